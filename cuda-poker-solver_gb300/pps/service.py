"""The solver service behind the HTTP front-end (pps/api.py).

It has the same operations, arguments and answers as the reference's
python/pps_api.py:
- a registry of solvers with LRU eviction;
- solve / continue / cancel / reset, and background jobs in iteration chunks;
- stats, strategy, decide-node listing with action paths, node navigation,
  range, root / node EVs, runout summaries;
- save / load sandboxed to a data directory;
- one-shot solves.

The difference is concurrency. The reference serializes every solve behind
one global lock (``SOLVE_LOCK``, python/pps_api.py:164-166). Here each solver
has its own CUDA stream and its own lock, so solves of different solvers run
at once on the GPU, while calls on one solver serialize. One-shot solves with
an exploitability target and nothing else asked go through one shared
:class:`pps.Batch` in serve mode (continuous batching): requests that arrive
while others are on the GPU join the same launches.

No web framework is needed here: errors are :class:`ServiceError` carrying
an HTTP status; pps/api.py maps them onto FastAPI.
"""
from __future__ import annotations

import os
import threading
import time
import uuid
from collections import OrderedDict
from typing import Any, Dict, List, Optional

import numpy as np

from . import pps_native as pn
from .batch import Batch


class ServiceError(Exception):
    """An error answer: HTTP status code and message."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status
        self.message = message


def _engine(fn, *args, **kwargs):
    """Runs an engine call, mapping its errors to status 400
    (python/pps_api.py:169-174)."""
    try:
        return fn(*args, **kwargs)
    except (ValueError, RuntimeError) as e:
        raise ServiceError(400, str(e)) from e


def jsonable(obj: Any) -> Any:
    """numpy arrays and scalars to plain JSON values."""
    if isinstance(obj, dict):
        return {k: jsonable(v) for k, v in obj.items()}
    if isinstance(obj, (list, tuple)):
        return [jsonable(v) for v in obj]
    if isinstance(obj, np.ndarray):
        return obj.tolist()
    if isinstance(obj, np.generic):
        return obj.item()
    return obj


def action_text(a: Dict[str, Any]) -> str:
    k = a["kind"]
    if k in ("bet", "raise"):
        return "%s %d" % (k, a.get("amount", 0))
    if k == "allin":
        return "all-in"
    return k


class _Entry:
    def __init__(self, solver: pn.Solver, board: str):
        self.solver = solver
        self.lock = threading.Lock()
        self.created = time.time()
        self.last_used = self.created
        self.board = board
        self.paths: Optional[List[str]] = None
        self.tree: Optional[Dict[str, List[int]]] = None
        self.decide_idx: Dict[int, int] = {}
        self.nodes: Optional[List[Dict[str, Any]]] = None
        self.job: Optional[Dict[str, Any]] = None


KIND_NAME = {0: "decide", 1: "showdown", 2: "fold", 3: "chance"}


class SolverService:
    """Solver registry, jobs and queries (python/pps_api.py's operations)."""

    def __init__(self, max_solvers: Optional[int] = None, max_iters: Optional[int] = None,
                 data_dir: Optional[str] = None, batch: Optional[Batch] = None):
        self.max_solvers = int(max_solvers or os.environ.get("PPS_API_MAX_SOLVERS", "8"))
        self.max_iters = int(max_iters or os.environ.get("PPS_API_MAX_ITERS", "1000000"))
        self.data_dir = os.path.abspath(data_dir or os.environ.get(
            "PPS_API_DATA_DIR", os.path.join(os.getcwd(), "api-solutions")))
        self._d: "OrderedDict[str, _Entry]" = OrderedDict()
        self._mu = threading.Lock()
        self._batch = batch
        self._batch_mu = threading.Lock()

    # ---- registry (python/pps_api.py:120-160) ----
    def _add(self, solver: pn.Solver, board: str) -> str:
        with self._mu:
            sid = uuid.uuid4().hex[:12]
            self._d[sid] = _Entry(solver, board)
            self._d.move_to_end(sid)
            while len(self._d) > self.max_solvers:
                self._d.popitem(last=False)
        return sid

    def _get(self, sid: str) -> _Entry:
        with self._mu:
            e = self._d.get(sid)
            if e is None:
                raise ServiceError(404, "no solver %s" % sid)
            e.last_used = time.time()
            self._d.move_to_end(sid)
            return e

    def _meta(self, sid: str, e: _Entry) -> Dict[str, Any]:
        s = e.solver
        return {"id": sid, "board": e.board, "num_nodes": s.num_nodes,
                "num_decide_nodes": s.num_decide_nodes, "max_depth": s.max_depth,
                "total_iterations": s.total_iterations, "iterations_run": s.iterations_run,
                "job": dict(e.job) if e.job else None}

    def _check_iters(self, n: int) -> int:
        if n <= 0 or n > self.max_iters:
            raise ServiceError(422, "max_iters must be in [1, %d]" % self.max_iters)
        return int(n)

    @staticmethod
    def _new_solver(spec: Dict[str, Any]) -> pn.Solver:
        return _engine(pn.Solver, board=spec["board"], oop=spec["oop"], ip=spec["ip"],
                       pot=spec["pot"], stack=spec["stack"], bets=spec.get("bets", "0.75,a"),
                       raises=spec.get("raises", "2.5,3"),
                       max_raises=spec.get("max_raises", 0))

    def health(self) -> Dict[str, Any]:
        with self._mu:
            n = len(self._d)
        return {"status": "ok", "solvers": n, "max_solvers": self.max_solvers,
                "max_iters": self.max_iters, "data_dir": self.data_dir,
                "solve_lock": False, "batch": self._batch is not None}

    def create_solver(self, spec: Dict[str, Any]) -> Dict[str, Any]:
        t0 = time.perf_counter()
        solver = self._new_solver(spec)
        ms = (time.perf_counter() - t0) * 1000.0
        sid = self._add(solver, spec["board"])
        out = self._meta(sid, self._get(sid))
        out["compile_ms"] = round(ms, 1)
        return jsonable(out)

    def list_solvers(self) -> List[Dict[str, Any]]:
        with self._mu:
            items = list(self._d.items())
        return [dict(id=sid, board=e.board, created=e.created, last_used=e.last_used,
                     total_iterations=e.solver.total_iterations,
                     iterations_run=e.solver.iterations_run, num_nodes=e.solver.num_nodes)
                for sid, e in items]

    def get_solver(self, sid: str) -> Dict[str, Any]:
        return self._meta(sid, self._get(sid))

    def delete_solver(self, sid: str) -> Dict[str, bool]:
        with self._mu:
            if self._d.pop(sid, None) is None:
                raise ServiceError(404, "no solver %s" % sid)
        return {"removed": True}

    # ---- solving (python/pps_api.py:347-452) ----
    def _job_worker(self, e: _Entry, kind: str, p: Dict[str, Any]) -> None:
        """Iteration chunks with progress; a chunked continuation follows the
        same DCFR schedule as one long solve."""
        s = e.solver
        target = p.get("target") or -1.0
        total = p["max_iters"]
        chunk = max(128, total // 50)
        remaining = total
        e.job["start"] = s.total_iterations
        try:
            if kind == "solve":
                take = min(chunk, remaining)
                with e.lock:
                    s.solve(take, p.get("algo", "dcfr"), target)
                e.job["done"] = s.total_iterations - e.job["start"]
                remaining -= s.iterations_run
                if s.iterations_run < take:
                    remaining = 0
            while remaining > 0 and not e.job["cancel"]:
                take = min(chunk, remaining)
                with e.lock:
                    s.continue_solve(take, target)
                e.job["done"] = s.total_iterations - e.job["start"]
                ran = s.iterations_run
                remaining -= ran
                if ran < take:
                    remaining = 0
            e.job["status"] = "cancelled" if e.job["cancel"] else "done"
        except Exception as ex:  # an engine error ends the job, not the service
            e.job["status"] = "error"
            e.job["error"] = str(ex)
        finally:
            e.job["running"] = False

    def _start_job(self, sid: str, e: _Entry, kind: str, p: Dict[str, Any]) -> Dict[str, Any]:
        with self._mu:  # check and claim at once: two requests cannot both start a job
            if e.job and e.job["running"]:
                raise ServiceError(409, "a solve job is already running on this solver "
                                        "(POST /solvers/{id}/cancel first)")
            e.job = {"running": True, "status": "running", "kind": kind, "done": 0,
                     "start": 0, "total": p["max_iters"], "target": p.get("target"),
                     "error": None, "cancel": False}
            job = dict(e.job)
        threading.Thread(target=self._job_worker, args=(e, kind, p), daemon=True).start()
        return {"id": sid, "job": job}

    def _busy(self, e: _Entry) -> None:
        if e.job and e.job["running"]:
            raise ServiceError(409, "a solve job is running on this solver")

    def solve(self, sid: str, p: Dict[str, Any]) -> Dict[str, Any]:
        e = self._get(sid)
        p = dict(p)
        p["max_iters"] = self._check_iters(p.get("max_iters", 2000))
        if not p.get("wait", True):
            return self._start_job(sid, e, "solve", p)
        self._busy(e)
        with e.lock:
            t0 = time.perf_counter()
            _engine(e.solver.solve, p["max_iters"], p.get("algo", "dcfr"),
                    p.get("target") or -1.0)
            ms = (time.perf_counter() - t0) * 1000.0
            st = _engine(e.solver.stats)
        return jsonable({"solve_ms": round(ms, 1), "iterations_run": e.solver.iterations_run,
                         "total_iterations": e.solver.total_iterations, "stats": st})

    def continue_solve(self, sid: str, p: Dict[str, Any]) -> Dict[str, Any]:
        e = self._get(sid)
        p = dict(p)
        p["max_iters"] = self._check_iters(p.get("max_iters", 2000))
        if not p.get("wait", True):
            return self._start_job(sid, e, "continue", p)
        self._busy(e)
        with e.lock:
            t0 = time.perf_counter()
            _engine(e.solver.continue_solve, p["max_iters"], p.get("target") or -1.0)
            ms = (time.perf_counter() - t0) * 1000.0
            st = _engine(e.solver.stats)
        return jsonable({"continue_ms": round(ms, 1), "iterations_run": e.solver.iterations_run,
                         "total_iterations": e.solver.total_iterations, "stats": st})

    def cancel(self, sid: str) -> Dict[str, Any]:
        e = self._get(sid)
        if not (e.job and e.job["running"]):
            return {"cancelled": False}
        e.job["cancel"] = True
        return {"cancelled": True}

    def wait_job(self, sid: str, timeout: float = 60.0) -> Dict[str, Any]:
        """Blocks until the solver's background job ends (or timeout)."""
        e = self._get(sid)
        t0 = time.time()
        while e.job and e.job["running"] and time.time() - t0 < timeout:
            time.sleep(0.01)
        return self._meta(sid, e)

    def reset(self, sid: str) -> Dict[str, Any]:
        e = self._get(sid)
        self._busy(e)
        with e.lock:
            _engine(e.solver.reset)
        return self._meta(sid, e)

    # ---- queries (python/pps_api.py:455-585) ----
    def _locked(self, sid: str, fn, *args):
        e = self._get(sid)
        with e.lock:
            return jsonable(_engine(fn(e), *args))

    def stats(self, sid: str) -> Dict[str, Any]:
        return self._locked(sid, lambda e: e.solver.stats)

    def strategy(self, sid: str, node: int = 0) -> Dict[str, Any]:
        return self._locked(sid, lambda e: e.solver.strategy, int(node))

    def root_ev(self, sid: str) -> Dict[str, Any]:
        return self._locked(sid, lambda e: e.solver.root_ev)

    def node_ev(self, sid: str, node: int = 0) -> Dict[str, Any]:
        return self._locked(sid, lambda e: e.solver.node_ev, int(node))

    def runout_summary(self, sid: str, node: int = 0, action: int = 0) -> Dict[str, Any]:
        return self._locked(sid, lambda e: e.solver.runout_summary, int(node), int(action))

    def range(self, sid: str, player: int = 0) -> Dict[str, Any]:
        if player not in (0, 1):
            raise ServiceError(422, "player must be 0 or 1")
        e = self._get(sid)
        with e.lock:
            cards = _engine(e.solver.player_cards, player)
            w = _engine(e.solver.player_weights, player)
        return {"player": player,
                "combos": [pn.card_text(cards[2 * i]) + pn.card_text(cards[2 * i + 1])
                           for i in range(len(w))],
                "weights": jsonable(np.asarray(w))}

    def _paths(self, e: _Entry) -> List[str]:
        """Action-path label per node (decide edges: the action; chance
        edges: "deal <card>"), built once per solver with the tree and the
        decide-node list (python/pps_api.py:184-236)."""
        if e.paths is not None:
            return e.paths
        with e.lock:
            tree = _engine(e.solver.tree_structure)
            dns = _engine(e.solver.decide_nodes)
        kinds, cb, ch, bd = tree["kinds"], tree["child_base"], tree["children"], tree["boards"]
        n = len(kinds)
        acts = {d["node_id"]: d["actions"] for d in dns}
        paths = [""] * n
        for u in range(n):
            p = paths[u]
            cnt = (cb[u + 1] if u + 1 < n else len(ch)) - cb[u]
            if cnt <= 0:
                continue
            if kinds[u] == 0:
                for i, a in enumerate(acts[u]):
                    c = ch[cb[u] + i]
                    lab = action_text(a)
                    paths[c] = "%s — %s" % (p, lab) if p else lab
            elif kinds[u] == 3:
                nb = 52 - cnt
                for i in range(cnt):
                    c = ch[cb[u] + i]
                    paths[c] = "%s — deal %s" % (p, self._dealt(bd, u, c, nb))
        e.tree = tree
        e.decide_idx = {d["node_id"]: d["index"] for d in dns}
        e.nodes = dns
        e.paths = paths
        return paths

    @staticmethod
    def _dealt(boards: List[int], parent: int, child: int, n_parent: int) -> str:
        """The card a chance branch added (card id 0 is 2c: slice by the
        parent's board length, not by nonzero slots)."""
        rest = list(boards[5 * child:5 * child + n_parent + 1])
        for c in boards[5 * parent:5 * parent + n_parent]:
            rest.remove(c)
        return pn.card_text(rest[0]) if len(rest) == 1 else "?"

    def _first_decide(self, e: _Entry, start: int) -> Optional[int]:
        kinds, cb, ch = e.tree["kinds"], e.tree["child_base"], e.tree["children"]
        n = len(kinds)
        q = [start]
        while q:
            u = q.pop(0)
            for i in range(cb[u], cb[u + 1] if u + 1 < n else len(ch)):
                c = ch[i]
                if kinds[c] == 0:
                    return c
                if kinds[c] == 3:
                    q.append(c)
        return None

    def decide_nodes(self, sid: str, offset: int = 0, limit: int = 200) -> Dict[str, Any]:
        if offset < 0 or not 0 < limit <= 2000:
            raise ServiceError(422, "offset >= 0 and 0 < limit <= 2000")
        e = self._get(sid)
        paths = self._paths(e)
        out = []
        for d in e.nodes[offset:offset + limit]:
            d = dict(d)
            d["path"] = paths[d["node_id"]] or "(root)"
            out.append(d)
        return jsonable({"total": len(e.nodes), "nodes": out})

    def node_nav(self, sid: str, node: int = 0) -> Dict[str, Any]:
        """One entry per action of decide node `node`: the child's kind and
        the first decide node reached through it, with per-card branches for
        a deal (python/pps_api.py:485-538)."""
        e = self._get(sid)
        paths = self._paths(e)
        if not 0 <= node < len(e.nodes):
            raise ServiceError(400, "decide node %d out of range" % node)
        d = e.nodes[node]
        kinds, cb, ch, bd = (e.tree["kinds"], e.tree["child_base"], e.tree["children"],
                             e.tree["boards"])
        n = len(kinds)

        def count(u):
            return (cb[u + 1] if u + 1 < n else len(ch)) - cb[u]

        actions = []
        for a, child in zip(d["actions"], d["children"]):
            item = {"label": action_text(a), "kind": a["kind"], "amount": a.get("amount", 0),
                    "child_node": child, "child_kind": KIND_NAME[kinds[child]]}
            nxt = child if kinds[child] == 0 else self._first_decide(e, child)
            item["next_decide"] = e.decide_idx[nxt] if nxt is not None else None
            if kinds[child] == 3:
                nb = 52 - count(child)
                branches = []
                for i in range(count(child)):
                    bc = ch[cb[child] + i]
                    bn = bc if kinds[bc] == 0 else self._first_decide(e, bc)
                    branches.append({"card": self._dealt(bd, child, bc, nb),
                                     "next_decide": e.decide_idx[bn] if bn is not None else None})
                item["branches"] = branches
            actions.append(item)
        return jsonable({"node": node, "path": paths[d["node_id"]] or "(root)",
                         "player": d["player"], "n_board": d["n_board"], "actions": actions})

    # ---- files (python/pps_api.py:587-627) ----
    def _data_path(self, name: str) -> str:
        if not name or "/" in name or "\\" in name or name in (".", ".."):
            raise ServiceError(400, "bad solution name %r" % name)
        os.makedirs(self.data_dir, exist_ok=True)
        return os.path.join(self.data_dir, name)

    def save(self, sid: str, name: str, compressed: bool = False) -> Dict[str, Any]:
        e = self._get(sid)
        path = self._data_path(name)
        with e.lock:
            _engine(e.solver.save, path, compressed)
        return {"saved": True, "name": name, "bytes": os.path.getsize(path),
                "compressed": bool(compressed)}

    def load(self, name: str) -> Dict[str, Any]:
        path = self._data_path(name)
        if not os.path.isfile(path):
            raise ServiceError(404, "no solution file %r" % name)
        solver = _engine(pn.Solver.load, path)
        sid = self._add(solver, name)
        out = self._meta(sid, self._get(sid))
        out["name"] = name
        return jsonable(out)

    def list_solutions(self) -> Dict[str, Any]:
        os.makedirs(self.data_dir, exist_ok=True)
        out = []
        for name in sorted(os.listdir(self.data_dir)):
            p = os.path.join(self.data_dir, name)
            if os.path.isfile(p):
                out.append({"name": name, "bytes": os.path.getsize(p)})
        return {"data_dir": self.data_dir, "solutions": out}

    # ---- one-shot (python/pps_api.py:630-656) ----
    def _shared_batch(self) -> Batch:
        with self._batch_mu:
            if self._batch is None:
                self._batch = Batch()
                self._batch.start()
            return self._batch

    def close(self) -> None:
        with self._batch_mu:
            if self._batch is not None:
                self._batch.stop()
                self._batch.close()
                self._batch = None

    def solve_oneshot(self, body: Dict[str, Any]) -> Dict[str, Any]:
        """Compile, solve, answer. A request with an exploitability target
        that asks for nothing but the solution's stats and root strategy is
        served by the shared batch (continuous batching with every other
        such request); otherwise a Solver of its own runs it."""
        iters = self._check_iters(body.get("max_iters", 2000))
        target = body.get("target")
        wants_solver = body.get("strategy_nodes") or body.get("root_ev") or body.get("keep")
        if target and not wants_solver and body.get("algo", "dcfr") == "dcfr":
            b = self._shared_batch()
            t0 = time.perf_counter()
            ticket = _engine(b.submit, body["board"], body["oop"], body["ip"], body["pot"],
                             body["stack"], bets=body.get("bets", "0.75,a"),
                             raises=body.get("raises", "2.5,3"),
                             max_raises=body.get("max_raises", 0), target=float(target))
            r = b.wait(ticket)
            ms = (time.perf_counter() - t0) * 1000.0
            if r["status"] != 0:
                raise ServiceError(400, r["error"])
            return jsonable({
                "served_by": "batch", "solve_ms": round(ms, 1),
                "iterations_run": r["iterations"],
                "stats": {"ev_oop": r["ev_oop"], "ev_ip": r["ev_ip"],
                          "exploitability": r["exploitability"], "pair_mass": r["pair_mass"]},
                "root_strategy": {"actions": r["root_actions"], "freqs": r["root_freqs"]},
                "converged": r["converged"]})
        t0 = time.perf_counter()
        solver = self._new_solver(body)
        compile_ms = (time.perf_counter() - t0) * 1000.0
        t1 = time.perf_counter()
        _engine(solver.solve, iters, body.get("algo", "dcfr"), target or -1.0)
        solve_ms = (time.perf_counter() - t1) * 1000.0
        out: Dict[str, Any] = {"served_by": "solver", "compile_ms": round(compile_ms, 1),
                               "solve_ms": round(solve_ms, 1),
                               "iterations_run": solver.iterations_run,
                               "stats": _engine(solver.stats)}
        for n in body.get("strategy_nodes") or []:
            out.setdefault("strategies", {})[n] = _engine(solver.strategy, n)
        if body.get("root_ev"):
            out["root_ev"] = _engine(solver.root_ev)
        if body.get("keep"):
            out["solver_id"] = self._add(solver, body["board"])
        return jsonable(out)
