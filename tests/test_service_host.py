"""The solver service (pps/service.py) on the host, over a fake solver: the
registry, jobs and errors, and the action paths / node navigation that the
reference API builds from the tree structure (python/pps_api.py:184-276,
485-538). tests/test_gpu_service.py runs the same operations on real
solvers."""
import os
import threading
import time

import numpy as np
import pytest

from pps.service import ServiceError, SolverService

BOARD = [49, 33, 13, 5]  # Qs 9h 2d 7c (card id = suit * 13 + rank, suits c d h s)


class FakeSolver:
    """A 54-node turn tree in DFS pre-order:

    0 decide OOP [check -> 1, bet 150 -> 53 (fold)]
    1 decide IP  [check -> 2 (deal), bet 150 -> 52 (fold)]
    2 chance, one branch per remaining card: 2c -> 3, the others -> 5..51
    3 decide OOP on the river 2c [check -> 4 (showdown)]
    """

    def __init__(self):
        rest = [c for c in range(52) if c not in BOARD]
        assert len(rest) == 48 and rest[0] == 0
        kinds = [0, 0, 3, 0, 1] + [1] * 47 + [2, 2]
        kids = {0: [1, 53], 1: [2, 52], 2: [3] + list(range(5, 52)), 3: [4]}
        cb, ch = [], []
        for u in range(len(kinds)):
            cb.append(len(ch))
            ch.extend(kids.get(u, []))
        boards = []
        river = {3: 0, 4: 0}
        for c, node in zip(rest[1:], range(5, 52)):
            river[node] = c
        for u in range(len(kinds)):
            boards.extend(BOARD + [river[u]] if u in river else BOARD + [0])
        self.tree = {"kinds": kinds, "child_base": cb, "children": ch, "boards": boards}
        chk, bet = {"kind": "check", "amount": 0}, {"kind": "bet", "amount": 150}
        self.nodes = [
            {"index": 0, "node_id": 0, "player": 0, "depth": 0, "n_board": 4, "n_combos": 3,
             "actions": [chk, bet], "children": [1, 53]},
            {"index": 1, "node_id": 1, "player": 1, "depth": 1, "n_board": 4, "n_combos": 3,
             "actions": [chk, bet], "children": [2, 52]},
            {"index": 2, "node_id": 3, "player": 0, "depth": 3, "n_board": 5, "n_combos": 3,
             "actions": [chk], "children": [4]},
        ]
        self.total_iterations = 0
        self.iterations_run = 0
        self.num_nodes = len(kinds)
        self.num_decide_nodes = len(self.nodes)
        self.max_depth = 4
        self.chunk_sleep = 0.0

    def tree_structure(self):
        return self.tree

    def decide_nodes(self):
        return [dict(d) for d in self.nodes]

    def solve(self, n, algo="dcfr", target=-1.0):
        if algo not in ("dcfr", "hs30"):
            raise ValueError("unknown algo " + algo)
        self.total_iterations = 0
        return self.continue_solve(n, target)

    def continue_solve(self, n, target=-1.0):
        time.sleep(self.chunk_sleep)
        self.iterations_run = n
        self.total_iterations += n

    def reset(self):
        self.total_iterations = self.iterations_run = 0

    def stats(self):
        return {"ev_oop": 40.0, "ev_ip": 60.0, "exploitability": 1.0, "pair_mass": 1}

    def strategy(self, idx=0):
        if not 0 <= idx < len(self.nodes):
            raise ValueError("decide node %d out of range" % idx)
        return {"index": idx, "freqs": np.full((2, 3), 0.5, dtype=np.float32)}

    def save(self, path, compressed=False):
        with open(path, "wb") as f:
            f.write(b"PPSG" + bytes([4 if compressed else 3]))

    def player_cards(self, player):
        return [0, 1, 2, 3]

    def player_weights(self, player):
        return np.array([0.5, 1.0])


@pytest.fixture
def svc(tmp_path):
    s = SolverService(max_solvers=2, max_iters=50000, data_dir=str(tmp_path / "sol"))
    yield s
    s.close()


def add(svc, solver=None):
    return svc._add(solver or FakeSolver(), "Qs9h2d7c")


def test_paths_and_navigation(svc):
    sid = add(svc)
    nodes = svc.decide_nodes(sid, 0, 10)
    assert nodes["total"] == 3
    assert [n["path"] for n in nodes["nodes"]] == ["(root)", "check", "check — check — deal 2c"]
    assert [n["index"] for n in svc.decide_nodes(sid, 1, 1)["nodes"]] == [1]

    nav = svc.node_nav(sid, 0)
    assert nav["path"] == "(root)" and nav["player"] == 0 and nav["n_board"] == 4
    acts = {a["label"]: a for a in nav["actions"]}
    assert set(acts) == {"check", "bet 150"}
    assert acts["check"]["child_kind"] == "decide" and acts["check"]["next_decide"] == 1
    assert acts["bet 150"]["child_kind"] == "fold" and acts["bet 150"]["next_decide"] is None

    deal = svc.node_nav(sid, 1)["actions"][0]
    assert deal["child_kind"] == "chance" and deal["next_decide"] == 2
    cards = [b["card"] for b in deal["branches"]]
    assert len(cards) == len(set(cards)) == 48 and cards[0] == "2c"  # card id 0 is a card
    assert not set(cards) & {"Qs", "9h", "2d", "7c"} and "?" not in cards
    assert deal["branches"][0]["next_decide"] == 2
    assert all(b["next_decide"] is None for b in deal["branches"][1:])

    with pytest.raises(ServiceError) as e:
        svc.node_nav(sid, 3)
    assert e.value.status == 400


def test_registry_eviction_and_errors(svc):
    a, b = add(svc), add(svc)
    svc.get_solver(a)  # a is now the most recently used
    c = add(svc)
    assert {s["id"] for s in svc.list_solvers()} == {a, c}
    with pytest.raises(ServiceError) as e:
        svc.stats(b)
    assert e.value.status == 404
    assert svc.delete_solver(a) == {"removed": True}
    with pytest.raises(ServiceError) as e:
        svc.delete_solver(a)
    assert e.value.status == 404
    with pytest.raises(ServiceError) as e:  # an engine ValueError is a bad request
        svc.strategy(c, 7)
    assert e.value.status == 400
    st = svc.strategy(c, 1)
    assert st["freqs"] == [[0.5] * 3] * 2  # numpy made JSON-ready
    for n in (0, 50001):
        with pytest.raises(ServiceError) as e:
            svc.solve(c, {"max_iters": n})
        assert e.value.status == 422
    h = svc.health()
    assert h["solve_lock"] is False and h["solvers"] == 1 and h["max_solvers"] == 2


def test_files_are_sandboxed(svc):
    sid = add(svc)
    for bad in ("", ".", "..", "../x", "a/b", "a\\b"):
        with pytest.raises(ServiceError) as e:
            svc.save(sid, bad)
        assert e.value.status == 400
    r = svc.save(sid, "spot1", compressed=True)
    assert r == {"saved": True, "name": "spot1", "bytes": 5, "compressed": True}
    assert os.path.isfile(os.path.join(svc.data_dir, "spot1"))
    assert svc.list_solutions()["solutions"] == [{"name": "spot1", "bytes": 5}]
    with pytest.raises(ServiceError) as e:
        svc.load("missing")
    assert e.value.status == 404


def test_background_job_cancel_and_conflicts(svc):
    fake = FakeSolver()
    fake.chunk_sleep = 0.02
    sid = add(svc, fake)
    job = svc.solve(sid, {"max_iters": 40000, "wait": False})["job"]
    assert job["running"] and job["total"] == 40000
    for call in (lambda: svc.solve(sid, {"max_iters": 10}),
                 lambda: svc.continue_solve(sid, {"max_iters": 10, "wait": False}),
                 lambda: svc.reset(sid)):
        with pytest.raises(ServiceError) as e:
            call()
        assert e.value.status == 409
    assert svc.cancel(sid) == {"cancelled": True}
    meta = svc.wait_job(sid, timeout=10.0)
    assert meta["job"]["status"] == "cancelled" and not meta["job"]["running"]
    assert 0 < fake.total_iterations < 40000
    assert svc.cancel(sid) == {"cancelled": False}
    r = svc.continue_solve(sid, {"max_iters": 100})
    assert r["iterations_run"] == 100 and r["stats"]["ev_oop"] == 40.0


def test_one_job_per_solver_under_concurrent_starts(svc):
    fake = FakeSolver()
    fake.chunk_sleep = 0.02
    sid = add(svc, fake)
    out, barrier = [], threading.Barrier(8)

    def start():
        barrier.wait()
        try:
            svc.solve(sid, {"max_iters": 20000, "wait": False})
            out.append("started")
        except ServiceError as e:
            out.append(e.status)

    threads = [threading.Thread(target=start) for _ in range(8)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert sorted(out, key=str) == [409] * 7 + ["started"]
    svc.cancel(sid)
    assert svc.wait_job(sid, timeout=10.0)["job"]["status"] == "cancelled"
