"""pps.Batch: many spots solved at once on one GPU (batched and served).

No reference counterpart: the reference solves one spot per Solver and its
API server (python/pps_api.py) runs solves one at a time behind a lock.
Here submitted spots are compiled on host threads, admitted into one
device-resident forest while their footprints fit the HBM budget, iterated
together (one CUDA graph per DCFR iteration over every resident spot) and
retired one by one once their FP64 exploitability check reaches the target.

    import pps
    b = pps.Batch(check_every=64)
    t = b.submit(board="Qs9h2d7c3h", oop="...", ip="...", pot=100, stack=200,
                 bets="0.5,1,a", raises="2.5", target_frac=0.005)
    b.run()                      # or b.start() ... b.wait(t) ... b.stop()
    r = b.result(t)              # {"ev_oop", "ev_ip", "exploitability", ...}

A result does not depend on which other spots shared the device: each spot
runs the same kernels on its own rows, and its checks (first after
min(32, check_every) iterations, then where its exploitability, taken as
falling like 1/t^2, would meet the target, at most ``check_every`` apart,
in steps of 16; every ``check_every`` with ``fixed_checks=True``) depend on
its own exploitability values only.
"""
from __future__ import annotations

import ctypes as C
from typing import Any, Dict, List, Optional, Sequence

import numpy as np

from . import _abi
from ._abi import check, lib
from .pps_native import _KIND, _bet_config, _range_arg, make_spot, parse_board


def _result_dict(r: _abi.BatchResult) -> Dict[str, Any]:
    acts = [{"kind": _KIND.get(r.root_action[a].kind, str(r.root_action[a].kind)),
             "amount": int(r.root_action[a].amount)} for a in range(r.root_actions)]
    return {
        "ticket": int(r.ticket), "status": int(r.status),
        "error": r.error.decode(errors="replace"), "converged": bool(r.converged),
        "iterations": int(r.iterations), "num_nodes": int(r.num_nodes),
        "ev_oop": r.ev0, "ev_ip": r.ev1, "exploitability": r.exploitability,
        "target": r.target, "pair_mass": int(r.pair_mass),
        "submit_ms": r.submit_ms, "admit_ms": r.admit_ms, "finish_ms": r.finish_ms,
        "latency_ms": r.finish_ms - r.submit_ms, "device_bytes": int(r.device_bytes),
        "root_actions": acts, "root_freqs": [r.root_freqs[a] for a in range(r.root_actions)],
        "root_combos": int(r.root_combos),
    }


def _cfg_array(bets: Any, raises: Any, max_raises: int,
               streets: Optional[Sequence[Dict[str, Any]]]):
    if streets is None:
        arr = (_abi.BetConfig * 1)()
        arr[0] = _bet_config(bets, raises, max_raises)
        return arr, 1
    if len(streets) != 3:
        raise RuntimeError("streets must hold 3 configs (flop, turn, river)")
    arr = (_abi.BetConfig * 3)()
    for k, sc in enumerate(streets):
        arr[k] = _bet_config(sc.get("bets", bets), sc.get("raises", raises),
                             sc.get("max_raises", max_raises))
    return arr, 3


class Batch:
    """Batched / served DCFR solving on the current CUDA device."""

    def __init__(self, hbm_budget: int = 0, check_every: int = 64, max_iterations: int = 4096,
                 compile_threads: int = 0, algo: str = "dcfr", fixed_checks: bool = False):
        cfg = _abi.BatchConfig()
        lib.pps_gb_batch_config_default(C.byref(cfg))
        cfg.hbm_budget = int(hbm_budget)
        cfg.check_every = int(check_every)
        cfg.fixed_checks = 1 if fixed_checks else 0
        cfg.max_iterations = int(max_iterations)
        cfg.compile_threads = int(compile_threads)
        cfg.algo = algo.encode()
        self._h = C.c_void_p()
        check(lib.pps_gb_batch_create(C.byref(cfg), C.byref(self._h)))

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h and h.value:
            lib.pps_gb_batch_destroy(h)
            self._h = C.c_void_p()

    def __del__(self):
        self.close()

    def __enter__(self) -> "Batch":
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    # -- requests --
    def submit(self, board: Any, oop: Any, ip: Any, pot: int, stack: int,
               bets: Any = "0.75,a", raises: Any = "2.5,3", max_raises: int = 0,
               streets: Optional[Sequence[Dict[str, Any]]] = None,
               target: Optional[float] = None, target_frac: Optional[float] = None) -> int:
        """Queues a spot (the Solver constructor's keywords). The spot is
        solved until its exploitability is at most ``target`` chips (or
        ``target_frac`` of the pot); with neither it runs to max_iterations."""
        spot = make_spot(parse_board(board), _range_arg(oop), _range_arg(ip), pot, stack)
        return self.submit_spot(spot, _cfg_array(bets, raises, max_raises, streets),
                                target if target is not None else
                                (target_frac * pot if target_frac is not None else -1.0))

    def submit_spot(self, spot: _abi.Spot, cfgs, target: float) -> int:
        arr, n = cfgs
        t = C.c_int64()
        check(lib.pps_gb_batch_submit(self._h, C.byref(spot), arr, n, float(target),
                                      C.byref(t)))
        return t.value

    def set_budget(self, hbm_budget: int) -> None:
        check(lib.pps_gb_batch_set_budget(self._h, int(hbm_budget)))

    # -- driving --
    def run(self, timeout: float = 0.0) -> bool:
        """Drives the batch on this thread until every request finished
        (True) or ``timeout`` seconds passed (False)."""
        rc = lib.pps_gb_batch_run(self._h, float(timeout))
        if rc == _abi.PENDING:
            return False
        check(rc)
        return True

    def start(self) -> None:
        """Serve mode: a library thread drives the batch until stop()."""
        check(lib.pps_gb_batch_start(self._h))

    def stop(self) -> None:
        check(lib.pps_gb_batch_stop(self._h))

    # -- results --
    def poll(self, ticket: int) -> Optional[Dict[str, Any]]:
        r = _abi.BatchResult()
        rc = lib.pps_gb_batch_poll(self._h, int(ticket), C.byref(r))
        if rc == _abi.PENDING:
            return None
        check(rc)
        return _result_dict(r)

    def wait(self, ticket: int, timeout: float = 0.0) -> Optional[Dict[str, Any]]:
        r = _abi.BatchResult()
        rc = lib.pps_gb_batch_wait(self._h, int(ticket), float(timeout), C.byref(r))
        if rc == _abi.PENDING:
            return None
        check(rc)
        return _result_dict(r)

    def result(self, ticket: int) -> Dict[str, Any]:
        r = self.poll(ticket)
        if r is None:
            raise RuntimeError("request %d has not finished" % ticket)
        return r

    def root_rows(self, ticket: int) -> np.ndarray:
        """Cumulative root strategy rows (root_actions x root_combos)."""
        r = self.result(ticket)
        n = C.c_int64()
        buf = np.zeros(max(1, len(r["root_actions"]) * r["root_combos"]), dtype=np.float32)
        check(lib.pps_gb_batch_root_rows(self._h, int(ticket),
                                         buf.ctypes.data_as(C.POINTER(C.c_float)), buf.size,
                                         C.byref(n)))
        return buf[:n.value].reshape(len(r["root_actions"]), r["root_combos"]) \
            if n.value else np.zeros((0, 0), dtype=np.float32)

    def collect(self, max_results: int = 1 << 16) -> List[Dict[str, Any]]:
        out = (_abi.BatchResult * max(1, max_results))()
        n = C.c_int()
        check(lib.pps_gb_batch_collect(self._h, out, max_results, C.byref(n)))
        return [_result_dict(out[i]) for i in range(n.value)]

    def info(self) -> Dict[str, int]:
        i = _abi.BatchInfo()
        check(lib.pps_gb_batch_get_info(self._h, C.byref(i)))
        return {k: (float if t is C.c_double else int)(getattr(i, k))
                for k, t in _abi.BatchInfo._fields_}


def footprint(board: Any, oop: Any, ip: Any, pot: int, stack: int, bets: Any = "0.75,a",
              raises: Any = "2.5,3", max_raises: int = 0,
              streets: Optional[Sequence[Dict[str, Any]]] = None) -> int:
    """Device bytes the spot occupies in a Batch (host-only compile)."""
    spot = make_spot(parse_board(board), _range_arg(oop), _range_arg(ip), pot, stack)
    arr, n = _cfg_array(bets, raises, max_raises, streets)
    b = C.c_int64()
    check(lib.pps_gb_batch_footprint(C.byref(spot), arr, n, C.byref(b)))
    return b.value
