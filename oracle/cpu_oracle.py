"""ctypes wrapper of the CPU oracle (oracle/oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference legs, to check the GPU solver against.
It never backs the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np
from typing import Dict

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

SCHEDULES = {"dcfr": 0, "hs30": 1, "dcfr-g2": 2, "dcfr-noreset": 3, "dcfr-g2-noreset": 4}


class OrcCfg(C.Structure):
    _fields_ = [("bets", C.c_double * 16), ("n_bets", C.c_int), ("raises", C.c_double * 16),
                ("n_raises", C.c_int), ("allin", C.c_int), ("geo", C.c_int),
                ("max_raises", C.c_int), ("add_t", C.c_double), ("force_t", C.c_double),
                ("merge_t", C.c_double)]


def build() -> str:
    subprocess.run(["sh", os.path.join(HERE, "build_oracle.sh")], check=True,
                   capture_output=True)
    return LIB


_lib = None


EXPORT_CB = C.CFUNCTYPE(None, C.c_void_p, C.c_char_p, C.c_char, C.c_void_p, C.c_int64)
_DT = {b"i": np.int32, b"q": np.int64, b"B": np.uint8, b"f": np.float32, b"d": np.float64}


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.POINTER(C.c_uint8), C.c_int, C.POINTER(C.c_double),
                                 C.POINTER(C.c_double), C.c_int64, C.c_int64,
                                 C.POINTER(OrcCfg), C.c_int, C.c_int]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_num_nodes.argtypes = [C.c_void_p]
        L.orc_row_total.restype = C.c_int64
        L.orc_row_total.argtypes = [C.c_void_p]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_iterate.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]
        L.orc_value.restype = C.c_double
        L.orc_value.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double)]
        L.orc_rows.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_float)]
        L.orc_set_rows.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_float)]
        L.orc_pair_mass.restype = C.c_double
        L.orc_pair_mass.argtypes = [C.c_void_p]
        L.orc_strength7.restype = C.c_uint64
        L.orc_strength7.argtypes = [C.POINTER(C.c_uint8)]
        L.orc_actions.argtypes = [C.c_int64, C.c_int64, C.POINTER(OrcCfg), C.c_int64, C.c_int64,
                                  C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int),
                                  C.POINTER(C.c_int64)]
        L.orc_export.argtypes = [C.c_void_p, EXPORT_CB, C.c_void_p]
        _lib = L
    return _lib


def make_cfg(bets, raises, allin=False, geo=False, max_raises=0, add_t=1.5, force_t=0.15,
             merge_t=0.1) -> OrcCfg:
    c = OrcCfg()
    c.n_bets = len(bets)
    for i, b in enumerate(bets):
        c.bets[i] = b
    c.n_raises = len(raises)
    for i, r in enumerate(raises):
        c.raises[i] = r
    c.allin, c.geo, c.max_raises = int(allin), int(geo), int(max_raises)
    c.add_t, c.force_t, c.merge_t = add_t, force_t, merge_t
    return c


def cfg_from(bc) -> OrcCfg:
    """From a workloads.BetCfg."""
    return make_cfg(bc.bets, bc.raises, bc.allin, bc.geometric, bc.max_raises, bc.add_allin,
                    bc.force_allin, bc.merging)


class Oracle:
    """One spot in the CPU restatement; rows in the reference dense layout."""

    def __init__(self, board, w0, w1, pot, stack, cfgs, precision=32, threads=None):
        L = lib()
        if threads:
            L.orc_set_threads(int(threads))
        b = (C.c_uint8 * 5)(*list(board))
        a0 = np.ascontiguousarray(w0, dtype=np.float64)
        a1 = np.ascontiguousarray(w1, dtype=np.float64)
        arr = (OrcCfg * len(cfgs))(*cfgs)
        self.h = L.orc_create(b, len(board), a0.ctypes.data_as(C.POINTER(C.c_double)),
                              a1.ctypes.data_as(C.POINTER(C.c_double)), int(pot), int(stack),
                              arr, len(cfgs), int(precision))
        if not self.h:
            raise ValueError("empty range after board filtering")
        self.total = 0

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    @property
    def num_nodes(self) -> int:
        return lib().orc_num_nodes(self.h)

    @property
    def row_total(self) -> int:
        return lib().orc_row_total(self.h)

    def iterate(self, n, planned=None, algo="dcfr", t0=None):
        t0 = self.total if t0 is None else t0
        lib().orc_iterate(self.h, int(t0), int(n), int(planned or n), SCHEDULES[algo])
        self.total = t0 + n

    def value(self, tr, mode):
        """mode 1 = EV vs the average strategy, 2 = best response (f64)."""
        return lib().orc_value(self.h, int(tr), int(mode), None)

    def value_row(self, tr, mode, n):
        row = np.zeros(n)
        v = lib().orc_value(self.h, int(tr), int(mode), row.ctypes.data_as(C.POINTER(C.c_double)))
        return v, row

    def stats(self, pot):
        ev0, ev1 = self.value(0, 1), self.value(1, 1)
        br0, br1 = self.value(0, 2), self.value(1, 2)
        return {"ev_oop": ev0, "ev_ip": ev1, "exploitability": (br0 + br1 - pot) / 2.0}

    def rows(self, which):
        out = np.zeros(self.row_total, dtype=np.float32)
        lib().orc_rows(self.h, int(which), out.ctypes.data_as(C.POINTER(C.c_float)))
        return out

    def set_rows(self, which, rows):
        a = np.ascontiguousarray(rows, dtype=np.float32)
        lib().orc_set_rows(self.h, int(which), a.ctypes.data_as(C.POINTER(C.c_float)))


def reference_layout(board, w0, w1, pot, stack, cfg) -> Dict[str, np.ndarray]:
    """The reference's device layout of a spot (the arrays its init()
    uploads, cuda/gpu_cfr.cu:1363-1827), restated by the oracle from its own
    tree: what the reference's kernels run on (oracle/ref_gpu.py). One bet
    config for every street, as in the reference. w0 / w1: 1326 weights."""
    o = Oracle(board, w0, w1, pot, stack, [cfg], 32, 1)
    out: Dict[str, np.ndarray] = {}

    def sink(_user, name, dt, data, n):
        t = _DT[dt]
        a = np.ctypeslib.as_array(C.cast(data, C.POINTER(C.c_uint8)), (int(n) * np.dtype(t).itemsize,)) \
            if n else np.zeros(0, dtype=np.uint8)
        out[name.decode()] = a.view(t).copy()

    cb = EXPORT_CB(sink)
    lib().orc_export(o.h, cb, None)
    return out


def oracle_for(spot, threads=None, precision=32, parse_range=None):
    """An Oracle for a workloads.Spot; string ranges need `parse_range`."""
    def w(r):
        if isinstance(r, str):
            if parse_range is None:
                raise ValueError("string range needs a parser")
            return np.asarray(parse_range(r), dtype=np.float64)
        return np.array(r, dtype=np.float64)
    cfgs = [cfg_from(c) for c in spot.street_cfgs] if spot.street_cfgs else [cfg_from(spot.cfg)]
    return Oracle(spot.board, w(spot.oop), w(spot.ip), spot.pot, spot.stack, cfgs, precision,
                  threads)


def strength7(cards) -> int:
    b = (C.c_uint8 * 7)(*[int(c) for c in cards])
    return int(lib().orc_strength7(b))


def actions(pot_base, stack, cfg: OrcCfg, sc0, sc1, actor, after_allin, num_bets, streets):
    kinds = (C.c_int * 64)()
    amts = (C.c_int64 * 64)()
    n = lib().orc_actions(pot_base, stack, C.byref(cfg), sc0, sc1, actor, int(after_allin),
                          num_bets, streets, kinds, amts)
    return [(kinds[i], int(amts[i])) for i in range(n)]
