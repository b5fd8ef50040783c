"""Helpers shared by the tests: spots -> product solvers / oracle solvers."""
import numpy as np

from pps import pps_native as pn
from pps import workloads as wl
from oracle import cpu_oracle as co


def weights(r):
    return pn.parse_range(r) if isinstance(r, str) else np.asarray(r, dtype=np.float64)


def abi_cfgs(spot):
    if spot.street_cfgs:
        return [pn.bet_config(c.bet_text(), c.raise_text(), c.max_raises) for c in spot.street_cfgs]
    return [pn.bet_config(spot.cfg.bet_text(), spot.cfg.raise_text(), spot.cfg.max_raises)]


def solver(spot, **kw):
    streets = None
    if spot.street_cfgs:
        streets = [{"bets": c.bet_text(), "raises": c.raise_text() or [],
                    "max_raises": c.max_raises} for c in spot.street_cfgs]
    return pn.Solver(board=spot.board_text(), oop=weights(spot.oop), ip=weights(spot.ip),
                     pot=spot.pot, stack=spot.stack, bets=spot.cfg.bet_text(),
                     raises=spot.cfg.raise_text() or [], max_raises=spot.cfg.max_raises,
                     streets=streets, **kw)


def oracle(spot, precision=32, threads=None):
    cfgs = [co.cfg_from(c) for c in spot.street_cfgs] if spot.street_cfgs else \
        [co.cfg_from(spot.cfg)]
    w0, w1 = weights(spot.oop), weights(spot.ip)
    bset = set(spot.board)
    for i, (a, b) in enumerate((a, b) for a in range(52) for b in range(a + 1, 52)):
        if a in bset or b in bset:
            w0[i] = w1[i] = 0.0
    return co.Oracle(spot.board, w0, w1, spot.pot, spot.stack, cfgs, precision, threads)


def seeded_rows(meta, row_total, mode):
    """The reference's GPU_CFR_SEED_STRAT profile (cuda/gpu_cfr.cu:2066-2097)
    from decide metadata rows (regOff, na, player, nC, depth, nBoard, node,
    actBase)."""
    rows = np.zeros(row_total, dtype=np.float32)
    for mi, m in enumerate(meta.reshape(-1, 8)):
        reg, na, _, nc, depth = int(m[0]), int(m[1]), int(m[2]), int(m[3]), int(m[4])
        turn = depth <= 2
        ok = {2: turn, 3: not turn, 4: depth == 0, 5: depth == 1, 6: depth == 2,
              7: mi == 1, 8: mi == 2, 9: depth == 1 and mi != 1}.get(mode, True)
        if not ok or na < 2:
            continue
        for c in range(nc):
            p0 = np.float32(0.15 + 0.7 * ((c % 8) / 7.0))
            rows[reg + c] = p0
            rows[reg + nc + c] = np.float32(1.0) - p0
    return rows


def root_strategy(rows, na, n, w):
    """Range-weighted root frequencies from dense rows (reference
    rootStrategy, cuda/gpu_cfr.cu:2148-2175)."""
    r = np.asarray(rows[:na * n], dtype=np.float64).reshape(na, n)
    tot = r.sum(axis=0)
    sig = np.where(tot > 0, r / np.where(tot > 0, tot, 1), 1.0 / na)
    return (sig * w[None, :]).sum(axis=1) / w.sum()
