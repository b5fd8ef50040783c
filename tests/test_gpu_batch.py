"""Batched and served solving (pps.Batch over the pps_gb_batch_* C ABI).

Gates:
* a spot's result is the same alone and in the mix: same iteration count,
  EVs and exploitability within 1e-9 chips, root strategy rows within the
  row tolerance of the parity tests (normwise 5e-5; the rows are computed
  by the same kernels on the spot's own rows, so they agree exactly in
  practice);
* a batch result equals a lone Solver run for the same number of
  iterations (same tolerances);
* every converged result is at or below its target, checked at multiples
  of 16 iterations (adaptive schedule) or of check_every (fixed schedule);
* EVs of river spots are within 0.01 chips of the FP64 CPU oracle run for
  the same iterations;
* served mode overlaps requests submitted at different times, and an HBM
  budget admits spots one at a time without changing any result.
"""
import time

import numpy as np
import pytest

from pps import workloads as wl

from helpers import oracle, solver, weights

pytestmark = pytest.mark.gpu

ROW_TOL = 5e-5
CHIP_TOL = 1e-9
CHECK = 32


def _spots():
    """Named spots plus draws of the batched distribution: its rivers and
    its turns small enough for a quick test (footprint under 64 MB)."""
    from pps import batch as pb
    out = [wl.river_c1(), wl.river_geo(), wl.turn_api(), wl.turn_short()]
    for sp in wl.batched(32, seed=505):
        if len(sp.board) == 4:
            fp = pb.footprint(sp.board_text(), weights(sp.oop), weights(sp.ip), sp.pot,
                              sp.stack, sp.cfg.bet_text(), sp.cfg.raise_text(),
                              sp.cfg.max_raises)
            if fp > (64 << 20):
                continue
        out.append(sp)
        if len(out) >= 12:
            break
    return out


def _submit(b, sp, frac=0.005):
    """frac: target exploitability as a fraction of the pot (< 0: none)."""
    streets = None
    if sp.street_cfgs:
        streets = [{"bets": c.bet_text(), "raises": c.raise_text() or [],
                    "max_raises": c.max_raises} for c in sp.street_cfgs]
    return b.submit(sp.board_text(), weights(sp.oop), weights(sp.ip), sp.pot, sp.stack,
                    bets=sp.cfg.bet_text(), raises=sp.cfg.raise_text() or [],
                    max_raises=sp.cfg.max_raises, streets=streets,
                    target=frac * sp.pot if frac > 0 else -1.0)


def _normwise(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if b.size == 0:
        return 0.0
    return float(np.max(np.abs(a - b))) / max(float(np.max(np.abs(b))), 1e-30)


def _solve_batch(spots, **kw):
    import pps
    b = pps.Batch(check_every=CHECK, max_iterations=1024, **kw)
    tickets = [_submit(b, sp) for sp in spots]
    assert b.run(timeout=300)
    res = [b.result(t) for t in tickets]
    rows = [b.root_rows(t) for t in tickets]
    info = b.info()
    b.close()
    return res, rows, info


@pytest.fixture(scope="module")
def mixed():
    spots = _spots()
    return spots, _solve_batch(spots)


def test_batch_converges_to_target(mixed):
    spots, (res, _, info) = mixed
    assert info["failed"] == 0 and info["done"] == len(spots)
    assert info["peak_active"] >= 2  # spots shared the device
    for sp, r in zip(spots, res):
        assert r["status"] == 0, r["error"]
        assert r["iterations"] % 16 == 0
        assert r["converged"], (sp.name, r["exploitability"], r["target"])
        assert r["exploitability"] <= 0.005 * sp.pot + 1e-12
        assert abs(sum(r["root_freqs"]) - 1.0) < 1e-6


def test_fixed_check_schedule():
    """fixed_checks: every spot is checked (and retired) at multiples of
    check_every. The adaptive default checks at most check_every apart, so
    it retires a spot within check_every iterations after the fixed
    schedule's passing check (exploitability falls between the two)."""
    spots = _spots()[:6]
    fixed, _, _ = _solve_batch(spots, fixed_checks=True)
    adaptive, _, _ = _solve_batch(spots)
    for sp, f, a in zip(spots, fixed, adaptive):
        assert f["converged"] and f["iterations"] % CHECK == 0, sp.name
        assert a["converged"] and a["iterations"] % 16 == 0, sp.name
        assert a["iterations"] <= f["iterations"] + CHECK, (sp.name, a["iterations"], f["iterations"])


def test_result_same_alone_and_in_the_mix(mixed):
    spots, (res, rows, _) = mixed
    for i in (0, 2, 4, len(spots) - 1):
        (alone,), (arows,), _ = _solve_batch([spots[i]])
        r = res[i]
        assert alone["iterations"] == r["iterations"], spots[i].name
        for k in ("ev_oop", "ev_ip", "exploitability"):
            assert abs(alone[k] - r[k]) <= CHIP_TOL, (spots[i].name, k, alone[k], r[k])
        assert _normwise(arows, rows[i]) <= ROW_TOL


def test_batch_equals_lone_solver(mixed):
    spots, (res, rows, _) = mixed
    for i in (0, 1, 2, 3):
        sp, r = spots[i], res[i]
        s = solver(sp)
        s.solve(r["iterations"])
        st = s.stats()
        # Same rows; the root values are summed in another order (device
        # reduction here, host loop in Solver.stats).
        for k in ("ev_oop", "ev_ip", "exploitability"):
            assert abs(st[k] - r[k]) <= 1e-7, (sp.name, k, st[k], r[k])
        na, n = rows[i].shape
        lone = np.asarray(s.read_rows(1))[:na * n].reshape(na, n)
        assert _normwise(rows[i], lone) <= ROW_TOL


def test_river_ev_within_a_hundredth_of_the_oracle():
    """River spots run in a batch to a fixed 512 iterations (no target):
    EVs within 0.01 chips of the FP64 CPU oracle after the same iterations.
    (Early on, regret matching amplifies f32 rounding wherever regrets sit
    at zero, so the gate is taken where the strategies have settled.)"""
    import pps
    spots = [wl.river_c1(), wl.river_geo()]
    b = pps.Batch(check_every=CHECK, max_iterations=512)
    tickets = [_submit(b, sp, frac=-1.0) for sp in spots]
    assert b.run(timeout=120)
    for sp, t in zip(spots, tickets):
        r = b.result(t)
        assert r["iterations"] == 512 and not r["converged"]
        o = oracle(sp, precision=64)
        o.iterate(512)
        st = o.stats(sp.pot)
        assert abs(st["ev_oop"] - r["ev_oop"]) < 0.01
        assert abs(st["ev_ip"] - r["ev_ip"]) < 0.01
    b.close()


def test_budget_admits_one_at_a_time_without_changing_results():
    """Two ~230 MB turn spots under a budget that holds one of them (plus
    the pools' mapping granularity) never share the device; small river
    spots still join; every result equals the unconstrained batch's."""
    from pps import batch as pb
    sub = [wl.turn_c2(seed=202, uniform_config=True), wl.turn_c2(seed=203, uniform_config=True),
           wl.river_c1(), wl.river_geo()]
    big = max(pb.footprint(sp.board_text(), weights(sp.oop), weights(sp.ip), sp.pot, sp.stack,
                           sp.cfg.bet_text(), sp.cfg.raise_text() or [], sp.cfg.max_raises)
              for sp in sub)
    budget = int(1.3 * big) + (64 << 20)
    free, _, _ = _solve_batch(sub)
    got, _, info = _solve_batch(sub, hbm_budget=budget)
    assert info["peak_active"] <= 3
    assert info["peak_used_bytes"] <= budget
    assert info["failed"] == 0
    for r, want in zip(got, free):
        assert r["iterations"] == want["iterations"]
        for k in ("ev_oop", "ev_ip", "exploitability"):
            assert abs(r[k] - want[k]) <= CHIP_TOL


def test_spot_over_budget_is_refused():
    import pps
    from pps import _abi
    b = pps.Batch(hbm_budget=1 << 20, check_every=CHECK)
    t = _submit(b, wl.turn_api())
    assert b.run(timeout=120)
    r = b.result(t)
    assert r["status"] == _abi.E_BUDGET
    assert "budget" in r["error"]
    b.close()


def test_served_requests_overlap_and_match(mixed):
    import pps
    spots, (res, _, _) = mixed
    b = pps.Batch(check_every=CHECK, max_iterations=1024)
    b.start()
    # Submitted while the serving thread runs, back to back: they are
    # compiled on host threads and admitted as they become ready, so several
    # share the device (a spacing between requests would let fast spots
    # finish alone).
    tickets = [_submit(b, sp) for sp in spots]
    got = [b.wait(t, timeout=300) for t in tickets]
    info = b.info()
    b.stop()
    b.close()
    assert info["peak_active"] >= 2
    for r, want in zip(got, res):
        assert r is not None and r["status"] == 0
        assert r["iterations"] == want["iterations"]
        assert abs(r["ev_oop"] - want["ev_oop"]) <= CHIP_TOL
        assert r["latency_ms"] >= r["finish_ms"] - r["admit_ms"]


def test_empty_range_spot_finishes_with_zero_stats():
    import pps
    b = pps.Batch(check_every=CHECK)
    sp = wl.river_empty()
    t = _submit(b, sp)
    assert b.run(timeout=60)
    r = b.result(t)
    assert r["status"] == 0 and r["iterations"] == 0
    assert r["ev_oop"] == 0.0 and r["exploitability"] == 0.0
    b.close()
