"""GPU parity: the sm_103a kernels (through the C ABI) against the CPU
oracle and the reference's known answers."""
import json
import os

import numpy as np
import pytest

from pps import workloads as wl

from helpers import oracle, seeded_rows, solver, root_strategy

pytestmark = pytest.mark.gpu

@pytest.mark.parametrize("tag,mode", [("TINY", None), ("M7", 7), ("M9", 9)])
def test_tiny_check_known_answers(golden_dir, tag, mode):
    """tools/tiny_check.cpp ground truth (1e-4, tools/quality/
    gpu_postflop_parity.sh:126-148) through the GPU value walk."""
    want = json.load(open(os.path.join(golden_dir, "tiny_check.json")))[tag]
    ref = np.load(os.path.join(golden_dir, "ref_turn_tiny.npz"))
    s = solver(wl.turn_tiny())
    s.solve(0)
    if mode:
        s.write_rows(1, seeded_rows(ref["decideMeta"], int(ref["regTotal"][0]), mode))
    v0, _ = s.walk(0, 0)
    v1, _ = s.walk(1, 0)
    assert abs(v0 - want["ev0"]) < 1e-4
    assert abs(v1 - want["ev1"]) < 1e-4


def test_seed_env_hook_matches(golden_dir, monkeypatch):
    """The reference's GPU_CFR_SEED_STRAT hook in stats() (cuda/gpu_cfr.cu:
    2066-2097) reproduces the M7 known answer."""
    want = json.load(open(os.path.join(golden_dir, "tiny_check.json")))["M7"]
    monkeypatch.setenv("GPU_CFR_SEED_STRAT", "7")
    s = solver(wl.turn_tiny())
    s.solve(0)
    assert abs(s.stats()["ev_oop"] - want["ev0"]) < 1e-4


ROW_CASES = [("river_c1", 1), ("river_c1", 2), ("river_c1", 10), ("turn_short", 1),
             ("turn_short", 2), ("turn_short", 10), ("river_geo", 1), ("river_geo", 2),
             ("river_geo", 10), ("turn_api", 1), ("flop_short", 1), ("flop_short", 2),
             ("turn_c3", 1)]


@pytest.mark.parametrize("name,iters", ROW_CASES)
def test_rows_match_oracle(name, iters):
    """Regret and strategy rows after 1, 2 and 10 iterations against the
    FP64 oracle. Tolerance: the error normwise (max |gpu - f64| / max |f64|)
    stays within 5e-5 and within twice the error of a plain f32
    restatement of the reference's arithmetic (the f32 oracle). Cases are
    the well-conditioned ones: where regret matching meets regrets that are
    exactly zero in exact arithmetic (turn_api after 2+ iterations), f32
    and f64 pick different strategies and rows are compared through the
    solution gates below instead."""
    spot = wl.NAMED[name]()
    s = solver(spot)
    s.solve(iters)
    o64 = oracle(spot, precision=64)
    o64.iterate(iters)
    o32 = oracle(spot, precision=32)
    o32.iterate(iters)
    for which in (0, 1):
        g, r, r32 = s.read_rows(which), o64.rows(which), o32.rows(which)
        assert g.shape == r.shape and np.all(np.isfinite(g))
        scale = max(float(np.max(np.abs(r))), 1e-30)
        err_gpu = float(np.max(np.abs(g.astype(np.float64) - r))) / scale
        err_f32 = float(np.max(np.abs(r32.astype(np.float64) - r))) / scale
        assert err_gpu <= 5e-5, (name, which, err_gpu, err_f32)
        assert err_gpu <= max(2.0 * err_f32, 1e-6), (name, which, err_gpu, err_f32)


@pytest.mark.parametrize("name,iters", [("turn_c3", 2), ("turn_c3", 10)])
def test_rows_no_worse_than_f32_where_ill_conditioned(name, iters):
    """The 48,255-node benchmark turn after 2 and 10 iterations. From the
    second iteration on, regret matching meets regrets that are exactly
    zero in exact arithmetic (combos whose actions all have equal values),
    and f32 rounding decides their strategy: even the plain f32 restatement
    of the reference's arithmetic (the f32 oracle) is 0.21 normwise away
    from FP64 after 2 iterations. The gate is therefore relative: the GPU's
    regret and strategy rows are no further from the FP64 oracle than the
    f32 restatement's (within 2x), and the same holds for the root EV of
    the average strategy (FP64 walks on both sides; within 2x plus 0.01
    chips)."""
    spot = wl.NAMED[name]()
    s = solver(spot)
    s.solve(iters)
    st = s.stats()
    o64 = oracle(spot, precision=64)
    o64.iterate(iters)
    o32 = oracle(spot, precision=32)
    o32.iterate(iters)
    for which in (0, 1):
        g, r, r32 = s.read_rows(which), o64.rows(which), o32.rows(which)
        assert g.shape == r.shape and np.all(np.isfinite(g))
        scale = max(float(np.max(np.abs(r))), 1e-30)
        err_gpu = float(np.max(np.abs(g.astype(np.float64) - r))) / scale
        err_f32 = float(np.max(np.abs(r32.astype(np.float64) - r))) / scale
        assert err_gpu <= max(2.0 * err_f32, 5e-5), (name, iters, which, err_gpu, err_f32)
    e64, e32 = o64.stats(spot.pot), o32.stats(spot.pot)
    d_gpu = abs(st["ev_oop"] - e64["ev_oop"])
    d_f32 = abs(e32["ev_oop"] - e64["ev_oop"])
    assert d_gpu <= 2.0 * d_f32 + 0.01, (d_gpu, d_f32)


@pytest.mark.parametrize("name,iters", [("river_c1", 1000), ("turn_api", 300),
                                        ("turn_c2_uniform", 100), ("turn_c2", 500)])
def test_solution_matches_oracle(name, iters):
    """Solution gates: root EV within 0.01 chips, root strategy
    within 0.10 L-inf, exploitability ratio in [0.5, 2], against the FP64
    oracle run of the same iterations. turn_c2 is the 6,333-node turn with
    per-street sizes (turn {33, 75}%, river {50, 100}%, 2.5x raises, max 3)
    at its full 500 iterations."""
    spot = wl.NAMED[name]()
    s = solver(spot)
    s.solve(iters)
    st = s.stats()
    o = oracle(spot, precision=64)
    o.iterate(iters)
    ost = o.stats(spot.pot)
    assert abs(st["ev_oop"] - ost["ev_oop"]) < 0.01
    assert abs(st["ev_ip"] - ost["ev_ip"]) < 0.01
    ratio = st["exploitability"] / max(ost["exploitability"], 1e-9)
    assert 0.5 <= ratio <= 2.0, (st, ost)
    na = s.decide_nodes()[0]["actions"]
    g = s.root_strategy()
    n0 = s.num_base_combos(0)
    w0 = s.player_weights(0)
    r = root_strategy(o.rows(1), len(na), n0, w0)
    assert np.max(np.abs(g - r)) <= 0.10


@pytest.mark.parametrize("name", ["river_c1", "turn_api", "turn_c2_uniform", "turn_c3"])
def test_fp64_walks_equal_oracle_on_the_same_rows(name):
    """The stats walks (FP64 on the device: EV against the average
    strategy, best responses) evaluate a given strategy exactly: the
    product's rows after 30 iterations, written into the FP64 oracle, give
    the same EVs and exploitability there to 1e-9 (observed: 1e-14). This
    pins the scorer that the solution gates and the batch checks use."""
    spot = wl.NAMED[name]()
    s = solver(spot)
    s.solve(30)
    mine = s.stats()
    o = oracle(spot, precision=64)
    o.set_rows(0, np.asarray(s.read_rows(0), dtype=np.float32))
    o.set_rows(1, np.asarray(s.read_rows(1), dtype=np.float32))
    ref = o.stats(spot.pot)
    for k in ("ev_oop", "ev_ip", "exploitability"):
        assert abs(mine[k] - ref[k]) <= 1e-9 * max(1.0, abs(ref[k])), (k, mine[k], ref[k])


def test_deterministic_rows():
    spot = wl.turn_api()
    a, b = solver(spot), solver(spot)
    a.solve(50)
    b.solve(50)
    for which in (0, 1):
        assert np.array_equal(a.read_rows(which), b.read_rows(which))
    a.reset()
    a.solve(50)
    assert np.array_equal(a.read_rows(1), b.read_rows(1))


@pytest.mark.parametrize("name", ["river_c1", "turn_api", "turn_short", "flop_short", "river_geo"])
def test_terminal_groups_match_per_node_kernels(name):
    """Engine 0 (showdown / fold nodes in groups of four, float4 lanes,
    128-position prefix blocks) and engine 1 (one CTA per terminal node,
    32-position blocks) evaluate the same formulas: after 1 iteration the
    rows agree to f32 rounding (normwise 1e-5); after 300 the solutions pass
    the oracle gates against each other (EV within 0.01 chips,
    exploitability ratio in [0.5, 2], or within 0.01 chips where it is ~0).
    In between, regret matching
    amplifies rounding wherever regrets sit at zero (see the row cases
    above), so rows are not compared there."""
    spot = wl.NAMED[name]()
    for iters in (1, 300):
        a, b = solver(spot), solver(spot)
        a.set_engine(0)
        b.set_engine(1)
        a.solve(iters)
        b.solve(iters)
        assert a.info().engine == 0 and b.info().engine == 1
        if iters == 1:
            for which in (0, 1):
                ra = np.asarray(a.read_rows(which), dtype=np.float64)
                rb = np.asarray(b.read_rows(which), dtype=np.float64)
                assert np.max(np.abs(ra - rb)) <= 1e-5 * max(np.max(np.abs(rb)), 1e-30)
            continue
        sa, sb = a.stats(), b.stats()
        assert abs(sa["ev_oop"] - sb["ev_oop"]) < 0.01
        assert abs(sa["ev_ip"] - sb["ev_ip"]) < 0.01
        ea, eb = sa["exploitability"], sb["exploitability"]
        assert abs(ea - eb) < 0.01 or 0.5 <= ea / max(eb, 1e-9) <= 2.0, (ea, eb)


def test_full_size_turn_c3_properties():
    """The 48,255-node turn tree (turn_c3): FP64 EVs sum to the pot, exploitability
    falls with iterations, rows stay finite and the strategy normalizes."""
    spot = wl.turn_c3()
    s = solver(spot)
    assert s.num_nodes == 48255
    s.solve(64)
    e64 = s.stats()
    s.solve(256)
    e256 = s.stats()
    for st in (e64, e256):
        assert abs(st["ev_oop"] + st["ev_ip"] - spot.pot) < 1e-3
    assert e256["exploitability"] < e64["exploitability"]
    rows = s.read_rows(1)
    assert np.all(np.isfinite(rows)) and np.all(rows >= 0)
    f = s.strategy(3)["freqs"]
    np.testing.assert_allclose(f.sum(axis=0), 1.0, atol=1e-9)


def test_flop_164k_rows_match_oracle():
    """The reference's 164,416-node flop bench spot (two chance streets):
    rows after one iteration against the FP64 oracle (normwise 5e-5)."""
    spot = wl.flop_164k()
    s = solver(spot)
    assert s.num_nodes == 164416
    s.solve(1)
    o64 = oracle(spot, precision=64)
    o64.iterate(1)
    for which in (0, 1):
        g, r = s.read_rows(which), o64.rows(which)
        scale = max(float(np.max(np.abs(r))), 1e-30)
        assert float(np.max(np.abs(g.astype(np.float64) - r))) / scale <= 5e-5


@pytest.mark.parametrize("name", ["turn_api", "turn_short", "flop_short", "turn_w52"])
def test_fused_plan_matches_staged_plan(name):
    """Engine 2 (one fused launch per backward level) runs the same record
    and group arithmetic as engine 0 in another launch order: the rows are
    bitwise identical after 1 and 50 iterations. The default (autotuned)
    solver picks one of the two and matches as well."""
    spot = wl.NAMED[name]()
    for iters in (1, 50):
        a, b, c = solver(spot), solver(spot), solver(spot)
        a.set_engine(0)
        b.set_engine(2)
        a.solve(iters)
        b.solve(iters)
        c.solve(iters)
        assert a.info().engine == 0 and b.info().engine == 2
        assert c.info().engine in (0, 2)
        for which in (0, 1):
            ra = a.read_rows(which)
            assert np.array_equal(ra, b.read_rows(which)), (name, iters, which)
            assert np.array_equal(ra, c.read_rows(which)), (name, iters, which)


def test_fused_plan_refused_for_wide_lists():
    s = solver(wl.turn_c2(uniform_config=True))
    with pytest.raises(RuntimeError, match="engine 2"):
        s.set_engine(2)


def _strategy_total(iters):
    """The exact per-combo total of the cumulative strategy after `iters`
    iterations of the "dcfr" schedule: every iteration adds a strategy that
    sums to 1 over the actions (strat = strat * avg + sigma, cuda/gpu_cfr.cu:
    512-523), so the total follows S = S * avg + 1, with avg the f32
    coefficient the device table holds, evaluated here in FP64."""
    s = 0.0
    for t in range(iters):
        k = 0
        if t > 0:
            k = 1
            while k * 4 <= t:
                k *= 4
        tg = float(t - k)
        avg = float(np.float32((tg / (tg + 1.0)) ** 3))
        s = s * avg + 1.0
    return s


def _total_deviation(rows, meta, total):
    """max over decide-node combos of |sum over actions - total| / total."""
    worst = 0.0
    for m in meta.reshape(-1, 8):
        reg, na, nc = int(m[0]), int(m[1]), int(m[3])
        r = np.asarray(rows[reg:reg + na * nc], dtype=np.float64).reshape(na, nc)
        worst = max(worst, float(np.max(np.abs(r.sum(axis=0) - total))) / total)
    return worst


@pytest.mark.parametrize("name,iters", [("river_c1", 1000), ("turn_api", 700),
                                        ("turn_c3", 1000)])
def test_compensated_strategy_sums(name, iters):
    """Compensated (two-float) cumulative-strategy sums against the plain
    f32 sums on the same solve. The regrets do not depend on the strategy
    sums, so they are bitwise equal. Every iteration adds a strategy that
    sums to 1, so each combo's strategy sums must total the schedule's
    weighted count (FP64 recurrence): the compensated rows meet it to f32
    rounding of the final sums (relative 1e-6) and at least as closely as
    the plain ones, whose error grows with the iterations accumulated since
    the last reset. On the spots the FP64 oracle runs in seconds, the
    strategy rows are also at least as close to its rows (within 1%)."""
    from pps import pps_native as pn
    from helpers import abi_cfgs
    spot = wl.NAMED[name]()
    plain, comp = solver(spot), solver(spot)
    plain.set_engine(0)
    comp.set_engine(0)
    comp.set_compensated(True)
    assert comp.info().compensated == 1 and plain.info().compensated == 0
    plain.solve(iters)
    comp.solve(iters)
    assert np.array_equal(plain.read_rows(0), comp.read_rows(0))
    meta = pn.compile_export(spot.board, spot.oop, spot.ip, spot.pot, spot.stack,
                             abi_cfgs(spot))["decideMeta"]
    total = _strategy_total(iters)
    dev_plain = _total_deviation(plain.read_rows(1), meta, total)
    dev_comp = _total_deviation(comp.read_rows(1), meta, total)
    assert dev_comp <= 1e-6, (dev_comp, dev_plain)
    assert dev_comp <= dev_plain, (dev_comp, dev_plain)
    if name != "turn_c3":
        o = oracle(spot, precision=64)
        o.iterate(iters)
        exact = o.rows(1)
        scale = float(np.max(np.abs(exact)))
        e_plain = float(np.max(np.abs(plain.read_rows(1) - exact))) / scale
        e_comp = float(np.max(np.abs(comp.read_rows(1) - exact))) / scale
        assert e_comp <= 1.01 * e_plain + 1e-7, (e_comp, e_plain)
    # Turning the option off keeps the sums (rounded high words).
    comp.set_compensated(False)
    comp.continue_solve(16)
    assert comp.info().compensated == 0
