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
             ("river_geo", 10), ("turn_api", 1), ("flop_short", 1), ("flop_short", 2)]


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


@pytest.mark.parametrize("name", ["river_c1", "turn_api", "turn_c2_uniform"])
def test_solution_matches_oracle(name):
    """Solution gates: root EV within 0.01 chips, root strategy
    within 0.10 L-inf, exploitability ratio in [0.5, 2], against the FP64
    oracle run of the same iterations."""
    spot = wl.NAMED[name]()
    iters = {"river_c1": 1000, "turn_api": 300, "turn_c2_uniform": 100}[name]
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
