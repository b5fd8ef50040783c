"""GPU parity against the REFERENCE's own kernels: cuda/gpu_cfr.cu compiled
from its source for sm_103a (oracle/_ref/gpu_cfr_kernels.fatbin) and run on
the same GPU, on the reference layout, graph and launch sequence
(oracle/ref/ref_gpu.cpp). The product solver, through the C ABI, must give
the reference's rows and solutions on the same inputs."""
import numpy as np
import pytest

from pps import workloads as wl
from oracle import cpu_oracle as co
from oracle import ref_gpu

from helpers import oracle, solver, weights

pytestmark = [
    pytest.mark.gpu,
    pytest.mark.skipif(not ref_gpu.fatbin_present(),
                       reason="reference kernels not built (oracle/ref/build_ref.sh needs "
                              "the reference sources)"),
]


def reference(spot):
    """The reference's kernels on the reference's layout of the spot, as the
    oracle restates it (bit-exact against the reference's init(), pinned in
    tests/test_oracle_golden.py): no product code builds their input."""
    exp = co.reference_layout(spot.board, weights(spot.oop), weights(spot.ip), spot.pot,
                              spot.stack, co.cfg_from(spot.cfg))
    return ref_gpu.RefKernels(exp, spot.pot)


def normwise(a, b):
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(np.asarray(a, dtype=np.float64) - b))) / \
        max(float(np.max(np.abs(b))), 1e-30)


ROW_CASES = [("river_c1", 1), ("river_c1", 2), ("river_c1", 10), ("turn_short", 1),
             ("turn_short", 2), ("turn_api", 1), ("river_geo", 1), ("river_geo", 2),
             ("flop_short", 1), ("flop_short", 2), ("turn_c2_uniform", 1), ("turn_c3", 1),
             ("turn_w52", 1)]


@pytest.mark.parametrize("name,iters", ROW_CASES)
def test_rows_match_reference_kernels(name, iters):
    """Regret and strategy rows after 1, 2 and 10 iterations: normwise
    (max |product - reference| / max |reference|) within 5e-5. The two
    differ only in f32 summation order (the reference's showdown scan is
    plain f32 and its fold sums use shared-memory atomics, so its own runs
    drift by rounding). Cases are the well-conditioned ones: where regret
    matching meets regrets that are exactly zero in exact arithmetic
    (turn_w52 after 2 iterations: there even the f32 and f64 oracles differ
    by 0.04 normwise), rounding picks the strategy, and the solutions are
    compared instead (below)."""
    spot = wl.NAMED[name]()
    r = reference(spot)
    r.solve(iters)
    s = solver(spot)
    s.solve(iters)
    for which in (0, 1):
        g, ref = s.read_rows(which), r.rows(which)
        assert g.shape == ref.shape
        assert np.all(np.isfinite(ref))
        assert normwise(g, ref) <= 5e-5, (name, iters, which, normwise(g, ref))
    r.close()


@pytest.mark.parametrize("name,iters", [("river_c1", 2), ("river_c1", 10),
                                        ("turn_short", 2), ("river_geo", 2)])
def test_at_least_as_accurate_as_reference_kernels(name, iters):
    """Against the FP64 oracle, the product's rows are no further off than
    the reference kernels' own (within 2x, or 1e-6 normwise)."""
    spot = wl.NAMED[name]()
    r = reference(spot)
    r.solve(iters)
    s = solver(spot)
    s.solve(iters)
    o = oracle(spot, precision=64)
    o.iterate(iters)
    for which in (0, 1):
        exact = o.rows(which)
        e_ref = normwise(r.rows(which), exact)
        e_gb = normwise(s.read_rows(which), exact)
        assert e_gb <= max(2.0 * e_ref, 1e-6), (name, which, e_gb, e_ref)
    r.close()


@pytest.mark.parametrize("name,iters", [("river_c1", 1000), ("turn_api", 300),
                                        ("turn_c2_uniform", 100), ("turn_c2_uniform", 500),
                                        ("turn_w52", 1000), ("turn_c3", 1000)])
def test_solution_matches_reference_kernels(name, iters):
    """After a full solve the product's strategy passes the solution gates
    against the reference kernels': EVs within 0.01 chips, root strategy
    within 0.10 L-inf (range-weighted frequencies of the root actions),
    exploitability no worse than twice the reference's (or within 0.01
    chips where it is ~0, or both within 0.5% of the pot - the batch and
    serve target - where f32 rounding sets it). The reference's average
    strategy is scored by the product's FP64 walks after writing its rows
    in (those walks equal the oracle's FP64 evaluation of the same rows to
    1e-12: test_gpu_parity).

    The reference's kernels are not deterministic (their fold sums use
    shared-memory atomics), and on turn_c3 their runs are erratic: four
    runs in one process gave exploitabilities of 0.062, 0.139, 0.747 and
    0.041 chips (pot 100) and root EVs of 47.414, 47.412, 47.373 and
    47.415, against the product's 0.093 and 47.413 on every run. So the
    reference is solved three times and the gates compare with its best
    run (lowest exploitability). Where a run is far from equilibrium the
    EVs cannot agree to 0.01 chips: a profile with exploitability e holds
    each player's EV within 2e of the game value, so the EV gate is 0.01
    chips or e_a + e_b (half of 2(e_a + e_b)), whichever is larger.
    turn_c3 is the benchmark's own workload (48,255 nodes, 1,000
    iterations), turn_c2_uniform the 6,333-node turn at 500."""
    spot = wl.NAMED[name]()
    runs = []
    for _ in range(3):
        r = reference(spot)
        r.solve(iters)
        scored = solver(spot)
        scored.solve(0)
        scored.write_rows(1, r.rows(1))
        runs.append((scored.stats(), np.asarray(scored.root_strategy())))
        r.close()
    theirs, ref = min(runs, key=lambda x: x[0]["exploitability"])
    s = solver(spot)
    s.solve(iters)
    mine = s.stats()
    a, b = mine["exploitability"], theirs["exploitability"]
    for side in ("ev_oop", "ev_ip"):
        assert abs(mine[side] - theirs[side]) < max(0.01, a + b), (side, mine, runs)
    # Where both solutions are within 0.5% of the pot of exact equilibrium,
    # their exploitability is set by f32 rounding, and the ratio is noise.
    converged = max(a, b) <= 0.005 * spot.pot
    assert abs(a - b) < 0.01 or converged or a <= 2.0 * b, (a, b, runs)
    g = np.asarray(s.root_strategy())
    assert g.shape == ref.shape
    assert float(np.max(np.abs(g - ref))) <= 0.10, (g, ref)
