"""The no-allocation entry point (pps_gb_solve_noalloc) against the regular
one (pps_gb_create + pps_gb_solve / pps_gb_continue), through the C ABI.

pps_gb_solve_noalloc serves callers that cannot call cudaMalloc (their
device memory belongs to another allocator, or they must avoid cudaMalloc's
implicit synchronization): they own the regret and strategy rows, and every
other buffer lives in the library's static device array. Here the caller's
rows are torch tensors on the current device. Two calls in a row must
continue the solve exactly as a regular solve followed by continue_solve
does, within the row tolerance of the parity tests (normwise 5e-5; the two
paths run the same kernels, so the rows come out identical in practice).

This file sorts last so that a run stopping at the first failure has run
every other test first.
"""
import ctypes as C

import numpy as np
import pytest

from pps import _abi
from pps import pps_native as pn
from pps import workloads as wl

from helpers import abi_cfgs, solver, weights

pytestmark = pytest.mark.gpu

TOL = 5e-5


def _abi_spot(spot):
    return pn.make_spot(spot.board, weights(spot.oop), weights(spot.ip), spot.pot, spot.stack)


def _noalloc(spot, regret, strat, first, iters, torch):
    n_rows = C.c_int64()
    stream = torch.cuda.current_stream().cuda_stream
    rc = _abi.lib.pps_gb_solve_noalloc(
        C.byref(_abi_spot(spot)), C.byref(abi_cfgs(spot)[0]), C.c_void_p(regret.data_ptr()),
        C.c_void_p(strat.data_ptr()), regret.numel(), first, iters, C.c_void_p(stream),
        C.byref(n_rows))
    return rc, n_rows.value


def _normwise(a, b):
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(np.asarray(a, dtype=np.float64) - b))) / max(
        float(np.max(np.abs(b))), 1e-30)


@pytest.mark.parametrize("name,iters", [("river_c1", 40), ("turn_api", 20)])
def test_noalloc_matches_regular_solve_over_two_calls(name, iters):
    torch = pytest.importorskip("torch")
    spot = wl.NAMED[name]()
    ref = solver(spot)
    n = ref.info().row_total
    regret = torch.zeros(n, dtype=torch.float32, device="cuda")
    strat = torch.zeros(n, dtype=torch.float32, device="cuda")

    ref.solve(iters)
    rc, rows = _noalloc(spot, regret, strat, 0, iters, torch)
    assert rc == 0, _abi.lib.pps_gb_last_error().decode()
    assert rows == n
    assert _normwise(regret.cpu().numpy(), ref.read_rows(0)) <= TOL
    assert _normwise(strat.cpu().numpy(), ref.read_rows(1)) <= TOL

    ref.continue_solve(iters)
    rc, _ = _noalloc(spot, regret, strat, iters, iters, torch)
    assert rc == 0, _abi.lib.pps_gb_last_error().decode()
    assert _normwise(regret.cpu().numpy(), ref.read_rows(0)) <= TOL
    assert _normwise(strat.cpu().numpy(), ref.read_rows(1)) <= TOL


def test_noalloc_rejects_spots_beyond_the_scratch():
    torch = pytest.importorskip("torch")
    spot = wl.turn_c3()  # ~1 GB of rows: far beyond the 64 MiB static scratch
    ref_rows = pn.compile_export(spot.board, spot.oop, spot.ip, spot.pot, spot.stack,
                                 abi_cfgs(spot))["regTotal"][0]
    regret = torch.zeros(int(ref_rows), dtype=torch.float32, device="cuda")
    strat = torch.zeros(int(ref_rows), dtype=torch.float32, device="cuda")
    rc, _ = _noalloc(spot, regret, strat, 0, 1, torch)
    assert rc == _abi.E_BUDGET
    msg = _abi.lib.pps_gb_last_error().decode()
    assert "scratch" in msg and str(64 << 20) in msg


@pytest.mark.parametrize("name", ["river_c1", "turn_api"])
def test_noalloc_spot_without_decide_nodes(name):
    """A zero behind-stack makes the root a showdown (river) or chance node
    (turn): the spot has no decide nodes and no rows. The call succeeds with
    NULL row buffers and reports 0 rows, as the regular solver does."""
    pytest.importorskip("torch")
    import dataclasses
    spot = dataclasses.replace(wl.NAMED[name](), stack=0)
    ref = solver(spot)
    ref.solve(3)
    assert ref.info().row_total == 0
    n_rows = C.c_int64(-1)
    rc = _abi.lib.pps_gb_solve_noalloc(
        C.byref(_abi_spot(spot)), C.byref(abi_cfgs(spot)[0]), None, None, 0, 0, 3, None,
        C.byref(n_rows))
    assert rc == 0, _abi.lib.pps_gb_last_error().decode()
    assert n_rows.value == 0


def test_noalloc_size_query_and_late_window():
    """row_capacity 0 is a size query: the call fails with PPS_GB_E_ARG and
    still reports the rows the spot needs. A continuation far into a solve
    (absolute iteration 6,000,000) holds only its own schedule window in the
    scratch, so it runs; its coefficients are those of the late iterations
    (positive regrets kept almost whole, the average weighted ~1)."""
    torch = pytest.importorskip("torch")
    spot = wl.river_c1()
    n_rows = C.c_int64(-1)
    rc = _abi.lib.pps_gb_solve_noalloc(
        C.byref(_abi_spot(spot)), C.byref(abi_cfgs(spot)[0]), None, None, 0, 0, 1, None,
        C.byref(n_rows))
    assert rc == _abi.E_ARG
    n = solver(spot).info().row_total
    assert n_rows.value == n

    regret = torch.zeros(n, dtype=torch.float32, device="cuda")
    strat = torch.zeros(n, dtype=torch.float32, device="cuda")
    rc, rows = _noalloc(spot, regret, strat, 0, 20, torch)
    assert rc == 0 and rows == n
    before = strat.clone()
    rc, _ = _noalloc(spot, regret, strat, 6_000_000, 2, torch)
    assert rc == 0, _abi.lib.pps_gb_last_error().decode()
    s = strat.cpu().numpy()
    assert np.all(np.isfinite(s)) and np.all(s >= 0)
    # Average weight ((t-k)/(t-k+1))^3 ~ 1 this late: the strategy sums grow
    # by about one strategy (1 per combo summed over actions) per iteration.
    grow = float(s.sum() - before.cpu().numpy().sum())
    assert grow > 0
