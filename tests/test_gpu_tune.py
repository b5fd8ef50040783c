"""Launch shapes and the autotuner (pps_gb_set_launch_shape, Engine::
autotune): the iteration graph's plan and the grids of its level and group
launches. A shape changes timing only: persistent grids stride over the same
(spot, node-range) tasks that one-CTA-per-task grids run, with the same
arithmetic, so the rows must come out bitwise identical under every shape.
The smallest caps (1 x SM count) make every CTA run many tasks in turn."""
import os
import subprocess
import sys

import numpy as np
import pytest

from pps import workloads as wl

from helpers import solver

pytestmark = pytest.mark.gpu

SHAPES = [dict(plan=0, fwd_cap=1, bwd_cap=1, sd_cap=1, fd_cap=1),
          dict(plan=0, fwd_cap=16, bwd_cap=16, sd_cap=2, fd_cap=3),
          dict(plan=0, fwd_cap=0, bwd_cap=0, sd_cap=1, fd_cap=0)]
FUSED = [dict(plan=2, fwd_cap=1, bwd_cap=1, sd_cap=0, fd_cap=0),
         dict(plan=2, fwd_cap=16, bwd_cap=16, sd_cap=0, fd_cap=0)]


@pytest.mark.parametrize("name", ["river_c1", "turn_api", "flop_short", "turn_c2_uniform",
                                  "turn_w52"])
def test_launch_shapes_give_identical_rows(name):
    spot = wl.NAMED[name]()
    base = solver(spot)
    base.set_launch_shape(plan=0, fwd_cap=0, bwd_cap=0, sd_cap=0, fd_cap=0)
    base.solve(40)
    want = [base.read_rows(k) for k in (0, 1)]
    shapes = SHAPES + (FUSED if name in ("turn_api", "flop_short", "turn_w52") else [])
    for shape in shapes:
        s = solver(spot)
        s.set_launch_shape(**shape)
        assert s.launch_shape() == shape
        s.solve(40)
        for k in (0, 1):
            assert np.array_equal(s.read_rows(k), want[k]), (name, shape, k)


def test_autotuner_caches_its_choice(tmp_path):
    """The first solve of 32+ iterations tunes the shape (and gives the same
    rows as an untuned solve); the choice is written to the cache file, and
    a new process takes it from there."""
    cache = str(tmp_path / "shapes")
    code = r'''
import json, os, sys
sys.path[:0] = [sys.argv[1], os.path.join(sys.argv[1], "cuda-poker-solver_gb300"),
                os.path.join(sys.argv[1], "tests")]
from pps import workloads as wl
from helpers import solver
s = solver(wl.turn_api())
s.solve(64)
print(json.dumps(s.launch_shape()))
'''
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, PPS_GB_TUNE_FILE=cache)
    shapes = []
    for _ in range(2):
        r = subprocess.run([sys.executable, "-c", code, repo], env=env, capture_output=True,
                           text=True, timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]
        shapes.append(r.stdout.strip().splitlines()[-1])
    assert shapes[0] == shapes[1]
    lines = open(cache).read().split("\n")
    assert any(line.strip() for line in lines)
    fields = [line.split() for line in lines if line.strip()]
    assert all(len(f) == 8 for f in fields)

    tuned, plain = solver(wl.turn_api()), solver(wl.turn_api())
    plain.set_launch_shape(plan=0, fwd_cap=0, bwd_cap=0, sd_cap=0, fd_cap=0)
    tuned.solve(64)
    plain.solve(64)
    for k in (0, 1):
        assert np.array_equal(tuned.read_rows(k), plain.read_rows(k))
