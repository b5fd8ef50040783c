"""The "PPS1" version-1 solution file against the reference's own writer and
loader (cuda/gpu_cfr.cu:2686-2853).

tests/golden/ref_solution_v1.pps was written by the reference's save() for
a small river spot (tests/golden/make_golden.py --solution-file, through
oracle/_ref/ref_capture: the reference engine compiled on a host CUDA stub),
with the rows set to a fixed pattern that `pattern()` reproduces. CPU tests
read the file's fields in the reference's order and, where the reference's
tools are built, run the reference's load constructor on it. The GPU test
loads it with this library, checks every row and the iteration count, and
saves it again: the bytes must equal the reference's, so files written here
load in the reference and the other way round.
"""
import json
import os
import struct
import subprocess
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "ref_solution_v1.pps")
META = json.load(open(os.path.join(HERE, "golden", "ref_solution_v1.json")))
REF_CAPTURE = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "ref_capture")


def pattern(which, n):
    """The rows ref_capture --save wrote (uint32 index arithmetic)."""
    i = np.arange(n, dtype=np.uint64)
    if which == 0:
        k = ((i * 2654435761) & 0xFFFFFFFF) % 20001
        return (k.astype(np.int64) - 10000).astype(np.float32) / np.float32(64.0)
    k = ((i * 40503) & 0xFFFFFFFF) % 1000
    return k.astype(np.float32) / np.float32(8.0)


def parse_v1(raw):
    """Field order of the reference's save() (cuda/gpu_cfr.cu:2743-2785)."""
    o = 0

    def take(fmt):
        nonlocal o
        v = struct.unpack_from("<" + fmt, raw, o)
        o += struct.calcsize("<" + fmt)
        return v if len(v) > 1 else v[0]

    def doubles():
        n = take("i")
        return list(take("%dd" % n)) if n > 1 else ([take("d")] if n == 1 else [])

    f = {"magic": take("I"), "version": take("I"), "n_board": take("i")}
    f["board"] = list(take("5B"))
    f["pot"], f["stack"] = take("q"), take("q")
    f["oop"] = np.frombuffer(raw, np.float64, 1326, o); o += 1326 * 8
    f["ip"] = np.frombuffer(raw, np.float64, 1326, o); o += 1326 * 8
    f["bets"], f["raises"] = doubles(), doubles()
    f["allin"], f["geometric"] = take("b"), take("b")
    f["max_raises"] = take("i")
    f["thresholds"] = [take("d"), take("d"), take("d")]
    f["num_nodes"], f["iterations"] = take("q"), take("q")
    n = take("i")
    f["algo"] = raw[o:o + n].decode(); o += n
    f["reg_total"] = take("q")
    f["regret"] = np.frombuffer(raw, np.float32, f["reg_total"], o); o += 4 * f["reg_total"]
    f["strat"] = np.frombuffer(raw, np.float32, f["reg_total"], o); o += 4 * f["reg_total"]
    f["end"] = o
    return f


def test_reference_file_fields():
    raw = open(GOLDEN, "rb").read()
    f = parse_v1(raw)
    assert f["magic"] == 0x31535050 and f["version"] == 1
    assert f["end"] == len(raw)
    assert f["n_board"] == 5 and f["pot"] == META["pot"] and f["stack"] == META["stack"]
    assert f["bets"] == [0.75] and f["raises"] == [2.5, 3.0] and f["allin"] == 1
    assert f["num_nodes"] == META["num_nodes"] and f["reg_total"] == META["reg_total"]
    assert f["iterations"] == META["iterations"] and f["algo"] == "dcfr"
    assert np.array_equal(f["regret"], pattern(0, f["reg_total"]))
    assert np.array_equal(f["strat"], pattern(1, f["reg_total"]))


@pytest.mark.skipif(not os.path.exists(REF_CAPTURE),
                    reason="reference tools not built (oracle/ref/build_ref.sh)")
def test_reference_loader_reads_the_golden():
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_golden import read_dump
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "load.bin")
        subprocess.run([REF_CAPTURE, "--load", GOLDEN, out], check=True, capture_output=True)
        d = read_dump(out)
    n = int(d["regTotal"][0])
    assert n == META["reg_total"] and int(d["totalIterations"][0]) == META["iterations"]
    assert int(d["counter"][0]) == META["iterations"]
    assert np.array_equal(d["regret"], pattern(0, n))
    assert np.array_equal(d["strat"], pattern(1, n))


@pytest.mark.gpu
def test_load_reference_file_and_save_identical(tmp_path):
    """pps.Solver.load reads the reference-written file (same rows, same
    iteration count); saving it again gives the reference's bytes exactly;
    the loaded solve continues."""
    import pps
    s = pps.Solver.load(GOLDEN)
    n = META["reg_total"]
    assert s.num_nodes == META["num_nodes"]
    assert s.total_iterations == META["iterations"]
    assert np.array_equal(s.read_rows(0), pattern(0, n))
    assert np.array_equal(s.read_rows(1), pattern(1, n))
    out = str(tmp_path / "again.pps")
    s.save(out)
    assert open(out, "rb").read() == open(GOLDEN, "rb").read()
    s.continue_solve(20)
    assert s.total_iterations == META["iterations"] + 20
    st = s.stats()
    assert np.isfinite(st["ev_oop"]) and np.isfinite(st["exploitability"])
