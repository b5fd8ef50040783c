"""Host-side product logic against the reference's golden vectors (CPU
only): evaluator, bet abstraction, range parser, C-ABI exports, file
errors that fail before any device use."""
import ctypes
import json
import os
import re
import struct

import numpy as np
import pytest

from pps import _abi
from pps import pps_native as pn

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def test_library_exports_every_declared_symbol():
    header = open(os.path.join(REPO, "include", "pps_gb.h")).read()
    declared = set(re.findall(r"\b(pps_gb_\w+)\s*\(", header))
    lib = ctypes.CDLL(_abi.LIB_PATH)
    missing = [s for s in sorted(declared) if not hasattr(lib, s)]
    assert not missing, missing
    assert set(_abi.SYMBOLS) <= declared


def test_hand_keys(golden_dir):
    g = np.load(os.path.join(golden_dir, "eval_keys.npz"))
    keys = pn.hand_keys(g["hands"])
    assert np.array_equal(keys, g["keys"])  # includes repeated-card hands


def test_bet_actions(golden_dir):
    for s in json.load(open(os.path.join(golden_dir, "bet_actions.json"))):
        cfg = pn.bet_config([b for b in s["bets"]] + (["a"] if s["allin"] else []) +
                            (["e"] if s["geo"] else []) or [0.5], s["raises"], s["max_raises"])
        if not s["bets"] and not s["allin"] and not s["geo"]:
            cfg.n_bet_fracs = 0
        cfg.add_allin_threshold = s["add"]
        cfg.force_allin_threshold = s["force"]
        cfg.merging_threshold = s["merge"]
        got = pn.bet_actions(s["pot"], s["stack"], cfg, s["sc0"], s["sc1"], s["actor"],
                             s["after_allin"], s["num_bets"], s["num_streets"])
        assert [list(a) for a in got] == s["out"], s


def test_range_parser(golden_dir):
    for text, want in json.load(open(os.path.join(golden_dir, "ranges.json"))).items():
        if want is None:
            with pytest.raises(RuntimeError):
                pn.parse_range(text)
        else:
            assert np.array_equal(pn.parse_range(text), np.asarray(want)), text


def test_range_totals():
    """tests/test_main.cpp:910-929 (RangeParser) of the reference."""
    cases = {"AA": 6, "AKs": 4, "AKo": 12, "AK": 16, "TT+": 30, "A9s+": 20, "T9s+": 20,
             "A5s-A2s": 16, "98s-65s": 16, "55-22": 24, "AA:0.5,KK": 9, "AK,AA": 22}
    for text, total in cases.items():
        assert abs(pn.parse_range(text).sum() - total) < 1e-9


def _write(path, chunks):
    with open(path, "wb") as f:
        for c in chunks:
            f.write(c)


def test_solution_file_errors_before_device(tmp_path):
    missing = str(tmp_path / "nope.sol")
    with pytest.raises(RuntimeError, match="cannot open"):
        pn.Solver.load(missing)
    bad = str(tmp_path / "bad.sol")
    _write(bad, [b"XXXX", struct.pack("<I", 1)])
    with pytest.raises(RuntimeError, match="not a solution file"):
        pn.Solver.load(bad)
    _write(bad, [struct.pack("<II", 0x31535050, 7)])
    with pytest.raises(RuntimeError, match="version"):
        pn.Solver.load(bad)
    _write(bad, [struct.pack("<IIi", 0x31535050, 1, 9)])
    with pytest.raises(RuntimeError, match="board size"):
        pn.Solver.load(bad)
    _write(bad, [struct.pack("<IIi", 0x31535050, 1, 5), bytes(3)])
    with pytest.raises(RuntimeError, match="truncated"):
        pn.Solver.load(bad)


def test_bad_inputs_rejected_on_host():
    with pytest.raises(RuntimeError):
        pn.Solver(board="Qs9h", oop="TT+", ip="99+", pot=100, stack=100)
    with pytest.raises(RuntimeError):
        pn.Solver(board="Qs9h2d7c", oop="XX", ip="99+", pot=100, stack=100)
    with pytest.raises(RuntimeError):
        pn.Solver(board="Qs9h2d7c", oop="TT+", ip="99+", pot=100, stack=100, bets="")
    with pytest.raises(RuntimeError):
        pn.Solver(board="QsQs2d7c", oop="TT+", ip="99+", pot=100, stack=100)
    # the reference binding's messages (python/pps_native.cpp:66, 74, 104, 152)
    for kw, msg in ((dict(board="QsXh2d"), "bad card rank 'X'"),
                    (dict(board="Qs9z2d"), "bad card suit 'z'"),
                    (dict(board="Qs9h"), 'board must be 3, 4 or 5 cards (e.g. "Qs9h2d")'),
                    (dict(bets="0.5,zz"), "bad bet size token 'zz'")):
        args = dict(board="Qs9h2d", oop="TT+", ip="99+", pot=100, stack=100)
        args.update(kw)
        with pytest.raises(RuntimeError) as e:
            pn.Solver(**args)
        assert str(e.value) == msg


def test_batch_footprint_host_only():
    """pps_gb_batch_footprint compiles on the host: footprints grow with
    the tree and the 48,255-node turn spot (turn_c3) needs ~1.7 GB (f32 rows, FP64 walk
    rows, tables, groups, records)."""
    from pps import batch as pb
    from pps import workloads as wl
    from helpers import weights

    def fp(sp):
        return pb.footprint(sp.board_text(), weights(sp.oop), weights(sp.ip), sp.pot,
                            sp.stack, sp.cfg.bet_text(), sp.cfg.raise_text() or [],
                            sp.cfg.max_raises)
    small, mid, big = fp(wl.river_c1()), fp(wl.turn_api()), fp(wl.turn_c3())
    assert 0 < small < mid < big
    assert 1.2e9 < big < 2.5e9


def test_batched_distribution():
    """The batched / served spot distribution: ~70% river / 30% turn,
    all-combo U(0,1) ranges, pot in [50, 200), stack/pot in [1, 8], 2-4
    distinct bet sizes from {25, 33, 50, 75, 100, 150}% plus all-in."""
    from pps import workloads as wl
    spots = wl.batched(256)
    rivers = sum(len(s.board) == 5 for s in spots)
    assert 150 <= rivers <= 210
    for s in spots:
        assert 50 <= s.pot < 200
        assert 0.99 <= s.stack / s.pot <= 8.01
        assert 2 <= len(s.cfg.bets) <= 4 and len(set(s.cfg.bets)) == len(s.cfg.bets)
        assert set(s.cfg.bets) <= {0.25, 0.33, 0.5, 0.75, 1.0, 1.5} and s.cfg.allin
        assert len(s.oop) == 1326 and 0.0 <= min(s.oop) and max(s.oop) < 1.0
    assert [s.board for s in wl.batched(8)] == [s.board for s in spots[:8]]  # seeded


def test_reference_kernel_argument_block(golden_dir):
    """The runner of the reference's own kernels (oracle/ref/ref_gpu.cpp)
    builds TreeBuf (cuda/gpu_cfr.cu:132-201) with the member order, offsets
    and size of the struct compiled from the reference source."""
    from oracle import ref_gpu
    want = json.load(open(os.path.join(golden_dir, "ref_treebuf.json")))
    members, size = ref_gpu.args_layout()
    assert size == want["size"] == 448
    assert [list(m) for m in members] == want["members"]


def test_layout_is_pinned_and_deterministic(golden_dir):
    """The device layout (tables built on several host threads, then merged
    in state order) is byte-identical run to run and equal to the committed
    digests, which the serial builder produced."""
    from pps import workloads as wl
    from helpers import abi_cfgs
    with open(os.path.join(golden_dir, "layout_digests.json")) as f:
        want = json.load(f)["digests"]
    for name, hexd in want.items():
        sp = wl.NAMED[name]()
        args = (sp.board, sp.oop, sp.ip, sp.pot, sp.stack, abi_cfgs(sp))
        got = [pn.layout_digest(*args) for _ in range(2)]
        assert got[0] == got[1] == int(hexd, 16), name


def test_layouts_built_concurrently_match(golden_dir):
    """Layouts built from several threads at once (as a batch's compile
    workers build them; each build also runs its own helper threads) are
    the pinned bytes."""
    import threading
    from pps import workloads as wl
    from helpers import abi_cfgs
    with open(os.path.join(golden_dir, "layout_digests.json")) as f:
        want = json.load(f)["digests"]
    names = ["turn_w52", "turn_c2_uniform", "flop_small", "turn_api"]
    got, errors = {}, []

    def work(k):
        try:
            for name in names[k % len(names):] + names[:k % len(names)]:
                sp = wl.NAMED[name]()
                d = pn.layout_digest(sp.board, sp.oop, sp.ip, sp.pot, sp.stack, abi_cfgs(sp))
                got.setdefault(name, []).append(d)
        except Exception as e:  # noqa: BLE001 - reported below
            errors.append(repr(e))

    threads = [threading.Thread(target=work, args=(k,)) for k in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    for name in names:
        assert got[name] == [int(want[name], 16)] * 4, name


def test_cli_argument_errors():
    """gpu_pfflop rejects bad arguments before any device use, with the
    reference CLI's messages and exit status 2 (tools/gpu_pfflop.cu:44-52,
    104-137)."""
    import subprocess
    exe = os.path.join(os.path.dirname(pn.__file__), "gpu_pfflop")
    ok = ["TT+", "AA", "100", "100", "0.5", "2", "10"]
    cases = [([], "usage: gpu_pfflop postflop"),
             (["postflop", "Qs9h"] + ok, "board must be 3, 4 or 5 cards"),
             (["postflop", "QsXh2d"] + ok, "bad card rank 'X'"),
             (["postflop", "Qs9z2d"] + ok, "bad card suit 'z'"),
             (["postflop", "Qs9h2d", "TT+", "AA", "100", "100", "0.5,zz", "2", "10"],
              "bad bet sizes '0.5,zz' (use fractions and/or 'a')")]
    for args, msg in cases:
        r = subprocess.run([exe] + args, capture_output=True, text=True, timeout=60)
        assert r.returncode == 2 and r.stdout == "" and r.stderr.startswith(msg), (args, r.stderr)
