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
