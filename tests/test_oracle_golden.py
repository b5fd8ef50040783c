"""The CPU oracle against the reference's own golden vectors (CPU only):
evaluator keys, bet abstraction and the tiny_check known answers."""
import json
import os

import numpy as np
import pytest

from oracle import cpu_oracle as co
from pps import workloads as wl

from helpers import oracle, seeded_rows


def test_evaluator_keys(golden_dir):
    g = np.load(os.path.join(golden_dir, "eval_keys.npz"))
    hands, keys = g["hands"], g["keys"]
    # The oracle evaluates distinct cards only (the first 20000 hands).
    for h, k in zip(hands[:20000], keys[:20000]):
        assert co.strength7(h) == int(k)


def test_bet_actions(golden_dir):
    states = json.load(open(os.path.join(golden_dir, "bet_actions.json")))
    for s in states:
        cfg = co.make_cfg(s["bets"], s["raises"], s["allin"], s["geo"], s["max_raises"],
                          s["add"], s["force"], s["merge"])
        got = co.actions(s["pot"], s["stack"], cfg, s["sc0"], s["sc1"], s["actor"],
                         s["after_allin"], s["num_bets"], s["num_streets"])
        assert [list(a) for a in got] == s["out"], s


@pytest.mark.parametrize("name", ["river_c1", "turn_api", "turn_tiny", "turn_short",
                                  "flop_short", "river_geo"])
def test_tree_shape(golden_dir, name):
    ref = np.load(os.path.join(golden_dir, "ref_%s.npz" % name))
    o = oracle(wl.NAMED[name]())
    assert o.num_nodes == int(ref["numNodes"][0])
    assert o.row_total == int(ref["regTotal"][0])


@pytest.mark.parametrize("tag,mode", [("TINY", None), ("M7", 7), ("M9", 9)])
def test_tiny_check_known_answers(golden_dir, tag, mode):
    """tools/tiny_check.cpp ground truth: EV under uniform and two seeded
    profiles, tolerance 1e-4 (tools/quality/gpu_postflop_parity.sh:126-148)."""
    want = json.load(open(os.path.join(golden_dir, "tiny_check.json")))[tag]
    ref = np.load(os.path.join(golden_dir, "ref_turn_tiny.npz"))
    spot = wl.turn_tiny()
    o = oracle(spot, precision=64)
    if mode:
        o.set_rows(1, seeded_rows(ref["decideMeta"], o.row_total, mode))
    assert abs(o.value(0, 1) - want["ev0"]) < 1e-4
    assert abs(o.value(1, 1) - want["ev1"]) < 1e-4


def test_oracle_river_converges():
    """A planted mistake in the oracle's rows is visible: exploitability is
    small after a solve and large for a perturbed strategy."""
    spot = wl.river_c1()
    o = oracle(spot, precision=32)
    o.iterate(300)
    st = o.stats(spot.pot)
    assert abs(st["ev_oop"] + st["ev_ip"] - spot.pot) < 1e-6
    assert 0 <= st["exploitability"] < 0.05
    rows = o.rows(1)
    rows[: rows.size // 3] = 0.0
    rows[rows.size // 3: 2 * rows.size // 3] += 5.0
    o.set_rows(1, rows)
    assert o.stats(spot.pot)["exploitability"] > 10 * st["exploitability"]


def _layout(spot):
    from helpers import weights
    return co.reference_layout(spot.board, weights(spot.oop), weights(spot.ip), spot.pot,
                               spot.stack, co.cfg_from(spot.cfg))


@pytest.mark.parametrize("name", ["river_c1", "turn_api", "turn_tiny", "turn_short",
                                  "flop_short", "river_geo"])
def test_reference_layout_bit_exact_small(golden_dir, name):
    """The oracle's restatement of the reference's device layout (the input
    of the reference's kernels) equals the reference's own init() arrays,
    every one bit for bit."""
    ref = dict(np.load(os.path.join(golden_dir, "ref_%s.npz" % name)))
    mine = _layout(wl.NAMED[name]())
    assert sorted(ref) == sorted(mine)
    for k, v in ref.items():
        assert mine[k].dtype == v.dtype and np.array_equal(mine[k], v), k


@pytest.mark.parametrize("name", ["turn_w52", "turn_c3", "turn_c2_uniform", "flop_small"])
def test_reference_layout_bit_exact_large(golden_dir, name):
    import hashlib
    hashes = json.load(open(os.path.join(golden_dir, "ref_hashes.json")))[name]
    mine = _layout(wl.NAMED[name]())
    assert sorted(hashes) == sorted(mine)
    for k, (digest, size) in hashes.items():
        a = np.ascontiguousarray(mine[k])
        assert a.size == size and hashlib.sha256(a.tobytes()).hexdigest() == digest, k
