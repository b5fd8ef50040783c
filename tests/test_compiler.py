"""The product tree compiler against the REFERENCE compiler's own artifacts
(captured from cuda/gpu_cfr.cu:1331-1827 by oracle/ref/ref_capture): every
array bit-exact for the small spots, sha256-equal for the large ones."""
import hashlib
import json
import os

import numpy as np
import pytest

from pps import pps_native as pn
from pps import workloads as wl

from helpers import abi_cfgs


def export(spot):
    return pn.compile_export(spot.board, spot.oop, spot.ip, spot.pot, spot.stack,
                             abi_cfgs(spot))


@pytest.mark.parametrize("name", ["river_c1", "turn_api", "turn_tiny", "turn_short",
                                  "flop_short", "river_geo", "river_empty"])
def test_bit_exact_small(golden_dir, name):
    ref = dict(np.load(os.path.join(golden_dir, "ref_%s.npz" % name)))
    mine = export(wl.NAMED[name]())
    assert sorted(ref) == sorted(mine)
    for k, v in ref.items():
        assert mine[k].dtype == v.dtype and np.array_equal(mine[k], v), k


@pytest.mark.parametrize("name", ["turn_w52", "turn_c3", "turn_c2_uniform", "flop_small"])
def test_bit_exact_large(golden_dir, name):
    hashes = json.load(open(os.path.join(golden_dir, "ref_hashes.json")))[name]
    mine = export(wl.NAMED[name]())
    assert sorted(hashes) == sorted(mine)
    for k, (digest, size) in hashes.items():
        a = np.ascontiguousarray(mine[k])
        assert a.size == size and hashlib.sha256(a.tobytes()).hexdigest() == digest, k


def test_per_street_config_changes_only_later_streets():
    """Per-street configs (extension): the turn config drives the turn
    nodes, the river config the river nodes."""
    spot = wl.turn_c2()
    per = export(spot)
    uni = export(wl.turn_c2(uniform_config=True))
    k0 = per["actAmount"][:per["na"][0]]
    assert np.array_equal(k0, uni["actAmount"][:uni["na"][0]])
    meta = per["decideMeta"].reshape(-1, 8)
    river = meta[meta[:, 5] == 5]
    assert len(river) and not np.array_equal(per["actAmount"], uni["actAmount"])
    # every river decide node's bets follow the river config {0.5, 1.0}
    first = river[0]
    pot = per["potBase"][first[6]]
    amounts = per["actAmount"][first[7]:first[7] + first[1]]
    assert round(0.5 * pot) in amounts or round(1.0 * pot) in amounts
