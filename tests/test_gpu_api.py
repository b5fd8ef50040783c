"""The reference's API invariants (python/test_pps.py:18-239) against this
solver, through the same pps.Solver surface."""
import os
import struct
import subprocess
import tempfile

import numpy as np
import pytest

import pps

pytestmark = pytest.mark.gpu

BOARD, OOP, IP, POT, STACK, BETS, RAISES = "Qs9h2d7c", "TT+,AKo", "AQ+,KQs", 200, 500, "0.75,a", "2.5,3"


def fresh():
    return pps.Solver(board=BOARD, oop=OOP, ip=IP, pot=POT, stack=STACK, bets=BETS, raises=RAISES)


def close(a, b, tol, what):
    d = np.max(np.abs(np.asarray(a, dtype=float) - np.asarray(b, dtype=float)))
    assert d <= tol, "%s: max diff %g > %g" % (what, d, tol)


def test_construct_and_solve():
    s = fresh()
    assert s.num_nodes > 0 and s.num_decide_nodes > 0
    s.solve(300)
    assert s.iterations_run == 300 and s.total_iterations == 300
    st = s.stats()
    close(st["ev_oop"] + st["ev_ip"], POT, 0.05, "EV zero-sum")
    assert 0.0 <= st["exploitability"] < 5.0


def test_labeled_tree():
    s = fresh()
    nodes = s.decide_nodes()
    assert len(nodes) == s.num_decide_nodes
    root = nodes[0]
    assert root["player"] == 0 and root["depth"] == 0
    assert [a["kind"] for a in root["actions"]] == ["check", "bet", "allin"]
    assert [a["amount"] for a in root["actions"]] == [0, 150, 500]
    assert all(0 <= c < s.num_nodes for c in root["children"])


def test_combo_strategy():
    s = fresh()
    s.solve(300)
    for idx in (0, 1, 2):
        r = s.strategy(idx)
        f = np.asarray(r["freqs"])
        assert f.ndim == 2 and f.shape[0] == len(r["actions"])
        assert f.shape[1] == len(r["cards"]) == len(r["combos"])
        close(f.sum(axis=0), 1.0, 1e-9, "strategy(%d) row sums" % idx)
        for c in r["cards"]:
            assert len(c) == 4 and c[0] in "23456789TJQKA" and c[1] in "cdhs"
    assert "aggregate" in s.strategy(0) and "aggregate" in s.strategy(1)
    deep = next(n["index"] for n in s.decide_nodes() if n["n_board"] == 5)
    assert "aggregate" not in s.strategy(deep)


def test_root_ev_consistency():
    s = fresh()
    s.solve(300)
    ev, st = s.root_ev(), s.stats()
    for p, agg, pl in (("oop", st["ev_oop"], 0), ("ip", st["ev_ip"], 1)):
        w = np.asarray(s.player_weights(pl))
        m, v = np.asarray(ev[p]["mass"]), np.asarray(ev[p]["ev"])
        ok = m > 0
        close((w[ok] * m[ok] * v[ok]).sum() / (w[ok] * m[ok]).sum(), agg, 2e-3, "root EV " + p)


def test_warm_start_is_exact():
    """DCFR's schedule depends only on the absolute iteration, and the
    kernels are deterministic: 150 + 150 equals 300 bit for bit."""
    a, b = fresh(), fresh()
    a.solve(300)
    b.solve(150)
    b.continue_solve(150)
    assert b.total_iterations == 300
    for which in (0, 1):
        assert np.array_equal(a.read_rows(which), b.read_rows(which))
    sa, sb = a.stats(), b.stats()
    close(sa["ev_oop"], sb["ev_oop"], 1e-12, "warm-start EV")
    b.reset()
    assert b.total_iterations == 0
    b.solve(300)
    close(sa["ev_oop"], b.stats()["ev_oop"], 1e-12, "post-reset EV")


def test_save_load(tmp_path):
    s = fresh()
    s.solve(300)
    path = str(tmp_path / "spot.sol")
    s.save(path)
    t = pps.Solver.load(path)
    assert t.num_nodes == s.num_nodes and t.total_iterations == 300
    close(s.stats()["ev_oop"], t.stats()["ev_oop"], 1e-9, "loaded EV")
    close(s.strategy(1)["freqs"], t.strategy(1)["freqs"], 1e-12, "loaded freqs")
    s.continue_solve(200)
    t.continue_solve(200)
    assert s.total_iterations == 500 == t.total_iterations
    assert np.array_equal(s.read_rows(0), t.read_rows(0))
    # truncated and mismatched files are rejected
    raw = open(path, "rb").read()
    open(str(tmp_path / "trunc.sol"), "wb").write(raw[:-100])
    with pytest.raises(RuntimeError, match="truncated"):
        pps.Solver.load(str(tmp_path / "trunc.sol"))
    with pytest.raises(RuntimeError):
        pps.Solver.load(str(tmp_path / "nonexistent.sol"))


def test_save_load_compressed(tmp_path):
    """Compressed solution files (16-bit codes, one f32 scale per action
    row): rows in about half the bytes, every entry within half a code step of its
    row's scale, the loaded solution passes the EV / exploitability gates
    against the saved one, and solving continues from it."""
    s = fresh()
    s.solve(300)
    full, comp = str(tmp_path / "full.sol"), str(tmp_path / "comp.sol")
    s.save(full)
    s.save(comp, compressed=True)
    rows = 2 * 4 * len(s.read_rows(0))  # f32 regret + strategy bytes
    header = os.path.getsize(full) - rows
    assert os.path.getsize(comp) - header < 0.55 * rows
    t = pps.Solver.load(comp)
    assert t.num_nodes == s.num_nodes and t.total_iterations == 300
    for which, q in ((0, 32767.0), (1, 65535.0)):
        a = np.asarray(s.read_rows(which), dtype=np.float64)
        b = np.asarray(t.read_rows(which), dtype=np.float64)
        assert np.max(np.abs(a - b)) <= (0.5 / q + 1e-6) * np.max(np.abs(a))
    sa, sb = s.stats(), t.stats()
    close(sa["ev_oop"], sb["ev_oop"], 1e-2, "compressed EV")
    assert abs(sa["exploitability"] - sb["exploitability"]) < 1e-2
    s.continue_solve(200)
    t.continue_solve(200)
    assert t.total_iterations == 500
    close(s.stats()["ev_oop"], t.stats()["ev_oop"], 1e-2, "continued EV")
    raw = open(comp, "rb").read()
    open(str(tmp_path / "trunc.sol"), "wb").write(raw[:-100])
    with pytest.raises(RuntimeError, match="truncated"):
        pps.Solver.load(str(tmp_path / "trunc.sol"))


def test_save_load_compressed_per_street(tmp_path):
    """Version 4: per-street bet configs with compressed rows."""
    from helpers import solver as spot_solver
    from pps import workloads as wl
    s = spot_solver(wl.turn_c2())
    s.solve(50)
    path = str(tmp_path / "c2.sol")
    s.save(path, compressed=True)
    assert struct.unpack_from("<I", open(path, "rb").read(), 4)[0] == 4
    t = pps.Solver.load(path)
    assert t.num_nodes == s.num_nodes == 6333
    close(s.stats()["ev_oop"], t.stats()["ev_oop"], 1e-2, "per-street compressed EV")


def test_errors():
    s = fresh()
    s.solve(300)
    with pytest.raises(RuntimeError):
        s.strategy(s.num_decide_nodes + 5)
    with pytest.raises(RuntimeError):
        s.solve(10, algo="cfr+")
    with pytest.raises(RuntimeError):
        s.node_ev(s.num_decide_nodes + 5)
    t = fresh()
    with pytest.raises(RuntimeError, match="no prior solve"):
        t.continue_solve(10)
    t.solve(10, algo="hs30")
    with pytest.raises(RuntimeError, match="DCFR only"):
        t.continue_solve(10)


def test_target_solve():
    s = fresh()
    s.solve(max_iters=100000, target=1.0)
    assert s.iterations_run < 100000
    assert s.stats()["exploitability"] <= 1.0
    it0 = s.total_iterations
    s.continue_solve(max_iters=100000, target=0.5)
    assert s.total_iterations > it0


def test_node_ev():
    s = fresh()
    s.solve(400)
    st = s.stats()
    ev = s.node_ev(0)
    close(ev["sides"]["oop"]["agg_ev"], st["ev_oop"], 1e-6, "node_ev root oop")
    close(ev["sides"]["ip"]["agg_ev"], st["ev_ip"], 1e-6, "node_ev root ip")
    side = ev["sides"]["oop"]
    freqs = np.asarray(s.strategy(0)["freqs"])
    mix = (freqs * np.asarray([a["per_combo"] for a in ev["action_ev"]])).sum(axis=0)
    live = np.asarray(side["mass"]) > 0
    close(mix[live], np.asarray(side["ev"])[live], 1e-4, "action mix identity")
    ev1 = s.node_ev(1)
    assert ev1["decider"] == 1 and len(ev1["action_ev"]) == len(ev1["actions"])


def test_runout_summary_and_tree():
    s = fresh()
    s.solve(200)
    nodes = s.decide_nodes()
    # OOP check, IP check behind -> deal: decide 1 action 0 leads to a chance node
    ts = s.tree_structure()
    idx, act = next((n["index"], a) for n in nodes for a, c in enumerate(n["children"])
                    if ts["kinds"][c] == 3)
    r = s.runout_summary(idx, act)
    assert len(r["branches"]) == 44 + 4  # turn spot: 48 river cards
    for br in r["branches"]:
        if br["next_decide"] >= 0 and len(br["freq"]):
            close(np.sum(br["freq"]), 1.0, 1e-9, "branch freq")
    assert len(ts["kinds"]) == s.num_nodes == len(ts["child_base"])
    assert len(ts["boards"]) == 5 * s.num_nodes


def test_queries_walk_only_what_they_read(monkeypatch):
    """node_ev and runout_summary walk the query node's subtree plus the
    forward path to it; the answers are identical to full-tree walks."""
    s = fresh()
    s.solve(200)
    nodes = s.decide_nodes()
    ts = s.tree_structure()
    deals = [(n["index"], a) for n in nodes for a, c in enumerate(n["children"])
             if ts["kinds"][c] == 3][:3]
    picks = sorted({1, 2, 5, len(nodes) // 2, len(nodes) - 1})

    def answers():
        return ([s.node_ev(i) for i in picks], [s.runout_summary(i, a) for i, a in deals])

    sub_ev, sub_run = answers()
    monkeypatch.setenv("PPS_GB_QUERY_FULL_WALKS", "1")
    full_ev, full_run = answers()
    for a, b in zip(sub_ev, full_ev):
        for side in ("oop", "ip"):
            for k in ("ev", "mass", "agg_ev"):
                assert np.array_equal(np.asarray(a["sides"][side][k]),
                                      np.asarray(b["sides"][side][k])), (side, k)
        for x, y in zip(a["action_ev"], b["action_ev"]):
            assert np.array_equal(np.asarray(x["per_combo"]), np.asarray(y["per_combo"]))
    for a, b in zip(sub_run, full_run):
        for x, y in zip(a["branches"], b["branches"]):
            assert x["agg_ev"] == y["agg_ev"] and list(x["freq"]) == list(y["freq"])


def test_cli_protocol():
    exe = os.path.join(os.path.dirname(pps.__file__), "gpu_pfflop")
    out = subprocess.run([exe, "postflop", "Qs9h2d7c", "TT+", "99+", "200", "3000", "0.5", "",
                          "0"], capture_output=True, text=True, check=True)
    lines = dict(l.split(" ", 1) for l in out.stdout.splitlines() if l)
    ev0 = float(out.stdout.split("EV 0 ")[1].split()[0])
    assert abs(ev0 - 116.649980) < 1e-4
    assert "EXPLOITABILITY" in lines
    assert "iters/s" in out.stderr and "nodes=1305" in out.stderr


def test_bounded_wait_gives_up_and_reports():
    """The device waits are bounded: a warp that waits on its barrier for a
    copy that is never issued gives up after its polls (the bulk-copied
    records' wait, then its drain rounds), sets the solver's device error
    word, and the host raises. No GPU fault is involved, and the solver
    afterwards solves exactly as a fresh one does."""
    import time
    s = fresh()
    t0 = time.time()
    with pytest.raises(RuntimeError, match="device wait timed out"):
        s.probe_bounded_wait(1024)
    assert time.time() - t0 < 120
    s.solve(30)
    f = fresh()
    f.solve(30)
    for which in (0, 1):
        assert np.array_equal(s.read_rows(which), f.read_rows(which))
