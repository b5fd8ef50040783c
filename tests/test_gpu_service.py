"""The solver service behind the HTTP front-end (pps/service.py) on the GPU:
the reference API's operations (python/pps_api.py) with real solvers,
without a global solve lock."""
import threading

import numpy as np
import pytest

from pps.service import ServiceError, SolverService

pytestmark = pytest.mark.gpu

SPOT = {"board": "Qs9h2d7c", "oop": "TT+,AKo", "ip": "AQ+,KQs", "pot": 200, "stack": 500,
        "bets": "0.75,a", "raises": "2.5,3"}


@pytest.fixture
def svc(tmp_path):
    s = SolverService(max_solvers=3, data_dir=str(tmp_path / "sol"))
    yield s
    s.close()


def test_registry_solve_and_queries(svc):
    meta = svc.create_solver(SPOT)
    sid = meta["id"]
    assert meta["num_nodes"] > 0 and meta["total_iterations"] == 0
    r = svc.solve(sid, {"max_iters": 300})
    assert r["iterations_run"] == 300 and abs(r["stats"]["ev_oop"] + r["stats"]["ev_ip"] - 200) < 1e-6
    st = svc.stats(sid)
    assert st == r["stats"]
    nodes = svc.decide_nodes(sid, 0, 5)
    assert nodes["total"] == meta["num_decide_nodes"] and nodes["nodes"][0]["path"] == "(root)"
    nav = svc.node_nav(sid, 0)
    assert len(nav["actions"]) == len(svc.strategy(sid, 0)["actions"])
    deal = next((a for n in range(min(nodes["total"], 20))
                 for a in svc.node_nav(sid, n)["actions"] if a["child_kind"] == "chance"), None)
    assert deal is not None and len(deal["branches"]) == 48
    rng = svc.range(sid, 1)
    assert len(rng["combos"]) == len(rng["weights"]) > 0
    assert set(svc.node_ev(sid, 1)["sides"]) == {"oop", "ip"}
    svc.continue_solve(sid, {"max_iters": 100})
    assert svc.get_solver(sid)["total_iterations"] == 400
    with pytest.raises(ServiceError) as e:
        svc.stats("nope")
    assert e.value.status == 404
    with pytest.raises(ServiceError) as e:
        svc.node_nav(sid, 10 ** 6)
    assert e.value.status == 400


def test_background_job_and_cancel(svc):
    sid = svc.create_solver(SPOT)["id"]
    job = svc.solve(sid, {"max_iters": 20000, "wait": False})["job"]
    assert job["running"]
    with pytest.raises(ServiceError) as e:
        svc.solve(sid, {"max_iters": 10})
    assert e.value.status == 409
    svc.cancel(sid)
    meta = svc.wait_job(sid)
    assert meta["job"]["status"] in ("cancelled", "done") and not meta["job"]["running"]
    done = svc.solve(sid, {"max_iters": 2000, "wait": False})
    meta = svc.wait_job(sid)
    assert meta["job"]["status"] == "done" and meta["total_iterations"] == 2000


def test_save_load_and_lru(svc):
    sid = svc.create_solver(SPOT)["id"]
    svc.solve(sid, {"max_iters": 200})
    assert svc.save(sid, "a.sol")["bytes"] > 0
    assert svc.save(sid, "b.sol", compressed=True)["compressed"]
    names = [f["name"] for f in svc.list_solutions()["solutions"]]
    assert names == ["a.sol", "b.sol"]
    lid = svc.load("b.sol")["id"]
    assert svc.get_solver(lid)["total_iterations"] == 200
    with pytest.raises(ServiceError):
        svc.save(sid, "../escape.sol")
    for _ in range(3):  # max_solvers = 3: the oldest entries are evicted
        svc.create_solver(SPOT)
    with pytest.raises(ServiceError):
        svc.get_solver(sid)


def test_solves_of_different_solvers_run_concurrently(svc):
    """No global solve lock: two threads solve two solvers at once and get
    the same answers as one after the other."""
    a, b = svc.create_solver(SPOT)["id"], svc.create_solver(SPOT)["id"]
    out = {}

    def run(sid):
        out[sid] = svc.solve(sid, {"max_iters": 400})["stats"]

    ts = [threading.Thread(target=run, args=(s,)) for s in (a, b)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert out[a] == out[b]
    c = svc.create_solver(SPOT)["id"]
    assert svc.solve(c, {"max_iters": 400})["stats"] == out[a]


def test_oneshot_served_by_the_batch(svc):
    """One-shot solves with a target go through the shared batch, several
    at once; asking for strategies falls back to a Solver of its own."""
    spots = [dict(SPOT, pot=200 + 20 * k) for k in range(3)]
    res = [None] * 3

    def run(k):
        res[k] = svc.solve_oneshot(dict(spots[k], target=0.005 * spots[k]["pot"]))

    ts = [threading.Thread(target=run, args=(k,)) for k in range(3)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    for k, r in enumerate(res):
        assert r["served_by"] == "batch" and r["converged"]
        assert r["stats"]["exploitability"] <= 0.005 * spots[k]["pot"] + 1e-9
        assert abs(sum(r["root_strategy"]["freqs"]) - 1.0) < 1e-6
    own = svc.solve_oneshot(dict(SPOT, max_iters=200, strategy_nodes=[0], root_ev=True))
    assert own["served_by"] == "solver" and "0" in {str(k) for k in own["strategies"]}
    assert "root_ev" in own


def test_paths_navigation_and_runouts(svc):
    """The reference API's navigation behaviour (python/test_pps_api.py:
    165-276): action paths with card-labelled deals, node-nav labels, a
    flop deal with 49 runouts (card 2c included, none on the board), and a
    runout summary consistent with node_ev at each branch."""
    sid = svc.create_solver(SPOT)["id"]
    svc.solve(sid, {"max_iters": 200})
    paths = [n["path"] for n in svc.decide_nodes(sid, 0, 50)["nodes"]]
    assert paths[0] == "(root)" and paths[1].startswith("check")
    deals = [p for p in paths if "deal" in p]
    assert deals
    for p in deals:
        for step in p.split(" — "):
            if step.startswith("deal "):
                card = step[5:]
                assert len(card) == 2 and card[0] in "23456789TJQKA" and card[1] in "cdhs"
    assert svc.decide_nodes(sid, 1, 1)["nodes"][0]["index"] == 1
    nav = svc.node_nav(sid, 0)
    assert {a["label"] for a in nav["actions"]} == {"check", "bet 150", "all-in"}
    assert next(a for a in nav["actions"] if a["label"] == "check")["next_decide"] == 1
    nav1 = {a["kind"]: a for a in svc.node_nav(sid, 1)["actions"]}
    assert "fold" not in nav1 and nav1["check"]["next_decide"] is not None
    rng = svc.range(sid, 0)
    assert all(len(c) == 4 for c in rng["combos"]) and sum(rng["weights"]) > 0
    st, ev0 = svc.stats(sid), svc.node_ev(sid, 0)
    assert abs(ev0["sides"]["oop"]["agg_ev"] - st["ev_oop"]) < 1e-4
    assert abs(ev0["sides"]["ip"]["agg_ev"] - st["ev_ip"]) < 1e-4
    with pytest.raises(ServiceError) as e:
        svc.node_ev(sid, 99999)
    assert e.value.status == 400

    fid = svc.create_solver(dict(SPOT, board="Qs9h2d"))["id"]
    svc.solve(fid, {"max_iters": 100})
    nav = svc.node_nav(fid, 1)
    check = next(a for a in nav["actions"] if a["kind"] == "check")
    assert check["child_kind"] == "chance"
    cards = [b["card"] for b in check["branches"]]
    assert len(cards) == len(set(cards)) == 49 and "2c" in cards and "?" not in cards
    assert not set(cards) & {"Qs", "9h", "2d"}
    rs = svc.runout_summary(fid, 1, [a["kind"] for a in nav["actions"]].index("check"))
    assert rs["decider"] == 0 and [b["card"] for b in rs["branches"]] == cards
    live = [b for b in rs["branches"] if b["next_decide"] >= 0]
    assert len(live) == 49
    for b in live:
        assert len(b["freq"]) == len(rs["actions"]) and abs(sum(b["freq"]) - 1.0) < 1e-5
    first = live[0]
    nev = svc.node_ev(fid, first["next_decide"])
    assert abs(nev["sides"]["oop"]["agg_ev"] - first["agg_ev"]["oop"]) < 1e-3
    with pytest.raises(ServiceError) as e:
        svc.runout_summary(fid, 0, 0)  # not a deal
    assert e.value.status == 400
