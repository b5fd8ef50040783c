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
