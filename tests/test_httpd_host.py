"""The framework-free HTTP front-end (pps/httpd.py) on the host: every route
of the reference's python/pps_api.py with the same method, the request
models' defaults and bounds (422), service errors mapped onto their status
codes, and a real HTTP round trip. The service calls are faked here (no
GPU); tests/test_gpu_api_http.py runs the reference's API tests over HTTP
against real solvers."""
import json
import os
import urllib.error
import urllib.request

from pps import httpd
from pps.service import ServiceError


class FakeService:
    """Answers with the call it received; sid "missing" is 404."""

    def __getattr__(self, name):
        def fn(*args):
            if args and args[0] == "missing":
                raise ServiceError(404, "no solver missing")
            return {"op": name, "args": list(args)}
        return fn


def test_every_reference_route_exists(golden_dir):
    want = {tuple(r) for r in json.load(open(os.path.join(golden_dir, "api_routes.json")))}
    have = set(httpd.route_set())
    assert want <= have, sorted(want - have)


def test_bodies_queries_and_errors():
    svc = FakeService()
    st, out = httpd.dispatch(svc, "POST", "/solvers/ab12/solve", {"max_iters": 300})
    assert st == 200 and out["op"] == "solve"
    assert out["args"] == ["ab12", {"max_iters": 300, "algo": "dcfr", "target": None,
                                    "wait": True}]
    st, out = httpd.dispatch(svc, "POST", "/solvers", {"board": "Qs9h2d7c", "oop": "TT+",
                                                       "ip": "AQ+", "pot": 200, "stack": 500})
    assert st == 201 and out["args"][0]["bets"] == "0.75,a" and out["args"][0]["max_raises"] == 0
    assert httpd.dispatch(svc, "POST", "/solvers", {"board": "Qs9h2d7c"})[0] == 422
    assert httpd.dispatch(svc, "POST", "/solvers/x/solve", {"max_iters": 0})[0] == 422
    assert httpd.dispatch(svc, "POST", "/solvers/x/solve", {"max_iters": "a"})[0] == 422
    assert httpd.dispatch(svc, "POST", "/solvers/x/solve", {"target": -1.0})[0] == 422
    st, out = httpd.dispatch(svc, "GET", "/solvers/x/decide-nodes?offset=3&limit=7")
    assert st == 200 and out["args"] == ["x", 3, 7]
    assert httpd.dispatch(svc, "GET", "/solvers/x/decide-nodes?limit=5000")[0] == 422
    assert httpd.dispatch(svc, "GET", "/solvers/x/range?player=2")[0] == 422
    assert httpd.dispatch(svc, "GET", "/solvers/x/strategy?node=-1")[0] == 422
    st, out = httpd.dispatch(svc, "GET", "/solvers/missing")
    assert st == 404 and "missing" in out["detail"]
    st, out = httpd.dispatch(svc, "POST", "/solvers/load", {"name": "a.sol"})
    assert st == 201 and out == {"op": "load", "args": ["a.sol"]}
    assert httpd.dispatch(svc, "GET", "/nowhere")[0] == 404
    assert httpd.dispatch(svc, "PUT", "/health")[0] == 405
    st, out = httpd.dispatch(svc, "POST", "/solve", {"board": "Qs9h2d7c", "oop": "TT+",
                                                     "ip": "AQ+", "pot": 200, "stack": 500,
                                                     "strategy_nodes": [0, 1], "keep": True})
    assert st == 200 and out["args"][0]["strategy_nodes"] == [0, 1]
    assert out["args"][0]["keep"] is True and out["args"][0]["root_ev"] is False


def test_http_round_trip():
    srv, base = httpd.serve_in_thread(FakeService())
    try:
        req = urllib.request.Request(base + "/solvers/ab/continue", method="POST",
                                     data=json.dumps({"max_iters": 5}).encode(),
                                     headers={"Content-Type": "application/json"})
        with urllib.request.urlopen(req, timeout=30) as r:
            assert r.status == 200
            assert json.loads(r.read())["args"][1]["max_iters"] == 5
        try:
            urllib.request.urlopen(base + "/solvers/missing/stats", timeout=30)
            raise AssertionError("expected 404")
        except urllib.error.HTTPError as e:
            assert e.code == 404 and "missing" in json.loads(e.read())["detail"]
    finally:
        srv.shutdown()
        srv.server_close()
