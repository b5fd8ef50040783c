"""The HTTP front-end (pps/api.py) on the host: every route of the
reference's python/pps_api.py exists with the same method, and service
errors map onto HTTP status codes. The service calls are faked here (no
GPU); tests/test_gpu_service.py runs the real service."""
import asyncio
import json
import os

import pytest

pytest.importorskip("fastapi")

from pps import api  # noqa: E402
from pps.service import ServiceError  # noqa: E402


def call(app, method, path, body=None, query=""):
    """One request through the ASGI app (no HTTP client needed)."""
    async def run():
        payload = json.dumps(body).encode() if body is not None else b""
        scope = {"type": "http", "asgi": {"version": "3.0"}, "http_version": "1.1",
                 "method": method, "scheme": "http", "path": path,
                 "raw_path": path.encode(), "query_string": query.encode(), "root_path": "",
                 "headers": [(b"content-type", b"application/json"),
                             (b"content-length", str(len(payload)).encode())],
                 "client": ("127.0.0.1", 1), "server": ("127.0.0.1", 80)}
        inbox = [{"type": "http.request", "body": payload, "more_body": False}]
        sent = []

        async def receive():
            return inbox.pop(0) if inbox else {"type": "http.disconnect"}

        async def send(msg):
            sent.append(msg)

        await app(scope, receive, send)
        status = next(m["status"] for m in sent if m["type"] == "http.response.start")
        data = b"".join(m.get("body", b"") for m in sent if m["type"] == "http.response.body")
        return status, (json.loads(data) if data else None)
    return asyncio.run(run())


class FakeService:
    """Answers with the arguments it was called with; sid "missing" is 404."""

    def __getattr__(self, name):
        def fn(*args):
            if args and args[0] == "missing":
                raise ServiceError(404, "no solver missing")
            return {"op": name, "args": list(args)}
        return fn


def test_every_reference_route_exists(golden_dir):
    want = {tuple(r) for r in json.load(open(os.path.join(golden_dir, "api_routes.json")))}
    app = api.create_app(FakeService())
    have = set()
    for r in app.routes:
        for m in getattr(r, "methods", None) or ():
            have.add((m, r.path))
    assert want <= have, sorted(want - have)


def test_requests_reach_the_service_and_errors_map():
    app = api.create_app(FakeService())
    st, body = call(app, "POST", "/solvers", {"board": "Qs9h2d7c", "oop": "TT+", "ip": "99+",
                                               "pot": 100, "stack": 200})
    assert st == 201 and body["op"] == "create_solver"
    assert body["args"][0]["bets"] == "0.75,a"  # the reference's defaults
    st, body = call(app, "GET", "/solvers/abc/node-ev", query="node=7")
    assert st == 200 and body == {"op": "node_ev", "args": ["abc", 7]}
    st, body = call(app, "POST", "/solvers/abc/save", {"name": "x.sol", "compressed": True})
    assert st == 200 and body["args"] == ["abc", "x.sol", True]
    st, body = call(app, "GET", "/solvers/missing/stats")
    assert st == 404 and "no solver" in body["detail"]
    st, _ = call(app, "GET", "/solvers/abc/range", query="player=3")
    assert st == 422  # validated before the service
    st, body = call(app, "POST", "/solve", {"board": "Qs9h2d7c3h", "oop": "TT+", "ip": "99+",
                                           "pot": 100, "stack": 100, "target": 0.5})
    assert st == 200 and body["op"] == "solve_oneshot" and body["args"][0]["target"] == 0.5
