"""HTTP front-end without a web framework: the reference API's routes
(python/pps_api.py) over pps.service.SolverService, served by the standard
library's threading HTTP server.

    python -m pps.httpd --host 127.0.0.1 --port 8070

pps/api.py serves the same routes through FastAPI where that is installed;
this module needs nothing beyond the standard library, so it also runs
where FastAPI is absent. Both map requests onto the same service calls:
the same bodies (field defaults and bounds as the reference's request
models), the same answers, the same status codes (400 engine and argument
errors, 404 unknown solver or file, 409 job conflict, 422 request
validation).
"""
from __future__ import annotations

import argparse
import json
import re
import threading
from http.server import BaseHTTPRequestHandler, ThreadingHTTPServer
from typing import Any, Callable, Dict, List, Optional, Tuple
from urllib.parse import parse_qs, urlsplit

from .service import ServiceError, SolverService

REQUIRED = object()


def _num(v, kind):
    if isinstance(v, bool) or not isinstance(v, (int, float)):
        raise ValueError("must be a number")
    if kind is int and isinstance(v, float):
        if not v.is_integer():
            raise ValueError("must be an integer")
        v = int(v)
    return kind(v)


# Field: (default or REQUIRED, converter, bound check or None)
def _field(default, conv, check=None):
    return (default, conv, check)


def _int(v):
    return _num(v, int)


def _float(v):
    return _num(v, float)


def _bool(v):
    if not isinstance(v, bool):
        raise ValueError("must be a boolean")
    return v


def _str(v):
    if not isinstance(v, str):
        raise ValueError("must be a string")
    return v


def _any(v):
    return v


def _opt(conv):
    return lambda v: None if v is None else conv(v)


def _int_list(v):
    if not isinstance(v, list):
        raise ValueError("must be a list")
    return [_int(x) for x in v]


SPOT = {"board": _field(REQUIRED, _str), "oop": _field(REQUIRED, _any),
        "ip": _field(REQUIRED, _any), "pot": _field(REQUIRED, _int, lambda x: x >= 0),
        "stack": _field(REQUIRED, _int, lambda x: x > 0), "bets": _field("0.75,a", _any),
        "raises": _field("2.5,3", _any), "max_raises": _field(0, _int, lambda x: x >= 0)}
SOLVE = {"max_iters": _field(2000, _int, lambda x: x > 0), "algo": _field("dcfr", _str),
         "target": _field(None, _opt(_float), lambda x: x is None or x > 0),
         "wait": _field(True, _bool)}
CONTINUE = {"max_iters": _field(2000, _int, lambda x: x > 0),
            "target": _field(None, _opt(_float), lambda x: x is None or x > 0),
            "wait": _field(True, _bool)}
SAVE = {"name": _field(REQUIRED, _str), "compressed": _field(False, _bool)}
LOAD = {"name": _field(REQUIRED, _str)}
ONESHOT = dict(SPOT, **SOLVE, strategy_nodes=_field([], _int_list),
               root_ev=_field(False, _bool), keep=_field(False, _bool))


class RequestError(Exception):
    """A request the route's schema rejects (HTTP 422)."""


def validate(schema: Dict[str, Tuple], body: Any) -> Dict[str, Any]:
    if not isinstance(body, dict):
        raise RequestError("body must be a JSON object")
    out = {}
    for name, (default, conv, check) in schema.items():
        if name not in body:
            if default is REQUIRED:
                raise RequestError("field %r is required" % name)
            out[name] = default
            continue
        try:
            v = conv(body[name])
        except (ValueError, TypeError) as e:
            raise RequestError("field %r: %s" % (name, e)) from e
        if check is not None and not check(v):
            raise RequestError("field %r out of range" % name)
        out[name] = v
    return out


def _query_int(q: Dict[str, List[str]], name: str, default: int, lo: Optional[int] = None,
               hi: Optional[int] = None, gt: Optional[int] = None) -> int:
    if name not in q:
        return default
    try:
        v = int(q[name][-1])
    except ValueError as e:
        raise RequestError("query %r must be an integer" % name) from e
    if (lo is not None and v < lo) or (hi is not None and v > hi) or (gt is not None and v <= gt):
        raise RequestError("query %r out of range" % name)
    return v


Handler = Callable[[SolverService, Dict[str, str], Dict[str, List[str]], Any], Any]

# (method, path template, status on success, handler)
ROUTES: List[Tuple[str, str, int, Handler]] = [
    ("GET", "/health", 200, lambda s, p, q, b: s.health()),
    ("POST", "/solvers", 201, lambda s, p, q, b: s.create_solver(validate(SPOT, b))),
    ("GET", "/solvers", 200, lambda s, p, q, b: s.list_solvers()),
    ("POST", "/solvers/load", 201, lambda s, p, q, b: s.load(validate(LOAD, b)["name"])),
    ("GET", "/solvers/{sid}", 200, lambda s, p, q, b: s.get_solver(p["sid"])),
    ("DELETE", "/solvers/{sid}", 200, lambda s, p, q, b: s.delete_solver(p["sid"])),
    ("POST", "/solvers/{sid}/solve", 200,
     lambda s, p, q, b: s.solve(p["sid"], validate(SOLVE, b))),
    ("POST", "/solvers/{sid}/continue", 200,
     lambda s, p, q, b: s.continue_solve(p["sid"], validate(CONTINUE, b))),
    ("POST", "/solvers/{sid}/cancel", 200, lambda s, p, q, b: s.cancel(p["sid"])),
    ("POST", "/solvers/{sid}/reset", 200, lambda s, p, q, b: s.reset(p["sid"])),
    ("GET", "/solvers/{sid}/stats", 200, lambda s, p, q, b: s.stats(p["sid"])),
    ("GET", "/solvers/{sid}/strategy", 200,
     lambda s, p, q, b: s.strategy(p["sid"], _query_int(q, "node", 0, lo=0))),
    ("GET", "/solvers/{sid}/decide-nodes", 200,
     lambda s, p, q, b: s.decide_nodes(p["sid"], _query_int(q, "offset", 0, lo=0),
                                       _query_int(q, "limit", 200, gt=0, hi=2000))),
    ("GET", "/solvers/{sid}/node-nav", 200,
     lambda s, p, q, b: s.node_nav(p["sid"], _query_int(q, "node", 0, lo=0))),
    ("GET", "/solvers/{sid}/range", 200,
     lambda s, p, q, b: s.range(p["sid"], _query_int(q, "player", 0, lo=0, hi=1))),
    ("GET", "/solvers/{sid}/root-ev", 200, lambda s, p, q, b: s.root_ev(p["sid"])),
    ("GET", "/solvers/{sid}/node-ev", 200,
     lambda s, p, q, b: s.node_ev(p["sid"], _query_int(q, "node", 0, lo=0))),
    ("GET", "/solvers/{sid}/runout-summary", 200,
     lambda s, p, q, b: s.runout_summary(p["sid"], _query_int(q, "node", 0, lo=0),
                                         _query_int(q, "action", 0, lo=0))),
    ("POST", "/solvers/{sid}/save", 200,
     lambda s, p, q, b: (lambda v: s.save(p["sid"], v["name"], v["compressed"]))(
         validate(SAVE, b))),
    ("GET", "/solutions", 200, lambda s, p, q, b: s.list_solutions()),
    ("POST", "/solve", 200, lambda s, p, q, b: s.solve_oneshot(validate(ONESHOT, b))),
]


def _compile(template: str):
    return re.compile("^" + re.sub(r"\{(\w+)\}", r"(?P<\1>[^/]+)", template) + "$")


_COMPILED = [(m, _compile(t), st, h) for m, t, st, h in ROUTES]


def route_set() -> List[Tuple[str, str]]:
    return sorted((m, t) for m, t, _, _ in ROUTES)


def dispatch(svc: SolverService, method: str, url: str, body: Any = None) -> Tuple[int, Any]:
    """One request: (status, JSON-able answer). Errors answer
    {"detail": message}, as FastAPI does."""
    parts = urlsplit(url)
    query = parse_qs(parts.query)
    allowed = False
    for m, rx, status, handler in _COMPILED:
        mt = rx.match(parts.path)
        if not mt:
            continue
        allowed = True
        if m != method:
            continue
        try:
            return status, handler(svc, mt.groupdict(), query, body if body is not None else {})
        except RequestError as e:
            return 422, {"detail": str(e)}
        except ServiceError as e:
            return e.status, {"detail": e.message}
    return (405, {"detail": "method not allowed"}) if allowed else (404, {"detail": "not found"})


def make_server(svc: SolverService, host: str = "127.0.0.1", port: int = 8070
                ) -> ThreadingHTTPServer:
    """A threading HTTP server answering the routes from `svc` (port 0:
    any free port, see server.server_address)."""

    class _Handler(BaseHTTPRequestHandler):
        protocol_version = "HTTP/1.1"

        def _answer(self, method):
            n = int(self.headers.get("Content-Length") or 0)
            raw = self.rfile.read(n) if n else b""
            try:
                body = json.loads(raw) if raw else None
            except json.JSONDecodeError:
                status, out = 422, {"detail": "body is not JSON"}
            else:
                status, out = dispatch(svc, method, self.path, body)
            data = json.dumps(out).encode()
            self.send_response(status)
            self.send_header("Content-Type", "application/json")
            self.send_header("Content-Length", str(len(data)))
            self.end_headers()
            self.wfile.write(data)

        def do_GET(self):
            self._answer("GET")

        def do_POST(self):
            self._answer("POST")

        def do_DELETE(self):
            self._answer("DELETE")

        def log_message(self, *args):
            pass

    return ThreadingHTTPServer((host, port), _Handler)


def serve_in_thread(svc: SolverService, host: str = "127.0.0.1", port: int = 0):
    """Starts make_server on a daemon thread; returns (server, base URL)."""
    srv = make_server(svc, host, port)
    threading.Thread(target=srv.serve_forever, daemon=True).start()
    h, p = srv.server_address[:2]
    return srv, "http://%s:%d" % (h, p)


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--host", default="127.0.0.1")
    ap.add_argument("--port", type=int, default=8070)
    args = ap.parse_args()
    srv = make_server(SolverService(), args.host, args.port)
    try:
        srv.serve_forever()
    finally:
        srv.server_close()


if __name__ == "__main__":
    main()
