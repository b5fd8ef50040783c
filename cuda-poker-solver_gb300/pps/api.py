"""HTTP front-end: the reference's python/pps_api.py endpoints over
pps.service.SolverService (needs FastAPI; the service itself does not).

    uvicorn pps.api:app --host 127.0.0.1 --port 8070

The routes, request bodies and answers are those of the reference API, so
its clients and UI work unchanged. The difference is concurrency: there is
no global solve lock. Solves of different solvers run at once, and one-shot
solves with a target share the GPU through continuous batching (see
pps/service.py). Added: ``POST /solvers/{id}/save`` takes ``compressed``,
and ``GET /health`` reports ``solve_lock: false``.
"""
from __future__ import annotations

from typing import Any, Dict, List, Optional, Union

from fastapi import FastAPI, HTTPException, Query
from pydantic import BaseModel, Field

from . import __version__
from .service import ServiceError, SolverService

RangeArg = Union[str, Dict[str, float], List[float]]
BetSizesArg = Union[str, List[Union[float, str]]]


class SpotSpec(BaseModel):
    board: str = Field(..., description='e.g. "Qs9h2d7c" (3-5 cards)')
    oop: RangeArg
    ip: RangeArg
    pot: int = Field(..., ge=0)
    stack: int = Field(..., gt=0)
    bets: BetSizesArg = "0.75,a"
    raises: Union[str, List[float]] = "2.5,3"
    max_raises: int = Field(0, ge=0)


class SolveParams(BaseModel):
    max_iters: int = Field(2000, gt=0)
    algo: str = "dcfr"
    target: Optional[float] = Field(None, gt=0.0)
    wait: bool = True


class ContinueParams(BaseModel):
    max_iters: int = Field(2000, gt=0)
    target: Optional[float] = Field(None, gt=0.0)
    wait: bool = True


class SaveParams(BaseModel):
    name: str
    compressed: bool = False


class LoadParams(BaseModel):
    name: str


class OneShot(SpotSpec, SolveParams):
    strategy_nodes: List[int] = Field(default_factory=list)
    root_ev: bool = False
    keep: bool = False


def _dump(m: BaseModel) -> Dict[str, Any]:
    return m.model_dump() if hasattr(m, "model_dump") else m.dict()


def create_app(service: Optional[SolverService] = None) -> FastAPI:
    svc = service if service is not None else SolverService()
    app = FastAPI(title="pps solver API (GB300)", version=__version__,
                  description="GPU postflop DCFR solver: the reference API's endpoints "
                              "without a global solve lock, one-shot solves served by "
                              "continuous batching.")

    def call(fn, *args):
        try:
            return fn(*args)
        except ServiceError as e:
            raise HTTPException(e.status, e.message) from e

    @app.get("/health")
    def health():
        return call(svc.health)

    @app.post("/solvers", status_code=201)
    def create_solver(spec: SpotSpec):
        return call(svc.create_solver, _dump(spec))

    @app.get("/solvers")
    def list_solvers():
        return call(svc.list_solvers)

    @app.get("/solvers/{sid}")
    def get_solver(sid: str):
        return call(svc.get_solver, sid)

    @app.delete("/solvers/{sid}")
    def delete_solver(sid: str):
        return call(svc.delete_solver, sid)

    @app.post("/solvers/{sid}/solve")
    def solve(sid: str, p: SolveParams):
        return call(svc.solve, sid, _dump(p))

    @app.post("/solvers/{sid}/continue")
    def continue_solve(sid: str, p: ContinueParams):
        return call(svc.continue_solve, sid, _dump(p))

    @app.post("/solvers/{sid}/cancel")
    def cancel(sid: str):
        return call(svc.cancel, sid)

    @app.post("/solvers/{sid}/reset")
    def reset(sid: str):
        return call(svc.reset, sid)

    @app.get("/solvers/{sid}/stats")
    def stats(sid: str):
        return call(svc.stats, sid)

    @app.get("/solvers/{sid}/strategy")
    def strategy(sid: str, node: int = Query(0, ge=0)):
        return call(svc.strategy, sid, node)

    @app.get("/solvers/{sid}/decide-nodes")
    def decide_nodes(sid: str, offset: int = Query(0, ge=0),
                     limit: int = Query(200, gt=0, le=2000)):
        return call(svc.decide_nodes, sid, offset, limit)

    @app.get("/solvers/{sid}/node-nav")
    def node_nav(sid: str, node: int = Query(0, ge=0)):
        return call(svc.node_nav, sid, node)

    @app.get("/solvers/{sid}/range")
    def player_range(sid: str, player: int = Query(0, ge=0, le=1)):
        return call(svc.range, sid, player)

    @app.get("/solvers/{sid}/root-ev")
    def root_ev(sid: str):
        return call(svc.root_ev, sid)

    @app.get("/solvers/{sid}/node-ev")
    def node_ev(sid: str, node: int = Query(0, ge=0)):
        return call(svc.node_ev, sid, node)

    @app.get("/solvers/{sid}/runout-summary")
    def runout_summary(sid: str, node: int = Query(0, ge=0), action: int = Query(0, ge=0)):
        return call(svc.runout_summary, sid, node, action)

    @app.post("/solvers/{sid}/save")
    def save(sid: str, p: SaveParams):
        return call(svc.save, sid, p.name, p.compressed)

    @app.post("/solvers/load", status_code=201)
    def load(p: LoadParams):
        return call(svc.load, p.name)

    @app.get("/solutions")
    def list_solutions():
        return call(svc.list_solutions)

    @app.post("/solve")
    def solve_oneshot(body: OneShot):
        return call(svc.solve_oneshot, _dump(body))

    app.state.service = svc
    return app


_app: Optional[FastAPI] = None


def __getattr__(name: str):
    """``pps.api:app`` for ASGI servers, built on first use, so that
    importing the module for create_app starts no service."""
    global _app
    if name == "app":
        if _app is None:
            _app = create_app()
        return _app
    raise AttributeError(name)
