"""pps: GB300-native heads-up postflop DCFR solver - Python interface.

The same programmatic surface as the reference's ``pps`` package
(python/pps/__init__.py:22-31): ``pps.Solver`` is ``pps.pps_native.Solver``.
``pps.Batch`` (an extension) solves many spots at once on one GPU.

    import pps
    s = pps.Solver(board="Qs9h2d", oop="TT+,AKo", ip="AQ+,KQs",
                   pot=200, stack=500, bets="0.75,a", raises="2.5,3")
    s.solve(2000)
    s.stats()

The native library (libpps_gb.so, sm_103a) is built in-tree by
``python cuda-poker-solver_gb300/build_ext.py``; importing without it
raises ImportError.
"""

__all__ = ["Solver", "Batch", "__version__"]

__version__ = "0.1.0"

from . import pps_native as _native  # noqa: E402

Solver = _native.Solver

from .batch import Batch  # noqa: E402
