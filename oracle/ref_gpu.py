"""ctypes wrapper of the reference-kernel runner (oracle/ref/ref_gpu.cpp).

TEST AND MEASUREMENT INFRASTRUCTURE ONLY: the reference's own GPU kernels
(cuda/gpu_cfr.cu, compiled from its source into
oracle/_ref/gpu_cfr_kernels.fatbin by oracle/ref/build_ref.sh) run on the
reference layout that the product compiler exports. The GPU parity tests
use it as a second checker and the bench's reference leg times it; the
product path never touches it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Dict

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libref_gpu.so")
FATBIN = os.path.join(HERE, "_ref", "gpu_cfr_kernels.fatbin")

_lib = None


def fatbin_present() -> bool:
    return os.path.exists(FATBIN)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            subprocess.run(["sh", os.path.join(HERE, "build_oracle.sh")], check=True,
                           capture_output=True)
        L = C.CDLL(LIB)
        L.refgpu_last_error.restype = C.c_char_p
        L.refgpu_create.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_char_p),
                                    C.POINTER(C.c_void_p), C.POINTER(C.c_int64),
                                    C.POINTER(C.c_int), C.c_int64, C.POINTER(C.c_void_p)]
        L.refgpu_destroy.argtypes = [C.c_void_p]
        L.refgpu_solve.argtypes = [C.c_void_p, C.c_int]
        L.refgpu_time.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double)]
        L.refgpu_rows.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_float), C.c_int64]
        L.refgpu_row_total.restype = C.c_int64
        L.refgpu_row_total.argtypes = [C.c_void_p]
        L.refgpu_args_layout.argtypes = [C.POINTER(C.c_char_p), C.POINTER(C.c_int64),
                                         C.c_int, C.POINTER(C.c_int64)]
        _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc != 0:
        raise RuntimeError("reference kernels: " + lib().refgpu_last_error().decode())


def args_layout():
    """(TreeBuf member names with their byte offsets, block size) as the
    runner builds the kernels' argument block."""
    names = (C.c_char_p * 64)()
    offs = (C.c_int64 * 64)()
    size = C.c_int64()
    n = lib().refgpu_args_layout(names, offs, 64, C.byref(size))
    return [(names[i].decode(), int(offs[i])) for i in range(n)], int(size.value)


class RefKernels:
    """One spot on the reference's kernels: `export` is the product
    compiler's reference-layout export (pps_native.compile_export)."""

    def __init__(self, export: Dict[str, np.ndarray], pot: int, fatbin: str = FATBIN):
        if not os.path.exists(fatbin):
            raise FileNotFoundError(fatbin)
        keep = [np.ascontiguousarray(v) for v in export.values()]
        n = len(keep)
        names = (C.c_char_p * n)(*[k.encode() for k in export])
        ptrs = (C.c_void_p * n)(*[a.ctypes.data for a in keep])
        counts = (C.c_int64 * n)(*[a.size for a in keep])
        elems = (C.c_int * n)(*[a.dtype.itemsize for a in keep])
        h = C.c_void_p()
        _check(lib().refgpu_create(fatbin.encode(), n, names, ptrs, counts, elems, int(pot),
                                   C.byref(h)))
        self._h = h

    def close(self) -> None:
        if self._h:
            lib().refgpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, iterations: int) -> None:
        _check(lib().refgpu_solve(self._h, int(iterations)))

    def rows(self, which: int) -> np.ndarray:
        n = lib().refgpu_row_total(self._h)
        out = np.zeros(n, dtype=np.float32)
        _check(lib().refgpu_rows(self._h, int(which),
                                 out.ctypes.data_as(C.POINTER(C.c_float)), n))
        return out

    def ms_per_iteration(self, warmup: int, iterations: int) -> float:
        ms = C.c_double()
        _check(lib().refgpu_time(self._h, int(warmup), int(iterations), C.byref(ms)))
        return ms.value
