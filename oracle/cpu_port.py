"""ctypes wrapper of the C restatement (oracle/kpm_cpu.c) - TEST INFRASTRUCTURE ONLY."""
from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse as sp

from .build_oracle import build

_lib = None


def _load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(build()))
        vp, i64 = C.c_void_p, C.c_int64
        lib.kpm1d_cpu.argtypes = [i64, vp, vp, vp, i64, i64, vp, vp, C.c_int, i64]
        lib.kpm1d_cpu.restype = C.c_int
        lib.kpm_cpu_max_threads.restype = C.c_int
        _lib = lib
    return _lib


def max_threads() -> int:
    return int(_load().kpm_cpu_max_threads())


def kpm1d_cpu(H, NC: int, psi: np.ndarray, nthreads: int = 0, last_n: int = -1) -> np.ndarray:
    """mu_all (NR, NC) from the C port; ``last_n`` bounds the number of steps."""
    lib = _load()
    H = sp.csc_matrix(H, dtype=np.complex128)
    H.sort_indices()
    colptr = np.ascontiguousarray(H.indptr, dtype=np.int64)
    rowval = np.ascontiguousarray(H.indices, dtype=np.int64)
    nz = np.ascontiguousarray(H.data, dtype=np.complex128)
    NH, NR = psi.shape
    p = np.asfortranarray(psi, dtype=np.complex128)
    mu = np.zeros((NR, NC), dtype=np.complex128, order="F")
    rc = lib.kpm1d_cpu(NH, colptr.ctypes.data, rowval.ctypes.data, nz.ctypes.data, NC, NR,
                       p.ctypes.data, mu.ctypes.data, int(nthreads), int(last_n))
    if rc != 0:
        raise ValueError(f"kpm1d_cpu failed with status {rc}")
    return np.ascontiguousarray(mu)
