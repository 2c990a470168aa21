"""Device-resident sparse operators (the analogue of the Julia shim's GB300CSR).

A ``GB300Operator`` owns a libkpmgb handle: the matrix is uploaded once, in
row-major CSR, and reused by every moment call, where the reference uploads
and converts it on every call (``src/moment.jl:432``).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse as sp

from . import _native


class GB300Operator:
    """A square sparse operator resident on the current CUDA device."""

    def __init__(self, M):
        if isinstance(M, GB300Operator):
            raise TypeError("already a GB300Operator")
        M = sp.csc_matrix(M, dtype=np.complex128)
        if M.shape[0] != M.shape[1]:
            raise _native.KPMArgumentError(f"operator must be square (got {M.shape})")
        M.sort_indices()
        lib = _native.load()
        colptr = np.ascontiguousarray(M.indptr, dtype=np.int64)
        rowval = np.ascontiguousarray(M.indices, dtype=np.int64)
        nzval = np.ascontiguousarray(M.data, dtype=np.complex128)
        h = C.c_void_p()
        rc = lib.kpmgb_operator_create(
            M.shape[0], M.nnz, colptr.ctypes.data, rowval.ctypes.data,
            nzval.ctypes.data if M.nnz else None, 0, C.byref(h))
        _native.check(rc)
        self._h = h
        self._lib = lib
        self.shape = M.shape
        # CSC pattern in the order the device operator was built from; the
        # gradient entry point returns values in this order.
        self.indptr = colptr
        self.indices = rowval
        self.nnz = int(M.nnz)
        n, nnz, real = C.c_int64(), C.c_int64(), C.c_int32()
        _native.check(lib.kpmgb_operator_info(h, C.byref(n), C.byref(nnz), C.byref(real)))
        self.is_real = bool(real.value)

    @property
    def handle(self):
        return self._h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.kpmgb_operator_destroy(h)
            self._h = None

    def __repr__(self):
        return f"GB300Operator(n={self.shape[0]}, nnz={self.nnz}, real={self.is_real})"


def as_operator(M) -> GB300Operator:
    return M if isinstance(M, GB300Operator) else GB300Operator(M)
