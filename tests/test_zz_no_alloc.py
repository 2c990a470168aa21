"""kpmgb_kpm1d_noalloc: the kpm_1d entry point for callers that cannot let the
library allocate device memory (it keeps its scratch in a static device
array).  Called through the C ABI with caller-owned device buffers, twice in
a row, and checked against kpmgb_kpm1d on the same inputs."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import relerr

pytestmark = pytest.mark.gpu


def test_noalloc_matches_kpm1d_twice(built_lib):
    import torch
    import kpm_gb300 as kg
    from kpm_gb300 import _native, models

    lib = _native.load()
    rng = np.random.default_rng(77)
    H = models.square_anderson(24, W=2.0, rng=rng)            # NH = 576
    Hn = sp.csr_matrix(H / 4.5, dtype=np.complex128)
    Hn.sort_indices()
    NH, NR, NC = Hn.shape[0], 12, 256
    psi = kg.random_phase_vectors(rng, NH, NR)
    ref = kg.kpm_1d(sp.csc_matrix(Hn), NC, NR, psi_in=psi, avg_output=False)

    dev = torch.device("cuda")
    rowptr = torch.from_numpy(Hn.indptr.astype(np.int32)).to(dev)
    col = torch.from_numpy(Hn.indices.astype(np.int32)).to(dev)
    val = torch.from_numpy(Hn.data.astype(np.complex128)).to(dev)
    psi_t = torch.from_numpy(np.ascontiguousarray(psi.T)).to(dev)   # column-major NH x NR
    stream = torch.cuda.Stream()
    for _ in range(2):
        mu_t = torch.full((NC, NR), float("nan"), dtype=torch.complex128, device=dev)
        # the uploads and the NaN fill run on torch's current stream; the
        # entry point works on `stream` (non-blocking), so order it after them
        stream.wait_stream(torch.cuda.current_stream())
        rc = lib.kpmgb_kpm1d_noalloc(NH, C.c_void_p(rowptr.data_ptr()), C.c_void_p(col.data_ptr()),
                                     C.c_void_p(val.data_ptr()), NC, NR,
                                     C.c_void_p(psi_t.data_ptr()), C.c_void_p(mu_t.data_ptr()),
                                     C.c_void_p(stream.cuda_stream))
        _native.check(rc)
        got = mu_t.cpu().numpy().T          # (NR, NC)
        assert relerr(got, ref) < 1e-12

    # sizes beyond the static scratch are rejected with an argument error
    rc = lib.kpmgb_kpm1d_noalloc(1 << 22, C.c_void_p(rowptr.data_ptr()), C.c_void_p(col.data_ptr()),
                                 C.c_void_p(val.data_ptr()), NC, 64, C.c_void_p(psi_t.data_ptr()),
                                 C.c_void_p(mu_t.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert rc == _native.ERR_ARGUMENT
    assert "static" in lib.kpmgb_last_error().decode()

    # host memory and misaligned device pointers are rejected before any work
    host_mu = np.zeros((NC, NR), dtype=np.complex128)
    rc = lib.kpmgb_kpm1d_noalloc(NH, C.c_void_p(rowptr.data_ptr()), C.c_void_p(col.data_ptr()),
                                 C.c_void_p(val.data_ptr()), NC, NR, C.c_void_p(psi_t.data_ptr()),
                                 C.c_void_p(host_mu.ctypes.data), C.c_void_p(stream.cuda_stream))
    assert rc == _native.ERR_ARGUMENT
    rc = lib.kpmgb_kpm1d_noalloc(NH, C.c_void_p(rowptr.data_ptr()), C.c_void_p(col.data_ptr()),
                                 C.c_void_p(val.data_ptr() + 8), NC, NR,
                                 C.c_void_p(psi_t.data_ptr()), C.c_void_p(mu_t.data_ptr()),
                                 C.c_void_p(stream.cuda_stream))
    assert rc == _native.ERR_ARGUMENT and "aligned" in lib.kpmgb_last_error().decode()
