"""Host CSC -> CSR conversion of kpmgb_operator_create (kpmgb_csr_host.h),
compiled with g++ into a small driver: against SciPy's transpose for random
operators, 0- and 1-based, with 1, 3 and 8 threads (identical output), and
the argument errors (row index out of range, non-monotone colptr)."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("csr") / "csr_driver"
    subprocess.run(["g++", "-std=c++17", "-O2", "-pthread",
                    f"-I{ROOT / 'kpm.jl_gb300' / 'csrc'}",
                    str(ROOT / "tests" / "csr_host_driver.cpp"), "-o", str(exe)], check=True)
    return exe


def _run(driver, tmp_path, n, colptr, rowval, nzval, base, threads):
    src, dst = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(src, "wb") as f:
        np.array([n, len(rowval), base], dtype=np.int64).tofile(f)
        np.asarray(colptr, dtype=np.int64).tofile(f)
        np.asarray(rowval, dtype=np.int64).tofile(f)
        np.ascontiguousarray(nzval, dtype=np.complex128).view(np.float64).tofile(f)
    subprocess.run([str(driver), str(src), str(dst), str(threads)], check=True)
    raw = dst.read_bytes()
    status = int(np.frombuffer(raw[:8], dtype=np.int64)[0])
    if status:
        return raw[8:].decode()
    nnz = len(rowval)
    o = 8
    is_real, max_row = np.frombuffer(raw[o:o + 16], dtype=np.int64); o += 16
    rmax = float(np.frombuffer(raw[o:o + 8], dtype=np.float64)[0]); o += 8
    rowptr = np.frombuffer(raw[o:o + 4 * (n + 1)], dtype=np.int32); o += 4 * (n + 1)
    col = np.frombuffer(raw[o:o + 4 * nnz], dtype=np.int32); o += 4 * nnz
    perm = np.frombuffer(raw[o:o + 4 * nnz], dtype=np.int32); o += 4 * nnz
    val = np.frombuffer(raw[o:o + 16 * nnz], dtype=np.complex128)
    return dict(is_real=int(is_real), max_row=int(max_row), rmax=rmax, rowptr=rowptr, col=col,
                perm=perm, val=val)


@pytest.mark.parametrize("n,density,complex_v", [(1, 1.0, False), (57, 0.08, True),
                                                 (700, 0.01, False), (3001, 0.002, True)])
@pytest.mark.parametrize("base", [0, 1])
def test_matches_scipy_transpose(driver, tmp_path, n, density, complex_v, base):
    rng = np.random.default_rng(n + base)
    A = sp.random(n, n, density=density, format="csc", random_state=rng,
                  data_rvs=lambda k: rng.standard_normal(k)).astype(np.complex128)
    if complex_v:
        A.data = A.data + 1j * rng.standard_normal(A.nnz)
    A.sort_indices()
    pos = sp.csc_matrix((np.arange(A.nnz, dtype=np.float64) + 1, A.indices, A.indptr), shape=A.shape)
    R, P = A.tocsr(), pos.tocsr()
    R.sort_indices()
    P.sort_indices()
    outs = [_run(driver, tmp_path, n, A.indptr + base, A.indices + base, A.data, base, t)
            for t in (1, 3, 8)]
    for out in outs:
        assert np.array_equal(out["rowptr"], R.indptr)
        assert np.array_equal(out["col"], R.indices)
        assert np.array_equal(out["val"], R.data)
        assert np.array_equal(out["perm"], P.data.astype(np.int64) - 1)
        assert out["is_real"] == int(not complex_v or A.nnz == 0)
        assert out["max_row"] == (int(np.diff(R.indptr).max()) if n else 0)
        rs = np.zeros(n)
        np.add.at(rs, np.repeat(np.arange(n), np.diff(R.indptr)), np.abs(R.data.real) + np.abs(R.data.imag))
        assert out["rmax"] == pytest.approx(rs.max(), rel=1e-14)
    for out in outs[1:]:
        for k in ("rowptr", "col", "perm", "val"):
            assert np.array_equal(out[k], outs[0][k])


@pytest.mark.parametrize("threads", [1, 4])
def test_argument_errors(driver, tmp_path, threads):
    colptr = np.array([0, 2, 3, 5])
    rows = np.array([0, 2, 1, 0, 3])          # row 3 of a 3 x 3 operator
    assert _run(driver, tmp_path, 3, colptr, rows, np.ones(5), 0, threads) == \
        "row index out of range"
    assert _run(driver, tmp_path, 3, np.array([0, 3, 2, 5]), np.array([0, 1, 2, 0, 1]),
                np.ones(5), 0, threads) == "colptr is not monotone"
