"""C-ABI checks that need no GPU: the library builds, loads, exports every
symbol declared in include/kpmgb.h, and rejects bad arguments before any
device work."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest
import scipy.sparse as sp

ROOT = Path(__file__).resolve().parent.parent


def _declared_symbols():
    text = (ROOT / "include" / "kpmgb.h").read_text()
    return sorted(set(re.findall(r"\b(kpmgb_[a-z0-9_]+)\s*\(", text)))


def test_header_and_binding_agree():
    from kpm_gb300 import _native
    assert set(_declared_symbols()) == set(_native.EXPORTED_SYMBOLS)


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(str(built_lib))
    missing = [s for s in _declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_version_and_error_without_gpu(built_lib):
    from kpm_gb300 import _native
    lib = _native.load()
    assert lib.kpmgb_version().decode().startswith("kpmgb")
    # a null operator is rejected with an argument error, no device work
    rc = lib.kpmgb_kpm1d(None, 4, 1, 4, None, None, None)
    assert rc == _native.ERR_ARGUMENT
    assert lib.kpmgb_last_error().decode()


def test_csc_validation_before_upload(built_lib):
    from kpm_gb300 import _native
    lib = _native.load()
    h = C.c_void_p()
    colptr = np.array([0, 1, 3], dtype=np.int64)   # claims 3 entries
    rowval = np.array([0, 1], dtype=np.int64)
    nz = np.ones(2, dtype=np.complex128)
    rc = lib.kpmgb_operator_create(2, 2, colptr.ctypes.data, rowval.ctypes.data,
                                   nz.ctypes.data, 0, C.byref(h))
    assert rc == _native.ERR_ARGUMENT
    colptr = np.array([0, 1, 2], dtype=np.int64)
    rowval = np.array([0, 5], dtype=np.int64)      # row out of range
    rc = lib.kpmgb_operator_create(2, 2, colptr.ctypes.data, rowval.ctypes.data,
                                   nz.ctypes.data, 0, C.byref(h))
    assert rc == _native.ERR_ARGUMENT
    assert "range" in lib.kpmgb_last_error().decode()


def test_python_argument_validation(built_lib):
    """Front-end checks mirror the reference's ArgumentErrors (src/frontend.jl:225-327)."""
    import kpm_gb300 as kg
    H = sp.identity(8, dtype=complex, format="csc") * 0.5
    h = kg.RescaledHamiltonian(H, 1.0, 0.0)
    with pytest.raises(kg.KPMArgumentError):
        kg.dos_moments(h, NC=63)
    with pytest.raises(kg.KPMArgumentError):
        kg.dos_moments(h, NC=64, rng=np.random.default_rng(1), psi_in=np.zeros((8, 2)))
    with pytest.raises(kg.KPMArgumentError):
        kg.dos_moments(h, NC=64, psi_in=np.zeros((7, 2)))
    with pytest.raises(kg.KPMArgumentError):
        kg.cond_moments(h, H, H, NC=32, psi_in=np.zeros((7, 2)))
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d(H, 8, 2, psi_in=np.zeros((8, 2)), psi_in_l=np.zeros((8, 2)))
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d(H, 8, 2, psi_in_l=np.zeros((8, 2)))
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_2d(H, H, H, 8, 2, 8, psi_in=np.zeros((8, 2)), moment_parity="BOTH")
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_2d(H, H, H, 8, 2, 8, psi_in=np.zeros((8, 2)), arr_size=1)
    with pytest.raises(kg.KPMArgumentError):
        kg.ConductivityMoments(np.zeros((3, 2), dtype=complex), 1.0, 0.0, 8, 1)


def test_blocking_rule_matches_reference_arithmetic():
    """src/moment.jl:759-810 as pinned by test/kpm2d_blocking_test.jl:119-152."""
    import kpm_gb300 as kg
    NH, NR, NC = 40, 3, 50
    one = NH * NR * 16
    c = kg.kpm_2d_blocking(NH, NR, NC, workspace_bytes=30 * one, right_block=4)
    assert c == dict(arr_size=18, right_block=4, bytes=11 * one + 18 * (one + 64))
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_2d_blocking(NH, NR, NC, workspace_bytes=10 * one - 1)
    c = kg.kpm_2d_blocking(NH, NR, NC, workspace_bytes=10 * one, arr_size=27, right_block=9)
    assert (c["arr_size"], c["right_block"]) == (27, 9)


def test_derivative_host_checks_and_tangent_scale(built_lib):
    """The forward-mode derivatives validate shapes and probes on the host
    before any device work; the tangent scale is an exact power of two near
    sqrt(NC) |dH|_inf (or |dJ| / |J|)."""
    import math
    import kpm_gb300 as kg
    from kpm_gb300 import moment
    H = sp.identity(8, dtype=complex, format="csc") * 0.5
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d_derivative(H, H[:4, :4], 8, 1, psi_in=np.ones((8, 1)))
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d_derivative(H, H, 8, 2, psi_in=np.ones((8, 1)))
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_2d_derivative(H, H, H, None, H, None, 8, 1, 8)
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_2d_derivative(H, H, H, None, H[:4, :4], None, 8, 1, 8, psi_in=np.ones((8, 1)))
    dH = sp.csr_matrix(H * 3.0)          # |dH|_inf = 1.5
    s = moment._tangent_scale(256, dH)   # sqrt(256) * 1.5 = 24 -> 2^-5
    assert s == math.ldexp(1.0, -5)
    J = sp.csr_matrix(H)
    s = moment._tangent_scale(4, dH * 0.0, ((J, J * 64.0),))   # |dJ| / |J| = 64
    assert s == math.ldexp(1.0, -6)
    assert moment._tangent_scale(16, sp.csr_matrix((8, 8))) == 1.0


def test_blocking_rule_agrees_with_oracle_everywhere():
    """The host blocking rule (kpm_gb300.kpm_2d_blocking) and the oracle's
    restatement of src/moment.jl:759-810 agree on random sizes, budgets and
    explicit block sizes, including which inputs are rejected."""
    import kpm_gb300 as kg
    from oracle import kpm_oracle as ko
    rng = np.random.default_rng(2024)
    for _ in range(3000):
        NH = int(rng.integers(1, 5000))
        NR = int(rng.integers(1, 64))
        NC = int(rng.integers(2, 600))
        one = NH * NR * 16
        budget = int(rng.integers(0, 60) * one + rng.integers(0, one))
        arr = "auto" if rng.random() < 0.5 else int(rng.integers(0, 40))
        rb = "auto" if rng.random() < 0.5 else int(rng.integers(1, 40))
        try:
            ref = ko.kpm_2d_blocking(NH, NR, NC, budget, arr_size=arr, right_block=rb)
        except ValueError:
            ref = None
        try:
            got = kg.kpm_2d_blocking(NH, NR, NC, workspace_bytes=budget, arr_size=arr,
                                     right_block=rb)
        except kg.KPMArgumentError:
            got = None
        if ref is None:
            assert got is None, (NH, NR, NC, budget, arr, rb, got)
        else:
            assert got is not None, (NH, NR, NC, budget, arr, rb)
            assert (got["arr_size"], got["right_block"], got["bytes"]) == ref, \
                (NH, NR, NC, budget, arr, rb, got, ref)


def test_dos_basis_and_jackson_match_oracle():
    """The host-side DOS map used for gradient losses (frontend.dos_basis) is
    the reconstruction of src/applications/dos.jl:76-161 as a matrix: Phi @ mu
    equals the oracle's rho on the same grid (points outside |E - b| < a
    give 0), and the Jackson factors match."""
    import kpm_gb300 as kg
    from oracle import kpm_oracle as ko
    rng = np.random.default_rng(8)
    for NC in (1, 2, 17, 128):
        n = np.arange(NC)
        assert np.allclose(kg.jackson_kernel(n, NC), ko.jackson_kernel(n, NC), rtol=0, atol=1e-15)
        mu = rng.standard_normal(NC)
        a, b = 1.7, -0.3
        E = np.linspace(b - 1.2 * a, b + 1.2 * a, 301)
        _, rho = ko.dos(mu, a, b=b, E_grid=E)
        got = kg.dos_basis(NC, a, b, E) @ mu
        assert np.abs(got - rho).max() <= 1e-12 * max(1.0, np.abs(rho).max())
