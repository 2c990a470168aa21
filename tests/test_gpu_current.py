"""kpm_1d_current (src/moment.jl:558-714) on the GPU: traces against dense
Chebyshev matrices (test/optical_cond_test.jl:278-335) and probe moments
against the oracle for a non-Hermitian J (test/kpm2d_blocking_test.jl:264-268)."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import relerr
import kpm_gb300 as kg
from kpm_gb300 import models
from oracle import kpm_oracle as ko

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def _haldane_jxx():
    H, Jx, _, _ = models.haldane(3, 3, t=1.0, t2=0.2)
    Hm, Jm = H.toarray(), Jx.toarray()
    dx = np.where(np.abs(Hm) > 0, Jm / np.where(Hm == 0, 1, Hm), 0)
    Jxx = sp.csc_matrix(Hm * dx ** 2)
    a, b, Hn = ko.normalizeH(H, center=True)
    return Hn, Jxx


@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_current_trace_vs_dense(prec):
    Hn, Jxx = _haldane_jxx()
    D, NC = Hn.shape[0], 16
    T = ko.chebyshev_matrices(Hn.toarray(), NC)
    ref = np.array([np.trace(Jxx.toarray() @ T[n]) / D for n in range(NC)])
    psi = np.eye(D, dtype=complex)
    mu = kg.kpm_1d_current(Hn, Jxx, NC, D, D, psi_in=psi, precision=prec)
    tol = 1e-12 if prec == "fp64" else 1e-9
    assert relerr(mu, ref) < tol
    if prec == "fp64":
        assert np.abs(mu.imag).max() < 1e-14
        ser = kg.kpm_1d_current(Hn, Jxx, NC, D, D, psi_in=psi, NR_parallel=False)
        assert relerr(ser, mu) < 1e-12
        allm = kg.kpm_1d_current(Hn, Jxx, NC, D, D, psi_in=psi, avg_output=False)
        assert allm.shape == (D, NC)
        assert relerr(allm.sum(axis=0) / D, mu) < 1e-12


def test_current_force_norm():
    Hn, Jxx = _haldane_jxx()
    D = Hn.shape[0]
    rng = np.random.default_rng(4242)
    psi_u = ko.random_phase_vectors(rng, D, 4) * np.array([1.0, 3.0, 0.25, 7.0])
    forced = kg.kpm_1d_current(Hn, Jxx, 16, 4, D, psi_in=psi_u.copy(), force_norm=True)
    pre = psi_u.copy()
    kg.normalize_by_col(pre)
    assert relerr(forced, kg.kpm_1d_current(Hn, Jxx, 16, 4, D, psi_in=pre)) < 1e-12


def test_current_antihermitian_ring():
    N, phi = 12, 0.35
    H = np.zeros((N, N), dtype=complex)
    disp = np.zeros((N, N))
    for i in range(N):
        j = (i + 1) % N
        H[j, i] = -np.exp(1j * phi / N)
        H[i, j] = np.conj(H[j, i])
        disp[j, i], disp[i, j] = 1.0, -1.0
    J = sp.csc_matrix(H * disp)
    assert np.abs((J + J.conj().T).toarray()).max() == 0
    a = 2 * np.abs(np.linalg.eigvalsh(H)).max() / (2 - 0.1)
    Hn = sp.csc_matrix(H / a)
    NC = 12
    T = ko.chebyshev_matrices(Hn.toarray(), NC)
    tr_J = np.array([np.trace(J.toarray() @ T[n]) / N for n in range(NC)])
    assert np.abs(tr_J).max() > 0.1   # the loop around the ring closes at n = N - 1
    mu = kg.kpm_1d_current(Hn, J, NC, N, N, psi_in=np.eye(N, dtype=complex))
    assert np.abs(mu - tr_J).max() <= 1e-12 * np.abs(tr_J).max() + 1e-14
    assert np.abs(mu.real).max() < 1e-14


def test_current_nonhermitian_j_probes():
    rng = np.random.default_rng(6)
    H = models.square_anderson(10, W=1.0, rng=rng)
    Hn = (H / 4.6).tocsc()
    J = sp.random(100, 100, density=0.05, random_state=3, dtype=float) \
        + 1j * sp.random(100, 100, density=0.05, random_state=4, dtype=float)
    psi = ko.random_phase_vectors(rng, 100, 6)
    ref = ko.kpm_1d_current(Hn, J, 40, psi)
    got = kg.kpm_1d_current(Hn, sp.csc_matrix(J), 40, 6, psi_in=psi, avg_output=False)
    assert relerr(got, ref) < 1e-12


def test_current_separate_bra_unimplemented():
    Hn, Jxx = _haldane_jxx()
    D = Hn.shape[0]
    p = np.ones((D, 1), dtype=complex)
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d_current(Hn, Jxx, 16, 1, D, psi_in_l=p, psi_in_r=p)
