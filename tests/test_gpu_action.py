"""chebyshev_action (src/utils/chebyshev_action.jl:47-122) on the GPU against
the oracle's direct recurrence (atol 1e-12, as test/chebyshev_action_test.jl)
and spectral sums from exact diagonalisation (1e-8)."""
import numpy as np
import pytest
import scipy.sparse as sp

import kpm_gb300 as kg
from kpm_gb300 import models
from oracle import kpm_oracle as ko

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def _prescaled(rng, n, margin=0.95):
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    Hd = (A + A.conj().T) / 2
    Hd /= np.abs(np.linalg.eigvalsh(Hd)).max() / margin
    return Hd, sp.csc_matrix(Hd)


def _crandn(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def test_action_matches_recurrence_and_ed():
    rng = np.random.default_rng(151)
    NH, NC, NR, K = 48, 16, 2, 3
    Hd, Hs = _prescaled(rng, NH)
    V = _crandn(rng, NH, NR)
    C = _crandn(rng, NC, K)
    ref = ko.chebyshev_action(Hs, V, C)
    got = kg.chebyshev_action(Hs, V, C)
    assert np.abs(got - ref).max() <= 1e-12
    lam, U = np.linalg.eigh(Hd)
    th = np.arccos(np.clip(lam, -1, 1))
    for k in range(K):
        f = np.array([np.sum(C[:, k] * np.cos(np.arange(NC) * t)) for t in th])
        assert np.abs(got[:, :, k] - U @ (f[:, None] * (U.conj().T @ V))).max() <= 1e-8


def test_action_promotion_and_vector_forms():
    rng = np.random.default_rng(157)
    NH, NC, NR = 40, 12, 2
    Hd, Hs = _prescaled(rng, NH)
    Vc, Vr = _crandn(rng, NH, NR), rng.standard_normal((NH, NR))
    Cr, Cc = rng.standard_normal(NC), _crandn(rng, NC)
    assert np.abs(kg.chebyshev_action(Hs, Vc, Cr)
                  - ko.chebyshev_action(Hs, Vc, Cr[:, None])[:, :, 0]).max() <= 1e-12
    assert np.abs(kg.chebyshev_action(Hs, Vr, Cc)
                  - ko.chebyshev_action(Hs, Vr, Cc[:, None])[:, :, 0]).max() <= 1e-12
    Hr = np.real(Hd)
    Hr /= np.abs(np.linalg.eigvalsh(Hr)).max() / 0.95
    assert np.abs(kg.chebyshev_action(sp.csc_matrix(Hr), Vr, Cc)
                  - ko.chebyshev_action(Hr, Vr, Cc[:, None])[:, :, 0]).max() <= 1e-12
    C = _crandn(rng, NC, 2)
    full = kg.chebyshev_action(Hs, Vc, C)
    assert np.abs(kg.chebyshev_action(Hs, Vc, C[:, 0]) - full[:, :, 0]).max() <= 1e-14
    assert np.abs(kg.chebyshev_action(Hs, Vc[:, 0], C) - full[:, 0, :]).max() <= 1e-14
    assert np.abs(kg.chebyshev_action(Hs, Vc[:, 0], C[:, 0]) - full[:, 0, 0]).max() <= 1e-14
    out = np.zeros((NH, NR, 2), dtype=complex)
    kg.chebyshev_action_bang(out, Hs, Vc, C)
    assert np.array_equal(out, full)


@pytest.mark.parametrize("NC,K", [(1, 1), (2, 3), (40, 6), (33, 9), (200, 10), (70, 13)])
def test_action_large_sparse(NC, K):
    """chunk boundaries (32 vectors) and output passes (1, 2, 4 or 8 outputs
    wide, the last one padded) at odd sizes"""
    rng = np.random.default_rng(NC + K)
    H = models.square_anderson(40, W=1.5, rng=rng)
    H = (H / 4.9).tocsc()
    V = ko.random_phase_vectors(rng, 1600, 5)
    C = _crandn(rng, NC, K) / np.sqrt(NC)
    ref = ko.chebyshev_action(H, V, C)
    got = kg.chebyshev_action(H, V, C)
    assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


def test_action_growth_guard():
    rng = np.random.default_rng(4)
    H = (models.square_anderson(12, W=0.0, rng=rng) / 3.0).tocsc()   # spectrum to +-4/3
    V = ko.random_phase_vectors(rng, 144, 2)
    C = np.ones((40, 1))
    with pytest.raises(kg.KPMNumericalError):
        kg.chebyshev_action(H, V, C, check_every=16)
    out = kg.chebyshev_action(H, V, C, check_every=0)
    assert np.all(np.isfinite(out))
    ok = (models.square_anderson(12, W=0.0, rng=rng) / 4.4).tocsc()
    kg.chebyshev_action(ok, V, C, check_every=1)


def test_action_argument_errors():
    H = (models.ring(16) / 2.2).tocsc()
    V = np.ones((16, 2), dtype=complex)
    with pytest.raises(kg.KPMArgumentError):
        kg.chebyshev_action(H, V, np.zeros((0, 1)))
    with pytest.raises(kg.KPMArgumentError):
        kg.chebyshev_action(H, V, np.zeros((4, 0)))
    with pytest.raises(kg.KPMArgumentError):
        kg.chebyshev_action(H, np.ones((15, 2)), np.ones(4))
    with pytest.raises(kg.KPMArgumentError):
        kg.chebyshev_action(H, V, np.ones(4), check_every=-1)
    with pytest.raises(kg.KPMArgumentError):
        kg.chebyshev_action_bang(np.zeros((16, 2, 2), dtype=complex), H, V, np.ones((4, 3)))
