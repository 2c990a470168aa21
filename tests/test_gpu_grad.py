"""Adjoint gradient of a loss on kpm_1d moments (kpmgb_kpm1d_grad).

Checked against central finite differences of the oracle's doubling moments
entry by entry on a small complex model, and against directional finite
differences of the GPU FP64 forward path on larger ones, including the
DOS-window loss int (rho - rho_t)^2 dE built from dos_basis.
"""
import numpy as np
import pytest

import kpm_gb300 as kg
from kpm_gb300 import models
from oracle import kpm_oracle as ko

pytestmark = pytest.mark.gpu


def _oracle_loss(H, NC, psi, g):
    mu = ko.kpm_1d_doubling(H, NC, psi)
    return float((mu.real.sum(axis=0) / psi.shape[1]) @ g)


def _gpu_loss(H, NC, psi, g):
    return float(kg.kpm_1d(H, NC, psi.shape[1], psi_in=psi.copy()) @ g)


def _hermitian_direction(rng, H):
    """Random Hermitian perturbation on H's (symmetric) pattern."""
    D = H.copy().tocoo()
    vals = rng.standard_normal(D.nnz) + 1j * rng.standard_normal(D.nnz)
    D.data = vals
    D = D.tocsc()
    D = (D + D.conj().T) / 2
    D = D.tocsc()
    D.sort_indices()
    return D


def _pairing(G, D):
    """dL along D = sum_k Re(conj(G_k) D_k) over stored entries."""
    Gd = G.toarray()
    Dd = D.toarray()
    return float(np.sum(Gd.real * Dd.real + Gd.imag * Dd.imag))


def test_grad_matches_oracle_finite_differences(built_lib):
    rng = np.random.default_rng(11)
    H, _, _, _ = models.haldane(2, 3, t2=0.2, m=0.15)
    H = (H / 3.6).tocsc()
    H.sort_indices()
    NC, NR = 24, 3
    psi = ko.random_phase_vectors(rng, H.shape[0], NR)
    g = rng.standard_normal(NC)
    G = kg.kpm_1d_grad(H, NC, psi, g, checkpoint_every=5)
    eps = 1e-6
    fd = H.copy()
    fd.data = np.zeros(H.nnz, dtype=np.complex128)
    for k in range(H.nnz):
        for unit in (1.0, 1j):
            Hp = H.copy()
            Hp.data[k] += eps * unit
            Hm = H.copy()
            Hm.data[k] -= eps * unit
            d = (_oracle_loss(Hp, NC, psi, g) - _oracle_loss(Hm, NC, psi, g)) / (2 * eps)
            fd.data[k] += d * unit
    ref = fd.toarray()
    got = G.toarray()
    # central differences at eps=1e-6: truncation ~1e-12, cancellation ~1e-10
    assert np.abs(got - ref).max() <= 1e-7 * np.abs(ref).max()


@pytest.mark.parametrize("C", [0, 1, 7, 64, 1000])
def test_grad_independent_of_checkpoint_spacing(built_lib, C):
    rng = np.random.default_rng(5)
    H = models.square_anderson(12, W=2.0, rng=rng)
    H = (H / 5.1).tocsc()
    NC, NR = 96, 4
    psi = ko.random_phase_vectors(rng, H.shape[0], NR)
    g = rng.standard_normal(NC)
    ref = kg.kpm_1d_grad(H, NC, psi, g, checkpoint_every=48).toarray()
    got = kg.kpm_1d_grad(H, NC, psi, g, checkpoint_every=C).toarray()
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()


def test_grad_directional_graphene(built_lib):
    rng = np.random.default_rng(21)
    H = models.graphene(16, 16, onsite=0.1 * rng.standard_normal(512))
    H = (H / 3.4).tocsc()
    NC, NR = 256, 8
    psi = ko.random_phase_vectors(rng, H.shape[0], NR)
    g = rng.standard_normal(NC) / np.sqrt(NC)
    G = kg.kpm_1d_grad(H, NC, psi, g, checkpoint_every=64)
    D = _hermitian_direction(rng, H)
    eps = 1e-5
    fd = (_gpu_loss(H + eps * D, NC, psi, g) - _gpu_loss(H - eps * D, NC, psi, g)) / (2 * eps)
    assert abs(_pairing(G, D) - fd) <= 1e-6 * max(abs(fd), 1e-3)


def test_grad_dos_window_loss(built_lib):
    """L = int_{-0.5}^{0.5} (rho - rho_t)^2 dE on graphene with random onsite
    energies; rho_t from a second disorder seed."""
    rng = np.random.default_rng(3)
    Lc = 12
    NH = 2 * Lc * Lc
    a, b = 3.4, 0.0
    H = (models.graphene(Lc, Lc, onsite=0.1 * rng.standard_normal(NH)) / a).tocsc()
    Ht = (models.graphene(Lc, Lc, onsite=0.1 * rng.standard_normal(NH)) / a).tocsc()
    NC, NR = 128, 6
    psi = ko.random_phase_vectors(rng, NH, NR)
    E = np.linspace(-0.5, 0.5, 201)
    w = np.full(E.size, E[1] - E[0])
    w[[0, -1]] /= 2
    Phi = kg.dos_basis(NC, a, b, E)
    rho_t = Phi @ kg.kpm_1d(Ht, NC, NR, psi_in=psi.copy())

    def loss(Hx):
        rho = Phi @ kg.kpm_1d(Hx, NC, NR, psi_in=psi.copy())
        return float(w @ (rho - rho_t) ** 2), rho

    L0, rho = loss(H)
    g = Phi.T @ (2 * w * (rho - rho_t))
    G = kg.kpm_1d_grad(H, NC, psi, g)
    D = _hermitian_direction(rng, H)
    eps = 1e-5
    fd = (loss(H + eps * D)[0] - loss(H - eps * D)[0]) / (2 * eps)
    assert L0 > 0
    assert abs(_pairing(G, D) - fd) <= 1e-5 * abs(fd) + 1e-12


def test_grad_argument_errors(built_lib):
    H = (models.ring(16) / 2.2).tocsc()
    psi = np.ones((16, 2), dtype=np.complex128)
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d_grad(H, 15, psi, np.zeros(15))
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d_grad(H, 16, psi, np.zeros(12))


def test_grad_column_batches():
    """NR = 40 runs as batches of 32 + 8 columns; the gradient is the
    probe-count-weighted sum of the per-batch gradients."""
    rng = np.random.default_rng(12)
    H = (models.square_anderson(10, W=2.0, rng=rng) / 5.1).tocsc()
    psi = ko.random_phase_vectors(rng, 100, 40)
    g = rng.standard_normal(48)
    full = kg.kpm_1d_grad(H, 48, psi, g).toarray()
    a = kg.kpm_1d_grad(H, 48, psi[:, :32], g).toarray()
    b = kg.kpm_1d_grad(H, 48, psi[:, 32:], g).toarray()
    ref = (32 * a + 8 * b) / 40
    assert np.abs(full - ref).max() <= 1e-13 * np.abs(ref).max()
