"""GPU directional derivatives of the moments (forward mode through the
block-triangular embedding) against the oracle's explicit product-rule
tangent recurrences.  FP64: 1e-12 norm-wise relative; float-float recurrence
and split contraction: 1e-9.  Also checked: consistency with the adjoint
gradient, and dsigma_xy/dt2 of the Haldane model against central differences
of the oracle's conductivity."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import relerr
from helpers import rand_herm
import kpm_gb300 as kg
from kpm_gb300 import models
from oracle import kpm_oracle as ko

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return built_lib


def _herm_on_pattern(rng, H, scale=0.1):
    """A Hermitian perturbation with H's sparsity pattern."""
    P = sp.csr_matrix(H, dtype=np.complex128).copy()
    P.data = rng.standard_normal(P.nnz) + 1j * rng.standard_normal(P.nnz)
    return ((P + P.conj().T) * (scale / 2)).tocsc()


def _haldane_direction(L, t2=0.2):
    (H, Jx, Jy, area), (H0, Jx0, Jy0, _), (H1, Jx1, Jy1, _) = (
        models.haldane(L, L, t2=t2), models.haldane(L, L, t2=0.0), models.haldane(L, L, t2=1.0))
    return H, Jx, Jy, area, H1 - H0, Jx1 - Jx0, Jy1 - Jy0


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("ff", 1e-9)])
def test_kpm1d_derivative_matches_oracle(prec, tol):
    rng = np.random.default_rng(21)
    H = (models.square_anderson(12, W=2.0, rng=rng) / 5.1).tocsc()
    dH = _herm_on_pattern(rng, H)
    psi = ko.random_phase_vectors(rng, 144, 5)
    got = kg.kpm_1d_derivative(H, dH, 64, 5, psi_in=psi, avg_output=False, precision=prec)
    ref = ko.kpm_1d_tangent(H, dH, 64, psi)
    assert relerr(got, ref) < tol
    avg = kg.kpm_1d_derivative(H, dH, 64, 5, psi_in=psi, precision=prec)
    assert relerr(avg, ref.sum(axis=0).real / 5) < tol


@pytest.mark.parametrize("prec,contraction,tol",
                         [("fp64", "fp64", 1e-12), ("ff", "fp64", 1e-9), ("fp64", "split", 1e-9)])
def test_kpm2d_derivative_matches_oracle(prec, contraction, tol):
    rng = np.random.default_rng(22)
    H, Jx, Jy, _, dH, dJx, dJy = _haldane_direction(5)
    a = 3.8
    NH, NR, NC = H.shape[0], 4, 40
    psl = ko.random_phase_vectors(rng, NH, NR)
    psr = ko.random_phase_vectors(rng, NH, NR)
    ref = ko.kpm_2d_tangent(H / a, dH / a, Jx, dJx, Jy, dJy, NC, psl, psr)
    got = kg.kpm_2d_derivative(H / a, dH / a, Jx, dJx, Jy, dJy, NC, NR, NH, psi_in_l=psl,
                               psi_in_r=psr, precision=prec, contraction=contraction)
    assert relerr(got, ref) < tol


def test_kpm2d_derivative_blocking_parity_and_fixed_currents():
    rng = np.random.default_rng(23)
    H, Jx, Jy, _, dH, dJx, dJy = _haldane_direction(4)
    NH, NR, NC = H.shape[0], 3, 30
    psi = ko.random_phase_vectors(rng, NH, NR)
    ref = ko.kpm_2d_tangent(H / 3.8, dH / 3.8, Jx, None, Jy, None, NC, psi, psi)
    # several left blocks and right blocks
    got = kg.kpm_2d_derivative(H / 3.8, dH / 3.8, Jx, None, Jy, None, NC, NR, NH, psi_in=psi,
                               arr_size=7, right_block=4)
    assert relerr(got, ref) < 1e-12
    n = np.arange(NC)
    odd = ((n[:, None] + n[None, :]) % 2 == 1)
    got = kg.kpm_2d_derivative(H / 3.8, dH / 3.8, Jx, None, Jy, None, NC, NR, NH, psi_in=psi,
                               moment_parity="ODD")
    assert relerr(got, np.where(odd, ref, 0)) < 1e-12


def test_derivative_consistent_with_adjoint_gradient():
    """sum_m g_m dmu_m (forward mode) = Re <grad, dH> (reverse mode)."""
    rng = np.random.default_rng(24)
    H = (models.square_anderson(10, W=3.0, rng=rng) / 5.6).tocsc()
    dH = _herm_on_pattern(rng, H)
    psi = ko.random_phase_vectors(rng, 100, 4)
    NC = 96
    g = rng.standard_normal(NC)
    fwd = float(g @ kg.kpm_1d_derivative(H, dH, NC, 4, psi_in=psi))
    grad = kg.kpm_1d_grad(H, NC, psi, g)
    # gradient stored on H's pattern, value k = dL/dRe + i dL/dIm
    Gd = sp.csc_matrix(grad)
    Dd = sp.csc_matrix(dH)
    rev = float(np.real(np.sum(Gd.conj().multiply(Dd))))
    assert abs(fwd - rev) <= 1e-10 * max(abs(fwd), 1.0)


def test_haldane_dsigma_dt2_matches_finite_difference():
    """dsigma_xy/dt2 at Ef = 0 (fixed rescaling) from the GPU derivative and
    the GPU reconstruction, against central differences of the oracle's
    sigma_xy (6x6 torus, t2 = 0.2, NC = 96, identity probes)."""
    t2, h = 0.2, 1e-5
    H, Jx, Jy, area, dH, dJx, dJy = _haldane_direction(6, t2)
    D = H.shape[0]
    a, b, Hn = ko.normalizeH(H, center=True)
    psi = np.eye(D, dtype=complex)
    dmu = kg.kpm_2d_derivative(Hn, dH / a, Jx, dJx, Jy, dJy, 96, D, D, psi_in=psi)
    ds = kg.kubo_bastin_cond(dmu, a, 0.0, b=b, NH=D, area=area)

    def sigma(tt):
        Ht, Jxt, Jyt, _ = models.haldane(6, 6, t2=tt)
        Hs = (Ht - b * sp.identity(D, dtype=complex, format="csr")) / a
        mu = ko.kpm_2d(Hs, Jxt, Jyt, 96, psi, psi, 96, 96)
        return ko.kubo_bastin_cond(mu, a, 0.0, b=b, NH=D, area=area)
    fd = (sigma(t2 + h) - sigma(t2 - h)) / (2 * h)
    assert abs(ds - fd) <= 1e-6 * abs(fd)
    assert abs(fd) > 0.1   # the check is not vacuous


def test_derivative_argument_errors():
    H = models.square_anderson(4, W=1.0).tocsc() / 5.0
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d_derivative(H, H[:8, :8], 8, 1, psi_in=np.ones((16, 1)))
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_2d_derivative(H, H, H, None, H, None, 8, 1, 16)
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d_derivative(kg.GB300Operator(H), H, 8, 1, psi_in=np.ones((16, 1)))
