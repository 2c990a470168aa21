"""Reverse-mode gradient of losses on the kpm_2d moments (kpmgb_kpm2d_grad)
and of the Kubo-Bastin conductivity (kpmgb_kubo_bastin_weights).

Checked entry by entry against central finite differences of the oracle's
kpm_2d on a small complex model (H, Ja, Jb as independent operators), and on
the Haldane model 64x64 (NC=256, NR=8): d sigma_xy(Ef=0) along random onsite
energies, t1 and t2 (the currents J = H (r_i - r_j) move with the hoppings)
against the oracle's exact dual-number derivative (fixture
tests/golden/fullsize_x1.npz) and against the GPU forward-mode derivative.
Tolerances: finite differences 1e-7 (entry-wise, relative to the largest
entry), exact derivatives 1e-8 relative.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import relerr
import fullsize_cases as fc
from helpers import GOLDEN
import kpm_gb300 as kg
from kpm_gb300 import models
from oracle import kpm_oracle as ko

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return built_lib


def _oracle_F(H, Ja, Jb, NC, pl, pr, G, parity="NONE"):
    mu = ko.kpm_2d(H, Ja, Jb, NC, pl, pr, NC, NC, moment_parity=parity)
    return float(np.sum(G * mu).real)


@pytest.mark.parametrize("parity", ["NONE", "ODD"])
def test_kpm2d_grad_matches_oracle_finite_differences(parity):
    rng = np.random.default_rng(31)
    H, Jx, Jy, _ = models.haldane(3, 3, t2=0.2, m=0.15)
    H = fc.rescaled_keep(H, 3.9, 0.05)
    NH, NC, NR = H.shape[0], 10, 3
    pl = ko.random_phase_vectors(rng, NH, NR)
    pr = ko.random_phase_vectors(rng, NH, NR)
    G = rng.standard_normal((NC, NC)) + 1j * rng.standard_normal((NC, NC))
    gH, gA, gB = kg.kpm_2d_grad(H, Jx, Jy, NC, G, psi_in_l=pl, psi_in_r=pr,
                                moment_parity=parity)
    eps = 1e-6
    for which, (M, got) in enumerate(((H, gH), (Jx, gA), (Jy, gB))):
        M = sp.csc_matrix(M)
        fd = np.zeros(M.nnz, dtype=np.complex128)
        for k in range(M.nnz):
            for unit in (1.0, 1j):
                Mp, Mm = M.copy(), M.copy()
                Mp.data = M.data.copy()
                Mm.data = M.data.copy()
                Mp.data[k] += eps * unit
                Mm.data[k] -= eps * unit
                ops_p = [H, Jx, Jy]
                ops_m = [H, Jx, Jy]
                ops_p[which], ops_m[which] = Mp, Mm
                d = (_oracle_F(*ops_p, NC, pl, pr, G, parity)
                     - _oracle_F(*ops_m, NC, pl, pr, G, parity)) / (2 * eps)
                fd[k] += d * unit
        g = sp.csc_matrix(got)
        assert np.array_equal(g.indptr, M.indptr) and np.array_equal(g.indices, M.indices)
        assert np.abs(g.data - fd).max() <= 1e-7 * np.abs(fd).max(), which


def test_kubo_bastin_weights_are_the_linear_map():
    rng = np.random.default_rng(8)
    NC, a, b, NH, area = 48, 3.3, 0.1, 200, 170.0
    mu = rng.standard_normal((NC, NC)) + 1j * rng.standard_normal((NC, NC))
    for Ef, beta in ((0.0, np.inf), (0.4, 20.0), (-1.2, np.inf)):
        W = kg.kubo_bastin_weights(NC, a, Ef, b=b, NH=NH, area=area, beta=beta)
        s = kg.kubo_bastin_cond(mu, a, Ef, b=b, NH=NH, area=area, beta=beta)
        s_ref = ko.kubo_bastin_cond(mu, a, Ef, b=b, NH=NH, area=area, beta=beta)
        assert abs(np.sum(W * mu).real - s_ref) <= 1e-11 * max(1.0, abs(s_ref))
        assert abs(s - s_ref) <= 1e-11 * max(1.0, abs(s_ref))


def test_haldane64_dsigma_against_oracle_and_forward_mode():
    f = np.load(GOLDEN / "fullsize_x1.npz")
    a, b, area = float(f["a"]), float(f["b"]), float(f["area"])
    H, Jx, Jy, _, dirs = fc.x1_model()
    Hn = fc.rescaled_keep(H, a, b)
    NH, NC, NR, Ef = Hn.shape[0], fc.X1["NC"], fc.X1["NR"], fc.X1["Ef"]
    psi = fc.x1_probes(NH)
    ops = [kg.GB300Operator(M) for M in (Hn, Jx, Jy)]
    mu = kg.kpm_2d(*ops, NC, NR, NH, psi_in=psi)
    sigma = kg.kubo_bastin_cond(mu, a, Ef, b=b, NH=NH, area=area)
    assert abs(sigma - float(f["sigma"])) <= 1e-9 * abs(float(f["sigma"]))
    W = kg.kubo_bastin_weights(NC, a, Ef, b=b, NH=NH, area=area)
    assert abs(np.sum(W * mu).real - sigma) <= 1e-11 * abs(sigma)
    gH, gJx, gJy = kg.kpm_2d_grad(Hn, Jx, Jy, NC, W, psi_in=psi)
    for k, (dH, dJx, dJy) in enumerate(dirs):
        d = fc.pairing(gH, dH / a) + fc.pairing(gJx, dJx) + fc.pairing(gJy, dJy)
        ref = float(f["dsigma"][k])
        assert abs(d - ref) <= 1e-8 * abs(ref), (k, d, ref)
        # forward mode through the block-triangular embedding: its power-of-two
        # pre-scaling balances the tangent half against the primal half, which
        # leaves ~1e-8 relative on a derivative 1000x smaller than sigma (t1)
        dmu = kg.kpm_2d_derivative(Hn, dH / a, Jx, dJx, Jy, dJy, NC, NR, NH, psi_in=psi)
        fwd = kg.kubo_bastin_cond(dmu, a, Ef, b=b, NH=NH, area=area)
        assert abs(d - fwd) <= 1e-6 * abs(ref), (k, d, fwd)


def test_kpm2d_grad_column_batches_and_errors():
    """NR = 40 runs as batches of 32 + 8 probe columns; the gradient is their
    sum.  mn_sym is not covered and Jb_adjoint is needed for device operators."""
    rng = np.random.default_rng(12)
    H, Jx, Jy, _ = models.haldane(4, 4, t2=0.1)
    H = fc.rescaled_keep(H, 3.6, 0.0)
    NH, NC = H.shape[0], 8
    psi = ko.random_phase_vectors(rng, NH, 40)
    G = rng.standard_normal((NC, NC)) + 1j * rng.standard_normal((NC, NC))
    full = kg.kpm_2d_grad(H, Jx, Jy, NC, G, psi_in=psi)
    a = kg.kpm_2d_grad(H, Jx, Jy, NC, G, psi_in=np.ascontiguousarray(psi[:, :32]))
    b = kg.kpm_2d_grad(H, Jx, Jy, NC, G, psi_in=np.ascontiguousarray(psi[:, 32:]))
    for g, ga, gb in zip(full, a, b):
        ref = (32 * ga.toarray() + 8 * gb.toarray()) / 40
        assert np.abs(g.toarray() - ref).max() <= 1e-13 * np.abs(ref).max()
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_2d_grad(H, Jx, kg.GB300Operator(Jy), NC, G, psi_in=psi)
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_2d_grad(H, Jx, Jy, NC, G[:4, :4], psi_in=psi)
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_2d_grad(H, Jx, Jy, NC, G, psi_in=psi, moment_parity="BOTH")
