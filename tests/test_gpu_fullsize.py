"""Parity at the benchmark sizes, through properties that hold at any size
(the oracle does not finish there): float-float against native FP64 moments,
the Chebyshev bound |mu_n| <= mu_0, the doubling identity against the full
bra/ket recurrence, independence of the probe columns (one wide call equals
two narrow ones), the split contraction against the FP64 one, the quantised
Hall conductance of the Haldane model, and the persistent ensemble launch
against per-member calls.  Tolerances: FP64 forms 1e-12, float-float and
split forms 1e-9 (norm-wise relative)."""
import numpy as np
import pytest

from conftest import relerr
import kpm_gb300 as kg
from kpm_gb300 import models

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return built_lib


@pytest.fixture(scope="module")
def anderson128():
    """3D Anderson L=128 periodic (NH=2097152, 7 nonzeros per row), W=16.5,
    centred rescaling, 64 random-phase probes: the headline workload."""
    rng = np.random.default_rng(42)
    h = kg.rescale(models.cubic_anderson(128, W=16.5, rng=rng), center=True)
    op = kg.GB300Operator(h.H)
    psi = kg.random_phase_vectors(np.random.default_rng(7), h.H.shape[0], 64)
    return op, psi


def test_anderson128_ff_vs_fp64_and_bounds(anderson128):
    op, psi = anderson128
    NC = 512
    ff = kg.kpm_1d(op, NC, 64, psi_in=psi, avg_output=False, precision="ff")
    f64 = kg.kpm_1d(op, NC, 64, psi_in=psi, avg_output=False, precision="fp64")
    assert relerr(ff, f64) < 1e-9
    # unit-norm probes: mu_0 = <psi|psi> = 1, and |mu_n| <= mu_0 (|T_n| <= 1 on the
    # rescaled spectrum)
    assert np.abs(f64[:, 0] - 1.0).max() <= 1e-12
    assert np.abs(f64).max() <= 1 + 1e-12
    assert np.abs(ff).max() <= 1 + 1e-12


def test_anderson128_doubling_vs_full_recurrence(anderson128):
    """mu_{2n} = 2<v_n|v_n> - mu_0 and mu_{2n+1} = 2<v_n|v_{n+1}> - mu_1 (doubling)
    against mu_n = <psi|T_n psi> step by step (the bra/ket path)."""
    op, psi = anderson128
    NC = 256
    dbl = kg.kpm_1d(op, NC, 64, psi_in=psi, avg_output=False, precision="fp64")
    lr = kg.kpm_1d(op, NC, 64, psi_in_l=psi, psi_in_r=psi.copy(), avg_output=False,
                   precision="fp64")
    assert relerr(dbl, lr) < 1e-12
    assert np.abs(lr.imag).max() <= 1e-12


def test_anderson128_probe_columns_independent(anderson128):
    op, psi = anderson128
    NC = 128
    both = kg.kpm_1d(op, NC, 64, psi_in=psi, avg_output=False, precision="ff")
    lo = kg.kpm_1d(op, NC, 32, psi_in=np.ascontiguousarray(psi[:, :32]), avg_output=False,
                   precision="ff")
    hi = kg.kpm_1d(op, NC, 32, psi_in=np.ascontiguousarray(psi[:, 32:]), avg_output=False,
                   precision="ff")
    assert relerr(both, np.vstack([lo, hi])) < 1e-12


def test_haldane256_split_contraction_and_quantised_hall():
    """Haldane 256x256 cells (NH=131072), t2 = 0.1 i, NC=512, NR=16."""
    H, Jx, Jy, area = models.haldane(256, 256, t=1.0, t2=0.1)
    h = kg.rescale(H, center=True)
    NH, NR, NC = H.shape[0], 16, 512
    psi = kg.random_phase_vectors(np.random.default_rng(42), NH, NR)
    ops = [kg.GB300Operator(M) for M in (h.H, Jx, Jy)]
    split = kg.kpm_2d(*ops, NC, NR, NH, psi_in=psi, precision="ff", contraction="split")
    f64 = kg.kpm_2d(*ops, NC, NR, NH, psi_in=psi, precision="fp64", contraction="fp64")
    assert relerr(split, f64) < 1e-9
    s = kg.kubo_bastin_cond(f64, h.a, np.array([-0.1, 0.0, 0.1]), b=h.b, NH=NH, area=area)
    assert np.abs(s - 1.0).max() < 0.02 or np.abs(s + 1.0).max() < 0.02


def test_ensemble256_vs_member_calls():
    """256 realisations of the 2D Anderson model, L ~ U{24..96}, W ~ U[1, 8],
    NC=512, NR=8: one persistent launch against per-member calls."""
    rng = np.random.default_rng(42)
    Hs, psis = [], []
    for _ in range(256):
        L = int(rng.integers(24, 97))
        W = float(rng.uniform(1.0, 8.0))
        Hs.append((models.square_anderson(L, W=W, rng=rng) / (4.0 + W / 2 + 0.1)).tocsc())
        psis.append(kg.random_phase_vectors(rng, L * L, 8))
    ens = kg.EnsembleOperator(Hs)
    got = kg.kpm_1d_ensemble(ens, 512, psis, avg_output=False)
    for i in range(0, 256, 17):
        ref = kg.kpm_1d(Hs[i], 512, 8, psi_in=psis[i], avg_output=False)
        assert relerr(got[i], ref) < 1e-12
