"""Parity at the benchmark sizes.

Against the oracle (fixtures from tests/golden/make_fullsize.py, inputs
rebuilt from seeds by fullsize_cases.py):
  c2  3D Anderson L=128, NC=4096, NR=64: all moments of eight probe columns
      against the C restatement of the reference CPU path, FP64 and
      float-float;
  c3  Haldane 256x256, NC=512, NR=16: the full moment matrix against the
      blocked NumPy kpm_2d (src/moment.jl:987-1088) for the FP64 and the
      split tensor-core contraction, and sigma_xy at 201 Fermi energies
      against the oracle's kubo_bastin_cond;
  c4  all 256 ensemble members against the oracle's doubling recurrence
      (FP64 and float-float per-step schedule, float-float persistent);
  c5  graphene 128x128, NC=1024, NR=16, checkpoints every 64: the adjoint
      gradient of the DOS-window loss along an onsite and a hopping direction
      against the oracle's exact directional derivative and against central
      differences of oracle moments.
Size-independent properties on top: the Chebyshev bound |mu_n| <= mu_0, the
doubling identity against the full bra/ket recurrence, independence of the
probe columns, the quantised Hall conductance.

Tolerances (norm-wise relative unless stated): FP64 moments 1e-12,
float-float and split forms 1e-9.
"""
import multiprocessing as mp
import os

import numpy as np
import pytest

from conftest import relerr
import fullsize_cases as fc
from helpers import GOLDEN
import kpm_gb300 as kg
from oracle import kpm_oracle as ko

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return built_lib


@pytest.fixture(scope="module")
def anderson128():
    """The headline workload with the fixture's rescaling."""
    f = np.load(GOLDEN / "fullsize_c2.npz")
    Hn = fc.rescaled(fc.c2_hamiltonian(), float(f["a"]), float(f["b"]))
    op = kg.GB300Operator(Hn)
    psi = fc.c2_probes(Hn.shape[0])
    return op, psi, f


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("ff", 1e-9)])
def test_c2_all_moments_against_cpu_port(anderson128, prec, tol):
    op, psi, f = anderson128
    NC = fc.C2["NC"]
    mu = kg.kpm_1d(op, NC, 64, psi_in=psi, avg_output=False, precision=prec)
    ref = f["mu"]
    got = mu[f["cols"]]
    assert relerr(got, ref) < tol
    for i in range(len(ref)):
        assert relerr(got[i], ref[i]) < tol
    # unit-norm probes: mu_0 = 1, and |mu_n| <= mu_0 on the rescaled spectrum
    assert np.abs(mu[:, 0] - 1.0).max() <= 1e-12
    assert np.abs(mu).max() <= 1 + 1e-12


def test_c2_doubling_vs_full_recurrence(anderson128):
    """mu_{2n} = 2<v_n|v_n> - mu_0 and mu_{2n+1} = 2<v_n|v_{n+1}> - mu_1 (doubling)
    against mu_n = <psi|T_n psi> step by step (the bra/ket path)."""
    op, psi, _ = anderson128
    NC = 256
    dbl = kg.kpm_1d(op, NC, 64, psi_in=psi, avg_output=False, precision="fp64")
    lr = kg.kpm_1d(op, NC, 64, psi_in_l=psi, psi_in_r=psi.copy(), avg_output=False,
                   precision="fp64")
    assert relerr(dbl, lr) < 1e-12
    assert np.abs(lr.imag).max() <= 1e-12


def test_c2_probe_columns_independent(anderson128):
    op, psi, _ = anderson128
    NC = 128
    both = kg.kpm_1d(op, NC, 64, psi_in=psi, avg_output=False, precision="ff")
    lo = kg.kpm_1d(op, NC, 32, psi_in=np.ascontiguousarray(psi[:, :32]), avg_output=False,
                   precision="ff")
    hi = kg.kpm_1d(op, NC, 32, psi_in=np.ascontiguousarray(psi[:, 32:]), avg_output=False,
                   precision="ff")
    assert relerr(both, np.vstack([lo, hi])) < 1e-12


def test_c3_moment_matrix_and_sigma_against_oracle():
    f = np.load(GOLDEN / "fullsize_c3.npz")
    a, b, area = float(f["a"]), float(f["b"]), float(f["area"])
    H, Jx, Jy, _ = fc.c3_model()
    Hn = fc.rescaled(H, a, b)
    NH, NR, NC = Hn.shape[0], fc.C3["NR"], fc.C3["NC"]
    psi = fc.c3_probes(NH)
    ops = [kg.GB300Operator(M) for M in (Hn, Jx, Jy)]
    f64 = kg.kpm_2d(*ops, NC, NR, NH, psi_in=psi, precision="fp64", contraction="fp64")
    split = kg.kpm_2d(*ops, NC, NR, NH, psi_in=psi, precision="ff", contraction="split")
    assert relerr(f64, f["mu"]) < 1e-12
    assert relerr(split, f["mu"]) < 1e-9
    Ef = fc.C3["Ef"]
    s64 = kg.kubo_bastin_cond(f64, a, Ef, b=b, NH=NH, area=area)
    ssp = kg.kubo_bastin_cond(split, a, Ef, b=b, NH=NH, area=area)
    # sigma is a linear functional of mu with weights up to (1 - x^2)^-1.5 near
    # the band edges, so its relative error may exceed that of mu
    assert relerr(s64, f["sigma"]) < 1e-9
    assert relerr(ssp, f["sigma"]) < 1e-6
    # quantised Hall conductance inside the gap
    mid = np.abs(Ef) <= 0.1 + 1e-12
    s = s64[mid]
    assert np.abs(s - 1.0).max() < 0.02 or np.abs(s + 1.0).max() < 0.02


def test_c4_every_member_against_oracle():
    """The 256-member persistent launch against the oracle's doubling
    recurrence for every member (oracle runs in a spawn pool)."""
    Hs, psis = fc.c4_members()
    ens = kg.EnsembleOperator(Hs)
    got = kg.kpm_1d_ensemble(ens, 512, psis, avg_output=False)
    got_ff = kg.kpm_1d_ensemble(ens, 512, psis, avg_output=False, precision="ff")
    got_ps = kg.kpm_1d_ensemble(ens, 512, psis, avg_output=False, precision="ff", kernel="single")
    ctx = mp.get_context("spawn")
    with ctx.Pool(max(1, min(16, os.cpu_count() or 1))) as pool:
        refs = pool.starmap(ko.kpm_1d_doubling, [(H, 512, p) for H, p in zip(Hs, psis)],
                            chunksize=8)
    for i in range(256):
        assert relerr(got[i], refs[i]) < 1e-12, i
        assert relerr(got_ff[i], refs[i]) < 1e-9, i
        assert relerr(got_ps[i], refs[i]) < 1e-9, i


def test_c5_dos_window_gradient_against_oracle():
    f = np.load(GOLDEN / "fullsize_c5.npz")
    H, Ht, psi = fc.c5_inputs()
    NC, NR, a = fc.C5["NC"], fc.C5["NR"], fc.C5["a"]
    Phi, q = fc.dos_weights(NC, a, fc.C5["E"])
    rho_t = f["rho_t"]
    assert relerr(Phi @ kg.kpm_1d(Ht, NC, NR, psi_in=psi.copy()), rho_t) < 1e-11
    rho = Phi @ kg.kpm_1d(H, NC, NR, psi_in=psi.copy())
    L0 = float(q @ (rho - rho_t) ** 2)
    assert abs(L0 - float(f["loss"])) <= 1e-8 * float(f["loss"])
    g = Phi.T @ (2 * q * (rho - rho_t))
    G = kg.kpm_1d_grad(H, NC, psi, g, checkpoint_every=fc.C5["checkpoint"])
    for k, D in enumerate(fc.c5_directions(H)):
        d = fc.pairing(G, D)
        # exact (dual-number) derivative of the oracle; central differences of
        # oracle moments at eps = 1e-5 agree with it to ~1e-7
        assert abs(d - f["exact"][k]) <= 1e-8 * abs(f["exact"][k])
        assert abs(d - f["fd"][k]) <= 5e-6 * abs(f["fd"][k])
