"""kpm_3d (src/moment.jl:1105-1280) on the GPU against the dense trace
formula of test/cpge_test.jl:319-338 and the oracle."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import relerr
from helpers import rand_herm
import kpm_gb300 as kg
from oracle import kpm_oracle as ko

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


def _cluster(seed=9, D=12):
    rng = np.random.default_rng(seed)
    H = rand_herm(rng, D)
    J = [rand_herm(rng, D, scale=1.0) for _ in range(3)]
    return H, J


def _dense_mu3(H, J, NC):
    T = ko.chebyshev_matrices(H, NC)
    D = H.shape[0]
    return np.array([[[np.trace(T[m] @ J[1] @ T[n] @ J[2] @ T[p] @ J[0]) / D
                       for p in range(NC)] for m in range(NC)] for n in range(NC)])


@pytest.mark.parametrize("prec,contraction,tol", [("fp64", "fp64", 1e-12), ("ff", "fp64", 1e-9),
                                                  ("fp64", "split", 1e-9)])
def test_kpm3d_trace_formula(prec, contraction, tol):
    H, J = _cluster()
    D, NC = H.shape[0], 8
    psi = np.eye(D, dtype=complex)
    mu = kg.kpm_3d(sp.csc_matrix(H), *(sp.csc_matrix(j) for j in J), NC, D, D, psi_in=psi,
                   precision=prec, contraction=contraction)
    assert mu.shape == (NC, NC, NC)
    assert relerr(mu, _dense_mu3(H, J, NC)) < tol


def test_kpm3d_probes_match_oracle():
    H, J = _cluster(seed=3, D=40)
    rng = np.random.default_rng(5)
    NC, NR = 6, 4
    pl = ko.random_phase_vectors(rng, 40, NR)
    pr = ko.random_phase_vectors(rng, 40, NR)
    Hs, Js = sp.csc_matrix(H), [sp.csc_matrix(j) for j in J]
    mu = kg.kpm_3d(Hs, *Js, NC, NR, 40, psi_in_l=pl, psi_in_r=pr, arr_size=3, right_block=2)
    assert relerr(mu, ko.kpm_3d(Hs, *Js, NC, pl, pr)) < 1e-12
