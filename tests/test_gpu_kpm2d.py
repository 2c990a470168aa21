"""GPU parity of the kpm_2d moment matrix (recurrences + contraction) against
dense Chebyshev references, the blocked oracle and exact diagonalisation."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import relerr
from helpers import blocking_model, load_golden
import kpm_gb300 as kg
from kpm_gb300 import models
from oracle import ed_reference as ed
from oracle import kpm_oracle as ko

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "ff": 1e-9}


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    return built_lib


@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_golden_haldane_moment_matrix(prec):
    f, mat = load_golden("haldane_3x3")
    NC = int(f["NC2"])
    NH = int(f["H_n"])
    mu = kg.kpm_2d(mat("H"), mat("Jx"), mat("Jy"), NC, 2, NH, psi_in_l=f["psi_l"],
                   psi_in_r=f["psi_r"], arr_size=4, right_block=3, precision=prec)
    assert relerr(mu, f["mu2d_dense"]) < TOL[prec]


@pytest.mark.parametrize("NC", [17, 24])
@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_blocked_vs_dense(NC, prec):
    """test/kpm2d_blocking_test.jl:73-95"""
    rng = np.random.default_rng(801)
    H, Ja, Jb = blocking_model(rng, 6)
    pl = ko.random_phase_vectors(rng, 36, 3)
    pr = ko.random_phase_vectors(rng, 36, 3)
    ref = ko.kpm2d_dense_reference(H, Ja, Jb, pl, pr, NC)
    got = kg.kpm_2d(sp.csc_matrix(H), sp.csc_matrix(Ja), sp.csc_matrix(Jb), NC, 3, 36,
                    psi_in_l=pl, psi_in_r=pr, arr_size=5, right_block=3, precision=prec)
    assert relerr(got, ref) < TOL[prec]


def test_blocking_invariance_and_auto():
    """test/kpm2d_blocking_test.jl:97-117, plus the resident (auto) plan."""
    rng = np.random.default_rng(802)
    NC = 17
    H, Ja, Jb = (kg.GB300Operator(sp.csc_matrix(M)) for M in blocking_model(rng, 6))
    psi = ko.random_phase_vectors(rng, 36, 3)
    base = kg.kpm_2d(H, Ja, Jb, NC, 3, 36, psi_in=psi, arr_size=3, right_block=3)
    for kl in (2, 3, 5, NC, NC + 7):
        for kr in (1, 3, 16, NC, NC + 7):
            got = kg.kpm_2d(H, Ja, Jb, NC, 3, 36, psi_in=psi, arr_size=kl, right_block=kr)
            assert relerr(got, base) < 1e-12, (kl, kr)
    auto = kg.kpm_2d(H, Ja, Jb, NC, 3, 36, psi_in=psi)
    assert relerr(auto, base) < 1e-12
    tight = kg.kpm_2d(H, Ja, Jb, NC, 3, 36, psi_in=psi, workspace_bytes=40 * 36 * 3 * 16)
    assert relerr(tight, base) < 1e-12


@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_parity_and_mn_sym(prec):
    """test/kpm2d_blocking_test.jl:154-207"""
    rng = np.random.default_rng(803)
    NC = 17
    H, Ja, Jb = (sp.csc_matrix(M) for M in blocking_model(rng, 6))
    psi = ko.random_phase_vectors(rng, 36, 3)
    full = ko.kpm_2d(H, Ja, Jb, NC, psi, psi, 5, 3)
    mask = (np.add.outer(np.arange(NC), np.arange(NC)) % 2) == 1
    kw = dict(psi_in=psi, arr_size=5, right_block=3, precision=prec)
    odd = kg.kpm_2d(H, Ja, Jb, NC, 3, 36, moment_parity="ODD", **kw)
    even = kg.kpm_2d(H, Ja, Jb, NC, 3, 36, moment_parity="EVEN", **kw)
    assert relerr(odd, full * mask) < TOL[prec]
    assert relerr(even, full * ~mask) < TOL[prec]
    sym = kg.kpm_2d(H, Ja, Jb, NC, 3, 36, mn_sym=True, **kw)
    assert relerr(sym, ko.kpm_2d(H, Ja, Jb, NC, psi, psi, 5, 3, mn_sym=True)) < TOL[prec]


@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_haldane_hall_quantized(prec):
    """test/kubo_bastin_test.jl:19-56: sigma_xy = C from GPU moments."""
    t2 = 0.2
    H, Jx, Jy, area = models.haldane(6, 6, t=1.0, t2=t2)
    D = H.shape[0]
    a, b, Hn = ko.normalizeH(H, center=True)
    psi = np.eye(D, dtype=complex)
    mu = kg.kpm_2d(Hn, Jx, Jy, 96, D, D, psi_in=psi, precision=prec)
    ref = ko.kpm_2d(Hn, Jx, Jy, 96, psi, psi, 96, 96)
    assert relerr(mu, ref) < TOL[prec]
    s_kpm = ko.kubo_bastin_cond(mu, a, 0.0, b=b, NH=D, area=area)
    s_ed = ed.ed_hall_conductivity_T0(H, Jx, Jy, area, 0.0)
    C = round(ed.chern_number_fhs(ed.haldane_bloch(t=1.0, t2=t2), Nk=30))
    assert abs(s_kpm - s_ed) < 0.03
    assert abs(s_kpm - C) < 0.05


def test_typed_cond_moments_delegates():
    NH = 64
    H = sp.diags([np.ones(NH - 1), np.ones(NH - 1)], [-1, 1], format="csc").astype(complex)
    Jx = sp.diags([-1j * np.ones(NH - 1), 1j * np.ones(NH - 1)], [-1, 1], format="csc")
    h = kg.rescale(H)
    psi = kg.random_phase_vectors(np.random.default_rng(11), NH, 4)
    m2 = kg.cond_moments(h, Jx, 0.7 * Jx, NC=32, psi_in=psi.copy())
    ref = kg.kpm_2d(h.H, Jx, 0.7 * Jx, 32, 4, NH, psi_in=psi.copy())
    assert np.array_equal(m2.mu, ref)
    assert relerr(ref, ko.kpm_2d(h.H, Jx, 0.7 * Jx, 32, psi, psi, 32, 32)) < 1e-12


@pytest.mark.parametrize("prec", ["fp64", "ff"])
@pytest.mark.parametrize("NC", [17, 24, 160])
def test_split_contraction_vs_dense(prec, NC):
    """BF16-digit tensor-core contraction (tcgen05) against the dense reference."""
    rng = np.random.default_rng(900 + NC)
    H, Ja, Jb = blocking_model(rng, 6)
    pl = ko.random_phase_vectors(rng, 36, 3)
    pr = ko.random_phase_vectors(rng, 36, 3)
    ref = ko.kpm2d_dense_reference(H, Ja, Jb, pl, pr, NC) if NC <= 24 else \
        ko.kpm_2d(H, Ja, Jb, NC, pl, pr, NC, NC)
    got = kg.kpm_2d(sp.csc_matrix(H), sp.csc_matrix(Ja), sp.csc_matrix(Jb), NC, 3, 36,
                    psi_in_l=pl, psi_in_r=pr, precision=prec, contraction="split")
    assert relerr(got, ref) < 1e-9


@pytest.mark.parametrize("kw", [dict(arr_size=5, right_block=3), dict(moment_parity="ODD"),
                                dict(mn_sym=True, arr_size=7, right_block=4)])
def test_split_contraction_blocking_parity(kw):
    rng = np.random.default_rng(803)
    NC = 17
    H, Ja, Jb = (sp.csc_matrix(M) for M in blocking_model(rng, 6))
    psi = ko.random_phase_vectors(rng, 36, 3)
    ref = kg.kpm_2d(H, Ja, Jb, NC, 3, 36, psi_in=psi, **kw)
    got = kg.kpm_2d(H, Ja, Jb, NC, 3, 36, psi_in=psi, contraction="split", **kw)
    assert relerr(got, ref) < 1e-9


def test_split_contraction_haldane_hall():
    """Quantized sigma_xy from tensor-core moments, and 1e-9 agreement with FP64."""
    t2 = 0.2
    H, Jx, Jy, area = models.haldane(6, 6, t=1.0, t2=t2)
    D = H.shape[0]
    a, b, Hn = ko.normalizeH(H, center=True)
    psi = np.eye(D, dtype=complex)
    ops = [kg.GB300Operator(M) for M in (Hn, Jx, Jy)]
    m64 = kg.kpm_2d(*ops, 96, D, D, psi_in=psi)
    msp = kg.kpm_2d(*ops, 96, D, D, psi_in=psi, precision="ff", contraction="split")
    assert relerr(msp, m64) < 1e-9
    s_kpm = ko.kubo_bastin_cond(msp, a, 0.0, b=b, NH=D, area=area)
    s_ed = ed.ed_hall_conductivity_T0(H, Jx, Jy, area, 0.0)
    assert abs(s_kpm - s_ed) < 0.03


def test_split_contraction_large_k():
    """K = NH*NR large enough for many exact 256-element chunks and K-splits."""
    rng = np.random.default_rng(5)
    H, Jx, Jy, _ = models.haldane(32, 32, t2=0.1)
    a, b, Hn = ko.normalizeH(H, center=True)
    NH = Hn.shape[0]
    psi = ko.random_phase_vectors(rng, NH, 16)
    ops = [kg.GB300Operator(M) for M in (Hn, Jx, Jy)]
    m64 = kg.kpm_2d(*ops, 64, 16, NH, psi_in=psi)
    msp = kg.kpm_2d(*ops, 64, 16, NH, psi_in=psi, contraction="split")
    assert relerr(msp, m64) < 1e-9


@pytest.mark.parametrize("NR", [16, 32])
@pytest.mark.parametrize("case", ["haldane", "peierls8"])
@pytest.mark.parametrize("kw", [{}, {"arr_size": 6, "right_block": 4},
                                {"moment_parity": "ODD"}, {"mn_sym": True}])
def test_column_pair_path_matches_oracle(NR, case, kw):
    """Float-float + split contraction with 16 or 32 probe columns on complex
    operators of at most 12 nonzeros per row runs the column-pair layout
    (k_step_ffcp: rows of up to 8 live slots in one anchored chunk, longer
    rows in two); against the blocked oracle and the FP64 path, with small
    blocks (left-chain wrap, right blocks recomputed), parity masks and
    mn_sym."""
    rng = np.random.default_rng(NR + len(case) + len(kw))
    if case == "haldane":
        H, Jx, Jy, _ = models.haldane(8, 8, t2=0.15, m=0.1)       # 10 nonzeros per row
        Hn = (H / 3.6).tocsc()
    else:
        Hn = (_peierls(8, rng) / 4.3).tocsc()                     # 5 nonzeros per row
        Jx = (1j * Hn).tocsc()
        Jy = ((0.3 - 0.7j) * Hn.conj()).tocsc()
    NH = Hn.shape[0]
    NC = 24
    pl = ko.random_phase_vectors(rng, NH, NR)
    pr = ko.random_phase_vectors(rng, NH, NR)
    ref = ko.kpm_2d(Hn, Jx, Jy, NC, pl, pr, NC, NC,
                    moment_parity=kw.get("moment_parity", "NONE"), mn_sym=kw.get("mn_sym", False))
    got = kg.kpm_2d(Hn, Jx, Jy, NC, NR, NH, psi_in_l=pl, psi_in_r=pr, precision="ff",
                    contraction="split", **kw)
    f64 = kg.kpm_2d(Hn, Jx, Jy, NC, NR, NH, psi_in_l=pl, psi_in_r=pr, **kw)
    assert relerr(got, ref) < TOL["ff"]
    assert relerr(got, f64) < TOL["ff"]


def _peierls(L, rng):
    """Square lattice with random U(1) phases on the bonds (complex, 5 per row)."""
    n = L * L
    rows, cols, vals = [], [], []
    for i in range(L):
        for j in range(L):
            s = i * L + j
            for t in (((i + 1) % L) * L + j, i * L + (j + 1) % L):
                ph = np.exp(2j * np.pi * rng.random())
                rows += [s, t]
                cols += [t, s]
                vals += [-ph, -np.conj(ph)]
            rows.append(s)
            cols.append(s)
            vals.append(rng.uniform(-0.5, 0.5))
    return sp.csc_matrix((vals, (rows, cols)), shape=(n, n))
