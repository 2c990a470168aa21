"""Pin the CPU oracle against the known answers the reference's tests use.

No GPU.  Each test restates one of the reference's own checks
(test/dos_test.jl, test/kpm2d_blocking_test.jl, test/kubo_bastin_test.jl,
test/frontend_test.jl) against the oracle, so the oracle is validated by exact
diagonalisation, dense Chebyshev matrices and analytic results rather than by
itself.
"""
import math

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import relerr
from kpm_gb300 import models
from oracle import ed_reference as ed
from oracle import kpm_oracle as ko


def _rand_herm(rng, n, scale=1.2):
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    H = (A + A.conj().T) / 2
    return H / (scale * np.linalg.norm(H, 2))


def _blocking_model(rng, L):
    """test/kpm2d_blocking_test.jl:7-23"""
    N = L * L
    H = np.zeros((N, N), dtype=complex)
    for y in range(L):
        for x in range(L):
            i = x + L * y
            if x < L - 1:
                H[i, i + 1] = H[i + 1, i] = -1
            if y < L - 1:
                H[i, i + L] = H[i + L, i] = -1
    A = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    H = H + 0.03 * (A + A.conj().T) / 2
    H = H / (1.2 * np.linalg.norm(H, 2))
    B = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    Cm = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    return H, (B + B.conj().T) / 2, (Cm + Cm.conj().T) / 2


def test_doubling_vs_direct_and_ed():
    """test/dos_test.jl:11-44"""
    rng = np.random.default_rng(42)
    NH, NC = 64, 32
    Hd = _rand_herm(rng, NH, scale=1 / 0.95)
    psi = rng.standard_normal((NH, 1)) + 1j * rng.standard_normal((NH, 1))
    psi /= np.linalg.norm(psi)
    mu = ko.kpm_1d(sp.csr_matrix(Hd), NC, 1, psi_in=psi)
    direct = np.zeros(NC)
    prev, cur = psi[:, 0].copy(), Hd @ psi[:, 0]
    direct[0], direct[1] = np.vdot(psi[:, 0], prev).real, np.vdot(psi[:, 0], cur).real
    for n in range(2, NC):
        prev, cur = cur, 2 * (Hd @ cur) - prev
        direct[n] = np.vdot(psi[:, 0], cur).real
    assert np.max(np.abs(mu - direct)) < 1e-10
    assert np.max(np.abs(mu - ed.ed_moments(Hd, psi, NC)[0])) < 1e-8


def test_kpm1d_equal_and_lr_vs_dense_chebyshev():
    """test/kpm2d_blocking_test.jl:237-269"""
    rng = np.random.default_rng(805)
    NH, NR, NC = 20, 3, 24
    H = _rand_herm(rng, NH)
    psi = ko.random_phase_vectors(rng, NH, NR)
    pl = ko.random_phase_vectors(rng, NH, NR)
    pr = ko.random_phase_vectors(rng, NH, NR)
    T = ko.chebyshev_matrices(H, NC)
    ref_eq = np.array([[np.vdot(psi[:, i], T[n] @ psi[:, i]) for n in range(NC)] for i in range(NR)])
    ref_lr = np.array([[np.vdot(pl[:, i], T[n] @ pr[:, i]) for n in range(NC)] for i in range(NR)])
    got_eq = ko.kpm_1d(sp.csr_matrix(H), NC, NR, psi_in=psi, avg_output=False)
    got_lr = ko.kpm_1d(sp.csr_matrix(H), NC, NR, psi_in_l=pl, psi_in_r=pr, avg_output=False)
    assert relerr(got_eq, ref_eq) < 1e-12
    assert relerr(got_lr, ref_lr) < 1e-12
    # odd NC is allowed on the bra/ket path only
    ko.kpm_1d_lr(sp.csr_matrix(H), 7, pl, pr)
    with pytest.raises(ValueError):
        ko.kpm_1d_doubling(sp.csr_matrix(H), 7, psi)


@pytest.mark.parametrize("NC", [17, 24])
def test_kpm2d_blocked_vs_dense(NC):
    """test/kpm2d_blocking_test.jl:73-95"""
    rng = np.random.default_rng(801)
    H, Ja, Jb = _blocking_model(rng, 6)
    pl = ko.random_phase_vectors(rng, 36, 3)
    pr = ko.random_phase_vectors(rng, 36, 3)
    ref = ko.kpm2d_dense_reference(H, Ja, Jb, pl, pr, NC)
    got = ko.kpm_2d(H, Ja, Jb, NC, pl, pr, K_left=5, K_right=3)
    assert relerr(got, ref) < 1e-12


def test_kpm2d_blocking_invariance_parity_mnsym():
    """test/kpm2d_blocking_test.jl:97-117 and :154-207"""
    rng = np.random.default_rng(802)
    NC = 17
    H, Ja, Jb = _blocking_model(rng, 6)
    psi = ko.random_phase_vectors(rng, 36, 3)
    base = ko.kpm_2d(H, Ja, Jb, NC, psi, psi, 3, 3)
    for kl in (2, 3, 5, NC, NC + 7):
        for kr in (1, 3, 16, NC, NC + 7):
            assert relerr(ko.kpm_2d(H, Ja, Jb, NC, psi, psi, kl, kr), base) < 1e-12
    odd = ko.kpm_2d(H, Ja, Jb, NC, psi, psi, 5, 3, moment_parity="ODD")
    even = ko.kpm_2d(H, Ja, Jb, NC, psi, psi, 5, 3, moment_parity="EVEN")
    mask = (np.add.outer(np.arange(NC), np.arange(NC)) % 2) == 1
    assert relerr(odd, base * mask) < 1e-12
    assert relerr(even, base * ~mask) < 1e-12
    sym_ref = base.copy()
    for m in range(NC):
        for n in range(m + 1, NC):
            sym_ref[m, n] = sym_ref[m, n].real
            sym_ref[n, m] = sym_ref[m, n]
    sym = ko.kpm_2d(H, Ja, Jb, NC, psi, psi, 5, 3, mn_sym=True)
    assert relerr(sym, sym_ref) < 1e-12


def test_blocking_choices():
    """test/kpm2d_blocking_test.jl:119-152"""
    NH, NR, NC = 40, 3, 50
    one = NH * NR * 16
    kl, kr, nbytes = ko.kpm_2d_blocking(NH, NR, NC, 30 * one, right_block=4)
    assert (kl, kr) == (18, 4)
    assert nbytes == 11 * one + 18 * (one + 64)
    with pytest.raises(ValueError):
        ko.kpm_2d_blocking(NH, NR, NC, 10 * one - 1)
    assert ko.kpm_2d_blocking(NH, NR, NC, 10 * one, arr_size=27, right_block=9)[:2] == (27, 9)


def test_estimator_semantics():
    """test/dos_test.jl:66-141: unbiased probes, |c|^2 scaling, force_norm."""
    rng = np.random.default_rng(21)
    D = 8
    u = np.full(D, 1 / math.sqrt(D))
    H = 0.8 * np.outer(u, u)
    psi = np.exp(2j * np.pi * rng.random((D, 512)))
    ko.normalize_by_col(psi)
    mu = ko.kpm_1d(sp.csr_matrix(H), 4, 512, psi_in=psi)
    assert abs(mu[1] - 0.8 / D) < 0.3 * 0.8 / D
    Hs = sp.csr_matrix(_rand_herm(rng, 32, scale=2.0))
    p = rng.standard_normal((32, 1)) + 1j * rng.standard_normal((32, 1))
    p /= np.linalg.norm(p)
    assert relerr(ko.kpm_1d(Hs, 16, 1, psi_in=2 * p), 4 * ko.kpm_1d(Hs, 16, 1, psi_in=p)) < 1e-10
    raw = ko.random_phase_vectors(rng, 32, 4) * np.array([1.0, 5.0, 0.2, 12.0])
    forced = raw.copy()
    m_forced = ko.kpm_1d(Hs, 16, 4, psi_in=forced, force_norm=True)
    pre = raw.copy()
    ko.normalize_by_col(pre)
    assert relerr(m_forced, ko.kpm_1d(Hs, 16, 4, psi_in=pre)) < 1e-12
    assert relerr(forced, pre) < 1e-12


def test_chain_dos_analytic_and_sum_rule():
    """test/dos_test.jl:214-249: shifted 1D chain DOS and the sum rule."""
    N, t, shift = 4000, 1.0, 0.7
    H = models.ring(N, t=t, shift=shift)
    a, b, Hn = ko.normalizeH(H, center=True)
    assert abs(b - shift) < 0.05
    rng = np.random.default_rng(7)
    psi = np.exp(2j * np.pi * rng.random((N, 24)))
    ko.normalize_by_col(psi)
    mu = ko.kpm_1d(Hn, 256, 24, psi_in=psi)
    E, rho = ko.dos(mu, a, b=b, N_tilde=1024)
    assert abs(np.sum(rho) * (E[1] - E[0]) - 1.0) < 2e-2
    idx = np.abs(E - shift) < 1.5 * t
    exact = 1 / (np.pi * np.sqrt(4 * t ** 2 - (E[idx] - shift) ** 2))
    assert np.max(np.abs(rho[idx] - exact)) < 0.02


def test_dos_sum_rule_identity_probes():
    """test/frontend_test.jl:173-187: with identity probes the sum rule is exact."""
    NH = 64
    H = sp.diags([np.ones(NH - 1), np.ones(NH - 1)], [-1, 1]).astype(complex)
    a, _, Hn = ko.normalizeH(H)
    mu = ko.kpm_1d(Hn, 128, NH, psi_in=np.eye(NH, dtype=complex))
    assert abs(mu[0] - 1.0) < 1e-12
    Nq = 512
    xq = np.cos((np.arange(1, Nq + 1) - 0.5) * np.pi / Nq)
    _, rho = ko.dos(mu, a, E_grid=a * xq)
    assert abs(np.sum(a * np.pi * np.sqrt(1 - xq ** 2) * rho) / Nq - 1.0) < 1e-12


def test_haldane_hall_quantized():
    """test/kubo_bastin_test.jl:19-56: sigma_xy = C from KPM moments and ED."""
    t2 = 0.2
    H, Jx, Jy, area = models.haldane(6, 6, t=1.0, t2=t2)
    D = H.shape[0]
    C_fhs = ed.chern_number_fhs(ed.haldane_bloch(t=1.0, t2=t2), Nk=30)
    C = round(C_fhs)
    assert abs(C) == 1 and abs(C_fhs - C) < 1e-10
    s_ed = ed.ed_hall_conductivity_T0(H, Jx, Jy, area, 0.0)
    assert abs(s_ed - C) < 0.02
    a, b, Hn = ko.normalizeH(H, center=True)
    psi = np.eye(D, dtype=complex)
    mu = ko.kpm_2d(Hn, Jx, Jy, 96, psi, psi, 96, 96)
    s_kpm = ko.kubo_bastin_cond(mu, a, 0.0, b=b, NH=D, area=area)
    assert abs(s_kpm - s_ed) < 0.03
    assert abs(s_kpm - C) < 0.05


def test_normalizeH():
    """test/dos_test.jl:176-195"""
    rng = np.random.default_rng(3)
    A = sp.random(100, 100, density=0.05, random_state=3,
                  data_rvs=lambda k: rng.standard_normal(k) + 1j * rng.standard_normal(k))
    with pytest.raises(ValueError):
        ko.normalizeH(A + 2 * A.conj().T)
    H = (A + A.conj().T).tocsr()
    a, _, Hn = ko.normalizeH(H)
    assert np.abs(np.linalg.eigvalsh(Hn.toarray())).max() < 1
    a, b, Hs = ko.normalizeH(H + 0.7 * sp.identity(100), center=True)
    ev = np.linalg.eigvalsh(Hs.toarray())
    assert abs(b - 0.7) < 0.1 * a and ev.min() > -1 and ev.max() < 1


@pytest.mark.parametrize("name", ["anderson2d_L8", "haldane_3x3", "ring_N64"])
def test_oracle_matches_golden(name):
    """The oracle reproduces every committed golden fixture."""
    from pathlib import Path
    f = np.load(Path(__file__).parent / "golden" / f"{name}.npz")
    H = sp.csc_matrix((f["H_data"], f["H_indices"], f["H_indptr"]), shape=(int(f["H_n"]),) * 2)
    NC = int(f["NC"])
    if name == "anderson2d_L8":
        mu = ko.kpm_1d(H, NC, 3, psi_in=f["psi"], avg_output=False)
        assert relerr(mu, f["mu_dense"]) < 1e-12
        assert relerr(mu, f["mu_ed"]) < 1e-10
    elif name == "haldane_3x3":
        mu = ko.kpm_1d(H, NC, 2, psi_in_l=f["psi_l"], psi_in_r=f["psi_r"], avg_output=False)
        assert relerr(mu, f["mu_lr_dense"]) < 1e-12
        J = lambda k: sp.csc_matrix((f[f"{k}_data"], f[f"{k}_indices"], f[f"{k}_indptr"]),
                                    shape=H.shape)
        m2 = ko.kpm_2d(H, J("Jx"), J("Jy"), int(f["NC2"]), f["psi_l"], f["psi_r"], 4, 3)
        assert relerr(m2, f["mu2d_dense"]) < 1e-12
    else:
        N = H.shape[0]
        mu = ko.kpm_1d(H, NC, N, psi_in=np.eye(N, dtype=complex))
        assert relerr(mu, f["mu_exact"]) < 1e-12


def test_c_port_matches_oracle():
    """The C restatement (CPU baseline) agrees with the NumPy oracle."""
    from oracle import cpu_port
    rng = np.random.default_rng(5)
    H = models.square_anderson(16, W=2.0, rng=rng)
    a, _, Hn = ko.normalizeH(H)
    psi = ko.random_phase_vectors(rng, 256, 5)
    ref = ko.kpm_1d_doubling(Hn, 128, psi)
    got = cpu_port.kpm1d_cpu(Hn, 128, psi, nthreads=2)
    assert relerr(got, ref) < 1e-12


def test_oracle_kpm3d_trace_formula():
    """test/cpge_test.jl:319-338: mu[n,m,p] = Tr[T_m Jb T_n Jc T_p Ja] / D with
    identity probes."""
    from helpers import rand_herm
    rng = np.random.default_rng(9)
    D, NC = 10, 5
    H = rand_herm(rng, D)
    J = [rand_herm(rng, D, scale=1.0) for _ in range(3)]
    T = ko.chebyshev_matrices(H, NC)
    ref = np.array([[[np.trace(T[m] @ J[1] @ T[n] @ J[2] @ T[p] @ J[0]) / D
                      for p in range(NC)] for m in range(NC)] for n in range(NC)])
    psi = np.eye(D, dtype=complex)
    got = ko.kpm_3d(H, J[0], J[1], J[2], NC, psi, psi)
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)


def test_oracle_chebyshev_action_ed():
    """test/chebyshev_action_test.jl:43-60: the action equals the spectral sum."""
    rng = np.random.default_rng(151)
    NH, NC, NR, K = 30, 14, 2, 3
    A = rng.standard_normal((NH, NH)) + 1j * rng.standard_normal((NH, NH))
    Hd = (A + A.conj().T) / 2
    Hd /= np.abs(np.linalg.eigvalsh(Hd)).max() / 0.95
    V = rng.standard_normal((NH, NR)) + 1j * rng.standard_normal((NH, NR))
    C = rng.standard_normal((NC, K)) + 1j * rng.standard_normal((NC, K))
    out = ko.chebyshev_action(Hd, V, C)
    lam, U = np.linalg.eigh(Hd)
    th = np.arccos(np.clip(lam, -1, 1))
    for k in range(K):
        f = np.array([np.sum(C[:, k] * np.cos(np.arange(NC) * t)) for t in th])
        assert np.abs(out[:, :, k] - U @ (f[:, None] * (U.conj().T @ V))).max() < 1e-8


def test_oracle_kpm1d_current_trace():
    """test/optical_cond_test.jl:278-287: kpm_1d_current with identity probes is
    Tr[J T_n] / D."""
    from helpers import rand_herm
    rng = np.random.default_rng(2)
    D, NC = 14, 10
    H = rand_herm(rng, D)
    J = rand_herm(rng, D, scale=1.0)
    T = ko.chebyshev_matrices(H, NC)
    ref = np.array([np.trace(J @ T[n]) / D for n in range(NC)])
    mu = ko.kpm_1d_current(H, J, NC, np.eye(D, dtype=complex)).sum(axis=0) / D
    assert np.linalg.norm(mu - ref) <= 1e-12 * np.linalg.norm(ref)


def test_oracle_tangent_trace_identity():
    """Directional derivative of the traced moments: with identity probes,
    d/dt Tr T_n(H + t dH) = n Tr[U_{n-1}(H) dH] (T_n' = n U_{n-1}), exactly."""
    from helpers import rand_herm
    rng = np.random.default_rng(5)
    D, NC = 16, 20
    H = rand_herm(rng, D)
    dH = rand_herm(rng, D, scale=3.0)
    U = [np.eye(D, dtype=complex), 2.0 * H]
    for n in range(2, NC):
        U.append(2.0 * H @ U[n - 1] - U[n - 2])
    ref = np.array([0.0] + [n * np.trace(U[n - 1] @ dH) for n in range(1, NC)])
    got = ko.kpm_1d_tangent(H, dH, NC, np.eye(D, dtype=complex)).sum(axis=0)
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)


def test_oracle_tangent_finite_difference():
    """kpm_1d / kpm_2d tangents against central differences of the moments in
    the Haldane t2 direction (H, Jx, Jy are affine in t2)."""
    def model(t2):
        H, Jx, Jy, _ = models.haldane(4, 4, t2=t2)
        return H / 3.8, Jx, Jy
    rng = np.random.default_rng(6)
    (H0, Jx0, Jy0), (H1, Jx1, Jy1) = model(0.0), model(1.0)
    t2, h, NC, NR = 0.2, 1e-5, 24, 3
    H, Jx, Jy = model(t2)
    NH = H.shape[0]
    psl = ko.random_phase_vectors(rng, NH, NR)
    psr = ko.random_phase_vectors(rng, NH, NR)
    d2 = ko.kpm_2d_tangent(H, H1 - H0, Jx, Jx1 - Jx0, Jy, Jy1 - Jy0, NC, psl, psr)
    fd2 = (ko.kpm2d_dense_reference(*model(t2 + h), psl, psr, NC)
           - ko.kpm2d_dense_reference(*model(t2 - h), psl, psr, NC)) / (2 * h)
    assert relerr(d2, fd2) < 1e-6
    d1 = ko.kpm_1d_tangent(H, H1 - H0, NC, psr)
    fd1 = (ko.kpm_1d_lr(model(t2 + h)[0], NC, psr, psr)
           - ko.kpm_1d_lr(model(t2 - h)[0], NC, psr, psr)) / (2 * h)
    assert relerr(d1, fd1) < 1e-6


def test_oracle_dos_derivatives():
    """test/dos_test.jl:143-193 on the oracle: dE_order = 1 against central
    differences (rtol 1e-5), dE_order = 2 against the five-point stencil
    (rtol 1e-7) and against dos0 at the band centre (rtol 1e-10)."""
    rng = np.random.default_rng(23)
    NC, a, b = 48, 1.7, 0.35
    mu = rng.standard_normal(NC)
    E_grid = b + a * np.array([-0.45, 0.2, 0.55])
    h = 1e-3 * a

    def rho0(E):
        return ko.dos(mu, a, b, E_grid=[E])[1][0]

    stencil = np.array([(-rho0(E + 2 * h) + 16 * rho0(E + h) - 30 * rho0(E)
                         + 16 * rho0(E - h) - rho0(E - 2 * h)) / (12 * h * h) for E in E_grid])
    assert np.allclose(ko.dos_derivative(mu, a, b, E_grid, 2), stencil, rtol=1e-7, atol=0)
    c = ko.dos_derivative(mu, a, b, [b], 2)[0]
    assert abs(c - ko.dos0(mu, a, dE_order=2)) <= 1e-10 * abs(c)
    assert abs(ko.dos0(mu, a) - ko.dos(mu, a, b, E_grid=[b])[1][0]) <= 1e-12 * abs(ko.dos0(mu, a))
    h1 = 1e-4 * a
    fd = (ko.dos(mu, a, b, E_grid=E_grid + h1)[1] - ko.dos(mu, a, b, E_grid=E_grid - h1)[1]) / (2 * h1)
    assert np.allclose(ko.dos_derivative(mu, a, b, E_grid, 1), fd, rtol=1e-5, atol=0)
    assert np.allclose(ko.dos_derivative(mu, a, b, E_grid, 0), ko.dos(mu, a, b, E_grid=E_grid)[1],
                       rtol=1e-13, atol=0)
