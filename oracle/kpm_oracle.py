"""CPU oracle for the KPM Chebyshev-moment hot path (TEST INFRASTRUCTURE ONLY).

This module is the checker, never the product: only the test suite,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may import it.
It restates, in NumPy/SciPy, the reference algorithms of KPM.jl that the GPU
library replaces, following the reference's index and doubling conventions
line by line.  Every function cites the reference file:line it follows.

Parity pinning: the reference is pure Julia and Julia is not available in
this environment, so the oracle cannot be compared with the reference's own
outputs.  It is pinned instead against the known-answer checks that the
reference's test suite uses (dense Chebyshev-matrix references, exact
diagonalisation, the quantized Haldane Hall conductance, the analytic 1D-chain
DOS and the DOS sum rule); see ``tests/test_oracle_pinning.py``.  Probe
vectors are always passed explicitly, because Julia's Xoshiro stream cannot be
reproduced here.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def _csr(H):
    if sp.issparse(H):
        return sp.csr_matrix(H, dtype=np.complex128)
    return np.asarray(H, dtype=np.complex128)


def normalize_by_col(psi: np.ndarray, centering: bool = False) -> None:
    """In-place column normalisation; no mean-centring by default.

    Follows ``src/utils/vectors.jl:14-19``.
    """
    for i in range(psi.shape[1]):
        col = psi[:, i]
        if centering:
            col -= col.mean()
        col /= np.linalg.norm(col)


def random_phase_vectors(rng: np.random.Generator, NH: int, NR: int) -> np.ndarray:
    """exp(2*pi*i*U[0,1)) columns, unit-normalised (``src/frontend.jl:212-216``).

    Uses a NumPy Generator instead of Julia's Xoshiro; the distribution is the
    same, the stream is not.
    """
    psi = np.exp(rng.random((NH, NR)) * (2j * np.pi))
    normalize_by_col(psi)
    return psi


def columnwise_dot(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """dot(A[:,i], B[:,i]) = sum(conj(A)*B) per column (``src/utils/vectors.jl:103-117``).

    The reference calls BLAS ``dot``; here each column's products are summed
    along a contiguous axis, where NumPy uses pairwise summation, so the
    rounding error grows like log(NH) as with a blocked BLAS kernel (a plain
    running sum over NH rows drifts by ~1e-12 relative over a few hundred
    moments)."""
    P = np.ascontiguousarray((A.conj() * B).T)
    if P.ndim == 1:
        return P.sum()
    return P.sum(axis=1)


def cheb_step(H, Vpp: np.ndarray, Vp: np.ndarray) -> np.ndarray:
    """V_pp <- 2 H V_p - V_pp (``src/utils/chebyshev_iteration.jl:59-75``)."""
    return 2.0 * (H @ Vp) - Vpp


def kpm_1d_doubling(H, NC: int, psi: np.ndarray) -> np.ndarray:
    """Equal-vector moments with the doubling trick; returns mu_all (NR, NC).

    Follows ``src/moment.jl:420-492``: alpha_0 = psi, alpha_1 = H psi,
    mu_0 = <a0|a0>, mu_1 = <a0|a1>; for n = 2..NC/2 after
    alpha_n = 2 H alpha_{n-1} - alpha_{n-2}:
    mu_{2n-2} = 2<a_{n-1}|a_{n-1}> - mu_0, mu_{2n-1} = 2<a_{n-1}|a_n> - mu_1.
    """
    H = _csr(H)
    if NC % 2 != 0:
        raise ValueError("Invalid NC: NC should be even.")
    NH, NR = psi.shape
    mu = np.zeros((NR, NC), dtype=np.complex128)
    a_prev = np.array(psi, dtype=np.complex128)
    a_cur = H @ a_prev
    mu[:, 0] = columnwise_dot(a_prev, a_prev)
    mu[:, 1] = columnwise_dot(a_prev, a_cur)
    for n in range(2, NC // 2 + 1):
        a_next = cheb_step(H, a_prev, a_cur)
        mu[:, 2 * n - 2] = 2.0 * columnwise_dot(a_cur, a_cur) - mu[:, 0]
        mu[:, 2 * n - 1] = 2.0 * columnwise_dot(a_cur, a_next) - mu[:, 1]
        a_prev, a_cur = a_cur, a_next
    return mu


def kpm_1d_lr(H, NC: int, psi_l: np.ndarray, psi_r: np.ndarray) -> np.ndarray:
    """Independent bra/ket moments mu[i, n] = <psil_i|T_n(H) psir_i> (NR, NC).

    Follows ``src/moment.jl:498-556`` (full NC-step recurrence, odd NC allowed).
    """
    H = _csr(H)
    if NC < 2:
        raise ValueError("Invalid NC: NC should be at least 2.")
    NH, NR = psi_r.shape
    mu = np.zeros((NR, NC), dtype=np.complex128)
    a_prev = np.array(psi_r, dtype=np.complex128)
    a_cur = H @ a_prev
    mu[:, 0] = columnwise_dot(psi_l, a_prev)
    mu[:, 1] = columnwise_dot(psi_l, a_cur)
    for n in range(2, NC):
        a_next = cheb_step(H, a_prev, a_cur)
        mu[:, n] = columnwise_dot(psi_l, a_next)
        a_prev, a_cur = a_cur, a_next
    return mu


def kpm_1d(H, NC: int, NR: int, psi_in=None, psi_in_l=None, psi_in_r=None,
           force_norm: bool = False, avg_output: bool = True):
    """Wrapper semantics of ``src/moment.jl:339-418`` (explicit probes only)."""
    lr = psi_in is None
    if lr:
        if psi_in_l is None or psi_in_r is None:
            raise ValueError("must set both psi_in_l and psi_in_r or neither")
        if force_norm:
            normalize_by_col(psi_in_l)
            normalize_by_col(psi_in_r)
        mu_all = kpm_1d_lr(H, NC, psi_in_l, psi_in_r)
    else:
        if force_norm:
            normalize_by_col(psi_in)
        mu_all = kpm_1d_doubling(H, NC, psi_in)
    if avg_output:
        avg = mu_all.sum(axis=0) / NR
        return avg if lr else avg.real
    return mu_all


def kpm_2d_blocking(NH: int, NR: int, NC: int, workspace_bytes, arr_size="auto",
                    right_block="auto"):
    """Block-size choice of ``src/moment.jl:759-810``; returns (K_left, K_right, bytes)."""
    if NH <= 0 or NR <= 0 or NC < 2:
        raise ValueError("bad sizes")
    block = NH * NR * 16
    budget = int(workspace_bytes)
    if budget < 0:
        raise ValueError("workspace_bytes must be nonnegative")
    if right_block == "auto":
        K_right = min(NC, 16)
    elif int(right_block) >= 1:
        K_right = int(right_block)
    else:
        raise ValueError("right_block must be auto or a positive integer")
    base = (K_right + 7) * block
    per_left = block + K_right * 16
    if arr_size == "auto":
        K_left_max = (budget - base) // per_left
        if K_left_max < 2:
            raise ValueError("workspace_bytes cannot fit the minimum kpm_2d workspace")
        K_left = min(K_left_max, NC)
    elif int(arr_size) >= 2:
        K_left = int(arr_size)
    else:
        raise ValueError("arr_size must be auto or an integer at least 2")
    return K_left, K_right, base + K_left * per_left


def kpm_2d(H, Ja, Jb, NC: int, psi_l: np.ndarray, psi_r: np.ndarray, K_left: int,
           K_right: int, moment_parity: str = "NONE", mn_sym: bool = False) -> np.ndarray:
    """Blocked 2D moments mu[n, m] (NC, NC) following ``src/moment.jl:987-1088``.

    Left chain T_{m}(H) psi_l in rings of K_left slots (``:1013-1031, :1075``),
    right chain Jb T_n(H) Ja psi_r recomputed per left block from n = 1
    (``:1034-1052``), block product mu_b = R^H L / NR (``:1055-1061``),
    mu[n, m] += conj(mu_b) under the (n+m) parity mask (``:1063-1072``),
    then the mn_sym symmetrisation (``:1078-1086``).
    """
    if moment_parity not in ("NONE", "ODD", "EVEN"):
        raise ValueError(f"moment_parity={moment_parity} not understood.")
    H, Ja, Jb = _csr(H), _csr(Ja), _csr(Jb)
    NH, NR = psi_r.shape
    if K_left < 2 or K_right < 1:
        raise ValueError("bad blocking")
    mu = np.zeros((NC, NC), dtype=np.complex128)
    left = [None] * K_left
    left[0] = np.array(psi_l, dtype=np.complex128)
    left[1] = H @ left[0]
    Jpsi0 = Ja @ psi_r
    reps = -(-NC // K_left)
    for rep in range(1, reps + 1):
        m1 = (rep - 1) * K_left + 1
        m2 = min(rep * K_left, NC)
        rep_size = m2 - m1 + 1
        for i in range(3, rep_size + 1):
            left[i - 1] = 2.0 * (H @ left[i - 2]) - left[i - 3]
        L = np.stack([v.reshape(-1, order="F") for v in left[:rep_size]], axis=1)
        nmax = m2 if mn_sym else NC
        ring = [None, None, None]
        for n1 in range(1, nmax + 1, K_right):
            n2 = min(n1 + K_right - 1, nmax)
            cols = []
            for n in range(n1, n2 + 1):
                if n == 1:
                    ring[0] = Jpsi0.copy()
                elif n == 2:
                    ring[1] = H @ Jpsi0
                else:
                    i_, ip, ipp = (n - 1) % 3, (n - 2) % 3, (n - 3) % 3
                    ring[i_] = 2.0 * (H @ ring[ip]) - ring[ipp]
                cols.append((Jb @ ring[(n - 1) % 3]).reshape(-1, order="F"))
            R = np.stack(cols, axis=1)
            mub = (R.conj().T @ L) / NR
            for jm in range(rep_size):
                m = m1 + jm
                for jn in range(n2 - n1 + 1):
                    n = n1 + jn
                    keep = (moment_parity == "NONE"
                            or (moment_parity == "ODD" and (m + n) % 2 == 1)
                            or (moment_parity == "EVEN" and (m + n) % 2 == 0))
                    if keep:
                        mu[n - 1, m - 1] += np.conj(mub[jn, jm])
        if rep < reps:
            a = 2.0 * (H @ left[K_left - 1]) - left[K_left - 2]
            b = 2.0 * (H @ a) - left[K_left - 1]
            left[0], left[1] = a, b
    if mn_sym:
        for m in range(NC):
            for n in range(m + 1, NC):
                mu[m, n] = mu[m, n].real
                mu[n, m] = mu[m, n]
    return mu


# ---------------------------------------------------------------- references
def chebyshev_matrices(H: np.ndarray, NC: int):
    """Dense T_n(H), n = 0..NC-1 (``test/kpm2d_blocking_test.jl:25-35``)."""
    H = np.asarray(H.toarray() if sp.issparse(H) else H, dtype=np.complex128)
    N = H.shape[0]
    T = [np.eye(N, dtype=np.complex128)]
    if NC > 1:
        T.append(H.copy())
    for n in range(2, NC):
        T.append(2.0 * H @ T[n - 1] - T[n - 2])
    return T


def kpm2d_dense_reference(H, Ja, Jb, psi_l, psi_r, NC):
    """mu[n, m] = sum_i <T_m psil_i | Jb T_n Ja psir_i> / NR (``test/kpm2d_blocking_test.jl:37-45``)."""
    dense = lambda M: np.asarray(M.toarray() if sp.issparse(M) else M, dtype=np.complex128)
    Ja, Jb = dense(Ja), dense(Jb)
    T = chebyshev_matrices(H, NC)
    NR = psi_l.shape[1]
    Lv = [T[m] @ psi_l for m in range(NC)]
    Rv = [Jb @ T[n] @ Ja @ psi_r for n in range(NC)]
    mu = np.zeros((NC, NC), dtype=np.complex128)
    for m in range(NC):
        for n in range(NC):
            mu[n, m] = np.sum(Lv[m].conj() * Rv[n]) / NR
    return mu


def kpm_1d_current(H, Ja, NC: int, psi: np.ndarray) -> np.ndarray:
    """mu[i, n] = <Ja^dagger psi_i | T_n(H) psi_i> (NR, NC) (``src/moment.jl:656-714``)."""
    H = _csr(H)
    Jd = sp.csr_matrix(_csr(Ja)).conj().T.tocsr()
    bra = Jd @ np.asarray(psi, dtype=np.complex128)
    return kpm_1d_lr(H, NC, bra, psi)


def kpm_3d(H, Ja, Jb, Jc, NC: int, psi_l: np.ndarray, psi_r: np.ndarray) -> np.ndarray:
    """mu[:, :, p] = kpm_2d(H, Jc, Jb; psi_l, T_p(H) Ja psi_r) (``src/moment.jl:1105-1228``)."""
    H = _csr(H)
    v_prev = _csr(Ja) @ np.asarray(psi_r, dtype=np.complex128)
    mu = np.zeros((NC, NC, NC), dtype=np.complex128)
    v_cur = None
    for p in range(NC):
        if p == 0:
            v = v_prev
        elif p == 1:
            v_cur = H @ v_prev
            v = v_cur
        else:
            v_prev, v_cur = v_cur, cheb_step(H, v_prev, v_cur)
            v = v_cur
        mu[:, :, p] = kpm_2d(H, Jc, Jb, NC, psi_l, v, NC, min(NC, 16))
    return mu


def chebyshev_action(H, V: np.ndarray, C: np.ndarray) -> np.ndarray:
    """out[:, :, k] = sum_n C[n, k] T_{n-1}(H) V, coefficients verbatim
    (``src/utils/chebyshev_action.jl:47-122``); V (NH, NR), C (NC, K)."""
    H = _csr(H)
    V = np.asarray(V, dtype=np.complex128)
    C = np.asarray(C, dtype=np.complex128)
    NH, NR = V.shape
    NC, K = C.shape
    out = np.zeros((NH, NR, K), dtype=np.complex128)
    a_prev = V.copy()
    out += a_prev[:, :, None] * C[0][None, None, :]
    if NC == 1:
        return out
    a_cur = H @ a_prev
    out += a_cur[:, :, None] * C[1][None, None, :]
    for n in range(2, NC):
        a_prev, a_cur = a_cur, cheb_step(H, a_prev, a_cur)
        out += a_cur[:, :, None] * C[n][None, None, :]
    return out


# ------------------------------------------------------------ reconstruction
def hn(n):
    """h_0 = 1, h_n = 2 (``src/kernels/kernels.jl:2``)."""
    n = np.asarray(n)
    return np.where(n != 0, 2.0, 1.0)


def jackson_kernel(n, N):
    """Jackson damping g_n (``src/kernels/jackson_kernel.jl:7-8``)."""
    n = np.asarray(n, dtype=np.float64)
    c = np.pi / (N + 1)
    g = ((N + 1 - n) * np.cos(c * n) + np.sin(c * n) / np.tan(c)) / (N + 1)
    return g * (n < N)


def lorentz_kernels(lam: float):
    """sinh(lam(1-n/N))/sinh(lam) (``src/kernels/lorentz_kernel.jl:10-18``)."""
    if not lam > 0:
        raise ValueError("lambda must be positive")
    return lambda n, N: np.sinh(lam * (1 - np.asarray(n, dtype=np.float64) / N)) / np.sinh(lam)


def chebyshev_lin_trans(x, mu_tilde):
    """sum_n mu~_n T_n(x) with T_n(x) = cos(n acos x) (``src/utils/chebyshev_lintrans.jl:6-27``)."""
    n = np.arange(len(mu_tilde))
    T = np.cos(np.outer(np.arccos(x), n))
    return T @ mu_tilde


def dos(mu, a, b=0.0, E_grid=None, N_tilde=0, E_range=None, NC=0, kernel=jackson_kernel):
    """rho(E) = sum_n h_n g_n mu_n T_n(x) / (a pi sqrt(1-x^2)) (``src/applications/dos.jl:76-161``)."""
    mu = np.asarray(mu)
    NC = len(mu) if NC == 0 else min(NC, len(mu))
    if E_grid is None:
        N_tilde = NC * 2 if N_tilde == 0 else N_tilde
        if E_range is None:
            E_range = [b - 0.99 * a, b + 0.99 * a]
        E_grid = np.arange(N_tilde + 1) * (E_range[1] - E_range[0]) / N_tilde + E_range[0]
    E_grid = np.asarray(E_grid, dtype=np.float64)
    rho = np.zeros_like(E_grid)
    idx = np.abs(E_grid - b) < a
    x = (E_grid[idx] - b) / a
    n = np.arange(NC)
    mut = mu[:NC] * kernel(n, NC) * hn(n)
    r = chebyshev_lin_trans(x, mut)
    rho[idx] = np.real(r / (a * np.pi * np.sqrt(1 - x ** 2)))
    return E_grid, rho


# Truncated Taylor series ("jets") f(E + h) = sum_k f[k] h^k, the arithmetic
# that nested forward-mode derivatives perform; used to restate the
# dE_order >= 1 branch of ``src/applications/dos.jl:128-139`` (ForwardDiff
# through ``_dos_single``, i.e. through cos(n acos x) and a pi sqrt(1 - x^2)).
def _jet_mul(f, g):
    K = len(f) - 1
    return [sum(f[j] * g[k - j] for j in range(k + 1)) for k in range(K + 1)]


def _jet_div(f, g):
    K = len(f) - 1
    r = []
    for k in range(K + 1):
        r.append((f[k] - sum(g[j] * r[k - j] for j in range(1, k + 1))) / g[0])
    return r


def _jet_sqrt(u):
    K = len(u) - 1
    s = [np.sqrt(u[0])]
    for k in range(1, K + 1):
        s.append((u[k] - sum(s[j] * s[k - j] for j in range(1, k))) / (2 * s[0]))
    return s


def _jet_integral_from_derivative(dv, v0):
    """v with v' = dv (jets): v[k] = dv[k-1] / k."""
    return [v0] + [dv[k - 1] / k for k in range(1, len(dv) + 1)]


def _jet_cos_sin(w):
    """cos(w), sin(w) jets from c' = -s w', s' = c w'."""
    K = len(w) - 1
    c, s = [np.cos(w[0])], [np.sin(w[0])]
    for k in range(1, K + 1):
        c.append(-sum(j * w[j] * s[k - j] for j in range(1, k + 1)) / k)
        s.append(sum(j * w[j] * c[k - j] for j in range(1, k + 1)) / k)
    return c, s


def dos_derivative(mu, a, b, E_grid, dE_order: int, NC=0, kernel=jackson_kernel):
    """d^k rho/dE^k of ``dos`` at each energy (``src/applications/dos.jl:128-139``)."""
    mu = np.asarray(mu)
    NC = len(mu) if NC == 0 else min(NC, len(mu))
    n = np.arange(NC)
    mut = np.real(mu[:NC]) * kernel(n, NC) * hn(n)
    E_grid = np.asarray(E_grid, dtype=np.float64)
    out = np.zeros_like(E_grid)
    K = int(dE_order)
    for i, E in enumerate(E_grid):
        if not abs(E - b) < a:
            continue
        x = [(E - b) / a, 1.0 / a] + [0.0] * (K - 1) if K >= 1 else [(E - b) / a]
        u = _jet_mul(x, x)
        u = [1.0 - u[0]] + [-v for v in u[1:]]
        sq = _jet_sqrt(u)
        # acos(x): derivative -x' / sqrt(1 - x^2)
        dth = _jet_div([-v for v in x[1:]] + [0.0], sq)[:K] if K >= 1 else []
        th = _jet_integral_from_derivative(dth, np.arccos(x[0]))
        c, _ = _jet_cos_sin([n * t for t in th])          # jets of cos(n theta), vectorised in n
        S = [float(np.dot(mut, ck)) for ck in c]
        rho = _jet_div(S, [a * np.pi * v for v in sq])
        out[i] = math.factorial(K) * rho[K]
    return out


def dos0(mu, a, NC=0, kernel=jackson_kernel, dE_order: int = 0):
    """DOS or its second energy derivative at x = 0 from the closed forms of
    ``src/applications/dos.jl:166-200``."""
    mu = np.real(np.asarray(mu))
    NC = len(mu) if NC == 0 else min(NC, len(mu))
    n0, n2 = np.arange(0, NC, 4), np.arange(2, NC, 4)
    t0 = mu[n0] * hn(n0) * kernel(n0, NC)
    t2 = mu[n2] * hn(n2) * kernel(n2, NC)
    if dE_order == 0:
        return (t0.sum() - t2.sum()) / (a * np.pi)
    if dE_order == 2:
        return ((t0 * (1 - n0 ** 2.0)).sum() + (t2 * (n2 ** 2.0 - 1)).sum()) / (a ** 3 * np.pi)
    raise ValueError(f"unimplemented for derivative of order {dE_order}.")


def gausschebyshevt(n: int):
    """Gauss-Chebyshev (first kind) nodes cos((2k-1)pi/2n) and weights pi/n."""
    k = np.arange(n, 0, -1)
    return np.cos((2 * k - 1) * np.pi / (2 * n)), np.full(n, np.pi / n)


def fermi_functions(Ef: float, beta: float):
    """T=0 step with weight 1/2 at Ef, or Fermi-Dirac (``src/utils/physics.jl:15-39``)."""
    if math.isinf(beta):
        return lambda x: ((x < Ef).astype(float) + (x <= Ef).astype(float)) / 2
    return lambda x: 1.0 / (np.exp((x - Ef) * beta) + 1.0)


def mu2d_apply_kernel_and_h(mu, NC, kernel=jackson_kernel):
    """mu~[n,m] = mu[n,m] g_n h_n g_m h_m (``src/kernels/kernels.jl:14-50``)."""
    n = np.arange(NC)
    kv = kernel(n, NC) * hn(n)
    return np.asarray(mu[:NC, :NC], dtype=np.complex128) * kv[:, None] * kv[None, :]


def kubo_bastin_cond(mu2d, a, Ef, b=0.0, NH=None, area=None, beta=math.inf,
                     kernel=jackson_kernel, NC=None, quad_N=None, edge_cutoff=1e-3):
    """sigma_ab(Ef) in e^2/h via Gauss-Chebyshev quadrature (``src/applications/conductivity.jl:101-157``)."""
    if not a > 0 or not area > 0 or not NH > 0:
        raise ValueError("a, area and NH must be positive")
    NC = min(NC or mu2d.shape[0], mu2d.shape[0], mu2d.shape[1])
    quad_N = quad_N or 8 * NC
    mut = mu2d_apply_kernel_and_h(mu2d, NC, kernel)
    ff = fermi_functions(float(Ef), float(beta))
    nodes, weights = gausschebyshevt(quad_N)
    fv = ff(a * nodes + b)
    keep = (np.abs(nodes) < 1 - edge_cutoff) & (fv != 0)
    if not keep.any():
        return 0.0
    x = nodes[keep]
    phi = weights[keep] * fv[keep] / (1 - x ** 2) ** 1.5
    ns = np.arange(NC)[:, None]
    th = np.arccos(x)[None, :]
    s = np.sqrt(1 - x ** 2)[None, :]
    C = np.cos(ns * th)
    E = np.exp(1j * ns * th)
    WM = (x[None, :] - 1j * ns * s) * E
    WN = (x[None, :] + 1j * ns * s) * np.conj(E)
    U = mut.T @ C
    V = mut @ C
    acc = np.sum(phi[None, :] * (U * WM)) + np.sum(phi[None, :] * (V * WN))
    return -2 * NH / (area * a ** 2) * acc.real


def normalizeH(H, eps: float = 0.1, fixed_a: float = 0.0, center: bool = False):
    """Rescale into (-1, 1) via an ARPACK edge estimate (``src/utils/external.jl:41-76``)."""
    Hs = sp.csr_matrix(H, dtype=np.complex128)
    dev = abs(Hs - Hs.conj().T).max() if Hs.nnz else 0.0
    if dev != 0 and not dev <= math.sqrt(np.finfo(float).eps) * abs(Hs).max():
        raise ValueError("normalizeH: H must be Hermitian")
    if fixed_a != 0:
        if center:
            raise ValueError("center=true is incompatible with fixed_a")
        return float(fixed_a), 0.0, Hs / fixed_a
    if center:
        emax = spla.eigsh(Hs, k=1, which="LA", tol=1e-3, maxiter=300 * Hs.shape[0],
                          return_eigenvectors=False)[0]
        emin = spla.eigsh(Hs, k=1, which="SA", tol=1e-3, maxiter=300 * Hs.shape[0],
                          return_eigenvectors=False)[0]
        a = (emax - emin) / (2 - eps)
        b = (emax + emin) / 2
        return float(a), float(b), (Hs - b * sp.identity(Hs.shape[0], format="csr")) / a
    emax = abs(spla.eigsh(Hs, k=1, which="LM", tol=1e-3, maxiter=300 * Hs.shape[0],
                          return_eigenvectors=False)[0])
    a = 2 * emax / (2 - eps)
    return float(a), 0.0, Hs / a


# ------------------------------------------------------ directional derivatives
# No reference counterpart: KPM.jl obtains these by pushing ForwardDiff duals
# through the recurrences of ``src/moment.jl:420-556`` and ``:887-1088``.  The
# restatement below is the dual-number arithmetic written out: every
# recurrence vector v carries its tangent dv along H + t dH, updated by the
# product rule.
def _tangent_chain(H, dH, v0, dv0, NC: int):
    """Vectors T_n(H) v0 and their tangents for n = 0..NC-1 (dual recurrence of
    ``src/chebyshev_iteration.jl:59-75``)."""
    v = [v0, H @ v0]
    dv = [dv0, dH @ v0 + H @ dv0]
    for n in range(2, NC):
        v.append(2.0 * (H @ v[n - 1]) - v[n - 2])
        dv.append(2.0 * (dH @ v[n - 1] + H @ dv[n - 1]) - dv[n - 2])
    return v[:NC], dv[:NC]


def kpm_1d_tangent(H, dH, NC: int, psi: np.ndarray) -> np.ndarray:
    """d/dt <psi_i|T_n(H + t dH)|psi_i> at t = 0, shape (NR, NC)."""
    H, dH = _csr(H), _csr(dH)
    psi = np.asarray(psi, dtype=np.complex128)
    # the dual recurrence of _tangent_chain, keeping only the last two vectors
    out = np.zeros((psi.shape[1], NC), dtype=np.complex128)
    v_pp, v_p = psi, H @ psi
    dv_pp, dv_p = np.zeros_like(psi), dH @ psi
    if NC > 1:
        out[:, 1] = columnwise_dot(psi, dv_p)
    for n in range(2, NC):
        v_n = 2.0 * (H @ v_p) - v_pp
        dv_n = 2.0 * (dH @ v_p + H @ dv_p) - dv_pp
        out[:, n] = columnwise_dot(psi, dv_n)
        v_pp, v_p, dv_pp, dv_p = v_p, v_n, dv_p, dv_n
    return out


def kpm_2d_tangent(H, dH, Ja, dJa, Jb, dJb, NC: int, psi_l, psi_r) -> np.ndarray:
    """d/dt of the kpm_2d moments mu[n, m] = sum_i <T_m psil_i|Jb T_n Ja psir_i>/NR
    along (H, Ja, Jb) + t (dH, dJa, dJb) at t = 0 (orientation of
    ``src/moment.jl:1055-1070``), shape (NC, NC)."""
    H, dH, Ja, Jb = _csr(H), _csr(dH), _csr(Ja), _csr(Jb)
    NH, NR = np.asarray(psi_r).shape
    zero = sp.csr_matrix((NH, NH), dtype=np.complex128)
    dJa = zero if dJa is None else _csr(dJa)
    dJb = zero if dJb is None else _csr(dJb)
    pl = np.asarray(psi_l, dtype=np.complex128)
    pr = np.asarray(psi_r, dtype=np.complex128)
    L, dL = _tangent_chain(H, dH, pl, np.zeros_like(pl), NC)
    S, dS = _tangent_chain(H, dH, Ja @ pr, dJa @ pr, NC)
    R = [Jb @ s for s in S]
    dR = [dJb @ s + Jb @ ds for s, ds in zip(S, dS)]
    Lm = np.stack([x.reshape(-1, order="F") for x in L], axis=1)
    dLm = np.stack([x.reshape(-1, order="F") for x in dL], axis=1)
    Rn = np.stack([x.reshape(-1, order="F") for x in R], axis=1)
    dRn = np.stack([x.reshape(-1, order="F") for x in dR], axis=1)
    # dmu[n, m] = (<dL_m|R_n> + <L_m|dR_n>) / NR
    return (Rn.T @ dLm.conj() + dRn.T @ Lm.conj()) / NR
