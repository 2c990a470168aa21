"""Typed front end mirroring ``src/frontend.jl`` of KPM.jl.

``RescaledHamiltonian`` carries the rescaling provenance (a, b) of
``H_norm = (H - b I)/a``; ``dos_moments`` / ``cond_moments`` validate their
inputs exactly as the reference does and delegate to the GPU moment engine.
``h.H`` may be a SciPy sparse matrix or a ``GB300Operator`` (already resident
on the device, reused across calls).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Any

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from ._native import KPMArgumentError
from .moment import kpm_1d, kpm_2d, normalize_by_col
from .operator import GB300Operator


@dataclass(frozen=True)
class RescaledHamiltonian:
    """``H`` with spectrum inside (-1, 1); ``a``, ``b`` in physical units (``src/frontend.jl:11-15``)."""

    H: Any
    a: float
    b: float

    def __repr__(self):
        return f"RescaledHamiltonian(NH={self.H.shape[0]}, a={self.a}, b={self.b})"


@dataclass(frozen=True)
class DosMoments:
    """DOS moments with provenance (``src/frontend.jl:32-44``)."""

    mu: np.ndarray
    a: float
    b: float
    NH: int
    NR: int

    def __post_init__(self):
        if not (self.NH > 0 and self.NR > 0):
            raise KPMArgumentError(
                f"DosMoments: NH and NR must be positive (got NH={self.NH}, NR={self.NR})")


@dataclass(frozen=True)
class ConductivityMoments:
    """kpm_2d moment matrix with provenance (``src/frontend.jl:53-72``)."""

    mu: np.ndarray
    a: float
    b: float
    NH: int
    NR: int

    def __post_init__(self):
        if self.mu.ndim != 2 or self.mu.shape[0] != self.mu.shape[1]:
            raise KPMArgumentError(
                f"ConductivityMoments: the moment matrix must be square (got {self.mu.shape})")
        if not (self.NH > 0 and self.NR > 0):
            raise KPMArgumentError(
                f"ConductivityMoments: NH and NR must be positive (got NH={self.NH}, NR={self.NR})")


def _hermitian_check(H):
    dev = abs(H - H.conj().T).max() if H.nnz else 0.0
    scale = abs(H).max() if H.nnz else 0.0
    if dev != 0 and not dev <= math.sqrt(np.finfo(float).eps) * scale:
        raise KPMArgumentError(f"normalizeH: H must be Hermitian (max |H - H'| = {dev}).")


def normalizeH(H, eps: float = 0.1, fixed_a: float = 0.0, center: bool = False):
    """ARPACK edge estimate and rescaling (``src/utils/external.jl:41-76``).

    Returns ``(a, H_norm)`` or, with ``center=True``, ``(a, b, H_norm)``.
    Host-side input preparation (ARPACK, tol 1e-3), as in the reference.
    """
    H = sp.csr_matrix(H, dtype=np.complex128)
    _hermitian_check(H)
    if fixed_a != 0:
        if center:
            raise KPMArgumentError(
                "normalizeH: center=true is incompatible with fixed_a — the center shift is "
                "derived from the spectral edges, which fixed_a skips.")
        return float(fixed_a), (H / fixed_a).tocsc()
    n = H.shape[0]
    kw = dict(k=1, tol=1e-3, maxiter=max(300, 30 * n), return_eigenvectors=False)
    if n <= 2:
        ev = np.linalg.eigvalsh(H.toarray())
        emax, emin, elm = ev.max(), ev.min(), np.abs(ev).max()
    if center:
        if n > 2:
            emax = spla.eigsh(H, which="LA", **kw)[0]
            emin = spla.eigsh(H, which="SA", **kw)[0]
        a = (emax - emin) / (2 - eps)
        b = (emax + emin) / 2
        return float(a), float(b), ((H - b * sp.identity(n, format="csr")) / a).tocsc()
    if n > 2:
        elm = abs(spla.eigsh(H, which="LM", **kw)[0])
    a = 2 * elm / (2 - eps)
    return float(a), (H / a).tocsc()


def rescale(H, *, center: bool = False, eps: float = 0.1, fixed_a: float = 0.0):
    """Rescale Hermitian ``H`` keeping its provenance (``src/frontend.jl:149-161``)."""
    if center:
        a, b, Hn = normalizeH(H, eps=eps, fixed_a=fixed_a, center=True)
    else:
        a, Hn = normalizeH(H, eps=eps, fixed_a=fixed_a)
        b = 0.0
    if not (math.isfinite(a) and math.isfinite(b)):
        raise KPMArgumentError(f"rescale: a and b must be finite as Float64 (got a={a}, b={b})")
    return RescaledHamiltonian(Hn, float(a), float(b))


def random_phase_vectors(rng: np.random.Generator, NH: int, NR: int) -> np.ndarray:
    """Unit-norm random-phase probes, no mean centring (``src/frontend.jl:212-216``)."""
    psi = np.exp(rng.random((NH, NR)) * (2j * np.pi))
    normalize_by_col(psi)
    return psi


def _probe_args(h, NR, rng, psi_in):
    if rng is not None and psi_in is not None:
        raise KPMArgumentError("pass either rng or psi_in, not both")
    NH = h.H.shape[0]
    NR = int(NR)
    if psi_in is not None:
        psi_in = np.asarray(psi_in)
        if psi_in.shape[0] != NH:
            raise KPMArgumentError(f"psi_in has {psi_in.shape[0]} rows; expected {NH}")
        NR = psi_in.shape[1]
    elif rng is not None:
        psi_in = random_phase_vectors(rng, NH, NR)
    return NH, NR, psi_in


def dos_moments(h: RescaledHamiltonian, *, NC: int = 1024, NR: int = 12, rng=None,
                psi_in=None, verbose: int = 0, precision: str = "fp64") -> DosMoments:
    """DOS moments of ``h`` (``src/frontend.jl:225-259``)."""
    if NC % 2 != 0:
        raise KPMArgumentError(
            "kpm_1d computes NC moments from NC/2 recurrence steps; NC must be even")
    NH, NR, psi_in = _probe_args(h, NR, rng, psi_in)
    if psi_in is None:
        psi_in = random_phase_vectors(np.random.default_rng(), NH, NR)
    mu = kpm_1d(h.H, int(NC), NR, NH, psi_in=psi_in, verbose=verbose, precision=precision)
    return DosMoments(mu, h.a, h.b, NH, NR)


def cond_moments(h: RescaledHamiltonian, Ja, Jb, *, NC: int = 256, NR: int = 8, rng=None,
                 psi_in=None, arr_size="auto", right_block="auto", workspace_bytes="auto",
                 precision: str = "fp64", contraction: str = "fp64",
                 **kwargs) -> ConductivityMoments:
    """Conductivity moments for ``h`` and currents ``Ja``, ``Jb`` (``src/frontend.jl:270-327``).

    The currents follow the bond convention (J_a)_ij = H_ij (r_i - r_j)_a of the
    original, unrescaled H.
    """
    NH, NR, psi_in = _probe_args(h, NR, rng, psi_in)
    if psi_in is None:
        psi_in = random_phase_vectors(np.random.default_rng(), NH, NR)
    mu = kpm_2d(h.H, Ja, Jb, int(NC), NR, NH, psi_in=psi_in, arr_size=arr_size,
                right_block=right_block, workspace_bytes=workspace_bytes, precision=precision,
                contraction=contraction, **kwargs)
    return ConductivityMoments(mu, h.a, h.b, NH, NR)


def on_device(h: RescaledHamiltonian) -> RescaledHamiltonian:
    """Same Hamiltonian with ``H`` uploaded once as a ``GB300Operator``."""
    if isinstance(h.H, GB300Operator):
        return h
    return RescaledHamiltonian(GB300Operator(h.H), h.a, h.b)


def jackson_kernel(n, N):
    """Jackson damping factors g_n for an N-moment expansion
    (``src/kernels/jackson_kernel.jl:7-8``)."""
    n = np.asarray(n, dtype=np.float64)
    c = np.pi / (N + 1)
    return ((N + 1 - n) * np.cos(c * n) + np.sin(c * n) / np.tan(c)) / (N + 1) * (n < N)


def dos_basis(NC: int, a: float, b: float, E_grid, kernel=jackson_kernel) -> np.ndarray:
    """Matrix Phi (len(E_grid), NC) with rho(E_e) = Phi[e] @ mu.

    The reconstruction of ``src/applications/dos.jl:76-161``
    (rho(E) = sum_n h_n g_n mu_n T_n(x) / (a pi sqrt(1 - x^2)), x = (E - b)/a,
    zero outside |E - b| < a) written as a linear map, so that a loss on the
    DOS turns into moment weights for :func:`kpm_1d_grad`:
    g = Phi.T @ dL/drho.
    """
    E = np.asarray(E_grid, dtype=np.float64)
    n = np.arange(int(NC))
    w = np.asarray(kernel(n, int(NC)), dtype=np.float64) * np.where(n != 0, 2.0, 1.0)
    Phi = np.zeros((E.size, int(NC)))
    inside = np.abs(E - b) < a
    x = (E[inside] - b) / a
    Phi[inside] = np.cos(np.outer(np.arccos(x), n)) * w / (a * np.pi * np.sqrt(1 - x * x))[:, None]
    return Phi


def _damping(kernel, NC: int):
    if kernel is None:
        return None
    g = np.ascontiguousarray(np.broadcast_to(kernel(np.arange(NC), NC), (NC,)), dtype=np.float64)
    return g


def kubo_bastin_cond(mu2D, a: float, Ef, *, b: float = 0.0, NH: int, area: float,
                     beta: float = math.inf, kernel=jackson_kernel, NC: int | None = None,
                     quad_N: int | None = None, edge_cutoff: float = 1e-3):
    """DC conductivity sigma_ab(Ef) in e^2/h (``src/applications/conductivity.jl:101-157``).

    ``mu2D``: NC x NC moments of ``kpm_2d``.  ``Ef`` may be a scalar (returns
    a float, as the reference) or an array of Fermi energies (returns an
    array): the Ef-independent node sums run once on the GPU for all of them.
    """
    import ctypes as C
    from . import _native
    if not a > 0:
        raise KPMArgumentError("kubo_bastin_cond: a must be positive.")
    if not area > 0:
        raise KPMArgumentError("kubo_bastin_cond: area must be positive.")
    if not NH > 0:
        raise KPMArgumentError("kubo_bastin_cond: NH must be positive.")
    mu = np.asfortranarray(mu2D, dtype=np.complex128)
    if mu.ndim != 2:
        raise KPMArgumentError("kubo_bastin_cond: mu2D must be a matrix")
    NCx = min(mu.shape) if NC is None else min(int(NC), *mu.shape)
    quad_N = 8 * NCx if quad_N is None else int(quad_N)
    if quad_N <= 0:
        raise KPMArgumentError("kubo_bastin_cond: quad_N must be positive.")
    if not 0 <= edge_cutoff < 1:
        raise KPMArgumentError("kubo_bastin_cond: edge_cutoff must be in [0, 1).")
    scalar = np.ndim(Ef) == 0
    ef = np.ascontiguousarray(np.atleast_1d(np.asarray(Ef, dtype=np.float64)))
    out = np.empty(ef.size, dtype=np.float64)
    g = _damping(kernel, NCx)
    lib = _native.load()
    rc = lib.kpmgb_kubo_bastin(mu.ctypes.data, mu.shape[0], NCx, float(a), float(b),
                               ef.ctypes.data, ef.size, int(NH), float(area), float(beta),
                               g.ctypes.data if g is not None else None, quad_N,
                               float(edge_cutoff), out.ctypes.data)
    _native.check(rc)
    return float(out[0]) if scalar else out


def kubo_bastin_weights(NC: int, a: float, Ef: float, *, b: float = 0.0, NH: int, area: float,
                        beta: float = math.inf, kernel=jackson_kernel, quad_N: int | None = None,
                        edge_cutoff: float = 1e-3) -> np.ndarray:
    """W (NC, NC) complex with ``kubo_bastin_cond(mu, a, Ef; ...) ==
    Re sum_{n,m} W[n,m] mu[n,m]``: the Kubo-Bastin reconstruction
    (``src/applications/conductivity.jl:101-157``) as a linear functional of
    the moments, i.e. d sigma / d mu, computed on the GPU.  Feed it (times
    dL/dsigma) to :func:`kpm_2d_grad`."""
    import ctypes as C  # noqa: F401
    from . import _native
    if not a > 0:
        raise KPMArgumentError("kubo_bastin_cond: a must be positive.")
    if not area > 0:
        raise KPMArgumentError("kubo_bastin_cond: area must be positive.")
    if not NH > 0:
        raise KPMArgumentError("kubo_bastin_cond: NH must be positive.")
    NC = int(NC)
    quad_N = 8 * NC if quad_N is None else int(quad_N)
    g = _damping(kernel, NC)
    W = np.empty((NC, NC), dtype=np.complex128, order="F")
    lib = _native.load()
    _native.check(lib.kpmgb_kubo_bastin_weights(NC, float(a), float(b), float(Ef), int(NH),
                                                float(area), float(beta),
                                                g.ctypes.data if g is not None else None,
                                                quad_N, float(edge_cutoff), W.ctypes.data))
    return W


def dos(mu_or_H, H_rescale_factor=None, *, b: float = 0.0, E_grid=None, N_tilde: int = 0,
        E_range=None, NC: int = 0, NR: int = 12, kernel=jackson_kernel, dE_order: int = 0,
        fix_normalization: float = 0.0, center: bool = False, rng=None):
    """Density of states (``src/applications/dos.jl:43-161``); returns (E_grid, rho).

    ``dos(mu, a; ...)`` reconstructs from moments on the GPU; ``dos(H; ...)``
    first rescales H (``normalizeH``) and computes NC moments with NR
    random-phase probes.
    """
    from . import _native
    if H_rescale_factor is None:
        H = mu_or_H
        NCm = 1024 if NC == 0 else int(NC)
        if center:
            a, b, Hn = normalizeH(H, fixed_a=fix_normalization, center=True)
        else:
            a, Hn = normalizeH(H, fixed_a=fix_normalization)
            b = 0.0
        NH = Hn.shape[0]
        psi = random_phase_vectors(np.random.default_rng() if rng is None else rng, NH, NR)
        mu = kpm_1d(Hn, NCm, NR, NH, psi_in=psi)
        return dos(mu, a, b=b, E_grid=E_grid, E_range=E_range, N_tilde=N_tilde, kernel=kernel,
                   NC=NCm, dE_order=dE_order)
    mu = np.asarray(mu_or_H)
    if mu.ndim != 1:
        raise KPMArgumentError("The input need to be 1D array")
    a = float(H_rescale_factor)
    if not a > 0:
        raise KPMArgumentError("the rescale factor must be positive")
    if not 0 <= int(dE_order) <= 4:
        raise KPMArgumentError("dos: dE_order must be in 0..4")
    NC = len(mu) if NC == 0 else min(int(NC), len(mu))
    if E_grid is None:
        N_tilde = NC * 2 if N_tilde == 0 else N_tilde
        if E_range is None:
            E_range = [b - 0.99 * a, b + 0.99 * a]
        E_grid = np.arange(N_tilde + 1) * (E_range[1] - E_range[0]) / N_tilde + E_range[0]
    else:
        if E_range is not None:
            raise KPMArgumentError("Should not set `E_grid` and `E_range` simultaneously.")
        if N_tilde != 0 and len(E_grid) != N_tilde:
            raise KPMArgumentError("`N_tilde` does not match with `E_grid`.")
    E = np.ascontiguousarray(E_grid, dtype=np.float64)
    m = np.ascontiguousarray(np.real(mu[:NC]), dtype=np.float64)
    g = _damping(kernel, NC)
    rho = np.empty(E.size, dtype=np.float64)
    lib = _native.load()
    _native.check(lib.kpmgb_dos_derivative(m.ctypes.data, NC, a, float(b),
                                           g.ctypes.data if g is not None else None,
                                           E.ctypes.data, E.size, int(dE_order),
                                           rho.ctypes.data))
    return E, rho


def dos0(mu, H_rescale_factor, *, NC: int = 0, kernel=jackson_kernel, dE_order: int = 0):
    """DOS (``dE_order=0``) or its second energy derivative (``dE_order=2``) at
    the centre of the rescaling, x = 0, from the closed-form values
    T_n(0) = 1, -1, 0 for n = 0, 2, odd (mod 4) and
    d^2/dx^2 [T_n(x)/sqrt(1-x^2)]_{x=0} = (-1)^{n/2} (1 - n^2) for even n
    (``src/applications/dos.jl:166-200``)."""
    a = float(H_rescale_factor)
    if not a > 0:
        raise KPMArgumentError("the rescale factor must be positive")
    mu = np.asarray(mu)
    NC = len(mu) if NC == 0 else min(int(NC), len(mu))
    n0 = np.arange(0, NC, 4)
    n2 = np.arange(2, NC, 4)
    w0 = np.real(mu[n0]) * np.where(n0 != 0, 2.0, 1.0) * kernel(n0, NC)
    w2 = np.real(mu[n2]) * 2.0 * kernel(n2, NC)
    if dE_order == 0:
        return float((w0.sum() - w2.sum()) / (a * np.pi))
    if dE_order == 2:
        return float(((w0 * (1 - n0 ** 2.0)).sum() + (w2 * (n2 ** 2.0 - 1)).sum()) / (a ** 3 * np.pi))
    raise KPMArgumentError(f"unimplemented for derivative of order {dE_order}.")
