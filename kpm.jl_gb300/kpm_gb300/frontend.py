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
