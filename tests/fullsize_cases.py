"""Inputs of the benchmark-size parity cases, shared by the GPU tests and by
tests/golden/make_fullsize.py (which computes their oracle references).

Every input is rebuilt from a seed here and on the GPU machine; only the
rescaling (a, b) is read from the fixture, because ARPACK's edge estimate
(tolerance 1e-3) may differ between machines in its last digits and the
moments depend on it.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from kpm_gb300 import models
from oracle import kpm_oracle as ko

# 3D Anderson L=128 periodic (NH = 2,097,152, 7 nonzeros per row), W = 16.5,
# centred rescaling, NC = 4096, NR = 64 random-phase probes: the headline
# kpm_1d workload.  The oracle covers eight of the 64 columns (both halves of
# the 64-column row).
C2 = dict(L=128, W=16.5, NC=4096, NR=64, seed_h=42, seed_psi=7,
          cols=np.array([0, 9, 18, 27, 36, 45, 54, 63]))
# Haldane 256x256 cells x 2 orbitals (NH = 131,072), t1 = 1, t2 = 0.1 i, M = 0,
# NC = 512, NR = 16; sigma_xy at 201 Fermi energies in [-3, 3].
C3 = dict(L=256, t2=0.1, NC=512, NR=16, seed_psi=42, K_left=64, K_right=16,
          Ef=np.linspace(-3.0, 3.0, 201))
# Graphene 128x128 (NH = 32,768), t = 1, onsite N(0, 0.1^2); target DOS from
# a second seeded realisation; NC = 1024, NR = 16, checkpoints every 64 steps;
# L = int_{-0.5}^{0.5} (rho - rho_t)^2 dE on 201 trapezoid nodes.
C5 = dict(L=128, NC=1024, NR=16, a=3.5, seed_h=11, seed_t=12, seed_psi=13, seed_dir=14,
          checkpoint=64, E=np.linspace(-0.5, 0.5, 201))


def rescaled(H, a: float, b: float):
    """(H - b I) / a as CSC complex128, the normalised operator of
    src/frontend.jl:149-161 for a given (a, b)."""
    Hn = (sp.csc_matrix(H, dtype=np.complex128) - b * sp.identity(H.shape[0], format="csc")) / a
    Hn = sp.csc_matrix(Hn)
    Hn.sort_indices()
    return Hn


# Haldane 64x64 cells (NH = 8192), t1 = 1, t2 = 0.2 i, M = 0, NC = 256, NR = 8:
# d sigma_xy(Ef = 0) along the onsite energies (a random direction), t1 and t2.
X1 = dict(L=64, t2=0.2, NC=256, NR=8, seed_psi=5, seed_dir=6, Ef=0.0)


def rescaled_keep(H, a: float, b: float):
    """(H - b I) / a on exactly H's stored pattern (H must store its diagonal),
    so that gradients on the pattern cover every parameter direction."""
    Hn = sp.csc_matrix(H, dtype=np.complex128, copy=True)
    Hn.sort_indices()
    rows = Hn.indices
    cols = np.repeat(np.arange(Hn.shape[1]), np.diff(Hn.indptr))
    diag = rows == cols
    if np.count_nonzero(diag) != Hn.shape[0]:
        raise ValueError("H must store its diagonal")
    Hn.data = Hn.data.copy()
    Hn.data[diag] -= b
    Hn.data /= a
    return Hn


def x1_model():
    """(H, Jx, Jy, area) and the three parameter directions (dH, dJx, dJy) of
    the unrescaled model: random onsite energies, t1, t2 (the builder is linear
    in each)."""
    L, t2 = X1["L"], X1["t2"]
    H, Jx, Jy, area = models.haldane(L, L, t=1.0, t2=t2)
    zero = models.haldane(L, L, t=0.0, t2=0.0)
    d_t1 = models.haldane(L, L, t=1.0, t2=0.0)
    d_t2 = models.haldane(L, L, t=0.0, t2=1.0)
    on = np.random.default_rng(X1["seed_dir"]).standard_normal(H.shape[0])
    dirs = [(sp.diags(on.astype(np.complex128), format="csc"), zero[1], zero[2])]
    for d in (d_t1, d_t2):
        dirs.append(tuple(sp.csc_matrix(d[k] - zero[k]) for k in range(3)))
    return H, Jx, Jy, area, dirs


def x1_probes(NH: int):
    return ko.random_phase_vectors(np.random.default_rng(X1["seed_psi"]), NH, X1["NR"])


def c2_hamiltonian():
    return models.cubic_anderson(C2["L"], W=C2["W"], rng=np.random.default_rng(C2["seed_h"]))


def c2_probes(NH: int):
    return ko.random_phase_vectors(np.random.default_rng(C2["seed_psi"]), NH, C2["NR"])


def c3_model():
    return models.haldane(C3["L"], C3["L"], t=1.0, t2=C3["t2"])


def c3_probes(NH: int):
    return ko.random_phase_vectors(np.random.default_rng(C3["seed_psi"]), NH, C3["NR"])


def c4_members():
    """256 realisations of the 2D Anderson model, L ~ U{24..96}, W ~ U[1, 8],
    each rescaled by 4 + W/2 + 0.1 (a bound on its spectral radius), with 8
    random-phase probes."""
    rng = np.random.default_rng(42)
    Hs, psis = [], []
    for _ in range(256):
        L = int(rng.integers(24, 97))
        W = float(rng.uniform(1.0, 8.0))
        Hs.append((models.square_anderson(L, W=W, rng=rng) / (4.0 + W / 2 + 0.1)).tocsc())
        psis.append(ko.random_phase_vectors(rng, L * L, 8))
    return Hs, psis


def c5_inputs():
    """(H, H_target, psi) of the DOS-window loss, rescaled by a = 3.5 (b = 0)."""
    L, a = C5["L"], C5["a"]
    NH = 2 * L * L
    on = 0.1 * np.random.default_rng(C5["seed_h"]).standard_normal(NH)
    on_t = 0.1 * np.random.default_rng(C5["seed_t"]).standard_normal(NH)
    H = rescaled(models.graphene(L, L, onsite=on), a, 0.0)
    Ht = rescaled(models.graphene(L, L, onsite=on_t), a, 0.0)
    psi = ko.random_phase_vectors(np.random.default_rng(C5["seed_psi"]), NH, C5["NR"])
    return H, Ht, psi


def c5_directions(H):
    """Two Hermitian directions on H's pattern: onsite energies only, and
    nearest-neighbour hoppings only (both real, as the model's parameters)."""
    rng = np.random.default_rng(C5["seed_dir"])
    Hc = sp.coo_matrix(H)
    diag = Hc.row == Hc.col
    d_on = np.where(diag, rng.standard_normal(Hc.nnz), 0.0)
    # one value per bond: symmetrise a random draw over (i, j) and (j, i)
    draw = rng.standard_normal(Hc.nnz)
    D_hop = sp.csc_matrix((np.where(diag, 0.0, draw), (Hc.row, Hc.col)), shape=H.shape)
    D_hop = sp.csc_matrix((D_hop + D_hop.T) / 2)
    D_on = sp.csc_matrix((d_on, (Hc.row, Hc.col)), shape=H.shape)
    out = []
    for D in (D_on, D_hop):
        D = sp.csc_matrix(D, dtype=np.complex128)
        D.sort_indices()
        out.append(D)
    return out


def dos_weights(NC: int, a: float, E):
    """Phi (len(E), NC) with rho(E) = Phi @ mu (src/applications/dos.jl:76-161,
    Jackson kernel, h_n = 1, 2, 2, ...), and trapezoid weights on E."""
    n = np.arange(NC)
    w = ko.jackson_kernel(n, NC) * ko.hn(n)
    x = np.asarray(E) / a
    Phi = np.cos(np.outer(np.arccos(x), n)) * w / (a * np.pi * np.sqrt(1 - x * x))[:, None]
    q = np.full(len(E), E[1] - E[0])
    q[[0, -1]] /= 2
    return Phi, q


def pairing(G, D) -> float:
    """dL along D = sum_k Re(conj(G_k) D_k) over stored entries."""
    Gc, Dc = sp.coo_matrix(G), sp.coo_matrix(D)
    Gd = {(i, j): v for i, j, v in zip(Gc.row, Gc.col, Gc.data)}
    return float(sum((np.conj(Gd.get((i, j), 0.0)) * v).real
                     for i, j, v in zip(Dc.row, Dc.col, Dc.data)))
