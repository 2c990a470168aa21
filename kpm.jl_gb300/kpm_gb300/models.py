"""Tight-binding model builders for the benchmark and test workloads.

Host-side input preparation (not timed).  Each builder follows the lattice
conventions of the reference's own builders, so that moments computed here are
comparable with the reference's tests and benchmarks:

* ``square_anderson``: periodic square lattice, hopping -t on the 4 nearest
  neighbours, onsite uniform[-W/2, W/2]  (``benchmarks/core_bench.jl:35-64``
  for the lattice, ``test/ed_reference.jl:396-441`` for the disorder draw).
* ``cubic_anderson``: periodic simple-cubic L^3 lattice, site index
  x + L(y-1) + L^2(z-1), hops -t along +x, +y, +z and their conjugates,
  onsite W*(U[0,1)-0.5), bond currents from minimum-image displacements
  (``test/ed_reference.jl:396-441``).
* ``haldane``: Haldane model on an Lx x Ly honeycomb torus, NN hopping -t,
  NNN t2*e^{+-i phi}, staggered mass, bond currents (J_a)_ij = H_ij (r_i-r_j)_a
  (``test/ed_reference.jl:69-141``).
* ``graphene``: honeycomb torus with onsite energies, hopping -t
  (``examples/GrapheneModel.jl:33-105``).

All matrices are returned as ``scipy.sparse.csc_matrix`` (complex128), the
storage order Julia's ``SparseMatrixCSC`` uses, which is what the C ABI takes.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp


def _coo_csc(rows, cols, vals, n):
    m = sp.coo_matrix((np.asarray(vals, dtype=np.complex128), (np.asarray(rows), np.asarray(cols))),
                      shape=(n, n))
    m = m.tocsc()
    m.sum_duplicates()
    m.sort_indices()
    return m


def square_anderson(L: int, t: float = 1.0, W: float = 0.0, rng=None, currents: bool = False):
    """Periodic L x L square lattice with onsite disorder uniform[-W/2, W/2]."""
    rng = np.random.default_rng(0) if rng is None else rng
    N = L * L
    idx = np.arange(N)
    x, y = idx % L, idx // L
    rows, cols, vals, dxs, dys = [], [], [], [], []
    for ddx, ddy in ((1, 0), (-1, 0), (0, 1), (0, -1)):
        j = (x + ddx) % L + L * ((y + ddy) % L)
        rows.append(idx)
        cols.append(j)
        vals.append(np.full(N, -t, dtype=np.complex128))
        # displacement r_i - r_j (minimum image)
        dxs.append(np.full(N, -ddx, dtype=np.float64))
        dys.append(np.full(N, -ddy, dtype=np.float64))
    onsite = W * (rng.random(N) - 0.5)
    rows.append(idx)
    cols.append(idx)
    vals.append(onsite.astype(np.complex128))
    dxs.append(np.zeros(N))
    dys.append(np.zeros(N))
    r, c, v = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
    H = _coo_csc(r, c, v, N)
    if not currents:
        return H
    Jx = _coo_csc(r, c, v * np.concatenate(dxs), N)
    Jy = _coo_csc(r, c, v * np.concatenate(dys), N)
    return H, Jx, Jy


def cubic_anderson(L: int, t: float = 1.0, W: float = 0.0, rng=None, currents: bool = False):
    """Periodic L^3 cubic lattice (``test/ed_reference.jl:396-441``), 7 nnz per row."""
    if L < 3:
        raise ValueError("cubic_anderson: L must be at least 3")
    rng = np.random.default_rng(1) if rng is None else rng
    N = L ** 3
    j = np.arange(N, dtype=np.int64)
    x, y, z = j % L, (j // L) % L, j // (L * L)
    site = lambda a, b, c: (a % L) + L * (b % L) + L * L * (c % L)
    rows, cols, vals, disp = [], [], [], []
    for d, (ox, oy, oz) in enumerate(((1, 0, 0), (0, 1, 0), (0, 0, 1))):
        i = site(x + ox, y + oy, z + oz)
        amp = np.full(N, -t, dtype=np.complex128)
        vec = np.zeros(3)
        vec[d] = 1.0
        rows += [i, j]
        cols += [j, i]
        vals += [amp, np.conj(amp)]
        disp += [np.tile(vec, (N, 1)), np.tile(-vec, (N, 1))]
    onsite = W * (rng.random(N) - 0.5)
    rows.append(j)
    cols.append(j)
    vals.append(onsite.astype(np.complex128))
    disp.append(np.zeros((N, 3)))
    r, c, v = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
    H = _coo_csc(r, c, v, N)
    if not currents:
        return H
    D = np.concatenate(disp)
    return (H,) + tuple(_coo_csc(r, c, v * D[:, k], N) for k in range(3)) + (float(N),)


def _honeycomb_vectors():
    a1 = np.array([math.sqrt(3), 0.0])
    a2 = np.array([math.sqrt(3) / 2, 1.5])
    dAB = np.array([math.sqrt(3) / 2, 0.5])
    return a1, a2, dAB


def haldane(Lx: int, Ly: int, t: float = 1.0, t2: float = 0.2, phi: float = math.pi / 2,
            m: float = 0.0):
    """Haldane model on a honeycomb torus; returns (H, Jx, Jy, area).

    Cell index (x, y) -> y + Ly*x (0-based), sites A = 2*cell, B = 2*cell+1,
    matching ``test/ed_reference.jl:69-141`` shifted to 0-based indices.
    """
    a1, a2, dAB = _honeycomb_vectors()
    N = 2 * Lx * Ly
    cx, cy = np.meshgrid(np.arange(Lx), np.arange(Ly), indexing="ij")
    cx, cy = cx.ravel(), cy.ravel()
    cell = lambda x, y: (y % Ly) + Ly * (x % Lx)
    A = lambda x, y: 2 * cell(x, y)
    B = lambda x, y: 2 * cell(x, y) + 1
    rows, cols, vals, dx, dy = [], [], [], [], []

    def addhop(i, j, amp, d):
        amp = np.broadcast_to(np.asarray(amp, dtype=np.complex128), i.shape)
        rows.extend([i, j])
        cols.extend([j, i])
        vals.extend([amp, np.conj(amp)])
        dx.extend([np.full(i.shape, d[0]), np.full(i.shape, -d[0])])
        dy.extend([np.full(i.shape, d[1]), np.full(i.shape, -d[1])])

    addhop(B(cx, cy), A(cx, cy), -t, dAB)
    addhop(B(cx, cy), A(cx + 1, cy), -t, dAB - a1)
    addhop(B(cx, cy), A(cx, cy + 1), -t, dAB - a2)
    for d, (ox, oy) in ((a1, (1, 0)), (a2 - a1, (-1, 1)), (-a2, (0, -1))):
        addhop(A(cx + ox, cy + oy), A(cx, cy), t2 * np.exp(1j * phi), d)
        addhop(B(cx + ox, cy + oy), B(cx, cy), t2 * np.exp(-1j * phi), d)
    # staggered mass; stored explicitly even when m == 0, like the reference
    for s, sign in ((A(cx, cy), 1.0), (B(cx, cy), -1.0)):
        rows.append(s)
        cols.append(s)
        vals.append(np.full(s.shape, sign * m, dtype=np.complex128))
        dx.append(np.zeros(s.shape))
        dy.append(np.zeros(s.shape))
    r, c, v = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
    DX, DY = np.concatenate(dx), np.concatenate(dy)
    H = _coo_keep_zeros(r, c, v, N)
    Jx = _coo_keep_zeros(r, c, v * DX, N)
    Jy = _coo_keep_zeros(r, c, v * DY, N)
    area = Lx * Ly * abs(a1[0] * a2[1] - a1[1] * a2[0])
    return H, Jx, Jy, area


def _coo_keep_zeros(r, c, v, n):
    """CSC assembly that sums duplicates but keeps explicit zeros (Julia's ``sparse``)."""
    order = np.lexsort((r, c))
    r, c, v = r[order], c[order], v[order]
    key = c.astype(np.int64) * n + r
    uniq, start = np.unique(key, return_index=True)
    vals = np.add.reduceat(v, start) if len(v) else v
    rows = (uniq % n).astype(np.int64)
    colsu = (uniq // n).astype(np.int64)
    indptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(indptr, colsu + 1, 1)
    indptr = np.cumsum(indptr)
    return sp.csc_matrix((vals, rows, indptr), shape=(n, n))


def graphene(Lx: int, Ly: int, t: float = 1.0, onsite=None):
    """Honeycomb torus with NN hopping -t and onsite energies (length 2*Lx*Ly)."""
    H, _, _, _ = haldane(Lx, Ly, t=t, t2=0.0, m=0.0)
    H = sp.csc_matrix(H)
    H.eliminate_zeros()
    N = H.shape[0]
    if onsite is not None:
        H = (H + sp.diags(np.asarray(onsite, dtype=np.complex128), format="csc")).tocsc()
    H.sort_indices()
    return H


def ring(N: int, t: float = 1.0, shift: float = 0.0):
    """N-site periodic chain, hopping -t, onsite shift (``test/dos_test.jl:214-249``)."""
    i = np.arange(N)
    r = np.concatenate([i, i, i])
    c = np.concatenate([(i + 1) % N, (i - 1) % N, i])
    v = np.concatenate([np.full(N, -t), np.full(N, -t), np.full(N, shift)]).astype(np.complex128)
    return _coo_csc(r, c, v, N)
