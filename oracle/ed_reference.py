"""Exact-diagonalisation references used to pin the oracle (TEST INFRASTRUCTURE ONLY).

Restates the known-answer routines of the reference's test module
``test/ed_reference.jl``; no KPM code is involved, so agreement between these
and the KPM oracle pins the oracle independently of the reference's runtime.
"""
from __future__ import annotations

import math

import numpy as np


def haldane_bloch(t=1.0, t2=0.2, phi=math.pi / 2, m=0.0):
    """2x2 Bloch Hamiltonian h(k1, k2) of the Haldane torus model (``test/ed_reference.jl:216-238``)."""
    nnn = ((1, 0), (-1, 1), (0, -1))

    def hk(k1, k2):
        phase = lambda off: np.exp(2j * np.pi * (k1 * off[0] + k2 * off[1]))
        hBA = -t * (1 + phase((1, 0)) + phase((0, 1)))
        hAA = m + 0j
        hBB = -m + 0j
        for off in nnn:
            hAA += t2 * np.exp(1j * phi) * np.conj(phase(off)) + t2 * np.exp(-1j * phi) * phase(off)
            hBB += t2 * np.exp(-1j * phi) * np.conj(phase(off)) + t2 * np.exp(1j * phi) * phase(off)
        return np.array([[hAA, np.conj(hBA)], [hBA, hBB]])

    return hk


def chern_number_fhs(hk, Nk=24, band=0):
    """Fukui-Hatsugai-Suzuki lattice Chern number (``test/ed_reference.jl:240-275``)."""
    u = np.empty((Nk, Nk, 2), dtype=np.complex128)
    for i in range(Nk):
        for j in range(Nk):
            w, v = np.linalg.eigh(hk(i / Nk, j / Nk))
            u[i, j] = v[:, band]
    total = 0.0
    for i in range(Nk):
        for j in range(Nk):
            u00, u10 = u[i, j], u[(i + 1) % Nk, j]
            u11, u01 = u[(i + 1) % Nk, (j + 1) % Nk], u[i, (j + 1) % Nk]
            total += np.angle(np.vdot(u00, u10) * np.vdot(u10, u11) * np.vdot(u11, u01)
                              * np.vdot(u01, u00))
    return -total / (2 * np.pi)


def ed_hall_conductivity_T0(H, Ja, Jb, area, Ef):
    """T=0 TKNN Hall conductivity in e^2/h (``test/ed_reference.jl:517-532``)."""
    dense = lambda M: np.asarray(M.toarray() if hasattr(M, "toarray") else M, dtype=np.complex128)
    ev, U = np.linalg.eigh(dense(H))
    Va = U.conj().T @ (dense(Ja) / 1j) @ U
    Vb = U.conj().T @ (dense(Jb) / 1j) @ U
    occ = ev <= Ef
    un = ~occ
    d = ev[occ][:, None] - ev[un][None, :]
    acc = np.sum(np.imag(Va[np.ix_(occ, un)] * Vb[np.ix_(un, occ)].T) / d ** 2)
    return 2 * np.pi * (-2 / area) * acc


def ed_moments(H, psi, NC):
    """mu_n = sum_k |<v_k|psi>|^2 T_n(lambda_k) per column (``test/dos_test.jl:36-43``)."""
    dense = np.asarray(H.toarray() if hasattr(H, "toarray") else H, dtype=np.complex128)
    lam, V = np.linalg.eigh(dense)
    w = np.abs(V.conj().T @ psi) ** 2
    th = np.arccos(np.clip(lam, -1, 1))
    T = np.cos(np.outer(np.arange(NC), th))
    return (T @ w).T
