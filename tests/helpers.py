"""Shared test inputs (seeded)."""
from pathlib import Path

import numpy as np
import scipy.sparse as sp

GOLDEN = Path(__file__).resolve().parent / "golden"


def rand_herm(rng, n, scale=1.2):
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    H = (A + A.conj().T) / 2
    return H / (scale * np.linalg.norm(H, 2))


def blocking_model(rng, L):
    """Dense nearest-neighbour + weak random Hermitian model of
    test/kpm2d_blocking_test.jl:7-23, with random Hermitian currents."""
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


def load_golden(name):
    f = np.load(GOLDEN / f"{name}.npz")
    n = int(f["H_n"])
    mat = lambda k: sp.csc_matrix((f[f"{k}_data"], f[f"{k}_indices"], f[f"{k}_indptr"]),
                                  shape=(n, n))
    return f, mat
