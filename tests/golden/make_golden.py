"""Generate the golden fixtures of tests/golden/*.npz.

Every fixture carries an input (operator in CSC form, probes) and references
computed WITHOUT the KPM recurrence: exact diagonalisation (mu_n from the
eigen-decomposition) or dense Chebyshev matrices T_n(H) built by dense
products, as the reference's tests do (test/dos_test.jl:36-43,
test/kpm2d_blocking_test.jl:25-45).  The GPU tests compare against these.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import scipy.sparse as sp

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "kpm.jl_gb300"))

from kpm_gb300 import models  # noqa: E402
from oracle import ed_reference, kpm_oracle  # noqa: E402

OUT = Path(__file__).resolve().parent


def csc_arrays(M):
    M = sp.csc_matrix(M, dtype=np.complex128)
    M.sort_indices()
    return dict(indptr=M.indptr.astype(np.int64), indices=M.indices.astype(np.int64),
                data=M.data, n=np.int64(M.shape[0]))


def dense_moments(H, psi_l, psi_r, NC):
    T = kpm_oracle.chebyshev_matrices(H, NC)
    return np.array([[np.vdot(psi_l[:, i], T[n] @ psi_r[:, i]) for n in range(NC)]
                     for i in range(psi_l.shape[1])])


def main():
    rng = np.random.default_rng(42)
    # 1) 2D Anderson L=8, W=2, rescaled by its exact spectral radius
    H = models.square_anderson(8, W=2.0, rng=rng)
    ev = np.linalg.eigvalsh(H.toarray())
    Hn = (H / (1.1 * np.abs(ev).max())).tocsc()
    psi = kpm_oracle.random_phase_vectors(rng, 64, 3)
    NC = 64
    np.savez_compressed(OUT / "anderson2d_L8.npz", **{f"H_{k}": v for k, v in csc_arrays(Hn).items()},
                        psi=psi, NC=NC, mu_ed=ed_reference.ed_moments(Hn, psi, NC),
                        mu_dense=dense_moments(Hn, psi, psi, NC))
    # 2) Haldane 3x3 (complex H), bra/ket moments and the 2D moment matrix
    H, Jx, Jy, area = models.haldane(3, 3, t2=0.2)
    ev = np.linalg.eigvalsh(H.toarray())
    Hn = (H / (1.05 * np.abs(ev).max())).tocsc()
    NH = Hn.shape[0]
    psl = kpm_oracle.random_phase_vectors(rng, NH, 2)
    psr = kpm_oracle.random_phase_vectors(rng, NH, 2)
    NC = 24
    NC2 = 12
    np.savez_compressed(
        OUT / "haldane_3x3.npz", **{f"H_{k}": v for k, v in csc_arrays(Hn).items()},
        **{f"Jx_{k}": v for k, v in csc_arrays(Jx).items()},
        **{f"Jy_{k}": v for k, v in csc_arrays(Jy).items()},
        psi_l=psl, psi_r=psr, NC=NC, mu_lr_dense=dense_moments(Hn, psl, psr, NC), NC2=NC2,
        mu2d_dense=kpm_oracle.kpm2d_dense_reference(Hn, Jx, Jy, psl, psr, NC2))
    # 3) periodic ring, identity probes: exact trace moments in closed form
    N = 64
    t = 1.0
    Hr = models.ring(N, t=t)
    a = 2.0 * t / 0.95
    Hn = (Hr / a).tocsc()
    eps = -2 * t * np.cos(2 * np.pi * np.arange(N) / N) / a
    NC = 128
    mu_exact = np.array([np.mean(np.cos(n * np.arccos(eps))) for n in range(NC)])
    np.savez_compressed(OUT / "ring_N64.npz", **{f"H_{k}": v for k, v in csc_arrays(Hn).items()},
                        NC=NC, mu_exact=mu_exact)
    print("wrote", sorted(p.name for p in OUT.glob("*.npz")))


if __name__ == "__main__":
    main()
