"""Probe / realisation sharding over processes (gloo, world_size 2, CPU).

The per-rank compute is replaced by a small dense Chebyshev evaluation
defined here, so that only the partitioning and the reduction are under
test; the GPU entry points behind them are covered by the gpu tests.
"""
import os
import socket

import numpy as np
import pytest
import scipy.sparse as sp

from kpm_gb300 import sharding


def _dense_mu_all(H, NC, psi):
    """<psi_i|T_n(H)|psi_i> per probe column, (NR, NC), by the plain recurrence."""
    Hd = np.asarray(H.todense()) if sp.issparse(H) else np.asarray(H)
    t0, t1 = psi, Hd @ psi
    out = np.zeros((psi.shape[1], NC), dtype=np.complex128)
    out[:, 0] = np.einsum("ij,ij->j", psi.conj(), t0)
    out[:, 1] = np.einsum("ij,ij->j", psi.conj(), t1)
    for n in range(2, NC):
        t0, t1 = t1, 2 * Hd @ t1 - t0
        out[:, n] = np.einsum("ij,ij->j", psi.conj(), t1)
    return out


def _dense_mu2d(H, Ja, Jb, NC, psi_l, psi_r):
    Hd, Ad, Bd = (np.asarray(M.todense()) for M in (H, Ja, Jb))
    def chain(v):
        vs = [v, Hd @ v]
        for _ in range(2, NC):
            vs.append(2 * Hd @ vs[-1] - vs[-2])
        return vs
    L = chain(psi_l)
    R = chain(Ad @ psi_r)
    mu = np.zeros((NC, NC), dtype=np.complex128)
    for n in range(NC):
        JR = Bd @ R[n]
        for m in range(NC):
            mu[n, m] = np.sum(L[m].conj() * JR) / psi_l.shape[1]
    return mu


def _problem(seed=3, n=24, NR=5):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    H = (A + A.conj().T) / 2
    H /= 1.2 * np.linalg.norm(H, 2)
    psi = np.exp(2j * np.pi * rng.random((n, NR))) / np.sqrt(n)
    B = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    return sp.csc_matrix(H), sp.csc_matrix((B + B.conj().T) / 2), psi


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, outdir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        H, J, psi = _problem()
        NC = 12
        mu_avg = sharding.kpm_1d_sharded(H, NC, psi, compute=_dense_mu_all)
        mu_all = sharding.kpm_1d_sharded(H, NC, psi, avg_output=False, compute=_dense_mu_all)
        mu2 = sharding.kpm_2d_sharded(H, J, H, 6, psi, compute=_dense_mu2d)
        Hs = [sp.csc_matrix(np.diag(np.linspace(-0.5, 0.5, k))) for k in (3, 9, 4, 7, 5)]
        psis = [np.ones((k, 2), dtype=complex) / np.sqrt(k) for k in (3, 9, 4, 7, 5)]
        ens = sharding.kpm_1d_ensemble_sharded(
            Hs, 8, psis, compute=lambda hs, nc, ps: [_dense_mu_all(h, nc, p) for h, p in zip(hs, ps)])
        np.savez(os.path.join(outdir, f"rank{rank}.npz"), mu_avg=mu_avg, mu_all=mu_all, mu2=mu2,
                 ens=np.array(ens))
    finally:
        dist.destroy_process_group()


def test_probe_slice_covers_columns():
    for NR in (1, 5, 64, 67):
        for world in range(1, min(NR, 9) + 1):
            cols = []
            sizes = []
            for r in range(world):
                sl = sharding.probe_slice(NR, world, r)
                cols.extend(range(NR)[sl])
                sizes.append(sl.stop - sl.start)
            assert cols == list(range(NR))
            assert max(sizes) - min(sizes) <= 1


def test_member_partition_balanced():
    rng = np.random.default_rng(0)
    costs = rng.integers(500, 9000, size=256)
    parts = sharding.member_partition(costs, 4)
    assert sorted(i for p in parts for i in p) == list(range(256))
    loads = [costs[p].sum() for p in parts]
    assert max(loads) - min(loads) <= costs.max()


def test_sharded_gloo_two_ranks(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       join=True, start_method="spawn")
    H, J, psi = _problem()
    ref_all = _dense_mu_all(H, 12, psi)
    ref2 = _dense_mu2d(H, J, H, 6, psi, psi)
    for r in range(world):
        f = np.load(tmp_path / f"rank{r}.npz")
        assert np.allclose(f["mu_all"], ref_all, rtol=0, atol=1e-13)
        assert np.allclose(f["mu_avg"], ref_all.sum(0).real / psi.shape[1], rtol=0, atol=1e-13)
        assert np.allclose(f["mu2"], ref2, rtol=0, atol=1e-12)
        assert f["ens"].shape == (5, 2, 8)
        d = np.linspace(-0.5, 0.5, 9)
        expect = [np.mean(np.cos(n * np.arccos(d))) for n in range(8)]
        assert np.allclose(f["ens"][1][0].real, expect, atol=1e-13)


def test_world_larger_than_probes_rejected():
    with pytest.raises(Exception):
        sharding.probe_slice(4, 2, 2)
