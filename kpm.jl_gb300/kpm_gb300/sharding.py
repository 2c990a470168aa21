"""Probe and realisation sharding across processes, one GPU per process.

The stochastic trace of KPM.jl averages over independent probe columns
(``src/moment.jl:410-411`` for kpm_1d, the GEMM over K = NH*NR at
``src/moment.jl:1055-1061`` for kpm_2d), and ensemble members are independent
realisations.  So the work shards with no per-step exchange: each rank runs
the single-GPU path on its own columns (or members) and one sum of the
partial moments over ranks finishes the job.  The sum goes through
``torch.distributed`` (NCCL for CUDA tensors, gloo on CPU); the process group
is the caller's.

Every function takes ``compute=`` (default: the GPU entry point) so the
partitioning and reduction can be exercised without a GPU.
"""
from __future__ import annotations

import numpy as np

from ._native import KPMArgumentError


def probe_slice(NR: int, world: int, rank: int) -> slice:
    """Contiguous, balanced block of probe columns owned by ``rank``."""
    if world < 1 or not 0 <= rank < world:
        raise KPMArgumentError(f"invalid rank {rank} of {world}")
    base, extra = divmod(int(NR), world)
    start = rank * base + min(rank, extra)
    return slice(start, start + base + (1 if rank < extra else 0))


def member_partition(costs, world: int) -> list[list[int]]:
    """Greedy longest-processing-time split of ensemble members by cost
    (e.g. nnz * NC); returns the member indices of every rank, each sorted."""
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(i)
        load[r] += float(costs[i])
    return [sorted(p) for p in parts]


def _dist():
    import torch.distributed as dist
    return dist


def _world(group):
    dist = _dist()
    if not dist.is_available() or not dist.is_initialized():
        return 1, 0
    return dist.get_world_size(group), dist.get_rank(group)


def _allreduce_sum(arr: np.ndarray, group) -> np.ndarray:
    """Sum a complex/real numpy array over the ranks of ``group``."""
    import torch
    dist = _dist()
    if not dist.is_available() or not dist.is_initialized():
        return arr
    t = torch.from_numpy(np.ascontiguousarray(arr))
    if t.is_complex():
        t = torch.view_as_real(t)
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    t = t.cpu()
    if np.iscomplexobj(arr):
        t = torch.view_as_complex(t.contiguous())
    return t.numpy().reshape(arr.shape)


def gather_probe_moments(mu_local: np.ndarray, NR_total: int, *, group=None) -> np.ndarray:
    """Assemble per-rank kpm_1d moments (this rank's (NR_g, NC) block of the
    columns ``probe_slice(NR_total, world, rank)``) into the full
    (NR_total, NC) matrix on every rank, by one sum over the ranks."""
    world, rank = _world(group)
    sl = probe_slice(NR_total, world, rank)
    mu_local = np.asarray(mu_local)
    if mu_local.shape[0] != sl.stop - sl.start:
        raise KPMArgumentError(f"rank {rank} holds {mu_local.shape[0]} columns; its slice has "
                               f"{sl.stop - sl.start}")
    full = np.zeros((int(NR_total), mu_local.shape[1]), dtype=np.complex128)
    full[sl] = mu_local
    return _allreduce_sum(full, group)


def kpm_1d_sharded(H, NC: int, psi_in, *, group=None, avg_output: bool = True, compute=None,
                   **kw):
    """``kpm_1d(H, NC, NR, psi_in=psi_in)`` with the NR probe columns split
    over the ranks of ``group``.  Every rank passes the full (NH, NR) probe
    block (or at least identical copies of it) and gets the full result: the
    real probe average (length NC), or the (NR, NC) matrix with
    ``avg_output=False``."""
    from .moment import kpm_1d
    compute = compute or (lambda H_, NC_, psi_: kpm_1d(H_, NC_, psi_.shape[1], psi_in=psi_,
                                                       avg_output=False, **kw))
    psi = np.asarray(psi_in)
    NR = psi.shape[1]
    world, rank = _world(group)
    if world > NR:
        raise KPMArgumentError(f"{world} ranks for {NR} probe columns")
    sl = probe_slice(NR, world, rank)
    mu_all = gather_probe_moments(compute(H, int(NC), np.array(psi[:, sl], dtype=np.complex128)),
                                  NR, group=group)
    if avg_output:
        return mu_all.sum(axis=0).real / NR
    return mu_all


def kpm_2d_sharded(H, Ja, Jb, NC: int, psi_in_l, psi_in_r=None, *, group=None, compute=None,
                   **kw):
    """``kpm_2d`` with the probe columns split over the ranks of ``group``:
    mu = (1/NR) sum_g NR_g mu_g, every rank gets the (NC, NC) result."""
    from .moment import kpm_2d
    psi_l = np.asarray(psi_in_l)
    psi_r = psi_l if psi_in_r is None else np.asarray(psi_in_r)
    NH, NR = psi_l.shape
    compute = compute or (lambda H_, Ja_, Jb_, NC_, l_, r_: kpm_2d(
        H_, Ja_, Jb_, NC_, l_.shape[1], NH, psi_in_l=l_, psi_in_r=r_, **kw))
    world, rank = _world(group)
    if world > NR:
        raise KPMArgumentError(f"{world} ranks for {NR} probe columns")
    sl = probe_slice(NR, world, rank)
    nr = sl.stop - sl.start
    mu = compute(H, Ja, Jb, int(NC), np.array(psi_l[:, sl], dtype=np.complex128),
                 np.array(psi_r[:, sl], dtype=np.complex128)) * (nr / NR)
    return _allreduce_sum(np.asarray(mu, dtype=np.complex128), group)


def kpm_1d_ensemble_sharded(Hs, NC: int, psis, *, group=None, compute=None, **kw):
    """``kpm_1d_ensemble`` with members balanced over the ranks by nnz; every
    rank gets the list of (NR, NC) moment matrices of all members."""
    from .moment import kpm_1d_ensemble
    compute = compute or (lambda Hs_, NC_, ps_: kpm_1d_ensemble(Hs_, NC_, ps_, avg_output=False,
                                                                **kw))
    if len(Hs) != len(psis) or not Hs:
        raise KPMArgumentError("Hs and psis must be non-empty lists of equal length")
    NR = np.asarray(psis[0]).shape[1]
    world, rank = _world(group)
    costs = [getattr(H, "nnz", H.shape[0]) + H.shape[0] for H in Hs]
    mine = member_partition(costs, world)[rank]
    out = np.zeros((len(Hs), NR, int(NC)), dtype=np.complex128)
    if mine:
        res = compute([Hs[i] for i in mine], int(NC), [psis[i] for i in mine])
        for i, m in zip(mine, res):
            out[i] = m
    out = _allreduce_sum(out, group)
    return [out[i] for i in range(len(Hs))]
