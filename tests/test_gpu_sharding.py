"""The sharded entry points with the GPU compute under a real NCCL process
group (one rank: this machine has one GPU; the partitioning and the sum over
ranks are also covered with gloo and two ranks in test_sharding.py).  The
all-reduce runs even for one rank, so the NCCL path executes on the device."""
import os
import socket

import numpy as np
import pytest

from conftest import relerr
import kpm_gb300 as kg
from kpm_gb300 import models, sharding
from oracle import kpm_oracle as ko

pytestmark = pytest.mark.gpu


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.fixture
def nccl_group(built_lib):
    import torch
    import torch.distributed as dist
    os.environ.setdefault("NCCL_NVLS_ENABLE", "0")
    store = dist.TCPStore("127.0.0.1", _free_port(), 1, True)
    dist.init_process_group("nccl", store=store, rank=0, world_size=1,
                            device_id=torch.device("cuda", 0))
    yield None
    dist.destroy_process_group()


def test_sharded_paths_on_gpu_with_nccl(nccl_group):
    rng = np.random.default_rng(14)
    H = (models.square_anderson(20, W=2.0, rng=rng) / 5.1).tocsc()
    psi = ko.random_phase_vectors(rng, 400, 12)
    got = sharding.kpm_1d_sharded(H, 96, psi, avg_output=False, precision="ff")
    assert relerr(got, ko.kpm_1d_doubling(H, 96, psi)) < 1e-9
    assert np.array_equal(got, kg.kpm_1d(H, 96, 12, psi_in=psi, avg_output=False,
                                         precision="ff"))
    Hh, Jx, Jy, _ = models.haldane(4, 4, t2=0.1)
    Hn = (Hh / 3.5).tocsc()
    ps = ko.random_phase_vectors(rng, Hn.shape[0], 6)
    mu2 = sharding.kpm_2d_sharded(Hn, Jx, Jy, 16, ps)
    assert relerr(mu2, ko.kpm_2d(Hn, Jx, Jy, 16, ps, ps, 16, 16)) < 1e-12
    Hs = [(models.square_anderson(L, W=2.0, rng=rng) / 5.1).tocsc() for L in (6, 9, 7)]
    psis = [ko.random_phase_vectors(rng, H_.shape[0], 4) for H_ in Hs]
    ens = sharding.kpm_1d_ensemble_sharded(Hs, 32, psis)
    for H_, p_, m in zip(Hs, psis, ens):
        assert relerr(m, ko.kpm_1d_doubling(H_, 32, p_)) < 1e-12
