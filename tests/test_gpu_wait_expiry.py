"""Failure detection on the GPU without a fault: the single-launch kernel's
grid barrier is made to wait for an arrival that never comes, so every block
gives up after a short bounded spin, records the timeout status and returns.
The host must report KPMGB_ERR_TIMEOUT, and the same operator (same context,
same workspace) must then produce oracle-exact moments."""
import numpy as np
import pytest

from conftest import relerr
import kpm_gb300 as kg
from kpm_gb300 import _native, models
from oracle import kpm_oracle as ko

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return built_lib


def test_barrier_wait_expires_and_context_survives():
    rng = np.random.default_rng(11)
    H = (models.square_anderson(16, W=2.0, rng=rng) / 5.1).tocsc()
    op = kg.GB300Operator(H)
    lib = _native.load()
    rc = lib.kpmgb_selftest_wait_expiry(op.handle)
    assert rc == _native.ERR_TIMEOUT
    assert b"bounded wait" in lib.kpmgb_last_error()
    psi = ko.random_phase_vectors(rng, 256, 4)
    ref = ko.kpm_1d_doubling(H, 64, psi)
    # the barrier counters are re-armed by the next launch of the same kernel
    got = kg.kpm_1d(op, 64, 4, psi_in=psi, avg_output=False, kernel="single")
    assert relerr(got, ref) < 1e-12
    got = kg.kpm_1d(op, 64, 4, psi_in=psi, avg_output=False)
    assert relerr(got, ref) < 1e-12
    # and the expiry is reported again, not latched or hung
    assert lib.kpmgb_selftest_wait_expiry(op.handle) == _native.ERR_TIMEOUT
    got = kg.kpm_1d(op, 64, 4, psi_in=psi, avg_output=False, precision="ff", kernel="single")
    assert relerr(got, ref) < 1e-9
