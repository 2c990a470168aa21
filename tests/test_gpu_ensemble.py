"""Batched ensemble (one persistent launch for many realisations) against the
per-member kpm_1d and the oracle."""
import numpy as np
import pytest

from conftest import relerr
import kpm_gb300 as kg
from kpm_gb300 import models
from oracle import kpm_oracle as ko

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "ff": 1e-9}


def _members(rng, count, lo, hi):
    Hs, psis = [], []
    for _ in range(count):
        L = int(rng.integers(lo, hi + 1))
        W = float(rng.uniform(1.0, 8.0))
        H = models.square_anderson(L, W=W, rng=rng)
        Hs.append((H / (4.0 + W / 2 + 0.1)).tocsc())   # Gershgorin bound keeps |E| < 1
        psis.append(ko.random_phase_vectors(rng, L * L, 8))
    return Hs, psis


@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_ensemble_matches_oracle(built_lib, prec):
    rng = np.random.default_rng(4)
    Hs, psis = _members(rng, 12, 6, 20)
    got = kg.kpm_1d_ensemble(Hs, 128, psis, precision=prec, avg_output=False)
    for H, psi, m in zip(Hs, psis, got):
        assert relerr(m, ko.kpm_1d_doubling(H, 128, psi)) < TOL[prec]


def test_ensemble_matches_single_calls(built_lib):
    rng = np.random.default_rng(8)
    Hs, psis = _members(rng, 40, 8, 24)
    got = kg.kpm_1d_ensemble(Hs, 64, psis, avg_output=False)
    for H, psi, m in zip(Hs, psis, got):
        ref = kg.kpm_1d(H, 64, 8, psi_in=psi, avg_output=False)
        assert relerr(m, ref) < 1e-12


def test_ensemble_validation(built_lib):
    rng = np.random.default_rng(1)
    Hs, psis = _members(rng, 2, 4, 5)
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d_ensemble(Hs, 63, psis)
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d_ensemble(Hs, 64, [psis[0], psis[1][:, :4]])


@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_ensemble_column_batches(built_lib, prec):
    """NR = 40 runs as column batches of 32 + 8."""
    rng = np.random.default_rng(31)
    Hs, psis = [], []
    for _ in range(5):
        L = int(rng.integers(5, 12))
        Hs.append((models.square_anderson(L, W=2.0, rng=rng) / 5.1).tocsc())
        psis.append(ko.random_phase_vectors(rng, L * L, 40))
    got = kg.kpm_1d_ensemble(Hs, 64, psis, precision=prec, avg_output=False)
    for H, psi, m in zip(Hs, psis, got):
        assert relerr(m, ko.kpm_1d_doubling(H, 64, psi)) < TOL[prec]


def test_ensemble_operator_reuse(built_lib):
    rng = np.random.default_rng(44)
    Hs, psis = _members(rng, 9, 6, 14)
    ens = kg.EnsembleOperator(Hs)
    a = kg.kpm_1d_ensemble(Hs, 48, psis, avg_output=False)
    b = kg.kpm_1d_ensemble(ens, 48, psis, avg_output=False)
    c = kg.kpm_1d_ensemble(ens, 48, psis, avg_output=False)
    for x, y, z in zip(a, b, c):
        assert np.array_equal(x, y) and np.array_equal(y, z)
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d_ensemble(ens, 48, psis[:-1])


def test_ensemble_autotune_cache_round_trip(built_lib, tmp_path, monkeypatch):
    """kernel="tune" times the candidate launch shapes once, writes the choice
    to the persistent cache, and a later call (a fresh operator, as a new
    process would build) reads it back without timing: it launches exactly as
    many kernels as an untuned call.  Both agree with the oracle."""
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("KPMGB_TUNE_CACHE", str(cache))
    rng = np.random.default_rng(19)
    Hs, psis = _members(rng, 24, 6, 18)
    ref = [ko.kpm_1d_doubling(H, 96, p) for H, p in zip(Hs, psis)]
    for prec in ("ff", "fp64"):
        n0 = kg.kernel_launch_count()
        got = kg.kpm_1d_ensemble(kg.EnsembleOperator(Hs), 96, psis, precision=prec,
                                 avg_output=False, kernel="tune")
        n_tuned = kg.kernel_launch_count() - n0
        lines = [l for l in cache.read_text().splitlines() if l.startswith("ensemble|")]
        assert any(f"|prec={1 if prec == 'ff' else 0}" in l for l in lines)
        n0 = kg.kernel_launch_count()
        again = kg.kpm_1d_ensemble(kg.EnsembleOperator(Hs), 96, psis, precision=prec,
                                   avg_output=False, kernel="tune")
        n_cached = kg.kernel_launch_count() - n0
        n0 = kg.kernel_launch_count()
        kg.kpm_1d_ensemble(kg.EnsembleOperator(Hs), 96, psis, precision=prec, avg_output=False)
        n_plain = kg.kernel_launch_count() - n0
        assert n_tuned > n_cached
        assert n_cached == n_plain
        for m, a, r in zip(got, again, ref):
            assert np.array_equal(m, a)
            assert relerr(m, r) < TOL[prec]


@pytest.mark.parametrize("threads", [256, 512, 1024])
def test_ensemble_padded_kernel_matches_oracle(built_lib, tmp_path, monkeypatch, threads):
    """The padded-row float-float ensemble kernel at every tuned CTA size
    (forced through a cache entry): parity with the oracle; the doubling
    moments' imaginary parts are exactly 0 (Hermitian members)."""
    rng = np.random.default_rng(23 + threads)
    Hs, psis = _members(rng, 16, 6, 20)
    ens = kg.EnsembleOperator(Hs)
    NH, nnz = ens.op.shape[0], ens.op.nnz
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("KPMGB_TUNE_CACHE", str(cache))
    # learn the exact key from a tuning run, then pin its value
    kg.kpm_1d_ensemble(ens, 64, psis, precision="ff", kernel="tune")
    key = [l.rsplit(" ", 1)[0] for l in cache.read_text().splitlines()
           if l.startswith("ensemble|") and f"|NH={NH}|nnz={nnz}|" in l and "|prec=1" in l][0]
    cache.write_text(f"{key} {threads},1\n")
    got = kg.kpm_1d_ensemble(ens, 128, psis, precision="ff", avg_output=False, kernel="tune")
    for H, p, m in zip(Hs, psis, got):
        assert relerr(m, ko.kpm_1d_doubling(H, 128, p)) < TOL["ff"]
        assert np.all(m.imag == 0.0)
