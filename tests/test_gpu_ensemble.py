"""Batched ensemble (many realisations in one call) against the per-member
kpm_1d and the oracle, for both schedules: one launch per step over CTAs of
at most 512 rows of a member ("gather", "padded", the default "auto") and one
persistent launch in which each CTA runs whole members ("single")."""
import numpy as np
import pytest
import scipy.sparse as sp

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


KERNELS = [("fp64", "auto"), ("fp64", "gather"), ("fp64", "single"), ("ff", "auto"),
           ("ff", "gather"), ("ff", "padded"), ("ff", "single")]


@pytest.mark.parametrize("prec,kernel", KERNELS)
def test_ensemble_matches_oracle(built_lib, prec, kernel):
    rng = np.random.default_rng(4)
    Hs, psis = _members(rng, 12, 6, 20)
    got = kg.kpm_1d_ensemble(Hs, 128, psis, precision=prec, avg_output=False, kernel=kernel)
    for H, psi, m in zip(Hs, psis, got):
        assert relerr(m, ko.kpm_1d_doubling(H, 128, psi)) < TOL[prec]


@pytest.mark.parametrize("prec,kernel", KERNELS)
def test_ensemble_members_over_many_ctas(built_lib, prec, kernel):
    """Members of 1..10 CTAs of the per-step schedule (512 rows each), with
    sizes at the CTA boundary (512, 513 rows: a 1-row CTA) and a 1-row member;
    every member against the oracle, and the two schedules against each
    other."""
    rng = np.random.default_rng(77)
    Hs, psis = [], []
    for n in (2304, 512, 513, 1, 4900, 1024, 37, 1025):
        if n == 1:
            H = sp.csc_matrix(np.array([[0.3 + 0j]]))
        else:
            L = int(round(np.sqrt(n))) if n in (2304, 4900, 1024) else None
            H = (models.square_anderson(L, W=3.0, rng=rng) / 5.6).tocsc() if L else \
                ((models.ring(n) + sp.diags(rng.uniform(-0.5, 0.5, n))) / 2.6).tocsc()
        Hs.append(H)
        psis.append(ko.random_phase_vectors(rng, H.shape[0], 8))
    got = kg.kpm_1d_ensemble(Hs, 64, psis, precision=prec, avg_output=False, kernel=kernel)
    other = kg.kpm_1d_ensemble(Hs, 64, psis, precision=prec, avg_output=False,
                               kernel="single" if kernel != "single" else "auto")
    for H, psi, m, o in zip(Hs, psis, got, other):
        assert relerr(m, ko.kpm_1d_doubling(H, 64, psi)) < TOL[prec]
        assert relerr(m, o) < TOL[prec]
    # the schedule is a pure function of the shape: repeated calls agree bitwise
    again = kg.kpm_1d_ensemble(Hs, 64, psis, precision=prec, avg_output=False, kernel=kernel)
    for m, a in zip(got, again):
        assert np.array_equal(m, a)


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
    # padded rows are float-float only
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d_ensemble(Hs, 64, psis, kernel="padded")
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d_ensemble(Hs, 64, psis, kernel="cluster")


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
    """kernel="tune" times the candidate schedules and shapes once, writes
    the choice to the persistent cache, and later calls (fresh operators, as
    a new process would build) read it back without timing: they launch the
    same number of kernels as each other and fewer than the tuning call.  All
    agree with the oracle."""
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
        kg.kpm_1d_ensemble(kg.EnsembleOperator(Hs), 96, psis, precision=prec, avg_output=False,
                           kernel="tune")
        n_third = kg.kernel_launch_count() - n0
        assert n_tuned > n_cached
        assert n_cached == n_third
        for m, a, r in zip(got, again, ref):
            assert np.array_equal(m, a)
            assert relerr(m, r) < TOL[prec]


@pytest.mark.parametrize("shape", ["256,1,0", "512,1,0", "1024,1,0", "256,1,256", "256,1,2048",
                                   "256,0,1024"])
def test_ensemble_tuned_shapes_match_oracle(built_lib, tmp_path, monkeypatch, shape):
    """Every tuned shape (threads per CTA, padded rows, rows per CTA of the
    per-step schedule or 0 for the persistent one; forced through a cache
    entry): parity with the oracle; the doubling moments' imaginary parts are
    exactly 0 with padded rows (Hermitian members)."""
    rng = np.random.default_rng(23 + sum(map(int, shape.split(","))))
    Hs, psis = _members(rng, 16, 6, 20)
    ens = kg.EnsembleOperator(Hs)
    NH, nnz = ens.op.shape[0], ens.op.nnz
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("KPMGB_TUNE_CACHE", str(cache))
    # learn the exact key from a tuning run, then pin its value
    kg.kpm_1d_ensemble(ens, 64, psis, precision="ff", kernel="tune")
    key = [l.rsplit(" ", 1)[0] for l in cache.read_text().splitlines()
           if l.startswith("ensemble|") and f"|NH={NH}|nnz={nnz}|" in l and "|prec=1" in l][0]
    cache.write_text(f"{key} {shape}\n")
    n0 = kg.kernel_launch_count()
    got = kg.kpm_1d_ensemble(ens, 128, psis, precision="ff", avg_output=False, kernel="tune")
    launches = kg.kernel_launch_count() - n0
    # the per-step schedule launches once per step (64), the persistent once
    assert (launches > 64) == (not shape.endswith(",0"))
    for H, p, m in zip(Hs, psis, got):
        assert relerr(m, ko.kpm_1d_doubling(H, 128, p)) < TOL["ff"]
        if shape.split(",")[1] == "1":
            assert np.all(m.imag == 0.0)


@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_ensemble_device_entry_matches_host_entry(built_lib, prec):
    """kpmgb_kpm1d_ensemble_device on torch tensors (stacked column-major
    probes in, (nseg, NC, NR) moments out) gives the host entry's moments
    bitwise."""
    import torch
    rng = np.random.default_rng(52)
    Hs, psis = _members(rng, 10, 20, 40)
    ens = kg.EnsembleOperator(Hs)
    NC, NR = 96, 8
    host = kg.kpm_1d_ensemble(ens, NC, psis, precision=prec, avg_output=False)
    stacked = np.vstack(psis)                     # (sum NH, NR)
    psi_t = torch.from_numpy(np.ascontiguousarray(stacked.T)).cuda()
    mu_t = torch.zeros((len(Hs), NC, NR), dtype=torch.complex128, device="cuda")
    kg.kpm_1d_ensemble_device(ens, NC, psi_t, mu_t, precision=prec)
    kg.sync(ens.op)
    torch.cuda.synchronize()
    got = mu_t.cpu().numpy()
    for i, m in enumerate(host):
        assert np.array_equal(got[i].T, m)
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d_ensemble_device(ens, NC, psi_t, mu_t[:, :64], precision=prec)


def _ragged_member(rng, n, max_row, complex_h):
    """Hermitian member with row lengths spread over 0..max_row, scaled into
    the Chebyshev domain."""
    rows, cols = [], []
    for i in range(n):
        for j in rng.choice(n, size=int(rng.integers(0, max_row // 2 + 1)), replace=False):
            rows.append(i)
            cols.append(int(j))
    vals = rng.standard_normal(len(rows)) + (1j * rng.standard_normal(len(rows)) if complex_h else 0)
    A = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    A = (A + A.conj().T).tocsr()
    A.sum_duplicates()
    keep = (np.diff(A.indptr) <= max_row).astype(float)
    A = sp.csc_matrix(sp.diags(keep) @ A @ sp.diags(keep))
    A.eliminate_zeros()
    return A / (1.05 * max(np.abs(np.linalg.eigvalsh(A.toarray())).max(), 1e-3))


@pytest.mark.parametrize("NR", [1, 3, 8, 13, 32])
@pytest.mark.parametrize("complex_h", [False, True])
def test_ensemble_padded_rows_widths_match_oracle(built_lib, NR, complex_h):
    """Float-float padded-row steps of real and complex members for 1..32
    probe columns and ragged rows of up to 8 nonzeros (empty rows included):
    every member against the oracle, and the padded and CSR-row kernels
    against each other (their float-float sums are anchored per padded row
    and per 8-nonzero chunk of a CSR row: agreement to ~1e-12)."""
    rng = np.random.default_rng(300 + NR + 7 * complex_h)
    Hs = [_ragged_member(rng, n, 8, complex_h) for n in (150, 700, 33, 520)]
    psis = [ko.random_phase_vectors(rng, H.shape[0], NR) for H in Hs]
    got = kg.kpm_1d_ensemble(Hs, 96, psis, precision="ff", avg_output=False, kernel="padded")
    auto = kg.kpm_1d_ensemble(Hs, 96, psis, precision="ff", avg_output=False)
    csr = kg.kpm_1d_ensemble(Hs, 96, psis, precision="ff", avg_output=False, kernel="gather")
    for H, psi, m, a, c in zip(Hs, psis, got, auto, csr):
        assert relerr(m, ko.kpm_1d_doubling(H, 96, psi)) < TOL["ff"]
        assert np.array_equal(m, a)
        assert relerr(m, c) < 1e-11
