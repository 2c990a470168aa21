"""GPU parity of the kpm_1d moment engine against the oracle and the golden
fixtures.  FP64 path: 1e-12 norm-wise relative (the reference's rtol);
float-float path: 1e-9."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import relerr
from helpers import load_golden, rand_herm
import kpm_gb300 as kg
from kpm_gb300 import models
from oracle import kpm_oracle as ko

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "ff": 1e-9}


@pytest.fixture(scope="module", autouse=True)
def _lib(built_lib):
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return built_lib


@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_golden_anderson(prec):
    f, mat = load_golden("anderson2d_L8")
    H = mat("H")
    mu = kg.kpm_1d(H, int(f["NC"]), 3, psi_in=f["psi"], avg_output=False, precision=prec)
    assert relerr(mu, f["mu_dense"]) < TOL[prec]
    assert relerr(mu, f["mu_ed"]) < max(TOL[prec], 1e-10)


@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_golden_haldane_lr(prec):
    f, mat = load_golden("haldane_3x3")
    mu = kg.kpm_1d(mat("H"), int(f["NC"]), 2, psi_in_l=f["psi_l"], psi_in_r=f["psi_r"],
                   avg_output=False, precision=prec)
    assert relerr(mu, f["mu_lr_dense"]) < TOL[prec]


@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_golden_ring_exact_trace(prec):
    f, mat = load_golden("ring_N64")
    H = mat("H")
    N = H.shape[0]
    mu = kg.kpm_1d(H, int(f["NC"]), N, psi_in=np.eye(N, dtype=complex), precision=prec)
    assert relerr(mu, f["mu_exact"]) < TOL[prec]


# small operators run as one cluster launch by default ("auto"); "gather"
# keeps the per-step kernels and their lane-group shapes under test
KERNELS = ["auto", "gather"]


@pytest.mark.parametrize("NR", [1, 2, 3, 4, 5, 8, 12, 16, 24, 32, 33, 64, 100, 128, 130, 200])
@pytest.mark.parametrize("prec", ["fp64", "ff"])
@pytest.mark.parametrize("kernel", KERNELS)
def test_probe_counts(NR, prec, kernel):
    """Every lane-group shape and the >128-column batching (per-step kernels),
    and every probe count on the cluster path."""
    rng = np.random.default_rng(100 + NR)
    H = models.square_anderson(16, W=2.0, rng=rng)
    a, _, Hn = ko.normalizeH(H)
    psi = ko.random_phase_vectors(rng, 256, NR)
    ref = ko.kpm_1d_doubling(Hn, 64, psi)
    got = kg.kpm_1d(Hn, 64, NR, psi_in=psi, avg_output=False, precision=prec, kernel=kernel)
    assert relerr(got, ref) < TOL[prec]


@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_config_2d_anderson_L64(prec):
    """2D Anderson L=64 (NH=4096), W=2, NC=1024, NR=12, the CPU-runnable workload."""
    rng = np.random.default_rng(42)
    H = models.square_anderson(64, W=2.0, rng=rng)
    a, _, Hn = ko.normalizeH(H)
    psi = ko.random_phase_vectors(rng, 4096, 12)
    ref = ko.kpm_1d_doubling(Hn, 1024, psi)
    got = kg.kpm_1d(Hn, 1024, 12, psi_in=psi, avg_output=False, precision=prec)
    assert relerr(got, ref) < TOL[prec]
    # per-moment relative error of the probe average against the largest moment
    err = np.max(np.abs(got.mean(0) - ref.mean(0))) / np.max(np.abs(ref.mean(0)))
    assert err < TOL[prec]


@pytest.mark.parametrize("prec", ["fp64", "ff"])
@pytest.mark.parametrize("lr", [False, True])
def test_complex_haldane(prec, lr):
    rng = np.random.default_rng(7)
    H, _, _, _ = models.haldane(24, 24, t2=0.1)
    a, b, Hn = ko.normalizeH(H, center=True)
    NH = Hn.shape[0]
    pl = ko.random_phase_vectors(rng, NH, 16)
    pr = ko.random_phase_vectors(rng, NH, 16)
    if lr:
        ref = ko.kpm_1d_lr(Hn, 257, pl, pr)  # odd NC, as test/gpu_smoke.jl:63-100
        got = kg.kpm_1d(Hn, 257, 16, psi_in_l=pl, psi_in_r=pr, avg_output=False, precision=prec)
    else:
        ref = ko.kpm_1d_doubling(Hn, 256, pr)
        got = kg.kpm_1d(Hn, 256, 16, psi_in=pr, avg_output=False, precision=prec)
    assert relerr(got, ref) < TOL[prec]


@pytest.mark.parametrize("prec", ["fp64", "ff"])
@pytest.mark.parametrize("kernel", KERNELS)
def test_ragged_empty_and_long_rows(prec, kernel):
    """Rows with 0, 1, ... 40 nonzeros (several float-float chunks), complex values."""
    rng = np.random.default_rng(3)
    n = 300
    rows, cols = [], []
    for i in range(n):
        k = (i * 7) % 41 if i % 10 else 0
        c = rng.choice(n, size=k, replace=False)
        rows += [i] * k
        cols += list(c)
    vals = rng.standard_normal(len(rows)) + 1j * rng.standard_normal(len(rows))
    A = sp.coo_matrix((vals, (rows, cols)), shape=(n, n)).tocsr()
    Hd = (A + A.conj().T).toarray() / 2
    Hd /= 1.1 * np.linalg.norm(Hd, 2)
    H = sp.csc_matrix(Hd)
    psi = ko.random_phase_vectors(rng, n, 6)
    ref = ko.kpm_1d_doubling(H, 96, psi)
    got = kg.kpm_1d(H, 96, 6, psi_in=psi, avg_output=False, precision=prec, kernel=kernel)
    assert relerr(got, ref) < TOL[prec]
    ref = ko.kpm_1d_lr(H, 95, psi[:, ::-1].copy(), psi)
    got = kg.kpm_1d(H, 95, 6, psi_in_l=psi[:, ::-1].copy(), psi_in_r=psi, avg_output=False,
                    precision=prec, kernel=kernel)
    assert relerr(got, ref) < TOL[prec]


@pytest.mark.parametrize("prec", ["fp64", "ff"])
@pytest.mark.parametrize("kernel", KERNELS)
def test_unnormalized_and_zero_columns(prec, kernel):
    """mu scales as |c|^2 (test/dos_test.jl:80-93); a zero probe gives zero moments."""
    rng = np.random.default_rng(13)
    H = sp.csc_matrix(rand_herm(rng, 32, scale=2.0))
    psi = ko.random_phase_vectors(rng, 32, 4) * np.array([1.0, 1e6, 1e-7, 0.0])
    ref = ko.kpm_1d_doubling(H, 16, psi)
    got = kg.kpm_1d(H, 16, 4, psi_in=psi, avg_output=False, precision=prec, kernel=kernel)
    for i in range(3):
        assert relerr(got[i], ref[i]) < TOL[prec]
    assert np.all(got[3] == 0)


@pytest.mark.parametrize("prec", ["fp64", "ff"])
@pytest.mark.parametrize("kernel", KERNELS)
def test_deterministic(prec, kernel):
    rng = np.random.default_rng(11)
    H = models.square_anderson(32, W=1.0, rng=rng)
    _, _, Hn = ko.normalizeH(H)
    op = kg.GB300Operator(Hn)
    psi = ko.random_phase_vectors(rng, 1024, 8)
    m1 = kg.kpm_1d(op, 128, 8, psi_in=psi, avg_output=False, precision=prec, kernel=kernel)
    m2 = kg.kpm_1d(op, 128, 8, psi_in=psi, avg_output=False, precision=prec, kernel=kernel)
    assert np.array_equal(m1, m2)


def test_errors():
    rng = np.random.default_rng(1)
    H = sp.csc_matrix(rand_herm(rng, 16))
    psi = ko.random_phase_vectors(rng, 16, 2)
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d(H, 7, 2, psi_in=psi)
    op = kg.GB300Operator(H)
    mu = np.zeros((2, 8), dtype=complex)
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d_bang(op, 8, 2, 15, mu, psi[:15])
    # spectrum outside (-1, 1): the recurrence grows, the guard reports it
    Hbad = sp.csc_matrix(3.0 * rand_herm(rng, 16, scale=1.0))
    with pytest.raises(kg.KPMNumericalError):
        kg.kpm_1d(Hbad, 64, 2, psi_in=psi, stability_check=True)
    # without the guard the reference semantics hold (finite growth is returned)
    mu_raw = kg.kpm_1d(Hbad, 16, 2, psi_in=psi)
    assert np.all(np.isfinite(mu_raw))
    # non-finite input is always reported
    bad = psi.copy()
    bad[0, 0] = np.nan
    with pytest.raises(kg.KPMNumericalError):
        kg.kpm_1d(H, 8, 2, psi_in=bad)


@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_wrapper_serial_columns_and_force_norm(prec):
    """kpm_1d with NR_parallel=False runs one call per column with the same
    options (src/moment.jl:339-418): the moments match the batched call, the
    stability guard still fires, and force_norm normalises the columns first
    (src/utils/vectors.jl:14-19)."""
    rng = np.random.default_rng(21)
    H = (models.square_anderson(20, W=2.0, rng=rng) / 5.1).tocsc()
    NR, NC = 6, 128
    psi = ko.random_phase_vectors(rng, 400, NR)
    both = kg.kpm_1d(H, NC, NR, psi_in=psi.copy(), avg_output=False, precision=prec)
    serial = kg.kpm_1d(H, NC, NR, psi_in=psi.copy(), avg_output=False, precision=prec,
                       NR_parallel=False, kernel="gather", use_graph=True)
    assert relerr(serial, both) < TOL[prec]
    assert relerr(serial, ko.kpm_1d_doubling(H, NC, psi)) < TOL[prec]
    Hbad = sp.csc_matrix(3.0 * rand_herm(rng, 16, scale=1.0))
    pb = ko.random_phase_vectors(rng, 16, 2)
    with pytest.raises(kg.KPMNumericalError):
        kg.kpm_1d(Hbad, 64, 2, psi_in=pb, stability_check=True, NR_parallel=False,
                  precision=prec)
    scaled = 3.7 * psi
    got = kg.kpm_1d(H, NC, NR, psi_in=scaled, avg_output=False, precision=prec, force_norm=True)
    assert np.allclose(np.linalg.norm(scaled, axis=0), 1.0)
    assert relerr(got, ko.kpm_1d_doubling(H, NC, psi)) < TOL[prec]


def test_device_api_matches_host():
    import torch
    rng = np.random.default_rng(9)
    H = models.square_anderson(32, W=2.0, rng=rng)
    _, _, Hn = ko.normalizeH(H)
    op = kg.GB300Operator(Hn)
    psi = ko.random_phase_vectors(rng, 1024, 12)
    host = kg.kpm_1d(op, 256, 12, psi_in=psi, avg_output=False)
    psi_t = torch.from_numpy(np.ascontiguousarray(psi.T)).cuda()
    mu_t = torch.zeros((256, 12), dtype=torch.complex128, device="cuda")
    kg.kpm_1d_device(op, 256, psi_t, mu_t)
    kg.sync(op)
    torch.cuda.synchronize()
    assert np.array_equal(mu_t.cpu().numpy().T, host)


def test_typed_frontend_delegates():
    """dos_moments delegates to kpm_1d exactly (test/frontend_test.jl:40-55)."""
    NH = 64
    H = sp.diags([np.ones(NH - 1), np.ones(NH - 1)], [-1, 1], format="csc").astype(complex)
    h = kg.rescale(H)
    psi = kg.random_phase_vectors(np.random.default_rng(11), NH, 4)
    m = kg.dos_moments(h, NC=64, psi_in=psi.copy())
    ref = kg.kpm_1d(h.H, 64, 4, psi_in=psi.copy())
    assert np.array_equal(m.mu, ref)
    assert (m.a, m.b, m.NH, m.NR) == (h.a, h.b, NH, 4)
    full = kg.dos_moments(h, NC=128, psi_in=np.eye(NH, dtype=complex))
    assert abs(full.mu[0] - 1.0) < 1e-12


@pytest.mark.parametrize("prec", ["fp64", "ff"])
@pytest.mark.parametrize("lr", [False, True])
def test_cuda_graph_replay_identical(prec, lr):
    """use_graph captures the per-step recurrence once and replays it:
    results are bitwise those of direct launches, on the first call and on
    replays, and a changed NC or probe count is captured afresh."""
    rng = np.random.default_rng(17)
    H = models.square_anderson(24, W=2.0, rng=rng)
    op = kg.GB300Operator((H / 5.1).tocsc())
    for NC, NR in ((128, 12), (128, 12), (64, 12), (64, 7)):
        psi = ko.random_phase_vectors(rng, 576, NR)
        kw = dict(psi_in_l=psi, psi_in_r=psi[:, ::-1].copy()) if lr else dict(psi_in=psi)
        ref = kg.kpm_1d(op, NC, NR, avg_output=False, precision=prec, kernel="gather", **kw)
        n0 = kg.kernel_launch_count()
        g1 = kg.kpm_1d(op, NC, NR, avg_output=False, precision=prec, use_graph=True,
                       kernel="gather", **kw)
        n1 = kg.kernel_launch_count()
        g2 = kg.kpm_1d(op, NC, NR, avg_output=False, precision=prec, use_graph=True,
                       kernel="gather", **kw)
        n2 = kg.kernel_launch_count()
        assert np.array_equal(g1, ref) and np.array_equal(g2, ref)
        assert n2 - n1 == n1 - n0 > 0


def test_cuda_graph_device_api_stream():
    import torch
    rng = np.random.default_rng(3)
    H = models.square_anderson(16, W=1.0, rng=rng)
    op = kg.GB300Operator((H / 4.6).tocsc())
    NC, NR = 96, 8
    psi = ko.random_phase_vectors(rng, 256, NR)
    psi_t = torch.from_numpy(np.ascontiguousarray(psi.T)).cuda()
    s = torch.cuda.Stream()
    outs = []
    mu_t = torch.zeros((NC, NR), dtype=torch.complex128, device="cuda")
    for use_graph in (False, True, True):
        mu_t.zero_()
        # the inputs and the zero fill were queued on torch's current stream;
        # s is a separate non-blocking stream, so order it after them
        s.wait_stream(torch.cuda.current_stream())
        kg.kpm_1d_device(op, NC, psi_t, mu_t, precision="ff", stream=s, use_graph=use_graph,
                         kernel="gather")
        kg.sync(op, s)
        outs.append(mu_t.cpu().numpy())
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])


@pytest.mark.parametrize("prec", ["fp64", "ff"])
@pytest.mark.parametrize("NR", [5, 12, 40, 64])
def test_autotuned_kernel_matches_oracle(prec, NR):
    rng = np.random.default_rng(NR)
    H = models.square_anderson(20, W=2.0, rng=rng)
    H = (H / 5.1).tocsc()
    op = kg.GB300Operator(H)
    psi = ko.random_phase_vectors(rng, 400, NR)
    ref = ko.kpm_1d_doubling(H, 64, psi)
    a = kg.kpm_1d(op, 64, NR, psi_in=psi, avg_output=False, precision=prec, kernel="tune")
    b = kg.kpm_1d(op, 64, NR, psi_in=psi, avg_output=False, precision=prec, kernel="tune",
                  use_graph=True)
    assert relerr(a, ref) < TOL[prec]
    assert np.array_equal(a, b)
    lr = kg.kpm_1d(op, 33, NR, psi_in_l=psi, psi_in_r=psi, avg_output=False, precision=prec,
                   kernel="tune")
    assert relerr(lr, ko.kpm_1d_lr(H, 33, psi, psi)) < TOL[prec]


def _peierls_square(L, rng):
    """Complex Hermitian square lattice (5 nonzeros per row)."""
    H = models.square_anderson(L, W=1.5, rng=rng).tocoo()
    ph = np.exp(1j * 0.37 * (H.row - H.col))
    return sp.csc_matrix((H.data * ph, (H.row, H.col)), shape=H.shape) / 4.9


@pytest.mark.parametrize("prec", ["fp64", "ff"])
@pytest.mark.parametrize("NR", [1, 5, 12, 64, 200, 256])
@pytest.mark.parametrize("lr", [False, True])
def test_single_launch_kernel_matches_oracle(prec, NR, lr):
    """kernel variant 6: the whole recurrence in one cooperative launch"""
    rng = np.random.default_rng(3 * NR + lr)
    H = _peierls_square(16, rng) if lr else (models.square_anderson(16, W=2.0, rng=rng) / 5.1).tocsc()
    psi = ko.random_phase_vectors(rng, 256, NR)
    if lr:
        psr = ko.random_phase_vectors(rng, 256, NR)
        got = kg.kpm_1d(H, 37, NR, psi_in_l=psi, psi_in_r=psr, avg_output=False, precision=prec,
                        kernel="single")
        ref = ko.kpm_1d_lr(H, 37, psi, psr)
    else:
        got = kg.kpm_1d(H, 128, NR, psi_in=psi, avg_output=False, precision=prec, kernel="single")
        ref = ko.kpm_1d_doubling(H, 128, psi)
    assert relerr(got, ref) < TOL[prec]


def test_single_launch_kernel_growth_and_limits():
    rng = np.random.default_rng(2)
    H = (models.square_anderson(12, W=0.0, rng=rng) / 3.0).tocsc()   # spectrum beyond [-1, 1]
    psi = ko.random_phase_vectors(rng, 144, 4)
    with pytest.raises(kg.KPMNumericalError):
        kg.kpm_1d(H, 64, 4, psi_in=psi, kernel="single", stability_check=True)
    ok = (models.square_anderson(12, W=0.0, rng=rng) / 4.4).tocsc()
    kg.kpm_1d(ok, 64, 4, psi_in=psi, kernel="single", stability_check=True)
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d(ok, 16, 257, psi_in=ko.random_phase_vectors(rng, 144, 257), kernel="single")


@pytest.mark.parametrize("NR", [33, 48, 64])
@pytest.mark.parametrize("lr", [False, True])
def test_padded_row_kernel_real_matches_oracle(NR, lr):
    """kernel variant 9: fixed-width padded rows; the recurrence vectors are
    bitwise those of the register-gather kernel, so the moments agree with it
    to rounding of the (differently partitioned) sums"""
    rng = np.random.default_rng(NR + 7 * lr)
    H = (models.cubic_anderson(7, W=4.0, rng=rng) / 8.2).tocsc()
    NH = H.shape[0]
    psi = ko.random_phase_vectors(rng, NH, NR)
    if lr:
        psr = ko.random_phase_vectors(rng, NH, NR)
        kw = dict(psi_in_l=psi, psi_in_r=psr)
        NC, ref = 41, ko.kpm_1d_lr(H, 41, psi, psr)
    else:
        kw = dict(psi_in=psi)
        NC, ref = 96, ko.kpm_1d_doubling(H, 96, psi)
    got = kg.kpm_1d(H, NC, NR, avg_output=False, precision="ff", kernel="padded", **kw)
    gat = kg.kpm_1d(H, NC, NR, avg_output=False, precision="ff", kernel="gather", **kw)
    assert relerr(got, ref) < TOL["ff"]
    assert relerr(got, gat) < 1e-13


@pytest.mark.parametrize("NR", [33, 40, 64])
@pytest.mark.parametrize("dot", ["doubling", "lr"])
@pytest.mark.parametrize("W", [5, 7, 8])
def test_streaming_kernel_matches_oracle(NR, dot, W):
    """kernel variant 11 (row-streaming, real H, 33..64 columns, rows of 5..8
    nonzeros, one anchored chunk per row, loads prefetched across rows): moments
    against the oracle and against the register-gather kernel; the doubling
    moments' imaginary parts are exactly 0 (Hermitian H)."""
    rng = np.random.default_rng(NR + 11 * W)
    if W == 7:
        H = (models.cubic_anderson(7, W=4.0, rng=rng) / 8.2).tocsc()
    else:
        H = _ragged_herm(rng, 300, W, False)
        while np.diff(H.tocsr().indptr).max() != W:       # exactly W in the longest row
            H = _ragged_herm(rng, 300, W, False)
    NH = H.shape[0]
    psi = ko.random_phase_vectors(rng, NH, NR)
    if dot == "lr":
        psr = ko.random_phase_vectors(rng, NH, NR)
        kw = dict(psi_in_l=psi, psi_in_r=psr)
        NC, ref = 41, ko.kpm_1d_lr(H, 41, psi, psr)
    else:
        kw = dict(psi_in=psi)
        NC, ref = 96, ko.kpm_1d_doubling(H, 96, psi)
    got = kg.kpm_1d(H, NC, NR, avg_output=False, precision="ff", kernel="streaming", **kw)
    gat = kg.kpm_1d(H, NC, NR, avg_output=False, precision="ff", kernel="gather", **kw)
    assert relerr(got, ref) < TOL["ff"]
    assert relerr(got, gat) < 1e-12
    if dot == "doubling":
        assert np.all(got.imag == 0.0)


@pytest.mark.parametrize("NR", [9, 16, 24, 32])
@pytest.mark.parametrize("dot", ["doubling", "lr"])
@pytest.mark.parametrize("case", ["peierls", "haldane", "ragged12", "ragged7"])
def test_streaming_kernel_complex_matches_oracle(NR, dot, case):
    """kernel variant 11 on complex operators (k_step_ffc: 9..32 columns, one
    column per lane, rows padded to 8 or 12 slots)."""
    rng = np.random.default_rng(NR + (7 if dot == "lr" else 0) + len(case))
    if case == "peierls":
        H = _peierls_square(16, rng)                        # 5 nonzeros per row
    elif case == "haldane":
        Hh, _, _, _ = models.haldane(8, 8, t2=0.2, m=0.1)   # 10 nonzeros per row
        H = (Hh / 3.8).tocsc()
    else:
        w = int(case[6:])
        H = _ragged_herm(rng, 240, w, True)
        while np.diff(H.tocsr().indptr).max() < w - 1:
            H = _ragged_herm(rng, 240, w, True)
    NH = H.shape[0]
    psi = ko.random_phase_vectors(rng, NH, NR)
    if dot == "lr":
        psr = ko.random_phase_vectors(rng, NH, NR)
        kw = dict(psi_in_l=psi, psi_in_r=psr)
        NC, ref = 37, ko.kpm_1d_lr(H, 37, psi, psr)
    else:
        kw = dict(psi_in=psi)
        NC, ref = 80, ko.kpm_1d_doubling(H, 80, psi)
    got = kg.kpm_1d(H, NC, NR, avg_output=False, precision="ff", kernel="streaming", **kw)
    gat = kg.kpm_1d(H, NC, NR, avg_output=False, precision="ff", kernel="gather", **kw)
    assert relerr(got, ref) < TOL["ff"]
    # both float-float; one anchored chunk per row here against chunks of 8
    # (+ the rest) in the CSR kernel: different roundings at ~1e-12
    assert relerr(got, gat) < 1e-11
    if dot == "doubling":
        assert np.all(got.imag == 0.0)


def test_streaming_kernel_limits():
    rng = np.random.default_rng(4)
    H = (models.cubic_anderson(5, W=1.0, rng=rng) / 7.0).tocsc()
    psi = ko.random_phase_vectors(rng, 125, 40)
    with pytest.raises(kg.KPMArgumentError):   # 8 columns
        kg.kpm_1d(H, 16, 8, psi_in=psi[:, :8], precision="ff", kernel="streaming")
    with pytest.raises(kg.KPMArgumentError):   # bra/ket path with 32 columns
        kg.kpm_1d(H, 16, 32, psi_in_l=psi[:, :32], psi_in_r=psi[:, 8:], precision="ff",
                  kernel="streaming")
    with pytest.raises(kg.KPMArgumentError):   # FP64
        kg.kpm_1d(H, 16, 40, psi_in=psi, precision="fp64", kernel="streaming")
    Hc = _peierls_square(8, rng)               # complex operator, 40 columns
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d(Hc, 16, 40, psi_in=ko.random_phase_vectors(rng, 64, 40), precision="ff",
                  kernel="streaming")
    with pytest.raises(kg.KPMArgumentError):   # complex operator, 8 columns
        kg.kpm_1d(Hc, 16, 8, psi_in=ko.random_phase_vectors(rng, 64, 8), precision="ff",
                  kernel="streaming")
    long_rows = _ragged_herm(rng, 80, 13, False)
    long_rows = long_rows if np.diff(long_rows.tocsr().indptr).max() > 8 else None
    if long_rows is not None:
        with pytest.raises(kg.KPMArgumentError):
            kg.kpm_1d(long_rows, 16, 40, psi_in=ko.random_phase_vectors(rng, 80, 40),
                      precision="ff", kernel="streaming")


def _ragged_herm(rng, n, max_row, complex_h):
    """Hermitian operator with row lengths spread over 0..max_row (some rows
    empty), scaled into the Chebyshev domain."""
    rows, cols = [], []
    for i in range(n):
        k = int(rng.integers(0, max_row // 2 + 1))
        for j in rng.choice(n, size=k, replace=False):
            rows.append(i)
            cols.append(int(j))
    vals = rng.standard_normal(len(rows)) + (1j * rng.standard_normal(len(rows)) if complex_h else 0)
    A = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    A = (A + A.conj().T).tocsc()
    A.sum_duplicates()
    deg = np.diff(A.indptr)
    keep = deg <= max_row
    A = sp.diags(keep.astype(float)) @ A @ sp.diags(keep.astype(float))
    A = sp.csc_matrix(A)
    A.eliminate_zeros()
    return A / (1.05 * max(np.abs(np.linalg.eigvalsh(A.toarray())).max(), 1e-3))


@pytest.mark.parametrize("max_row", [3, 8, 13, 16])
@pytest.mark.parametrize("complex_h,NR", [(False, 6), (False, 12), (False, 40), (False, 64),
                                          (True, 5), (True, 16), (True, 32)])
def test_padded_row_kernel_ragged_rows(max_row, complex_h, NR):
    """padding of short, empty and 4k+r rows for every table width 4..16, on
    every lane shape (8, 16 and 32 lanes per row, one or two columns each)"""
    rng = np.random.default_rng(max_row * 3 + NR)
    H = _ragged_herm(rng, 150, max_row, complex_h)
    psi = ko.random_phase_vectors(rng, 150, NR)
    got = kg.kpm_1d(H, 64, NR, psi_in=psi, avg_output=False, precision="ff", kernel="padded")
    ref = ko.kpm_1d_doubling(H, 64, psi)
    gat = kg.kpm_1d(H, 64, NR, psi_in=psi, avg_output=False, precision="ff", kernel="gather")
    assert relerr(got, ref) < TOL["ff"]
    # bitwise recurrence vectors where both kernels chunk by 4 (real H with 33..64
    # columns, complex H with 9..32); chunks of 8 in k_step_ff elsewhere
    same_chunks = (NR > 32) if not complex_h else (8 < NR <= 32)
    assert relerr(got, gat) < (1e-13 if same_chunks else 1e-12)


def test_padded_row_kernel_limits():
    rng = np.random.default_rng(9)
    H = (models.cubic_anderson(5, W=1.0, rng=rng) / 7.0).tocsc()
    psi = ko.random_phase_vectors(rng, 125, 16)
    with pytest.raises(kg.KPMArgumentError):   # 4 columns
        kg.kpm_1d(H, 16, 4, psi_in=psi[:, :4], precision="ff", kernel="padded")
    dense = _ragged_herm(rng, 60, 40, False)   # rows longer than 16
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d(dense, 16, 40, psi_in=ko.random_phase_vectors(rng, 60, 40), precision="ff",
                  kernel="padded")


@pytest.mark.parametrize("prec", ["fp64", "ff"])
@pytest.mark.parametrize("case", ["anderson16", "anderson64", "anderson_150", "peierls19",
                                  "cubic28", "anderson_220"])
@pytest.mark.parametrize("lr", [False, True])
def test_cluster_kernel_matches_oracle(prec, case, lr):
    """kernel variant 10: one thread-block cluster per probe column, the
    recurrence in distributed shared memory (1, 8 and 16 CTAs per cluster; the
    operator's rows cached in shared memory or read from global memory)"""
    rng = np.random.default_rng(len(case) + 3 * lr)
    if case == "anderson16":
        H = (models.square_anderson(16, W=2.0, rng=rng) / 5.1).tocsc()      # 1 CTA
    elif case == "anderson64":
        H = (models.square_anderson(64, W=2.0, rng=rng) / 5.1).tocsc()      # 8 CTAs
    elif case == "anderson_150":
        H = (models.square_anderson(150, W=2.0, rng=rng) / 5.1).tocsc()     # 16 x 1407 rows
    elif case == "anderson_220":
        H = (models.square_anderson(220, W=2.0, rng=rng) / 5.1).tocsc()     # 16 x 3025 rows:
        # the CTAs' rows of the operator do not fit beside the slots (uncached path)
    elif case == "cubic28":
        H = (models.cubic_anderson(28, W=4.0, rng=rng) / 8.2).tocsc()       # 16 x 1372 rows
    else:
        H = _peierls_square(19, rng)                                        # complex, 361 rows
    NH = H.shape[0]
    NR = 5 if case != "anderson64" else 12
    psi = ko.random_phase_vectors(rng, NH, NR)
    if lr:
        psr = ko.random_phase_vectors(rng, NH, NR)
        got = kg.kpm_1d(H, 37, NR, psi_in_l=psi, psi_in_r=psr, avg_output=False, precision=prec,
                        kernel="cluster")
        ref = ko.kpm_1d_lr(H, 37, psi, psr)
        tol = TOL[prec]
    else:
        got = kg.kpm_1d(H, 96, NR, psi_in=psi, avg_output=False, precision=prec, kernel="cluster")
        ref = ko.kpm_1d_doubling(H, 96, psi)
        # FP64 noise floor of the doubling moments on this operator: the oracle's
        # own doubling and step-by-step paths differ by up to 2e-12 on 22500 rows
        floor = relerr(ref, ko.kpm_1d_lr(H, 96, psi, psi))
        tol = max(TOL[prec], 3 * floor)
    assert relerr(got, ref) < tol


def test_cluster_kernel_growth_and_capacity():
    rng = np.random.default_rng(4)
    H = (models.square_anderson(12, W=0.0, rng=rng) / 3.0).tocsc()   # spectrum beyond [-1, 1]
    psi = ko.random_phase_vectors(rng, 144, 4)
    with pytest.raises(kg.KPMNumericalError):
        kg.kpm_1d(H, 64, 4, psi_in=psi, kernel="cluster", stability_check=True)
    big = (models.cubic_anderson(50, W=1.0, rng=rng) / 7.0).tocsc()  # 125000 rows per column
    with pytest.raises(kg.KPMArgumentError):
        kg.kpm_1d(big, 8, 2, psi_in=ko.random_phase_vectors(rng, 125000, 2), kernel="cluster")
    # the operator and context stay usable
    ok = (models.square_anderson(12, W=1.0, rng=rng) / 5.0).tocsc()
    got = kg.kpm_1d(ok, 32, 4, psi_in=psi, avg_output=False, kernel="cluster")
    assert relerr(got, ko.kpm_1d_doubling(ok, 32, psi)) < TOL["fp64"]


@pytest.mark.parametrize("lr", [False, True])
def test_pinned_host_probes_match_pageable(lr):
    """Probe blocks in pinned host memory are read by the copy kernel (from
    1 MiB up), pageable ones by cudaMemcpyAsync: the moments agree bitwise."""
    import torch
    rng = np.random.default_rng(61)
    H = (models.square_anderson(96, W=2.0, rng=rng) / 5.1).tocsc()
    NH, NR, NC = H.shape[0], 16, 64
    psi = ko.random_phase_vectors(rng, NH, NR)          # 2.4 MB
    op = kg.GB300Operator(H)
    pinned = torch.empty((NR, NH), dtype=torch.complex128, pin_memory=True)
    pinned.numpy()[...] = psi.T
    host_psi = pinned.numpy().T
    a = np.zeros((NR, NC), dtype=np.complex128)
    b = np.zeros((NR, NC), dtype=np.complex128)
    if lr:
        kg.kpm_1d_bang(op, NC, NR, NH, a, np.asfortranarray(psi), np.asfortranarray(psi))
        kg.kpm_1d_bang(op, NC, NR, NH, b, host_psi, host_psi)
    else:
        kg.kpm_1d_bang(op, NC, NR, NH, a, np.asfortranarray(psi))
        kg.kpm_1d_bang(op, NC, NR, NH, b, host_psi)
    assert np.array_equal(a, b)
    assert relerr(a, ko.kpm_1d_lr(H, NC, psi, psi) if lr else ko.kpm_1d_doubling(H, NC, psi)) < 1e-12
    # the library's own page-locked buffers (kpmgb_host_alloc)
    own = kg.pinned_empty((NH, NR), np.complex128, "F")
    own[...] = psi
    c = np.zeros((NR, NC), dtype=np.complex128)
    if lr:
        kg.kpm_1d_bang(op, NC, NR, NH, c, own, own)
    else:
        kg.kpm_1d_bang(op, NC, NR, NH, c, own)
    assert np.array_equal(a, c)


@pytest.mark.parametrize("NR", [9, 12, 16, 17, 24, 32, 33, 40, 48, 63, 64])
@pytest.mark.parametrize("W", [5, 7, 8])
def test_packed_kernels_match_oracle(NR, W):
    """Float-float doubling steps of real operators with 9..64 columns run on
    packed FP32 pairs in the paired vector layout: one column per lane for
    9..32 columns (k_step_ffpk1), two per lane for 33..64 (k_step_ffpk, idle
    lanes masked below 64).  Against the oracle and the register-gather
    kernel; the doubling moments' imaginary parts are exactly 0."""
    rng = np.random.default_rng(100 + NR + 7 * W)
    if W == 7:
        H = (models.cubic_anderson(7, W=4.0, rng=rng) / 8.2).tocsc()
    else:
        H = _ragged_herm(rng, 300, W, False)
        while np.diff(H.tocsr().indptr).max() != W:
            H = _ragged_herm(rng, 300, W, False)
    NH = H.shape[0]
    psi = ko.random_phase_vectors(rng, NH, NR)
    got = kg.kpm_1d(H, 96, NR, psi_in=psi, avg_output=False, precision="ff", kernel="streaming")
    gat = kg.kpm_1d(H, 96, NR, psi_in=psi, avg_output=False, precision="ff", kernel="gather")
    assert relerr(got, ko.kpm_1d_doubling(H, 96, psi)) < TOL["ff"]
    assert relerr(got, gat) < 1e-12
    assert np.all(got.imag == 0.0)


@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_operators_rebuilt_on_cached_blocks(prec):
    """Operators and workspaces built and destroyed in a loop reuse released
    device blocks (the library's block cache): every rebuilt operator gives
    its first build's moments bitwise, and the oracle's."""
    rng = np.random.default_rng(91)
    Hs = [(models.square_anderson(L, W=2.0, rng=rng) / 5.1).tocsc() for L in (40, 23, 40, 57)]
    psis = [ko.random_phase_vectors(rng, H.shape[0], 12) for H in Hs]
    first = {}
    for rep in range(3):
        for i, (H, psi) in enumerate(zip(Hs, psis)):
            op = kg.GB300Operator(H)
            mu = kg.kpm_1d(op, 128, 12, psi_in=psi, avg_output=False, precision=prec)
            del op
            if rep == 0:
                first[i] = mu
                assert relerr(mu, ko.kpm_1d_doubling(H, 128, psi)) < TOL[prec]
            else:
                assert np.array_equal(mu, first[i])
