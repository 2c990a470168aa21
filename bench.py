#!/usr/bin/env python
"""Benchmark of the kpm_1d Chebyshev-moment path on GB300.

Workload (default): kpm_1d DOS at scale on a 3D cubic Anderson model, L=128
periodic (NH = 2,097,152, 7 nonzeros per row), t = 1, onsite uniform
[-8.25, 8.25] (W = 16.5), ComplexF64, centred rescaling, NC = 4096 moments,
NR = 64 random-phase probes.  Synthetic seeded inputs; the vectors (2.1 GB per
slot) are far larger than L2, so no flush is needed between steps.

A step is one full kpm_1d call (NC/2 = 2048 recurrence launches).  `value` is
vector-steps/s (NR * NC/2 per call) with the probes resident in HBM, timed with
CUDA events on the launching stream; `e2e` is the same metric through the
public host API (pinned host probes copied in, moments copied out, every step).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for _p in (ROOT, ROOT / "kpm.jl_gb300"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

import numpy as np  # noqa: E402

METRIC = "kpm_1d vector-steps/s"
UNIT = "vector-steps/s"
FALLBACK_HBM_GBS = 6800.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--precision", default="ff", choices=["ff", "fp64"])
    p.add_argument("--L", type=int, default=128)
    p.add_argument("--W", type=float, default=16.5)
    p.add_argument("--NC", type=int, default=4096)
    p.add_argument("--NR", type=int, default=64)
    p.add_argument("--cpu-steps", type=int, default=16,
                   help="recurrence steps in the bounded CPU-baseline sample")
    p.add_argument("--kernel", default="auto",
                   choices=["auto", "gather", "tune", "padded", "streaming"],
                   help="float-float step kernel of the headline call")
    p.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-cond", action="store_true",
                   help="skip the kpm_2d (tensor-core contraction) summary of the headline line")
    p.add_argument("--no-secondary", action="store_true",
                   help="skip the c1 / c4 / c5 summary of the headline line")
    p.add_argument("--workload", default="dos",
                   choices=["dos", "dos-small", "cond", "ensemble", "grad", "action", "dsigma",
                            "published"],
                   help="dos (default): the headline kpm_1d line on the 3D Anderson model; "
                        "the others print one JSON line each: dos-small (2D Anderson L=64), "
                        "cond (kpm_2d + Kubo-Bastin on the Haldane model), ensemble (256 "
                        "realisations), grad (adjoint gradient on graphene), action "
                        "(chebyshev_action)")
    p.add_argument("--haldane-L", type=int, default=256, help="cond: Haldane cells per side")
    p.add_argument("--cond-NC", type=int, default=512, help="cond: Chebyshev moments per side")
    p.add_argument("--contraction", default="both", choices=["both", "split", "fp64"],
                   help="cond: which kpm_2d contraction(s) to time")
    return p.parse_args()


def workload(args, rank):
    from kpm_gb300 import models, rescale, random_phase_vectors
    rng = np.random.default_rng(42)
    H = models.cubic_anderson(args.L, t=1.0, W=args.W, rng=rng)
    h = rescale(H, center=True)
    psi = random_phase_vectors(np.random.default_rng(1000 + rank), H.shape[0], args.NR)
    return h, psi


def config(args, scaling_note=None):
    NH = args.L ** 3
    return {
        "workload": (f"kpm_1d DOS, 3D cubic Anderson L={args.L} periodic (NH={NH}, 7 nnz/row), "
                     f"W={args.W}, centred rescaling, NC={args.NC}, NR={args.NR}"),
        "NH": NH, "NC": args.NC, "NR": args.NR, "nnz_per_row": 7,
        "precision": args.precision,
        "step_kernel": args.kernel,
        "l2": "inputs larger than L2 (2.1 GB per recurrence slot), no flush needed",
        "step": "one kpm_1d call = NC/2 recurrence launches with fused moments",
    }


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.f = None

    def __enter__(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.f:
            return None
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return None
        def num(x):
            try:
                return float(x)
            except ValueError:
                return math.nan
        sm = [num(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" == r[5 + i]})
        return {"sm_mhz": statistics.median([s for s in sm if not math.isnan(s)] or [0]),
                "sm_max_mhz": max(num(r[2]) for r in rows), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(num(r[3]) for r in rows)}


def measured_hbm():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return float(json.loads(f.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return FALLBACK_HBM_GBS, "fallback"


def profile_traffic(precision):
    """DRAM bytes per step launch from the committed ncu summary, if present."""
    f = ROOT / "profiles" / f"kpm1d_step_{precision}_traffic.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch_full_size:"):
            return float(line.split(":", 1)[1])
    return None


def cpu_sample(h, psi, args, nthreads):
    """The C port of the reference CPU algorithm on a bounded sample of the workload."""
    from oracle import cpu_port
    steps = max(2, min(args.cpu_steps, args.NC // 2))
    t0 = time.perf_counter()
    mu = cpu_port.kpm1d_cpu(h.H, args.NC, psi, nthreads=nthreads, last_n=steps)
    dt = time.perf_counter() - t0
    return {"value": args.NR * steps / dt, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": (f"first {steps} of {args.NC // 2} recurrence steps of the same workload "
                       f"(NR={args.NR} columns each), C/OpenMP restatement of the reference "
                       f"CPU path, {nthreads} threads"),
            "seconds": dt}, mu, steps


def run_reference(args, rank, world):
    """--impl reference: the reference CPU algorithm (C port) on this machine's host cores."""
    if rank != 0:
        return
    from oracle import cpu_port
    h, psi = workload(args, 0)
    nthreads = cpu_port.max_threads()
    for _ in range(args.warmup):
        cpu_sample(h, psi, args, nthreads)
    times, vals = [], []
    for _ in range(args.steps):
        res, _, steps = cpu_sample(h, psi, args, nthreads)
        times.append(res["seconds"])
        vals.append(res["value"])
    value = args.NR * steps * args.steps / sum(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(times) / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config(args),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": res["sample"]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": ("KPM.jl is Julia and Julia is not installed; the reference arm runs the "
                 "C/OpenMP restatement of its CPU algorithm (oracle/kpm_cpu.c)"),
    }
    print(json.dumps(line), flush=True)


def measured_bf16():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return float(json.loads(f.read_text())["bf16_tflops"]), "measured"
        except (KeyError, ValueError):
            pass
    return 1900.0, "fallback"


# FP64 operations of the plain recurrence per row x column x step for a real
# operator: 2 FMAs per nonzero (re, im), the update alpha*acc + beta*z (2 MUL +
# 2 FMA) and the doubling dots <x|x> (2 FMA) and <x|y> (4 FMA); an FMA counts 2.
def fp64_flop_per_row_col(nnz_per_row, real=True):
    per_nz = 4 if real else 8
    return per_nz * nnz_per_row + 6 + 12


def cond_summary(args):
    """kpm_2d on the Haldane model 256x256 cells (NH=131072), t2 = 0.1 i,
    NC=512, NR=16: the split tensor-core contraction against the FP64 one,
    the contraction kernel's own device time (CUDA events around its launch on
    the launching stream), and sigma_xy(Ef=0)."""
    import torch
    import kpm_gb300 as kg
    from kpm_gb300 import _native, models, rescale
    H, Jx, Jy, area = models.haldane(256, 256, t=1.0, t2=0.1)
    h = rescale(H, center=True)
    NH, NR, NC = H.shape[0], 16, 512
    psi = kg.random_phase_vectors(np.random.default_rng(42), NH, NR)
    ops = [kg.GB300Operator(M) for M in (h.H, Jx, Jy)]
    s = torch.cuda.Stream()
    psi_t = torch.from_numpy(np.ascontiguousarray(psi.T)).cuda()
    K = NH * NR
    F = 8.0 * NC * NC * K               # complex-FP64-equivalent flop per call
    F_bf16 = 15 * F                     # 15 digit-pair BF16 products per real product
    out = {"workload": f"kpm_2d, Haldane 256x256x2 (NH={NH}), t2=0.1i, NC={NC}, NR={NR}; "
                       "sigma_xy(Ef=0)"}
    res = {}
    for prec, contraction, steps in (("ff", "split", 3), ("fp64", "fp64", 1)):
        mu_t = torch.zeros((NC, NC), dtype=torch.complex128, device="cuda")
        call = lambda: kg.kpm_2d_device(ops[0], ops[1], ops[2], NC, psi_t, psi_t, mu_t,
                                        precision=prec, contraction=contraction, stream=s)
        call()
        kg.sync(ops[0], s)
        kname = "contract_split" if contraction == "split" else "contract_fp64"
        _native.timing_read(kname)               # drop the warm-up call's events
        _native.timing_enable(True)
        try:
            ms = _time_device(call, s, 0, steps, lambda: kg.sync(ops[0], s))
        finally:
            _native.timing_enable(False)
        kms, klaunch = _native.timing_read(kname)
        res[contraction] = mu_t.cpu().numpy().T.copy()
        out[f"{prec}_recurrence_{contraction}_contraction_ms"] = ms
        out[f"{contraction}_contraction_kernel_ms_per_call"] = kms / steps
        out[f"{contraction}_contraction_launches_per_call"] = klaunch / steps
    peak, kind = measured_bf16()
    tc_ms = out["split_contraction_kernel_ms_per_call"]
    achieved = F_bf16 / (tc_ms / 1e3) / 1e12
    out["split_contraction_roofline"] = {
        "bound": "tensor", "kernel": "k_contract_tc", "achieved": achieved, "peak": peak,
        "unit": "TFLOP/s", "frac": achieved / peak,
        "peak_source": f"{kind} (MEASURED_PEAKS.json bf16_tflops, burst)",
        "bf16_flop_per_call": F_bf16,
        "note": "BF16 work = 15 digit-pair products x 8*NC^2*NH*NR"}
    out["fp64_contraction_kernel_tflops"] = F / (out["fp64_contraction_kernel_ms_per_call"] / 1e3) / 1e12
    out["split_vs_fp64_rel_err"] = float(np.linalg.norm(res["split"] - res["fp64"])
                                         / np.linalg.norm(res["fp64"]))
    out["speedup_split_vs_fp64"] = (out["fp64_recurrence_fp64_contraction_ms"]
                                    / out["ff_recurrence_split_contraction_ms"])
    sig = kg.kubo_bastin_cond(res["split"], h.a, np.array([0.0]), b=h.b, NH=NH, area=area)
    sig64 = kg.kubo_bastin_cond(res["fp64"], h.a, np.array([0.0]), b=h.b, NH=NH, area=area)
    out["sigma_xy_at_Ef0_split"] = float(sig[0])
    out["sigma_xy_at_Ef0_fp64"] = float(sig64[0])
    return out


# ------------------------------------------------------------ secondary workloads
def _events(stream):
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _time_device(fn, stream, warmup, steps, sync):
    """Average ms of fn() over `steps` calls on `stream` (CUDA events), after warm-up."""
    import torch
    for _ in range(warmup):
        fn()
    sync()
    torch.cuda.synchronize()
    e0, e1 = _events(stream)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    sync()
    return e0.elapsed_time(e1) / steps


def secondary_summary(args):
    """Compact numbers of the other benchmark configurations for the headline
    line: c1 (2D Anderson L=64, NC=1024, NR=12, device-resident), c4 (256
    ensemble members, NC=512, NR=8, device-resident) and c5 (gradient of a
    DOS-window loss, graphene 128x128, NC=1024, NR=16, host API)."""
    import torch
    import kpm_gb300 as kg
    from kpm_gb300 import models, rescale
    out = {}
    # c1
    H = models.square_anderson(64, W=2.0, rng=np.random.default_rng(42))
    h = rescale(H)
    NH, NR, NC = 4096, 12, 1024
    psi = kg.random_phase_vectors(np.random.default_rng(42), NH, NR)
    op = kg.GB300Operator(h.H)
    st = torch.cuda.Stream()
    psi_t = torch.from_numpy(np.ascontiguousarray(psi.T)).cuda()
    mu_t = torch.zeros((NC, NR), dtype=torch.complex128, device="cuda")
    c1 = {"workload": "kpm_1d, 2D square Anderson L=64 (NH=4096), NC=1024, NR=12"}
    for prec in ("fp64", "ff"):
        ms = _time_device(lambda: kg.kpm_1d_device(op, NC, psi_t, mu_t, precision=prec, stream=st),
                          st, 3, 10, lambda: kg.sync(op, st))
        c1[prec] = {"ms_per_call": ms, "value": NR * NC / 2 / (ms / 1e3)}
    # the reference's own CPU configuration: the C port of its CPU path, the
    # whole call on the host cores
    from oracle import cpu_port
    nt = cpu_port.max_threads()
    t0 = time.perf_counter()
    cpu_port.kpm1d_cpu(h.H, NC, psi, nthreads=nt)
    dt = time.perf_counter() - t0
    c1["cpu_baseline"] = {"ms_per_call": dt * 1e3, "value": NR * NC / 2 / dt, "cores": nt,
                          "kind": "port", "sample": "the whole call (512 steps)"}
    out["c1"] = c1
    # c4
    rng = np.random.default_rng(42)
    Hs, psis = [], []
    for _ in range(256):
        L = int(rng.integers(24, 97))
        W = float(rng.uniform(1.0, 8.0))
        Hs.append((models.square_anderson(L, W=W, rng=rng) / (4.0 + W / 2 + 0.1)).tocsc())
        psis.append(kg.random_phase_vectors(rng, L * L, 8))
    ens = kg.EnsembleOperator(Hs)
    NC4, NR4 = 512, 8
    epsi = torch.from_numpy(np.ascontiguousarray(np.vstack(psis).T)).cuda()
    emu = torch.zeros((256, NC4, NR4), dtype=torch.complex128, device="cuda")
    cur = torch.cuda.current_stream()
    c4 = {"workload": "256 x kpm_1d, 2D Anderson L~U{24..96}, NC=512, NR=8 (device-resident)"}
    for prec in ("fp64", "ff"):
        ms = _time_device(lambda: kg.kpm_1d_ensemble_device(ens, NC4, epsi, emu, precision=prec),
                          cur, 1, 3, lambda: kg.sync(ens.op))
        c4[prec] = {"ms_per_call": ms, "value": 256 * NR4 * NC4 / 2 / (ms / 1e3)}
    c4["ff_over_fp64"] = c4["fp64"]["ms_per_call"] / c4["ff"]["ms_per_call"]
    out["c4"] = c4
    # c5
    rng = np.random.default_rng(42)
    NH5 = 2 * 128 * 128
    H5 = (models.graphene(128, 128, onsite=0.1 * rng.standard_normal(NH5)) / 3.4).tocsc()
    NC5, NR5 = 1024, 16
    psi5 = kg.random_phase_vectors(rng, NH5, NR5)
    g5 = rng.standard_normal(NC5)
    op5 = kg.GB300Operator(H5)
    tf = _time_host(lambda: kg.kpm_1d(op5, NC5, NR5, psi_in=psi5), 1, 3)
    tg = _time_host(lambda: kg.kpm_1d_grad(op5, NC5, psi5, g5), 1, 3)
    out["c5"] = {"workload": "gradient of sum_m g_m mu_m, graphene 128x128, NC=1024, NR=16",
                 "forward_ms": tf, "gradient_ms": tg, "gradient_over_forward": tg / tf}
    return out


def _time_host(fn, warmup, steps):
    for _ in range(warmup):
        fn()
    t0 = time.perf_counter()
    for _ in range(steps):
        fn()
    return (time.perf_counter() - t0) * 1e3 / steps


def workload_dos_small(args):
    """2D square Anderson L=64 (NH=4096, 5 nnz/row), W=2, NC=1024, NR=12: the
    L2-resident configuration the CPU port runs in full."""
    import torch
    import kpm_gb300 as kg
    from kpm_gb300 import models, rescale
    from oracle import cpu_port
    H = models.square_anderson(64, W=2.0, rng=np.random.default_rng(42))
    h = rescale(H)
    NH, NR, NC = 4096, 12, 1024
    psi = kg.random_phase_vectors(np.random.default_rng(42), NH, NR)
    op = kg.GB300Operator(h.H)
    s = torch.cuda.Stream()
    psi_t = torch.from_numpy(np.ascontiguousarray(psi.T)).cuda()
    mu_t = torch.zeros((NC, NR), dtype=torch.complex128, device="cuda")
    vs = NR * NC // 2
    out = {"workload": "kpm_1d, 2D square Anderson L=64 (NH=4096), W=2, NC=1024, NR=12",
           "metric": METRIC, "unit": UNIT}
    for prec in ("fp64", "ff"):
        for mode in ("launches", "graph", "single", "cluster"):
            ms = _time_device(lambda: kg.kpm_1d_device(op, NC, psi_t, mu_t, precision=prec,
                                                       stream=s, use_graph=mode == "graph",
                                                       kernel=mode if mode in ("single", "cluster")
                                                       else "auto"),
                              s, args.warmup, max(args.steps, 10), lambda: kg.sync(op, s))
            out[f"{prec}_{mode}"] = {"ms_per_call": ms, "value": vs / (ms / 1e3)}
    ms_h = _time_host(lambda: kg.kpm_1d(op, NC, NR, psi_in=psi, use_graph=True), 2, 10)
    out["e2e_fp64_graph"] = {"ms_per_call": ms_h, "value": vs / (ms_h / 1e3)}
    nt = cpu_port.max_threads()
    t0 = time.perf_counter()
    cpu_port.kpm1d_cpu(h.H, NC, psi, nthreads=nt)
    dt = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": vs / dt, "unit": UNIT, "cores": nt, "kind": "port",
                           "sample": "the whole call (512 steps)"}
    return out


def workload_cond(args):
    """kpm_2d on the Haldane model 256x256 cells (NH=131072), NC=512, NR=16, then
    sigma_xy at 201 Fermi energies in [-3, 3]."""
    import torch
    import kpm_gb300 as kg
    from kpm_gb300 import models, rescale
    Lh = args.haldane_L
    H, Jx, Jy, area = models.haldane(Lh, Lh, t=1.0, t2=0.1)
    h = rescale(H, center=True)
    NH, NR, NC = H.shape[0], 16, args.cond_NC
    psi = kg.random_phase_vectors(np.random.default_rng(42), NH, NR)
    ops = [kg.GB300Operator(M) for M in (h.H, Jx, Jy)]
    s = torch.cuda.Stream()
    psi_t = torch.from_numpy(np.ascontiguousarray(psi.T)).cuda()
    F = 8.0 * NC * NC * NH * NR
    out = {"workload": f"kpm_2d, Haldane {Lh}x{Lh}x2 (NH={NH}), t2=0.1i, NC={NC}, NR=16; "
                       "sigma_xy at 201 Ef",
           "flop_per_call_complex_fp64_equivalent": F}
    mus = {}
    forms = {"split": [("ff", "split"), ("fp64", "split")], "fp64": [("fp64", "fp64")]}
    which = (forms["split"] + forms["fp64"]) if args.contraction == "both" else forms[args.contraction]
    for prec, contraction in which:
        key = f"{prec}_recurrence_{contraction}_contraction"
        mu_t = torch.zeros((NC, NC), dtype=torch.complex128, device="cuda")
        steps = 1 if contraction == "fp64" else max(args.steps, 1)
        ms = _time_device(lambda: kg.kpm_2d_device(ops[0], ops[1], ops[2], NC, psi_t, psi_t, mu_t,
                                                   precision=prec, contraction=contraction,
                                                   stream=s),
                          s, 1, steps, lambda: kg.sync(ops[0], s))
        mus[key] = mu_t.cpu().numpy().T.copy()
        out[key] = {"ms_per_call": ms, "TFLOP/s": F / (ms / 1e3) / 1e12}
    ref_key = "fp64_recurrence_fp64_contraction"
    if ref_key in mus:
        b = mus[ref_key]
        for k, a in mus.items():
            if k != ref_key:
                out[f"{k}_rel_err_vs_fp64"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    Efs = np.linspace(-3, 3, 201)
    t0 = time.perf_counter()
    last = f"{which[-1][0]}_recurrence_{which[-1][1]}_contraction"
    sig = kg.kubo_bastin_cond(mus[last], h.a, Efs, b=h.b, NH=NH, area=area)
    out["kubo_bastin_201_Ef_ms"] = (time.perf_counter() - t0) * 1e3
    out["sigma_xy_at_Ef0"] = float(sig[100])
    return out


def workload_dsigma(args):
    """dsigma_xy/dt2 at Ef=0 of the Haldane model, 64x64 cells (NH=8192), t2=0.2,
    NC=256, NR=8, fixed rescaling: host-API kpm_2d + reconstruction (forward)
    against kpm_2d_derivative (forward mode over the 2NH block operators) +
    reconstruction, both end to end from host arrays."""
    import kpm_gb300 as kg
    from kpm_gb300 import models, rescale
    L, t2, NC, NR = 64, 0.2, 256, 8
    H, Jx, Jy, area = models.haldane(L, L, t2=t2)
    H0, Jx0, Jy0, _ = models.haldane(L, L, t2=0.0)
    H1, Jx1, Jy1, _ = models.haldane(L, L, t2=1.0)
    h = rescale(H, center=True)
    NH = H.shape[0]
    dH, dJx, dJy = (H1 - H0) / h.a, Jx1 - Jx0, Jy1 - Jy0
    psi = kg.random_phase_vectors(np.random.default_rng(42), NH, NR)
    out = {"workload": "dsigma_xy/dt2 at Ef=0, Haldane 64x64x2 (NH=8192), t2=0.2, NC=256, NR=8"}
    steps = max(args.steps, 3)
    for contraction in ("fp64", "split"):
        res = {}

        def fwd():
            mu = kg.kpm_2d(h.H, Jx, Jy, NC, NR, NH, psi_in=psi, contraction=contraction)
            res["sigma"] = kg.kubo_bastin_cond(mu, h.a, 0.0, b=h.b, NH=NH, area=area)

        def der():
            dmu = kg.kpm_2d_derivative(h.H, dH, Jx, dJx, Jy, dJy, NC, NR, NH, psi_in=psi,
                                       contraction=contraction)
            res["dsigma"] = kg.kubo_bastin_cond(dmu, h.a, 0.0, b=h.b, NH=NH, area=area)
        tf = _time_host(fwd, 1, steps)
        td = _time_host(der, 1, steps)
        out[f"{contraction}_contraction"] = {
            "forward_ms": tf, "derivative_ms": td, "derivative_over_forward": td / tf,
            "sigma_xy": res["sigma"], "dsigma_xy_dt2": res["dsigma"]}
    # reverse mode: the gradient of sigma_xy(Ef=0) with respect to every stored
    # entry of H, Jx and Jy at once (kpmgb_kubo_bastin_weights + kpmgb_kpm2d_grad)
    def grad():
        W = kg.kubo_bastin_weights(NC, h.a, 0.0, b=h.b, NH=NH, area=area)
        res["grads"] = kg.kpm_2d_grad(h.H, Jx, Jy, NC, W, psi_in=psi)
    tfwd = out["fp64_contraction"]["forward_ms"]
    tg = _time_host(grad, 1, steps)
    gH, gJx, gJy = res["grads"]
    d_rev = _pair(gH, dH) + _pair(gJx, dJx) + _pair(gJy, dJy)
    out["reverse_mode_gradient"] = {
        "gradient_ms": tg, "gradient_over_forward_fp64": tg / tfwd,
        "entries": int(gH.nnz + gJx.nnz + gJy.nnz),
        "dsigma_xy_dt2_from_gradient": d_rev,
        "note": "one reverse pass gives d sigma / d (every stored entry of H, Jx, Jy); "
                "dsigma/dt2 follows by pairing with the t2 direction"}
    return out


def _pair(G, D):
    """sum_k Re(conj(G_k) D_k) over the stored entries of D (G: a gradient on a
    pattern that contains D's)."""
    import scipy.sparse as sp
    g, d = sp.coo_matrix(G), sp.coo_matrix(D)
    gd = {(i, j): v for i, j, v in zip(g.row, g.col, g.data)}
    return float(sum((np.conj(gd.get((i, j), 0.0)) * v).real for i, j, v in zip(d.row, d.col, d.data)))


def _square_lattice(L):
    """Periodic square lattice with hopping -1 on the four directed nearest-
    neighbour entries of every site and no diagonal, as the reference's own
    benchmark builds it (benchmarks/core_bench.jl:35-63); with currents."""
    import scipy.sparse as sp
    x, y = np.meshgrid(np.arange(L), np.arange(L), indexing="ij")
    x, y = x.ravel(), y.ravel()
    site = lambda a, b: (a % L) + L * (b % L)
    rows, cols, dxs, dys = [], [], [], []
    for ddx, ddy in ((1, 0), (-1, 0), (0, 1), (0, -1)):
        rows.append(site(x, y))
        cols.append(site(x + ddx, y + ddy))
        dxs.append(np.full(x.shape, -ddx))
        dys.append(np.full(x.shape, -ddy))
    r, c = np.concatenate(rows), np.concatenate(cols)
    v = -np.ones(r.shape, dtype=np.complex128)
    n = L * L
    H = sp.csc_matrix((v, (r, c)), shape=(n, n))
    Jx = sp.csc_matrix((v * np.concatenate(dxs), (r, c)), shape=(n, n))
    Jy = sp.csc_matrix((v * np.concatenate(dys), (r, c)), shape=(n, n))
    return H, Jx, Jy


def workload_published(args):
    """The reference's own benchmark suite (benchmarks/core_bench.jl), whose
    A100 times it publishes: kpm_1d DOS on the 256x256 (NC=1024, NR=8) and
    512x512 (NC=512, NR=4) periodic square lattices, kpm_2d on 128x128
    (NC=64, NR=4; default blocking and arr_size=64), chebyshev_action on
    256x256 (NC=1024, NR=8, K=2).  Timed end to end through the host API from
    host arrays: `per_call_operator` builds the device operator inside every
    call (as the reference converts and uploads H per call), `resident` reuses
    it.  Default (FP64) precision, as the reference; `resident_ff` and
    `resident_ff_split` add the chosen forms (float-float recurrences, split
    tensor-core contraction)."""
    import kpm_gb300 as kg
    rng = np.random.default_rng(42)
    steps = max(args.steps, 3)
    out = {"workload": "KPM.jl benchmarks/core_bench.jl suite (periodic square lattices)",
           "reference_a100_s": {"kpm_1d_NH65536_NC1024_NR8": 0.056766,
                                "kpm_1d_NH262144_NC512_NR4": 0.058475,
                                "kpm_2d_NH16384_NC64_NR4_default": 0.010318,
                                "kpm_2d_NH16384_NC64_NR4_arr64": 0.006348},
           "reference_a100_source": "benchmarks/results/perf-core-mike-a100.json:8-12"}
    for L, NC, NR in ((256, 1024, 8), (512, 512, 4)):
        H, _, _ = _square_lattice(L)
        a, Hn = kg.normalizeH(H)
        NH = L * L
        psi = kg.random_phase_vectors(rng, NH, NR)
        op = kg.GB300Operator(Hn)
        key = f"kpm_1d_NH{NH}_NC{NC}_NR{NR}"
        out[key] = {
            "per_call_operator_s": _time_host(lambda: kg.kpm_1d(Hn, NC, NR, NH, psi_in=psi), 1,
                                              steps) / 1e3,
            "resident_s": _time_host(lambda: kg.kpm_1d(op, NC, NR, NH, psi_in=psi), 1, steps) / 1e3,
            "resident_ff_s": _time_host(lambda: kg.kpm_1d(op, NC, NR, NH, psi_in=psi,
                                                          precision="ff"), 1, steps) / 1e3}
    H, Jx, Jy = _square_lattice(128)
    a, Hn = kg.normalizeH(H)
    NH = 128 * 128
    psi = kg.random_phase_vectors(rng, NH, 4)
    ops = [kg.GB300Operator(M) for M in (Hn, Jx, Jy)]
    for tag, kw in (("default", {}), ("arr64", {"arr_size": 64})):
        split = dict(kw, precision="ff", contraction="split")
        ref = kg.kpm_2d(*ops, 64, 4, NH, psi_in=psi, **kw)
        got = kg.kpm_2d(*ops, 64, 4, NH, psi_in=psi, **split)
        out[f"kpm_2d_NH16384_NC64_NR4_{tag}"] = {
            "per_call_operator_s": _time_host(lambda: kg.kpm_2d(Hn, Jx, Jy, 64, 4, NH, psi_in=psi,
                                                                **kw), 1, steps) / 1e3,
            "resident_s": _time_host(lambda: kg.kpm_2d(*ops, 64, 4, NH, psi_in=psi, **kw), 1,
                                     steps) / 1e3,
            # the chosen form: float-float recurrences, split tensor-core contraction
            "resident_ff_split_s": _time_host(lambda: kg.kpm_2d(*ops, 64, 4, NH, psi_in=psi,
                                                                **split), 1, steps) / 1e3,
            "ff_split_vs_fp64_rel_err": float(np.linalg.norm(got - ref) / np.linalg.norm(ref))}
    H, _, _ = _square_lattice(256)
    a, Hn = kg.normalizeH(H)
    V = kg.random_phase_vectors(rng, 65536, 8)
    n = np.arange(1024)
    C = np.stack([np.where(n == 0, 1.0, 2.0) * np.cos(n * np.pi / 2),
                  np.where(n == 0, 1.0, 2.0) * np.cos(n * 1.3)], axis=1)
    op = kg.GB300Operator(Hn)
    out["chebyshev_action_NH65536_NC1024_NR8_K2"] = {
        "resident_s": _time_host(lambda: kg.chebyshev_action(op, V, C, check_every=0), 1,
                                 steps) / 1e3}
    for k, ref in out["reference_a100_s"].items():
        ours = out[k]["per_call_operator_s"]
        out[k]["reference_a100_over_ours_per_call"] = ref / ours
    return out


def workload_ensemble(args):
    """256 realisations of the 2D Anderson model, L ~ U{24..96}, W ~ U[1, 8],
    NC=512, NR=8: the ensemble call (per-step schedule, persistent schedule,
    autotuned) against per-member calls."""
    import kpm_gb300 as kg
    from kpm_gb300 import models
    rng = np.random.default_rng(42)
    Hs, psis = [], []
    for _ in range(256):
        L = int(rng.integers(24, 97))
        W = float(rng.uniform(1.0, 8.0))
        Hs.append((models.square_anderson(L, W=W, rng=rng) / (4.0 + W / 2 + 0.1)).tocsc())
        psis.append(kg.random_phase_vectors(rng, L * L, 8))
    NC, NR = 512, 8
    vs = 256 * NR * NC // 2
    out = {"workload": "256 x kpm_1d, 2D Anderson L~U{24..96}, W~U[1,8], NC=512, NR=8",
           "metric": METRIC, "unit": UNIT, "mean_NH": float(np.mean([H.shape[0] for H in Hs]))}
    t0 = time.perf_counter()
    ens = kg.EnsembleOperator(Hs)
    out["ensemble_operator_build_ms"] = (time.perf_counter() - t0) * 1e3
    suffix = {"auto": "", "single": "_persistent", "tune": "_tuned"}
    for prec in ("fp64", "ff"):
        for kernel in ("auto", "single", "tune"):
            ms = _time_host(lambda: kg.kpm_1d_ensemble(ens, NC, psis, precision=prec,
                                                       kernel=kernel), 1, max(args.steps, 3))
            out[f"ensemble_{prec}{suffix[kernel]}"] = {"ms_per_call": ms, "value": vs / (ms / 1e3)}
    out["ff_over_fp64"] = out["ensemble_fp64"]["ms_per_call"] / out["ensemble_ff"]["ms_per_call"]
    # device-resident form: probes and moments stay in HBM, CUDA events on the
    # launching stream (the GPU time of the call)
    import torch
    psi_t = torch.from_numpy(np.ascontiguousarray(np.vstack(psis).T)).cuda()
    mu_t = torch.zeros((len(Hs), NC, NR), dtype=torch.complex128, device="cuda")
    stream = torch.cuda.current_stream()
    for prec in ("fp64", "ff"):
        for kernel in ("auto", "single"):
            def call():
                kg.kpm_1d_ensemble_device(ens, NC, psi_t, mu_t, precision=prec, kernel=kernel)
            call()
            kg.sync(ens.op)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            reps = max(args.steps, 3)
            e0.record(stream)
            for _ in range(reps):
                call()
            e1.record(stream)
            kg.sync(ens.op)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            out[f"ensemble_{prec}{suffix[kernel]}_device"] = {"ms_per_call": ms,
                                                             "value": vs / (ms / 1e3)}
    out["ff_over_fp64_device"] = (out["ensemble_fp64_device"]["ms_per_call"]
                                  / out["ensemble_ff_device"]["ms_per_call"])
    out["ff_tuned_over_fp64_tuned"] = (out["ensemble_fp64_tuned"]["ms_per_call"]
                                       / out["ensemble_ff_tuned"]["ms_per_call"])
    ops = [kg.GB300Operator(H) for H in Hs]
    def loop():
        for op, p in zip(ops, psis):
            kg.kpm_1d(op, NC, NR, psi_in=p, use_graph=True)
    ms = _time_host(loop, 1, max(args.steps, 3))
    out["per_member_calls_fp64_graph"] = {"ms_per_call": ms, "value": vs / (ms / 1e3)}
    return out


def workload_grad(args):
    """Adjoint gradient: graphene 128x128 (NH=32768), onsite N(0, 0.1^2),
    NC=1024, NR=16; forward kpm_1d vs kpmgb_kpm1d_grad."""
    import kpm_gb300 as kg
    from kpm_gb300 import models
    rng = np.random.default_rng(42)
    NH = 2 * 128 * 128
    H = (models.graphene(128, 128, onsite=0.1 * rng.standard_normal(NH)) / 3.4).tocsc()
    NC, NR = 1024, 16
    psi = kg.random_phase_vectors(rng, NH, NR)
    g = rng.standard_normal(NC)
    op = kg.GB300Operator(H)
    out = {"workload": "gradient of sum_m g_m mu_m, graphene 128x128 (NH=32768), NC=1024, NR=16"}
    tf = _time_host(lambda: kg.kpm_1d(op, NC, NR, psi_in=psi), 1, max(args.steps, 3))
    out["forward_ms"] = tf
    for C in (0, 64):
        tg = _time_host(lambda: kg.kpm_1d_grad(op, NC, psi, g, checkpoint_every=C), 1,
                        max(args.steps, 3))
        out[f"grad_checkpoint_{C or 'auto'}_ms"] = tg
        out[f"grad_over_forward_{C or 'auto'}"] = tg / tf
    return out


def workload_action(args):
    """chebyshev_action: 256x256 periodic square (NH=65536), NC=1024, NR=8, K=2
    (the reference benchmark's configuration), stability guard off."""
    import kpm_gb300 as kg
    from kpm_gb300 import models
    H = (models.square_anderson(256, W=0.0) / 4.2).tocsc()
    V = kg.random_phase_vectors(np.random.default_rng(42), 65536, 8)
    n = np.arange(1024)
    C = np.stack([np.where(n == 0, 1.0, 2.0) * np.cos(n * np.pi / 2) * np.exp(-n / 300),
                  np.where(n == 0, 1.0, 2.0) * np.cos(n * 1.3) * np.exp(-n / 300)], axis=1)
    op = kg.GB300Operator(H)
    ms = _time_host(lambda: kg.chebyshev_action(op, V, C, check_every=0), 1, max(args.steps, 3))
    NH, NR, NC, K = 65536, 8, 1024, 2
    return {"workload": "chebyshev_action, square 256x256 (NH=65536), NC=1024, NR=8, K=2",
            "ms_per_call_e2e": ms, "vector_steps_per_s": NR * (NC - 1) / (ms / 1e3),
            "h2d_bytes": NH * NR * 16 + NC * K * 16, "d2h_bytes": NH * NR * K * 16}


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload != "dos":
        import torch
        torch.cuda.set_device(local)
        fn = {"dos-small": workload_dos_small, "cond": workload_cond,
              "ensemble": workload_ensemble, "grad": workload_grad,
              "action": workload_action, "dsigma": workload_dsigma,
              "published": workload_published}[args.workload]
        res = fn(args)
        res["version"] = __import__("kpm_gb300").version()
        if rank == 0:
            print(json.dumps(res), flush=True)
        return
    import torch
    import torch.distributed as dist
    import kpm_gb300 as kg

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    h, psi = workload(args, rank)
    NH, NR, NC = h.H.shape[0], args.NR, args.NC
    op = kg.GB300Operator(h.H)
    # a dedicated stream: every library kernel and both timing events go here
    stream = torch.cuda.Stream()
    psi_t = torch.from_numpy(np.ascontiguousarray(psi.T)).cuda()
    mu_t = torch.zeros((NC, NR), dtype=torch.complex128, device="cuda")

    def call(prec):
        kg.kpm_1d_device(op, NC, psi_t, mu_t, precision=prec, stream=stream,
                         kernel=args.kernel if prec == "ff" else "auto")

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        call(args.precision)
    kg.sync(op, stream)
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n0 = kg.kernel_launch_count()
    with ClockSampler(local) as clk:
        barrier()
        w0 = time.perf_counter()
        ev0.record(stream)
        for _ in range(args.steps):
            call(args.precision)
        ev1.record(stream)
        barrier()
        wall_ms = (time.perf_counter() - w0) * 1e3 / args.steps
    launches = kg.kernel_launch_count() - n0
    kg.sync(op, stream)
    ms = ev0.elapsed_time(ev1) / args.steps
    t = torch.tensor([ms], device="cuda")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    value = world * NR * (NC // 2) / (ms / 1e3)
    mu_chosen = mu_t.cpu().numpy().T.copy()
    if world > 1:
        # every rank ran its own NR probe columns (weak scaling); one sum over
        # the ranks assembles all world * NR columns (kpm_gb300.sharding)
        from kpm_gb300 import sharding
        mu_global = sharding.gather_probe_moments(mu_chosen, world * NR)
        mu_avg = mu_global.sum(axis=0).real / (world * NR)

    # roofline of the dominant kernel (the fused recurrence step)
    nnz = h.H.nnz
    B_step = 48 * NH * NR + 20 * nnz + 4 * (NH + 1)
    step_launches = (NC // 2) * math.ceil(NR / 128)
    avg_launch_s = (ms / 1e3) / step_launches
    peak, peak_kind = measured_hbm()
    achieved = B_step / avg_launch_s / 1e9
    traffic = profile_traffic(args.precision)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                else "fallback 6.8 TB/s",
                "bytes_per_launch": B_step,
                "avg_launch_ms": avg_launch_s * 1e3}

    # end to end through the public host API: pinned host probes in, moments out
    e2e = None
    if not args.no_e2e:
        pinned = torch.empty((NR, NH), dtype=torch.complex128, pin_memory=True)
        pinned.numpy()[...] = psi.T
        host_psi = pinned.numpy().T  # (NH, NR) column-major view of pinned memory
        mu_host = np.zeros((NR, NC), dtype=np.complex128)
        kg.kpm_1d_bang(op, NC, NR, NH, mu_host, host_psi, precision=args.precision,
                       kernel=args.kernel if args.precision == "ff" else "auto")
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            kg.kpm_1d_bang(op, NC, NR, NH, mu_host, host_psi, precision=args.precision,
                           kernel=args.kernel if args.precision == "ff" else "auto")
        barrier()
        te = (time.perf_counter() - t0) / args.steps
        tt = torch.tensor([te], device="cuda")
        if world > 1:
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        te = float(tt.item())
        e2e = {"value": world * NR * (NC // 2) / te, "unit": UNIT,
               "h2d_bytes_per_step": NH * NR * 16, "d2h_bytes_per_step": NR * NC * 16,
               "ms_per_step": te * 1e3}

    # chosen form vs the plain FP64 path on the same inputs
    plain = None
    if not args.no_plain and args.precision != "fp64":
        mu64 = torch.zeros_like(mu_t)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        kg.kpm_1d_device(op, NC, psi_t, mu64, precision="fp64", stream=stream)
        e1.record(stream)
        barrier()
        kg.sync(op, stream)
        m64 = mu64.cpu().numpy().T
        avg_c, avg_p = mu_chosen.mean(0).real, m64.mean(0).real
        plain_ms = e0.elapsed_time(e1)
        fp64_peak = kg.measure_fp64_peak()
        fl = fp64_flop_per_row_col(nnz / NH, real=True) * NH * NR
        plain_launch_s = (plain_ms / 1e3) / step_launches
        plain_hbm = B_step / plain_launch_s / 1e9
        plain = {"ms_per_step": e0.elapsed_time(e1),
                 "value": NR * (NC // 2) / (e0.elapsed_time(e1) / 1e3),
                 "speedup_chosen_vs_plain": e0.elapsed_time(e1) / ms,
                 "moment_rel_err_normwise": float(np.linalg.norm(mu_chosen - m64)
                                                  / np.linalg.norm(m64)),
                 "moment_rel_err_max": float(np.max(np.abs(avg_c - avg_p)) / np.max(np.abs(avg_p))),
                 "roofline": {
                     "bound": "fp64", "achieved": fl / plain_launch_s / 1e12,
                     "peak": fp64_peak, "unit": "TFLOP/s",
                     "frac": fl / plain_launch_s / 1e12 / fp64_peak,
                     "peak_source": "measured in this run (kpmgb_measure_fp64_peak: independent "
                                    "FP64 FMA chains on every SM)",
                     "flop_per_launch": fl,
                     "flop_model": "per row x column x step: 4 per nonzero (real H) + 6 "
                                   "(update) + 12 (doubling dots)",
                     "hbm": {"achieved": plain_hbm, "peak": peak, "unit": "GB/s",
                             "frac": plain_hbm / peak}}}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        from oracle import cpu_port
        cpu, mu_cpu, steps = cpu_sample(h, psi, args, cpu_port.max_threads())
        k = 2 * steps
        cpu["check_rel_err_first_moments"] = float(
            np.linalg.norm(mu_cpu[:, :k] - mu_chosen[:, :k]) / np.linalg.norm(mu_cpu[:, :k]))
        cpu.pop("seconds", None)

    cond = None
    if rank == 0 and world == 1 and not args.no_cond:
        cond = cond_summary(args)

    secondary = None
    if rank == 0 and world == 1 and not args.no_secondary:
        secondary = secondary_summary(args)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "wall_ms_per_step": wall_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": ("f64 emulated as float-float on the FP32 pipe" if args.precision == "ff"
                      else "f64"),
            "data": "synthetic (seeded 3D Anderson model and random-phase probes)",
            "config": config(args),
            "roofline": roofline,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "plain_fp64": plain,
            "cpu_baseline": cpu,
            "kpm2d_tensor_core": cond,
            "other_configs": secondary,
            "version": kg.version(),
        }
        if world > 1:
            line["sharded"] = {"probe_columns": world * NR, "mu0_average": float(mu_avg[0]),
                               "reduction": "kpm_gb300.sharding.gather_probe_moments (NCCL)"}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
