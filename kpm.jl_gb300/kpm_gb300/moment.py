"""Moment engine entry points mirroring KPM.jl's ``kpm_1d`` / ``kpm_2d``.

Same names, argument meaning and error behaviour as ``src/moment.jl``:

* ``kpm_1d(H, NC, NR, NH=None, *, psi_in, psi_in_l, psi_in_r, force_norm,
  avg_output, NR_parallel)``  (``src/moment.jl:339-418``)
* ``kpm_1d_bang(H, NC, NR, NH, mu_all, psi_in)`` / ``(..., psi_in_l, psi_in_r)``
  (the reference's ``kpm_1d!``, ``src/moment.jl:420-556``)
* ``kpm_2d(H, Ja, Jb, NC, NR, NH, *, psi_in | psi_in_l+psi_in_r, arr_size,
  right_block, workspace_bytes, moment_parity, mn_sym)``
  (``src/moment.jl:812-1103``)
* ``kpm_2d_blocking`` (``src/moment.jl:759-810``)

All arithmetic runs in libkpmgb on the GPU.  Probe blocks are NumPy arrays of
shape (NH, NR) (column i = probe i, as in Julia) or torch CUDA tensors for the
``*_device`` forms.  ``precision="fp64"`` is native double precision;
``precision="ff"`` is the emulated-double (float-float) recurrence.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _native
from ._native import KPMArgumentError
from .operator import GB300Operator, as_operator

_PREC = {"fp64": _native.PREC_FP64, "ff": _native.PREC_FF}
_CONTRACT = {"fp64": _native.CONTRACT_FP64, "split": _native.CONTRACT_SPLIT}


def _prec(precision) -> int:
    try:
        return _PREC[precision]
    except KeyError:
        raise KPMArgumentError(f"precision must be one of {sorted(_PREC)} (got {precision!r})")


def normalize_by_col(psi: np.ndarray, centering: bool = False) -> None:
    """In-place column normalisation (``src/utils/vectors.jl:14-19``)."""
    for i in range(psi.shape[1]):
        col = psi[:, i]
        if centering:
            col -= col.mean()
        col /= np.linalg.norm(col)


def _colmajor(psi, NH, NR, name):
    a = np.asarray(psi)
    if a.shape != (NH, NR):
        raise KPMArgumentError(
            f"Invalid `{name}` with size {a.shape}. Expecting ({NH}, {NR})")
    return np.asfortranarray(a, dtype=np.complex128)


_VARIANT = {"auto": 0, "gather": 1, "tune": 4, "single": 6, "padded": 9, "cluster": 10,
            "streaming": 11}


def _opts1d(precision, stability_check, kernel="auto", use_graph=False):
    if kernel not in _VARIANT:
        raise KPMArgumentError(f"kernel must be one of {sorted(_VARIANT)}")
    return _native.Kpm1dOptions(_prec(precision), 1 if stability_check else 0,
                                1 if use_graph else 0, _VARIANT[kernel])


def kpm_1d_bang(H, NC: int, NR: int, NH: int, mu_all: np.ndarray, psi_in=None, psi_in_r=None,
                *, precision: str = "fp64", stability_check: bool = False,
                kernel: str = "auto", use_graph: bool = False) -> None:
    """``kpm_1d!``: fill ``mu_all`` (NR, NC) in place.

    ``kpm_1d_bang(H, NC, NR, NH, mu_all, psi_in)`` is the doubling path
    (NC even); ``kpm_1d_bang(H, NC, NR, NH, mu_all, psi_in_l, psi_in_r)`` the
    bra/ket path.  ``use_graph`` replays the recurrence as a CUDA graph
    (captured on the first call, reused while sizes and buffers repeat).
    """
    op = as_operator(H)
    lib = _native.load()
    if mu_all.shape != (NR, NC):
        raise KPMArgumentError(f"mu_all has size {mu_all.shape}; expected ({NR}, {NC})")
    out = np.empty((NR, NC), dtype=np.complex128, order="F")
    opts = _opts1d(precision, stability_check, kernel, use_graph)
    if psi_in_r is None:
        if NC % 2 != 0:
            raise KPMArgumentError("Invalid NC: NC should be even.")
        psi = _colmajor(psi_in, NH, NR, "psi_in")
        rc = lib.kpmgb_kpm1d(op.handle, NC, NR, NH, psi.ctypes.data, out.ctypes.data, C.byref(opts))
    else:
        if NC < 2:
            raise KPMArgumentError("Invalid NC: NC should be at least 2.")
        pl = _colmajor(psi_in, NH, NR, "psi_in_l")
        pr = _colmajor(psi_in_r, NH, NR, "psi_in_r")
        rc = lib.kpmgb_kpm1d_lr(op.handle, NC, NR, NH, pl.ctypes.data, pr.ctypes.data,
                                out.ctypes.data, C.byref(opts))
    _native.check(rc)
    mu_all[...] = out


def kpm_1d(H, NC: int, NR: int, NH: int | None = None, *, psi_in=None, psi_in_l=None,
           psi_in_r=None, force_norm: bool = False, verbose: int = 0, avg_output: bool = True,
           NR_parallel: bool = True, rng=None, precision: str = "fp64",
           stability_check: bool = False, kernel: str = "auto", use_graph: bool = False):
    """Stochastic-trace Chebyshev moments (``src/moment.jl:339-418``).

    Returns the real probe average (length NC) for equal bra/ket, the complex
    average for ``psi_in_l``/``psi_in_r``, or the (NR, NC) matrix with
    ``avg_output=False``.  Without probes, random-phase probes are drawn from
    ``rng`` (a NumPy Generator; the reference draws from Xoshiro).

    ``kernel`` picks the recurrence kernel (``include/kpmgb.h``,
    ``kernel_variant``): ``"auto"`` (one thread-block-cluster launch per call
    for small operators, else per-step launches of the row-streaming kernels
    -- on packed FP32 pairs for real operators with 9..64 columns,
    float-float doubling -- where they apply, else of the register-gather
    kernel), ``"gather"``,
    ``"padded"``, ``"streaming"``, ``"cluster"``, ``"single"``, ``"tune"``.
    ``use_graph`` replays the per-step launches from a CUDA graph.  With
    ``NR_parallel=False`` the columns run one call each, with the same
    options.
    """
    NH = H.shape[0] if NH is None else int(NH)
    NC, NR = int(NC), int(NR)
    mu_all = np.zeros((NR, NC), dtype=np.complex128)
    lr = False
    if psi_in is None:
        if psi_in_l is not None or psi_in_r is not None:
            if psi_in_l is None or psi_in_r is None:
                raise KPMArgumentError("must set both `psi_in_l` and `psi_in_r` or neither.")
            lr = True
            if force_norm:
                normalize_by_col(psi_in_l)
                normalize_by_col(psi_in_r)
        else:
            from .frontend import random_phase_vectors
            rng = np.random.default_rng() if rng is None else rng
            psi_in = random_phase_vectors(rng, NH, NR)
    else:
        if psi_in_l is not None or psi_in_r is not None:
            raise KPMArgumentError(
                "must either set `psi_in` or set `psi_in_l` and `psi_in_r`, but not both.")
        if force_norm:
            normalize_by_col(psi_in)
    op = as_operator(H)
    if NR_parallel:
        if lr:
            kpm_1d_bang(op, NC, NR, NH, mu_all, psi_in_l, psi_in_r, precision=precision,
                        stability_check=stability_check, kernel=kernel, use_graph=use_graph)
        else:
            kpm_1d_bang(op, NC, NR, NH, mu_all, psi_in, precision=precision,
                        stability_check=stability_check, kernel=kernel, use_graph=use_graph)
    else:
        for i in range(NR):
            row = np.zeros((1, NC), dtype=np.complex128)
            if lr:
                kpm_1d_bang(op, NC, 1, NH, row, np.asarray(psi_in_l)[:, i:i + 1],
                            np.asarray(psi_in_r)[:, i:i + 1], precision=precision,
                            stability_check=stability_check, kernel=kernel,
                            use_graph=use_graph)
            else:
                kpm_1d_bang(op, NC, 1, NH, row, np.asarray(psi_in)[:, i:i + 1],
                            precision=precision, stability_check=stability_check,
                            kernel=kernel, use_graph=use_graph)
            mu_all[i] = row[0]
    if avg_output:
        avg = mu_all.sum(axis=0) / NR
        return avg if lr else avg.real
    return mu_all


def kpm_2d_blocking(NH: int, NR: int, NC: int, *, workspace_bytes="auto", arr_size="auto",
                    right_block="auto"):
    """Block sizes of the reference rule (``src/moment.jl:759-810``).

    Returns ``dict(arr_size=K_left, right_block=K_right, bytes=footprint)``.
    The automatic budget is ``KPM_WORKSPACE_BYTES`` or half the free device
    memory.
    """
    if NH <= 0:
        raise KPMArgumentError(f"NH must be positive (got {NH})")
    if NR <= 0:
        raise KPMArgumentError(f"NR must be positive (got {NR})")
    if NC < 2:
        raise KPMArgumentError(f"NC must be at least 2 (got {NC})")
    block = NH * NR * 16
    if workspace_bytes == "auto":
        env = os.environ.get("KPM_WORKSPACE_BYTES", "")
        if env:
            budget = int(env)
        else:
            import torch
            free, _ = torch.cuda.mem_get_info()
            budget = free // 2
    elif isinstance(workspace_bytes, (int, np.integer)):
        budget = int(workspace_bytes)
    else:
        raise KPMArgumentError("workspace_bytes must be :auto or an integer")
    if budget < 0:
        raise KPMArgumentError("workspace_bytes must be nonnegative")
    if right_block == "auto":
        K_right = min(NC, 16)
    elif isinstance(right_block, (int, np.integer)) and right_block >= 1:
        K_right = int(right_block)
    else:
        raise KPMArgumentError("right_block must be :auto or a positive integer")
    base = (K_right + 7) * block
    per_left = block + K_right * 16
    if arr_size == "auto":
        kmax = (budget - base) // per_left
        if kmax < 2:
            raise KPMArgumentError(
                f"workspace_bytes={budget} cannot fit the minimum kpm_2d workspace "
                f"({base + 2 * per_left} bytes at right_block={K_right})")
        K_left = min(kmax, NC)
    elif isinstance(arr_size, (int, np.integer)) and arr_size >= 2:
        K_left = int(arr_size)
    else:
        raise KPMArgumentError("arr_size must be :auto or an integer at least 2")
    return dict(arr_size=K_left, right_block=K_right, bytes=base + K_left * per_left)


def _opts2d(arr_size, right_block, workspace_bytes, moment_parity, mn_sym, precision,
            contraction):
    if moment_parity not in _native.PARITY:
        raise KPMArgumentError(f"moment_parity={moment_parity} not understood.")
    if arr_size == "auto":
        kl = 0
    elif isinstance(arr_size, (int, np.integer)) and arr_size >= 2:
        kl = int(arr_size)
    else:
        raise KPMArgumentError("arr_size must be :auto or an integer at least 2")
    if right_block == "auto":
        kr = 0
    elif isinstance(right_block, (int, np.integer)) and right_block >= 1:
        kr = int(right_block)
    else:
        raise KPMArgumentError("right_block must be :auto or a positive integer")
    if workspace_bytes == "auto":
        env = os.environ.get("KPM_WORKSPACE_BYTES", "")
        wb = int(env) if env else -1
    elif isinstance(workspace_bytes, (int, np.integer)) and workspace_bytes >= 0:
        wb = int(workspace_bytes)
    else:
        raise KPMArgumentError("workspace_bytes must be :auto or a nonnegative integer")
    if contraction not in _CONTRACT:
        raise KPMArgumentError(f"contraction must be one of {sorted(_CONTRACT)}")
    return _native.Kpm2dOptions(kl, kr, wb, _native.PARITY[moment_parity], 1 if mn_sym else 0,
                                _prec(precision), _CONTRACT[contraction])


def kpm_2d_bang(H, Ja, Jb, NC: int, NR: int, NH: int, mu: np.ndarray, psi_in_l, psi_in_r=None,
                *, arr_size="auto", right_block="auto", workspace_bytes="auto",
                moment_parity="NONE", mn_sym=False, precision="fp64", contraction="fp64",
                verbose=0) -> None:
    """``kpm_2d!``: overwrite ``mu`` (NC, NC) (``src/moment.jl:887-1088``)."""
    if psi_in_r is None:
        psi_in_r = psi_in_l
    opts = _opts2d(arr_size, right_block, workspace_bytes, moment_parity, mn_sym, precision,
                   contraction)
    pl = _colmajor(psi_in_l, NH, NR, "psi_in_l")
    pr = _colmajor(psi_in_r, NH, NR, "psi_in_r")
    h, a, b = as_operator(H), as_operator(Ja), as_operator(Jb)
    out = np.empty((NC, NC), dtype=np.complex128, order="F")
    lib = _native.load()
    rc = lib.kpmgb_kpm2d(h.handle, a.handle, b.handle, NC, NR, NH, pl.ctypes.data,
                         pr.ctypes.data, out.ctypes.data, C.byref(opts))
    _native.check(rc)
    mu[...] = out


def kpm_2d(H, Ja, Jb, NC: int, NR: int, NH: int, *, psi_in=None, psi_in_l=None, psi_in_r=None,
           arr_size="auto", right_block="auto", workspace_bytes="auto", moment_parity="NONE",
           mn_sym=False, verbose=0, rng=None, precision="fp64", contraction="fp64"):
    """Two-dimensional moments mu[n, m] (NC, NC) (``src/moment.jl:812-885``)."""
    NC, NR, NH = int(NC), int(NR), int(NH)
    mu = np.zeros((NC, NC), dtype=np.complex128)
    kw = dict(arr_size=arr_size, right_block=right_block, workspace_bytes=workspace_bytes,
              moment_parity=moment_parity, mn_sym=mn_sym, precision=precision,
              contraction=contraction)
    if psi_in is None and psi_in_l is None and psi_in_r is None:
        from .frontend import random_phase_vectors
        rng = np.random.default_rng() if rng is None else rng
        psi = random_phase_vectors(rng, NH, NR)
        kpm_2d_bang(H, Ja, Jb, NC, NR, NH, mu, psi, psi, **kw)
    elif psi_in is not None and psi_in_l is None and psi_in_r is None:
        kpm_2d_bang(H, Ja, Jb, NC, NR, NH, mu, psi_in, psi_in, **kw)
    elif psi_in is None and psi_in_l is not None and psi_in_r is not None:
        kpm_2d_bang(H, Ja, Jb, NC, NR, NH, mu, psi_in_l, psi_in_r, **kw)
    else:
        raise KPMArgumentError("unimplemented")
    return mu


# ------------------------------------------------- directional derivatives
def _host_sparse(M, name):
    import scipy.sparse as sp
    if isinstance(M, GB300Operator):
        raise KPMArgumentError(f"{name}: the derivative forms need host matrices, "
                               "not device operators")
    return sp.csr_matrix(M, dtype=np.complex128)


def _lower_block(A, dA, n):
    """[[A, 0], [dA, A]]: T_n of it is [[T_n(A), 0], [D T_n(A)[dA], T_n(A)]], and a
    product of such blocks carries the product rule in its lower-left block."""
    import scipy.sparse as sp
    dA = sp.csr_matrix((n, n), dtype=np.complex128) if dA is None else dA
    return sp.bmat([[A, None], [dA, A]], format="csc")


def _inf_norm(M) -> float:
    return float(abs(M).sum(axis=1).max()) if M is not None and M.nnz else 0.0


def _tangent_scale(NC: int, dH, J_pairs=()) -> float:
    """Power of two s applied to the tangent direction and undone on the result
    (both exact).  The tangent halves of the augmented vectors grow relative
    to the value halves like n |dH| for probes spread over the band interior
    (T_n' = n U_{n-1}; the worst-case bound n^2 |dH| needs band-edge weight);
    s near the geometric mean sqrt(NC) |dH| of that growth keeps the halves
    within a factor ~sqrt(NC) of each other, which the per-vector scaling of
    the float-float rows and of the split contraction's digit planes needs
    (the smaller half loses log2 of the ratio in bits)."""
    import math
    g = math.sqrt(int(NC)) * _inf_norm(dH)
    for J, dJ in J_pairs:
        nj = _inf_norm(J)
        if nj > 0:
            g = max(g, _inf_norm(dJ) / nj)
    if not g > 0 or not math.isfinite(g):
        return 1.0
    return math.ldexp(1.0, -round(math.log2(g)))


def kpm_1d_derivative(H, dH, NC: int, NR: int, NH: int | None = None, *, psi_in,
                      avg_output: bool = True, precision: str = "fp64", kernel: str = "auto"):
    """Directional derivative of ``kpm_1d`` moments along ``H + t dH`` at t = 0:
    ``dmu_n = sum_i <psi_i| D T_n(H)[dH] |psi_i>`` (forward mode, one scalar
    parameter; ``kpm_1d_grad`` is the reverse mode for many).

    Runs the l/r recurrence of ``kpm_1d`` on the GPU over the 2NH operator
    ``[[H, 0], [dH, H]]`` with ket ``[psi; 0]`` and bra ``[0; psi]``: the lower
    half of ``T_n`` applied to the ket is the Frechet derivative of ``T_n(H)``
    applied to psi.  Costs about twice a forward call.  Returns the real
    probe average (length NC; ``dH`` Hermitian) or the complex (NR, NC) matrix
    with ``avg_output=False``.  No reference counterpart: KPM.jl differentiates
    ``src/moment.jl:420-556`` with ForwardDiff duals.
    """
    import scipy.sparse as sp
    Hh, dHh = _host_sparse(H, "H"), _host_sparse(dH, "dH")
    NH = Hh.shape[0] if NH is None else int(NH)
    if Hh.shape != (NH, NH) or dHh.shape != (NH, NH):
        raise KPMArgumentError(f"H and dH must both be ({NH}, {NH})")
    psi = np.asarray(psi_in, dtype=np.complex128)
    if psi.shape != (NH, int(NR)):
        raise KPMArgumentError(f"Invalid `psi_in` with size {psi.shape}. Expecting ({NH}, {NR})")
    z = np.zeros_like(psi)
    sc = _tangent_scale(NC, dHh)
    mu = kpm_1d(_lower_block(Hh, dHh * sc, NH), NC, NR, 2 * NH,
                psi_in_l=np.vstack([z, psi]), psi_in_r=np.vstack([psi, z]),
                avg_output=False, precision=precision, kernel=kernel) / sc
    return mu.sum(axis=0).real / int(NR) if avg_output else mu


def kpm_2d_derivative(H, dH, Ja, dJa, Jb, dJb, NC: int, NR: int, NH: int, *, psi_in=None,
                      psi_in_l=None, psi_in_r=None, **kw):
    """Directional derivative of ``kpm_2d`` moments along ``H + t dH``,
    ``Ja + t dJa``, ``Jb + t dJb`` at t = 0 (``dJa`` / ``dJb`` may be None):
    ``dmu[n, m] = (1/NR) sum_i d<T_m psi_l_i | Jb T_n Ja psi_r_i>``.

    One GPU ``kpm_2d`` call over 2NH operators: ``[[H, 0], [dH, H]]``,
    ``[[Ja, 0], [dJa, Ja]]`` and ``[[dJb, Jb], [Jb, 0]]`` (the lower-triangular
    embedding of Jb with its halves swapped), probes ``[psi_l; 0]`` and
    ``[psi_r; 0]``: the left chain carries ``[L_m; dL_m]``, the right one
    ``[dR_n; R_n]``, so the contraction sums ``<L|dR> + <dL|R>``.  The
    direction is pre-scaled by a power of two (``_tangent_scale``).  Every
    ``kpm_2d`` keyword (blocking, parity, mn_sym, precision, contraction)
    applies.  ``kubo_bastin_cond`` is linear in the moments, so at fixed
    rescaling ``kubo_bastin_cond(dmu, ...)`` is the derivative of the
    conductivity (e.g. dsigma_xy/dt2 of the Haldane model).  No reference
    counterpart (``src/moment.jl:887-1088`` is differentiated with duals).
    """
    import scipy.sparse as sp
    NH, NR = int(NH), int(NR)
    Hh, dHh = _host_sparse(H, "H"), _host_sparse(dH, "dH")
    A, B = _host_sparse(Ja, "Ja"), _host_sparse(Jb, "Jb")
    dA = None if dJa is None else _host_sparse(dJa, "dJa")
    dB = None if dJb is None else _host_sparse(dJb, "dJb")
    for M, name in ((Hh, "H"), (dHh, "dH"), (A, "Ja"), (B, "Jb"), (dA, "dJa"), (dB, "dJb")):
        if M is not None and M.shape != (NH, NH):
            raise KPMArgumentError(f"{name} must be ({NH}, {NH}) (got {M.shape})")
    if psi_in is not None:
        if psi_in_l is not None or psi_in_r is not None:
            raise KPMArgumentError("unimplemented")
        psi_in_l = psi_in_r = psi_in
    if psi_in_l is None or psi_in_r is None:
        raise KPMArgumentError("kpm_2d_derivative needs explicit probes "
                               "(`psi_in` or `psi_in_l` and `psi_in_r`)")
    pl = np.asarray(psi_in_l, dtype=np.complex128)
    pr = np.asarray(psi_in_r, dtype=np.complex128)
    if pl.shape != (NH, NR) or pr.shape != (NH, NR):
        raise KPMArgumentError(f"probes must be ({NH}, {NR})")
    z = np.zeros((NH, NR), dtype=np.complex128)
    sc = _tangent_scale(NC, dHh, ((A, dA), (B, dB)))
    dA = None if dA is None else dA * sc
    Bs = sp.csr_matrix((NH, NH), dtype=np.complex128) if dB is None else dB * sc
    Jb_aug = sp.bmat([[Bs, B], [B, None]], format="csc")
    mu = kpm_2d(_lower_block(Hh, dHh * sc, NH), _lower_block(A, dA, NH), Jb_aug, NC, NR, 2 * NH,
                psi_in_l=np.vstack([pl, z]), psi_in_r=np.vstack([pr, z]), **kw)
    return mu / sc


# ------------------------------------------------------------ device forms
def _stream_ptr(stream):
    if stream is None:
        import torch
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return C.c_void_p(getattr(stream, "cuda_stream", stream))


def kpm_1d_device(op: GB300Operator, NC: int, psi_t, mu_t, *, psi_l_t=None,
                  precision="fp64", stability_check=False, stream=None,
                  kernel="auto", use_graph=False) -> None:
    """Enqueue kpm_1d on torch CUDA tensors without host copies.

    ``psi_t``: complex128 tensor of shape (NR, NH) (row-contiguous, i.e. the
    column-major NH x NR block); ``mu_t``: complex128 (NC, NR).  Runs on
    ``stream`` (default: torch's current stream) and returns immediately.
    """
    lib = _native.load()
    NR, NH = psi_t.shape
    for t, name in ((psi_t, "psi"), (mu_t, "mu")):
        if not t.is_contiguous():
            raise KPMArgumentError(f"{name} tensor must be contiguous")
    if tuple(mu_t.shape) != (NC, NR):
        raise KPMArgumentError(f"mu tensor must have shape ({NC}, {NR})")
    opts = _opts1d(precision, stability_check, kernel, use_graph)
    if psi_l_t is None:
        rc = lib.kpmgb_kpm1d_device(op.handle, NC, NR, NH, C.c_void_p(psi_t.data_ptr()),
                                    C.c_void_p(mu_t.data_ptr()), C.byref(opts), _stream_ptr(stream))
    else:
        rc = lib.kpmgb_kpm1d_lr_device(op.handle, NC, NR, NH, C.c_void_p(psi_l_t.data_ptr()),
                                       C.c_void_p(psi_t.data_ptr()), C.c_void_p(mu_t.data_ptr()),
                                       C.byref(opts), _stream_ptr(stream))
    _native.check(rc)


def kpm_2d_device(H: GB300Operator, Ja: GB300Operator, Jb: GB300Operator, NC: int, psi_l_t,
                  psi_r_t, mu_t, *, arr_size="auto", right_block="auto",
                  workspace_bytes="auto", moment_parity="NONE", mn_sym=False,
                  precision="fp64", contraction="fp64", stream=None) -> None:
    """Enqueue kpm_2d on torch CUDA tensors; ``mu_t`` is complex128 (NC, NC) holding
    the column-major moment matrix (mu_t[m, n] = mu[n, m])."""
    lib = _native.load()
    NR, NH = psi_r_t.shape
    opts = _opts2d(arr_size, right_block, workspace_bytes, moment_parity, mn_sym, precision,
                   contraction)
    rc = lib.kpmgb_kpm2d_device(H.handle, Ja.handle, Jb.handle, NC, NR, NH,
                                C.c_void_p(psi_l_t.data_ptr()), C.c_void_p(psi_r_t.data_ptr()),
                                C.c_void_p(mu_t.data_ptr()), C.byref(opts), _stream_ptr(stream))
    _native.check(rc)


def sync(op: GB300Operator, stream=None) -> None:
    """Wait for enqueued work on ``op`` and raise deferred numerical failures."""
    _native.check(_native.load().kpmgb_operator_sync(op.handle, _stream_ptr(stream)))


class EnsembleOperator:
    """The members of an ensemble stacked once as a block-diagonal operator
    resident on the device, with its segment table; reusable across
    :func:`kpm_1d_ensemble` calls."""

    def __init__(self, Hs):
        import scipy.sparse as sp
        if not Hs:
            raise KPMArgumentError("Hs must be a non-empty list")
        self.sizes = [int(H.shape[0]) for H in Hs]
        Hb = sp.block_diag([sp.csc_matrix(H, dtype=np.complex128) for H in Hs], format="csc")
        self.op = GB300Operator(Hb)
        self.seg = np.zeros(len(Hs) + 1, dtype=np.int64)
        self.seg[1:] = np.cumsum(self.sizes)
        self._staging = None

    def staging(self, NR: int):
        """The stacked column-major probe block (sum NH_i, NR) in page-locked
        host memory, kept between calls (the library reads it with its copy
        kernel instead of staging pageable memory)."""
        if self._staging is None or self._staging.shape[1] != NR:
            self._staging = None
            self._staging = _native.pinned_empty((int(self.seg[-1]), NR), np.complex128, "F")
        return self._staging

    def __len__(self):
        return len(self.sizes)


def kpm_1d_ensemble(Hs, NC: int, psis, *, precision: str = "fp64", avg_output: bool = True,
                    kernel: str = "auto"):
    """Doubling moments of many independent members in one call.

    ``Hs``: list of (rescaled) sparse operators of any sizes, or an
    :class:`EnsembleOperator` built from them; ``psis``: list of probe blocks
    (NH_i, NR) with a common NR (run in batches of 32 columns).
    Equivalent to
    ``[kpm_1d(H_i, NC, NR, psi_in=psi_i) for ...]`` (``src/moment.jl:339-492``
    per member).  Returns a list of length-NC real averages, or of (NR, NC)
    matrices with ``avg_output=False``.

    ``kernel``: ``"auto"`` (one launch per step over the stacked members,
    padded float-float rows where the members allow them); ``"gather"`` (one
    launch per step, CSR rows); ``"padded"`` (one launch per step, padded
    float-float rows, at most 8 nonzeros per row); ``"single"`` (one
    persistent launch, each CTA runs whole members); ``"tune"`` (times the
    schedules and shapes once per ensemble shape and device and keeps the
    choice in the persistent autotuning cache, ``KPMGB_TUNE_CACHE``, default
    ``~/.cache/kpmgb/tune.txt``).
    """
    ens = Hs if isinstance(Hs, EnsembleOperator) else None
    if ens is None:
        if not Hs or len(Hs) != len(psis):
            raise KPMArgumentError("Hs and psis must be non-empty lists of equal length")
        sizes = [H.shape[0] for H in Hs]
    else:
        sizes = ens.sizes
        if len(psis) != len(sizes):
            raise KPMArgumentError("one probe block per ensemble member")
    NR = int(np.asarray(psis[0]).shape[1])
    for n, p in zip(sizes, psis):
        if np.asarray(p).shape != (n, NR):
            raise KPMArgumentError("every probe block must be (NH_i, NR) with a common NR")
    if NC % 2 != 0:
        raise KPMArgumentError("Invalid NC: NC should be even.")
    if ens is None:
        ens = EnsembleOperator(Hs)
    op, seg = ens.op, ens.seg
    # one pass into the stacked column-major probe block (pinned, reused)
    psi = ens.staging(NR)
    for i, p in enumerate(psis):
        psi[int(seg[i]):int(seg[i + 1])] = p
    out = np.empty((len(sizes), NC, NR), dtype=np.complex128)
    if kernel not in ("auto", "tune", "gather", "padded", "single"):
        raise KPMArgumentError("kernel must be 'auto', 'tune', 'gather', 'padded' or 'single' "
                               "for the ensemble")
    opts = _opts1d(precision, False, kernel)
    lib = _native.load()
    rc = lib.kpmgb_kpm1d_ensemble(op.handle, len(sizes), seg.ctypes.data, NC, NR, psi.ctypes.data,
                                  out.ctypes.data, C.byref(opts))
    _native.check(rc)
    if avg_output:
        # column by column in order: the same sums as kpm_1d's averaging
        acc = out[:, :, 0].copy()
        for r in range(1, NR):
            acc += out[:, :, r]
        return list(acc.real / NR)
    return [np.ascontiguousarray(out[i].T) for i in range(len(sizes))]


def kpm_1d_ensemble_device(ens: "EnsembleOperator", NC: int, psi_t, mu_t, *,
                           precision: str = "fp64", kernel: str = "auto", stream=None) -> None:
    """Enqueue the ensemble call on torch CUDA tensors without host copies.

    ``psi_t``: complex128 tensor of shape (NR, sum NH_i) (row-contiguous, i.e.
    the column-major stacked probe block, member i's probes in its rows);
    ``mu_t``: complex128 (nseg, NC, NR), member i's moments mu_t[i, n, r].
    Runs on ``stream`` (default: torch's current stream) and returns
    immediately; :func:`sync` waits and raises deferred failures.
    """
    lib = _native.load()
    NR, NH = psi_t.shape
    nseg = len(ens.sizes)
    for t, name in ((psi_t, "psi"), (mu_t, "mu")):
        if not t.is_contiguous():
            raise KPMArgumentError(f"{name} tensor must be contiguous")
    if NH != int(ens.seg[-1]):
        raise KPMArgumentError("psi must hold the stacked rows of every member")
    if tuple(mu_t.shape) != (nseg, NC, NR):
        raise KPMArgumentError(f"mu tensor must have shape ({nseg}, {NC}, {NR})")
    if kernel not in ("auto", "tune", "gather", "padded", "single"):
        raise KPMArgumentError("kernel must be 'auto', 'tune', 'gather', 'padded' or 'single' "
                               "for the ensemble")
    opts = _opts1d(precision, False, kernel)
    rc = lib.kpmgb_kpm1d_ensemble_device(ens.op.handle, nseg, ens.seg.ctypes.data, NC, NR,
                                         C.c_void_p(psi_t.data_ptr()), C.c_void_p(mu_t.data_ptr()),
                                         C.byref(opts), _stream_ptr(stream))
    _native.check(rc)


def kpm_1d_grad(H, NC: int, psi_in, g, *, checkpoint_every: int = 0):
    """Gradient of ``L = sum_m g[m] * kpm_1d(H, NC, NR, psi_in=psi_in)[m]``.

    ``g`` holds the real weights dL/dmu_m (length NC), e.g. from
    :func:`kpm_gb300.frontend.dos_basis` for a loss on the reconstructed DOS.
    Runs the adjoint Chebyshev recurrence on the GPU (checkpoints every
    ``checkpoint_every`` steps; 0 keeps every vector resident when half of the
    free device memory holds them) and returns the gradient on H's sparsity
    pattern: a CSC matrix whose stored value k is dL/dRe(H_k) + i dL/dIm(H_k)
    (H_ij and H_ji are independent entries; for a Hermitian parameter t on
    both, dL/dt sums the two).  No reference counterpart: KPM.jl obtains such
    derivatives by ForwardDiff duals through ``src/moment.jl:420-492``.
    """
    import scipy.sparse as sp
    op = as_operator(H)
    NH = op.shape[0]
    a = np.asarray(psi_in)
    if a.ndim != 2 or a.shape[0] != NH:
        raise KPMArgumentError(f"Invalid `psi_in` with size {a.shape}. Expecting ({NH}, NR)")
    NR = a.shape[1]
    psi = _colmajor(a, NH, NR, "psi_in")
    gw = np.ascontiguousarray(g, dtype=np.float64)
    if gw.shape != (int(NC),):
        raise KPMArgumentError(f"g must have length NC={NC} (got {gw.shape})")
    out = np.empty(op.nnz, dtype=np.complex128)
    lib = _native.load()
    rc = lib.kpmgb_kpm1d_grad(op.handle, int(NC), NR, NH, psi.ctypes.data, gw.ctypes.data,
                              int(checkpoint_every), out.ctypes.data)
    _native.check(rc)
    return sp.csc_matrix((out, op.indices, op.indptr), shape=op.shape)


def kpm_2d_grad(H, Ja, Jb, NC: int, G, NR: int | None = None, NH: int | None = None, *,
                psi_in=None, psi_in_l=None, psi_in_r=None, moment_parity: str = "NONE",
                Jb_adjoint=None):
    """Gradient of ``F = Re sum_{n,m} G[n,m] mu[n,m]`` with respect to the
    stored entries of H, Ja and Jb, for the kpm_2d moments
    ``mu = kpm_2d(H, Ja, Jb, NC, NR, NH; psi_in_l, psi_in_r, moment_parity)``
    (``src/moment.jl:812-1088``).

    ``G`` (NC, NC) complex: dF/dmu, e.g. :func:`kubo_bastin_weights` for a
    loss on sigma(Ef).  Returns ``(gH, gJa, gJb)``: CSC matrices on each
    operator's pattern whose stored value k is dF/dRe(X_k) + i dF/dIm(X_k).
    Runs the adjoint Chebyshev recurrences of both chains on the GPU (FP64),
    keeping every forward vector of a batch of 32 probe columns resident.
    ``Jb_adjoint``: Jb^dagger as a matrix or operator (built from ``Jb`` when
    that is a SciPy matrix).  No reference counterpart: KPM.jl obtains such
    derivatives by ForwardDiff duals.
    """
    import scipy.sparse as sp
    if moment_parity not in _native.PARITY:
        raise KPMArgumentError(f"moment_parity={moment_parity} not understood.")
    if Jb_adjoint is None:
        if isinstance(Jb, GB300Operator):
            raise KPMArgumentError("Jb_adjoint is required when Jb is a GB300Operator")
        Jb_adjoint = sp.csc_matrix(Jb, dtype=np.complex128).conj().T.tocsc()
    op, oa, ob, obh = (as_operator(M) for M in (H, Ja, Jb, Jb_adjoint))
    NH = op.shape[0] if NH is None else int(NH)
    if psi_in is not None:
        if psi_in_l is not None or psi_in_r is not None:
            raise KPMArgumentError(
                "must either set `psi_in` or set `psi_in_l` and `psi_in_r`, but not both.")
        psi_in_l = psi_in_r = psi_in
    if psi_in_l is None or psi_in_r is None:
        raise KPMArgumentError("probe vectors are required (psi_in, or psi_in_l and psi_in_r)")
    NR = np.asarray(psi_in_r).shape[1] if NR is None else int(NR)
    pl = _colmajor(psi_in_l, NH, NR, "psi_in_l")
    pr = _colmajor(psi_in_r, NH, NR, "psi_in_r")
    Gm = np.asfortranarray(G, dtype=np.complex128)
    if Gm.shape != (int(NC), int(NC)):
        raise KPMArgumentError(f"G must be ({NC}, {NC}) (got {Gm.shape})")
    outs = [np.empty(o.nnz, dtype=np.complex128) for o in (op, oa, ob)]
    lib = _native.load()
    rc = lib.kpmgb_kpm2d_grad(op.handle, oa.handle, ob.handle, obh.handle, int(NC), NR, NH,
                              pl.ctypes.data, pr.ctypes.data, Gm.ctypes.data,
                              _native.PARITY[moment_parity], outs[0].ctypes.data,
                              outs[1].ctypes.data, outs[2].ctypes.data)
    _native.check(rc)
    return tuple(sp.csc_matrix((g, o.indices, o.indptr), shape=o.shape)
                 for g, o in zip(outs, (op, oa, ob)))


def chebyshev_action_bang(out, Hn, V, C, *, check_every: int = 16, verbose: int = 0) -> None:
    """``chebyshev_action!``: out[:, :, k] = sum_n C[n, k] T_{n-1}(Hn) V
    (``src/utils/chebyshev_action.jl:47-122``), overwriting ``out``.

    Coefficients are used verbatim (no h_n, no damping).  ``V``: (NH, NR) or
    (NH,); ``C``: (NC, K) or (NC,); ``out``: complex (NH, NR, K), or the shape
    with the vector axes of ``V`` / ``C`` dropped.  ``check_every`` runs the
    reference's growth guard (0 disables it).
    """
    op = as_operator(Hn)
    Vm = np.asarray(V)
    Cm = np.asarray(C)
    Vm2 = Vm.reshape(Vm.shape[0], -1) if Vm.ndim == 1 else Vm
    Cm2 = Cm.reshape(-1, 1) if Cm.ndim == 1 else Cm
    if Vm2.ndim != 2 or Cm2.ndim != 2:
        raise KPMArgumentError("V and C must be vectors or matrices")
    NH, NR = Vm2.shape
    NC, K = Cm2.shape
    if NC < 1:
        raise KPMArgumentError("C must have at least one coefficient row")
    if NR < 1:
        raise KPMArgumentError("V must have at least one column")
    if K < 1:
        raise KPMArgumentError("C must have at least one coefficient column")
    if op.shape[1] != NH:
        raise KPMArgumentError(f"size(Hn, 2) = {op.shape[1]} must equal size(V, 1) = {NH}")
    if check_every < 0:
        raise KPMArgumentError("check_every must be >= 0")
    if not isinstance(out, np.ndarray) or not np.iscomplexobj(out):
        raise KPMArgumentError("out must be a complex numpy array")
    if np.shares_memory(out, Vm):
        raise KPMArgumentError("out must not alias V")
    expect = [NH, NR, K]
    if out.ndim == 2 and Cm.ndim == 1:
        expect = [NH, NR]
    elif out.ndim == 2 and Vm.ndim == 1:
        expect = [NH, K]
    elif out.ndim == 1:
        expect = [NH]
    if list(out.shape) != expect:
        raise KPMArgumentError(f"out must be {' x '.join(map(str, expect))}, got {out.shape}")
    Vf = np.asfortranarray(Vm2, dtype=np.complex128)
    Cf = np.asfortranarray(Cm2, dtype=np.complex128)
    res = np.empty((NH, NR, K), dtype=np.complex128, order="F")
    lib = _native.load()
    _native.check(lib.kpmgb_chebyshev_action(op.handle, NH, NR, Vf.ctypes.data, NC, K,
                                             Cf.ctypes.data, int(check_every), res.ctypes.data))
    out[...] = res.reshape(out.shape, order="F") if out.ndim < 3 else res


def chebyshev_action(Hn, V, C, **kw):
    """Allocating form of :func:`chebyshev_action_bang`; vector ``V`` drops the
    probe axis, vector ``C`` the coefficient axis (``src/utils/chebyshev_action.jl:148-160``)."""
    Vm, Cm = np.asarray(V), np.asarray(C)
    NH = Vm.shape[0]
    shape = [NH]
    if Vm.ndim == 2:
        shape.append(Vm.shape[1])
    if Cm.ndim == 2:
        shape.append(Cm.shape[1])
    out = np.zeros(shape, dtype=np.complex128)
    chebyshev_action_bang(out, Hn, V, C, **kw)
    return out


def kpm_1d_current(H, Ja, NC: int, NR: int, NH: int | None = None, *, psi_in=None,
                   psi_in_l=None, psi_in_r=None, force_norm: bool = False, verbose: int = 0,
                   avg_output: bool = True, NR_parallel: bool = True, rng=None,
                   precision: str = "fp64", kernel: str = "auto"):
    """Current moments mu_n = <psi| J_a T_n(H) |psi> (``src/moment.jl:558-714``).

    No doubling: the bra J_a^dagger psi is formed on the GPU once and the
    bra/ket recurrence runs NC - 1 steps.  ``Ja`` may be a SciPy matrix (its
    adjoint is uploaded) or a ``GB300Operator`` that already holds
    J_a^dagger.  Returns the complex probe average (length NC), or the
    (NR, NC) matrix with ``avg_output=False``.  The separate-bra form
    (``psi_in_l``/``psi_in_r``) is unimplemented, as in the reference.
    """
    import scipy.sparse as sp
    NH = H.shape[0] if NH is None else int(NH)
    NC, NR = int(NC), int(NR)
    if psi_in is None:
        if psi_in_l is not None or psi_in_r is not None:
            if psi_in_l is None or psi_in_r is None:
                raise KPMArgumentError("must set both `psi_in_l` and `psi_in_r` or neither.")
            raise KPMArgumentError("unimplemented.")
        from .frontend import random_phase_vectors
        rng = np.random.default_rng() if rng is None else rng
        psi_in = random_phase_vectors(rng, NH, NR)
    elif psi_in_l is not None or psi_in_r is not None:
        raise KPMArgumentError(
            "must either set `psi_in` or set `psi_in_l` and `psi_in_r`, but not both.")
    elif force_norm:
        normalize_by_col(psi_in)
    op = as_operator(H)
    jadj = Ja if isinstance(Ja, GB300Operator) else GB300Operator(
        sp.csc_matrix(Ja, dtype=np.complex128).conj().T)
    psi = _colmajor(psi_in, NH, NR, "psi_in")
    lib = _native.load()
    opts = _opts1d(precision, False, kernel)
    out = np.empty((NR, NC), dtype=np.complex128, order="F")
    if NR_parallel:
        _native.check(lib.kpmgb_kpm1d_current(op.handle, jadj.handle, NC, NR, NH,
                                              psi.ctypes.data, out.ctypes.data, C.byref(opts)))
    else:
        for i in range(NR):
            col = np.asfortranarray(psi[:, i:i + 1])
            row = np.empty((1, NC), dtype=np.complex128, order="F")
            _native.check(lib.kpmgb_kpm1d_current(op.handle, jadj.handle, NC, 1, NH,
                                                  col.ctypes.data, row.ctypes.data, C.byref(opts)))
            out[i] = row[0]
    mu_all = np.ascontiguousarray(out)
    if avg_output:
        return mu_all.sum(axis=0) / NR
    return mu_all


def kpm_3d(H, Ja, Jb, Jc, NC: int, NR: int, NH: int, *, arr_size="auto", right_block="auto",
           verbose: int = 0, psi_in_l=None, psi_in_r=None, psi_in=None, precision="fp64",
           contraction="fp64", rng=None):
    """Three-operator moments mu[n, m, p] (NC, NC, NC) (``src/moment.jl:1105-1280``).

    ``mu[:, :, p] = kpm_2d(H, Jc, Jb; psi_l, T_p(H) Ja psi_r)``.  Probe rules
    follow the reference: ``psi_in`` wins over ``psi_in_l``/``psi_in_r``; one
    of the pair alone is used for both; none draws random phases.
    """
    import warnings
    NC, NR, NH = int(NC), int(NR), int(NH)
    if psi_in is not None:
        if psi_in_l is not None or psi_in_r is not None:
            warnings.warn("`psi_in_l`, `psi_in_r` and `psi_in` are simultaneously set. "
                          "Taking `psi_in` and discarding the others")
        psi_in_l = psi_in_r = psi_in
    elif psi_in_l is not None or psi_in_r is not None:
        if psi_in_l is None or psi_in_r is None:
            warnings.warn("only one of `psi_in_l` and `psi_in_r` is set. Setting them as the same.")
            psi_in_l = psi_in_r = psi_in_l if psi_in_l is not None else psi_in_r
    else:
        from .frontend import random_phase_vectors
        rng = np.random.default_rng() if rng is None else rng
        psi_in_l = psi_in_r = random_phase_vectors(rng, NH, NR)
    pl = _colmajor(psi_in_l, NH, NR, "psi_in_l")
    pr = _colmajor(psi_in_r, NH, NR, "psi_in_r")
    ops = [as_operator(M) for M in (H, Ja, Jb, Jc)]
    opts = _opts2d(arr_size, right_block, "auto", "NONE", False, precision, contraction)
    mu = np.zeros((NC, NC, NC), dtype=np.complex128, order="F")
    lib = _native.load()
    _native.check(lib.kpmgb_kpm3d(ops[0].handle, ops[1].handle, ops[2].handle, ops[3].handle, NC,
                                  NR, NH, pl.ctypes.data, pr.ctypes.data, mu.ctypes.data,
                                  C.byref(opts)))
    return mu
