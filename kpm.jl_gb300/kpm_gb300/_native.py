"""ctypes binding of libkpmgb (the C ABI declared in include/kpmgb.h).

The library must be present: there is no CPU fallback.  Importing this module
does not load it; the first call that needs it does, and raises
``KPMLibraryError`` if it has not been built.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libkpmgb.so"

# status classes (include/kpmgb.h)
OK, ERR_ARGUMENT, ERR_NUMERICAL, ERR_CUDA, ERR_ALLOC, ERR_TIMEOUT = range(6)
PREC_FP64, PREC_FF = 0, 1
CONTRACT_FP64, CONTRACT_SPLIT = 0, 1
PARITY = {"NONE": 0, "ODD": 1, "EVEN": 2}

EXPORTED_SYMBOLS = (
    "kpmgb_version",
    "kpmgb_last_error",
    "kpmgb_operator_create",
    "kpmgb_operator_destroy",
    "kpmgb_operator_info",
    "kpmgb_kpm1d",
    "kpmgb_kpm1d_lr",
    "kpmgb_kpm2d",
    "kpmgb_kpm1d_device",
    "kpmgb_kpm1d_lr_device",
    "kpmgb_kpm2d_device",
    "kpmgb_operator_sync",
    "kpmgb_kernel_launch_count",
    "kpmgb_kpm1d_noalloc",
    "kpmgb_kpm1d_ensemble",
    "kpmgb_kpm1d_ensemble_device",
    "kpmgb_kpm1d_grad",
    "kpmgb_kubo_bastin",
    "kpmgb_dos",
    "kpmgb_dos_derivative",
    "kpmgb_kubo_bastin_weights",
    "kpmgb_kpm2d_grad",
    "kpmgb_chebyshev_action",
    "kpmgb_kpm1d_current",
    "kpmgb_kpm3d",
    "kpmgb_selftest_wait_expiry",
    "kpmgb_timing_enable",
    "kpmgb_timing_read",
    "kpmgb_measure_fp64_peak",
    "kpmgb_host_alloc",
    "kpmgb_host_free",
)


class KPMLibraryError(RuntimeError):
    """libkpmgb.so is missing or cannot be loaded."""


class KPMArgumentError(ValueError):
    """Invalid arguments (the reference's ArgumentError / AssertionError)."""


class KPMNumericalError(RuntimeError):
    """Recurrence left the stable region or produced non-finite moments."""


class KPMDeviceError(RuntimeError):
    """CUDA runtime, allocation or timeout failure."""


class Kpm1dOptions(C.Structure):
    _fields_ = [("precision", C.c_int32), ("stability_check", C.c_int32),
                ("use_graph", C.c_int32), ("kernel_variant", C.c_int32)]


class Kpm2dOptions(C.Structure):
    _fields_ = [("arr_size", C.c_int64), ("right_block", C.c_int64),
                ("workspace_bytes", C.c_int64), ("moment_parity", C.c_int32),
                ("mn_sym", C.c_int32), ("precision", C.c_int32), ("contraction", C.c_int32)]


_lib = None
_lock = threading.Lock()


def _declare(lib):
    vp, i32, i64, dp = C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_double)
    f64 = C.c_double
    lib.kpmgb_version.restype = C.c_char_p
    lib.kpmgb_last_error.restype = C.c_char_p
    lib.kpmgb_kernel_launch_count.restype = i64
    lib.kpmgb_operator_create.argtypes = [i64, i64, vp, vp, vp, i32, C.POINTER(vp)]
    lib.kpmgb_operator_destroy.argtypes = [vp]
    lib.kpmgb_operator_info.argtypes = [vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i32)]
    lib.kpmgb_kpm1d.argtypes = [vp, i64, i64, i64, vp, vp, C.POINTER(Kpm1dOptions)]
    lib.kpmgb_kpm1d_lr.argtypes = [vp, i64, i64, i64, vp, vp, vp, C.POINTER(Kpm1dOptions)]
    lib.kpmgb_kpm2d.argtypes = [vp, vp, vp, i64, i64, i64, vp, vp, vp, C.POINTER(Kpm2dOptions)]
    lib.kpmgb_kpm1d_device.argtypes = [vp, i64, i64, i64, vp, vp, C.POINTER(Kpm1dOptions), vp]
    lib.kpmgb_kpm1d_lr_device.argtypes = [vp, i64, i64, i64, vp, vp, vp,
                                          C.POINTER(Kpm1dOptions), vp]
    lib.kpmgb_kpm2d_device.argtypes = [vp, vp, vp, i64, i64, i64, vp, vp, vp,
                                       C.POINTER(Kpm2dOptions), vp]
    lib.kpmgb_operator_sync.argtypes = [vp, vp]
    lib.kpmgb_kpm1d_ensemble.argtypes = [vp, i32, vp, i64, i64, vp, vp, C.POINTER(Kpm1dOptions)]
    lib.kpmgb_kpm1d_ensemble_device.argtypes = [vp, i32, vp, i64, i64, vp, vp,
                                                C.POINTER(Kpm1dOptions), vp]
    lib.kpmgb_kubo_bastin.argtypes = [vp, i64, i64, f64, f64, vp, i64, i64, f64, f64, vp, i64,
                                      f64, vp]
    lib.kpmgb_kpm1d_current.argtypes = [vp, vp, i64, i64, i64, vp, vp, C.POINTER(Kpm1dOptions)]
    lib.kpmgb_selftest_wait_expiry.argtypes = [vp]
    lib.kpmgb_kpm3d.argtypes = [vp, vp, vp, vp, i64, i64, i64, vp, vp, vp, C.POINTER(Kpm2dOptions)]
    lib.kpmgb_chebyshev_action.argtypes = [vp, i64, i64, vp, i64, i64, vp, i64, vp]
    lib.kpmgb_dos.argtypes = [vp, i64, f64, f64, vp, vp, i64, vp]
    lib.kpmgb_dos_derivative.argtypes = [vp, i64, f64, f64, vp, vp, i64, i32, vp]
    lib.kpmgb_kubo_bastin_weights.argtypes = [i64, f64, f64, f64, i64, f64, f64, vp, i64, f64, vp]
    lib.kpmgb_kpm2d_grad.argtypes = [vp, vp, vp, vp, i64, i64, i64, vp, vp, vp, i32, vp, vp, vp]
    lib.kpmgb_kpm1d_grad.argtypes = [vp, i64, i64, i64, vp, vp, i64, vp]
    lib.kpmgb_kpm1d_noalloc.argtypes = [i64, vp, vp, vp, i64, i64, vp, vp, vp]
    lib.kpmgb_timing_enable.argtypes = [i32]
    lib.kpmgb_timing_read.argtypes = [i32, dp, C.POINTER(i64)]
    lib.kpmgb_measure_fp64_peak.argtypes = [dp]
    lib.kpmgb_host_alloc.argtypes = [i64, C.POINTER(vp)]
    lib.kpmgb_host_free.argtypes = [vp]
    for name in EXPORTED_SYMBOLS:
        if name not in ("kpmgb_version", "kpmgb_last_error", "kpmgb_kernel_launch_count"):
            getattr(lib, name).restype = C.c_int


def load(path: Path | None = None):
    """Load (once) and return the ctypes library handle."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise KPMLibraryError(
                f"{p} is missing: build it with kpm_gb300.build.build() (nvcc, sm_103a); "
                "this package has no CPU fallback")
        try:
            lib = C.CDLL(str(p))
        except OSError as e:  # pragma: no cover - depends on the host
            raise KPMLibraryError(f"cannot load {p}: {e}") from e
        _declare(lib)
        _lib = lib
        return lib


def check(rc: int) -> None:
    """Raise the exception class matching a non-zero status."""
    if rc == OK:
        return
    msg = (_lib.kpmgb_last_error() or b"").decode(errors="replace")
    if rc == ERR_ARGUMENT:
        raise KPMArgumentError(msg)
    if rc == ERR_NUMERICAL:
        raise KPMNumericalError(msg)
    raise KPMDeviceError(f"status {rc}: {msg}")


def pinned_empty(shape, dtype=np.complex128, order="C"):
    """An uninitialised NumPy array in page-locked host memory
    (kpmgb_host_alloc), freed when the array is collected."""
    import weakref
    lib = load()
    dt = np.dtype(dtype)
    n = int(np.prod(shape)) * dt.itemsize
    ptr = C.c_void_p()
    check(lib.kpmgb_host_alloc(max(n, 1), C.byref(ptr)))
    buf = (C.c_char * max(n, 1)).from_address(ptr.value)
    arr = np.frombuffer(buf, dtype=dt, count=int(np.prod(shape)))
    arr = arr.reshape(shape, order=order)
    weakref.finalize(buf, lib.kpmgb_host_free, C.c_void_p(ptr.value))
    return arr


def version() -> str:
    return load().kpmgb_version().decode()


def kernel_launch_count() -> int:
    return int(load().kpmgb_kernel_launch_count())


TIMED = {"contract_split": 0, "contract_fp64": 1}


def timing_enable(on: bool) -> None:
    """Bracket the instrumented kernels' launches with CUDA events (or stop)."""
    check(load().kpmgb_timing_enable(1 if on else 0))


def timing_read(kernel: str):
    """(summed device ms, launches) of one instrumented kernel since the last
    read; waits for the recorded events."""
    ms, n = C.c_double(0.0), C.c_int64(0)
    check(load().kpmgb_timing_read(TIMED[kernel], C.byref(ms), C.byref(n)))
    return ms.value, n.value


def measure_fp64_peak() -> float:
    """Measured FP64 FMA rate of the current device, TFLOP/s."""
    t = C.c_double(0.0)
    check(load().kpmgb_measure_fp64_peak(C.byref(t)))
    return t.value
