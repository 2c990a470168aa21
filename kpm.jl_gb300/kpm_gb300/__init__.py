"""GB300 Chebyshev-moment engine: a drop-in for KPM.jl's kpm_1d / kpm_2d path.

Host-side mirror of the reference interface over the C ABI of libkpmgb
(include/kpmgb.h).  All moment arithmetic runs in hand-written sm_103a CUDA;
there is no CPU fallback.
"""
from ._native import (KPMArgumentError, KPMDeviceError, KPMLibraryError, KPMNumericalError,
                      kernel_launch_count, measure_fp64_peak, pinned_empty, timing_enable,
                      timing_read, version)
from .frontend import (ConductivityMoments, DosMoments, RescaledHamiltonian, cond_moments,
                       dos, dos0, dos_basis, dos_moments, jackson_kernel, kubo_bastin_cond, kubo_bastin_weights, normalizeH, on_device, random_phase_vectors, rescale)
from .moment import (EnsembleOperator, chebyshev_action, chebyshev_action_bang, kpm_1d, kpm_1d_bang, kpm_1d_current, kpm_1d_derivative, kpm_2d_derivative, kpm_1d_device, kpm_1d_ensemble, kpm_1d_ensemble_device, kpm_1d_grad, kpm_2d, kpm_2d_bang, kpm_2d_blocking, kpm_2d_grad, kpm_3d,
                     kpm_2d_device, normalize_by_col, sync)
from .operator import GB300Operator, as_operator

__all__ = [
    "KPMArgumentError", "KPMDeviceError", "KPMLibraryError", "KPMNumericalError",
    "kernel_launch_count", "measure_fp64_peak", "pinned_empty", "timing_enable", "timing_read", "version", "ConductivityMoments", "DosMoments",
    "RescaledHamiltonian", "cond_moments", "dos", "dos0", "dos_basis", "dos_moments", "jackson_kernel", "kubo_bastin_cond", "kubo_bastin_weights", "normalizeH", "on_device",
    "random_phase_vectors", "rescale", "EnsembleOperator", "chebyshev_action", "chebyshev_action_bang", "kpm_1d", "kpm_1d_bang", "kpm_1d_current", "kpm_1d_derivative", "kpm_2d_derivative", "kpm_1d_device", "kpm_1d_ensemble", "kpm_1d_ensemble_device", "kpm_1d_grad", "kpm_2d",
    "kpm_2d_bang", "kpm_2d_blocking", "kpm_2d_grad", "kpm_3d", "kpm_2d_device", "normalize_by_col", "sync",
    "GB300Operator", "as_operator",
]
