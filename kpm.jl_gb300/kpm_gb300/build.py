"""Build libkpmgb.so in-tree with nvcc for sm_103a.

Each CUDA translation unit is compiled in parallel, then linked into a shared
library with the CUDA runtime linked statically (no dependency on a
particular libcudart.so at load time).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
ROOT = PKG_DIR.parent                    # kpm.jl_gb300/
CSRC = ROOT / "csrc"
INCLUDE = ROOT.parent / "include"
LIB_DIR = PKG_DIR / "_lib"
LIB_PATH = LIB_DIR / "libkpmgb.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = [
    "kpmgb_api.cu",
    "kpmgb_recurrence.cu",
    "kpmgb_step_f64.cu",
    "kpmgb_step_ff.cu",
    "kpmgb_step_ffe.cu",
    "kpmgb_small.cu",
    "kpmgb_cluster.cu",
    "kpmgb_contract.cu",
    "kpmgb_contract_tc.cu",
    "kpmgb_noalloc.cu",
    "kpmgb_ensemble.cu",
    "kpmgb_adjoint.cu",
    "kpmgb_recon.cu",
    "kpmgb_action.cu",
    "kpmgb_timing.cu",
    "kpmgb_tune.cu",
    "kpmgb_alloc.cu",
    "kpmgb_hostio.cu",
    "kpmgb_step_ffpk.cu",
]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libkpmgb")
    return exe


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False, defines=(), out: Path | None = None,
          objdir: Path | None = None) -> Path:
    """Compile libkpmgb.so if any source or header is newer than the library.

    ``defines`` (e.g. ``["KPMGB_FF_MIN_BLOCKS=2"]``) set the kernels' tuning
    macros; a tuned variant is written to ``out`` with objects in ``objdir``.
    """
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    objdir = Path(objdir) if objdir else ROOT / "_build"
    objdir.mkdir(parents=True, exist_ok=True)
    lib_path = Path(out) if out else LIB_PATH
    lib_path.parent.mkdir(parents=True, exist_ok=True)
    flags = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                    f"-I{INCLUDE}", f"-I{CSRC}"] + [f"-D{d}" for d in defines]
    cc = nvcc()

    def compile_one(src: str) -> Path:
        s = CSRC / src
        o = objdir / (s.stem + ".o")
        if force or _stale(o, [s] + headers):
            cmd = [cc, *flags, "-c", str(s), "-o", str(o)]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
            if verbose:
                print(f"compiled {src}", file=sys.stderr)
        return o

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(SOURCES), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    if force or _stale(lib_path, objs):
        tmp = lib_path.with_suffix(".so.tmp")
        cmd = [cc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
