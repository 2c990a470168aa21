"""Build the C oracle (kpm_cpu.c) into oracle/_build/libkpm_cpu.so (TEST INFRASTRUCTURE).

The reference itself is Julia and has no C/C++ sources, so there is no
oracle/_ref build: nothing of the reference can be compiled here.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "kpm_cpu.c"
OUT = HERE / "_build" / "libkpm_cpu.so"


def build(force: bool = False) -> Path:
    OUT.parent.mkdir(exist_ok=True)
    if not force and OUT.exists() and OUT.stat().st_mtime >= SRC.stat().st_mtime:
        return OUT
    cc = shutil.which("gcc") or "cc"
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [cc, "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", str(SRC), "-o", str(tmp)]
    subprocess.run(cmd, check=True, capture_output=True)
    tmp.replace(OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
