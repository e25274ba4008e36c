"""Build recipe for the GB300 library (libcovof_gpu.so) -- sm_103a only.

Compiles each CUDA translation unit with nvcc in parallel and links them into
an in-tree shared library at covof_2d-fortran_gb300/_build/libcovof_gpu.so.
No cmake and no pip install: the .so stays next to the sources so that a
process loading it can be traced back to this tree.

-fmad=false: every kernel evaluates expressions exactly as written (no fused
multiply-add contraction), which is what makes the VOF step and the operator
applications bit-identical to a serial FP64 evaluation.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_build"
LIB = OUT_DIR / "libcovof_gpu.so"
SOURCES = ["poisson.cu", "momentum.cu", "vof.cu", "svof.cu", "adjoint.cu", "capi.cu", "batch.cu", "static_scratch.cu", "output.cu", "precond.cu", "peak.cu"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-std=c++17", "-lineinfo", "-fmad=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
    # host arithmetic (the history sums) in program order, no FMA contraction
    "-Xcompiler", "-ffp-contract=off",
    "-diag-suppress", "177,550",
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


CHECKED_DIR = PKG / "_build_checked"


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> Path:
    """Compile (if needed) and return the path of libcovof_gpu.so.
    checked: the bounds-check build (-DCOVOF_CHECKED) into _build_checked/,
    for tests that run the parity cases with every stencil index checked."""
    nvcc = _nvcc()
    out_dir = CHECKED_DIR if checked else OUT_DIR
    lib = out_dir / "libcovof_gpu.so"
    flags = NVCC_FLAGS + (["-DCOVOF_CHECKED"] if checked else [])
    out_dir.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "covof_gpu.h"]
    objs = []
    jobs = []
    for src in SOURCES:
        s = CSRC / src
        o = out_dir / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc] + flags + ["-c", str(s), "-o", str(o)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed: " + " ".join(cmd))

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(lib, objs):
        run([nvcc] + ARCH + ["-shared", "-o", str(lib)] + [str(o) for o in objs] + ["-lcudart"])
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, checked="--checked" in sys.argv))
