"""Builds the in-tree native libraries of mpifdtd_gb300.

* ``_build/libmpifdtd_gb300.so``  CUDA engine (C ABI of include/mpifdtd_gb300.h),
  compiled for sm_103a only.
* ``_build/libmpifdtd_upml.so``   drop-in entry points of the reference
  (include/mpifdtd_upml.h); needs the host program's field_*/models_* symbols.
* ``_build/libmpifdtd_field.so``  the library's own implementation of the
  reference's field.h / models.h host API (for programs without field.c).
* ``_build/libmpifdtd_surrogate.so`` the far-field surrogate's kernels
  (tcgen05 BF16 GEMM, element-wise forward/backward, Adam), sm_103a.

Translation units compile in parallel; no cmake.  Host code is compiled with
-ffp-contract=off because it evaluates the reference's one-time formulas
(sigma profiles, coefficients, NTFF shifts) and must round as the reference.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"

ENGINE_SO = BUILD / "libmpifdtd_gb300.so"
UPML_SO = BUILD / "libmpifdtd_upml.so"
FIELD_SO = BUILD / "libmpifdtd_field.so"
SURROGATE_SO = BUILD / "libmpifdtd_surrogate.so"
SURROGATE_SOURCES = ["surrogate_gemm.cu", "surrogate_ops.cu"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     f"-I{INCLUDE}"]
CC_FLAGS = ["-O2", "-fPIC", "-ffp-contract=off", "-Wall", f"-I{INCLUDE}"]

ENGINE_SOURCES = ["fdtd_kernels.cu", "fdtd_tblock.cu", "fdtd_tblock_serial.cu", "fdtd_batch.cu", "fdtd_api.cu", "fdtd_setup.cu", "ntff_noalloc.cu",
                  "fdtd_farfield.cu", "fdtd_dft.cu", "fdtd_split.cu", "fdtd_checkpoint.cu"]
# The model evaluators classify sub-cell samples with comparisons such as
# px*px + py*py <= r*r (circleModel.c:45-57); a fused multiply-add could flip a
# sample on the boundary, so that file is compiled without contraction.
# The split-field / NS update rounds every operation as the reference's C does.
PER_FILE_FLAGS = {"fdtd_setup.cu": ["-fmad=false"], "fdtd_split.cu": ["-fmad=false"]}


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _run(cmd, verbose):
    if verbose:
        print(" ".join(str(c) for c in cmd), flush=True)
    r = subprocess.run([str(c) for c in cmd], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    return r


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _headers():
    return list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile every extension for sm_103a; returns the engine library path."""
    BUILD.mkdir(parents=True, exist_ok=True)
    hdrs = _headers()
    objs = []
    jobs = []
    sobjs = []
    for src in ENGINE_SOURCES + SURROGATE_SOURCES:
        s = CSRC / src
        o = BUILD / (s.stem + ".o")
        (objs if src in ENGINE_SOURCES else sobjs).append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([nvcc()] + NVCC_FLAGS + PER_FILE_FLAGS.get(src, []) + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(lambda c: _run(c, verbose), jobs))
    if force or _stale(ENGINE_SO, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", ENGINE_SO] + objs, verbose)
    if force or _stale(SURROGATE_SO, sobjs):
        _run([nvcc()] + ARCH + ["-shared", "-o", SURROGATE_SO] + sobjs, verbose)
    # drop-in layer (C) and the library's own field/models host API, both
    # linked against the engine and finding it next to themselves ($ORIGIN)
    link = [f"-L{BUILD}", "-lmpifdtd_gb300", "-Wl,-rpath,$ORIGIN", "-lm"]
    for src, so in ((CSRC / "compat_upml.c", UPML_SO), (CSRC / "field_host.c", FIELD_SO)):
        if force or _stale(so, [src] + hdrs + [ENGINE_SO]):
            _run([os.environ.get("CC", "gcc"), "-std=gnu99"] + CC_FLAGS + [f"-I{CSRC}", "-shared", "-o", so, src]
                 + link, verbose)
    return ENGINE_SO


if __name__ == "__main__":
    import sys
    build(verbose=True, force="--force" in sys.argv)
    print("built", ENGINE_SO)
