"""Build the native library and CLI in-tree (nvcc + g++, no CMake).

Outputs:
  lulesh_gb300/lib/liblulesh_gb300.so   the C ABI of include/lulesh_gb300.h
  lulesh_gb300/bin/lulesh_gpu           the drop-in command line (lulesh2.0 options)

Every CUDA translation unit is compiled for sm_103a only.  The FP64 parity
kernels are compiled with --fmad=false so each operation rounds like the
reference's -ffp-contract=off build; the other copy allows FMA contraction.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
BINDIR = os.path.join(PKG, "bin")
LIB = os.path.join(LIBDIR, "liblulesh_gb300.so")
CLI = os.path.join(BINDIR, "lulesh_gpu")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                      "-I" + CSRC, "-I" + os.path.join(ROOT, "include")]

# (source, extra nvcc flags)
CUDA_UNITS = [
    ("lg_kernels_fp64.cu", ["--fmad=false"]),
    ("lg_kernels_fma.cu", ["--fmad=true"]),
    ("lg_kernels_mixed.cu", ["--fmad=true"]),
    ("lg_api.cu", []),
    ("lg_ensemble.cu", []),
    ("lg_adjoint.cu", ["--fmad=true"]),
    ("lg_peak.cu", ["--fmad=true"]),
    ("lg_noalloc.cu", ["--fmad=false"]),
    ("lg_setup.cu", ["--fmad=false"]),
    ("lg_halo.cu", ["--fmad=false"]),
]
HOST_UNITS = ["lg_problem.cc"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
          if f.endswith((".h", ".cuh", ".inc"))]
    return hs + [os.path.join(ROOT, "include", "lulesh_gb300.h")]


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile everything that is out of date; return the library path."""
    nvcc = _nvcc()
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BINDIR, exist_ok=True)
    hdrs = _headers()
    steps = []
    objs = []
    for src, extra in CUDA_UNITS:
        s = os.path.join(CSRC, src)
        if not os.path.exists(s):
            continue
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            steps.append([nvcc] + NVCC_COMMON + extra + ["-c", s, "-o", o])
    for src in HOST_UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src + ".o")
        objs.append(o)
        if _stale(o, [s] + hdrs):
            # no FMA contraction: set-up arithmetic (volumes, masses, the first
            # time step) must round exactly as the reference's on every host
            # (GCC contracts by default on aarch64)
            steps.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I" + CSRC,
                          "-I" + os.path.join(ROOT, "include"), "-c", s, "-o", o])
    cli_src = os.path.join(CSRC, "lulesh_gpu.cc")
    cli_obj = os.path.join(OBJ, "lulesh_gpu.cc.o")
    if _stale(cli_obj, [cli_src] + hdrs):
        steps.append(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                      "-I" + os.path.join(ROOT, "include"), "-c", cli_src, "-o", cli_obj])
    with ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        for cmd in steps:
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
        list(ex.map(_run, steps))
    exports = os.path.join(CSRC, "exports.map")
    if _stale(LIB, objs + [exports]):
        # only the C ABI (lg_*) is exported; internal C++ symbols stay local
        _run([nvcc] + ARCH + ["-shared", "-Xlinker", "--version-script=" + exports, "-o", LIB]
             + objs)
    if _stale(CLI, [cli_obj, LIB]):
        _run(["g++", "-o", CLI, cli_obj, "-L" + LIBDIR, "-llulesh_gb300",
              "-Wl,-rpath,$ORIGIN/../lib"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
