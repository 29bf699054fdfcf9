"""Builds the CUDA engine into sbd_gb300/_build/libsbdgb.so (sm_103a only).

Each translation unit is compiled by its own nvcc process (in parallel) and
the objects are linked into one shared library with the C ABI of
include/sbdgb.h.  No CMake, no torch extension machinery: plain nvcc.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libsbdgb.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OUT, os.path.basename(src).replace(".cu", ".o"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(
            os.path.getmtime(src), *[os.path.getmtime(os.path.join(CSRC, h)) for h in os.listdir(CSRC)
                                     if h.endswith((".cuh", ".h"))],
            os.path.getmtime(os.path.join(ROOT, "include", "sbdgb.h"))):
        return obj
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(OUT, exist_ok=True)
    extra = list(extra or [])
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    _build_rates(extra)
    if verbose:
        print(LIB)
    return LIB


RATES_SRC = os.path.join(HERE, "bench_csrc", "rates.cu")
RATES_LIB = os.path.join(OUT, "libsbdgb_rates.so")


def _build_rates(extra: list[str]) -> str:
    """The FP64 rate probe of the benchmark (bench_csrc/rates.cu), a library of
    its own: it is a measurement utility, not part of the engine's ABI."""
    if os.path.exists(RATES_LIB) and os.path.getmtime(RATES_LIB) >= os.path.getmtime(RATES_SRC):
        return RATES_LIB
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-shared", RATES_SRC, "-o", RATES_LIB, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {RATES_SRC}:\n{r.stdout}\n{r.stderr}")
    return RATES_LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
