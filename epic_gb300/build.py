"""Build the in-tree CUDA library epic_gb300/_lib/libepic_gb300.so for sm_103a.

nvcc compiles each translation unit in parallel (one -gencode, -lineinfo) and links one
shared library with the C ABI of include/epic_gb300.h.  Host code is compiled with
-ffp-contract=off so the host-side set-up gives the same bits on x86-64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libepic_gb300.so")
SOURCES = ["epic_model.cu", "k_filter.cu", "k_filter_gemm.cu", "k_column.cu", "k_column_acc.cu", "k_stencil.cu", "k_turb.cu", "epic_setup.cpp",
           "epic_dropin.cpp"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags() -> list[str]:
    # -fmad=false keeps every binary64 operation separately rounded (the FP64 form matches the
    # reference bit for bit); -prec-div/-prec-sqrt=false make binary32 division and square root
    # (used by the mixed form only) the fast approximate instructions, within 2 ulp
    extra = os.environ.get("EPIC_NVCC_EXTRA", "").split()
    return ["-O3", "-std=c++17", ARCH, "-lineinfo", "-fmad=false", "-prec-div=false", "-prec-sqrt=false",
            "-Xcompiler", "-fPIC,-ffp-contract=off",
            "-I" + os.path.join(ROOT, "include"), "-I" + SRC, "--expt-relaxed-constexpr", *extra]


def _compile(src: str) -> str:
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    deps = [os.path.join(SRC, src)] + [os.path.join(SRC, h) for h in os.listdir(SRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(ROOT, "include", "epic_gb300.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    cmd = [_nvcc(), *_flags(), "-c", os.path.join(SRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    stamp = os.path.join(OUT, "build_flags.txt")
    flags = " ".join(_flags())
    if not os.path.exists(stamp) or open(stamp).read() != flags:
        for f in os.listdir(OUT):
            if f.endswith(".o") or f.endswith(".so"):
                os.remove(os.path.join(OUT, f))
        with open(stamp, "w") as fh:
            fh.write(flags)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [_nvcc(), ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
