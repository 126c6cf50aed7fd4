"""Builds libevrgpu.so (the sm_103a H.psi library) in-tree with nvcc.

The translation units are compiled in parallel and linked against the CUDA runtime,
the CUDA runtime only (no BLAS or LAPACK library).  Output: elvibrot-tnumtana_gb300/_build/libevrgpu.so.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG_ROOT, "csrc")
BUILD = os.path.join(PKG_ROOT, "_build")
LIB = os.path.join(BUILD, "libevrgpu.so")
SOURCES = ["evr_setup.cpp", "evr_kernels.cu", "evr_capi.cu", "evr_davidson.cu", "evr_propagate.cu", "evr_peaks.cu",
           "evr_noalloc.cu", "evr_tc_test.cu", "evr_filter.cu", "evr_lanczos.cu", "evr_wpio.cpp", "evr_stages.cu", "evr_control.cu", "evr_batch.cu", "evr_kern_items_d0.cu", "evr_kern_items_d1.cu",
           "evr_kern_items_f0.cu", "evr_kern_items_f1.cu", "evr_kern_slab_d0.cu", "evr_kern_slab_d1.cu",
           "evr_kern_slab_f0.cu", "evr_kern_slab_f1.cu", "evr_kern_slab_f0tc.cu", "evr_kern_slab_f1tc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(os.path.dirname(PKG_ROOT), "include", "evr_gpu.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    common = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3"]

    def comp(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [cc] + common + ["-c", os.path.join(CSRC, src), "-o", obj]
        if src.endswith(".cpp"):
            cmd = [cc, "-x", "cu"] + common + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(comp, srcs))
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
