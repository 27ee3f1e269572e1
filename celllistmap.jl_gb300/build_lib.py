"""Build recipe of libcelllist_cuda.so (sm_103a).

Compiles the CUDA translation units in parallel with nvcc and links them into
``celllistmap.jl_gb300/_build/libcelllist_cuda.so``.  Host code is compiled
with -ffp-contract=off so that the box geometry keeps the reference's
separately rounded arithmetic; device code on the exact path uses explicit
round-to-nearest intrinsics.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libcelllist_cuda.so")
SOURCES = ["clm_api.cu", "clm_build.cu", "clm_pairs.cu", "clm_pairs_f32.cu", "clm_pairs_f64.cu", "clm_pairs_batch.cu",
           "clm_batched.cu", "clm_noalloc.cu"]
PEAKS_SRC = "clm_peaks.cu"
PEAKS_LIB = os.path.join(OUT_DIR, "libclm_peaks.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcelllist_cuda.so")


def _flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                   "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
                   "-I", os.path.join(ROOT, "include"), "-I", CSRC] + list(extra)


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "celllistmap_gb300.h"),
                                                                 __file__]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_info else []

    def compile_one(src):
        obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        cmd = [cc, "-c", os.path.join(CSRC, src), "-o", obj] + _flags(extra)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    if verbose or ptxas_info:
        for obj, err in results:
            if err:
                print(err)
    tmp = LIB + ".tmp"
    cmd = [cc, "-shared", "-o", tmp] + [o for o, _ in results] + ARCH + ["-Xcompiler", "-fPIC"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr)
    os.replace(tmp, LIB)
    # FMA-pipe peak probes used by bench.py for the pair-kernel roofline
    cmd = [cc, "-shared", "-o", PEAKS_LIB, os.path.join(CSRC, PEAKS_SRC)] + _flags()
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on clm_peaks.cu:\n" + r.stderr)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
