"""In-tree build of the CUDA library ``glphase_gb300/libglphase_gpu.so``.

Five translation units (the host side and four tables of generation-kernel
instantiations) compiled in parallel with nvcc, one ``-gencode`` (sm_103a),
then linked; host code with ``-ffp-contract=off`` so host-side float
arithmetic rounds identically on x86-64 and aarch64.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJDIR = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libglphase_gpu.so")
SOURCES = ["glp_api.cu", "glp_gen_single_f32.cu", "glp_gen_single_vq.cu",
           "glp_gen_multi_f32.cu", "glp_gen_multi_vq.cu", "glp_gen_single_f32_sub4.cu",
           "glp_gen_single_vq_sub4.cu", "glp_gen_multi_f32_sub4.cu", "glp_gen_multi_vq_sub4.cu"]
HEADERS = ["glp_kernels.cuh", "glp_rng.h", "glp_launch.h", "glp_knn.cuh", "glp_tract.h",
           "glp_tally.cuh", "glp_vq.cuh", "glp_server_core.h"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
         "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return "nvcc"


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(ROOT, "include", "glphase_gpu.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str], verbose: bool) -> subprocess.CompletedProcess:
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    return subprocess.run(cmd, capture_output=True, text=True)


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> str:
    if not force and not needs_build():
        return LIB
    os.makedirs(OBJDIR, exist_ok=True)
    extra = ["-Xptxas=-v"] if ptxas_v else []
    # extra nvcc flags for tuning experiments, e.g. GLP_NVCC_FLAGS=-maxrregcount=96
    extra += os.environ.get("GLP_NVCC_FLAGS", "").split()
    jobs = []
    for s in SOURCES:
        obj = os.path.join(OBJDIR, s.replace(".cu", ".o"))
        jobs.append((obj, [nvcc(), ARCH] + FLAGS + extra +
                     ["-c", os.path.join(CSRC, s), "-o", obj]))
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        results = list(ex.map(lambda j: _run(j[1], verbose), jobs))
    for (obj, _), res in zip(jobs, results):
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(obj)}:\n" + res.stdout +
                               res.stderr)
        if ptxas_v or verbose:
            print(res.stderr, file=sys.stderr)
    link = [nvcc(), ARCH, "-shared", "-o", LIB + ".tmp"] + [o for o, _ in jobs]
    res = _run(link, verbose)
    if res.returncode != 0:
        raise RuntimeError("nvcc link failed:\n" + res.stdout + res.stderr)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    build(force=True, verbose=True, ptxas_v="-v" in sys.argv)
