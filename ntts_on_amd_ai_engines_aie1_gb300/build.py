"""Builds libgb300ntt.so in-tree for sm_103a (nvcc + g++, no cmake).

    python -m ntts_on_amd_ai_engines_aie1_gb300.build      # or __graft_entry__.build()

Translation units compile in parallel; objects go to _build/, the ptxas
resource report of every kernel to _build/ptxas.log.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libgb300ntt.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["abi.cu", "batch.cu", "batch_k16.cu", "batch_k16_w64.cu", "batch_k16_w32.cu", "batch_k16_w32g.cu", "batch_k16_w16.cu", "batch_k16_w16g.cu", "batch_k16_zc.cu", "batch_k32.cu", "batch_k32_w16.cu", "noalloc.cu", "kernels_r2.cu", "kernels_r2_32.cu", "kernels_r4_r8.cu", "kernels_misc.cu", "kernels_large.cu", "serve.cu", "canon_tables.cu", "kernels_c16.cu", "kernels_c32.cu", "batch_c16.cu", "batch_c16_small.cu", "batch_c32.cu", "kernels_c32_large.cu"]
CXX_SOURCES = ["tables.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(PKG), "include", "gb300_ntt.h"))
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                         "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-v",
                         "-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                         "-Wall", "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        logs = list(ex.map(_run, jobs))
    if logs:
        with open(os.path.join(BUILD, "ptxas.log"), "w") as f:
            f.write("\n".join(logs))
    if force or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lpthread", "-Xlinker", "--no-undefined"])
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
