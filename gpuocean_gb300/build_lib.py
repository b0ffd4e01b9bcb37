"""Builds ``libgpuocean_gb300.so`` (sm_103a) from ``csrc/`` with nvcc.

The translation units are compiled in parallel and linked in-tree next to this
file, so the library is found by ``gpuocean_gb300._lib`` without installation.
Run ``python -m gpuocean_gb300.build_lib`` or call :func:`build`.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_obj")
LIB = os.path.join(HERE, "libgpuocean_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
BASE = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "--expt-relaxed-constexpr"]
# the reference builds its step kernel with flush-to-zero and approximate
# division and square root (S/CDKLM16.py:277-281); most of this library does
# the same.  Files in DEFAULT_MATH keep CUDA's default (IEEE) arithmetic, as
# the reference's boundary kernels are built (U/Common.py:1140-1151).
COMMON = BASE + ["-ftz=true", "-prec-div=false", "-prec-sqrt=false"]
DEFAULT_MATH = {"sponge.cu"}
# per-file extra flags.  The step translation units keep every multiply and
# add separately rounded (no FMA contraction), as the reference compiles its
# step kernel (--fmad=false): with the same operation order this makes the
# RK2 step bit-identical to the reference's kernel.  The random numbers, the
# SOAR field and the KL model error use fast math, as the reference's noise
# kernels do; the transfer of the SOAR field to the state is built like the
# ensemble step, whose fused epilogue runs the same code (noise_transfer.cuh)
# and must round identically; so must the single-collection drifter kernels
# and the drifter work of the ensemble step.  The adjoint (cdklm_adjoint.cu)
# contracts multiply-adds: it is tested against FP64 autograd, not for bits.
EXTRA = {"noise.cu": ["-use_fast_math"],
         "noise_transfer.cu": ["-fmad=false"],
         "drift.cu": ["-fmad=false"],
         "cdklm_step.cu": ["-fmad=false"],
         "ensemble.cu": ["-fmad=false"],
         **{f"ensemble_shape_{tx}x{ty}.cu": ["-fmad=false"]
            for tx, ty in ((32, 16), (32, 8), (16, 16), (64, 8), (32, 24))}}


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found; the CUDA toolkit is required to build gpuocean_gb300")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _needs(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    nvcc = nvcc_path()
    os.makedirs(OBJ, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "gpuocean_gb300.h"))
    jobs = []
    for src in sources():
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src[:-3] + ".o")
        if force or _needs(o, [s] + headers):
            flags = BASE if src in DEFAULT_MATH else COMMON
            cmd = [nvcc, *ARCH, *flags, *EXTRA.get(src, []), "-c", s, "-o", o]
            jobs.append((src, cmd))
    failed = []

    def run(job):
        name, cmd = job
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        return name, r

    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for name, r in ex.map(run, jobs):
                if r.returncode != 0:
                    failed.append((name, r.stderr + r.stdout))
                elif verbose and (r.stderr or r.stdout):
                    print(r.stderr + r.stdout)
    if failed:
        msg = "\n".join(f"--- {n} ---\n{e}" for n, e in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    objs = [os.path.join(OBJ, s[:-3] + ".o") for s in sources()]
    if force or jobs or _needs(LIB, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr + r.stdout)
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
