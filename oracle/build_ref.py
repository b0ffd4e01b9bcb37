"""Compiles the reference's kernel sources to sm_103a cubins in oracle/_ref/.

TEST INFRASTRUCTURE ONLY (the second oracle; see ``oracle/ref_kernels.py``).

For every entry of ``REF_CONFIGS`` a two-line translation unit is written to
``oracle/_ref/src/<name>.cu``: the ``#define``s the reference's Python host
would pass to PyCUDA, then an ``#include`` of the unmodified reference source
from the reference checkout.  It is compiled with nvcc to
``oracle/_ref/<name>.cubin`` with the reference's own options for that kernel.
Nothing from the reference is copied into this repository; the cubins are
build products (git-ignored).  Without the reference checkout this is a no-op
and the tests that need the cubins skip.

    python -m oracle.build_ref [--reference PATH] [-f]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle.ref_kernels import REF_CONFIGS, REF_DIR, cubin_path  # noqa: E402

KERNEL_SUBDIR = os.path.join("src", "gpuocean", "gpu_kernels")


def kernel_dir(reference=None):
    """The reference's kernel directory: ``reference`` or, if None,
    ``$GPUOCEAN_REFERENCE``; None when neither names a checkout."""
    reference = reference or os.environ.get("GPUOCEAN_REFERENCE")
    if not reference:
        return None
    d = os.path.join(reference, KERNEL_SUBDIR)
    return d if os.path.isdir(d) else None


def build(reference=None, force=False, verbose=False):
    kdir = kernel_dir(reference)
    if kdir is None:
        return []
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    src_dir = os.path.join(REF_DIR, "src")
    os.makedirs(src_dir, exist_ok=True)
    jobs = []
    for name, (kernel, defines, flags) in REF_CONFIGS.items():
        tu = os.path.join(src_dir, name + ".cu")
        text = "".join(f"#define {k} {v}\n" for k, v in defines.items())
        text += f'#include "{os.path.join(kdir, kernel)}"\n'
        old = open(tu).read() if os.path.exists(tu) else None
        if old != text:
            with open(tu, "w") as f:
                f.write(text)
        out = cubin_path(name)
        if force or old != text or not os.path.exists(out):
            cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", *flags, "-I", kdir, tu, "-o", out]
            jobs.append((name, cmd))

    def run(job):
        name, cmd = job
        if verbose:
            print(" ".join(cmd), flush=True)
        return name, subprocess.run(cmd, capture_output=True, text=True)

    failed = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for name, r in ex.map(run, jobs):
                if r.returncode != 0:
                    failed.append(f"--- {name} ---\n{r.stderr}{r.stdout}")
    if failed:
        raise RuntimeError("reference kernel build failed:\n" + "\n".join(failed))
    return [n for n, _ in jobs]


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    ap.add_argument("-f", action="store_true")
    a = ap.parse_args()
    print(build(a.reference, a.f, verbose=True))
