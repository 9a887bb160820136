"""Builds libptgpu.so (the CUDA engine behind include/ptgpu.h) in-tree with nvcc for sm_103a.

Translation units compile in parallel; the field kernels and the FP64 multigrid kernels are
compiled without FMA contraction so that they round exactly like the reference's expressions (see
csrc/pt_fields.cu, csrc/pt_mg.cu); kernels that want a fused multiply-add call fma() explicitly.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libptgpu.so")
BUILD = os.path.join(HERE, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off",
          "-Xptxas", "-O3", "--expt-relaxed-constexpr"]
EXTRA = {"pt_fields.cu": ["--fmad=false"], "pt_mg.cu": ["--fmad=false"], "pt_direct.cu": ["--fmad=false"],
         "pt_io.cu": ["--fmad=false"], "pt_equalize.cu": ["--fmad=false"]}
SOURCES = ["pt_setup.cpp", "pt_fields.cu", "pt_tracers.cu", "pt_mg.cu", "pt_mixed.cu", "pt_api.cu", "pt_unet.cu",
           "pt_direct.cu", "pt_io.cu", "pt_equalize.cu"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "ptgpu.h"))
    return any(os.path.getmtime(d) > os.path.getmtime(obj) for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        if force or _stale(o, s):
            cmd = [cc] + ARCH + COMMON + EXTRA.get(src, []) + ["-c", s, "-o", o]
            if src.endswith(".cpp"):
                cmd = [cc, "-x", "cu"] + cmd[1:]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r.returncode

    with ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        codes = list(ex.map(run, jobs))
    if any(codes):
        raise RuntimeError("nvcc failed")
    objs = [os.path.join(BUILD, s + ".o") for s in SOURCES]
    if force or jobs or not os.path.exists(OUT):
        cmd = [cc] + ARCH + ["-shared", "-o", OUT] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"]
        if run(cmd):
            raise RuntimeError("link failed")
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
