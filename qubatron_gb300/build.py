"""Build libqbcuda.so in-tree with nvcc for sm_103a.

The traversal must stay bit-exact with the shader's FP32 arithmetic, so the
device code is compiled with -fmad=false (no fused multiply-add), IEEE division
and square root and no flush-to-zero, and the host code with
-ffp-contract=off.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libqbcuda.so")

SOURCES = ["qbcuda.cu", "frame.cu", "proposal.cu", "build.cu", "boxes.cu", "mlp.cu", "host.cpp"]
HEADERS = ["trace.cuh", "walker.cuh", "render.cuh", "qbc_internal.h", "qbc_ctx.h", "mlp.h", "mlp_device.cuh"]

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-lineinfo", "-O3", "-std=c++17",
    "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    "-shared",
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(ROOT, "include", "qbcuda.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile libqbcuda.so if any source is newer; return its path. The
    translation units compile in parallel, then link into one shared library."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    inc = ["-I", os.path.join(ROOT, "include")]
    compile_flags = [f for f in NVCC_FLAGS if f != "-shared"]
    procs = []
    objs = []
    for src in SOURCES:
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        cmd = [_nvcc(), *compile_flags, *inc, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd += ["-Xptxas", "-v"]
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)))
    errors = []
    for src, p in procs:
        out, err = p.communicate()
        if p.returncode != 0:
            errors.append(f"--- {src}\n{out}{err}")
        elif verbose:
            sys.stderr.write(err)
    if errors:
        raise RuntimeError("nvcc failed building libqbcuda:\n" + "\n".join(errors))
    tmp = LIB + ".tmp"
    link = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-Xcompiler", "-fPIC", "-o", tmp, *objs]
    res = subprocess.run(link, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("nvcc failed linking libqbcuda:\n" + res.stdout + res.stderr)
    os.replace(tmp, LIB)
    for o in objs:
        os.remove(o)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
