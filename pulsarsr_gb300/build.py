"""Build libpsr.so (sm_103a) in-tree: pulsarsr_gb300/_build/libpsr.so.

Each CUDA translation unit is compiled in parallel with nvcc for
compute_103a/sm_103a, then linked into one shared library.  --fmad=false
keeps nvcc from contracting a*b+c: the parity kernels use explicit
__fmaf_rn/__fadd_rn intrinsics wherever an FMA is intended.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpsr.so")
CLI = os.path.join(OUT, "psr")

NVCC_FLAGS = [
    "-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo",
    "--fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
    "-Xptxas", "-warn-spills",
]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpsr")
    return path


def sources() -> list[str]:
    return sorted(os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith(".cu")
                  and not f.startswith("cli_"))


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
    deps = [src] + [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith(".h")]
    deps.append(os.path.join(HERE, "..", "include", "psr.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc(), *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip():
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(OUT, exist_ok=True)
    extra = extra or []
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), sources()))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [nvcc(), "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", LIB, *objs,
               "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    cli_src = os.path.join(SRC, "cli_psr.cpp")
    if os.path.exists(cli_src):
        if not os.path.exists(CLI) or os.path.getmtime(CLI) < max(os.path.getmtime(cli_src),
                                                                  os.path.getmtime(LIB)):
            cmd = ["g++", "-O2", "-std=c++17", "-o", CLI, cli_src,
                   f"-I{os.path.join(HERE, '..', 'include')}", f"-L{OUT}", "-lpsr",
                   f"-Wl,-rpath,$ORIGIN", "-pthread"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"cli build failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
