"""Build libasmooth_gb300.so in-tree for sm_103a with nvcc.

Each CUDA translation unit under csrc/ is compiled in parallel into
csrc/_build/*.o and linked into asmooth_gb300/libasmooth_gb300.so (CUDA
runtime linked statically, so the library only needs the driver).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libasmooth_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
UNITS = ["asg_index", "asg_knn", "asg_deposit", "asg_fof", "asg_output", "asg_shell", "asg_decode", "asg_capi", "asg_noalloc"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build asmooth_gb300")


def _sources_mtime() -> float:
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
             if f.endswith((".cu", ".cuh", ".h"))]
    paths.append(os.path.join(INCLUDE, "asmooth_gb300.h"))
    paths.append(os.path.abspath(__file__))
    return max(os.path.getmtime(p) for p in paths)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if stale) and return the path of the shared library."""
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) >= _sources_mtime():
        return OUT
    cc = nvcc()
    bdir = os.path.join(CSRC, "_build")
    os.makedirs(bdir, exist_ok=True)

    def compile_unit(u: str) -> str:
        obj = os.path.join(bdir, u + ".o")
        cmd = [cc, *ARCH, *FLAGS, "-c", os.path.join(CSRC, u + ".cu"), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {u}.cu:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, UNITS))
    tmp = OUT + f".{os.getpid()}.tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True, verbose=True))
