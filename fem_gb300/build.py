"""Build the GB300 LinA shared library (sm_103a) in-tree with nvcc.

Output: fem_gb300/_build/libLinA_gb300.so.  Translation units are compiled in
parallel; only what changed since the last build is recompiled.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INC = os.path.join(ROOT, "include")
LIB = os.path.join(OUT, "libLinA_gb300.so")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off",
                   f"-I{INC}", f"-I{SRC}"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", f"-I{INC}", f"-I{SRC}",
             "-I/usr/local/cuda/include"]
C_FLAGS = ["-O2", "-std=c11", "-fPIC", "-fopenmp", "-ffp-contract=off", f"-I{INC}", f"-I{SRC}",
           "-I/usr/local/cuda/include"]


def _sources():
    out = []
    for f in sorted(os.listdir(SRC)):
        if f.endswith((".cu", ".cpp", ".c")):
            out.append(os.path.join(SRC, f))
    return out


def _headers_mtime():
    m = 0.0
    for d in (SRC, INC):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh", ".hpp")):
                m = max(m, os.path.getmtime(os.path.join(d, f)))
    return m


def _compile(src, force):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    if not force and os.path.exists(obj):
        if os.path.getmtime(obj) >= max(os.path.getmtime(src), _headers_mtime()):
            return obj, None
    if src.endswith(".cu"):
        cmd = [NVCC] + CU_FLAGS + ["-c", src, "-o", obj]
    elif src.endswith(".cpp"):
        cmd = [os.environ.get("CXX", "g++")] + CXX_FLAGS + ["-c", src, "-o", obj]
    else:
        cmd = [os.environ.get("CC", "gcc")] + C_FLAGS + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}"
    return obj, None


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, force), srcs))
    errs = [e for _, e in results if e]
    if errs:
        raise RuntimeError("compilation failed:\n" + "\n".join(errs))
    objs = [o for o, _ in results]
    newest = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [NVCC, "-shared"] + ARCH + ["-Xcompiler", "-fopenmp", "-Xlinker", "-Bsymbolic", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
