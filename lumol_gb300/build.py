"""Build recipe of the engine's shared library (sm_103a, in-tree).

`build()` compiles every CUDA translation unit of `csrc/` in parallel with nvcc
for `sm_103a` and links `liblumol_gb300.so` next to this file.  It is also what
`__graft_entry__.build()` calls.
"""
from __future__ import annotations

import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblumol_gb300.so")
SOURCES = ["nlist.cu", "forces.cu", "mixed.cu", "persist.cu", "md.cu", "diag.cu", "mc.cu", "noalloc.cu",
           "lower.cu", "runtime.cu", "capi.cu", "capi_mc.cu"]

NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17",
    # host code restates the reference's arithmetic: keep products and sums unfused
    "-Xcompiler", "-fPIC,-ffp-contract=off",
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _compile(src: str) -> tuple[str, int, str]:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [_nvcc(), *NVCC_FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    return obj, proc.returncode, proc.stdout + proc.stderr


def _stale(objs: list[str]) -> bool:
    if not os.path.exists(LIB):
        return True
    lib_t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(HERE, "..", "include", "lumol_gb300.h"))
    return any(os.path.getmtime(d) > lib_t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles the CUDA sources and links the shared library; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    objs = [os.path.join(BUILD, os.path.splitext(s)[0] + ".o") for s in SOURCES]
    if not force and not _stale(objs):
        return LIB
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as pool:
        results = list(pool.map(_compile, SOURCES))
    failed = [(o, log) for o, rc, log in results if rc != 0]
    if verbose:
        for _, _, log in results:
            sys.stdout.write(log)
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(log for _, log in failed))
    tmp = LIB + ".tmp"
    link = [_nvcc(), "-shared", "-o", tmp, *objs, "-lcudart"]
    proc = subprocess.run(link, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("link failed:\n" + proc.stdout + proc.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
