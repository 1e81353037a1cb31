"""Build the C-ABI shared library ``libtatva_gb300.so`` in-tree for sm_103a.

Every translation unit is compiled by nvcc in parallel with
``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and linked into one
shared library next to this file.  Objects are cached under ``_build/`` and
rebuilt when a source, a header or the flags change.
"""

from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_NAME = "libtatva_gb300.so"
LIB_PATH = os.path.join(PKG_DIR, LIB_NAME)

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON_FLAGS = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "--expt-relaxed-constexpr",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-fvisibility=hidden",
    "-I" + INCLUDE,
    "-I" + CSRC,
]


def _nvcc() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    for p in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(p):
            return p
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build tatva_gb300")


def _cuda_lib_dir() -> str:
    nvcc = _nvcc()
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "lib64")


def _sources():
    return sorted(
        os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp"))
    )


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return sorted(hs)


def _digest(paths, extra):
    h = hashlib.sha256()
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    h.update(" ".join(extra).encode())
    h.update(b"cudart-shared")
    return h.hexdigest()[:16]


def build(verbose: bool = False, jobs: int | None = None, extra_flags=()) -> str:
    """Compile (if stale) and link the library; returns its path."""
    nvcc = _nvcc()
    os.makedirs(BUILD_DIR, exist_ok=True)
    flags = ARCH_FLAGS + COMMON_FLAGS + list(extra_flags)
    hdr = _digest(_headers(), flags)
    objs, cmds = [], []
    for src in _sources():
        tag = _digest([src], [hdr])
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + "." + tag + ".o")
        objs.append(obj)
        if not os.path.exists(obj):
            x = ["-x", "cu"] if src.endswith(".cu") else []
            cmds.append([nvcc, *flags, *x, "-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {cmd[-3]}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, flush=True)
        return r

    if cmds:
        n = jobs or min(len(cmds), os.cpu_count() or 4)
        with ThreadPoolExecutor(max_workers=n) as ex:
            list(ex.map(run, cmds))
    stamp = os.path.join(BUILD_DIR, "lib.stamp")
    want = _digest(objs, []) if all(os.path.exists(o) for o in objs) else ""
    have = open(stamp).read() if os.path.exists(stamp) else None
    if not os.path.exists(LIB_PATH) or have != want or cmds:
        tmp = LIB_PATH + ".tmp"
        # One CUDA runtime per process: link the shared libcudart.so.13 (the one torch
        # has already loaded resolves it by soname), so that stream handles created by
        # the host framework are valid in this library.
        run([nvcc, *ARCH_FLAGS, "-shared", "-cudart", "shared", "-o", tmp, *objs, "-lpthread",
             "-Xlinker", "-rpath," + _cuda_lib_dir()])
        os.replace(tmp, LIB_PATH)
        with open(stamp, "w") as f:
            f.write(want)
    # drop stale objects of older builds
    keep = set(objs)
    for f in os.listdir(BUILD_DIR):
        p = os.path.join(BUILD_DIR, f)
        if f.endswith(".o") and p not in keep:
            os.remove(p)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True))
