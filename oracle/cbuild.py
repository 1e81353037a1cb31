"""Build and bind the plain-C oracle restatements (test infrastructure only).

``csparse.c`` restates the reference's sparsity pattern and natural-order greedy
distance-2 colouring for sizes where the Python oracle in ``sparse.py`` is too slow.
It is compiled with the host C compiler into ``oracle/_build/`` (not part of the
product, which never loads it)."""

from __future__ import annotations

import ctypes
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csparse.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle_sparse.so")
_LIB = None


def build() -> str:
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = shutil.which("cc") or shutil.which("gcc")
    if not cc:
        raise RuntimeError("no C compiler for the oracle")
    tmp = LIB + ".tmp"
    subprocess.run([cc, "-O2", "-shared", "-fPIC", SRC, "-o", tmp], check=True)
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _LIB
    if _LIB is None:
        L = ctypes.CDLL(build())
        P, I64 = ctypes.c_void_p, ctypes.c_int64
        L.oracle_pattern.argtypes = [P, I64, ctypes.c_int, I64, ctypes.c_int, P, P]
        L.oracle_pattern.restype = ctypes.c_int
        L.oracle_d2_colors.argtypes = [P, P, I64, P]
        L.oracle_d2_colors.restype = ctypes.c_int
        _LIB = L
    return _LIB


def pattern(elements, n_nodes, ndpn):
    """(indptr int64, indices int32) of _create_sparse_structure (_extraction.py:37-102)."""
    conn = np.ascontiguousarray(elements, dtype=np.int32)
    n = int(n_nodes) * ndpn
    indptr = np.zeros(n + 1, np.int64)
    L = lib()
    if L.oracle_pattern(conn.ctypes.data, conn.shape[0], conn.shape[1], int(n_nodes), ndpn,
                        indptr.ctypes.data, None):
        raise MemoryError("oracle_pattern")
    indices = np.empty(int(indptr[-1]), np.int32)
    if L.oracle_pattern(conn.ctypes.data, conn.shape[0], conn.shape[1], int(n_nodes), ndpn,
                        indptr.ctypes.data, indices.ctypes.data):
        raise MemoryError("oracle_pattern")
    return indptr, indices


def d2_colors(indptr, indices):
    """Natural-order greedy distance-2 colours (_coloring.py:27-48, 136-153, 270-283)."""
    indptr = np.ascontiguousarray(indptr, dtype=np.int64)
    indices = np.ascontiguousarray(indices, dtype=np.int32)
    n = indptr.size - 1
    colors = np.empty(n, np.int32)
    if lib().oracle_d2_colors(indptr.ctypes.data, indices.ctypes.data, n, colors.ctypes.data) < 0:
        raise MemoryError("oracle_d2_colors")
    return colors
