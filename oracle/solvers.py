"""Reference solvers (oracle, test infrastructure only).

The reference ships no solver: users compose ``jax.scipy.sparse.linalg.cg``
with the matrix-free HVP (``README.md:93``).  This is the plain FP64
Jacobi-preconditioned CG used to check the device solvers.
"""

from __future__ import annotations

import numpy as np


def jacobi_cg(apply, b, diag, x0=None, rtol=1e-10, maxiter=100000):
    x = np.zeros_like(b) if x0 is None else x0.copy()
    r = b - apply(x)
    z = r / diag
    p = z.copy()
    rz = r @ z
    bn = np.linalg.norm(b)
    it = 0
    while np.linalg.norm(r) > rtol * bn and it < maxiter:
        q = apply(p)
        alpha = rz / (p @ q)
        x += alpha * p
        r -= alpha * q
        z = r / diag
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
        it += 1
    return x, it
