"""Sparsity pattern, distance-2 colouring and colored Jacobians (oracle, test only).

Restates:
  * ``_create_sparse_structure`` / ``pattern_from_mesh``
        tatva/sparse/_extraction.py:37-102  (dof = node*ndpn + comp, rows/cols by
        repeat/tile, linearised ``np.unique`` ordering, int8 ones)
  * ``get_distance2_adjacency`` (A @ A)          tatva/sparse/_coloring.py:27-48
  * ``greedy_coloring`` (natural order, smallest free colour)
                                                 tatva/sparse/_coloring.py:136-153
  * ``distance2_colors``                         tatva/sparse/_coloring.py:270-283
  * ``compute_rows_cols``                        tatva/sparse/base.py:108-136
  * ``colored_jacobian_batch`` (one JVP per colour with seed = (colors==c))
                                                 tatva/sparse/base.py:230-270
  * ``jacfwd`` decompression ``data = Jc[rows, col_colors]``
                                                 tatva/sparse/base.py:163-176

The reference obtains its colours from the external ``tatva_coloring``
package (``tatva/sparse/base.py:32,66``), whose source is not part of the
reference tree; the in-repo natural-order greedy colouring restated here is
the one this project pins to.  Hessian values do not depend on which valid
distance-2 colouring is used.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sps


def create_sparse_structure(elements, n_dofs_per_node, K_shape):
    elements_np = np.asarray(elements, dtype=np.int64)
    n_el, npe = elements_np.shape
    nde = npe * n_dofs_per_node
    dofs = elements_np[..., None] * n_dofs_per_node + np.arange(n_dofs_per_node, dtype=np.int64)
    element_dofs = dofs.reshape(n_el, -1)
    rows = np.repeat(element_dofs, nde, axis=1).ravel()
    cols = np.tile(element_dofs, (1, nde)).ravel()
    lin = np.unique(rows * K_shape[1] + cols)
    r, c = lin // K_shape[1], lin % K_shape[1]
    return sps.csr_matrix((np.ones(r.shape[0], dtype=np.int8), (r, c)), shape=K_shape)


def pattern_from_mesh(coords, elements, n_dofs_per_node):
    n = n_dofs_per_node * np.asarray(coords).shape[0]
    return create_sparse_structure(elements, n_dofs_per_node, (n, n))


def distance2_adjacency(n_dofs, indptr, indices):
    A = sps.csr_matrix(
        (np.ones(len(indices), dtype=bool), np.asarray(indices), np.asarray(indptr)),
        shape=(n_dofs, n_dofs),
    )
    A2 = (A @ A).tocsr()
    A2.sort_indices()
    return A2.indptr, A2.indices


def greedy_colors(n_dofs, a2_ptr, a2_idx):
    """Natural-order greedy: colour i = smallest colour unused among coloured
    distance-2 neighbours (pure Python loop: small cases only)."""
    colors = -np.ones(n_dofs, dtype=np.int32)
    for i in range(n_dofs):
        nb = colors[a2_idx[a2_ptr[i]:a2_ptr[i + 1]]]
        used = set(nb[nb >= 0].tolist())
        c = 0
        while c in used:
            c += 1
        colors[i] = c
    return colors


def distance2_colors(indptr, indices, n_dofs):
    p, i = distance2_adjacency(n_dofs, indptr, indices)
    return greedy_colors(n_dofs, p, i)


def compute_rows_cols(indptr, indices, colors):
    indptr = np.asarray(indptr)
    rows = np.repeat(np.arange(len(indptr) - 1), np.diff(indptr))
    col_colors = np.asarray(colors)[np.asarray(indices)]
    return rows, col_colors


def colored_jacobian(jvp, n_dofs, colors, n_colors=None):
    """Jc (N, C) with Jc[:, c] = jvp(seed_c), seed_c = (colors == c) as 1.0/0.0."""
    colors = np.asarray(colors)
    n_colors = int(colors.max()) + 1 if n_colors is None else n_colors
    Jc = np.zeros((n_dofs, n_colors))
    for c in range(n_colors):
        seed = np.where(colors == c, 1.0, 0.0)
        Jc[:, c] = jvp(seed)
    return Jc


def decompress(Jc, rows, col_colors):
    return Jc[rows, col_colors]


def check_distance2(indptr, indices, colors):
    """True when every row's columns carry pairwise distinct colours and each
    column's colour differs from the row's (structurally valid Hessian compression)."""
    indptr, indices, colors = map(np.asarray, (indptr, indices, colors))
    for r in range(len(indptr) - 1):
        cc = colors[indices[indptr[r]:indptr[r + 1]]]
        if len(np.unique(cc)) != len(cc):
            return False
    return True


def element_colors(elements, n_nodes):
    """Greedy natural-order element colouring: elements sharing a node differ."""
    elements = np.asarray(elements)
    E = elements.shape[0]
    inc = [[] for _ in range(n_nodes)]
    for e in range(E):
        for a in elements[e]:
            inc[a].append(e)
    col = -np.ones(E, dtype=np.int32)
    for e in range(E):
        used = set()
        for a in elements[e]:
            for f in inc[a]:
                if col[f] >= 0:
                    used.add(int(col[f]))
        c = 0
        while c in used:
            c += 1
        col[e] = c
    return col
