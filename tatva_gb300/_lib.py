"""ctypes binding of the C ABI (``include/tatva_gb300.h``).

The shared library is built in-tree by ``tatva_gb300.build()``.  There is no
fallback: if the library is missing every compute call raises.
"""

from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32, c_int64, c_size_t, c_void_p

from . import _build

TG_OK, TG_ERR_VALUE, TG_ERR_TYPE, TG_ERR_CUDA, TG_ERR_UNSUPPORTED = 0, 1, 2, 3, 4
TG_ERR_NOT_CONVERGED, TG_ERR_WORKSPACE, TG_ERR_BREAKDOWN = 5, 6, 7
TG_TRI3, TG_TET4, TG_HEX8 = 0, 1, 2
TG_F32, TG_F64 = 0, 1
TG_POISSON, TG_LINEAR_ELASTIC, TG_NEO_HOOKEAN = 0, 1, 2
TG_MODE_RESIDUAL, TG_MODE_HVP, TG_MODE_DIAG = 0, 1, 2


class NotConvergedError(RuntimeError):
    """A solver reached its iteration budget before the tolerance."""


class BreakdownError(RuntimeError):
    """CG breakdown: p.Ap <= 0 or a non-finite value appeared."""


_EXC = {
    TG_ERR_VALUE: ValueError,
    TG_ERR_TYPE: TypeError,
    TG_ERR_CUDA: RuntimeError,
    TG_ERR_UNSUPPORTED: NotImplementedError,
    TG_ERR_NOT_CONVERGED: NotConvergedError,
    TG_ERR_WORKSPACE: RuntimeError,
    TG_ERR_BREAKDOWN: BreakdownError,
}


class BlockPlan(ctypes.Structure):
    _fields_ = [
        ("n_blocks", c_int32),
        ("n_elems", c_int32),
        ("nodes_per_elem_padded", c_int32),
        ("max_local_nodes", c_int32),
        ("n_shared", c_int32),
        ("n_partials", c_int32),
        ("threads", c_int32),
        ("n_affine_blocks", c_int32),
        ("n_diag_blocks", c_int32),
        ("max_block_elems", c_int32),
        ("blk_elem_ptr", c_void_p),
        ("blk_color_ptr", c_void_p),
        ("color_ofs", c_void_p),
        ("blk_node_ptr", c_void_p),
        ("lconn", c_void_p),
        ("elem_id", c_void_p),
        ("lnode_gid", c_void_p),
        ("lnode_slot", c_void_p),
        ("lnode_smem", c_void_p),
        ("shared_node", c_void_p),
        ("shared_ptr", c_void_p),
        ("shared_slots", c_void_p),
        ("box_geom32", c_void_p),
        ("n_lattice_blocks", c_int32),
        ("reserved0", c_int32),
        ("grid_nodes", c_int32 * 3),
        ("grid_reserved", c_int32),
        ("grid_h", c_double * 3),
    ]


class Material(ctypes.Structure):
    _fields_ = [
        ("kind", c_int32),
        ("reserved", c_int32),
        ("p0", c_double),
        ("p1", c_double),
        ("p2", c_double),
        ("p3", c_double),
        ("elem_param", c_void_p),
    ]


class SolveStats(ctypes.Structure):
    _fields_ = [
        ("status", c_int32),
        ("iterations", c_int32),
        ("outer", c_int32),
        ("reserved", c_int32),
        ("rel_res", c_double),
    ]


class BrickRequest(ctypes.Structure):
    _fields_ = [
        ("nodes", c_int32 * 3),
        ("reserved", c_int32),
        ("h", c_double * 3),
        ("mu", c_double),
        ("lam", c_double),
        ("b", c_void_p),
        ("x", c_void_p),
        ("fixed", c_void_p),
        ("workspace", c_void_p),
        ("workspace_bytes", c_size_t),
        ("rtol", c_double),
        ("inner_rtol", c_double),
        ("max_outer", c_int32),
        ("max_inner", c_int32),
    ]


class BrickState(ctypes.Structure):
    _fields_ = [
        ("phase", c_int32),
        ("status", c_int32),
        ("iterations", c_int32),
        ("outer", c_int32),
        ("rel_res", c_double),
    ]


TG_BRICK_MAX_SLOTS = 64
TG_BRICK_FREE, TG_BRICK_REFINE, TG_BRICK_RUN, TG_BRICK_DONE, TG_BRICK_FAILED = 0, 1, 2, 3, 4


class BatchDesc(ctypes.Structure):
    _fields_ = [
        ("n_systems", c_int32),
        ("max_rows", c_int32),
        ("row_ofs", c_void_p),
        ("ell_ofs", c_void_p),
        ("ell_width", c_void_p),
        ("order", c_void_p),
        ("ell_col", c_void_p),
        ("ell_val32", c_void_p),
        ("ell_val64", c_void_p),
    ]


class OperatorDesc(ctypes.Structure):
    _fields_ = [
        ("elem", c_int32),
        ("prec", c_int32),
        ("mat", Material),
        ("plan", c_void_p),
        ("coords", c_void_p),
        ("n_nodes", c_int64),
        ("u", c_void_p),
        ("fixed", c_void_p),
        ("n_rows", c_int64),
        ("csr_indptr", c_void_p),
        ("csr_indices", c_void_p),
        ("csr_data", c_void_p),
        ("csr_node_ptr", c_void_p),
        ("csr_node_indices", c_void_p),
    ]


P = c_void_p
I = c_int
L = c_int64
D = c_double
S = c_size_t

# name -> (restype, argtypes)
SIGNATURES = {
    "tg_last_error": (c_char_p, []),
    "tg_version": (c_int, []),
    "tg_device_sm_count": (c_int, []),
    "tg_stream_create": (I, [POINTER(c_void_p)]),
    "tg_stream_destroy": (I, [P]),
    "tg_stream_synchronize": (I, [P]),
    "tg_device_synchronize": (I, []),
    "tg_eval": (I, [I, I, P, L, I, P, L, P, P]),
    "tg_grad": (I, [I, I, P, P, L, I, P, L, P, P]),
    "tg_integration_weights": (I, [I, I, P, L, P, L, P, P]),
    "tg_integrate_quad": (I, [I, P, P, L, I, I, P, P]),
    "tg_sum_rows_workspace_bytes": (S, [I, I]),
    "tg_sum_rows": (I, [I, P, L, I, P, P, S, P]),
    "tg_gather_nodal": (I, [I, P, L, I, P, L, I, P, P]),
    "tg_integrate_quad_transpose": (I, [I, P, P, L, I, I, P, P]),
    "tg_scatter_nodal": (I, [I, P, L, I, I, P, P, P, P]),
    "tg_grad_transpose_workspace_bytes": (S, [I, I, L, I]),
    "tg_grad_transpose": (I, [I, I, P, P, L, I, P, L, P, P, P, P, S, P]),
    "tg_eval_transpose": (I, [I, I, P, L, I, P, L, P, P, P, P]),
    "tg_plan_build": (I, [I, P, L, L, P, I, I, I, POINTER(c_void_p)]),
    "tg_plan_sizes": (I, [P, P]),
    "tg_plan_export": (I, [P] + [P] * 12),
    "tg_plan_free": (None, [P]),
    "tg_grid_detect": (I, [I, P, L, L, P, I, P, P]),
    "tg_plan_box_geometry": (I, [P, P, P, P, P]),
    "tg_apply_workspace_bytes": (S, [I, I, I, P]),
    "tg_apply": (I, [I, I, I, P, P, P, L, P, P, P, P, P, S, P]),
    "tg_apply_noalloc": (I, [I, I, I, P, P, P, L, P, P, P, P, P]),
    "tg_energy_per_element": (I, [I, I, P, P, L, P, L, P, P, P]),
    "tg_compressed_hessian": (I, [I, I, P, P, L, P, L, P, P, P, P, I, P, P]),
    "tg_rows_cols": (I, [P, P, P, L, L, P, P, P]),
    "tg_decompress": (I, [I, P, I, P, P, L, P, P]),
    "tg_color_seeds": (I, [I, P, L, I, I, P, P]),
    "tg_set_column": (I, [I, P, L, I, I, P, P]),
    "tg_spmv": (I, [I, L, P, P, P, P, P, P]),
    "tg_csr_node_blocks3": (I, [L, P, P, P, P, P, P]),
    "tg_spmv_blocks3": (I, [I, L, P, P, P, P, P, P, P]),
    "tg_csr_diagonal": (I, [I, L, P, P, P, P, P]),
    "tg_csr_apply_dirichlet": (I, [I, L, P, P, P, P, P]),
    "tg_operator_workspace_bytes": (S, [P]),
    "tg_operator_apply": (I, [P, P, P, P, S, P]),
    "tg_dot_workspace_bytes": (S, []),
    "tg_dot": (I, [I, P, P, L, P, P, S, P]),
    "tg_axpby": (I, [I, L, D, P, D, P, P]),
    "tg_convert": (I, [I, P, I, P, L, P]),
    "tg_cg_workspace_bytes": (S, [P]),
    "tg_cg_solve": (I, [P, P, P, P, D, I, I, P, S, P, P]),
    "tg_mixed_workspace_bytes": (S, [P, P]),
    "tg_mixed_solve": (I, [P, P, P, P, P, D, D, I, I, I, P, S, P, P]),
    "tg_brick_batch_create": (I, [POINTER(c_void_p)]),
    "tg_brick_batch_destroy": (None, [P]),
    "tg_brick_workspace_bytes": (S, [P]),
    "tg_brick_admit": (I, [P, P, P, P]),
    "tg_brick_step": (I, [P, I, P]),
    "tg_brick_poll": (I, [P, P, I, P]),
    "tg_batch_ell_from_csr": (I, [P, L, P, P, P, P, P]),
    "tg_batch_workspace_bytes": (S, [L]),
    "tg_batch_solve": (I, [P, L, P, P, D, D, I, I, I, I, P, S, P, P, P, P, P]),
    "tg_pattern_build": (I, [P, L, I, L, I, POINTER(c_void_p)]),
    "tg_pattern_nnz": (I, [P, P]),
    "tg_pattern_export": (I, [P, P, P]),
    "tg_pattern_free": (None, [P]),
    "tg_distance2_colors": (I, [P, P, L, P, P]),
    "tg_element_colors": (I, [P, L, I, L, P, P, P, P]),
    "tg_node_incidence": (I, [P, L, I, L, P, P]),
}

_LIB = None


def library_path() -> str:
    return _build.LIB_PATH


def lib():
    """Load the library once; raise if it has not been built."""
    global _LIB
    if _LIB is None:
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(
                f"{os.path.basename(path)} is not built: call tatva_gb300.build() first "
                "(there is no non-CUDA fallback)"
            )
        import torch  # noqa: F401  (loads the process's CUDA runtime first)

        handle = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = handle
    return _LIB


def check(rc: int) -> None:
    if rc != TG_OK:
        msg = lib().tg_last_error().decode(errors="replace")
        raise _EXC.get(rc, RuntimeError)(msg)


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))
