"""The C-ABI library: it loads, exports every entry point the header declares, maps
status codes to the reference's exception types, and the package refuses to run
compute on host tensors (no CPU fallback).  No GPU compute here."""

import ctypes
import os
import re

import numpy as np
import pytest
import torch

from tatva_gb300 import Mesh, Operator, _lib, element, materials

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "tatva_gb300.h")).read()
    return sorted(set(re.findall(r"TG_API\s+[\w\s\*]+?\b(tg_\w+)\s*\(", src)))


def test_every_declared_symbol_is_exported():
    names = _declared()
    assert len(names) >= 40
    L = _lib.lib()
    for n in names:
        assert hasattr(L, n), n
    # and the ctypes binding covers exactly the header
    assert set(names) == set(_lib.SIGNATURES)


def test_version_and_error_string():
    L = _lib.lib()
    assert L.tg_version() >= 1
    assert isinstance(L.tg_last_error(), bytes)


def test_status_codes_map_to_reference_exceptions():
    L = _lib.lib()
    conn = np.array([[0, 1, 5]], np.int32)
    h = ctypes.c_void_p()
    rc = L.tg_pattern_build(conn.ctypes.data, 1, 3, 3, 1, ctypes.byref(h))
    assert rc == _lib.TG_ERR_VALUE
    with pytest.raises(ValueError, match="outside the mesh coordinates array"):
        _lib.check(rc)
    conn = np.array([[0, -1, 2]], np.int32)
    with pytest.raises(ValueError, match="negative node indices"):
        _lib.check(L.tg_pattern_build(conn.ctypes.data, 1, 3, 3, 1, ctypes.byref(h)))
    with pytest.raises(TypeError):
        _lib.check(L.tg_convert(7, None, 0, None, 1, None))
    with pytest.raises(ValueError):
        _lib.check(L.tg_apply(0, 0, 0, None, None, None, 1, None, None, None, None, None, 0, None))


def test_compute_on_host_tensors_fails_loudly():
    m = Mesh.unit_square(2, 2, device="cpu")
    op = Operator(m, element.Tri3())
    u = torch.zeros(m.n_nodes, dtype=torch.float64)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        op.grad(u)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        materials.Poisson(op, 1.0).residual(u)


def test_operator_validation_matches_reference_messages():
    nodes = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0]])
    with pytest.raises(ValueError, match="references nodes outside"):
        Operator(Mesh(nodes, np.array([[0, 1, 3]], np.int32), device="cpu"), element.Tri3())
    with pytest.raises(ValueError, match="negative node indices"):
        Operator(Mesh(nodes, np.array([[0, -1, 2]], np.int32), device="cpu"), element.Tri3())
    with pytest.raises(ValueError, match="at least one element"):
        Operator(Mesh(nodes, np.zeros((0, 3), np.int32), device="cpu"), element.Tri3())
    with pytest.raises(TypeError, match="integer indices"):
        Mesh(nodes, np.array([[0.0, 1.0, 2.0]]), device="cpu")
    with pytest.raises(NotImplementedError):
        element.Tri3(quad_points=np.zeros((1, 2)), quad_weights=np.ones(1))


def test_lifter_semantics_on_host():
    """tests/test_lifter.py known answers with Fixed (torch on the host)."""
    from tatva_gb300.lifter import Fixed, Lifter

    lf = Lifter(6, Fixed(np.array([0, 5])))
    full = lf.lift_from_zeros(torch.tensor([10.0, 20.0, 30.0, 40.0], dtype=torch.float64))
    np.testing.assert_array_equal(full.numpy(), [0, 10, 20, 30, 40, 0])
    np.testing.assert_array_equal(lf.reduce(full).numpy(), [10, 20, 30, 40])
    np.testing.assert_array_equal(
        lf.reduce_adjoint(torch.arange(6.0, dtype=torch.float64)).numpy(), [1, 2, 3, 4])
    lf2 = Lifter(6, Fixed(np.array([0, 5]), np.array([0.0, 1.0])))
    np.testing.assert_array_equal(
        lf2.lift_from_zeros(torch.zeros(4, dtype=torch.float64)).numpy(), [0, 0, 0, 0, 0, 1])
    assert lf2.fixed_mask("cpu").tolist() == [1, 0, 0, 0, 0, 1]


def test_node_block_spmv_argument_checks():
    """The node-block entry points reject row counts that are not multiples of 3 and
    missing buffers before any launch."""
    L = _lib.lib()
    with pytest.raises(ValueError, match="multiple of 3"):
        _lib.check(L.tg_csr_node_blocks3(4, None, None, None, None, None, None))
    with pytest.raises(ValueError, match="multiple of 3"):
        _lib.check(L.tg_spmv_blocks3(_lib.TG_F32, 5, None, None, None, None, None, None, None))
    with pytest.raises(ValueError):
        _lib.check(L.tg_spmv_blocks3(_lib.TG_F32, 6, None, None, None, None, None, None, None))
    assert L.tg_spmv_blocks3(_lib.TG_F32, 0, None, None, None, None, None, None, None) == _lib.TG_OK



def test_brick_workspace_bytes_is_a_host_query():
    """The request engine's per-request workspace size (host arithmetic, no device):
    FP64 residual, five FP32 vectors, the node mask and the partials, each 256-byte
    aligned; zero for a brick with fewer than two nodes on an axis."""
    L = _lib.lib()
    q = lambda n: int(L.tg_brick_workspace_bytes((ctypes.c_int32 * 3)(*n)))
    assert q((1, 3, 3)) == 0 and q((3, 3, 1)) == 0
    small, big = q((3, 3, 3)), q((17, 17, 17))
    assert small > 0 and big > small and small % 256 == 0 and big % 256 == 0
    ndof = 3 * 17 ** 3
    assert big >= 8 * ndof + 5 * 4 * ndof + 17 ** 3
