"""CPU oracle for the tatva FEM hot path -- TEST INFRASTRUCTURE ONLY.

This package is a plain numpy/scipy FP64 restatement of the reference
(smec-ethz/tatva 0.11.1) algorithms on the hot path.  It exists to check the
CUDA implementation in ``tatva_gb300``; it is never the thing measured and
never a fallback.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it.

Pinning: the restatement is checked against golden fixtures in
``tests/golden/`` that were produced by executing the reference's own Python
modules (``tatva/element/base.py``, ``tatva/operator.py``, ``tatva/mesh.py``,
``tatva/sparse/_extraction.py``, ``tatva/sparse/_coloring.py``,
``tatva/sparse/base.py``) with numpy standing in for ``jax.numpy``
(``tests/golden/make_golden.py``), and against the known answers of the
reference's tests (``tests/test_operator.py``, ``tests/test_element.py``,
``tests/test_sparse.py``).  Derivatives (residual, HVP, Hessian) are pinned by
complex-step differentiation of the reference-computed energy.

Modules:
  elements  -- Tri3 / Tetrahedron4 / Hexahedron8 shape functions + quadrature
  mesh      -- structured mesh generators (Tri3 square, Kuhn Tet4 box, Hex8 brick)
  operator  -- eval / grad / integration weights / integrate / map
  materials -- Poisson, linear elastic, Neo-Hookean: energy, residual, HVP, tangent
  sparse    -- sparsity pattern, distance-2 greedy colouring, rows/cols,
               compressed Jacobian, decompression
  lifter    -- Dirichlet (Fixed) lift / reduce / reduce_adjoint
  solvers   -- Jacobi-preconditioned CG in FP64
"""
