"""Generate golden fixtures by executing the reference tatva's own Python code.

Run from the repository root, in a container that has the reference tree:

    python tests/golden/make_golden.py /path/to/reference
    python tests/golden/make_golden.py /path/to/reference compound   # compound_golden.npz

JAX is not installed where this runs, so a minimal numpy stand-in for the
handful of ``jax`` entry points the reference modules touch at import time
(``jax.numpy`` -> numpy, ``jax.vmap`` / ``jax.lax.map`` -> Python loops,
``jax.jit`` / ``register_dataclass`` -> identity) is installed in
``sys.modules`` before ``tatva`` is imported.  The arithmetic that produces the
fixtures is therefore the reference's own code paths (element shape functions,
``Operator.eval/grad/get_integration_weights/integrate_per_element``,
``Mesh.unit_square``, ``_create_sparse_structure``, ``_coloring.distance2_colors``,
``compute_rows_cols``) evaluated in numpy FP64.

Derivatives, which the reference takes with ``jax.grad`` / ``jax.jvp``, are
produced here by complex-step differentiation of the reference-computed element
energies (exact to rounding: no subtractive cancellation).  Second derivatives
of the non-quadratic Neo-Hookean energy are a Richardson-extrapolated central
difference of complex-step gradients (accurate to ~1e-10, stated in the test).

Output: ``tests/golden/*.npz`` (small; committed).  Nothing at run time reads
the reference tree.
"""

from __future__ import annotations

import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


# ---------------------------------------------------------------------------
# numpy stand-in for the jax entry points used at import / call time
# ---------------------------------------------------------------------------


def _install_jax_standin():
    jax = types.ModuleType("jax")
    jnp = types.ModuleType("jax.numpy")

    def _jnp_getattr(name):
        return getattr(np, name)

    jnp.__getattr__ = _jnp_getattr  # type: ignore[attr-defined]

    def repeat(a, repeats, axis=None, total_repeat_length=None):
        return np.repeat(a, repeats, axis=axis)

    jnp.repeat = repeat
    jnp.linalg = np.linalg

    def vmap(f, in_axes=0, out_axes=0):
        def wrapped(*args):
            n = len(args[0])
            outs = [f(*[a[i] for a in args]) for i in range(n)]
            if isinstance(outs[0], tuple):
                return tuple(np.stack([o[k] for o in outs]) for k in range(len(outs[0])))
            return np.stack([np.asarray(o) for o in outs])

        return wrapped

    lax = types.ModuleType("jax.lax")

    def lax_map(f, xs, batch_size=None):
        if isinstance(xs, tuple):
            n = len(xs[0])
            outs = [f(tuple(x[i] for x in xs)) for i in range(n)]
        else:
            n = len(xs)
            outs = [f(xs[i]) for i in range(n)]
        if isinstance(outs[0], tuple):
            return tuple(np.stack([o[k] for o in outs]) for k in range(len(outs[0])))
        return np.stack([np.asarray(o) for o in outs])

    lax.map = lax_map

    def jit(f=None, **kw):
        if f is None:
            return lambda g: g
        return f

    tree_util = types.ModuleType("jax.tree_util")
    tree_util.register_dataclass = lambda cls=None, **kw: (cls if cls is not None else (lambda c: c))
    tree_util.register_pytree_node_class = lambda cls: cls
    tree_util.tree_map = lambda f, *t: f(*t)

    errors = types.ModuleType("jax.errors")

    class TracerBoolConversionError(Exception):
        pass

    errors.TracerBoolConversionError = TracerBoolConversionError

    jtyping = types.ModuleType("jax.typing")
    jtyping.ArrayLike = object

    config = types.SimpleNamespace(update=lambda *a, **k: None)

    experimental = types.ModuleType("jax.experimental")
    jsparse = types.ModuleType("jax.experimental.sparse")
    jsparse.BCOO = object
    jsparse.BCSR = object
    experimental.sparse = jsparse

    jax.numpy = jnp
    jax.lax = lax
    jax.vmap = vmap
    jax.jit = jit
    jax.tree_util = tree_util
    jax.errors = errors
    jax.typing = jtyping
    jax.config = config
    jax.Array = np.ndarray
    jax.experimental = experimental

    autovmap_mod = types.ModuleType("jax_autovmap")
    autovmap_mod.autovmap = lambda *a, **k: (lambda f: f)

    sys.modules.update(
        {
            "jax": jax,
            "jax.numpy": jnp,
            "jax.lax": lax,
            "jax.tree_util": tree_util,
            "jax.errors": errors,
            "jax.typing": jtyping,
            "jax.experimental": experimental,
            "jax.experimental.sparse": jsparse,
            "jax_autovmap": autovmap_mod,
        }
    )


def _load_file(modname, path):
    spec = importlib.util.spec_from_file_location(modname, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[modname] = mod
    spec.loader.exec_module(mod)
    return mod


def load_reference(ref_root):
    sys.dont_write_bytecode = True
    _install_jax_standin()
    sys.path.insert(0, ref_root)
    import tatva  # noqa: F401  (element, mesh, operator)
    from tatva import element as el
    from tatva.mesh import Mesh
    from tatva.operator import Operator

    # sparse submodules without the package __init__ (which pulls in the jaxpr tracer)
    sp_dir = os.path.join(ref_root, "tatva", "sparse")
    pkg = types.ModuleType("tatva.sparse")
    pkg.__path__ = [sp_dir]
    sys.modules["tatva.sparse"] = pkg
    coloring = _load_file("tatva.sparse._coloring", os.path.join(sp_dir, "_coloring.py"))
    tc = types.ModuleType("tatva_coloring")
    tc.distance2_colors = coloring.distance2_colors
    sys.modules["tatva_coloring"] = tc
    extraction = _load_file("tatva.sparse._extraction", os.path.join(sp_dir, "_extraction.py"))
    sbase = _load_file("tatva.sparse.base", os.path.join(sp_dir, "base.py"))
    return types.SimpleNamespace(
        el=el, Mesh=Mesh, Operator=Operator, coloring=coloring,
        extraction=extraction, sbase=sbase,
    )


# ---------------------------------------------------------------------------
# energy densities (numpy restatements of the test materials; complex-safe)
# ---------------------------------------------------------------------------


def dens_poisson(kappa, f):
    def psi(H, uq):
        return 0.5 * kappa * np.sum(H * H, axis=-1) - f * uq

    return psi


def dens_linear_elastic(mu, lmbda):
    def psi(H):
        eps = 0.5 * (H + np.swapaxes(H, -1, -2))
        tr = np.trace(eps, axis1=-2, axis2=-1)
        sig = 2 * mu * eps + lmbda * tr[..., None, None] * np.eye(H.shape[-1])
        return 0.5 * np.einsum("...ij,...ij->...", sig, eps)

    return psi


def dens_neo_hookean(mu, lmbda):
    def psi(H):
        F = np.eye(3) + H
        J = np.linalg.det(F)
        C = np.swapaxes(F, -1, -2) @ F
        I1 = np.trace(C, axis1=-2, axis2=-1)
        return (mu / 2) * (I1 - 3 - 2 * np.log(J)) + (lmbda / 2) * np.log(J) ** 2

    return psi


def element_energy(ref, op, law, kind, u_flat, nv):
    """Per-element energies through the reference Operator."""
    u = u_flat.reshape(-1, nv) if nv > 1 else u_flat
    if kind == "poisson":
        H = op.grad(u)
        uq = op.eval(u)
        return op.integrate_per_element(law(H, uq))
    return op.integrate_per_element(law(op.grad(u)))


def cs_gradient(ref, op, law, kind, u, nv, colors, elements):
    """Complex-step gradient of the reference energy, colour by colour."""
    h = 1e-30
    n = u.shape[0]
    g = np.zeros(n)
    dofs = (elements[:, :, None] * nv + np.arange(nv)).reshape(elements.shape[0], -1)
    for c in range(int(colors.max()) + 1):
        seed = (colors == c).astype(np.float64)
        Ee = element_energy(ref, op, law, kind, u + 1j * h * seed, nv)
        d = np.imag(Ee) / h  # per-element derivative along the seed
        # each element holds at most one dof of colour c: give it the value
        for e in range(elements.shape[0]):
            sel = dofs[e][colors[dofs[e]] == c]
            if sel.size:
                assert sel.size == 1
                g[sel[0]] += d[e]
    return g


def make(ref_root):
    ref = load_reference(ref_root)
    el, Mesh, Operator = ref.el, ref.Mesh, ref.Operator
    out = {}
    rng = np.random.default_rng(1234)

    # ---- element tables + exact-gradient checks (tests/test_element.py:45-149)
    for name, cls in (("tri3", el.Tri3), ("tet4", el.Tetrahedron4), ("hex8", el.Hexahedron8)):
        e = cls()
        qp, qw = np.asarray(e.quad_points), np.asarray(e.quad_weights)
        out[f"{name}_qp"] = qp
        out[f"{name}_qw"] = qw
        out[f"{name}_N"] = np.stack([np.asarray(e.shape_function(x)) for x in qp])
        out[f"{name}_dN"] = np.stack([np.asarray(e.shape_function_derivative(x)) for x in qp])
        X = np.asarray(e._reference_nodes()) * 0.9 + 0.05 * rng.standard_normal(
            np.asarray(e._reference_nodes()).shape)
        U = rng.standard_normal((X.shape[0], 3))
        out[f"{name}_el_X"] = X
        out[f"{name}_el_U"] = U
        out[f"{name}_el_grad"] = np.stack([np.asarray(e.gradient(x, U, X)) for x in qp])
        out[f"{name}_el_interp"] = np.stack([np.asarray(e.interpolate(x, U, X)) for x in qp])
        out[f"{name}_el_detJ"] = np.stack([np.asarray(e.get_jacobian(x, X)[1]) for x in qp])

    # ---- reference mesh generator (mesh.py:146-205)
    for nx, ny in ((3, 2), (8, 8)):
        m = Mesh.unit_square(nx, ny)
        out[f"usq_{nx}x{ny}_coords"] = np.asarray(m.coords)
        out[f"usq_{nx}x{ny}_elements"] = np.asarray(m.elements)

    # ---- meshes for operator / pattern / colouring fixtures
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle import mesh as om

    meshes = {}
    m = Mesh.unit_square(4, 3)
    meshes["tri"] = (np.asarray(m.coords), np.asarray(m.elements), el.Tri3())
    c, e_ = om.kuhn_box((1.0, 1.0, 1.0), (2, 2, 2))
    c = om.jitter_interior(c, 0.5, 0.2, seed=7)
    meshes["tet"] = (c, e_, el.Tetrahedron4())
    c, e_ = om.brick(2, 2, 2)
    c = om.jitter_interior(c, 0.5, 0.2, seed=11)
    meshes["hexj"] = (c, e_, el.Hexahedron8())
    c, e_ = om.brick(3, 2, 2, lengths=(1.5, 1.0, 0.8))
    meshes["hexa"] = (c, e_, el.Hexahedron8())

    for key, (coords, elements, elem) in meshes.items():
        mesh = Mesh(coords=coords, elements=elements)
        op = Operator(mesh, elem)
        n = coords.shape[0]
        us = rng.standard_normal(n)
        uv = rng.standard_normal((n, coords.shape[1]))
        out[f"{key}_coords"] = coords
        out[f"{key}_elements"] = elements
        out[f"{key}_us"] = us
        out[f"{key}_uv"] = uv
        out[f"{key}_eval_s"] = np.asarray(op.eval(us))
        out[f"{key}_eval_v"] = np.asarray(op.eval(uv))
        out[f"{key}_grad_s"] = np.asarray(op.grad(us))
        out[f"{key}_grad_v"] = np.asarray(op.grad(uv))
        out[f"{key}_weights"] = np.asarray(op.get_integration_weights())
        out[f"{key}_int_pe_s"] = np.asarray(op.integrate_per_element(us))
        out[f"{key}_int_pe_v"] = np.asarray(op.integrate_per_element(uv))

        for ndpn in (1, 2, 3) if coords.shape[1] == 3 else (1, 2):
            shp = (n * ndpn, n * ndpn)
            csr = ref.extraction._create_sparse_structure(elements, ndpn, shp)
            colors = np.asarray(ref.coloring.distance2_colors(csr.indptr, csr.indices, shp[0]))
            cm = ref.sbase.ColoredMatrix.from_csr(csr, colors=colors)
            rows, col_colors = ref.sbase.compute_rows_cols(cm)
            out[f"{key}_pat{ndpn}_indptr"] = np.asarray(csr.indptr)
            out[f"{key}_pat{ndpn}_indices"] = np.asarray(csr.indices)
            out[f"{key}_pat{ndpn}_colors"] = colors.astype(np.int32)
            out[f"{key}_pat{ndpn}_rows"] = np.asarray(rows)
            out[f"{key}_pat{ndpn}_colcolors"] = np.asarray(col_colors)

        # ---- energies and complex-step residuals through the reference Operator
        dim = coords.shape[1]
        cases = [("poisson", dens_poisson(1.7, 0.9), 1)]
        cases.append(("linear_elastic", dens_linear_elastic(0.8, 1.3), dim))
        if dim == 3:
            cases.append(("neo_hookean", dens_neo_hookean(1.0, 10.0), 3))
        for kind, law, nv in cases:
            colors = out[f"{key}_pat{nv}_colors"]
            u = 0.05 * rng.standard_normal(n * nv)
            Ee = element_energy(ref, op, law, kind, u, nv)
            g = cs_gradient(ref, op, law, kind, u, nv, colors, elements)
            out[f"{key}_{kind}_u"] = u
            out[f"{key}_{kind}_energy_pe"] = np.real(np.asarray(Ee))
            out[f"{key}_{kind}_residual"] = g
            v = rng.standard_normal(n * nv)
            out[f"{key}_{kind}_v"] = v
            if kind == "neo_hookean":
                # Richardson-extrapolated central difference of complex-step gradients
                def gdir(t):
                    return cs_gradient(ref, op, law, kind, u + t * v, nv, colors, elements)

                d = 1e-4
                D1 = (gdir(d) - gdir(-d)) / (2 * d)
                D2 = (gdir(2 * d) - gdir(-2 * d)) / (4 * d)
                out[f"{key}_{kind}_hvp"] = (4 * D1 - D2) / 3
            else:
                # quadratic energy: HVP = grad E(v) with the linear (source) part removed
                g0 = cs_gradient(ref, op, law, kind, np.zeros_like(u), nv, colors, elements)
                out[f"{key}_{kind}_hvp"] = (
                    cs_gradient(ref, op, law, kind, v, nv, colors, elements) - g0)

    # ---- test_sparse.py:48-80 fixture: Tri3 8x8, 2-dof elasticity mu=1, lambda=0
    m = Mesh.unit_square(8, 8)
    op = Operator(m, el.Tri3())
    coords, elements = np.asarray(m.coords), np.asarray(m.elements)
    n2 = coords.shape[0] * 2
    csr = ref.extraction._create_sparse_structure(elements, 2, (n2, n2))
    colors = np.asarray(ref.coloring.distance2_colors(csr.indptr, csr.indices, n2))
    law = dens_linear_elastic(1.0, 0.0)
    K = np.zeros((n2, n2))
    for j in range(n2):
        ej = np.zeros(n2)
        ej[j] = 1.0
        K[:, j] = cs_gradient(ref, op, law, "le", ej, 2, colors, elements)
    out["sq8_pat2_indptr"] = np.asarray(csr.indptr)
    out["sq8_pat2_indices"] = np.asarray(csr.indices)
    out["sq8_pat2_colors"] = colors.astype(np.int32)
    out["sq8_le_dense_K"] = K

    np.savez_compressed(os.path.join(HERE, "reference_golden.npz"), **out)
    print(f"wrote {len(out)} arrays to {os.path.join(HERE, 'reference_golden.npz')}")


def make_compound(ref_root):
    """Compound layouts and pattern_from_compound of the reference
    (tatva/compound/__init__.py, tatva/sparse/_extraction.py:117-245) for three states on
    small meshes; written to tests/golden/compound_golden.npz."""
    ref = load_reference(ref_root)
    import warnings

    from tatva import compound as C

    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle import mesh as om

    out = {}
    ct, et = om.kuhn_box((1, 1, 1), (2, 2, 1), origin=(0, 0, 0))
    mt = ref.Mesh(ct, et)
    cq, eq = om.unit_square(3, 2)
    mq = ref.Mesh(cq, eq)

    class TwoNodal(C.Compound, mesh=mt):
        u = C.field((C.FieldSize.AUTO, 3))
        theta = C.field((C.FieldSize.AUTO,))

    class NodalAndLocal(C.Compound, mesh=mt):
        u = C.field((C.FieldSize.AUTO, 3))
        p = C.field((5,))

    class PartialNodal(C.Compound, mesh=mq):
        u = C.field((C.FieldSize.AUTO, 2))
        lam = C.field((4,), field_type=C.field_types.Nodal(node_ids=np.array([0, 3, 5, 11])))

    for name, cls in (("two_nodal", TwoNodal), ("nodal_local", NodalAndLocal),
                      ("partial_nodal", PartialNodal)):
        out[f"{name}_size"] = np.array(cls.size)
        for fname, f in cls.fields:
            out[f"{name}_field_{fname}"] = np.asarray(f.indices(slice(None))).reshape(-1)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            pat = ref.extraction.pattern_from_compound(cls)
            blocks = ref.extraction.pattern_from_compound(cls, block_wise=True)
        out[f"{name}_indptr"] = pat.indptr.astype(np.int64)
        out[f"{name}_indices"] = pat.indices.astype(np.int64)
        out[f"{name}_block_shapes"] = np.array([[b.shape[0], b.shape[1], b.nnz]
                                                for row in blocks for b in row])
    np.savez_compressed(os.path.join(HERE, "compound_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "compound_golden.npz"), len(out), "arrays")


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[2] == "compound":
        make_compound(sys.argv[1])
        sys.exit(0)
    make(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
