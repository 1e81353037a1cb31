"""Compound states: named fields packed into one flat vector, and their sparsity.

Drop-in for ``tatva.compound`` (tatva/compound/__init__.py:73-470) on the host side
and ``tatva.sparse.pattern_from_compound`` (tatva/sparse/_extraction.py:117-245):

* ``class S(Compound, mesh=m): u = field((FieldSize.AUTO, 3)); p = field((5,))``
  declares fields; ``S.size`` is the flat length, ``S.fields`` the fields in
  declaration order.
* Layout: when two or more fields are full nodal fields (first dimension
  ``FieldSize.AUTO`` or ``field_type=Nodal()``, stackable), they share one block
  whose rows are nodes and whose columns are the fields' components side by side;
  that block comes first, the other fields follow in declaration order (a lone
  nodal field is laid out first on its own).  ``@stack_fields("a", "b")`` stacks the
  named fields the same way (along their last axis) starting at the first one's
  offset, and lays the later fields out again after the block.
* ``S.u[i, j]`` / ``S.u.indices(sl)`` give flat indices; ``state.u`` reads a field,
  ``state.at("u").set(x)`` returns an updated state, ``for f in state`` unpacks the
  fields, ``state + other`` adds the flat vectors.
* ``pattern_from_compound(S, block_wise=False)``: nodal fields couple all their dofs
  within each element of ``S``'s mesh; every other field only its diagonal.

Each field carries an explicit integer index map into the flat vector (host numpy),
so every view is one gather and every update one scatter on the flat tensor.
"""

from __future__ import annotations

import warnings
from dataclasses import dataclass
from enum import IntEnum
from math import prod
from typing import Callable

import numpy as np
import scipy.sparse as sps
import torch


class CompoundError(ValueError):
    """Inconsistent Compound declaration or use."""


class CompoundStackError(CompoundError):
    pass


class FieldSize(IntEnum):
    AUTO = -1


@dataclass
class Nodal:
    node_ids: np.ndarray | None = None
    stack: bool = True

    def get(self):
        return self


@dataclass
class Local:
    def get(self):
        return self


@dataclass
class Shared:
    def get(self):
        return self


class FieldType(IntEnum):
    LOCAL = 0
    NODAL = 1
    SHARED = 2

    def get(self):
        return {FieldType.LOCAL: Local, FieldType.NODAL: Nodal, FieldType.SHARED: Shared}[self]()


@dataclass(frozen=True)
class field:  # noqa: N801 - the reference's spelling
    """Field declaration: shape (first entry may be FieldSize.AUTO), optional default
    factory, field type (FieldType or Nodal/Local/Shared instance)."""

    shape: tuple
    default_factory: Callable | None = None
    field_type: object = FieldType.LOCAL


class Field:
    """A laid-out field: its shape and the flat index of each of its entries."""

    def __init__(self, name, shape, index, field_type, default_factory, root):
        self.name = name
        self.shape = tuple(int(s) for s in shape)
        self._index = np.asarray(index, dtype=np.int64).reshape(self.shape)
        self.field_type = field_type
        self.default_factory = default_factory
        self.root = root  # (start, stop) of the contiguous block holding the field

    def __getitem__(self, idx) -> np.ndarray:
        return self._index[idx]

    def indices(self, idx=slice(None)) -> np.ndarray:
        return np.asarray(self._index[idx]).reshape(-1)

    def _gather(self, arr: torch.Tensor) -> torch.Tensor:
        idx = torch.as_tensor(self._index.reshape(-1), device=arr.device)
        return arr[idx].reshape(self.shape)

    def _scatter(self, arr: torch.Tensor, value) -> torch.Tensor:
        idx = torch.as_tensor(self._index.reshape(-1), device=arr.device)
        v = torch.as_tensor(value, dtype=arr.dtype, device=arr.device)
        return arr.index_put((idx,), torch.broadcast_to(v, self.shape).reshape(-1))

    def __get__(self, instance, owner):
        if instance is None:
            return self
        return self._gather(instance.arr)

    def __repr__(self):
        return f"Field({self.name}, shape={self.shape})"


def _ftype(spec: field):
    ft = spec.field_type
    return ft.get() if hasattr(ft, "get") else ft


def _stacked(items, base, leading):
    """Index maps for fields stacked along their last axis: rows = leading entries,
    columns = the fields' last-axis components side by side."""
    widths = [1 if len(shape) == len(leading) else shape[-1] for _, shape in items]
    K = sum(widths)
    rows = np.arange(int(prod(leading)), dtype=np.int64).reshape(leading)[..., None] * K
    out, col = {}, 0
    for (name, shape), w in zip(items, widths):
        out[name] = (base + rows + col + np.arange(w)).reshape(shape)
        col += w
    return out, int(prod(leading)) * K


class Compound:
    fields: tuple = ()
    size: int = 0
    _mesh = None

    def __init_subclass__(cls, *, mesh=None, **kwargs):
        super().__init_subclass__(**kwargs)
        inherited = []
        for base in cls.__mro__[1:]:
            if issubclass(base, Compound) and base is not Compound:
                inherited = list(base.fields)
                break
        offset = sum(int(prod(f.shape)) for _, f in inherited)
        specs = [(k, v) for k, v in cls.__dict__.items() if isinstance(v, field)]
        reserved = set(dir(Compound)) | {"arr"}
        resolved = []
        for name, spec in specs:
            if name in reserved:
                raise CompoundError(f"Field name '{name}' is reserved and cannot be used in "
                                    "Compound class.")
            shape = tuple(spec.shape)
            ft = _ftype(spec)
            if shape and shape[0] == FieldSize.AUTO:
                if isinstance(ft, Nodal) and ft.node_ids is not None:
                    n = len(ft.node_ids)
                else:
                    if mesh is None:
                        raise CompoundError(
                            f"Mesh must be provided to resolve AUTO size for field '{name}'.")
                    n = int(mesh.coords.shape[0])
                shape = (n,) + shape[1:]
                if not isinstance(ft, Nodal):
                    ft = Nodal()
            resolved.append((name, shape, ft, spec.default_factory))
        stack = [r for r in resolved
                 if isinstance(r[2], Nodal) and r[2].node_ids is None and r[2].stack]
        laid = {}
        if len(stack) >= 2:
            n = stack[0][1][0]
            maps, total = _stacked([(r[0], r[1]) for r in stack], offset, (n,))
            for r in stack:
                laid[r[0]] = (maps[r[0]], (offset, offset + total))
            offset += total
            rest = [r for r in resolved if r[0] not in laid]
        else:
            rest = stack + [r for r in resolved if r not in stack]
        for name, shape, ft, df in rest:
            size = int(prod(shape))
            laid[name] = (offset + np.arange(size, dtype=np.int64).reshape(shape),
                          (offset, offset + size))
            offset += size
        new = []
        for name, shape, ft, df in resolved:
            f = Field(name, shape, laid[name][0], ft, df, laid[name][1])
            setattr(cls, name, f)
            new.append((name, f))
        cls.fields = tuple(inherited + new)
        cls.size = offset
        cls._mesh = mesh

    def __init__(self, arr=None, **kwargs):
        if arr is not None:
            arr = torch.as_tensor(arr)
            if arr.numel() != self.size:
                raise CompoundError(f"Array size {arr.numel()} does not match expected size "
                                    f"{self.size}.")
            self.arr = arr.reshape(-1)
        else:
            self.arr = torch.zeros(self.size, dtype=torch.float64)
            for name, f in self.fields:
                if name in kwargs:
                    self.arr = f._scatter(self.arr, kwargs[name])
                elif f.default_factory is not None:
                    self.arr = f._scatter(self.arr, f.default_factory())

    def __len__(self):
        return len(self.fields)

    def __iter__(self):
        for name, _ in self.fields:
            yield getattr(self, name)

    def __add__(self, other):
        return self.__class__(self.arr + other.arr)

    def __repr__(self):
        return f"{type(self).__name__}(" + ", ".join(
            f"{n}={f.shape}" for n, f in self.fields) + ")"

    def at(self, name: str):
        f = dict(self.fields).get(name)
        if f is None:
            raise AttributeError(f"Unknown field name: {name}")
        state = self

        class _At:
            def set(self, value):
                return state.__class__(f._scatter(state.arr, value))

        return _At()

    def flatten(self) -> torch.Tensor:
        return self.arr


class CompoundEnergy:
    """Energy of a Compound state as a sum over its fields, E(s) = sum_f E_f(s.f), each
    term one of the fused energies (``materials.Poisson / LinearElastic / NeoHookean``)
    on an Operator over the compound's mesh.

    The reference writes such energies as user JAX code over the fields of a state
    (tatva/compound/__init__.py:73-300) and differentiates them with jax.grad / jax.jvp /
    tatva.sparse.jacfwd on the pattern of ``pattern_from_compound``.  Here each field's
    values are gathered from the flat state on the device through the field's index map,
    the field's energy kernels compute its residual, HVP or compressed Hessian, and the
    result is scattered back to the field's flat indices.  Only full nodal fields (one
    row per mesh node, columns = the energy's components) can carry an energy; fields
    without one contribute nothing (their rows are zero)."""

    def __init__(self, compound_cls, **energies):
        self.compound_cls = compound_cls
        fields = dict(compound_cls.fields)
        self.terms = []
        for name, en in energies.items():
            if name not in fields:
                raise CompoundError(f"Unknown field name: {name}")
            f = fields[name]
            n_nodes = en.op.n_nodes
            if not (isinstance(f.field_type, Nodal) and f.field_type.node_ids is None
                    and f.shape[0] == n_nodes and int(prod(f.shape)) == en.n_dofs):
                raise CompoundError(
                    f"field '{name}' of shape {f.shape} is not a full nodal field with the "
                    f"{en.n_values} components per node of its energy")
            self.terms.append((name, f, en))
        self._idx: dict = {}

    @property
    def n_dofs(self) -> int:
        return self.compound_cls.size

    def _index(self, f, device) -> torch.Tensor:
        key = (f.name, str(device))
        if key not in self._idx:
            self._idx[key] = torch.as_tensor(f.indices(), device=device)
        return self._idx[key]

    def _flat(self, s):
        arr = s.arr if isinstance(s, Compound) else s
        if arr.numel() != self.n_dofs:
            raise CompoundError(f"Array size {arr.numel()} does not match expected size "
                                f"{self.n_dofs}.")
        return arr.reshape(-1)

    def _apply(self, method: str, s, v=None, fixed=None) -> torch.Tensor:
        u = self._flat(s)
        vv = self._flat(v) if v is not None else None
        ref = u if u is not None else vv
        out = torch.zeros(self.n_dofs, dtype=ref.dtype, device=ref.device)
        for _, f, en in self.terms:
            idx = self._index(f, ref.device)
            mask = fixed[idx].contiguous() if fixed is not None else None
            uf = u[idx].contiguous()
            if method == "residual":
                y = en.residual(uf, fixed=mask)
            elif method == "hvp":
                y = en.hvp(uf, vv[idx].contiguous(), fixed=mask)
            else:
                y = en.diagonal(uf, fixed=mask)
            out[idx] = y.reshape(-1)
        return out

    def residual(self, s, fixed=None) -> torch.Tensor:
        """dE/ds (jax.grad of the summed field energies), flat, in the compound layout."""
        return self._apply("residual", s, fixed=fixed)

    def hvp(self, s, v, fixed=None) -> torch.Tensor:
        """d2E/ds2 . v (jax.jvp(jax.grad(E))), flat, in the compound layout."""
        return self._apply("hvp", s, v, fixed=fixed)

    def diagonal(self, s, fixed=None) -> torch.Tensor:
        return self._apply("diagonal", s, fixed=fixed)

    def value(self, s) -> torch.Tensor:
        u = self._flat(s)
        return sum(en.value(u[self._index(f, u.device)].contiguous()) for _, f, en in self.terms)

    __call__ = value

    def compressed_hessian(self, s, colors: torch.Tensor, n_colors: int,
                           dtype=None) -> torch.Tensor:
        """Jc (size, n_colors) on a distance-2 colouring of the compound pattern: each
        field's rows from its energy's compressed Hessian with the colours of its own
        columns (the energy couples no two fields, so the other columns add nothing)."""
        u = self._flat(s)
        dtype = dtype or u.dtype
        Jc = torch.zeros((self.n_dofs, n_colors), dtype=dtype, device=u.device)
        for _, f, en in self.terms:
            idx = self._index(f, u.device)
            Jc[idx] = en.compressed_hessian(u[idx].contiguous(), colors[idx].contiguous(),
                                            n_colors, dtype=dtype)
        return Jc


def stack_fields(*names: str, axis: int = -1):
    """Class decorator: lay the named fields out as one block stacked along their last
    axis, starting where the first of them started; later fields follow the block."""
    if not names:
        raise CompoundError("At least one field name is required.")
    if axis != -1:
        raise CompoundStackError("only axis=-1 stacking is supported")

    def deco(cls):
        fmap = dict(cls.fields)
        for n in names:
            if n not in fmap:
                raise CompoundStackError(f"Unknown field name in stack_fields: {n}")
        lead = {fmap[n].shape[:-1] if len(fmap[n].shape) > 1 else fmap[n].shape for n in names}
        if len(lead) != 1:
            raise CompoundStackError("stacked fields must share their leading dimensions")
        leading = lead.pop()
        first = min(i for i, (n, _) in enumerate(cls.fields) if n in names)
        base = int(cls.fields[first][1]._index.min()) if cls.fields[first][1]._index.size else 0
        maps, total = _stacked([(n, fmap[n].shape) for n in names], base, leading)
        offset = base + total
        new = []
        for i, (n, f) in enumerate(cls.fields):
            if i >= first:
                if n in maps:
                    f = Field(n, f.shape, maps[n], f.field_type, f.default_factory,
                              (base, base + total))
                else:
                    size = int(prod(f.shape))
                    f = Field(n, f.shape, offset + np.arange(size), f.field_type,
                              f.default_factory, (offset, offset + size))
                    offset += size
                setattr(cls, n, f)
            new.append((n, f))
        cls.fields = tuple(new)
        cls.size = offset
        return cls

    return deco


def pattern_from_compound(compound_cls, block_wise: bool = False):
    """Sparsity of a Compound state on its mesh: the dofs of all nodal fields are
    coupled within each element; other fields get their diagonal only (with a
    warning).  ``block_wise``: the pattern cut into the fields' blocks (a stacked
    block is one block) as a list of lists."""
    mesh = compound_cls._mesh
    if mesh is None:
        raise CompoundError("Mesh must be set on Compound class to create sparsity pattern.")
    n_nodes = int(mesh.coords.shape[0])
    el = np.asarray(mesh.elements_host(), dtype=np.int64)
    coupled, diag = [], []
    for name, f in compound_cls.fields:
        ft = f.field_type
        if isinstance(ft, Nodal):
            idx = f.indices()
            n_items = len(ft.node_ids) if ft.node_ids is not None else n_nodes
            if n_items == 0:
                continue
            per = idx.size // n_items
            node_dofs = np.full((n_nodes, per), -1, dtype=np.int64)
            if ft.node_ids is None:
                node_dofs[:] = idx.reshape(n_nodes, per)
            else:
                ids = np.asarray(ft.node_ids, dtype=np.int64)
                ok = (ids >= 0) & (ids < n_nodes)
                node_dofs[ids[ok]] = idx.reshape(-1, per)[ok]
            coupled.append(node_dofs[el].reshape(el.shape[0], -1))
        else:
            warnings.warn(f"Custom space detected for field '{name}'. Only diagonal entries "
                          "added to the sparsity pattern. Please provide your own sparsity "
                          "pattern if cross-coupling is required.", UserWarning)
            diag.append(f.indices())
    n = compound_cls.size
    keys = []
    if coupled:
        ed = np.concatenate(coupled, axis=1)
        m = ed.shape[1]
        r = np.repeat(ed, m, axis=1).ravel()
        c = np.tile(ed, (1, m)).ravel()
        ok = (r >= 0) & (c >= 0)
        keys.append(r[ok] * n + c[ok])
    if diag:
        d = np.concatenate(diag)
        keys.append(d * n + d)
    if keys:
        u = np.unique(np.concatenate(keys))
        full = sps.csr_matrix((np.ones(u.size, dtype=np.int8), (u // n, u % n)), shape=(n, n))
    else:
        full = sps.csr_matrix((n, n), dtype=np.int8)
    if not block_wise:
        return full
    roots = sorted({f.root for _, f in compound_cls.fields})
    return [[full[a0:a1, b0:b1] for (b0, b1) in roots] for (a0, a1) in roots]


__all__ = ["Compound", "CompoundEnergy", "CompoundError", "CompoundStackError", "Field", "FieldSize",
           "FieldType",
           "Local", "Nodal", "Shared", "field", "pattern_from_compound", "stack_fields"]
