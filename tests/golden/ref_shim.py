"""A minimal stand-in for ``jax``/``jax.numpy``/``lineax`` built on ``torch.func``.

Purpose: JAX is not installable in the environment that generates the golden
fixtures, so the reference package (``updes``) is imported *unmodified* from its
source tree with these modules placed in ``sys.modules`` first.  Every
operation the reference's solve path uses is mapped onto float64 torch:

* ``jax.vmap`` / ``jax.grad`` / ``jax.jacfwd``  -> ``torch.func`` equivalents
  (automatic differentiation, not closed forms, exactly like the reference);
* ``x.at[idx].set(v)``                           -> functional index_put on a clone;
* ``jax.lax.fori_loop``                          -> a Python loop;
* ``jnp.linalg.inv``                             -> ``torch.linalg.inv`` (LAPACK getrf/getri);
* ``lineax.linear_solve(..., lx.QR())``          -> Householder QR + triangular solve.

The shim is test infrastructure for ``tests/golden/make_golden.py`` only.
Nothing in the product imports it.
"""
from __future__ import annotations

import functools
import sys
import types
import warnings

import numpy as np
import torch

warnings.filterwarnings("ignore")
torch.set_default_dtype(torch.float64)


def _dt(dtype):
    if dtype is None:
        return None
    if dtype is int:
        return torch.int64
    if dtype is float:
        return torch.float64
    if dtype is bool:
        return torch.bool
    if isinstance(dtype, torch.dtype):
        return dtype
    return torch.float64


def _t(x, dtype=None):
    """Convert anything array-like into a torch tensor (float64 / int64)."""
    if isinstance(x, torch.Tensor):
        return x if dtype is None else x.to(_dt(dtype))
    if isinstance(x, (list, tuple)):
        if len(x) and any(isinstance(e, (torch.Tensor, list, tuple, np.ndarray)) for e in x):
            out = torch.stack([_t(e) for e in x])
            return out if dtype is None else out.to(_dt(dtype))
        return torch.tensor(x, dtype=_dt(dtype))
    if isinstance(x, np.ndarray):
        out = torch.from_numpy(np.ascontiguousarray(x))
        return out if dtype is None else out.to(_dt(dtype))
    return torch.tensor(x, dtype=_dt(dtype))


class _AtIndex:
    def __init__(self, arr, idx):
        self.arr, self.idx = arr, idx

    def _index(self):
        idx = self.idx if isinstance(self.idx, tuple) else (self.idx,)
        return tuple(_t(i) if isinstance(i, (list, np.ndarray)) else i for i in idx)

    def set(self, v):
        out = self.arr.clone()
        v = _t(v)
        out[self._index()] = v.to(out.dtype)
        return out

    def add(self, v):
        idx = self._index()
        if all(isinstance(i, slice) and i == slice(None) for i in idx):
            # the whole array: out of place, so that a batched value under vmap broadcasts into the result
            return self.arr + _t(v).to(self.arr.dtype)
        out = self.arr.clone()
        out[idx] += _t(v).to(out.dtype)
        return out

    def get(self):
        return self.arr[self._index()]


class _At:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _AtIndex(self.arr, idx)


torch.Tensor.at = property(lambda self: _At(self))


def _wrap1(fn):
    return lambda x, *a, **k: fn(_t(x), *a, **k)


def _batched_out(fn, args, in_axes):
    """Make non-tensor outputs tensors (vmap needs tensors)."""
    out = fn(*args)
    if not isinstance(out, torch.Tensor):
        out = torch.as_tensor(out, dtype=torch.float64)
    return out


def vmap(fn, in_axes=0, out_axes=0):
    def wrapped(*args):
        n = len(args)
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * n
        args = tuple(_t(a) if (ax is not None and not isinstance(a, torch.Tensor)) else a
                     for a, ax in zip(args, axes))
        return torch.func.vmap(lambda *a: _batched_out(fn, a, axes),
                               in_dims=tuple(axes), out_dims=out_axes)(*args)
    return wrapped


def grad(fn, argnums=0):
    assert argnums == 0

    def inner(x, *a, **k):
        out = fn(x, *a, **k)
        if not isinstance(out, torch.Tensor):
            out = torch.as_tensor(out, dtype=x.dtype)
        return out + 0.0 * x.sum()

    def g(x, *a, **k):
        return torch.func.grad(lambda x_: inner(x_, *a, **k))(_t(x))
    return g


def jacfwd(fn, argnums=0):
    assert argnums == 0

    def j(x, *a, **k):
        return torch.func.jacfwd(lambda x_: fn(x_, *a, **k))(_t(x))
    return j


def jit(fn=None, static_argnums=None, static_argnames=None, **kw):
    if fn is None:
        return lambda f: f
    return fn


def fori_loop(lo, hi, body, init):
    val = init
    for i in range(int(lo), int(hi)):
        val = body(i, val)
    return val


def tree_map(f, tree):
    if isinstance(tree, dict):
        return {k: tree_map(f, v) for k, v in tree.items()}
    if isinstance(tree, list):
        return [tree_map(f, v) for v in tree]
    if isinstance(tree, tuple):
        return tuple(tree_map(f, v) for v in tree)
    return f(tree)


def _random_unavailable(*a, **k):
    raise RuntimeError("jax.random is not provided by the shim: inject node coordinates instead")


def _make_jnp():
    jnp = types.ModuleType("jax.numpy")
    jnp.zeros = lambda shape, dtype=None: torch.zeros(shape, dtype=_dt(dtype) or torch.float64)
    jnp.ones = lambda shape, dtype=None: torch.ones(shape, dtype=_dt(dtype) or torch.float64)
    jnp.array = lambda x, dtype=None: _t(x, dtype)
    jnp.asarray = jnp.array
    jnp.stack = lambda seq, axis=0: torch.stack([_t(e) for e in seq], dim=axis)
    jnp.concatenate = lambda seq, axis=0: torch.cat([_t(e) for e in seq], dim=axis)
    for name in ("sqrt", "exp", "log", "sin", "cos", "tan", "sinh", "cosh", "tanh", "abs",
                 "isnan", "isinf", "floor"):
        setattr(jnp, name, _wrap1(getattr(torch, name)))
    jnp.nan_to_num = lambda x, nan=0.0, posinf=None, neginf=None: torch.nan_to_num(
        _t(x), nan=nan, posinf=posinf, neginf=neginf)
    jnp.trace = lambda x: torch.trace(_t(x))
    jnp.dot = lambda a, b: torch.dot(_t(a), _t(b)) if (_t(a).dim() == 1 and _t(b).dim() == 1) \
        else torch.matmul(_t(a), _t(b))
    jnp.matmul = lambda a, b: torch.matmul(_t(a), _t(b))
    jnp.arange = lambda *a, dtype=None: torch.arange(*a, dtype=_dt(dtype))
    jnp.linspace = lambda a, b, n: torch.linspace(float(a), float(b), int(n), dtype=torch.float64)
    jnp.meshgrid = lambda *xs, indexing="xy": torch.meshgrid(*[_t(x) for x in xs], indexing=indexing)
    jnp.newaxis = None
    jnp.flip = lambda x, axis=None: torch.flip(_t(x), dims=(axis,) if axis is not None else tuple(range(_t(x).dim())))
    jnp.set_printoptions = lambda *a, **k: None
    jnp.inf = float("inf")
    jnp.pi = float(np.pi)
    jnp.sum = lambda x, axis=None: torch.sum(_t(x)) if axis is None else torch.sum(_t(x), dim=axis)
    jnp.mean = lambda x, axis=None: torch.mean(_t(x)) if axis is None else torch.mean(_t(x), dim=axis)
    jnp.clip = lambda x, lo, hi: torch.clamp(_t(x), lo, hi)
    jnp.where = lambda c, a, b: torch.where(_t(c), _t(a), _t(b))
    jnp.ndarray = torch.Tensor
    jnp.float64 = torch.float64
    jnp.int32 = torch.int32
    linalg = types.ModuleType("jax.numpy.linalg")
    linalg.inv = lambda a: torch.linalg.inv(_t(a))
    linalg.norm = lambda a, *x, **k: torch.linalg.norm(_t(a), *x, **k)
    linalg.solve = lambda a, b: torch.linalg.solve(_t(a), _t(b))
    jnp.linalg = linalg
    return jnp, linalg


def _make_lineax():
    lx = types.ModuleType("lineax")

    class MatrixLinearOperator:
        def __init__(self, matrix):
            self.matrix = _t(matrix)

    class QR:
        pass

    class _Solution:
        def __init__(self, value):
            self.value = value

    def linear_solve(operator, vector, solver=None):
        assert isinstance(solver, QR), "only the QR solver is provided by the shim"
        q, r = torch.linalg.qr(operator.matrix, mode="reduced")
        y = q.T @ _t(vector)
        x = torch.linalg.solve_triangular(r, y[:, None], upper=True)[:, 0]
        return _Solution(x)

    lx.MatrixLinearOperator = MatrixLinearOperator
    lx.QR = QR
    lx.linear_solve = linear_solve
    return lx


class _Anything(types.ModuleType):
    """A module whose every attribute is a no-op callable (plotting stubs)."""

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Anything(name)

    def __call__(self, *a, **k):
        return _Anything("call")


def install():
    """Place the shim modules in ``sys.modules`` (idempotent)."""
    if "jax" in sys.modules and getattr(sys.modules["jax"], "_is_shim", False):
        return
    jax = types.ModuleType("jax")
    jax._is_shim = True
    jnp, linalg = _make_jnp()
    jax.numpy = jnp
    jax.vmap, jax.grad, jax.jacfwd, jax.jit = vmap, grad, jacfwd, jit
    lax = types.ModuleType("jax.lax")
    lax.fori_loop = fori_loop
    jax.lax = lax
    tu = types.ModuleType("jax.tree_util")
    tu.Partial = functools.partial
    tu.tree_map = tree_map
    jax.tree_util = tu
    cfg = types.SimpleNamespace(update=lambda *a, **k: None)
    jax.config = cfg
    rnd = types.ModuleType("jax.random")
    rnd.PRNGKey = rnd.split = rnd.uniform = rnd.permutation = _random_unavailable
    jax.random = rnd
    sys.modules.update({
        "jax": jax, "jax.numpy": jnp, "jax.numpy.linalg": linalg, "jax.lax": lax,
        "jax.tree_util": tu, "jax.random": rnd, "lineax": _make_lineax(),
    })
    for stub in ("matplotlib", "matplotlib.pyplot", "matplotlib.animation", "seaborn",
                 "pyvista", "mpl_toolkits", "mpl_toolkits.mplot3d"):
        sys.modules.setdefault(stub, _Anything(stub))
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
