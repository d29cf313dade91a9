"""NumPy stand-in for the part of the JAX API that GO-MELT's reference code uses.

TEST INFRASTRUCTURE ONLY.  This module exists so that the unmodified reference
sources (``go_melt/computeFunctions.py`` and ``go_melt/go_melt.py`` of
JLnorthwestern/GO-MELT) can be imported and executed on a machine without JAX,
to produce golden input/output vectors.  Nothing in the product imports it.

The reference pins ``jax[cuda12_pip]==0.4.16`` (``requirements.txt:2-3``),
which is not installed here.  The reference uses JAX only for array
primitives whose semantics are public and simple:

* ``jax.numpy`` array functions  -> the same-named NumPy functions, in FP64
  (this is the behaviour of JAX with ``jax_enable_x64`` switched on, i.e.
  "an FP64 run of the reference");
* immutable ``x.at[i].set(v)`` / ``.add(v)`` updates -> copy, then NumPy
  assignment / ``np.add.at``;
* ``jax.jit`` -> identity (tracing changes nothing observable for pure code);
* ``jax.vmap(f)(xs)`` -> ``f`` applied to each leading-axis slice, outputs
  stacked leaf by leaf;
* ``jax.lax.scan(f, init, xs)`` -> the documented Python loop
  (carry, y) = f(carry, x), with the ``y`` leaves stacked;
* ``jax.lax.select(p, a, b)`` -> ``np.where``;
* ``jax.experimental.sparse.BCOO((data, idx), shape) @ v`` -> a scatter-add of
  ``data * v[idx[:, 1]]`` into ``idx[:, 0]``.

``dill`` is replaced by ``pickle`` and ``pyevtk.hl.gridToVTK`` by a function
that records its call (file output is not compared).
"""

from __future__ import annotations

import functools
import pickle
import sys
import types

import numpy as np


# ---------------------------------------------------------------------------
# Array type with JAX's functional update syntax
# ---------------------------------------------------------------------------
class JArray(np.ndarray):
    """ndarray whose in-place operators do not mutate (JAX arrays are immutable)."""

    def __array_finalize__(self, obj):  # noqa: D401 - numpy hook
        pass

    @property
    def at(self):
        return _At(self)

    # JAX arrays have no in-place operators; Python then falls back to
    # ``x = x op y``.  Emulate that so no aliased array is ever mutated.
    def __iadd__(self, o):
        return np.add(self, o)

    def __isub__(self, o):
        return np.subtract(self, o)

    def __imul__(self, o):
        return np.multiply(self, o)

    def __itruediv__(self, o):
        return np.true_divide(self, o)


def _w(a):
    """Wrap a NumPy result as JArray (scalars stay NumPy scalars)."""
    if isinstance(a, np.ndarray) and not isinstance(a, JArray):
        return a.view(JArray)
    return a


class _AtIdx:
    def __init__(self, arr, idx):
        self.arr = arr
        self.idx = idx

    def set(self, v):
        out = np.array(self.arr, copy=True)
        v = np.asarray(v)
        if v.dtype != out.dtype and out.dtype == bool:
            v = v.astype(bool)
        out[self.idx] = v
        return _w(out)

    def add(self, v):
        out = np.array(self.arr, copy=True)
        np.add.at(out, self.idx, v)
        return _w(out)

    def get(self):
        return _w(np.asarray(self.arr)[self.idx])


class _At:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _AtIdx(self.arr, idx)


# ---------------------------------------------------------------------------
# jax.numpy
# ---------------------------------------------------------------------------
def _wrapfn(fn):
    @functools.wraps(fn)
    def inner(*a, **k):
        r = fn(*a, **k)
        if isinstance(r, tuple):
            return tuple(_w(x) for x in r)
        return _w(r)

    return inner


def _bincount(x, weights=None, length=None, minlength=0):
    x = np.asarray(x).reshape(-1)
    n = length if length is not None else minlength
    r = np.bincount(x, weights=None if weights is None else np.asarray(weights).reshape(-1),
                    minlength=int(n))
    if length is not None:
        r = r[: int(length)]
    return _w(r)


def _array(obj, dtype=None, **kw):
    return _w(np.array(obj, dtype=dtype))


def _make_jnp():
    m = types.ModuleType("jax.numpy")
    names = [
        "zeros", "ones", "linspace", "arange", "concatenate", "clip", "floor", "stack",
        "matmul", "sum", "mean", "diag", "exp", "sqrt", "round", "isclose", "maximum",
        "minimum", "divmod", "tile", "repeat", "logical_and", "zeros_like", "ones_like",
        "abs", "diff", "multiply", "where", "asarray", "full", "min", "max", "any", "all",
        "reshape", "dot", "einsum", "prod", "cumsum", "sort", "argmax", "argmin",
        "logical_or", "logical_not", "ceil", "sign", "power", "log", "square", "array_equal",
        "nonzero", "take", "meshgrid", "outer", "eye", "full_like", "transpose",
    ]
    for n in names:
        setattr(m, n, _wrapfn(getattr(np, n)))
    m.array = _array
    m.bincount = _bincount
    m.size = np.size
    m.shape = np.shape
    m.pi = np.pi
    m.inf = np.inf
    m.nan = np.nan
    m.float32 = np.float32
    m.float64 = np.float64
    m.int32 = np.int32
    m.int64 = np.int64
    m.bool_ = np.bool_
    m.ndarray = np.ndarray
    m.savez = np.savez
    m.load = np.load
    linalg = types.ModuleType("jax.numpy.linalg")
    linalg.det = _wrapfn(np.linalg.det)
    linalg.norm = _wrapfn(np.linalg.norm)
    linalg.inv = _wrapfn(np.linalg.inv)
    m.linalg = linalg
    return m


# ---------------------------------------------------------------------------
# pytree helpers for vmap / scan
# ---------------------------------------------------------------------------
def _stack_tree(items):
    first = items[0]
    if isinstance(first, (list, tuple)):
        cols = [_stack_tree([it[i] for it in items]) for i in range(len(first))]
        return type(first)(cols) if isinstance(first, tuple) else cols
    if isinstance(first, dict):
        return {k: _stack_tree([it[k] for it in items]) for k in first}
    return _w(np.stack([np.asarray(x) for x in items], axis=0))


def vmap(f, in_axes=0, out_axes=0):
    if in_axes not in (0, (0,)):
        raise NotImplementedError("only in_axes=0 is used by the reference")

    def mapped(*args):
        n = len(args[0])
        outs = [f(*[a[i] for a in args]) for i in range(n)]
        return _stack_tree(outs)

    return mapped


def scan(f, init, xs, length=None):
    carry = init
    ys = []
    seq = xs if xs is not None else range(length)
    for x in seq:
        carry, y = f(carry, x)
        ys.append(y)
    return carry, _stack_tree(ys)


def select(pred, a, b):
    return _w(np.where(pred, a, b))


def jit(fun=None, **kw):
    if fun is None:
        return lambda f: f
    return fun


# ---------------------------------------------------------------------------
# jax.experimental.sparse.BCOO
# ---------------------------------------------------------------------------
class BCOO:
    def __init__(self, args, shape):
        data, indices = args
        self.data = np.asarray(data)
        self.indices = np.asarray(indices)
        self.shape = tuple(int(s) for s in shape)

    def __matmul__(self, v):
        v = np.asarray(v)
        out = np.zeros(self.shape[0], dtype=np.result_type(self.data, v))
        np.add.at(out, self.indices[:, 0], self.data * v[self.indices[:, 1]])
        return _w(out)


# ---------------------------------------------------------------------------
# installation into sys.modules
# ---------------------------------------------------------------------------
VTK_CALLS: list = []


def install():
    """Register fake ``jax``, ``dill`` and ``pyevtk`` modules in sys.modules."""
    jax = types.ModuleType("jax")
    jnp = _make_jnp()
    lax = types.ModuleType("jax.lax")
    lax.scan = scan
    lax.select = select
    experimental = types.ModuleType("jax.experimental")
    sparse = types.ModuleType("jax.experimental.sparse")
    sparse.BCOO = BCOO
    experimental.sparse = sparse
    config = types.SimpleNamespace(update=lambda *a, **k: None)
    jax.numpy = jnp
    jax.lax = lax
    jax.experimental = experimental
    jax.jit = jit
    jax.vmap = vmap
    jax.config = config
    sys.modules["jax"] = jax
    sys.modules["jax.numpy"] = jnp
    sys.modules["jax.lax"] = lax
    sys.modules["jax.experimental"] = experimental
    sys.modules["jax.experimental.sparse"] = sparse

    dill = types.ModuleType("dill")
    dill.dump = pickle.dump
    dill.load = pickle.load
    dill.HIGHEST_PROTOCOL = pickle.HIGHEST_PROTOCOL
    sys.modules["dill"] = dill

    pyevtk = types.ModuleType("pyevtk")
    hl = types.ModuleType("pyevtk.hl")

    def gridToVTK(path, *a, **k):
        VTK_CALLS.append(path)

    hl.gridToVTK = gridToVTK
    pyevtk.hl = hl
    sys.modules["pyevtk"] = pyevtk
    sys.modules["pyevtk.hl"] = hl
    return jax
