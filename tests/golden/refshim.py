"""A numpy stand-in for ``jax``/``equinox``/``lineax`` so the reference's own forward code runs here.

Test infrastructure only: it exists to generate golden vectors from the reference package itself
(``make_golden.py``) in a container where JAX is not installed.  It evaluates the reference's
forward arithmetic in float64 numpy; it does no differentiation, tracing or compilation.  Any jax
API the forward path does not use resolves to an inert placeholder so that the reference's package
``__init__`` modules import.
"""
from __future__ import annotations

import abc
import dataclasses
import functools
import sys
import types

import numpy as np


class JArr(np.ndarray):
    """ndarray with jax's functional ``.at[idx].set/add/...`` update syntax."""

    def __array_finalize__(self, obj):  # noqa: D401 - numpy hook
        pass

    @property
    def at(self):
        return _At(self)

    def block_until_ready(self):
        return self


class _At:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _AtIdx(self.arr, idx)


class _AtIdx:
    def __init__(self, arr, idx):
        self.arr, self.idx = arr, _unwrap(idx)

    def set(self, v, **_):
        out = np.array(self.arr, copy=True)
        out[self.idx] = _unwrap(v)
        return _wrap(out)

    def add(self, v, **_):
        out = np.array(self.arr, copy=True)
        np.add.at(out, self.idx, _unwrap(v))
        return _wrap(out)

    def multiply(self, v, **_):
        out = np.array(self.arr, copy=True)
        np.multiply.at(out, self.idx, _unwrap(v))
        return _wrap(out)

    def max(self, v, **_):
        out = np.array(self.arr, copy=True)
        np.maximum.at(out, self.idx, _unwrap(v))
        return _wrap(out)

    def min(self, v, **_):
        out = np.array(self.arr, copy=True)
        np.minimum.at(out, self.idx, _unwrap(v))
        return _wrap(out)

    def get(self, **_):
        return _wrap(np.asarray(self.arr)[self.idx])


def _unwrap(x):
    if isinstance(x, JArr):
        return x.view(np.ndarray)
    if isinstance(x, tuple):
        return tuple(_unwrap(v) for v in x)
    if isinstance(x, list):
        return [_unwrap(v) for v in x]
    return x


def _wrap(x):
    if isinstance(x, np.ndarray) and not isinstance(x, JArr):
        return x.view(JArr)
    if isinstance(x, np.generic):
        return np.asarray(x).view(JArr)
    if isinstance(x, tuple):
        return tuple(_wrap(v) for v in x)
    if isinstance(x, list):
        return [_wrap(v) for v in x]
    return x


class _Inert:
    """Placeholder for any jax/lineax API the forward path never executes."""

    def __init__(self, name="inert"):
        self._name = name

    def __call__(self, *a, **k):
        if len(a) == 1 and callable(a[0]) and not k:
            return a[0]  # used as a decorator
        return _Inert(self._name + "()")

    def __getattr__(self, name):
        if name.startswith("__") and name.endswith("__"):
            raise AttributeError(name)
        return _Inert(f"{self._name}.{name}")

    def __mro_entries__(self, bases):
        return (object,)

    def __repr__(self):
        return f"<inert {self._name}>"


class _InertModule(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__") and name.endswith("__"):
            raise AttributeError(name)
        return _Inert(f"{self.__name__}.{name}")


def _np_fn(fn):
    @functools.wraps(fn)
    def wrapped(*a, **k):
        a = tuple(_unwrap(v) for v in a)
        k = {kk: _unwrap(v) for kk, v in k.items()}
        return _wrap(fn(*a, **k))

    return wrapped


class _JnpModule(types.ModuleType):
    ndarray = np.ndarray
    integer = np.integer
    floating = np.floating
    float64 = np.float64
    float32 = np.float32
    int32 = np.int32
    int64 = np.int64
    bool_ = np.bool_
    inf = np.inf
    nan = np.nan
    pi = np.pi
    newaxis = None

    def __getattr__(self, name):
        if name.startswith("__") and name.endswith("__"):
            raise AttributeError(name)
        target = getattr(np, name)
        if isinstance(target, types.ModuleType):
            return _NpSub(target)
        if callable(target) and not isinstance(target, type):
            return _np_fn(target)
        return target

    @staticmethod
    def asarray(x, dtype=None):
        return np.asarray(_unwrap(x), dtype=dtype).view(JArr)

    @staticmethod
    def clip(a, a_min=None, a_max=None, **_):
        return _wrap(np.clip(_unwrap(a), a_min, a_max))

    @staticmethod
    def array(x, dtype=None):
        return np.array(_unwrap(x), dtype=dtype).view(JArr)


class _NpSub:
    def __init__(self, mod):
        self._mod = mod

    def __getattr__(self, name):
        t = getattr(self._mod, name)
        return _np_fn(t) if callable(t) else t


def _segment(reducer, init):
    def seg(data, segment_ids, num_segments=None, **_):
        data = np.asarray(_unwrap(data))
        ids = np.asarray(_unwrap(segment_ids))
        n = int(num_segments) if num_segments is not None else int(ids.max()) + 1
        out = np.full((n,) + data.shape[1:], init, dtype=data.dtype)
        reducer.at(out, ids, data)
        return _wrap(out)

    return seg


def _scan(f, init, xs=None, length=None, **_):
    carry = init
    ys = []
    n = length if xs is None else len(xs)
    for i in range(n):
        carry, y = f(carry, None if xs is None else xs[i])
        ys.append(y)
    return carry, ys


def _cond(pred, true_fun, false_fun, *ops):
    return true_fun(*ops) if bool(pred) else false_fun(*ops)


def _fori(lo, hi, body, init):
    v = init
    for i in range(lo, hi):
        v = body(i, v)
    return v


def _while(cond, body, init):
    v = init
    while bool(cond(v)):
        v = body(v)
    return v


def _lax_map(f, xs, **_):
    return _wrap(np.stack([_unwrap(f(x)) for x in xs]))


# ---------------------------------------------------------------- equinox
class _StaticField:
    pass


def _eqx_field(*, static=False, default=dataclasses.MISSING, default_factory=dataclasses.MISSING,
               converter=None, **_):
    kw = {}
    if default is not dataclasses.MISSING:
        kw["default"] = default
    if default_factory is not dataclasses.MISSING:
        kw["default_factory"] = default_factory
    md = {"converter": converter} if converter is not None else {}
    return dataclasses.field(metadata=md, **kw)


class _ModuleMeta(abc.ABCMeta):
    def __new__(mcls, name, bases, ns, **kw):
        cls = super().__new__(mcls, name, bases, ns, **kw)
        has_init = "__init__" in ns
        # Mutable class-level defaults (arrays) are not allowed by dataclasses; wrap them.
        for k, ann in list(ns.get("__annotations__", {}).items()):
            v = ns.get(k, dataclasses.MISSING)
            if isinstance(v, (np.ndarray, list, dict, set)):
                setattr(cls, k, dataclasses.field(default_factory=(lambda vv=v: vv)))
        cls = dataclasses.dataclass(init=not has_init, eq=False, repr=False)(cls)
        return cls

    def __call__(cls, *a, **k):
        obj = cls.__new__(cls)
        object.__setattr__(obj, "_eqx_init", True)
        cls.__init__(obj, *a, **k)
        for f in dataclasses.fields(cls):
            conv = f.metadata.get("converter")
            if conv is not None and hasattr(obj, f.name):
                object.__setattr__(obj, f.name, conv(getattr(obj, f.name)))
        object.__setattr__(obj, "_eqx_init", False)
        post = getattr(obj, "__post_init__", None)
        if post is not None and "__init__" in cls.__dict__:
            pass
        check = getattr(obj, "__check_init__", None)
        if check is not None:
            check()
        return obj


class Module(metaclass=_ModuleMeta):
    def __setattr__(self, name, value):
        if getattr(self, "_eqx_init", False):
            object.__setattr__(self, name, value)
        else:
            raise AttributeError(f"cannot set {name} on a frozen Module")


def _tree_at(where, pytree, replace=None, replace_fn=None, is_leaf=None):
    import copy

    # Only the attribute-path form ``lambda m: m.a`` / ``lambda m: (m.a, m.b)`` is needed here.
    class _Rec:
        def __init__(self, path=()):
            self._path = path

        def __getattr__(self, name):
            return _Rec(self._path + (name,))

    rec = where(_Rec())
    paths = [r._path for r in (rec if isinstance(rec, tuple) else (rec,))]
    values = replace if isinstance(rec, tuple) else (replace,)

    def setp(obj, path, value):
        new = copy.copy(obj)
        if len(path) == 1:
            object.__setattr__(new, path[0], value)
        else:
            object.__setattr__(new, path[0], setp(getattr(obj, path[0]), path[1:], value))
        return new

    out = pytree
    for p, v in zip(paths, values):
        out = setp(out, p, v)
    return out


def _grad(f, argnums=0, **_):
    """``jax.grad`` of a scalar function by complex-step differentiation (exact to rounding).

    Used by the reference only on elementwise closed-form wall functions; one complex evaluation
    per input element with step ``1e-30`` gives the derivative without subtractive cancellation.
    """
    assert argnums == 0

    def g(x, *rest):
        x = np.asarray(_unwrap(x), dtype=float)
        out = np.zeros_like(x)
        flat = x.ravel()
        h = 1e-30
        for i in range(flat.size):
            xc = flat.astype(complex)
            xc[i] += 1j * h
            val = _unwrap(f(_wrap(xc.reshape(x.shape)), *rest))
            out.flat[i] = np.imag(val) / h
        return _wrap(out)

    return g


def _error_if(x, pred, msg):
    if bool(np.any(_unwrap(pred))):
        raise RuntimeError(msg)
    return x


def install() -> None:
    """Register the stand-in modules in ``sys.modules`` (idempotent)."""
    if "jax" in sys.modules and getattr(sys.modules["jax"], "_refshim", False):
        return
    jax = _InertModule("jax")
    jax._refshim = True
    jnp = _JnpModule("jax.numpy")
    ops = types.ModuleType("jax.ops")
    ops.segment_sum = _segment(np.add, 0.0)
    ops.segment_max = _segment(np.maximum, -np.inf)
    ops.segment_min = _segment(np.minimum, np.inf)
    lax = _InertModule("jax.lax")
    lax.scan, lax.cond, lax.fori_loop, lax.while_loop, lax.map = _scan, _cond, _fori, _while, _lax_map
    lax.stop_gradient = lambda x: x
    config = types.SimpleNamespace(update=lambda *a, **k: None)
    jax.numpy, jax.ops, jax.lax, jax.config = jnp, ops, lax, config
    jax.Array = np.ndarray
    jax.core = types.SimpleNamespace(Tracer=type("Tracer", (), {}))
    jax.errors = types.SimpleNamespace(TracerArrayConversionError=type("E1", (Exception,), {}),
                                       ConcretizationTypeError=type("E2", (Exception,), {}))
    jax.ShapeDtypeStruct = _Inert("ShapeDtypeStruct")
    jax.jit = lambda f=None, **k: (f if f is not None else (lambda g: g))
    jax.grad = _grad
    jax.tree_util = _InertModule("jax.tree_util")
    jax.tree = _InertModule("jax.tree")
    jax.scipy = _InertModule("jax.scipy")
    jax.experimental = _InertModule("jax.experimental")
    jax.random = _InertModule("jax.random")
    jax.debug = types.SimpleNamespace(callback=lambda *a, **k: None, print=lambda *a, **k: None)
    mods = {"jax": jax, "jax.numpy": jnp, "jax.ops": ops, "jax.lax": lax,
            "jax.tree_util": jax.tree_util, "jax.scipy": jax.scipy,
            "jax.experimental": jax.experimental, "jax.random": jax.random}
    for sub in ("jax.scipy.sparse", "jax.scipy.sparse.linalg", "jax.scipy.linalg",
                "jax.experimental.sparse", "jax.sharding", "jax.experimental.shard_map",
                "jax.typing", "jax.flatten_util", "jax.dtypes"):
        mods[sub] = _InertModule(sub)
    eqx = _InertModule("equinox")
    eqx.Module = Module
    eqx.field = _eqx_field
    eqx.tree_at = _tree_at
    eqx.filter_jit = lambda f=None, **k: (f if f is not None else (lambda g: g))
    eqx.error_if = _error_if
    eqx.AbstractVar = type("AbstractVar", (), {"__class_getitem__": classmethod(lambda c, i: object)})
    mods["equinox"] = eqx
    for name in ("lineax", "diffrax", "optimistix", "petsc4py", "petsc4py.PETSc", "jaxtyping"):
        mods[name] = _InertModule(name)
    sys.modules.update(mods)
