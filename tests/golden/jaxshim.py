"""A numpy-backed stand-in for the parts of ``jax`` that JAX-Fluids touches,
so that the reference's own Python source can run in a container without
jax/jaxlib and produce golden vectors.

Test infrastructure only: it is installed into ``sys.modules`` by
``make_ref_fixtures.py`` and by nothing else.

What it reproduces:

* ``jax.numpy``: numpy's functions, with results viewed as ``JArray`` (an
  ``ndarray`` subclass with JAX's functional ``x.at[idx].set/add/mul/min/max/get``
  and ``block_until_ready``).  Elementwise float64 arithmetic rounds each
  operation once (IEEE), as XLA does without contraction.  ``jnp.power`` with an
  integer exponent is evaluated like ``lax.integer_pow`` (binary powering of
  the base by repeated squaring), not through libm's ``pow``.
* ``jax.jit`` / ``jax.checkpoint`` / ``custom_vjp`` / ``stop_gradient``: run the
  function eagerly (no tracing, no differentiation).
* ``jax.lax`` control flow (``fori_loop``, ``while_loop``, ``scan``, ``cond``,
  ``switch``) as Python loops; collectives are single-device identities.
* ``jax.vmap`` as a Python loop over the mapped axis.

Differentiation is not reproduced: gradients come from elsewhere.
"""
from __future__ import annotations

import functools
import sys
import types

import numpy as np


class JArray(np.ndarray):
    """numpy array with JAX's functional update syntax."""

    def __array_finalize__(self, obj):
        pass

    @property
    def at(self):
        return _At(self)

    def block_until_ready(self):
        return self

    def __hash__(self):
        return id(self)

    # ``x != None`` is a plain bool for a JAX array (its comparison operators
    # defer on operands they do not recognise, so Python compares identities)
    def __eq__(self, o):
        return False if o is None else np.ndarray.__eq__(self, o)

    def __ne__(self, o):
        return True if o is None else np.ndarray.__ne__(self, o)

    # JAX arrays are immutable: ``x += y`` rebinds x to a new array.  numpy
    # would write through x, and through every view that shares its memory.
    def __iadd__(self, o):
        return np.add(self, o)

    def __isub__(self, o):
        return np.subtract(self, o)

    def __imul__(self, o):
        return np.multiply(self, o)

    def __itruediv__(self, o):
        return np.true_divide(self, o)

    def __ipow__(self, o):
        return np.power(self, o)

    def __setitem__(self, k, v):
        raise TypeError("JAX arrays are immutable: use x.at[idx].set(v)")


def _wrap(x):
    if isinstance(x, np.ndarray) and not isinstance(x, JArray):
        return x.view(JArray)
    if isinstance(x, tuple):
        return tuple(_wrap(v) for v in x)
    if isinstance(x, list):
        return [_wrap(v) for v in x]
    return x


class _AtIndex:
    def __init__(self, arr, idx):
        self.arr, self.idx = arr, idx

    def _apply(self, op, val):
        out = np.array(self.arr, copy=True)  # plain ndarray while it is written
        val = np.asarray(val)
        if op == "set":
            out[self.idx] = val
        elif op == "add":
            if _fancy(self.idx):
                np.add.at(out, self.idx, val)
            else:
                out[self.idx] = out[self.idx] + val
        elif op == "mul":
            out[self.idx] = out[self.idx] * val
        elif op == "min":
            out[self.idx] = np.minimum(out[self.idx], val)
        elif op == "max":
            out[self.idx] = np.maximum(out[self.idx], val)
        return out.view(JArray)

    def set(self, val, **kw):
        return self._apply("set", val)

    def add(self, val, **kw):
        return self._apply("add", val)

    def multiply(self, val, **kw):
        return self._apply("mul", val)

    mul = multiply

    def min(self, val, **kw):
        return self._apply("min", val)

    def max(self, val, **kw):
        return self._apply("max", val)

    def get(self, **kw):
        return _wrap(np.asarray(self.arr)[self.idx])


def _fancy(idx):
    idx = idx if isinstance(idx, tuple) else (idx,)
    return any(isinstance(i, (np.ndarray, list)) for i in idx)


class _At:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _AtIndex(self.arr, idx)


# ---------------------------------------------------------------- jax.numpy
def _integer_pow(x, n):
    """lax.integer_pow: binary powering (square-and-multiply), as XLA expands it."""
    x = np.asarray(x)
    if n == 0:
        return np.ones_like(x)
    neg = n < 0
    n = abs(n)
    acc = None
    base = x
    while n:
        if n & 1:
            acc = base if acc is None else acc * base
        n >>= 1
        if n:
            base = base * base
    return 1.0 / acc if neg else acc


def _power(x, y):
    if isinstance(y, (int, np.integer)) and not isinstance(y, bool):
        return _wrap(_integer_pow(x, int(y)))
    return _wrap(np.power(x, y))


def _make_jnp():
    jnp = types.ModuleType("jax.numpy")
    special = {
        "power": _power,
        "s_": np.s_,
        "index_exp": np.index_exp,
        "ndarray": JArray,
        "newaxis": None,
        "pi": np.pi,
        "inf": np.inf,
        "nan": np.nan,
        "e": np.e,
    }

    def array(x, dtype=None, copy=True, **kw):
        return _wrap(np.array(x, dtype=dtype))

    def asarray(x, dtype=None, **kw):
        return _wrap(np.asarray(x, dtype=dtype))

    special["array"] = array
    special["asarray"] = asarray

    def square(x):
        x = np.asarray(x)
        return _wrap(x * x)

    special["square"] = square

    def _getattr(name):
        if name in special:
            return special[name]
        obj = getattr(np, name)
        if isinstance(obj, type) or not callable(obj):
            return obj

        @functools.wraps(obj)
        def f(*a, **k):
            k.pop("precision", None)
            for key in ("where", "initial"):  # JAX's None means "no mask" / "no initial value"
                if key in k and k[key] is None:
                    del k[key]
            return _wrap(obj(*a, **k))

        return f

    jnp.__getattr__ = _attr_only(_getattr)
    for n in ("float32", "float64", "int32", "int64", "bool_", "uint8", "finfo", "iinfo", "dtype"):
        setattr(jnp, n, getattr(np, n))
    for n, v in special.items():
        setattr(jnp, n, v)
    linalg = types.ModuleType("jax.numpy.linalg")
    linalg.__getattr__ = _attr_only(lambda name: (lambda *a, **k: _wrap(getattr(np.linalg, name)(*a, **k))))
    jnp.linalg = linalg
    return jnp


# ---------------------------------------------------------------- jax.lax
def _make_lax():
    lax = types.ModuleType("jax.lax")

    def fori_loop(lo, hi, body, init, **kw):
        v = init
        for i in range(int(lo), int(hi)):
            v = body(i, v)
        return v

    def while_loop(cond, body, init):
        v = init
        while bool(cond(v)):
            v = body(v)
        return v

    def scan(f, init, xs=None, length=None, **kw):
        carry = init
        ys = []
        n = length if xs is None else len(_leaves(xs)[0])
        for i in range(n):
            x = None if xs is None else _tree_map(lambda a: a[i], xs)
            carry, y = f(carry, x)
            ys.append(y)
        if ys and ys[0] is not None:
            stacked = _tree_map(lambda *a: _wrap(np.stack(a)), *ys)
        else:
            stacked = None
        return carry, stacked

    def cond(pred, tf, ff, *ops):
        return tf(*ops) if bool(pred) else ff(*ops)

    def switch(i, branches, *ops):
        return branches[int(i)](*ops)

    def select(p, a, b):
        return _wrap(np.where(p, a, b))

    ident = lambda x, *a, **k: x
    lax.fori_loop, lax.while_loop, lax.scan, lax.cond, lax.switch, lax.select = (
        fori_loop, while_loop, scan, cond, switch, select)
    lax.stop_gradient = ident
    for n in ("psum", "pmax", "pmin", "pmean", "all_gather"):
        setattr(lax, n, ident)
    lax.ppermute = lambda x, *a, **k: x
    lax.axis_index = lambda *a, **k: 0
    lax.integer_pow = lambda x, n: _wrap(_integer_pow(x, n))
    lax.sqrt = lambda x: _wrap(np.sqrt(x))
    lax.rsqrt = lambda x: _wrap(1.0 / np.sqrt(x))
    lax.max = lambda a, b: _wrap(np.maximum(a, b))
    lax.min = lambda a, b: _wrap(np.minimum(a, b))
    return lax


def _leaves(t):
    if isinstance(t, dict):
        return [l for v in t.values() for l in _leaves(v)]
    if isinstance(t, (list, tuple)):
        return [l for v in t for l in _leaves(v)]
    if t is None:
        return []
    return [t]


def _tree_map(f, t, *rest):
    if isinstance(t, dict):
        return {k: _tree_map(f, t[k], *(r[k] for r in rest)) for k in t}
    if isinstance(t, tuple) and hasattr(t, "_fields"):
        return type(t)(*(_tree_map(f, a, *(r[i] for r in rest)) for i, a in enumerate(t)))
    if isinstance(t, (list, tuple)):
        return type(t)(_tree_map(f, a, *(r[i] for r in rest)) for i, a in enumerate(t))
    if t is None:
        return None
    return f(t, *rest)


# ---------------------------------------------------------------- jax
class _Config:
    def __init__(self):
        self.values = {"jax_enable_x64": True}

    def update(self, k, v):
        if k == "jax_enable_x64" and not v:
            raise RuntimeError("the numpy stand-in runs in float64 only")
        self.values[k] = v

    def read(self, k):
        return self.values.get(k)

    def __getattr__(self, k):
        return self.values.get(k)


def jit(fun=None, **kw):
    if fun is None:
        return lambda f: f
    return fun


def checkpoint(fun=None, **kw):
    if fun is None:
        return lambda f: f
    return fun


class custom_vjp:
    def __init__(self, fun, nondiff_argnums=()):
        self.fun = fun
        functools.update_wrapper(self, fun)

    def defvjp(self, fwd, bwd):
        pass

    def __call__(self, *a, **k):
        return self.fun(*a, **k)

    def __get__(self, obj, objtype=None):
        return self if obj is None else functools.partial(self, obj)


def vmap(fun, in_axes=0, out_axes=0, **kw):
    def mapped(*args):
        axes = in_axes if isinstance(in_axes, (list, tuple)) else [in_axes] * len(args)
        n = next(np.shape(a)[ax] for a, ax in zip(args, axes) if ax is not None)
        outs = [fun(*(a if ax is None else np.take(a, i, axis=ax) for a, ax in zip(args, axes))) for i in range(n)]
        return _tree_map(lambda *o: _wrap(np.stack(o, axis=out_axes)), *outs)
    return mapped


def pmap(fun=None, **kw):
    """Decorates (the reference decorates methods at class definition); calling raises."""
    if fun is None:
        return lambda f: pmap(f)

    @functools.wraps(fun)
    def f(*a, **k):
        raise NotImplementedError("jax.pmap is not available in the numpy stand-in")
    return f


def _attr_only(fn):
    """Module __getattr__ answering ordinary names only: dunder lookups
    (__file__, __path__, ...) raise AttributeError as for a real module."""
    def getattr_(name):
        if name.startswith("__"):
            raise AttributeError(name)
        return fn(name)
    return getattr_


def _no(name):
    def f(*a, **k):
        raise NotImplementedError(f"jax.{name} is not available in the numpy stand-in")
    return f


class _Anything:
    """Stand-in for any attribute of a stubbed third-party package: callable,
    subclassable, and every attribute is another stand-in."""

    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _Anything()

    def __getattr__(self, k):
        return _Anything()


class _StubFinder:
    """Import hook answering for packages the reference imports at module level
    but never calls on this path (flax, haiku, optax, h5py, matplotlib, yaml,
    git): their modules exist and every attribute is a stand-in."""

    def __init__(self, names):
        self.names = set(names)

    def find_spec(self, name, path, target=None):
        import importlib.machinery
        if name.split(".")[0] in self.names:
            return importlib.machinery.ModuleSpec(name, self, is_package=True)
        return None

    def create_module(self, spec):
        m = types.ModuleType(spec.name)
        m.__path__ = []
        m.__getattr__ = _attr_only(lambda k: _Anything)
        return m

    def exec_module(self, m):
        pass


def install_stubs(names=("flax", "haiku", "optax", "h5py", "matplotlib", "mpl_toolkits", "yaml", "git")):
    """Stub the packages in `names` that are not importable here."""
    import importlib.util
    missing = [n for n in names if n not in sys.modules and importlib.util.find_spec(n) is None]
    if missing:
        sys.meta_path.insert(0, _StubFinder(missing))
    return missing


def install():
    """Put the stand-in into sys.modules as jax, jax.numpy, jax.lax, ..."""
    if "jax" in sys.modules and getattr(sys.modules["jax"], "_numpy_standin", False):
        return sys.modules["jax"]
    jax = types.ModuleType("jax")
    jax._numpy_standin = True
    jnp = _make_jnp()
    lax = _make_lax()
    jax.numpy, jax.lax = jnp, lax
    jax.Array = JArray
    jax.ndarray = JArray
    jax.config = _Config()
    jax.jit, jax.checkpoint, jax.remat, jax.custom_vjp, jax.vmap = jit, checkpoint, checkpoint, custom_vjp, vmap
    jax.pmap = pmap
    jax.grad = _no("grad")
    jax.value_and_grad = _no("value_and_grad")
    jax.stop_gradient = lambda x: x
    jax.device_count = lambda *a: 1
    jax.local_device_count = lambda *a: 1
    jax.process_index = lambda *a: 0
    jax.process_count = lambda *a: 1
    jax.devices = lambda *a: ["cpu:0"]
    jax.local_devices = lambda *a: ["cpu:0"]
    jax.default_backend = lambda: "cpu"
    jax.device_put = lambda x, *a, **k: _wrap(np.asarray(x)) if isinstance(x, np.ndarray) else x
    jax.device_put_sharded = _no("device_put_sharded")
    jax.block_until_ready = lambda x: x
    tree = types.ModuleType("jax.tree")
    tree.map = _tree_map
    tree.leaves = _leaves
    jax.tree = tree
    tree_util = types.ModuleType("jax.tree_util")
    tree_util.tree_map = _tree_map
    tree_util.tree_leaves = _leaves
    tree_util.register_pytree_node_class = lambda c: c
    tree_util.register_pytree_node = lambda *a, **k: None
    jax.tree_util = tree_util
    nn = types.ModuleType("jax.nn")
    nn.relu = lambda x: _wrap(np.maximum(x, 0.0))
    jax.nn = nn
    random = types.ModuleType("jax.random")
    random.PRNGKey = lambda s: np.random.default_rng(s)
    random.uniform = lambda key, shape=(), minval=0.0, maxval=1.0, **k: _wrap(key.uniform(minval, maxval, shape))
    jax.random = random
    scipy = types.ModuleType("jax.scipy")
    special = types.ModuleType("jax.scipy.special")
    special.__getattr__ = _attr_only(_no)
    scipy.special = special
    jax.scipy = scipy
    experimental = types.ModuleType("jax.experimental")
    mh = types.ModuleType("jax.experimental.multihost_utils")
    mh.process_allgather = lambda x, *a, **k: x
    mh.sync_global_devices = lambda *a, **k: None
    mh.broadcast_one_to_all = lambda x, *a, **k: x
    experimental.multihost_utils = mh
    jax.experimental = experimental
    version = types.ModuleType("jax.version")
    version.__version__ = "numpy-stand-in"
    jax.version = version
    jaxlib = types.ModuleType("jaxlib")
    jaxlib.__path__ = []
    jaxlib_version = types.ModuleType("jaxlib.version")
    jaxlib_version.__version__ = "numpy-stand-in"
    jaxlib.version = jaxlib_version
    typing = types.ModuleType("jax.typing")
    typing.ArrayLike = object
    jax.typing = typing
    for name, mod in {"jax": jax, "jax.numpy": jnp, "jax.lax": lax, "jax.tree": tree, "jax.tree_util": tree_util,
                      "jax.nn": nn, "jax.random": random, "jax.scipy": scipy, "jax.scipy.special": special,
                      "jax.experimental": experimental, "jax.experimental.multihost_utils": mh,
                      "jax.numpy.linalg": jnp.linalg, "jax.typing": typing, "jax.version": version,
                      "jaxlib": jaxlib, "jaxlib.version": jaxlib_version}.items():
        sys.modules[name] = mod
    return jax
