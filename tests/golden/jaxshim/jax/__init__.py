"""numpy stand-in for jax (see tests/golden/jaxshim/README.txt)."""
import copy as _copy
import functools as _ft

import numpy as _np

from . import numpy as numpy  # noqa: F401
from .numpy import JArr as Array, _wrap, _unwrap, X64

_np_ = _np


def _leading(a, ax):
    return _np.shape(a)[ax]


def _take(a, ax, i):
    if ax is None:
        return a
    if isinstance(a, (list, tuple)):
        return type(a)(_take(x, ax, i) for x in a)
    return _wrap(_np.take(_unwrap(a), i, axis=ax))


def _stack(outs):
    o0 = outs[0]
    if isinstance(o0, tuple):
        return tuple(_stack([o[k] for o in outs]) for k in range(len(o0)))
    if isinstance(o0, list):
        return [_stack([o[k] for o in outs]) for k in range(len(o0))]
    if o0 is None:
        return None
    return _wrap(_np.stack([_unwrap(o) for o in outs]))


def vmap(f, in_axes=0, out_axes=0):
    def g(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        n = None
        for a, ax in zip(args, axes):
            if ax is not None:
                n = _leading(_unwrap(a) if not isinstance(a, (list, tuple)) else a[0], ax)
                break
        outs = [f(*[_take(a, ax, i) for a, ax in zip(args, axes)]) for i in range(n)]
        return _stack(outs)
    return g


def grad(f):
    """Complex-step derivative of a scalar analytic function of one scalar."""
    def g(x):
        xr = _np.asarray(_unwrap(x))
        cdt = _np.complex128 if (X64 or xr.dtype == _np.float64) else _np.complex64
        h = 1e-30 if cdt == _np.complex128 else 1e-20
        xc = (xr.astype(cdt) + 1j * h).astype(cdt)
        y = _np.asarray(_unwrap(f(_wrap(xc))))
        yr = _np.asarray(_unwrap(f(_wrap(xr))))
        d = _np.imag(y) / h
        d = _np.where(_np.isnan(yr), _np.nan, d)
        return _wrap(d.astype(xr.dtype if xr.dtype.kind == "f" else _np.float32))
    return g


def _trace_leaves(obj, memo):
    """What jit does to a module argument: Python float fields become f32 scalars."""
    from equinox import Module
    if isinstance(obj, list):
        return [_trace_leaves(o, memo) for o in obj]
    if isinstance(obj, tuple):
        return tuple(_trace_leaves(o, memo) for o in obj)
    if isinstance(obj, Module):
        if id(obj) in memo:
            return memo[id(obj)]
        new = _copy.copy(obj)
        memo[id(obj)] = new
        static = type(obj)._shim_static_fields()
        for k, v in list(vars(obj).items()):
            if k in static:
                continue
            if isinstance(v, float) and not isinstance(v, bool):
                object.__setattr__(new, k, _wrap(_np.asarray(v, _np.float64 if X64 else _np.float32)))
            elif isinstance(v, (list, tuple, Module)):
                object.__setattr__(new, k, _trace_leaves(v, memo))
        return new
    return obj


def jit(f=None, static_argnames=None, **kw):
    if f is None:
        return lambda g: jit(g, static_argnames=static_argnames, **kw)

    @_ft.wraps(f)
    def g(*args, **kwargs):
        memo = {}
        args = [_trace_leaves(a, memo) for a in args]
        return f(*args, **kwargs)
    return g


def block_until_ready(x):
    return x


from . import random as random  # noqa: E402,F401
from . import lax as lax  # noqa: E402,F401
from . import ops as ops  # noqa: E402,F401
from . import tree_util as tree_util  # noqa: E402,F401
