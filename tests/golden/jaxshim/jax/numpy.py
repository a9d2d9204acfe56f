"""numpy with JAX's dtype rules (x64 disabled unless JAXSHIM_X64=1)."""
import os as _os
import sys as _sys
import types as _types

import numpy as _np

X64 = _os.environ.get("JAXSHIM_X64") == "1"

_CANON = {} if X64 else {_np.dtype(_np.float64): _np.float32, _np.dtype(_np.int64): _np.int32,
                         _np.dtype(_np.uint64): _np.uint32, _np.dtype(_np.complex128): _np.complex64}


def _canon(a):
    t = _CANON.get(a.dtype)
    return a.astype(t) if t is not None else a


def _unwrap(x):
    if isinstance(x, JArr):
        return x.view(_np.ndarray)
    if isinstance(x, (list, tuple)):
        return type(x)(_unwrap(v) for v in x)
    if isinstance(x, dict):
        return {k: _unwrap(v) for k, v in x.items()}
    if isinstance(x, _np.generic) and not X64 and x.dtype in _CANON:
        return _CANON[x.dtype](x)
    return x


def _wrap(r):
    if isinstance(r, JArr):
        return r
    if isinstance(r, _np.ndarray):
        return _canon(r).view(JArr)
    if isinstance(r, _np.generic):
        return _canon(_np.asarray(r)).view(JArr)
    if isinstance(r, tuple):
        return tuple(_wrap(v) for v in r)
    if isinstance(r, list):
        return [_wrap(v) for v in r]
    return r


def _matmul(a, b):
    a, b = _np.asarray(a), _np.asarray(b)
    if a.ndim == 2 and b.ndim == 2:  # sum of products, k order
        return _np.add.reduce(a[:, :, None] * b[None, :, :], axis=1)
    if a.ndim == 2 and b.ndim == 1:
        return _np.add.reduce(a * b[None, :], axis=1)
    return _np.matmul(a, b)


class _At:
    def __init__(self, a):
        self.a = a

    def __getitem__(self, idx):
        return _AtIdx(self.a, _unwrap(idx))


class _AtIdx:
    def __init__(self, a, idx):
        self.a, self.idx = a, idx

    def set(self, v):
        r = _np.array(_unwrap(self.a))
        r[self.idx] = _unwrap(v)
        return _wrap(r)

    def add(self, v):
        r = _np.array(_unwrap(self.a))
        _np.add.at(r, self.idx, _unwrap(v))
        return _wrap(r)

    def get(self):
        return _wrap(_np.asarray(_unwrap(self.a))[self.idx])


class JArr(_np.ndarray):
    __array_priority__ = 100

    def __array_ufunc__(self, ufunc, method, *inputs, **kw):
        if ufunc is _np.matmul:
            return _wrap(_matmul(*_unwrap(inputs)))
        ins = _unwrap(inputs)
        if "out" in kw:
            kw["out"] = _unwrap(kw["out"])
        return _wrap(getattr(ufunc, method)(*ins, **kw))

    def __array_function__(self, func, types, args, kwargs):
        return _wrap(func(*_unwrap(args), **_unwrap(kwargs)))

    def __getitem__(self, idx):
        return _wrap(_np.ndarray.__getitem__(self.view(_np.ndarray), _unwrap(idx)))

    def __matmul__(self, o):
        return _wrap(_matmul(_unwrap(self), _unwrap(o)))

    def __rmatmul__(self, o):
        return _wrap(_matmul(_unwrap(o), _unwrap(self)))

    def astype(self, dt, **kw):
        return _wrap(_np.asarray(self.view(_np.ndarray)).astype(dt))

    @property
    def at(self):
        return _At(self)

    def __bool__(self):
        return bool(self.view(_np.ndarray))

    def __float__(self):
        return float(self.view(_np.ndarray))

    def __int__(self):
        return int(self.view(_np.ndarray))

    def __index__(self):
        return int(self.view(_np.ndarray))

    def tolist(self):
        return self.view(_np.ndarray).tolist()

    def block_until_ready(self):
        return self


def _fn(name):
    f = getattr(_np, name)

    def g(*a, **k):
        return _wrap(f(*_unwrap(a), **_unwrap(k)))
    g.__name__ = name
    return g


def array(x, dtype=None, **k):
    return _wrap(_np.array(_unwrap(x), dtype=dtype))


asarray = array


def dot(a, b):
    a, b = _np.asarray(_unwrap(a)), _np.asarray(_unwrap(b))
    if a.ndim == 1 and b.ndim == 1:
        return _wrap(_np.add.reduce(a * b))
    return _wrap(_matmul(a, b))


def einsum(spec, *ops, **k):
    return _wrap(_np.einsum(spec, *[_np.asarray(_unwrap(o)) for o in ops], optimize=False))


def _norm(x, ord=None, axis=None, keepdims=False):
    x = _np.asarray(_unwrap(x))
    if axis is None:
        x = x.ravel()
        axis = 0
    return _wrap(_np.sqrt(_np.add.reduce(x * x, axis=axis, keepdims=keepdims)))


linalg = _types.SimpleNamespace(norm=_norm)

_PASS = {"pi", "inf", "nan", "e", "newaxis", "float32", "float64", "int32", "int64", "uint32", "bool_", "complex64",
         "complex128", "ndarray", "dtype", "float16", "int8", "uint8", "int16"}


def __getattr__(name):
    if name in _PASS:
        return getattr(_np, name)
    if hasattr(_np, name) and callable(getattr(_np, name)):
        return _fn(name)
    raise AttributeError(name)


_sys.modules[__name__ + ".linalg"] = linalg
