"""Keys are uint32 pairs; every draw seeds numpy's Generator from the key."""
import numpy as _np

from .numpy import _unwrap, _wrap, X64

LOG = []  # (kind, shape, values) of every draw, for fixtures that want them


def _rng(key):
    k = _np.asarray(_unwrap(key)).astype(_np.uint64).ravel().tolist()
    return _np.random.default_rng([int(v) for v in k] + [0x1ACE])


def PRNGKey(seed):
    return _wrap(_np.array([0, int(seed) & 0xFFFFFFFF], _np.uint32))


key = PRNGKey


def split(key, num=2):
    r = _rng(key)
    return _wrap(r.integers(0, 2**32, size=(num, 2), dtype=_np.uint64).astype(_np.uint32))


def _shape(shape):
    return tuple(shape) if isinstance(shape, (tuple, list)) else ((shape,) if shape is not None else ())


def _ft():
    return _np.float64 if X64 else _np.float32


def uniform(key, shape=(), dtype=None, minval=0.0, maxval=1.0):
    u = _rng(key).random(_shape(shape)).astype(dtype or _ft())
    u = u * (maxval - minval) + minval
    LOG.append(("uniform", _shape(shape), _np.array(u)))
    return _wrap(u.astype(dtype or _ft()))


def normal(key, shape=(), dtype=None):
    v = _rng(key).standard_normal(_shape(shape)).astype(dtype or _ft())
    LOG.append(("normal", _shape(shape), _np.array(v)))
    return _wrap(v)


def choice(key, a, shape=(), replace=True, p=None, axis=0):
    p = None if p is None else _np.asarray(_unwrap(p), _np.float64)
    if p is not None:
        p = p / p.sum()
    n = a if isinstance(a, int) else len(a)
    v = _rng(key).choice(n, size=_shape(shape), replace=replace, p=p).astype(_np.int32)
    LOG.append(("choice", _shape(shape), _np.array(v)))
    return _wrap(v)
