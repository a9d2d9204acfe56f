"""Minimal equinox stand-in: Module, field, tree_at."""
import copy as _copy


class _Field:
    def __init__(self, static=False, **kw):
        self.static = static


def field(static=False, **kw):
    return _Field(static)


class Module:
    def __init_subclass__(cls, **kw):
        super().__init_subclass__(**kw)
        if "__init__" not in cls.__dict__:
            names = []
            for klass in reversed(cls.__mro__):
                for n in getattr(klass, "__annotations__", {}):
                    if n not in names and not isinstance(klass.__dict__.get(n), property):
                        names.append(n)

            def __init__(self, *args, **kwargs):
                for n, v in zip(names, args):
                    object.__setattr__(self, n, v)
                for n, v in kwargs.items():
                    object.__setattr__(self, n, v)
            cls.__init__ = __init__

    @classmethod
    def _shim_static_fields(cls):
        out = set()
        for klass in cls.__mro__:
            for n, v in klass.__dict__.items():
                if isinstance(v, _Field) and v.static:
                    out.add(n)
        return out


class _Rec:
    def __init__(self, path):
        self._path = path

    def __getattr__(self, n):
        return _Rec(self._path + [n])


def _set(obj, path, val):
    if len(path) == 1:
        object.__setattr__(obj, path[0], val)
        return
    child = _copy.copy(getattr(obj, path[0]))
    _set(child, path[1:], val)
    object.__setattr__(obj, path[0], child)


def tree_at(where, pytree, replace=None, replace_fn=None, is_leaf=None):
    sel = where(_Rec([]))
    new = _copy.copy(pytree)
    if isinstance(sel, tuple):
        for s, v in zip(sel, replace):
            _set(new, s._path, v)
    else:
        _set(new, sel._path, replace)
    return new


def filter_jit(f=None, **kw):
    return f if f is not None else (lambda g: g)
