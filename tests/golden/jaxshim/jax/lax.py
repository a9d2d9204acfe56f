from . import _stack


def scan(f, init, xs=None, length=None, **kw):
    carry = init
    n = length if xs is None else len(xs)
    ys = []
    for i in range(n):
        carry, y = f(carry, None if xs is None else xs[i])
        ys.append(y)
    if not ys or all(y is None for y in ys):
        return carry, None
    return carry, _stack(ys)


def cond(pred, true_fun, false_fun, operand=None):
    return true_fun(operand) if bool(pred) else false_fun(operand)
