import numpy as _np

from .numpy import _wrap


def cond(pred, true_fun, false_fun, *operands):
    return true_fun(*operands) if bool(pred) else false_fun(*operands)


def switch(index, branches, *operands):
    i = int(_np.clip(int(index), 0, len(branches) - 1))
    return branches[i](*operands)


def _stack_tree(outs):
    first = outs[0]
    if isinstance(first, (tuple, list)):
        return type(first)(_stack_tree([o[k] for o in outs]) for k in range(len(first)))
    return _wrap(_np.stack([_np.asarray(o) for o in outs]))


def _slice_tree(xs, i):
    if isinstance(xs, (tuple, list)):
        return type(xs)(_slice_tree(x, i) for x in xs)
    return _wrap(_np.asarray(xs)[i])


def _length(xs):
    if isinstance(xs, (tuple, list)):
        return _length(xs[0])
    return _np.shape(xs)[0]


def scan(f, init, xs, length=None):
    n = length if xs is None else _length(xs)
    carry = init
    ys = []
    for i in range(n):
        x = None if xs is None else _slice_tree(xs, i)
        carry, y = f(carry, x)
        ys.append(y)
    return carry, (_stack_tree(ys) if ys else None)


def map(f, xs):
    n = _length(xs)
    return _stack_tree([f(_slice_tree(xs, i)) for i in range(n)])


def dynamic_slice(x, start_indices, slice_sizes):
    x = _np.asarray(x)
    sl = []
    for s, size, dim in zip(start_indices, slice_sizes, x.shape):
        s = int(min(max(int(s), 0), dim - size))
        sl.append(slice(s, s + size))
    return _wrap(x[tuple(sl)])


def zeros_like_array(x):
    return _wrap(_np.zeros_like(_np.asarray(x)))
