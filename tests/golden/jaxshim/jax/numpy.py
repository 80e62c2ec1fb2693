"""jax.numpy stand-in: NumPy with JAX's clamped gathers, dropped out-of-range
scatters, ``.at[...]`` updates, stable argsort and ``size=`` arguments."""
import numpy as _np

_np.seterr(all="ignore")

complex128 = _np.complex128
float64 = _np.float64
int32 = _np.int32
int64 = _np.int64
bool_ = _np.bool_
ndarray = _np.ndarray
pi = _np.pi
inf = _np.inf
nan = _np.nan


def _is_int(x):
    return isinstance(x, (int, _np.integer)) and not isinstance(x, (bool, _np.bool_)) or (
        isinstance(x, _np.ndarray) and x.ndim == 0 and _np.issubdtype(x.dtype, _np.integer))


def _fix_index(idx, shape, mode):
    """Normalise a (tuple) index.  mode 'clip' clamps ints; mode 'drop' returns None
    when an int index is out of range."""
    if not isinstance(idx, tuple):
        idx = (idx,)
    n_real = sum(1 for e in idx if e is not None and e is not Ellipsis and not (
        isinstance(e, _np.ndarray) and e.dtype == bool))
    out = []
    dim = 0
    for e in idx:
        if e is Ellipsis:
            out.append(e)
            dim += len(shape) - n_real
            continue
        if e is None:
            out.append(e)
            continue
        if _is_int(e):
            n = shape[dim]
            i = int(e)
            if i < 0:
                i += n
            if i < 0 or i >= n:
                if mode == "drop":
                    return None
                i = min(max(i, 0), n - 1)
            out.append(i)
        elif isinstance(e, (list, _np.ndarray)) and _np.asarray(e).dtype != bool and _np.issubdtype(_np.asarray(e).dtype, _np.integer):
            n = shape[dim]
            a = _np.asarray(e).astype(_np.int64)
            a = _np.where(a < 0, a + n, a)
            if mode == "drop" and (_np.any(a < 0) or _np.any(a >= n)):
                keep = (a >= 0) & (a < n)
                a = a[keep]
            out.append(_np.clip(a, 0, n - 1))
        else:
            out.append(e)
        dim += 1
    return tuple(out)


class _At:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _AtIdx(self.arr, idx)


class _AtIdx:
    def __init__(self, arr, idx):
        self.arr, self.idx = arr, idx

    def set(self, values, *args, **kwargs):
        out = _np.array(self.arr, copy=True)
        idx = _fix_index(self.idx, out.shape, "drop")
        if idx is not None:
            out[idx] = _np.asarray(values)
        return _wrap(out)

    def add(self, values, *args, **kwargs):
        out = _np.array(self.arr, copy=True)
        idx = _fix_index(self.idx, out.shape, "drop")
        if idx is not None:
            out[idx] += _np.asarray(values)
        return _wrap(out)

    def get(self, *args, **kwargs):
        return self.arr[self.idx]


class Array(_np.ndarray):
    def __new__(cls, x):
        return _np.asarray(x).view(cls)

    @property
    def at(self):
        return _At(self)

    def __getitem__(self, idx):
        fixed = _fix_index(idx, self.shape, "clip")
        r = _np.ndarray.__getitem__(self.view(_np.ndarray), fixed)
        return _wrap(r)

    def __iter__(self):
        for i in range(self.shape[0]):
            yield self[i]

    # JAX arrays are immutable: augmented assignment rebinds instead of mutating
    def __iadd__(self, o):
        return _wrap(_np.add(self.view(_np.ndarray), _unwrap(o)))

    def __isub__(self, o):
        return _wrap(_np.subtract(self.view(_np.ndarray), _unwrap(o)))

    def __imul__(self, o):
        return _wrap(_np.multiply(self.view(_np.ndarray), _unwrap(o)))

    def __itruediv__(self, o):
        return _wrap(_np.true_divide(self.view(_np.ndarray), _unwrap(o)))

    def __array_wrap__(self, arr, context=None, return_scalar=False):
        if return_scalar:
            return arr[()]
        return arr.view(Array) if isinstance(arr, _np.ndarray) else arr


def _wrap(x):
    if isinstance(x, Array):
        return x
    if isinstance(x, _np.ndarray):
        return x.view(Array)
    if isinstance(x, tuple):
        return tuple(_wrap(e) for e in x)
    if isinstance(x, list):
        return [_wrap(e) for e in x]
    return x


def _unwrap(x):
    if isinstance(x, Array):
        return x.view(_np.ndarray)
    if isinstance(x, (list, tuple)):
        return type(x)(_unwrap(e) for e in x)
    return x


def array(x, dtype=None, copy=True):
    return _wrap(_np.array(_unwrap(x), dtype=dtype))


def asarray(x, dtype=None):
    return _wrap(_np.asarray(_unwrap(x), dtype=dtype))


def argsort(a, axis=-1, kind=None, order=None):
    return _wrap(_np.argsort(_unwrap(a), axis=axis, kind="stable"))


def sort(a, axis=-1, kind=None, order=None):
    return _wrap(_np.sort(_unwrap(a), axis=axis, kind="stable"))


def trapz(y, x=None, dx=1.0, axis=-1):
    return _wrap(_np.trapezoid(_unwrap(y), x=_unwrap(x), dx=dx, axis=axis))


def argwhere(a, *, size=None, fill_value=None):
    r = _np.argwhere(_unwrap(a))
    if size is not None:
        fv = 0 if fill_value is None else fill_value
        out = _np.full((size, r.shape[1]), fv, dtype=r.dtype)
        m = min(size, r.shape[0])
        out[:m] = r[:m]
        r = out
    return _wrap(r)


def unique(a, return_index=False, size=None, fill_value=None, **kw):
    a = _np.asarray(_unwrap(a))
    if return_index:
        u, ix = _np.unique(a, return_index=True)
        if size is not None:
            uu = _np.full(size, u[0] if fill_value is None else fill_value, dtype=u.dtype)
            ii = _np.zeros(size, dtype=ix.dtype)
            m = min(size, len(u))
            uu[:m], ii[:m] = u[:m], ix[:m]
            u, ix = uu, ii
        return _wrap(u), _wrap(ix)
    u = _np.unique(a)
    if size is not None:
        uu = _np.full(size, u[0] if fill_value is None else fill_value, dtype=u.dtype)
        m = min(size, len(u))
        uu[:m] = u[:m]
        u = uu
    return _wrap(u)


def __getattr__(name):
    f = getattr(_np, name)
    if callable(f):
        def g(*args, **kwargs):
            return _wrap(f(*_unwrap(args), **{k: _unwrap(v) for k, v in kwargs.items()}))
        return g
    return f
