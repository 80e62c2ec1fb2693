"""jax.random stand-in.  The reference draws only small warm-start
perturbations from it (extended_source.py:76-85, 144-148).  JAX's threefry
stream cannot be reproduced here, so the stand-in returns a documented fixed
pattern instead: for the two keys split from PRNGKey(0), row t of the drawn
array is +-(maxval - minval)/4, the sign taken from bit 0 (first key) or bit 1
(second key) of t.  The oracle and the CUDA kernels perturb warm starts with the
same pattern."""
import hashlib

import numpy as _np

from .numpy import _wrap


def PRNGKey(seed):
    return _np.array([0, int(seed) & 0xFFFFFFFF], dtype=_np.uint32)


def _derive(key, salt):
    h = hashlib.sha256(_np.asarray(key, dtype=_np.uint32).tobytes() + salt.to_bytes(4, "little")).digest()
    return _np.frombuffer(h[:8], dtype=_np.uint32).copy()


def split(key, num=2):
    return _np.stack([_derive(key, i + 1) for i in range(num)])


def uniform(key, shape=(), dtype=None, minval=0.0, maxval=1.0):
    key = _np.asarray(key, dtype=_np.uint32)
    first, second = split(PRNGKey(0))
    shape = tuple(shape) if _np.ndim(shape) else (shape,)
    half = 0.25 * (maxval - minval)
    if len(shape) >= 1 and (_np.array_equal(key, first) or _np.array_equal(key, second)):
        bit = 0 if _np.array_equal(key, first) else 1
        t = _np.arange(shape[0]).reshape((-1,) + (1,) * (len(shape) - 1))
        out = _np.broadcast_to(_np.where((t >> bit) & 1, half, -half) + 0.5 * (maxval + minval), shape)
        return _wrap(_np.array(out, dtype=_np.float64))
    seed = int.from_bytes(key.tobytes(), "little")
    return _wrap(_np.random.default_rng(seed).uniform(minval, maxval, size=shape))
