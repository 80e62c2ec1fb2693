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
    seed = int.from_bytes(_np.asarray(key, dtype=_np.uint32).tobytes(), "little")
    rng = _np.random.default_rng(seed)
    return _wrap(rng.uniform(minval, maxval, size=shape))
