"""A NumPy stand-in for the small part of the JAX API that the reference
caustics package uses.  Test infrastructure only: it lets tests/golden/make_golden.py
run the reference's unmodified Python source in a container without JAX, to
produce golden fixtures.  Semantics emulated on purpose:

* out-of-range integer gathers clamp to the last element (JAX gather "clip");
  out-of-range scatters through ``.at[i].set`` are dropped;
* ``lax.cond`` / ``lax.switch`` are lazy (only the taken branch runs);
* ``argsort`` is stable;
* ``random`` draws are deterministic per key but are NOT JAX's threefry stream
  (only used for +-1e-6 / +-1e-9 jitter in the reference).
"""
import numpy as _np

from . import numpy  # noqa: F401
from . import lax  # noqa: F401
from . import random  # noqa: F401
from . import config as _config_mod  # noqa: F401
from . import scipy  # noqa: F401
from .numpy import _wrap

config = _config_mod.config


def jit(fun=None, **kwargs):
    if fun is None:
        return lambda f: f
    return fun


def _take(a, i, ax):
    return _wrap(_np.take(_np.asarray(a), i, axis=ax))


def _stack_tree(outs):
    first = outs[0]
    if isinstance(first, (tuple, list)):
        return type(first)(_stack_tree([o[k] for o in outs]) for k in range(len(first)))
    return _wrap(_np.stack([_np.asarray(o) for o in outs]))


def vmap(fun, in_axes=0, out_axes=0):
    def mapped(*args):
        axes = list(in_axes) if isinstance(in_axes, (list, tuple)) else [in_axes] * len(args)
        n = None
        for a, ax in zip(args, axes):
            if ax is not None:
                n = _np.shape(a)[ax]
                break
        outs = []
        for i in range(n):
            call = [(_take(a, i, ax) if ax is not None else a) for a, ax in zip(args, axes)]
            outs.append(fun(*call))
        return _stack_tree(outs)

    return mapped


def jacfwd(*a, **k):
    raise NotImplementedError("autodiff is not available in the NumPy stand-in")


jacrev = jacfwd
grad = jacfwd
