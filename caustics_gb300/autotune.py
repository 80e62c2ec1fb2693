"""Launch-shape autotuner for the batched light-curve kernels.

Tunes, by timing candidates on (a sample of) the caller's workload:
* the persistent grid of the contour kernel (CTAs per SM),
* the device work-queue chunk (items taken per queue grab),
* the lanes that share one contour point's Gauss-Legendre nodes.
Results are cached per (device, npts_limb, limb darkening, npts_ld, precision).
"""
import itertools

import numpy as np
import torch

DEFAULT = dict(grid=0, queue_chunk=1, ld_group=1)
_CACHE = {}


def _sample(offsets, t, curves, max_points):
    off = offsets.cpu().numpy()
    c = int(np.searchsorted(off, max_points, side="right")) - 1
    c = max(1, min(c, len(off) - 1))
    n = int(off[c])
    return offsets[:c + 1], t[:n], curves[:c]


def tune(offsets, t, curves, npts_limb=200, limb_darkening=False, npts_ld=100, roots_itmax=2500, precision="mixed",
         max_points=4096, reps=2, verbose=False, labelling="reference"):
    from . import api
    offsets, _ = api._to_device(offsets, torch.int64)
    t, _ = api._to_device(t, torch.float64)
    curves, _ = api._to_device(curves, torch.float64)
    dev = t.device
    key = (torch.cuda.get_device_name(dev), int(npts_limb), bool(limb_darkening), int(npts_ld), str(precision),
           str(labelling))
    if key in _CACHE:
        return dict(_CACHE[key])
    so, st, sc = _sample(offsets, t, curves, max_points)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    kw = dict(npts_limb=npts_limb, limb_darkening=limb_darkening, npts_ld=npts_ld, roots_itmax=roots_itmax,
              precision=precision, labelling=labelling)
    best, best_ms, table = None, float("inf"), []
    for per_sm, chunk, group in itertools.product((1, 2), (1, 2, 4), (1, 2, 4)):
        cfg = dict(grid=per_sm * sms, queue_chunk=chunk, ld_group=group)
        api.mag_lc_batched(so, st, sc, **kw, **cfg)
        ms = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            api.mag_lc_batched(so, st, sc, **kw, **cfg)
            e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        m = float(np.median(ms))
        table.append((cfg, m))
        if m < best_ms:
            best, best_ms = cfg, m
    if verbose:
        for cfg, m in table:
            print(cfg, f"{m:.3f} ms")
    _CACHE[key] = dict(best)
    return dict(best)
