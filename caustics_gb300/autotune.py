"""Launch-shape autotuner for the batched light-curve kernels.

Tunes, by timing candidates on (a sample of) the caller's workload:
* threads per contour-kernel CTA (128 or 256): with one CTA per extended-source
  evaluation this sets how many limb points and contour points a block works
  on at once, and how many evaluations share an SM;
* the persistent grid of the contour kernel (occupancy-sized, or one CTA per SM);
* the device work-queue chunk (items taken per queue grab);
* the lanes that share one contour point's Gauss-Legendre nodes;
* threads per polynomial in the per-point pass (one thread per point, or a
  group of 8 lanes with one lane per root), tried on the best shape found.
Results are cached per (device, npts_limb, limb darkening, npts_ld, precision,
labelling, workload size bucket, share of points on curves with q < 0.01): the
last two decide how many evaluations reach the contour kernel and how uneven
they are.
"""
import itertools
import math

import numpy as np
import torch

DEFAULT = dict(grid=0, queue_chunk=1, ld_group=1, cta_threads=0, point_lanes=0)
_CACHE = {}


def _sample(offsets, t, curves, max_points):
    off = offsets.cpu().numpy()
    c = int(np.searchsorted(off, max_points, side="right")) - 1
    c = max(1, min(c, len(off) - 1))
    n = int(off[c])
    return offsets[:c + 1], t[:n], curves[:c]


def cache_key(dev, offsets, curves, **kw):
    """(device, options..., log2 bucket of the point count, share of points on
    curves with q < 0.01 in tenths)."""
    off = offsets.cpu().numpy()
    lens = np.diff(off)
    q = curves[:, 1].cpu().numpy()
    n = int(off[-1])
    small_q = float((lens * (q < 0.01)).sum()) / max(n, 1)
    return (torch.cuda.get_device_name(dev), tuple(sorted(kw.items())), int(math.log2(max(n, 1))),
            int(round(10 * small_q)))


def tune(offsets, t, curves, npts_limb=200, limb_darkening=False, npts_ld=100, roots_itmax=2500, precision="mixed",
         max_points=4096, reps=2, verbose=False, labelling="reference"):
    from . import api
    offsets, _ = api._to_device(offsets, torch.int64)
    t, _ = api._to_device(t, torch.float64)
    curves, _ = api._to_device(curves, torch.float64)
    dev = t.device
    kw = dict(npts_limb=npts_limb, limb_darkening=limb_darkening, npts_ld=npts_ld, roots_itmax=roots_itmax,
              precision=precision, labelling=labelling)
    key = cache_key(dev, offsets, curves, **kw)
    if key in _CACHE:
        return dict(_CACHE[key])
    so, st, sc = _sample(offsets, t, curves, max_points)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    cands = []
    for threads, chunk, group in itertools.product((128, 256), (1, 2, 4), (1, 2, 4)):
        cands.append(dict(grid=0, queue_chunk=chunk, ld_group=group, cta_threads=threads))
    cands += [dict(grid=sms, queue_chunk=c, ld_group=g, cta_threads=256) for c, g in itertools.product((1, 2), (1, 2))]
    best, best_ms, table = None, float("inf"), []

    def trial(cfg):
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
        return m

    for cfg in cands:
        m = trial(dict(cfg, point_lanes=1))
        if m < best_ms:
            best, best_ms = dict(cfg, point_lanes=1), m
    cfg = dict(best, point_lanes=8)
    m = trial(cfg)
    if m < best_ms:
        best, best_ms = cfg, m
    if verbose:
        for cfg, m in table:
            print(cfg, f"{m:.3f} ms")
    _CACHE[key] = dict(best)
    return dict(best)
