"""Light curves across ranks (one process per GPU): the units are independent,
so each rank evaluates its own subset and nothing crosses ranks on the data
path; the magnifications are gathered at the end.

Curves are assigned by estimated cost (length x the expected fraction of points
that need the contour integral: every point when q < 0.01, because the
reference's planetary-caustic test always fails there, and about half
otherwise), greedily to the least-loaded rank, heaviest first."""
import numpy as np


def curve_costs(offsets, curves):
    offsets = np.asarray(offsets, dtype=np.int64)
    curves = np.asarray(curves, dtype=np.float64)
    lengths = np.diff(offsets).astype(np.float64)
    full_fraction = np.where(curves[:, 1] < 0.01, 1.0, 0.5)
    return lengths * full_fraction


def partition(offsets, curves, world_size):
    """List of curve-index arrays, one per rank (sorted within a rank)."""
    cost = curve_costs(offsets, curves)
    load = np.zeros(world_size)
    parts = [[] for _ in range(world_size)]
    for c in np.argsort(-cost, kind="stable"):
        r = int(np.argmin(load))
        parts[r].append(int(c))
        load[r] += cost[c]
    return [np.array(sorted(p), dtype=np.int64) for p in parts]


def local_problem(offsets, t, curves, indices):
    """(offsets, t, curves) of the given curves, renumbered from 0, and the
    global point index of every local point."""
    offsets = np.asarray(offsets, dtype=np.int64)
    pts = [np.arange(offsets[c], offsets[c + 1]) for c in indices]
    idx = np.concatenate(pts) if pts else np.zeros(0, dtype=np.int64)
    lens = np.array([len(p) for p in pts], dtype=np.int64)
    loc_off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    return loc_off, np.asarray(t)[idx], np.asarray(curves)[indices], idx


def gather(local_values, global_index, npoints, group=None):
    """Every rank's local results into the global order on every rank
    (torch.distributed all_gather of (index, value) pairs of uneven sizes)."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    vals = torch.as_tensor(np.asarray(local_values, dtype=np.float64))
    idx = torch.as_tensor(np.asarray(global_index, dtype=np.int64))
    n = torch.tensor([vals.numel()], dtype=torch.int64)
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    cap = int(max(int(s) for s in sizes))
    pv = torch.zeros(cap, dtype=torch.float64)
    pi = torch.full((cap,), -1, dtype=torch.int64)
    pv[:vals.numel()] = vals
    pi[:idx.numel()] = idx
    all_v = [torch.zeros(cap, dtype=torch.float64) for _ in range(world)]
    all_i = [torch.zeros(cap, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(all_v, pv, group=group)
    dist.all_gather(all_i, pi, group=group)
    out = np.full(npoints, np.nan)
    for v, i, s in zip(all_v, all_i, sizes):
        k = int(s)
        out[i[:k].numpy()] = v[:k].numpy()
    return out
