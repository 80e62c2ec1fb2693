#!/usr/bin/env python
"""Benchmark of the extended-source magnification hot path on one GB300.

Headline workload (the largest single-GPU configuration): 4096 binary-lens
limb-darkened light curves of uneven lengths, seed 2: per curve s ~ logU[0.3,
3], q ~ logU[1e-4, 1], rho ~ logU[1e-3, 1e-1], u0 ~ U[-0.3, 0.3], alpha ~
U[0, 2pi], u1 ~ U[0.2, 0.8], tE ~ logU[5, 100], t0 = 0, length ~ U{200..5000},
times uniform on [t0 - 2tE, t0 + 2tE]; npts_limb 200, npts_ld 100 (mag()'s
defaults).  10,596,037 points, of which 5,833,735 take the contour integral
(every point of the curves with q < 0.01, where the reference's planetary test
rejects the hexadecapole).

A step is one batched mixed-precision pass (CUDA-graph replay of the per-point
pass, the first-point ordering kernel and the persistent contour kernel) over
one batch of curves: the 4096 curves are dealt, in order, into K contiguous
batches of about equal estimated cost, so the K timed steps evaluate the whole
workload exactly once.

value   = light-curve magnification evaluations/s (every point counts),
          device-timed (CUDA events on the launching stream), inputs resident
          in HBM, L2 flushed between timed steps (256 MiB write > 129 MB L2);
e2e     = the same through the public API (mag_lc_batched) from pinned host
          buffers, host->device and device->host copies inside the timed region;
vjp     = VJP evaluations/s (mag_lc_batched_vjp) on 256 curves x 1000 points
          (seed 3), N(0,1) cotangent, with its own roofline.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--quick]
"""
import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NCURVES, SEED, NMIN, NMAX = 4096, 2, 200, 5000
LC = dict(npts_limb=200, limb_darkening=True, npts_ld=100)
WL = dict(workload="binary-ld-lightcurves-4096-uneven", ncurves=NCURVES, seed=SEED, lengths="U{200..5000}",
          npoints=10596037, npts_limb=200, npts_ld=100, limb_darkening=True,
          params="s~logU[0.3,3], q~logU[1e-4,1], rho~logU[1e-3,1e-1], u0~U[-0.3,0.3], alpha~U[0,2pi], "
                 "u1~U[0.2,0.8], tE~logU[5,100], t0=0, t~U[t0-2tE, t0+2tE]")
METRIC = "extended-source magnification evals/s (light-curve points, batched mixed precision, <=1e-4 rel err)"
UNIT = "evals/s"
VJP_METRIC = "extended-source magnification VJP evals/s (light-curve points, batched mixed precision)"
# Nominal FP64-equivalent work (flop) per unit: a full contour evaluation at
# npts_limb = L, npts_ld = G is L root solves (5.7e3 flop) + ~3.1 L contour points
# x 2G nodes x 60 flop; a hexadecapole-routed point is one binary point-source
# solve (5.7e3) + the hexadecapole and tests (8e3); the VJP is ~3x its forward.
F_PS2, F_HEX = 5.7e3, 8e3


def f_es(L, G):
    return L * 5.7e3 + 3.1 * L * G * 2 * 60


# Per contour evaluation of es_kernel<2, MIXED> (npts_limb 200, npts_ld 100),
# from one ncu capture of a contour-kernel launch (profiles/), divided by the
# evaluations of that launch: DRAM bytes read + written (instructions,
# constants, spills; the inputs are 24 B per point), and the executed FP64 and
# FP32 arithmetic (dadd + dmul + 2 dfma, fadd + fmul + 2 ffma thread
# instructions).
NCU_EVALS = 2764
DRAM_BYTES_PER_EVAL = 6.547e6 / NCU_EVALS
FP64_FLOP_PER_EVAL = 1.2939e9 / NCU_EVALS
FP32_FLOP_PER_EVAL = 2.3732e10 / NCU_EVALS
FP64_PIPE_BUSY_NCU = 0.581
# the same for es_kernel<2, MIXED, GRAD> (the VJP's contour kernel), one
# launch over 2000 contour evaluations of the gradient workload
NCU_EVALS_VJP = 2000
DRAM_BYTES_PER_EVAL_VJP = 13.89e6 / NCU_EVALS_VJP
FP64_FLOP_PER_EVAL_VJP = 3.3826e9 / NCU_EVALS_VJP
FP32_FLOP_PER_EVAL_VJP = 6.1482e10 / NCU_EVALS_VJP
FP64_PIPE_BUSY_NCU_VJP = 0.671


def draw_batched(ncurves_total, seed, nmin, nmax, take):
    """Curves drawn as the reference-scale batched workloads: per curve
    s ~ logU[0.3, 3], q ~ logU[1e-4, 1], rho ~ logU[1e-3, 1e-1], u0 ~ U[-0.3, 0.3],
    alpha ~ U[0, 2pi], u1 ~ U[0.2, 0.8], tE ~ logU[5, 100], t0 = 0, length
    ~ U{nmin..nmax}, times uniform on [t0 - 2tE, t0 + 2tE]; the first `take`
    curves of the full draw."""
    rng = np.random.default_rng(seed)
    n = ncurves_total
    lens = rng.integers(nmin, nmax + 1, n)
    cv = np.stack([10 ** rng.uniform(np.log10(0.3), np.log10(3), n), 10 ** rng.uniform(-4, 0, n),
                   10 ** rng.uniform(-3, -1, n), rng.uniform(0.2, 0.8, n), rng.uniform(-0.3, 0.3, n),
                   rng.uniform(0, 2 * np.pi, n), np.zeros(n), 10 ** rng.uniform(np.log10(5), 2, n)], axis=1)
    ts = [np.sort(rng.uniform(-2 * te, 2 * te, m)) for te, m in zip(cv[:take, 7], lens[:take])]
    offsets = np.concatenate([[0], np.cumsum(lens[:take])]).astype(np.int64)
    return offsets, np.concatenate(ts), cv[:take]


def batches(offsets, cv, k):
    """Contiguous curve ranges [c0, c1) of about equal estimated cost (points x
    1 for q < 0.01, where every point takes the contour integral, else x 0.15)."""
    lens = np.diff(offsets)
    cost = lens * np.where(cv[:, 1] < 0.01, 1.0, 0.15)
    cum = np.cumsum(cost)
    edges = [0] + [int(np.searchsorted(cum, cum[-1] * j / k)) + 1 for j in range(1, k)] + [len(lens)]
    edges = np.maximum.accumulate(np.minimum(edges, len(lens)))
    return [(int(a), int(b)) for a, b in zip(edges[:-1], edges[1:]) if b > a]


def trajectory(t, cv):
    tau = (t - cv[6]) / cv[7]
    return (cv[4] * np.cos(cv[5]) + tau * np.sin(cv[5])) + 1j * (-cv[4] * np.sin(cv[5]) + tau * np.cos(cv[5]))


# ---------------------------------------------------------------------------
# CPU baseline (the oracle restatement of the reference, process pool)
# ---------------------------------------------------------------------------

def _oracle_points(job):
    sys.path.insert(0, ROOT)
    from oracle import caustics_oracle as O
    out = []
    for t, cv in job:
        out.append(float(O.mag(np.atleast_1d(trajectory(t, cv)), cv[2], u1=cv[3], s=cv[0], q=cv[1], **LC)[0]))
    return out


def _cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def make_pool(n):
    ctx = mp.get_context("spawn")
    pool = ctx.Pool(n)
    pool.map(_oracle_points, [[(0.0, np.array([1.0, 0.5, 1e-2, 0.5, 1.0, 0.3, 0.0, 10.0]))]] * n)  # warm each worker
    return pool


_DRAW = None


def cpu_rate(pool, cores, per_core, seed):
    """Light-curve points/s of the oracle on a uniform random sample of the
    workload's points (each with its own curve's parameters)."""
    global _DRAW
    if _DRAW is None:
        _DRAW = draw_batched(NCURVES, SEED, NMIN, NMAX, NCURVES)
    off, t, cv = _DRAW
    rng = np.random.default_rng(100 + seed)
    pick = np.sort(rng.choice(len(t), size=per_core * cores, replace=False))
    cid = np.searchsorted(off, pick, side="right") - 1
    jobs = [[(t[i], cv[c]) for i, c in zip(pick[j::cores], cid[j::cores])] for j in range(cores)]
    t0 = time.perf_counter()
    pool.map(_oracle_points, jobs)
    return len(pick) / (time.perf_counter() - t0), len(pick)


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        time.sleep(0.3)
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# reference arm
# ---------------------------------------------------------------------------

def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = _cores()
    pool = make_pool(cores)
    for k in range(args.warmup):
        cpu_rate(pool, cores, per_core=2, seed=1000 + k)
    rates, n = [], 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        r, n = cpu_rate(pool, cores, per_core=6, seed=k)
        rates.append(r)
    wall = time.perf_counter() - t0
    pool.close()
    value = float(np.mean(rates))
    sample = (f"{n} points per step drawn uniformly from the workload's 10,596,037 (each with its curve's "
              f"parameters); oracle restatement of the reference (NumPy + C solver), spawn pool")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(WL),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------

def timed(stream, fn, reps=1, flush=None):
    import torch
    ms = []
    for _ in range(reps):
        if flush is not None:
            flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    return float(np.mean(ms))


def _counted(nfull, ms, peaks, vjp=False):
    """The contour evaluations' executed arithmetic (ncu counts per evaluation)
    at the measured rate, against the live FMA peaks of each pipe."""
    f64e, f32e, busy = ((FP64_FLOP_PER_EVAL_VJP, FP32_FLOP_PER_EVAL_VJP, FP64_PIPE_BUSY_NCU_VJP) if vjp else
                        (FP64_FLOP_PER_EVAL, FP32_FLOP_PER_EVAL, FP64_PIPE_BUSY_NCU))
    f64 = f64e * nfull / (ms * 1e-3) / 1e12
    f32 = f32e * nfull / (ms * 1e-3) / 1e12
    kern = "es_kernel<2,MIXED,GRAD>" if vjp else "es_kernel<2,MIXED>"
    return {"fp64_flop_per_eval": f64e, "fp32_flop_per_eval": f32e,
            "fp64_tflops": f64, "fp64_frac": f64 / peaks["fp64"], "fp32_tflops": f32, "fp32_frac": f32 / peaks["fp32"],
            "fp64_pipe_busy_ncu": busy,
            "source": f"ncu thread-instruction counters (dadd, dmul, dfma; fadd, fmul, ffma) of one {kern} launch over "
                      "the evaluations it ran (profiles/); contour evaluations only"}


def fma_peaks(dev, stream):
    """FP32 and FP64 FMA rates (TFLOP/s) of this GPU from the benchmark-only
    probe (csrc/bench/probe_fma.cu): the SIMT roofline denominators."""
    import ctypes
    import torch
    from caustics_gb300 import build as B
    probe = ctypes.CDLL(B.BENCH_LIB)
    probe.cgb_probe_fma.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    buf = torch.empty(sms * 8, dtype=torch.float64, device=dev)
    out = {}
    for fp64 in (0, 1):
        iters, blocks = (4096, sms * 8) if not fp64 else (512, sms * 8)
        launch = lambda: probe.cgb_probe_fma(fp64, iters, blocks, ctypes.c_void_p(buf.data_ptr()),
                                             ctypes.c_void_p(stream.cuda_stream))
        launch()
        out["fp64" if fp64 else "fp32"] = blocks * 256 * iters * 256 / (timed(stream, launch, reps=3) * 1e-3) / 1e12
    return out


def headline(C, dev, stream, flush, args, clocks):
    """The K timed steps over the 4096-curve workload."""
    import torch
    off, t, cv = draw_batched(NCURVES, SEED, NMIN, NMAX, args.curves or NCURVES)
    parts = batches(off, cv, args.steps)
    evs, host = [], []
    config = None
    for a, b in parts:
        o = off[a:b + 1] - off[a]
        tt = t[off[a]:off[b]]
        if config is None and args.tune:
            from caustics_gb300 import autotune
            config = autotune.tune(o, tt, cv[a:b], precision="mixed", **LC)
        ev = C.BatchedLightCurves(o, tt, curves_for_tuning=cv[a:b], precision="mixed", tune=False,
                                  config=config or {"grid": 0, "queue_chunk": 1, "ld_group": 1}, **LC)
        evs.append((ev, torch.as_tensor(cv[a:b], device=dev)))
        host.append((torch.as_tensor(o).pin_memory(), torch.as_tensor(tt).pin_memory(),
                     torch.as_tensor(cv[a:b]).pin_memory()))
    npts = [int(ev.t.numel()) for ev, _ in evs]
    for k in range(args.warmup):
        ev, c = evs[k % len(evs)]
        ev(c)
    torch.cuda.synchronize()
    clocks.start()
    times = []
    for ev, c in evs:
        flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ev(c)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    clk = clocks.stop()
    nfull = [int(ev.route.sum().item()) for ev, _ in evs]
    status = np.concatenate([ev.status.cpu().numpy() for ev, _ in evs])
    return dict(evs=evs, host=host, parts=parts, npts=npts, nfull=nfull, times=times, clk=clk, config=config,
                status=status, off=off, t=t, cv=cv)


def e2e_run(C, H):
    """The same batches through the public API from pinned host buffers."""
    import torch
    cfg = H["config"] or {}
    o, tt, c = H["host"][0]
    C.mag_lc_batched(o, tt, c, precision="mixed", **LC, **cfg).cpu()
    torch.cuda.synchronize()
    h2d = d2h = 0
    t0 = time.perf_counter()
    for o, tt, c in H["host"]:
        m = C.mag_lc_batched(o, tt, c, precision="mixed", **LC, **cfg).cpu()
        h2d += (o.numel() + tt.numel() + c.numel()) * 8
        d2h += m.numel() * 8
    wall = time.perf_counter() - t0
    k = len(H["host"])
    return {"value": sum(H["npts"]) / wall, "unit": UNIT, "h2d_bytes_per_step": h2d // k,
            "d2h_bytes_per_step": d2h // k, "host_timed_s": wall}


def vjp_line(C, dev, stream, flush, peaks, args):
    """VJP of the 256 x 1000-point workload (seed 3) with respect to (s, q,
    rho, u1, u0, alpha, t0, tE), N(0,1) cotangent per point."""
    import torch
    off, t, cv = draw_batched(256, 3, 1000, 1000, args.vjp_curves)
    offd, td, cvd = (torch.as_tensor(x, device=dev) for x in (off, t, cv))
    cot = torch.as_tensor(np.random.default_rng(3).normal(size=len(t)), device=dev)
    g32, _ = C.mag_lc_batched_vjp(offd, td, cvd, cot, precision="mixed", **LC)
    reps = 3
    vms = timed(stream, lambda: C.mag_lc_batched_vjp(offd, td, cvd, cot, precision="mixed", **LC), reps=reps,
                flush=flush)
    fms = timed(stream, lambda: C.mag_lc_batched(offd, td, cvd, precision="mixed", **LC), reps=reps, flush=flush)
    _, route = C.mag_lc_batched(offd, td, cvd, precision="mixed", return_route=True, **LC)
    nfull = int(route.sum().item())
    g64, _ = C.mag_lc_batched_vjp(offd, td, cvd, cot, precision="fp64", **LC)
    g2, _ = C.mag_lc_batched_vjp(offd, td, cvd, cot, precision="mixed", **LC)
    d = (g32 - g64).abs()
    comp = (d / g64.abs().clamp(min=1e-300)).max().item()  # near-zero components included
    gn = g64.norm(dim=1, keepdim=True).clamp(min=1e-300)
    reln = d.norm(dim=1, keepdim=True) / gn
    norm = reln.max().item()
    norm_p99 = torch.quantile(reln.flatten(), 0.99).item()
    comp_n = (d / gn).max().item()  # each component's error against its curve's gradient norm
    n = len(t)
    flop = 3.0 * (nfull * f_es(LC["npts_limb"], LC["npts_ld"]) + (n - nfull) * (F_PS2 + F_HEX))
    achieved = flop / (vms * 1e-3) / 1e12
    return {"metric": VJP_METRIC, "value": n / (vms * 1e-3), "unit": UNIT, "ms_per_call": vms,
            "workload": f"{len(cv)} curves x 1000 points, seed 3 (drawn as the headline workload), npts_limb 200, "
                        "npts_ld 100, LD, cotangent N(0,1) (seed 3); gradient w.r.t. (s, q, rho, u1, u0, alpha, t0, tE)",
            "points": n, "full_contour_points": nfull, "full_contour_evals_per_s": nfull / (vms * 1e-3),
            "forward_evals_per_s": n / (fms * 1e-3), "vjp_over_forward_time": vms / fms,
            "mixed_vs_fp64_grad_max_rel_component": comp, "mixed_vs_fp64_grad_max_rel_norm_per_curve": norm,
            "mixed_vs_fp64_grad_p99_rel_norm_per_curve": norm_p99,
            "mixed_vs_fp64_grad_max_component_err_over_curve_norm": comp_n,
            "bit_identical_repeat": bool(torch.equal(g32, g2)),
            "roofline": {"bound": "fp32-fma", "achieved": achieved, "peak": peaks["fp32"], "unit": "TFLOP/s",
                         "frac": achieved / peaks["fp32"], "traffic": DRAM_BYTES_PER_EVAL_VJP * nfull,
                         "counted": _counted(nfull, vms, peaks, vjp=True),
                         "flop_per_unit": "3 x forward: contour point 3 x 8.58e6, hexadecapole point 3 x 1.37e4",
                         "kernel": "cgb_mag_lc_batched_vjp (point pass, first-point ordering, es_kernel<2,MIXED,GRAD>, "
                                   "curve sums), CUDA events around the call",
                         "peak_source": "measured live (csrc/bench/probe_fma.cu, FP32 FMA burst)"}}


def extras_plain_and_fp64(C, dev, stream, flush, H, args):
    """The per-call FP64 form (one mag_extended_source launch per point, grid 1:
    the reference's lax.map over points, on the GPU) on full-contour points of
    the workload, and batched FP64 on the first batch against batched mixed."""
    import torch
    ev, c = H["evs"][0]
    o, tt, cvh = H["host"][0]
    m32 = ev(c).clone()
    od, td, cd_ = o.cuda(), tt.cuda(), cvh.cuda()
    m64 = C.mag_lc_batched(od, td, cd_, precision="fp64", **LC)
    f64_ms = timed(stream, lambda: C.mag_lc_batched(od, td, cd_, precision="fp64", **LC), flush=flush)
    err = float(((m32 - m64).abs() / m64.abs()).max().item())
    full = np.flatnonzero(ev.route.bool().cpu().numpy())
    pick = full[np.linspace(0, len(full) - 1, min(args.plain_points, len(full))).astype(int)]
    off, t, cvn = o.numpy(), tt.numpy(), cvh.numpy()
    cid = np.searchsorted(off, pick, side="right") - 1
    calls = [(torch.tensor(trajectory(t[i], cvn[k]), dtype=torch.complex128, device=dev).reshape(1), cvn[k])
             for i, k in zip(pick, cid)]

    def plain():
        for w, cv in calls:
            C.mag_extended_source(w, cv[2], u1=cv[3], s=cv[0], q=cv[1], precision="fp64", grid=1, **LC)
    plain()
    pms = timed(stream, plain)
    nfull0 = H["nfull"][0]
    return {"plain_fp64_per_call_full_contour_evals_per_s": len(calls) / (pms * 1e-3),
            "batched_fp64_first_batch": {"points": H["npts"][0], "full_contour_points": nfull0,
                                         "evals_per_s": H["npts"][0] / (f64_ms * 1e-3),
                                         "full_contour_evals_per_s": nfull0 / (f64_ms * 1e-3)},
            "mixed_vs_fp64_max_rel_err_first_batch": err}


def extras_lightcurve_2000(C, dev, stream, flush):
    """The reference's limb-darkened light curve (s 1.1, q 5e-3, rho 1e-2, u1
    0.5, npts_limb 500, npts_ld 100, 2000 points u0 0.05, alpha 0.6, t0 0,
    tE 20): every point through the contour integral."""
    import torch
    t = np.linspace(-40.0, 40.0, 2000)
    cv = np.array([[1.1, 5e-3, 1e-2, 0.5, 0.05, 0.6, 0.0, 20.0]])
    off = np.array([0, 2000])
    kw = dict(npts_limb=500, limb_darkening=True, npts_ld=100)
    ev = C.BatchedLightCurves(off, t, curves_for_tuning=cv, precision="mixed", **kw)
    cvd = torch.as_tensor(cv, device=dev)
    ev(cvd)
    ms = timed(stream, lambda: ev(cvd), reps=5, flush=flush)
    od, td = torch.as_tensor(off, device=dev), torch.as_tensor(t, device=dev)
    m64 = C.mag_lc_batched(od, td, cvd, precision="fp64", **kw)
    ms64 = timed(stream, lambda: C.mag_lc_batched(od, td, cvd, precision="fp64", **kw), reps=1, flush=flush)
    ones = torch.ones(2000, dtype=torch.float64, device=dev)
    vms = timed(stream, lambda: C.mag_lc_batched_vjp(od, td, cvd, ones, precision="mixed", **kw), reps=2,
                flush=flush)
    return {"workload": "binary-ld-lightcurve-2000pt (s 1.1, q 5e-3, rho 1e-2, u1 0.5, npts_limb 500, npts_ld 100)",
            "mixed_evals_per_s": 2000 / (ms * 1e-3), "fp64_evals_per_s": 2000 / (ms64 * 1e-3),
            "vjp_evals_per_s": 2000 / (vms * 1e-3),
            "mixed_vs_fp64_max_rel_err": float(((ev.mag - m64).abs() / m64).max().item()), "autotuned": ev.config}


def extras_triple_lightcurves(C, dev, stream, flush, ncurves=64, seed=11):
    """Triple-lens limb-darkened light curves in one batched call (every point
    through the contour integral, as the reference's mag()): lenses drawn as
    the triple point-source workload (s, r3 ~ U[0.5, 2], q ~ logU[1e-4, 1], q3 ~
    logU[1e-4, 1e-1], psi ~ U[0, 2pi]), rho ~ logU[1e-3, 10^-1.5], sources and
    trajectories as the batched workload, 200-400 points per curve; forward in
    both precisions and the VJP w.r.t. the 11 curve parameters."""
    import torch
    rng = np.random.default_rng(seed)
    n = ncurves
    lens = rng.integers(200, 401, n)
    cv = np.stack([rng.uniform(0.5, 2, n), 10 ** rng.uniform(-4, 0, n), 10 ** rng.uniform(-4, -1, n),
                   rng.uniform(0.5, 2, n), rng.uniform(0, 2 * np.pi, n), 10 ** rng.uniform(-3, -1.5, n),
                   rng.uniform(0.2, 0.8, n), rng.uniform(-0.3, 0.3, n), rng.uniform(0, 2 * np.pi, n), np.zeros(n),
                   10 ** rng.uniform(np.log10(5), 2, n)], axis=1)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    t = np.concatenate([np.sort(rng.uniform(-te, te, m)) for te, m in zip(cv[:, 10], lens)])
    od, td, cvd = (torch.as_tensor(x, device=dev) for x in (off, t, cv))
    cot = torch.as_tensor(np.random.default_rng(seed).normal(size=len(t)), device=dev)
    f32 = lambda: C.mag_lc_batched(od, td, cvd, precision="mixed", **LC)
    f64 = lambda: C.mag_lc_batched(od, td, cvd, precision="fp64", **LC)
    fv = lambda: C.mag_lc_batched_vjp(od, td, cvd, cot, precision="mixed", **LC)
    m32, m64 = f32(), f64()
    fv()
    ms, ms64, vms = (timed(stream, f, reps=2, flush=flush) for f in (f32, f64, fv))
    npts = len(t)
    return {"workload": f"{n} triple-lens curves x 200-400 points (seed {seed}), npts_limb 200, npts_ld 100, LD; "
                        "grad w.r.t. (s, q, q3, r3, psi, rho, u1, u0, alpha, t0, tE)",
            "points": npts, "mixed_evals_per_s": npts / (ms * 1e-3), "fp64_evals_per_s": npts / (ms64 * 1e-3),
            "vjp_evals_per_s": npts / (vms * 1e-3), "vjp_over_forward_time": vms / ms,
            "mixed_vs_fp64_max_rel_err": float(((m32 - m64).abs() / m64.abs()).max().item())}


def extras_triple(C, dev, stream, nsys=1000, npos=1000):
    """Triple-lens point source over the whole triple workload (seed 1: 1000
    systems s1, s2 ~ U[0.5, 2], q1 ~ logU[1e-4, 1], q2 ~ logU[1e-4, 1e-1], psi ~
    U[0, 2pi]; 1000 positions each, x then y ~ U[-1.5, 1.5]; s = s1, q = q1,
    q3 = q2, r3 = s2): FP64 point-source throughput, and the mixed solver
    against FP64 on the same polynomials (roots as sets, image counts, mu)."""
    import torch
    rng = np.random.default_rng(1)
    s1, s2 = rng.uniform(0.5, 2.0, nsys), rng.uniform(0.5, 2.0, nsys)
    q1, q2 = 10 ** rng.uniform(-4, 0, nsys), 10 ** rng.uniform(-4, -1, nsys)
    psi = rng.uniform(0, 2 * np.pi, nsys)
    w = rng.uniform(-1.5, 1.5, (nsys, npos)) + 1j * rng.uniform(-1.5, 1.5, (nsys, npos))
    wd = torch.as_tensor(w, device=dev)
    prm = [dict(s=s1[k], q=q1[k], q3=q2[k], r3=s2[k], psi=psi[k]) for k in range(nsys)]

    def ps_all():
        for k in range(nsys):
            C.mag_point_source(wd[k], nlenses=3, precision="fp64", **prm[k])
    ps_all()
    ps_ms = timed(stream, ps_all)
    e1 = q1 / (1 + q1 + q2)
    emin = np.minimum(np.minimum(e1, q1 * e1), 1 - e1 - q1 * e1)
    mixed_sys = np.flatnonzero(emin >= 1e-2)  # the others run the FP64 solver under "mixed" (FP32 cannot
    worst_root, worst_mu, mismatch, p9999 = 0.0, 0.0, 0, []  # separate the images around a small mass)
    t_mixed = t_fp64 = 0.0
    for k in mixed_sys:
        c = C.lens_polynomial(wd[k], nlenses=3, **prm[k])
        t_fp64 += timed(stream, lambda: C.ehrlich_aberth(c, None, itmax=2500, precision="fp64"))
        t_mixed += timed(stream, lambda: C.ehrlich_aberth(c, None, itmax=2500, precision="mixed"))
        z64 = C.ehrlich_aberth(c, None, itmax=2500, precision="fp64").reshape(-1, 10)
        z32 = C.ehrlich_aberth(c, None, itmax=2500, precision="mixed").reshape(-1, 10)
        dist = (z64[:, :, None] - z32[:, None, :]).abs().min(dim=-1).values / z64.abs().clamp(min=1.0)
        worst_root = max(worst_root, float(dist.max()))
        p9999.append(float(torch.quantile(dist.reshape(-1), 0.9999)))
        # image filter |lens_eq(z) - w| < 1e-6 and mu = sum 1/|det J| in FP64 on the device
        q, q3 = prm[k]["q"], prm[k]["q3"]
        a, e1 = 0.5 * prm[k]["s"], q / (1 + q + q3)
        r = [complex(a), complex(-a), prm[k]["r3"] * np.exp(1j * prm[k]["psi"])]
        eps = [e1, q * e1, 1 - e1 - q * e1]
        wc = wd[k] + a * (1 - q) / (1 + q)

        def filt(z):
            zb = z.conj()
            res = (z - sum(ej / (zb - np.conj(rj)) for rj, ej in zip(r, eps)) - wc[:, None]).abs()
            lam = sum(ej / (zb - np.conj(rj)) ** 2 for rj, ej in zip(r, eps))
            det = 1.0 - lam.abs() ** 2
            return res, torch.where(res < 1e-6, 1.0 / det.abs(), torch.zeros_like(det)).sum(1)
        r64, mu64 = filt(z64)
        r32, mu32 = filt(z32)
        amb = ((r64 > 1e-6 / 30) & (r64 < 1e-6 * 30)).any(1) | ((r32 > 1e-6 / 30) & (r32 < 1e-6 * 30)).any(1)
        mismatch += int((((r64 < 1e-6).sum(1) != (r32 < 1e-6).sum(1)) & ~amb).sum())
        worst_mu = max(worst_mu, float(((mu32 - mu64).abs() / mu64)[~amb].max()))
    n, nm = nsys * npos, len(mixed_sys) * npos
    return {"workload": "1000 triple systems x 1000 positions (seed 1)",
            "point_source_fp64_evals_per_s": n / (ps_ms * 1e-3),
            "mixed_solver_systems": f"{len(mixed_sys)} of {nsys} (every mass fraction >= 1e-2; the others take "
                                    "the FP64 solver under mixed precision)",
            "roots_fp64_polys_per_s": nm / (t_fp64 * 1e-3), "roots_mixed_polys_per_s": nm / (t_mixed * 1e-3),
            "mixed_vs_fp64_root_rel_dist_max": worst_root,
            "mixed_vs_fp64_root_rel_dist_p9999_max_over_systems": float(np.max(p9999)),
            "image_count_mismatch_outside_ambiguous_band": mismatch, "mixed_vs_fp64_mu_max_rel": worst_mu}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--plain-points", type=int, default=24)
    ap.add_argument("--curves", type=int, default=0, help="first N curves only (profiling case); 0 = all 4096")
    ap.add_argument("--vjp-curves", type=int, default=256)
    ap.add_argument("--no-tune", dest="tune", action="store_false", help="default launch shape, no autotuner")
    ap.add_argument("--quick", action="store_true", help="headline steps only: no e2e, VJP, CPU baseline or extras")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--only-vjp", action="store_true",
                    help="one VJP call on --vjp-curves curves of the gradient workload (profiling case)")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.only_vjp:
        import torch
        import caustics_gb300 as C
        off, t, cv = draw_batched(256, 3, 1000, 1000, args.vjp_curves)
        cot = np.random.default_rng(3).normal(size=len(t))
        t0 = time.perf_counter()
        g, _ = C.mag_lc_batched_vjp(off, t, cv, cot, precision="mixed", **LC)
        torch.cuda.synchronize()
        s = time.perf_counter() - t0
        _, route = C.mag_lc_batched(off, t, cv, precision="mixed", return_route=True, **LC)  # after the VJP's launches
        print(json.dumps({"only_vjp": True, "points": len(t), "full_contour_points": int(route.sum().item()), "s": s,
                          "grad_finite": bool(torch.isfinite(g).all())}))
        return
    if args.quick:
        args.no_cpu = True

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    cores = _cores()
    pool = make_pool(cores) if (rank == 0 and not args.no_cpu) else None  # before the first GPU call

    import torch
    import caustics_gb300 as C

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    if dist is not None:
        dist.barrier()
    H = headline(C, dev, stream, flush, args, Clocks(local))
    total_ms = float(np.sum(H["times"]))
    if dist is not None:
        t_ = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t_, op=dist.ReduceOp.MAX)
        total_ms = float(t_.item())
    npoints, nfull = sum(H["npts"]), sum(H["nfull"])
    value = world * npoints / (total_ms * 1e-3)
    peaks = fma_peaks(dev, stream)
    flop = nfull * f_es(LC["npts_limb"], LC["npts_ld"]) + (npoints - nfull) * (F_PS2 + F_HEX)
    achieved = flop / (total_ms * 1e-3) / 1e12
    st = H["status"]
    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": len(H["times"]),
        "warmup": args.warmup, "ms_per_step": total_ms / len(H["times"]), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 (mixed)", "data": "synthetic",
        "config": {**WL, "npoints": npoints, "curves": int(H["cv"].shape[0]),
                   "step": f"one batch of curves; the {len(H['times'])} timed steps cover the workload once",
                   "l2": "flushed between timed steps (256 MiB write)", "parallelism": "replicas",
                   "autotuned": H["config"], "cuda_graph": all(ev.graph is not None for ev, _ in H["evs"])},
        "full_contour_points": nfull,
        "full_contour_evals_per_s": world * nfull / (total_ms * 1e-3),
        "step_ms": H["times"],
        "status_counts": {"noconv": int(((st & 1) != 0).sum()), "ambiguous": int(((st & 2) != 0).sum()),
                          "fallback": int(((st & 4) != 0).sum()), "merge": int(((st & 8) != 0).sum()),
                          "capacity": int(((st & 16) != 0).sum()), "invalid": int(((st & 32) != 0).sum())},
        "roofline": {"bound": "fp32-fma", "achieved": achieved, "peak": peaks["fp32"], "unit": "TFLOP/s",
                     "frac": achieved / peaks["fp32"], "traffic": DRAM_BYTES_PER_EVAL * nfull / len(H["times"]),
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of a contour-kernel launch "
                                       "(profiles/), per contour evaluation, times a step's mean contour evaluations",
                     "kernel": "es_kernel<2,MIXED> with its per-point pass and first-point ordering (the step's "
                               "graph replay, CUDA events on the launching stream)",
                     "flop_per_unit": "contour evaluation 8.58e6 (npts_limb 200, npts_ld 100), hexadecapole point "
                                      "1.37e4",
                     "peak_source": "measured live in bench.py (csrc/bench/probe_fma.cu, FP32 FMA burst); the path "
                                    "moves 24 B per point, so neither the HBM nor the tensor peak bounds it",
                     "fp64_fma_peak": peaks["fp64"],
                     "counted": _counted(nfull, total_ms, peaks),
                     "hbm_sanity": {"bytes_per_point": 24,
                                    "achieved_gbs": 24 * npoints / (total_ms * 1e-3) / 1e9,
                                    "peak_gbs_measured": _measured_peaks().get("hbm_gbs")}},
        "clocks": H["clk"],
        "gpu_launches": 3 * len(H["times"]),  # per step: per-point pass, first-point ordering, contour kernel
    }
    if not args.quick:
        res["e2e"] = e2e_run(C, H)
        res["vjp"] = vjp_line(C, dev, stream, flush, peaks, args)
        res.update(extras_plain_and_fp64(C, dev, stream, flush, H, args))
        plain = res["plain_fp64_per_call_full_contour_evals_per_s"]
        fwd_full = res["full_contour_evals_per_s"] / world
        res["batched_mixed_vs_plain_fp64"] = fwd_full / plain
        res["vjp_plus_forward_vs_plain_fp64"] = 1.0 / ((1.0 / fwd_full + 1.0 / res["vjp"]["full_contour_evals_per_s"])
                                                       * plain)
        res["binary_ld_lightcurve_2000pt"] = extras_lightcurve_2000(C, dev, stream, flush)
        res["triple_lens"] = extras_triple(C, dev, stream)
        res["triple_lens_lightcurves"] = extras_triple_lightcurves(C, dev, stream, flush)
    if pool is not None:
        rate, n = cpu_rate(pool, cores, per_core=48, seed=99)
        pool.close()
        res["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                               "sample": f"{n} points drawn uniformly from the workload's points (each with its "
                                         "curve's parameters), oracle restatement (NumPy + C solver), spawn pool"}
    if rank == 0:
        print(json.dumps(res))
    if dist is not None:
        dist.destroy_process_group()


def _measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


if __name__ == "__main__":
    main()
