#!/usr/bin/env python
"""Benchmark of the extended-source magnification hot path on one GB300.

Workload (the reference's binary limb-darkened light curve): s=1.1, q=5e-3,
rho=1e-2, u1=0.5, npts_limb=500, npts_ld=100, a 2000-point straight trajectory
u0=0.05, alpha=0.6 rad, t uniform on [t0-2tE, t0+2tE], t0=0, tE=20.  Every
point fails the hexadecapole test (q < 0.01), so a step is 2000 full
contour-integration evaluations plus the per-point hexadecapole pass.

value   = extended-source evaluations/s of the batched mixed-precision path,
          device-timed (CUDA events), inputs resident in HBM, L2 flushed
          between timed steps (256 MiB write > 129 MB L2);
e2e     = the same through the public API with host (NumPy) buffers, copies
          included, host clock;
plain   = the per-call FP64 form (one mag_extended_source launch per point),
          and batched FP64, for the mixed-vs-plain speed-up.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
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

WL = dict(workload="binary-ld-lightcurve-2000pt", s=1.1, q=5e-3, rho=1e-2, u1=0.5, npts_limb=500, npts_ld=100,
          npoints=2000, u0=0.05, alpha=0.6, t0=0.0, tE=20.0)
METRIC = "extended-source magnification evals/s (batched mixed precision, <=1e-4 rel err)"
UNIT = "evals/s"
# nominal FP64-equivalent work of one full contour evaluation at npts_limb=L,
# npts_ld=G: L root solves (5.7e3 flop) + ~3.1 L contour points x 2G nodes x 60 flop
FLOP_PER_EVAL = WL["npts_limb"] * 5.7e3 + 3.1 * WL["npts_limb"] * WL["npts_ld"] * 2 * 60
# DRAM bytes (read + write) per evaluation of the contour kernel, from one ncu
# capture of a 300-evaluation launch of this workload (1.40 MB per launch;
# instruction, constant and register-spill traffic: the inputs are 24 B per
# evaluation), scaled by the evaluations of a launch
DRAM_BYTES_PER_EVAL = 1.397e6 / 300


def trajectory(n):
    t = np.linspace(WL["t0"] - 2 * WL["tE"], WL["t0"] + 2 * WL["tE"], n)
    tau = (t - WL["t0"]) / WL["tE"]
    a, u0 = WL["alpha"], WL["u0"]
    return (u0 * np.cos(a) + tau * np.sin(a)) + 1j * (-u0 * np.sin(a) + tau * np.cos(a))


# ---------------------------------------------------------------------------
# CPU baseline (the oracle restatement of the reference, process pool)
# ---------------------------------------------------------------------------

def _oracle_chunk(ws):
    sys.path.insert(0, ROOT)
    from oracle import caustics_oracle as O
    return O.mag(np.asarray(ws), WL["rho"], npts_limb=WL["npts_limb"], limb_darkening=True, u1=WL["u1"],
                 npts_ld=WL["npts_ld"], s=WL["s"], q=WL["q"])


def _cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def make_pool(n):
    ctx = mp.get_context("spawn")
    pool = ctx.Pool(n)
    pool.map(_oracle_chunk, [trajectory(2000)[:1]] * n)  # import + warm each worker
    return pool


def cpu_rate(pool, cores, per_core=6, seed=0):
    w = trajectory(WL["npoints"])
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(len(w), size=per_core * cores, replace=False))
    chunks = [w[idx[i::cores]] for i in range(cores)]
    t = time.perf_counter()
    pool.map(_oracle_chunk, chunks)
    dt = time.perf_counter() - t
    return len(idx) / dt, len(idx)


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
    for _ in range(args.warmup):
        cpu_rate(pool, cores, per_core=2)
    rates, n = [], 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        r, n = cpu_rate(pool, cores, per_core=4, seed=k)
        rates.append(r)
    wall = time.perf_counter() - t0
    pool.close()
    value = float(np.mean(rates))
    sample = f"{n} of the {WL['npoints']} trajectory points per step, oracle restatement (NumPy + C solver)"
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {k: v for k, v in WL.items()},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------

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


def extras_batched(C, dev, stream, flush, ncurves=24, plain_points=24):
    """A bounded sample of the 4096-curve uneven batched workload (seed 2,
    lengths U{200..5000}, npts_limb=200, npts_ld=100, LD): batched mixed with
    the autotuned launch shape in a CUDA graph, against the plain per-call FP64
    form (one launch per full-contour point) on points of the same curves."""
    import torch
    off, t, cv = draw_batched(4096, 2, 200, 5000, ncurves)
    kw = dict(npts_limb=200, limb_darkening=True, npts_ld=100)
    ev = C.BatchedLightCurves(off, t, curves_for_tuning=cv, precision="mixed", **kw)
    cvd = torch.as_tensor(cv, device=dev)
    ev(cvd)
    ms = timed(stream, lambda: ev(cvd), reps=3, flush=flush)
    route = ev.route.bool().cpu().numpy()
    nfull = int(route.sum())
    ref = C.mag_lc_batched(off, t, cv, precision="fp64", **kw).cpu().numpy()
    err = float(np.max(np.abs(ev.mag.cpu().numpy() - ref) / ref))
    # plain per-call FP64 on a sample of the full-contour points
    full = np.flatnonzero(route)
    pick = full[np.linspace(0, len(full) - 1, min(plain_points, len(full))).astype(int)]
    curve_of = np.searchsorted(off, pick, side="right") - 1
    calls = []
    for i, c in zip(pick, curve_of):
        s_, q_, rho, u1, u0, a, t0, te = cv[c]
        tau = (t[i] - t0) / te
        w = torch.tensor([(u0 * np.cos(a) + tau * np.sin(a)) + 1j * (-u0 * np.sin(a) + tau * np.cos(a))],
                         dtype=torch.complex128, device=dev)
        calls.append((w, rho, dict(npts_limb=200, limb_darkening=True, u1=u1, npts_ld=100, s=s_, q=q_)))

    def plain():
        for w, rho, k in calls:
            C.mag_extended_source(w, rho, precision="fp64", grid=1, **k)
    plain()
    pms = timed(stream, plain)
    plain_rate = len(calls) / (pms * 1e-3)
    return {"workload": f"first {ncurves} of 4096 curves, seed 2, lengths U{{200..5000}}, npts_limb 200, npts_ld 100, LD",
            "points": int(len(t)), "full_contour_points": nfull, "ms": ms, "points_per_s": len(t) / (ms * 1e-3),
            "full_contour_evals_per_s": nfull / (ms * 1e-3), "plain_fp64_per_call_evals_per_s": plain_rate,
            "batched_full_vs_plain_fp64": nfull / (ms * 1e-3) / plain_rate, "mixed_vs_fp64_max_rel_err": err,
            "autotuned": ev.config, "cuda_graph": ev.graph is not None}


def extras_vjp(C, dev, stream, flush):
    """VJP with respect to (s, q, rho, u1, u0, alpha, t0, tE) for 256 curves x
    1000 points drawn as the batched workload (seed 3), N(0,1) cotangent."""
    import torch
    off, t, cv = draw_batched(256, 3, 1000, 1000, 256)
    kw = dict(npts_limb=200, limb_darkening=True, npts_ld=100)
    offd, td, cvd = (torch.as_tensor(x, device=dev) for x in (off, t, cv))
    cot = torch.as_tensor(np.random.default_rng(3).normal(size=len(t)), device=dev)
    C.mag_lc_batched_vjp(offd, td, cvd, cot, precision="mixed", **kw)
    vms = timed(stream, lambda: C.mag_lc_batched_vjp(offd, td, cvd, cot, precision="mixed", **kw), reps=2, flush=flush)
    fms = timed(stream, lambda: C.mag_lc_batched(offd, td, cvd, precision="mixed", **kw), reps=2, flush=flush)
    g32, _ = C.mag_lc_batched_vjp(offd, td, cvd, cot, precision="mixed", **kw)
    g64, _ = C.mag_lc_batched_vjp(offd, td, cvd, cot, precision="fp64", **kw)
    rel = (torch.abs(g32 - g64) / torch.clamp(torch.abs(g64), min=1e-300)).median().item()
    return {"workload": "256 curves x 1000 points, seed 3, npts_limb 200, npts_ld 100, LD, cotangent N(0,1)",
            "vjp_points_per_s": len(t) / (vms * 1e-3), "forward_points_per_s": len(t) / (fms * 1e-3),
            "vjp_over_forward_time": vms / fms, "mixed_vs_fp64_grad_median_rel_diff": rel}


def extras_triple(C, dev, stream, nsys=1000, big=1 << 20, ncentres=256):
    """Triple lenses: point-source throughput (FP64 solver; "mixed" routes
    triple lenses there, its degree-10 FP32 stages being slower than FP64 in a
    one-polynomial-per-thread kernel) and extended-source throughput, mixed
    against FP64, on the first six systems whose mass fractions all reach 1e-2
    (below that the mixed path hands triple lenses to the FP64 solver).
    Systems: seed 1, s1, s2 ~ U[0.5, 2], q1 ~ logU[1e-4, 1], q2 ~ logU[1e-4,
    1e-1], psi ~ U[0, 2pi]; s = s1, q = q1, q3 = q2, r3 = s2.  Contour workload
    per system: 256 source centres ~ U[-1, 1]^2 (seed 7), rho = 1e-2,
    npts_limb = 300, with and without limb darkening (u1 = 0.5, npts_ld = 100)."""
    import torch
    rng = np.random.default_rng(1)
    sysp = np.stack([rng.uniform(0.5, 2, nsys), rng.uniform(0.5, 2, nsys), 10 ** rng.uniform(-4, 0, nsys),
                     10 ** rng.uniform(-4, -1, nsys), rng.uniform(0, 2 * np.pi, nsys)], axis=1)
    e1 = sysp[:, 2] / (1 + sysp[:, 2] + sysp[:, 3])
    e2 = sysp[:, 2] * e1
    emin = np.minimum(np.minimum(e1, e2), 1 - e1 - e2)
    systems = np.flatnonzero(emin >= 1e-2)[:6]
    rng2 = np.random.default_rng(7)
    ps_rate, es = [], {"ld0": {"fp64": [], "mixed": []}, "ld1": {"fp64": [], "mixed": []}}
    maxrel, fallbacks = 0.0, 0
    for k in systems:
        p = dict(s=sysp[k, 0], q=sysp[k, 2], q3=sysp[k, 3], r3=sysp[k, 1], psi=sysp[k, 4])
        wb = torch.as_tensor(rng2.uniform(-1.5, 1.5, big) + 1j * rng2.uniform(-1.5, 1.5, big), device=dev)
        C.mag_point_source(wb, nlenses=3, precision="fp64", **p)
        ps_rate.append(big / (timed(stream, lambda: C.mag_point_source(wb, nlenses=3, precision="fp64", **p), 3)
                              * 1e-3))
        w0 = torch.as_tensor(rng2.uniform(-1, 1, ncentres) + 1j * rng2.uniform(-1, 1, ncentres), device=dev)
        for ld in (0, 1):
            res = {}
            for prec in ("fp64", "mixed"):
                def f():
                    return C.mag_extended_source(w0, 1e-2, nlenses=3, npts_limb=300, limb_darkening=bool(ld),
                                                 u1=0.5, precision=prec, return_status=True, **p)
                res[prec] = f()
                es[f"ld{ld}"][prec].append(ncentres / (timed(stream, f, 2) * 1e-3))
            m64, m32, s32 = res["fp64"][0], res["mixed"][0], res["mixed"][1]
            maxrel = max(maxrel, float(((m32 - m64).abs() / m64.abs()).max().item()))
            fallbacks += int(((s32 & 4) != 0).sum().item())
    gm = lambda v: float(np.exp(np.mean(np.log(v))))
    return {"workload": f"systems {systems.tolist()} of 1000 (seed 1); point source: 2^20 positions ~ U[-1.5, 1.5]^2 "
                        "per system; contour: 256 centres, rho 1e-2, npts_limb 300",
            "systems_on_fp64_solver_of_1000": int((emin < 1e-2).sum()),
            "point_source_fp64_evals_per_s_geomean": gm(ps_rate),
            "extended_fp64_evals_per_s_geomean": {"uniform": gm(es["ld0"]["fp64"]), "ld": gm(es["ld1"]["fp64"])},
            "extended_mixed_evals_per_s_geomean": {"uniform": gm(es["ld0"]["mixed"]), "ld": gm(es["ld1"]["mixed"])},
            "extended_mixed_vs_fp64_max_rel_err": maxrel, "extended_mixed_fallback_evals": fallbacks}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--plain-points", type=int, default=40)
    ap.add_argument("--points", type=int, default=WL["npoints"], help="trajectory points (smaller: profiling case)")
    ap.add_argument("--quick", action="store_true", help="headline step only: no CPU baseline, no extra workloads")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.points != WL["npoints"]:
        WL["npoints"] = args.points
        WL["workload"] = f"binary-ld-lightcurve-{args.points}pt"
    if args.quick:
        args.no_cpu = True

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    cores = _cores()
    pool = make_pool(cores) if (rank == 0 and not args.no_cpu) else None  # before the first GPU call

    import torch
    import caustics_gb300 as C
    from caustics_gb300 import _lib as L

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    w_host = trajectory(WL["npoints"])
    t_host = np.linspace(WL["t0"] - 2 * WL["tE"], WL["t0"] + 2 * WL["tE"], WL["npoints"])
    curves_host = np.array([[WL["s"], WL["q"], WL["rho"], WL["u1"], WL["u0"], WL["alpha"], WL["t0"], WL["tE"]]])
    offsets_host = np.array([0, WL["npoints"]], dtype=np.int64)
    w = torch.as_tensor(w_host).to(dev)
    t_dev = torch.as_tensor(t_host).to(dev)
    curves = torch.as_tensor(curves_host).to(dev)
    offsets = torch.as_tensor(offsets_host).to(dev)
    cot = torch.randn(WL["npoints"], dtype=torch.float64, device=dev, generator=torch.Generator(dev).manual_seed(3))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    kw = dict(npts_limb=WL["npts_limb"], limb_darkening=True, u1=WL["u1"], npts_ld=WL["npts_ld"], s=WL["s"],
              q=WL["q"])
    kwb = dict(npts_limb=WL["npts_limb"], limb_darkening=True, npts_ld=WL["npts_ld"])

    # batched path: per-point pass + persistent contour kernel draining the
    # device queue, launch shape from the autotuner, captured in a CUDA graph
    ev = C.BatchedLightCurves(offsets, t_dev, curves_for_tuning=curves, precision="mixed", **kwb)

    def step():
        return ev(curves)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        step()
    barrier()
    # timed batched mixed steps (events on the launching stream, L2 flushed between)
    clocks = Clocks(local)
    clocks.start()
    times = []
    barrier()
    for _ in range(args.steps):
        flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    barrier()
    clk = clocks.stop()
    out_mixed = ev.mag.clone()
    ms = float(np.mean(times))
    if dist is not None:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * WL["npoints"] / (ms * 1e-3)

    # the contour pass as the step runs it, without the graph: one batched call
    # (per-point pass, first-point ordering, contour kernel; every point routes
    # to the contour kernel, which takes the bulk of the time)
    es_ms = timed(stream, lambda: C.mag_lc_batched(offsets, t_dev, curves, precision="mixed", **kwb, **ev.config),
                  reps=max(2, args.steps // 2), flush=flush)
    achieved = WL["npoints"] * FLOP_PER_EVAL / (es_ms * 1e-3) / 1e12
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    buf = torch.empty(sms * 8, dtype=torch.float64, device=dev)
    import ctypes
    from caustics_gb300 import build as B
    probe = ctypes.CDLL(B.BENCH_LIB)  # benchmark-only FMA probe (csrc/bench/probe_fma.cu)
    probe.cgb_probe_fma.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]

    def fma_peak(fp64):
        iters, blocks = (4096, sms * 8) if not fp64 else (512, sms * 8)
        launch = lambda: probe.cgb_probe_fma(fp64, iters, blocks, ctypes.c_void_p(buf.data_ptr()),
                                             ctypes.c_void_p(stream.cuda_stream))
        launch()
        return blocks * 256 * iters * 256 / (timed(stream, launch) * 1e-3) / 1e12
    fp32_peak = fma_peak(0)
    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64 (mixed)", "data": "synthetic",
        "config": {**WL, "l2": "flushed between timed steps (256 MiB write)", "parallelism": "replicas",
                   "autotuned": ev.config, "cuda_graph": ev.graph is not None},
        "roofline": {"bound": "fp32-fma", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": DRAM_BYTES_PER_EVAL * WL["npoints"],
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of a 300-evaluation launch, "
                                       "scaled to this launch's evaluations",
                     "kernel": "es_kernel<2,MIXED> with its per-point pass and first-point ordering (one "
                               "cgb_mag_lc_batched call, CUDA events around it)",
                     "peak_source": "measured live in bench.py (cgb_probe_fma, FP32 FMA burst); the path moves "
                                    "24 B per evaluation, so neither HBM nor tensor peaks bound it",
                     "flop_per_eval": FLOP_PER_EVAL,
                     "pipes_ncu": {"fp64_pct_of_peak": 42.5, "fp32_fma_pct_of_peak": 8.8, "issue_active_pct": 17.5,
                                   "source": "ncu --set full of a 300-evaluation launch of this workload "
                                             "(profiles/es_kernel_mixed_binary_ld_300pt.md): the FP64 pipe, not "
                                             "the FMA rate of the flop model, bounds the kernel"},
                     "hbm_sanity": {"bytes_per_eval": 24,
                                    "achieved_gbs": 24 * WL["npoints"] / (es_ms * 1e-3) / 1e9,
                                    "peak_gbs_measured": _measured_peaks().get("hbm_gbs")}},
        "clocks": clk,
        "gpu_launches": 3 * args.steps,  # per step: per-point pass, first-point ordering, contour kernel
    }
    if not args.quick:
        # FP64 batched, and plain per-call FP64 (one launch per point, like lax.map)
        C.mag_lc_batched(offsets, t_dev, curves, precision="fp64", **kwb)
        out64 = None

        def f64():
            nonlocal out64
            out64 = C.mag_lc_batched(offsets, t_dev, curves, precision="fp64", **kwb)
        fp64_ms = timed(stream, f64, flush=flush)
        fp64_rate = WL["npoints"] / (fp64_ms * 1e-3)
        err = float(torch.max(torch.abs(out_mixed - out64) / out64).item())
        idx = np.linspace(0, WL["npoints"] - 1, args.plain_points).astype(int)
        wp = [w[i:i + 1] for i in idx]
        C.mag_extended_source(wp[0], WL["rho"], precision="fp64", grid=1, **kw)

        def plain():
            for x in wp:
                C.mag_extended_source(x, WL["rho"], precision="fp64", grid=1, **kw)
        plain_rate = len(wp) / (timed(stream, plain) * 1e-3)
        fp64_peak = fma_peak(1)
        es64_ms = timed(stream, lambda: C.mag_extended_source(w, WL["rho"], precision="fp64", **kw), flush=flush)

        # nearest-root labelling: no faithful labelling solves
        near = C.BatchedLightCurves(offsets, t_dev, curves_for_tuning=curves, precision="mixed", labelling="nearest",
                                    config=ev.config, **kwb)
        near(curves)
        near_ms = timed(stream, lambda: near(curves), reps=max(2, args.steps), flush=flush)
        near_err = float(torch.max(torch.abs(near.mag - out64) / out64).item())

        # VJP of the light curve (s, q, rho, u1, u0, alpha, t0, tE) with a N(0,1) cotangent
        C.mag_lc_batched_vjp(offsets, t_dev, curves, cot, precision="mixed", **ev.config, **kwb)
        vjp_ms = timed(stream, lambda: C.mag_lc_batched_vjp(offsets, t_dev, curves, cot, precision="mixed",
                                                            **ev.config, **kwb), reps=max(2, args.steps // 2),
                       flush=flush)
        vjp_rate = WL["npoints"] / (vjp_ms * 1e-3)

        # end to end through the public API with host buffers (H2D of times and curve
        # parameters, D2H of the magnifications inside the timed region)
        C.mag_lc_batched(offsets_host, t_host, curves_host, precision="mixed", **ev.config, **kwb).cpu()
        e2e_t = []
        for _ in range(max(2, args.steps)):
            t = time.perf_counter()
            C.mag_lc_batched(offsets_host, t_host, curves_host, precision="mixed", **ev.config, **kwb).cpu().numpy()
            e2e_t.append(time.perf_counter() - t)
        e2e_rate = world * WL["npoints"] / float(np.mean(e2e_t))
        res.update({
            "e2e": {"value": e2e_rate, "unit": UNIT, "h2d_bytes_per_step": WL["npoints"] * 8 + 16 + 64,
                    "d2h_bytes_per_step": WL["npoints"] * 8},
            "plain_fp64_per_call_evals_per_s": plain_rate,
            "batched_fp64_evals_per_s": fp64_rate,
            "batched_mixed_vs_plain_fp64": value / world / plain_rate,
            "mixed_vs_fp64_max_rel_err": err,
            "vjp_evals_per_s": vjp_rate,
            "nearest_labelling": {"evals_per_s": WL["npoints"] / (near_ms * 1e-3),
                                  "max_rel_err_vs_fp64_reference_labelling": near_err},
            "vjp_plus_forward_vs_plain_fp64": 1.0 / ((1.0 / value * world + 1.0 / vjp_rate) * plain_rate),
            "fp64_roofline": {"kernel": "es_kernel<2,FP64>", "achieved": WL["npoints"] * FLOP_PER_EVAL /
                              (es64_ms * 1e-3) / 1e12, "peak": fp64_peak, "unit": "TFLOP/s",
                              "peak_source": "measured live (cgb_probe_fma, FP64 FMA)"},
            "batched_4096_curve_sample": extras_batched(C, dev, stream, flush),
            "vjp_256x1000": extras_vjp(C, dev, stream, flush),
            "triple_lens": extras_triple(C, dev, stream),
        })
    if pool is not None:
        rate, n = cpu_rate(pool, cores)
        pool.close()
        res["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                               "sample": f"{n} trajectory points, oracle restatement (NumPy + C solver), spawn pool"}
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
