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

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--plain-points", type=int, default=40)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return

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
    w = torch.as_tensor(w_host).to(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    kw = dict(npts_limb=WL["npts_limb"], limb_darkening=True, u1=WL["u1"], npts_ld=WL["npts_ld"], s=WL["s"],
              q=WL["q"])

    def step(prec):
        return C.mag(w, WL["rho"], precision=prec, **kw)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    # warm-up
    for _ in range(args.warmup):
        out_mixed = step("mixed")
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
        out_mixed = step("mixed")
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    barrier()
    clk = clocks.stop()
    ms = float(np.mean(times))
    if dist is not None:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * WL["npoints"] / (ms * 1e-3)

    # dominant kernel alone: the contour pass over all points (every point routes to it)
    es_ms = []
    for _ in range(max(2, args.steps // 2)):
        flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        C.mag_extended_source(w, WL["rho"], precision="mixed", **kw)
        e1.record(stream)
        e1.synchronize()
        es_ms.append(e0.elapsed_time(e1))
    es_ms = float(np.mean(es_ms))

    # FP64 batched, and plain per-call FP64 (one launch per point, like lax.map)
    step("fp64")
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    out64 = step("fp64")
    e1.record(stream)
    e1.synchronize()
    fp64_rate = WL["npoints"] / (e0.elapsed_time(e1) * 1e-3)
    err = float(torch.max(torch.abs(out_mixed - out64) / out64).item())
    idx = np.linspace(0, WL["npoints"] - 1, args.plain_points).astype(int)
    wp = [w[i:i + 1] for i in idx]
    C.mag_extended_source(wp[0], WL["rho"], precision="fp64", grid=1, **kw)
    torch.cuda.synchronize()
    e0.record(stream)
    for x in wp:
        C.mag_extended_source(x, WL["rho"], precision="fp64", grid=1, **kw)
    e1.record(stream)
    e1.synchronize()
    plain_rate = len(wp) / (e0.elapsed_time(e1) * 1e-3)

    # end to end through the public API with host buffers
    C.mag(w_host, WL["rho"], precision="mixed", **kw)
    e2e_t = []
    for _ in range(max(2, args.steps)):
        t = time.perf_counter()
        res = C.mag(w_host, WL["rho"], precision="mixed", **kw)
        e2e_t.append(time.perf_counter() - t)
    e2e_rate = world * WL["npoints"] / float(np.mean(e2e_t))

    # live FMA-pipe peak (FP32) for the roofline denominator
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    buf = torch.empty(sms * 8, dtype=torch.float64, device=dev)
    iters, blocks = 4096, sms * 8
    import ctypes
    L.lib().cgb_probe_fma(0, iters, blocks, ctypes.c_void_p(buf.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    e0.record(stream)
    L.lib().cgb_probe_fma(0, iters, blocks, ctypes.c_void_p(buf.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    e1.record(stream)
    e1.synchronize()
    fp32_peak = blocks * 256 * iters * 256 / (e0.elapsed_time(e1) * 1e-3) / 1e12
    achieved = WL["npoints"] * FLOP_PER_EVAL / (es_ms * 1e-3) / 1e12

    cpu = None
    if pool is not None:
        rate, n = cpu_rate(pool, cores)
        pool.close()
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{n} trajectory points, oracle restatement (NumPy + C solver), spawn pool"}

    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64 (mixed)", "data": "synthetic",
            "config": {**WL, "l2": "flushed between timed steps (256 MiB write)", "parallelism": "replicas"},
            "roofline": {"bound": "fp32-fma", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp32_peak, "traffic": None, "kernel": "es_kernel<2,MIXED>",
                         "peak_source": "measured live in bench.py (cgb_probe_fma, FP32 FMA burst)",
                         "flop_per_eval": FLOP_PER_EVAL},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_rate, "unit": UNIT, "h2d_bytes_per_step": WL["npoints"] * 16,
                    "d2h_bytes_per_step": WL["npoints"] * 8},
            "clocks": clk,
            "gpu_launches": 2 * args.steps,
            "plain_fp64_per_call_evals_per_s": plain_rate,
            "batched_fp64_evals_per_s": fp64_rate,
            "batched_mixed_vs_plain_fp64": value / world / plain_rate,
            "mixed_vs_fp64_max_rel_err": err,
            "vjp_evals_per_s": None,
        }))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
