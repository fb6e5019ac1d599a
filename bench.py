"""Benchmark of the SB hot path: nnz*agent*steps/s on one GB300.

Workload (the metric's headline configuration): MaxCut on a 2-D torus 100x100
(n = 10,000, degree 4, weights +-1 from seed 1234), 1024 agents, dt = 0.5,
fused kernel, 20,000 steps, update window on (early exit once every agent has
bifurcated).  A bench "step" is one complete solve of that instance (device
init from the seed, the SB loop, windows, the cut reduction).  `value` is the
BF16-state run with the problem resident on the device; the FP32-state run of
the same instance and the FP64 run (energy-error reference) are reported
beside it.  `e2e` repeats the BF16 solve through the C ABI from host buffers:
the CSR upload, the solve and the per-agent cut read-back are inside the timed
region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "sparse-ising-solver_gb300")
ORACLE = os.path.join(ROOT, "oracle")
for p in (PKG, ORACLE):
    if p not in sys.path:
        sys.path.insert(0, p)

CONFIG = dict(workload="maxcut-torus-100x100-pm1", n=10000, degree=4, agents=1024, dt=0.5,
              sb_steps=20000, update_window=1, fused=1, graph_seed=1234, init_seed=1)
METRIC = "nnz*agent*steps/s"


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample(g, A, sb_steps, seconds=12.0, nthreads=0):
    """The FP64 oracle (OpenMP over rows, all host threads) on a bounded sample
    of the workload: the same graph and agents for `s` SB steps."""
    import sbo
    og = sbo.Graph(g.n, g.rowptr, g.col, g.val, g.wsum)
    t = []
    for k in (2, 6):   # the difference removes the init cost
        t0 = time.perf_counter()
        sbo.maxcut_solve(og, sbo.params(dt=CONFIG["dt"], steps=k, period=k, agents=A,
                                        seed=CONFIG["init_seed"], nthreads=nthreads))
        t.append(time.perf_counter() - t0)
    per_step = max((t[1] - t[0]) / 4.0, 1e-4)
    s = int(max(2, min(sb_steps, seconds / per_step)))
    t0 = time.perf_counter()
    o = sbo.maxcut_solve(og, sbo.params(dt=CONFIG["dt"], steps=s, period=s, agents=A,
                                        seed=CONFIG["init_seed"], nthreads=nthreads))
    dt = time.perf_counter() - t0
    cores = nthreads if nthreads > 0 else (os.cpu_count() or 1)
    return g.nnz * A * o["result"]["steps_run"] / dt, cores, s, dt


def run_reference(args, rank):
    """--impl reference: the reference path has no CPU solver, so its CPU
    implementation here is the FP64 oracle port, all host threads."""
    if rank != 0:
        return
    import sbx
    import sbo
    sbo.lib()
    g = sbx.gen_torus(100, 100, seed=CONFIG["graph_seed"])
    A = CONFIG["agents"]
    vals = []
    samples = []
    for i in range(args.warmup + args.steps):
        v, cores, s, dt = cpu_sample(g, A, CONFIG["sb_steps"], seconds=8.0)
        if i >= args.warmup:
            vals.append(v)
            samples.append((s, dt))
    value = sum(vals) / len(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "nnz*agent*steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * sum(d for _, d in samples) / len(samples),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": dict(CONFIG),
        "cpu_baseline": {"value": value, "unit": "nnz*agent*steps/s", "cores": cores,
                         "kind": "port",
                         "sample": "%d SB steps of the workload per bench step" % samples[0][0]},
        "e2e": {"value": value, "unit": "nnz*agent*steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--sb-steps", type=int, default=CONFIG["sb_steps"],
                    help="SB steps per solve (profiling cases use fewer)")
    ap.add_argument("--legs", default="all", choices=["all", "bf16"],
                    help="bf16: only the timed BF16 solves (profiling)")
    args = ap.parse_args()
    CONFIG["sb_steps"] = args.sb_steps

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return

    import numpy as np
    import torch
    import sbx

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    # a created stream: the engine captures CUDA graphs on it (the legacy
    # default stream cannot be captured)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = sbx.Context(local)
    ctx.set_stream(stream.cuda_stream)
    g = sbx.gen_torus(100, 100, seed=CONFIG["graph_seed"])
    A = CONFIG["agents"]
    prob = ctx.problem(g)
    seed = CONFIG["init_seed"] + rank   # each rank: an independent replica (weak scaling)

    def prm(prec, flags=0):
        return sbx.params(dt=CONFIG["dt"], steps=CONFIG["sb_steps"], agents=A,
                          fused=CONFIG["fused"], update_window=CONFIG["update_window"],
                          seed=seed, precision=prec, flags=flags)

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def timed(prec, k, w):
        for _ in range(w):
            ctx.solve(prob, prm(prec))
        evs = []
        units = 0
        launches = 0
        res = None
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        with Clocks(local) as clk:
            for _ in range(k):
                flush.fill_(1)   # L2 flush between iterations
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                res, vals = ctx.solve(prob, prm(prec))
                e1.record(stream)
                evs.append((e0, e1))
                units += g.nnz * A * res["steps_run"]
                launches += res["gpu_launches"]
            torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in evs)
        if dist is not None:
            t = torch.tensor([ms], device="cuda", dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
            u = torch.tensor([units], device="cuda", dtype=torch.float64)
            dist.all_reduce(u)
            units = float(u.item())
        return units / (ms / 1000.0), ms / k, res, vals, clk.summary(), launches // max(k, 1)

    v_bf16, ms_bf16, r_bf16, cuts_bf16, clocks, launches = timed(sbx.BF16, args.steps, args.warmup)
    if args.legs == "bf16":
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": v_bf16, "ms_per_step": ms_bf16,
                              "config": dict(CONFIG), "legs": "bf16"}), flush=True)
        ctx.close()
        return
    v_f32, ms_f32, r_f32, cuts_f32, _, _ = timed(sbx.F32, 1, 1)
    r64, cuts64 = ctx.solve(prob, prm(sbx.F64))

    # e2e: through the C ABI from host buffers, CSR upload + solve + read-back.
    t_e2e = []
    units_e2e = 0
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p2 = ctx.problem(g)
        r2, _ = ctx.solve(p2, prm(sbx.BF16))
        p2.close()
        torch.cuda.synchronize()
        if i >= args.warmup:
            t_e2e.append(time.perf_counter() - t0)
            units_e2e += g.nnz * A * r2["steps_run"]
    e2e = units_e2e / sum(t_e2e)

    # Dominant kernel: the streaming step kernel, timed launch by launch.
    rp, _ = ctx.solve(prob, prm(sbx.BF16, sbx.FLAG_PROFILE))
    peaks, peak_kind = load_peaks()
    sx = sy = 2
    b_step = 2 * g.n * A * (sx + sy) + 8 * g.nnz + 4 * (g.n + 1)
    roof = None
    if rp["kernel_launches"] and rp["kernel_ms"] > 0:
        per_launch_s = rp["kernel_ms"] / 1000.0 / rp["kernel_launches"]
        achieved = b_step / per_launch_s / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "traffic": None,
                "peak_kind": peak_kind, "kernel": "k_step<bf16,fused>",
                "bytes_per_launch": b_step, "launch_us": per_launch_s * 1e6}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        v, cores, s, dt = cpu_sample(g, A, CONFIG["sb_steps"])
        cpu = {"value": v, "unit": "nnz*agent*steps/s", "cores": cores, "kind": "port",
               "sample": "FP64 oracle, %d SB steps of the workload (%.1f s)" % (s, dt)}

    if rank == 0:
        best64 = r64["max"]
        line = {
            "metric": METRIC, "value": v_bf16, "unit": "nnz*agent*steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_bf16,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
            "data": "synthetic (seeded torus, weights +-1)",
            "config": dict(CONFIG, precision="bf16 state, fp32 arithmetic, exact integer force",
                           l2="flushed between iterations (256 MB write)",
                           parallelism="replicas" if world > 1 else "single"),
            "e2e": {"value": e2e, "unit": "nnz*agent*steps/s",
                    "h2d_bytes_per_step": int(g.rowptr.nbytes + g.col.nbytes + g.val.nbytes),
                    "d2h_bytes_per_step": int(8 * A + 32)},
            "gpu_launches": launches,
            "roofline": roof,
            "cpu_baseline": cpu,
            "clocks": clocks,
            "fp32": {"value": v_f32, "ms_per_step": ms_f32, "best_cut": r_f32["max"],
                     "steps_run": r_f32["steps_run"]},
            "quality": {"best_cut_bf16": r_bf16["max"], "best_cut_fp32": r_f32["max"],
                        "best_cut_fp64": best64,
                        "energy_error_bf16": abs(r_bf16["max"] - best64) / abs(best64),
                        "energy_error_fp32": abs(r_f32["max"] - best64) / abs(best64),
                        "steps_run_bf16": r_bf16["steps_run"], "kernel": r_bf16["kernel_used"]},
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
