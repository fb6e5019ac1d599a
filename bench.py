"""Benchmark of the SB hot path: nnz*agent*steps/s on one GB300.

Default workload (the configuration the metric names, "BF16-batched vs
FP32-plain"): 512 independent MaxCut instances, n log-uniform in [100, 20000],
Erdos-Renyi and random geometric graphs of average degree 6-40, weights +-1,
64 agents each, BF16 state, dt 0.5, 10,000 steps, all instances in one
launch per SB step (a CUDA graph per window).  A bench "step" is one complete
batched solve (device init from the seeds, the SB loop, windows, the exact
cuts).  `value` has the problems resident on the device; `e2e` goes through
the C ABI from host buffers (every instance's CSR uploaded, the solve, the
per-agent cuts read back).  FP32-plain (each instance solved alone in FP32),
the FP64 run of the same seeds (the energy error) and the time to reach
FP32-plain's best cuts are reported beside it.

Other workloads (--workload): torus (torus 100x100, 1024 agents, BF16,
update window), er800 (ER n=800, 1024 agents, FP32 plain), rmat20 (R-MAT
2^20, 256 agents, BF16), tsp30 (30 cities, 1024 agents, FP32).

`--workload loaders` times the MTX and TSPLIB loaders instead (engine, the
oracle's restatement, and the reference's own where it was compiled).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload batch512|torus|er800|rmat20|tsp30|loaders]
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

METRIC = "nnz*agent*steps/s"
WORKLOADS = {
    "torus": dict(kind="maxcut", workload="maxcut-torus-100x100-pm1", graph=("torus", 100, 100),
                  agents=1024, dt=0.5, sb_steps=20000, update_window=1, fused=1,
                  precision="bf16", compare=("f32", "f64")),
    "er800": dict(kind="maxcut", workload="maxcut-er-800-p0.0601-unit",
                  graph=("er", 800, 0.0601, False), agents=1024, dt=0.1, sb_steps=10000,
                  update_window=0, fused=1, precision="f32", compare=("bf16", "f64")),
    "rmat20": dict(kind="maxcut", workload="maxcut-rmat-scale20-ef4-unit",
                   graph=("rmat", 20, 4), agents=256, dt=0.5, sb_steps=10000, update_window=0,
                   fused=1, precision="bf16", compare=("f32",)),
    # 30 cities uniform in the unit square, scaled by 1000: the reference's
    # fixed xi0 = 0.002 (ising_tsp.cu:61) suits TSPLIB-sized distances; at
    # unit scale its dynamics find no valid tour (checked with the oracle)
    "tsp30": dict(kind="tsp", workload="tsp-30-unit-square-x1000-penalty1.5maxd", cities=30,
                  coord_scale=1000.0, agents=1024, dt=0.1, sb_steps=20000, precision="f16",
                  compare=("bf16", "f32", "f64")),
    "loaders": dict(kind="loaders", workload="loaders", sb_steps=0),
    "batch512": dict(kind="batch", workload="batch-512-maxcut-er+rgg-n100..20000-pm1",
                     instances=512, agents=64, dt=0.5, sb_steps=10000, fused=1,
                     precision="bf16", compare=("f32",)),
}
GRAPH_SEED, INIT_SEED = 1234, 1
PBYTES = {"f32": 4, "bf16": 2, "f16": 2, "f64": 8}
# time to target with restarts: each restart round solves copies of the
# missed instances, as many as keep the round's batch near this share of the
# full batch's rows (at least one copy, at most RESTART_MAX_COPIES)
RESTART_ROWS = 0.1
RESTART_MAX_COPIES = 32


def restart_copies(rows_missed, rows_total):
    """Copies of each missed instance in a restart round: as many as keep the
    round's batch near RESTART_ROWS of the full batch's rows, at least one
    and at most RESTART_MAX_COPIES."""
    return int(min(RESTART_MAX_COPIES, max(1, RESTART_ROWS * rows_total // max(1, rows_missed))))


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) per launch of
# each workload's dominant kernel, from one ncu capture of the same kernel
# and tile (the command is in the source string); the resident kernels'
# launch covers the whole solve.
TRAFFIC = {
    "torus": (45.85e6, "ncu --set full -k regex:k_resident_rs -c 1: bench.py --workload torus "
                       "--profile 20000 --kernel split (one 20,000-step launch)"),
    # per SB step: the k_row launch plus 1/100 of the isolated rows' k_iso
    "rmat20": (9.814e8, "ncu --set full -k regex:k_row|k_iso: bench.py --workload rmat20 "
                        "--profile 100 (k_row launch + k_iso / 100)"),
    "batch512": (1.0662e9, "ncu --set full -k regex:k_bsm -s 4 -c 1: bench.py --workload batch512 "
                           "--profile 100 (one k_bsm launch)"),
    # the whole 2,000-step solve is one launch; per launch of the bench's
    # 20,000-step solve the state read once is the same
    "tsp30": (3.870e6, "ncu --set full -k regex:k_tsp_tc -c 1: bench.py --workload tsp30 "
                       "--profile 2000 --kernel tensor --precision bf16 (one launch)"),
}


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
        self.lines = []

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
        for l in self.lines:
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


def batch_specs(count):
    """The batched workload's instances as (kind, n, degree, seed): n
    log-uniform in [100, 20000], even positions Erdos-Renyi with average
    degree uniform in [6, 40], odd ones random geometric graphs of the same
    degree range; weights +-1."""
    import numpy as np
    rng = np.random.default_rng(GRAPH_SEED)
    out = []
    for i in range(count):
        n = int(round(np.exp(rng.uniform(np.log(100), np.log(20000)))))
        deg = float(rng.uniform(6, 40))
        out.append(("er" if i % 2 == 0 else "rgg", n, deg, GRAPH_SEED + i))
    return out


def batch_graph(spec, gen):
    """One batched instance from its spec, built by `gen`: the engine's
    generators (sbx) or their restatement on the oracle side (sbo), which
    give the same arrays."""
    kind, n, deg, seed = spec
    if kind == "er":
        return gen.gen_er(n, min(1.0, deg / (n - 1)), pm1=True, seed=seed)
    return gen.gen_rgg(n, deg, seed=seed)


def batch_instances(wl, gen=None, count=0):
    """The batch's graphs (the first `count` when given)."""
    if gen is None:
        import sbx as gen
    specs = batch_specs(wl["instances"])
    if count:
        specs = specs[:count]
    return [batch_graph(sp, gen) for sp in specs]


def build_instance(wl, gen=None):
    """The seeded synthetic instance: a Graph, or a dict with the TSP data,
    built by `gen` (sbx by default; sbo on the CPU legs)."""
    if gen is None:
        import sbx as gen
    if wl["kind"] == "maxcut":
        g = wl["graph"]
        if g[0] == "torus":
            return gen.gen_torus(g[1], g[2], seed=GRAPH_SEED)
        if g[0] == "er":
            return gen.gen_er(g[1], g[2], pm1=g[3], seed=GRAPH_SEED)
        return gen.gen_rmat(g[1], g[2], seed=GRAPH_SEED)
    xc, yc = gen.gen_cities(wl["cities"], wl.get("coord_scale", 1.0), seed=GRAPH_SEED)
    packed = gen.tsp_distances(xc, yc, 2)   # EUC_2D_FLOAT: no truncation
    mx = float(packed.max())
    return dict(xc=xc, yc=yc, packed=packed, N=wl["cities"], A=1.0, B=1.5 * mx, C=1.5 * mx)


def oracle_tsp(inst):
    import sbo
    return sbo.Tsp(inst["xc"], inst["yc"], sbo.DIST_EUC_2D_FLOAT, A=inst["A"], B=inst["B"],
                   C_=inst["C"])


def instance_sizes(wl, inst):
    if wl["kind"] == "maxcut":
        return inst.n, inst.nnz
    t = oracle_tsp(inst)
    return t.graph.n, t.graph.nnz


def config_of(wl):
    """The workload's configuration, printed identically by both arms."""
    c = {k: v for k, v in wl.items() if k not in ("compare", "graph")}
    if "graph" in wl:
        c["graph"] = list(wl["graph"])
    c["graph_seed"], c["init_seed"] = GRAPH_SEED, INIT_SEED
    c["l2"] = "flushed between timed iterations (256 MB write)"
    return c


def cpu_sample(wl, inst, seconds=12.0, nthreads=0):
    """The FP64 oracle on a bounded sample of the workload: the same instance
    and agents for s SB steps (OpenMP over rows, every host thread, for MaxCut;
    one thread for TSP).  Returns (nnz*agent*steps/s, cores, s, seconds)."""
    import sbo
    A = wl["agents"]
    if wl["kind"] == "maxcut":
        og = sbo.Graph(inst.n, inst.rowptr, inst.col, inst.val, inst.wsum)
        nnz = inst.nnz
        cores = nthreads if nthreads > 0 else (os.cpu_count() or 1)

        def run(k):
            t0 = time.perf_counter()
            o = sbo.maxcut_solve(og, sbo.params(dt=wl["dt"], steps=k, period=k, agents=A,
                                                seed=INIT_SEED, nthreads=nthreads))
            return time.perf_counter() - t0, o["result"]["steps_run"]
    else:
        t = oracle_tsp(inst)
        nnz = t.graph.nnz
        cores = 1

        def run(k):
            t0 = time.perf_counter()
            o = t.solve(sbo.params(dt=wl["dt"], steps=k, agents=A, seed=INIT_SEED, threshold=50))
            return time.perf_counter() - t0, o["result"]["steps_run"]
    ta, _ = run(10)
    tb, _ = run(30)   # the difference removes the init cost
    per_step = max((tb - ta) / 20.0, 1e-5)
    s = int(max(10, min(wl["sb_steps"], seconds / per_step)))
    s = (s // 10) * 10
    dt, steps = run(s)
    return nnz * A * steps / dt, cores, s, dt


def cpu_batch_sample(wl, graphs, seconds=10.0, cores=0):
    """The FP64 oracle's fused step (the restatement of the reference kernel)
    on every instance of the batch, s steps each, instances spread over the
    host threads (one thread per instance at a time).  The initial state is
    made before the timed region.  Returns (nnz*agent*steps/s, cores, s,
    seconds)."""
    import sbo
    from concurrent.futures import ThreadPoolExecutor
    cores = cores or (os.cpu_count() or 1)
    A, dt, steps = wl["agents"], wl["dt"], wl["sb_steps"]
    st = []
    for i, g in enumerate(graphs):
        og = sbo.Graph(g.n, g.rowptr, g.col, g.val, g.wsum)
        x, y = sbo.init_maxcut(g.n, A, INIT_SEED + i)
        sbo.update_xy(x, y, 0, steps, dt)
        st.append([og, x, y, sbo.xi0(og), 0])
    order = sorted(range(len(st)), key=lambda i: -st[i][0].nnz)

    def run(k):
        def work(i):
            og, x, y, x0, k0 = st[i]
            for j in range(k):
                sbo.fused_step(og, x, y, A, k0 + j, steps, dt, x0, nthreads=1)
            st[i][4] = k0 + k
        t0 = time.perf_counter()
        with ThreadPoolExecutor(cores) as ex:
            list(ex.map(work, order))
        return time.perf_counter() - t0
    t1 = run(1)
    s = int(max(1, min(wl["sb_steps"] // 2, seconds / max(t1, 1e-6))))
    sec = run(s)
    return sum(g.nnz for g in graphs) * A * s / sec, cores, s, sec


def reference_gpu_batch(wl, graphs, seed, every=16):
    """The reference's own kernels on this GPU (oracle/_ref, where they were
    compiled) on every `every`-th instance of the batch, one after another as
    its CLI would run them, full runs: their nnz*agent*steps/s and best cuts.
    None where the reference's kernels were not compiled."""
    import numpy as np
    import sbo
    if not sbo.ref_gpu_available():
        return None
    t_us, units, best = 0.0, 0, []
    for i in range(0, len(graphs), every):
        g = graphs[i]
        og = sbo.Graph(g.n, g.rowptr, g.col, g.val, g.wsum)
        r = sbo.ref_gpu_maxcut(og, wl["agents"], wl["sb_steps"], wl["dt"], seed + i,
                               fused=wl["fused"])
        t_us += r["time_us"]
        units += g.nnz * wl["agents"] * r["steps_run"]
        best.append(r["max"])
    return {"value": units / (t_us / 1e6), "unit": "nnz*agent*steps/s",
            "sample": "every %dth instance (%d), full runs, one after another, the reference's "
                      "kernels and launch shapes, its host-clock time" % (every, len(best)),
            "seconds": t_us / 1e6, "kernels": "src/kernels.cu compiled to PTX, driven as "
                                              "src/ising.cu drives them",
            "best_cuts_mean": float(np.mean(best))}


def run_reference(args, wl, rank):
    """--impl reference: the reference path has no CPU solver, so its CPU
    implementation here is the FP64 oracle port, every host thread."""
    if rank != 0:
        return
    import sbo
    sbo.lib()
    vals, samples, cores = [], [], 1
    if wl["kind"] == "batch":
        # the instances through the oracle's generators: nothing of the
        # engine is loaded by this arm
        graphs = batch_instances(wl, gen=sbo, count=args.instances)
        for i in range(args.warmup + args.steps):
            v, cores, s, dt = cpu_batch_sample(wl, graphs, seconds=4.0)
            if i >= args.warmup:
                vals.append(v)
                samples.append((s, dt))
        what = "FP64 oracle fused step, %d SB steps of each of the %d instances per bench step" % (
            samples[0][0], len(graphs))
    else:
        inst = build_instance(wl, gen=sbo)
        for i in range(args.warmup + args.steps):
            v, cores, s, dt = cpu_sample(wl, inst, seconds=8.0)
            if i >= args.warmup:
                vals.append(v)
                samples.append((s, dt))
        what = "%d SB steps of the workload per bench step" % samples[0][0]
    value = sum(vals) / len(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "nnz*agent*steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000.0 * sum(d for _, d in samples) / len(samples),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generators)", "config": config_of(wl),
        "cpu_baseline": {"value": value, "unit": "nnz*agent*steps/s", "cores": cores,
                         "kind": "port", "sample": what},
        "e2e": {"value": value, "unit": "nnz*agent*steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    # the CPU arm runs the reference's path as the oracle restates it, and
    # nothing of the engine
    if "sbx" in sys.modules:
        raise RuntimeError("the reference arm loaded the engine")
    print(json.dumps(line), flush=True)


def run_loaders(args):
    """--workload loaders: the file loaders of the path (src/csr.cpp:15-192,
    src/tsp_cpu.cpp:9-45) on files of the workloads' sizes -- the R-MAT
    scale-20 graph as a symmetric pattern MTX and 100,000 cities as a TSPLIB
    EUC_2D file, both written here from the seeded generators.  Timed: the
    engine's loader (sbx_load_mtx / sbx_load_tsplib, every host thread), the
    oracle's single-thread restatement, and the reference's own loaders
    compiled from its sources (oracle/_ref, only where they were built: the
    GPU machine has no reference sources).  Each is the fastest of `--steps`
    parses, with the arrays allocated beforehand."""
    import ctypes as C
    import tempfile
    import numpy as np
    import sbo
    import sbx
    reps = max(1, args.steps)
    tmp = tempfile.mkdtemp(prefix="sbx_loaders_")
    g = sbo.gen_rmat(20, 4, seed=GRAPH_SEED)
    rows = np.repeat(np.arange(g.n, dtype=np.int64), np.diff(g.rowptr))
    up = g.col > rows
    mtx = os.path.join(tmp, "rmat20.mtx")
    with open(mtx, "w") as f:
        f.write("%%%%MatrixMarket matrix coordinate pattern symmetric\n%d %d %d\n" % (g.n, g.n, int(up.sum())))
        np.savetxt(f, np.stack([rows[up] + 1, g.col[up].astype(np.int64) + 1], 1), fmt="%d")
    ncity = 100000
    rng = np.random.default_rng(GRAPH_SEED)
    tsp = os.path.join(tmp, "c100k.tsp")
    with open(tsp, "w") as f:
        f.write("NAME: c100k\nTYPE: TSP\nDIMENSION: %d\nEDGE_WEIGHT_TYPE: EUC_2D\nNODE_COORD_SECTION\n" % ncity)
        np.savetxt(f, np.column_stack([np.arange(1, ncity + 1), rng.uniform(0, 1e6, ncity),
                                       rng.uniform(0, 1e6, ncity)]), fmt=["%d", "%.3f", "%.3f"])
        f.write("EOF\n")

    def best(fn):
        t = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            t.append(time.perf_counter() - t0)
        return min(t)

    def mtx_timer(lib_fn):
        n, nnz, w = C.c_int64(), C.c_int64(), C.c_double()
        rc = lib_fn(mtx.encode(), C.byref(n), C.byref(nnz), None, None, None, C.byref(w))
        if rc != 0:
            raise RuntimeError("MTX load failed: %d" % rc)
        rp = np.empty(n.value + 1, np.int32)
        col = np.empty(nnz.value, np.int32)
        val = np.empty(nnz.value)
        args_ = (mtx.encode(), C.byref(n), C.byref(nnz), rp.ctypes.data_as(C.c_void_p),
                 col.ctypes.data_as(C.c_void_p), val.ctypes.data_as(C.c_void_p), C.byref(w))
        return best(lambda: lib_fn(*args_)), int(n.value), int(nnz.value)

    def tsp_timer(lib_fn):
        N, kind = C.c_int32(), C.c_int32()
        if lib_fn(tsp.encode(), C.byref(N), None, None, C.byref(kind)) != 0:
            raise RuntimeError("TSPLIB load failed")
        xc, yc = np.empty(N.value), np.empty(N.value)
        a_ = (tsp.encode(), C.byref(N), xc.ctypes.data_as(C.c_void_p), yc.ctypes.data_as(C.c_void_p),
              C.byref(kind))
        return best(lambda: lib_fn(*a_))

    mb = os.path.getsize(mtx) / 1e6
    tb = os.path.getsize(tsp) / 1e6
    te, n, nnz = mtx_timer(sbx.lib().sbx_load_mtx)
    to, _, _ = mtx_timer(sbo.lib().sbo_mtx_load)
    tte = tsp_timer(sbx.lib().sbx_load_tsplib)
    tto = tsp_timer(sbo.lib().sbo_tsplib_load)
    ref = os.path.join(ORACLE, "_ref", "ref_kernels")
    refl = {"unavailable": "the reference's loaders are built only where its sources are "
                           "(oracle/_ref); none on this machine"}
    if os.path.exists(ref):
        try:
            o1 = subprocess.run([ref, "mtx-time", mtx, str(reps)], capture_output=True, text=True, check=True)
            o2 = subprocess.run([ref, "tsplib-time", tsp, str(reps)], capture_output=True, text=True,
                                check=True)
            # the timing is the last line (the reference's loader prints too)
            tr1 = float(o1.stdout.strip().splitlines()[-1].split()[0])
            tr2 = float(o2.stdout.strip().splitlines()[-1].split()[0])
            refl = {"mtx_s": tr1, "mtx_MB_per_s": mb / tr1, "tsplib_s": tr2, "tsplib_MB_per_s": tb / tr2,
                    "cores": 1, "kind": "reference",
                    "code": "src/csr.cpp CSR(path) and src/tsp_cpu.cpp TSP_CPU(path), compiled with g++ -O2"}
        except Exception as e:   # noqa: BLE001
            refl = {"unavailable": "reference loader run failed: %s" % e}
    import shutil
    shutil.rmtree(tmp, ignore_errors=True)
    host_threads = min(os.cpu_count() or 1, 64)
    line = {"metric": "MTX parse + CSR build MB/s", "value": mb / te, "unit": "MB/s",
            "higher_is_better": True, "workload": "loaders", "steps": reps,
            "data": "synthetic (seeded generators), written as text files",
            "config": {"workload": "loaders", "mtx": "R-MAT scale 20, edge factor 4, pattern symmetric",
                       "mtx_MB": mb, "n": n, "nnz": nnz, "tsplib": "100,000 cities EUC_2D (the loader's largest)",
                       "tsplib_MB": tb},
            "engine": {"mtx_s": te, "mtx_MB_per_s": mb / te, "tsplib_s": tte, "tsplib_MB_per_s": tb / tte,
                       "cores": host_threads},
            "oracle_port": {"mtx_s": to, "mtx_MB_per_s": mb / to, "tsplib_s": tto,
                            "tsplib_MB_per_s": tb / tto, "cores": 1},
            "reference": refl}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batch512", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--sb-steps", type=int, default=0,
                    help="SB steps per solve (profiling cases use fewer)")
    ap.add_argument("--profile", type=int, default=0, metavar="STEPS",
                    help="one solve of STEPS SB steps of the workload and exit, kernels "
                         "launched directly: the case the ncu summaries capture")
    ap.add_argument("--kernel", default="auto", choices=["auto", "stream", "resident", "split", "tensor"],
                    help="--profile: kernel family")
    ap.add_argument("--tile", default="", metavar="V,LR,BT,CM",
                    help="--profile: streaming tile (agents per lane, lanes per row, threads, "
                         "count mode 1 bytes / 2 bit planes / 4 shared-memory planes, batched); "
                         "default: the fixed heuristic")
    ap.add_argument("--legs", default="all", choices=["all", "main"],
                    help="main: only the timed solves of the main precision (profiling)")
    ap.add_argument("--instances", type=int, default=0, metavar="K",
                    help="batch512: only the first K instances (sub-batch sizes)")
    ap.add_argument("--step-times", action="store_true",
                    help="--profile: time every step kernel (events) and print microseconds per step")
    ap.add_argument("--precision", default="", choices=["", "f32", "bf16", "f16", "f64"],
                    help="--profile: the state precision (default: the workload's)")
    args = ap.parse_args()
    wl = dict(WORKLOADS[args.workload])
    if args.sb_steps:
        wl["sb_steps"] = args.sb_steps
    if args.precision and args.profile:
        wl["precision"] = args.precision

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.workload == "loaders":
        if rank == 0:
            run_loaders(args)
        return
    if args.impl == "reference":
        run_reference(args, wl, rank)
        return
    if args.profile:
        run_profile_case(args, wl)
        return
    if wl["kind"] == "batch":
        run_batch(args, wl, rank, world, local)
        return

    import torch
    import sbx
    import replicas

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
    inst = build_instance(wl)
    A = wl["agents"]
    n, nnz = instance_sizes(wl, inst)

    def make_problem():
        if wl["kind"] == "maxcut":
            return ctx.problem(inst)
        return ctx.tsp_problem(inst["packed"], inst["N"], A=inst["A"], B=inst["B"], C_=inst["C"])

    prob = make_problem()
    seed = INIT_SEED + rank   # each rank: an independent replica (weak scaling)

    def prm(prec, flags=0):
        kw = dict(dt=wl["dt"], steps=wl["sb_steps"], agents=A, seed=seed,
                  precision=sbx.PRECISIONS[prec], flags=flags)
        if wl["kind"] == "maxcut":
            kw.update(fused=wl["fused"], update_window=wl["update_window"])
        return sbx.params(**kw)

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def quality(r):
        return r["max"] if wl["kind"] == "maxcut" else r["min"]

    def timed(prec, k, w):
        for _ in range(w):
            ctx.solve(prob, prm(prec))
        evs, units, launches, res = [], 0, 0, None
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        with Clocks(local) as clk:
            for _ in range(k):
                flush.fill_(1)   # L2 flush between iterations
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                res, _ = ctx.solve(prob, prm(prec))
                e1.record(stream)
                evs.append((e0, e1))
                units += nnz * A * res["steps_run"]
                launches += res["gpu_launches"]
            torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in evs)
        # replicas: the slowest rank's time, all ranks' work
        ms, units = replicas.reduce_timing(ms, units, device="cuda")
        return units / (ms / 1000.0), ms / k, res, clk.summary(), launches // max(k, 1)

    main_prec = wl["precision"]
    v_main, ms_main, r_main, clocks, launches = timed(main_prec, args.steps, args.warmup)
    if args.legs == "main":
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": v_main, "ms_per_step": ms_main,
                              "config": config_of(wl), "legs": "main"}), flush=True)
        ctx.close()
        return

    # The same solve in the other precisions: throughput and best result.
    others = {}
    for prec in wl["compare"]:
        if prec == "f64":
            rr, _ = ctx.solve(prob, prm("f64"))
            others["f64"] = {"best": quality(rr), "steps_run": rr["steps_run"],
                             "ms": rr["time_us"] / 1000.0}
        else:
            v, ms, rr, _, _ = timed(prec, 1, 1)
            others[prec] = {"value": v, "ms_per_step": ms, "best": quality(rr),
                            "steps_run": rr["steps_run"]}

    # Time to target: the first window whose best cut reaches the FP32-plain
    # best cut less 0.1%, in the main precision and in FP32 (device clock from
    # the loop start; the per-window cut is part of the timed loop).
    ttt = None
    if wl["kind"] == "maxcut" and main_prec != "f32" and "f32" in others:
        b32 = others["f32"]["best"]
        target = b32 - 1e-3 * abs(b32)

        def prm_t(prec):
            p = prm(prec)
            p.target = target
            return p
        rt, _ = ctx.solve(prob, prm_t(main_prec))
        r32, _ = ctx.solve(prob, prm_t("f32"))
        ttt = {"target": target, "rule": "FP32-plain best cut less 0.1%",
               main_prec + "_us": rt["time_to_target_us"], main_prec + "_steps": rt["steps_to_target"],
               "f32_plain_us": r32["time_to_target_us"], "f32_plain_steps": r32["steps_to_target"],
               "speedup": (r32["time_to_target_us"] / rt["time_to_target_us"]
                           if rt["time_to_target_us"] > 0 and r32["time_to_target_us"] > 0 else None)}

    # e2e: through the C ABI from host buffers, upload + solve + read-back.
    t_e2e, units_e2e = [], 0
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p2 = make_problem()
        r2, _ = ctx.solve(p2, prm(main_prec))
        p2.close()
        torch.cuda.synchronize()
        if i >= args.warmup:
            t_e2e.append(time.perf_counter() - t0)
            units_e2e += nnz * A * r2["steps_run"]
    e2e = units_e2e / sum(t_e2e)
    if wl["kind"] == "maxcut":
        h2d = int(inst.rowptr.nbytes + inst.col.nbytes + inst.val.nbytes)
    else:
        h2d = int(inst["packed"].nbytes)
    d2h = int(8 * A + 64)

    # Dominant kernel, timed launch by launch (SBX_FLAG_PROFILE).
    rp, _ = ctx.solve(prob, prm(main_prec, sbx.FLAG_PROFILE))
    peaks, peak_kind = load_peaks()
    s = PBYTES[main_prec]
    b_step = 2 * n * A * (s + s) + 8 * nnz + 4 * (n + 1)
    roof = None
    if rp["kernel_launches"] and rp["kernel_ms"] > 0:
        per_launch_s = rp["kernel_ms"] / 1000.0 / rp["kernel_launches"]
        niso = int((inst.rowptr[1:] == inst.rowptr[:-1]).sum()) if wl["kind"] == "maxcut" else 0
        if rp["kernel_used"] == sbx.KERNEL_STREAM and niso and wl["fused"]:
            # isolated rows advance a window per k_iso launch (in registers):
            # the unit is one SB step, its k_row launch plus 1/100 of k_iso
            bytes_per_launch = b_step
            kname = ("k_row + k_iso/100 (one SB step; %d isolated rows advanced a 100-step window "
                     "per k_iso launch, effective bytes)" % niso)
        elif rp["kernel_used"] == sbx.KERNEL_STREAM:
            bytes_per_launch, kname = b_step, "k_row (one SB step per launch)"
        elif rp["kernel_used"] == sbx.KERNEL_TENSOR:
            bytes_per_launch, kname = None, "k_tsp_tc (the whole solve in one launch)"
        else:
            # on-chip kernels run many steps per launch: B_step per step run
            bytes_per_launch = b_step * rp["steps_run"] / rp["kernel_launches"]
            kname = "resident (many steps per launch; state on chip, effective bytes)"
        tr = TRAFFIC.get(args.workload)
        if bytes_per_launch is None:
            # the TSP distance product on the tensor cores: 2 N^3 FLOP per
            # agent and step (the algorithm's), against the bf16 peak; the
            # MMAs issue 12 per 128-row tile (D in three exact parts, both
            # neighbour positions, 32-padded cities)
            Nc = wl["cities"]
            flops = 2.0 * Nc ** 3 * A * rp["steps_run"] / rp["kernel_launches"]
            tiles = -(-Nc * 8 // 128)
            issued = 12 * tiles * 2 * 128 * 32 * 16 * (-(-A // 8)) * rp["steps_run"] / rp["kernel_launches"]
            achieved = flops / per_launch_s / 1e12
            roof = {"bound": "tensor", "achieved": achieved, "peak": peaks["bf16_tflops"],
                    "unit": "TFLOP/s", "frac": achieved / peaks["bf16_tflops"],
                    "traffic": tr[0] if tr else None, "traffic_source": tr[1] if tr else None,
                    "peak_kind": peak_kind + " (bf16 burst)", "kernel": kname,
                    "flops_per_launch": flops, "issued_mma_flops_per_launch": issued,
                    "launch_us": per_launch_s * 1e6, "launches": rp["kernel_launches"],
                    "step_us": per_launch_s * 1e6 * rp["kernel_launches"] / rp["steps_run"]}
        else:
            achieved = bytes_per_launch / per_launch_s / 1e9
            roof = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                    "frac": achieved / peaks["hbm_gbs"], "traffic": tr[0] if tr else None,
                    "traffic_source": tr[1] if tr else None, "peak_kind": peak_kind,
                    "kernel": kname, "bytes_per_launch": bytes_per_launch,
                    "launch_us": per_launch_s * 1e6, "launches": rp["kernel_launches"]}

    ref_gpu = None
    if rank == 0 and world == 1 and wl["kind"] == "tsp":
        import sbo
        if sbo.ref_gpu_available():
            rr = sbo.ref_gpu_tsp(oracle_tsp(inst), A, wl["sb_steps"], wl["dt"], seed)
            ref_gpu = {"value": nnz * A * rr["steps_run"] / (rr["time_us"] / 1e6),
                       "unit": "nnz*agent*steps/s", "seconds": rr["time_us"] / 1e6,
                       "best": rr["min"], "valid": rr["valid"], "steps_run": rr["steps_run"],
                       "kernels": "src/kernels.cu compiled to PTX, driven as src/ising_tsp.cu "
                                  "drives them (FP64 CSR, its launch shapes, host-clock time)"}
    if rank == 0 and world == 1 and wl["kind"] == "maxcut":
        import sbo
        if sbo.ref_gpu_available():
            og = sbo.Graph(inst.n, inst.rowptr, inst.col, inst.val, inst.wsum)
            rr = sbo.ref_gpu_maxcut(og, A, wl["sb_steps"], wl["dt"], seed, uw=wl["update_window"],
                                    fused=wl["fused"])
            ref_gpu = {"value": nnz * A * rr["steps_run"] / (rr["time_us"] / 1e6),
                       "unit": "nnz*agent*steps/s", "seconds": rr["time_us"] / 1e6,
                       "best": rr["max"], "steps_run": rr["steps_run"],
                       "kernels": "src/kernels.cu compiled to PTX, driven as src/ising.cu "
                                  "drives them (FP64, its launch shapes, host-clock time)"}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        v, cores, s_cpu, dt = cpu_sample(wl, inst)
        cpu = {"value": v, "unit": "nnz*agent*steps/s", "cores": cores, "kind": "port",
               "sample": "FP64 oracle, %d SB steps of the workload (%.1f s)" % (s_cpu, dt)}

    if rank == 0:
        refk = "f64" if "f64" in others else ("f32" if "f32" in others else None)
        ref = others.get(refk) if refk else None
        err = None
        if ref and ref["best"] and abs(ref["best"]) < 1e300 and abs(quality(r_main)) < 1e300:
            err = abs(quality(r_main) - ref["best"]) / abs(ref["best"])
        qual = {"best_" + main_prec: quality(r_main), "steps_run": r_main["steps_run"],
                "kernel": r_main["kernel_used"], "energy_error_vs_%s" % refk: err}
        if wl["kind"] == "tsp":
            qual["valid_agents"] = r_main["valid"]
        else:
            qual["ps"] = r_main["ps"]
        line = {
            "metric": METRIC, "value": v_main, "unit": "nnz*agent*steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_main,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": main_prec, "data": "synthetic (seeded generators)",
            "config": config_of(wl),
            "shape": {"n": n, "nnz": nnz, "parallelism": "replicas" if world > 1 else "single",
                      "state": "%s storage, fp32 arithmetic, exact integer force" % main_prec},
            "e2e": {"value": e2e, "unit": "nnz*agent*steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "roofline": roof,
            "cpu_baseline": cpu,
            "reference_gpu": ref_gpu,
            "clocks": clocks,
            "other_precisions": others,
            "quality": qual,
            "time_to_target": ttt,
            "tile": {k: r_main[k] for k in ("lane_agents", "row_lanes", "block_threads",
                                            "count_mode", "staging", "agents_per_block")},
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()



def run_profile_case(args, wl):
    """--profile STEPS: one solve (batched: one solve_batch) of the workload
    with STEPS SB steps of its schedule, no CUDA graph, the tile pinned --
    a small, repeatable case for ncu captures."""
    import sbx
    kern = {"auto": sbx.KERNEL_AUTO, "stream": sbx.KERNEL_STREAM, "resident": sbx.KERNEL_RESIDENT,
            "split": sbx.KERNEL_RESIDENT_SPLIT, "tensor": sbx.KERNEL_TENSOR}[args.kernel]
    kw = dict(dt=wl["dt"], steps=wl["sb_steps"], run_steps=args.profile, seed=INIT_SEED,
              precision=sbx.PRECISIONS[wl["precision"]], kernel=kern,
              flags=sbx.FLAG_NO_GRAPH | sbx.FLAG_NO_TUNE | (sbx.FLAG_PROFILE if args.step_times else 0))
    if args.tile:
        v, lr, bt, cm = (int(t) for t in args.tile.split(","))
        if cm == 4:   # the shared-memory-plane batch kernel: its CTA size only
            kw.update(block_threads=bt, count_mode=cm)
        else:
            kw.update(lane_agents=v, row_lanes=lr, block_threads=bt, count_mode=cm)
    ctx = sbx.Context(0)
    size = {}
    if wl["kind"] == "batch":
        graphs = batch_instances(wl, count=args.instances)
        size = {"instances": len(graphs), "rows": sum(g.n for g in graphs), "nnz": sum(g.nnz for g in graphs)}
        probs = [ctx.problem(g) for g in graphs]
        res, _, t = ctx.solve_batch(probs, [wl["agents"]] * len(probs), sbx.params(fused=wl["fused"], **kw))
        r = res[0]
    else:
        inst = build_instance(wl)
        if wl["kind"] == "maxcut":
            prob = ctx.problem(inst)
            kw.update(fused=wl["fused"], update_window=wl["update_window"])
        else:
            prob = ctx.tsp_problem(inst["packed"], inst["N"], A=inst["A"], B=inst["B"], C_=inst["C"])
        r, _ = ctx.solve(prob, sbx.params(agents=wl["agents"], **kw))
    line = {"profile": wl["workload"], "steps_run": r["steps_run"], "kernel": r["kernel_used"],
            "tile": [r["lane_agents"], r["row_lanes"], r["block_threads"], r["count_mode"]],
            "time_us": r["time_us"], **size}
    if args.step_times and r["steps_run"]:
        line["step_us"] = 1000.0 * r["kernel_ms"] / r["steps_run"]
    print(json.dumps(line), flush=True)
    ctx.close()


def run_batch(args, wl, rank, world, local):
    """The batched workload: every instance packed into one block-diagonal
    run per bench step (sbx_solve_batch), against the FP32-plain mode (each
    instance solved alone, FP32 state) for throughput, best cut and time to
    target, and against the FP64 run of the same seeds for the energy error."""
    import numpy as np
    import torch
    import sbx
    import replicas
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = sbx.Context(local)
    ctx.set_stream(stream.cuda_stream)
    graphs = batch_instances(wl, count=args.instances)
    A = wl["agents"]
    agents = [A] * len(graphs)
    probs = [ctx.problem(g) for g in graphs]
    n_tot = sum(g.n for g in graphs)
    nnz_tot = sum(g.nnz for g in graphs)
    units_per = nnz_tot * A
    seed = INIT_SEED + rank
    prm = lambda prec, flags=0: sbx.params(dt=wl["dt"], steps=wl["sb_steps"], seed=seed,
                                           fused=wl["fused"], precision=sbx.PRECISIONS[prec],
                                           flags=flags)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        ctx.solve_batch(probs, agents, prm(wl["precision"]))
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    evs, res = [], None
    with Clocks(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1)   # L2 flush between iterations
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            res, vals, _ = ctx.solve_batch(probs, agents, prm(wl["precision"]))
            e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in evs) / args.steps
    steps_run = res[0]["steps_run"]
    # replicas: the slowest rank's time, all ranks' work
    ms, units_all = replicas.reduce_timing(ms, units_per * steps_run, device="cuda")
    value = units_all / (ms / 1000.0)
    if args.legs == "main":
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "ms_per_step": ms,
                              "config": config_of(wl), "legs": "main"}), flush=True)
        ctx.close()
        return
    best_b = np.array([r["max"] for r in res])
    launches = res[0]["gpu_launches"]

    # e2e through the C ABI from host buffers: every instance's CSR uploaded
    # (sbx_problem_csr), the batched solve, the per-agent cuts read back
    e2e_w, e2e_k = min(args.warmup, 2), max(1, min(args.steps, 5))
    t_e2e = []
    for i in range(e2e_w + e2e_k):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        p2 = [ctx.problem(g) for g in graphs]
        ctx.solve_batch(p2, agents, prm(wl["precision"]))
        for p in p2:
            p.close()
        torch.cuda.synchronize()
        if i >= e2e_w:
            t_e2e.append(time.perf_counter() - t0)
    e2e = units_per * steps_run / (sum(t_e2e) / len(t_e2e))

    # FP32-plain: each instance alone (seed + i, as the batch seeds it)
    t_plain, best_p = 0.0, []
    for i, p in enumerate(probs):
        r, _ = ctx.solve(p, sbx.params(dt=wl["dt"], steps=wl["sb_steps"], agents=A, seed=seed + i,
                                       fused=wl["fused"], precision=sbx.F32))
        t_plain += r["time_us"] / 1e6
        best_p.append(r["max"])
    best_p = np.array(best_p)
    v_plain = units_per * wl["sb_steps"] / t_plain
    rel = (best_p - best_b) / np.abs(best_p)
    # the FP64 run of the same seeds (bit-exact with the FP64 oracle): the
    # energy error of the batch's best cuts
    r64, _, _ = ctx.solve_batch(probs, agents, prm("f64"))
    best_64 = np.array([r["max"] for r in r64])
    err64 = np.abs(best_b - best_64) / np.abs(best_64)
    # Time to target: per instance, the FP32-plain best cut less 0.1%.  The
    # batch reaches all targets when its slowest instance does; FP32-plain
    # solves the instances one after another.
    targets = best_p - 1e-3 * np.abs(best_p)
    rt, _, _ = ctx.solve_batch(probs, agents, prm(wl["precision"]), targets=targets)
    tb = np.array([r["time_to_target_us"] for r in rt])
    tp = []
    for i, p in enumerate(probs):
        r, _ = ctx.solve(p, sbx.params(dt=wl["dt"], steps=wl["sb_steps"], agents=A, seed=seed + i,
                                       fused=wl["fused"], precision=sbx.F32, target=targets[i]))
        tp.append(r["time_to_target_us"])
    tp = np.array(tp)
    reached = tb > 0
    # Restarts: the instances the batch missed are solved again from other
    # seeds, several copies of each in one smaller batch (every copy has its
    # own seed, the batch seeding entry k with seed + k; the copy count keeps
    # the round near RESTART_ROWS of the full batch's rows, so a round costs
    # about a tenth of the first and the last few instances get many seeds),
    # until every instance has reached its target (at most 8 rounds).  An
    # instance is reached in a round when one of its copies is, at that
    # copy's time.  The first round counts whole (its misses are known only
    # at its end), so does every round that still misses one; the round that
    # reaches the last targets counts up to its slowest instance.
    t_restart = float(np.max(tb)) if reached.all() else None
    rounds, missed = 0, np.nonzero(~reached)[0]
    left, round_us, copies_used = [int(len(missed))], [], []
    if not reached.all():
        t_restart = float(rt[0]["time_us"]) if rt[0]["time_us"] > 0 else None
        while len(missed) and rounds < 8 and t_restart is not None:
            rounds += 1
            copies = restart_copies(sum(graphs[i].n for i in missed), n_tot)
            copies_used.append(copies)
            rep = np.repeat(missed, copies)
            rr, _, t_sub = ctx.solve_batch([probs[i] for i in rep], [A] * len(rep), sbx.params(
                dt=wl["dt"], steps=wl["sb_steps"], seed=seed + 100000 * rounds, fused=wl["fused"],
                precision=sbx.PRECISIONS[wl["precision"]]), targets=targets[rep])
            tr_ = np.array([r["time_to_target_us"] for r in rr]).reshape(len(missed), copies)
            hit = np.where(tr_ > 0, tr_, np.inf).min(axis=1)
            ok = np.isfinite(hit)
            t_round = float(hit.max()) if ok.all() else float(t_sub)
            t_restart += t_round
            round_us.append(t_round)
            missed = missed[~ok]
            left.append(int(len(missed)))
        if len(missed):
            t_restart = None
    ttt = {"rule": "per instance: FP32-plain best cut less 0.1%",
           "batched_reached": float(np.mean(reached)),
           "batched_all_us": float(tb.max()) if reached.all() else None,
           "batched_reached_us": float(tb[reached].max()) if reached.any() else None,
           "fp32_plain_us": float(tp.sum()),
           "speedup": float(tp.sum() / tb.max()) if reached.all() else None,
           "missed": [int(i) for i in np.nonzero(~reached)[0]],
           "with_restarts": {"rounds": rounds, "all_reached": t_restart is not None,
                             "copies_per_round": copies_used,
                             "missed_after_each_round": left,
                             "round_us": round_us,
                             "missed_rows": [int(graphs[i].n) for i in missed],
                             "batched_us": t_restart,
                             "speedup": float(tp.sum() / t_restart) if t_restart else None}}
    peaks, peak_kind = load_peaks()
    b_step = 2 * n_tot * A * (PBYTES[wl["precision"]] * 2) + 8 * nnz_tot + 4 * (n_tot + len(graphs))
    rp, _, _ = ctx.solve_batch(probs, agents, prm(wl["precision"], sbx.FLAG_PROFILE))
    roof = None
    if rp[0]["kernel_ms"] > 0:
        per_launch_s = rp[0]["kernel_ms"] / 1000.0 / rp[0]["steps_run"]
        achieved = b_step / per_launch_s / 1e9
        tr = TRAFFIC.get("batch512") if not args.instances else None
        roof = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "traffic": tr[0] if tr else None,
                "traffic_source": tr[1] if tr else None, "peak_kind": peak_kind,
                "kernel": "step kernel, one launch per SB step over all instances",
                "bytes_per_launch": b_step, "launch_us": per_launch_s * 1e6,
                "launches": rp[0]["kernel_launches"]}
    # the same instances in FP16 state, and in FP32 from other seeds (the
    # seed-to-seed spread of the best cut that any other trajectory shows)
    spread = {}
    for label, prec, off in (("f16", "f16", 0), ("f32_other_seeds", "f32", 100000)):
        rs, _, _ = ctx.solve_batch(probs, agents, sbx.params(
            dt=wl["dt"], steps=wl["sb_steps"], seed=seed + off, fused=wl["fused"],
            precision=sbx.PRECISIONS[prec]))
        b = np.array([r["max"] for r in rs])
        g_ = (best_p - b) / np.abs(best_p)
        spread[label] = {"within_0.1pct_of_fp32_plain": float(np.mean(g_ <= 1e-3)),
                         "mean_rel_gap": float(np.mean(g_)), "max_rel_gap": float(np.max(g_))}
    ref_gpu = reference_gpu_batch(wl, graphs, seed) if rank == 0 and world == 1 else None
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        v, cores, s_cpu, dt = cpu_batch_sample(wl, graphs, seconds=10.0)
        cpu = {"value": v, "unit": "nnz*agent*steps/s", "cores": cores, "kind": "port",
               "sample": "FP64 oracle fused step, %d SB steps of each of the %d instances "
                         "(%.1f s)" % (s_cpu, len(graphs), dt)}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "nnz*agent*steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": wl["precision"], "data": "synthetic (seeded generators)",
            "config": config_of(wl),
            "shape": {"instances": len(graphs), "rows": n_tot, "nnz": nnz_tot,
                      "parallelism": "replicas" if world > 1 else "single"},
            "e2e": {"value": e2e, "unit": "nnz*agent*steps/s",
                    "h2d_bytes_per_step": int(sum(g.rowptr.nbytes + g.col.nbytes + g.val.nbytes
                                                  for g in graphs)),
                    "d2h_bytes_per_step": int(8 * A * len(graphs)),
                    "warmup": e2e_w, "samples": e2e_k},
            "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "fp32_plain": {"value": v_plain, "speedup_of_batched": value / v_plain,
                           "seconds": t_plain},
            "quality": {"instances": len(graphs),
                        "within_0.1pct_of_fp32_plain": float(np.mean(rel <= 1e-3)),
                        "mean_rel_gap": float(np.mean(rel)), "max_rel_gap": float(np.max(rel)),
                        "energy_error_vs_f64": {"mean": float(np.mean(err64)),
                                                "max": float(np.max(err64))},
                        "other_runs": spread},
            "reference_gpu": ref_gpu,
            "time_to_target": ttt,
            "tile": {k: res[0][k] for k in ("kernel_used", "lane_agents", "row_lanes",
                                            "block_threads", "count_mode", "staging")},
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
