"""The reference's own CUDA kernels on the same GPU, beside the engine.

oracle/_ref/ref_kernels.ptx is the reference's src/kernels.cu compiled to PTX
where the reference sources are (oracle/Makefile); oracle/_ref/libref_gpu.so
drives those kernels as src/ising.cu does.  The tests skip where the PTX was
not built.

* The set-up (configuration 1: ER n=800, 1024 agents, dt 0.1): the
  reference's initial state after its pre-step Update_XY equals the oracle's
  (to the rounding of its compiler's fused multiply-adds).
* Its trajectories are not reproducible: the kernel updates X in place while
  other threads gather it (src/kernels.cu:225-262), and early in a run, when
  many x sit near zero, a gathered neighbour that has already moved this step
  flips sign often.  After one window the reference's state is a different
  trajectory from the Jacobi restatement's (and from another run's), so the
  comparison is on whole runs:
* Whole runs of configurations 1 and 2: the reference's best cut, and the
  engine's FP32-plain best cut from the same seed within 0.5% of it.
"""
import numpy as np
import pytest

import bench
import sbx
from conftest import oracle_graph

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def oracle_ref(oracle):
    if not oracle.ref_gpu_available():
        pytest.skip("the reference's kernels were not compiled to PTX (no reference sources here)")
    return oracle


def test_reference_gpu_setup_matches_the_oracle(oracle_ref):
    oracle = oracle_ref
    wl = bench.WORKLOADS["er800"]
    g = bench.build_instance(wl, oracle)
    A, steps, dt = wl["agents"], wl["sb_steps"], wl["dt"]
    r = oracle.ref_gpu_maxcut(g, A, steps, dt, 1, run_windows=-1, want_state=True)
    assert r["steps_run"] == 0 and r["windows_run"] == 0
    x, y = oracle.init_maxcut(g.n, A, 1)
    oracle.update_xy(x, y, 0, steps, dt)
    assert np.max(np.abs(r["x"] - x)) <= 1e-15 and np.max(np.abs(r["y"] - y)) <= 1e-15


@pytest.mark.parametrize("name", ["er800", "torus"])
def test_reference_gpu_whole_run_and_engine_fp32_plain(oracle_ref, name):
    oracle = oracle_ref
    wl = bench.WORKLOADS[name]
    g = bench.build_instance(wl, oracle)
    A, steps, dt, uw = wl["agents"], wl["sb_steps"], wl["dt"], wl["update_window"]
    r = oracle.ref_gpu_maxcut(g, A, steps, dt, 1, uw=uw)
    assert r["max"] > 0 and r["time_us"] > 0
    ctx = sbx.Context(0)
    gs = bench.build_instance(wl)
    e, cut = ctx.solve(ctx.problem(gs), sbx.params(dt=dt, steps=steps, agents=A, seed=1,
                                                   update_window=uw, precision=sbx.F32))
    assert abs(e["max"] - r["max"]) <= 5e-3 * r["max"]
    # the cut of the reference's reported best equals an exact cut evaluation
    # of some spin assignment: integer-valued for integer weights
    assert r["max"] == np.floor(r["max"])
    ctx.close()


def test_reference_gpu_tsp_whole_run_and_engine(oracle_ref):
    # TSP with 30 cities and 1024 agents (the TSP workload, its 20,000
    # steps): the reference's kernels (FP64, X updated in place) and the
    # engine's FP64 run and FP16 / BF16 tensor-core runs from the same seed
    # find valid tours of comparable length.  The best of 1024 agents is
    # still noisy at a fifth of the steps: BF16 state (8-bit mantissa) ended
    # 6.7% above the reference's best at 4,000 steps, while at 20,000 steps
    # all of them lie within 1%.
    oracle = oracle_ref
    wl = dict(bench.WORKLOADS["tsp30"])
    inst = bench.build_instance(wl, oracle)
    t = bench.oracle_tsp(inst)
    A, steps, dt = wl["agents"], wl["sb_steps"], wl["dt"]
    r = oracle.ref_gpu_tsp(t, A, steps, dt, 1)
    assert r["steps_run"] == steps and r["time_us"] > 0
    assert r["valid"] > 0 and np.isfinite(r["min"])
    ctx = sbx.Context(0)
    prob = ctx.tsp_problem(inst["packed"], inst["N"], A=inst["A"], B=inst["B"], C_=inst["C"])
    for prec in (sbx.F64, sbx.F16, sbx.BF16):
        e, lengths = ctx.solve(prob, sbx.params(dt=dt, steps=steps, agents=A, seed=1, precision=prec))
        assert e["valid"] > 0
        # within 5% of the reference's best tour (different trajectories)
        assert abs(e["min"] - r["min"]) <= 0.05 * r["min"]
    ctx.close()
