"""Failure detection without a GPU fault: the bounded device waits give up,
flag the error and return, and the solve reports SBX_ERR_CUDA; the context
then runs the next solve correctly.

A test-only flag (SBX_FLAG_TEST_GIVEUP) makes every bounded wait of a solve
give up at its first check, the path a wait that never completes takes after
its limit: the co-resident window barrier of the register + shared-memory
resident kernel (its target raised past what the CTAs can reach, a short
limit), the staged-row copy waits of the streaming step kernel (the copies
still land before the kernel returns) and the MMA-completion wait of the TSP
tensor-core kernel (the MMAs finish and TMEM is freed before it returns).
Nothing faults, traps or hangs.
"""
import numpy as np
import pytest

import sbx
from conftest import oracle_graph

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = sbx.Context(0)
    yield c
    c.close()


def _expect_wait_failure(fn):
    with pytest.raises(sbx.SbxError) as e:
        fn()
    assert e.value.rc == sbx.ERR_CUDA
    assert b"bounded wait" in sbx.lib().sbx_last_error()


def test_window_barrier_gives_up_and_the_context_recovers(ctx, oracle):
    g = sbx.gen_torus(40, 40, seed=5)
    prob = ctx.problem(g)
    base = dict(dt=0.5, steps=2000, agents=1024, seed=3, precision=sbx.BF16,
                kernel=sbx.KERNEL_RESIDENT_SPLIT, update_window=1)
    _expect_wait_failure(lambda: ctx.solve(prob, sbx.params(flags=sbx.FLAG_TEST_GIVEUP, **base)))
    # the next solve runs normally: bit-exact with the oracle's BF16 mode
    r, cut = ctx.solve(prob, sbx.params(run_steps=300, **base))
    assert r["kernel_used"] == sbx.KERNEL_RESIDENT_SPLIT and r["steps_run"] == 300
    o = oracle.maxcut_solve_lp(oracle_graph(oracle, g),
                               oracle.params(dt=0.5, steps=2000, agents=1024, seed=3, uw=1,
                                             run_steps=300), oracle.BF16, want_state=True)
    x, y, s = ctx.state(g.n, 1024)
    assert np.array_equal(x, o["x"]) and np.array_equal(y, o["y"])
    assert np.array_equal(cut, o["cut"])


def test_staged_row_waits_give_up_single_and_batched(ctx, oracle):
    g = sbx.gen_er(3000, 0.004, pm1=True, seed=2)
    prob = ctx.problem(g)
    base = dict(dt=0.5, steps=500, run_steps=100, agents=64, seed=1, precision=sbx.F32,
                kernel=sbx.KERNEL_STREAM, staging=2)
    _expect_wait_failure(lambda: ctx.solve(prob, sbx.params(flags=sbx.FLAG_TEST_GIVEUP, **base)))
    # batched solves read the same error flag
    g2 = sbx.gen_rgg(2000, 10.0, seed=4)
    probs = [prob, ctx.problem(g2)]
    bp = dict(base)
    bp.pop("kernel")
    _expect_wait_failure(lambda: ctx.solve_batch(probs, [64, 64], sbx.params(
        flags=sbx.FLAG_TEST_GIVEUP, kernel=sbx.KERNEL_STREAM, **bp)))
    # and the context goes on: the staged kernel's next solve is bit-exact
    r, cut = ctx.solve(prob, sbx.params(**base))
    assert r["staging"] == 2 and r["steps_run"] == 100
    o = oracle.maxcut_solve_lp(oracle_graph(oracle, g),
                               oracle.params(dt=0.5, steps=500, agents=64, seed=1, run_steps=100),
                               oracle.F32, want_state=True)
    x, y, s = ctx.state(g.n, 64)
    assert np.array_equal(x, o["x"]) and np.array_equal(y, o["y"])
    assert np.array_equal(cut, o["cut"])


def test_tensor_core_wait_gives_up_and_the_context_recovers(ctx):
    # The TSP tensor-core kernel waits (bounded) for its MMAs on an mbarrier;
    # giving up flags the error, drains the MMAs in flight, frees TMEM and
    # returns.  The next solve is bit-identical to a solve on a fresh start.
    xc, yc = sbx.gen_cities(16, 1000.0, seed=2)
    packed = sbx.tsp_distances(xc, yc, sbx.DIST_EUC_2D_FLOAT)
    mx = float(packed.max())
    prob = ctx.tsp_problem(packed, 16, A=1.0, B=1.5 * mx, C_=1.5 * mx)
    base = dict(dt=0.1, steps=400, agents=64, seed=4, precision=sbx.BF16, kernel=sbx.KERNEL_TENSOR)
    r0, l0 = ctx.solve(prob, sbx.params(**base))
    x0, y0, _ = ctx.state(256, 64)
    _expect_wait_failure(lambda: ctx.solve(prob, sbx.params(flags=sbx.FLAG_TEST_GIVEUP, **base)))
    r1, l1 = ctx.solve(prob, sbx.params(**base))
    x1, y1, _ = ctx.state(256, 64)
    assert r1["kernel_used"] == sbx.KERNEL_TENSOR and r1["steps_run"] == 400
    assert np.array_equal(x0, x1) and np.array_equal(y0, y1)
    assert np.array_equal(np.nan_to_num(l0), np.nan_to_num(l1))
