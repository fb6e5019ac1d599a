"""The TSP distance product on the tensor cores (SBX_KERNEL_TENSOR, 16-bit
state) against the CUDA-core resident kernel (SBX_KERNEL_RESIDENT: the same
update with the product on the FP32 pipes) and the FP64 oracle.

The tensor cores take D as three 16-bit parts whose sum is D exactly (FP16
after an exact power-of-two scale) and the state as it is stored, so every
product is exact and only the order of the FP32 sums differs from the
CUDA-core kernel (src/kernels.cu:561-597 sums l in order).  So after one step
the two states agree within one unit in the last place of the storage type
(a sum next to a rounding boundary may round the other way), and over a
longer run the tensor-core state is no further from FP64 than the CUDA-core
state is, with a margin of two."""
import numpy as np
import pytest

import sbx

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = sbx.Context(0)
    yield c
    c.close()


def ulp(v, prec):
    """Spacing of the storage type at each value (normal range)."""
    v = np.abs(np.asarray(v, np.float64))
    if prec == sbx.BF16:
        return np.spacing(v.astype(np.float32)).astype(np.float64) * 65536.0
    return np.spacing(v.astype(np.float16)).astype(np.float64)


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


def _problem(ctx, N, scale, seed):
    xc, yc = sbx.gen_cities(N, scale, seed=seed)
    packed = sbx.tsp_distances(xc, yc, sbx.DIST_EUC_2D_FLOAT)
    mx = float(packed.max())
    return ctx.tsp_problem(packed, N, A=1.0, B=1.5 * mx, C_=1.5 * mx), (xc, yc, mx)


def _run(ctx, prob, N, A, prec, kernel, **kw):
    r, lengths = ctx.solve(prob, sbx.params(agents=A, precision=prec, kernel=kernel, **kw))
    assert r["kernel_used"] == kernel
    x, y, _ = ctx.state(N * N, A)
    return r, x, y, lengths


@pytest.mark.parametrize("prec", [sbx.BF16, sbx.F16])
@pytest.mark.parametrize("N,scale", [(3, 1000.0), (12, 1000.0), (16, 1000.0), (30, 1000.0),
                                     (32, 1000.0), (17, 3.0e6)])
def test_one_step_within_one_ulp_of_cuda_core(ctx, prec, N, scale):
    # 3 cities: the smallest the kernel takes; 16: one full 128-row tile;
    # 32: two full tiles and every bit of the 32-city masks; (17, 3e6):
    # distances far past FP16's range, so the FP16 operands are scaled, and
    # 17 cities with 8 agents per CTA leave rows of the second tile idle
    prob, _ = _problem(ctx, N, scale, seed=N)
    A = 72   # not a multiple of 8: the last CTA holds padded agents
    kw = dict(dt=0.1, steps=1000, run_steps=1, period=1, seed=9)
    _, xt, yt, _ = _run(ctx, prob, N, A, prec, sbx.KERNEL_TENSOR, **kw)
    _, xc, yc, _ = _run(ctx, prob, N, A, prec, sbx.KERNEL_RESIDENT, **kw)
    for got, want in ((xt, xc), (yt, yc)):
        d = np.abs(got - want)
        assert np.all(d <= ulp(want, prec)), float(d.max())
        assert np.mean(d == 0) > 0.99


@pytest.mark.parametrize("prec", [sbx.BF16, sbx.F16])
def test_trajectory_no_further_from_fp64_than_cuda_core(ctx, prec):
    N, A, max_steps = 12, 40, 1000
    prob, _ = _problem(ctx, N, 1000.0, seed=11)
    for k in (50, 100):
        kw = dict(dt=0.1, steps=max_steps, run_steps=k, period=25, seed=77)
        _, xt, yt, _ = _run(ctx, prob, N, A, prec, sbx.KERNEL_TENSOR, **kw)
        _, xc, yc, _ = _run(ctx, prob, N, A, prec, sbx.KERNEL_RESIDENT, **kw)
        _, x64, y64, _ = _run(ctx, prob, N, A, sbx.F64, sbx.KERNEL_STREAM, **kw)
        floor = 2.0 ** -8 if prec == sbx.BF16 else 2.0 ** -11
        assert rel_err(xt, x64) <= max(2 * rel_err(xc, x64), floor)
        assert rel_err(yt, y64) <= max(2 * rel_err(yc, y64), floor)


@pytest.mark.parametrize("prec", [sbx.BF16, sbx.F16])
def test_config_shape_runs_decodes_and_is_deterministic(ctx, oracle, prec):
    # 30 cities, 1024 agents (the TSP workload's shape), 2000 steps: every
    # valid tour is a permutation whose length the oracle gives exactly, the
    # CUDA-core kernel finds valid tours too, and a rerun is bit-identical.
    N, A = 30, 1024
    prob, (xc, yc, mx) = _problem(ctx, N, 1000.0, seed=1234)
    kw = dict(dt=0.1, steps=2000, seed=5)
    r, xt, yt, lengths = _run(ctx, prob, N, A, prec, sbx.KERNEL_TENSOR, **kw)
    assert r["agents_per_block"] == 8 and r["steps_run"] == 2000
    tours, valid = ctx.tours(N, A)
    t = oracle.Tsp(xc, yc, oracle.DIST_EUC_2D_FLOAT, A=1.0, B=1.5 * mx, C_=1.5 * mx)
    nvalid = 0
    for a in range(A):
        if valid[a] > 0:
            nvalid += 1
            assert sorted(tours[a].tolist()) == list(range(N))
            assert lengths[a] == t.tour_length(tours[a])
        else:
            assert np.isnan(lengths[a])
    assert nvalid == r["valid"]
    rc, _, _, _ = _run(ctx, prob, N, A, prec, sbx.KERNEL_RESIDENT, **kw)
    assert (r["valid"] > 0) == (rc["valid"] > 0)
    r2, x2, y2, _ = _run(ctx, prob, N, A, prec, sbx.KERNEL_TENSOR, **kw)
    assert np.array_equal(x2, xt) and np.array_equal(y2, yt) and r2["valid"] == r["valid"]


def test_auto_picks_tensor_for_16_bit_tsp_only(ctx):
    prob, _ = _problem(ctx, 10, 1000.0, seed=3)
    kw = dict(dt=0.1, steps=200, agents=32, seed=1)
    for prec, want in ((sbx.BF16, sbx.KERNEL_TENSOR), (sbx.F16, sbx.KERNEL_TENSOR),
                       (sbx.F32, sbx.KERNEL_RESIDENT), (sbx.F64, sbx.KERNEL_STREAM)):
        r, _ = ctx.solve(prob, sbx.params(precision=prec, **kw))
        assert r["kernel_used"] == want
    # refused where it does not apply: FP32 state, two cities, MaxCut
    with pytest.raises(sbx.SbxError) as e:
        ctx.solve(prob, sbx.params(precision=sbx.F32, kernel=sbx.KERNEL_TENSOR, **kw))
    assert e.value.rc == sbx.ERR_UNSUPPORTED
    p2, _ = _problem(ctx, 2, 1000.0, seed=3)
    with pytest.raises(sbx.SbxError) as e:
        ctx.solve(p2, sbx.params(precision=sbx.BF16, kernel=sbx.KERNEL_TENSOR, **kw))
    assert e.value.rc == sbx.ERR_UNSUPPORTED
    g = ctx.problem(sbx.gen_er(100, 0.1, pm1=True, seed=1))
    with pytest.raises(sbx.SbxError) as e:
        ctx.solve(g, sbx.params(precision=sbx.BF16, kernel=sbx.KERNEL_TENSOR, **kw))
    assert e.value.rc == sbx.ERR_UNSUPPORTED


@pytest.mark.parametrize("threads", [1, 2, 4])
@pytest.mark.parametrize("N", [13, 30])
def test_threads_per_row_agree(ctx, N, threads):
    # 1, 2 or 4 threads share a row's cities (row_lanes): the same arithmetic
    # in the same order, so the states are bit-identical
    prob, _ = _problem(ctx, N, 1000.0, seed=N + 1)
    A = 48
    kw = dict(dt=0.1, steps=600, run_steps=300, seed=3)
    r, xt, yt, lt = _run(ctx, prob, N, A, sbx.BF16, sbx.KERNEL_TENSOR, row_lanes=threads, **kw)
    assert r["row_lanes"] == threads
    r1, x1, y1, l1 = _run(ctx, prob, N, A, sbx.BF16, sbx.KERNEL_TENSOR, row_lanes=1, **kw)
    assert np.array_equal(xt, x1) and np.array_equal(yt, y1)
    assert np.array_equal(np.nan_to_num(lt), np.nan_to_num(l1)) and r["valid"] == r1["valid"]
