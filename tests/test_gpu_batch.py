"""The batched step kernel with per-instance sign planes in shared memory
(count_mode 4), against the oracle and against the streaming batch kernels.

Every instance of a batch must evolve bit for bit as the oracle's restatement
of the engine's 16-bit arithmetic from seed + its position: x, y, window
spins and cuts, fused and unfused, at 32, 64 and 128 agents (one, two and
four sign words per row), with +-1 and all-positive weights, isolated rows,
and instances large enough to be split over several CTAs.
"""
import numpy as np
import pytest

import sbx
from conftest import oracle_graph

pytestmark = pytest.mark.gpu

LP = {sbx.BF16: 1, sbx.F16: 2}


@pytest.fixture(scope="module")
def ctx():
    c = sbx.Context(0)
    yield c
    c.close()


def _graphs(allpos=False):
    if allpos:
        return [sbx.gen_er(700, 0.03, pm1=False, seed=1), sbx.gen_er(5200, 0.004, pm1=False, seed=2),
                sbx.gen_er(90, 0.2, pm1=False, seed=3)]
    # RGG at low degree has isolated vertices; the 9,000-row instance spans
    # several CTAs' row runs
    return [sbx.gen_er(600, 0.04, pm1=True, seed=1), sbx.gen_rgg(1500, 3.0, seed=2),
            sbx.gen_torus(30, 40, seed=3), sbx.gen_er(9000, 0.003, pm1=True, seed=4),
            sbx.gen_rgg(120, 12.0, seed=5), sbx.gen_er(2500, 0.016, pm1=True, seed=6)]


def _check(ctx, oracle, graphs, A, prec, fused, run=150, period=50, steps=3000, seed=20, **kw):
    probs = [ctx.problem(g) for g in graphs]
    res, vals, _ = ctx.solve_batch(probs, [A] * len(probs),
                                   sbx.params(dt=0.5, steps=steps, run_steps=run, period=period,
                                              seed=seed, precision=prec, fused=fused, **kw))
    for i, g in enumerate(graphs):
        o = oracle.maxcut_solve_lp(oracle_graph(oracle, g),
                                   oracle.params(dt=0.5, steps=steps, agents=A, seed=seed + i,
                                                 period=period, fused=fused, run_steps=run),
                                   LP[prec], want_state=True)
        x, y, s = ctx.batch_state(i, g.n, A)
        what = "instance %d (n=%d)" % (i, g.n)
        assert np.array_equal(x, o["x"]), what + ": x"
        assert np.array_equal(y, o["y"]), what + ": y"
        assert np.array_equal(s, o["spins"]), what + ": spins"
        assert np.array_equal(vals[i * A:(i + 1) * A], o["cut"]), what + ": cuts"
    for p in probs:
        p.close()
    return res


@pytest.mark.parametrize("prec", [sbx.BF16, sbx.F16])
@pytest.mark.parametrize("agents", [32, 64, 128])
@pytest.mark.parametrize("fused", [1, 0])
def test_shared_plane_kernel_bitexact(ctx, oracle, prec, agents, fused):
    res = _check(ctx, oracle, _graphs(), agents, prec, fused)
    assert res[0]["count_mode"] == 4


def test_shared_plane_kernel_all_positive_weights(ctx, oracle):
    res = _check(ctx, oracle, _graphs(allpos=True), 64, sbx.BF16, 1)
    assert res[0]["count_mode"] == 4


@pytest.mark.parametrize("threads", [512, 640, 1024])
def test_shared_plane_kernel_cta_sizes_agree(ctx, oracle, threads):
    res = _check(ctx, oracle, _graphs(), 64, sbx.BF16, 1, count_mode=4, block_threads=threads)
    assert res[0]["count_mode"] == 4 and res[0]["block_threads"] == threads


def test_shared_plane_and_streaming_batch_kernels_agree(ctx):
    graphs = _graphs()
    probs = [ctx.problem(g) for g in graphs]
    A = [64] * len(probs)
    base = dict(dt=0.5, steps=2000, seed=7, precision=sbx.BF16)
    r4, v4, _ = ctx.solve_batch(probs, A, sbx.params(**base))
    r2, v2, _ = ctx.solve_batch(probs, A, sbx.params(count_mode=2, **base))
    assert r4[0]["count_mode"] == 4 and r2[0]["count_mode"] == 2
    assert np.array_equal(v4, v2)
    for p in probs:
        p.close()


def test_instances_past_the_16_bit_columns_take_the_streaming_kernel(ctx, oracle):
    # An instance of more than 32,767 rows cannot be addressed by the
    # shared-plane kernel's 16-bit columns (at 32 agents its 132 KB plane
    # would fit in shared memory): the batch runs on the streaming kernel
    # instead (bit-exact with the oracle), and asking for count mode 4 is
    # refused with the reason.
    graphs = [sbx.gen_er(33000, 0.0002, pm1=True, seed=8), sbx.gen_rgg(500, 9.0, seed=9)]
    res = _check(ctx, oracle, graphs, 32, sbx.BF16, 1, run=100, steps=2000)
    assert res[0]["count_mode"] != 4
    probs = [ctx.problem(g) for g in graphs]
    with pytest.raises(sbx.SbxError) as e:
        ctx.solve_batch(probs, [32, 32], sbx.params(dt=0.5, steps=200, seed=1, precision=sbx.BF16,
                                                   count_mode=4))
    assert e.value.rc == sbx.ERR_UNSUPPORTED
    for p in probs:
        p.close()
