"""The register + shared-memory resident kernel (GPU, through the C ABI):
its state, window spins, cuts and steps equal the streaming kernel's bit for
bit (same arithmetic), with and without the update-window exit, for +-1 and
real weights, and whichever configuration (register rows) the size picks."""
import numpy as np
import pytest

from conftest import oracle_graph

import sbx

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = sbx.Context(0)
    yield c
    c.close()


def _real_graph(n, p, seed):
    rng = np.random.default_rng(seed)
    iu = np.triu_indices(n, 1)
    keep = rng.random(iu[0].size) < p
    r, c = iu[0][keep], iu[1][keep]
    w = np.round(rng.normal(0.0, 1.0, r.size), 3)
    rows = np.concatenate([r, c])
    cols = np.concatenate([c, r])
    vals = np.concatenate([w, w])
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    rowptr = np.zeros(n + 1, np.int64)
    np.add.at(rowptr, rows + 1, 1)
    return sbx.Graph(n, np.cumsum(rowptr), cols, vals, float(w.sum()))


CASES = [
    # (graph, agents): sizes that put 0, 2 and 4 register rows per thread
    ("torus40", lambda: sbx.gen_torus(40, 40, seed=1234), 96),
    ("torus100", lambda: sbx.gen_torus(100, 100, seed=1234), 64),
    ("torus80x100", lambda: sbx.gen_torus(80, 100, seed=7), 64),
    ("er3000", lambda: sbx.gen_er(3000, 0.004, pm1=True, seed=2), 40),
    ("rgg9000", lambda: sbx.gen_rgg(9000, 10.0, seed=3), 72),
    ("real1500", lambda: _real_graph(1500, 0.01, 4), 32),
    # ~400 isolated rows: the streaming solve advances them a window per launch
    ("er4000iso", lambda: sbx.gen_er(4000, 0.0006, pm1=True, seed=5), 64),
]


@pytest.mark.parametrize("prec", [sbx.BF16, sbx.F16])
@pytest.mark.parametrize("uw", [0, 1])
@pytest.mark.parametrize("name,make,agents", CASES)
def test_split_resident_equals_streaming(ctx, oracle, prec, uw, name, make, agents):
    g = make()
    prob = ctx.problem(g)
    base = dict(dt=0.5, steps=1500, agents=agents, seed=9, precision=prec, update_window=uw,
                threshold=3 if uw else 0)
    r1, cut1 = ctx.solve(prob, sbx.params(kernel=sbx.KERNEL_RESIDENT_SPLIT, **base))
    assert r1["kernel_used"] == sbx.KERNEL_RESIDENT_SPLIT
    x1, y1, s1 = ctx.state(g.n, agents)
    r2, cut2 = ctx.solve(prob, sbx.params(kernel=sbx.KERNEL_STREAM, **base))
    x2, y2, s2 = ctx.state(g.n, agents)
    np.testing.assert_array_equal(x1, x2)
    np.testing.assert_array_equal(y1, y2)
    np.testing.assert_array_equal(s1, s2)
    np.testing.assert_array_equal(cut1, cut2)
    for k in ("steps_run", "windows_run", "bifurcated", "max", "ps"):
        assert r1[k] == r2[k], k
    np.testing.assert_array_equal(oracle.cut(oracle_graph(oracle, g), s1, agents), cut1)


def test_split_resident_refusals(ctx):
    g = sbx.gen_torus(20, 20, seed=1)
    prob = ctx.problem(g)
    for kw in (dict(precision=sbx.F32), dict(precision=sbx.BF16, fused=0)):
        with pytest.raises(sbx.SbxError) as e:
            ctx.solve(prob, sbx.params(steps=100, agents=64, kernel=sbx.KERNEL_RESIDENT_SPLIT, **kw))
        assert e.value.rc == sbx.ERR_UNSUPPORTED
    hub = sbx.gen_rmat(12, 8, seed=1234)   # rows above 127 neighbours
    with pytest.raises(sbx.SbxError):
        ctx.solve(ctx.problem(hub), sbx.params(steps=100, agents=64, precision=sbx.BF16,
                                               kernel=sbx.KERNEL_RESIDENT_SPLIT))


@pytest.mark.parametrize("prec", [sbx.BF16, sbx.F16])
def test_resident_batch_equals_streaming_batch(ctx, prec):
    # instances packed into bins of the resident batch kernel (here more rows
    # than one bin holds, so several bins) against the streaming batch:
    # identical per-agent cuts and statistics (batches take integer weights)
    gs = [sbx.gen_rgg(9000, 8.0, seed=31), sbx.gen_er(8500, 0.002, pm1=True, seed=32),
          sbx.gen_torus(90, 100, seed=33), sbx.gen_er(300, 0.04, pm1=True, seed=1),
          sbx.gen_torus(20, 30, seed=3), sbx.gen_er(150, 0.1, pm1=False, seed=5)]
    agents = [64, 64, 40, 64, 32, 96]
    probs = [ctx.problem(g) for g in gs]
    base = dict(dt=0.5, steps=1200, seed=77, precision=prec)
    res_r, vals_r, _ = ctx.solve_batch(probs, agents, sbx.params(kernel=sbx.KERNEL_RESIDENT, **base))
    res_s, vals_s, _ = ctx.solve_batch(probs, agents, sbx.params(kernel=sbx.KERNEL_STREAM, **base))
    assert all(r["kernel_used"] == sbx.KERNEL_RESIDENT for r in res_r)
    assert all(r["kernel_used"] == sbx.KERNEL_STREAM for r in res_s)
    np.testing.assert_array_equal(vals_r, vals_s)
    for a, b in zip(res_r, res_s):
        for k in ("max", "min", "mean", "std", "ps", "steps_run"):
            assert a[k] == b[k], k
    # by itself (AUTO) the resident batch is taken for low-degree classes
    # (mean degree <= 8), the streaming kernel otherwise
    res_a, vals_a, _ = ctx.solve_batch(probs, agents, sbx.params(**base))
    nnz, rows = sum(g.nnz for g in gs), sum(g.n for g in gs)
    assert res_a[0]["kernel_used"] == (sbx.KERNEL_RESIDENT if nnz <= 8 * rows else sbx.KERNEL_STREAM)
    np.testing.assert_array_equal(vals_a, vals_r)
