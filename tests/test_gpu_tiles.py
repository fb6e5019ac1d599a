"""Streaming tiles, the autotuner and the per-window trace (GPU, through the C
ABI).

Bars:
  * every tile the step kernels are built for (agents per lane, lanes per
    row, threads per CTA) gives a state bit-identical to every other tile, at
    FP64 and BF16, with +-1 and with real weights, and with a row count that
    leaves lanes of the last warp without a row;
  * FP64 through a several-rows-per-warp tile stays bit-exact with the oracle;
  * the autotuner reports a tile the kernels accept and changes no result;
  * the trace holds one record per window whose last best cut is the solve's
    best cut, and time-to-target is the first window reaching the target.
"""
import numpy as np
import pytest

from conftest import oracle_first_steps, oracle_graph

import sbx

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = sbx.Context(0)
    yield c
    c.close()


def _tiles(prec, Ap, heavy=False):
    """The tiles (agents per lane, lanes per row, threads per CTA) a solve
    with Ap padded agents accepts (mirror of tile_ok)."""
    vm = {sbx.F64: 2, sbx.F32: 4, sbx.BF16: 8, sbx.F16: 8}[prec]
    out = []
    for v in (8, 4, 2, 1):
        if v > vm:
            continue
        for lr in (32, 16, 8, 4):
            if lr == 32:
                ok = Ap % (32 * v) == 0
            else:
                ok = not heavy and v in (vm, vm // 2) and v * lr == Ap
            if ok:
                out += [(v, lr, 256), (v, lr, 128)]
    return out


def _real_graph(n=203, p=0.05, seed=9):
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


@pytest.mark.parametrize("prec", [sbx.F64, sbx.BF16])
@pytest.mark.parametrize("weights", ["pm1", "real"])
@pytest.mark.parametrize("agents", [64, 32, 128])
def test_every_tile_gives_the_same_state(ctx, prec, weights, agents):
    # 203 rows: not a multiple of 2, 4 or 8 rows per warp; degrees up to ~20,
    # so bit-plane counting splits rows over several lanes
    g = sbx.gen_er(203, 0.05, pm1=True, seed=7) if weights == "pm1" else _real_graph()
    prob = ctx.problem(g)
    Ap = (agents + 31) // 32 * 32
    tiles = _tiles(prec, Ap)
    assert any(lr < 32 for _, lr, _ in tiles) or prec == sbx.F64
    modes = (1, 2) if weights == "pm1" else (1,)
    ref = None
    for (v, lr, bt), cm in [(t, m) for t in tiles for m in modes]:
        r, cut = ctx.solve(prob, sbx.params(dt=0.4, steps=600, agents=agents, seed=11,
                                            precision=prec, update_window=1,
                                            kernel=sbx.KERNEL_STREAM, lane_agents=v,
                                            row_lanes=lr, block_threads=bt, count_mode=cm))
        assert (r["lane_agents"], r["row_lanes"], r["block_threads"], r["count_mode"]) == \
            (v, lr, bt, cm)
        x, y, s = ctx.state(g.n, agents)
        if ref is None:
            ref = (x, y, s, cut, r["steps_run"])
            continue
        np.testing.assert_array_equal(x, ref[0])
        np.testing.assert_array_equal(y, ref[1])
        np.testing.assert_array_equal(s, ref[2])
        np.testing.assert_array_equal(cut, ref[3])
        assert r["steps_run"] == ref[4]


@pytest.mark.parametrize("fused", [1, 0])
@pytest.mark.parametrize("count_mode", [1, 2])
def test_fp64_rows_per_warp_tile_bitexact_with_oracle(ctx, oracle, fused, count_mode):
    g = sbx.gen_er(203, 0.05, pm1=True, seed=7)
    A, max_steps, dt, seed = 32, 2000, 0.3, 5
    prob = ctx.problem(g)
    ctx.solve(prob, sbx.params(dt=dt, steps=max_steps, run_steps=300, agents=A, fused=fused,
                               seed=seed, precision=sbx.F64, kernel=sbx.KERNEL_STREAM,
                               lane_agents=2, row_lanes=16, count_mode=count_mode))
    x, y, s = ctx.state(g.n, A)
    og = oracle_graph(oracle, g)
    ox, oy = oracle_first_steps(oracle, og, A, seed, dt, max_steps, 300, fused)
    np.testing.assert_array_equal(x, ox)
    np.testing.assert_array_equal(y, oy)


def test_heavy_rows_refuse_rows_per_warp_tiles(ctx):
    g = sbx.gen_rmat(12, 8, seed=1234)
    assert np.diff(g.rowptr).max() > 128
    prob = ctx.problem(g)
    with pytest.raises(sbx.SbxError) as e:
        ctx.solve(prob, sbx.params(dt=0.5, steps=100, agents=64, precision=sbx.BF16,
                                   kernel=sbx.KERNEL_STREAM, row_lanes=8))
    assert e.value.rc == sbx.ERR_ARG
    r, _ = ctx.solve(prob, sbx.params(dt=0.5, steps=100, agents=64, precision=sbx.BF16,
                                      kernel=sbx.KERNEL_STREAM))
    assert r["row_lanes"] == 32


@pytest.mark.parametrize("agents", [64, 1024])
def test_autotuned_tile_is_valid_and_changes_nothing(ctx, agents):
    g = sbx.gen_torus(30, 30, seed=1234)
    prob = ctx.problem(g)
    base = dict(dt=0.5, steps=500, agents=agents, seed=3, precision=sbx.BF16,
                kernel=sbx.KERNEL_STREAM)
    r, cut = ctx.solve(prob, sbx.params(**base))
    tile = (r["lane_agents"], r["row_lanes"], r["block_threads"])
    assert tile in _tiles(sbx.BF16, agents)
    x, y, s = ctx.state(g.n, agents)
    r2, cut2 = ctx.solve(prob, sbx.params(flags=sbx.FLAG_NO_TUNE, **base))
    assert (r2["lane_agents"], r2["row_lanes"], r2["block_threads"], r2["count_mode"]) == \
        ({64: 2, 1024: 8}[agents], 32, 256, 1)
    x2, y2, s2 = ctx.state(g.n, agents)
    np.testing.assert_array_equal(x, x2)
    np.testing.assert_array_equal(y, y2)
    np.testing.assert_array_equal(cut, cut2)
    # the tuned tile is cached by matrix shape: the same tile again, also for a
    # fresh upload of the same graph
    r3, _ = ctx.solve(prob, sbx.params(**base))
    assert (r3["lane_agents"], r3["row_lanes"], r3["block_threads"]) == tile
    prob2 = ctx.problem(g)
    r4, cut4 = ctx.solve(prob2, sbx.params(**base))
    assert (r4["lane_agents"], r4["row_lanes"], r4["block_threads"]) == tile
    np.testing.assert_array_equal(cut4, cut)


def test_trace_and_time_to_target(ctx, oracle):
    g = sbx.gen_torus(40, 40, seed=1234)
    A, steps = 96, 3000
    prob = ctx.problem(g)
    base = dict(dt=0.5, steps=steps, agents=A, seed=21, precision=sbx.F32,
                kernel=sbx.KERNEL_STREAM)
    r0, cut0 = ctx.solve(prob, sbx.params(**base))
    r, cut = ctx.solve(prob, sbx.params(trace=1, **base))
    np.testing.assert_array_equal(cut, cut0)          # tracing changes no result
    st, best, t_us = ctx.trace()
    assert len(st) == steps // 100
    np.testing.assert_array_equal(st, np.arange(1, steps // 100 + 1) * 100)
    assert best[-1] == r["max"]
    assert np.all(np.diff(t_us) >= 0) and t_us[0] > 0
    assert r["time_to_target_us"] == -1 and r["steps_to_target"] == -1
    # each record is the exact best cut of that window's spins
    assert np.all(best == np.floor(best))
    target = float(np.max(best[: len(best) // 2]))
    r2, _ = ctx.solve(prob, sbx.params(trace=0, target=target, **base))
    st2, best2, t2 = ctx.trace()
    k = int(np.argmax(best2 >= target))
    assert r2["steps_to_target"] == st2[k] and r2["time_to_target_us"] == t2[k]
    assert r2["steps_to_target"] <= st2[len(st2) // 2 - 1]
    r3, _ = ctx.solve(prob, sbx.params(target=r["max"] + 1e6, **base))
    assert r3["time_to_target_us"] == -1 and r3["steps_to_target"] == -1


def test_trace_with_early_exit_records_only_closed_windows(ctx, oracle):
    # windows of 10 steps, threshold 2: the oracle exits at step 2210 of 3000;
    # the engine polls the exit flag late and runs up to three idle windows
    # past it, which must leave no record
    g = sbx.gen_er(60, 0.1, pm1=False, seed=3)
    prm = dict(dt=0.2, steps=3000, agents=32, seed=2, period=10, threshold=2)
    ref = oracle.maxcut_solve(oracle_graph(oracle, g),
                              oracle.params(fused=1, uw=1, **prm))["result"]
    assert ref["steps_run"] < 3000
    prob = ctx.problem(g)
    r, cut = ctx.solve(prob, sbx.params(update_window=1, precision=sbx.F64,
                                        kernel=sbx.KERNEL_STREAM, trace=1, **prm))
    assert r["steps_run"] == ref["steps_run"] and r["max"] == ref["max"]
    st, best, t_us = ctx.trace()
    assert len(st) == r["windows_run"] and st[-1] == r["steps_run"]
    assert best[-1] == r["max"]


def test_trace_refused_where_not_built(ctx):
    g = sbx.gen_er(100, 0.1, seed=1)
    prob = ctx.problem(g)
    with pytest.raises(sbx.SbxError) as e:
        ctx.solve(prob, sbx.params(steps=100, agents=64, kernel=sbx.KERNEL_RESIDENT, trace=1))
    assert e.value.rc == sbx.ERR_UNSUPPORTED
    with pytest.raises(sbx.SbxError) as e:
        ctx.solve_batch([prob], [64], sbx.params(steps=100, target=10.0))
    assert e.value.rc == sbx.ERR_ARG


@pytest.mark.parametrize("prec", [sbx.BF16, sbx.F64])
def test_batch_time_to_target_matches_single_traced_solves(ctx, prec):
    # A batched instance runs exactly as alone from seed + i, so its first
    # window reaching a target is the single traced solve's first window.
    gs = [sbx.gen_er(300, 0.04, pm1=True, seed=1), sbx.gen_rgg(900, 8.0, seed=2),
          sbx.gen_torus(20, 30, seed=3), sbx.gen_er(150, 0.1, pm1=False, seed=5)]
    agents = [64, 64, 40, 64]
    probs = [ctx.problem(g) for g in gs]
    base = dict(dt=0.5, steps=1500, seed=100, precision=prec, kernel=sbx.KERNEL_STREAM)
    res0, vals0, _ = ctx.solve_batch(probs, agents, sbx.params(**base))
    # targets: a little under each instance's final best, and one out of reach
    targets = [r["max"] - 2.0 for r in res0]
    targets[2] = res0[2]["max"] + 1e6
    res, vals, _ = ctx.solve_batch(probs, agents, sbx.params(**base), targets=targets)
    np.testing.assert_array_equal(vals, vals0)       # the trace changes no result
    for i, (p, a) in enumerate(zip(probs, agents)):
        r1, _ = ctx.solve(p, sbx.params(agents=a, target=targets[i], **dict(base, seed=100 + i)))
        assert res[i]["steps_to_target"] == r1["steps_to_target"]
        if i == 2:
            assert res[i]["steps_to_target"] == -1 and res[i]["time_to_target_us"] == -1
        else:
            assert 0 < res[i]["steps_to_target"] <= 1500 and res[i]["time_to_target_us"] > 0


@pytest.mark.parametrize("agents", [32, 256])
@pytest.mark.parametrize("count_mode", [1, 2])
def test_dense_unit_rows_count_modes_bitexact_with_oracle(ctx, oracle, agents, count_mode):
    # degrees ~100 (just under the heavy-row split at 127): every lane of a
    # bit-plane group holds many neighbours and the planes fill up
    g = sbx.gen_er(240, 0.42, pm1=True, seed=13)
    deg = np.diff(g.rowptr)
    assert deg.max() <= 127 and deg.mean() > 90
    A, max_steps, dt, seed = agents, 2000, 0.2, 3
    prob = ctx.problem(g)
    # 200 steps: two windows of 100
    ctx.solve(prob, sbx.params(dt=dt, steps=max_steps, run_steps=200, agents=A, fused=1, seed=seed,
                               precision=sbx.F64, kernel=sbx.KERNEL_STREAM, count_mode=count_mode))
    x, y, s = ctx.state(g.n, A)
    og = oracle_graph(oracle, g)
    ox, oy = oracle_first_steps(oracle, og, A, seed, dt, max_steps, 200, 1)
    np.testing.assert_array_equal(x, ox)
    np.testing.assert_array_equal(y, oy)


@pytest.mark.parametrize("count_mode", [1, 2, 3])
def test_heavy_rows_count_modes_bitexact_with_oracle(ctx, oracle, count_mode):
    # R-MAT: heavy rows (split into chunks), light rows on both sides of the
    # mixed mode's degree threshold (12), and empty rows
    g = sbx.gen_rmat(12, 8, seed=1234)
    deg = np.diff(g.rowptr)
    assert deg.max() > 127 and ((deg >= 12) & (deg <= 127)).sum() > 100 and ((deg > 0) & (deg < 12)).sum() > 100
    A, max_steps, dt, seed = 64, 2000, 0.5, 9
    prob = ctx.problem(g)
    r, _ = ctx.solve(prob, sbx.params(dt=dt, steps=max_steps, run_steps=200, agents=A, fused=1,
                                      seed=seed, precision=sbx.F64, kernel=sbx.KERNEL_STREAM,
                                      count_mode=count_mode))
    assert r["count_mode"] == count_mode
    x, y, s = ctx.state(g.n, A)
    og = oracle_graph(oracle, g)
    ox, oy = oracle_first_steps(oracle, og, A, seed, dt, max_steps, 200, 1)
    np.testing.assert_array_equal(x, ox)
    np.testing.assert_array_equal(y, oy)


@pytest.mark.parametrize("count_mode", [1, 2])
@pytest.mark.parametrize("A,tile", [(64, (2, 32)), (32, (1, 32)), (32, (2, 16))])
def test_isolated_rows_bitexact_with_oracle(ctx, oracle, A, tile, count_mode):
    # ~40 isolated rows (degree 0), advanced a window at a time by their own
    # kernel, the others by the step kernel (byte counters or bit planes):
    # FP64 state equal to the oracle's
    g = sbx.gen_er(400, 0.006, pm1=True, seed=21)
    assert (np.diff(g.rowptr) == 0).sum() > 20
    max_steps, dt, seed = 2000, 0.5, 4
    prob = ctx.problem(g)
    ctx.solve(prob, sbx.params(dt=dt, steps=max_steps, run_steps=200, agents=A, fused=1, seed=seed,
                               precision=sbx.F64, kernel=sbx.KERNEL_STREAM, lane_agents=tile[0],
                               row_lanes=tile[1], count_mode=count_mode))
    x, y, s = ctx.state(g.n, A)
    og = oracle_graph(oracle, g)
    ox, oy = oracle_first_steps(oracle, og, A, seed, dt, max_steps, 200, 1)
    np.testing.assert_array_equal(x, ox)
    np.testing.assert_array_equal(y, oy)


def test_mixed_count_mode_needs_heavy_rows(ctx):
    g = sbx.gen_er(300, 0.05, pm1=True, seed=2)
    prob = ctx.problem(g)
    with pytest.raises(sbx.SbxError) as e:
        ctx.solve(prob, sbx.params(dt=0.5, steps=100, agents=64, precision=sbx.BF16,
                                   kernel=sbx.KERNEL_STREAM, count_mode=3))
    assert e.value.rc == sbx.ERR_ARG


@pytest.mark.parametrize("prec", [sbx.BF16, sbx.F32, sbx.F64])
@pytest.mark.parametrize("count_mode", [1, 2])
def test_staged_rows_give_the_same_state(ctx, prec, count_mode):
    # rows copied ahead into shared memory (bulk asynchronous copies) against
    # direct loads: heavy rows (R-MAT) and plain rows, every lane width
    for g, A in ((sbx.gen_rmat(13, 6, seed=77), 256), (sbx.gen_er(700, 0.02, pm1=True, seed=8), 64)):
        prob = ctx.problem(g)
        ref = None
        for staging in (1, 2):
            r, cut = ctx.solve(prob, sbx.params(dt=0.5, steps=400, agents=A, seed=5, precision=prec,
                                                kernel=sbx.KERNEL_STREAM, row_lanes=32,
                                                count_mode=count_mode, staging=staging))
            assert r["staging"] == staging
            x, y, s = ctx.state(g.n, A)
            if ref is None:
                ref = (x, y, s, cut)
                continue
            np.testing.assert_array_equal(x, ref[0])
            np.testing.assert_array_equal(y, ref[1])
            np.testing.assert_array_equal(s, ref[2])
            np.testing.assert_array_equal(cut, ref[3])
