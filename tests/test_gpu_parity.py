"""Parity of the CUDA engine (through the C ABI) with the FP64 oracle and the
reference fixtures.

Bars (SURVEY parity clauses):
  * FP64 state: bit-exact with the oracle / the reference's kernels run in
    Jacobi order (trajectories, window flags, cuts, steps run).
  * FP32 state: trajectories within 1e-4 (normwise, relative to max |x|) of
    the FP64 oracle over the first 100 steps.
  * Cuts: bit-exact for the spins the engine returns, at every precision.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

import sbx

pytestmark = pytest.mark.gpu

TRAJ_TOL = 1e-4


@pytest.fixture(scope="module")
def ctx():
    c = sbx.Context(0)
    yield c
    c.close()


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


JACOBI_CASES = ["mc_er40_fused_jacobi", "mc_er40_unfused", "mc_er40_uw", "mc_er40_real",
                "mc_ring24_dt05"]


@pytest.mark.parametrize("name", JACOBI_CASES)
def test_fp64_maxcut_bitexact_with_reference_fixture(ctx, name):
    ref = golden(name)
    g = sbx.load_mtx(os.path.join(GOLDEN, str(ref["source"])))
    A = int(ref["agents"])
    prob = ctx.problem(g)
    prm = sbx.params(dt=float(ref["dt"]), steps=int(ref["steps"]), agents=A,
                     fused=int(ref["fused"]), update_window=int(ref["uw"]),
                     threshold=int(ref["threshold"]), seed=int(ref["seed"]),
                     precision=sbx.F64, kernel=sbx.KERNEL_STREAM)
    r, cut = ctx.solve(prob, prm)
    x, y, s = ctx.state(g.n, A)
    np.testing.assert_array_equal(x, ref["x"])
    np.testing.assert_array_equal(y, ref["y"])
    np.testing.assert_array_equal(s, ref["cur"].astype(np.int32))
    np.testing.assert_array_equal(cut, ref["cut"])
    assert r["steps_run"] == ref["steps_windows"][0]
    assert r["windows_run"] == ref["steps_windows"][1]
    assert r["bifurcated"] == int(ref["bif"].sum())
    assert r["xi0"] == float(ref["xi0"])


def _oracle_graph(oracle, g):
    return oracle.Graph(g.n, g.rowptr, g.col, g.val, g.wsum)


@pytest.mark.parametrize("kernel", [sbx.KERNEL_STREAM, sbx.KERNEL_RESIDENT])
@pytest.mark.parametrize("fused", [1, 0])
@pytest.mark.parametrize("gname", ["er40", "er800"])
def test_fp32_trajectory_within_1e4(ctx, oracle, kernel, fused, gname):
    if gname == "er40":
        g = sbx.load_mtx(os.path.join(GOLDEN, "er40_pm1.mtx"))
        A = 33
    else:
        g = sbx.gen_er(800, 0.0601, pm1=False, seed=1234)
        A = 64
    steps, dt, seed = 100, 0.1, 99
    prob = ctx.problem(g)
    prm = sbx.params(dt=dt, steps=steps, agents=A, fused=fused, seed=seed, precision=sbx.F32,
                     kernel=kernel)
    r, cut = ctx.solve(prob, prm)
    assert r["kernel_used"] == kernel
    x, y, s = ctx.state(g.n, A)
    og = _oracle_graph(oracle, g)
    o = oracle.maxcut_solve(og, oracle.params(dt=dt, steps=steps, agents=A, fused=fused,
                                              seed=seed), want_state=True)
    assert rel_err(x, o["x"]) < TRAJ_TOL
    assert rel_err(y, o["y"]) < TRAJ_TOL
    # cut evaluation is exact for whatever spins the engine holds
    np.testing.assert_array_equal(oracle.cut(og, s, A), cut)
    assert r["steps_run"] == o["result"]["steps_run"] == 100


@pytest.mark.parametrize("prec", [sbx.F32, sbx.BF16, sbx.F16])
@pytest.mark.parametrize("kernel", [sbx.KERNEL_STREAM, sbx.KERNEL_RESIDENT])
def test_cut_exact_and_close_to_fp64_on_torus(ctx, oracle, prec, kernel):
    # 2-D torus 40x40 (+-1 weights), 96 agents, dt 0.5, 2000 steps with the
    # update window: a scaled copy of the torus workload.
    g = sbx.gen_torus(40, 40, seed=1234)
    A, steps = 96, 2000
    prob = ctx.problem(g)
    prm = sbx.params(dt=0.5, steps=steps, agents=A, update_window=1, seed=4321, precision=prec,
                     kernel=kernel)
    r, cut = ctx.solve(prob, prm)
    x, y, s = ctx.state(g.n, A)
    og = _oracle_graph(oracle, g)
    np.testing.assert_array_equal(oracle.cut(og, s, A), cut)
    assert r["max"] == cut.max() and r["min"] == cut.min()
    r64, cut64 = ctx.solve(prob, sbx.params(dt=0.5, steps=steps, agents=A, update_window=1,
                                            seed=4321, precision=sbx.F64,
                                            kernel=sbx.KERNEL_STREAM))
    # energy error against the FP64 run from the same seed: best cuts within 2%
    assert abs(r["max"] - r64["max"]) <= 0.02 * abs(r64["max"])
    assert r["steps_run"] % 100 == 0 and 0 < r["steps_run"] <= steps


def test_fp64_large_init_matches_oracle(ctx, oracle):
    # 10^4 rows x 64 agents: the device rand() stream spans many jump chunks.
    g = sbx.gen_torus(100, 100, seed=1)
    A = 64
    prob = ctx.problem(g)
    prm = sbx.params(dt=0.5, steps=1, period=1, agents=A, seed=2024, precision=sbx.F64,
                     kernel=sbx.KERNEL_STREAM)
    r, cut = ctx.solve(prob, prm)
    x, y, s = ctx.state(g.n, A)
    og = _oracle_graph(oracle, g)
    o = oracle.maxcut_solve(og, oracle.params(dt=0.5, steps=1, period=1, agents=A, seed=2024),
                            want_state=True)
    np.testing.assert_array_equal(x, o["x"])
    np.testing.assert_array_equal(y, o["y"])
    np.testing.assert_array_equal(cut, o["cut"])


TSP_CASES = ["tsp_euc5", "tsp_geo6"]


@pytest.mark.parametrize("name", TSP_CASES)
def test_fp64_tsp_bitexact_with_reference_fixture(ctx, oracle, name):
    ref = golden(name)
    xc, yc, kind = sbx.load_tsplib(os.path.join(GOLDEN, str(ref["source"])))
    packed = sbx.tsp_distances(xc, yc, kind)
    np.testing.assert_array_equal(packed, ref["dist"])
    N, A = len(xc), int(ref["agents"])
    prob = ctx.tsp_problem(packed, N)
    prm = sbx.params(dt=0.1, steps=int(ref["steps"]), agents=A, seed=int(ref["seed"]),
                     precision=sbx.F64, kernel=sbx.KERNEL_STREAM)
    r, lengths = ctx.solve(prob, prm)
    x, y, s = ctx.state(N * N, A)
    np.testing.assert_array_equal(x, ref["x"])
    np.testing.assert_array_equal(y, ref["y"])
    tours, valid = ctx.tours(N, A)
    np.testing.assert_array_equal(valid, ref["valid"])
    t = oracle.Tsp(xc, yc, kind)
    for a in range(A):
        if ref["valid"][a] > 0:
            assert lengths[a] == t.tour_length(tours[a])
        else:
            assert np.isnan(lengths[a])
    assert r["valid"] == int((ref["valid"] > 0).sum())
    assert r["steps_run"] == int(ref["steps_run"][0])


@pytest.mark.parametrize("kernel", [sbx.KERNEL_RESIDENT, sbx.KERNEL_STREAM])
def test_fp32_tsp_trajectory_within_1e4(ctx, oracle, kernel):
    xc, yc = sbx.gen_cities(12, 1000.0, seed=11)
    kind = sbx.DIST_EUC_2D
    packed = sbx.tsp_distances(xc, yc, kind)
    N, A, steps = 12, 40, 100
    prob = ctx.tsp_problem(packed, N)
    prm = sbx.params(dt=0.1, steps=steps, agents=A, seed=77, precision=sbx.F32, kernel=kernel)
    r, lengths = ctx.solve(prob, prm)
    assert r["kernel_used"] == kernel
    x, y, s = ctx.state(N * N, A)
    t = oracle.Tsp(xc, yc, kind)
    o = t.solve(oracle.params(dt=0.1, steps=steps, agents=A, seed=77, threshold=50),
                want_state=True)
    assert rel_err(x, o["x"]) < TRAJ_TOL
    assert rel_err(y, o["y"]) < TRAJ_TOL


def test_tsp_config_shape_runs_and_decodes(ctx, oracle):
    # 30 cities in the unit square (float distances), penalty 1.5 max d,
    # 1024 agents: the TSP workload's shape, 2000 steps.
    xc, yc = sbx.gen_cities(30, 1.0, seed=1234)
    kind = sbx.DIST_EUC_2D_FLOAT
    packed = sbx.tsp_distances(xc, yc, kind)
    mx = packed.max()
    prob = ctx.tsp_problem(packed, 30, A=1.0, B=1.5 * mx, C_=1.5 * mx)
    r, lengths = ctx.solve(prob, sbx.params(dt=0.1, steps=2000, agents=1024, seed=5,
                                            precision=sbx.F32))
    tours, valid = ctx.tours(30, 1024)
    t = oracle.Tsp(xc, yc, kind, A=1.0, B=1.5 * mx, C_=1.5 * mx)
    nvalid = 0
    for a in range(1024):
        if valid[a] > 0:
            nvalid += 1
            assert sorted(tours[a].tolist()) == list(range(30))
            assert lengths[a] == t.tour_length(tours[a])
    assert nvalid == r["valid"]
