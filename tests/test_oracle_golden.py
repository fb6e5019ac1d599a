"""Pin the FP64 oracle to the reference: bit-exact against the fixtures that
tests/golden/make_golden.py produced by running the reference's own
src/kernels.cu, src/csr.cpp and src/tsp_cpu.cpp on the CPU."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

MAXCUT = ["mc_er40_fused_jacobi", "mc_er40_fused_serial", "mc_er40_unfused",
          "mc_er40_uw", "mc_er40_real", "mc_ring24_dt05"]
TSP = ["tsp_euc5", "tsp_euc5_serial", "tsp_geo6"]


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


@pytest.mark.parametrize("name,src", [("load_er40_pm1", "er40_pm1.mtx"),
                                      ("load_er40_real", "er40_real.mtx"),
                                      ("load_ring24_pattern", "ring24_pattern.mtx"),
                                      ("load_gen4_integer", "gen4_integer.mtx")])
def test_mtx_loader_matches_reference(oracle, name, src):
    ref = load(name)
    g = oracle.mtx_load(os.path.join(GOLDEN, src))
    assert g.n == ref["size_nnz"][0] and g.nnz == ref["size_nnz"][1]
    np.testing.assert_array_equal(g.rowptr, ref["rowptr"])
    np.testing.assert_array_equal(g.col, ref["col"])
    np.testing.assert_array_equal(g.val, ref["val"])
    assert g.wsum == ref["wsum"][0]


@pytest.mark.parametrize("name,src", [("load_euc5", "euc5.tsp"), ("load_geo6", "geo6.tsp")])
def test_tsplib_loader_matches_reference(oracle, name, src):
    ref = load(name)
    xc, yc, kind = oracle.tsplib_load(os.path.join(GOLDEN, src))
    assert len(xc) == ref["n_geo"][0]
    assert kind == (oracle.DIST_GEO if ref["n_geo"][1] else oracle.DIST_EUC_2D)
    np.testing.assert_array_equal(xc, ref["lat"])
    np.testing.assert_array_equal(yc, ref["lon"])


@pytest.mark.parametrize("name", MAXCUT)
def test_maxcut_trajectory_and_cut_bitexact(oracle, name):
    ref = load(name)
    g = oracle.mtx_load(os.path.join(GOLDEN, str(ref["source"])))
    np.testing.assert_array_equal(g.rowptr, ref["rowptr"])
    A, steps, dt = int(ref["agents"]), int(ref["steps"]), float(ref["dt"])
    xi0 = oracle.xi0(g)
    assert xi0 == float(ref["xi0"])
    x, y = oracle.init_maxcut(g.n, A, int(ref["seed"]))
    oracle.update_xy(x, y, 0, steps, dt)
    np.testing.assert_array_equal(x, ref["x_pre"])
    np.testing.assert_array_equal(y, ref["y_pre"])
    dumps = set(int(d) for d in ref["dumps"])
    for k in range(max(dumps) if dumps else 0):
        if int(ref["fused"]):
            oracle.fused_step(g, x, y, A, k, steps, dt, xi0, int(ref["schedule"]))
        else:
            oracle.unfused_step(g, x, y, A, k, steps, dt, xi0)
        if k + 1 in dumps:
            np.testing.assert_array_equal(x, ref["x_%d" % (k + 1)], err_msg="step %d" % (k + 1))
            np.testing.assert_array_equal(y, ref["y_%d" % (k + 1)], err_msg="step %d" % (k + 1))
    p = oracle.params(dt=dt, steps=steps, agents=A, fused=int(ref["fused"]), uw=int(ref["uw"]),
                      threshold=int(ref["threshold"]), seed=int(ref["seed"]),
                      schedule=int(ref["schedule"]))
    out = oracle.maxcut_solve(g, p, want_state=True)
    np.testing.assert_array_equal(out["x"], ref["x"])
    np.testing.assert_array_equal(out["y"], ref["y"])
    np.testing.assert_array_equal(out["spins"], ref["cur"].astype(np.int32))
    np.testing.assert_array_equal(out["cut"], ref["cut"])
    assert out["result"]["steps_run"] == ref["steps_windows"][0]
    assert out["result"]["windows_run"] == ref["steps_windows"][1]
    assert out["result"]["bifurcated"] == int(ref["bif"].sum())
    # the cut of the final spins, recomputed from spins alone
    np.testing.assert_array_equal(oracle.cut(g, out["spins"], A), ref["cut"])


@pytest.mark.parametrize("name", TSP)
def test_tsp_trajectory_and_tours_bitexact(oracle, name):
    ref = load(name)
    xc, yc, kind = oracle.tsplib_load(os.path.join(GOLDEN, str(ref["source"])))
    t = oracle.Tsp(xc, yc, kind)
    np.testing.assert_array_equal(t.packed, ref["dist"])
    np.testing.assert_array_equal(t.rowsum, ref["rowsum"])
    np.testing.assert_array_equal(t.graph.rowptr, ref["rowptr"])
    np.testing.assert_array_equal(t.graph.col, ref["col"])
    np.testing.assert_array_equal(t.graph.val, ref["val"])
    A, steps, dt = int(ref["agents"]), int(ref["steps"]), float(ref["dt"])
    n = t.N * t.N
    x, y = oracle.init_tsp(n, A, int(ref["seed"]))
    oracle.update_xy(x, y, 0, steps, dt)
    np.testing.assert_array_equal(x, ref["x_pre"])
    np.testing.assert_array_equal(y, ref["y_pre"])
    dumps = set(int(d) for d in ref["dumps"])
    for k in range(max(dumps)):
        t.step(x, y, A, k, steps, dt, int(ref["schedule"]))
        if k + 1 in dumps:
            np.testing.assert_array_equal(x, ref["x_%d" % (k + 1)], err_msg="step %d" % (k + 1))
            np.testing.assert_array_equal(y, ref["y_%d" % (k + 1)], err_msg="step %d" % (k + 1))
    p = oracle.params(dt=dt, steps=steps, agents=A, threshold=50, seed=int(ref["seed"]),
                      schedule=int(ref["schedule"]))
    out = t.solve(p, want_state=True)
    np.testing.assert_array_equal(out["x"], ref["x"])
    np.testing.assert_array_equal(out["y"], ref["y"])
    np.testing.assert_array_equal(out["valid"], ref["valid"])
    assert out["result"]["steps_run"] == ref["steps_run"][0]
    fin = ref["fin"].astype(np.int32).reshape(n, A)
    for c in range(A):
        if ref["valid"][c] > 0:
            order = [city for o in range(t.N) for city in range(t.N)
                     if fin[o * t.N + city, c] == 1]
            assert list(out["tours"][c]) == order
            assert out["lengths"][c] == t.tour_length(order)
        else:
            assert np.isnan(out["lengths"][c])
