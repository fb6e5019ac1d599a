"""The oracle's lower-precision mode and its generator restatement, on the CPU.

* Rounding to the storage types equals torch's (bfloat16) and numpy's
  (float16) round-to-nearest-even conversions, subnormals included.
* The FP32 mode follows the FP64 restatement of the reference to 1e-4 over
  the first 100 steps (the parity clause the engine's FP32 mode meets).
* The oracle-side generators build the same instances as the engine's
  (sbx_gen_*): the benchmark's CPU legs use them without loading the engine.
"""
import os

import numpy as np
import pytest

import bench
from conftest import GOLDEN


def _random_floats(n, seed):
    rng = np.random.default_rng(seed)
    bits = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
    f = bits.view(np.float32)
    f = f[np.isfinite(f)]
    # plus values around the storage types' subnormal and overflow ranges
    extra = np.concatenate([rng.uniform(-1, 1, 2000) * 2.0 ** -14, rng.uniform(-1, 1, 2000) * 2.0 ** -126,
                            rng.uniform(-1, 1, 2000) * 65520.0, rng.uniform(-1, 1, 2000)])
    return np.concatenate([f, extra.astype(np.float32)])


def test_bf16_rounding_matches_torch(oracle):
    torch = pytest.importorskip("torch")
    v = _random_floats(20000, 1)
    got = oracle.round_storage(oracle.BF16, v)
    want = torch.from_numpy(v).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_f16_rounding_matches_numpy(oracle):
    v = _random_floats(20000, 2)
    got = oracle.round_storage(oracle.F16, v)
    with np.errstate(over="ignore"):
        want = v.astype(np.float16).astype(np.float32)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_f32_mode_follows_fp64_for_100_steps(oracle):
    g = oracle.mtx_load(os.path.join(GOLDEN, "er40_pm1.mtx"))
    A, steps, dt, seed = 48, 10000, 0.1, 9
    o = oracle.maxcut_solve_lp(g, oracle.params(dt=dt, steps=steps, agents=A, seed=seed,
                                                period=100, run_steps=100), oracle.F32,
                               want_state=True)
    x, y = oracle.init_maxcut(g.n, A, seed)
    oracle.update_xy(x, y, 0, steps, dt)
    x0 = oracle.xi0(g)
    for k in range(100):
        oracle.fused_step(g, x, y, A, k, steps, dt, x0)
    err = np.max(np.abs(o["x"] - x)) / np.max(np.abs(x))
    assert 0 < err < 1e-4
    # BF16 keeps its sign planes consistent: the window spins are the signs
    # of the stored state
    ob = oracle.maxcut_solve_lp(g, oracle.params(dt=dt, steps=steps, agents=A, seed=seed,
                                                 period=100, run_steps=100), oracle.BF16,
                                want_state=True)
    assert np.array_equal(np.where(np.signbit(ob["x"]), -1, 1), ob["spins"])
    assert np.array_equal(oracle.round_storage(oracle.BF16, ob["x"].astype(np.float32)),
                          ob["x"].astype(np.float32))


def _same(a, b):
    return (a.n == b.n and np.array_equal(a.rowptr, b.rowptr) and np.array_equal(a.col, b.col)
            and np.array_equal(a.val, b.val) and a.wsum == b.wsum)


@pytest.mark.parametrize("name", ["er800", "torus"])
def test_generators_match_the_engine(oracle, name):
    import sbx
    wl = bench.WORKLOADS[name]
    assert _same(bench.build_instance(wl, oracle), bench.build_instance(wl, sbx))


def test_batch_and_tsp_generators_match_the_engine(oracle):
    import sbx
    wl = bench.WORKLOADS["batch512"]
    specs = bench.batch_specs(wl["instances"])
    for sp in specs[:24]:
        assert _same(bench.batch_graph(sp, oracle), bench.batch_graph(sp, sbx)), sp
    assert _same(oracle.gen_rmat(14, 4, seed=5), sbx.gen_rmat(14, 4, seed=5))
    a = bench.build_instance(bench.WORKLOADS["tsp30"], oracle)
    b = bench.build_instance(bench.WORKLOADS["tsp30"], sbx)
    for k in ("xc", "yc", "packed"):
        assert np.array_equal(a[k], b[k])
    assert a["B"] == b["B"] and a["C"] == b["C"]
