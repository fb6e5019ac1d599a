"""Known-answer tests: instances whose answers are known without the
reference -- the 4-cycle (max cut 4), the triangle K3 (max cut 2), +-1
graphs of 16 vertices whose optimum is found by enumerating all 2^16
assignments, and 4 cities at the corners of a square of side 1000 (shortest
tour 4000, the others 2000 + 2000 sqrt 2; the reference's fixed xi0 = 0.002
suits distances of that size).

The oracle's exact cut and tour length must give these values, and SB with
enough agents must reach the optimum -- in the oracle (CPU) and in the
engine (GPU)."""
import itertools
import math

import numpy as np
import pytest

import sbx


def csr_of_edges(n, edges):
    """Symmetric CSR (both triangles, rows sorted by column) of weighted
    undirected edges (u, v, w); W = sum of w over the edges."""
    rows = [[] for _ in range(n)]
    for u, v, w in edges:
        rows[u].append((v, w))
        rows[v].append((u, w))
    rp, col, val = [0], [], []
    for r in rows:
        for c, w in sorted(r):
            col.append(c)
            val.append(float(w))
        rp.append(len(col))
    return (np.array(rp, np.int32), np.array(col, np.int32), np.array(val),
            float(sum(w for _, _, w in edges)))


def brute_max_cut(n, edges):
    """The optimum over all 2^n assignments (spin 0 fixed: a cut and its
    complement are equal)."""
    e = np.array(edges)
    u, v, w = e[:, 0].astype(int), e[:, 1].astype(int), e[:, 2]
    s = np.array(list(itertools.product([1, -1], repeat=n - 1)))
    s = np.hstack([np.ones((len(s), 1), int), s])
    return float(np.max(((1 - s[:, u] * s[:, v]) / 2 * w).sum(axis=1)))


def pm1_graph(n, p, seed):
    rng = np.random.default_rng(seed)
    edges = [(i, j, int(rng.choice([-1, 1]))) for i in range(n) for j in range(i + 1, n)
             if rng.random() < p]
    return edges


CASES = {
    "c4": (4, [(0, 1, 1), (1, 2, 1), (2, 3, 1), (3, 0, 1)], 4.0),
    "k3": (3, [(0, 1, 1), (1, 2, 1), (0, 2, 1)], 2.0),
}
for _seed in (1, 2, 3):
    _e = pm1_graph(16, 0.35, _seed)
    CASES["pm1_16_%d" % _seed] = (16, _e, brute_max_cut(16, _e))


def test_brute_force_optima_are_as_stated():
    assert brute_max_cut(4, CASES["c4"][1]) == 4.0
    assert brute_max_cut(3, CASES["k3"][1]) == 2.0


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_exact_cut_and_sb_reach_the_optimum(oracle, name):
    n, edges, best = CASES[name]
    rp, col, val, W = csr_of_edges(n, edges)
    g = oracle.Graph(n, rp, col, val, W)
    # the exact cut of two assignments: all spins equal (cut 0) and the
    # brute-force optimum's value is an upper bound of every agent's cut
    ones = np.ones(n * 2, np.int32)
    assert np.all(oracle.cut(g, ones, 2) == 0.0)
    o = oracle.maxcut_solve(g, oracle.params(dt=0.5, steps=2000, agents=64, seed=7))
    assert np.all(o["cut"] <= best)
    assert o["result"]["max"] == best


DIAG = 2000.0 + 2000.0 * math.sqrt(2)


def square_tsp(oracle):
    xc = np.array([0.0, 1000.0, 1000.0, 0.0])
    yc = np.array([0.0, 0.0, 1000.0, 1000.0])
    return xc, yc, oracle.Tsp(xc, yc, oracle.DIST_EUC_2D_FLOAT)


def test_oracle_square_tours(oracle):
    xc, yc, t = square_tsp(oracle)
    assert t.tour_length([0, 1, 2, 3]) == 4000.0
    assert math.isclose(t.tour_length([0, 2, 1, 3]), DIAG, rel_tol=1e-6)
    o = t.solve(oracle.params(dt=0.1, steps=2000, agents=64, seed=3, threshold=50))
    lengths = o["lengths"][o["valid"] > 0]
    assert len(lengths) > 0
    assert np.min(lengths) == 4000.0


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("prec", [sbx.F32, sbx.BF16])
def test_engine_reaches_the_optimum(name, prec):
    n, edges, best = CASES[name]
    rp, col, val, W = csr_of_edges(n, edges)
    ctx = sbx.Context(0)
    r, cut = ctx.solve(ctx.problem(sbx.Graph(n, rp, col, val, W)),
                       sbx.params(dt=0.5, steps=2000, agents=64, seed=7, precision=prec))
    assert np.all(cut <= best) and r["max"] == best
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [sbx.F32, sbx.BF16, sbx.F16])
def test_engine_square_tour(oracle, prec):
    xc, yc, t = square_tsp(oracle)
    ctx = sbx.Context(0)
    prob = ctx.tsp_problem(t.packed, 4)
    r, lengths = ctx.solve(prob, sbx.params(dt=0.1, steps=2000, agents=64, seed=3, precision=prec))
    ok = np.isfinite(lengths)
    assert ok.any() and np.nanmin(lengths) == 4000.0
    assert np.all(np.isclose(lengths[ok], 4000.0) | np.isclose(lengths[ok], DIAG))
    ctx.close()
