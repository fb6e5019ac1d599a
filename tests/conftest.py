import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "sparse-ising-solver_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import sbo
    sbo.lib()
    return sbo


def oracle_graph(oracle, g):
    """The oracle's CSR of an sbx.Graph."""
    return oracle.Graph(g.n, g.rowptr, g.col, g.val, g.wsum)


def oracle_first_steps(oracle, og, A, seed, dt, max_steps, k, fused):
    """The oracle's state after the pre-step and the first k steps of a
    max_steps schedule (src/ising.cu:188 then k kernel launches)."""
    x, y = oracle.init_maxcut(og.n, A, seed)
    oracle.update_xy(x, y, 0, max_steps, dt)
    x0 = oracle.xi0(og)
    for step in range(k):
        if fused:
            oracle.fused_step(og, x, y, A, step, max_steps, dt, x0)
        else:
            oracle.unfused_step(og, x, y, A, step, max_steps, dt, x0)
    return x, y
