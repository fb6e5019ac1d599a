"""sbx_fused_steps_noalloc: SB steps for callers that cannot allocate device
memory (all of it held by their own arena, or a loop that cannot take the
synchronisation cudaMalloc may bring).  The entry point is called through the
C ABI on buffers the caller owns; its result must match sbx_solve's, call
after call -- from odd and even steps, and on a second graph whose signs the
array does not hold -- because it shares one static scratch array between
calls.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

import sbx

pytestmark = pytest.mark.gpu

TOL = 1e-4


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


def _entry():
    f = sbx.lib().sbx_fused_steps_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p,
                  C.c_void_p, C.c_double, C.c_double, C.c_int32, C.c_int32, C.c_int32,
                  C.c_void_p]
    f.restype = C.c_int
    return f


def test_noalloc_steps_match_sbx_solve_on_two_calls():
    torch = pytest.importorskip("torch")
    f = _entry()
    g = sbx.gen_er(600, 0.05, pm1=True, seed=3)
    A, max_steps, dt, seed = 64, 1000, 0.2, 5
    ctx = sbx.Context(0)
    prob = ctx.problem(g)
    # period 1: the reference run can stop after any number of steps
    base = dict(dt=dt, steps=max_steps, period=1, agents=A, seed=seed, precision=sbx.F32,
                kernel=sbx.KERNEL_STREAM)
    r, _ = ctx.solve(prob, sbx.params(run_steps=1, **base))
    x0, y0, _ = ctx.state(g.n, A)

    dev = torch.device("cuda", 0)
    rowptr = torch.tensor(g.rowptr, dtype=torch.int32, device=dev)
    col = torch.tensor(g.col, dtype=torch.int32, device=dev)
    val = torch.tensor(g.val.astype(np.float32), device=dev)
    x = torch.tensor(x0.astype(np.float32).reshape(g.n, A), device=dev)
    y = torch.tensor(y0.astype(np.float32).reshape(g.n, A), device=dev)
    stream = torch.cuda.current_stream().cuda_stream

    done = 1
    for nsteps in (40, 60):
        rc = f(rowptr.data_ptr(), col.data_ptr(), val.data_ptr(), g.n, A, x.data_ptr(),
               y.data_ptr(), dt, r["xi0"], done, nsteps, max_steps, stream)
        assert rc == sbx.OK, sbx.lib().sbx_last_error()
        torch.cuda.synchronize()
        done += nsteps
        ctx.solve(prob, sbx.params(run_steps=done, **base))
        xe, ye, _ = ctx.state(g.n, A)
        assert rel(x.cpu().numpy().ravel(), xe) < TOL
        assert rel(y.cpu().numpy().ravel(), ye) < TOL

    # A third call on another graph, from an even step: the planes the first
    # two calls left in the shared array are wrong for it, and it starts on
    # the other plane.  It must still match sbx_solve.
    g2 = sbx.gen_er(420, 0.08, pm1=True, seed=11)
    prob2 = ctx.problem(g2)
    base2 = dict(base, seed=seed + 1)
    r2, _ = ctx.solve(prob2, sbx.params(run_steps=2, **base2))
    x2, y2, _ = ctx.state(g2.n, A)
    rowptr2 = torch.tensor(g2.rowptr, dtype=torch.int32, device=dev)
    col2 = torch.tensor(g2.col, dtype=torch.int32, device=dev)
    val2 = torch.tensor(g2.val.astype(np.float32), device=dev)
    xb = torch.tensor(x2.astype(np.float32).reshape(g2.n, A), device=dev)
    yb = torch.tensor(y2.astype(np.float32).reshape(g2.n, A), device=dev)
    rc = f(rowptr2.data_ptr(), col2.data_ptr(), val2.data_ptr(), g2.n, A, xb.data_ptr(),
           yb.data_ptr(), dt, r2["xi0"], 2, 30, max_steps, stream)
    assert rc == sbx.OK, sbx.lib().sbx_last_error()
    torch.cuda.synchronize()
    ctx.solve(prob2, sbx.params(run_steps=32, **base2))
    xe, ye, _ = ctx.state(g2.n, A)
    assert rel(xb.cpu().numpy().ravel(), xe) < TOL
    assert rel(yb.cpu().numpy().ravel(), ye) < TOL

    # a null column or value array is refused, whatever the matrix holds
    rc = f(rowptr.data_ptr(), None, val.data_ptr(), g.n, A, x.data_ptr(), y.data_ptr(), dt,
           r["xi0"], 0, 1, max_steps, stream)
    assert rc == -1 and b"null pointer" in sbx.lib().sbx_last_error()
    rc = f(rowptr.data_ptr(), col.data_ptr(), None, g.n, A, x.data_ptr(), y.data_ptr(), dt,
           r["xi0"], 0, 1, max_steps, stream)
    assert rc == -1 and b"null pointer" in sbx.lib().sbx_last_error()

    # beyond the static array: refused before any work, with the reason
    n_big = sbx.NOALLOC_MAX_WORDS + 1   # agents = 32: one word per row
    rc = f(rowptr.data_ptr(), col.data_ptr(), val.data_ptr(), n_big, 32, x.data_ptr(),
           y.data_ptr(), dt, r["xi0"], 0, 1, max_steps, stream)
    assert rc == -1 and b"exceeds SBX_NOALLOC_MAX_WORDS" in sbx.lib().sbx_last_error()
    ctx.close()
