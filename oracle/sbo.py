"""ctypes binding of the FP64 CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline leg of bench.py, always as the checker.  The product never
imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

JACOBI, SERIAL = 0, 1
DIST_EUC_2D, DIST_GEO, DIST_EUC_2D_FLOAT = 0, 1, 2

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


class Csr(C.Structure):
    _fields_ = [("n", C.c_int64), ("nnz", C.c_int64), ("rowptr", C.c_void_p),
                ("col", C.c_void_p), ("val", C.c_void_p), ("wsum", C.c_double)]


class Params(C.Structure):
    _fields_ = [("dt", C.c_double), ("steps", C.c_int32), ("agents", C.c_int32),
                ("fused", C.c_int32), ("uw", C.c_int32), ("period", C.c_int32),
                ("threshold", C.c_int32), ("seed", C.c_uint32),
                ("schedule", C.c_int32), ("nthreads", C.c_int32), ("run_steps", C.c_int32)]


class Result(C.Structure):
    _fields_ = [("min", C.c_double), ("max", C.c_double), ("mean", C.c_double),
                ("std", C.c_double), ("ps", C.c_double), ("xi0", C.c_double),
                ("steps_run", C.c_int64), ("windows_run", C.c_int64),
                ("bifurcated", C.c_int64), ("valid", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def build():
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = C.CDLL(LIB_PATH)
        _lib.sbo_xi0.restype = C.c_double
        _lib.sbo_tsp_tour_length.restype = C.c_double
        _lib.sbo_dense_to_csr.restype = C.c_int64
    return _lib


class Graph:
    """A CSR matrix held in numpy arrays, with the reference's weight sum W."""

    def __init__(self, n, rowptr, col, val, wsum):
        self.n = int(n)
        self.rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
        self.col = np.ascontiguousarray(col, dtype=np.int32)
        self.val = np.ascontiguousarray(val, dtype=np.float64)
        self.wsum = float(wsum)

    @property
    def nnz(self):
        return int(self.col.size)

    def cstruct(self):
        return Csr(self.n, self.nnz, self.rowptr.ctypes.data, self.col.ctypes.data,
                   self.val.ctypes.data, self.wsum)


class _GenGraph(C.Structure):
    _fields_ = [("n", C.c_int64), ("nnz", C.c_int64), ("rowptr", C.c_void_p),
                ("col", C.c_void_p), ("val", C.c_void_p), ("wsum", C.c_double)]


def _gen(fn, *args):
    g = _GenGraph()
    f = getattr(lib(), fn)
    rc = f(*args, C.byref(g))
    if rc != 0:
        raise ValueError("%s failed: %d" % (fn, rc))
    try:
        n, nnz = g.n, g.nnz
        rp = np.ctypeslib.as_array((C.c_int32 * (n + 1)).from_address(g.rowptr)).copy()
        col = (np.ctypeslib.as_array((C.c_int32 * nnz).from_address(g.col)).copy()
               if nnz else np.empty(0, np.int32))
        val = (np.ctypeslib.as_array((C.c_double * nnz).from_address(g.val)).copy()
               if nnz else np.empty(0))
    finally:
        lib().sbo_graph_free(C.byref(g))
    return Graph(n, rp, col, val, g.wsum)


# The engine's seeded synthetic instances (sbx.gen_*), restated in sbo_gen.c:
# the same arguments give the same arrays.
def gen_er(n, p, pm1=False, seed=1234):
    return _gen("sbo_gen_er", C.c_int64(n), C.c_double(p), C.c_int(1 if pm1 else 0),
                C.c_uint64(seed))


def gen_torus(rows, cols, seed=1234):
    return _gen("sbo_gen_torus", C.c_int32(rows), C.c_int32(cols), C.c_uint64(seed))


def gen_rmat(scale, edge_factor=4, a=0.57, b=0.19, c=0.19, seed=1234):
    return _gen("sbo_gen_rmat", C.c_int32(scale), C.c_int32(edge_factor), C.c_double(a),
                C.c_double(b), C.c_double(c), C.c_uint64(seed))


def gen_rgg(n, avg_degree, seed=1234):
    return _gen("sbo_gen_rgg", C.c_int64(n), C.c_double(avg_degree), C.c_uint64(seed))


def gen_cities(N, scale=1.0, seed=1234):
    xc = np.empty(N)
    yc = np.empty(N)
    rc = lib().sbo_gen_cities(C.c_int32(N), C.c_double(scale), C.c_uint64(seed),
                              xc.ctypes.data_as(C.c_void_p), yc.ctypes.data_as(C.c_void_p))
    if rc != 0:
        raise ValueError("sbo_gen_cities failed")
    return xc, yc


def tsp_distances(xc, yc, kind):
    N = len(xc)
    xc = np.ascontiguousarray(xc, np.float64)
    yc = np.ascontiguousarray(yc, np.float64)
    packed = np.empty(N * (N - 1) // 2)
    if lib().sbo_tsp_distances(C.c_int32(N), xc.ctypes.data_as(C.c_void_p),
                               yc.ctypes.data_as(C.c_void_p), C.c_int(kind),
                               packed.ctypes.data_as(C.c_void_p)) != 0:
        raise ValueError("bad TSP instance")
    return packed


def params(dt=0.1, steps=10000, agents=1024, fused=1, uw=0, period=100,
           threshold=25, seed=1234, schedule=JACOBI, nthreads=0, run_steps=0):
    return Params(dt, steps, agents, fused, uw, period, threshold, seed, schedule,
                  nthreads, run_steps)


def rand_stream(seed, count):
    out = np.empty(count, np.int32)
    lib().sbo_rand_stream(C.c_uint32(seed), C.c_int64(count), out.ctypes.data_as(C.c_void_p))
    return out


def xi0(g):
    c = g.cstruct()
    return lib().sbo_xi0(C.byref(c))


def init_maxcut(n, A, seed):
    x = np.empty(n * A)
    y = np.empty(n * A)
    lib().sbo_init_maxcut(C.c_int64(n), C.c_int64(A), C.c_uint32(seed),
                          x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p))
    return x, y


def fused_step(g, x, y, A, step, max_steps, dt, xi0v, schedule=JACOBI, nthreads=0):
    c = g.cstruct()
    lib().sbo_fused_step(C.byref(c), x.ctypes.data_as(C.c_void_p),
                         y.ctypes.data_as(C.c_void_p), C.c_int64(A), C.c_int32(step),
                         C.c_int32(max_steps), C.c_double(dt), C.c_double(xi0v),
                         C.c_int(schedule), C.c_int(nthreads))


def update_xy(x, y, step, max_steps, dt):
    lib().sbo_update_xy(x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p),
                        C.c_int64(x.size), C.c_int32(step), C.c_int32(max_steps),
                        C.c_double(dt))


def unfused_step(g, x, y, A, step, max_steps, dt, xi0v):
    c = g.cstruct()
    lib().sbo_unfused_step(C.byref(c), x.ctypes.data_as(C.c_void_p),
                           y.ctypes.data_as(C.c_void_p), C.c_int64(A), C.c_int32(step),
                           C.c_int32(max_steps), C.c_double(dt), C.c_double(xi0v))


def init_tsp(n, A, seed):
    x = np.empty(n * A)
    y = np.empty(n * A)
    lib().sbo_init_tsp(C.c_int64(n), C.c_int64(A), C.c_uint32(seed),
                       x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p))
    return x, y


def cut(g, spins, A):
    c = g.cstruct()
    spins = np.ascontiguousarray(spins, dtype=np.int32)
    out = np.empty(A)
    lib().sbo_cut(C.byref(c), spins.ctypes.data_as(C.c_void_p), C.c_int64(A),
                  out.ctypes.data_as(C.c_void_p))
    return out


def maxcut_solve(g, p, want_state=False):
    c = g.cstruct()
    A = p.agents
    r = Result()
    cutv = np.empty(A)
    x = np.empty(g.n * A) if want_state else None
    y = np.empty(g.n * A) if want_state else None
    s = np.empty(g.n * A, np.int32) if want_state else None
    vp = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)
    rc = lib().sbo_maxcut_solve(C.byref(c), C.byref(p), C.byref(r), vp(cutv), vp(x),
                                vp(y), vp(s))
    if rc != 0:
        raise ValueError("sbo_maxcut_solve failed: %d" % rc)
    out = {"result": r.as_dict(), "cut": cutv}
    if want_state:
        out.update(x=x, y=y, spins=s)
    return out


F32, BF16, F16 = 0, 1, 2   # the engine's lower-precision storage modes


def round_storage(prec, v):
    """float32 values rounded to the storage type (returned as float32)."""
    v = np.ascontiguousarray(v, np.float32)
    f = lib().sbo_round_storage
    f.restype = C.c_float
    return np.array([f(C.c_int(prec), C.c_float(float(a))) for a in v.ravel()],
                    np.float32).reshape(v.shape)


def init_maxcut_lp(n, A, seed, prec):
    x = np.empty(n * A, np.float32)
    y = np.empty(n * A, np.float32)
    lib().sbo_init_maxcut_lp(C.c_int64(n), C.c_int64(A), C.c_uint32(seed), C.c_int(prec),
                             x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p))
    return x, y


def maxcut_solve_lp(g, p, prec, want_state=False):
    """The MaxCut solve in the engine's FP32 / BF16 / FP16 state mode: float
    arithmetic in the engine's operation order, rounded to the storage type
    on every store.  State is returned as float64 (exact)."""
    c = g.cstruct()
    A = p.agents
    r = Result()
    cutv = np.empty(A)
    x = np.empty(g.n * A, np.float32) if want_state else None
    y = np.empty(g.n * A, np.float32) if want_state else None
    s = np.empty(g.n * A, np.int32) if want_state else None
    vp = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)
    rc = lib().sbo_maxcut_solve_lp(C.byref(c), C.byref(p), C.c_int(prec), C.byref(r), vp(cutv),
                                   vp(x), vp(y), vp(s))
    if rc != 0:
        raise ValueError("sbo_maxcut_solve_lp failed: %d" % rc)
    out = {"result": r.as_dict(), "cut": cutv}
    if want_state:
        out.update(x=x.astype(np.float64), y=y.astype(np.float64), spins=s)
    return out


def mtx_load(path):
    n = C.c_int64()
    nnz = C.c_int64()
    w = C.c_double()
    rc = lib().sbo_mtx_load(path.encode(), C.byref(n), C.byref(nnz), None, None, None,
                            C.byref(w))
    if rc != 0:
        raise ValueError("sbo_mtx_load(%s) failed: %d" % (path, rc))
    rp = np.empty(n.value + 1, np.int32)
    col = np.empty(nnz.value, np.int32)
    val = np.empty(nnz.value)
    rc = lib().sbo_mtx_load(path.encode(), C.byref(n), C.byref(nnz),
                            rp.ctypes.data_as(C.c_void_p), col.ctypes.data_as(C.c_void_p),
                            val.ctypes.data_as(C.c_void_p), C.byref(w))
    return Graph(n.value, rp, col, val, w.value)


def tsplib_load(path):
    N = C.c_int32()
    kind = C.c_int()
    rc = lib().sbo_tsplib_load(path.encode(), C.byref(N), None, None, C.byref(kind))
    if rc != 0:
        raise ValueError("sbo_tsplib_load(%s) failed: %d" % (path, rc))
    xc = np.empty(N.value)
    yc = np.empty(N.value)
    rc = lib().sbo_tsplib_load(path.encode(), C.byref(N), xc.ctypes.data_as(C.c_void_p),
                               yc.ctypes.data_as(C.c_void_p), C.byref(kind))
    if rc != 0:
        raise ValueError("sbo_tsplib_load(%s) failed: %d" % (path, rc))
    return xc, yc, kind.value


class Tsp:
    """TSP instance: packed distances, per-city sums, the QUBO as CSR."""

    def __init__(self, xc, yc, kind, A=1.0, B=None, C_=None, penalty_scale=1.0):
        self.N = N = int(len(xc))
        self.kind = kind
        self.xc = np.ascontiguousarray(xc, np.float64)
        self.yc = np.ascontiguousarray(yc, np.float64)
        self.packed = np.empty(N * (N - 1) // 2)
        rc = lib().sbo_tsp_distances(C.c_int32(N), self.xc.ctypes.data_as(C.c_void_p),
                                     self.yc.ctypes.data_as(C.c_void_p), C.c_int(kind),
                                     self.packed.ctypes.data_as(C.c_void_p))
        if rc != 0:
            raise ValueError("bad TSP instance")
        self.rowsum = np.empty(N)
        mx = C.c_double()
        sm = C.c_double()
        lib().sbo_tsp_rowsums(C.c_int32(N), self.packed.ctypes.data_as(C.c_void_p),
                              self.rowsum.ctypes.data_as(C.c_void_p), C.byref(mx),
                              C.byref(sm))
        self.maxd = mx.value
        self.qa = float(A)
        self.qb = float(B) if B is not None else penalty_scale * mx.value
        self.qc = float(C_) if C_ is not None else penalty_scale * mx.value
        m = N * N
        dense = np.empty(m * m)
        lib().sbo_tsp_qubo_dense(C.c_int32(N), self.packed.ctypes.data_as(C.c_void_p),
                                 C.c_double(self.qa), C.c_double(self.qb),
                                 C.c_double(self.qc), dense.ctypes.data_as(C.c_void_p))
        nnz = lib().sbo_dense_to_csr(C.c_int64(m), dense.ctypes.data_as(C.c_void_p),
                                     None, None, None)
        rp = np.empty(m + 1, np.int32)
        col = np.empty(nnz, np.int32)
        val = np.empty(nnz)
        lib().sbo_dense_to_csr(C.c_int64(m), dense.ctypes.data_as(C.c_void_p),
                               rp.ctypes.data_as(C.c_void_p), col.ctypes.data_as(C.c_void_p),
                               val.ctypes.data_as(C.c_void_p))
        self.graph = Graph(m, rp, col, val, 0.0)

    def tour_length(self, tour):
        t = np.ascontiguousarray(tour, np.int32)
        return lib().sbo_tsp_tour_length(C.c_int32(self.N),
                                         self.packed.ctypes.data_as(C.c_void_p),
                                         t.ctypes.data_as(C.c_void_p))

    def step(self, x, y, A, step, max_steps, dt, schedule=JACOBI):
        c = self.graph.cstruct()
        lib().sbo_tsp_step(C.byref(c), self.rowsum.ctypes.data_as(C.c_void_p),
                           x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p),
                           C.c_int64(A), C.c_int32(step), C.c_int32(max_steps),
                           C.c_double(dt), C.c_double(0.002), C.c_int32(self.N),
                           C.c_double(self.qa), C.c_double(self.qb), C.c_double(self.qc),
                           C.c_int(schedule))

    def solve(self, p, want_state=False):
        c = self.graph.cstruct()
        A = p.agents
        r = Result()
        lengths = np.empty(A)
        tours = np.full(A * self.N, -1, np.int32)
        valid = np.empty(A, np.int32)
        n = self.N * self.N
        x = np.empty(n * A) if want_state else None
        y = np.empty(n * A) if want_state else None
        vp = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)
        rc = lib().sbo_tsp_solve(C.byref(c), C.c_int32(self.N),
                                 self.packed.ctypes.data_as(C.c_void_p),
                                 self.rowsum.ctypes.data_as(C.c_void_p),
                                 C.c_double(self.qa), C.c_double(self.qb),
                                 C.c_double(self.qc), C.byref(p), C.byref(r),
                                 vp(lengths), vp(tours), vp(x), vp(y), vp(valid))
        if rc != 0:
            raise ValueError("sbo_tsp_solve failed: %d" % rc)
        out = {"result": r.as_dict(), "lengths": lengths,
               "tours": tours.reshape(A, self.N), "valid": valid}
        if want_state:
            out.update(x=x, y=y)
        return out


# ---- the reference's own CUDA kernels on the GPU (test infrastructure) ----
# oracle/_ref/ref_kernels.ptx is the reference's src/kernels.cu compiled to
# PTX where the reference sources are; oracle/_ref/libref_gpu.so
# (oracle/ref/ref_gpu.cpp) loads it and drives the kernels as
# src/ising.cu:85-271 does.
REF_PTX = os.path.join(HERE, "_ref", "ref_kernels.ptx")
REF_GPU_LIB = os.path.join(HERE, "_ref", "libref_gpu.so")
_ref_gpu = None


def ref_gpu_available():
    return os.path.exists(REF_PTX) and os.path.exists(REF_GPU_LIB)


def _ref_lib():
    global _ref_gpu
    if _ref_gpu is None:
        _ref_gpu = C.CDLL(REF_GPU_LIB)
        _ref_gpu.ref_gpu_last_error.restype = C.c_char_p
    return _ref_gpu


def ref_gpu_maxcut(g, agents, steps, dt, seed, uw=0, fused=1, run_windows=0, want_state=False,
                   device=0):
    """One MaxCut run of the reference's GPU path (its kernels, its launch
    shapes, its graph of 100 steps + window).  Returns the statistics line
    (time_us is the reference's own host-clock region), the per-agent cuts,
    and x, y when asked."""
    st = np.zeros(8)
    cut = np.empty(agents)
    x = np.empty(g.n * agents) if want_state else None
    y = np.empty(g.n * agents) if want_state else None
    vp = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)
    rc = _ref_lib().ref_gpu_maxcut(REF_PTX.encode(), C.c_int(device), C.c_int64(g.n),
                                   C.c_int64(g.nnz), vp(g.rowptr), vp(g.col), vp(g.val),
                                   C.c_double(g.wsum), C.c_int(agents), C.c_int(steps),
                                   C.c_double(dt), C.c_uint(seed), C.c_int(uw), C.c_int(fused),
                                   C.c_int(run_windows), vp(st), vp(x), vp(y), vp(cut))
    if rc != 0:
        raise RuntimeError("ref_gpu_maxcut: " + _ref_lib().ref_gpu_last_error().decode())
    out = {"time_us": st[0], "min": st[1], "max": st[2], "mean": st[3], "std": st[4],
           "ps": st[5], "steps_run": int(st[6]), "windows_run": int(st[7]), "cut": cut}
    if want_state:
        out.update(x=x, y=y)
    return out


def ref_gpu_tsp(t, agents, steps, dt, seed, device=0):
    """One TSP run of the reference's GPU path (symplectic_kernel_tsp and
    update_window_tsp in its launch shapes, a graph of steps/10 steps + the
    window) on the oracle's QUBO and distance sums (pinned to the
    reference's).  Returns the statistics of the valid agents' tour lengths
    (time_us is the reference's own host-clock region) and every agent's
    length (NaN without a valid tour)."""
    st = np.zeros(8)
    lengths = np.empty(agents)
    g = t.graph
    vp = lambda a: a.ctypes.data_as(C.c_void_p)
    rc = _ref_lib().ref_gpu_tsp(REF_PTX.encode(), C.c_int(device), C.c_int(t.N), C.c_int64(g.nnz),
                                vp(g.rowptr), vp(g.col), vp(g.val), vp(t.rowsum), vp(t.packed),
                                C.c_double(t.qa), C.c_double(t.qb), C.c_double(t.qc), C.c_int(agents),
                                C.c_int(steps), C.c_double(dt), C.c_uint(seed), vp(st), vp(lengths))
    if rc != 0:
        raise RuntimeError("ref_gpu_tsp: " + _ref_lib().ref_gpu_last_error().decode())
    return {"time_us": st[0], "min": st[1], "max": st[2], "mean": st[3], "std": st[4],
            "valid": int(st[5]), "steps_run": int(st[6]), "lengths": lengths}
