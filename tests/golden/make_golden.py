"""Generate the golden fixtures in this directory from the REFERENCE's own code.

Runs oracle/_ref/ref_kernels -- the reference's src/kernels.cu, src/csr.cpp and
src/tsp_cpu.cpp compiled for the CPU by `make -C oracle ref` -- on small seeded
inputs, and stores inputs and outputs as .npz files.  The tests compare the
FP64 oracle against these files bit for bit, and the CUDA engine against the
oracle.  Needs the reference sources (REF_SRC, default /root/reference/src);
the fixtures it writes are committed, so nothing else needs them.

    python tests/golden/make_golden.py
"""
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import sbo  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "ref_kernels")


def write_arrays(path, arrays):
    with open(path, "wb") as f:
        for name, a in arrays.items():
            a = np.asarray(a)
            t = {np.dtype(np.int32): b"i", np.dtype(np.float64): b"d",
                 np.dtype(np.uint8): b"b"}[a.dtype]
            f.write(name.encode().ljust(32, b"\0"))
            f.write(t)
            f.write(struct.pack("<q", a.size))
            f.write(a.tobytes())


def read_arrays(path):
    out = {}
    with open(path, "rb") as f:
        while True:
            name = f.read(32)
            if len(name) < 32:
                break
            t = f.read(1)
            (cnt,) = struct.unpack("<q", f.read(8))
            dt = {b"i": np.int32, b"d": np.float64, b"b": np.uint8}[t]
            out[name.rstrip(b"\0").decode()] = np.frombuffer(
                f.read(cnt * np.dtype(dt).itemsize), dtype=dt).copy()
    return out


def run_ref(mode, inp, arrays=None):
    if not os.path.exists(REF_BIN):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    with tempfile.TemporaryDirectory() as td:
        ip = os.path.join(td, "in.bin")
        op = os.path.join(td, "out.bin")
        if arrays is not None:
            write_arrays(ip, arrays)
        else:
            ip = inp
        subprocess.run([REF_BIN, mode, ip, op], check=True, stdout=subprocess.DEVNULL)
        return read_arrays(op)


# ---------------------------------------------------------------- inputs

def er_edges(n, p, rng):
    iu, ju = np.triu_indices(n, 1)
    keep = rng.random(iu.size) < p
    return iu[keep], ju[keep]


def write_mtx(path, n, i, j, w, field="integer", symmetry="symmetric", comments=()):
    with open(path, "w") as f:
        f.write("%%%%MatrixMarket matrix coordinate %s %s\n" % (field, symmetry))
        for c in comments:
            f.write("%" + c + "\n")
        f.write("%d %d %d\n" % (n, n, len(i)))
        for a, b, v in zip(i, j, w if w is not None else [0] * len(i)):
            if field == "pattern":
                f.write("%d %d\n" % (a + 1, b + 1))
            elif field == "integer":
                f.write("%d %d %d\n" % (a + 1, b + 1, int(v)))
            else:
                f.write("%d %d %.17g\n" % (a + 1, b + 1, v))


def write_tsp(path, name, coords, kind):
    with open(path, "w") as f:
        f.write("NAME: %s\nTYPE: TSP\nCOMMENT: seeded synthetic instance\n" % name)
        f.write("DIMENSION: %d\nEDGE_WEIGHT_TYPE: %s\nNODE_COORD_SECTION\n" % (len(coords), kind))
        for k, (a, b) in enumerate(coords):
            f.write("%d %s %s\n" % (k + 1, a, b))
        f.write("EOF\n")


def make_inputs():
    rng = np.random.default_rng(20240601)
    files = {}
    # ER graph, +-1 integer weights, symmetric, every vertex with an edge.
    n = 40
    while True:
        i, j = er_edges(n, 0.15, rng)
        deg = np.bincount(np.concatenate([i, j]), minlength=n)
        if deg.min() > 0:
            break
    w = rng.choice([-1, 1], size=i.size)
    files["er40_pm1"] = os.path.join(HERE, "er40_pm1.mtx")
    write_mtx(files["er40_pm1"], n, i, j, w, comments=("seeded ER(40, 0.15), weights +-1",))
    # Same shape, real weights (FP64 order matters in the cut sum).
    wr = np.round(rng.normal(0, 1, size=i.size), 3)
    files["er40_real"] = os.path.join(HERE, "er40_real.mtx")
    write_mtx(files["er40_real"], n, i, j, wr, field="real")
    # Pattern (unweighted) ring-plus-chords, 24 vertices.
    m = 24
    pi = list(range(m)) + list(range(0, m, 3))
    pj = [(k + 1) % m for k in range(m)] + [(k + 7) % m for k in range(0, m, 3)]
    pi, pj = np.minimum(pi, pj), np.maximum(pi, pj)
    files["ring24_pattern"] = os.path.join(HERE, "ring24_pattern.mtx")
    write_mtx(files["ring24_pattern"], m, pi, pj, None, field="pattern")
    # General (non-mirrored) integer file with a diagonal entry that is dropped.
    gi = np.array([0, 1, 2, 3, 1, 2, 0, 3, 2])
    gj = np.array([1, 0, 3, 2, 2, 1, 3, 0, 2])
    gw = np.array([2, 2, -1, -1, 3, 3, 1, 1, 5])
    files["gen4_integer"] = os.path.join(HERE, "gen4_integer.mtx")
    write_mtx(files["gen4_integer"], 4, gi, gj, gw, symmetry="general")
    # TSP EUC_2D, 5 cities, integer coordinates.
    c5 = rng.integers(0, 1000, size=(5, 2))
    files["euc5"] = os.path.join(HERE, "euc5.tsp")
    write_tsp(files["euc5"], "euc5", [(str(a), str(b)) for a, b in c5], "EUC_2D")
    # TSP GEO, 6 cities, DDD.MM coordinates.
    lat = rng.uniform(10, 30, 6)
    lon = rng.uniform(90, 100, 6)
    g6 = [("%.2f" % (int(a) + 0.6 * (a - int(a))), "%.2f" % (int(b) + 0.6 * (b - int(b))))
          for a, b in zip(lat, lon)]
    files["geo6"] = os.path.join(HERE, "geo6.tsp")
    write_tsp(files["geo6"], "geo6", g6, "GEO")
    return files


# ---------------------------------------------------------------- cases

MAXCUT_CASES = [
    # name, file, agents, steps, fused, jacobi, uw, threshold, dt, seed, dumps
    ("mc_er40_fused_jacobi", "er40_pm1", 33, 300, 1, 1, 0, 25, 0.1, 7, [1, 2, 10, 100]),
    ("mc_er40_fused_serial", "er40_pm1", 33, 200, 1, 0, 0, 25, 0.1, 7, [1, 100]),
    ("mc_er40_unfused", "er40_pm1", 33, 250, 0, 1, 0, 25, 0.1, 11, [1, 100]),
    ("mc_er40_uw", "er40_pm1", 8, 3000, 1, 1, 1, 3, 0.5, 5, []),
    ("mc_er40_real", "er40_real", 33, 200, 1, 1, 0, 25, 0.3, 3, [1, 100]),
    ("mc_ring24_dt05", "ring24_pattern", 40, 400, 1, 1, 0, 25, 0.5, 1234, [100]),
]

TSP_CASES = [
    # name, file, agents, steps, jacobi, seed, dumps
    ("tsp_euc5", "euc5", 33, 200, 1, 9, [1, 20, 100]),
    ("tsp_euc5_serial", "euc5", 8, 100, 0, 9, [1]),
    ("tsp_geo6", "geo6", 16, 300, 1, 21, [30]),
]


def main():
    files = make_inputs()
    for name, key in [("load_er40_pm1", "er40_pm1"), ("load_er40_real", "er40_real"),
                      ("load_ring24_pattern", "ring24_pattern"),
                      ("load_gen4_integer", "gen4_integer")]:
        out = run_ref("mtx", files[key])
        np.savez_compressed(os.path.join(HERE, name + ".npz"), source=os.path.basename(files[key]),
                            **out)
    for name, key in [("load_euc5", "euc5"), ("load_geo6", "geo6")]:
        out = run_ref("tsplib", files[key])
        np.savez_compressed(os.path.join(HERE, name + ".npz"), source=os.path.basename(files[key]),
                            **out)
    for (name, key, A, steps, fused, jacobi, uw, thr, dt, seed, dumps) in MAXCUT_CASES:
        g = sbo.mtx_load(files[key])
        xi0 = sbo.xi0(g)
        arrays = {
            "path": np.frombuffer(files[key].encode(), np.uint8),
            "agents": np.array([A], np.int32), "steps": np.array([steps], np.int32),
            "period": np.array([100], np.int32), "fused": np.array([fused], np.int32),
            "jacobi": np.array([jacobi], np.int32), "uw": np.array([uw], np.int32),
            "threshold": np.array([thr], np.int32), "dt": np.array([dt]),
            "xi0": np.array([xi0]), "seed": np.array([seed], np.int32),
            "dump_steps": np.array(dumps, np.int32),
        }
        out = run_ref("maxcut", None, arrays)
        meta = dict(source=os.path.basename(files[key]), agents=A, steps=steps, fused=fused,
                    schedule=sbo.JACOBI if jacobi else sbo.SERIAL, uw=uw, threshold=thr,
                    dt=dt, seed=seed, xi0=xi0, dumps=np.array(dumps, np.int32))
        out = {k: (v.astype(np.int8) if k in ("cur", "fin") else v) for k, v in out.items()}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **meta, **out)
        print(name, "cuts", out["cut"][:4], "steps/windows", out["steps_windows"])
    for (name, key, A, steps, jacobi, seed, dumps) in TSP_CASES:
        arrays = {
            "path": np.frombuffer(files[key].encode(), np.uint8),
            "agents": np.array([A], np.int32), "steps": np.array([steps], np.int32),
            "threshold": np.array([50], np.int32), "jacobi": np.array([jacobi], np.int32),
            "dt": np.array([0.1]), "seed": np.array([seed], np.int32),
            "dump_steps": np.array(dumps, np.int32),
        }
        out = run_ref("tsp", None, arrays)
        meta = dict(source=os.path.basename(files[key]), agents=A, steps=steps,
                    schedule=sbo.JACOBI if jacobi else sbo.SERIAL, dt=0.1, seed=seed,
                    threshold=50, dumps=np.array(dumps, np.int32))
        out = {k: (v.astype(np.int8) if k in ("cur", "fin") else v) for k, v in out.items()}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **meta, **out)
        print(name, "valid agents", int((out["valid"] > 0).sum()), "steps", out["steps_run"])


if __name__ == "__main__":
    main()
