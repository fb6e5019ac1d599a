/*
 * ref_kernels.cpp -- drives the REFERENCE's own code on the CPU, to pin the
 * oracle (oracle/sbo_*.c) to it.  TEST INFRASTRUCTURE ONLY; built by
 * oracle/Makefile into oracle/_ref/ (git-ignored) only where the reference
 * sources are present, and used only by tests/golden/make_golden.py.
 *
 * Linked with, unmodified, from the reference tree:
 *   src/kernels.cu   (through oracle/ref/shim/cuda_runtime.h; each launch
 *                     below runs the kernel once per CUDA thread)
 *   src/csr.cpp      (CSR::from_file, CSR::from_matrix, construct_csr)
 *   src/tsp_cpu.cpp  (TSP_CPU::read_file)
 * Restated here (they sit in files that also hold <<<>>> launches): the
 * host orchestration of src/ising.cu:85-236 and src/ising_tsp.cu:50-176, and
 * the host parts of src/tsp_gpu.cu:51-112.
 *
 * I/O: a stream of named arrays, each
 *   char name[32]; char type ('i' int32, 'd' double, 'b' uint8); int64 count;
 *   then count elements.
 */
#include "cuda_runtime.h"

#include "csr.cuh"
#include "kernels.cuh"

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

dim3 threadIdx, blockIdx, blockDim, gridDim;

namespace {

struct Arr {
    char type;
    std::vector<char> bytes;
    template <class T> T *as() { return reinterpret_cast<T *>(bytes.data()); }
    int64_t count() const
    {
        size_t es = type == 'd' ? 8 : type == 'i' ? 4 : 1;
        return (int64_t)(bytes.size() / es);
    }
};

std::map<std::string, Arr> read_arrays(const char *path)
{
    std::map<std::string, Arr> m;
    FILE *f = fopen(path, "rb");
    if (!f) {
        perror(path);
        exit(2);
    }
    char name[32];
    while (fread(name, 1, 32, f) == 32) {
        Arr a;
        int64_t cnt;
        if (fread(&a.type, 1, 1, f) != 1 || fread(&cnt, 8, 1, f) != 1) break;
        size_t es = a.type == 'd' ? 8 : a.type == 'i' ? 4 : 1;
        a.bytes.resize((size_t)cnt * es);
        if (cnt && fread(a.bytes.data(), es, (size_t)cnt, f) != (size_t)cnt) break;
        m[std::string(name)] = std::move(a);
    }
    fclose(f);
    return m;
}

struct Writer {
    FILE *f;
    explicit Writer(const char *p) : f(fopen(p, "wb")) {}
    ~Writer() { fclose(f); }
    void put(const char *nm, char type, const void *p, int64_t cnt)
    {
        char name[32] = {0};
        strncpy(name, nm, 31);
        fwrite(name, 1, 32, f);
        fwrite(&type, 1, 1, f);
        fwrite(&cnt, 8, 1, f);
        size_t es = type == 'd' ? 8 : type == 'i' ? 4 : 1;
        if (cnt) fwrite(p, es, (size_t)cnt, f);
    }
};

double getd(std::map<std::string, Arr> &m, const char *k) { return m[k].as<double>()[0]; }
int geti(std::map<std::string, Arr> &m, const char *k) { return m[k].as<int32_t>()[0]; }

/* Run `kern` once for every CUDA thread of a (ceil(nx/32), ceil(ny/32)) grid
 * of 32x32 blocks, in CUDA's linear order (block x fastest, then thread x). */
template <class F> void launch_serial(int nx, int ny, F kern)
{
    blockDim = {32, 32, 1};
    gridDim = {(unsigned)((nx + 31) / 32), (unsigned)((ny + 31) / 32), 1};
    for (unsigned by = 0; by < gridDim.y; by++)
        for (unsigned bx = 0; bx < gridDim.x; bx++)
            for (unsigned ty = 0; ty < 32; ty++)
                for (unsigned tx = 0; tx < 32; tx++) {
                    blockIdx = {bx, by, 0};
                    threadIdx = {tx, ty, 0};
                    kern();
                }
}

/* As launch_serial, but every thread sees the memory as it was when the
 * launch began: after each thread its own X/Y element and the step counter
 * are put back, and all writes are applied when every thread has run.  The
 * step kernels write nothing else. */
template <class F>
void launch_jacobi(int ncols, int nrows, double *X, double *Y, int *step, F kern)
{
    const int64_t sz = (int64_t)ncols * nrows;
    std::vector<double> nx(X, X + sz), ny(Y, Y + sz);
    const int step0 = *step;
    int step_after = step0;
    blockDim = {32, 32, 1};
    gridDim = {(unsigned)((ncols + 31) / 32), (unsigned)((nrows + 31) / 32), 1};
    for (unsigned by = 0; by < gridDim.y; by++)
        for (unsigned bx = 0; bx < gridDim.x; bx++)
            for (unsigned ty = 0; ty < 32; ty++)
                for (unsigned tx = 0; tx < 32; tx++) {
                    int col = bx * 32 + tx, row = by * 32 + ty;
                    blockIdx = {bx, by, 0};
                    threadIdx = {tx, ty, 0};
                    if (row >= nrows || col >= ncols) {
                        kern();
                        continue;
                    }
                    int64_t i = (int64_t)row * ncols + col;
                    double x0 = X[i], y0 = Y[i];
                    kern();
                    nx[i] = X[i];
                    ny[i] = Y[i];
                    X[i] = x0;
                    Y[i] = y0;
                    if (*step != step0) step_after = *step;
                    *step = step0;
                }
    memcpy(X, nx.data(), sizeof(double) * sz);
    memcpy(Y, ny.data(), sizeof(double) * sz);
    *step = step_after;
}

void init_xy(int64_t sz, unsigned seed, double *x, double *y, bool tsp)
{
    srand(seed);   /* ising.cu:91-95 / ising_tsp.cu:55-59 */
    for (int64_t i = 0; i < sz; i++) {
        if (tsp) {
            x[i] = 0;
            y[i] = (((double)rand() / RAND_MAX) * 2 - 1) / 10;
        } else {
            x[i] = (((double)rand() / RAND_MAX) * 2 - 1) / 10;
            y[i] = (((double)rand() / RAND_MAX) * 2 - 1) / 10;
        }
    }
}

/* MaxCut: load the .mtx with the reference's CSR class, then the host flow
 * of Ising::symplectic_update with emulated launches. */
int run_maxcut(const char *in, const char *out)
{
    auto m = read_arrays(in);
    std::string path(m["path"].as<char>(), m["path"].bytes.size());
    CSR csr(path);
    const int nrows = csr.size, ncols = geti(m, "agents");
    const int max_steps = geti(m, "steps"), period = geti(m, "period");
    const int fused = geti(m, "fused"), jacobi = geti(m, "jacobi");
    const int uw = geti(m, "uw"), threshold = geti(m, "threshold");
    const double dt = getd(m, "dt"), xi0 = getd(m, "xi0");
    const unsigned seed = (unsigned)geti(m, "seed");
    Arr &dumps = m["dump_steps"];
    const int64_t sz = (int64_t)nrows * ncols;
    std::vector<double> X(sz), Y(sz), cut(sz), fcut(ncols);
    std::vector<int> cur(sz, -1), fin(sz, -1), stab(ncols, 0);
    bool *bif = new bool[ncols](), *prev = new bool[ncols]();
    init_xy(sz, seed, X.data(), Y.data(), false);
    int *ap = csr.csr_row_indices.data(), *ai = csr.csr_columns.data();
    double *av = csr.csr_data.data();
    int step = 0;
    Writer w(out);
    w.put("rowptr", 'i', ap, (int64_t)csr.csr_row_indices.size());
    w.put("col", 'i', ai, (int64_t)csr.csr_columns.size());
    w.put("val", 'd', av, (int64_t)csr.csr_data.size());
    w.put("wsum", 'd', &csr.sum, 1);
    launch_serial(ncols, nrows, [&] {
        Update_XY(X.data(), Y.data(), &step, max_steps, dt, ncols, nrows);
    });
    w.put("x_pre", 'd', X.data(), sz);
    w.put("y_pre", 'd', Y.data(), sz);
    int64_t host_step = 0, windows = 0;
    bool run = host_step < max_steps;
    auto maybe_dump = [&](int s) {
        for (int64_t k = 0; k < dumps.count(); k++)
            if (dumps.as<int32_t>()[k] == s) {
                std::string nx = "x_" + std::to_string(s), ny = "y_" + std::to_string(s);
                w.put(nx.c_str(), 'd', X.data(), sz);
                w.put(ny.c_str(), 'd', Y.data(), sz);
            }
    };
    while (run) {
        for (int i = 0; i < period; i++) {
            if (fused) {
                auto k = [&] {
                    symplectic_kernel_maxcut(ap, ai, av, X.data(), Y.data(), 0.01, dt,
                                             &step, max_steps, xi0, ncols, nrows);
                };
                if (jacobi) launch_jacobi(ncols, nrows, X.data(), Y.data(), &step, k);
                else launch_serial(ncols, nrows, k);
            } else {
                launch_serial(ncols, nrows, [&] {
                    Update_XY(X.data(), Y.data(), &step, max_steps, dt, ncols, nrows);
                });
                launch_serial(ncols, nrows, [&] {
                    mat_mult(ap, ai, av, X.data(), Y.data(), 0.01, dt, &step, max_steps,
                             xi0, ncols, nrows);
                });
                launch_serial(ncols, nrows, [&] { confine(X.data(), Y.data(), ncols, nrows); });
                launch_serial(ncols, nrows, [&] { step_forward(&step); });
            }
            maybe_dump(step);
        }
        launch_serial(ncols, nrows, [&] {
            update_window(X.data(), cur.data(), fin.data(), bif, prev, stab.data(),
                          threshold, ncols, nrows);
        });
        windows++;
        host_step += period;
        run = host_step < max_steps;
        if (uw) {
            int s = 0;
            for (int c = 0; c < ncols; c++) s += bif[c];
            if (s == ncols) run = false;
        }
    }
    launch_serial(ncols, nrows, [&] {
        compute_max_cut(ap, ai, av, cur.data(), cut.data(), ncols, nrows);
    });
    launch_serial(ncols, nrows, [&] {
        sum_max_cut(cut.data(), fcut.data(), csr.sum, ncols, nrows);
    });
    std::vector<uint8_t> b(ncols);
    for (int c = 0; c < ncols; c++) b[c] = bif[c];
    w.put("x", 'd', X.data(), sz);
    w.put("y", 'd', Y.data(), sz);
    w.put("cur", 'i', cur.data(), sz);
    w.put("fin", 'i', fin.data(), sz);
    w.put("stab", 'i', stab.data(), ncols);
    w.put("bif", 'b', b.data(), ncols);
    w.put("cut", 'd', fcut.data(), ncols);
    int sw[2] = {step, (int)windows};
    w.put("steps_windows", 'i', sw, 2);
    delete[] bif;
    delete[] prev;
    return 0;
}

/* TSP: TSP_CPU + the reference distance kernel + CSR::from_matrix, then the
 * host flow of Ising_TSP::symplectic_update with emulated launches. */
int run_tsp(const char *in, const char *out)
{
    auto m = read_arrays(in);
    std::string path(m["path"].as<char>(), m["path"].bytes.size());
    TSP_CPU tsp(path);
    const int N = tsp.ncities, nd = tsp.nonzeros;
    std::vector<double> dist(nd), rowsum(N, 0.0);
    launch_serial(N, N, [&] {
        if (tsp.dtype == "GEO")
            TSP_distances_GEO(dist.data(), tsp.latitudes.data(), tsp.longitudes.data(), N);
        else
            TSP_distances_EUC_2D(dist.data(), tsp.latitudes.data(), tsp.longitudes.data(), N);
    });
    double maximum = 0, sumd = 0;
    {   /* tsp_gpu.cu:51-68 */
        int i = 0, j = 0;
        for (int k = 0; k < nd; k++) {
            if (j == N - 1) {
                i++;
                j = i;
            }
            j++;
            rowsum[i] += dist[k];
            rowsum[j] += dist[k];
            sumd += dist[k];
            if (dist[k] > maximum) maximum = dist[k];
        }
    }
    const double A = 1, B = maximum, C = maximum;   /* tsp_gpu.cu:81-83 */
    std::vector<double> full;
    for (int i = 0; i < N; i++)   /* tsp_gpu.cu:84-108 */
        for (int k = 0; k < N; k++)
            for (int j = 0; j < N; j++)
                for (int l = 0; l < N; l++) {
                    if (i != j && k == l) full.push_back(C / 4);
                    else if ((i == j + 1 || j == i + 1 || (i == 0 && j == N - 1) ||
                              (i == N - 1 && j == 0)) && k != l) {
                        int c1 = std::min(k, l), c2 = std::max(k, l);
                        int pos = ((2 * N - c1 - 3) * c1) / 2 + c2 - 1;
                        full.push_back(A * dist[pos] / 8);
                    } else if (i == j && k != l) full.push_back(B / 4);
                    else if (i == j && k == l) full.push_back((B + C) / 4);
                    else full.push_back(0);
                }
    CSR csr(full, N * N);
    const int nrows = csr.size, ncols = geti(m, "agents");
    const int max_steps = geti(m, "steps"), threshold = geti(m, "threshold");
    const int jacobi = geti(m, "jacobi");
    const double dt = getd(m, "dt"), xi0 = 0.002;
    const unsigned seed = (unsigned)geti(m, "seed");
    Arr &dumps = m["dump_steps"];
    const int64_t sz = (int64_t)nrows * ncols;
    std::vector<double> X(sz), Y(sz);
    std::vector<int> cur(sz, -1), fin(sz, -1), stab(sz, 0), valid(ncols, 0);
    std::vector<int> cv(N * ncols, 0), ov(N * ncols, 0);
    bool *bif = new bool[ncols](), *prev = new bool[ncols]();
    init_xy(sz, seed, X.data(), Y.data(), true);
    int *ap = csr.csr_row_indices.data(), *ai = csr.csr_columns.data();
    double *av = csr.csr_data.data();
    Writer w(out);
    std::vector<double> coords;
    for (int c = 0; c < N; c++) {
        coords.push_back(tsp.latitudes[c]);
        coords.push_back(tsp.longitudes[c]);
    }
    w.put("coords", 'd', coords.data(), 2 * N);
    w.put("dist", 'd', dist.data(), nd);
    w.put("rowsum", 'd', rowsum.data(), N);
    w.put("rowptr", 'i', ap, (int64_t)csr.csr_row_indices.size());
    w.put("col", 'i', ai, (int64_t)csr.csr_columns.size());
    w.put("val", 'd', av, (int64_t)csr.csr_data.size());
    int step = 0;
    const int period = max_steps / 10, n = 2;
    launch_serial(ncols, nrows, [&] {
        Update_XY(X.data(), Y.data(), &step, max_steps, dt, ncols, nrows);
    });
    w.put("x_pre", 'd', X.data(), sz);
    w.put("y_pre", 'd', Y.data(), sz);
    int64_t host_step = 0;
    bool run = true;
    while (run) {
        for (int i = 0; i < period; i++) {
            auto k = [&] {
                symplectic_kernel_tsp(ap, ai, av, rowsum.data(), X.data(), Y.data(), dt,
                                      &step, max_steps, xi0, n, A, B, C, N, ncols, nrows);
            };
            if (jacobi) launch_jacobi(ncols, nrows, X.data(), Y.data(), &step, k);
            else launch_serial(ncols, nrows, k);
            for (int64_t q = 0; q < dumps.count(); q++)
                if (dumps.as<int32_t>()[q] == step) {
                    std::string nx = "x_" + std::to_string(step), ny = "y_" + std::to_string(step);
                    w.put(nx.c_str(), 'd', X.data(), sz);
                    w.put(ny.c_str(), 'd', Y.data(), sz);
                }
        }
        launch_serial(ncols, nrows, [&] {
            update_window_tsp(X.data(), cur.data(), fin.data(), bif, prev, stab.data(),
                              valid.data(), threshold, cv.data(), ov.data(), &step, N,
                              ncols, nrows);
        });
        host_step += period;
        run = host_step < max_steps;
    }
    w.put("x", 'd', X.data(), sz);
    w.put("y", 'd', Y.data(), sz);
    w.put("cur", 'i', cur.data(), sz);
    w.put("fin", 'i', fin.data(), sz);
    w.put("valid", 'i', valid.data(), ncols);
    w.put("steps_run", 'i', &step, 1);
    delete[] bif;
    delete[] prev;
    return 0;
}

/* Loader dumps: the reference's CSR / TSP_CPU objects as parsed. */
int dump_mtx(const char *path, const char *out)
{
    CSR csr(path);
    Writer w(out);
    w.put("rowptr", 'i', csr.csr_row_indices.data(), (int64_t)csr.csr_row_indices.size());
    w.put("col", 'i', csr.csr_columns.data(), (int64_t)csr.csr_columns.size());
    w.put("val", 'd', csr.csr_data.data(), (int64_t)csr.csr_data.size());
    w.put("wsum", 'd', &csr.sum, 1);
    int meta[2] = {csr.size, csr.nonzeros};
    w.put("size_nnz", 'i', meta, 2);
    return 0;
}

int dump_tsp(const char *path, const char *out)
{
    TSP_CPU tsp(path);
    Writer w(out);
    w.put("lat", 'd', tsp.latitudes.data(), (int64_t)tsp.latitudes.size());
    w.put("lon", 'd', tsp.longitudes.data(), (int64_t)tsp.longitudes.size());
    int meta[2] = {tsp.ncities, tsp.dtype == "GEO" ? 1 : 0};
    w.put("n_geo", 'i', meta, 2);
    return 0;
}

/* Loader timing: the reference's CSR (src/csr.cpp) or TSP_CPU
 * (src/tsp_cpu.cpp) constructor on one file, `reps` times, one thread as the
 * reference runs it; prints the fastest wall time in seconds and the sizes. */
int time_loader(const char *kind, const char *path, int reps)
{
    double best = 1e300;
    long long a = 0, b = 0;
    for (int i = 0; i < reps; i++) {
        const auto t0 = std::chrono::steady_clock::now();
        if (std::string(kind) == "mtx-time") {
            CSR csr(path);
            a = csr.size;
            b = csr.nonzeros;
        } else {
            TSP_CPU tsp(path);
            a = tsp.ncities;
        }
        const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        best = s < best ? s : best;
    }
    printf("%.9f %lld %lld\n", best, a, b);
    return 0;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc == 4 && (std::string(argv[1]) == "mtx-time" || std::string(argv[1]) == "tsplib-time"))
        return time_loader(argv[1], argv[2], atoi(argv[3]));
    if (argc != 4) {
        fprintf(stderr, "usage: ref_kernels maxcut|tsp|mtx|tsplib <in> <out>\n"
                        "       ref_kernels mtx-time|tsplib-time <in> <repetitions>\n");
        return 2;
    }
    std::string mode = argv[1];
    if (mode == "maxcut") return run_maxcut(argv[2], argv[3]);
    if (mode == "tsp") return run_tsp(argv[2], argv[3]);
    if (mode == "mtx") return dump_mtx(argv[2], argv[3]);
    if (mode == "tsplib") return dump_tsp(argv[2], argv[3]);
    return 2;
}
