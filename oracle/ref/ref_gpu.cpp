// ref_gpu.cpp -- TEST INFRASTRUCTURE ONLY: runs the reference's own CUDA
// kernels on the GPU (MaxCut and TSP), for the differential against the
// engine.
//
// The kernels are the reference's src/kernels.cu, compiled to PTX from the
// reference sources by oracle/Makefile (`ref-ptx`, output oracle/_ref/); this
// file loads that PTX with the CUDA driver API and drives the kernels as
// Ising::reset_initialization + Ising::symplectic_update do
// (src/ising.cu:85-271): the rand() initial state and xi0 on the host, 32x32
// thread blocks over (agents, rows), the pre-step Update_XY, a captured graph
// of `sampling_period` (100) fused steps -- or the unfused Update_XY /
// mat_mult / confine / step_forward quartet -- plus update_window, launched
// and synchronised window by window, timed on the host clock; then
// compute_max_cut, sum_max_cut and the statistics line.  Nothing of the
// engine is used.  The reference's kernels update X in place while other
// threads gather it, so two runs from one seed may differ.
#include <cuda.h>

#include <chrono>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

std::string g_err;

int fail(const std::string &m)
{
    g_err = m;
    return -1;
}

#define DRV(call)                                                                   \
    do {                                                                            \
        CUresult r_ = (call);                                                       \
        if (r_ != CUDA_SUCCESS) {                                                   \
            const char *s_ = nullptr;                                               \
            cuGetErrorString(r_, &s_);                                              \
            return fail(std::string(#call) + ": " + (s_ ? s_ : "?"));               \
        }                                                                           \
    } while (0)

// The kernels by their source names (the PTX holds C++-mangled names:
// _Z<length><name><parameters>).
struct Kernels {
    CUfunction update_xy = nullptr, fused = nullptr, mat_mult = nullptr, confine = nullptr,
               step_forward = nullptr, window = nullptr, cut = nullptr, sum_cut = nullptr,
               tsp_step = nullptr, tsp_window = nullptr;
};

std::string base_name(const char *mangled)
{
    if (std::strncmp(mangled, "_Z", 2) != 0) return mangled;
    const char *p = mangled + 2;
    int len = 0;
    while (*p >= '0' && *p <= '9') len = len * 10 + (*p++ - '0');
    return std::string(p, (size_t)len);
}

int find_kernels(CUmodule mod, Kernels &k)
{
    unsigned int count = 0;
    DRV(cuModuleGetFunctionCount(&count, mod));
    std::vector<CUfunction> fs(count);
    DRV(cuModuleEnumerateFunctions(fs.data(), count, mod));
    for (CUfunction f : fs) {
        const char *nm = nullptr;
        DRV(cuFuncGetName(&nm, f));
        const std::string b = base_name(nm);
        if (b == "Update_XY") k.update_xy = f;
        else if (b == "symplectic_kernel_maxcut") k.fused = f;
        else if (b == "mat_mult") k.mat_mult = f;
        else if (b == "confine") k.confine = f;
        else if (b == "step_forward") k.step_forward = f;
        else if (b == "update_window") k.window = f;
        else if (b == "compute_max_cut") k.cut = f;
        else if (b == "sum_max_cut") k.sum_cut = f;
        else if (b == "symplectic_kernel_tsp") k.tsp_step = f;
        else if (b == "update_window_tsp") k.tsp_window = f;
    }
    if (!k.update_xy || !k.fused || !k.mat_mult || !k.confine || !k.step_forward || !k.window || !k.cut ||
        !k.sum_cut || !k.tsp_step || !k.tsp_window)
        return fail("a reference kernel is missing from the PTX");
    return 0;
}

int read_file(const char *path, std::string &out)
{
    FILE *f = std::fopen(path, "rb");
    if (!f) return fail(std::string("cannot open ") + path);
    char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, got);
    std::fclose(f);
    return 0;
}

}  // namespace

extern "C" const char *ref_gpu_last_error(void) { return g_err.c_str(); }

// One TSP run of the reference's GPU path, as Ising_TSP::reset_initialization
// + symplectic_update drive it (src/ising_tsp.cu:50-100, 111-248): x = 0 and y
// from the rand() stream, xi0 = 0.002, n = 2, 32x32 blocks over (agents,
// rows), the pre-step Update_XY, a captured graph of max_steps / 10
// symplectic_kernel_tsp launches + update_window_tsp, launched and
// synchronised until max_steps; then the tours of the valid agents from the
// final spins (src/ising_tsp.cu:200-215) and their lengths over the packed
// distances (calculate_distance_of_tour).  The QUBO in CSR and the per-city
// distance sums are the caller's (the oracle's, pinned to the reference's).
// stats[8]: loop time in microseconds (the reference's chrono region), min,
// max, mean, std of the valid tours' lengths, valid agents, SB steps run.
// lengths[agents] (NaN for agents without a valid tour) is optional.
extern "C" int ref_gpu_tsp(const char *ptx_path, int device, int ncities, int64_t nnz, const int32_t *rowptr,
                           const int32_t *col, const double *val, const double *rowsum, const double *packed,
                           double A, double B, double C, int agents, int max_steps, double dt, unsigned seed,
                           double *stats, double *lengths)
{
    if (!ptx_path || ncities < 3 || agents <= 0 || max_steps < 10 || !rowptr || !col || !val || !rowsum ||
        !packed || !stats)
        return fail("bad arguments");
    const int nrows = ncities * ncities, ncols = agents;
    const int convergence_threshold = 50;   // src/csr.cuh:167
    std::string ptx;
    if (read_file(ptx_path, ptx)) return -1;
    DRV(cuInit(0));
    CUdevice dev;
    DRV(cuDeviceGet(&dev, device));
    CUcontext ctx;
    DRV(cuDevicePrimaryCtxRetain(&ctx, dev));
    DRV(cuCtxPushCurrent(ctx));
    CUmodule mod = nullptr;
    CUstream stream = nullptr;
    CUgraph graph = nullptr;
    CUgraphExec exec = nullptr;
    CUdeviceptr d_rp = 0, d_col = 0, d_val = 0, d_rs = 0, d_x = 0, d_y = 0, d_step = 0, d_stab = 0, d_cur = 0,
                d_fin = 0, d_bif = 0, d_prev = 0, d_valid = 0, d_cv = 0, d_ov = 0;
    auto body = [&]() -> int {
        DRV(cuModuleLoadData(&mod, ptx.c_str()));
        Kernels k;
        if (find_kernels(mod, k)) return -1;
        const size_t size = (size_t)nrows * ncols;
        std::vector<double> X(size, 0.0), Y(size);
        std::srand(seed);
        for (size_t i = 0; i < size; i++) Y[i] = (((double)std::rand() / RAND_MAX) * 2 - 1) / 10;
        DRV(cuMemAlloc(&d_rp, sizeof(int) * (nrows + 1)));
        DRV(cuMemAlloc(&d_col, sizeof(int) * (nnz > 0 ? nnz : 1)));
        DRV(cuMemAlloc(&d_val, sizeof(double) * (nnz > 0 ? nnz : 1)));
        DRV(cuMemAlloc(&d_rs, sizeof(double) * ncities));
        DRV(cuMemAlloc(&d_x, sizeof(double) * size));
        DRV(cuMemAlloc(&d_y, sizeof(double) * size));
        DRV(cuMemAlloc(&d_step, sizeof(int)));
        DRV(cuMemAlloc(&d_stab, sizeof(int) * size));
        DRV(cuMemAlloc(&d_cur, sizeof(int) * size));
        DRV(cuMemAlloc(&d_fin, sizeof(int) * size));
        DRV(cuMemAlloc(&d_bif, ncols));
        DRV(cuMemAlloc(&d_prev, ncols));
        DRV(cuMemAlloc(&d_valid, sizeof(int) * ncols));
        DRV(cuMemAlloc(&d_cv, sizeof(int) * ncols * ncities));
        DRV(cuMemAlloc(&d_ov, sizeof(int) * ncols * ncities));
        DRV(cuMemcpyHtoD(d_rp, rowptr, sizeof(int) * (nrows + 1)));
        if (nnz > 0) {
            DRV(cuMemcpyHtoD(d_col, col, sizeof(int) * nnz));
            DRV(cuMemcpyHtoD(d_val, val, sizeof(double) * nnz));
        }
        DRV(cuMemcpyHtoD(d_rs, rowsum, sizeof(double) * ncities));
        DRV(cuMemcpyHtoD(d_x, X.data(), sizeof(double) * size));
        DRV(cuMemcpyHtoD(d_y, Y.data(), sizeof(double) * size));
        DRV(cuMemsetD32(d_step, 0, 1));
        DRV(cuMemsetD32(d_cur, 0xffffffffu, size));
        DRV(cuMemsetD32(d_fin, 0xffffffffu, size));
        DRV(cuMemsetD8(d_bif, 0, ncols));
        DRV(cuMemsetD8(d_prev, 0, ncols));
        DRV(cuMemsetD32(d_valid, 0, ncols));
        DRV(cuMemsetD32(d_cv, 0, (size_t)ncols * ncities));
        DRV(cuMemsetD32(d_ov, 0, (size_t)ncols * ncities));
        // the reference never initialises stability; zero it as the oracle
        // does, so that runs are reproducible where the kernels are
        DRV(cuMemsetD32(d_stab, 0, size));

        const unsigned gx = (unsigned)((ncols + 31) / 32), gy = (unsigned)((nrows + 31) / 32);
        int ms = max_steps, nc = ncols, nr = nrows, nci = ncities, thr = convergence_threshold, n2 = 2;
        double ts = dt, x0 = 0.002, a_ = A, b_ = B, c_ = C;
        void *a_xy[] = {&d_x, &d_y, &d_step, &ms, &ts, &nc, &nr};
        void *a_tsp[] = {&d_rp, &d_col, &d_val, &d_rs, &d_x, &d_y, &ts, &d_step, &ms, &x0, &n2,
                         &a_, &b_, &c_, &nci, &nc, &nr};
        void *a_win[] = {&d_x, &d_cur, &d_fin, &d_bif, &d_prev, &d_stab, &d_valid, &thr, &d_cv, &d_ov, &d_step,
                         &nci, &nc, &nr};
        const int period = max_steps / 10;
        DRV(cuStreamCreate(&stream, CU_STREAM_NON_BLOCKING));
        DRV(cuStreamBeginCapture(stream, CU_STREAM_CAPTURE_MODE_GLOBAL));
        for (int i = 0; i < period; i++)
            DRV(cuLaunchKernel(k.tsp_step, gx, gy, 1, 32, 32, 1, 0, stream, a_tsp, nullptr));
        DRV(cuLaunchKernel(k.tsp_window, gx, gy, 1, 32, 32, 1, 0, stream, a_win, nullptr));
        DRV(cuStreamEndCapture(stream, &graph));
        DRV(cuGraphInstantiate(&exec, graph, 0));
        DRV(cuCtxSynchronize());

        const auto t0 = std::chrono::high_resolution_clock::now();
        DRV(cuLaunchKernel(k.update_xy, gx, gy, 1, 32, 32, 1, 0, nullptr, a_xy, nullptr));
        DRV(cuCtxSynchronize());
        int64_t step = 0;
        bool run = true;
        while (run) {
            DRV(cuGraphLaunch(exec, stream));
            DRV(cuStreamSynchronize(stream));
            step += period;
            run = step < max_steps;
        }
        const auto t1 = std::chrono::high_resolution_clock::now();
        const double us = (double)std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count();

        std::vector<int> fin(size), valid((size_t)ncols);
        DRV(cuMemcpyDtoH(fin.data(), d_fin, sizeof(int) * size));
        DRV(cuMemcpyDtoH(valid.data(), d_valid, sizeof(int) * ncols));
        // tours of the valid agents and their lengths (src/ising_tsp.cu:
        // 200-239, calculate_distance_of_tour at :272-287)
        std::vector<double> all;
        double total = 0, mn = DBL_MAX, mx = -DBL_MAX;
        for (int a = 0; a < ncols; a++) {
            double len = NAN;
            if (valid[(size_t)a] > 0) {
                std::vector<int> cities;
                for (int order = 0; order < ncities; order++)
                    for (int city = 0; city < ncities; city++)
                        if (fin[(size_t)(order * ncities + city) * ncols + a] == 1) cities.push_back(city);
                if ((int)cities.size() != ncities) return fail("a valid agent without a tour");
                len = 0;
                for (int i = 0; i < ncities; i++) {
                    const int u = cities[(size_t)i], v = cities[(size_t)((i + 1) % ncities)];
                    const int c1 = u < v ? u : v, c2 = u < v ? v : u;
                    len += packed[c2 + c1 * ncities - (c1 + 2) * (c1 + 1) / 2];
                }
                all.push_back(len);
                total += len;
                mn = len < mn ? len : mn;
                mx = len > mx ? len : mx;
            }
            if (lengths) lengths[a] = len;
        }
        const double avg = total / (double)all.size();
        double sd = 0;
        for (double v : all) sd += std::pow(v - avg, 2);
        stats[0] = us;
        stats[1] = mn;
        stats[2] = mx;
        stats[3] = avg;
        stats[4] = std::pow(sd / ((double)all.size() - 1), 0.5);
        stats[5] = (double)all.size();
        int dstep = 0;
        DRV(cuMemcpyDtoH(&dstep, d_step, sizeof(int)));
        stats[6] = dstep;
        stats[7] = 0;
        return 0;
    };
    const int rc = body();
    if (exec) cuGraphExecDestroy(exec);
    if (graph) cuGraphDestroy(graph);
    if (stream) cuStreamDestroy(stream);
    CUdeviceptr ptrs[] = {d_rp, d_col, d_val, d_rs, d_x, d_y, d_step, d_stab, d_cur, d_fin, d_bif, d_prev,
                          d_valid, d_cv, d_ov};
    for (CUdeviceptr q : ptrs)
        if (q) cuMemFree(q);
    if (mod) cuModuleUnload(mod);
    CUcontext popped;
    cuCtxPopCurrent(&popped);
    cuDevicePrimaryCtxRelease(dev);
    return rc;
}

// One MaxCut run of the reference's GPU path.  stats[8] receives: SB loop
// time in microseconds (the reference's chrono region), min, max, mean, std,
// ps of the cuts, SB steps run, windows run.  x, y (n * agents, row-major)
// and cut (agents) are optional outputs.  run_windows > 0 stops after that
// many windows (the first run_windows * 100 steps of the max_steps
// schedule); run_windows < 0 runs the pre-step Update_XY only.
extern "C" int ref_gpu_maxcut(const char *ptx_path, int device, int64_t n64, int64_t nnz,
                              const int32_t *rowptr, const int32_t *col, const double *val, double wsum,
                              int agents, int max_steps, double dt, unsigned seed, int uw, int fused,
                              int run_windows, double *stats, double *x_out, double *y_out, double *cut_out)
{
    if (!ptx_path || n64 <= 0 || agents <= 0 || !rowptr || (nnz > 0 && (!col || !val)) || !stats)
        return fail("bad arguments");
    const int nrows = (int)n64, ncols = agents;
    const int convergence_threshold = 25, sampling_period = 100;   // src/csr.cuh:108-109
    const double pressure_slope = 0.01;                            // src/csr.cuh:113
    FILE *f = std::fopen(ptx_path, "rb");
    if (!f) return fail(std::string("cannot open ") + ptx_path);
    std::string ptx;
    char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) ptx.append(buf, got);
    std::fclose(f);

    DRV(cuInit(0));
    CUdevice dev;
    DRV(cuDeviceGet(&dev, device));
    CUcontext ctx;
    DRV(cuDevicePrimaryCtxRetain(&ctx, dev));
    DRV(cuCtxPushCurrent(ctx));
    int rc = 0;
    CUmodule mod = nullptr;
    CUstream stream = nullptr;
    CUgraph graph = nullptr;
    CUgraphExec exec = nullptr;
    CUdeviceptr d_rp = 0, d_col = 0, d_val = 0, d_x = 0, d_y = 0, d_step = 0, d_stab = 0, d_cur = 0, d_fin = 0,
                d_bif = 0, d_prev = 0, d_cuts = 0, d_final = 0;
    auto body = [&]() -> int {
        DRV(cuModuleLoadData(&mod, ptx.c_str()));
        Kernels k;
        if (find_kernels(mod, k)) return -1;
        const size_t size = (size_t)nrows * ncols;
        // src/ising.cu:85-138: X then Y from one rand() stream, xi0
        std::vector<double> X(size), Y(size);
        std::srand(seed);
        for (size_t i = 0; i < size; i++) {
            X[i] = (((double)std::rand() / RAND_MAX) * 2 - 1) / 10;
            Y[i] = (((double)std::rand() / RAND_MAX) * 2 - 1) / 10;
        }
        const double nn = (double)nrows * (double)nrows;
        double sum = 0.0, nonzero = 0.0;
        for (int64_t i = 0; i < nnz; i++) sum += val[i];
        const double mean = sum / nn;
        for (int64_t i = 0; i < nnz; i++) nonzero += std::pow(val[i] - mean, 2);
        const double zero = (nn - (double)nnz) * mean * mean;
        const double variance = std::pow((nonzero + zero) / (nn - 1), 0.5);
        const double xi0 = 0.7 / (variance * std::pow((double)nrows, 0.5));

        DRV(cuMemAlloc(&d_rp, sizeof(int) * (nrows + 1)));
        DRV(cuMemAlloc(&d_col, sizeof(int) * (nnz > 0 ? nnz : 1)));
        DRV(cuMemAlloc(&d_val, sizeof(double) * (nnz > 0 ? nnz : 1)));
        DRV(cuMemAlloc(&d_x, sizeof(double) * size));
        DRV(cuMemAlloc(&d_y, sizeof(double) * size));
        DRV(cuMemAlloc(&d_step, sizeof(int)));
        DRV(cuMemAlloc(&d_stab, sizeof(int) * ncols));
        DRV(cuMemAlloc(&d_cur, sizeof(int) * size));
        DRV(cuMemAlloc(&d_fin, sizeof(int) * size));
        DRV(cuMemAlloc(&d_bif, ncols));
        DRV(cuMemAlloc(&d_prev, ncols));
        DRV(cuMemAlloc(&d_cuts, sizeof(double) * size));
        DRV(cuMemAlloc(&d_final, sizeof(double) * ncols));
        DRV(cuMemcpyHtoD(d_rp, rowptr, sizeof(int) * (nrows + 1)));
        if (nnz > 0) {
            DRV(cuMemcpyHtoD(d_col, col, sizeof(int) * nnz));
            DRV(cuMemcpyHtoD(d_val, val, sizeof(double) * nnz));
        }
        DRV(cuMemsetD32(d_step, 0, 1));
        DRV(cuMemsetD32(d_cur, 0xffffffffu, size));
        DRV(cuMemsetD32(d_fin, 0xffffffffu, size));
        DRV(cuMemsetD8(d_bif, 0, ncols));
        DRV(cuMemsetD8(d_prev, 0, ncols));
        // the reference never initialises stability (src/ising.cu:73); zero
        // it, as the oracle does, so that window runs are reproducible
        DRV(cuMemsetD32(d_stab, 0, ncols));
        DRV(cuMemcpyHtoD(d_x, X.data(), sizeof(double) * size));
        DRV(cuMemcpyHtoD(d_y, Y.data(), sizeof(double) * size));

        const unsigned gx = (unsigned)((ncols + 31) / 32), gy = (unsigned)((nrows + 31) / 32);
        int ms = max_steps, nc = ncols, nr = nrows, thr = convergence_threshold;
        double ps_ = pressure_slope, ts = dt, x0 = xi0;
        void *a_xy[] = {&d_x, &d_y, &d_step, &ms, &ts, &nc, &nr};
        void *a_fused[] = {&d_rp, &d_col, &d_val, &d_x, &d_y, &ps_, &ts, &d_step, &ms, &x0, &nc, &nr};
        void *a_conf[] = {&d_x, &d_y, &nc, &nr};
        void *a_stepf[] = {&d_step};
        void *a_win[] = {&d_x, &d_cur, &d_fin, &d_bif, &d_prev, &d_stab, &thr, &nc, &nr};
        DRV(cuStreamCreate(&stream, CU_STREAM_NON_BLOCKING));
        DRV(cuStreamBeginCapture(stream, CU_STREAM_CAPTURE_MODE_GLOBAL));
        for (int i = 0; i < sampling_period; i++) {
            if (fused) {
                DRV(cuLaunchKernel(k.fused, gx, gy, 1, 32, 32, 1, 0, stream, a_fused, nullptr));
            } else {
                DRV(cuLaunchKernel(k.update_xy, gx, gy, 1, 32, 32, 1, 0, stream, a_xy, nullptr));
                DRV(cuLaunchKernel(k.mat_mult, gx, gy, 1, 32, 32, 1, 0, stream, a_fused, nullptr));
                DRV(cuLaunchKernel(k.confine, gx, gy, 1, 32, 32, 1, 0, stream, a_conf, nullptr));
                DRV(cuLaunchKernel(k.step_forward, gx, gy, 1, 32, 32, 1, 0, stream, a_stepf, nullptr));
            }
        }
        DRV(cuLaunchKernel(k.window, gx, gy, 1, 32, 32, 1, 0, stream, a_win, nullptr));
        DRV(cuStreamEndCapture(stream, &graph));
        DRV(cuGraphInstantiate(&exec, graph, 0));
        DRV(cuCtxSynchronize());

        const auto t0 = std::chrono::high_resolution_clock::now();
        // the pre-step, src/ising.cu:188 (on the legacy stream, as the
        // reference launches it)
        DRV(cuLaunchKernel(k.update_xy, gx, gy, 1, 32, 32, 1, 0, nullptr, a_xy, nullptr));
        DRV(cuCtxSynchronize());
        int64_t step = 0, windows = 0;
        bool run = step < max_steps && run_windows >= 0;
        std::vector<unsigned char> bif((size_t)ncols);
        while (run) {
            DRV(cuGraphLaunch(exec, stream));
            DRV(cuStreamSynchronize(stream));
            step += sampling_period;
            windows++;
            run = step < max_steps;
            if (uw) {
                DRV(cuMemcpyDtoH(bif.data(), d_bif, ncols));
                int s = 0;
                for (int i = 0; i < ncols; i++) s += bif[(size_t)i];
                if (s == ncols) run = false;
            }
            if (run_windows > 0 && windows >= run_windows) run = false;
        }
        const auto t1 = std::chrono::high_resolution_clock::now();
        const double us = (double)std::chrono::duration_cast<std::chrono::microseconds>(t1 - t0).count();

        double wsum_ = wsum;
        void *a_cut[] = {&d_rp, &d_col, &d_val, &d_cur, &d_cuts, &nc, &nr};
        void *a_sum[] = {&d_cuts, &d_final, &wsum_, &nc, &nr};
        DRV(cuLaunchKernel(k.cut, gx, gy, 1, 32, 32, 1, 0, nullptr, a_cut, nullptr));
        DRV(cuLaunchKernel(k.sum_cut, gx, gy, 1, 32, 32, 1, 0, nullptr, a_sum, nullptr));
        std::vector<double> cuts((size_t)ncols);
        DRV(cuMemcpyDtoH(cuts.data(), d_final, sizeof(double) * ncols));
        // the statistics line, src/ising.cu:238-265
        double mx = -DBL_MAX, mn = DBL_MAX, total = 0, sd = 0;
        for (double v : cuts) {
            if (v > mx) mx = v;
            if (v < mn) mn = v;
            total += v;
        }
        const double avg = total / ncols;
        int nmax = 0;
        for (double v : cuts) {
            sd += std::pow(v - avg, 2);
            if (v == mx) nmax++;
        }
        stats[0] = us;
        stats[1] = mn;
        stats[2] = mx;
        stats[3] = avg;
        stats[4] = std::pow(sd / (ncols - 1), 0.5);
        stats[5] = (double)nmax / ncols;
        int dstep = 0;
        DRV(cuMemcpyDtoH(&dstep, d_step, sizeof(int)));
        stats[6] = dstep;
        stats[7] = (double)windows;
        if (cut_out) std::memcpy(cut_out, cuts.data(), sizeof(double) * ncols);
        if (x_out) DRV(cuMemcpyDtoH(x_out, d_x, sizeof(double) * size));
        if (y_out) DRV(cuMemcpyDtoH(y_out, d_y, sizeof(double) * size));
        return 0;
    };
    rc = body();
    if (exec) cuGraphExecDestroy(exec);
    if (graph) cuGraphDestroy(graph);
    if (stream) cuStreamDestroy(stream);
    CUdeviceptr ptrs[] = {d_rp, d_col, d_val, d_x, d_y, d_step, d_stab, d_cur, d_fin, d_bif, d_prev, d_cuts, d_final};
    for (CUdeviceptr p : ptrs)
        if (p) cuMemFree(p);
    if (mod) cuModuleUnload(mod);
    CUcontext popped;
    cuCtxPopCurrent(&popped);
    cuDevicePrimaryCtxRelease(dev);
    return rc;
}
