// program.cpp -- drop-in replacement for the reference's ./build/program
// (src/main.cu:214-312): same positional arguments, same stdout lines, same
// appended output-file line (src/ising.cu:267 + src/main.cu:223 for MaxCut,
// src/ising_tsp.cu:248 for TSP), through the C ABI of libsbx.so.
//
//   program <default?> <.mtx/.tsp> <output file>
//   program 0 <file> <output file> <maxcut|tsp> <update_window> <fused> <random>
//           <time_step> <max_steps> <agents>
//
// Options after the positional arguments (all optional):
//   --seed=N         srand seed (default: time(0), as the reference)
//   --precision=P    f32 (default) | bf16 | f16 | f64
//   --kernel=K       auto (default) | stream | resident | split (registers +
//                    shared memory, 16-bit fused state) | tensor (TSP, 16-bit
//                    state: the distance product on the tensor cores)
//   --period=N       steps per window (default: the reference's)
//   --device=N       CUDA device (default 0)
//   --compat-stoi    parse time_step with std::stoi as the reference does
//                    (main.cu:303 truncates 0.1 to 0); default parses a double
//   --tsp-use-args   let TSP honour time_step/max_steps/agents (the reference
//                    fixes 0.1 / 10000 / 10000, csr.cuh:169-171, main.cu:238)
#include "../../include/sbx.h"

#include <cmath>
#include <cstdlib>
#include <ctime>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

namespace {

bool ends_with(const std::string &v, const std::string &e)
{
    return e.size() <= v.size() && std::equal(e.rbegin(), e.rend(), v.rbegin());
}

int die(const char *what, int rc)
{
    std::cerr << "program: " << what << ": " << sbx_strerror(rc) << "\n";
    return 1;
}

struct Opts {
    unsigned seed = (unsigned)std::time(0);
    int precision = SBX_F32, kernel = SBX_KERNEL_AUTO, period = 0, device = 0;
    bool compat_stoi = false, tsp_args = false;
};

int max_cut(bool uw, bool fused, double time_step, int max_steps, int agents, const std::string &ifile,
            const std::string &ofile, const Opts &o)
{
    std::ofstream file(ofile, std::ios::app);
    int64_t n = 0, nnz = 0;
    double wsum = 0;
    int rc = sbx_load_mtx(ifile.c_str(), &n, &nnz, nullptr, nullptr, nullptr, &wsum);
    if (rc) return die(ifile.c_str(), rc);
    std::vector<int32_t> rp(n + 1), col(nnz);
    std::vector<double> val(nnz);
    rc = sbx_load_mtx(ifile.c_str(), &n, &nnz, rp.data(), col.data(), val.data(), &wsum);
    if (rc) return die(ifile.c_str(), rc);
    sbx_ctx *ctx;
    if ((rc = sbx_create(&ctx, o.device))) return die("sbx_create", rc);
    sbx_problem *p;
    if ((rc = sbx_problem_csr(ctx, n, nnz, rp.data(), col.data(), val.data(), wsum, &p)))
        return die("sbx_problem_csr", rc);
    sbx_params pr;
    sbx_params_default(&pr);
    pr.dt = time_step;
    pr.steps = max_steps;
    pr.agents = agents;
    pr.fused = fused;
    pr.update_window = uw;
    pr.seed = o.seed;
    pr.precision = o.precision;
    pr.kernel = o.kernel;
    pr.period = o.period;
    sbx_result r;
    std::cout << "file: " << ifile << ", ";
    if ((rc = sbx_solve(ctx, p, &pr, &r, nullptr))) return die("sbx_solve", rc);
    const long int total_time = (long int)r.time_us;
    file << total_time << "," << r.min << "," << r.max << "," << r.mean << "," << r.std << "," << r.ps << ",";
    std::cout << "time: " << total_time << ", steps: " << max_steps << ", max: " << r.max << ", min: " << r.min
              << ", average: " << r.mean << ", Std Dev: " << r.std << ", P(s): " << r.ps
              << ", time step: " << time_step << ", # agents: " << agents << "\n";
    file << ifile << "," << n << "," << nnz << "," << max_steps << "," << time_step << "," << agents << "\n";
    sbx_problem_destroy(p);
    sbx_destroy(ctx);
    return 0;
}

int traveling_salesman(double time_step, int max_steps, int agents, const std::string &ifile,
                       const std::string &ofile, const Opts &o)
{
    std::ofstream file(ofile, std::ios::app);
    int32_t N = 0, kind = 0;
    int rc = sbx_load_tsplib(ifile.c_str(), &N, nullptr, nullptr, &kind);
    if (rc) return die(ifile.c_str(), rc);
    std::vector<double> xc(N), yc(N), packed((size_t)N * (N - 1) / 2);
    if ((rc = sbx_load_tsplib(ifile.c_str(), &N, xc.data(), yc.data(), &kind))) return die(ifile.c_str(), rc);
    std::cout << N << "\n" << (kind == SBX_DIST_GEO ? "GEO" : "EUC_2D") << "\n";   // tsp_cpu.cpp:29,33
    sbx_tsp_distances(N, xc.data(), yc.data(), kind, packed.data());
    double maximum = 0;
    for (double d : packed)
        if (d > maximum) maximum = d;
    std::cout << "\n" << maximum << "\n";   // tsp_gpu.cu:70-71
    sbx_ctx *ctx;
    if ((rc = sbx_create(&ctx, o.device))) return die("sbx_create", rc);
    sbx_problem *p;
    // construct_matrix: A = 1, B = C = max distance (tsp_gpu.cu:81-83)
    if ((rc = sbx_problem_tsp(ctx, N, packed.data(), 1.0, maximum, maximum, &p))) return die("sbx_problem_tsp", rc);
    sbx_params pr;
    sbx_params_default(&pr);
    pr.dt = o.tsp_args ? time_step : 0.1;
    pr.steps = o.tsp_args ? max_steps : 10000;
    pr.agents = o.tsp_args ? agents : 10000;
    pr.seed = o.seed;
    pr.precision = o.precision;
    pr.kernel = o.kernel;
    pr.period = o.period;
    sbx_result r;
    if ((rc = sbx_solve(ctx, p, &pr, &r, nullptr))) return die("sbx_solve", rc);
    if (r.valid == 0) std::cout << "no agent had a valid solution\n";
    const long int total_time = (long int)r.time_us;
    file << total_time << ", " << r.min << ", " << r.max << ", " << r.mean << ", " << r.std << ", " << r.valid << ", ";
    std::cout << "time: " << total_time << ", vagents: " << r.valid << ", steps: " << pr.steps << ", max: " << r.max
              << ", min: " << r.min << ", average: " << r.mean << ", Std Dev: " << r.std << "\n";
    // Ising_TSP::generate_random (ising_tsp.cu:255-270): a random tour from
    // the same rand() stream, after the n*agents draws of the init.
    srand(o.seed);
    for (int64_t i = 0; i < (int64_t)N * N * pr.agents; i++) rand();
    std::vector<int> cities(N);
    for (int i = 0; i < N; i++) cities[i] = i;
    for (int i = 1; i < N; i++) {   // random_shuffle's swap walk
        const int j = rand() % (i + 1);
        if (i != j) std::swap(cities[i], cities[j]);
    }
    double len = 0;
    for (int i = 0; i < N; i++) {
        const int a = cities[i], b = cities[(i + 1) % N], c1 = std::min(a, b), c2 = std::max(a, b);
        len += packed[(size_t)c2 + (size_t)c1 * N - (size_t)(c1 + 2) * (c1 + 1) / 2];
    }
    std::cout << "\n" << "traveling salesman distance from random spin assignment: " << len << "\n";
    sbx_problem_destroy(p);
    sbx_destroy(ctx);
    return 0;
}

}  // namespace

int main(int argc, char *argv[])
{
    std::vector<std::string> pos;
    Opts o;
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        if (a.rfind("--", 0) != 0) {
            pos.push_back(a);
            continue;
        }
        const size_t eq = a.find('=');
        const std::string k = a.substr(2, eq == std::string::npos ? std::string::npos : eq - 2);
        const std::string v = eq == std::string::npos ? "" : a.substr(eq + 1);
        if (k == "seed") o.seed = (unsigned)std::stoul(v);
        else if (k == "precision") o.precision = v == "bf16" ? SBX_BF16 : v == "f16" ? SBX_F16 : v == "f64" ? SBX_F64 : SBX_F32;
        else if (k == "kernel")
            o.kernel = v == "stream"     ? SBX_KERNEL_STREAM
                       : v == "resident" ? SBX_KERNEL_RESIDENT
                       : v == "split"    ? SBX_KERNEL_RESIDENT_SPLIT
                       : v == "tensor"   ? SBX_KERNEL_TENSOR
                                         : SBX_KERNEL_AUTO;
        else if (k == "period") o.period = std::stoi(v);
        else if (k == "device") o.device = std::stoi(v);
        else if (k == "compat-stoi") o.compat_stoi = true;
        else if (k == "tsp-use-args") o.tsp_args = true;
        else {
            std::cerr << "program: unknown option " << a << "\n";
            return -1;
        }
    }
    if (pos.size() < 3) {
        std::cout << "usage: ./program <default?> <.mtx/.tsp> <output file>\n";
        return -1;
    }
    bool mtx = false, tsp = false, update_window = false, fused = true;
    double time_step = 0.1;
    int max_steps = 10000, agents = 1024;
    const bool default_settings = (bool)std::stoi(pos[0]);
    const std::string input_file = pos[1], output_file = pos[2];
    if (default_settings) {
        if (ends_with(input_file, ".mtx")) mtx = true;
        else if (ends_with(input_file, ".tsp")) tsp = true;
    } else {
        if (pos.size() != 10) {
            std::cout << "usage: ./program <default?> <.mtx/.tsp> <output file> <maxcut/tsp> <update window?> "
                         "<fused?> <random?> <time_step> <max_steps> <agents>\n";
            return -1;
        }
        if (pos[3] == "maxcut") mtx = true;
        else if (pos[3] == "tsp") tsp = true;
        update_window = (bool)std::stoi(pos[4]);
        fused = (bool)std::stoi(pos[5]);
        (void)std::stoi(pos[6]);   // `random`: parsed, unused (main.cu:302)
        time_step = o.compat_stoi ? (double)std::stoi(pos[7]) : std::stod(pos[7]);
        max_steps = std::stoi(pos[8]);
        agents = std::stoi(pos[9]);
    }
    if (mtx) return max_cut(update_window, fused, time_step, max_steps, agents, input_file, output_file, o);
    if (tsp) return traveling_salesman(time_step, max_steps, agents, input_file, output_file, o);
    return 0;
}
