// Times the reference's own CPU ComputeUnit (built from its sources into
// oracle/_ref/libsymref.so by oracle/Makefile) on one of the project's
// synthetic workloads, as a measured CPU baseline beside the CPU restatement
// timed by `bench.py --impl reference`.  Test infrastructure only.
//
//   make -C oracle refbench
//   cd <scratch dir> && <repo>/oracle/_ref/ref_bench ata 100 8
//
// Device(VecWidth(4), NumThreads(threads)) as in the reference's Tutorial; one
// execute() (setArgs + run) is timed: median of 100 after 10 warm-ups.  The
// reference writes its generated code into the current directory.  Prints one
// JSON line.
#include "ComputeUnit.hpp"
#include "Symbolic.hpp"
#include "SymbolicUtilities.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "../symboliclib_gb300/csrc/workloads/workloads.hpp"

using namespace symgb_workloads;

namespace {

std::vector<Sym::Symbolic> variables(std::size_t n, int group) {
    std::vector<Sym::Symbolic> v;
    v.reserve(n);
    for (std::size_t i = 0; i < n; ++i) v.emplace_back((int)i, group);
    return v;
}

double seconds() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: ref_bench <ata|cotan> <size> <threads> [seed]\n");
        return 2;
    }
    const std::string w = argv[1];
    const int size = std::atoi(argv[2]);
    const int threads = std::atoi(argv[3]);
    const std::uint64_t seed = argc > 4 ? std::strtoull(argv[4], nullptr, 10) : 2024;
    Sym::Symbolic::varIdCounter = 0;
    std::vector<double> in;
    std::vector<Sym::Symbolic> outs, syms;
    std::vector<double> numeric;
    const double t0 = seconds();
    if (w == "ata") {
        CSC<double> A = stencilMatrix(size, 2, seed);
        syms = variables(A.nnz(), 0);
        CSC<Sym::Symbolic> B = ataPlusA(A, syms);
        outs = B.values;
        in = A.values;
        numeric = ataPlusA(A, A.values).values;
    } else if (w == "cotan") {
        TriMesh m = cotanMesh(size, seed);
        syms = variables(m.V.size(), 0);
        outs = cotanLaplacian(syms, m.nv, m.F).values;
        in = m.V;
        numeric = cotanLaplacian(m.V, m.nv, m.F).values;
    } else {
        std::fprintf(stderr, "unknown workload %s\n", w.c_str());
        return 2;
    }
    const double tModel = seconds() - t0;
    auto* cu = new Sym::ComputeUnit<double>(Sym::Device(Sym::VecWidth(4), Sym::NumThreads(threads)), syms, outs);
    const double t1 = seconds();
    cu->compile();
    const double tCompile = seconds() - t1;
    std::vector<double> res(outs.size());
    for (int i = 0; i < 10; ++i) cu->execute(in);
    std::vector<double> times;
    for (int i = 0; i < 100; ++i) {
        const double a = seconds();
        cu->execute(in);
        times.push_back(seconds() - a);
    }
    cu->getResults(res);
    std::sort(times.begin(), times.end());
    const double t = times[times.size() / 2];
    double err = 0, mx = 0;
    for (double v : numeric) mx = std::max(mx, std::fabs(v));
    for (std::size_t i = 0; i < res.size(); ++i)
        err = std::max(err, std::fabs(res[i] - numeric[i]) / std::max(std::fabs(numeric[i]), 1e-10 * mx));
    std::printf(
        "{\"impl\": \"reference CPU ComputeUnit\", \"workload\": \"%s %d\", \"device\": \"VecWidth(4), NumThreads(%d)\", "
        "\"output_nnz\": %zu, \"ms_per_execute\": %.6f, \"nnz_per_s\": %.6e, \"max_rel_err_vs_fp64_model\": %.3e, "
        "\"model_s\": %.2f, \"compile_s\": %.2f}\n",
        w.c_str(), size, threads, res.size(), t * 1e3, res.size() / t, err, tModel, tCompile);
    std::fflush(stdout);
    std::_Exit(0);  // the reference unloads its OpenMP library in ~ComputeUnit, which crashes
}
