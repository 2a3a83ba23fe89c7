// Runs the reference SymbolicLib front end (oracle/_ref/libsymref.so, built
// from the reference's own sources by oracle/Makefile) on one of the project's
// synthetic workloads and keeps what its ComputeUnit generates, so that the
// reference's own execution paths can be compiled and timed next to the GPU:
//
//   cuda: cudaCode.cu   - the reference's generated CUDA source for
//                         Device(UseCuda(), ThreadsPerBlock(tpb))
//                         (ComputeUnit.cpp:364-450, StringResources.h:16-162)
//   cpu:  cpuCode.cpp   - its generated C++ for Device(VecWidth(w)) (same
//                         code path, StringResources.h:312-480); the thread
//                         count is a compile-time define (-DNUMTHREADS)
//
// plus the table files the reference writes beside the source (indexData,
// constData, outIndexData: Utilities.hpp:156-161) and the workload's input
// values (inputs.bin, float64, input containers concatenated).
// Test and baseline infrastructure only: nothing of the engine links it.
//
//   ref_codegen <outdir> <workload> <size> <seed> cuda <threads_per_block>
//   ref_codegen <outdir> <workload> <size> <seed> cpu  <vec_width>
//
// The reference writes its files into the current directory; this program
// changes into <outdir> first.  See oracle/ref_paths.sh for the recipe.
#include "ComputeUnit.hpp"
#include "Symbolic.hpp"
#include "SymbolicDifferentiation.hpp"
#include "SymbolicUtilities.hpp"

#include <unistd.h>

#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>

#include "../symboliclib_gb300/csrc/workloads/workloads.hpp"

using namespace symgb_workloads;

namespace {

// Read access to the generated source, a private member of the reference's
// ComputeUnit: an explicit template instantiation may name a private member,
// and the friend function it defines hands out the member pointer.
template <class Tag, auto M>
struct Expose {
    friend constexpr auto member(Tag) { return M; }
};
struct TCode {
    friend constexpr auto member(TCode);
};
template struct Expose<TCode, &Sym::ComputeUnit<double>::code>;

struct RefFix {
    template <class A>
    void operator()(A& K9, A& D9) const {
        Sym::makeFixed(K9, D9);
    }
};

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
    if (argc < 7) {
        std::fprintf(stderr, "usage: ref_codegen <outdir> <workload> <size> <seed> <cuda|cpu> <tpb|vecwidth>\n");
        return 2;
    }
    const std::string dir = argv[1], w = argv[2], kind = argv[5];
    const int size = std::atoi(argv[3]);
    const std::uint64_t seed = std::strtoull(argv[4], nullptr, 10);
    const int param = std::atoi(argv[6]);
    if (chdir(dir.c_str()) != 0) {
        std::perror("chdir");
        return 2;
    }
    Sym::Symbolic::varIdCounter = 0;
    const double t0 = seconds();
    std::vector<Sym::Symbolic> outs;
    std::vector<std::vector<Sym::Symbolic>> syms;
    std::vector<double> in;
    if (w == "ata") {
        CSC<double> A = stencilMatrix(size, 2, seed);
        syms.push_back(variables(A.nnz(), 0));
        outs = ataPlusA(A, syms[0]).values;
        in = A.values;
    } else if (w == "cotan") {
        TriMesh m = cotanMesh(size, seed);
        syms.push_back(variables(m.V.size(), 0));
        outs = cotanLaplacian(syms[0], m.nv, m.F).values;
        in = m.V;
    } else if (w == "cloth") {
        ClothRest r = clothRest(size);
        std::vector<double> X, vel;
        clothState(r, seed, X, vel);
        syms.push_back(variables(X.size(), 0));
        syms.push_back(variables(vel.size(), 1));
        outs = clothMatrix(r, syms[0], syms[1], RefFix()).values;
        in = X;
        in.insert(in.end(), vel.begin(), vel.end());
    } else if (w == "neohookean") {
        TetMesh m = tetMesh(size);
        in = tetState(m, seed);
        syms.push_back(variables(in.size(), 0));
        auto E = neoHookeanEnergies(m, syms[0]);
        auto upper = Sym::hessianSparse(Sym::Symbolic(Sym::ADD, E), syms[0]);
        outs = symmetricFromUpper((int)in.size(), upper).values;
    } else {
        std::fprintf(stderr, "unknown workload %s\n", w.c_str());
        return 2;
    }
    const double t1 = seconds();
    Sym::Device dev = kind == "cuda" ? Sym::Device(Sym::UseCuda(), Sym::ThreadsPerBlock(param))
                                     : Sym::Device(Sym::VecWidth(param));
    Sym::ComputeUnit<double>* u = nullptr;
    if (syms.size() == 1)
        u = new Sym::ComputeUnit<double>(dev, syms[0], outs);
    else
        u = new Sym::ComputeUnit<double>(dev, syms[0], syms[1], outs);
    const double t2 = seconds();
    {
        std::ofstream f(kind == "cuda" ? "cudaCode.cu" : "cpuCode.cpp");
        f << ((*u).*member(TCode{}));
    }
    {
        std::ofstream f("inputs.bin", std::ios::binary);
        f.write((const char*)in.data(), in.size() * sizeof(double));
    }
    std::printf("{\"workload\": \"%s\", \"size\": %d, \"seed\": %llu, \"device\": \"%s\", \"param\": %d, "
                "\"outputs\": %zu, \"inputs\": %zu, \"model_s\": %.2f, \"front_end_s\": %.2f}\n",
                w.c_str(), size, (unsigned long long)seed, kind.c_str(), param, outs.size(), in.size(), t1 - t0,
                t2 - t1);
    std::fflush(stdout);
    // The unit is never compiled and never destroyed (its destructor would
    // dlclose a library it never opened).
    std::_Exit(0);
}
