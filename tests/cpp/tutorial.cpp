// The reference's Tutorial (examples/Tutorial/main.cpp) against the engine's
// C++ API: known answers of evaluate/differentiate, then B = A^T A + A through
// ComputeUnit<double>(Device(UseCuda(), ThreadsPerBlock(128)), AS, BS) when run
// with --gpu.  Exit status 0 on success.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "symgb/ComputeUnit.hpp"
#include "symgb/differentiation.hpp"
#include "../../symboliclib_gb300/csrc/workloads/workloads.hpp"

using namespace Sym;

static int failures = 0;
static void expect(bool ok, const char* what, double got, double want) {
    std::printf("%s %s: %.6f (expected %.6f)\n", ok ? "ok  " : "FAIL", what, got, want);
    if (!ok) ++failures;
}

int main(int argc, char** argv) {
    const bool gpu = argc > 1 && std::strcmp(argv[1], "--gpu") == 0;
    // Known answers of the reference README / Tutorial (main.cpp:27-33).
    Symbolic a(0, 0), b(1, 0);
    Symbolic c = a + b * sqrt(a * b);
    const std::vector<double> ab{1.0, 2.0};
    const double v = evaluate(c, ab);
    expect(std::fabs(v - 3.82843) < 5e-6, "evaluate(a + b sqrt(ab))", v, 3.82843);
    auto dc = differentiate(c, std::vector<Symbolic>{a, b});
    const double d0 = evaluate(dc[0], ab), d1 = evaluate(dc[1], ab);
    expect(std::fabs(d0 - 2.41421) < 5e-6, "d/da", d0, 2.41421);
    expect(std::fabs(d1 - 2.12132) < 5e-6, "d/db", d1, 2.12132);

    // B = A^T A + A planned by the ComputeUnit constructor.
    using namespace symgb_workloads;
    CSC<double> A = stencilMatrix(20, 2, 7);
    std::vector<Symbolic> AS;
    for (std::size_t i = 0; i < A.nnz(); ++i) AS.emplace_back((int)i, 0);
    CSC<Symbolic> BS = ataPlusA(A, AS);
    ComputeUnit<double> unit(Device(UseCuda(), ThreadsPerBlock(128)), AS, BS.values);
    const std::size_t nk = unit.planDesc().num_kernels;
    expect(nk > 0, "kernels planned", (double)nk, 1.0);
    // a block size the engine cannot honour is an error, not silently replaced
    bool rejected = false;
    try {
        Device bad(UseCuda(), ThreadsPerBlock(100));
    } catch (const std::invalid_argument&) {
        rejected = true;
    }
    expect(rejected, "ThreadsPerBlock(100) rejected", rejected, 1.0);
    // An engine error (here ValueSets(0), refused by symgb_set_num_sets) throws
    // by default; with OnError(ErrorPolicy::Print) it is printed and compile()
    // returns; with OnError(ErrorPolicy::Exit) the process exits (--exit-policy).
    {
        bool threw = false;
        try {
            ComputeUnit<double> bad(Device(UseCuda(), ValueSets(0)), AS, BS.values);
            bad.compile();
        } catch (const std::runtime_error&) {
            threw = true;
        }
        expect(threw, "engine error throws by default", threw, 1.0);
        bool printed = true;
        try {
            ComputeUnit<double> quiet(Device(UseCuda(), ValueSets(0), OnError(ErrorPolicy::Print)), AS, BS.values);
            quiet.compile();
        } catch (const std::exception&) {
            printed = false;
        }
        expect(printed, "OnError(Print) carries on", printed, 1.0);
        if (argc > 1 && std::strcmp(argv[1], "--exit-policy") == 0) {
            ComputeUnit<double> fatal(Device(UseCuda(), ValueSets(0), OnError(ErrorPolicy::Exit)), AS, BS.values);
            fatal.compile();
            std::printf("not reached\n");
            return 0;
        }
    }
    if (gpu) {
        std::vector<double> B(BS.nnz(), 0.0);
        unit.compile().execute(A.values).getResults(B);
        const std::vector<double> ref = ataPlusA(A, A.values).values;
        double err = 0.0, scale = 0.0;
        for (std::size_t i = 0; i < B.size(); ++i) {
            err = std::fmax(err, std::fabs(B[i] - ref[i]));
            scale = std::fmax(scale, std::fabs(ref[i]));
        }
        expect(err <= 1e-12 * scale, "ComputeUnit A^T A + A max abs error / scale", err / scale, 0.0);
        // a second execute with other values, results fetched by index
        std::vector<double> A2(A.values);
        for (double& x : A2) x *= -0.5;
        std::vector<double> B2(BS.nnz(), 0.0);
        unit.execute(A2).getResults(B2, 0);
        const std::vector<double> ref2 = ataPlusA(A, A2).values;
        double err2 = 0.0;
        for (std::size_t i = 0; i < B2.size(); ++i) err2 = std::fmax(err2, std::fabs(B2[i] - ref2[i]));
        expect(err2 <= 1e-12 * scale, "second execute, getResults(x, 0)", err2 / scale, 0.0);
        unit.close();
    }
    return failures ? 1 : 0;
}
