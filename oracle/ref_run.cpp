// Loads a library built from the reference's generated source (cudaCode.cu or
// cpuCode.cpp, kept by ref_codegen) through the five calls the reference's
// ComputeUnit binds (ComputeUnit.cpp:146-167: init, run, setArg, getResult,
// finish), feeds it the workload's inputs and times it.  Test and baseline
// infrastructure only.
//
//   ref_run <gen_dir> <library> <warmup> <steps> [<results.bin>]
//
// <gen_dir> holds the table files (indexData, constData, outIndexData) and
// inputs.bin.  The plan sizes (numIndizes, argLength[], ...) are globals of
// the generated library and are read with dlsym.  Built with -DREF_CUDA for
// the CUDA path: run() is then also timed with CUDA events on the library's
// own stream (the global `stream`), with the L2 cleared by a 256 MiB write
// before every timed run.  Prints one JSON line; medians.
#include <dlfcn.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#ifdef REF_CUDA
#include <cuda_runtime.h>
#endif

namespace {

template <class T>
std::vector<T> readFile(const std::string& path, std::size_t count) {
    std::vector<T> v(count);
    std::ifstream f(path, std::ios::binary);
    if (count && !f.read(reinterpret_cast<char*>(v.data()), count * sizeof(T))) {
        std::fprintf(stderr, "ref_run: cannot read %zu values from %s\n", count, path.c_str());
        std::exit(2);
    }
    return v;
}

double now() { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); }

double median(std::vector<double> v) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    return v.size() % 2 ? v[v.size() / 2] : 0.5 * (v[v.size() / 2 - 1] + v[v.size() / 2]);
}

void* sym(void* h, const char* name) {
    void* p = dlsym(h, name);
    if (!p) {
        std::fprintf(stderr, "ref_run: symbol %s missing\n", name);
        std::exit(2);
    }
    return p;
}

#ifdef REF_CUDA
void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        std::fprintf(stderr, "ref_run: %s: %s\n", what, cudaGetErrorString(e));
        std::exit(3);
    }
}
#endif

}  // namespace

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: ref_run <gen_dir> <library> <warmup> <steps> [<results.bin>]\n");
        return 2;
    }
    const std::string dir = argv[1];
    const int warmup = std::atoi(argv[3]), steps = std::atoi(argv[4]);
    void* h = dlopen(argv[2], RTLD_NOW | RTLD_LOCAL);
    if (!h) {
        std::fprintf(stderr, "ref_run: %s\n", dlerror());
        return 2;
    }
    using InitF = void (*)(const unsigned*, const unsigned*, const double*);
    auto init = reinterpret_cast<InitF>(sym(h, "init"));
    auto run = reinterpret_cast<void (*)()>(sym(h, "run"));
    auto setArg = reinterpret_cast<void (*)(const double*, int)>(sym(h, "setArg"));
    auto getResult = reinterpret_cast<void (*)(double*, int)>(sym(h, "getResult"));
    const std::size_t numIndizes = *static_cast<std::size_t*>(sym(h, "numIndizes"));
    const std::size_t numConst = *static_cast<std::size_t*>(sym(h, "numConst"));
    const std::size_t numOutputValues = *static_cast<std::size_t*>(sym(h, "numOutputValues"));
    const std::size_t numOuts = *static_cast<std::size_t*>(sym(h, "numOuts"));
    const std::size_t numKernels = *static_cast<std::size_t*>(sym(h, "numKernels"));
    const std::size_t* argLength = static_cast<std::size_t*>(sym(h, "argLength"));
    const std::size_t* outLength = static_cast<std::size_t*>(sym(h, "outputIndexLength"));

    auto idx = readFile<unsigned>(dir + "/indexData", numIndizes);
    auto cst = readFile<double>(dir + "/constData", numConst);
    auto outIds = readFile<unsigned>(dir + "/outIndexData", numOutputValues);
    std::ifstream inf(dir + "/inputs.bin", std::ios::binary | std::ios::ate);
    const std::size_t inCount = static_cast<std::size_t>(inf.tellg()) / sizeof(double);
    auto in = readFile<double>(dir + "/inputs.bin", inCount);
    std::vector<const double*> args;
    std::size_t off = 0;
    for (int i = 0; off < inCount; ++i) {
        args.push_back(in.data() + off);
        off += argLength[i];
    }
    const double t0 = now();
    init(idx.data(), outIds.data(), cst.data());
    const double tInit = now() - t0;
    auto setArgs = [&] {
        for (std::size_t i = 0; i < args.size(); ++i) setArg(args[i], (int)i);
    };
    setArgs();
    for (int i = 0; i < warmup; ++i) run();

    std::vector<double> runS, execS, eventMs;
#ifdef REF_CUDA
    cudaStream_t stream = *static_cast<cudaStream_t*>(sym(h, "stream"));
    void* flush = nullptr;
    const std::size_t flushBytes = 256u << 20;
    check(cudaMalloc(&flush, flushBytes), "cudaMalloc");
    cudaEvent_t e0, e1;
    check(cudaEventCreate(&e0), "event");
    check(cudaEventCreate(&e1), "event");
    for (int i = 0; i < steps; ++i) {
        check(cudaMemsetAsync(flush, i & 0xff, flushBytes, stream), "memset");
        check(cudaStreamSynchronize(stream), "sync");
        check(cudaEventRecord(e0, stream), "record");
        const double t = now();
        run();  // launches every kernel and waits for the stream
        runS.push_back(now() - t);
        check(cudaEventRecord(e1, stream), "record");
        check(cudaEventSynchronize(e1), "sync");
        float ms = 0;
        check(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
        eventMs.push_back(ms);
    }
    check(cudaFree(flush), "cudaFree");
#else
    for (int i = 0; i < steps; ++i) {
        const double t = now();
        run();
        runS.push_back(now() - t);
    }
#endif
    for (int i = 0; i < steps; ++i) {
        const double t = now();
        setArgs();
        run();
        execS.push_back(now() - t);
    }
    std::vector<double> res;
    for (std::size_t k = 0; k < numOuts; ++k) {
        std::vector<double> r(outLength[k]);
        getResult(r.data(), (int)k);
        res.insert(res.end(), r.begin(), r.end());
    }
    if (argc > 5) {
        std::ofstream f(argv[5], std::ios::binary);
        f.write(reinterpret_cast<const char*>(res.data()), res.size() * sizeof(double));
    }
    std::printf("{\"kernels\": %zu, \"outputs\": %zu, \"init_s\": %.4f, \"run_ms\": %.6f, \"execute_ms\": %.6f",
                numKernels, res.size(), tInit, median(runS) * 1e3, median(execS) * 1e3);
#ifdef REF_CUDA
    std::printf(", \"run_event_ms\": %.6f", median(eventMs));
#endif
    std::printf(", \"steps\": %d, \"warmup\": %d}\n", steps, warmup);
    std::fflush(stdout);
    // The reference's finish() frees nothing on the CUDA path and its library
    // is never unloaded by the reference either.
    std::_Exit(0);
}
