// Run-time compilation of the compiled executor's modules: NVRTC for
// sm_103a, loaded with the runtime's library API (cudaLibraryLoadData), cached
// per process by source text and, when SYMGB_JIT_CACHE names a directory, on
// disk as cubin files keyed by a hash of the source and the options.
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "codegen.hpp"

namespace symgb {
namespace engine {

namespace {

const char* const kOptions[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-lineinfo", "--fmad=false"};

std::uint64_t fnv1a(const std::string& s, std::uint64_t h = 1469598103934665603ull) {
    for (unsigned char ch : s) {
        h ^= ch;
        h *= 1099511628211ull;
    }
    return h;
}

struct Entry {
    std::shared_ptr<JitModule> module;
    cudaLibrary_t library = nullptr;  // kept loaded until the process exits
};

std::mutex g_mutex;
std::map<std::string, Entry> g_cache;  // source text -> module

int compile(const std::string& source, std::vector<char>* cubin, std::string* err) {
    nvrtcProgram prog;
    nvrtcResult r = nvrtcCreateProgram(&prog, source.c_str(), "symgb_module.cu", 0, nullptr, nullptr);
    if (r != NVRTC_SUCCESS) {
        *err = std::string("nvrtcCreateProgram: ") + nvrtcGetErrorString(r);
        return SYMGB_ERR_ARGUMENT;
    }
    r = nvrtcCompileProgram(prog, (int)(sizeof kOptions / sizeof kOptions[0]), kOptions);
    if (r != NVRTC_SUCCESS) {
        std::size_t n = 0;
        nvrtcGetProgramLogSize(prog, &n);
        std::string log(n, '\0');
        if (n) nvrtcGetProgramLog(prog, &log[0]);
        if (log.size() > 2000) log.resize(2000);
        *err = std::string("NVRTC compilation failed: ") + nvrtcGetErrorString(r) + "\n" + log;
        nvrtcDestroyProgram(&prog);
        return SYMGB_ERR_ARGUMENT;
    }
    std::size_t n = 0;
    r = nvrtcGetCUBINSize(prog, &n);
    if (r == NVRTC_SUCCESS) {
        cubin->resize(n);
        r = nvrtcGetCUBIN(prog, cubin->data());
    }
    nvrtcDestroyProgram(&prog);
    if (r != NVRTC_SUCCESS) {
        *err = std::string("nvrtcGetCUBIN: ") + nvrtcGetErrorString(r);
        return SYMGB_ERR_ARGUMENT;
    }
    return SYMGB_OK;
}

std::string cachePath(const std::string& source) {
    const char* dir = std::getenv("SYMGB_JIT_CACHE");
    if (!dir || !*dir) return std::string();
    std::uint64_t h = fnv1a(source);
    for (const char* o : kOptions) h = fnv1a(o, h);
    char name[64];
    std::snprintf(name, sizeof name, "/symgb_%016llx.cubin", (unsigned long long)h);
    return std::string(dir) + name;
}

}  // namespace

int compileOnly(const std::string& source, double* seconds, std::string* err) {
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<char> cubin;
    const int e = compile(source, &cubin, err);
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return e;
}

int loadModule(const JitSource& src, std::shared_ptr<const JitModule>* out, std::string* err) {
    std::lock_guard<std::mutex> lock(g_mutex);
    auto it = g_cache.find(src.source);
    if (it != g_cache.end()) {
        *out = it->second.module;
        return SYMGB_OK;
    }
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<char> cubin;
    const std::string path = cachePath(src.source);
    if (!path.empty()) {
        std::ifstream f(path, std::ios::binary);
        if (f) cubin.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    }
    if (cubin.empty()) {
        if (int e = compile(src.source, &cubin, err)) return e;
        if (!path.empty()) {
            const std::string tmp = path + ".tmp" + std::to_string((unsigned long long)(std::uintptr_t)&cubin);
            std::ofstream f(tmp, std::ios::binary);
            f.write(cubin.data(), (std::streamsize)cubin.size());
            f.close();
            if (f) std::rename(tmp.c_str(), path.c_str());
        }
    }
    Entry e;
    cudaError_t ce = cudaLibraryLoadData(&e.library, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (ce != cudaSuccess) {
        *err = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(ce);
        return SYMGB_ERR_CUDA;
    }
    auto m = std::make_shared<JitModule>();
    m->launches = src.launches;
    m->grouped = src.grouped;
    m->direct = src.direct;
    for (const JitLaunch& L : src.launches) {
        cudaKernel_t k;
        ce = cudaLibraryGetKernel(&k, e.library, L.name.c_str());
        if (ce != cudaSuccess) {
            *err = "cudaLibraryGetKernel(" + L.name + "): " + cudaGetErrorString(ce);
            cudaLibraryUnload(e.library);
            return SYMGB_ERR_CUDA;
        }
        cudaFuncAttributes fa{};
        ce = cudaFuncGetAttributes(&fa, (const void*)k);
        if (ce != cudaSuccess) {
            *err = "cudaFuncGetAttributes(" + L.name + "): " + cudaGetErrorString(ce);
            cudaLibraryUnload(e.library);
            return SYMGB_ERR_CUDA;
        }
        m->kernels.push_back((const void*)k);
        m->registers.push_back(fa.numRegs);
    }
    m->compileSeconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    e.module = m;
    g_cache.emplace(src.source, e);
    *out = m;
    return SYMGB_OK;
}

}  // namespace engine
}  // namespace symgb
