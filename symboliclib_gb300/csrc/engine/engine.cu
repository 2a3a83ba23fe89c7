// Device engine: interpreter kernels for ComputeKernel programs, the unit
// runtime and the C ABI declared in include/symgb.h.
//
// Memory layout in HBM (one unit):
//   x   [num_total_memory][S] float64: inputs, then every kernel's output rows
//       in kernel order (reference numTotalMemory layout), value sets innermost
//       so that one gathered index serves S consecutive doubles;
//   p   uint32 index table, per kernel [row][instance] (reference positionData);
//   c   float64 constant table, per kernel [row][instance];
//   ids uint32 x slot of every output value, container order.
// A work item is (instance i, value set s), numbered w = i * S + s; thread
// blocks cover consecutive work items, so for S >= 32 a warp shares one
// instance and its index loads are broadcasts, and for S = 1 a warp covers 32
// consecutive instances and its index loads are one coalesced 128-byte line.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "program.hpp"
#include "symgb.h"

using symgb::engine::Program;

namespace {

thread_local std::string g_lastError;

int fail(int code, const std::string& msg) {
    g_lastError = msg;
    return code;
}

#define SYMGB_CUDA(call)                                                                            \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return fail(e_ == cudaErrorMemoryAllocation ? SYMGB_ERR_NOMEM : SYMGB_ERR_CUDA,        \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                        \
    } while (0)

// ------------------------------------------------------------------ device side

struct DevKernel {
    const std::uint64_t* prog;  // device program
    const std::uint32_t* p;     // index table of this kernel
    const double* c;            // constant table of this kernel
    std::uint64_t yoff;         // first x slot written by this kernel
    std::uint64_t n;            // instances
    std::uint32_t regs;         // register-file slots used
    std::uint32_t pad;
};

struct Tile {
    std::uint32_t kernel;
    std::uint32_t count;   // work items in this tile
    std::uint64_t start;   // first work item
};

struct BarrierState {
    unsigned int count;
    unsigned int generation;
    int error;  // set by a block whose wait timed out
    int pad;
};

enum : int { LOAD_CACHED = 0, LOAD_L2 = 1 };

template <int LOAD>
__device__ __forceinline__ double loadX(const double* a) {
    if (LOAD == LOAD_L2) return __ldcg(a);
    return __ldg(a);
}

__device__ __forceinline__ double dfma(double a, double b, double c, int flags) {
    if (flags & symgb::engine::FMA_NEG_PRODUCT) a = -a;
    if (flags & symgb::engine::FMA_NEG_ADDEND) c = -c;
    return __fma_rn(a, b, c);
}

// Executes one program for one work item.  R points at this thread's first
// register; registers are `stride` doubles apart (one shared-memory column per
// thread, so a warp's register access is conflict-free).
template <int LOAD>
__device__ __forceinline__ void runProgram(const std::uint64_t* __restrict__ prog, double* R, unsigned stride,
                                           const double* x, double* xw, const std::uint32_t* __restrict__ p,
                                           const double* __restrict__ c, std::uint64_t n, std::uint64_t i,
                                           std::uint64_t yoff, unsigned S, unsigned s) {
    using namespace symgb::engine;
#define REG(k) R[(unsigned)(k) * stride]
    for (const std::uint64_t* ip = prog;;) {
        const std::uint64_t w = *ip++;
        const unsigned op = (unsigned)(w & 0xff);
        const unsigned d = (unsigned)(w >> 8) & 0xff;
        const unsigned a = (unsigned)(w >> 16) & 0xff;
        const unsigned b = (unsigned)(w >> 24) & 0xff;
        switch (op) {
            case OP_END: return;
            case OP_LDX: {
                const unsigned row = (unsigned)(w >> 16) & 0xffff;
                const int off = (int)(unsigned)(w >> 32);
                const std::uint64_t slot = (std::uint64_t)((long long)__ldg(p + row * n + i) + off);
                REG(d) = loadX<LOAD>(x + slot * S + s);
                break;
            }
            case OP_LDC: REG(d) = __ldg(c + (std::uint64_t)(unsigned)(w >> 32) * n + i); break;
            case OP_LDK: REG(d) = __longlong_as_double((long long)*ip++); break;
            case OP_ST: xw[(yoff + (std::uint64_t)(unsigned)(w >> 32) * n + i) * S + s] = REG(a); break;
            case OP_ADD: REG(d) = __dadd_rn(REG(a), REG(b)); break;
            case OP_SUB: REG(d) = __dsub_rn(REG(a), REG(b)); break;
            case OP_MUL: REG(d) = __dmul_rn(REG(a), REG(b)); break;
            case OP_DIV: REG(d) = __ddiv_rn(REG(a), REG(b)); break;
            case OP_NEG: REG(d) = -REG(a); break;
            case OP_SQRT: REG(d) = __dsqrt_rn(REG(a)); break;
            case OP_REC: REG(d) = __ddiv_rn(1.0, REG(a)); break;
            case OP_FMA: {
                const unsigned cr = (unsigned)(w >> 32) & 0xff;
                const int fl = (int)((w >> 40) & 0x3);
                REG(d) = dfma(REG(a), REG(b), REG(cr), fl);
                break;
            }
            case OP_MOV: REG(d) = REG(a); break;
            case OP_SIN: REG(d) = sin(REG(a)); break;
            case OP_COS: REG(d) = cos(REG(a)); break;
            case OP_TAN: REG(d) = tan(REG(a)); break;
            case OP_ASIN: REG(d) = asin(REG(a)); break;
            case OP_ACOS: REG(d) = acos(REG(a)); break;
            case OP_ATAN: REG(d) = atan(REG(a)); break;
            case OP_EXP: REG(d) = exp(REG(a)); break;
            case OP_LOG: REG(d) = log(REG(a)); break;
            case OP_POW: REG(d) = pow(REG(a), REG(b)); break;
            default: return;
        }
    }
#undef REG
}

// One launch per ComputeKernel (the reference's K(i) launch shape).
__global__ void plainKernel(DevKernel k, const double* x, double* xw, unsigned S) {
    extern __shared__ double regs[];
    const std::uint64_t w = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= k.n * S) return;
    const std::uint64_t i = w / S;
    const unsigned s = (unsigned)(w - i * S);
    runProgram<LOAD_CACHED>(k.prog, regs + threadIdx.x, blockDim.x, x, xw, k.p, k.c, k.n, i, k.yoff, S, s);
}

__device__ __forceinline__ unsigned long long globalTimerNs() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier for a cooperative launch.  The wait is bounded: after
// `timeoutNs` the waiting block records SYMGB_ERR_TIMEOUT in bar->error and in
// the host-mapped flag `hostError`, and leaves.  Every block checks bar->error
// after each barrier and returns when it is set.
__device__ bool gridBarrier(BarrierState* bar, int* hostError, unsigned long long timeoutNs) {
    __syncthreads();
    __shared__ int failed;
    if (threadIdx.x == 0) {
        volatile unsigned int* gen = &bar->generation;
        volatile int* err = &bar->error;
        const unsigned int g = *gen;
        __threadfence();
        if (atomicAdd(&bar->count, 1u) == gridDim.x - 1) {
            atomicExch(&bar->count, 0u);
            __threadfence();
            atomicAdd(&bar->generation, 1u);
        } else {
            const unsigned long long t0 = globalTimerNs();
            while (*gen == g) {
                if (*err) break;
                if (globalTimerNs() - t0 > timeoutNs) {
                    atomicExch(&bar->error, SYMGB_ERR_TIMEOUT);
                    *(volatile int*)hostError = SYMGB_ERR_TIMEOUT;
                    break;
                }
                __nanosleep(100);
            }
        }
        __threadfence();
        failed = *err != 0;
    }
    __syncthreads();
    return !failed;
}

// Tiles of all kernels of levels [levelBegin, levelEnd); levels separated by a
// grid barrier when the range holds more than one level.
template <int LOAD>
__global__ void fusedKernel(const DevKernel* __restrict__ ks, const Tile* __restrict__ tiles,
                            const std::uint32_t* __restrict__ levelTiles, int levelBegin, int levelEnd,
                            const double* x, double* xw, unsigned S, BarrierState* bar, int* hostError,
                            unsigned long long timeoutNs) {
    extern __shared__ double regs[];
    for (int L = levelBegin; L < levelEnd; ++L) {
        const std::uint32_t t0 = levelTiles[L], t1 = levelTiles[L + 1];
        for (std::uint32_t t = t0 + blockIdx.x; t < t1; t += gridDim.x) {
            const Tile tile = tiles[t];
            const DevKernel k = ks[tile.kernel];
            for (unsigned j = threadIdx.x; j < tile.count; j += blockDim.x) {
                const std::uint64_t w = tile.start + j;
                const std::uint64_t i = w / S;
                const unsigned s = (unsigned)(w - i * S);
                runProgram<LOAD>(k.prog, regs + threadIdx.x, blockDim.x, x, xw, k.p, k.c, k.n, i, k.yoff, S, s);
            }
        }
        if (L + 1 < levelEnd)
            if (!gridBarrier(bar, hostError, timeoutNs)) return;
    }
}

// out[s * len + j] = x[ids[j] * S + s]  (reference gatherResult, per value set)
__global__ void gatherKernel(const double* __restrict__ x, const std::uint32_t* __restrict__ ids, std::uint64_t len,
                             unsigned S, double* __restrict__ out) {
    const std::uint64_t w = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= len * S) return;
    const std::uint64_t j = w / S;
    const unsigned s = (unsigned)(w - j * S);
    out[(std::uint64_t)s * len + j] = __ldg(x + (std::uint64_t)__ldg(ids + j) * S + s);
}

// x[(start + j) * S + s] = in[s * len + j]
__global__ void scatterKernel(const double* __restrict__ in, std::uint64_t start, std::uint64_t len, unsigned S,
                              double* __restrict__ x) {
    const std::uint64_t w = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= len * S) return;
    const std::uint64_t j = w / S;
    const unsigned s = (unsigned)(w - j * S);
    x[(start + j) * S + s] = __ldg(in + (std::uint64_t)s * len + j);
}

// ------------------------------------------------------------------ host side

struct HostKernel {
    symgb_kernel_desc desc;
    std::vector<symgb_node> nodes;
    std::vector<std::int32_t> access;
    Program prog[2];  // exact, fast
};

template <class T>
struct DevBuf {
    T* ptr = nullptr;
    std::size_t count = 0;
    ~DevBuf() { reset(); }
    void reset() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        count = 0;
    }
    cudaError_t alloc(std::size_t n) {
        reset();
        if (n == 0) n = 1;
        cudaError_t e = cudaMalloc(&ptr, n * sizeof(T));
        if (e == cudaSuccess) count = n;
        return e;
    }
};

}  // namespace

struct symgb_unit {
    // plan
    std::vector<HostKernel> kernels;
    std::vector<std::uint64_t> argStart, argLength, outStart, outLength;
    std::uint64_t numTotalMemory = 0, numIndices = 0, numOutputValues = 0, numConstants = 0;
    int threadsPerBlock = 128;
    int numLevels = 0;
    symgb_schedule sched{SYMGB_SCHEDULE_PLAIN, SYMGB_MATH_FAST, 0, 0, 0, 0};
    int numSets = 1;

    // device state
    bool initialized = false;
    int device = 0;
    int smCount = 0;
    cudaStream_t ownStream = nullptr, stream = nullptr;
    DevBuf<double> x, c, staging, outBuf;
    DevBuf<std::uint32_t> p, ids;
    DevBuf<std::uint64_t> progs;
    DevBuf<DevKernel> devKernels;
    DevBuf<Tile> tiles;
    DevBuf<std::uint32_t> levelTiles;
    DevBuf<BarrierState> barrier;
    int* errorHost = nullptr;  // mapped pinned flag written by the device
    int* errorDev = nullptr;
    std::vector<DevKernel> hostDevKernels;
    std::vector<std::uint32_t> hostLevelTiles;
    std::vector<Tile> hostTiles;
    std::vector<int> kernelOrderByLevel;
    std::size_t tilesFor = 0;  // configuration the tile table was built for
    int tilesSets = -1, tilesItems = -1, tilesMath = -1;
    cudaGraphExec_t graph = nullptr;
    bool graphValid = false;
    int lastLaunches = 0;
    int launchesPerRun = 0;
    unsigned long long barrierTimeoutNs = 2000000000ull;

    ~symgb_unit() { release(); }

    void dropGraph() {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
        graphValid = false;
    }

    void release() {
        dropGraph();
        x.reset();
        c.reset();
        staging.reset();
        outBuf.reset();
        p.reset();
        ids.reset();
        progs.reset();
        devKernels.reset();
        tiles.reset();
        levelTiles.reset();
        barrier.reset();
        if (errorHost) cudaFreeHost(errorHost);
        errorHost = nullptr;
        errorDev = nullptr;
        if (ownStream) cudaStreamDestroy(ownStream);
        ownStream = nullptr;
        stream = nullptr;
        initialized = false;
    }

    int mathIndex() const { return sched.math == SYMGB_MATH_EXACT ? 0 : 1; }
    int tpb() const { return sched.threads_per_block > 0 ? sched.threads_per_block : threadsPerBlock; }
};

namespace {

int uploadPrograms(symgb_unit* u) {
    const int mi = u->mathIndex();
    std::vector<std::uint64_t> all;
    std::vector<std::size_t> offs;
    for (auto& k : u->kernels) {
        offs.push_back(all.size());
        all.insert(all.end(), k.prog[mi].words.begin(), k.prog[mi].words.end());
    }
    SYMGB_CUDA(u->progs.alloc(all.size()));
    SYMGB_CUDA(cudaMemcpy(u->progs.ptr, all.data(), all.size() * 8, cudaMemcpyHostToDevice));
    u->hostDevKernels.clear();
    for (std::size_t k = 0; k < u->kernels.size(); ++k) {
        const auto& d = u->kernels[k].desc;
        DevKernel dk;
        dk.prog = u->progs.ptr + offs[k];
        dk.p = u->p.ptr + d.index_offset;
        dk.c = u->c.ptr + d.constants_offset;
        dk.yoff = d.output_offset;
        dk.n = d.num_instances;
        dk.regs = (std::uint32_t)std::max(1, u->kernels[k].prog[mi].registers);
        dk.pad = 0;
        u->hostDevKernels.push_back(dk);
    }
    SYMGB_CUDA(u->devKernels.alloc(u->hostDevKernels.size()));
    SYMGB_CUDA(cudaMemcpy(u->devKernels.ptr, u->hostDevKernels.data(), u->hostDevKernels.size() * sizeof(DevKernel),
                          cudaMemcpyHostToDevice));
    u->dropGraph();
    u->tilesSets = -1;
    return SYMGB_OK;
}

// Tile table for the fused schedules: per level, every kernel's work items cut
// into tiles of `items` consecutive work items.
int buildTiles(symgb_unit* u) {
    const int S = u->numSets;
    int items = u->sched.items_per_tile > 0 ? u->sched.items_per_tile : 2 * u->tpb();
    if (u->tilesSets == S && u->tilesItems == items && u->tilesMath == u->mathIndex()) return SYMGB_OK;
    u->hostTiles.clear();
    u->hostLevelTiles.assign(1, 0);
    for (int L = 0; L < u->numLevels; ++L) {
        for (std::size_t k = 0; k < u->kernels.size(); ++k) {
            if (u->kernels[k].desc.level != L) continue;
            const std::uint64_t total = u->kernels[k].desc.num_instances * (std::uint64_t)S;
            for (std::uint64_t st = 0; st < total; st += items)
                u->hostTiles.push_back({(std::uint32_t)k, (std::uint32_t)std::min<std::uint64_t>(items, total - st), st});
        }
        u->hostLevelTiles.push_back((std::uint32_t)u->hostTiles.size());
    }
    SYMGB_CUDA(u->tiles.alloc(u->hostTiles.size()));
    if (!u->hostTiles.empty())
        SYMGB_CUDA(cudaMemcpy(u->tiles.ptr, u->hostTiles.data(), u->hostTiles.size() * sizeof(Tile), cudaMemcpyHostToDevice));
    SYMGB_CUDA(u->levelTiles.alloc(u->hostLevelTiles.size()));
    SYMGB_CUDA(cudaMemcpy(u->levelTiles.ptr, u->hostLevelTiles.data(), u->hostLevelTiles.size() * 4, cudaMemcpyHostToDevice));
    u->tilesSets = S;
    u->tilesItems = items;
    u->tilesMath = u->mathIndex();
    return SYMGB_OK;
}

std::size_t regBytes(const symgb_unit* u, int kbegin, int kend, int tpb, int level = -1) {
    std::uint32_t r = 1;
    for (int k = kbegin; k < kend; ++k)
        if (level < 0 || u->kernels[k].desc.level == level) r = std::max(r, u->hostDevKernels[k].regs);
    return (std::size_t)r * tpb * sizeof(double);
}

int setSmemLimit(const void* fn, std::size_t bytes) {
    if (bytes > 48 * 1024) SYMGB_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return SYMGB_OK;
}

// Enqueues one evaluation on the unit's stream.
int enqueueRun(symgb_unit* u) {
    const unsigned S = (unsigned)u->numSets;
    const int tpb = u->tpb();
    int launches = 0;
    switch (u->sched.kind) {
        case SYMGB_SCHEDULE_PLAIN: {
            for (std::size_t k = 0; k < u->kernels.size(); ++k) {
                const DevKernel& dk = u->hostDevKernels[k];
                const std::uint64_t work = dk.n * S;
                if (work == 0) continue;
                const std::size_t smem = (std::size_t)dk.regs * tpb * sizeof(double);
                if (setSmemLimit((const void*)plainKernel, smem)) return SYMGB_ERR_CUDA;
                const unsigned grid = (unsigned)((work + tpb - 1) / tpb);
                plainKernel<<<grid, tpb, smem, u->stream>>>(dk, u->x.ptr, u->x.ptr, S);
                ++launches;
            }
            break;
        }
        case SYMGB_SCHEDULE_LEVELS: {
            if (int e = buildTiles(u)) return e;
            for (int L = 0; L < u->numLevels; ++L) {
                const std::uint32_t nt = u->hostLevelTiles[L + 1] - u->hostLevelTiles[L];
                if (!nt) continue;
                const std::size_t smem = regBytes(u, 0, (int)u->kernels.size(), tpb, L);
                if (setSmemLimit((const void*)fusedKernel<LOAD_CACHED>, smem)) return SYMGB_ERR_CUDA;
                fusedKernel<LOAD_CACHED><<<nt, tpb, smem, u->stream>>>(u->devKernels.ptr, u->tiles.ptr, u->levelTiles.ptr, L,
                                                                      L + 1, u->x.ptr, u->x.ptr, S, u->barrier.ptr,
                                                                      u->errorDev, u->barrierTimeoutNs);
                ++launches;
            }
            break;
        }
        case SYMGB_SCHEDULE_PERSISTENT: {
            if (int e = buildTiles(u)) return e;
            const std::size_t smem = regBytes(u, 0, (int)u->kernels.size(), tpb);
            const void* fn = (const void*)fusedKernel<LOAD_L2>;
            if (setSmemLimit(fn, smem)) return SYMGB_ERR_CUDA;
            int perSm = 0;
            SYMGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, fusedKernel<LOAD_L2>, tpb, smem));
            if (perSm < 1) return fail(SYMGB_ERR_ARGUMENT, "persistent schedule: register file does not fit on an SM");
            if (u->sched.blocks_per_sm > 0) perSm = std::min(perSm, u->sched.blocks_per_sm);
            unsigned grid = (unsigned)(perSm * u->smCount);
            std::uint32_t maxTiles = 0;
            for (int L = 0; L < u->numLevels; ++L)
                maxTiles = std::max(maxTiles, u->hostLevelTiles[L + 1] - u->hostLevelTiles[L]);
            grid = std::max(1u, std::min<unsigned>(grid, maxTiles));
            const DevKernel* ks = u->devKernels.ptr;
            const Tile* tl = u->tiles.ptr;
            const std::uint32_t* lt = u->levelTiles.ptr;
            int lb = 0, le = u->numLevels;
            const double* xr = u->x.ptr;
            double* xw = u->x.ptr;
            BarrierState* bar = u->barrier.ptr;
            int* err = u->errorDev;
            unsigned long long to = u->barrierTimeoutNs;
            void* args[] = {(void*)&ks, (void*)&tl, (void*)&lt, (void*)&lb, (void*)&le, (void*)&xr,
                            (void*)&xw, (void*)&S, (void*)&bar, (void*)&err, (void*)&to};
            SYMGB_CUDA(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(tpb), args, smem, u->stream));
            ++launches;
            break;
        }
        default: return fail(SYMGB_ERR_ARGUMENT, "unknown schedule kind");
    }
    SYMGB_CUDA(cudaGetLastError());
    u->launchesPerRun = launches;
    return SYMGB_OK;
}

int runAsync(symgb_unit* u) {
    if (!u->initialized) return fail(SYMGB_ERR_STATE, "run before init");
    if (u->sched.use_graph && u->sched.kind != SYMGB_SCHEDULE_PERSISTENT) {
        if (!u->graphValid) {
            if (u->sched.kind != SYMGB_SCHEDULE_PLAIN)
                if (int e = buildTiles(u)) return e;
            // smem attributes must be set outside capture
            cudaGraph_t g;
            SYMGB_CUDA(cudaStreamBeginCapture(u->stream, cudaStreamCaptureModeThreadLocal));
            int e = enqueueRun(u);
            cudaError_t ce = cudaStreamEndCapture(u->stream, &g);
            if (e) return e;
            if (ce != cudaSuccess) return fail(SYMGB_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
            SYMGB_CUDA(cudaGraphInstantiate(&u->graph, g, 0));
            cudaGraphDestroy(g);
            u->graphValid = true;
        }
        SYMGB_CUDA(cudaGraphLaunch(u->graph, u->stream));
        u->lastLaunches = u->launchesPerRun;
        return SYMGB_OK;
    }
    int e = enqueueRun(u);
    u->lastLaunches = u->launchesPerRun;
    return e;
}

int checkDeviceError(symgb_unit* u) {
    if (u->errorHost && *(volatile int*)u->errorHost) {
        const int code = *(volatile int*)u->errorHost;
        *(volatile int*)u->errorHost = 0;
        cudaMemset(u->barrier.ptr, 0, sizeof(BarrierState));
        return fail(code, "device-side wait timed out (grid barrier)");
    }
    return SYMGB_OK;
}

int copyDesc(symgb_unit* u, const symgb_plan_desc* d) {
    if (!d || (d->num_kernels && !d->kernels)) return fail(SYMGB_ERR_ARGUMENT, "null plan");
    u->kernels.resize(d->num_kernels);
    int maxLevel = -1;
    for (std::uint32_t k = 0; k < d->num_kernels; ++k) {
        HostKernel& hk = u->kernels[k];
        hk.desc = d->kernels[k];
        hk.nodes.assign(d->kernels[k].nodes, d->kernels[k].nodes + d->kernels[k].num_nodes);
        hk.access.assign(d->kernels[k].access, d->kernels[k].access + 2 * (std::size_t)d->kernels[k].num_access);
        hk.desc.nodes = hk.nodes.data();
        hk.desc.access = hk.access.data();
        if (hk.desc.level < 0) return fail(SYMGB_ERR_ARGUMENT, "negative kernel level");
        maxLevel = std::max(maxLevel, hk.desc.level);
        // Bounds of everything the kernel touches, checked once on the host.
        const std::uint64_t n = hk.desc.num_instances;
        if (hk.desc.output_offset + n * hk.desc.num_output_rows > d->num_total_memory)
            return fail(SYMGB_ERR_ARGUMENT, "kernel output rows exceed x");
        if (hk.desc.index_offset + n * hk.desc.num_index_rows > d->num_indices)
            return fail(SYMGB_ERR_ARGUMENT, "kernel index rows exceed the index table");
        if (hk.desc.constants_offset + n * hk.desc.num_constant_rows > d->num_constants)
            return fail(SYMGB_ERR_ARGUMENT, "kernel constant rows exceed the constant table");
        try {
            hk.prog[0] = symgb::engine::compileTemplate(hk.desc, SYMGB_MATH_EXACT);
            hk.prog[1] = symgb::engine::compileTemplate(hk.desc, SYMGB_MATH_FAST);
        } catch (const std::exception& ex) {
            return fail(SYMGB_ERR_ARGUMENT, std::string("kernel ") + std::to_string(k) + ": " + ex.what());
        }
    }
    u->numLevels = maxLevel + 1;
    u->argStart.assign(d->arg_start, d->arg_start + d->num_args);
    u->argLength.assign(d->arg_length, d->arg_length + d->num_args);
    u->outStart.assign(d->output_start, d->output_start + d->num_outputs);
    u->outLength.assign(d->output_length, d->output_length + d->num_outputs);
    for (std::uint32_t a = 0; a < d->num_args; ++a)
        if (u->argStart[a] + u->argLength[a] > d->num_total_memory) return fail(SYMGB_ERR_ARGUMENT, "input exceeds x");
    for (std::uint32_t o = 0; o < d->num_outputs; ++o)
        if (u->outStart[o] + u->outLength[o] > d->num_output_values) return fail(SYMGB_ERR_ARGUMENT, "output range exceeds ids");
    u->numTotalMemory = d->num_total_memory;
    u->numIndices = d->num_indices;
    u->numOutputValues = d->num_output_values;
    u->numConstants = d->num_constants;
    u->threadsPerBlock = d->threads_per_block ? (int)d->threads_per_block : 128;
    return SYMGB_OK;
}

}  // namespace

extern "C" {

const char* symgb_last_error(void) { return g_lastError.c_str(); }

int symgb_unit_create(const symgb_plan_desc* plan, symgb_unit_t* out) {
    if (!out) return fail(SYMGB_ERR_ARGUMENT, "null output handle");
    *out = nullptr;
    std::unique_ptr<symgb_unit> u(new symgb_unit());
    if (int e = copyDesc(u.get(), plan)) return e;
    *out = u.release();
    return SYMGB_OK;
}

int symgb_init(symgb_unit_t u, const uint32_t* index_data, const uint32_t* out_index_data, const double* const_data) {
    if (!u) return fail(SYMGB_ERR_ARGUMENT, "null unit");
    if ((u->numIndices && !index_data) || (u->numOutputValues && !out_index_data) || (u->numConstants && !const_data))
        return fail(SYMGB_ERR_ARGUMENT, "null table");
    // Every index must address x; checked once here so the kernels need no bounds checks.
    for (const auto& k : u->kernels) {
        const auto& d = k.desc;
        for (std::uint32_t a = 0; a < d.num_access; ++a) {
            const std::uint32_t row = (std::uint32_t)k.access[2 * a];
            const long long off = k.access[2 * a + 1];
            const std::uint32_t* pr = index_data + d.index_offset + (std::uint64_t)row * d.num_instances;
            for (std::uint64_t i = 0; i < d.num_instances; ++i) {
                const long long slot = (long long)pr[i] + off;
                if (slot < 0 || (std::uint64_t)slot >= u->numTotalMemory)
                    return fail(SYMGB_ERR_ARGUMENT, "index table entry outside x");
            }
        }
    }
    for (std::uint64_t j = 0; j < u->numOutputValues; ++j)
        if (out_index_data[j] >= u->numTotalMemory) return fail(SYMGB_ERR_ARGUMENT, "output id outside x");
    u->release();
    SYMGB_CUDA(cudaGetDevice(&u->device));
    SYMGB_CUDA(cudaDeviceGetAttribute(&u->smCount, cudaDevAttrMultiProcessorCount, u->device));
    SYMGB_CUDA(cudaStreamCreateWithFlags(&u->ownStream, cudaStreamNonBlocking));
    u->stream = u->ownStream;
    SYMGB_CUDA(u->x.alloc(u->numTotalMemory * (std::size_t)u->numSets));
    SYMGB_CUDA(cudaMemset(u->x.ptr, 0, u->x.count * sizeof(double)));
    SYMGB_CUDA(u->p.alloc(u->numIndices));
    if (u->numIndices) SYMGB_CUDA(cudaMemcpy(u->p.ptr, index_data, u->numIndices * 4, cudaMemcpyHostToDevice));
    SYMGB_CUDA(u->c.alloc(u->numConstants));
    if (u->numConstants) SYMGB_CUDA(cudaMemcpy(u->c.ptr, const_data, u->numConstants * 8, cudaMemcpyHostToDevice));
    SYMGB_CUDA(u->ids.alloc(u->numOutputValues));
    if (u->numOutputValues)
        SYMGB_CUDA(cudaMemcpy(u->ids.ptr, out_index_data, u->numOutputValues * 4, cudaMemcpyHostToDevice));
    SYMGB_CUDA(u->barrier.alloc(1));
    SYMGB_CUDA(cudaMemset(u->barrier.ptr, 0, sizeof(BarrierState)));
    SYMGB_CUDA(cudaHostAlloc((void**)&u->errorHost, sizeof(int), cudaHostAllocMapped));
    *u->errorHost = 0;
    SYMGB_CUDA(cudaHostGetDevicePointer((void**)&u->errorDev, u->errorHost, 0));
    if (int e = uploadPrograms(u)) return e;
    u->initialized = true;
    return SYMGB_OK;
}

int symgb_set_arg(symgb_unit_t u, const double* d, int i) {
    if (!u || !u->initialized) return fail(SYMGB_ERR_STATE, "set_arg before init");
    if (i < 0 || (std::size_t)i >= u->argStart.size() || !d) return fail(SYMGB_ERR_ARGUMENT, "bad argument index");
    if (u->numSets != 1) return symgb_set_arg_sets(u, d, i);
    SYMGB_CUDA(cudaMemcpyAsync(u->x.ptr + u->argStart[i], d, u->argLength[i] * 8, cudaMemcpyHostToDevice, u->stream));
    SYMGB_CUDA(cudaStreamSynchronize(u->stream));
    return SYMGB_OK;
}

int symgb_run(symgb_unit_t u) {
    if (!u) return fail(SYMGB_ERR_ARGUMENT, "null unit");
    if (int e = runAsync(u)) return e;
    SYMGB_CUDA(cudaStreamSynchronize(u->stream));
    return checkDeviceError(u);
}

int symgb_run_async(symgb_unit_t u) {
    if (!u) return fail(SYMGB_ERR_ARGUMENT, "null unit");
    return runAsync(u);
}

int symgb_synchronize(symgb_unit_t u) {
    if (!u || !u->initialized) return fail(SYMGB_ERR_STATE, "synchronize before init");
    SYMGB_CUDA(cudaStreamSynchronize(u->stream));
    return checkDeviceError(u);
}

static int ensureOutBuf(symgb_unit* u, std::size_t n) {
    if (u->outBuf.count < n) SYMGB_CUDA(u->outBuf.alloc(n));
    return SYMGB_OK;
}

int symgb_get_result_sets_device(symgb_unit_t u, double* d, int k) {
    if (!u || !u->initialized) return fail(SYMGB_ERR_STATE, "get_result before init");
    if (k < 0 || (std::size_t)k >= u->outStart.size() || !d) return fail(SYMGB_ERR_ARGUMENT, "bad result index");
    const std::uint64_t len = u->outLength[k];
    const std::uint64_t work = len * u->numSets;
    if (work) {
        gatherKernel<<<(unsigned)((work + 255) / 256), 256, 0, u->stream>>>(u->x.ptr, u->ids.ptr + u->outStart[k], len,
                                                                            (unsigned)u->numSets, d);
        SYMGB_CUDA(cudaGetLastError());
    }
    return SYMGB_OK;
}

int symgb_get_result_sets(symgb_unit_t u, double* d, int k) {
    if (!u || !u->initialized) return fail(SYMGB_ERR_STATE, "get_result before init");
    if (k < 0 || (std::size_t)k >= u->outStart.size() || !d) return fail(SYMGB_ERR_ARGUMENT, "bad result index");
    const std::size_t n = u->outLength[k] * (std::size_t)u->numSets;
    if (int e = ensureOutBuf(u, n)) return e;
    if (int e = symgb_get_result_sets_device(u, u->outBuf.ptr, k)) return e;
    SYMGB_CUDA(cudaMemcpyAsync(d, u->outBuf.ptr, n * 8, cudaMemcpyDeviceToHost, u->stream));
    SYMGB_CUDA(cudaStreamSynchronize(u->stream));
    return checkDeviceError(u);
}

int symgb_get_result(symgb_unit_t u, double* d, int k) { return symgb_get_result_sets(u, d, k); }

int symgb_set_arg_sets_device(symgb_unit_t u, const double* d, int i) {
    if (!u || !u->initialized) return fail(SYMGB_ERR_STATE, "set_arg before init");
    if (i < 0 || (std::size_t)i >= u->argStart.size() || !d) return fail(SYMGB_ERR_ARGUMENT, "bad argument index");
    const std::uint64_t len = u->argLength[i];
    if (u->numSets == 1) {
        SYMGB_CUDA(cudaMemcpyAsync(u->x.ptr + u->argStart[i], d, len * 8, cudaMemcpyDeviceToDevice, u->stream));
        return SYMGB_OK;
    }
    const std::uint64_t work = len * u->numSets;
    if (work) {
        scatterKernel<<<(unsigned)((work + 255) / 256), 256, 0, u->stream>>>(d, u->argStart[i], len, (unsigned)u->numSets,
                                                                             u->x.ptr);
        SYMGB_CUDA(cudaGetLastError());
    }
    return SYMGB_OK;
}

int symgb_set_arg_sets(symgb_unit_t u, const double* d, int i) {
    if (!u || !u->initialized) return fail(SYMGB_ERR_STATE, "set_arg before init");
    if (i < 0 || (std::size_t)i >= u->argStart.size() || !d) return fail(SYMGB_ERR_ARGUMENT, "bad argument index");
    const std::size_t n = u->argLength[i] * (std::size_t)u->numSets;
    if (u->numSets == 1) {
        SYMGB_CUDA(cudaMemcpyAsync(u->x.ptr + u->argStart[i], d, n * 8, cudaMemcpyHostToDevice, u->stream));
    } else {
        if (u->staging.count < n) SYMGB_CUDA(u->staging.alloc(n));
        SYMGB_CUDA(cudaMemcpyAsync(u->staging.ptr, d, n * 8, cudaMemcpyHostToDevice, u->stream));
        if (int e = symgb_set_arg_sets_device(u, u->staging.ptr, i)) return e;
    }
    SYMGB_CUDA(cudaStreamSynchronize(u->stream));
    return SYMGB_OK;
}

int symgb_finish(symgb_unit_t u) {
    if (!u) return fail(SYMGB_ERR_ARGUMENT, "null unit");
    if (u->initialized) cudaStreamSynchronize(u->stream);
    u->release();
    return SYMGB_OK;
}

void symgb_unit_destroy(symgb_unit_t u) {
    if (!u) return;
    if (u->initialized) cudaStreamSynchronize(u->stream);
    delete u;
}

int symgb_set_schedule(symgb_unit_t u, const symgb_schedule* s) {
    if (!u || !s) return fail(SYMGB_ERR_ARGUMENT, "null argument");
    if (s->kind < 0 || s->kind > 2 || s->math < 0 || s->math > 1) return fail(SYMGB_ERR_ARGUMENT, "bad schedule");
    if (s->threads_per_block < 0 || s->threads_per_block > 1024 || (s->threads_per_block % 32))
        return fail(SYMGB_ERR_ARGUMENT, "threads_per_block must be a multiple of 32 up to 1024");
    const bool mathChanged = s->math != u->sched.math;
    u->sched = *s;
    u->dropGraph();
    u->tilesSets = -1;
    if (mathChanged && u->initialized) return uploadPrograms(u);
    return SYMGB_OK;
}

int symgb_get_schedule(symgb_unit_t u, symgb_schedule* s) {
    if (!u || !s) return fail(SYMGB_ERR_ARGUMENT, "null argument");
    *s = u->sched;
    return SYMGB_OK;
}

int symgb_set_num_sets(symgb_unit_t u, int num_sets) {
    if (!u || num_sets < 1) return fail(SYMGB_ERR_ARGUMENT, "num_sets must be >= 1");
    if (num_sets == u->numSets) return SYMGB_OK;
    u->numSets = num_sets;
    u->dropGraph();
    u->tilesSets = -1;
    if (u->initialized) {
        SYMGB_CUDA(cudaStreamSynchronize(u->stream));
        SYMGB_CUDA(u->x.alloc(u->numTotalMemory * (std::size_t)num_sets));
        SYMGB_CUDA(cudaMemset(u->x.ptr, 0, u->x.count * sizeof(double)));
    }
    return SYMGB_OK;
}

int symgb_num_sets(symgb_unit_t u) { return u ? u->numSets : 0; }

int symgb_set_stream(symgb_unit_t u, void* stream) {
    if (!u || !u->initialized) return fail(SYMGB_ERR_STATE, "set_stream before init");
    u->stream = stream ? (cudaStream_t)stream : u->ownStream;
    u->dropGraph();
    return SYMGB_OK;
}

int symgb_get_stats(symgb_unit_t u, symgb_stats* s) {
    if (!u || !s) return fail(SYMGB_ERR_ARGUMENT, "null argument");
    std::memset(s, 0, sizeof(*s));
    s->num_kernels = u->kernels.size();
    s->num_levels = (std::uint64_t)u->numLevels;
    for (auto l : u->argLength) s->num_inputs += l;
    s->num_outputs = u->numOutputValues;
    std::uint64_t slots = 0;
    const int mi = u->mathIndex();
    for (const auto& k : u->kernels) {
        const auto& d = k.desc;
        slots += d.num_instances * d.num_output_rows;
        s->index_entries += d.num_instances * d.num_index_rows;
        s->constant_entries += d.num_instances * d.num_constant_rows;
        const auto& st = k.prog[mi].stats;
        s->flops += st.flops * d.num_instances;
        s->divs += st.divs * d.num_instances;
        s->sqrts += st.sqrts * d.num_instances;
        s->transcendentals += st.transcendentals * d.num_instances;
        s->gathers += st.gathers * d.num_instances;
        s->max_registers = std::max<std::uint64_t>(s->max_registers, (std::uint64_t)k.prog[mi].registers);
        s->program_words += k.prog[mi].words.size();
    }
    s->num_intermediates = slots > s->num_outputs ? slots - s->num_outputs : 0;
    return SYMGB_OK;
}

uint64_t symgb_algorithmic_bytes(symgb_unit_t u, int num_sets) {
    symgb_stats s;
    if (symgb_get_stats(u, &s)) return 0;
    const std::uint64_t S = (std::uint64_t)std::max(1, num_sets);
    return S * (8 * s.num_inputs + 8 * s.num_outputs + 16 * s.num_intermediates) + 4 * s.index_entries +
           8 * s.constant_entries;
}

int symgb_last_launch_count(symgb_unit_t u) { return u ? u->lastLaunches : 0; }

}  // extern "C"
