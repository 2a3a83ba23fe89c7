// Device-side code shared by the engine's translation units: the interpreter
// for ComputeKernel programs (evalTile / evalKernel), the bounded grid barrier
// and the result gather.  Included inside an anonymous namespace, so every
// translation unit instantiates its own kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "program.hpp"
#include "symgb.h"

namespace symgb {
namespace engine {

struct DevKernel {
    const std::uint64_t* prog;  // device program: loads section, then compute words
    const std::uint32_t* p;     // index table of this kernel
    const double* c;            // constant table of this kernel
    std::uint64_t yoff;         // first x slot written by this kernel
    std::uint64_t n;            // instances
    std::uint32_t regs;         // register-file slots used
    std::uint32_t nloads;       // words in the loads section
    std::uint32_t nwords;       // total program words (loads + compute)
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

struct EvalArgs {
    const DevKernel* ks;
    const Tile* tiles;
    const std::uint32_t* segments;  // tile index boundaries of the segments
    int segBegin, segEnd;           // segments run by this launch, barrier between them
    const double* x;
    double* xw;
    unsigned S;
    unsigned progCap;               // program words that fit in shared memory (0: read from global)
    unsigned regStride;             // unused, reserved
    BarrierState* bar;
    int* hostError;
    unsigned long long timeoutNs;
};

}  // namespace engine
}  // namespace symgb

namespace {

using namespace symgb::engine;

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


// Evaluates one tile: ITEMS work items per thread.  Shared memory holds the
// program (when it fits) followed by the register file, laid out
// [register][item][thread] so a warp's accesses are conflict-free.
template <int ITEMS, int LOAD>
__device__ __forceinline__ void evalTile(const DevKernel& k, const std::uint64_t* prog, double* regs, const Tile& t,
                                         const EvalArgs& A) {
    using namespace symgb::engine;
    const unsigned T = blockDim.x;
    const unsigned S = A.S;
    for (std::uint64_t base = 0; base < t.count; base += (std::uint64_t)T * ITEMS) {
        std::uint64_t ii[ITEMS];
        unsigned ss[ITEMS];
        bool valid[ITEMS];
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            std::uint64_t off = base + (std::uint64_t)j * T + threadIdx.x;
            valid[j] = off < t.count;
            if (!valid[j]) off = t.count - 1;  // duplicate the last item; its stores are skipped
            const std::uint64_t w = t.start + off;
            ii[j] = w / S;
            ss[j] = (unsigned)(w - ii[j] * S);
        }
#define REG(r, j) regs[((unsigned)(r) * ITEMS + (j)) * T + threadIdx.x]
        // Loads: up to 8 entries at a time, all index loads, then all gathers.
        const unsigned nl = k.nloads;
        for (unsigned b = 0; b < nl; b += 8) {
            std::uint64_t wv[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) wv[u] = (b + u < nl) ? prog[b + u] : 0ull;
            long long idx[8][ITEMS];
#pragma unroll
            for (int u = 0; u < 8; ++u)
#pragma unroll
                for (int j = 0; j < ITEMS; ++j) {
                    idx[u][j] = 0;
                    if ((wv[u] & 0xff) == OP_LDX) {
                        const unsigned row = (unsigned)(wv[u] >> 16) & 0xffff;
                        idx[u][j] = (long long)__ldg(k.p + row * k.n + ii[j]) + (int)(unsigned)(wv[u] >> 32);
                    }
                }
            double v[8][ITEMS];
#pragma unroll
            for (int u = 0; u < 8; ++u)
#pragma unroll
                for (int j = 0; j < ITEMS; ++j) {
                    const unsigned op = (unsigned)(wv[u] & 0xff);
                    if (op == OP_LDX)
                        v[u][j] = loadX<LOAD>(A.x + (std::uint64_t)idx[u][j] * S + ss[j]);
                    else if (op == OP_LDC)
                        v[u][j] = __ldg(k.c + (std::uint64_t)(unsigned)(wv[u] >> 32) * k.n + ii[j]);
                    else
                        v[u][j] = 0.0;
                }
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (b + u < nl) {
                    const unsigned d = (unsigned)(wv[u] >> 8) & 0xff;
#pragma unroll
                    for (int j = 0; j < ITEMS; ++j) REG(d, j) = v[u][j];
                }
        }
        // Arithmetic and stores.  `acc` holds the last result (per item); flag
        // bits route single-use values through it instead of shared memory.
        double acc[ITEMS];
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) acc[j] = 0.0;
        for (const std::uint64_t* ip = prog + nl;;) {
            const std::uint64_t w = *ip++;
            const unsigned op = (unsigned)(w & 0xff);
            const unsigned d = (unsigned)(w >> 8) & 0xff;
            const unsigned a = (unsigned)(w >> 16) & 0xff;
            const unsigned bb = (unsigned)(w >> 24) & 0xff;
            const bool aAcc = (w & F_A_ACC) != 0, bAcc = (w & F_B_ACC) != 0, keep = (w & F_NOSTORE) == 0;
            if (op == OP_END) break;
#define OPA(j) (aAcc ? acc[j] : REG(a, j))
#define OPB(j) (bAcc ? acc[j] : REG(bb, j))
#define RESULT(j, v)              \
    {                             \
        const double r_ = (v);    \
        acc[j] = r_;              \
        if (keep) REG(d, j) = r_; \
    }
            switch (op) {
                case OP_LDK: {
                    const double cv = __longlong_as_double((long long)*ip++);
#pragma unroll
                    for (int j = 0; j < ITEMS; ++j) RESULT(j, cv)
                    break;
                }
                case OP_ST: {
                    const std::uint64_t row = (std::uint64_t)((w >> 32) & 0xffffff);
#pragma unroll
                    for (int j = 0; j < ITEMS; ++j)
                        if (valid[j]) A.xw[(k.yoff + row * k.n + ii[j]) * S + ss[j]] = OPA(j);
                    break;
                }
#define BIN(OPC, EXPR)                                                 \
    case OPC: {                                                        \
        _Pragma("unroll") for (int j = 0; j < ITEMS; ++j) {            \
            const double x1 = OPA(j), x2 = OPB(j);                     \
            RESULT(j, (EXPR))                                          \
        }                                                              \
        break;                                                         \
    }
#define UN(OPC, EXPR)                                                  \
    case OPC: {                                                        \
        _Pragma("unroll") for (int j = 0; j < ITEMS; ++j) {            \
            const double x1 = OPA(j);                                  \
            RESULT(j, (EXPR))                                          \
        }                                                              \
        break;                                                         \
    }
                BIN(OP_ADD, __dadd_rn(x1, x2))
                BIN(OP_SUB, __dsub_rn(x1, x2))
                BIN(OP_MUL, __dmul_rn(x1, x2))
                BIN(OP_DIV, __ddiv_rn(x1, x2))
                BIN(OP_POW, pow(x1, x2))
                UN(OP_NEG, -x1)
                UN(OP_SQRT, __dsqrt_rn(x1))
                UN(OP_REC, __ddiv_rn(1.0, x1))
                UN(OP_MOV, x1)
                UN(OP_SIN, sin(x1))
                UN(OP_COS, cos(x1))
                UN(OP_TAN, tan(x1))
                UN(OP_ASIN, asin(x1))
                UN(OP_ACOS, acos(x1))
                UN(OP_ATAN, atan(x1))
                UN(OP_EXP, exp(x1))
                UN(OP_LOG, log(x1))
#undef BIN
#undef UN
                case OP_FMA: {
                    const unsigned cr = (unsigned)(w >> 32) & 0xff;
                    const int fl = (int)((w >> 40) & 0x3);
                    const bool cAcc = (w & F_C_ACC) != 0;
#pragma unroll
                    for (int j = 0; j < ITEMS; ++j) {
                        const double x3 = cAcc ? acc[j] : REG(cr, j);
                        RESULT(j, dfma(OPA(j), OPB(j), x3, fl))
                    }
                    break;
                }
                default: break;
            }
#undef OPA
#undef OPB
#undef RESULT
        }
#undef REG
    }
}

// Runs the tiles of segments [segBegin, segEnd); a grid barrier separates
// segments (cooperative launches only when the range holds several segments).
template <int ITEMS, int LOAD>
__global__ void evalKernel(EvalArgs A) {
    extern __shared__ double smem[];
    std::uint64_t* progSmem = reinterpret_cast<std::uint64_t*>(smem);
    double* regs = smem + A.progCap;
    int cur = -1;
    const std::uint64_t* prog = nullptr;
    DevKernel k;
    for (int sg = A.segBegin; sg < A.segEnd; ++sg) {
        const std::uint32_t t0 = A.segments[sg], t1 = A.segments[sg + 1];
        for (std::uint32_t ti = t0 + blockIdx.x; ti < t1; ti += gridDim.x) {
            const Tile t = A.tiles[ti];
            if ((int)t.kernel != cur) {
                k = A.ks[t.kernel];
                cur = (int)t.kernel;
                if (k.nwords <= A.progCap) {
                    __syncthreads();  // previous program no longer in use
                    for (unsigned q = threadIdx.x; q < k.nwords; q += blockDim.x) progSmem[q] = k.prog[q];
                    __syncthreads();
                    prog = progSmem;
                } else {
                    prog = k.prog;
                }
            }
            evalTile<ITEMS, LOAD>(k, prog, regs, t, A);
        }
        if (sg + 1 < A.segEnd)
            if (!gridBarrier(A.bar, A.hostError, A.timeoutNs)) return;
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

}  // namespace
