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
    const std::uint64_t* prog;  // device program: load section, compute bundles, literal table
    const std::uint32_t* p;     // index table of this kernel
    const double* c;            // constant table of this kernel
    std::uint64_t yoff;         // first x slot written by this kernel
    std::uint64_t n;            // instances
    std::uint32_t regs;         // register-file slots used
    std::uint32_t nloads;       // words in the loads section
    std::uint32_t nwords;       // total program words (loads + compute + literals)
    std::uint32_t litoff;       // first word of the literal table
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

// Interpreter variants: MODE_L2 reads x through L2 only (x written earlier in
// the same launch); MODE_LIB adds the library operations (pow, sin, ...),
// whose code needs many registers, so programs without them run a variant
// with a smaller register footprint and higher occupancy.
enum : int { MODE_L2 = 1, MODE_LIB = 2 };

struct EvalArgs {
    const DevKernel* ks;
    const Tile* tiles;
    const std::uint32_t* segments;  // tile index boundaries of the segments
    int segBegin, segEnd;           // segments run by this launch, barrier between them
    const double* x;
    double* xw;
    unsigned S;
    unsigned progCap;               // program words that fit in shared memory (0: read from global)
    unsigned barrierExtra;          // arrivals beyond the grid a barrier waits for (timeout tests; 0)
    BarrierState* bar;
    int* hostError;
    unsigned long long timeoutNs;
};

}  // namespace engine
}  // namespace symgb

namespace {

using namespace symgb::engine;

// Gather of x: through L2 only when other SMs write x during the launch.
template <int L2_ONLY>
__device__ __forceinline__ double loadX(const double* a) {
    if (L2_ONLY) return __ldcg(a);
    return __ldg(a);
}

#include "jit_prelude.cuh"

__device__ __forceinline__ double negate(double x) { return symgbNegate(x); }

struct AddOp {
    __device__ double operator()(double x, double y, double) const { return __dadd_rn(x, y); }
};
struct SubOp {
    __device__ double operator()(double x, double y, double) const { return __dsub_rn(x, y); }
};
struct MulOp {
    __device__ double operator()(double x, double y, double) const { return __dmul_rn(x, y); }
};
struct DivOp {
    __device__ double operator()(double x, double y, double) const { return __ddiv_rn(x, y); }
};
template <bool NEG_PRODUCT, bool NEG_ADDEND>
struct FmaOp {  // (+-)(x * y) (+-) z, one rounding
    __device__ double operator()(double x, double y, double z) const {
        return __fma_rn(NEG_PRODUCT ? negate(x) : x, y, NEG_ADDEND ? negate(z) : z);
    }
};
struct NegOp {
    __device__ double operator()(double x, double, double) const { return negate(x); }
};
struct MovOp {
    __device__ double operator()(double x, double, double) const { return x; }
};
struct SqrtOp {
    __device__ double operator()(double x, double, double) const { return __dsqrt_rn(x); }
};
struct RecOp {
    __device__ double operator()(double x, double, double) const { return __ddiv_rn(1.0, x); }
};

// Fast-mode division, reciprocal and square root (jit_prelude.cuh).
struct FastDivOp {
    __device__ double operator()(double a, double b, double) const { return symgbFastDiv(a, b); }
};
struct FastRecOp {
    __device__ double operator()(double x, double, double) const { return symgbFastRec(x); }
};
struct FastSqrtOp {
    __device__ double operator()(double x, double, double) const { return symgbFastSqrt(x); }
};
template <int OPC>
struct LibOp {  // CUDA's double-precision math library
    __device__ double operator()(double x, double y, double) const {
        switch (OPC) {
            case symgb::engine::OP_POW: return pow(x, y);
            case symgb::engine::OP_SIN: return sin(x);
            case symgb::engine::OP_COS: return cos(x);
            case symgb::engine::OP_TAN: return tan(x);
            case symgb::engine::OP_ASIN: return asin(x);
            case symgb::engine::OP_ACOS: return acos(x);
            case symgb::engine::OP_ATAN: return atan(x);
            case symgb::engine::OP_EXP: return exp(x);
            default: return log(x);
        }
    }
};

// Entries of a bundle processed together: their operand reads, operations and
// result writes are issued as three batches, so GROUP operations (times the
// items per thread) of one thread are in flight at once.
constexpr unsigned GROUP = 4;
constexpr unsigned LONG_GROUP = 2;  // division and square root: long sequences with many temporaries

__device__ __forceinline__ unsigned field(std::uint32_t e, int f) { return (e >> (8 * f)) & 0xffu; }

// Register file view of one thread: R[r * stride + j * T] is register r of item j.
struct RegFile {
    double* R;
    unsigned stride, T;
    __device__ __forceinline__ double& at(unsigned r, int j) const { return R[r * stride + j * T]; }
};

// Runs a bundle of `cnt` entries on the P lanes of each work item.  Round r
// gives lane l entry r * P + l; rounds are processed four, then two, then one
// at a time, the same count on every lane of the warp.  A lane whose entry
// index passes the end takes the last entry instead: it computes the same
// value into the same register as that entry's own lane, which is harmless,
// and keeps every lane on one instruction stream.  Single-entry bundles may
// take operands from, and leave their result only in, the accumulator `acc`
// (header flags; see program.hpp).
template <int ITEMS, int NSRC, unsigned G, class F>
__device__ __forceinline__ void runGroup(const std::uint32_t* e, unsigned cnt, unsigned first, unsigned lane,
                                         unsigned P, const RegFile& rf, unsigned flags, double (&acc)[ITEMS], F f) {
    std::uint32_t ee[G];
#pragma unroll
    for (unsigned u = 0; u < G; ++u) ee[u] = e[min(first + u * P + lane, cnt - 1)];
    double v[G][NSRC][ITEMS];
#pragma unroll
    for (unsigned u = 0; u < G; ++u)
#pragma unroll
        for (int s = 0; s < NSRC; ++s)
#pragma unroll
            for (int j = 0; j < ITEMS; ++j)
                v[u][s][j] = (G == 1 && (flags & (H_A_ACC << s))) ? acc[j] : rf.at(field(ee[u], s + 1), j);
    double r[G][ITEMS];
#pragma unroll
    for (unsigned u = 0; u < G; ++u)
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) r[u][j] = f(v[u][0][j], v[u][NSRC > 1 ? 1 : 0][j], v[u][NSRC > 2 ? 2 : 0][j]);
    if (G == 1) {
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) acc[j] = r[0][j];
        if (flags & H_NOSTORE) return;
    }
#pragma unroll
    for (unsigned u = 0; u < G; ++u)
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) rf.at(field(ee[u], 0), j) = r[u][j];
}

template <int ITEMS, int NSRC, unsigned GROUP, class F>
__device__ __forceinline__ void runBundle(const std::uint32_t* e, unsigned cnt, const RegFile& rf, unsigned lane,
                                          unsigned P, unsigned flags, double (&acc)[ITEMS], F f) {
    const unsigned rounds = (cnt + P - 1) / P;
    unsigned r = 0;
    for (; r + GROUP <= rounds; r += GROUP) runGroup<ITEMS, NSRC, GROUP>(e, cnt, r * P, lane, P, rf, 0, acc, f);
    if (GROUP > 2 && r + 2 <= rounds) {
        runGroup<ITEMS, NSRC, 2>(e, cnt, r * P, lane, P, rf, 0, acc, f);
        r += 2;
    }
    if (r < rounds) runGroup<ITEMS, NSRC, 1>(e, cnt, r * P, lane, P, rf, flags, acc, f);
}

// One entry at a time (long library sequences: keeps the code small).  Not a
// call: a call makes every live register of the caller survive it.
template <int ITEMS, int NSRC, class F>
__device__ __forceinline__ void runBundleSerial(const std::uint32_t* e, unsigned cnt, const RegFile& rf, unsigned lane,
                                                unsigned P, F f) {
    for (unsigned q = lane; q < cnt; q += P) {
        const std::uint32_t e0 = e[q];
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            const double x = rf.at(field(e0, 1), j);
            const double y = NSRC > 1 ? rf.at(field(e0, 2), j) : 0.0;
            rf.at(field(e0, 0), j) = f(x, y, 0.0);
        }
    }
}

// Grid-wide barrier of the persistent and fused schedules (bounded wait,
// jit_prelude.cuh).  `extra` raises the number of arrivals the barrier waits
// for beyond the grid (only for testing the timeout path; 0 otherwise).
__device__ __forceinline__ bool gridBarrier(BarrierState* bar, int* hostError, unsigned long long timeoutNs,
                                            unsigned extra) {
    return symgbGridBarrier(bar, hostError, timeoutNs, gridDim.x + extra);
}

// Stores of G rounds of an OP_ST bundle: y[row * n + i] for this lane's
// entries (a lane past the end stores the last entry's value again, to the
// same place).  A single-entry bundle may store the accumulator.
template <unsigned G, int ITEMS>
__device__ __forceinline__ void runStores(const std::uint32_t* e, unsigned cnt, unsigned first, unsigned P,
                                          const RegFile& rf, unsigned flags, const double (&acc)[ITEMS],
                                          const DevKernel& k, const EvalArgs& A, const std::uint64_t (&ii)[ITEMS],
                                          const unsigned (&ss)[ITEMS], const bool (&valid)[ITEMS]) {
    std::uint32_t ee[G];
    double v[G][ITEMS];
#pragma unroll
    for (unsigned u = 0; u < G; ++u) ee[u] = e[min(first + u * P, cnt - 1)];
#pragma unroll
    for (unsigned u = 0; u < G; ++u)
#pragma unroll
        for (int j = 0; j < ITEMS; ++j)
            v[u][j] = (G == 1 && (flags & symgb::engine::H_A_ACC)) ? acc[j] : rf.at(field(ee[u], 0), j);
#pragma unroll
    for (unsigned u = 0; u < G; ++u)
#pragma unroll
        for (int j = 0; j < ITEMS; ++j)
            if (valid[j]) A.xw[(k.yoff + (std::uint64_t)(ee[u] >> 8) * k.n + ii[j]) * A.S + ss[j]] = v[u][j];
}

// Load entries first, first + P, ..., first + (W - 1) P of the load section
// (this lane's share of W rounds; entries past the end are skipped): all
// index loads, then all gathers, constant and literal reads, then the
// register writes, so up to W x ITEMS independent loads are in flight.  x slots fit in 32 bits (checked when the
// unit is created).
template <int W, int ITEMS, int MODE>
__device__ __forceinline__ void runLoads(const std::uint64_t* prog, unsigned first, unsigned nl, unsigned P,
                                         const DevKernel& k, const EvalArgs& A, const std::uint64_t (&ii)[ITEMS],
                                         const unsigned (&ss)[ITEMS], const RegFile& rf) {
    using namespace symgb::engine;
    unsigned meta[W];
    unsigned slot[W][ITEMS];
#pragma unroll
    for (int u = 0; u < W; ++u) {
        const std::uint64_t w = (first + u * P < nl) ? prog[first + u * P] : 0ull;
        meta[u] = (unsigned)w & 0xffffu;  // op, destination register
        const unsigned op = (unsigned)w & 0xffu;
        const unsigned imm = (unsigned)(w >> 32);
#pragma unroll
        for (int j = 0; j < ITEMS; ++j)
            slot[u][j] = op == OP_LDX ? __ldg(k.p + ((unsigned)(w >> 16) & 0xffffu) * k.n + ii[j]) + imm : imm;
    }
    const double* lit = reinterpret_cast<const double*>(prog + k.litoff);
    double v[W][ITEMS];
#pragma unroll
    for (int u = 0; u < W; ++u)
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            const unsigned op = meta[u] & 0xffu;
            if (op == OP_LDX)
                v[u][j] = loadX<MODE & MODE_L2>(A.x + (std::uint64_t)slot[u][j] * A.S + ss[j]);
            else if (op == OP_LDC)
                v[u][j] = __ldg(k.c + (std::uint64_t)slot[u][j] * k.n + ii[j]);
            else if (op == OP_LDK)
                v[u][j] = lit[slot[u][j]];
            else
                v[u][j] = 0.0;
        }
#pragma unroll
    for (int u = 0; u < W; ++u)
        if (first + u * P < nl) {
#pragma unroll
            for (int j = 0; j < ITEMS; ++j) rf.at(meta[u] >> 8, j) = v[u][j];
        }
}

// Evaluates one tile.  A work item (one instance for one value set) is run by
// P = LANES threads of one warp: warp lane l serves item slot l % (32 / P)
// of its warp as lane l / (32 / P), so each half-warp touches consecutive
// slots.  Each thread serves ITEMS item slots per pass.  Shared memory holds
// the program (when it fits) followed by the register file, laid out
// [register][item][slot] so a warp's accesses are conflict-free.  The lanes of
// an item split every bundle; a warp barrier after each bundle makes their
// results visible to each other.
template <int ITEMS, int LANES, int MODE>
__device__ __forceinline__ void evalTile(const DevKernel& k, const std::uint64_t* prog, double* regs, const Tile& t,
                                         const EvalArgs& A) {
    using namespace symgb::engine;
    constexpr unsigned P = LANES;
    constexpr unsigned perWarp = 32u / P;
    const unsigned lane = (threadIdx.x & 31u) / perWarp;
    const unsigned T = blockDim.x / P;  // item slots per block
    const unsigned me = (threadIdx.x >> 5) * perWarp + (threadIdx.x & (perWarp - 1));
    const unsigned S = A.S;
    const RegFile rf{regs + me, (unsigned)ITEMS * T, T};
    const double* lit = reinterpret_cast<const double*>(prog + k.litoff);
    for (std::uint64_t base = 0; base < t.count; base += (std::uint64_t)T * ITEMS) {
        std::uint64_t ii[ITEMS];
        unsigned ss[ITEMS];
        bool valid[ITEMS];
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) {
            std::uint64_t off = base + (std::uint64_t)j * T + me;
            valid[j] = off < t.count;
            if (!valid[j]) off = t.count - 1;  // duplicate the last item; its stores are skipped
            const std::uint64_t w = t.start + off;
            if (S == 1) {
                ii[j] = w;
                ss[j] = 0;
            } else if (w < 0xffffffffull) {
                ii[j] = (std::uint32_t)w / S;
                ss[j] = (unsigned)w - (unsigned)ii[j] * S;
            } else {
                ii[j] = w / S;
                ss[j] = (unsigned)(w - ii[j] * S);
            }
        }
        // Loads: in rounds of 8, 4, 2 and 1 entries per lane (the same count on
        // every lane), all index loads, then all gathers.
        const unsigned nl = k.nloads;
        const unsigned rounds = (nl + P - 1) / P;
        unsigned r = 0;
        for (; r + 8 <= rounds; r += 8) runLoads<8, ITEMS, MODE>(prog, r * P + lane, nl, P, k, A, ii, ss, rf);
        if (r + 4 <= rounds) {
            runLoads<4, ITEMS, MODE>(prog, r * P + lane, nl, P, k, A, ii, ss, rf);
            r += 4;
        }
        if (r + 2 <= rounds) {
            runLoads<2, ITEMS, MODE>(prog, r * P + lane, nl, P, k, A, ii, ss, rf);
            r += 2;
        }
        if (r < rounds) runLoads<1, ITEMS, MODE>(prog, r * P + lane, nl, P, k, A, ii, ss, rf);
        if (P > 1) __syncwarp();
        // Compute bundles.
        double acc[ITEMS];
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) acc[j] = 0.0;
        for (const std::uint64_t* ip = prog + nl;;) {
            const std::uint64_t h = *ip;
            const unsigned op = (unsigned)h & 0xffu;
            if (op == OP_END) break;
            const unsigned cnt = (unsigned)(h >> 8) & 0xffffu;
            const unsigned flags = (unsigned)h & 0xff000000u;
            const std::uint32_t* e = reinterpret_cast<const std::uint32_t*>(ip + 1);
            ip += 1 + ((cnt + 1) >> 1);
            switch (op) {
                case OP_ADD: runBundle<ITEMS, 2, GROUP>(e, cnt, rf, lane, P, flags, acc, AddOp{}); break;
                case OP_SUB: runBundle<ITEMS, 2, GROUP>(e, cnt, rf, lane, P, flags, acc, SubOp{}); break;
                case OP_MUL: runBundle<ITEMS, 2, GROUP>(e, cnt, rf, lane, P, flags, acc, MulOp{}); break;
                case OP_DIV: runBundle<ITEMS, 2, LONG_GROUP>(e, cnt, rf, lane, P, flags, acc, DivOp{}); break;
                case OP_FMA: runBundle<ITEMS, 3, GROUP>(e, cnt, rf, lane, P, flags, acc, FmaOp<false, false>{}); break;
                case OP_FMS: runBundle<ITEMS, 3, GROUP>(e, cnt, rf, lane, P, flags, acc, FmaOp<false, true>{}); break;
                case OP_FNMA: runBundle<ITEMS, 3, GROUP>(e, cnt, rf, lane, P, flags, acc, FmaOp<true, false>{}); break;
                case OP_FNMS: runBundle<ITEMS, 3, GROUP>(e, cnt, rf, lane, P, flags, acc, FmaOp<true, true>{}); break;
                case OP_NEG: runBundle<ITEMS, 1, GROUP>(e, cnt, rf, lane, P, flags, acc, NegOp{}); break;
                case OP_MOV: runBundle<ITEMS, 1, GROUP>(e, cnt, rf, lane, P, flags, acc, MovOp{}); break;
                case OP_SQRT: runBundle<ITEMS, 1, LONG_GROUP>(e, cnt, rf, lane, P, flags, acc, SqrtOp{}); break;
                case OP_REC: runBundle<ITEMS, 1, LONG_GROUP>(e, cnt, rf, lane, P, flags, acc, RecOp{}); break;
                case OP_FDIV: runBundle<ITEMS, 2, LONG_GROUP>(e, cnt, rf, lane, P, flags, acc, FastDivOp{}); break;
                case OP_FSQRT: runBundle<ITEMS, 1, LONG_GROUP>(e, cnt, rf, lane, P, flags, acc, FastSqrtOp{}); break;
                case OP_FREC: runBundle<ITEMS, 1, LONG_GROUP>(e, cnt, rf, lane, P, flags, acc, FastRecOp{}); break;
                case OP_POW: if (MODE & MODE_LIB) runBundleSerial<ITEMS, 2>(e, cnt, rf, lane, P, LibOp<OP_POW>{}); break;
                case OP_SIN: if (MODE & MODE_LIB) runBundleSerial<ITEMS, 1>(e, cnt, rf, lane, P, LibOp<OP_SIN>{}); break;
                case OP_COS: if (MODE & MODE_LIB) runBundleSerial<ITEMS, 1>(e, cnt, rf, lane, P, LibOp<OP_COS>{}); break;
                case OP_TAN: if (MODE & MODE_LIB) runBundleSerial<ITEMS, 1>(e, cnt, rf, lane, P, LibOp<OP_TAN>{}); break;
                case OP_ASIN: if (MODE & MODE_LIB) runBundleSerial<ITEMS, 1>(e, cnt, rf, lane, P, LibOp<OP_ASIN>{}); break;
                case OP_ACOS: if (MODE & MODE_LIB) runBundleSerial<ITEMS, 1>(e, cnt, rf, lane, P, LibOp<OP_ACOS>{}); break;
                case OP_ATAN: if (MODE & MODE_LIB) runBundleSerial<ITEMS, 1>(e, cnt, rf, lane, P, LibOp<OP_ATAN>{}); break;
                case OP_EXP: if (MODE & MODE_LIB) runBundleSerial<ITEMS, 1>(e, cnt, rf, lane, P, LibOp<OP_EXP>{}); break;
                case OP_LOG: if (MODE & MODE_LIB) runBundleSerial<ITEMS, 1>(e, cnt, rf, lane, P, LibOp<OP_LOG>{}); break;
                case OP_LDK:
                    for (unsigned r = 0; r < (cnt + P - 1) / P; ++r) {  // rounds, as in runBundle
                        const std::uint32_t e0 = e[min(r * P + lane, cnt - 1)];
                        const double c = lit[e0 >> 8];
#pragma unroll
                        for (int j = 0; j < ITEMS; ++j) {
                            acc[j] = c;
                            if (!(flags & H_NOSTORE)) rf.at(field(e0, 0), j) = c;
                        }
                    }
                    break;
                case OP_ST: {
                    // Rounds of 4, 2 and 1 entries as in runBundle.
                    const unsigned rounds = (cnt + P - 1) / P;
                    unsigned r = 0;
                    for (; r + GROUP <= rounds; r += GROUP)
                        runStores<GROUP, ITEMS>(e, cnt, r * P + lane, P, rf, 0, acc, k, A, ii, ss, valid);
                    if (r + 2 <= rounds) {
                        runStores<2, ITEMS>(e, cnt, r * P + lane, P, rf, 0, acc, k, A, ii, ss, valid);
                        r += 2;
                    }
                    if (r < rounds) runStores<1, ITEMS>(e, cnt, r * P + lane, P, rf, flags, acc, k, A, ii, ss, valid);
                    break;
                }
                default: break;
            }
            if (P > 1) __syncwarp();
        }
    }
}

// Runs the tiles of segments [segBegin, segEnd); a grid barrier separates
// segments (cooperative launches only when the range holds several segments).
// Register cap per variant: the interpreter's occupancy is what hides the
// latency of its shared-memory operands and FP64 results.  With a cap of 72,
// ptxas fits the two-item variant without library operations into 64
// registers with no spills (96 allowed it 80; cotan 500 per execute: 153 us
// against 163 us).
template <int ITEMS>
struct EvalRegs {
    static constexpr int value = ITEMS == 1 ? 64 : ITEMS == 2 ? 72 : 96;
};

template <int ITEMS, int LANES, int MODE>
__global__ void __maxnreg__(EvalRegs<ITEMS>::value) evalKernel(EvalArgs A) {
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
            evalTile<ITEMS, LANES, MODE>(k, prog, regs, t, A);
        }
        if (sg + 1 < A.segEnd)
            if (!gridBarrier(A.bar, A.hostError, A.timeoutNs, A.barrierExtra)) return;
    }
}

// out[s * len + j] = x[ids[j] * S + s]  (reference gatherResult, per value set).
// Threads run along the output (j fastest), so the writes are contiguous; they
// may go straight to page-locked host memory.
__global__ void gatherKernel(const double* __restrict__ x, const std::uint32_t* __restrict__ ids, std::uint64_t len,
                             unsigned S, double* __restrict__ out) {
    const std::uint64_t w = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= len * S) return;
    const std::uint64_t s = S == 1 ? 0 : w / len;
    const std::uint64_t j = w - s * len;
    out[w] = __ldg(x + (std::uint64_t)__ldg(ids + j) * S + s);
}

}  // namespace
