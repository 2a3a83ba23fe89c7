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
#include <chrono>
#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "codegen.hpp"
#include "device.cuh"
#include "kernels.hpp"
#include "program.hpp"
#include "symgb.h"
#include "unit.hpp"

using namespace symgb::engine;

namespace {

thread_local std::string g_lastError;

int fail(int code, const std::string& msg) {
    g_lastError = msg;
    return code;
}

}  // namespace

int symgb::engine::setLastError(int code, const std::string& msg) { return fail(code, msg); }

namespace {

#define SYMGB_CUDA(call)                                                                            \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return fail(e_ == cudaErrorMemoryAllocation ? SYMGB_ERR_NOMEM : SYMGB_ERR_CUDA,        \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                        \
    } while (0)

// ------------------------------------------------------------------ device side

// x[(start + j) * S + s] = in[s * len + j]
__global__ void scatterKernel(const double* __restrict__ in, std::uint64_t start, std::uint64_t len, unsigned S,
                              double* __restrict__ x) {
    const std::uint64_t w = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= len * S) return;
    const std::uint64_t j = w / S;
    const unsigned s = (unsigned)(w - j * S);
    x[(start + j) * S + s] = __ldg(in + (std::uint64_t)s * len + j);
}

// The same two copies for many value sets, through a 32 x 32 tile in shared
// memory: one warp reads the 32 consecutive sets of one slot (256 contiguous
// bytes of x) and writes 32 consecutive positions of one set, so both sides
// are coalesced (the one-thread-per-value kernels above read 8 bytes per
// 32-byte sector on one side).  Grid: (ceil(len / 32), ceil(S / 32)), 256
// threads.
constexpr unsigned kSetTile = 32;

// out[s * len + j] = x[ids[j] * S + s]
__global__ void __launch_bounds__(256) gatherSetsKernel(const double* __restrict__ x,
                                                        const std::uint32_t* __restrict__ ids, std::uint64_t len,
                                                        unsigned S, double* __restrict__ out) {
    __shared__ double tile[kSetTile][kSetTile + 1];
    const std::uint64_t j0 = (std::uint64_t)blockIdx.x * kSetTile;
    const unsigned s0 = blockIdx.y * kSetTile;
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (unsigned p = warp; p < kSetTile; p += 8) {
        const std::uint64_t j = j0 + p;
        if (j < len && s0 + lane < S) tile[p][lane] = __ldg(x + (std::uint64_t)__ldg(ids + j) * S + s0 + lane);
    }
    __syncthreads();
    for (unsigned q = warp; q < kSetTile; q += 8) {
        const std::uint64_t j = j0 + lane;
        if (s0 + q < S && j < len) out[(std::uint64_t)(s0 + q) * len + j] = tile[lane][q];
    }
}

// x[(start + j) * S + s] = in[s * len + j]
__global__ void __launch_bounds__(256) scatterSetsKernel(const double* __restrict__ in, std::uint64_t start,
                                                         std::uint64_t len, unsigned S, double* __restrict__ x) {
    __shared__ double tile[kSetTile][kSetTile + 1];
    const std::uint64_t j0 = (std::uint64_t)blockIdx.x * kSetTile;
    const unsigned s0 = blockIdx.y * kSetTile;
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (unsigned q = warp; q < kSetTile; q += 8) {
        const std::uint64_t j = j0 + lane;
        if (s0 + q < S && j < len) tile[lane][q] = __ldg(in + (std::uint64_t)(s0 + q) * len + j);
    }
    __syncthreads();
    for (unsigned p = warp; p < kSetTile; p += 8) {
        const std::uint64_t j = j0 + p;
        if (j < len && s0 + lane < S) x[(start + j) * S + s0 + lane] = tile[p][lane];
    }
}

// Padded copy of one kernel's table rows for the compiled executor's grouped
// item layout: dst[r * stride + i] = src[r * n + min(i, n - 1)] (the last
// instance's entry fills the padding, so padded loads stay valid).
template <class T>
__global__ void padRowsKernel(const T* __restrict__ src, T* __restrict__ dst, std::uint64_t n, std::uint64_t stride,
                              std::uint64_t rows) {
    const std::uint64_t w = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= rows * stride) return;
    const std::uint64_t r = w / stride, i = w - r * stride;
    dst[w] = src[r * n + (i < n ? i : n - 1)];
}

// res[pos[t]] = x[slot[t]]: the results of the rows that are not written
// straight into res (one value set).
__global__ void restGatherKernel(const double* __restrict__ x, const std::uint32_t* __restrict__ pos,
                                 const std::uint32_t* __restrict__ slot, std::uint64_t count, double* __restrict__ res) {
    const std::uint64_t t = (std::uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < count) res[__ldg(pos + t)] = __ldg(x + __ldg(slot + t));
}

// Value-set counts from which the tiled kernels are used.
constexpr unsigned kTiledSets = 8;

// ------------------------------------------------------------------ host side

}  // namespace

namespace {

int uploadPrograms(symgb_unit* u) {
    const int mi = u->mathIndex();
    std::vector<std::uint64_t> all;
    std::vector<std::size_t> offs;
    u->maxProgWords = 0;
    for (auto& k : u->kernels) {
        offs.push_back(all.size());
        const Program& pr = k.prog[mi];
        all.insert(all.end(), pr.loads.begin(), pr.loads.end());
        all.insert(all.end(), pr.words.begin(), pr.words.end());
        u->maxProgWords = std::max<std::uint32_t>(u->maxProgWords, (std::uint32_t)(pr.loads.size() + pr.words.size()));
    }
    SYMGB_CUDA(u->progs.alloc(all.size()));
    SYMGB_CUDA(cudaMemcpy(u->progs.ptr, all.data(), all.size() * 8, cudaMemcpyHostToDevice));
    u->hostDevKernels.clear();
    for (std::size_t k = 0; k < u->kernels.size(); ++k) {
        const auto& d = u->kernels[k].desc;
        const Program& pr = u->kernels[k].prog[mi];
        DevKernel dk;
        dk.prog = u->progs.ptr + offs[k];
        dk.p = u->p.ptr + d.index_offset;
        dk.c = u->c.ptr + d.constants_offset;
        dk.yoff = d.output_offset;
        dk.n = d.num_instances;
        dk.regs = (std::uint32_t)std::max(1, pr.registers);
        dk.nloads = (std::uint32_t)pr.loads.size();
        dk.nwords = (std::uint32_t)(pr.loads.size() + pr.words.size());
        dk.litoff = (std::uint32_t)(pr.loads.size() + pr.literalOffset);
        u->hostDevKernels.push_back(dk);
    }
    SYMGB_CUDA(u->devKernels.alloc(u->hostDevKernels.size()));
    SYMGB_CUDA(cudaMemcpy(u->devKernels.ptr, u->hostDevKernels.data(), u->hostDevKernels.size() * sizeof(DevKernel),
                          cudaMemcpyHostToDevice));
    u->dropGraph();
    u->tilesSets = -1;
    return SYMGB_OK;
}

// Tile table: per level, every kernel's work items cut into tiles of
// consecutive work items; tiles of one kernel are contiguous.  Segments give the
// tile boundaries per level (fused schedules) and per kernel (plain schedule).
int buildTiles(symgb_unit* u) {
    const int S = u->numSets;
    const int items = u->sched.items_per_tile > 0 ? u->sched.items_per_tile : u->launchTpb() / u->lanes() * u->items();
    if (u->tilesSets == S && u->tilesItems == items && u->tilesMath == u->mathIndex() &&
        u->tilesShapes == u->shapesVersion)
        return SYMGB_OK;
    u->hostTiles.clear();
    u->hostLevelSeg.assign(1, 0);
    u->hostKernelSeg.assign(1, 0);
    for (int L = 0; L < u->numLevels; ++L) {
        for (std::size_t k = 0; k < u->kernels.size(); ++k) {
            if (u->kernels[k].desc.level != L) continue;
            const std::uint64_t total = u->kernels[k].desc.num_instances * (std::uint64_t)S;
            if (!total) continue;
            // One pass of the kernel's launch shape per tile (unless the
            // schedule fixes the tile size).
            const symgb_unit::Shape sh = u->shapeOf(k);
            const std::uint64_t tile = u->sched.items_per_tile > 0 ? (std::uint64_t)u->sched.items_per_tile
                                                                   : (std::uint64_t)(sh.tpb / sh.lanes * sh.items);
            for (std::uint64_t st = 0; st < total; st += tile)
                u->hostTiles.push_back({(std::uint32_t)k, (std::uint32_t)std::min<std::uint64_t>(tile, total - st), st});
            u->hostKernelSeg.push_back((std::uint32_t)u->hostTiles.size());
        }
        u->hostLevelSeg.push_back((std::uint32_t)u->hostTiles.size());
    }
    SYMGB_CUDA(u->tiles.alloc(u->hostTiles.size()));
    if (!u->hostTiles.empty())
        SYMGB_CUDA(cudaMemcpy(u->tiles.ptr, u->hostTiles.data(), u->hostTiles.size() * sizeof(Tile), cudaMemcpyHostToDevice));
    SYMGB_CUDA(u->levelSeg.alloc(u->hostLevelSeg.size()));
    SYMGB_CUDA(cudaMemcpy(u->levelSeg.ptr, u->hostLevelSeg.data(), u->hostLevelSeg.size() * 4, cudaMemcpyHostToDevice));
    SYMGB_CUDA(u->kernelSeg.alloc(u->hostKernelSeg.size()));
    SYMGB_CUDA(cudaMemcpy(u->kernelSeg.ptr, u->hostKernelSeg.data(), u->hostKernelSeg.size() * 4, cudaMemcpyHostToDevice));
    u->tilesSets = S;
    u->tilesItems = items;
    u->tilesShapes = u->shapesVersion;
    u->tilesMath = u->mathIndex();
    return SYMGB_OK;
}

std::uint32_t maxRegs(const symgb_unit* u, int level = -1) {
    std::uint32_t r = 1;
    for (std::size_t k = 0; k < u->kernels.size(); ++k)
        if (level < 0 || u->kernels[k].desc.level == level) r = std::max(r, u->hostDevKernels[k].regs);
    return r;
}

std::uint32_t maxWords(const symgb_unit* u, int level = -1) {
    std::uint32_t w = 0;
    for (std::size_t k = 0; k < u->kernels.size(); ++k)
        if (level < 0 || u->kernels[k].desc.level == level) w = std::max(w, u->hostDevKernels[k].nwords);
    return w;
}

// Program words that may be staged in shared memory per CTA.  A launch stages
// its programs whenever they fit beside the register file: read from global
// memory instead, every bundle header and entry is an L1 access that the
// gathers compete with, and misses go to L2.  Larger programs are read from
// global memory (all threads of a warp read the same word).
constexpr std::uint32_t kProgCapWords = 4096;

std::size_t smemBytes(std::uint32_t progCap, std::uint32_t regs, int items, int tpb, int lanes) {
    return (std::size_t)progCap * 8 + (std::size_t)regs * items * (tpb / lanes) * sizeof(double);
}

// Largest block size <= tpb (a multiple of 32) whose register file (and
// staged program) fit in shared memory; 0 if not even one warp fits.
int fitBlock(const symgb_unit* u, std::uint32_t progCap, std::uint32_t regs, int items, int tpb, int lanes) {
    while (tpb >= 32 && smemBytes(progCap, regs, items, tpb, lanes) > u->smemOptin) tpb -= 32;
    return tpb >= 32 ? tpb : 0;
}

int setSmemLimit(const void* fn, std::size_t bytes) {
    if (bytes > 48 * 1024) SYMGB_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return SYMGB_OK;
}

const void* evalFunction(int items, int lanes, bool l2, bool lib) {
    return symgb::engine::evalKernelFor(items, lanes, (l2 ? MODE_L2 : 0) | (lib ? MODE_LIB : 0));
}

// ------------------------------------------------------------------ compiled executor

// Module configuration of the compiled executor for schedule `kind`: block
// sizes as the interpreter's (per-kernel shapes for plain launches, the
// heaviest kernel's shape for a level, the schedule's for the persistent
// kernel).
JitConfig jitConfig(const symgb_unit* u, int kind) {
    JitConfig c;
    c.kind = kind == SYMGB_SCHEDULE_PLAIN ? JIT_PLAIN : kind == SYMGB_SCHEDULE_LEVELS ? JIT_LEVELS : JIT_PERSISTENT;
    c.math = u->sched.math;
    c.numSets = (unsigned)u->numSets;
    c.minBlocks = std::max(0, u->sched.blocks_per_sm);
    c.loadPath = u->loadPath;
    c.itemLayout = u->itemLayout;
    if (u->directOutputs && u->numSets == 1 && u->directRows) c.directBase = u->directBase;
    for (std::size_t k = 0; k < u->kernels.size(); ++k) {
        c.kernelTpb.push_back(u->shapeOf(k).tpb);
        c.kernelItems.push_back(u->shapeOf(k).items);
    }
    if (c.kind == JIT_PERSISTENT) {
        c.levelTpb.assign(1, u->tpb());
        c.levelItems.assign(1, u->items());
    } else {
        c.levelTpb.assign((std::size_t)std::max(1, u->numLevels), u->tpb());
        c.levelItems.assign(c.levelTpb.size(), u->items());
        std::vector<double> most(c.levelTpb.size(), -1.0);
        for (std::size_t k = 0; k < u->kernels.size(); ++k) {
            const auto& d = u->kernels[k].desc;
            const double work = (double)d.num_instances * (double)(d.num_nodes + 1);
            if (d.level >= 0 && (std::size_t)d.level < most.size() && work > most[d.level]) {
                most[d.level] = work;
                c.levelTpb[d.level] = u->shapeOf(k).tpb;
                c.levelItems[d.level] = u->shapeOf(k).items;
            }
        }
    }
    return c;
}

std::string jitKeyOf(const JitConfig& c) {
    std::string k = std::to_string(c.kind) + "/" + std::to_string(c.math) + "/" + std::to_string(c.numSets) + "/";
    for (int t : c.kernelTpb) k += std::to_string(t) + ",";
    k += "/";
    for (int t : c.levelTpb) k += std::to_string(t) + ",";
    k += "/";
    for (int t : c.kernelItems) k += std::to_string(t) + ",";
    k += "/";
    for (int t : c.levelItems) k += std::to_string(t) + ",";
    k += "/" + std::to_string(c.minBlocks) + "/" + std::to_string(c.loadPath) + "/" + std::to_string(c.itemLayout) +
         "/" + std::to_string(c.directBase.empty() ? 0 : 1);
    return k;
}

// The padded tables of the grouped item layout, made once per init on the
// unit's stream (which is then synchronised: a later capture must not see it).
int buildGroupedTables(symgb_unit* u) {
    if (u->groupedBuilt) return SYMGB_OK;
    std::vector<symgb_kernel_desc> descs;
    for (const auto& k : u->kernels) descs.push_back(k.desc);
    const GroupedTables t = groupedTables(descs);
    SYMGB_CUDA(u->p4.alloc(t.indexSize));
    SYMGB_CUDA(u->c4.alloc(t.constSize));
    for (std::size_t k = 0; k < descs.size(); ++k) {
        const symgb_kernel_desc& d = descs[k];
        if (!d.num_instances) continue;
        const std::uint64_t iw = t.stride[k] * d.num_index_rows, cw = t.stride[k] * d.num_constant_rows;
        if (iw)
            padRowsKernel<std::uint32_t><<<(unsigned)((iw + 255) / 256), 256, 0, u->stream>>>(
                u->p.ptr + d.index_offset, u->p4.ptr + t.indexBase[k], d.num_instances, t.stride[k], d.num_index_rows);
        if (cw)
            padRowsKernel<double><<<(unsigned)((cw + 255) / 256), 256, 0, u->stream>>>(
                u->c.ptr + d.constants_offset, u->c4.ptr + t.constBase[k], d.num_instances, t.stride[k],
                d.num_constant_rows);
    }
    SYMGB_CUDA(cudaGetLastError());
    SYMGB_CUDA(cudaStreamSynchronize(u->stream));
    u->groupedBuilt = true;
    return SYMGB_OK;
}

// The compiled module of schedule `kind` in the unit's current configuration,
// generated and compiled on first use.  `seconds` receives the compile time
// (0 when the module was already loaded).
int getModule(symgb_unit* u, int kind, std::shared_ptr<const JitModule>* out, double* seconds = nullptr) {
    if (seconds) *seconds = 0.0;
    const JitConfig cfg = jitConfig(u, kind);
    if (cfg.itemLayout == SYMGB_ITEMS_GROUPED && u->initialized)
        if (int e = buildGroupedTables(u)) return e;
    const std::string key = jitKeyOf(cfg);
    auto it = u->jitModules.find(key);
    if (it != u->jitModules.end()) {
        *out = it->second;
        return SYMGB_OK;
    }
    std::vector<symgb_kernel_desc> descs;
    for (const auto& k : u->kernels) descs.push_back(k.desc);
    JitSource src;
    try {
        src = generateModule(descs, u->numLevels, cfg);
    } catch (const std::exception& e) {
        return fail(SYMGB_ERR_ARGUMENT, std::string("compiled executor: ") + e.what());
    }
    for (const JitLaunch& L : src.launches)
        if (L.blocks > 0x7fffffffull) return fail(SYMGB_ERR_ARGUMENT, "compiled executor: grid too large");
    std::string err;
    std::shared_ptr<const JitModule> m;
    const auto t0 = std::chrono::steady_clock::now();
    if (int e = loadModule(src, &m, &err)) return fail(e, err);
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    u->jitModules[key] = m;
    *out = m;
    return SYMGB_OK;
}

// Enqueues one evaluation with the compiled executor.  Launches after the
// first overlap their start-up with the previous launch (programmatic
// dependent launch; each kernel waits for its predecessor before reading x).
// With `kernelEvents`, runs the plain module without that overlap and
// records an event before and after each kernel's launch.
int enqueueCompiled(symgb_unit* u, const std::vector<cudaEvent_t>* kernelEvents) {
    std::shared_ptr<const JitModule> m;
    if (int e = getModule(u, kernelEvents ? SYMGB_SCHEDULE_PLAIN : u->sched.kind, &m)) return e;
    const double* x = u->x.ptr;
    double* xw = u->x.ptr;
    const std::uint32_t* p = m->grouped ? u->p4.ptr : u->p.ptr;
    const double* c = m->grouped ? u->c4.ptr : u->c.ptr;
    double* res = m->direct ? u->res.ptr : nullptr;
    const std::uint32_t* dp = m->direct ? u->dp.ptr : nullptr;
    BarrierState* bar = u->barrier.ptr;
    int* hostError = u->errorDev;
    unsigned long long timeoutNs = u->barrierTimeoutNs;
    unsigned extra = u->barrierExtra;
    void* args[] = {(void*)&x,   (void*)&xw,  (void*)&p,         (void*)&c,         (void*)&res,
                    (void*)&dp,  (void*)&bar, (void*)&hostError, (void*)&timeoutNs, (void*)&extra};

    int launches = 0;
    for (std::size_t j = 0; j < m->launches.size(); ++j) {
        const JitLaunch& L = m->launches[j];
        cudaLaunchAttribute at[2];
        unsigned na = 0;
        unsigned grid = (unsigned)L.blocks;
        if (L.cooperative) {
            int perSm = 0;
            SYMGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, m->kernels[j], L.tpb, 0));
            if (perSm < 1) return fail(SYMGB_ERR_ARGUMENT, "persistent schedule: kernel does not fit on an SM");
            if (u->sched.blocks_per_sm > 0) perSm = std::min(perSm, u->sched.blocks_per_sm);
            grid = std::max(1u, std::min<unsigned>(grid, (unsigned)(perSm * u->smCount)));
            at[na].id = cudaLaunchAttributeCooperative;
            at[na].val.cooperative = 1;
            ++na;
        }
        if (j > 0 && !kernelEvents) {
            at[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            at[na].val.programmaticStreamSerializationAllowed = 1;
            ++na;
        }
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(grid);
        cfg.blockDim = dim3((unsigned)L.tpb);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = u->stream;
        cfg.attrs = na ? at : nullptr;
        cfg.numAttrs = na;
        if (kernelEvents && L.kernel >= 0) SYMGB_CUDA(cudaEventRecord((*kernelEvents)[2 * L.kernel], u->stream));
        SYMGB_CUDA(cudaLaunchKernelExC(&cfg, m->kernels[j], args));
        if (kernelEvents && L.kernel >= 0) SYMGB_CUDA(cudaEventRecord((*kernelEvents)[2 * L.kernel + 1], u->stream));
        ++launches;
    }
    u->launchesPerRun = launches;
    u->lastRunDirect = m->direct;
    return SYMGB_OK;
}

// Enqueues one evaluation on the unit's stream.  With `kernelEvents`, runs the
// plain schedule whatever the unit's and records an event before and after
// each kernel's launch (per-kernel timing).
int enqueueRun(symgb_unit* u, const std::vector<cudaEvent_t>* kernelEvents = nullptr) {
    if (u->compiledExec()) return enqueueCompiled(u, kernelEvents);
    u->lastRunDirect = false;
    if (int e = buildTiles(u)) return e;
    const int items = u->items();
    const int tpb = u->launchTpb();
    const int lanes = u->lanes();
    int launches = 0;
    EvalArgs A;
    A.ks = u->devKernels.ptr;
    A.tiles = u->tiles.ptr;
    A.x = u->x.ptr;
    A.xw = u->x.ptr;
    A.S = (unsigned)u->numSets;
    A.barrierExtra = u->barrierExtra;
    A.bar = u->barrier.ptr;
    A.hostError = u->errorDev;
    A.timeoutNs = u->barrierTimeoutNs;
    auto launch = [&](bool l2, std::uint32_t regs, std::uint32_t words, unsigned grid, bool coop,
                      symgb_unit::Shape sh) -> int {
        const int items = sh.items, lanes = sh.lanes, tpb = sh.tpb;
        const void* fn = evalFunction(items, lanes, l2, u->usesLibrary);
        if (!fn) return fail(SYMGB_ERR_ARGUMENT, "several lanes per item need one item per thread");
        const int bt = fitBlock(u, 0, regs, items, tpb, lanes);
        if (!bt) return fail(SYMGB_ERR_ARGUMENT, "kernel register file exceeds shared memory");
        const std::array<std::uint32_t, 6> key{(std::uint32_t)l2, regs, words, (std::uint32_t)items, (std::uint32_t)tpb,
                                                (std::uint32_t)lanes};
        auto it = u->stagingCache.find(key);
        if (it == u->stagingCache.end()) {
            std::uint32_t c = std::min(words, kProgCapWords);
            if (words > kProgCapWords || fitBlock(u, c, regs, items, tpb, lanes) != bt) c = 0;
            it = u->stagingCache.emplace(key, c).first;
        }
        const std::uint32_t cap = it->second;
        const std::size_t smem = smemBytes(cap, regs, items, bt, lanes);
        if (setSmemLimit(fn, smem)) return SYMGB_ERR_CUDA;
        A.progCap = cap;
        if (coop) {
            int perSm = 0;
            SYMGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, fn, bt, smem));
            if (perSm < 1) return fail(SYMGB_ERR_ARGUMENT, "persistent schedule: register file does not fit on an SM");
            if (u->sched.blocks_per_sm > 0) perSm = std::min(perSm, u->sched.blocks_per_sm);
            grid = std::max(1u, std::min<unsigned>(grid, (unsigned)(perSm * u->smCount)));
            void* args[] = {(void*)&A};
            SYMGB_CUDA(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(bt), args, smem, u->stream));
        } else {
            // A CTA loops over tiles; capping the grid makes each CTA take
            // several tiles (fewer CTA launches, one program staging per CTA).
            if (u->sched.blocks_per_sm > 0)
                grid = std::max(1u, std::min<unsigned>(grid, (unsigned)(u->sched.blocks_per_sm * u->smCount)));
            void* args[] = {(void*)&A};
            SYMGB_CUDA(cudaLaunchKernel(fn, dim3(grid), dim3(bt), args, smem, u->stream));
        }
        ++launches;
        return SYMGB_OK;
    };
    const symgb_unit::Shape unitShape{items, lanes, tpb};
    switch (kernelEvents ? SYMGB_SCHEDULE_PLAIN : u->sched.kind) {
        case SYMGB_SCHEDULE_PLAIN: {
            A.segments = u->kernelSeg.ptr;
            for (std::size_t sgi = 0; sgi + 1 < u->hostKernelSeg.size(); ++sgi) {
                const std::uint32_t nt = u->hostKernelSeg[sgi + 1] - u->hostKernelSeg[sgi];
                const std::uint32_t k = u->hostTiles[u->hostKernelSeg[sgi]].kernel;
                A.segBegin = (int)sgi;
                A.segEnd = (int)sgi + 1;
                if (kernelEvents) SYMGB_CUDA(cudaEventRecord((*kernelEvents)[2 * k], u->stream));
                if (int e = launch(false, u->hostDevKernels[k].regs, u->hostDevKernels[k].nwords, nt, false,
                                   u->shapeOf(k)))
                    return e;
                if (kernelEvents) SYMGB_CUDA(cudaEventRecord((*kernelEvents)[2 * k + 1], u->stream));
            }
            break;
        }
        case SYMGB_SCHEDULE_LEVELS: {
            // Consecutive levels in groups of `fusion_depth`; a group of several
            // levels is one cooperative launch with grid barriers between them.
            A.segments = u->levelSeg.ptr;
            const int depth = std::max(1, u->sched.fusion_depth);
            for (int L = 0; L < u->numLevels; L += depth) {
                const int L1 = std::min(u->numLevels, L + depth);
                std::uint32_t maxTiles = 0, regs = 1, words = 0;
                for (int q = L; q < L1; ++q) {
                    maxTiles = std::max(maxTiles, u->hostLevelSeg[q + 1] - u->hostLevelSeg[q]);
                    regs = std::max(regs, maxRegs(u, q));
                    words = std::max(words, maxWords(u, q));
                }
                if (!maxTiles) continue;
                A.segBegin = L;
                A.segEnd = L1;
                // A single level runs in the launch shape of its largest kernel.
                symgb_unit::Shape sh = unitShape;
                if (L1 - L == 1) {
                    double most = -1;
                    for (std::size_t k = 0; k < u->kernels.size(); ++k) {
                        if (u->kernels[k].desc.level != L) continue;
                        const double work = (double)u->kernels[k].desc.num_instances *
                                            (double)(u->kernels[k].prog[u->mathIndex()].operations + 1);
                        if (work > most) {
                            most = work;
                            sh = u->shapeOf(k);
                        }
                    }
                }
                if (int e = launch(L1 - L > 1, regs, words, maxTiles, L1 - L > 1, sh)) return e;
            }
            break;
        }
        case SYMGB_SCHEDULE_PERSISTENT: {
            A.segments = u->levelSeg.ptr;
            A.segBegin = 0;
            A.segEnd = u->numLevels;
            std::uint32_t maxTiles = 1;
            for (int L = 0; L < u->numLevels; ++L)
                maxTiles = std::max(maxTiles, u->hostLevelSeg[L + 1] - u->hostLevelSeg[L]);
            if (int e = launch(true, maxRegs(u), maxWords(u), maxTiles, true, unitShape)) return e;
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
    // A run that writes its results straight into res waits (on the unit's
    // stream) for the asynchronous copies still reading the previous ones.
    if (u->compiledExec() && u->directOutputs && u->directRows && u->numSets == 1)
        for (cudaEvent_t e : u->copyDone)
            if (e) SYMGB_CUDA(cudaStreamWaitEvent(u->stream, e, 0));
    if (u->sched.use_graph) {
        if (!u->graphValid) {
            if (u->compiledExec()) {  // nothing may be compiled or loaded during the capture
                std::shared_ptr<const JitModule> m;
                if (int e = getModule(u, u->sched.kind, &m)) return e;
            }
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
    // The interpreter addresses x slots with 32-bit indices (as the
    // reference's u32 positionData does).
    if (d->num_total_memory > 0xffffffffull) return fail(SYMGB_ERR_ARGUMENT, "plan needs more than 2^32 x slots");
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
            if (hk.prog[0].stats.transcendentals || hk.prog[1].stats.transcendentals) u->usesLibrary = true;
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
    // Every index must address x; checked once here so the kernels need no
    // bounds checks.  The slots some kernel reads are noted for the direct
    // result plan.
    std::vector<std::uint8_t> slotRead(u->numTotalMemory, 0);
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
                slotRead[(std::size_t)slot] = 1;
            }
        }
    }
    for (std::uint64_t j = 0; j < u->numOutputValues; ++j)
        if (out_index_data[j] >= u->numTotalMemory) return fail(SYMGB_ERR_ARGUMENT, "output id outside x");
    u->release();
    u->jitModules.clear();  // their direct result rows belong to the previous tables
    // Direct result plan: an output row is direct when each of its slots is
    // read by no kernel and is the slot of exactly one result position
    // (positions are 32-bit in the table: larger result sets are gathered).
    if (u->numOutputValues < 0xfffffffeull) {
        constexpr std::uint32_t kNone = 0xffffffffu, kMany = 0xfffffffeu;
        std::vector<std::uint32_t> posOf(u->numTotalMemory, kNone);
        for (std::uint64_t j = 0; j < u->numOutputValues; ++j) {
            std::uint32_t& q = posOf[out_index_data[j]];
            q = q == kNone ? (std::uint32_t)j : kMany;
        }
        std::vector<std::uint8_t> covered(u->numOutputValues, 0);
        std::vector<std::uint32_t> dpHost;
        u->directBase.assign(u->kernels.size(), {});
        for (std::size_t k = 0; k < u->kernels.size(); ++k) {
            const auto& d = u->kernels[k].desc;
            const std::uint64_t n = d.num_instances;
            u->directBase[k].assign(d.num_output_rows, -1);
            for (std::uint32_t r = 0; r < d.num_output_rows && n; ++r) {
                const std::uint64_t base = d.output_offset + (std::uint64_t)r * n;
                bool ok = true;
                for (std::uint64_t i = 0; i < n && ok; ++i)
                    ok = !slotRead[base + i] && posOf[base + i] < kMany;
                if (!ok) continue;
                u->directBase[k][r] = (std::int64_t)dpHost.size();
                for (std::uint64_t i = 0; i < n; ++i) {
                    dpHost.push_back(posOf[base + i]);
                    covered[posOf[base + i]] = 1;
                }
            }
        }
        std::vector<std::uint32_t> restPos, restSlot;
        for (std::uint64_t j = 0; j < u->numOutputValues; ++j)
            if (!covered[j]) {
                restPos.push_back((std::uint32_t)j);
                restSlot.push_back(out_index_data[j]);
            }
        u->directRows = !dpHost.empty();
        u->restCount = restPos.size();
        if (u->directRows) {
            SYMGB_CUDA(u->dp.alloc(dpHost.size()));
            SYMGB_CUDA(cudaMemcpy(u->dp.ptr, dpHost.data(), dpHost.size() * 4, cudaMemcpyHostToDevice));
            SYMGB_CUDA(u->res.alloc(u->numOutputValues));
            if (u->restCount) {
                SYMGB_CUDA(u->restPos.alloc(u->restCount));
                SYMGB_CUDA(u->restSlot.alloc(u->restCount));
                SYMGB_CUDA(cudaMemcpy(u->restPos.ptr, restPos.data(), u->restCount * 4, cudaMemcpyHostToDevice));
                SYMGB_CUDA(cudaMemcpy(u->restSlot.ptr, restSlot.data(), u->restCount * 4, cudaMemcpyHostToDevice));
            }
        }
    }
    SYMGB_CUDA(cudaGetDevice(&u->device));
    SYMGB_CUDA(cudaDeviceGetAttribute(&u->smCount, cudaDevAttrMultiProcessorCount, u->device));
    int optin = 0;
    SYMGB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, u->device));
    u->smemOptin = (std::size_t)optin;
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
    if (u->copyStream) SYMGB_CUDA(cudaStreamSynchronize(u->copyStream));
    return checkDeviceError(u);
}

static int ensureOutBuf(symgb_unit* u, std::size_t n) {
    if (u->outBuf.count < n) SYMGB_CUDA(u->outBuf.alloc(n));
    return SYMGB_OK;
}

// When the last run wrote its results straight into res (compiled executor,
// one value set), completes res with the other rows' results on the unit's
// stream and returns true: the results are then read from res.
static bool resultsInRes(symgb_unit* u, int* err) {
    *err = SYMGB_OK;
    if (!u->lastRunDirect || u->numSets != 1) return false;
    if (u->restCount) {
        restGatherKernel<<<(unsigned)((u->restCount + 255) / 256), 256, 0, u->stream>>>(
            u->x.ptr, u->restPos.ptr, u->restSlot.ptr, u->restCount, u->res.ptr);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) *err = fail(SYMGB_ERR_CUDA, std::string("rest gather: ") + cudaGetErrorString(e));
    }
    return true;
}

int symgb_get_result_sets_device(symgb_unit_t u, double* d, int k) {
    if (!u || !u->initialized) return fail(SYMGB_ERR_STATE, "get_result before init");
    if (k < 0 || (std::size_t)k >= u->outStart.size() || !d) return fail(SYMGB_ERR_ARGUMENT, "bad result index");
    int err = SYMGB_OK;
    if (resultsInRes(u, &err)) {
        if (err) return err;
        if (u->outLength[k])
            SYMGB_CUDA(cudaMemcpyAsync(d, u->res.ptr + u->outStart[k], u->outLength[k] * 8, cudaMemcpyDefault,
                                       u->stream));
        return SYMGB_OK;
    }
    const std::uint64_t len = u->outLength[k];
    const std::uint64_t work = len * u->numSets;
    if (work && u->numSets >= kTiledSets) {
        const dim3 grid((unsigned)((len + kSetTile - 1) / kSetTile), (unsigned)((u->numSets + kSetTile - 1) / kSetTile));
        gatherSetsKernel<<<grid, 256, 0, u->stream>>>(u->x.ptr, u->ids.ptr + u->outStart[k], len, (unsigned)u->numSets, d);
        SYMGB_CUDA(cudaGetLastError());
    } else if (work) {
        gatherKernel<<<(unsigned)((work + 255) / 256), 256, 0, u->stream>>>(u->x.ptr, u->ids.ptr + u->outStart[k], len,
                                                                            (unsigned)u->numSets, d);
        SYMGB_CUDA(cudaGetLastError());
    }
    return SYMGB_OK;
}

// Device-side address of a page-locked host buffer (cudaHostAlloc or
// cudaHostRegister with mapping), or null for any other pointer.
static double* mappedHost(double* d) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, d) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? static_cast<double*>(a.devicePointer) : nullptr;
}

int symgb_get_result_sets(symgb_unit_t u, double* d, int k) {
    if (!u || !u->initialized) return fail(SYMGB_ERR_STATE, "get_result before init");
    if (k < 0 || (std::size_t)k >= u->outStart.size() || !d) return fail(SYMGB_ERR_ARGUMENT, "bad result index");
    // Page-locked destination: the gather writes the results there directly
    // (one pass over the outputs instead of gather + copy).
    if (double* dd = mappedHost(d)) {
        if (int e = symgb_get_result_sets_device(u, dd, k)) return e;
        SYMGB_CUDA(cudaStreamSynchronize(u->stream));
        return checkDeviceError(u);
    }
    const std::size_t n = u->outLength[k] * (std::size_t)u->numSets;
    int err = SYMGB_OK;
    if (resultsInRes(u, &err)) {
        if (err) return err;
        if (n) SYMGB_CUDA(cudaMemcpyAsync(d, u->res.ptr + u->outStart[k], n * 8, cudaMemcpyDeviceToHost, u->stream));
        SYMGB_CUDA(cudaStreamSynchronize(u->stream));
        return checkDeviceError(u);
    }
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
    if (work && u->numSets >= kTiledSets) {
        const dim3 grid((unsigned)((len + kSetTile - 1) / kSetTile), (unsigned)((u->numSets + kSetTile - 1) / kSetTile));
        scatterSetsKernel<<<grid, 256, 0, u->stream>>>(d, u->argStart[i], len, (unsigned)u->numSets, u->x.ptr);
        SYMGB_CUDA(cudaGetLastError());
    } else if (work) {
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

int symgb_set_arg_sets_async(symgb_unit_t u, const double* d, int i) {
    if (!u || !u->initialized) return fail(SYMGB_ERR_STATE, "set_arg before init");
    if (i < 0 || (std::size_t)i >= u->argStart.size() || !d) return fail(SYMGB_ERR_ARGUMENT, "bad argument index");
    if (!mappedHost(const_cast<double*>(d))) return fail(SYMGB_ERR_ARGUMENT, "async set_arg needs page-locked memory");
    const std::size_t n = u->argLength[i] * (std::size_t)u->numSets;
    if (u->numSets == 1) {
        SYMGB_CUDA(cudaMemcpyAsync(u->x.ptr + u->argStart[i], d, n * 8, cudaMemcpyHostToDevice, u->stream));
        return SYMGB_OK;
    }
    if (u->staging.count < n) {
        SYMGB_CUDA(cudaStreamSynchronize(u->stream));  // the staging buffer may be in use
        SYMGB_CUDA(u->staging.alloc(n));
    }
    SYMGB_CUDA(cudaMemcpyAsync(u->staging.ptr, d, n * 8, cudaMemcpyHostToDevice, u->stream));
    return symgb_set_arg_sets_device(u, u->staging.ptr, i);
}

// The result is gathered on the unit's stream into a device buffer (or, when
// the run wrote it straight into res, taken from there) and copied to the
// host by the copy engine on the unit's copy stream, which the unit's stream
// does not wait for: the next execute's input copy and evaluation overlap
// this one's result copy.  (Gathering straight into page-locked memory
// would hold SMs for the whole transfer over the host link.)
int symgb_get_result_sets_async(symgb_unit_t u, double* d, int k) {
    if (!u || !u->initialized) return fail(SYMGB_ERR_STATE, "get_result before init");
    if (k < 0 || (std::size_t)k >= u->outStart.size() || !d) return fail(SYMGB_ERR_ARGUMENT, "bad result index");
    if (!mappedHost(d)) return fail(SYMGB_ERR_ARGUMENT, "async get_result needs page-locked memory");
    const std::size_t nk = u->outStart.size();
    if (!u->copyStream) {
        SYMGB_CUDA(cudaStreamCreateWithFlags(&u->copyStream, cudaStreamNonBlocking));
        SYMGB_CUDA(cudaEventCreateWithFlags(&u->gatherDone, cudaEventDisableTiming));
        u->copyDone.assign(nk, nullptr);
    }
    if (u->asyncOutSets != u->numSets) {
        SYMGB_CUDA(cudaStreamSynchronize(u->copyStream));  // copies may still read the old buffer
        std::size_t total = 0;
        for (std::size_t j = 0; j < nk; ++j) total += u->outLength[j];
        SYMGB_CUDA(u->asyncOut.alloc(std::max<std::size_t>(1, total * (std::size_t)u->numSets)));
        u->asyncOutSets = u->numSets;
    }
    std::size_t off = 0;
    for (int j = 0; j < k; ++j) off += u->outLength[j];
    off *= (std::size_t)u->numSets;
    const std::size_t n = u->outLength[k] * (std::size_t)u->numSets;
    double* buf = u->asyncOut.ptr + off;
    if (u->copyDone[k]) {
        SYMGB_CUDA(cudaStreamWaitEvent(u->stream, u->copyDone[k], 0));
    } else {
        SYMGB_CUDA(cudaEventCreateWithFlags(&u->copyDone[k], cudaEventDisableTiming));
    }
    // Results written straight into res are copied from there (the next run
    // waits for this copy before it rewrites res).
    int err = SYMGB_OK;
    if (resultsInRes(u, &err)) {
        if (err) return err;
        buf = u->res.ptr + u->outStart[k];
    } else if (int e = symgb_get_result_sets_device(u, buf, k)) {
        return e;
    }
    SYMGB_CUDA(cudaEventRecord(u->gatherDone, u->stream));
    // Chunks of at least 8 MiB, one per copy stream in use.
    const std::size_t minChunk = (8u << 20) / 8;
    const std::size_t chunks = std::max<std::size_t>(1, std::min<std::size_t>((std::size_t)u->copyStreams, n / minChunk));
    while (u->extraCopy.size() + 1 < chunks) {
        cudaStream_t st;
        cudaEvent_t ev;
        SYMGB_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        SYMGB_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        u->extraCopy.push_back(st);
        u->extraDone.push_back(ev);
    }
    const std::size_t per = (n + chunks - 1) / chunks;
    for (std::size_t c = 0; c < chunks; ++c) {
        cudaStream_t st = c == 0 ? u->copyStream : u->extraCopy[c - 1];
        const std::size_t b0 = c * per, len = std::min(n, b0 + per) - std::min(n, b0);
        SYMGB_CUDA(cudaStreamWaitEvent(st, u->gatherDone, 0));
        if (len) SYMGB_CUDA(cudaMemcpyAsync(d + b0, buf + b0, len * 8, cudaMemcpyDeviceToHost, st));
        if (c > 0) {
            SYMGB_CUDA(cudaEventRecord(u->extraDone[c - 1], st));
            SYMGB_CUDA(cudaStreamWaitEvent(u->copyStream, u->extraDone[c - 1], 0));
        }
    }
    SYMGB_CUDA(cudaEventRecord(u->copyDone[k], u->copyStream));
    return SYMGB_OK;
}

int symgb_set_direct_outputs(symgb_unit_t u, int on) {
    if (!u || (on != 0 && on != 1)) return fail(SYMGB_ERR_ARGUMENT, "direct outputs must be 0 or 1");
    if ((bool)on != u->directOutputs) {
        u->directOutputs = on;
        u->dropGraph();
    }
    return SYMGB_OK;
}

int symgb_set_item_layout(symgb_unit_t u, int layout) {
    if (!u || (layout != SYMGB_ITEMS_STRIDED && layout != SYMGB_ITEMS_GROUPED))
        return fail(SYMGB_ERR_ARGUMENT, "bad item layout");
    if (layout != u->itemLayout) {
        u->itemLayout = layout;
        u->dropGraph();
    }
    return SYMGB_OK;
}

int symgb_set_load_path(symgb_unit_t u, int path) {
    if (!u || path < SYMGB_LOAD_READONLY || path > SYMGB_LOAD_L2) return fail(SYMGB_ERR_ARGUMENT, "bad load path");
    if (path != u->loadPath) {
        u->loadPath = path;
        u->dropGraph();
    }
    return SYMGB_OK;
}

int symgb_set_copy_streams(symgb_unit_t u, int n) {
    if (!u || n < 1 || n > 8) return fail(SYMGB_ERR_ARGUMENT, "copy streams must be in [1, 8]");
    u->copyStreams = n;
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
    if (s->items_per_thread != 0 && s->items_per_thread != 1 && s->items_per_thread != 2 && s->items_per_thread != 4)
        return fail(SYMGB_ERR_ARGUMENT, "items_per_thread must be 1, 2 or 4");
    if (s->items_per_tile < 0 || s->blocks_per_sm < 0 || s->fusion_depth < 0)
        return fail(SYMGB_ERR_ARGUMENT, "negative schedule parameter");
    if (s->threads_per_block < 0 || s->threads_per_block > 1024 || (s->threads_per_block % 32))
        return fail(SYMGB_ERR_ARGUMENT, "threads_per_block must be a multiple of 32 up to 1024");
    if (s->lanes_per_item != 0 && s->lanes_per_item != 1 && s->lanes_per_item != 2 && s->lanes_per_item != 4 &&
        s->lanes_per_item != 8)
        return fail(SYMGB_ERR_ARGUMENT, "lanes_per_item must be 1, 2, 4 or 8");
    if (s->lanes_per_item > 1 && s->items_per_thread > 1)
        return fail(SYMGB_ERR_ARGUMENT, "several lanes per item need one item per thread");
    if (s->executor != SYMGB_EXEC_COMPILED && s->executor != SYMGB_EXEC_INTERPRETER)
        return fail(SYMGB_ERR_ARGUMENT, "unknown executor");
    const bool mathChanged = s->math != u->sched.math;
    u->sched = *s;
    u->dropGraph();
    u->tilesSets = -1;
    if (mathChanged && u->initialized) return uploadPrograms(u);
    return SYMGB_OK;
}

int symgb_set_kernel_shape(symgb_unit_t u, int k, int items_per_thread, int lanes_per_item, int threads_per_block) {
    if (!u) return fail(SYMGB_ERR_ARGUMENT, "null unit");
    if (k < 0 || (std::size_t)k >= u->kernels.size()) return fail(SYMGB_ERR_ARGUMENT, "bad kernel index");
    if (items_per_thread != 0 && items_per_thread != 1 && items_per_thread != 2 && items_per_thread != 4)
        return fail(SYMGB_ERR_ARGUMENT, "items_per_thread must be 0, 1, 2 or 4");
    if (lanes_per_item != 0 && lanes_per_item != 1 && lanes_per_item != 2 && lanes_per_item != 4 && lanes_per_item != 8)
        return fail(SYMGB_ERR_ARGUMENT, "lanes_per_item must be 0, 1, 2, 4 or 8");
    if (lanes_per_item > 1 && items_per_thread > 1)
        return fail(SYMGB_ERR_ARGUMENT, "several lanes per item need one item per thread");
    if (threads_per_block < 0 || threads_per_block > 1024 || (threads_per_block % 32))
        return fail(SYMGB_ERR_ARGUMENT, "threads_per_block must be a multiple of 32 up to 1024");
    u->kernelShape.resize(u->kernels.size(), symgb_unit::Shape{0, 0, 0});
    u->kernelShape[k] = symgb_unit::Shape{items_per_thread, lanes_per_item, threads_per_block};
    ++u->shapesVersion;
    u->dropGraph();
    return SYMGB_OK;
}

int symgb_prepare(symgb_unit_t u, double* compile_seconds) {
    if (compile_seconds) *compile_seconds = 0.0;
    if (!u) return fail(SYMGB_ERR_ARGUMENT, "null unit");
    if (!u->compiledExec()) return SYMGB_OK;
    std::shared_ptr<const JitModule> m;
    return getModule(u, u->sched.kind, &m, compile_seconds);
}

int64_t symgb_compiled_source(symgb_unit_t u, int kind, char* buf, uint64_t cap) {
    if (!u || kind < 0 || kind > 2) return fail(SYMGB_ERR_ARGUMENT, "bad unit or schedule kind");
    std::vector<symgb_kernel_desc> descs;
    for (const auto& k : u->kernels) descs.push_back(k.desc);
    std::string src;
    try {
        src = generateModule(descs, u->numLevels, jitConfig(u, kind)).source;
    } catch (const std::exception& e) {
        return fail(SYMGB_ERR_ARGUMENT, std::string("compiled executor: ") + e.what());
    }
    if (buf && cap) {
        const std::size_t n = std::min<std::size_t>(cap, src.size() + 1);
        std::memcpy(buf, src.c_str(), n);
    }
    return (int64_t)src.size();
}

int symgb_compile_check(symgb_unit_t u, int kind, double* seconds) {
    if (seconds) *seconds = 0.0;
    if (!u || kind < 0 || kind > 2) return fail(SYMGB_ERR_ARGUMENT, "bad unit or schedule kind");
    std::vector<symgb_kernel_desc> descs;
    for (const auto& k : u->kernels) descs.push_back(k.desc);
    std::string src, err;
    try {
        src = generateModule(descs, u->numLevels, jitConfig(u, kind)).source;
    } catch (const std::exception& e) {
        return fail(SYMGB_ERR_ARGUMENT, std::string("compiled executor: ") + e.what());
    }
    if (int e = compileOnly(src, seconds, &err)) return fail(e, err);
    return SYMGB_OK;
}

int symgb_compiled_registers(symgb_unit_t u, int kind, int* registers, int cap) {
    if (!u || kind < 0 || kind > 2 || cap < 0 || (cap > 0 && !registers)) return fail(SYMGB_ERR_ARGUMENT, "bad argument");
    if (!u->initialized) return fail(SYMGB_ERR_STATE, "compiled_registers before init");
    std::shared_ptr<const JitModule> m;
    if (int e = getModule(u, kind, &m)) return e;
    for (int i = 0; i < cap && i < (int)m->registers.size(); ++i) registers[i] = m->registers[i];
    return (int)m->registers.size();
}

int symgb_set_barrier_limits(symgb_unit_t u, uint64_t timeout_ns, int extra_arrivals) {
    if (!u || timeout_ns == 0 || extra_arrivals < 0) return fail(SYMGB_ERR_ARGUMENT, "bad barrier limits");
    u->barrierTimeoutNs = timeout_ns;
    u->barrierExtra = (unsigned)extra_arrivals;
    u->dropGraph();
    return SYMGB_OK;
}

int symgb_time_kernels(symgb_unit_t u, int reps, void* flush, uint64_t flush_bytes, double* us_per_kernel) {
    if (!u || !us_per_kernel || reps < 1) return fail(SYMGB_ERR_ARGUMENT, "bad argument");
    if (!u->initialized) return fail(SYMGB_ERR_STATE, "time_kernels before init");
    if (int e = buildTiles(u)) return e;
    const std::size_t nk = u->kernels.size();
    const std::size_t per = 2 * nk;
    while (u->timingEvents.size() < per * (std::size_t)reps) {
        cudaEvent_t ev;
        SYMGB_CUDA(cudaEventCreate(&ev));
        u->timingEvents.push_back(ev);
    }
    for (std::size_t k = 0; k < nk; ++k) us_per_kernel[k] = 0.0;
    for (int r = 0; r < reps; ++r) {
        if (flush && flush_bytes) SYMGB_CUDA(cudaMemsetAsync(flush, r & 0xff, flush_bytes, u->stream));
        const std::vector<cudaEvent_t> evs(u->timingEvents.begin() + per * r, u->timingEvents.begin() + per * (r + 1));
        // kernels without work are not launched: their two events are recorded back to back
        for (std::size_t k = 0; k < nk; ++k)
            if (!u->kernels[k].desc.num_instances) {
                SYMGB_CUDA(cudaEventRecord(evs[2 * k], u->stream));
                SYMGB_CUDA(cudaEventRecord(evs[2 * k + 1], u->stream));
            }
        if (int e = enqueueRun(u, &evs)) return e;
    }
    SYMGB_CUDA(cudaStreamSynchronize(u->stream));
    for (int r = 0; r < reps; ++r)
        for (std::size_t k = 0; k < nk; ++k) {
            float ms = 0.f;
            SYMGB_CUDA(cudaEventElapsedTime(&ms, u->timingEvents[per * r + 2 * k], u->timingEvents[per * r + 2 * k + 1]));
            us_per_kernel[k] += ms * 1e3 / reps;
        }
    return checkDeviceError(u);
}

int symgb_get_schedule(symgb_unit_t u, symgb_schedule* s) {
    if (!u || !s) return fail(SYMGB_ERR_ARGUMENT, "null argument");
    *s = u->sched;
    return SYMGB_OK;
}

int symgb_set_num_sets(symgb_unit_t u, int num_sets) {
    if (!u || num_sets < 1 || num_sets > (1 << 20)) return fail(SYMGB_ERR_ARGUMENT, "num_sets must be in [1, 2^20]");
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
        s->bundles += (std::uint64_t)k.prog[mi].bundles * d.num_instances;
        s->bundle_entries += (std::uint64_t)k.prog[mi].operations * d.num_instances;
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

struct symgb_batch {
    std::vector<symgb_unit_t> units;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    int launches = 0;
    ~symgb_batch() {
        if (exec) cudaGraphExecDestroy(exec);
        if (stream) cudaStreamDestroy(stream);
    }
};

int symgb_batch_create(symgb_unit_t* units, int n, int streams, symgb_batch_t* out) {
    if (!out || !units || n <= 0) return fail(SYMGB_ERR_ARGUMENT, "empty batch");
    *out = nullptr;
    streams = std::max(1, std::min(streams, 32));
    std::unique_ptr<symgb_batch> b(new symgb_batch());
    for (int i = 0; i < n; ++i) {
        if (!units[i] || !units[i]->initialized) return fail(SYMGB_ERR_STATE, "batch unit not initialized");
        if (int e = buildTiles(units[i])) return e;  // no allocation may happen inside the capture
        if (units[i]->compiledExec()) {               // nor any compilation or module load
            std::shared_ptr<const JitModule> m;
            if (int e = getModule(units[i], units[i]->sched.kind, &m)) return e;
        }
        b->units.push_back(units[i]);
    }
    SYMGB_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    std::vector<cudaStream_t> branch(streams);
    std::vector<cudaEvent_t> done(streams);
    cudaEvent_t fork;
    SYMGB_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    for (int k = 0; k < streams; ++k) {
        SYMGB_CUDA(cudaStreamCreateWithFlags(&branch[k], cudaStreamNonBlocking));
        SYMGB_CUDA(cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming));
    }
    // Fork: every branch waits on the capture stream; units go round-robin.
    int err = SYMGB_OK;
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        err = fail(SYMGB_ERR_CUDA, "batch: begin capture failed");
    } else {
        cudaEventRecord(fork, b->stream);
        for (int k = 0; k < streams; ++k) cudaStreamWaitEvent(branch[k], fork, 0);
        for (int i = 0; i < n && !err; ++i) {
            symgb_unit* u = b->units[i];
            cudaStream_t saved = u->stream;
            u->stream = branch[i % streams];
            err = enqueueRun(u);
            u->stream = saved;
            b->launches += u->launchesPerRun;
        }
        for (int k = 0; k < streams; ++k) {
            cudaEventRecord(done[k], branch[k]);
            cudaStreamWaitEvent(b->stream, done[k], 0);
        }
        const cudaError_t ce = cudaStreamEndCapture(b->stream, &graph);
        if (!err && ce != cudaSuccess) err = fail(SYMGB_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(ce));
    }
    if (!err && cudaGraphInstantiate(&b->exec, graph, 0) != cudaSuccess) err = fail(SYMGB_ERR_CUDA, "batch: graph instantiation failed");
    if (graph) cudaGraphDestroy(graph);
    cudaEventDestroy(fork);
    for (int k = 0; k < streams; ++k) {
        cudaEventDestroy(done[k]);
        cudaStreamDestroy(branch[k]);
    }
    if (err) return err;
    *out = b.release();
    return SYMGB_OK;
}

int symgb_batch_run_async(symgb_batch_t b, void* stream) {
    if (!b) return fail(SYMGB_ERR_ARGUMENT, "null batch");
    SYMGB_CUDA(cudaGraphLaunch(b->exec, stream ? (cudaStream_t)stream : b->stream));
    return SYMGB_OK;
}

int symgb_batch_run(symgb_batch_t b) {
    if (int e = symgb_batch_run_async(b, nullptr)) return e;
    SYMGB_CUDA(cudaStreamSynchronize(b->stream));
    for (auto* u : b->units)
        if (int e = checkDeviceError(u)) return e;
    return SYMGB_OK;
}

int symgb_batch_launch_count(symgb_batch_t b) { return b ? b->launches : 0; }

void symgb_batch_destroy(symgb_batch_t b) {
    if (!b) return;
    cudaStreamSynchronize(b->stream);
    delete b;
}

int64_t symgb_kernel_program(symgb_unit_t u, int k, int math, uint64_t* words, uint64_t cap, int* registers,
                             int* num_loads) {
    if (!u || k < 0 || (std::size_t)k >= u->kernels.size() || math < 0 || math > 1)
        return fail(SYMGB_ERR_ARGUMENT, "bad kernel or math mode");
    const Program& pr = u->kernels[k].prog[math];
    std::vector<std::uint64_t> all(pr.loads);
    all.insert(all.end(), pr.words.begin(), pr.words.end());
    if (words) std::memcpy(words, all.data(), std::min<std::uint64_t>(cap, all.size()) * sizeof(std::uint64_t));
    if (registers) *registers = pr.registers;
    if (num_loads) *num_loads = (int)pr.loads.size();
    return (int64_t)all.size();
}

}  // extern "C"
