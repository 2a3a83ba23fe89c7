// Allocation-free evaluation entry point (symgb_run_static).
//
// Some callers cannot call cudaMalloc: code running under a framework that owns
// all device memory through its own pool, code that must not allocate once set
// up (real-time loops), and code whose memory budget forbids new allocations.
// They still own device buffers for their inputs and outputs, but the engine's
// normal path (symgb_init) allocates its working memory - the x array with all
// intermediate values, the index and constant tables, the device programs, the
// tile table and the grid-barrier state.  This entry point keeps all of that in
// one file-scope device array of SYMGB_STATIC_SCRATCH_BYTES, reserved on every
// GPU that loads this module until the process exits, and calls no cudaMalloc,
// cudaFree or other allocating routine.
//
// Host code cannot use the array's name as a device address: on the host it is
// only a stand-in symbol.  The device address is obtained once per device with
// cudaGetSymbolAddress (the first call on a device does this, so make that first
// call before any stream capture) and passed to the kernels.  Every call shares
// the array and leaves its contents behind; the barrier state is cleared at the
// start of each call.  Calls whose GPU work overlaps (different host threads or
// streams) race on the array; serialise them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "device.cuh"
#include "kernels.hpp"
#include "program.hpp"
#include "symgb.h"
#include "unit.hpp"

static __device__ __align__(256) unsigned char g_staticScratch[SYMGB_STATIC_SCRATCH_BYTES];

namespace {

using namespace symgb::engine;

// Errors are reported through symgb_last_error(), like every other call.
int failStatic(int code, const std::string& msg) { return symgb::engine::setLastError(code, msg); }

#define STATIC_CUDA(call)                                                                            \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return failStatic(SYMGB_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

constexpr int kMaxDevices = 64;
std::mutex g_addrMutex;
void* g_scratchAddr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once.
int scratchAddress(int dev, unsigned char** out) {
    if (dev < 0 || dev >= kMaxDevices) return failStatic(SYMGB_ERR_ARGUMENT, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_addrMutex);
    if (!g_scratchAddr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_staticScratch);
        if (e != cudaSuccess || !p)
            return failStatic(SYMGB_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_scratchAddr[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_scratchAddr[dev]);
    return SYMGB_OK;
}

// Bump layout of the scratch array, every region 256-byte aligned.
struct Layout {
    std::size_t used = 0;
    std::size_t take(std::size_t bytes) {
        const std::size_t at = used;
        used = (used + bytes + 255) & ~std::size_t(255);
        return at;
    }
};

}  // namespace

extern "C" int symgb_run_static(symgb_unit_t u, const uint32_t* index_data, const uint32_t* out_index_data,
                                const double* const_data, const double* const* inputs, double* const* outputs,
                                void* stream_) {
    if (!u) return failStatic(SYMGB_ERR_ARGUMENT, "null unit");
    if ((u->numIndices && !index_data) || (u->numOutputValues && !out_index_data) || (u->numConstants && !const_data))
        return failStatic(SYMGB_ERR_ARGUMENT, "null table");
    if (!inputs || !outputs) return failStatic(SYMGB_ERR_ARGUMENT, "null input or output list");
    for (std::size_t i = 0; i < u->argStart.size(); ++i)
        if (!inputs[i] && u->argLength[i]) return failStatic(SYMGB_ERR_ARGUMENT, "null input pointer");
    for (std::size_t k = 0; k < u->outStart.size(); ++k)
        if (!outputs[k] && u->outLength[k]) return failStatic(SYMGB_ERR_ARGUMENT, "null output pointer");
    cudaStream_t stream = (cudaStream_t)stream_;

    // Programs of the unit's math mode, tiles and level segments (host images).
    const int mi = u->mathIndex();
    const int items = u->items();
    const int tileItems = u->sched.items_per_tile > 0 ? u->sched.items_per_tile : u->tpb() * items;
    std::vector<std::uint64_t> progWords;
    std::vector<std::size_t> progOff;
    std::uint32_t maxWords = 0, maxRegs = 1;
    for (const auto& k : u->kernels) {
        const Program& pr = k.prog[mi];
        progOff.push_back(progWords.size());
        progWords.insert(progWords.end(), pr.loads.begin(), pr.loads.end());
        progWords.insert(progWords.end(), pr.words.begin(), pr.words.end());
        maxWords = std::max<std::uint32_t>(maxWords, (std::uint32_t)(pr.loads.size() + pr.words.size()));
        maxRegs = std::max<std::uint32_t>(maxRegs, (std::uint32_t)std::max(1, pr.registers));
    }
    std::vector<Tile> tiles;
    std::vector<std::uint32_t> segments(1, 0);
    for (int L = 0; L < u->numLevels; ++L) {
        for (std::size_t k = 0; k < u->kernels.size(); ++k) {
            if (u->kernels[k].desc.level != L) continue;
            const std::uint64_t total = u->kernels[k].desc.num_instances;
            for (std::uint64_t st = 0; st < total; st += tileItems)
                tiles.push_back({(std::uint32_t)k, (std::uint32_t)std::min<std::uint64_t>(tileItems, total - st), st});
        }
        segments.push_back((std::uint32_t)tiles.size());
    }

    // Scratch layout and the size limit.
    Layout lay;
    const std::size_t oKernels = lay.take(sizeof(DevKernel) * std::max<std::size_t>(1, u->kernels.size()));
    const std::size_t oProg = lay.take(8 * std::max<std::size_t>(1, progWords.size()));
    const std::size_t oTiles = lay.take(sizeof(Tile) * std::max<std::size_t>(1, tiles.size()));
    const std::size_t oSeg = lay.take(4 * segments.size());
    const std::size_t oIdx = lay.take(4 * std::max<std::uint64_t>(1, u->numIndices));
    const std::size_t oConst = lay.take(8 * std::max<std::uint64_t>(1, u->numConstants));
    const std::size_t oIds = lay.take(4 * std::max<std::uint64_t>(1, u->numOutputValues));
    const std::size_t oBar = lay.take(sizeof(BarrierState) + sizeof(int));
    const std::size_t oX = lay.take(8 * std::max<std::uint64_t>(1, u->numTotalMemory));
    if (lay.used > (std::size_t)SYMGB_STATIC_SCRATCH_BYTES)
        return failStatic(SYMGB_ERR_ARGUMENT, "plan needs " + std::to_string(lay.used) +
                                                  " bytes of scratch; the allocation-free entry point has " +
                                                  std::to_string((unsigned long long)SYMGB_STATIC_SCRATCH_BYTES));

    // Every index must address x (checked on the host; the kernels do not check).
    for (const auto& k : u->kernels) {
        const auto& d = k.desc;
        for (std::uint32_t a = 0; a < d.num_access; ++a) {
            const std::uint32_t row = (std::uint32_t)k.access[2 * a];
            const long long off = k.access[2 * a + 1];
            const std::uint32_t* pr = index_data + d.index_offset + (std::uint64_t)row * d.num_instances;
            for (std::uint64_t i = 0; i < d.num_instances; ++i) {
                const long long slot = (long long)pr[i] + off;
                if (slot < 0 || (std::uint64_t)slot >= u->numTotalMemory)
                    return failStatic(SYMGB_ERR_ARGUMENT, "index table entry outside x");
            }
        }
    }
    for (std::uint64_t j = 0; j < u->numOutputValues; ++j)
        if (out_index_data[j] >= u->numTotalMemory) return failStatic(SYMGB_ERR_ARGUMENT, "output id outside x");

    int dev = 0, sms = 0, optin = 0;
    STATIC_CUDA(cudaGetDevice(&dev));
    STATIC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    STATIC_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    unsigned char* base = nullptr;
    if (int e = scratchAddress(dev, &base)) return e;

    std::vector<DevKernel> dks;
    for (std::size_t k = 0; k < u->kernels.size(); ++k) {
        const auto& d = u->kernels[k].desc;
        const Program& pr = u->kernels[k].prog[mi];
        DevKernel dk;
        dk.prog = reinterpret_cast<const std::uint64_t*>(base + oProg) + progOff[k];
        dk.p = reinterpret_cast<const std::uint32_t*>(base + oIdx) + d.index_offset;
        dk.c = reinterpret_cast<const double*>(base + oConst) + d.constants_offset;
        dk.yoff = d.output_offset;
        dk.n = d.num_instances;
        dk.regs = (std::uint32_t)std::max(1, pr.registers);
        dk.nloads = (std::uint32_t)pr.loads.size();
        dk.nwords = (std::uint32_t)(pr.loads.size() + pr.words.size());
        dk.litoff = (std::uint32_t)(pr.loads.size() + pr.literalOffset);
        dks.push_back(dk);
    }

    // Uploads (plain copies into the array; nothing is allocated).
    if (!dks.empty()) STATIC_CUDA(cudaMemcpyAsync(base + oKernels, dks.data(), dks.size() * sizeof(DevKernel), cudaMemcpyHostToDevice, stream));
    if (!progWords.empty()) STATIC_CUDA(cudaMemcpyAsync(base + oProg, progWords.data(), progWords.size() * 8, cudaMemcpyHostToDevice, stream));
    if (!tiles.empty()) STATIC_CUDA(cudaMemcpyAsync(base + oTiles, tiles.data(), tiles.size() * sizeof(Tile), cudaMemcpyHostToDevice, stream));
    STATIC_CUDA(cudaMemcpyAsync(base + oSeg, segments.data(), segments.size() * 4, cudaMemcpyHostToDevice, stream));
    if (u->numIndices) STATIC_CUDA(cudaMemcpyAsync(base + oIdx, index_data, u->numIndices * 4, cudaMemcpyHostToDevice, stream));
    if (u->numConstants) STATIC_CUDA(cudaMemcpyAsync(base + oConst, const_data, u->numConstants * 8, cudaMemcpyHostToDevice, stream));
    if (u->numOutputValues) STATIC_CUDA(cudaMemcpyAsync(base + oIds, out_index_data, u->numOutputValues * 4, cudaMemcpyHostToDevice, stream));
    STATIC_CUDA(cudaMemsetAsync(base + oBar, 0, sizeof(BarrierState) + sizeof(int), stream));  // must start at zero
    double* x = reinterpret_cast<double*>(base + oX);
    for (std::size_t i = 0; i < u->argStart.size(); ++i)
        if (u->argLength[i])
            STATIC_CUDA(cudaMemcpyAsync(x + u->argStart[i], inputs[i], u->argLength[i] * 8, cudaMemcpyDeviceToDevice, stream));

    // One cooperative launch over all levels (the persistent schedule).
    if (!tiles.empty()) {
        const std::uint32_t progCap = std::min<std::uint32_t>(maxWords, 4096);
        int bt = u->tpb();
        auto smemFor = [&](int t) { return (std::size_t)progCap * 8 + (std::size_t)maxRegs * items * t * 8; };
        while (bt >= 32 && smemFor(bt) > (std::size_t)optin) bt -= 32;
        if (bt < 32) return failStatic(SYMGB_ERR_ARGUMENT, "kernel register file exceeds shared memory");
        const std::size_t smem = smemFor(bt);
        const void* fn = symgb::engine::evalKernelFor(items, 1, MODE_L2 | (u->usesLibrary ? MODE_LIB : 0));
        if (!fn) return failStatic(SYMGB_ERR_ARGUMENT, "unsupported items per thread");
        if (smem > 48 * 1024) STATIC_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int perSm = 0;
        STATIC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, fn, bt, smem));
        if (perSm < 1) return failStatic(SYMGB_ERR_ARGUMENT, "register file does not fit on an SM");
        std::uint32_t maxTiles = 1;
        for (std::size_t L = 0; L + 1 < segments.size(); ++L) maxTiles = std::max(maxTiles, segments[L + 1] - segments[L]);
        const unsigned grid = std::max(1u, std::min<unsigned>(maxTiles, (unsigned)(perSm * sms)));
        EvalArgs A;
        A.ks = reinterpret_cast<const DevKernel*>(base + oKernels);
        A.tiles = reinterpret_cast<const Tile*>(base + oTiles);
        A.segments = reinterpret_cast<const std::uint32_t*>(base + oSeg);
        A.segBegin = 0;
        A.segEnd = u->numLevels;
        A.x = x;
        A.xw = x;
        A.S = 1;
        A.progCap = progCap;
        A.barrierExtra = 0;
        A.bar = reinterpret_cast<BarrierState*>(base + oBar);
        A.hostError = reinterpret_cast<int*>(base + oBar + sizeof(BarrierState));
        A.timeoutNs = u->barrierTimeoutNs;
        void* args[] = {(void*)&A};
        STATIC_CUDA(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(bt), args, smem, stream));
    }
    const std::uint32_t* ids = reinterpret_cast<const std::uint32_t*>(base + oIds);
    for (std::size_t k = 0; k < u->outStart.size(); ++k) {
        const std::uint64_t len = u->outLength[k];
        if (len)
            gatherKernel<<<(unsigned)((len + 255) / 256), 256, 0, stream>>>(x, ids + u->outStart[k], len, 1u, outputs[k]);
    }
    STATIC_CUDA(cudaGetLastError());
    // The status word is read back on the caller's stream, so the call waits
    // for its own work only, not for other streams of the device.
    int err = 0;
    STATIC_CUDA(cudaMemcpyAsync(&err, base + oBar + sizeof(BarrierState), sizeof(int), cudaMemcpyDeviceToHost, stream));
    STATIC_CUDA(cudaStreamSynchronize(stream));
    if (err) return failStatic(err, "device-side wait timed out (grid barrier)");
    return SYMGB_OK;
}
