// Host-side state of an engine unit, shared by the engine's translation units
// (engine.cu: the C ABI; static_scratch.cu: the allocation-free entry point).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "codegen.hpp"
#include "device.cuh"
#include "program.hpp"
#include "symgb.h"

namespace symgb {
namespace engine {

// Records the message returned by symgb_last_error() on this thread and
// returns `code`.
int setLastError(int code, const std::string& msg);

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

}  // namespace engine
}  // namespace symgb

struct symgb_unit {
    using HostKernel = symgb::engine::HostKernel;
    template <class T>
    using DevBuf = symgb::engine::DevBuf<T>;
    // plan
    std::vector<HostKernel> kernels;
    std::vector<std::uint64_t> argStart, argLength, outStart, outLength;
    std::uint64_t numTotalMemory = 0, numIndices = 0, numOutputValues = 0, numConstants = 0;
    int threadsPerBlock = 128;
    int numLevels = 0;
    symgb_schedule sched{SYMGB_SCHEDULE_PLAIN, SYMGB_MATH_FAST, 0, 0, 0, 0, 1, 0, 1, SYMGB_EXEC_COMPILED};
    int numSets = 1;
    bool usesLibrary = false;  // some program calls pow, sin, ... (interpreter variant MODE_LIB)

    // device state
    bool initialized = false;
    int device = 0;
    int smCount = 0;
    std::size_t smemOptin = 48 * 1024;  // max dynamic shared memory per block
    cudaStream_t ownStream = nullptr, stream = nullptr;
    DevBuf<double> x, c, staging, outBuf;
    // Asynchronous result copies (symgb_get_result_sets_async): gathered into
    // asyncOut (every output container, value sets included, at its own
    // offset) on `stream`, copied to the host on copyStream; copyDone[k] marks
    // the end of container k's last copy, which the next gather into that
    // region waits for.
    cudaStream_t copyStream = nullptr;
    cudaEvent_t gatherDone = nullptr;
    std::vector<cudaEvent_t> copyDone;
    // Large result copies are split over copyStreams (symgb_set_copy_streams):
    // copyStream and extraCopy[i], each chunk on its own stream so several
    // copy engines move it; extraDone[i] joins chunk i + 1 back into copyStream.
    int copyStreams = 1;
    int loadPath = SYMGB_LOAD_READONLY;  // compiled executor's load data path (symgb_set_load_path)
    std::vector<cudaStream_t> extraCopy;
    std::vector<cudaEvent_t> extraDone;
    DevBuf<double> asyncOut;
    int asyncOutSets = 0;
    DevBuf<std::uint32_t> p, ids;
    // Padded copies of p and c for the compiled executor's grouped item
    // layout (GroupedTables), made on the device at first use.
    int itemLayout = SYMGB_ITEMS_STRIDED;
    DevBuf<std::uint32_t> p4;
    DevBuf<double> c4;
    bool groupedBuilt = false;
    // Direct result writes of the compiled executor with one value set
    // (symgb_set_direct_outputs), planned at init: output rows whose slots no
    // kernel reads and that each name one result position are stored straight
    // into `res` at those positions - directBase[k][row] is the row's start in
    // dp (the positions, [row][instance]) or -1 - and the results of the other
    // rows are gathered into `res` (restPos / restSlot pairs) when they are
    // read.  lastRunDirect: the last enqueued run wrote res.
    bool directOutputs = true;
    bool directRows = false;  // some row is direct
    std::vector<std::vector<std::int64_t>> directBase;
    DevBuf<std::uint32_t> dp, restPos, restSlot;
    std::uint64_t restCount = 0;
    DevBuf<double> res;
    bool lastRunDirect = false;
    DevBuf<std::uint64_t> progs;
    DevBuf<DevKernel> devKernels;
    DevBuf<Tile> tiles;
    DevBuf<std::uint32_t> levelSeg, kernelSeg;
    DevBuf<BarrierState> barrier;
    int* errorHost = nullptr;  // mapped pinned flag written by the device
    int* errorDev = nullptr;
    std::vector<DevKernel> hostDevKernels;
    std::vector<std::uint32_t> hostLevelSeg, hostKernelSeg;  // tile boundaries per level / per kernel
    std::vector<Tile> hostTiles;
    std::uint32_t maxProgWords = 0;
    // program words staged in shared memory, per (L2 loads, registers, program
    // words, items per thread, threads per block, lanes per item) of a launch
    std::map<std::array<std::uint32_t, 6>, std::uint32_t> stagingCache;
    std::size_t tilesFor = 0;  // configuration the tile table was built for
    int tilesSets = -1, tilesItems = -1, tilesMath = -1;
    cudaGraphExec_t graph = nullptr;
    bool graphValid = false;
    // Compiled executor: modules by configuration key (schedule kind, math,
    // value sets, block sizes); `jit` is the current schedule's.
    std::map<std::string, std::shared_ptr<const symgb::engine::JitModule>> jitModules;
    std::shared_ptr<const symgb::engine::JitModule> jit;
    std::string jitKey;
    int lastLaunches = 0;
    int launchesPerRun = 0;
    unsigned long long barrierTimeoutNs = 2000000000ull;
    unsigned barrierExtra = 0;  // arrivals beyond the grid each barrier waits for (failure tests only)

    ~symgb_unit() { release(); }

    void dropGraph() {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
        graphValid = false;
    }

    void release() {
        if (copyStream) cudaStreamSynchronize(copyStream);  // copies may still read asyncOut
        for (cudaEvent_t e : copyDone)
            if (e) cudaEventDestroy(e);
        copyDone.clear();
        if (gatherDone) cudaEventDestroy(gatherDone);
        gatherDone = nullptr;
        for (cudaStream_t e : extraCopy) {
            cudaStreamSynchronize(e);
            cudaStreamDestroy(e);
        }
        extraCopy.clear();
        for (cudaEvent_t e : extraDone) cudaEventDestroy(e);
        extraDone.clear();
        if (copyStream) cudaStreamDestroy(copyStream);
        copyStream = nullptr;
        asyncOut.reset();
        asyncOutSets = 0;
        dropGraph();
        for (cudaEvent_t e : timingEvents) cudaEventDestroy(e);
        timingEvents.clear();
        x.reset();
        c.reset();
        staging.reset();
        outBuf.reset();
        p.reset();
        ids.reset();
        p4.reset();
        c4.reset();
        groupedBuilt = false;
        dp.reset();
        restPos.reset();
        restSlot.reset();
        res.reset();
        directRows = false;
        directBase.clear();
        restCount = 0;
        lastRunDirect = false;
        progs.reset();
        devKernels.reset();
        tiles.reset();
        levelSeg.reset();
        kernelSeg.reset();
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
    bool compiledExec() const { return sched.executor == SYMGB_EXEC_COMPILED; }
    int tpb() const { return sched.threads_per_block > 0 ? sched.threads_per_block : threadsPerBlock; }
    int items() const { return sched.items_per_thread == 2 || sched.items_per_thread == 4 ? sched.items_per_thread : 1; }
    int lanes() const { return sched.lanes_per_item > 1 ? sched.lanes_per_item : 1; }
    // Block size of a launch: whole warps when several lanes share an item.
    int launchTpb() const { return lanes() > 1 ? std::max(32, tpb() / 32 * 32) : tpb(); }

    // Per-kernel launch shape (symgb_set_kernel_shape); zeros take the schedule's.
    struct Shape {
        int items, lanes, tpb;
    };
    std::vector<Shape> kernelShape;
    int shapesVersion = 0, tilesShapes = -1;
    std::vector<cudaEvent_t> timingEvents;
    Shape shapeOf(std::size_t k) const {
        Shape s{items(), lanes(), tpb()};
        if (k < kernelShape.size()) {
            const Shape& o = kernelShape[k];
            if (o.items || o.lanes || o.tpb) {
                s.items = o.items ? o.items : 1;
                s.lanes = o.lanes ? o.lanes : 1;
                if (o.tpb) s.tpb = o.tpb;
            }
        }
        if (s.lanes > 1) s.tpb = std::max(32, s.tpb / 32 * 32);
        return s;
    }
};

