// The ComputeUnit API of the reference (src/ComputeUnit.hpp:14-222), running on
// the GB300 engine:
//
//   ComputeUnit<double> unit(Device(UseCuda(), ThreadsPerBlock(128)), AS, BS);
//   unit.compile().execute(A).getResults(B);
//
// Containers are anything with .data()/.size() of Symbolic (inputs: VAR(0..n-1, g)
// of one group; outputs: expressions), a single Symbolic, or an Eigen-style
// sparse matrix (valuePtr()/nonZeros()).  execute() takes the input value
// containers in constructor order; getResults() fills the output containers in
// constructor order (getResults(x, k) fills the k-th).  Planning (decomposition,
// kernel grouping, tables) follows the reference's method; compile() uploads
// the plan to the GPU instead of generating and building source code.
//
// Differences from the reference, by design: RealT must be double (the engine
// evaluates in FP64); an engine error throws std::runtime_error by default
// instead of exiting the process - OnError(ErrorPolicy::Print) prints it and
// carries on, OnError(ErrorPolicy::Exit) prints it and exits as the
// reference's generated library does (StringResources.h:28-34); several units
// can be live at once (no fixed file names).  Engine
// extensions: ValueSets(S) evaluates S value sets per execute (inputs and
// results hold S consecutive copies of each container), ExactMath() selects
// the bit-exact mode, and PlainSchedule / LevelSchedule / PersistentSchedule
// choose the launch structure.
#pragma once
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../symgb.h"
#include "frontend.hpp"
#include "plan_image.hpp"
#include "symbolic.hpp"
#include "utilities.hpp"

namespace symgb {

template <class T, class Tag>
struct NamedType {
    T x;
    explicit NamedType(const T& v) : x(v) {}
};

using ThreadsPerBlock = NamedType<int, struct ThreadsPerBlockTag>;
using NumThreads = NamedType<int, struct NumThreadsTag>;
using VecWidth = NamedType<int, struct VecWidthTag>;
using DecompositionThreshold = NamedType<int, struct DecompositionThresholdTag>;
using ValueSets = NamedType<int, struct ValueSetsTag>;
using ItemsPerThread = NamedType<int, struct ItemsPerThreadTag>;

// What the ComputeUnit does when an engine call fails.
enum class ErrorPolicy { Throw, Print, Exit };
using OnError = NamedType<ErrorPolicy, struct OnErrorTag>;

struct UseCuda {};
struct UseHIP {};
struct UseSinglePrecision {};
struct ExactMath {};
struct PlainSchedule {};
struct LevelSchedule {};
struct PersistentSchedule {};

class Device {
public:
    unsigned vectorWidth = 1;
    unsigned numThreads = 1;        // NumThreads: host threads of a CPU device
    unsigned threadsPerBlock = 0;   // ThreadsPerBlock: CUDA block size (0: engine default)
    unsigned decompositionThreshold = 6;
    bool singlePrecision = false;
    bool cudaDevice = false;
    bool hipDevice = false;
    int valueSets = 1;
    int math = SYMGB_MATH_FAST;
    int schedule = SYMGB_SCHEDULE_LEVELS;
    int itemsPerThread = 1;
    ErrorPolicy onError = ErrorPolicy::Throw;

    template <class... Args>
    explicit Device(const Args&... args) {
        (set(args), ...);
    }

private:
    void set(const DecompositionThreshold& v) { decompositionThreshold = (unsigned)v.x; }
    // The engine's kernels work in whole warps: a block size that is not a
    // multiple of 32 in [32, 1024] is rejected rather than rounded.
    void set(const ThreadsPerBlock& v) {
        if (v.x < 32 || v.x > 1024 || v.x % 32)
            throw std::invalid_argument("ThreadsPerBlock: the engine needs a multiple of 32 in [32, 1024]");
        threadsPerBlock = (unsigned)v.x;
    }
    void set(const VecWidth& v) { vectorWidth = (unsigned)v.x; }
    void set(const NumThreads& v) { numThreads = (unsigned)v.x; }
    void set(const ValueSets& v) { valueSets = v.x; }
    void set(const ItemsPerThread& v) { itemsPerThread = v.x; }
    void set(const OnError& v) { onError = v.x; }
    void set(const UseSinglePrecision&) { singlePrecision = true; }
    void set(const UseHIP&) { throw std::invalid_argument("UseHIP: the GB300 engine runs CUDA only"); }
    void set(const UseCuda&) {
        cudaDevice = true;
        vectorWidth = 0;
    }
    void set(const ExactMath&) { math = SYMGB_MATH_EXACT; }
    void set(const PlainSchedule&) { schedule = SYMGB_SCHEDULE_PLAIN; }
    void set(const LevelSchedule&) { schedule = SYMGB_SCHEDULE_LEVELS; }
    void set(const PersistentSchedule&) { schedule = SYMGB_SCHEDULE_PERSISTENT; }
};

namespace detail {

template <class C, class = void>
struct IsSparse : std::false_type {};
template <class C>
struct IsSparse<C, std::void_t<decltype(std::declval<C&>().valuePtr()), decltype(std::declval<C&>().nonZeros())>>
    : std::true_type {};

template <class C>
auto contPtr(C& c) {
    if constexpr (std::is_same<std::decay_t<C>, Symbolic>::value)
        return &c;
    else if constexpr (IsSparse<C>::value)
        return c.valuePtr();
    else
        return c.data();
}

template <class C>
std::size_t contSize(const C& c) {
    if constexpr (std::is_same<std::decay_t<C>, Symbolic>::value)
        return 1;
    else if constexpr (IsSparse<C>::value)
        return (std::size_t)const_cast<C&>(c).nonZeros();
    else
        return (std::size_t)c.size();
}

}  // namespace detail

template <class RealT>
class ComputeUnit {
    static_assert(std::is_same<RealT, double>::value, "the GB300 engine evaluates ComputeUnits in FP64 (RealT = double)");

public:
    template <class... Containers>
    explicit ComputeUnit(Device device, const Containers&... containers) : device_(device) {
        DeviceConfig cfg;
        cfg.vectorWidth = 0;  // device table layout
        cfg.numThreads = device.numThreads;
        cfg.decompositionThreshold = device.decompositionThreshold;
        cfg.cudaDevice = true;
        PlanBuilder pb(cfg);
        (pb.addContainer(detail::contPtr(const_cast<Containers&>(containers)), detail::contSize(containers)), ...);
        plan_ = pb.build();
        buildPlanImage(plan_, image_, device.threadsPerBlock ? device.threadsPerBlock : 128);
    }

    ComputeUnit(const ComputeUnit&) = delete;
    ComputeUnit& operator=(const ComputeUnit&) = delete;
    ~ComputeUnit() { close(); }

    // Creates the device unit and uploads the plan (reference: generate, build
    // and load the device library, then init()).
    ComputeUnit& compile() {
        close();
        check(symgb_unit_create(&image_.desc, &unit_));
        symgb_schedule s{device_.schedule, device_.math, (int)device_.threadsPerBlock, 0, 0, 0, device_.itemsPerThread, 0};
        check(symgb_set_schedule(unit_, &s));
        check(symgb_set_num_sets(unit_, device_.valueSets));
        check(symgb_init(unit_, image_.indexData.data(), image_.outIndexData.data(), image_.constData.data()));
        return *this;
    }

    // setArg for every input container, then run().  Synchronous copies from
    // the containers' own memory; containers that are page-locked
    // (cudaHostRegister) are copied by DMA at full link speed.  Overlapped
    // copies are the C ABI's *_async calls.
    template <class... Values>
    ComputeUnit& execute(const Values&... values) {
        requireCompiled();
        int i = 0;
        (setArg(i++, values), ...);
        check(symgb_run(unit_));
        return *this;
    }

    template <class... Outs>
    ComputeUnit& getResults(Outs&... outs) {
        requireCompiled();
        int k = 0;
        (getResult(k++, outs), ...);
        return *this;
    }

    template <class Out>
    ComputeUnit& getResults(Out& out, int k) {
        requireCompiled();
        getResult(k, out);
        return *this;
    }

    void close() {
        if (unit_) symgb_unit_destroy(unit_);
        unit_ = nullptr;
    }

    // Engine-side access for benchmarks and schedulers.
    symgb_unit_t handle() const { return unit_; }
    const Plan& plan() const { return plan_; }
    const symgb_plan_desc& planDesc() const { return image_.desc; }

private:
    void check(int rc) const {
        if (rc == SYMGB_OK) return;
        const std::string msg = std::string("symgb: ") + symgb_last_error();
        if (device_.onError == ErrorPolicy::Throw) throw std::runtime_error(msg);
        std::fprintf(stderr, "%s\n", msg.c_str());
        if (device_.onError == ErrorPolicy::Exit) std::exit(EXIT_FAILURE);
    }
    void requireCompiled() const {
        if (!unit_) throw std::logic_error("ComputeUnit: compile() first");
    }
    template <class V>
    void setArg(int i, const V& v) {
        if ((std::size_t)i >= image_.argLength.size()) throw std::invalid_argument("execute(): too many input containers");
        const std::size_t need = image_.argLength[i] * (std::size_t)device_.valueSets;
        if (detail::contSize(v) != need) throw std::invalid_argument("execute(): input container size mismatch");
        check(symgb_set_arg_sets(unit_, detail::contPtr(const_cast<V&>(v)), i));
    }
    template <class V>
    void getResult(int k, V& v) {
        if ((std::size_t)k >= image_.outLength.size()) throw std::invalid_argument("getResults(): no such output container");
        const std::size_t need = image_.outLength[k] * (std::size_t)device_.valueSets;
        if (detail::contSize(v) != need) throw std::invalid_argument("getResults(): output container size mismatch");
        check(symgb_get_result_sets(unit_, detail::contPtr(v), k));
    }

    Device device_;
    Plan plan_;
    PlanImage image_;
    symgb_unit_t unit_ = nullptr;
};

}  // namespace symgb

// The reference's namespace name, for drop-in source compatibility.
namespace Sym = symgb;
