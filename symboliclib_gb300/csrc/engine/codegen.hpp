// Compiled executor: source generation (codegen.cpp) and run-time compilation
// (jit.cu).  A unit's kernels are emitted as straight-line CUDA C++ - the
// form of the reference's generated kernels (ComputeUnit.cpp:409-421), with
// 1, 2 or 4 work items per thread - compiled for sm_103a by NVRTC at first use
// and cached by source text, and launched in one of three schedules.
#pragma once
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "symgb.h"

namespace symgb {
namespace engine {

enum JitKind : int {
    JIT_PLAIN = 0,       // one kernel per ComputeKernel, launched in plan order
    JIT_LEVELS = 1,      // one kernel per dependency level, all its ComputeKernels
    JIT_PERSISTENT = 2,  // one cooperative kernel over all levels, grid barriers between them
};

struct JitConfig {
    int kind = JIT_LEVELS;
    int math = SYMGB_MATH_FAST;
    unsigned numSets = 1;
    std::vector<int> kernelTpb;    // per ComputeKernel (JIT_PLAIN)
    std::vector<int> levelTpb;     // per level (JIT_LEVELS); [0] for JIT_PERSISTENT
    std::vector<int> kernelItems;  // work items per thread, per ComputeKernel (JIT_PLAIN)
    std::vector<int> levelItems;   // per level (JIT_LEVELS); [0] for JIT_PERSISTENT
    int minBlocks = 0;  // > 0: __launch_bounds__ minimum CTAs per SM (caps registers)
    int loadPath = 0;   // SYMGB_LOAD_*: data path of the table and x loads
    int itemLayout = 0;  // SYMGB_ITEMS_*: which work items a thread takes
    // Direct result writes (one value set): per kernel and output row, the
    // row's start in the result-position table `dp` - the row's results go to
    // res[dp[start + i]] instead of x - or -1; empty when none is direct.
    std::vector<std::vector<std::int64_t>> directBase;
};

// Grouped item layout (SYMGB_ITEMS_GROUPED): copies of the index and constant
// tables whose rows are padded to a multiple of 4 entries (the row's last
// entry repeated), so that a thread reads the entries of 1, 2 or 4
// consecutive instances of a row with one aligned vector load.  Kernel k's
// row r starts at indexBase[k] + r * stride[k] (constBase[k] + r * stride[k]
// for constants); stride[k] = n_k rounded up to a multiple of 4.
struct GroupedTables {
    std::vector<std::uint64_t> indexBase, constBase, stride;
    std::uint64_t indexSize = 0, constSize = 0;  // entries of the padded copies
};
GroupedTables groupedTables(const std::vector<symgb_kernel_desc>& descs);

// One launch of a module: entry name, ComputeKernel (plain) or level (levels)
// it covers, blocks needed to cover its work items, block size.
struct JitLaunch {
    std::string name;
    int kernel;
    int level;
    std::uint64_t blocks;
    int tpb;
    int items;  // work items per thread
    bool cooperative;  // persistent: grid capped at the co-resident maximum
};

struct JitSource {
    std::string source;
    std::vector<JitLaunch> launches;  // in execution order
    bool grouped = false;             // reads the padded tables (GroupedTables)
    bool direct = false;              // writes some results straight into res
};

// Generates the module for a unit's kernels (host only; throws
// std::runtime_error for templates it cannot express).
JitSource generateModule(const std::vector<symgb_kernel_desc>& descs, int numLevels, const JitConfig& cfg);

// A compiled and loaded module (jit.cu).  `kernels[j]` is the cudaKernel_t
// of launches[j], stored as void* (the form the runtime's launch calls take).
struct JitModule {
    std::vector<JitLaunch> launches;
    std::vector<const void*> kernels;
    std::vector<int> registers;  // per launch: registers per thread of the compiled kernel
    double compileSeconds = 0;
    bool grouped = false;        // launch with the padded tables (GroupedTables)
    bool direct = false;         // writes some results straight into res
};

// Compiles `source` with NVRTC without loading it (no device needed).
int compileOnly(const std::string& source, double* seconds, std::string* err);

// Compiles (or finds in the process-wide cache) the module for `src`.
// Returns 0 or a SYMGB_ERR_* code with the message in *err.
int loadModule(const JitSource& src, std::shared_ptr<const JitModule>* out, std::string* err);

}  // namespace engine
}  // namespace symgb
