// Front-end passes of the engine: decomposition into reusable sub-expressions,
// template simplification, kernel (template + tables) construction and the
// ComputeUnit plan (kernel order, memory layout, index/constant tables).
//
// These passes restate the reference's method (src/Decomposition.cpp,
// src/Simplify.cpp, src/ComputeKernel.cpp, src/ComputeUnit.cpp:231-451) so that
// the kernel list, the per-kernel tables and the per-kernel operation order
// equal the reference's for the same expressions.  That equality is what makes
// the device results bit-identical to the reference's in exact mode.
#pragma once
#include <algorithm>
#include <array>
#include <cstddef>
#include <ostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "symbolic.hpp"

namespace symgb {

// Splits expressions into blocks of reusable sub-expressions
// (reference src/Decomposition.cpp:234-490).
std::vector<ExpressionBlock> decompose(const std::vector<Symbolic>& expr, unsigned char complexityThreshold = 3,
                                       int variableGroupId = 255, bool mergeSingleParent = true);

// Template rewrites (reference src/Simplify.cpp).
Symbolic simplify(const Symbolic& x);
Symbolic removeConstantExpressions(const Symbolic& x);
Symbolic referenceRedundant(const Symbolic& x);
Symbolic makeSymbolic(OpType op, std::vector<Symbolic> operands);
Symbolic flattenAdditions(const Symbolic& x);
Symbolic flattenMultiplications(const Symbolic& x);
Symbolic optimizeProducts(const Symbolic& x);
Symbolic optimizeSum(const Symbolic& x);
Symbolic pullFactor(Symbolic x);

// Kahn topological order: node list of a graph given as "node -> successors"
// (reference src/Utilities.hpp:54-83).  Empty on a cycle.
template <class Succ>
std::vector<int> topologicalOrder(const std::vector<Succ>& graph) {
    const std::size_t n = graph.size();
    std::vector<int> incoming(n, 0);
    for (auto& nbh : graph)
        for (int i : nbh) ++incoming[i];
    std::vector<int> S, L;
    for (std::size_t i = 0; i < n; ++i)
        if (!incoming[i]) S.push_back((int)i);
    while (!S.empty()) {
        const int node = S.back();
        S.pop_back();
        L.push_back(node);
        for (int m : graph[node])
            if (--incoming[m] == 0) S.push_back(m);
    }
    for (int i : incoming)
        if (i) return {};
    return L;
}

// Row layout of a per-instance table (reference src/Utilities.hpp:103-133):
// pack 0 = row-major [row][instance] (the GPU layout), pack 1 = [instance][row],
// pack k = blocks of k instances per row.  Returns the pack length used.
template <class T>
int appendTransposed(const std::vector<std::vector<T>>& src, std::vector<T>& dst, std::size_t packLength) {
    if (src.empty()) return (int)packLength;
    const std::size_t seg = src.front().size();
    const std::size_t n0 = dst.size();
    dst.resize(n0 + seg * src.size());
    auto out = dst.begin() + n0;
    if (packLength == 0 || seg % packLength) {
        for (auto& s : src) out = std::copy(s.begin(), s.end(), out);
        return 0;
    }
    const std::size_t packs = seg / packLength;
    for (std::size_t i = 0; i < packs; ++i)
        for (auto& s : src) out = std::copy_n(s.begin() + packLength * i, packLength, out);
    return (int)packLength;
}

// Thrown when the blocks given to a ComputeKernel are not structurally
// identical.  The reference groups blocks by (structure hash, level), and in
// rare cases two different structures share that key; the reference then
// fails its assertion in the kernel constructor (ComputeKernel.cpp:166).
struct GroupMismatch : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// One group of structurally identical blocks: a template expression over
// per-instance tables (reference src/ComputeKernel.cpp:27-268).
class ComputeKernel {
public:
    struct Access {
        int baseRow;  // index-table row
        int offset;   // literal added to the gathered index
    };

    ComputeKernel(const std::vector<Symbolic>& instances, int simdWidth);

    std::size_t numInstances() const { return n_; }
    int simdWidth() const { return simdWidth_; }
    const Symbolic& templateExpression() const { return template_; }

    // Tables, computed on first use in the reference's order.
    const std::vector<std::array<int, 2>>& outputVariableData();
    const std::vector<double>& constantData();
    const std::vector<std::array<int, 2>>& variableData();
    const std::vector<Access>& access() const { return access_; }

    std::size_t numOutputRows() const { return outputTable_.size(); }
    std::size_t numVariableRows() const { return variableTable_.size(); }
    std::size_t numConstantRows() const { return constantTable_.size(); }
    int packLength() const { return variablePack_; }

    std::size_t outputOffset = 0;     // first x slot written by this kernel
    std::size_t indexOffset = 0;      // first entry in the index table
    std::size_t constantsOffset = 0;  // first entry in the constant table

private:
    void optimizeTemplate();
    void findCorrelatedVariables();

    std::size_t n_;
    int simdWidth_;
    Symbolic template_;
    int outputPack_ = -1, constantsPack_ = -1, variablePack_ = -1;
    std::vector<std::array<int, 2>> outputData_;
    std::vector<std::vector<std::array<int, 2>>> outputTable_;
    std::vector<double> constantData_;
    std::vector<std::vector<double>> constantTable_;
    std::vector<std::array<int, 2>> variableData_;
    std::vector<std::vector<std::array<int, 2>>> variableTable_;
    std::vector<Access> access_;
};

// Device parameters (reference src/ComputeUnit.hpp:14-101).
struct DeviceConfig {
    unsigned vectorWidth = 1;
    unsigned numThreads = 1;
    unsigned decompositionThreshold = 6;
    bool singlePrecision = false;
    bool cudaDevice = false;
};

// The compiled form of a ComputeUnit: kernels in execution order and the
// memory plan (reference src/ComputeUnit.cpp:231-451).
struct Plan {
    DeviceConfig device;
    std::vector<std::size_t> argStart, argLength;  // input containers in x
    std::vector<ComputeKernel> kernels;
    std::vector<unsigned> positionData;  // absolute x offsets per kernel index row
    std::vector<double> constantData;
    std::vector<int> outputIdsFlat;  // x slot of every output value, container order
    std::vector<std::size_t> outputIndexStart, outputIndexLength;
    std::size_t numTotalMemory = 0;
    std::size_t inputDataSize = 0;
    std::vector<int> kernelLevel;  // longest-path level of each kernel (0 = no kernel inputs)
};

// Accumulates input and output containers and builds the plan.
class PlanBuilder {
public:
    explicit PlanBuilder(const DeviceConfig& device) { plan_.device = device; }
    // Container of VAR(0..len-1, g) (an input) or of output expressions.
    void addContainer(const Symbolic* expr, std::size_t len);
    // Builds the plan once; releases the output expressions it was given.
    Plan build();

private:
    Plan plan_;
    std::vector<Symbolic> outputExpressions_;
    std::vector<std::vector<int>> outputIds_;
    std::vector<std::size_t> inputSizes_;
    std::vector<std::pair<int, std::size_t>> inputOffsets_;  // group -> offset
    std::size_t inputDataSize_ = 0;
    int outputCount_ = 0;
};

// Canonical text of a plan: kernels, templates (as s-expressions with exact
// constants), access tables and all data tables.  Used to compare plans.
void dumpPlan(Plan& plan, std::ostream& os);
std::string templateText(const Symbolic& t);

}  // namespace symgb
