// ComputeUnit planning: containers -> decomposition -> kernels -> execution
// order -> memory layout and tables (reference src/ComputeUnit.cpp:172-451).
#include <atomic>
#include <cstring>
#include <iomanip>
#include <map>
#include <set>
#include <sstream>
#include <stdexcept>
#include <unordered_map>

#include "symgb/frontend.hpp"
#include "symgb/parallel.hpp"
#include "symgb/stage_clock.hpp"
#include "symgb/traverse.hpp"

namespace symgb {

namespace {

// Structure fingerprint with non-linear mixing (operation, child count and
// child fingerprints, leaves by kind only).  Used only to split a kernel group
// whose blocks collide on the reference's CRC-based structure hash, which is
// linear over GF(2) and so has systematic collisions.
std::uint64_t structureFingerprint(const Symbolic& x) {
    return traverseGenerateIdentity<std::uint64_t>(x, [](const Symbolic& y, const std::vector<std::uint64_t>& cs) {
        std::uint64_t h = 0x9e3779b97f4a7c15ULL * (std::uint64_t)(y.op() + 1) + cs.size();
        for (std::uint64_t c : cs) {
            h ^= c + 0x9e3779b97f4a7c15ULL + (h << 6) + (h >> 2);
            h *= 0xbf58476d1ce4e5b9ULL;
            h ^= h >> 31;
        }
        return h;
    });
}

}  // namespace

// A container whose entries are all variables is an input: they must be
// VAR(0..len-1, g) of one group g.  Any other container holds outputs, each
// wrapped as ASSIGN(VAR(i, -10 - k), expr) for the k-th output container
// (reference ComputeUnit.cpp:172-228).
void PlanBuilder::addContainer(const Symbolic* expr, std::size_t len) {
    if (!len) return;
    bool isInput = true;
    for (std::size_t i = 0; i < len; ++i)
        if (expr[i].op() != VAR) {
            isInput = false;
            break;
        }
    if (isInput) {
        const int group = expr[0].variable()[1];
        for (std::size_t i = 0; i < len; ++i) {
            if (expr[i].variable()[0] != (int)i) throw std::invalid_argument("input variables are not numbered 0..n-1 in order");
            if (expr[i].variable()[1] != group) throw std::invalid_argument("input container mixes variable groups");
        }
        inputSizes_.push_back(len);
        inputOffsets_.emplace_back(group, inputDataSize_);
        inputDataSize_ += len;
    } else {
        for (std::size_t i = 0; i < len; ++i)
            outputExpressions_.emplace_back(ASSIGN, Symbolic((int)i, -10 - outputCount_), expr[i]);
        outputIds_.push_back(std::vector<int>(len, -1));
        ++outputCount_;
    }
}

Plan PlanBuilder::build() {
    Plan& P = plan_;
    const DeviceConfig& dev = P.device;
    StageClock clock;
    std::vector<ExpressionBlock> blocks =
        decompose(outputExpressions_, (unsigned char)dev.decompositionThreshold, GLOBAL_INTERMEDIATE, true);
    clock.mark("decompose (total)");

    // Group blocks by (structure hash, level) in first-seen order (ComputeUnit.cpp:34-56).
    std::unordered_map<hash_t, int> groupMap;
    std::vector<std::vector<int>> groups;
    for (int i = 0; i < (int)blocks.size(); ++i) {
        const hash_t h = hashPair(blocks[i].structureHash, blocks[i].level);
        int& id = groupMap[h];
        if (id) {
            groups[id - 1].push_back(i);
        } else {
            groups.push_back({i});
            id = (int)groups.size();
        }
    }
    // A group whose blocks turn out to differ in structure (where the reference
    // aborts) is split by structure fingerprint, in first-seen order;
    // groups of identical blocks - every case the reference handles - are
    // built exactly as the reference builds them.
    std::vector<int> blockGroup(blocks.size());
    std::vector<ComputeKernel> kernels;
    kernels.reserve(groups.size());
    auto widthFor = [&](std::size_t count) {
        if (dev.vectorWidth == 0) return 0;
        return count > dev.vectorWidth ? (int)dev.vectorWidth : 1;
    };
    for (std::size_t g = 0; g < groups.size(); ++g) {
        std::vector<Symbolic> inst(groups[g].size());
        for (std::size_t j = 0; j < groups[g].size(); ++j) inst[j] = blocks[groups[g][j]].x;
        try {
            kernels.emplace_back(inst, widthFor(inst.size()));
            for (int b : groups[g]) blockGroup[b] = (int)kernels.size() - 1;
        } catch (const GroupMismatch&) {
            std::vector<std::vector<int>> parts;
            std::unordered_map<std::uint64_t, int> partOf;
            for (int b : groups[g]) {
                int& p = partOf[structureFingerprint(blocks[b].x)];
                if (!p) {
                    parts.push_back({});
                    p = (int)parts.size();
                }
                parts[p - 1].push_back(b);
            }
            for (auto& part : parts) {
                std::vector<Symbolic> pi;
                for (int b : part) pi.push_back(blocks[b].x);
                kernels.emplace_back(pi, widthFor(pi.size()));
                for (int b : part) blockGroup[b] = (int)kernels.size() - 1;
            }
        }
    }

    clock.mark("kernels");

    // Execution order: children before parents (ComputeUnit.cpp:279-296).
    std::vector<std::set<int>> deps(kernels.size());
    for (int i = 0; i < (int)blocks.size(); ++i)
        for (int j : blocks[i].childs)
            if (j != -1) deps[blockGroup[j]].insert(blockGroup[i]);
    std::vector<int> order = topologicalOrder(deps);
    if (order.size() != kernels.size()) throw std::runtime_error("kernel dependency graph has a cycle");

    // Longest-path level of every kernel (0 = reads only inputs).
    std::vector<int> levelOf(kernels.size(), 0);
    for (int k : order)
        for (int parent : deps[k]) levelOf[parent] = std::max(levelOf[parent], levelOf[k] + 1);

    P.kernels.clear();
    P.kernels.reserve(kernels.size());
    for (int k : order) {
        P.kernels.push_back(std::move(kernels[k]));
        P.kernelLevel.push_back(levelOf[k]);
    }

    // Memory layout: x = [inputs | output and intermediate slots in kernel order].
    std::size_t variableDataSize = 0;
    std::size_t slots = 0;
    for (auto& k : P.kernels) slots += k.outputVariableData().size();
    KeyMap<std::size_t> intermediatePositions(slots);  // sized up front: no rehashing
    for (auto& k : P.kernels) {
        k.outputOffset = inputDataSize_ + variableDataSize;
        for (auto var : k.outputVariableData()) {
            if (var[1] <= -10) {
                outputIds_[-(10 + var[1])][var[0]] = (int)(inputDataSize_ + variableDataSize++);
            } else {
                if (var[0] != -1) intermediatePositions[hashVariable(var)] = variableDataSize;
                ++variableDataSize;
            }
        }
    }
    for (auto& ids : outputIds_) P.outputIdsFlat.insert(P.outputIdsFlat.end(), ids.begin(), ids.end());

    for (auto& k : P.kernels) {
        k.constantsOffset = P.constantData.size();
        const auto& cd = k.constantData();
        P.constantData.insert(P.constantData.end(), cd.begin(), cd.end());
    }

    clock.mark("order, layout");

    // Index table: every kernel's variable slots, filled in parallel (the maps
    // are only read here).  An input group without an offset reads from 0.
    const std::map<int, std::size_t> inputOffsets(inputOffsets_.begin(), inputOffsets_.end());
    std::size_t indices = 0;
    for (auto& k : P.kernels) {
        k.indexOffset = indices;
        indices += k.variableData().size();
    }
    P.positionData.resize(indices);
    for (auto& k : P.kernels) {
        const auto& vd = k.variableData();
        unsigned* out = P.positionData.data() + k.indexOffset;
        std::atomic<bool> missing{false};
        parallelFor(vd.size(), 4096, [&](std::size_t b, std::size_t e) {
            for (std::size_t i = b; i < e; ++i) {
                const auto& x = vd[i];
                if (x[1] == GLOBAL_INTERMEDIATE || x[1] == EXPLICIT_INTERMEDIATE) {
                    const std::size_t* pos = intermediatePositions.find(hashVariable(x));
                    if (!pos) {
                        missing = true;
                        continue;
                    }
                    out[i] = (unsigned)(inputDataSize_ + *pos);
                } else {
                    auto it = inputOffsets.find(x[1]);
                    out[i] = (unsigned)((it == inputOffsets.end() ? 0 : it->second) + x[0]);
                }
            }
        });
        if (missing) throw std::runtime_error("intermediate read before it is produced");
    }

    std::size_t acc = 0;
    for (std::size_t s : inputSizes_) {
        P.argStart.push_back(acc);
        P.argLength.push_back(s);
        acc += s;
    }
    acc = 0;
    for (auto& ids : outputIds_) {
        P.outputIndexStart.push_back(acc);
        P.outputIndexLength.push_back(ids.size());
        acc += ids.size();
    }
    P.inputDataSize = inputDataSize_;
    P.numTotalMemory = inputDataSize_ + variableDataSize;
    clock.mark("index table");

    // The blocks' expressions are released in parallel (most of their nodes
    // belong to one block; reference counts are atomic meanwhile).
    // So are the output expressions this builder holds (the containers' whole
    // expression graph, often hundreds of millions of nodes): build() consumes
    // them.
    {
        Symbolic::ConcurrentRefs concurrent;
        parallelFor(blocks.size(), 1024, [&](std::size_t b, std::size_t e) {
            for (std::size_t i = b; i < e; ++i) blocks[i] = ExpressionBlock();
        });
        parallelFor(outputExpressions_.size(), 1024, [&](std::size_t b, std::size_t e) {
            for (std::size_t i = b; i < e; ++i) outputExpressions_[i] = Symbolic();
        });
    }
    outputExpressions_.clear();
    clock.mark("release");
    return std::move(plan_);
}

namespace {

const char* opName(OpType op) {
    static const char* names[NUM_OPS] = {"NOOP", "CONST", "VAR", "ADD", "MUL", "MULC", "DIV", "SQRT", "SIN", "COS",
                                         "TAN", "COT", "ASIN", "ACOS", "ATAN", "EXP", "LOG", "POW", "ASSIGN", "GROUP",
                                         "CONDPOS", "CONDNONZERO", "CONDZERO", "NEG", "DEFINE", "BLOCK", "REC",
                                         "FIXED", "FUNC", "CALL"};
    return op < NUM_OPS ? names[op] : "?";
}

void writeTemplate(const Symbolic& x, std::ostream& os) {
    switch (x.op()) {
        case CONST: {
            std::uint64_t bits;
            double c = x.constant();
            std::memcpy(&bits, &c, 8);
            os << "#" << std::hex << bits << std::dec;
            return;
        }
        case VAR: os << "v(" << x.variable()[0] << "," << x.variable()[1] << ")"; return;
        default:
            os << "(" << opName(x.op());
            for (auto& c : x) {
                os << " ";
                writeTemplate(c, os);
            }
            os << ")";
    }
}

template <class T>
void writeList(std::ostream& os, const char* name, const std::vector<T>& v) {
    os << name << " " << v.size() << ":";
    for (auto& e : v) os << " " << e;
    os << "\n";
}

}  // namespace

std::string templateText(const Symbolic& t) {
    std::ostringstream os;
    writeTemplate(t, os);
    return os.str();
}

void dumpPlan(Plan& P, std::ostream& os) {
    os << "kernels " << P.kernels.size() << "\n";
    for (std::size_t k = 0; k < P.kernels.size(); ++k) {
        auto& K = P.kernels[k];
        os << "kernel " << k << " n=" << K.numInstances() << " outOff=" << K.outputOffset << " idxOff=" << K.indexOffset
           << " constOff=" << K.constantsOffset << "\n";
        os << "access";
        for (auto& a : K.access()) os << " " << a.baseRow << ":" << a.offset;
        os << "\n";
        os << "template " << templateText(K.templateExpression()) << "\n";
    }
    writeList(os, "argStart", P.argStart);
    writeList(os, "argLength", P.argLength);
    writeList(os, "outputIndexStart", P.outputIndexStart);
    writeList(os, "outputIndexLength", P.outputIndexLength);
    os << "numTotalMemory " << P.numTotalMemory << "\n";
    writeList(os, "positionData", P.positionData);
    writeList(os, "outputIds", P.outputIdsFlat);
    os << "constantData " << P.constantData.size() << ":";
    for (double c : P.constantData) {
        std::uint64_t bits;
        std::memcpy(&bits, &c, 8);
        os << " " << std::hex << bits << std::dec;
    }
    os << "\n";
}

}  // namespace symgb
