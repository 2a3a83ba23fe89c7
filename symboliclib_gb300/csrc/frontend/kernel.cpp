// ComputeKernel: one template expression applied over per-instance tables.
//
// Restates reference src/ComputeKernel.cpp:27-484.  The instances of a group
// are walked in lockstep; wherever the instances differ only in a leaf, the
// leaf becomes a table row: output variables (group -2), variables read through
// the index table (group -3) and per-instance constants (group -4).  The
// template is then rewritten (constant folding, local common-sub-expression
// extraction into DEFINE statements, simplification) and its statements are
// put into dependency order.
#include <atomic>
#include <map>
#include <unordered_set>

#include "symgb/frontend.hpp"
#include "symgb/parallel.hpp"
#include "symgb/traverse.hpp"

namespace symgb {

namespace {

// The lockstep cursor: the same child position across all instances.  It
// holds pointers to the instances' handles (kept alive by the instance list),
// so walking a template over many instances copies no reference counts.
struct Lockstep {
    std::vector<const Symbolic*> x;
    hash_t h = 0;
    unsigned childCounter = 0;

    explicit Lockstep(const std::vector<Symbolic>& xs) {
        x.reserve(xs.size());
        for (auto& s : xs) x.push_back(&s);
        init();
    }
    // The instances are read in parallel (memory-latency bound: one pointer
    // chase per instance); the hash is then taken in instance order.
    Lockstep(const std::vector<const Symbolic*>& parents, unsigned child) {
        x.resize(parents.size());
        std::vector<hash_t> hs(parents.size());
        parallelFor(parents.size(), kGrain, [&](std::size_t b, std::size_t e) {
            for (std::size_t i = b; i < e; ++i) {
                x[i] = &(*parents[i])[child];
                hs[i] = x[i]->ahash();
            }
        });
        if (!x.empty()) h = hashVectorParallel(hs);
    }
    // Hash of the instances' algebraic hashes (reference ComputeKernel.cpp:14-20).
    void init() {
        if (x.empty()) return;
        std::vector<hash_t> hs(x.size());
        parallelFor(x.size(), kGrain, [&](std::size_t b, std::size_t e) {
            for (std::size_t i = b; i < e; ++i) hs[i] = x[i]->ahash();
        });
        h = hashVectorParallel(hs);
    }
    // True if any instance differs from the first in operation or child count.
    bool mixed() const {
        if (x.empty()) return false;
        const OpType op0 = x.front()->op();
        const unsigned nc0 = x.front()->numChilds();
        std::atomic<bool> bad{false};
        parallelFor(x.size(), kGrain, [&](std::size_t b, std::size_t e) {
            for (std::size_t i = b; i < e && !bad.load(std::memory_order_relaxed); ++i)
                if (x[i]->op() != op0 || x[i]->numChilds() != nc0) bad.store(true, std::memory_order_relaxed);
        });
        return bad.load();
    }
    static constexpr std::size_t kGrain = 2048;
    unsigned numChilds() const { return x.empty() ? 0 : x.front()->numChilds(); }
    OpType op() const { return x.empty() ? NOOP : x.front()->op(); }
    bool visit() { return childCounter++ == x.front()->numChilds(); }

    // The variable of every instance.  The table is never collapsed to a single
    // entry: the reference's all-identical test (ComputeKernel.cpp:92) is
    // inverted and always fails.
    std::vector<std::array<int, 2>> variables() const {
        std::vector<std::array<int, 2>> v(x.size());
        parallelFor(x.size(), kGrain, [&](std::size_t b, std::size_t e) {
            for (std::size_t i = b; i < e; ++i) v[i] = x[i]->variable();
        });
        return v;
    }
    // The constant of every instance, or one value if all are equal.
    std::vector<double> constants() const {
        std::vector<double> v(x.size());
        parallelFor(x.size(), kGrain, [&](std::size_t b, std::size_t e) {
            for (std::size_t i = b; i < e; ++i) v[i] = x[i]->constant();
        });
        bool allEqual = true;
        for (std::size_t i = 1; i < v.size() && allEqual; ++i)
            if (v[0] != v[i]) allEqual = false;
        if (allEqual) v.resize(1);
        return v;
    }
};

}  // namespace

ComputeKernel::ComputeKernel(const std::vector<Symbolic>& instances, int simdWidth)
    : n_(instances.size()), simdWidth_(simdWidth) {
    std::map<hash_t, Symbolic> seen;  // instance-list hash -> template sub-tree
    std::vector<Lockstep> stack;
    stack.emplace_back(instances);
    std::vector<Symbolic> built;

    while (!stack.empty()) {
        Lockstep& cur = stack.back();
        if (cur.visit()) {
            const unsigned nc = cur.numChilds();
            Symbolic t(cur.op(), std::vector<Symbolic>(built.end() - nc, built.end()));
            built.erase(built.end() - nc, built.end());
            built.push_back(t);
            if (seen.find(cur.h) == seen.end()) seen[cur.h] = t;
            stack.pop_back();
            continue;
        }
        const OpType parentOp = cur.op();
        const unsigned childPos = cur.childCounter;  // 1-based position of this child
        // Every instance must have the same operation and child count here
        // (the reference asserts this, ComputeKernel.cpp:166).
        if (childPos == 1 && cur.mixed()) throw GroupMismatch("kernel group holds structurally different blocks");
        Lockstep data(cur.x, childPos - 1);
        if ((data.op() == VAR || data.op() == CONST) && data.mixed())  // leaf lists are never visited as `cur`
            throw GroupMismatch("kernel group holds structurally different blocks");
        auto it = seen.find(data.h);
        if (it != seen.end()) {
            built.push_back(it->second);
        } else if (data.op() == VAR) {
            auto values = data.variables();
            if (parentOp == ASSIGN && childPos == 1) {
                built.push_back(Symbolic((int)outputTable_.size(), TEMPLATE_OUTPUT));
                outputTable_.push_back(std::move(values));
            } else {
                built.push_back(Symbolic((int)variableTable_.size(), TEMPLATE_INDEX));
                variableTable_.push_back(std::move(values));
            }
            seen[data.h] = built.back();
        } else if (data.op() == CONST) {
            auto values = data.constants();
            if (values.size() == 1) {
                built.push_back(Symbolic(values.front()));
            } else {
                built.push_back(Symbolic((int)constantTable_.size(), TEMPLATE_CONSTANT));
                constantTable_.push_back(std::move(values));
            }
            seen[data.h] = built.back();
        } else {
            stack.push_back(std::move(data));  // invalidates `cur`
        }
    }

    // Pad to a multiple of the SIMD width (reference ComputeKernel.cpp:241-259).
    if (simdWidth_ > 1 && n_ > (std::size_t)simdWidth_ && n_ % simdWidth_) {
        const std::size_t pad = simdWidth_ - n_ % simdWidth_;
        for (auto& c : constantTable_) c.insert(c.end(), pad, 0.0);
        for (auto& v : variableTable_) {
            const std::array<int, 2> last = v.back();
            v.insert(v.end(), pad, last);
        }
        for (auto& v : outputTable_) v.insert(v.end(), pad, std::array<int, 2>{-1, -1});
        n_ += pad;
    }

    assert(built.size() == 1);
    template_ = built.front();
    optimizeTemplate();
}

// Reference ComputeKernel.cpp:270-323.
void ComputeKernel::optimizeTemplate() {
    template_ = removeConstantExpressions(template_);
    template_ = removeConstantExpressions(template_);
    template_ = referenceRedundant(template_);

    std::vector<ExpressionBlock> blocks = decompose({template_}, 0, LOCAL_VAR, false);
    for (auto& b : blocks) b.x = simplify(b.x);
    for (auto& b : blocks)
        if (b.x.op() == ASSIGN && b.x[0].variable()[1] == LOCAL_VAR) b.x = Symbolic(DEFINE, b.x[0], b.x[1]);

    std::vector<std::unordered_set<int>> graph(blocks.size());
    for (int i = 0; i < (int)blocks.size(); ++i)
        for (int c : blocks[i].childs) graph[c].insert(i);
    std::vector<int> order = topologicalOrder(graph);
    std::vector<Symbolic> statements;
    for (int i : order) statements.push_back(blocks[i].x);
    template_ = Symbolic(BLOCK, statements);
}

const std::vector<std::array<int, 2>>& ComputeKernel::outputVariableData() {
    if (outputData_.empty()) outputPack_ = appendTransposed(outputTable_, outputData_, simdWidth_);
    return outputData_;
}

const std::vector<double>& ComputeKernel::constantData() {
    if (constantData_.empty()) constantsPack_ = appendTransposed(constantTable_, constantData_, simdWidth_);
    return constantData_;
}

const std::vector<std::array<int, 2>>& ComputeKernel::variableData() {
    if (variableData_.empty()) {
        findCorrelatedVariables();
        variablePack_ = appendTransposed(variableTable_, variableData_, simdWidth_);
    }
    return variableData_;
}

// Index rows whose entries differ from an earlier row by one constant offset
// (same input group, same relative pattern) share that row; the template reads
// them as x[p[base] + offset] (reference ComputeKernel.cpp:413-484).
void ComputeKernel::findCorrelatedVariables() {
    std::map<hash_t, int> patterns;
    int i = 0;
    for (auto& vars : variableTable_) {
        std::vector<int> vals;
        bool sameGroup = true;
        vals.push_back(vars[0][1]);
        for (auto& v : vars) {
            if (v[1] != vars[0][1]) {
                sameGroup = false;
                break;
            }
            vals.push_back(v[0] - vars[0][0]);
        }
        if (!sameGroup || vars[0][1] == GLOBAL_INTERMEDIATE || vars[0][1] == EXPLICIT_INTERMEDIATE) {
            access_.push_back({i, 0});
        } else {
            const hash_t h = hashVector(vals);
            auto it = patterns.find(h);
            if (it == patterns.end()) {
                patterns[h] = i;
                access_.push_back({i, 0});
            } else {
                access_.push_back({it->second, vars[0][0] - variableTable_[it->second][0][0]});
            }
        }
        ++i;
    }
    // Keep only the rows that are read explicitly, renumbered densely.
    std::map<int, int> kept;
    std::vector<std::vector<std::array<int, 2>>> table;
    int next = 0;
    for (auto& a : access_) {
        auto it = kept.find(a.baseRow);
        if (it == kept.end()) {
            kept[a.baseRow] = next;
            table.push_back(variableTable_[a.baseRow]);
            a.baseRow = next++;
        } else {
            a.baseRow = it->second;
        }
    }
    variableTable_.swap(table);
}

}  // namespace symgb
