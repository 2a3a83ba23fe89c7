// Symbolic differentiation of the front end.
//
// differentiate(): reverse mode over the expression DAG with the rules of the
// reference (src/Operations.cpp:9-61, src/SymbolicDifferentiation.cpp:12-44).
// hessianCached(): forward-mode gradient and Hessian with a hash-keyed
// expression cache (src/SymbolicDifferentiation.hpp:70-147), including its
// quirks - a product with a constant falls through to the general product
// rule, and a variable outside the list counts as the first variable.
// hessianSparse(): per summand of a sum, the Hessian of that summand with
// respect to the variables it contains, made fixed, as (row, col, expr)
// triplets of the upper triangle (src/SymbolicDifferentiation.hpp:234-278).
// Rules exist for +, *, constant *, /, sqrt, 1/x - as in the reference.
#pragma once
#include <iostream>
#include <tuple>
#include <unordered_map>
#include <utility>
#include <vector>

#include "parallel.hpp"
#include "symbolic.hpp"
#include "traverse.hpp"
#include "utilities.hpp"

namespace symgb {

// Memoises built nodes by algebraic hash; expressions whose hash is a small
// integer (|h| <= 32) become that constant (reference Symbolic.hpp:175-189).
class CachedFactory {
public:
    template <class... Args>
    Symbolic operator()(const Args&... args) {
        Symbolic x(args...);
        if (x.ahash() <= 32 && x.ahash() >= -32) return Symbolic((double)x.ahash());
        Symbolic& y = cache_[x.ahash()];
        if (y.op() == NOOP) y = x;
        return y;
    }

private:
    std::unordered_map<hash_t, Symbolic> cache_;
};

// One reverse-mode step: pushes (child, adjoint) pairs of `x = (expr, adjoint)`.
inline void differentiateStep(const std::pair<Symbolic, Symbolic>& x, std::vector<std::pair<Symbolic, Symbolic>>& stack) {
    const Symbolic& e = x.first;
    const Symbolic& d = x.second;
    switch (e.op()) {
        case ASSIGN: stack.emplace_back(e[1], d); break;
        case ADD:
            for (const auto& c : e) stack.emplace_back(c, d);
            break;
        case MUL:
            for (unsigned i = 0; i < e.numChilds(); ++i) {
                std::vector<Symbolic> others;
                for (unsigned j = 0; j < e.numChilds(); ++j)
                    if (j != i) others.push_back(e[j]);
                others.push_back(d);
                stack.emplace_back(e[i], Symbolic(MUL, others));
            }
            break;
        case MULC: stack.emplace_back(e[1], d * e[0]); break;
        case DIV:
            stack.emplace_back(e[0], Symbolic(1.0) / e[1] * d);
            stack.emplace_back(e[1], -e[0] / (e[1] * e[1]) * d);
            break;
        case RECIPROCAL: stack.emplace_back(e[0], Symbolic(-1.0) / (e[0] * e[0]) * d); break;
        case SQRT: stack.emplace_back(e[0], Symbolic(0.5) / Symbolic(SQRT, e[0]) * d); break;
        default: std::cout << opInfo(e.op()).symbol << " not implemented\n"; break;
    }
}

// Gradient of `expr` with respect to `vars` (reverse mode).
inline std::vector<Symbolic> differentiate(const Symbolic& expr, const std::vector<Symbolic>& vars) {
    std::vector<Symbolic> grad(vars.size(), Symbolic(0.0));
    std::vector<std::pair<Symbolic, Symbolic>> stack{{expr, Symbolic(1.0)}};
    std::unordered_map<hash_t, int> varMap;
    for (int i = 0; i < (int)vars.size(); ++i) varMap[vars[i].ahash()] = i;
    while (!stack.empty()) {
        auto x = stack.back();
        stack.pop_back();
        const OpType op = x.first.op();
        if (op == VAR) {
            auto it = varMap.find(x.first.ahash());
            if (it != varMap.end()) grad[it->second] += x.second;
        } else if (op != CONST) {
            differentiateStep(x, stack);
        }
    }
    return grad;
}

// Gradient and Hessian by forward differentiation with a shared cache.
inline std::vector<std::vector<Symbolic>> hessianCached(const Symbolic& x, const std::vector<Symbolic>& vars) {
    std::unordered_map<hash_t, std::size_t> varId;
    for (std::size_t i = 0; i < vars.size(); ++i) varId[vars[i].ahash()] = i;
    CachedFactory cf;
    const std::size_t nv = vars.size();
    auto diff = [&](const Symbolic& y, const std::vector<std::vector<Symbolic>>& cg) {
        std::vector<Symbolic> ret(nv, Symbolic(0.0));
        switch (y.op()) {
            case ADD:
                for (std::size_t j = 0; j < nv; ++j) ret[j] = cf(ADD, cg[0][j], cg[1][j]);
                break;
            case MULC:
                for (std::size_t j = 0; j < nv; ++j)
                    if (cg[1][j].ahash()) ret[j] = cf(MULC, y[0], cg[1][j]);
                [[fallthrough]];
            case MUL:
                for (std::size_t j = 0; j < nv; ++j)
                    if (cg[0][j].ahash() || cg[1][j].ahash())
                        ret[j] = cf(ADD, cf(MUL, y[1], cg[0][j]), cf(MUL, y[0], cg[1][j]));
                break;
            case DIV:
                for (std::size_t j = 0; j < nv; ++j)
                    if (cg[0][j].ahash() || cg[1][j].ahash())
                        ret[j] = cf(ADD, cf(DIV, cg[0][j], y[1]),
                                    cf(MULC, Symbolic(-1.0), cf(DIV, cf(MUL, y[0], cg[1][j]), cf(MUL, y[1], y[1]))));
                break;
            case SQRT:
                for (std::size_t j = 0; j < nv; ++j)
                    if (cg[0][j].ahash()) ret[j] = cf(DIV, cg[0][j], cf(MULC, Symbolic(2.0), y));
                break;
            case VAR: ret[varId[y.ahash()]] = Symbolic(1.0); break;
            case CONST: break;
            default: std::cout << "diff rule not implemented" << std::endl;
        }
        return ret;
    };
    NodeMap<std::vector<Symbolic>> cache;
    auto grad = traverseGenerateIdentity<std::vector<Symbolic>>(x, diff, cache, true);
    std::vector<std::vector<Symbolic>> hess(nv);
    for (std::size_t i = 0; i < nv; ++i) hess[i] = traverseGenerateIdentity<std::vector<Symbolic>>(grad[i], diff, cache, true);
    return hess;
}

// (row, col, expression) entries of the upper triangle of the Hessian of a sum
// of energies; each summand's Hessian block is made fixed.  The summands are
// independent: their blocks are built on the front end's worker pool, the
// fixed blocks' variables numbered from per-summand counts in summand order
// (the numbers the summand-by-summand loop gives), and the entries emitted in
// summand order, so the result does not depend on the thread count.
inline std::vector<std::tuple<int, int, Symbolic>> hessianSparse(const Symbolic& x, const std::vector<Symbolic>& vars) {
    std::unordered_map<hash_t, std::size_t> varId;
    for (std::size_t i = 0; i < vars.size(); ++i) varId[vars[i].ahash()] = i;
    if (x.op() != ADD) throw std::invalid_argument("hessianSparse expects a sum of energies");
    const std::size_t n = x.numChilds();
    std::vector<std::vector<std::vector<Symbolic>>> blocks(n);
    std::vector<std::vector<std::size_t>> ids(n);
    std::vector<int> first(n + 1, 0);
    auto rowSpans = [&](std::size_t t) {
        std::vector<std::pair<Symbolic*, std::size_t>> d;
        for (auto& r : blocks[t]) d.emplace_back(r.data(), r.size());
        return d;
    };
    {
        Symbolic::ConcurrentRefs concurrent;
        parallelFor(n, 16, [&](std::size_t b, std::size_t e) {
            for (std::size_t t = b; t < e; ++t) {
                const Symbolic& c = x[t];
                std::vector<Symbolic> local;
                for (auto& v : harvestOp(VAR, c)) {
                    auto it = varId.find(v.ahash());
                    if (it != varId.end()) {
                        local.push_back(v);
                        ids[t].push_back(it->second);
                    }
                }
                blocks[t] = hessianCached(c, local);
                first[t + 1] = fixedVariableCount(rowSpans(t));
            }
        });
        int& counter = Symbolic::uniqueVariableCounter();
        first[0] = counter;
        for (std::size_t t = 0; t < n; ++t) first[t + 1] += first[t];
        parallelFor(n, 16, [&](std::size_t b, std::size_t e) {
            for (std::size_t t = b; t < e; ++t) makeFixedSpansAt(rowSpans(t), first[t]);
        });
        counter = first[n];
    }
    std::vector<std::tuple<int, int, Symbolic>> ret;
    for (std::size_t t = 0; t < n; ++t) {
        const auto& h = blocks[t];
        for (std::size_t i = 0; i < ids[t].size(); ++i)
            for (std::size_t j = 0; j < ids[t].size(); ++j)
                if (ids[t][i] <= ids[t][j]) ret.emplace_back((int)ids[t][i], (int)ids[t][j], h[i][j]);
    }
    {
        Symbolic::ConcurrentRefs concurrent;
        parallelFor(n, 256, [&](std::size_t b, std::size_t e) {
            for (std::size_t t = b; t < e; ++t) blocks[t] = {};
        });
    }
    return ret;
}

}  // namespace symgb
