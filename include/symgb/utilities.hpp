// Container helpers of the symbolic front end.
#pragma once
#include <unordered_map>
#include <utility>
#include <vector>

#include "symbolic.hpp"
#include "traverse.hpp"

namespace symgb {

namespace detail {
inline void collect(std::vector<std::pair<Symbolic*, std::size_t>>&) {}
template <class C, class... Rest>
void collect(std::vector<std::pair<Symbolic*, std::size_t>>& out, C& c, Rest&... rest) {
    out.emplace_back(c.data(), (std::size_t)c.size());
    collect(out, rest...);
}
}  // namespace detail

// Marks the given entries as one fixed block: every distinct expression (by
// algebraic hash) gets a fresh EXPLICIT_INTERMEDIATE variable, all of them are
// assigned inside one BLOCK, and each entry becomes FIXED(variable, block).
// The decomposition never splits a fixed block, so the block is evaluated as
// one kernel instance (reference src/SymbolicUtilities.hpp:52-86).
// The variables are numbered firstId, firstId + 1, ... in entry order;
// returns how many were used.
inline int makeFixedSpansAt(const std::vector<std::pair<Symbolic*, std::size_t>>& data, int firstId) {
    if (data.empty()) return 0;
    std::unordered_map<hash_t, Symbolic, IdentityHash> exprMap;
    std::vector<Symbolic> assignments;
    int next = firstId;
    for (auto& d : data)
        for (std::size_t i = 0; i < d.second; ++i) {
            Symbolic& var = exprMap[d.first[i].ahash()];
            if (var.op() == NOOP) {
                var = Symbolic(next++, EXPLICIT_INTERMEDIATE);
                assignments.emplace_back(ASSIGN, var, d.first[i]);
            }
        }
    Symbolic block(BLOCK, assignments);
    for (auto& d : data)
        for (std::size_t i = 0; i < d.second; ++i) d.first[i] = Symbolic(FIXED, exprMap[d.first[i].ahash()], block);
    return next - firstId;
}

// Number of variables makeFixedSpansAt would use (distinct algebraic hashes).
inline int fixedVariableCount(const std::vector<std::pair<Symbolic*, std::size_t>>& data) {
    std::unordered_map<hash_t, char, IdentityHash> seen;
    for (auto& d : data)
        for (std::size_t i = 0; i < d.second; ++i) seen.emplace(d.first[i].ahash(), 0);
    return (int)seen.size();
}

// Numbers the variables from the process-wide unique-variable counter, as
// Symbolic::generateUniqueVariable does.
inline void makeFixedSpans(const std::vector<std::pair<Symbolic*, std::size_t>>& data) {
    if (data.empty()) return;
    int& counter = Symbolic::uniqueVariableCounter();
    counter += makeFixedSpansAt(data, counter);
}

template <class... Conts>
void makeFixed(Conts&... conts) {
    std::vector<std::pair<Symbolic*, std::size_t>> data;
    detail::collect(data, conts...);
    makeFixedSpans(data);
}

// makeFixed over the rows of a matrix stored as a vector of rows.
inline void makeFixedRows(std::vector<std::vector<Symbolic>>& rows) {
    std::vector<std::pair<Symbolic*, std::size_t>> data;
    for (auto& r : rows) data.emplace_back(r.data(), r.size());
    makeFixedSpans(data);
}

// Evaluates an expression with values for the variables of one group
// (reference src/SymbolicDifferentiation.hpp:16-26).
template <class Cont>
double evaluate(const Symbolic& x, const Cont& values) {
    const auto* v = values.data();
    return traverseGenerateIdentity<double>(x, [&](const Symbolic& y, const std::vector<double>& c) {
        if (y.op() == CONST) return y.constant();
        if (y.op() == VAR) return (double)v[y.variable()[0]];
        return evaluateOp(y.op(), c.data(), (unsigned)c.size());
    });
}

}  // namespace symgb
