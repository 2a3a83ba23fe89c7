// Expression traversals with the visiting orders of reference src/Traverse.cpp
// and src/Traverse.hpp.  The orders matter: the decomposition numbers repeated
// sub-expressions in first-visit order, and memoised rewrites key their caches
// by node identity or algebraic hash.
#pragma once
#include <unordered_map>
#include <unordered_set>
#include <utility>
#include <vector>

#include "symbolic.hpp"

namespace symgb {

struct IdentityHash {
    std::size_t operator()(long long h) const { return (std::size_t)h; }
};

template <class T>
using NodeMap = std::unordered_map<long long, T, IdentityHash>;

// Depth-first pre-order with an explicit stack: a node's children are pushed
// in order and popped last-first (reference Traverse.cpp:11-37).  `fun`
// returns whether to descend.  With `unique`, each node identity is visited once.
template <class F>
void preOrderTraverse(const Symbolic& root, F&& fun, bool unique = false) {
    std::unordered_set<long long> visited;
    std::vector<const Symbolic*> stack;
    stack.push_back(&root);
    while (!stack.empty()) {
        const Symbolic* x = stack.back();
        stack.pop_back();
        if (unique && !visited.insert(x->id()).second) continue;
        if (fun(*x)) {
            const unsigned nc = x->numChilds();
            for (unsigned i = 0; i < nc; ++i) stack.push_back(&(*x)[i]);
        }
    }
}

// Children visited in order 0..n-1; `pre` decides whether to enter a node,
// `post` runs after all entered children (reference Traverse.cpp:39-63).
template <class Pre, class Post>
void prePostOrderTraverse(const Symbolic& root, Pre&& pre, Post&& post) {
    if (!pre(root)) return;
    std::vector<std::pair<const Symbolic*, unsigned>> stack;
    stack.emplace_back(&root, 0u);
    while (!stack.empty()) {
        const Symbolic* x = stack.back().first;
        const unsigned cnt = stack.back().second;
        const unsigned nc = x->numChilds();
        if (cnt == nc) {
            post(*x);
            stack.pop_back();
        } else {
            ++stack.back().second;
            const Symbolic* c = &(*x)[cnt];
            if (pre(*c)) stack.emplace_back(c, 0u);
        }
    }
}

template <class Post>
void postOrderTraverse(const Symbolic& root, Post&& post) {
    prePostOrderTraverse(root, [](const Symbolic&) { return true; }, post);
}

// Memoised bottom-up rewrite (reference Traverse.hpp:18-51).  `pre` maps a node
// before it is entered, `post(node, childValues)` produces its value.  The memo
// is keyed by node identity or, with `byHash`, by algebraic hash; values are
// stored under the key of the pre-mapped node and looked up with the key of the
// original child, as in the reference.
template <class T, class Pre, class Post>
T traverseGenerate(const Symbolic& root, Pre&& pre, Post&& post, NodeMap<T>& memo, bool byHash = false) {
    std::vector<std::pair<Symbolic, unsigned>> stack;
    std::vector<T> values;
    stack.emplace_back(pre(root), 0u);
    while (!stack.empty()) {
        const unsigned cnt = stack.back().second;
        const unsigned nc = stack.back().first.numChilds();
        if (cnt == nc) {
            Symbolic x = stack.back().first;
            std::vector<T> childValues(values.end() - nc, values.end());
            T val = post(x, childValues);
            memo[byHash ? x.ahash() : x.id()] = val;
            values.erase(values.end() - nc, values.end());
            values.push_back(std::move(val));
            stack.pop_back();
        } else {
            ++stack.back().second;
            const Symbolic& c = stack.back().first[cnt];
            auto it = memo.find(byHash ? c.ahash() : c.id());
            if (it != memo.end()) {
                values.push_back(it->second);
            } else {
                Symbolic pc = pre(c);
                stack.emplace_back(std::move(pc), 0u);
            }
        }
    }
    assert(values.size() == 1);
    return values.front();
}

template <class T, class Pre, class Post>
T traverseGenerate(const Symbolic& root, Pre&& pre, Post&& post, bool byHash = false) {
    NodeMap<T> memo;
    return traverseGenerate<T>(root, pre, post, memo, byHash);
}

template <class T, class Post>
T traverseGenerateIdentity(const Symbolic& root, Post&& post, NodeMap<T>& memo, bool byHash = false) {
    return traverseGenerate<T>(root, [](const Symbolic& x) { return x; }, post, memo, byHash);
}

template <class T, class Post>
T traverseGenerateIdentity(const Symbolic& root, Post&& post) {
    NodeMap<T> memo;
    return traverseGenerate<T>(root, [](const Symbolic& x) { return x; }, post, memo, false);
}

// All distinct nodes of one operation type, in unique pre-order
// (reference Traverse.cpp:69-77).
inline std::vector<Symbolic> harvestOp(OpType op, const Symbolic& x) {
    std::vector<Symbolic> ret;
    preOrderTraverse(x, [&](const Symbolic& y) {
        if (y.op() == op) ret.push_back(y);
        return true;
    }, true);
    return ret;
}

}  // namespace symgb
