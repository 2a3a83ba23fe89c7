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

// Open-addressing map from a 64-bit key (a node identity or hash) to V, for
// the front end's hot lookup tables.  Only lookup and insert are offered, so
// unlike an iterated container it cannot change any result order.
template <class V>
class KeyMap {
public:
    explicit KeyMap(std::size_t expected = 16) {
        std::size_t cap = 16;
        while (cap < 2 * expected) cap <<= 1;
        keys_.assign(cap, kEmpty);
        vals_.resize(cap);
    }
    V& operator[](long long key) {
        if (2 * (size_ + 1) > keys_.size()) grow();
        std::size_t i = slot(key);
        if (keys_[i] == kEmpty) {
            keys_[i] = key;
            vals_[i] = V();
            ++size_;
        }
        return vals_[i];
    }
    V* find(long long key) {
        const std::size_t i = slot(key);
        return keys_[i] == kEmpty ? nullptr : &vals_[i];
    }
    std::size_t size() const { return size_; }

private:
    static constexpr long long kEmpty = (long long)0x8000000000000001ULL;
    std::size_t slot(long long key) const {
        const std::size_t mask = keys_.size() - 1;
        std::size_t i = (std::size_t)(((unsigned long long)key * 0x9e3779b97f4a7c15ULL) >> 17) & mask;
        while (keys_[i] != kEmpty && keys_[i] != key) i = (i + 1) & mask;
        return i;
    }
    void grow() {
        std::vector<long long> k;
        std::vector<V> v;
        k.swap(keys_);
        v.swap(vals_);
        keys_.assign(k.size() * 2, kEmpty);
        vals_.resize(k.size() * 2);
        size_ = 0;
        for (std::size_t j = 0; j < k.size(); ++j)
            if (k[j] != kEmpty) {
                const std::size_t i = slot(k[j]);
                keys_[i] = k[j];
                vals_[i] = std::move(v[j]);
                ++size_;
            }
    }
    std::vector<long long> keys_;
    std::vector<V> vals_;
    std::size_t size_ = 0;
};

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
