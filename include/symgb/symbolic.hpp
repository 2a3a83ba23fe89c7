// Symbolic expression IR of the engine's front end.
//
// A Symbolic is a reference-counted handle to an immutable expression node.
// Nodes are shared by handle copies, never hash-consed: the decomposition
// counts repeated sub-expressions by node identity (reference
// src/Decomposition.cpp:266-288 keys its counts by Symbolic::id()), so two
// structurally equal expressions built separately stay two nodes, exactly as in
// the reference.  Hashes and complexities follow src/Symbolic.cpp:61-131 and
// src/Symbolic.cpp:168-174; the arithmetic operators build the same node shapes
// as src/Operations.cpp:114-166.
#pragma once
#include <array>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include "hashing.hpp"
#include "ops.hpp"

namespace symgb {

class Symbolic {
public:
    struct Node {
        std::uint32_t ref;
        OpType op;
        std::uint8_t complexity;
        std::uint32_t numChilds;
        hash_t algebraicHash;
        union {
            Symbolic* childs;
            double constant;
            std::array<int, 2> variable;
        };
    };

    Node* data = nullptr;

    Symbolic() = default;
    Symbolic(double c);  // constant leaf (implicit, like the reference)
    Symbolic(int id, int group);  // variable leaf
    Symbolic(OpType op, const Symbolic& c0);
    Symbolic(OpType op, const Symbolic& c0, const Symbolic& c1);
    Symbolic(OpType op, const std::vector<Symbolic>& childs);
    // Takes ownership of `childs`, an array from childArray(n).
    Symbolic(OpType op, Symbolic* childs, unsigned n);
    // An array of n empty handles for the constructor above (pooled for
    // short arrays).
    static Symbolic* childArray(unsigned n);

    Symbolic(const Symbolic& a) : data(a.data) {
        if (data) addRef(data);
    }
    Symbolic(Symbolic&& a) noexcept : data(a.data) { a.data = nullptr; }
    Symbolic& operator=(const Symbolic& a) {
        if (a.data) addRef(a.data);
        release();
        data = a.data;
        return *this;
    }
    Symbolic& operator=(Symbolic&& a) noexcept {
        if (this != &a) {
            release();
            data = a.data;
            a.data = nullptr;
        }
        return *this;
    }
    ~Symbolic() { release(); }

    static Symbolic generateUniqueVariable();
    static int& uniqueVariableCounter();

    OpType op() const { return data ? data->op : NOOP; }
    const std::array<int, 2>& variable() const { return data->variable; }
    double constant() const { return data->constant; }
    unsigned numChilds() const { return (data && op() != CONST && op() != VAR) ? data->numChilds : 0; }
    const Symbolic& operator[](std::size_t i) const {
        assert(data && i < numChilds());
        return data->childs[i];
    }
    const Symbolic* begin() const { return numChilds() ? data->childs : nullptr; }
    const Symbolic* end() const { return numChilds() ? data->childs + data->numChilds : nullptr; }
    hash_t algebraicHash() const { return data ? data->algebraicHash : NOOPHash; }
    hash_t ahash() const { return algebraicHash(); }
    unsigned char complexity() const { return data->complexity; }
    long long id() const { return (long long)(std::uintptr_t)data; }
    bool operator<(const Symbolic& x) const { return ahash() < x.ahash(); }
    bool operator==(const Symbolic& x) const { return ahash() == x.ahash(); }

    hash_t computeStructureHash() const;

    // Reference counts are plain integers, except inside a ConcurrentRefs
    // scope, where several threads may copy and drop handles to shared nodes
    // and every count update is atomic.
    struct ConcurrentRefs {
        ConcurrentRefs();
        ~ConcurrentRefs();
        ConcurrentRefs(const ConcurrentRefs&) = delete;
        ConcurrentRefs& operator=(const ConcurrentRefs&) = delete;
    };
    static bool concurrentRefs() { return __atomic_load_n(&concurrentScopes_, __ATOMIC_RELAXED) != 0; }

private:
    static inline int concurrentScopes_ = 0;  // open ConcurrentRefs scopes, any thread
    static void addRef(Node* n) {
        if (concurrentRefs())
            __atomic_add_fetch(&n->ref, 1u, __ATOMIC_RELAXED);
        else
            ++n->ref;
    }
    void release();
    void finish();  // computes hash and complexity of a freshly built node
    static Node* allocate(OpType op, unsigned numChilds);
    static void freeChildArray(Symbolic* p, unsigned n);
};

struct AlgebraicHashLess {
    bool operator()(const Symbolic& a, const Symbolic& b) const { return a.ahash() < b.ahash(); }
};

// Live node count (diagnostics and leak tests); exact while no other thread
// is creating or freeing nodes.
long long liveNodeCount();

// Arithmetic with the reference's node shapes.
Symbolic operator*(const Symbolic& a, const Symbolic& b);
Symbolic operator+(const Symbolic& a, const Symbolic& b);
Symbolic operator/(const Symbolic& a, const Symbolic& b);
Symbolic operator-(const Symbolic& a, const Symbolic& b);
Symbolic operator-(const Symbolic& a);
inline Symbolic& operator*=(Symbolic& a, const Symbolic& b) { return a = a * b; }
inline Symbolic& operator+=(Symbolic& a, const Symbolic& b) { return a = a + b; }
inline Symbolic& operator/=(Symbolic& a, const Symbolic& b) { return a = a / b; }
inline Symbolic& operator-=(Symbolic& a, const Symbolic& b) { return a = a - b; }
Symbolic sqrt(const Symbolic& a);

// Scalar evaluation of one operation (reference src/Operations.cpp:64-96 plus
// the remaining unary functions the engine executes).
double evaluateOp(OpType op, const double* childValues, unsigned n);

// A decomposed sub-expression (reference src/Symbolic.hpp:189-203).
struct ExpressionBlock {
    Symbolic x;
    hash_t structureHash = 0;
    int level = 0;
    std::vector<int> childs;
};

}  // namespace symgb
