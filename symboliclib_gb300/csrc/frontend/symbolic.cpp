// Symbolic node construction, hashing and arithmetic.
#include "symgb/symbolic.hpp"

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <mutex>
#include <new>

#include "symgb/parallel.hpp"
#include "symgb/traverse.hpp"

namespace symgb {

namespace {

// Reflected CRC-64 table of the Jones polynomial (0xad93d23594c935a9, bit
// reversed 0x95ac9329ac4bc9b5), generated rather than written out.
struct Crc64Table {
    std::uint64_t t[256];
    Crc64Table() {
        const std::uint64_t poly = 0x95ac9329ac4bc9b5ULL;
        for (int i = 0; i < 256; ++i) {
            std::uint64_t c = (std::uint64_t)i;
            for (int k = 0; k < 8; ++k) c = (c & 1) ? (c >> 1) ^ poly : (c >> 1);
            t[i] = c;
        }
    }
};

// Live node count: one counter per thread (a single shared atomic would be
// contended by every allocation of the parallel front-end passes), summed on
// demand.  Counters are never freed, so a thread's net count survives it.
struct LiveCounters {
    std::mutex m;
    std::vector<long long*> all;
};
LiveCounters& liveCounters() {
    static LiveCounters* c = new LiveCounters();
    return *c;
}
long long& liveNodes() {
    static thread_local long long* mine = [] {
        auto* p = new long long(0);
        std::lock_guard<std::mutex> g(liveCounters().m);
        liveCounters().all.push_back(p);
        return p;
    }();
    return *mine;
}

// Nodes are small and created by the million; a per-thread free list keeps
// allocation off the general-purpose heap.  The list is threaded through the
// free nodes themselves (the link lives in the union of a dead node), so
// freeing the hundreds of millions of nodes of a large expression graph
// touches no other memory.
struct NodePool {
    Symbolic::Node* head = nullptr;
    static Symbolic::Node*& link(Symbolic::Node* p) { return *reinterpret_cast<Symbolic::Node**>(&p->childs); }
    Symbolic::Node* get() {
        if (!head) {
            const std::size_t n = 4096;
            auto* slab = static_cast<Symbolic::Node*>(std::malloc(n * sizeof(Symbolic::Node)));
            if (!slab) throw std::bad_alloc();
            for (std::size_t i = 0; i < n; ++i) link(slab + i) = i + 1 < n ? slab + i + 1 : nullptr;
            head = slab;
        }
        Symbolic::Node* p = head;
        head = link(p);
        return p;
    }
    void put(Symbolic::Node* p) {
        link(p) = head;
        head = p;
    }
};

// One global pool guarded by a mutex would serialise the front end; nodes are
// instead returned to the free list of the thread that frees them.  Slabs are
// never returned to the heap, so a node may be freed by any thread and handles
// with static storage duration stay valid until exit.
NodePool& pool() {
    static thread_local NodePool p;
    return p;
}

// Child arrays of up to kPooledChilds handles come from per-size free lists
// (same ownership rules as nodes, linked through their first handle's
// storage); longer arrays use new[].
constexpr unsigned kPooledChilds = 8;
struct ChildPool {
    void* head[kPooledChilds + 1] = {};
    static void*& link(void* p) { return *static_cast<void**>(p); }
    void* get(unsigned n) {
        void*& h = head[n];
        if (!h) {
            const std::size_t count = 2048, bytes = n * sizeof(Symbolic);
            char* slab = static_cast<char*>(std::malloc(count * bytes));
            if (!slab) throw std::bad_alloc();
            for (std::size_t i = 0; i < count; ++i) link(slab + i * bytes) = i + 1 < count ? slab + (i + 1) * bytes : nullptr;
            h = slab;
        }
        void* p = h;
        h = link(p);
        return p;
    }
    void put(void* p, unsigned n) {
        link(p) = head[n];
        head[n] = p;
    }
};

ChildPool& childPool() {
    static thread_local ChildPool p;
    return p;
}

}  // namespace

const std::uint64_t* crc64Table() {
    static const Crc64Table table;
    return table.t;
}

namespace {

// Zero-byte steps of the CRC as 64x64 matrices over GF(2), one per power of
// two: column j of step[k] is the state that 2^k zero bytes make of bit j.
struct Crc64Shifts {
    std::uint64_t step[64][64];
    static std::uint64_t apply(const std::uint64_t (&m)[64], std::uint64_t v) {
        std::uint64_t r = 0;
        for (int j = 0; v; ++j, v >>= 1)
            if (v & 1) r ^= m[j];
        return r;
    }
    Crc64Shifts() {
        const std::uint64_t* tab = crc64Table();
        for (int j = 0; j < 64; ++j) {
            const std::uint64_t c = 1ULL << j;
            step[0][j] = tab[(std::uint8_t)c] ^ (c >> 8);
        }
        for (int k = 1; k < 64; ++k)
            for (int j = 0; j < 64; ++j) step[k][j] = apply(step[k - 1], step[k - 1][j]);
    }
};

const Crc64Shifts& crc64Shifts() {
    static const Crc64Shifts s;
    return s;
}

}  // namespace

std::uint64_t crc64Shift(std::uint64_t crc, std::uint64_t zeroBytes) {
    const Crc64Shifts& s = crc64Shifts();
    for (int k = 0; zeroBytes; ++k, zeroBytes >>= 1)
        if (zeroBytes & 1) crc = Crc64Shifts::apply(s.step[k], crc);
    return crc;
}

hash_t hashVectorParallel(const std::vector<hash_t>& v) {
    constexpr std::size_t kChunk = 4096;  // hashes per chunk
    if (v.size() < 4 * kChunk) return hashVector(v);
    const std::size_t chunks = (v.size() + kChunk - 1) / kChunk;
    std::vector<std::uint64_t> part(chunks);
    parallelFor(chunks, 1, [&](std::size_t b, std::size_t e) {
        for (std::size_t i = b; i < e; ++i) {
            const std::size_t n = std::min(kChunk, v.size() - i * kChunk);
            part[i] = (std::uint64_t)crc64(v.data() + i * kChunk, n * sizeof(hash_t));
        }
    });
    std::uint64_t crc = 0;
    for (std::size_t i = 0; i < chunks; ++i) {
        const std::size_t n = std::min(kChunk, v.size() - i * kChunk);
        crc = crc64Shift(crc, n * sizeof(hash_t)) ^ part[i];
    }
    return (hash_t)crc;
}

long long liveNodeCount() {
    std::lock_guard<std::mutex> g(liveCounters().m);
    long long n = 0;
    for (long long* p : liveCounters().all) n += __atomic_load_n(p, __ATOMIC_RELAXED);
    return n;
}

// One counter per thread: the expressions a thread builds are numbered as a
// program that builds them alone numbers them, whatever other threads build
// at the same time (several front ends may run side by side; the worker
// pool's threads never draw from it).
int& Symbolic::uniqueVariableCounter() {
    static thread_local int counter = 0;
    return counter;
}

Symbolic Symbolic::generateUniqueVariable() {
    return Symbolic(uniqueVariableCounter()++, EXPLICIT_INTERMEDIATE);
}

Symbolic::Node* Symbolic::allocate(OpType op, unsigned numChilds) {
    Node* n = pool().get();
    n->ref = 1;
    n->op = op;
    n->complexity = 0;
    n->numChilds = numChilds;
    n->algebraicHash = 0;
    n->childs = nullptr;
    ++liveNodes();
    return n;
}

Symbolic* Symbolic::childArray(unsigned n) {
    if (n == 0) return nullptr;
    if (n > kPooledChilds) return new Symbolic[n];
    Symbolic* p = static_cast<Symbolic*>(childPool().get(n));
    for (unsigned i = 0; i < n; ++i) new (p + i) Symbolic();
    return p;
}

void Symbolic::freeChildArray(Symbolic* p, unsigned n) {
    if (!p) return;
    if (n > kPooledChilds) {
        delete[] p;
        return;
    }
    for (unsigned i = 0; i < n; ++i) p[i].~Symbolic();
    childPool().put(p, n);
}

Symbolic::ConcurrentRefs::ConcurrentRefs() { __atomic_add_fetch(&concurrentScopes_, 1, __ATOMIC_SEQ_CST); }
Symbolic::ConcurrentRefs::~ConcurrentRefs() { __atomic_sub_fetch(&concurrentScopes_, 1, __ATOMIC_SEQ_CST); }

void Symbolic::release() {
    if (!data) return;
    const bool last = concurrentRefs() ? __atomic_sub_fetch(&data->ref, 1u, __ATOMIC_ACQ_REL) == 0 : --data->ref == 0;
    if (last) {
        if (data->op != CONST && data->op != VAR && data->numChilds) freeChildArray(data->childs, data->numChilds);
        pool().put(data);
        --liveNodes();
    }
    data = nullptr;
}

Symbolic::Symbolic(double c) {
    data = allocate(CONST, 0);
    data->constant = c;
    finish();
}

Symbolic::Symbolic(int id, int group) {
    data = allocate(VAR, 0);
    data->variable = {id, group};
    finish();
}

Symbolic::Symbolic(OpType op, const Symbolic& c0) {
    data = allocate(op, 1);
    data->childs = childArray(1);
    data->childs[0] = c0;
    finish();
}

Symbolic::Symbolic(OpType op, const Symbolic& c0, const Symbolic& c1) {
    data = allocate(op, 2);
    data->childs = childArray(2);
    data->childs[0] = c0;
    data->childs[1] = c1;
    finish();
}

Symbolic::Symbolic(OpType op, const std::vector<Symbolic>& childs) {
    data = allocate(op, (unsigned)childs.size());
    if (!childs.empty()) {
        data->childs = childArray((unsigned)childs.size());
        std::copy(childs.begin(), childs.end(), data->childs);
    }
    finish();
}

Symbolic::Symbolic(OpType op, Symbolic* childs, unsigned n) {
    data = allocate(op, n);
    data->childs = n ? childs : nullptr;
    finish();
}

// Algebraic hash (reference Symbolic.cpp:61-116): sums and products combine
// child hashes commutatively (wrapping integer + and *), constants hash to their
// integer value when integral, everything else chains CRC hashes.
void Symbolic::finish() {
    Node& d = *data;
    const unsigned n = d.numChilds;
    const Symbolic* ch = (d.op == CONST || d.op == VAR) ? nullptr : d.childs;
    std::uint64_t h = 0;
    bool done = false;
    switch (d.op) {
        case MUL:
        case MULC:
            h = 1;
            for (unsigned i = 0; i < n; ++i) {
                const std::uint64_t ci = ch[i].op() == ADD ? (std::uint64_t)hashPair(opInfo(ADD).seed, ch[i].ahash())
                                                           : (std::uint64_t)ch[i].ahash();
                h *= ci;
            }
            break;
        case ADD:
            h = 0;
            for (unsigned i = 0; i < n; ++i) {
                const std::uint64_t ci = (ch[i].op() == MUL || ch[i].op() == MULC)
                                             ? (std::uint64_t)hashPair(opInfo(MUL).seed, ch[i].ahash())
                                             : (std::uint64_t)ch[i].ahash();
                h += ci;
            }
            break;
        case CONST: {
            const double c = d.constant;
            if (c == 0.0) {
                h = 0;
            } else if (c == (double)(hash_t)c) {
                h = (std::uint64_t)(hash_t)c;
            } else {
                h = (std::uint64_t)hashValue(c);
            }
            break;
        }
        case VAR:
            h = (std::uint64_t)hashPair(opInfo(VAR).seed, hashVariable(d.variable));
            break;
        default:
            if (d.op == DIV) {
                if (ch[0].ahash() == 0) {
                    h = 0;
                    done = true;
                } else if (ch[0].ahash() == ch[1].ahash()) {
                    h = 1;
                    done = true;
                }
            }
            if (!done) {
                hash_t hh = opInfo(d.op).seed;
                for (unsigned i = 0; i < n; ++i) {
                    const OpType opi = ch[i].op();
                    if (opi == MULC || opi == MUL || opi == ADD)
                        hh = hashPair(hh, hashPair(opInfo(opi).seed, ch[i].ahash()));
                    else
                        hh = hashPair(hh, ch[i].ahash());
                }
                h = (std::uint64_t)hh;
            }
    }
    d.algebraicHash = (hash_t)h;

    // Complexity (reference Symbolic.cpp:119-131), saturating at 255.
    if (!n || d.op == CONST || d.op == VAR) {
        d.complexity = opInfo(d.op).cost;
    } else {
        unsigned tmp = 0;
        for (unsigned i = 0; i < n; ++i) tmp += ch[i].complexity();
        d.complexity = (std::uint8_t)std::min(255u, n * opInfo(d.op).cost + tmp);
    }
}

// Structure hash: post-order CRC chain of child structure hashes and the
// operation seed; leaves hash to their seed (reference Symbolic.cpp:168-174).
hash_t Symbolic::computeStructureHash() const {
    return traverseGenerateIdentity<hash_t>(*this, [](const Symbolic& x, const std::vector<hash_t>& hs) {
        if (hs.empty()) return opInfo(x.op()).seed;
        std::vector<hash_t> all(hs);
        all.push_back(opInfo(x.op()).seed);
        return hashVector(all);
    });
}

Symbolic operator*(const Symbolic& a, const Symbolic& b) {
    if (a.op() == CONST) return Symbolic(MULC, a, b);
    if (b.op() == CONST) return Symbolic(MULC, b, a);
    return Symbolic(MUL, a, b);
}

Symbolic operator+(const Symbolic& a, const Symbolic& b) { return Symbolic(ADD, a, b); }

Symbolic operator/(const Symbolic& a, const Symbolic& b) { return Symbolic(DIV, a, b); }

Symbolic operator-(const Symbolic& a, const Symbolic& b) {
    return Symbolic(ADD, a, Symbolic(MULC, Symbolic(-1.0), b));
}

Symbolic operator-(const Symbolic& a) { return Symbolic(MULC, Symbolic(-1.0), a); }

Symbolic sqrt(const Symbolic& a) { return Symbolic(SQRT, a); }

double evaluateOp(OpType op, const double* v, unsigned n) {
    switch (op) {
        case ADD: {
            double r = 0.0;
            for (unsigned i = 0; i < n; ++i) r += v[i];
            return r;
        }
        case MUL: {
            double r = 1.0;
            for (unsigned i = 0; i < n; ++i) r *= v[i];
            return r;
        }
        case MULC: return v[0] * v[1];
        case DIV: return v[0] / v[1];
        case SQRT: return std::sqrt(v[0]);
        case NEG: return -v[0];
        case RECIPROCAL: return 1.0 / v[0];
        case SIN: return std::sin(v[0]);
        case COS: return std::cos(v[0]);
        case TAN: return std::tan(v[0]);
        case ASIN: return std::asin(v[0]);
        case ACOS: return std::acos(v[0]);
        case ATAN: return std::atan(v[0]);
        case EXP: return std::exp(v[0]);
        case LOG: return std::log(v[0]);
        case POW: return std::pow(v[0], v[1]);
        default: return -1.0;
    }
}

}  // namespace symgb
