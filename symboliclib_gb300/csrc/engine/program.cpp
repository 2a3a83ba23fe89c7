// Template -> device program compiler (see program.hpp).
#include "program.hpp"

#include <algorithm>
#include <array>
#include <cstring>
#include <functional>
#include <sstream>
#include <stdexcept>
#include <unordered_map>

namespace symgb {
namespace engine {

namespace {

enum : int {
    N_CONST = 1, N_VAR = 2, N_ADD = 3, N_MUL = 4, N_MULC = 5, N_DIV = 6, N_SQRT = 7, N_SIN = 8, N_COS = 9,
    N_TAN = 10, N_ASIN = 12, N_ACOS = 13, N_ATAN = 14, N_EXP = 15, N_LOG = 16, N_POW = 17, N_ASSIGN = 18,
    N_NEG = 23, N_DEFINE = 24, N_BLOCK = 25, N_REC = 26
};
constexpr int G_OUTPUT = -2, G_INDEX = -3, G_CONSTANT = -4, G_LOCAL = 253;

struct Val {
    int reg;
    bool temp;  // the register may be overwritten / released by the consumer
};

class Compiler {
public:
    Compiler(const symgb_kernel_desc& k, int math) : k_(k), fast_(math == SYMGB_MATH_FAST) {
        const int n = (int)k.num_nodes;
        if (n == 0) throw std::runtime_error("empty template");
        kids_.resize(n);
        std::vector<int> stack;
        for (int j = 0; j < n; ++j) {
            const int nc = k.nodes[j].nchild;
            if (nc < 0 || nc > (int)stack.size()) throw std::runtime_error("malformed template node list");
            kids_[j].assign(stack.end() - nc, stack.end());
            stack.erase(stack.end() - nc, stack.end());
            stack.push_back(j);
        }
        if (stack.size() != 1) throw std::runtime_error("template is not a single tree");
        root_ = stack.back();
        countLocalUses(root_);
        collectLoads(root_);
    }

    Program run() {
        // Load section: one register per distinct load, in first-use order.
        for (auto& key : loadOrder_) {
            const int d = alloc();
            loadReg_[key] = d;
            const int kind = (int)(key >> 62);
            if (kind == 1) {  // gather
                const int row = (int)((key >> 32) & 0xffff);
                const std::int32_t off = (std::int32_t)(std::uint32_t)(key & 0xffffffffu);
                prog_.loads.push_back((std::uint64_t)OP_LDX | ((std::uint64_t)d << 8) | ((std::uint64_t)row << 16) |
                                      ((std::uint64_t)(std::uint32_t)off << 32));
                ++prog_.stats.gathers;
            } else {  // per-instance constant
                const std::uint32_t row = (std::uint32_t)(key & 0xffffffffu);
                prog_.loads.push_back(encode(OP_LDC, d, 0, 0, row));
            }
        }
        scheduleStatements();
        prog_.words.push_back(encode(OP_END, 0, 0, 0, 0));
        prog_.registers = maxReg_;
        return std::move(prog_);
    }

private:
    const symgb_node& node(int j) const { return k_.nodes[j]; }

    // Key of a load leaf: kind (1 gather, 2 constant) in bits 62-63.
    std::uint64_t loadKey(const symgb_node& nd) const {
        if (nd.b == G_INDEX) {
            if (nd.a < 0 || (std::uint32_t)nd.a >= k_.num_access) throw std::runtime_error("index variable out of range");
            const int row = k_.access[2 * nd.a], off = k_.access[2 * nd.a + 1];
            if (row < 0 || row > 0xffff || (std::uint32_t)row >= k_.num_index_rows)
                throw std::runtime_error("index row out of range");
            return (1ull << 62) | ((std::uint64_t)row << 32) | (std::uint64_t)(std::uint32_t)off;
        }
        if (nd.a < 0 || (std::uint32_t)nd.a >= k_.num_constant_rows) throw std::runtime_error("constant row out of range");
        return (2ull << 62) | (std::uint64_t)(std::uint32_t)nd.a;
    }

    void collectLoads(int j) {
        const symgb_node& nd = node(j);
        if (nd.op == N_VAR && (nd.b == G_INDEX || nd.b == G_CONSTANT)) {
            const std::uint64_t key = loadKey(nd);
            if (loadUses_[key]++ == 0) loadOrder_.push_back(key);
        }
        for (int c : kids_[j]) collectLoads(c);
    }

    // Flattens nested BLOCKs into the statement list, in order.
    void flatten(int j, std::vector<int>& out) const {
        if (node(j).op == N_BLOCK) {
            for (int c : kids_[j]) flatten(c, out);
        } else {
            out.push_back(j);
        }
    }

    void localsRead(int j, std::vector<int>& out) const {
        const symgb_node& nd = node(j);
        if (nd.op == N_VAR && nd.b == G_LOCAL && std::find(out.begin(), out.end(), nd.a) == out.end()) out.push_back(nd.a);
        for (int c : kids_[j]) localsRead(c, out);
    }

    // Emits statements in demand order: every output assignment in template
    // order, each preceded by the definitions it still needs (depth first).
    // This keeps definitions close to their uses, so fewer values are live
    // at once.  Statements only assign distinct outputs or locals, so their
    // order does not change any value.  Definitions no output needs are dropped.
    void scheduleStatements() {
        std::vector<int> stmts;
        flatten(root_, stmts);
        std::unordered_map<int, int> defOf;  // local id -> statement
        for (int st : stmts)
            if (node(st).op == N_DEFINE) defOf[node(kids_[st][0]).a] = st;
        std::unordered_map<int, char> emitted;
        std::function<void(int)> emit = [&](int st) {
            if (emitted[st]) return;
            emitted[st] = 1;
            std::vector<int> needs;
            localsRead(kids_[st][1], needs);
            for (int l : needs) {
                auto it = defOf.find(l);
                if (it != defOf.end()) emit(it->second);
            }
            statement(st);
        };
        for (int st : stmts)
            if (node(st).op != N_DEFINE) emit(st);
    }

    void countLocalUses(int j) {
        const symgb_node& nd = node(j);
        if (nd.op == N_VAR && nd.b == G_LOCAL) ++uses_[nd.a];
        const bool isDef = nd.op == N_DEFINE;
        for (std::size_t c = 0; c < kids_[j].size(); ++c) {
            if (isDef && c == 0) continue;  // the defined name is not a use
            countLocalUses(kids_[j][c]);
        }
    }

    int alloc() {
        int r;
        if (!free_.empty()) {
            r = free_.back();
            free_.pop_back();
        } else {
            r = maxReg_++;
            if (maxReg_ > MAX_REGISTERS) throw std::runtime_error("template needs more than 255 live values");
        }
        return r;
    }
    void release(int r) { free_.push_back(r); }
    void consume(const Val& v) {
        if (v.temp) release(v.reg);
    }

    void emit(std::uint64_t w) { prog_.words.push_back(w); }

    // Destination for an operation on the given operands: reuse the first
    // temporary operand register and release the other temporaries.  Sources
    // are read before the destination is written, so reuse is safe.
    int dstFor(std::initializer_list<Val> ops) {
        int temps[4];
        int nt = 0;
        for (const Val& v : ops)
            if (v.temp && std::find(temps, temps + nt, v.reg) == temps + nt) temps[nt++] = v.reg;
        for (int t = 1; t < nt; ++t) release(temps[t]);
        return nt ? temps[0] : alloc();
    }

    Val binary(int op, Val a, Val b) {
        const int d = dstFor({a, b});
        emit(encode(op, d, a.reg, b.reg, 0));
        ++prog_.stats.flops;
        return {d, true};
    }

    Val unary(int op, Val a) {
        const int d = dstFor({a});
        emit(encode(op, d, a.reg, 0, 0));
        return {d, true};
    }

    Val fma(Val a, Val b, Val c, int flags) {
        const int d = dstFor({a, b, c});
        emit(encode(OP_FMA, d, a.reg, b.reg, (std::uint32_t)(c.reg & 0xff) | ((std::uint32_t)flags << 8)));
        prog_.stats.flops += 2;
        return {d, true};
    }

    bool isProduct(int j) const {
        const symgb_node& nd = node(j);
        return (nd.op == N_MUL && kids_[j].size() >= 2) || nd.op == N_MULC;
    }

    // Compiles all factors but the last of a product; returns (partial, last).
    std::pair<Val, Val> productOperands(int j) {
        const auto& ks = kids_[j];
        Val acc = expr(ks[0]);
        for (std::size_t c = 1; c + 1 < ks.size(); ++c) acc = binary(OP_MUL, acc, expr(ks[c]));
        Val last = expr(ks.back());
        return {acc, last};
    }

    Val sum(int j) {
        const auto& ks = kids_[j];
        if (ks.size() == 1) return expr(ks[0]);
        bool have = false, pending = false;
        Val acc{0, false}, pa{0, false}, pb{0, false};
        int pflags = 0;
        for (std::size_t c = 0; c < ks.size(); ++c) {
            const int ch = ks[c];
            const bool negated = node(ch).op == N_NEG;
            const int inner = negated ? kids_[ch][0] : ch;
            if (fast_ && isProduct(inner)) {
                auto pr = productOperands(inner);
                const int fl = negated ? FMA_NEG_PRODUCT : 0;
                if (have) {
                    acc = fma(pr.first, pr.second, acc, fl);
                } else if (pending) {
                    Val prev = binary(OP_MUL, pa, pb);
                    if (pflags & FMA_NEG_PRODUCT) prev = unary(OP_NEG, prev);
                    acc = fma(pr.first, pr.second, prev, fl);
                    pending = false;
                    have = true;
                } else {
                    pa = pr.first;
                    pb = pr.second;
                    pflags = fl;
                    pending = true;
                }
                continue;
            }
            if (have && negated) {  // acc + -(e) == acc - e exactly
                acc = binary(OP_SUB, acc, expr(inner));
                continue;
            }
            Val v = expr(ch);
            if (pending) {
                acc = fma(pa, pb, v, pflags);
                pending = false;
                have = true;
            } else if (!have) {
                acc = v;
                have = true;
            } else {
                acc = binary(OP_ADD, acc, v);
            }
        }
        if (pending) {
            acc = binary(OP_MUL, pa, pb);
            if (pflags & FMA_NEG_PRODUCT) acc = unary(OP_NEG, acc);
        }
        return acc;
    }

    Val product(int j) {
        const auto& ks = kids_[j];
        Val acc = expr(ks[0]);
        for (std::size_t c = 1; c < ks.size(); ++c) acc = binary(OP_MUL, acc, expr(ks[c]));
        return acc;
    }

    Val expr(int j) {
        const symgb_node& nd = node(j);
        switch (nd.op) {
            case N_CONST: {
                const int d = alloc();
                emit(encode(OP_LDK, d, 0, 0, 0));
                std::uint64_t bits;
                std::memcpy(&bits, &nd.value, 8);
                emit(bits);
                ++prog_.stats.constLoads;
                return {d, true};
            }
            case N_VAR: {
                if (nd.b == G_LOCAL) {
                    auto it = regOf_.find(nd.a);
                    if (it == regOf_.end()) throw std::runtime_error("local value used before its definition");
                    const bool last = --uses_[nd.a] == 0;
                    return {it->second, last};
                }
                if (nd.b == G_INDEX || nd.b == G_CONSTANT) {
                    const std::uint64_t key = loadKey(nd);
                    const bool last = --loadUses_[key] == 0;
                    return {loadReg_.at(key), last};
                }
                throw std::runtime_error("unsupported variable group in template");
            }
            case N_ADD: return sum(j);
            case N_MUL: return product(j);
            case N_MULC: return product(j);
            case N_DIV: {
                Val a = expr(kids_[j][0]);
                Val b = expr(kids_[j][1]);
                Val r = binary(fast_ ? OP_FDIV : OP_DIV, a, b);
                --prog_.stats.flops;
                ++prog_.stats.divs;
                return r;
            }
            case N_NEG: {
                Val r = unary(OP_NEG, expr(kids_[j][0]));
                ++prog_.stats.flops;
                return r;
            }
            case N_SQRT: {
                Val r = unary(fast_ ? OP_FSQRT : OP_SQRT, expr(kids_[j][0]));
                ++prog_.stats.sqrts;
                return r;
            }
            case N_REC: {
                Val r = unary(fast_ ? OP_FREC : OP_REC, expr(kids_[j][0]));
                ++prog_.stats.divs;
                return r;
            }
            case N_POW: {
                Val a = expr(kids_[j][0]);
                Val b = expr(kids_[j][1]);
                const int d = dstFor({a, b});
                emit(encode(OP_POW, d, a.reg, b.reg, 0));
                ++prog_.stats.transcendentals;
                return {d, true};
            }
            case N_SIN: case N_COS: case N_TAN: case N_ASIN: case N_ACOS: case N_ATAN: case N_EXP: case N_LOG: {
                static const std::unordered_map<int, int> m = {{N_SIN, OP_SIN}, {N_COS, OP_COS}, {N_TAN, OP_TAN},
                                                               {N_ASIN, OP_ASIN}, {N_ACOS, OP_ACOS}, {N_ATAN, OP_ATAN},
                                                               {N_EXP, OP_EXP}, {N_LOG, OP_LOG}};
                Val r = unary(m.at(nd.op), expr(kids_[j][0]));
                ++prog_.stats.transcendentals;
                return r;
            }
            default:
                throw std::runtime_error("operation " + std::to_string(nd.op) + " cannot be executed on the device");
        }
    }

    void statement(int j) {
        const symgb_node& nd = node(j);
        if (nd.op == N_BLOCK) {  // nested statement list
            for (int s : kids_[j]) statement(s);
        } else if (nd.op == N_DEFINE) {
            const symgb_node& name = node(kids_[j][0]);
            if (name.op != N_VAR || name.b != G_LOCAL) throw std::runtime_error("DEFINE of a non-local");
            Val v = expr(kids_[j][1]);
            if (uses_[name.a] == 0) {  // defined but never read
                consume(v);
                return;
            }
            if (!v.temp) {  // alias of another live local: copy
                const int d = alloc();
                emit(encode(OP_MOV, d, v.reg, 0, 0));
                v = {d, true};
            }
            regOf_[name.a] = v.reg;
        } else if (nd.op == N_ASSIGN) {
            const symgb_node& out = node(kids_[j][0]);
            if (out.op != N_VAR || out.b != G_OUTPUT) throw std::runtime_error("ASSIGN to a non-output");
            if (out.a < 0 || (std::uint32_t)out.a >= k_.num_output_rows) throw std::runtime_error("output row out of range");
            if ((std::uint32_t)out.a >= ENTRY_FIELD_LIMIT) throw std::runtime_error("more than 2^24 output rows");
            Val v = expr(kids_[j][1]);
            emit(encode(OP_ST, 0, v.reg, 0, (std::uint32_t)out.a));
            ++prog_.stats.stores;
            consume(v);
        } else {
            throw std::runtime_error("template statement is neither DEFINE nor ASSIGN");
        }
    }

    const symgb_kernel_desc& k_;
    bool fast_;
    std::vector<std::vector<int>> kids_;
    int root_ = 0;
    std::unordered_map<int, int> uses_, regOf_;
    std::unordered_map<std::uint64_t, int> loadUses_, loadReg_;
    std::vector<std::uint64_t> loadOrder_;
    std::vector<int> free_;
    int maxReg_ = 0;
    Program prog_;
};


// ------------------------------------------------------------------ bundling

bool isBinary(int op) {
    return op == OP_ADD || op == OP_SUB || op == OP_MUL || op == OP_DIV || op == OP_FDIV || op == OP_POW;
}
bool isFma(int op) { return op == OP_FMA || op == OP_FMS || op == OP_FNMA || op == OP_FNMS; }

std::vector<LinOp> parseLinear(const std::vector<std::uint64_t>& w) {
    std::vector<LinOp> ops;
    for (std::size_t pc = 0; pc < w.size();) {
        const std::uint64_t x = w[pc++];
        const int op = (int)(x & 0xff);
        if (op == OP_END) break;
        const int d = (int)((x >> 8) & 0xff), a = (int)((x >> 16) & 0xff), b = (int)((x >> 24) & 0xff);
        LinOp L;
        L.op = op;
        switch (op) {
            case OP_LDK:
                L.d = d;
                if (pc >= w.size()) throw std::runtime_error("truncated literal");
                L.lit = w[pc++];
                break;
            case OP_ST:
                L.src[0] = a;
                L.nsrc = 1;
                L.row = (std::uint32_t)((x >> 32) & 0xffffff);
                break;
            case OP_FMA: {
                static const int byFlags[4] = {OP_FMA, OP_FNMA, OP_FMS, OP_FNMS};
                L.op = byFlags[(x >> 40) & 3];
                L.d = d;
                L.src[0] = a;
                L.src[1] = b;
                L.src[2] = (int)((x >> 32) & 0xff);
                L.nsrc = 3;
                break;
            }
            default:
                L.d = d;
                L.src[0] = a;
                L.nsrc = 1;
                if (isBinary(op)) {
                    L.src[1] = b;
                    L.nsrc = 2;
                }
        }
        ops.push_back(L);
    }
    return ops;
}

// Schedules the linear code into bundles and assigns registers (see the
// description of the program format).
Program bundle(const Program& lin, int window, int literalLoads) {
    std::vector<LinOp> ops = parseLinear(lin.words);
    const int n = (int)ops.size();
    const int nl = (int)lin.loads.size();

    // Value numbering: loads are values 0..nl-1, then one value per definition.
    std::vector<int> cur(256, -1);
    for (int i = 0; i < nl; ++i) cur[(lin.loads[i] >> 8) & 0xff] = i;
    std::vector<int> defOf(n, -1), producer(nl, -1);
    std::vector<std::array<int, 3>> use(n, {-1, -1, -1});
    std::vector<std::vector<int>> deps(n);
    std::unordered_map<std::uint32_t, int> lastStore;
    for (int j = 0; j < n; ++j) {
        const LinOp& L = ops[j];
        for (int s = 0; s < L.nsrc; ++s) {
            const int v = cur[L.src[s]];
            if (v < 0) throw std::runtime_error("program reads a register before writing it");
            use[j][s] = v;
            if (producer[v] >= 0) deps[j].push_back(producer[v]);
        }
        if (L.op == OP_ST) {  // two stores to one output keep their order
            auto it = lastStore.find(L.row);
            if (it != lastStore.end()) deps[j].push_back(it->second);
            lastStore[L.row] = j;
        }
        if (L.d >= 0) {
            defOf[j] = (int)producer.size();
            producer.push_back(j);
            cur[L.d] = defOf[j];
        }
    }
    // Negations folded into their readers, values unchanged: a + -x = a - x and
    // -x + b = b - x (IEEE defines a - b as a + -b, and addition commutes),
    // a - -x = a + x, and an FMA multiplicand or addend -x flips the FMA's sign
    // (the interpreter computes FNMA and FMS as FMAs of negated operands).  A
    // negation is dropped when every reader takes it.
    std::vector<char> dropped(n, 0);
    {
        std::vector<std::vector<int>> readersOf(producer.size());
        for (int j = 0; j < n; ++j)
            for (int s = 0; s < ops[j].nsrc; ++s)
                if (readersOf[use[j][s]].empty() || readersOf[use[j][s]].back() != j) readersOf[use[j][s]].push_back(j);
        auto fmaFlags = [](int op) {
            return op == OP_FNMA ? FMA_NEG_PRODUCT
                   : op == OP_FMS ? FMA_NEG_ADDEND
                   : op == OP_FNMS ? FMA_NEG_PRODUCT | FMA_NEG_ADDEND
                                   : 0;
        };
        static const int fmaOf[4] = {OP_FMA, OP_FNMA, OP_FMS, OP_FNMS};
        auto redirect = [&](int j, int from, int to) {  // j's dependency on `from` becomes one on `to`
            const auto d = std::find(deps[j].begin(), deps[j].end(), from);
            if (d != deps[j].end()) deps[j].erase(d);
            if (to >= 0 && std::find(deps[j].begin(), deps[j].end(), to) == deps[j].end()) deps[j].push_back(to);
        };
        for (int g = 0; g < n; ++g) {
            if (ops[g].op != OP_NEG || defOf[g] < 0) continue;
            const int v = defOf[g], x = use[g][0];
            const std::vector<int>& rs = readersOf[v];
            bool ok = !rs.empty();
            for (int j : rs) {
                const LinOp& L = ops[j];
                const bool at0 = use[j][0] == v, at1 = L.nsrc > 1 && use[j][1] == v;
                if (L.op == OP_ADD)
                    ok = ok && !(at0 && at1);
                else if (L.op == OP_SUB)
                    ok = ok && !at0;
                else if (!isFma(L.op))
                    ok = false;
            }
            if (!ok) continue;
            for (int j : rs) {
                LinOp& L = ops[j];
                if (L.op == OP_ADD || L.op == OP_SUB) {
                    if (L.op == OP_ADD && use[j][0] == v) {
                        std::swap(L.src[0], L.src[1]);
                        std::swap(use[j][0], use[j][1]);
                    }
                    L.op = L.op == OP_ADD ? OP_SUB : OP_ADD;
                    use[j][1] = x;
                } else {
                    int flags = fmaFlags(L.op);
                    for (int q = 0; q < 3; ++q)
                        if (use[j][q] == v) {
                            use[j][q] = x;
                            flags ^= q < 2 ? FMA_NEG_PRODUCT : FMA_NEG_ADDEND;
                        }
                    L.op = fmaOf[flags];
                }
                redirect(j, g, producer[x]);
                readersOf[x].push_back(j);
            }
            dropped[g] = 1;
        }
    }

    // Literal loads of the load section: the `literalLoads` most read distinct
    // literals become values nv0 .. nv - 1, loaded before any arithmetic; every
    // read of one of their literal-load operations reads that value instead,
    // and those operations are dropped.
    const int nv0 = (int)producer.size();
    std::vector<std::uint64_t> loadedLiterals;
    {
        auto literalRead = [&](int v) { return v < nv0 && producer[v] >= 0 && ops[producer[v]].op == OP_LDK; };
        std::unordered_map<std::uint64_t, int> reads;
        for (int j = 0; j < n; ++j)
            for (int s = 0; !dropped[j] && s < ops[j].nsrc; ++s)
                if (literalRead(use[j][s])) ++reads[ops[producer[use[j][s]]].lit];
        std::vector<std::pair<int, std::uint64_t>> order;
        for (const auto& r : reads) order.push_back({r.second, r.first});
        std::sort(order.begin(), order.end(), [](const auto& a, const auto& b) {
            return a.first != b.first ? a.first > b.first : a.second < b.second;
        });
        if ((int)order.size() > literalLoads) order.resize(std::max(0, literalLoads));
        std::unordered_map<std::uint64_t, int> valueOf;
        for (const auto& o : order) {
            valueOf[o.second] = (int)producer.size();
            producer.push_back(-1);
            loadedLiterals.push_back(o.second);
        }
        for (int j = 0; j < n; ++j)
            for (int s = 0; !dropped[j] && s < ops[j].nsrc; ++s) {
                const int v = use[j][s];
                if (!literalRead(v)) continue;
                const auto it = valueOf.find(ops[producer[v]].lit);
                if (it == valueOf.end()) continue;
                const auto d = std::find(deps[j].begin(), deps[j].end(), producer[v]);
                if (d != deps[j].end()) deps[j].erase(d);
                use[j][s] = it->second;
            }
        std::vector<int> readers(producer.size(), 0);
        for (int j = 0; j < n; ++j)
            for (int s = 0; !dropped[j] && s < ops[j].nsrc; ++s) ++readers[use[j][s]];
        for (int j = 0; j < n; ++j)
            if (ops[j].op == OP_LDK && readers[defOf[j]] == 0) dropped[j] = 1;
    }
    const int nv = (int)producer.size();

    // List scheduling: among the next `window` unscheduled operations, take
    // every ready operation of the most frequent opcode as one bundle.
    constexpr int NOWHERE = 1 << 30;  // bundle index of a dropped operation
    std::vector<int> bundleOf(n, -1);
    for (int j = 0; j < n; ++j)
        if (dropped[j]) bundleOf[j] = NOWHERE;
    std::vector<std::vector<int>> bundles;
    int frontier = 0;
    while (frontier < n && bundleOf[frontier] >= 0) ++frontier;
    std::vector<std::vector<int>> byOp(NUM_OPCODES);
    while (frontier < n) {
        for (auto& v : byOp) v.clear();
        int firstOp = -1;
        for (int j = frontier, seen = 0; j < n && seen < std::max(1, window); ++j) {
            if (bundleOf[j] >= 0) continue;
            ++seen;
            bool ready = true;
            for (int p : deps[j])
                if (bundleOf[p] < 0) {
                    ready = false;
                    break;
                }
            if (!ready) continue;
            byOp[ops[j].op].push_back(j);
            if (firstOp < 0) firstOp = ops[j].op;
        }
        int best = firstOp;
        for (int o = 0; o < NUM_OPCODES; ++o)
            if (byOp[o].size() > byOp[best].size()) best = o;
        std::vector<int>& chosen = byOp[best];
        if (chosen.size() > 0xffff) chosen.resize(0xffff);
        const int b = (int)bundles.size();
        for (int j : chosen) bundleOf[j] = b;
        bundles.push_back(chosen);
        while (frontier < n && bundleOf[frontier] >= 0) ++frontier;
    }

    // Accumulator forwarding between consecutive single-entry bundles: a value
    // whose every read is in the next bundle stays in the accumulator.
    const int nb = (int)bundles.size();
    auto viaBundle = [](int op) {  // operations the interpreter runs through runBundle
        return op == OP_LDK || op == OP_ADD || op == OP_SUB || op == OP_MUL || op == OP_DIV || op == OP_NEG ||
               op == OP_MOV || op == OP_SQRT || op == OP_REC || op == OP_FDIV || op == OP_FSQRT || op == OP_FREC ||
               isFma(op);
    };
    std::vector<int> useCount(nv, 0);
    for (int j = 0; j < n; ++j)
        for (int s = 0; !dropped[j] && s < ops[j].nsrc; ++s) ++useCount[use[j][s]];
    std::vector<std::uint32_t> headerFlags(nb, 0);
    std::vector<char> inAccOnly(nv, 0);
    for (int b = 0; b + 1 < nb; ++b) {
        if (bundles[b].size() != 1 || bundles[b + 1].size() != 1) continue;
        const int j = bundles[b][0], k = bundles[b + 1][0];
        const int v = defOf[j];
        if (v < 0 || !viaBundle(ops[j].op) || !(viaBundle(ops[k].op) || ops[k].op == OP_ST) || ops[k].op == OP_LDK)
            continue;
        int here = 0;
        std::uint32_t f = 0;
        for (int s = 0; s < ops[k].nsrc; ++s)
            if (use[k][s] == v) {
                ++here;
                f |= H_A_ACC << s;
            }
        if (here == 0 || here != useCount[v]) continue;
        headerFlags[b + 1] |= f;
        headerFlags[b] |= H_NOSTORE;
        inAccOnly[v] = 1;
    }

    // Registers: a value occupies its register from its defining bundle (or the
    // load section) through its last reading bundle.
    std::vector<int> lastUse(nv, -1);
    for (int j = 0; j < n; ++j)
        for (int s = 0; !dropped[j] && s < ops[j].nsrc; ++s)
            lastUse[use[j][s]] = std::max(lastUse[use[j][s]], bundleOf[j]);
    std::vector<std::vector<int>> freeAfter(nb + 1);
    std::vector<int> slot(nv, -1), pool;
    int nregs = 0;
    auto alloc = [&]() {
        if (!pool.empty()) {
            const int r = pool.back();
            pool.pop_back();
            return r;
        }
        if (nregs >= MAX_REGISTERS) throw std::runtime_error("template needs more than 255 live values");
        return nregs++;
    };
    auto loadValue = [&](int v) {
        slot[v] = alloc();
        freeAfter[std::max(0, lastUse[v])].push_back(v);
    };
    for (int v = 0; v < nl; ++v) loadValue(v);
    for (int v = nv0; v < nv; ++v) loadValue(v);
    Program out;
    out.stats = lin.stats;
    for (int b = 0; b < nb; ++b) {
        for (int j : bundles[b])
            if (defOf[j] >= 0) {
                const int v = defOf[j];
                if (inAccOnly[v]) {
                    slot[v] = 0;  // never written to the register file
                    continue;
                }
                slot[v] = alloc();
                freeAfter[std::max(b, lastUse[v])].push_back(v);
            }
        for (int v : freeAfter[b]) pool.push_back(slot[v]);
    }
    out.registers = nregs;

    std::vector<std::uint64_t> literals;
    std::unordered_map<std::uint64_t, std::uint32_t> literalIndex;
    auto literalOf = [&](std::uint64_t bits) {
        auto it = literalIndex.find(bits);
        if (it == literalIndex.end()) {
            it = literalIndex.emplace(bits, (std::uint32_t)literals.size()).first;
            literals.push_back(bits);
        }
        if (it->second >= ENTRY_FIELD_LIMIT) throw std::runtime_error("too many literals");
        return it->second;
    };
    for (int i = 0; i < nl; ++i)
        out.loads.push_back((lin.loads[i] & ~0xff00ull) | ((std::uint64_t)slot[i] << 8));
    for (int t = 0; t < nv - nv0; ++t)
        out.loads.push_back((std::uint64_t)OP_LDK | ((std::uint64_t)slot[nv0 + t] << 8) |
                            ((std::uint64_t)literalOf(loadedLiterals[t]) << 32));

    for (int b = 0; b < nb; ++b) {
        const auto& B = bundles[b];
        const int op = ops[B[0]].op;
        out.words.push_back((std::uint64_t)op | ((std::uint64_t)B.size() << 8) | headerFlags[b]);
        std::uint64_t pair = 0;
        for (std::size_t q = 0; q < B.size(); ++q) {
            const int j = B[q];
            const LinOp& L = ops[j];
            std::uint32_t e = 0;
            if (op == OP_ST) {
                e = (std::uint32_t)slot[use[j][0]] | (L.row << 8);
            } else if (op == OP_LDK) {
                e = (std::uint32_t)slot[defOf[j]] | (literalOf(L.lit) << 8);
            } else {
                e = (std::uint32_t)slot[defOf[j]];
                for (int s = 0; s < L.nsrc; ++s) e |= (std::uint32_t)slot[use[j][s]] << (8 * (s + 1));
            }
            if (q & 1) {
                out.words.push_back(pair | ((std::uint64_t)e << 32));
            } else {
                pair = e;
                if (q + 1 == B.size()) out.words.push_back(pair);
            }
        }
        out.operations += (int)B.size();
    }
    out.bundles = nb;
    out.words.push_back(OP_END);
    out.literalOffset = (std::uint32_t)out.words.size();
    out.words.insert(out.words.end(), literals.begin(), literals.end());
    return out;
}

}  // namespace

std::vector<LinOp> linearCode(const symgb_kernel_desc& k, int math, std::vector<std::uint64_t>* loads) {
    Compiler c(k, math);
    Program linear = c.run();
    if (loads) *loads = linear.loads;
    return parseLinear(linear.words);
}

Program compileTemplate(const symgb_kernel_desc& k, int math, int window, int literalLoads) {
    Compiler c(k, math);
    Program linear = c.run();
    // A wide window can keep more than MAX_REGISTERS values live; narrower
    // windows keep fewer (window 1 is the linear code's own order).  Literals
    // loaded up front are live from the start: without them as the last resort.
    for (int lits : {literalLoads, 0}) {
        for (int w = window;; w /= 2) {
            try {
                return bundle(linear, w, lits);
            } catch (const std::runtime_error&) {
                if (w <= 1 && lits == 0) throw;
                if (w <= 1) break;
            }
        }
    }
    throw std::runtime_error("template needs more than 255 live values");
}

std::string disassemble(const Program& p) {
    static const char* names[NUM_OPCODES] = {"end", "ldx", "ldc", "ldk", "st", "add", "sub", "mul", "div",
                                             "neg", "sqrt", "rec", "fma", "sin", "cos", "tan", "asin", "acos",
                                             "atan", "exp", "log", "pow", "mov", "fms", "fnma", "fnms",
                                             "fdiv", "fsqrt", "frec"};
    std::ostringstream os;
    for (std::uint64_t w : p.loads) {
        const int op = (int)(w & 0xff), d = (int)((w >> 8) & 0xff);
        const std::int32_t imm = (std::int32_t)(w >> 32);
        if (op == OP_LDX) {
            os << "ldx r" << d << " row" << ((w >> 16) & 0xffff) << " off" << imm << "\n";
        } else if (op == OP_LDK) {
            double v;
            std::memcpy(&v, &p.words[p.literalOffset + (std::uint32_t)imm], 8);
            os << "ldk r" << d << " " << v << "\n";
        } else {
            os << "ldc r" << d << " crow" << imm << "\n";
        }
    }
    for (std::size_t pc = 0; pc < p.words.size();) {
        const std::uint64_t h = p.words[pc++];
        const int op = (int)(h & 0xff);
        if (op == OP_END) break;
        const unsigned cnt = (unsigned)((h >> 8) & 0xffff);
        os << (op < NUM_OPCODES ? names[op] : "?") << " x" << cnt;
        if (h & H_A_ACC) os << " a=acc";
        if (h & H_B_ACC) os << " b=acc";
        if (h & H_C_ACC) os << " c=acc";
        if (h & H_NOSTORE) os << " nostore";
        os << ":";
        for (unsigned q = 0; q < cnt; ++q) {
            const std::uint32_t e = (std::uint32_t)(p.words[pc + q / 2] >> (32 * (q & 1)));
            const unsigned f0 = e & 0xff, f1 = (e >> 8) & 0xff, f2 = (e >> 16) & 0xff, f3 = e >> 24;
            os << " [";
            if (op == OP_ST) {
                os << "y" << (e >> 8) << "=r" << f0;
            } else if (op == OP_LDK) {
                double v;
                std::memcpy(&v, &p.words[p.literalOffset + (e >> 8)], 8);
                os << "r" << f0 << "=" << v;
            } else {
                os << "r" << f0 << "=r" << f1;
                if (isBinary(op) || isFma(op)) os << ",r" << f2;
                if (isFma(op)) os << ",r" << f3;
            }
            os << "]";
        }
        pc += (cnt + 1) / 2;
        os << "\n";
    }
    return os.str();
}

}  // namespace engine
}  // namespace symgb
