// Source generator of the compiled executor: turns a unit's ComputeKernel
// templates into one CUDA C++ module for NVRTC (see codegen.hpp).
//
// Every template is emitted from the same linear code the interpreter's
// programs are bundled from (program.cpp: linearCode), one statement per
// operation, each with the same CUDA rounding intrinsic the interpreter
// executes (__dadd_rn, __fma_rn, the prelude's fast division ...).  The
// compiler is therefore free to schedule and allocate registers, but not to
// change any value: results are bit-identical to the interpreter's in both
// math modes, and in exact mode to the reference's generated code built
// without FP contraction.  Plan constants (instance counts, table offsets,
// output slots, value sets) are literals of the source, so index arithmetic
// folds at compile time.
//
// A thread takes 1, 2 or 4 work items, either tpb items apart (strided) or as
// consecutive instances of one value set whose index and constant entries it
// reads with vector loads from padded copies of the tables (grouped).  With
// one value set, output rows that no kernel reads may store their results
// straight at their final positions in the unit's result buffer (direct
// result rows, planned by the engine at init).
#include "codegen.hpp"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <sstream>
#include <stdexcept>

#include "program.hpp"

namespace symgb {
namespace engine {

namespace {

std::string u64(std::uint64_t v) { return std::to_string(v) + "ull"; }

std::string literal(std::uint64_t bits) {
    char buf[64];
    std::snprintf(buf, sizeof buf, "__longlong_as_double((long long)0x%016llxull)", (unsigned long long)bits);
    return buf;
}

const char* libName(int op) {
    switch (op) {
        case OP_SIN: return "sin";
        case OP_COS: return "cos";
        case OP_TAN: return "tan";
        case OP_ASIN: return "asin";
        case OP_ACOS: return "acos";
        case OP_ATAN: return "atan";
        case OP_EXP: return "exp";
        case OP_LOG: return "log";
        default: return nullptr;
    }
}

// Emits the device function evaluating kernel k.
//   Strided items (grouped == nullptr): symgbBody<k><L2>(..., i, s) evaluates
//     one work item (instance i, value set s) and loads its own index and
//     constant entries.
//   Grouped items: symgbGroup<k><L2, IT, FULL>(..., g, s) evaluates the IT
//     consecutive instances g*IT .. g*IT+IT-1 of value set s; each index and
//     constant row is read with one vector load from the padded copies of the
//     tables (`grouped` gives their row bases), the instances' gathers,
//     arithmetic and stores follow, unrolled.  FULL = false guards the
//     instances past the kernel's end (the last group).
// Output rows with a start in `direct` (>= 0) store their results into
// res[dp[start + i]] (their final positions) instead of x.  L2 = 1 reads x
// through L2 only (values written earlier in the same launch, persistent
// schedule).  Returns the number of operations of the template.
std::size_t emitBody(std::ostringstream& os, int k, const symgb_kernel_desc& d, int math, unsigned S,
                     const GroupedTables* grouped, const std::vector<std::int64_t>* direct) {
    std::vector<std::uint64_t> loads;
    const std::vector<LinOp> ops = linearCode(d, math, &loads);
    const std::uint64_t n = d.num_instances;
    const bool g = grouped != nullptr;
    const char* in = g ? "        " : "    ";
    os << "// kernel " << k << ": " << n << " instances, level " << d.level << ", " << loads.size() << " loads, "
       << ops.size() << " operations\n";
    if (g)
        os << "template <int L2, int IT, bool FULL>\n__device__ __forceinline__ void symgbGroup" << k
           << "(const double* SYMGB_XR x, double* SYMGB_XR xw, const unsigned* __restrict__ p, "
              "const double* __restrict__ c, double* __restrict__ res, const unsigned* __restrict__ dp, "
              "unsigned long long g, unsigned s) {\n";
    else
        os << "template <int L2>\n__device__ __forceinline__ void symgbBody" << k
           << "(const double* SYMGB_XR x, double* SYMGB_XR xw, const unsigned* __restrict__ p, "
              "const double* __restrict__ c, double* __restrict__ res, const unsigned* __restrict__ dp, "
              "unsigned long long i, unsigned s) {\n";
    std::vector<std::string> cur(256);
    int next = 0;
    auto fresh = [&](int reg) -> std::string {
        std::string v = "v" + std::to_string(next++);
        if (reg < 0 || reg >= (int)cur.size()) throw std::runtime_error("codegen: register out of range");
        cur[reg] = v;
        return v;
    };
    auto use = [&](int reg) -> const std::string& {
        if (reg < 0 || reg >= (int)cur.size() || cur[reg].empty())
            throw std::runtime_error("codegen: register read before written");
        return cur[reg];
    };
    const std::string xs = S == 1 ? std::string() : " * " + std::to_string(S) + "ull + s";
    // Index rows read by the gathers, each loaded once (correlated index
    // variables share a row and differ by their offsets); constant rows
    // likewise in the grouped layout.
    std::vector<int> rowVar(d.num_index_rows, -1);
    int rows = 0;
    for (std::uint64_t w : loads) {
        if ((int)(w & 0xff) != OP_LDX) continue;
        const std::uint64_t row = (w >> 16) & 0xffff;
        if (row >= d.num_index_rows) throw std::runtime_error("codegen: index row out of range");
        if (rowVar[row] >= 0) continue;
        rowVar[row] = rows++;
        if (g)
            os << "    unsigned q" << rowVar[row] << "[IT];\n    symgbLoadIdx<IT>(p + "
               << u64(grouped->indexBase[k] + row * grouped->stride[k]) << " + g * IT, q" << rowVar[row] << ");\n";
        else
            os << "    const unsigned q" << rowVar[row] << " = SYMGB_LD(p + " << u64(d.index_offset + row * n)
               << " + i);\n";
    }
    std::vector<int> constVar;
    if (g) {
        constVar.assign(d.num_constant_rows, -1);
        int consts = 0;
        for (std::uint64_t w : loads) {
            if ((int)(w & 0xff) != OP_LDC) continue;
            const std::uint32_t row = (std::uint32_t)(w >> 32);
            if (row >= d.num_constant_rows) throw std::runtime_error("codegen: constant row out of range");
            if (constVar[row] >= 0) continue;
            constVar[row] = consts++;
            os << "    double k" << constVar[row] << "[IT];\n    symgbLoadConst<IT>(c + "
               << u64(grouped->constBase[k] + row * grouped->stride[k]) << " + g * IT, k" << constVar[row] << ");\n";
        }
        os << "    #pragma unroll\n    for (int j = 0; j < IT; ++j) {\n"
           << "        const unsigned long long i = g * IT + j;\n"
           << "        if (!FULL && i >= " << u64(n) << ") break;\n";
    }
    const std::string qj = g ? "[j]" : "";
    for (std::uint64_t w : loads) {
        const int op = (int)(w & 0xff), dst = (int)((w >> 8) & 0xff);
        const std::uint32_t imm = (std::uint32_t)(w >> 32);
        if (op == OP_LDX) {
            const std::uint64_t row = (w >> 16) & 0xffff;
            const std::string v = fresh(dst);
            os << in << "const double " << v << " = symgbLoadX<L2>(x + (unsigned long long)(q" << rowVar[row] << qj
               << " + " << imm << "u)" << xs << ");\n";
        } else if (op == OP_LDC) {
            const std::string v = fresh(dst);
            if (g)
                os << in << "const double " << v << " = k" << constVar[imm] << "[j];\n";
            else
                os << in << "const double " << v << " = SYMGB_LD(c + "
                   << u64(d.constants_offset + (std::uint64_t)imm * n) << " + i);\n";
        } else {
            throw std::runtime_error("codegen: unknown load word");
        }
    }
    for (const LinOp& L : ops) {
        std::string rhs;
        switch (L.op) {
            case OP_ST:
                if (direct && L.row < direct->size() && (*direct)[L.row] >= 0)
                    os << in << "res[SYMGB_LD(dp + " << u64((std::uint64_t)(*direct)[L.row]) << " + i)] = "
                       << use(L.src[0]) << ";\n";
                else
                    os << in << "xw[(" << u64(d.output_offset + (std::uint64_t)L.row * n) << " + i)" << xs
                       << "] = " << use(L.src[0]) << ";\n";
                continue;
            case OP_MOV: {
                const std::string src = use(L.src[0]);
                cur[L.d] = src;
                continue;
            }
            case OP_LDK: rhs = literal(L.lit); break;
            case OP_ADD: rhs = "__dadd_rn(" + use(L.src[0]) + ", " + use(L.src[1]) + ")"; break;
            case OP_SUB: rhs = "__dsub_rn(" + use(L.src[0]) + ", " + use(L.src[1]) + ")"; break;
            case OP_MUL: rhs = "__dmul_rn(" + use(L.src[0]) + ", " + use(L.src[1]) + ")"; break;
            case OP_DIV: rhs = "__ddiv_rn(" + use(L.src[0]) + ", " + use(L.src[1]) + ")"; break;
            case OP_NEG: rhs = "symgbNegate(" + use(L.src[0]) + ")"; break;
            case OP_SQRT: rhs = "__dsqrt_rn(" + use(L.src[0]) + ")"; break;
            case OP_REC: rhs = "__ddiv_rn(1.0, " + use(L.src[0]) + ")"; break;
            case OP_FDIV: rhs = "symgbFastDiv(" + use(L.src[0]) + ", " + use(L.src[1]) + ")"; break;
            case OP_FSQRT: rhs = "symgbFastSqrt(" + use(L.src[0]) + ")"; break;
            case OP_FREC: rhs = "symgbFastRec(" + use(L.src[0]) + ")"; break;
            case OP_FMA: rhs = "__fma_rn(" + use(L.src[0]) + ", " + use(L.src[1]) + ", " + use(L.src[2]) + ")"; break;
            case OP_FMS:
                rhs = "__fma_rn(" + use(L.src[0]) + ", " + use(L.src[1]) + ", symgbNegate(" + use(L.src[2]) + "))";
                break;
            case OP_FNMA:
                rhs = "__fma_rn(symgbNegate(" + use(L.src[0]) + "), " + use(L.src[1]) + ", " + use(L.src[2]) + ")";
                break;
            case OP_FNMS:
                rhs = "__fma_rn(symgbNegate(" + use(L.src[0]) + "), " + use(L.src[1]) + ", symgbNegate(" +
                      use(L.src[2]) + "))";
                break;
            case OP_POW: rhs = "pow(" + use(L.src[0]) + ", " + use(L.src[1]) + ")"; break;
            default: {
                const char* f = libName(L.op);
                if (!f) throw std::runtime_error("codegen: operation " + std::to_string(L.op) + " not supported");
                rhs = std::string(f) + "(" + use(L.src[0]) + ")";
            }
        }
        const std::string v = fresh(L.d);
        os << in << "const double " << v << " = " << rhs << ";\n";
    }
    if (g) os << "    }\n";
    os << "}\n\n";
    return ops.size();
}

// Templates of at most this many operations per thread (operations x items)
// get a second, unguarded copy of the items loop for threads whose items are
// all in range: without a bounds check per item the compiler can issue every
// item's index and gather loads before the first item's arithmetic, which is
// what a light, memory-bound template needs.  Heavier templates keep one
// guarded loop (their loads are hidden by arithmetic, and the copy would
// double their compile time).
constexpr std::size_t kSplitOps = 1024;

// Work items of kernel k for block `b0` (relative to the kernel's first
// block): `items` per thread, consecutive threads on consecutive items in
// each of the thread's rounds (coalesced), rounds unrolled so the items'
// loads are in flight together.  `split`: threads whose items are all in
// range take an unguarded copy of the loop (kSplitOps).
void emitItems(std::ostringstream& os, int k, std::uint64_t total, unsigned S, int tpb, int items, int l2,
               const std::string& b0, const char* indent, bool split) {
    os << indent << "const unsigned long long w0 = (" << b0 << ") * " << (std::uint64_t)tpb * items
       << "ull + threadIdx.x;\n";
    if (items > 1 && split) {
        os << indent << "if (w0 + " << u64((std::uint64_t)(items - 1) * tpb) << " < " << u64(total) << ") {\n"
           << indent << "    #pragma unroll\n" << indent << "    for (int j = 0; j < " << items << "; ++j) {\n"
           << indent << "        const unsigned long long w = w0 + (unsigned long long)j * " << tpb << "ull;\n"
           << indent << "        symgbBody" << k << "<" << l2 << ">(x, xw, p, c, res, dp, w / " << S
           << "ull, (unsigned)(w % " << S << "ull));\n"
           << indent << "    }\n" << indent << "} else {\n";
    }
    if (items > 1) os << indent << "#pragma unroll\n" << indent << "for (int j = 0; j < " << items << "; ++j) {\n";
    else os << indent << "{\n" << indent << "    const int j = 0;\n";
    os << indent << "    const unsigned long long w = w0 + (unsigned long long)j * " << tpb << "ull;\n"
       << indent << "    if (w < " << u64(total) << ") symgbBody" << k << "<" << l2 << ">(x, xw, p, c, res, dp, w / "
       << S << "ull, (unsigned)(w % " << S << "ull));\n"
       << indent << "}\n";
    if (items > 1 && split) os << indent << "}\n";
}

std::uint64_t blocksFor(std::uint64_t total, int tpb, int items) {
    const std::uint64_t per = (std::uint64_t)tpb * items;
    return (total + per - 1) / per;
}

// Blocks of kernel k: strided, n*S work items at tpb*items per block;
// grouped, ceil(n / items) groups per value set, one thread each.
std::uint64_t kernelBlocks(const symgb_kernel_desc& d, unsigned S, int tpb, int items, bool grouped) {
    if (!grouped) return blocksFor(d.num_instances * S, tpb, items);
    const std::uint64_t groups = (d.num_instances + items - 1) / items;
    return (groups * S + tpb - 1) / tpb;
}

// Grouped work of kernel k for block `b0` (relative to the kernel's first
// block): thread t takes group t / S of value set t % S (consecutive threads
// on consecutive sets, then groups).  Full groups run without per-instance
// guards when the template is light (`split`), as in emitItems.
void emitGroups(std::ostringstream& os, int k, const symgb_kernel_desc& d, unsigned S, int tpb, int items, int l2,
                const std::string& b0, const char* indent, bool split) {
    const std::uint64_t n = d.num_instances;
    const std::uint64_t groups = (n + items - 1) / items, full = n / items;
    os << indent << "const unsigned long long t = (" << b0 << ") * " << tpb << "ull + threadIdx.x;\n"
       << indent << "const unsigned long long g = t / " << S << "ull;\n"
       << indent << "const unsigned s = (unsigned)(t % " << S << "ull);\n";
    if (split && full)
        os << indent << "if (g < " << u64(full) << ") symgbGroup" << k << "<" << l2 << ", " << items
           << ", true>(x, xw, p, c, res, dp, g, s);\n"
           << indent << "else if (g < " << u64(groups) << ") symgbGroup" << k << "<" << l2 << ", " << items
           << ", false>(x, xw, p, c, res, dp, g, s);\n";
    else
        os << indent << "if (g < " << u64(groups) << ") symgbGroup" << k << "<" << l2 << ", " << items
           << ", false>(x, xw, p, c, res, dp, g, s);\n";
}

// The work of kernel k in either item layout.
void emitWork(std::ostringstream& os, int k, const symgb_kernel_desc& d, std::size_t ops, unsigned S, int tpb,
              int items, int l2, const std::string& b0, const char* indent, bool grouped) {
    const bool split = ops * (std::size_t)items <= kSplitOps;
    if (grouped) emitGroups(os, k, d, S, tpb, items, l2, b0, indent, split);
    else emitItems(os, k, d.num_instances * S, S, tpb, items, l2, b0, indent, split);
}

// Dispatch of block `b` over the kernels of one launch (kernel-major block
// ranges, each kernel's work items in consecutive blocks).
void emitDispatch(std::ostringstream& os, const std::vector<int>& ks, const std::vector<symgb_kernel_desc>& descs,
                  const std::vector<std::size_t>& opCount, unsigned S, int tpb, int items, int l2, const char* indent,
                  bool grouped) {
    std::uint64_t first = 0;
    const std::string inner = std::string(indent) + "    ";
    for (std::size_t q = 0; q < ks.size(); ++q) {
        const int k = ks[q];
        const std::uint64_t blocks = kernelBlocks(descs[k], S, tpb, items, grouped);
        os << indent << (q ? "else " : "") << "if (b < " << u64(first + blocks) << ") {\n";
        emitWork(os, k, descs[k], opCount[k], S, tpb, items, l2, "b - " + u64(first), inner.c_str(), grouped);
        os << indent << "}\n";
        first += blocks;
    }
}

std::uint64_t blocksOf(const std::vector<int>& ks, const std::vector<symgb_kernel_desc>& descs, unsigned S, int tpb,
                       int items, bool grouped) {
    std::uint64_t b = 0;
    for (int k : ks) b += kernelBlocks(descs[k], S, tpb, items, grouped);
    return b;
}

int checkedItems(int items) {
    if (items != 1 && items != 2 && items != 4) throw std::runtime_error("codegen: items per thread must be 1, 2 or 4");
    return items;
}

}  // namespace

extern const char* const kJitPrelude;

namespace {

// `__launch_bounds__(tpb)` or, with a minimum CTA count per SM that fits the
// SM's 2048 threads, `__launch_bounds__(tpb, minBlocks)`.
std::string launchBounds(int tpb, int minBlocks) {
    std::string s = "__launch_bounds__(" + std::to_string(tpb);
    const int fit = std::min(minBlocks, 2048 / std::max(1, tpb));
    if (fit > 0) s += ", " + std::to_string(fit);
    return s + ")";
}

}  // namespace

GroupedTables groupedTables(const std::vector<symgb_kernel_desc>& descs) {
    GroupedTables t;
    for (const auto& d : descs) {
        const std::uint64_t stride = (d.num_instances + 3) / 4 * 4;
        t.stride.push_back(stride);
        t.indexBase.push_back(t.indexSize);
        t.constBase.push_back(t.constSize);
        t.indexSize += stride * d.num_index_rows;
        t.constSize += stride * d.num_constant_rows;
    }
    return t;
}

JitSource generateModule(const std::vector<symgb_kernel_desc>& descs, int numLevels, const JitConfig& cfg) {
    JitSource out;
    std::ostringstream os;
    const unsigned S = cfg.numSets;
    if (cfg.itemLayout != SYMGB_ITEMS_STRIDED && cfg.itemLayout != SYMGB_ITEMS_GROUPED)
        throw std::runtime_error("codegen: unknown item layout");
    const bool grouped = cfg.itemLayout == SYMGB_ITEMS_GROUPED;
    out.grouped = grouped;
    GroupedTables gt;
    if (grouped) gt = groupedTables(descs);
    os << "// symgb compiled module: " << descs.size() << " kernels, " << numLevels << " levels, " << S
       << " value sets, math " << (cfg.math == SYMGB_MATH_FAST ? "fast" : "exact") << ", schedule " << cfg.kind
       << "\n";
    os << (cfg.kind == JIT_PERSISTENT ? "#define SYMGB_XR\n" : "#define SYMGB_XR __restrict__\n");
    os << kJitPrelude << "\n";
    // Loads of the tables and of x: the read-only data path (ld.global.nc),
    // cached in L1 (ld.global.ca) or in L2 only (ld.global.cg); values written
    // earlier in the same launch (L2 = 1) always come from L2.
    static const char* const kLoad[] = {"__ldg", "__ldca", "__ldcg"};
    if (cfg.loadPath < 0 || cfg.loadPath > 2) throw std::runtime_error("codegen: load path must be 0, 1 or 2");
    os << "#define SYMGB_LD(a) " << kLoad[cfg.loadPath] << "(a)\n";
    os << "template <int L2>\n__device__ __forceinline__ double symgbLoadX(const double* a) {\n"
          "    return L2 ? __ldcg(a) : SYMGB_LD(a);\n}\n\n";
    if (grouped)
        os << "// Entries of IT consecutive instances of one padded table row (aligned).\n"
              "template <int IT>\n__device__ __forceinline__ void symgbLoadIdx(const unsigned* a, unsigned (&q)[IT]) {\n"
              "    if constexpr (IT == 4) {\n"
              "        const uint4 v = SYMGB_LD(reinterpret_cast<const uint4*>(a));\n"
              "        q[0] = v.x; q[1] = v.y; q[2] = v.z; q[3] = v.w;\n"
              "    } else if constexpr (IT == 2) {\n"
              "        const uint2 v = SYMGB_LD(reinterpret_cast<const uint2*>(a));\n"
              "        q[0] = v.x; q[1] = v.y;\n"
              "    } else {\n"
              "        q[0] = SYMGB_LD(a);\n"
              "    }\n}\n"
              "template <int IT>\n__device__ __forceinline__ void symgbLoadConst(const double* a, double (&v)[IT]) {\n"
              "    if constexpr (IT >= 2) {\n"
              "        #pragma unroll\n"
              "        for (int h = 0; h < IT; h += 2) {\n"
              "            const double2 u = SYMGB_LD(reinterpret_cast<const double2*>(a + h));\n"
              "            v[h] = u.x; v[h + 1] = u.y;\n"
              "        }\n"
              "    } else {\n"
              "        v[0] = SYMGB_LD(a);\n"
              "    }\n}\n\n";
    std::vector<std::size_t> opCount(descs.size());
    if (!cfg.directBase.empty() && (cfg.directBase.size() != descs.size() || S != 1))
        throw std::runtime_error("codegen: direct result rows need one value set and a row table per kernel");
    for (std::size_t k = 0; k < descs.size(); ++k) {
        const std::vector<std::int64_t>* direct = cfg.directBase.empty() ? nullptr : &cfg.directBase[k];
        if (direct)
            for (std::int64_t b : *direct) out.direct |= b >= 0;
        opCount[k] = emitBody(os, (int)k, descs[k], cfg.math, S, grouped ? &gt : nullptr, direct);
    }
    const char* params = "(const double* SYMGB_XR x, double* SYMGB_XR xw, const unsigned* __restrict__ p, "
                         "const double* __restrict__ c, double* __restrict__ res, const unsigned* __restrict__ dp";
    // Kernels of each level, heaviest first (their blocks are dispatched first).
    std::vector<std::vector<int>> byLevel(numLevels);
    for (std::size_t k = 0; k < descs.size(); ++k) {
        const int L = descs[k].level;
        if (L < 0 || L >= numLevels) throw std::runtime_error("codegen: kernel level out of range");
        if (descs[k].num_instances) byLevel[L].push_back((int)k);
    }
    if (cfg.kind == JIT_PLAIN) {
        for (std::size_t k = 0; k < descs.size(); ++k) {
            const std::uint64_t total = descs[k].num_instances * S;
            if (!total) continue;
            const int tpb = cfg.kernelTpb.at(k);
            const int items = checkedItems(cfg.kernelItems.at(k));
            const std::string name = "symgb_k" + std::to_string(k);
            os << "extern \"C\" __global__ void " << launchBounds(tpb, cfg.minBlocks) << " " << name << params << ") {\n"
               << "    symgbDependencyWait();\n    symgbLaunchDependents();\n";
            emitWork(os, (int)k, descs[k], opCount[k], S, tpb, items, 0, "(unsigned long long)blockIdx.x", "    ",
                     grouped);
            os << "}\n\n";
            out.launches.push_back({name, (int)k, -1, kernelBlocks(descs[k], S, tpb, items, grouped), tpb, items,
                                    false});
        }
    } else if (cfg.kind == JIT_LEVELS) {
        for (int L = 0; L < numLevels; ++L) {
            std::vector<int> ks = byLevel[L];
            if (ks.empty()) continue;
            std::stable_sort(ks.begin(), ks.end(), [&](int a, int b) {
                return descs[a].num_instances * (descs[a].num_nodes + 1) > descs[b].num_instances * (descs[b].num_nodes + 1);
            });
            const int tpb = cfg.levelTpb.at(L);
            const int items = checkedItems(cfg.levelItems.at(L));
            const std::string name = "symgb_l" + std::to_string(L);
            os << "extern \"C\" __global__ void " << launchBounds(tpb, cfg.minBlocks) << " " << name << params << ") {\n"
               << "    symgbDependencyWait();\n    symgbLaunchDependents();\n"
               << "    const unsigned long long b = blockIdx.x;\n";
            emitDispatch(os, ks, descs, opCount, S, tpb, items, 0, "    ", grouped);
            os << "}\n\n";
            out.launches.push_back({name, -1, L, blocksOf(ks, descs, S, tpb, items, grouped), tpb, items, false});
        }
    } else if (cfg.kind == JIT_PERSISTENT) {
        const int tpb = cfg.levelTpb.at(0);
        const int items = checkedItems(cfg.levelItems.at(0));
        os << "struct SymgbBarrier { unsigned count; unsigned generation; int error; int pad; };\n";
        os << "extern \"C\" __global__ void " << launchBounds(tpb, cfg.minBlocks) << " symgb_persistent" << params
           << ", SymgbBarrier* bar, int* hostError, unsigned long long timeoutNs, unsigned extra) {\n"
           << "    symgbDependencyWait();\n";
        std::uint64_t most = 1;
        bool firstLevel = true;
        for (int L = 0; L < numLevels; ++L) {
            const std::vector<int>& ks = byLevel[L];
            if (ks.empty()) continue;
            if (!firstLevel)
                os << "    if (!symgbGridBarrier(bar, hostError, timeoutNs, gridDim.x + extra)) return;\n";
            const std::uint64_t nb = blocksOf(ks, descs, S, tpb, items, grouped);
            most = std::max(most, nb);
            os << "    for (unsigned long long b = blockIdx.x; b < " << u64(nb) << "; b += gridDim.x) {\n";
            emitDispatch(os, ks, descs, opCount, S, tpb, items, firstLevel ? 0 : 1, "        ", grouped);
            os << "    }\n";
            firstLevel = false;
        }
        os << "}\n\n";
        out.launches.push_back({"symgb_persistent", -1, -1, most, tpb, items, true});
    } else {
        throw std::runtime_error("codegen: unknown schedule");
    }
    out.source = os.str();
    return out;
}

}  // namespace engine
}  // namespace symgb
