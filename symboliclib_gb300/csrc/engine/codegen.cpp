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

// Emits the device function evaluating kernel k for one work item
// (instance i, value set s).  L2 = 1 reads x through L2 only (values written
// earlier in the same launch, persistent schedule).  Returns the number of
// operations of the template.
std::size_t emitBody(std::ostringstream& os, int k, const symgb_kernel_desc& d, int math, unsigned S) {
    std::vector<std::uint64_t> loads;
    const std::vector<LinOp> ops = linearCode(d, math, &loads);
    const std::uint64_t n = d.num_instances;
    os << "// kernel " << k << ": " << n << " instances, level " << d.level << ", " << loads.size() << " loads, "
       << ops.size() << " operations\n";
    os << "template <int L2>\n__device__ __forceinline__ void symgbBody" << k
       << "(const double* SYMGB_XR x, double* SYMGB_XR xw, const unsigned* __restrict__ p, "
          "const double* __restrict__ c, unsigned long long i, unsigned s) {\n";
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
    // variables share a row and differ by their offsets).
    std::vector<int> rowVar(d.num_index_rows, -1);
    int rows = 0;
    for (std::uint64_t w : loads) {
        if ((int)(w & 0xff) != OP_LDX) continue;
        const std::uint64_t row = (w >> 16) & 0xffff;
        if (row >= d.num_index_rows) throw std::runtime_error("codegen: index row out of range");
        if (rowVar[row] >= 0) continue;
        rowVar[row] = rows++;
        os << "    const unsigned q" << rowVar[row] << " = SYMGB_LD(p + " << u64(d.index_offset + row * n) << " + i);\n";
    }
    for (std::uint64_t w : loads) {
        const int op = (int)(w & 0xff), dst = (int)((w >> 8) & 0xff);
        const std::uint32_t imm = (std::uint32_t)(w >> 32);
        if (op == OP_LDX) {
            const std::uint64_t row = (w >> 16) & 0xffff;
            const std::string v = fresh(dst);
            os << "    const double " << v << " = symgbLoadX<L2>(x + (unsigned long long)(q" << rowVar[row] << " + "
               << imm << "u)" << xs << ");\n";
        } else if (op == OP_LDC) {
            const std::string v = fresh(dst);
            os << "    const double " << v << " = SYMGB_LD(c + " << u64(d.constants_offset + (std::uint64_t)imm * n)
               << " + i);\n";
        } else {
            throw std::runtime_error("codegen: unknown load word");
        }
    }
    for (const LinOp& L : ops) {
        std::string rhs;
        switch (L.op) {
            case OP_ST:
                os << "    xw[(" << u64(d.output_offset + (std::uint64_t)L.row * n) << " + i)" << xs
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
        os << "    const double " << v << " = " << rhs << ";\n";
    }
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
           << indent << "        symgbBody" << k << "<" << l2 << ">(x, xw, p, c, w / " << S << "ull, (unsigned)(w % "
           << S << "ull));\n"
           << indent << "    }\n" << indent << "} else {\n";
    }
    if (items > 1) os << indent << "#pragma unroll\n" << indent << "for (int j = 0; j < " << items << "; ++j) {\n";
    else os << indent << "{\n" << indent << "    const int j = 0;\n";
    os << indent << "    const unsigned long long w = w0 + (unsigned long long)j * " << tpb << "ull;\n"
       << indent << "    if (w < " << u64(total) << ") symgbBody" << k << "<" << l2 << ">(x, xw, p, c, w / " << S
       << "ull, (unsigned)(w % " << S << "ull));\n"
       << indent << "}\n";
    if (items > 1 && split) os << indent << "}\n";
}

std::uint64_t blocksFor(std::uint64_t total, int tpb, int items) {
    const std::uint64_t per = (std::uint64_t)tpb * items;
    return (total + per - 1) / per;
}

// Dispatch of block `b` over the kernels of one launch (kernel-major block
// ranges, each kernel's work items in consecutive blocks).
void emitDispatch(std::ostringstream& os, const std::vector<int>& ks, const std::vector<symgb_kernel_desc>& descs,
                  const std::vector<std::size_t>& opCount, unsigned S, int tpb, int items, int l2, const char* indent) {
    std::uint64_t first = 0;
    const std::string inner = std::string(indent) + "    ";
    for (std::size_t q = 0; q < ks.size(); ++q) {
        const int k = ks[q];
        const std::uint64_t total = descs[k].num_instances * S;
        const std::uint64_t blocks = blocksFor(total, tpb, items);
        os << indent << (q ? "else " : "") << "if (b < " << u64(first + blocks) << ") {\n";
        emitItems(os, k, total, S, tpb, items, l2, "b - " + u64(first), inner.c_str(),
                  opCount[k] * (std::size_t)items <= kSplitOps);
        os << indent << "}\n";
        first += blocks;
    }
}

std::uint64_t blocksOf(const std::vector<int>& ks, const std::vector<symgb_kernel_desc>& descs, unsigned S, int tpb,
                       int items) {
    std::uint64_t b = 0;
    for (int k : ks) b += blocksFor(descs[k].num_instances * S, tpb, items);
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

JitSource generateModule(const std::vector<symgb_kernel_desc>& descs, int numLevels, const JitConfig& cfg) {
    JitSource out;
    std::ostringstream os;
    const unsigned S = cfg.numSets;
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
    std::vector<std::size_t> opCount(descs.size());
    for (std::size_t k = 0; k < descs.size(); ++k) opCount[k] = emitBody(os, (int)k, descs[k], cfg.math, S);
    const char* params = "(const double* SYMGB_XR x, double* SYMGB_XR xw, const unsigned* __restrict__ p, "
                         "const double* __restrict__ c";
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
            emitItems(os, (int)k, total, S, tpb, items, 0, "(unsigned long long)blockIdx.x", "    ",
                      opCount[k] * (std::size_t)items <= kSplitOps);
            os << "}\n\n";
            out.launches.push_back({name, (int)k, -1, blocksFor(total, tpb, items), tpb, items, false});
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
            emitDispatch(os, ks, descs, opCount, S, tpb, items, 0, "    ");
            os << "}\n\n";
            out.launches.push_back({name, -1, L, blocksOf(ks, descs, S, tpb, items), tpb, items, false});
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
            const std::uint64_t nb = blocksOf(ks, descs, S, tpb, items);
            most = std::max(most, nb);
            os << "    for (unsigned long long b = blockIdx.x; b < " << u64(nb) << "; b += gridDim.x) {\n";
            emitDispatch(os, ks, descs, opCount, S, tpb, items, firstLevel ? 0 : 1, "        ");
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
