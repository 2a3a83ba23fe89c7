// Device programs: the form in which the engine's interpreter kernels execute
// a ComputeKernel template.
//
// A template (post-order nodes of a BLOCK of DEFINE / ASSIGN statements) is
// first compiled into a linear sequence of operations over virtual registers.
// In exact mode each template operation is one rounded operation in the
// template's order (n-ary sums and products left to right, as C evaluates the
// reference's generated code), so results are bit-identical to the reference
// compiled without FP contraction.  In fast mode, products feeding a sum are
// fused into FMA.
//
// The linear code is then list-scheduled into bundles: a bundle applies one
// operation to many independent operand tuples (no entry reads another
// entry's result), so the interpreter decodes one header per bundle and keeps
// several FP64 operations of one thread in flight.  Registers are assigned
// after scheduling; a register freed by a bundle is reused only by later
// bundles.  Scheduling only reorders operations whose inputs are ready, so
// every value is computed by the same operations on the same operands.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "symgb.h"

namespace symgb {
namespace engine {

// Load-section word: op (bits 0-7), dst (8-15), imm (32-63), see OP_LDX/OP_LDC/OP_LDK.
// Compute bundle: header word (op bits 0-7, entry count bits 8-23, accumulator
// flags bits 24-27), then the
// 32-bit entries, two per word (entry 2q in the low half of word q).  Entry
// fields: d bits 0-7, a 8-15, b 16-23, c 24-31; OP_ST entries hold the source
// register in bits 0-7 and the output row in bits 8-31; OP_LDK entries hold d
// and the index of the literal in the program's literal table in bits 8-31.
enum Opcode : std::uint8_t {
    OP_END = 0,
    OP_LDX = 1,   // r[dst] = x[p[row * n + i] + off]; row = bits 16-31, off = imm (signed)
    OP_LDC = 2,   // r[dst] = c[row * n + i]; row = imm
    OP_LDK = 3,   // r[d] = literal (load section: imm = its index in the literal table)
    OP_ST = 4,    // y[row * n + i] = r[a]
    OP_ADD = 5,
    OP_SUB = 6,   // r[a] - r[b]  (== r[a] + -(r[b]) exactly)
    OP_MUL = 7,
    OP_DIV = 8,
    OP_NEG = 9,
    OP_SQRT = 10,
    OP_REC = 11,  // 1 / r[a]
    OP_FMA = 12,  // r[d] = r[a] * r[b] + r[c], one rounding
    OP_SIN = 13,
    OP_COS = 14,
    OP_TAN = 15,
    OP_ASIN = 16,
    OP_ACOS = 17,
    OP_ATAN = 18,
    OP_EXP = 19,
    OP_LOG = 20,
    OP_POW = 21,
    OP_MOV = 22,
    OP_FMS = 23,   // r[a] * r[b] - r[c]
    OP_FNMA = 24,  // -(r[a] * r[b]) + r[c]
    OP_FNMS = 25,  // -(r[a] * r[b]) - r[c]
    OP_FDIV = 26,  // r[a] / r[b], fast mode: refined hardware reciprocal, within one ulp
    OP_FSQRT = 27, // sqrt(r[a]), fast mode
    OP_FREC = 28,  // 1 / r[a], fast mode
    NUM_OPCODES
};

constexpr int FMA_NEG_PRODUCT = 1;
constexpr int FMA_NEG_ADDEND = 2;
constexpr int MAX_REGISTERS = 255;

constexpr std::uint32_t ENTRY_FIELD_LIMIT = 1u << 24;  // OP_ST row / OP_LDK literal index

// Accumulator flags, header bits 24-27, set only on single-entry bundles.  The
// interpreter keeps the result of every single-entry bundle in a hardware
// register (the accumulator); a value whose only reader is the next bundle,
// itself a single entry, is passed there instead of through the shared-memory
// register file.  Values and their order are unchanged, only where they live.
constexpr std::uint32_t H_A_ACC = 1u << 24;     // operand a (ST: the stored value) is the accumulator
constexpr std::uint32_t H_B_ACC = 1u << 25;     // operand b is the accumulator
constexpr std::uint32_t H_C_ACC = 1u << 26;     // FMA addend is the accumulator
constexpr std::uint32_t H_NOSTORE = 1u << 27;   // the result stays in the accumulator only

struct ProgramStats {
    std::uint64_t flops = 0, divs = 0, sqrts = 0, transcendentals = 0, gathers = 0, constLoads = 0, stores = 0;
};

// A program has two sections.  `loads` holds every distinct gather (LDX) and
// per-instance constant read (LDC) of the template, and its most used
// distinct literals (LDK, up to LITERAL_LOADS), each loaded once into its own
// register before any arithmetic, so the interpreter can issue them all back
// to back (a literal so loaded takes one register and no compute entry,
// instead of one literal-load entry and one register per use site).  `words` holds the compute bundles (arithmetic, literal loads
// and output stores), an OP_END word, then the literal table (one double per
// word) starting at word `literalOffset`.
struct Program {
    std::vector<std::uint64_t> loads;
    std::vector<std::uint64_t> words;
    std::uint32_t literalOffset = 0;
    int registers = 0;
    int bundles = 0;      // compute bundles
    int operations = 0;   // compute entries over all bundles
    ProgramStats stats;
};

// Operations a bundle may gather from: the next `window` not yet scheduled
// operations of the linear code (larger windows give larger bundles and more
// live registers; a template that would need more than MAX_REGISTERS is
// scheduled again with half the window).  64 against 128 on the GB300: the
// multi-pattern cloth batch 3.70 -> 3.38 ms and Neo-Hookean 15^3 x 4 sets
// 252 -> 230 us faster with 64 (fewer registers, more resident items);
// Neo-Hookean 10^3 x 1 set 70 -> 58 us faster with 128.
constexpr int BUNDLE_WINDOW = 64;

// Distinct literals loaded in the load section.  ComputeKernel templates use
// few distinct literals (6-8 in the cloth and Neo-Hookean Hessians) at many
// sites (185 literal loads in the largest cloth kernel).
constexpr int LITERAL_LOADS = 32;

// Compiles one kernel template.  Throws std::runtime_error on templates the
// engine cannot execute (unknown operations, more than MAX_REGISTERS live
// values).  Loads are deduplicated: a gather that the template reads several
// times is loaded once; the value is the same, so results do not change.
Program compileTemplate(const symgb_kernel_desc& k, int math, int window = BUNDLE_WINDOW,
                        int literalLoads = LITERAL_LOADS);

// One operation of a template's linear code (before bundling): the form the
// code generator of the compiled executor reads.  Registers are the linear
// code's (reused once a value is dead); `d` is -1 for stores.  FMA variants
// carry their sign in the opcode (OP_FMA / OP_FMS / OP_FNMA / OP_FNMS).
struct LinOp {
    int op = OP_END;
    int d = -1;             // register written, -1 if none
    int src[3] = {-1, -1, -1};
    int nsrc = 0;
    std::uint32_t row = 0;  // OP_ST: output row
    std::uint64_t lit = 0;  // OP_LDK: the literal's bits
};

// The linear code of a template and, in `loads`, its load section (OP_LDX /
// OP_LDC words as in Program::loads).  Same operations, operands and rounding
// as the device program compileTemplate bundles from it.
std::vector<LinOp> linearCode(const symgb_kernel_desc& k, int math, std::vector<std::uint64_t>* loads);

// Human-readable listing (tests and debugging).
std::string disassemble(const Program& p);

inline std::uint64_t encode(int op, int dst, int a, int b, std::uint32_t imm) {
    return (std::uint64_t)(op & 0xff) | ((std::uint64_t)(dst & 0xff) << 8) | ((std::uint64_t)(a & 0xff) << 16) |
           ((std::uint64_t)(b & 0xff) << 24) | ((std::uint64_t)imm << 32);
}

}  // namespace engine
}  // namespace symgb
