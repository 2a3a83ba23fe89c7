// Device programs: the form in which the engine's interpreter kernels execute
// a ComputeKernel template.
//
// A template (post-order nodes of a BLOCK of DEFINE / ASSIGN statements) is
// compiled into a linear sequence of 64-bit instructions over a per-thread
// register file.  Every thread runs the same program for its own instance and
// value set, so instruction fetch and decode are warp-uniform.  In exact mode
// each template operation is one rounded operation in the template's order
// (n-ary sums and products left to right, as C evaluates the reference's
// generated code), so results are bit-identical to the reference compiled
// without FP contraction.  In fast mode, products feeding a sum are fused into
// FMA.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "symgb.h"

namespace symgb {
namespace engine {

// Instruction word: op (bits 0-7), dst (8-15), a (16-23), b (24-31), imm (32-63).
enum Opcode : std::uint8_t {
    OP_END = 0,
    OP_LDX = 1,   // r[dst] = x[p[row * n + i] + off]; row = bits 16-31, off = imm (signed)
    OP_LDC = 2,   // r[dst] = c[row * n + i]; row = imm
    OP_LDK = 3,   // r[dst] = next word as double
    OP_ST = 4,    // y[row * n + i] = r[a]; row = imm
    OP_ADD = 5,
    OP_SUB = 6,   // r[a] - r[b]  (== r[a] + -(r[b]) exactly)
    OP_MUL = 7,
    OP_DIV = 8,
    OP_NEG = 9,
    OP_SQRT = 10,
    OP_REC = 11,  // 1 / r[a]
    OP_FMA = 12,  // r[dst] = (+-)(r[a] * r[b]) (+-) r[c]; c = bits 32-39, flags bits 40-41
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
    NUM_OPCODES
};

constexpr int FMA_NEG_PRODUCT = 1;
constexpr int FMA_NEG_ADDEND = 2;
constexpr int MAX_REGISTERS = 255;

// Accumulator flags, bits 56-63 of a compute word.  The interpreter keeps the
// result of every instruction in a hardware register (the accumulator); a
// value consumed only by the very next instruction is passed there instead of
// through the shared-memory register file.
constexpr std::uint64_t F_A_ACC = 1ull << 56;    // operand a is the accumulator
constexpr std::uint64_t F_B_ACC = 2ull << 56;    // operand b is the accumulator
constexpr std::uint64_t F_C_ACC = 4ull << 56;    // FMA addend is the accumulator
constexpr std::uint64_t F_NOSTORE = 8ull << 56;  // result only in the accumulator
constexpr std::uint32_t ST_ROW_LIMIT = 1u << 24; // OP_ST row field: bits 32-55

struct ProgramStats {
    std::uint64_t flops = 0, divs = 0, sqrts = 0, transcendentals = 0, gathers = 0, constLoads = 0, stores = 0;
};

// A program has two sections.  `loads` holds every distinct gather (LDX) and
// per-instance constant read (LDC) of the template, each loaded once into its
// own register before any arithmetic, so the interpreter can issue them all
// back to back.  `words` holds the arithmetic, literal loads (LDK) and output
// stores, ending with OP_END.
struct Program {
    std::vector<std::uint64_t> loads;
    std::vector<std::uint64_t> words;
    int registers = 0;
    ProgramStats stats;
};

// Compiles one kernel template.  Throws std::runtime_error on templates the
// engine cannot execute (unknown operations, more than MAX_REGISTERS live
// values).  Loads are deduplicated: a gather that the template reads several
// times is loaded once; the value is the same, so results do not change.
Program compileTemplate(const symgb_kernel_desc& k, int math);

// Human-readable listing (tests and debugging).
std::string disassemble(const Program& p);

inline std::uint64_t encode(int op, int dst, int a, int b, std::uint32_t imm) {
    return (std::uint64_t)(op & 0xff) | ((std::uint64_t)(dst & 0xff) << 8) | ((std::uint64_t)(a & 0xff) << 16) |
           ((std::uint64_t)(b & 0xff) << 24) | ((std::uint64_t)imm << 32);
}

}  // namespace engine
}  // namespace symgb
