// Operation codes and per-operation properties of the symbolic IR.
//
// The numbering, the 64-bit per-operation hash seeds and the costs are the ones
// of the reference IR (src/Operations.hpp:9-38 and the OpInfos table at
// src/Operations.hpp:54-85).  They feed the structure and algebraic hashes that
// decide how expressions are grouped into kernels, so they must be identical
// for the engine's kernel lists to equal the reference's.
#pragma once
#include <cstdint>

namespace symgb {

using OpType = std::uint8_t;
using hash_t = long long;

enum : OpType {
    NOOP = 0, CONST = 1, VAR = 2, ADD = 3, MUL = 4, MULC = 5, DIV = 6, SQRT = 7,
    SIN = 8, COS = 9, TAN = 10, COT = 11, ASIN = 12, ACOS = 13, ATAN = 14,
    EXP = 15, LOG = 16, POW = 17, ASSIGN = 18, GROUP = 19, CONDPOS = 20,
    CONDNONZERO = 21, CONDZERO = 22, NEG = 23, DEFINE = 24, BLOCK = 25,
    RECIPROCAL = 26, FIXED = 27, FUNCTIONHANDLE = 28, CALL = 29,
    NUM_OPS = 30
};

// Reserved variable groups (reference src/Symbolic.hpp:14-16).
constexpr int GLOBAL_INTERMEDIATE = 254;
constexpr int EXPLICIT_INTERMEDIATE = 252;
constexpr int LOCAL_VAR = 253;

// Variable groups used inside kernel templates (reference ComputeKernel.cpp:189-221).
constexpr int TEMPLATE_OUTPUT = -2;    // y[slot]
constexpr int TEMPLATE_INDEX = -3;     // x[p[row] + offset]
constexpr int TEMPLATE_CONSTANT = -4;  // c[row]

struct OpInfo {
    std::uint8_t operands;  // 0 leaf, 1..3, or 255 (n-ary)
    bool infix;
    bool commutative;
    bool leaf;
    const char* symbol;
    hash_t seed;
    std::uint8_t cost;
};

inline const OpInfo& opInfo(OpType op) {
    static const OpInfo table[NUM_OPS] = {
        {255, false, false, false, "", (hash_t)0xcc9259a104c6ea35ULL, 0},            // NOOP
        {0, false, false, true, "", (hash_t)0x720980970d2b9f05ULL, 0},               // CONST
        {0, false, false, true, "", (hash_t)0x6f916152447e9041ULL, 1},               // VAR
        {255, true, true, false, "+", (hash_t)0xd457fa26b0562106ULL, 1},             // ADD
        {255, true, true, false, "*", (hash_t)0xb3beedbf7c3186ccULL, 1},             // MUL
        {2, true, false, false, "*", (hash_t)0x26530d4374e5c7c7ULL, 0},              // MULC
        {2, true, false, false, "/", (hash_t)0x52d63751b598c8bfULL, 1},              // DIV
        {1, false, false, false, "sqrt", (hash_t)0x280e56b8cfae0b37ULL, 5},          // SQRT
        {1, false, false, false, "sin", (hash_t)0x9c2ae07a9b27fff6ULL, 1},           // SIN
        {1, false, false, false, "cos", (hash_t)0x676e6b1a2c59ee19ULL, 1},           // COS
        {1, false, false, false, "tan", (hash_t)0x84b3c10ba829371dULL, 1},           // TAN
        {1, false, false, false, "cot", (hash_t)0x7dced0e9233a0853ULL, 1},           // COT
        {1, false, false, false, "asin", (hash_t)0x5ca0b0b777eb6ac5ULL, 1},          // ASIN
        {1, false, false, false, "acos", (hash_t)0xd994629b6eeb5b85ULL, 1},          // ACOS
        {1, false, false, false, "atan", (hash_t)0x07c437f90eccf490ULL, 1},          // ATAN
        {1, false, false, false, "exp", (hash_t)0x856822d27ac0754dULL, 1},           // EXP
        {1, false, false, false, "log", (hash_t)0x962e1816878fff6dULL, 1},           // LOG
        {2, false, false, false, "pow", (hash_t)0xe7db1b947e581812ULL, 1},           // POW
        {2, true, false, false, "=", (hash_t)0x6f2c602bf486949aULL, 1},              // ASSIGN
        {255, true, false, false, ";", (hash_t)0x3046da41a8716cbfULL, 1},            // GROUP
        {3, false, false, false, "selectpos", (hash_t)0xc17d952f1162e824ULL, 1},     // CONDPOS
        {3, false, false, false, "selectnonzero", (hash_t)0x5534ce8f1320b090ULL, 1}, // CONDNONZERO
        {3, false, false, false, "selectzero", (hash_t)0x78e0b29e0546e0eeULL, 1},    // CONDZERO
        {1, false, false, false, "-", (hash_t)0x18e0b23b05a6e0e3ULL, 0},             // NEG
        {2, false, false, false, "def", (hash_t)0x6f2c602bf486949aULL, 1},           // DEFINE
        {255, true, false, false, ";", (hash_t)0x1e66b3b5e487934cULL, 0},            // BLOCK
        {1, false, false, false, "1./", (hash_t)0xf512ee2a5d3a5323ULL, 1},           // RECIPROCAL
        {2, false, false, false, "FIXED", (hash_t)0x1fde2a735a3b5301ULL, 0},         // FIXED
        {0, false, false, false, "FUNC", (hash_t)0x6fe2fe2d5d20d4a1ULL, 0},          // FUNCTIONHANDLE
        {255, false, false, false, "CALL", (hash_t)0x1ef0462c532553afULL, 1},        // CALL
    };
    return table[op < NUM_OPS ? op : NOOP];
}

// Hash seeds used for leaves in structure hashes (reference src/Symbolic.hpp:10-12).
constexpr hash_t VarHash = (hash_t)0x6f916152447e9041ULL;
constexpr hash_t ConstHash = (hash_t)0x720980970d2b9f05ULL;
constexpr hash_t NOOPHash = (hash_t)0x2f2a32bb2a0f2e0dULL;

}  // namespace symgb
