"""CPU model of the device interpreter (TEST INFRASTRUCTURE ONLY).

Runs the programs the engine compiles for its ComputeKernels (read back with
symgb_kernel_program) with numpy, one vector element per instance, following
the interpreter's semantics (evalTile in symboliclib_gb300/csrc/engine/
device.cuh):

* load section: LDX r = x[p[row * n + i] + off] (u32 slot arithmetic),
  LDC r = c[off * n + i], LDK r = literal table[off];
* compute bundles: one header word (opcode bits 0-7, entry count 8-23, flags
  24-27), then 32-bit entries `d | a << 8 | b << 16 | c << 24`, two per word;
  no entry of a bundle reads another entry's result; LDK entries hold the
  literal index in bits 8-31, ST entries the output row; a single-entry
  bundle may take operands from, and leave its result only in, the
  accumulator (the result of the previous single-entry bundle);
* stores: x[yoff + row * n + i] = r[src];
* an END word, then the literal table.

Exact-mode programs round every operation separately, which numpy does too,
so the model reproduces the device bit for bit.  FMA is evaluated exactly
(rational arithmetic, one rounding); the fast division and reciprocal are
modelled as the IEEE operations (the device's agree bit for bit on every
operand measured) and the fast square root as the IEEE one (the device's is
within one unit in the last place)."""
from __future__ import annotations

import ctypes as C
import math
from fractions import Fraction

import numpy as np

OP_END, OP_LDX, OP_LDC, OP_LDK, OP_ST = 0, 1, 2, 3, 4
OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_NEG, OP_SQRT, OP_REC, OP_FMA = 5, 6, 7, 8, 9, 10, 11, 12
OP_SIN, OP_COS, OP_TAN, OP_ASIN, OP_ACOS, OP_ATAN, OP_EXP, OP_LOG, OP_POW = 13, 14, 15, 16, 17, 18, 19, 20, 21
OP_MOV, OP_FMS, OP_FNMA, OP_FNMS, OP_FDIV, OP_FSQRT, OP_FREC = 22, 23, 24, 25, 26, 27, 28
H_A_ACC, H_B_ACC, H_C_ACC, H_NOSTORE = 1 << 24, 1 << 25, 1 << 26, 1 << 27

BINARY = {OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_FDIV, OP_POW}
FMAS = {OP_FMA: (False, False), OP_FMS: (False, True), OP_FNMA: (True, False), OP_FNMS: (True, True)}


def _fma_scalar(x: float, y: float, z: float) -> float:
    if not (math.isfinite(x) and math.isfinite(y) and math.isfinite(z)):
        return x * y + z
    return float(Fraction(x) * Fraction(y) + Fraction(z))


_fma_vec = np.frompyfunc(_fma_scalar, 3, 1)


def fma(x, y, z) -> np.ndarray:
    """x * y + z with one rounding (round to nearest even)."""
    x, y, z = np.broadcast_arrays(x, y, z)
    return _fma_vec(x, y, z).astype(np.float64)


def _apply(op: int, a, b, c):
    with np.errstate(all="ignore"):
        if op == OP_ADD:
            return a + b
        if op == OP_SUB:
            return a - b
        if op == OP_MUL:
            return a * b
        if op in (OP_DIV, OP_FDIV):
            return a / b
        if op == OP_NEG:
            return -a
        if op == OP_MOV:
            return a.copy()
        if op in (OP_SQRT, OP_FSQRT):
            return np.sqrt(a)
        if op in (OP_REC, OP_FREC):
            return 1.0 / a
        if op in FMAS:
            neg_p, neg_c = FMAS[op]
            return fma(-a if neg_p else a, b, -c if neg_c else c)
        lib = {OP_SIN: np.sin, OP_COS: np.cos, OP_TAN: np.tan, OP_ASIN: np.arcsin, OP_ACOS: np.arccos,
               OP_ATAN: np.arctan, OP_EXP: np.exp, OP_LOG: np.log}
        if op in lib:
            return lib[op](a)
        if op == OP_POW:
            return np.power(a, b)
    raise ValueError(f"unknown opcode {op}")


def nsrc(op: int) -> int:
    return 3 if op in FMAS else 2 if op in BINARY else 1


def kernel_program(lib, unit_handle, k: int, math_mode: int):
    """(words, registers, number of load words) of kernel k's device program."""
    regs, nl = C.c_int(), C.c_int()
    n = lib.symgb_kernel_program(unit_handle, k, math_mode, None, 0, C.byref(regs), C.byref(nl))
    if n < 0:
        raise RuntimeError(f"symgb_kernel_program failed: {n}")
    buf = (C.c_uint64 * n)()
    lib.symgb_kernel_program(unit_handle, k, math_mode, buf, n, C.byref(regs), C.byref(nl))
    return np.frombuffer(buf, np.uint64).copy(), regs.value, nl.value


def run_kernel(words: np.ndarray, nl: int, x: np.ndarray, p: np.ndarray, c: np.ndarray, n: int, yoff: int) -> dict:
    """Runs one kernel's program over its n instances, writing its outputs into
    x; returns statistics (bundles, entries) of what it ran."""
    w = [int(v) for v in words]
    i = np.arange(n, dtype=np.int64)
    # the literal table follows the END word
    pc = nl
    while w[pc] & 0xff != OP_END:
        cnt = (w[pc] >> 8) & 0xffff
        pc += 1 + (cnt + 1) // 2
    lit = np.array(w[pc + 1:], dtype=np.uint64).view(np.float64)
    R: dict[int, np.ndarray] = {}
    for q in range(nl):
        op, d, imm = w[q] & 0xff, (w[q] >> 8) & 0xff, (w[q] >> 32) & 0xffffffff
        if op == OP_LDX:
            row = (w[q] >> 16) & 0xffff
            slot = (p[row * n + i].astype(np.uint64) + np.uint64(imm)) & np.uint64(0xffffffff)
            R[d] = x[slot.astype(np.int64)].copy()
        elif op == OP_LDC:
            R[d] = c[imm * n + i].copy()
        elif op == OP_LDK:
            R[d] = np.full(n, lit[imm])
        else:
            raise ValueError(f"opcode {op} in the load section")

    acc = np.zeros(n)
    pc, bundles, entries = nl, 0, 0
    while True:
        h = w[pc]
        op, cnt, flags = h & 0xff, (h >> 8) & 0xffff, h & 0xff000000
        if op == OP_END:
            break
        ents = [(w[pc + 1 + q // 2] >> (32 * (q & 1))) & 0xffffffff for q in range(cnt)]
        pc += 1 + (cnt + 1) // 2
        bundles += 1
        entries += cnt
        if cnt != 1 and flags:
            raise ValueError("accumulator flags on a bundle of several entries")
        if op == OP_ST:
            for e in ents:
                v = acc if flags & H_A_ACC else R[e & 0xff]
                row = e >> 8
                x[yoff + row * n + i] = v
            continue
        results = []
        for e in ents:
            d = e & 0xff
            if op == OP_LDK:
                v = np.full(n, lit[e >> 8])
            else:
                ins = []
                for s in range(nsrc(op)):
                    ins.append(acc if flags & (H_A_ACC << s) else R[(e >> (8 * (s + 1))) & 0xff])
                while len(ins) < 3:
                    ins.append(ins[0])
                v = _apply(op, *ins)
            results.append((d, v))
        if cnt == 1:
            acc = results[0][1]
            if flags & H_NOSTORE:
                continue
        for d, v in results:
            R[d] = v
    return {"bundles": bundles, "entries": entries}


def evaluate(lib, unit_handle, plan, index_data, out_index_data, const_data, inputs, math_mode: int):
    """execute() + getResults() of one value set, with every kernel's device
    program run by the model in kernel order."""
    d = plan.contents
    x = np.zeros(max(1, d.num_total_memory), np.float64)
    for a, v in enumerate(inputs):
        s = int(d.arg_start[a])
        x[s:s + int(d.arg_length[a])] = v
    idx = np.ascontiguousarray(index_data, np.uint32)
    cst = np.ascontiguousarray(const_data, np.float64)
    for k in range(d.num_kernels):
        kd = d.kernels[k]
        n = int(kd.num_instances)
        words, _, nl = kernel_program(lib, unit_handle, k, math_mode)
        p = idx[int(kd.index_offset):int(kd.index_offset) + int(kd.num_index_rows) * n]
        c = cst[int(kd.constants_offset):int(kd.constants_offset) + int(kd.num_constant_rows) * n]
        run_kernel(words, nl, x, p, c, n, int(kd.output_offset))
    ids = np.ascontiguousarray(out_index_data, np.uint32)
    outs = []
    for k in range(d.num_outputs):
        s, n = int(d.output_start[k]), int(d.output_length[k])
        outs.append(x[ids[s:s + n].astype(np.int64)])
    return outs
