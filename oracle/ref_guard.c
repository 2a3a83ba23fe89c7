/* Zero bytes placed directly in front of the reference's CRC table in
 * oracle/_ref/libsymref.so.  The reference's hash of a variable id pair
 * (Hashing.cpp:154-162) indexes the table with x % 255 + 1, which is negative
 * for negative variable groups (-2, -3, -4 in kernel templates, -10-k for
 * outputs).  Those reads land in front of the table; this guard makes them read
 * 0 in the oracle build, so the reference's hash-ordered simplification has a
 * fixed, reproducible operand order.  The engine's front end uses the same 0. */
__attribute__((section(".rodata.symref_guard"), aligned(64), used))
const unsigned char symref_zero_guard[4096] = {0};
