// Byte hashing used by the symbolic front end.
//
// The hash is a table-driven, reflected CRC-64 with the Jones polynomial, zero
// initial value and no final xor - the function the reference applies to raw
// bytes (src/Hashing.cpp:142-152).  The table is generated from the polynomial
// at start-up.  Variable pairs are hashed as in src/Hashing.cpp:154-162, whose
// table index x % 255 + 1 is negative for negative variable groups; those
// reads yield 0 here, matching the oracle build of the reference, which places
// zeros in front of its table.
#pragma once
#include <array>
#include <cstdint>
#include <cstring>
#include <vector>

#include "ops.hpp"

namespace symgb {

const std::uint64_t* crc64Table();

inline hash_t crc64(const void* bytes, std::size_t len) {
    const std::uint64_t* tab = crc64Table();
    const unsigned char* s = static_cast<const unsigned char*>(bytes);
    std::uint64_t crc = 0;
    for (std::size_t j = 0; j < len; ++j) crc = tab[(std::uint8_t)crc ^ s[j]] ^ (crc >> 8);
    return (hash_t)crc;
}

// Hash of the concatenated object representations of two values.
template <class T1, class T2>
inline hash_t hashPair(const T1& a, const T2& b) {
    unsigned char buf[sizeof(T1) + sizeof(T2)];
    std::memcpy(buf, &a, sizeof(T1));
    std::memcpy(buf + sizeof(T1), &b, sizeof(T2));
    return crc64(buf, sizeof(buf));
}

template <class T>
inline hash_t hashVector(const std::vector<T>& v) {
    return crc64(v.data(), sizeof(T) * v.size());
}

// The CRC above starts from 0 and has no final XOR, so it is linear over
// GF(2): crc64(A || B) = crc64Shift(crc64(A), |B|) ^ crc64(B), where
// crc64Shift(c, n) is the state reached from c by n zero bytes.
std::uint64_t crc64Shift(std::uint64_t crc, std::uint64_t zeroBytes);

// hashVector of a vector of hashes, with chunks of a long vector hashed in
// parallel and combined in order; the same value as hashVector.
hash_t hashVectorParallel(const std::vector<hash_t>& v);

template <class T>
inline hash_t hashValue(const T& v) {
    return crc64(&v, sizeof(T));
}

// Table entry used for one component of a variable pair.
inline std::uint64_t varTableEntry(int x) {
    const int idx = x % 255 + 1;  // C++ remainder: negative for negative x
    return idx >= 0 ? crc64Table()[idx] : 0;
}

inline hash_t hashVariable(const std::array<int, 2>& x) {
    hash_t data[2];
    data[0] = (hash_t)(varTableEntry(x[0]) + (std::uint64_t)(std::int64_t)x[0]);
    data[1] = (hash_t)(varTableEntry(x[1]) + (std::uint64_t)(std::int64_t)x[1]);
    return crc64(data, sizeof(data));
}

inline bool isSmallConstant(hash_t h) {
    if (h < 0) h = -h;
    return (h >> 4) == 0;
}

}  // namespace symgb
