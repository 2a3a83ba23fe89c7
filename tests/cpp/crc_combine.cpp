// The parallel vector hash of the front end against the serial one: the same
// CRC-64 value for vectors of many lengths (the combination of chunk CRCs by
// zero-byte shifts is exact), and crc64(A || B) = crc64Shift(crc64(A), |B|) ^
// crc64(B) for split points across a buffer.
#include <cstdio>
#include <random>
#include <vector>

#include "symgb/hashing.hpp"

int main() {
    std::mt19937_64 rng(12345);
    int failures = 0;
    for (std::size_t n : {0ul, 1ul, 7ul, 16383ul, 16384ul, 16385ul, 28322ul, 100000ul, 123457ul}) {
        std::vector<symgb::hash_t> v(n);
        for (auto& x : v) x = (symgb::hash_t)rng();
        if (symgb::hashVectorParallel(v) != symgb::hashVector(v)) {
            std::printf("hashVectorParallel differs at n = %zu\n", n);
            ++failures;
        }
    }
    std::vector<unsigned char> buf(1000);
    for (auto& b : buf) b = (unsigned char)rng();
    for (std::size_t split : {0ul, 1ul, 8ul, 333ul, 999ul, 1000ul}) {
        const std::uint64_t a = (std::uint64_t)symgb::crc64(buf.data(), split);
        const std::uint64_t b = (std::uint64_t)symgb::crc64(buf.data() + split, buf.size() - split);
        const std::uint64_t whole = (std::uint64_t)symgb::crc64(buf.data(), buf.size());
        if ((symgb::crc64Shift(a, buf.size() - split) ^ b) != whole) {
            std::printf("crc64Shift combination differs at split %zu\n", split);
            ++failures;
        }
    }
    std::printf(failures ? "FAILED\n" : "ok\n");
    return failures ? 1 : 0;
}
