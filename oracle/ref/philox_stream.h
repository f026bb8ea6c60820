// Counter-based Philox4x32-10 (Salmon, Moraes, Dror & Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC'11), restated for the oracle build of the
// reference.  The draw mapping below is the project's RNG contract; the CUDA
// engine and the oracle port implement the same contract independently.
//
//   key     = (seed, replica)
//   counter = (block_lo, block_hi, stream, 0), block = draw >> 1
//   draw n  = 64-bit word (w[2*(n&1)] << 32) | w[2*(n&1)+1] of block n >> 1
//   uniform_real()      = (x >> 11) * 2^-53                in [0, 1)
//   uniform_int(lo, hi) = lo + floor(x * (hi - lo + 1) / 2^64)
#pragma once
#include <cstdint>

namespace ldo_ref {

inline void philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

struct Stream {
    uint32_t key[2] {0, 0};
    uint32_t stream {0};
    uint64_t draws {0};

    uint64_t next64() {
        uint64_t block = draws >> 1;
        uint32_t ctr[4] = {(uint32_t)block, (uint32_t)(block >> 32), stream, 0u};
        uint32_t w[4];
        philox4x32_10(ctr, key, w);
        int j = (int)(draws & 1) * 2;
        ++draws;
        return ((uint64_t)w[j] << 32) | w[j + 1];
    }
    double uniform_real() { return (double)(next64() >> 11) * 0x1.0p-53; }
    int uniform_int(int lo, int hi) {
        uint64_t range = (uint64_t)((int64_t)hi - (int64_t)lo) + 1u;
        unsigned __int128 prod = (unsigned __int128)next64() * range;
        return lo + (int)(uint64_t)(prod >> 64);
    }
};

} // namespace ldo_ref
