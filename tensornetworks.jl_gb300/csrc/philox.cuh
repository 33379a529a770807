// Philox4x32-10 (Salmon, Moraes, Dror & Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC 2011), on the host and the device: ten rounds of two
// 32x32->64 multiplications with the published multipliers and Weyl key
// increments.
#pragma once

#include <stdint.h>

namespace tn {

__host__ __device__ inline void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// Draw k of trajectory `traj` under `seed`, in [0, 1): the 64-bit word
// (k % 2) of Philox4x32-10(counter = (k / 2 low, traj, k / 2 high, 0), key =
// (seed low, seed high)), its top 53 bits.
__host__ __device__ inline double philox_uniform(uint64_t seed, uint32_t traj, uint64_t k) {
    const uint64_t h = k >> 1;
    uint32_t c[4] = {(uint32_t)h, traj, (uint32_t)(h >> 32), 0u};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    const uint64_t w = (k & 1) ? (((uint64_t)c[3] << 32) | c[2]) : (((uint64_t)c[1] << 32) | c[0]);
    return (double)(w >> 11) * (1.0 / 9007199254740992.0);
}

}  // namespace tn
