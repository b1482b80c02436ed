// qew_philox.cuh -- Philox4x32-10 counter-based generator (J. Salmon,
// M. Moraes, R. Dror, D. Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC'11) and a Box-Muller (1958) normal pair. Increment i of step s comes from
// the block of counter (i/2, 0, s_lo, s_hi) under key (seed_lo, seed_hi):
// two 53-bit uniforms u1 in (0,1], u2 in [0,1), r = sqrt(-2 ln u1),
// xi_{2j} = r cos(2 pi u2), xi_{2j+1} = r sin(2 pi u2).
#pragma once

#include <stdint.h>

__host__ __device__ __forceinline__ void philox_round(uint32_t c[4], uint32_t k0, uint32_t k1) {
#ifdef __CUDA_ARCH__
    const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]);
    const uint32_t lo0 = 0xD2511F53u * c[0];
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]);
    const uint32_t lo1 = 0xCD9E8D57u * c[2];
#else
    const uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
    const uint32_t n0 = hi1 ^ c[1] ^ k0;
    const uint32_t n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
}

__host__ __device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint64_t seed) {
    uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        philox_round(c, k0, k1);
    }
}

// The two N(0,1) increments of sites 2j and 2j+1 at step `step`.
__device__ __forceinline__ void philox_normal_pair(uint64_t seed, uint64_t step, uint32_t j,
                                                   double &z0, double &z1) {
    uint32_t c[4] = {j, 0u, (uint32_t)step, (uint32_t)(step >> 32)};
    philox4x32_10(c, seed);
    const uint64_t a = ((((uint64_t)c[0]) << 32) | c[1]) >> 11;
    const uint64_t b = ((((uint64_t)c[2]) << 32) | c[3]) >> 11;
    const double u1 = ((double)a + 1.0) * (1.0 / 9007199254740992.0);
    const double u2 = (double)b * (1.0 / 9007199254740992.0);
    const double r = sqrt(-2.0 * log(u1));
    const double ang = 6.283185307179586476925286766559 * u2;
    z0 = r * cos(ang);
    z1 = r * sin(ang);
}
