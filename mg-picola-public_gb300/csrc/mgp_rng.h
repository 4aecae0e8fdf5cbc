/*
 * Counter-based white-noise streams for the 2LPT initial conditions.
 *
 * The reference seeds GSL's ranlxd1 generator once with `Seed` to fill the
 * seed table and re-seeds it per (i,j) column of the k-space grid
 * (src/2LPT.c:259-271, 344-354).  This library keeps that structure but uses
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) as the generator: the
 * stream for integer seed s returns, on its n-th call, the 53-bit uniform
 * built from the first two output words of Philox(counter = (n_lo, n_hi, 0, 0),
 * key = (s, 0x4D475043)).  Counter-based draws let a GPU thread jump straight
 * to any draw without replaying the stream.
 */
#ifndef MGP_RNG_H
#define MGP_RNG_H
#include <stdint.h>

#if defined(__CUDACC__)
#define MGP_HD __host__ __device__ __forceinline__
#else
#define MGP_HD static inline
#endif

MGP_HD void mgp_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                       uint32_t *o0, uint32_t *o1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    c1 = (uint32_t)p1;
    c3 = (uint32_t)p0;
    c0 = n0;
    c2 = n2;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  *o0 = c0;
  *o1 = c1;
}

/* Draw n of stream `seed`, uniform in [0, 1). */
MGP_HD double mgp_uniform(uint32_t seed, uint64_t n) {
  uint32_t o0, o1;
  mgp_philox((uint32_t)n, (uint32_t)(n >> 32), 0u, 0u, seed, 0x4D475043u, &o0, &o1);
  uint64_t u53 = ((uint64_t)o0 << 21) | (uint64_t)(o1 >> 11);
  return (double)u53 * (1.0 / 9007199254740992.0);
}

#endif
