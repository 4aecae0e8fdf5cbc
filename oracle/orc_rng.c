/*
 * Oracle random numbers (test infrastructure only).
 *
 * The reference draws its white noise from GSL's ranlxd1 generator
 * (src/2LPT.c:259-271 seed table, 344-354 per-column streams).  GSL is not
 * available and its generator is not reproduced here; the project defines a
 * counter-based stand-in with the same call structure: a "stream" is keyed
 * by the integer seed that gsl_rng_set() would receive, and the n-th call of
 * gsl_rng_uniform() on that stream returns draw n.
 *
 * Generator: Philox4x32-10, J. K. Salmon, M. A. Moraes, R. O. Dror,
 * D. E. Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11.
 * Stream draw n: counter = (n_lo, n_hi, 0, 0), key = (seed, 0x4D475043);
 * u = ((out0 << 21) | (out1 >> 11)) * 2^-53, a double in [0, 1).
 */
#include "orc.h"

void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; r++) {
    if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

double orc_stream_uniform(uint32_t seed, uint64_t n) {
  uint32_t ctr[4] = {(uint32_t)n, (uint32_t)(n >> 32), 0u, 0u};
  uint32_t key[2] = {seed, 0x4D475043u};
  uint32_t o[4];
  orc_philox4x32_10(ctr, key, o);
  uint64_t u53 = ((uint64_t)o[0] << 21) | (uint64_t)(o[1] >> 11);
  return (double)u53 * (1.0 / 9007199254740992.0);
}
