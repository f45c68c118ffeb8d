/* Host restatement of Philox4x32-10 and of the Box-Muller normal mapping.
 *
 * TEST INFRASTRUCTURE ONLY: this header belongs to the oracle. It is the
 * checker that the CUDA kernels are compared with; no product code includes it.
 *
 * Philox4x32-10 is the counter-based generator of Salmon, Moraes, Dror and
 * Shaw, "Parallel Random Numbers: As Easy as 1, 2, 3" (SC'11). It is written
 * here from the paper's definition: ten rounds of two 32x32->64 multiplies
 * with the round multipliers 0xD2511F53 / 0xCD9E8D57 and a Weyl key schedule
 * with increments 0x9E3779B9 / 0xBB67AE85. The known-answer vectors in
 * tests/golden/philox_kat.json pin this implementation.
 *
 * Stream layout shared with the device kernels (one Philox block = 4 words =
 * 4 standard normals, one per path of a path quad):
 *   key     = (seed & 0xffffffff, seed >> 32)
 *   counter = (quad & 0xffffffff, step, stream, (tag << 16) | (quad >> 32))
 * "quad" is path_index / 4 (or antithetic pair index / 4), "step" the time or
 * asset index, "stream" the contract id, "tag" the pricing method.
 *
 * Uniforms: u = (2*(x >> 9) + 1) * 2^-24, exactly representable in binary32
 * and binary64, strictly inside (0,1).
 * Normals: (z0,z1) = sqrt(-2 ln u0) * (cos, sin)(pi*(2*u1 - 1)), and likewise
 * (z2,z3) from (u2,u3).
 */
#pragma once
#include <stdint.h>
#include <math.h>

namespace orc {

static inline void philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2],
                                 uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int round = 0; round < 10; ++round) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * (uint64_t)c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * (uint64_t)c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static inline double uniform_from_word(uint32_t x) {
  return (double)(2u * (x >> 9) + 1u) * 0x1p-24;
}

/* Four FP64 standard normals for (seed, stream, tag, quad, step). */
static inline void normals4(uint64_t seed, uint32_t stream, uint32_t tag, uint64_t quad,
                            uint32_t step, double z[4]) {
  uint32_t ctr[4] = {(uint32_t)quad, step, stream,
                     (tag << 16) | (uint32_t)((quad >> 32) & 0xffffu)};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  uint32_t x[4];
  philox4x32_10(ctr, key, x);
  const double pi = 3.14159265358979323846;
  for (int h = 0; h < 2; ++h) {
    const double u0 = uniform_from_word(x[2 * h]);
    const double u1 = uniform_from_word(x[2 * h + 1]);
    const double rad = sqrt(-2.0 * log(u0));
    const double th = pi * (2.0 * u1 - 1.0);
    z[2 * h] = rad * cos(th);
    z[2 * h + 1] = rad * sin(th);
  }
}

}  // namespace orc
