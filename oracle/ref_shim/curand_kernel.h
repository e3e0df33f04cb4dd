/*
 * curand_kernel.h stand-in for the host build of the reference.
 *
 * TEST INFRASTRUCTURE ONLY.  It keeps the three cuRAND names the reference
 * calls (SwimmerArray.cu:13,173,179) and routes them to the project's own
 * counter-based stream (Philox4x32-10, keyed by seed, swimmer and move step;
 * implemented in oracle/lbswim_oracle.c).  The reference draws exactly one
 * uniform per Move call, so the number of uniform draws so far is the move
 * step; the normals of a tumble belong to the step of the last uniform draw.
 */
#ifndef LBSWIM_CURAND_STUB_H
#define LBSWIM_CURAND_STUB_H
#include <stdint.h>

extern "C" float orc_rng_uniform(uint64_t seed, uint32_t swimmer, uint64_t step);
extern "C" void orc_rng_normal3(uint64_t seed, uint32_t swimmer, uint64_t step, double out[3]);

struct curandStateXORWOW {
  unsigned long long seed;
  unsigned long long subsequence;
  unsigned long long calls;
  unsigned long long step;
  int k;
};

static inline void curand_init(unsigned long long seed, unsigned long long subsequence,
                               unsigned long long, curandStateXORWOW* s) {
  s->seed = seed;
  s->subsequence = subsequence;
  s->calls = 0;
  s->step = 0;
  s->k = 0;
}
static inline float curand_uniform(curandStateXORWOW* s) {
  s->step = s->calls++;
  s->k = 0;
  return orc_rng_uniform(s->seed, (uint32_t)s->subsequence, s->step);
}
static inline double curand_normal_double(curandStateXORWOW* s) {
  double g[3];
  orc_rng_normal3(s->seed, (uint32_t)s->subsequence, s->step, g);
  return g[(s->k++) % 3];
}
#endif
