/*
 * odp_rng.h -- the random stream behind the ODP graph utilities.
 *
 * The reference draws every random choice of its generators and 2-opt
 * mutations from libc rand() (utils.c:361-364 get_random, seeded by
 * ODP_Srand -> srand, utils.c:1036-1039).  To make seeded graphs reproducible
 * bit for bit, and to let many graphs be generated in parallel without the
 * global lock inside rand(), this header carries a private copy of the same
 * stream: glibc's TYPE_3 additive feedback generator (degree 31, separation 3),
 * as published in P. Selinger, "The GLIBC pseudo-random number generator":
 *
 *   r[0] = seed (0 is replaced by 1)
 *   r[i] = 16807 * r[i-1] mod (2^31 - 1),   i = 1..30   (Schrage's method)
 *   r[i] = r[i-31],                         i = 31..33
 *   r[i] = r[i-31] + r[i-3]  (mod 2^32),    i >= 34
 *   output k = r[k + 344] >> 1
 *
 * A stream flagged `libc` forwards to rand() instead, so the public
 * ODP_Srand/ODP_Generate_* entry points keep sharing the caller's rand()
 * state exactly as the reference does (its SA clients interleave random()).
 * The tests check the private stream against rand() output.
 */
#ifndef ODP_RNG_H
#define ODP_RNG_H
#include <stdint.h>
#include <stdlib.h>

/* The stream is produced in blocks: line[0..30] holds the 31 words before
 * the block, r[i-31..i-1]; a refill computes the next ODP_RNG_BLOCK words into
 * line[31..] in a straight loop (r[i] = r[i-31] + r[i-3]), then copies the
 * block's last 31 words down to line[0..30] as the next block's history.
 * Outputs r[i] >> 1 are handed out from line[31 + pos]. */
#define ODP_RNG_BLOCK 2046     /* a multiple of 3: the refill runs 3 lanes */

typedef struct odp_rng {
  uint32_t line[31 + ODP_RNG_BLOCK];
  int pos;                    /* next unread output in line[31..] */
  int libc;
} odp_rng;

static inline void odp_rng_refill(odp_rng *g)
{
  /* r[i-3], r[i-2], r[i-1] stay in registers: going through memory makes each
   * word wait on a store issued three iterations earlier. */
  uint32_t *r = g->line;
  uint32_t a = r[28], b = r[29], c = r[30];
  for(int i = 31; i < 31 + ODP_RNG_BLOCK; i += 3){
    a += r[i - 31]; b += r[i - 30]; c += r[i - 29];
    r[i] = a; r[i + 1] = b; r[i + 2] = c;
  }
  for(int i = 0; i < 31; i++) r[i] = r[ODP_RNG_BLOCK + i];
  g->pos = 0;
}

static inline int32_t odp_rng_step(odp_rng *g)
{
  if(g->pos == ODP_RNG_BLOCK) odp_rng_refill(g);
  return (int32_t)(g->line[31 + g->pos++] >> 1);
}

static inline void odp_rng_seed(odp_rng *g, unsigned int seed)
{
  uint32_t r[344];
  g->libc = 0;
  r[0] = (seed == 0) ? 1u : seed;
  /* the recurrence runs on the seed read as a signed 32-bit word */
  int64_t x = (seed == 0) ? 1 : (int64_t)(int32_t)seed;
  for(int i = 1; i < 31; i++){
    int64_t hi = x / 127773, lo = x % 127773;
    x = 16807 * lo - 2836 * hi;
    if(x < 0) x += 2147483647;
    r[i] = (uint32_t)x;
  }
  for(int i = 31; i < 34; i++) r[i] = r[i - 31];
  for(int i = 34; i < 344; i++) r[i] = r[i - 31] + r[i - 3];
  /* outputs start at r[344]; keep r[313..343] as the history */
  for(int i = 0; i < 31; i++) g->line[i] = r[313 + i];
  g->pos = ODP_RNG_BLOCK;
}

static inline int odp_rng_next(odp_rng *g)
{
  return g->libc ? rand() : (int)odp_rng_step(g);
}

/* Uniform integer in [0, max): the reference's get_random (utils.c:361-364),
 * same double arithmetic so the truncation matches for every max. */
static inline int odp_rng_below(odp_rng *g, int max)
{
  int x = odp_rng_next(g);
  /* x * max < 2^53 makes the double product exact and the division by 2^31
   * exact, so the truncated quotient equals the integer shift. */
  if(max >= 0 && max <= (1 << 22))
    return (int)(((uint64_t)(uint32_t)x * (uint64_t)max) >> 31);
  return (int)(x * ((double)max) / (1.0 + 2147483647.0));
}

#endif
