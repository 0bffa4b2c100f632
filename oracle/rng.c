/*
 * Oracle restatement of the random draws behind KMeans::kmeans_plus_plus.
 * TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * smartcore picks its generator in src/rand_custom.rs:1-32:
 *   - default features: rand::rngs::SmallRng, seeded by seed_from_u64(seed),
 *     seed None -> 0 (rand_custom.rs:26-27);
 *   - feature std_rand: rand::rngs::StdRng.
 * rand is pinned at 0.8.5 (Cargo.toml:28), which is not vendored here.  Its
 * published algorithms, restated below:
 *   - SmallRng on 64-bit targets = xoshiro256++ (Blackman & Vigna), whose
 *     seed_from_u64 fills the 256-bit state with four SplitMix64 outputs;
 *   - StdRng = ChaCha with 12 rounds (Bernstein), 256-bit key, 64-bit block
 *     counter and 64-bit stream id 0; seed_from_u64 (rand_core 0.6 default)
 *     fills the key with eight PCG32 (XSH-RR) outputs; words are consumed
 *     four blocks at a time and next_u64 joins two words low-first;
 *   - gen::<f64>() = (next_u64 >> 11) * 2^-53;
 *   - gen_range(low..high) over usize = widening-multiply rejection with the
 *     zone (range << lzcnt(range)) - 1.
 * No reference test pins a seeded draw: parity of these draws is unpinned.
 */
#include "oracle.h"

#include <string.h>

typedef struct {
  int kind;
  uint64_t s[4];     /* xoshiro256++ state */
  uint32_t key[8];   /* chacha key */
  uint64_t counter;  /* chacha block counter */
  uint32_t buf[64];  /* four chacha blocks */
  int idx;           /* next unread word of buf */
} orc_rng;

static uint64_t rotl64(uint64_t v, int r) { return (v << r) | (v >> (64 - r)); }
static uint32_t rotl32(uint32_t v, int r) { return (v << r) | (v >> (32 - r)); }
static uint32_t rotr32(uint32_t v, unsigned r) {
  r &= 31u;
  return r ? (v >> r) | (v << (32 - r)) : v;
}

/* The ChaCha block function (Bernstein; RFC 7539 section 2.3 for 20 rounds):
 * state = the four constants, the 256-bit key, words 12..15 as given;
 * `rounds` rounds (column and diagonal rounds alternating), then the input
 * added word by word. */
void orc_chacha_block(const uint32_t key[8], const uint32_t w12_15[4], int rounds, uint32_t out[16]) {
  uint32_t in[16], w[16];
  in[0] = 0x61707865u; in[1] = 0x3320646eu; in[2] = 0x79622d32u; in[3] = 0x6b206574u;
  for (int i = 0; i < 8; ++i) in[4 + i] = key[i];
  for (int i = 0; i < 4; ++i) in[12 + i] = w12_15[i];
  memcpy(w, in, sizeof w);
#define QR(a, b, c, d)                                   \
  w[a] += w[b]; w[d] ^= w[a]; w[d] = rotl32(w[d], 16);   \
  w[c] += w[d]; w[b] ^= w[c]; w[b] = rotl32(w[b], 12);   \
  w[a] += w[b]; w[d] ^= w[a]; w[d] = rotl32(w[d], 8);    \
  w[c] += w[d]; w[b] ^= w[c]; w[b] = rotl32(w[b], 7);
  for (int r = 0; r < rounds; r += 2) { /* a column round and a diagonal round */
    QR(0, 4, 8, 12) QR(1, 5, 9, 13) QR(2, 6, 10, 14) QR(3, 7, 11, 15)
    QR(0, 5, 10, 15) QR(1, 6, 11, 12) QR(2, 7, 8, 13) QR(3, 4, 9, 14)
  }
#undef QR
  for (int i = 0; i < 16; ++i) out[i] = w[i] + in[i];
}

/* One ChaCha quarter round on (a, b, c, d) (RFC 7539 section 2.1). */
void orc_chacha_quarter_round(uint32_t v[4]) {
  v[0] += v[1]; v[3] ^= v[0]; v[3] = rotl32(v[3], 16);
  v[2] += v[3]; v[1] ^= v[2]; v[1] = rotl32(v[1], 12);
  v[0] += v[1]; v[3] ^= v[0]; v[3] = rotl32(v[3], 8);
  v[2] += v[3]; v[1] ^= v[2]; v[1] = rotl32(v[1], 7);
}

/* rand's ChaCha12 block: 64-bit block counter in words 12-13, stream id 0. */
static void chacha_block(const uint32_t key[8], uint64_t ctr, uint32_t out[16]) {
  const uint32_t w[4] = {(uint32_t)ctr, (uint32_t)(ctr >> 32), 0u, 0u};
  orc_chacha_block(key, w, 12, out);
}

/* xoshiro256++ (Blackman & Vigna): output rotl(s0 + s3, 23) + s0, then the
 * state update. */
static uint64_t xoshiro_next(uint64_t s[4]) {
  uint64_t r = rotl64(s[0] + s[3], 23) + s[0];
  uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = rotl64(s[3], 45);
  return r;
}

void orc_xoshiro256pp(const uint64_t state[4], int64_t count, uint64_t *out) {
  uint64_t s[4] = {state[0], state[1], state[2], state[3]};
  for (int64_t i = 0; i < count; ++i) out[i] = xoshiro_next(s);
}

/* SplitMix64 (Steele, Lea & Flood): state += golden gamma, then the mix. */
static uint64_t splitmix_next(uint64_t *st) {
  *st += 0x9e3779b97f4a7c15ull;
  uint64_t z = *st;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

void orc_splitmix64(uint64_t seed, int64_t count, uint64_t *out) {
  uint64_t st = seed;
  for (int64_t i = 0; i < count; ++i) out[i] = splitmix_next(&st);
}

/* PCG32 output function XSH-RR (O'Neill) of a 64-bit LCG state. */
static uint32_t pcg_xsh_rr(uint64_t st) {
  uint32_t xs = (uint32_t)(((st >> 18) ^ st) >> 27);
  return rotr32(xs, (unsigned)(st >> 59));
}

/* count outputs of the LCG state' = state * 6364136223846793005 + inc with
 * the XSH-RR output of the state before the step (after_step = 0, the PCG
 * paper's pcg32) or after it (after_step = 1, rand_core's seed filler). */
void orc_pcg32(uint64_t state, uint64_t inc, int after_step, int64_t count, uint32_t *out) {
  for (int64_t i = 0; i < count; ++i) {
    const uint64_t old = state;
    state = state * 6364136223846793005ull + inc;
    out[i] = pcg_xsh_rr(after_step ? state : old);
  }
}

static void chacha_refill(orc_rng *g) {
  for (int b = 0; b < 4; ++b) chacha_block(g->key, g->counter + (uint64_t)b, g->buf + 16 * b);
  g->counter += 4;
  g->idx = 0;
}

static void rng_seed(orc_rng *g, int kind, uint64_t seed) {
  memset(g, 0, sizeof *g);
  g->kind = kind;
  if (kind == ORC_RNG_SMALL) {
    uint64_t st = seed;
    for (int i = 0; i < 4; ++i) g->s[i] = splitmix_next(&st);
    /* an all-zero state would be reseeded from 0; SplitMix64 never yields it */
  } else {
    orc_pcg32(seed, 11634580456548205067ull, 1, 8, g->key);
    g->counter = 0;
    g->idx = 64; /* empty: first read generates */
  }
}

static uint64_t rng_next_u64(orc_rng *g) {
  if (g->kind == ORC_RNG_SMALL) return xoshiro_next(g->s);
  if (g->idx >= 64) chacha_refill(g);
  if (g->idx == 63) { /* a u64 straddling two refills: low word first */
    uint64_t lo = g->buf[63];
    chacha_refill(g);
    uint64_t hi = g->buf[0];
    g->idx = 1;
    return (hi << 32) | lo;
  }
  uint64_t lo = g->buf[g->idx], hi = g->buf[g->idx + 1];
  g->idx += 2;
  return (hi << 32) | lo;
}

static double rng_gen_f64(orc_rng *g) {
  return (double)(rng_next_u64(g) >> 11) * (1.0 / 9007199254740992.0);
}

static uint64_t rng_gen_below(orc_rng *g, uint64_t n) {
  uint64_t range = n; /* low = 0, high = n - 1 inclusive */
  if (range == 0) return rng_next_u64(g);
  int lz = __builtin_clzll(range);
  uint64_t zone = (range << lz) - 1;
  for (;;) {
    uint64_t v = rng_next_u64(g);
    unsigned __int128 p = (unsigned __int128)v * range;
    uint64_t lo = (uint64_t)p, hi = (uint64_t)(p >> 64);
    if (lo <= zone) return hi;
  }
}

void orc_kmeanspp_draws(int rng_kind, uint64_t seed, int64_t n, int64_t k,
                        int64_t *first_index, double *uniforms) {
  orc_rng g;
  rng_seed(&g, rng_kind, seed);
  *first_index = (int64_t)rng_gen_below(&g, (uint64_t)n);
  for (int64_t j = 0; j + 1 < k; ++j) uniforms[j] = rng_gen_f64(&g);
}

void orc_rng_u64(int rng_kind, uint64_t seed, int64_t count, uint64_t *out) {
  orc_rng g;
  rng_seed(&g, rng_kind, seed);
  for (int64_t i = 0; i < count; ++i) out[i] = rng_next_u64(&g);
}
