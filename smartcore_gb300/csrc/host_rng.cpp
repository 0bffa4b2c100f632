// Host-side draws of KMeans::kmeans_plus_plus for callers that are not the
// Rust crate itself (a Rust shim passes the crate's own draws instead).
//
// smartcore selects its generator in src/rand_custom.rs:1-32 (rand 0.8.5,
// Cargo.toml:28): SmallRng by default, StdRng with the std_rand feature;
// seed None means seed 0 without std_rand.  Published algorithms restated:
//   SmallRng (64-bit targets): xoshiro256++; seed_from_u64 expands the seed
//     with SplitMix64 into the four state words.
//   StdRng: ChaCha, 12 rounds; seed_from_u64 (rand_core 0.6) fills the key
//     with PCG32 (XSH RR) outputs; the block counter is 64-bit, the stream
//     id 0, and four 16-word blocks are buffered; a u64 is two words, low
//     word first.
//   gen::<f64>():      (next_u64 >> 11) * 2^-53
//   gen_range(0..n):   widening multiply of next_u64 by n with rejection
//                      zone (n << leading_zeros(n)) - 1, result = high word.
// The draw sequence used by kmeans.rs is gen_range(0..n) (:359), then one
// gen::<f64>() per further seed (:385).
#include <stdint.h>
#include <string.h>

#include "../../include/smartcore_gb300.h"

namespace sc {
void set_error(const char *fmt, ...);

namespace {

class Xoshiro256pp {
 public:
  explicit Xoshiro256pp(uint64_t seed) {
    uint64_t z0 = seed;
    for (auto &w : s_) {
      z0 += 0x9e3779b97f4a7c15ull;
      uint64_t z = z0;
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
      w = z ^ (z >> 31);
    }
  }
  uint64_t next() {
    const uint64_t out = rotl(s_[0] + s_[3], 23) + s_[0];
    const uint64_t t = s_[1] << 17;
    s_[2] ^= s_[0];
    s_[3] ^= s_[1];
    s_[1] ^= s_[2];
    s_[0] ^= s_[3];
    s_[2] ^= t;
    s_[3] = rotl(s_[3], 45);
    return out;
  }

 private:
  static uint64_t rotl(uint64_t v, int r) { return (v << r) | (v >> (64 - r)); }
  uint64_t s_[4];
};

class ChaCha12 {
 public:
  explicit ChaCha12(uint64_t seed) {
    uint64_t st = seed;
    for (auto &k : key_) {
      st = st * 6364136223846793005ull + 11634580456548205067ull;
      const uint32_t x = (uint32_t)(((st >> 18) ^ st) >> 27);
      const unsigned rot = (unsigned)(st >> 59) & 31u;
      k = rot ? (x >> rot) | (x << (32 - rot)) : x;
    }
  }
  uint64_t next() {
    if (pos_ >= 64) refill();
    if (pos_ == 63) {
      const uint64_t lo = words_[63];
      refill();
      pos_ = 1;
      return ((uint64_t)words_[0] << 32) | lo;
    }
    const uint64_t v = ((uint64_t)words_[pos_ + 1] << 32) | words_[pos_];
    pos_ += 2;
    return v;
  }

 private:
  static uint32_t rotl(uint32_t v, int r) { return (v << r) | (v >> (32 - r)); }
  static void quarter(uint32_t *w, int a, int b, int c, int d) {
    w[a] += w[b]; w[d] = rotl(w[d] ^ w[a], 16);
    w[c] += w[d]; w[b] = rotl(w[b] ^ w[c], 12);
    w[a] += w[b]; w[d] = rotl(w[d] ^ w[a], 8);
    w[c] += w[d]; w[b] = rotl(w[b] ^ w[c], 7);
  }
  void block(uint64_t ctr, uint32_t *out) const {
    static const uint32_t sigma[4] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u};
    uint32_t init[16], w[16];
    memcpy(init, sigma, sizeof sigma);
    memcpy(init + 4, key_, sizeof key_);
    init[12] = (uint32_t)ctr;
    init[13] = (uint32_t)(ctr >> 32);
    init[14] = init[15] = 0u;
    memcpy(w, init, sizeof w);
    for (int r = 0; r < 12; r += 2) {
      quarter(w, 0, 4, 8, 12); quarter(w, 1, 5, 9, 13);
      quarter(w, 2, 6, 10, 14); quarter(w, 3, 7, 11, 15);
      quarter(w, 0, 5, 10, 15); quarter(w, 1, 6, 11, 12);
      quarter(w, 2, 7, 8, 13); quarter(w, 3, 4, 9, 14);
    }
    for (int i = 0; i < 16; ++i) out[i] = w[i] + init[i];
  }
  void refill() {
    for (int b = 0; b < 4; ++b) block(counter_ + (uint64_t)b, words_ + 16 * b);
    counter_ += 4;
    pos_ = 0;
  }
  uint32_t key_[8];
  uint64_t counter_ = 0;
  uint32_t words_[64];
  int pos_ = 64;
};

template <class G>
void draws(G &g, int64_t n, int64_t k, int64_t *first, double *u) {
  const uint64_t range = (uint64_t)n;
  const uint64_t zone = (range << __builtin_clzll(range)) - 1;
  for (;;) {
    const unsigned __int128 p = (unsigned __int128)g.next() * range;
    if ((uint64_t)p <= zone) {
      *first = (int64_t)(uint64_t)(p >> 64);
      break;
    }
  }
  for (int64_t j = 0; j + 1 < k; ++j) u[j] = (double)(g.next() >> 11) * 0x1.0p-53;
}

}  // namespace
}  // namespace sc

extern "C" sc_status sc_kmeanspp_draws(int32_t rng, uint64_t seed, int64_t n,
                                       int64_t k, int64_t *first_index,
                                       double *uniforms) {
  if (n < 1) {
    sc::set_error("cannot sample empty range");  // gen_range(0..0) panics in rand
    return SC_ERR_INVALID;
  }
  if (k < 1 || !first_index || (k > 1 && !uniforms)) {
    sc::set_error("invalid number of clusters: %lld", (long long)k);
    return SC_ERR_INVALID;
  }
  if (rng == SC_RNG_SMALL) {
    sc::Xoshiro256pp g(seed);
    sc::draws(g, n, k, first_index, uniforms);
  } else if (rng == SC_RNG_STD) {
    sc::ChaCha12 g(seed);
    sc::draws(g, n, k, first_index, uniforms);
  } else {
    sc::set_error("unknown generator %d", (int)rng);
    return SC_ERR_INVALID;
  }
  return SC_OK;
}
