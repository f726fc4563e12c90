// ts_common.h — primitives shared by the host driver and the CUDA kernels.
//
// PCG32 (rand_pcg 0.3.1 Lcg64Xsh32) seeded through rand_core 0.6.3's
// seed_from_u64, and rand 0.8.5's integer gen_range: the reference draws every
// random number through these (ms.rs:386, 454-458, 549-564, 804).
// ts_exp64 is the exponential used for the neighbour weights (ms.rs:1198-1203).
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define TS_HD __host__ __device__ __forceinline__
#else
#define TS_HD inline
#include <math.h>
#endif

namespace ts {

constexpr uint64_t kPcgMul = 6364136223846793005ULL;
constexpr uint64_t kPcgSeedInc = 11634580027462260723ULL;
constexpr uint32_t kOutside = 0xFF000000u;  // Rgba([0, 0, 0, 255]) packed little-endian

struct Pcg32 {
  uint64_t state, inc;
};

// XSH RR output function (PCG paper, O'Neill 2014).
TS_HD uint32_t pcg_output(uint64_t s) {
  uint32_t x = (uint32_t)(((s >> 18) ^ s) >> 27);
  uint32_t r = (uint32_t)(s >> 59);
  return (x >> r) | (x << ((32u - r) & 31u));
}

// seed_from_u64: four words of a fixed-increment PCG32 stream form the
// 16-byte seed (state, increment | 1); from_seed adds the increment and steps.
TS_HD Pcg32 pcg_from_u64(uint64_t seed) {
  uint32_t w0, w1, w2, w3;
  seed = seed * kPcgMul + kPcgSeedInc;
  w0 = pcg_output(seed);
  seed = seed * kPcgMul + kPcgSeedInc;
  w1 = pcg_output(seed);
  seed = seed * kPcgMul + kPcgSeedInc;
  w2 = pcg_output(seed);
  seed = seed * kPcgMul + kPcgSeedInc;
  w3 = pcg_output(seed);
  Pcg32 g;
  g.inc = ((uint64_t)w2 | ((uint64_t)w3 << 32)) | 1ULL;
  g.state = ((uint64_t)w0 | ((uint64_t)w1 << 32)) + g.inc;
  g.state = g.state * kPcgMul + g.inc;
  return g;
}

TS_HD uint32_t pcg_u32(Pcg32 &g) {
  uint64_t s = g.state;
  g.state = s * kPcgMul + g.inc;
  return pcg_output(s);
}

TS_HD uint64_t pcg_u64(Pcg32 &g) {
  uint64_t lo = pcg_u32(g);
  uint64_t hi = pcg_u32(g);
  return lo | (hi << 32);
}

TS_HD uint32_t clz32(uint32_t v) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__clz(v);
#else
  return (uint32_t)__builtin_clz(v);
#endif
}
TS_HD uint32_t clz64(uint64_t v) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__clzll(v);
#else
  return (uint32_t)__builtin_clzll(v);
#endif
}
TS_HD uint64_t mulhi64(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// Rng::gen_range(0..n) for u32: widening multiply, rejection zone
// (n << clz(n)) - 1.  n > 0.
TS_HD uint32_t gen_range_u32(Pcg32 &g, uint32_t n) {
  uint32_t zone = (n << clz32(n)) - 1u;
  for (;;) {
    uint64_t m = (uint64_t)pcg_u32(g) * n;
    if ((uint32_t)m <= zone) return (uint32_t)(m >> 32);
  }
}

// The same for usize on 64-bit targets.  n > 0.
TS_HD uint64_t gen_range_u64(Pcg32 &g, uint64_t n) {
  uint64_t zone = (n << clz64(n)) - 1u;
  for (;;) {
    uint64_t v = pcg_u64(g);
    if (v * n <= zone) return mulhi64(v, n);
  }
}

// Bounded variant for device loops: gives up (returns false) after
// max_draws rejected draws instead of spinning.
TS_HD bool gen_range_u32_bounded(Pcg32 &g, uint32_t n, uint32_t max_draws, uint32_t &out) {
  uint32_t zone = (n << clz32(n)) - 1u;
  for (uint32_t i = 0; i < max_draws; ++i) {
    uint64_t m = (uint64_t)pcg_u32(g) * n;
    if ((uint32_t)m <= zone) {
      out = (uint32_t)(m >> 32);
      return true;
    }
  }
  return false;
}
TS_HD bool gen_range_u64_bounded(Pcg32 &g, uint64_t n, uint32_t max_draws, uint64_t &out) {
  uint64_t zone = (n << clz64(n)) - 1u;
  for (uint32_t i = 0; i < max_draws; ++i) {
    uint64_t v = pcg_u64(g);
    if (v * n <= zone) {
      out = mulhi64(v, n);
      return true;
    }
  }
  return false;
}

// exp(x) in double: Cody-Waite reduction x = n*ln2 + r (ln2 split in a
// high part with trailing zero bits and a low part), Taylor series of e^r to
// degree 13 in Horner form with fused multiply-adds, times 2^n.  Every step
// is a correctly rounded IEEE operation, so host and device agree bit for
// bit.  Inputs below -700 return 0 (the weights are rounded to f32, where
// anything under 2^-150 is 0).
TS_HD double ts_exp64(double x) {
  if (x != x) return x;
  if (x < -700.0) return 0.0;
  if (x > 700.0) return __builtin_huge_val();
  const double inv_ln2 = 1.44269504088896338700e+00;
  const double ln2_hi = 6.93147180369123816490e-01;
  const double ln2_lo = 1.90821492927058770002e-10;
#ifdef __CUDA_ARCH__
  double n = rint(__dmul_rn(x, inv_ln2));
  double r = __dsub_rn(x, __dmul_rn(n, ln2_hi));
  r = __dsub_rn(r, __dmul_rn(n, ln2_lo));
#define TS_FMA(a, b, c) __fma_rn(a, b, c)
#else
  double n = rint(x * inv_ln2);
  double r = x - n * ln2_hi;
  r = r - n * ln2_lo;
#define TS_FMA(a, b, c) fma(a, b, c)
#endif
  double p = 1.0 / 6227020800.0;
  p = TS_FMA(p, r, 1.0 / 479001600.0);
  p = TS_FMA(p, r, 1.0 / 39916800.0);
  p = TS_FMA(p, r, 1.0 / 3628800.0);
  p = TS_FMA(p, r, 1.0 / 362880.0);
  p = TS_FMA(p, r, 1.0 / 40320.0);
  p = TS_FMA(p, r, 1.0 / 5040.0);
  p = TS_FMA(p, r, 1.0 / 720.0);
  p = TS_FMA(p, r, 1.0 / 120.0);
  p = TS_FMA(p, r, 1.0 / 24.0);
  p = TS_FMA(p, r, 1.0 / 6.0);
  p = TS_FMA(p, r, 0.5);
  p = TS_FMA(p, r, 1.0);
  p = TS_FMA(p, r, 1.0);
#undef TS_FMA
  return ldexp(p, (int)n);
}

}  // namespace ts
