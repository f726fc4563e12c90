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
// rand 0.8.5 UniformInt<u8>::sample_single(0, 255) with a Pcg32 seeded by
// seed_from_u64(seed): for 8- and 16-bit types the rejection zone is
// u32::MAX - (u32::MAX - range + 1) % range (range = 255 here), the draw
// (v * range) >> 32 of a u32 v.  The colour of an id in the debug maps
// (ms.rs:604-636).
TS_HD uint8_t id_colour(uint64_t seed) {
  Pcg32 g = pcg_from_u64(seed);
  const uint32_t range = 255u;
  const uint32_t zone = 0xffffffffu - (uint32_t)((0x100000000ull - range) % range);
  uint64_t m = 0;
  for (int t = 0; t < 64; ++t) {  // a draw is rejected with probability 2^-32
    m = (uint64_t)pcg_u32(g) * range;
    if ((uint32_t)m <= zone) break;
  }
  return (uint8_t)(m >> 32);
}

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

// 2^(j/64), j = 0..63, each the nearest double (gen_exp_table.py).
#define TS_EXP2_TABLE_VALUES \
  0x1.0000000000000p+0, 0x1.02c9a3e778061p+0, \
  0x1.059b0d3158574p+0, 0x1.0874518759bc8p+0, \
  0x1.0b5586cf9890fp+0, 0x1.0e3ec32d3d1a2p+0, \
  0x1.11301d0125b51p+0, 0x1.1429aaea92de0p+0, \
  0x1.172b83c7d517bp+0, 0x1.1a35beb6fcb75p+0, \
  0x1.1d4873168b9aap+0, 0x1.2063b88628cd6p+0, \
  0x1.2387a6e756238p+0, 0x1.26b4565e27cddp+0, \
  0x1.29e9df51fdee1p+0, 0x1.2d285a6e4030bp+0, \
  0x1.306fe0a31b715p+0, 0x1.33c08b26416ffp+0, \
  0x1.371a7373aa9cbp+0, 0x1.3a7db34e59ff7p+0, \
  0x1.3dea64c123422p+0, 0x1.4160a21f72e2ap+0, \
  0x1.44e086061892dp+0, 0x1.486a2b5c13cd0p+0, \
  0x1.4bfdad5362a27p+0, 0x1.4f9b2769d2ca7p+0, \
  0x1.5342b569d4f82p+0, 0x1.56f4736b527dap+0, \
  0x1.5ab07dd485429p+0, 0x1.5e76f15ad2148p+0, \
  0x1.6247eb03a5585p+0, 0x1.6623882552225p+0, \
  0x1.6a09e667f3bcdp+0, 0x1.6dfb23c651a2fp+0, \
  0x1.71f75e8ec5f74p+0, 0x1.75feb564267c9p+0, \
  0x1.7a11473eb0187p+0, 0x1.7e2f336cf4e62p+0, \
  0x1.82589994cce13p+0, 0x1.868d99b4492edp+0, \
  0x1.8ace5422aa0dbp+0, 0x1.8f1ae99157736p+0, \
  0x1.93737b0cdc5e5p+0, 0x1.97d829fde4e50p+0, \
  0x1.9c49182a3f090p+0, 0x1.a0c667b5de565p+0, \
  0x1.a5503b23e255dp+0, 0x1.a9e6b5579fdbfp+0, \
  0x1.ae89f995ad3adp+0, 0x1.b33a2b84f15fbp+0, \
  0x1.b7f76f2fb5e47p+0, 0x1.bcc1e904bc1d2p+0, \
  0x1.c199bdd85529cp+0, 0x1.c67f12e57d14bp+0, \
  0x1.cb720dcef9069p+0, 0x1.d072d4a07897cp+0, \
  0x1.d5818dcfba487p+0, 0x1.da9e603db3285p+0, \
  0x1.dfc97337b9b5fp+0, 0x1.e502ee78b3ff6p+0, \
  0x1.ea4afa2a490dap+0, 0x1.efa1bee615a27p+0, \
  0x1.f50765b6e4540p+0, 0x1.fa7c1819e90d8p+0,

// exp(x) in double, table driven: x = (64 m + j) ln2/64 + r with
// |r| <= ln2/128 (Cody-Waite reduction with ln2/64 split in a high part whose
// trailing bits are zero and a low part), e^r by its Taylor series to degree 5
// in Horner form with fused multiply-adds, times 2^(j/64) from the table and
// 2^m.  Every step is a correctly rounded IEEE operation, so host and device
// produce the same double, within a few ulp of the true exponential.  Inputs
// below -700 return 0 (the weights are rounded to f32, where anything under
// 2^-150 is 0).  `table` holds TS_EXP2_TABLE_VALUES.
TS_HD double ts_exp64(double x, const double *table) {
  if (x != x) return x;
  if (x < -700.0) return 0.0;
  if (x > 700.0) return __builtin_huge_val();
  const double inv_step = 0x1.71547652b82fep+6;
  const double step_hi = 0x1.62e42fee00000p-7;
  const double step_lo = 0x1.a39ef35793c76p-39;
#ifdef __CUDA_ARCH__
  const double k = rint(__dmul_rn(x, inv_step));
#define TS_FMA(a, b, c) __fma_rn(a, b, c)
#else
  const double k = rint(x * inv_step);
#define TS_FMA(a, b, c) fma(a, b, c)
#endif
  double r = TS_FMA(-k, step_hi, x);
  r = TS_FMA(-k, step_lo, r);
  double p = 1.0 / 120.0;
  p = TS_FMA(p, r, 1.0 / 24.0);
  p = TS_FMA(p, r, 1.0 / 6.0);
  p = TS_FMA(p, r, 0.5);
  p = TS_FMA(p, r, 1.0);
  p = TS_FMA(p, r, 1.0);
#undef TS_FMA
  const int ki = (int)k;
#ifdef __CUDA_ARCH__
  const double t = __dmul_rn(table[ki & 63], p);
#else
  const double t = table[ki & 63] * p;
#endif
  return ldexp(t, ki >> 6);
}

// a / b correctly rounded from y = RN(1/b): q0 = RN(a y), r = a - b q0
// (exact with a fused multiply-add), q = RN(q0 + r y) -- Markstein's
// correction, exact for operands whose quotient neither overflows nor
// underflows; a / 0 and 0 / 0 propagate as inf and NaN through q0.
TS_HD double ts_div_markstein(double a, double b, double y) {
#ifdef __CUDA_ARCH__
  const double q0 = __dmul_rn(a, y);
  const double r = __fma_rn(-q0, b, a);
  return __fma_rn(r, y, q0);
#else
  const double q0 = a * y;
  const double r = fma(-q0, b, a);
  return fma(r, y, q0);
#endif
}

// Bit casts shared by host and device code.
TS_HD uint64_t dbl_bits(double v) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(v);
#else
  uint64_t u;
  __builtin_memcpy(&u, &v, 8);
  return u;
#endif
}
TS_HD double bits_dbl(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double v;
  __builtin_memcpy(&v, &u, 8);
  return v;
#endif
}
TS_HD uint32_t flt_bits(float v) {
#ifdef __CUDA_ARCH__
  return (uint32_t)__float_as_uint(v);
#else
  uint32_t u;
  __builtin_memcpy(&u, &v, 4);
  return u;
#endif
}
TS_HD float bits_flt(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float v;
  __builtin_memcpy(&v, &u, 4);
  return v;
#endif
}

// ---------------------------------------------------------------------------
// IEEE round-to-nearest-even addition of non-negative doubles in integer
// arithmetic, for the in-order sum of the 4x-duplicated distance list
// (ms.rs:417-421), and integer division of that sum.  The kernels sum with
// hardware f64 adds: as one thread's dependent chain these integer steps
// measured slower on GB300 (16.8k against 14.1k cycles at k = 50).  They
// stay as the bit-exact statement of the binade rule (within one binade
// every add rounds the addend to the sum's ulp) that an exact parallel sum
// builds on, and the CPU and GPU tests hold them to hardware f64.
// Operands are the bit patterns of finite doubles >= 0 (zero or normal).
// ---------------------------------------------------------------------------
constexpr uint64_t kFrac52 = (1ULL << 52) - 1;

// RN(x + y): align with guard, round and sticky bits, add, renormalise once,
// round to nearest even.
TS_HD uint64_t ts_add_rn(uint64_t bx, uint64_t by) {
  if (bx < by) {
    const uint64_t t = bx;
    bx = by;
    by = t;
  }
  if (by == 0) return bx;
  uint32_t ex = (uint32_t)(bx >> 52);
  const uint32_t ey = (uint32_t)(by >> 52);
  const uint64_t mx = (bx & kFrac52) | (1ULL << 52);
  const uint64_t my = (by & kFrac52) | (1ULL << 52);
  const uint32_t sh = ex - ey;
  uint64_t y;
  if (sh >= 58) {
    y = 1;  // only the sticky bit survives
  } else {
    const uint64_t y3 = my << 3;
    y = (y3 >> sh) | ((y3 & ((1ULL << sh) - 1)) != 0 ? 1u : 0u);
  }
  uint64_t z = (mx << 3) + y;
  if (z >> 56) {
    z = (z >> 1) | (z & 1u);
    ++ex;
  }
  uint64_t m = z >> 3;
  const uint32_t low = (uint32_t)(z & 7u);
  if (low > 4u || (low == 4u && (m & 1u))) ++m;
  if (m >> 53) {
    m >>= 1;
    ++ex;
  }
  return ((uint64_t)ex << 52) | (m & kFrac52);
}

// RN(RN(RN(RN(s + d) + d) + d) + d).  When all four sums stay in s's binade,
// s is on that binade's grid u and every step adds d rounded to u: the bit
// pattern advances by 4 * round(d / u) (exact ties alternate by parity).
// ts_add4_fast handles that case (and d = 0) and returns false otherwise.
TS_HD bool ts_add4_fast(uint64_t bs, uint64_t bd, uint64_t &out) {
  if (bd == 0) {
    out = bs;
    return true;
  }
  if (bs == 0 || bs <= bd) return false;
  const uint32_t es = (uint32_t)(bs >> 52), ed = (uint32_t)(bd >> 52);
  const uint32_t sh = es - ed;
  if (sh == 0) return false;  // same binade: a carry is likely
  uint64_t a, rem, half;
  if (sh >= 54) {
    a = 0;
    rem = 1;  // below half an ulp: rounds down
    half = 2;
  } else {
    const uint64_t md = (bd & kFrac52) | (1ULL << 52);
    a = md >> sh;
    rem = md & ((1ULL << sh) - 1);
    half = 1ULL << (sh - 1);
  }
  if ((bs & kFrac52) + 4 * (a + 1) >= (1ULL << 52)) return false;  // may leave the binade
  if (rem != half) {
    out = bs + 4 * (a + (rem > half ? 1u : 0u));
    return true;
  }
  uint64_t b = bs;
  for (int i = 0; i < 4; ++i) {
    b += a;
    b += b & 1u;  // the tie goes to the even neighbour
  }
  out = b;
  return true;
}

TS_HD uint64_t ts_add4_rn(uint64_t bs, uint64_t bd) {
  uint64_t out;
  if (ts_add4_fast(bs, bd, out)) return out;
  bs = ts_add_rn(bs, bd);
  bs = ts_add_rn(bs, bd);
  bs = ts_add_rn(bs, bd);
  return ts_add_rn(bs, bd);
}

// RN(s / n) for a double s >= 0 (zero or normal) and an integer 1 <= n < 2^20,
// in integer arithmetic: a 96-bit quotient from two 64-by-32 divisions,
// normalised to 53 bits plus guard bits and a sticky bit, rounded to nearest
// even.
TS_HD uint64_t ts_div_int_rn(uint64_t bs, uint32_t n) {
  if (bs == 0) return 0;
  const uint32_t e = (uint32_t)(bs >> 52);
  const uint64_t m = (bs & kFrac52) | (1ULL << 52);
  const uint64_t num = m << 11;  // [2^63, 2^64)
  const uint64_t q1 = num / n, r1 = num - q1 * n;
  const uint64_t n2 = r1 << 32;  // < 2^52
  const uint64_t q2 = n2 / n, r2 = n2 - q2 * n;
  // quotient Q = q1 * 2^32 + q2 (value = Q * 2^(e - 1118)), sticky = r2 != 0
  uint64_t hi = q1 >> 32, lo = (q1 << 32) | q2;
  bool sticky = r2 != 0;
  const uint32_t bl = hi ? 128u - clz64(hi) : 64u - clz64(lo);
  const uint32_t t = bl - 56;  // keep 56 bits: 53 + guard, round, sticky
  uint64_t z;
  if (t == 0) {
    z = lo;
  } else if (t < 64) {
    sticky = sticky || (lo & ((1ULL << t) - 1)) != 0;
    z = (lo >> t) | (hi << (64 - t));
  } else {
    sticky = sticky || lo != 0 || (hi & ((1ULL << (t - 64)) - 1)) != 0;
    z = hi >> (t - 64);
  }
  z |= sticky ? 1u : 0u;
  uint64_t mq = z >> 3;
  uint32_t ee = e - 40 + t;
  const uint32_t low = (uint32_t)(z & 7u);
  if (low > 4u || (low == 4u && (mq & 1u))) ++mq;
  if (mq >> 53) {
    mq >>= 1;
    ++ee;
  }
  return ((uint64_t)ee << 52) | (mq & kFrac52);
}

// ---------------------------------------------------------------------------
// Neighbour weight w = (f32) exp(-(d / mean)) without f64 arithmetic on the
// common path (GB300's f64 rate is a small fraction of its f32 rate).
//
// d and mean are the reference's exact doubles.  They are split into
// double-f32 pairs (48 significant bits), divided and exponentiated in
// double-f32 arithmetic (error-free transformations: two-sum, fused
// two-product), giving z ~ exp(-q) / 2^m within z * (2^-44 + q * 2^-45) of
// the value the exact f64 path produces.  The f32 result is returned only
// when z lies farther than err from every f32 rounding boundary; then
// rounding the exact f64 value gives the same f32.
// Otherwise (about one weight in 2^14) the caller falls back to the exact f64
// path (ts_div_markstein + ts_exp64).  The bound err = 2^-40 + q 2^-42 is at
// least four times the error above.  q > 80, NaN and operands outside the
// normal f32 exponent range always fall back.
// ---------------------------------------------------------------------------
#define TS_EXP2_FF_TABLE_VALUES \
  0x1.0000000000000p+0f, 0x0.0p+0f, 0x1.02c9a40000000p+0f, -0x1.887fa00000000p-28f, \
  0x1.059b0e0000000p+0f, -0x1.9d4f520000000p-25f, 0x1.0874520000000p+0f, -0x1.e2990e0000000p-26f, \
  0x1.0b55860000000p+0f, 0x1.9f31220000000p-25f, 0x1.0e3ec40000000p+0f, -0x1.a585cc0000000p-25f, \
  0x1.11301e0000000p+0f, -0x1.fdb4960000000p-25f, 0x1.1429aa0000000p+0f, 0x1.d525bc0000000p-25f, \
  0x1.172b840000000p+0f, -0x1.c157420000000p-27f, 0x1.1a35be0000000p+0f, 0x1.6df96e0000000p-25f, \
  0x1.1d48740000000p+0f, -0x1.d2e8ca0000000p-25f, 0x1.2063b80000000p+0f, 0x1.0c519a0000000p-25f, \
  0x1.2387a60000000p+0f, 0x1.ceac480000000p-25f, 0x1.26b4560000000p+0f, 0x1.789f380000000p-26f, \
  0x1.29e9e00000000p+0f, -0x1.5c04240000000p-25f, 0x1.2d285a0000000p+0f, 0x1.b900c20000000p-26f, \
  0x1.306fe00000000p+0f, 0x1.4636e20000000p-25f, 0x1.33c08c0000000p+0f, -0x1.b37d200000000p-25f, \
  0x1.371a740000000p+0f, -0x1.18aac60000000p-25f, 0x1.3a7db40000000p+0f, -0x1.634c020000000p-25f, \
  0x1.3dea640000000p+0f, 0x1.8246840000000p-25f, 0x1.4160a20000000p+0f, 0x1.f72e2a0000000p-28f, \
  0x1.44e0860000000p+0f, 0x1.8624b40000000p-30f, 0x1.486a2c0000000p+0f, -0x1.47d8660000000p-25f, \
  0x1.4bfdae0000000p+0f, -0x1.593abc0000000p-25f, 0x1.4f9b280000000p+0f, -0x1.2c5a6c0000000p-25f, \
  0x1.5342b60000000p+0f, -0x1.2c56100000000p-25f, 0x1.56f4740000000p+0f, -0x1.295b040000000p-25f, \
  0x1.5ab07e0000000p+0f, -0x1.5bd5ec0000000p-27f, 0x1.5e76f20000000p+0f, -0x1.4a5bd60000000p-25f, \
  0x1.6247ec0000000p+0f, -0x1.f8b5500000000p-25f, 0x1.6623880000000p+0f, 0x1.2a91120000000p-27f, \
  0x1.6a09e60000000p+0f, 0x1.9fcef40000000p-26f, 0x1.6dfb240000000p+0f, -0x1.cd72e80000000p-27f, \
  0x1.71f75e0000000p+0f, 0x1.1d8bee0000000p-25f, 0x1.75feb60000000p+0f, -0x1.37b3060000000p-25f, \
  0x1.7a11480000000p+0f, -0x1.829fd00000000p-25f, 0x1.7e2f340000000p+0f, -0x1.2616340000000p-25f, \
  0x1.82589a0000000p+0f, -0x1.accc7c0000000p-26f, 0x1.868d9a0000000p+0f, -0x1.2edb440000000p-26f, \
  0x1.8ace540000000p+0f, 0x1.15506e0000000p-27f, 0x1.8f1aea0000000p+0f, -0x1.baa2320000000p-26f, \
  0x1.93737c0000000p+0f, -0x1.e647440000000p-25f, 0x1.97d82a0000000p+0f, -0x1.0d8d840000000p-31f, \
  0x1.9c49180000000p+0f, 0x1.51f8480000000p-27f, 0x1.a0c6680000000p+0f, -0x1.2886a60000000p-26f, \
  0x1.a5503c0000000p+0f, -0x1.b83b540000000p-25f, 0x1.a9e6b60000000p+0f, -0x1.50c0480000000p-25f, \
  0x1.ae89fa0000000p+0f, -0x1.a94b140000000p-26f, 0x1.b33a2c0000000p+0f, -0x1.ec3a820000000p-26f, \
  0x1.b7f7700000000p+0f, -0x1.a094380000000p-25f, 0x1.bcc1ea0000000p+0f, -0x1.f687c60000000p-25f, \
  0x1.c199be0000000p+0f, -0x1.3d56b20000000p-27f, 0x1.c67f120000000p+0f, 0x1.cafa2a0000000p-25f, \
  0x1.cb720e0000000p+0f, -0x1.8837cc0000000p-27f, 0x1.d072d40000000p+0f, 0x1.40f1300000000p-25f, \
  0x1.d5818e0000000p+0f, -0x1.822dbc0000000p-27f, 0x1.da9e600000000p+0f, 0x1.ed99420000000p-27f, \
  0x1.dfc9740000000p+0f, -0x1.908c940000000p-25f, 0x1.e502ee0000000p+0f, 0x1.e2cffe0000000p-26f, \
  0x1.ea4afa0000000p+0f, 0x1.52486c0000000p-27f, 0x1.efa1be0000000p+0f, 0x1.cc2b440000000p-25f, \
  0x1.f507660000000p+0f, -0x1.246eb00000000p-26f, 0x1.fa7c180000000p+0f, 0x1.9e90d80000000p-28f,

#ifdef __CUDA_ARCH__
#define TS_FADD(a, b) __fadd_rn(a, b)
#define TS_FSUB(a, b) __fsub_rn(a, b)
#define TS_FMUL(a, b) __fmul_rn(a, b)
#define TS_FFMA(a, b, c) __fmaf_rn(a, b, c)
#define TS_FDIV(a, b) __fdiv_rn(a, b)
#else
#define TS_FADD(a, b) ((a) + (b))
#define TS_FSUB(a, b) ((a) - (b))
#define TS_FMUL(a, b) ((a) * (b))
#define TS_FFMA(a, b, c) fmaf(a, b, c)
#define TS_FDIV(a, b) ((a) / (b))
#endif

TS_HD void ff_two_sum(float a, float b, float &s, float &e) {
  s = TS_FADD(a, b);
  const float bb = TS_FSUB(s, a);
  e = TS_FADD(TS_FSUB(a, TS_FSUB(s, bb)), TS_FSUB(b, bb));
}
TS_HD void ff_fast_two_sum(float a, float b, float &s, float &e) {  // |a| >= |b|
  s = TS_FADD(a, b);
  e = TS_FSUB(b, TS_FSUB(s, a));
}

// v > 0 with unbiased exponent in [-74, 127]: v ~ hi + lo to 2^-48 relative.
TS_HD bool ff_split(double v, float &hi, float &lo) {
  const uint64_t b = dbl_bits(v);
  const int32_t e = (int32_t)((b >> 52) & 0x7ffu) - 1023;
  if ((b >> 63) || e < -74 || e > 127) return false;
  const uint64_t m = (b & 0xFFFFFFFFFFFFFULL) | (1ULL << 52);
  hi = bits_flt(((uint32_t)(e + 127) << 23) | ((uint32_t)(m >> 29) & 0x7FFFFFu));
  const uint32_t ml = (uint32_t)(m & ((1u << 29) - 1u));
  lo = TS_FMUL((float)ml, bits_flt((uint32_t)(e - 52 + 127) << 23));
  return true;
}

TS_HD bool ts_weight_ff(double d, double mean, const float *tab_ff, float &w) {
  float q_hi, q_lo, a_hi, a_lo;
  // a zero or tiny mean (all distances 0 gives 0/0 = NaN) takes the exact path
  if (!ff_split(mean, a_hi, a_lo)) return false;
  if (dbl_bits(d) == 0) {
    q_hi = 0.0f;
    q_lo = 0.0f;
  } else {
    float d_hi, d_lo;
    if (!ff_split(d, d_hi, d_lo)) return false;
    const float q1 = TS_FDIV(d_hi, a_hi);
    const float p = TS_FMUL(q1, a_hi);
    const float pe = TS_FFMA(q1, a_hi, -p);
    float r = TS_FSUB(d_hi, p);
    r = TS_FSUB(TS_FSUB(TS_FADD(r, d_lo), pe), TS_FMUL(q1, a_lo));
    const float q2 = TS_FDIV(r, a_hi);
    ff_fast_two_sum(q1, q2, q_hi, q_lo);
  }
  if (!(q_hi >= 0.0f && q_hi <= 80.0f)) return false;
  const float x_hi = -q_hi, x_lo = -q_lo;
  const float ff_inv = 0x1.7154760000000p+6f, c1 = 0x1.6300000000000p-7f, c2 = -0x1.bd01060000000p-19f, c3 = 0x1.cf79ac0000000p-46f;
  const float kf = rintf(TS_FMUL(x_hi, ff_inv));
  const float t = TS_FFMA(-kf, c1, x_hi);
  const float p2 = TS_FMUL(kf, c2);
  const float e2 = TS_FFMA(kf, c2, -p2);
  float s, se;
  ff_two_sum(t, -p2, s, se);
  const float rl = TS_FSUB(TS_FSUB(TS_FADD(se, x_lo), e2), TS_FMUL(kf, c3));
  float r_hi, r_lo;
  ff_two_sum(s, rl, r_hi, r_lo);
  // e^r = 1 + r + r^2/2 + r^3/6 + r^4/24 + r^5/120, |r| <= ln2/128
  const float pp = TS_FMUL(r_hi, r_hi);
  const float ppe = TS_FFMA(r_hi, r_hi, -pp);
  const float h2 = TS_FMUL(pp, 0.5f);
  const float l2 = TS_FADD(TS_FMUL(ppe, 0.5f), TS_FMUL(r_hi, r_lo));
  const float t3 = TS_FMUL(TS_FMUL(r_hi, pp),
                           TS_FFMA(r_hi, TS_FFMA(r_hi, 1.0f / 120.0f, 1.0f / 24.0f), 1.0f / 6.0f));
  float u_hi, u_lo, b_hi, b_lo;
  ff_two_sum(1.0f, r_hi, u_hi, u_lo);
  ff_two_sum(u_hi, h2, b_hi, b_lo);
  const float lo = TS_FADD(TS_FADD(TS_FADD(TS_FADD(t3, l2), r_lo), b_lo), u_lo);
  float y_hi, y_lo;
  ff_fast_two_sum(b_hi, lo, y_hi, y_lo);
  const int32_t ki = (int32_t)kf;
  const float th = tab_ff[2 * (ki & 63)], tl = tab_ff[2 * (ki & 63) + 1];
  const float zp = TS_FMUL(y_hi, th);
  float ze = TS_FFMA(y_hi, th, -zp);
  ze = TS_FADD(ze, TS_FADD(TS_FMUL(y_hi, tl), TS_FMUL(y_lo, th)));
  float z_hi, z_lo;
  ff_fast_two_sum(zp, ze, z_hi, z_lo);
  // f32 rounding of z and its distance to the rounding boundaries
  const float f = TS_FADD(z_hi, z_lo);
  const float dlt = TS_FADD(TS_FSUB(z_hi, f), z_lo);
  const uint32_t fb = flt_bits(f);
  const float ulp = bits_flt(((fb >> 23) - 23u) << 23);
  const float half_up = TS_FMUL(ulp, 0.5f);
  const float half_dn = (fb & 0x7FFFFFu) == 0 ? TS_FMUL(ulp, 0.25f) : half_up;
  const float margin = dlt >= 0.0f ? TS_FSUB(half_up, dlt) : TS_FADD(half_dn, dlt);
  const float err = TS_FFMA(q_hi, 0x1p-42f, 0x1p-40f);
  if (!(margin > err)) return false;
  const int32_t m = ki >> 6;  // w = f * 2^m, normal for q <= 80
  w = TS_FMUL(f, bits_flt((uint32_t)(m + 127) << 23));
  return true;
}

// units * 2^qe as the bits of a double, exactly (units < 2^53, normal
// result): the neighbour distances and their sums of outputs whose sides
// are powers of two, without f64 arithmetic.
TS_HD uint64_t ts_units_bits(uint64_t units, int32_t qe) {
  if (units == 0) return 0;
  const int32_t p = 63 - (int32_t)clz64(units);
  const uint64_t m = units << (52 - p);
  return ((uint64_t)(uint32_t)(p + 1023 + qe) << 52) | (m & kFrac52);
}

#undef TS_FADD
#undef TS_FSUB
#undef TS_FMUL
#undef TS_FFMA
#undef TS_FDIV

}  // namespace ts
