/*
 * ms_oracle.c — CPU oracle for the texture-synthesis hot loop.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links, loads or calls
 * this file: it is built into oracle/_build/libtsoracle.so and used by the
 * parity tests, by __graft_entry__.smoke() as the checker, and by bench.py's
 * CPU-baseline leg.
 *
 * It restates, in plain C, the reference's multiresolution stochastic
 * synthesis (EmbarkStudios/texture-synthesis, Rust):
 *   lib/src/ms.rs          Generator::{new,new_from_inpaint,update,flush_resolved,
 *                          pick_random_unresolved,resolve_random_batch,
 *                          resolve_at_random,find_candidates,next_pyramid_level,
 *                          resolve}, better_match, find_best_match,
 *                          metric_cauchy, metric_l2, check_coord_validity
 *   lib/src/img_pyramid.rs ImagePyramid::build_gaussian
 *   lib/src/session.rs     Session::run (random init then resolve)
 * and, because the reference delegates to them, the published algorithms of
 * three third-party crates pinned in its Cargo.lock but absent here:
 *   rand_core 0.6.3  SeedableRng::seed_from_u64 (PCG32 seed expansion)
 *   rand_pcg 0.3.1   Lcg64Xsh32 (PCG XSH RR 64/32)
 *   rand 0.8.5       UniformInt::sample_single (Rng::gen_range, widening multiply)
 *   image 0.23.12    imageops::resize (separable filter, f32 intermediate,
 *                    round-to-nearest u8 output)
 *   rstar 0.7.1      nearest_neighbor_iter: replaced by an exact k-NN with the
 *                    tie rule stated below (rstar's order among equal
 *                    distances is tree-shape dependent and not reproducible).
 *
 * PARITY UNPINNED: the reference cannot be compiled here (no Rust toolchain,
 * no crates), and its own tests (lib/tests/diff.rs) compare 8x8 perceptual
 * hashes of JPEG-decoded photos, which need the absent `image` and `img_hash`
 * crates.  This oracle is therefore a restatement checked only by its own
 * properties and by the GPU path agreeing with it.
 *
 * Two semantics are stated here and shared with the GPU path:
 *  (1) k-NN tie rule: neighbours are ordered by (squared distance, y, x)
 *      ascending, x and y being the point's coordinates in the output plane
 *      (tiling mirrors may lie outside [0,W)x[0,H)).  The reference sorts
 *      rstar's output stably by squared distance (ms.rs:1523).
 *  (2) Batch-snapshot schedule: the items of a stage are processed in
 *      batches; every item of a batch reads the state as it was when the
 *      batch started, then the batch commits in item order.  A batch holds
 *      max(1, R / batch_divisor) items (R = resolved-list length at batch
 *      start), capped at max_batch when max_batch > 0.  batch_divisor = 0
 *      means batches of one item, which is the reference's
 *      max_thread_count(1) semantics.
 *
 * All float arithmetic is compiled with -ffp-contract=off: the reference's
 * Rust code never fuses a multiply and an add except where it calls mul_add.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/tsgpu.h" /* TS_MAX_SAMPLE_DRAWS, the one bound shared with the GPU path */

#define TSO_OK 0
#define TSO_ERR_ARG 1
#define TSO_ERR_NO_VALID_SAMPLE 2
#define TSO_ERR_INDEX 3
#define TSO_ERR_ALLOC 4

/* ------------------------------------------------------------------------ */
/* PCG32 as used through rand_pcg 0.3.1 / rand_core 0.6.3 / rand 0.8.5.      */
/* ------------------------------------------------------------------------ */
#define PCG_MUL 6364136223846793005ULL
#define PCG_SEED_INC 11634580027462260723ULL

typedef struct {
  uint64_t state, inc;
} pcg32;

/* XSH RR output permutation of the published PCG family (O'Neill 2014). */
static inline uint32_t pcg_out(uint64_t s) {
  uint32_t xs = (uint32_t)(((s >> 18) ^ s) >> 27);
  uint32_t rot = (uint32_t)(s >> 59);
  return (xs >> rot) | (xs << ((32u - rot) & 31u));
}

/* rand_core SeedableRng::seed_from_u64: a PCG32 stream with a fixed increment
 * advances first and emits four u32 words (little endian) that form the
 * 16-byte seed; Lcg64Xsh32::from_seed reads state = bytes[0..8],
 * increment = bytes[8..16] | 1, adds the increment and steps once. */
static pcg32 pcg_seed_from_u64(uint64_t x) {
  uint32_t w[4];
  for (int c = 0; c < 4; c++) {
    x = x * PCG_MUL + PCG_SEED_INC;
    w[c] = pcg_out(x);
  }
  pcg32 r;
  r.state = (uint64_t)w[0] | ((uint64_t)w[1] << 32);
  r.inc = ((uint64_t)w[2] | ((uint64_t)w[3] << 32)) | 1ULL;
  r.state = r.state + r.inc;
  r.state = r.state * PCG_MUL + r.inc;
  return r;
}

static inline uint32_t pcg_next_u32(pcg32 *r) {
  uint64_t s = r->state;
  r->state = s * PCG_MUL + r->inc;
  return pcg_out(s);
}

/* rand_core impls::next_u64_via_u32: low word first. */
static inline uint64_t pcg_next_u64(pcg32 *r) {
  uint64_t lo = pcg_next_u32(r);
  uint64_t hi = pcg_next_u32(r);
  return (hi << 32) | lo;
}

/* rand 0.8.5 UniformInt<u32>::sample_single(0, n): widening multiply with the
 * "conservative" rejection zone (range << leading_zeros(range)) - 1. */
static inline uint32_t gen_range_u32(pcg32 *r, uint32_t n) {
  uint32_t zone = (n << __builtin_clz(n)) - 1u;
  for (;;) {
    uint32_t v = pcg_next_u32(r);
    uint64_t m = (uint64_t)v * (uint64_t)n;
    if ((uint32_t)m <= zone) return (uint32_t)(m >> 32);
  }
}

/* Same for usize (64-bit targets): u64 draws, 128-bit product. */
static inline uint64_t gen_range_u64(pcg32 *r, uint64_t n) {
  uint64_t zone = (n << __builtin_clzll(n)) - 1u;
  for (;;) {
    uint64_t v = pcg_next_u64(r);
    unsigned __int128 m = (unsigned __int128)v * (unsigned __int128)n;
    if ((uint64_t)m <= zone) return (uint64_t)(m >> 64);
  }
}

/* Exported for the RNG unit tests. */
void tso_pcg_seed(uint64_t seed, uint64_t *state, uint64_t *inc) {
  pcg32 r = pcg_seed_from_u64(seed);
  *state = r.state;
  *inc = r.inc;
}
void tso_pcg_stream(uint64_t seed, uint32_t n, uint32_t *out) {
  pcg32 r = pcg_seed_from_u64(seed);
  for (uint32_t i = 0; i < n; i++) out[i] = pcg_next_u32(&r);
}
uint32_t tso_gen_range_u32(uint64_t seed, uint32_t n) {
  pcg32 r = pcg_seed_from_u64(seed);
  return gen_range_u32(&r, n);
}
uint64_t tso_gen_range_u64(uint64_t seed, uint64_t n) {
  pcg32 r = pcg_seed_from_u64(seed);
  return gen_range_u64(&r, n);
}

/* ------------------------------------------------------------------------ */
/* exp for the neighbour weights (ms.rs:1198-1203 calls f64::exp).           */
/* Table driven: x = (64 m + j) ln2/64 + r, |r| <= ln2/128 (Cody & Waite      */
/* reduction, ln2/64 split in a high part with zero trailing bits and a low  */
/* part), the Taylor series of e^r to degree 5 by Horner's rule with fused   */
/* multiply-adds, times 2^(j/64) (nearest doubles) and 2^m.  The GPU path     */
/* evaluates the identical operation sequence, so both sides produce the     */
/* same double, within a few ulp of the true exponential; the weights are    */
/* rounded to f32 afterwards.                                                */
/* ------------------------------------------------------------------------ */
static const double exp2_64[64] = {
  0x1.0000000000000p+0, 0x1.02c9a3e778061p+0,
  0x1.059b0d3158574p+0, 0x1.0874518759bc8p+0,
  0x1.0b5586cf9890fp+0, 0x1.0e3ec32d3d1a2p+0,
  0x1.11301d0125b51p+0, 0x1.1429aaea92de0p+0,
  0x1.172b83c7d517bp+0, 0x1.1a35beb6fcb75p+0,
  0x1.1d4873168b9aap+0, 0x1.2063b88628cd6p+0,
  0x1.2387a6e756238p+0, 0x1.26b4565e27cddp+0,
  0x1.29e9df51fdee1p+0, 0x1.2d285a6e4030bp+0,
  0x1.306fe0a31b715p+0, 0x1.33c08b26416ffp+0,
  0x1.371a7373aa9cbp+0, 0x1.3a7db34e59ff7p+0,
  0x1.3dea64c123422p+0, 0x1.4160a21f72e2ap+0,
  0x1.44e086061892dp+0, 0x1.486a2b5c13cd0p+0,
  0x1.4bfdad5362a27p+0, 0x1.4f9b2769d2ca7p+0,
  0x1.5342b569d4f82p+0, 0x1.56f4736b527dap+0,
  0x1.5ab07dd485429p+0, 0x1.5e76f15ad2148p+0,
  0x1.6247eb03a5585p+0, 0x1.6623882552225p+0,
  0x1.6a09e667f3bcdp+0, 0x1.6dfb23c651a2fp+0,
  0x1.71f75e8ec5f74p+0, 0x1.75feb564267c9p+0,
  0x1.7a11473eb0187p+0, 0x1.7e2f336cf4e62p+0,
  0x1.82589994cce13p+0, 0x1.868d99b4492edp+0,
  0x1.8ace5422aa0dbp+0, 0x1.8f1ae99157736p+0,
  0x1.93737b0cdc5e5p+0, 0x1.97d829fde4e50p+0,
  0x1.9c49182a3f090p+0, 0x1.a0c667b5de565p+0,
  0x1.a5503b23e255dp+0, 0x1.a9e6b5579fdbfp+0,
  0x1.ae89f995ad3adp+0, 0x1.b33a2b84f15fbp+0,
  0x1.b7f76f2fb5e47p+0, 0x1.bcc1e904bc1d2p+0,
  0x1.c199bdd85529cp+0, 0x1.c67f12e57d14bp+0,
  0x1.cb720dcef9069p+0, 0x1.d072d4a07897cp+0,
  0x1.d5818dcfba487p+0, 0x1.da9e603db3285p+0,
  0x1.dfc97337b9b5fp+0, 0x1.e502ee78b3ff6p+0,
  0x1.ea4afa2a490dap+0, 0x1.efa1bee615a27p+0,
  0x1.f50765b6e4540p+0, 0x1.fa7c1819e90d8p+0,
};

static double tso_exp(double x) {
  if (x != x) return x;
  if (x < -700.0) return 0.0; /* far below the smallest f32 after rounding */
  if (x > 700.0) return INFINITY;
  const double inv_step = 0x1.71547652b82fep+6;
  const double step_hi = 0x1.62e42fee00000p-7;
  const double step_lo = 0x1.a39ef35793c76p-39;
  double k = rint(x * inv_step);
  double r = fma(-k, step_hi, x);
  r = fma(-k, step_lo, r);
  double p = 1.0 / 120.0;
  p = fma(p, r, 1.0 / 24.0);
  p = fma(p, r, 1.0 / 6.0);
  p = fma(p, r, 0.5);
  p = fma(p, r, 1.0);
  p = fma(p, r, 1.0);
  int ki = (int)k;
  return ldexp(exp2_64[ki & 63] * p, ki >> 6);
}
double tso_exp_export(double x) { return tso_exp(x); }

/* Audit of tso_exp against the C library's exp, which the reference calls
 * (f64::exp, ms.rs:1198-1203): while on, every weight a run computes is
 * also computed with exp(), and the inputs whose f32 weights differ are
 * counted.  Test instrumentation; off by default. */
static int g_exp_audit;
static uint64_t g_exp_audit_n, g_exp_audit_diff;
void tso_exp_audit(int on) {
  g_exp_audit = on;
  __atomic_store_n(&g_exp_audit_n, 0, __ATOMIC_SEQ_CST);
  __atomic_store_n(&g_exp_audit_diff, 0, __ATOMIC_SEQ_CST);
}
void tso_exp_audit_counts(uint64_t *n, uint64_t *diff) {
  *n = __atomic_load_n(&g_exp_audit_n, __ATOMIC_SEQ_CST);
  *diff = __atomic_load_n(&g_exp_audit_diff, __ATOMIC_SEQ_CST);
}

/* ------------------------------------------------------------------------ */
/* image 0.23.12 imageops::resize restated (img_pyramid.rs:27-32 calls it     */
/* with FilterType::Gaussian; utils.rs:67-72 with CatmullRom).                */
/* ------------------------------------------------------------------------ */
enum { TSO_FILTER_NEAREST = 0, TSO_FILTER_TRIANGLE = 1, TSO_FILTER_CATMULLROM = 2, TSO_FILTER_GAUSSIAN = 3, TSO_FILTER_BLUR = 4 };

/* imageops::blur's kernel: gaussian(x, sigma) = 1/(sqrt(2 pi) sigma) *
 * exp(-x^2 / (2 sigma^2)), support 2 sigma */
static float k_gauss_sigma(float x, float r) {
  float a = 1.0f / (sqrtf(2.0f * 3.14159265358979323846f) * r);
  float b = expf(-(x * x) / (2.0f * (r * r)));
  return a * b;
}

static float k_gauss(float x) {
  /* gaussian(x, r = 0.5) = 1/(sqrt(2 pi) r) * exp(-x^2 / (2 r^2)) */
  const float r = 0.5f;
  float a = 1.0f / (sqrtf(2.0f * 3.14159265358979323846f) * r);
  float b = expf(-(x * x) / (2.0f * (r * r)));
  return a * b;
}
static float k_triangle(float x) {
  float a = fabsf(x);
  return a < 1.0f ? 1.0f - a : 0.0f;
}
static float k_catmullrom(float x) {
  /* cubic_bc(b = 0, c = 0.5, x) */
  const float b = 0.0f, c = 0.5f;
  float a = fabsf(x), k;
  if (a < 1.0f) {
    k = (12.0f - 9.0f * b - 6.0f * c) * (a * a * a) + (-18.0f + 12.0f * b + 6.0f * c) * (a * a) +
        (6.0f - 2.0f * b);
  } else if (a < 2.0f) {
    k = (-b - 6.0f * c) * (a * a * a) + (6.0f * b + 30.0f * c) * (a * a) + (-12.0f * b - 48.0f * c) * a +
        (8.0f * b + 24.0f * c);
  } else {
    k = 0.0f;
  }
  return k / 6.0f;
}
static float k_box(float x) { return (x >= -0.5f && x < 0.5f) ? 1.0f : 0.0f; }

static float filt_eval(int f, float x, float sigma) {
  switch (f) {
    case TSO_FILTER_BLUR: return k_gauss_sigma(x, sigma);
    case TSO_FILTER_TRIANGLE: return k_triangle(x);
    case TSO_FILTER_CATMULLROM: return k_catmullrom(x);
    case TSO_FILTER_GAUSSIAN: return k_gauss(x);
    default: return k_box(x);
  }
}
static float filt_support(int f, float sigma) {
  switch (f) {
    case TSO_FILTER_BLUR: return 2.0f * sigma;
    case TSO_FILTER_TRIANGLE: return 1.0f;
    case TSO_FILTER_CATMULLROM: return 2.0f;
    case TSO_FILTER_GAUSSIAN: return 3.0f;
    default: return 0.0f;
  }
}

static int64_t clamp_i64(int64_t a, int64_t lo, int64_t hi) {
  if (a < lo) return lo;
  if (a > hi) return hi;
  return a;
}

/* Taps of one output index along an axis: [left, right) and normalised
 * weights.  Returns the tap count; writes at most cap weights. */
static int axis_taps(int f, float sigma, uint32_t in_len, uint32_t out_len, uint32_t o, uint32_t *left_out,
                     float *ws, int cap) {
  float ratio = (float)in_len / (float)out_len;
  float sratio = ratio < 1.0f ? 1.0f : ratio;
  float src_support = filt_support(f, sigma) * sratio;
  float c = ((float)o + 0.5f) * ratio;
  int64_t left = (int64_t)floorf(c - src_support);
  left = clamp_i64(left, 0, (int64_t)in_len - 1);
  int64_t right = (int64_t)ceilf(c + src_support);
  right = clamp_i64(right, left + 1, (int64_t)in_len);
  c = c - 0.5f;
  int n = 0;
  float sum = 0.0f;
  for (int64_t i = left; i < right; i++) {
    float w = filt_eval(f, ((float)i - c) / sratio, sigma);
    if (n < cap) ws[n] = w;
    n++;
    sum += w;
  }
  for (int i = 0; i < n && i < cap; i++) ws[i] /= sum;
  *left_out = (uint32_t)left;
  return n;
}

/* Resize an RGBA8 image: vertical pass into an f32 image, then horizontal
 * pass with clamping to [0,255] and rounding half away from zero. */
static int resize_sigma(const uint8_t *src, uint32_t w, uint32_t h, uint8_t *dst, uint32_t nw, uint32_t nh, int filter,
                        float sigma) {
  if (nw == 0 || nh == 0) return TSO_OK;
  float *tmp = (float *)calloc((size_t)w * nh * 4 + 4, sizeof(float));
  float rv = nh ? (float)h / (float)nh : 1.0f, rh = nw ? (float)w / (float)nw : 1.0f;
  float rmax = rv > rh ? rv : rh;
  if (rmax < 1.0f) rmax = 1.0f;
  int cap = (int)(2.0f * filt_support(filter, sigma) * rmax) + 16;
  float *ws = (float *)malloc(sizeof(float) * cap);
  if (!tmp || !ws) {
    free(tmp);
    free(ws);
    return TSO_ERR_ALLOC;
  }
  /* vertical_sample(image, nh) */
  if (h > 0) {
    for (uint32_t oy = 0; oy < nh; oy++) {
      uint32_t left;
      int n = axis_taps(filter, sigma, h, nh, oy, &left, ws, cap);
      if (n > cap) {
        free(tmp);
        free(ws);
        return TSO_ERR_ARG;
      }
      for (uint32_t x = 0; x < w; x++) {
        float t0 = 0.0f, t1 = 0.0f, t2 = 0.0f, t3 = 0.0f;
        for (int i = 0; i < n; i++) {
          const uint8_t *p = src + (((size_t)(left + i) * w + x) * 4);
          float wt = ws[i];
          t0 += (float)p[0] * wt;
          t1 += (float)p[1] * wt;
          t2 += (float)p[2] * wt;
          t3 += (float)p[3] * wt;
        }
        float *q = tmp + ((size_t)oy * w + x) * 4;
        q[0] = t0;
        q[1] = t1;
        q[2] = t2;
        q[3] = t3;
      }
    }
  }
  /* horizontal_sample(tmp, nw) */
  for (uint32_t ox = 0; ox < nw; ox++) {
    uint32_t left = 0;
    int n = 0;
    if (w > 0) {
      n = axis_taps(filter, sigma, w, nw, ox, &left, ws, cap);
      if (n > cap) {
        free(tmp);
        free(ws);
        return TSO_ERR_ARG;
      }
    }
    for (uint32_t y = 0; y < nh; y++) {
      float t[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      for (int i = 0; i < n; i++) {
        const float *p = tmp + ((size_t)y * w + (left + i)) * 4;
        float wt = ws[i];
        t[0] += p[0] * wt;
        t[1] += p[1] * wt;
        t[2] += p[2] * wt;
        t[3] += p[3] * wt;
      }
      uint8_t *q = dst + ((size_t)y * nw + ox) * 4;
      for (int c = 0; c < 4; c++) {
        float v = t[c];
        if (v < 0.0f) v = 0.0f;
        if (v > 255.0f) v = 255.0f;
        q[c] = (uint8_t)roundf(v);
      }
    }
  }
  free(tmp);
  free(ws);
  return TSO_OK;
}

int tso_resize(const uint8_t *src, uint32_t w, uint32_t h, uint8_t *dst, uint32_t nw, uint32_t nh, int filter) {
  return resize_sigma(src, w, h, dst, nw, nh, filter, 0.0f);
}

/* transform_to_guide_map + match_histograms (utils.rs:101-183, used by
 * lib.rs:575-582 for examples without a guide when a target guide is set):
 * imageops::blur (sigma 2: the resize passes at the same size with the
 * kernel above), DynamicImage::grayscale (image 0.23 rgb_to_luma: 0.2126 R +
 * 0.7152 G + 0.0722 B in f32, left to right, truncated to u8), then the
 * histogram of that luma matched to channel 0 of the target guide:
 * f32 cumulative distributions normalised by their last entry, and
 * v -> (first index whose target cdf exceeds cdf_src[v], else v + 1 in u8)
 * as u8 minus 1, both in wrapping u8 arithmetic (the reference's release
 * build).  The transform's own resize discards its result (utils.rs:110-114)
 * and is left out.  out: (n, n, n, 255) per texel. */
int tso_guide_map(const uint8_t *src, uint32_t w, uint32_t h, const uint8_t *target, uint32_t tw, uint32_t th,
                  uint8_t *out) {
  size_t n = (size_t)w * h;
  uint8_t *blur = (uint8_t *)malloc(n * 4 + 4);
  uint8_t *luma = (uint8_t *)malloc(n + 1);
  if (!blur || !luma) {
    free(blur);
    free(luma);
    return TSO_ERR_ALLOC;
  }
  int rc = resize_sigma(src, w, h, blur, w, h, TSO_FILTER_BLUR, 2.0f);
  if (rc != TSO_OK) {
    free(blur);
    free(luma);
    return rc;
  }
  uint32_t hs[256] = {0}, ht[256] = {0};
  for (size_t i = 0; i < n; i++) {
    const uint8_t *p = blur + 4 * i;
    float l = 0.2126f * (float)p[0];
    l = l + 0.7152f * (float)p[1];
    l = l + 0.0722f * (float)p[2];
    luma[i] = (uint8_t)l;
    hs[luma[i]]++;
  }
  for (size_t i = 0; i < (size_t)tw * th; i++) ht[target[4 * i]]++;
  float cs[256], ct[256];
  cs[0] = (float)hs[0];
  ct[0] = (float)ht[0];
  for (int i = 1; i < 256; i++) {
    cs[i] = cs[i - 1] + (float)hs[i];
    ct[i] = ct[i - 1] + (float)ht[i];
  }
  float ms = cs[255], mt = ct[255];
  for (int i = 0; i < 256; i++) {
    cs[i] /= ms;
    ct[i] /= mt;
  }
  uint8_t map[256];
  for (int v = 0; v < 256; v++) {
    int pos = -1;
    for (int i = 0; i < 256; i++)
      if (ct[i] > cs[v]) {
        pos = i;
        break;
      }
    uint32_t idx = pos >= 0 ? (uint32_t)pos : (uint32_t)(uint8_t)(v + 1);
    map[v] = (uint8_t)((uint8_t)idx - 1u);
  }
  for (size_t i = 0; i < n; i++) {
    uint8_t v = map[luma[i]];
    out[4 * i] = out[4 * i + 1] = out[4 * i + 2] = v;
    out[4 * i + 3] = 255;
  }
  free(blur);
  free(luma);
  return TSO_OK;
}

/* ImagePyramid::build_gaussian (img_pyramid.rs:20-37): level i of `levels`
 * is resize(resize(img, w/2^(levels-1-i), h/...), w, h), the last level is the
 * image itself.  out holds max(levels,1) images of w*h*4 bytes. */
int tso_pyramid(const uint8_t *img, uint32_t w, uint32_t h, uint32_t levels, uint8_t *out) {
  size_t sz = (size_t)w * h * 4;
  uint32_t nl = levels == 0 ? 1 : levels;
  for (uint32_t l = 0; l + 1 < nl; l++) {
    uint32_t i = nl - 1 - l; /* 2^i downscale */
    uint32_t p = 1u << i;
    uint32_t sw = w / p, sh = h / p;
    uint8_t *small = (uint8_t *)calloc((size_t)sw * sh * 4 + 4, 1);
    if (!small) return TSO_ERR_ALLOC;
    int rc = tso_resize(img, w, h, small, sw, sh, TSO_FILTER_GAUSSIAN);
    if (rc == TSO_OK) rc = tso_resize(small, sw, sh, out + (size_t)l * sz, w, h, TSO_FILTER_GAUSSIAN);
    free(small);
    if (rc) return rc;
  }
  memcpy(out + (size_t)(nl - 1) * sz, img, sz);
  return TSO_OK;
}

/* ------------------------------------------------------------------------ */
/* Session inputs.                                                           */
/* ------------------------------------------------------------------------ */
typedef struct {
  const uint8_t *rgba; /* w*h*4 */
  uint32_t w, h;
  const uint8_t *guide; /* NULL, or gw*gh*4: the example's guide map */
  uint32_t gw, gh;
  int32_t sample_method; /* 0 All, 1 Ignore, 2 Image */
  const uint8_t *mask;   /* w*h*4 when sample_method == 2 */
} tso_example;

typedef struct {
  uint32_t k;           /* nearest_neighbors */
  uint32_t pad0;
  uint64_t m;           /* random_sample_locations */
  float cauchy;         /* cauchy_dispersion */
  float p;              /* backtrack_percent */
  uint32_t stages;      /* backtrack_stages */
  uint32_t pad1;
  uint64_t seed;
  float alpha;          /* guide_alpha */
  int32_t tiling;
  int32_t has_random_init;
  uint32_t pad2;
  uint64_t random_init;
  uint32_t out_w, out_h;
  uint32_t batch_divisor;
  uint32_t max_batch;
  int32_t nthreads;
  uint32_t pad3;
} tso_params;

typedef struct {
  uint64_t evals;       /* candidate-cost evaluations (candidates scored) */
  uint64_t resolves;    /* items processed in the stage loop */
  uint64_t batches;     /* batch steps */
  uint64_t n_resolved;  /* final resolved-list length */
} tso_stats;

/* Per-map level image: packed RGBA (byte 0 = R). */
typedef struct {
  uint32_t w, h;
  const uint32_t *px;
} img_t;

typedef struct {
  int32_t x, y;
  int64_t d2;
} nb_t;

typedef struct {
  int32_t x, y;  /* candidate source coordinate */
  int32_t map;
  uint32_t patch, idmap;
  int32_t sign;  /* +1: neighbourhood c + (n - p); -1: c + (p - n) */
} cand_t;

typedef struct {
  uint32_t pixel;
  uint32_t sx, sy, smap;
  uint32_t patch, idmap;
  float score;
  int append;
  int mirrors;
  int err;
  uint32_t ncand;
} result_t;

typedef struct {
  /* static */
  uint32_t W, H;
  size_t N;
  int tiling;
  int32_t x_l, x_r, y_b, y_t;
  uint32_t k;
  uint64_t m;
  int guided;
  /* maps of the current level, filtered (non-ignored) */
  uint32_t n_maps;
  img_t *maps;
  const uint8_t **masks; /* per filtered map: NULL = All, else mask rgba */
  /* guides of the current level, unfiltered, and the target guide */
  uint32_t n_guides;
  img_t *guides;
  img_t tguide;
  /* live state */
  uint32_t *color;
  uint32_t *cx, *cy, *cmap;
  uint32_t *ipatch, *imap;
  uint8_t *occ, *mir;
  uint32_t *resolved;
  float *rscore;
  size_t n_resolved;
  uint32_t *unresolved;
  size_t n_unresolved;
  size_t locked;
  /* stage */
  float lut_c[256], lut_g[256];
  uint64_t stage_seed;
} gen_t;

static inline uint32_t pack_rgba(const uint8_t *p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
#define OUTSIDE_COLOR 0xFF000000u /* Rgba([0,0,0,255]) */

/* Tree membership of an output-plane point, mirrors included
 * (flush_resolved, ms.rs:296-331). */
static inline int occupied(const gen_t *g, int32_t x, int32_t y) {
  int inx = x >= 0 && x < (int32_t)g->W, iny = y >= 0 && y < (int32_t)g->H;
  if (inx && iny) return g->occ[(size_t)y * g->W + x];
  if (!g->tiling || (!inx && !iny)) return 0;
  if (!inx) {
    if (x >= (int32_t)g->W) {
      int32_t xs = x - (int32_t)g->W;
      return xs < g->x_l && g->mir[(size_t)y * g->W + xs];
    }
    int32_t xs = x + (int32_t)g->W;
    return xs >= 0 && xs > g->x_r && g->mir[(size_t)y * g->W + xs];
  }
  if (y >= (int32_t)g->H) {
    int32_t ys = y - (int32_t)g->H;
    return ys < g->y_b && g->mir[(size_t)ys * g->W + x];
  }
  int32_t ys = y + (int32_t)g->H;
  return ys >= 0 && ys > g->y_t && g->mir[(size_t)ys * g->W + x];
}

static int nb_cmp(const void *a, const void *b) {
  const nb_t *u = (const nb_t *)a, *v = (const nb_t *)b;
  if (u->d2 != v->d2) return u->d2 < v->d2 ? -1 : 1;
  if (u->y != v->y) return u->y < v->y ? -1 : 1;
  if (u->x != v->x) return u->x < v->x ? -1 : 1;
  return 0;
}

/* Exact k nearest tree points of (px,py) under the (d2, y, x) order: expand
 * Chebyshev rings until at least k collected points lie within distance r of
 * the centre; every point outside ring r is farther than r. */
static size_t knn(const gen_t *g, int32_t px, int32_t py, uint32_t k, nb_t *out, nb_t *col, size_t col_cap) {
  if (k == 0) return 0;
  int32_t xmin = 0, xmax = (int32_t)g->W - 1, ymin = 0, ymax = (int32_t)g->H - 1;
  if (g->tiling) {
    xmin = -g->x_l;
    xmax = (int32_t)g->W + g->x_l;
    ymin = -g->y_b;
    ymax = (int32_t)g->H + g->y_b;
  }
  int32_t rmax = px - xmin;
  if (xmax - px > rmax) rmax = xmax - px;
  if (py - ymin > rmax) rmax = py - ymin;
  if (ymax - py > rmax) rmax = ymax - py;
  size_t n = 0, le = 0;
  for (int32_t r = 0; r <= rmax; r++) {
    /* points collected in earlier rings with d2 in ((r-1)^2, r^2] now count */
    int64_t r2 = (int64_t)r * r;
    for (int32_t dy = -r; dy <= r; dy++) {
      int32_t y = py + dy;
      if (y < ymin || y > ymax) continue;
      int full = (dy == -r || dy == r);
      for (int32_t dx = -r; dx <= r; dx += full ? 1 : 2 * r) {
        int32_t x = px + dx;
        if (r == 0 && dx != 0) break;
        if (x >= xmin && x <= xmax && occupied(g, x, y)) {
          if (n < col_cap) {
            col[n].x = x;
            col[n].y = y;
            col[n].d2 = (int64_t)dx * dx + (int64_t)dy * dy;
            n++;
          }
        }
        if (r == 0) break;
      }
    }
    le = 0;
    for (size_t i = 0; i < n; i++)
      if (col[i].d2 <= r2) le++;
    if (le >= k) break;
  }
  qsort(col, n, sizeof(nb_t), nb_cmp);
  size_t kk = n < k ? n : k;
  memcpy(out, col, kk * sizeof(nb_t));
  return kk;
}

static inline uint32_t get_texel(const img_t *im, int32_t x, int32_t y) {
  if (x >= 0 && y >= 0 && x < (int32_t)im->w && y < (int32_t)im->h) return im->px[(size_t)y * im->w + x];
  return OUTSIDE_COLOR;
}

static inline int32_t modulo_i32(int32_t a, int32_t b) {
  int32_t r = a % b;
  return r < 0 ? r + b : r;
}

/* check_coord_validity (ms.rs:1534-1549) */
static inline int coord_valid(const gen_t *g, int32_t x, int32_t y, uint32_t map) {
  const img_t *im = &g->maps[map];
  if (!(x >= 0 && y >= 0 && x < (int32_t)im->w && y < (int32_t)im->h)) return 0;
  const uint8_t *mk = g->masks[map];
  if (!mk) return 1;
  return mk[((size_t)y * im->w + x) * 4] != 0;
}

typedef struct {
  nb_t *nb;
  nb_t *col;
  size_t col_cap;
  cand_t *cand;
  uint8_t *pat, *gpat;
  double *dist;
  float *wt;
} scratch_t;

/* resolve_at_random (ms.rs:447-475): three fresh Pcg32(seed) streams pick the
 * map (usize range), x and y. */
static void random_coord(uint64_t seed, uint32_t n_maps, const img_t *maps, uint32_t *map, uint32_t *x,
                         uint32_t *y) {
  pcg32 r = pcg_seed_from_u64(seed);
  *map = (uint32_t)gen_range_u64(&r, n_maps);
  r = pcg_seed_from_u64(seed);
  *x = gen_range_u32(&r, maps[*map].w);
  r = pcg_seed_from_u64(seed);
  *y = gen_range_u32(&r, maps[*map].h);
}

/* One work item against the current (snapshot) state. */
static void resolve_item(const gen_t *g, uint32_t pixel, int is_new, uint64_t loop_seed, scratch_t *s,
                         result_t *res) {
  int32_t px = (int32_t)(pixel % g->W), py = (int32_t)(pixel / g->W);
  res->pixel = pixel;
  res->err = 0;
  res->ncand = 0;
  size_t nk = knn(g, px, py, g->k, s->nb, s->col, s->col_cap);
  if (nk == 0) {
    /* no resolved neighbours: resolve at random with the stage seed, keep the
     * pixel, insert it without tiling mirrors (ms.rs:1002-1010, 473) */
    uint32_t map, x, y;
    random_coord(g->stage_seed, g->n_maps, g->maps, &map, &x, &y);
    res->sx = x;
    res->sy = y;
    res->smap = map;
    res->patch = pixel;
    res->idmap = map;
    res->score = 0.0f;
    res->append = 1;
    res->mirrors = 0;
    return;
  }
  /* get_distances_to_k_neighs (ms.rs:405-425) */
  double dimx = (double)g->W, dimy = (double)g->H;
  double x2 = (double)px / dimx, y2 = (double)py / dimy;
  double sum = 0.0;
  for (size_t j = 0; j < nk; j++) {
    double x1 = (double)s->nb[j].x / dimx, y1 = (double)s->nb[j].y / dimy;
    double dx = x1 - x2, dy = y1 - y2;
    double d = fma(dx, dx, dy * dy);
    s->dist[j] = d;
    sum += d;
    sum += d;
    sum += d;
    sum += d;
  }
  double avg = sum / (double)(nk * 4);
  for (size_t j = 0; j < nk; j++) {
    double d = s->dist[j] / avg;
    s->wt[j] = (float)tso_exp(-1.0 * d);
    if (g_exp_audit) {
      __atomic_fetch_add(&g_exp_audit_n, 1, __ATOMIC_RELAXED);
      if ((float)exp(-1.0 * d) != s->wt[j]) __atomic_fetch_add(&g_exp_audit_diff, 1, __ATOMIC_RELAXED);
    }
  }
  /* find_candidates (ms.rs:478-602) */
  size_t nc = 0;
  for (size_t j = 0; j < nk; j++) {
    int32_t nx = s->nb[j].x, ny = s->nb[j].y;
    int32_t shx = px - nx, shy = py - ny;
    int32_t wx = modulo_i32(nx, (int32_t)g->W), wy = modulo_i32(ny, (int32_t)g->H);
    size_t f = (size_t)wy * g->W + (size_t)wx;
    uint32_t nmap = g->imap[f];
    if (nmap >= g->n_maps) {
      res->err = TSO_ERR_INDEX;
      return;
    }
    int32_t cxv = (int32_t)g->cx[f] + shx, cyv = (int32_t)g->cy[f] + shy;
    if (coord_valid(g, cxv, cyv, nmap)) {
      cand_t *c = &s->cand[nc++];
      c->x = cxv;
      c->y = cyv;
      c->map = (int32_t)nmap;
      c->patch = g->ipatch[f];
      c->idmap = nmap;
      c->sign = 1;
    }
  }
  pcg32 rng = pcg_seed_from_u64(loop_seed + 1);
  for (uint64_t t = 0; t < g->m; t++) {
    uint32_t map = (uint32_t)gen_range_u64(&rng, g->n_maps);
    uint32_t w = g->maps[map].w, h = g->maps[map].h;
    int32_t rx, ry;
    uint64_t tries = 0;
    for (;;) {
      rx = (int32_t)gen_range_u32(&rng, w);
      ry = (int32_t)gen_range_u32(&rng, h);
      if (coord_valid(g, rx, ry, map)) break;
      /* the reference draws without end; both sides stop after the same
       * number of pairs (TS_MAX_SAMPLE_DRAWS, include/tsgpu.h) */
      if (++tries >= TS_MAX_SAMPLE_DRAWS) {
        res->err = TSO_ERR_NO_VALID_SAMPLE;
        return;
      }
    }
    cand_t *c = &s->cand[nc++];
    c->x = rx;
    c->y = ry;
    c->map = (int32_t)map;
    c->patch = (uint32_t)ry * w + (uint32_t)rx;
    c->idmap = map;
    c->sign = -1;
  }
  res->ncand = (uint32_t)nc;
  /* k_neighs_to_precomputed_reference_pattern (ms.rs:1151-1181) */
  for (size_t j = 0; j < nk; j++) {
    int32_t nx = s->nb[j].x, ny = s->nb[j].y;
    int32_t qx = nx, qy = ny;
    if (g->tiling) {
      qx = modulo_i32(nx, (int32_t)g->W);
      qy = modulo_i32(ny, (int32_t)g->H);
    }
    uint32_t c;
    if (qx >= 0 && qy >= 0 && qx < (int32_t)g->W && qy < (int32_t)g->H)
      c = g->color[(size_t)qy * g->W + qx];
    else
      c = OUTSIDE_COLOR;
    memcpy(s->pat + 4 * j, &c, 4);
    if (g->guided) {
      int32_t gx = nx, gy = ny;
      if (g->tiling) {
        gx = modulo_i32(nx, (int32_t)g->tguide.w);
        gy = modulo_i32(ny, (int32_t)g->tguide.h);
      }
      uint32_t gc = get_texel(&g->tguide, gx, gy);
      memcpy(s->gpat + 4 * j, &gc, 4);
    }
  }
  /* find_best_match / better_match (ms.rs:1184-1288) */
  size_t best = 0;
  float lowest = 3.40282346638528859812e+38f; /* f32::MAX */
  for (size_t ci = 0; ci < nc; ci++) {
    const cand_t *c = &s->cand[ci];
    float score = 0.0f;
    int better = 1;
    const img_t *im = &g->maps[c->map];
    const img_t *gim = g->guided ? &g->guides[c->map] : NULL;
    if (g->guided && (uint32_t)c->map >= g->n_guides) {
      res->err = TSO_ERR_INDEX;
      return;
    }
    for (size_t j = 0; j < nk; j++) {
      int32_t ox = s->nb[j].x - px, oy = s->nb[j].y - py;
      int32_t qx = c->x + c->sign * ox, qy = c->y + c->sign * oy;
      uint32_t t = get_texel(im, qx, qy);
      const uint8_t *tb = (const uint8_t *)&t;
      const uint8_t *pb = s->pat + 4 * j;
      float nps = 0.0f;
      for (int ch = 0; ch < 4; ch++) {
        int d = (int)pb[ch] - (int)tb[ch];
        nps += g->lut_c[d < 0 ? -d : d];
      }
      if (g->guided) {
        uint32_t gt = get_texel(gim, qx, qy);
        const uint8_t *gb = (const uint8_t *)&gt;
        const uint8_t *gp = s->gpat + 4 * j;
        for (int ch = 0; ch < 4; ch++) {
          int d = (int)gp[ch] - (int)gb[ch];
          nps += g->lut_g[d < 0 ? -d : d];
        }
      }
      score += nps * s->wt[j];
      if (score >= lowest) {
        better = 0;
        break;
      }
    }
    if (better) {
      lowest = score;
      best = ci;
    }
  }
  const cand_t *b = &s->cand[best];
  res->sx = (uint32_t)b->x;
  res->sy = (uint32_t)b->y;
  res->smap = (uint32_t)b->map;
  res->patch = b->patch;
  res->idmap = b->idmap;
  res->score = lowest;
  res->append = is_new;
  res->mirrors = 1;
}

/* update + flush_resolved (ms.rs:296-377) */
static void commit(gen_t *g, const result_t *r, const img_t *maps) {
  uint32_t p = r->pixel;
  g->cx[p] = r->sx;
  g->cy[p] = r->sy;
  g->cmap[p] = r->smap;
  g->ipatch[p] = r->patch;
  g->imap[p] = r->idmap;
  g->color[p] = maps[r->smap].px[(size_t)r->sy * maps[r->smap].w + r->sx];
  if (r->append) {
    g->occ[p] = 1;
    if (g->tiling && r->mirrors) g->mir[p] = 1;
    g->resolved[g->n_resolved] = p;
    g->rscore[g->n_resolved] = r->score;
    g->n_resolved++;
  }
}

/* pick_random_unresolved (ms.rs:380-389) */
static int pick_unresolved(gen_t *g, uint64_t seed, uint32_t *out) {
  if (g->n_unresolved == 0) return 0;
  pcg32 r = pcg_seed_from_u64(seed);
  uint64_t idx = gen_range_u64(&r, g->n_unresolved);
  *out = g->unresolved[idx];
  g->unresolved[idx] = g->unresolved[g->n_unresolved - 1];
  g->n_unresolved--;
  return 1;
}

/* ------------------------------------------------------------------------ */
/* Threaded batch evaluation.                                                */
/* ------------------------------------------------------------------------ */
typedef struct {
  const gen_t *g;
  const uint32_t *pix;
  const int *is_new;
  const uint64_t *seeds;
  result_t *res;
  size_t begin, end;
  scratch_t *s;
} job_t;

static void *job_run(void *arg) {
  job_t *j = (job_t *)arg;
  for (size_t i = j->begin; i < j->end; i++) resolve_item(j->g, j->pix[i], j->is_new[i], j->seeds[i], j->s, &j->res[i]);
  return NULL;
}

static int scratch_init(scratch_t *s, size_t N_ext, uint32_t k, uint64_t m) {
  memset(s, 0, sizeof(*s));
  size_t kk = k ? k : 1;
  s->col_cap = N_ext;
  s->nb = (nb_t *)malloc(sizeof(nb_t) * kk);
  s->col = (nb_t *)malloc(sizeof(nb_t) * N_ext);
  s->cand = (cand_t *)malloc(sizeof(cand_t) * (kk + m));
  s->pat = (uint8_t *)malloc(4 * kk);
  s->gpat = (uint8_t *)malloc(4 * kk);
  s->dist = (double *)malloc(sizeof(double) * kk);
  s->wt = (float *)malloc(sizeof(float) * kk);
  return (s->nb && s->col && s->cand && s->pat && s->gpat && s->dist && s->wt) ? 0 : -1;
}
static void scratch_free(scratch_t *s) {
  free(s->nb);
  free(s->col);
  free(s->cand);
  free(s->pat);
  free(s->gpat);
  free(s->dist);
  free(s->wt);
}

static void set_level(gen_t *g, uint32_t n_ex, const tso_example *ex, uint32_t **ex_levels, uint32_t **gd_levels,
                      uint32_t *tg_levels, uint32_t level) {
  uint32_t fi = 0;
  for (uint32_t e = 0; e < n_ex; e++) {
    size_t sz = (size_t)ex[e].w * ex[e].h;
    if (ex[e].sample_method != 1) {
      g->maps[fi].w = ex[e].w;
      g->maps[fi].h = ex[e].h;
      g->maps[fi].px = ex_levels[e] + (size_t)level * sz;
      fi++;
    }
    if (g->guided) {
      size_t gsz = (size_t)ex[e].gw * ex[e].gh;
      g->guides[e].w = ex[e].gw;
      g->guides[e].h = ex[e].gh;
      g->guides[e].px = gd_levels[e] + (size_t)level * gsz;
    }
  }
  if (g->guided) {
    g->tguide.w = g->W;
    g->tguide.h = g->H;
    g->tguide.px = tg_levels + (size_t)level * g->N;
  }
}

/* Build pyramids of packed pixels: levels (>=1) images. */
static uint32_t *build_levels(const uint8_t *rgba, uint32_t w, uint32_t h, uint32_t stages, int *rc) {
  uint32_t nl = stages == 0 ? 1 : stages;
  size_t sz = (size_t)w * h;
  uint8_t *tmp = (uint8_t *)malloc(sz * 4 * nl + 4);
  uint32_t *out = (uint32_t *)malloc(sz * 4 * nl + 4);
  if (!tmp || !out) {
    free(tmp);
    free(out);
    *rc = TSO_ERR_ALLOC;
    return NULL;
  }
  *rc = tso_pyramid(rgba, w, h, stages, tmp);
  for (size_t i = 0; i < sz * nl; i++) out[i] = pack_rgba(tmp + 4 * i);
  free(tmp);
  return out;
}

/*
 * Run a session.  Inputs are RGBA8, already at their final sizes (the
 * session builder's resizes are tso_resize calls made by the caller).
 * inpaint_mask (out_w*out_h*4) marks R<255 pixels as unresolved; the
 * inpaint example (index inpaint_index, unfiltered) supplies the initial
 * colours and must be out_w x out_h.
 * Outputs: out_rgba (N*4), out_coord (N*3: x,y,map), out_id (N*2: patch,map),
 * out_resolved / out_rscore (N entries max; the resolved list), stats.
 */
int tso_run(const tso_params *prm, uint32_t n_ex, const tso_example *ex, const uint8_t *target_guide,
            const uint8_t *inpaint_mask, int32_t inpaint_index, uint8_t *out_rgba, uint32_t *out_coord,
            uint32_t *out_id, uint32_t *out_resolved, float *out_rscore, tso_stats *stats) {
  int rc = TSO_OK;
  gen_t g;
  memset(&g, 0, sizeof(g));
  g.W = prm->out_w;
  g.H = prm->out_h;
  g.N = (size_t)g.W * g.H;
  g.tiling = prm->tiling != 0;
  g.k = prm->k;
  g.m = prm->m;
  g.guided = target_guide != NULL;
  if (g.N == 0 || n_ex == 0 || prm->m == 0) return TSO_ERR_ARG;
  g.x_l = (int32_t)((float)g.W * 0.05f);
  g.x_r = (int32_t)g.W - g.x_l;
  g.y_b = (int32_t)((float)g.H * 0.05f);
  g.y_t = (int32_t)g.H - g.y_b;
  uint32_t stages = prm->stages;
  uint32_t nl = stages == 0 ? 1 : stages;

  uint32_t n_maps = 0;
  for (uint32_t e = 0; e < n_ex; e++)
    if (ex[e].sample_method != 1) n_maps++;
  if (n_maps == 0) return TSO_ERR_ARG;
  g.n_maps = n_maps;
  g.n_guides = g.guided ? n_ex : 0;

  uint32_t **ex_levels = (uint32_t **)calloc(n_ex, sizeof(uint32_t *));
  uint32_t **gd_levels = (uint32_t **)calloc(n_ex, sizeof(uint32_t *));
  uint32_t *tg_levels = NULL;
  g.maps = (img_t *)calloc(n_maps, sizeof(img_t));
  g.masks = (const uint8_t **)calloc(n_maps, sizeof(uint8_t *));
  g.guides = (img_t *)calloc(n_ex + 1, sizeof(img_t));
  g.color = (uint32_t *)calloc(g.N, 4);
  g.cx = (uint32_t *)calloc(g.N, 4);
  g.cy = (uint32_t *)calloc(g.N, 4);
  g.cmap = (uint32_t *)calloc(g.N, 4);
  g.ipatch = (uint32_t *)calloc(g.N, 4);
  g.imap = (uint32_t *)calloc(g.N, 4);
  g.occ = (uint8_t *)calloc(g.N, 1);
  g.mir = (uint8_t *)calloc(g.N, 1);
  size_t res_cap = g.N * 8 + 16;
  g.resolved = (uint32_t *)calloc(res_cap, 4);
  g.rscore = (float *)calloc(res_cap, 4);
  g.unresolved = (uint32_t *)calloc(g.N, 4);
  int nthreads = prm->nthreads < 1 ? 1 : prm->nthreads;
  scratch_t *scr = (scratch_t *)calloc((size_t)nthreads, sizeof(scratch_t));
  result_t *res = NULL;
  uint32_t *bpix = NULL;
  int *bnew = NULL;
  uint64_t *bseed = NULL;
  size_t N_ext = g.N;
  if (g.tiling) N_ext = (size_t)(g.W + 2 * g.x_l + 2) * (g.H + 2 * g.y_b + 2);
  if (!ex_levels || !gd_levels || !g.maps || !g.masks || !g.guides || !g.color || !g.cx || !g.cy || !g.cmap ||
      !g.ipatch || !g.imap || !g.occ || !g.mir || !g.resolved || !g.rscore || !g.unresolved || !scr) {
    rc = TSO_ERR_ALLOC;
    goto done;
  }
  for (int t = 0; t < nthreads; t++)
    if (scratch_init(&scr[t], N_ext, g.k, g.m)) {
      rc = TSO_ERR_ALLOC;
      goto done;
    }

  /* pyramids (session.rs:395-398, lib.rs:570) */
  {
    uint32_t fi = 0;
    for (uint32_t e = 0; e < n_ex; e++) {
      ex_levels[e] = build_levels(ex[e].rgba, ex[e].w, ex[e].h, stages, &rc);
      if (rc) goto done;
      if (g.guided) {
        if (!ex[e].guide) {
          rc = TSO_ERR_ARG;
          goto done;
        }
        gd_levels[e] = build_levels(ex[e].guide, ex[e].gw, ex[e].gh, stages, &rc);
        if (rc) goto done;
      }
      if (ex[e].sample_method != 1) {
        if (ex[e].sample_method == 2) {
          const uint8_t *mk = ex[e].mask;
          size_t any = 0;
          for (size_t i = 0; i < (size_t)ex[e].w * ex[e].h && !any; i++) any = mk[4 * i] != 0;
          if (!any) {
            rc = TSO_ERR_NO_VALID_SAMPLE;
            goto done;
          }
          g.masks[fi] = mk;
        }
        fi++;
      }
    }
    if (g.guided) {
      tg_levels = build_levels(target_guide, g.W, g.H, stages, &rc);
      if (rc) goto done;
    }
  }

  /* Generator::new / new_from_inpaint (ms.rs:220-293) */
  g.n_unresolved = 0;
  g.n_resolved = 0;
  if (inpaint_mask) {
    if (inpaint_index < 0 || (uint32_t)inpaint_index >= n_ex || ex[inpaint_index].w != g.W ||
        ex[inpaint_index].h != g.H) {
      rc = TSO_ERR_ARG;
      goto done;
    }
    for (size_t i = 0; i < g.N; i++) {
      g.color[i] = pack_rgba(ex[inpaint_index].rgba + 4 * i);
      if (inpaint_mask[4 * i] < 255) {
        g.unresolved[g.n_unresolved++] = (uint32_t)i;
      } else {
        g.resolved[g.n_resolved] = (uint32_t)i;
        g.rscore[g.n_resolved] = 0.0f;
        g.n_resolved++;
        g.cx[i] = (uint32_t)(i % g.W);
        g.cy[i] = (uint32_t)(i / g.W);
        g.cmap[i] = (uint32_t)inpaint_index;
      }
    }
    g.locked = g.n_resolved;
  } else {
    for (size_t i = 0; i < g.N; i++) g.unresolved[i] = (uint32_t)i;
    g.n_unresolved = g.N;
  }

  /* Session::run random init (session.rs:42-52, ms.rs:427-475): all examples,
   * ignored ones included, at their full-resolution level. */
  if (prm->has_random_init) {
    uint64_t count = prm->random_init;
    if (count > g.n_unresolved) {
      rc = TSO_ERR_ARG; /* the reference's redo count underflows and it indexes past its resolved list */
      goto done;
    }
    img_t *all = (img_t *)calloc(n_ex, sizeof(img_t));
    if (!all) {
      rc = TSO_ERR_ALLOC;
      goto done;
    }
    for (uint32_t e = 0; e < n_ex; e++) {
      all[e].w = ex[e].w;
      all[e].h = ex[e].h;
      all[e].px = ex_levels[e] + (size_t)(nl - 1) * ex[e].w * ex[e].h;
    }
    for (uint64_t i = 0; i < count; i++) {
      uint32_t p;
      if (!pick_unresolved(&g, prm->seed + i, &p)) continue;
      uint32_t map, x, y;
      random_coord(prm->seed + i + (uint64_t)p, n_ex, all, &map, &x, &y);
      result_t r;
      memset(&r, 0, sizeof(r));
      r.pixel = p;
      r.sx = x;
      r.sy = y;
      r.smap = map;
      r.patch = p;
      r.idmap = map;
      r.score = 0.0f;
      r.append = 1;
      r.mirrors = 0;
      commit(&g, &r, all);
    }
    free(all);
    g.locked += count;
  }

  /* resolve (ms.rs:702-1051) */
  {
    size_t total = g.n_unresolved;
    /* the tree is rebuilt from the resolved list with tiling mirrors */
    memset(g.occ, 0, g.N);
    memset(g.mir, 0, g.N);
    for (size_t i = 0; i < g.n_resolved; i++) {
      g.occ[g.resolved[i]] = 1;
      if (g.tiling) g.mir[g.resolved[i]] = 1;
    }
    float sig2 = prm->cauchy * prm->cauchy;
    float cauchy_lut[256], l2_lut[256];
    for (int d = 0; d < 256; d++) {
      float x = ((float)d - 0.0f) / 255.0f;
      float x2 = x * x;
      cauchy_lut[d] = log1pf(x2 / sig2);
      l2_lut[d] = x2;
    }
    int32_t pyramid_level = 0;
    size_t bcap = 0;
    for (int32_t ps = (int32_t)stages; ps >= 0; ps--) {
      set_level(&g, n_ex, ex, ex_levels, gd_levels, tg_levels, (uint32_t)pyramid_level);
      if (pyramid_level > 0) {
        /* next_pyramid_level (ms.rs:687-700) */
        for (size_t i = 0; i < g.n_resolved; i++) {
          uint32_t p = g.resolved[i];
          uint32_t mp = g.cmap[p];
          if (mp >= g.n_maps) {
            rc = TSO_ERR_INDEX;
            goto done;
          }
          g.color[p] = g.maps[mp].px[(size_t)g.cy[p] * g.maps[mp].w + g.cx[p]];
        }
      }
      pyramid_level += 1;
      if (pyramid_level > (int32_t)stages - 1) pyramid_level = (int32_t)stages - 1;

      pcg32 sr = pcg_seed_from_u64(prm->seed + (uint64_t)ps);
      g.stage_seed = (uint64_t)pcg_next_u32(&sr);

      float fp = powf(prm->p, (float)ps) * (float)total;
      size_t P = (fp >= 0.0f) ? (size_t)fp : 0;
      size_t redo = g.n_resolved - g.locked;

      float adaptive = 0.0f;
      if (g.guided && ps > 0) {
        float a = prm->alpha * (1.0f - ((float)g.n_resolved / (float)total));
        adaptive = (a * a) * a;
      }
      for (int d = 0; d < 256; d++) {
        if (g.guided) {
          g.lut_c[d] = (1.0f - adaptive) * cauchy_lut[d];
          g.lut_g[d] = adaptive * l2_lut[d];
        } else {
          g.lut_c[d] = cauchy_lut[d];
          g.lut_g[d] = 0.0f;
        }
      }
      size_t P_eff = P;
      if (P_eff > redo + g.n_unresolved) P_eff = redo + g.n_unresolved;

      size_t i = 0;
      while (i < P_eff) {
        size_t b = 1;
        if (prm->batch_divisor) {
          b = g.n_resolved / prm->batch_divisor;
          if (b < 1) b = 1;
          if (prm->max_batch && b > prm->max_batch) b = prm->max_batch;
        }
        if (b > P_eff - i) b = P_eff - i;
        if (b > bcap) {
          free(res);
          free(bpix);
          free(bnew);
          free(bseed);
          bcap = b;
          res = (result_t *)malloc(sizeof(result_t) * bcap);
          bpix = (uint32_t *)malloc(4 * bcap);
          bnew = (int *)malloc(sizeof(int) * bcap);
          bseed = (uint64_t *)malloc(8 * bcap);
          if (!res || !bpix || !bnew || !bseed) {
            rc = TSO_ERR_ALLOC;
            goto done;
          }
        }
        for (size_t t = 0; t < b; t++) {
          size_t it = i + t;
          uint64_t loop_seed = g.stage_seed + (uint64_t)it;
          bseed[t] = loop_seed;
          if (it < redo) {
            bpix[t] = g.resolved[it + g.locked];
            bnew[t] = 0;
          } else {
            pick_unresolved(&g, loop_seed, &bpix[t]);
            bnew[t] = 1;
          }
        }
        int nt = nthreads;
        if ((size_t)nt > b) nt = (int)b;
        if (nt <= 1) {
          for (size_t t = 0; t < b; t++) resolve_item(&g, bpix[t], bnew[t], bseed[t], &scr[0], &res[t]);
        } else {
          pthread_t th[256];
          job_t jobs[256];
          if (nt > 256) nt = 256;
          size_t per = (b + nt - 1) / nt;
          for (int t = 0; t < nt; t++) {
            jobs[t].g = &g;
            jobs[t].pix = bpix;
            jobs[t].is_new = bnew;
            jobs[t].seeds = bseed;
            jobs[t].res = res;
            jobs[t].begin = (size_t)t * per;
            jobs[t].end = jobs[t].begin + per > b ? b : jobs[t].begin + per;
            jobs[t].s = &scr[t];
            if (jobs[t].begin >= jobs[t].end) continue;
            if (t == 0) continue;
            pthread_create(&th[t], NULL, job_run, &jobs[t]);
          }
          if (jobs[0].begin < jobs[0].end) job_run(&jobs[0]);
          for (int t = 1; t < nt; t++)
            if (jobs[t].begin < jobs[t].end) pthread_join(th[t], NULL);
        }
        for (size_t t = 0; t < b; t++) {
          if (res[t].err) {
            rc = res[t].err;
            goto done;
          }
          if (res[t].smap >= g.n_maps) {
            rc = TSO_ERR_INDEX;
            goto done;
          }
          if (stats) stats->evals += res[t].ncand;
        }
        for (size_t t = 0; t < b; t++) commit(&g, &res[t], g.maps);
        if (stats) {
          stats->resolves += b;
          stats->batches += 1;
        }
        i += b;
      }
    }
  }

  for (size_t i = 0; i < g.N; i++) {
    memcpy(out_rgba + 4 * i, &g.color[i], 4);
    if (out_coord) {
      out_coord[3 * i] = g.cx[i];
      out_coord[3 * i + 1] = g.cy[i];
      out_coord[3 * i + 2] = g.cmap[i];
    }
    if (out_id) {
      out_id[2 * i] = g.ipatch[i];
      out_id[2 * i + 1] = g.imap[i];
    }
  }
  if (out_resolved || out_rscore) {
    size_t n = g.n_resolved < g.N * 8 ? g.n_resolved : g.N * 8;
    for (size_t i = 0; i < n; i++) {
      if (out_resolved) out_resolved[i] = g.resolved[i];
      if (out_rscore) out_rscore[i] = g.rscore[i];
    }
  }
  if (stats) stats->n_resolved = g.n_resolved;

done:
  if (ex_levels)
    for (uint32_t e = 0; e < n_ex; e++) free(ex_levels[e]);
  if (gd_levels)
    for (uint32_t e = 0; e < n_ex; e++) free(gd_levels[e]);
  free(ex_levels);
  free(gd_levels);
  free(tg_levels);
  free(g.maps);
  free(g.masks);
  free(g.guides);
  free(g.color);
  free(g.cx);
  free(g.cy);
  free(g.cmap);
  free(g.ipatch);
  free(g.imap);
  free(g.occ);
  free(g.mir);
  free(g.resolved);
  free(g.rscore);
  free(g.unresolved);
  if (scr) {
    for (int t = 0; t < nthreads; t++) scratch_free(&scr[t]);
    free(scr);
  }
  free(res);
  free(bpix);
  free(bnew);
  free(bseed);
  return rc;
}

/* The k-NN under the tie rule for one query against an explicit occupancy
 * plane (for unit tests of the GPU k-NN). occ/mir: W*H bytes. */
size_t tso_knn(uint32_t W, uint32_t H, int tiling, const uint8_t *occ, const uint8_t *mir, int32_t px, int32_t py,
               uint32_t k, int32_t *out_xy) {
  gen_t g;
  memset(&g, 0, sizeof(g));
  g.W = W;
  g.H = H;
  g.N = (size_t)W * H;
  g.tiling = tiling;
  g.x_l = (int32_t)((float)W * 0.05f);
  g.x_r = (int32_t)W - g.x_l;
  g.y_b = (int32_t)((float)H * 0.05f);
  g.y_t = (int32_t)H - g.y_b;
  g.occ = (uint8_t *)occ;
  g.mir = (uint8_t *)mir;
  size_t cap = (size_t)(W + 2 * g.x_l + 2) * (H + 2 * g.y_b + 2);
  nb_t *col = (nb_t *)malloc(sizeof(nb_t) * cap);
  nb_t *nb = (nb_t *)malloc(sizeof(nb_t) * (k ? k : 1));
  size_t n = knn(&g, px, py, k, nb, col, cap);
  for (size_t i = 0; i < n; i++) {
    out_xy[2 * i] = nb[i].x;
    out_xy[2 * i + 1] = nb[i].y;
  }
  free(col);
  free(nb);
  return n;
}


/* ---- debug maps (ms.rs:604-653) ------------------------------------------
 * Colour of an id: Pcg32::seed_from_u64(seed).gen_range(0..255) for u8
 * (rand 0.8.5 UniformInt<u8>::sample_single: zone u32::MAX - (u32::MAX -
 * 255 + 1) % 255, draw (v * 255) >> 32 of a u32 v). */
uint8_t tso_id_colour(uint64_t seed) {
  pcg32 r = pcg_seed_from_u64(seed);
  const uint32_t range = 255u;
  const uint32_t zone = 0xffffffffu - (uint32_t)((0x100000000ull - range) % range);
  for (;;) {
    uint64_t m = (uint64_t)pcg_next_u32(&r) * range;
    if ((uint32_t)m <= zone) return (uint8_t)(m >> 32);
  }
}

/* get_id_maps and get_uncertainty_map: RGBA8 per pixel; ids holds (patch,
 * map) per pixel, (flat, score) the resolved list. */
void tso_debug_maps(const uint32_t *ids, size_t n, const uint32_t *flat, const float *score, size_t n_res,
                    uint8_t *patch, uint8_t *map, uint8_t *unc) {
  for (size_t i = 0; i < n; i++) {
    uint32_t p = ids[2 * i], m = ids[2 * i + 1];
    patch[4 * i] = tso_id_colour(p);
    patch[4 * i + 1] = tso_id_colour((uint32_t)(p * 5u + 21u));
    patch[4 * i + 2] = tso_id_colour((uint32_t)(p / 4u + 12u));
    patch[4 * i + 3] = 255;
    map[4 * i] = tso_id_colour((uint64_t)m * 200u);
    map[4 * i + 1] = tso_id_colour((uint32_t)(m * 5u + 341u));
    map[4 * i + 2] = tso_id_colour((uint32_t)(m * 1200u - 35412u));
    map[4 * i + 3] = 255;
    unc[4 * i] = unc[4 * i + 1] = unc[4 * i + 2] = unc[4 * i + 3] = 0;
  }
  for (size_t i = 0; i < n_res; i++) {
    float s = score[i];
    float mn = (s != s) ? 1.0f : (s < 1.0f ? s : 1.0f); /* f32::min ignores NaN */
    float v = mn * 255.0f;
    uint32_t ns = v >= 255.0f ? 255u : (v > 0.0f ? (uint32_t)v : 0u); /* `as u8` truncates, saturates */
    size_t f = flat[i];
    if (f >= n) continue;
    unc[4 * f] = (uint8_t)ns;
    unc[4 * f + 1] = (uint8_t)(255u - ns);
    unc[4 * f + 2] = 0;
    unc[4 * f + 3] = 255;
  }
}
