// ts_kernels.cu — sm_103a kernels of the texture-synthesis hot loop.
//
// One batch step of a synthesis stage is five launches:
//   knn_walk        warp per work item: the k nearest resolved points under
//                   the (d2, y, x) order, by walking a table of lattice offsets
//                   sorted in that order and testing a resolved-point bitmap
//                   (replaces TreeGrid::get_k_nearest_neighbors, ms.rs:1363-1530)
//   knn_exhaustive  CTA per item the walk could not finish (sparse regions):
//                   radix-select over the resolved list
//   mean            thread per item: the mean of the 4x-duplicated distance
//                   list (ms.rs:417-423), the in-order f64 sum, one item per
//                   lane (large batches); for whole small batches the
//                   exhaustive k-NN computes it on one thread in integer
//                   arithmetic, whose dependent chain is shorter than f64's
//   resolve         warp per item: neighbour weights (ms.rs:1198-1203) in
//                   double-f32 arithmetic with an exact f64 fallback,
//                   coherence + random candidates (ms.rs:478-602), own
//                   pattern (ms.rs:1151-1181), candidate cost and first-min
//                   argmin (ms.rs:1184-1288), lanes over candidates
// The k-NN kernels also write each neighbour's exact squared normalised
// distance (ms.rs:410-415), one f64 fused multiply-add from per-pixel tables.
//   commit          thread per item: update + flush_resolved (ms.rs:296-377)
// Every item of a batch reads the state as it was when the batch started;
// commit runs after all of them.  Per stage, random_candidates precomputes the
// m random candidates of every item (they depend only on the seed), and
// level_switch recolours the resolved pixels (ms.rs:687-700).
//
// Floating point follows the reference operation by operation: f32 sums are
// sequential, multiplies and adds are never fused (the file is compiled with
// --fmad=false and uses __fadd_rn/__fmul_rn where it matters), and the f64
// distances use an explicit fused multiply-add exactly where ms.rs:415 calls
// mul_add.
#include <float.h>
#include <stdint.h>

#include <cuda_pipeline.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <utility>

#include "tsgpu.h"
#include "ts_common.h"
#include "ts_kernels.cuh"

namespace ts {

namespace {

constexpr int kWarp = 32;
constexpr int kResolveWarps = 4;
constexpr int kWalkWarps = 8;
constexpr int kExhThreads = 256;
constexpr int kTeamThreads = 128;
constexpr int kTeamFullThreads = 256;  // the full-evaluation form: batches of at most ~1000 items
constexpr int kStepWideThreads = 512;  // the fused small-step kernel on steps of at most one item per SM
constexpr int kExhCap = 2048;      // keys kept by the exhaustive k-NN at the cut distance
constexpr int kExhAllKeys = 8192;  // keys the exhaustive k-NN sorts in shared memory directly
constexpr int kExhSortAll = 256;   // at most this many keys are sorted without a select
constexpr uint32_t kMaxDraws = TS_MAX_SAMPLE_DRAWS;  // (x, y) pairs per random candidate
constexpr uint32_t kRcandFailed = 0x7fffu;              // map field of a random candidate whose draws ran out

__device__ const double g_exp2_64[64] = {TS_EXP2_TABLE_VALUES};
__device__ const float g_exp2_ff[128] = {TS_EXP2_FF_TABLE_VALUES};

__device__ __forceinline__ void set_err(int *err, int code) {
  if (*err == 0) atomicCAS(err, 0, code);
}

__device__ __forceinline__ int off_dx(int32_t off) { return (int)(int16_t)(off & 0xffff); }
__device__ __forceinline__ int off_dy(int32_t off) { return off >> 16; }
__device__ __forceinline__ int32_t pack_off(int dx, int dy) { return (int32_t)((uint32_t)(dx & 0xffff) | ((uint32_t)dy << 16)); }

__device__ __forceinline__ int modi(int a, int b) {
  int r = a % b;
  return r < 0 ? r + b : r;
}

// Tree membership of an output-plane point, tiling mirrors included
// (flush_resolved, ms.rs:296-331).
__device__ __forceinline__ bool occupied(const SessionDev &s, int x, int y) {
  const bool inx = (unsigned)x < s.W, iny = (unsigned)y < s.H;
  if (inx && iny) return (__ldg(&s.occ[(size_t)y * s.wpr + (x >> 5)]) >> (x & 31)) & 1u;
  if (!s.tiling || (!inx && !iny)) return false;
  int xs = x, ys = y;
  if (!inx) {
    if (x >= (int)s.W) {
      xs = x - (int)s.W;
      if (xs >= s.x_l) return false;
    } else {
      xs = x + (int)s.W;
      if (xs < 0 || xs <= s.x_r) return false;
    }
  } else {
    if (y >= (int)s.H) {
      ys = y - (int)s.H;
      if (ys >= s.y_b) return false;
    } else {
      ys = y + (int)s.H;
      if (ys < 0 || ys <= s.y_t) return false;
    }
  }
  return (__ldg(&s.mir[(size_t)ys * s.wpr + (xs >> 5)]) >> (xs & 31)) & 1u;
}

// Whether pixel p is in a tree of n points (SessionDev::rank); always true
// when the bitmap is the tree itself.
__device__ __forceinline__ bool in_tree(const SessionDev &s, uint32_t p, uint32_t n) {
  return !s.rank || __ldg(&s.rank[p]) - 1u < n;
}

// occupied() against the tree of an item whose batch starts with n points:
// with SessionDev::rank the bitmap may hold later points too, so a set bit
// is checked against the tree position of the pixel it stands for.
__device__ __forceinline__ bool occupied_n(const SessionDev &s, int x, int y, uint32_t n) {
  if (!occupied(s, x, y)) return false;
  if (!s.rank) return true;
  const int xs = modi(x, (int)s.W), ys = modi(y, (int)s.H);  // a mirror stands for its wrapped pixel
  return in_tree(s, (uint32_t)ys * s.W + (uint32_t)xs, n);
}

// Resolved-list length at the start of the batch of stage item `item`
// (BatchDev::btab), else the launch's own.
__device__ __forceinline__ uint32_t item_nres(const BatchDev &b, uint32_t item) {
  if (!b.btab) return b.n_res;
  uint32_t lo = 0, hi = b.nbt;
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (__ldg(&b.btab[mid].x) <= item)
      lo = mid;
    else
      hi = mid;
  }
  return __ldg(&b.btab[lo].y);
}

__device__ __forceinline__ bool mir_bit(const SessionDev &s, uint32_t x, uint32_t y) {
  return (s.mir[(size_t)y * s.wpr + (x >> 5)] >> (x & 31)) & 1u;
}

// check_coord_validity (ms.rs:1534-1549)
__device__ __forceinline__ bool coord_valid(const SessionDev &s, const MapDesc &md, int x, int y) {
  if (x < 0 || y < 0 || x >= (int)md.w || y >= (int)md.h) return false;
  if (md.mask_off < 0) return true;
  return __ldg(&s.masks[md.mask_off + (size_t)y * md.w + x]) != 0;
}

// ---------------------------------------------------------------------------
// Random candidates of every item of a stage (ms.rs:549-599): the stream is
// Pcg32::seed_from_u64(stage_seed + item + 1); per candidate a map
// (usize range), then (x, y) redrawn until valid.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void random_candidates_body(const SessionDev &s, const StageDev &st, uint32_t vb) {
  const uint32_t item = vb * blockDim.x + threadIdx.x;
  if (item >= st.n_items) return;
  Pcg32 g = pcg_from_u64(st.stage_seed + (uint64_t)item + 1ULL);
  uint2 *out = st.rcand + (size_t)item * s.m;
  for (uint32_t t = 0; t < s.m; ++t) {
    uint64_t map64 = 0;
    bool ok = gen_range_u64_bounded(g, s.n_maps, 256, map64);
    const uint32_t map = ok ? (uint32_t)map64 : 0u;
    const MapDesc md = s.maps[map];
    uint32_t x = 0, y = 0;
    if (ok) {
      ok = false;
      for (uint32_t tries = 0; tries < kMaxDraws; ++tries) {
        if (!gen_range_u32_bounded(g, md.w, 256, x) || !gen_range_u32_bounded(g, md.h, 256, y)) break;
        if (coord_valid(s, md, (int)x, (int)y)) {
          ok = true;
          break;
        }
      }
    }
    if (!ok) {
      // Only an item with resolved neighbours uses its random candidates
      // (an item without any resolves at random, ms.rs:1002-1010), so the
      // failure is left for the resolve kernel to report when it reads one.
      for (; t < s.m; ++t) out[t] = make_uint2(0u, kRcandFailed);
      return;
    }
    out[t] = make_uint2(x | (y << 16), map);
  }
}

// A random candidate as the resolve kernels store it: {x | y<<16, map}.  A
// failed draw (kRcandFailed) reports TS_ERR_NO_VALID_SAMPLE and is replaced
// by texel (0, 0) of map 0, so that nothing reads past the map table; the
// run's result is discarded.
__device__ __forceinline__ uint2 use_rcand(const SessionDev &s, uint2 v) {
  if (v.y == kRcandFailed) {
    set_err(s.err, kDevErrNoSample);
    v = make_uint2(0u, 0u);
  }
  return v;
}

// Exact squared normalised distance of a neighbour at offset (dx, dy).
__device__ __forceinline__ double neighbour_dist(const SessionDev &s, int px, int py, int dx, int dy, double x2,
                                                  double y2) {
  const int R = s.dtab_r;
  if (dx >= -R && dx <= R && dy >= -R && dy <= R) {
    const double ddx = __ldg(&s.dxt[(size_t)px * (2 * R + 1) + dx + R]);
    return __fma_rn(ddx, ddx, __ldg(&s.dy2t[(size_t)py * (2 * R + 1) + dy + R]));
  }
  const double ddx = __dsub_rn(s.xdiv[px + dx + s.xdiv_off], x2);
  const double ddy = __dsub_rn(s.ydiv[py + dy + s.ydiv_off], y2);
  return __fma_rn(ddx, ddx, __dmul_rn(ddy, ddy));
}

// The same from the per-pixel tables only, for offsets within their radius
// (every offset the walk's table holds): one f64 instruction, and no
// predicated far-offset path beside it.
__device__ __forceinline__ double neighbour_dist_near(const SessionDev &s, int px, int py, int dx, int dy) {
  const int R = s.dtab_r;
  const double ddx = __ldg(&s.dxt[(size_t)px * (2 * R + 1) + dx + R]);
  return __fma_rn(ddx, ddx, __ldg(&s.dy2t[(size_t)py * (2 * R + 1) + dy + R]));
}

// ---------------------------------------------------------------------------
// The mean of a distance list whose sums are exact (SessionDev::exact_sum):
// the in-order sum of the 4x-duplicated list (ms.rs:417-421) never rounds,
// so it equals 4 * (the list's sum in any order of exact adds), and the mean
// is that divided by 4n, rounded once, as the reference divides.
// ---------------------------------------------------------------------------
// A neighbour's distance in units of SessionDev::exact_q: an integer (the
// distances are exact), summed in integers instead of f64 adds.
__device__ __forceinline__ unsigned long long exact_units(const SessionDev &s, int dx, int dy) {
  return ((unsigned long long)(uint32_t)(dx * dx) << s.exact_sx) + ((unsigned long long)(uint32_t)(dy * dy) << s.exact_sy);
}
__device__ __forceinline__ unsigned long long warp_sum_units(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// A neighbour's distance from its packed offset, for sessions with exact
// sums: its units, converted (exact below 2^53) and scaled by the power of
// two exact_q, equal fma(dx, dx, dy * dy) of get_distances_to_k_neighs
// (ms.rs:405-425) bit for bit.
__device__ __forceinline__ double exact_dist(const SessionDev &s, int32_t off) {
  return __dmul_rn(__ull2double_rn(exact_units(s, off_dx(off), off_dy(off))), s.exact_q);
}
// The mean from the list's sum in units: below 2^53, so its conversion and
// the scaling by the power of two exact_q are exact; 4 * that is the
// reference's in-order sum, divided by 4n and rounded once.
// Integer arithmetic only (ts_units_bits, ts_div_int_rn): GB300's FP64 pipe
// is narrow, and an f64 division takes it for a whole warp.
__device__ __forceinline__ double exact_mean(const SessionDev &s, unsigned long long units, uint32_t n) {
  return bits_dbl(ts_div_int_rn(ts_units_bits(units, s.exact_qe), n));
}

__device__ __forceinline__ unsigned long long nb_key(uint32_t d2, int x, int y) {
  return ((unsigned long long)d2 << 32) | ((uint32_t)(y + 32768) << 16) | (uint32_t)(x + 32768);
}

// ---------------------------------------------------------------------------
// k-NN by walking the sorted offset table.  The table holds every lattice
// offset with d2 <= its radius^2, in (d2, dy, dx) order, so the first k
// occupied entries are exactly the k nearest points under the tie rule.
// Items for which the table holds fewer than k points (sparse steps, image
// edges) go to the exhaustive k-NN; sparse steps send every item there.
// ---------------------------------------------------------------------------
// Walk window: the bitmap square [-R, R]^2 around an item (R the table
// radius), kWinWords 32-bit words per row, bit i of word w of row r = point
// (px - R + 32w + i, py - R + r).
constexpr int kWinRows = 2 * kKnnTabRadius + 1;
constexpr int kWinWords = (2 * kKnnTabRadius + 1 + 31) / 32;
constexpr uint32_t kWalkDirect = 128;  // expected entries still to scan above which the window is built
constexpr size_t kWalkWinBytes = (size_t)kWalkWarps * kWinRows * kWinWords * 4;  // dynamic shared memory

// Bits of bitmap row `row` for x in [x0, x0 + 32) (bit i = x0 + i), zero
// outside [0, W).
__device__ __forceinline__ uint32_t row_bits(const uint32_t *row, int x0, const SessionDev &s) {
  const int W = (int)s.W;
  if (x0 >= W || x0 + 32 <= 0) return 0u;
  const int q = x0 >> 5, sh = x0 & 31;  // floor division
  const uint32_t lo = (q >= 0 && q < (int)s.wpr) ? __ldg(&row[q]) : 0u;
  const uint32_t hi = (sh && q + 1 >= 0 && q + 1 < (int)s.wpr) ? __ldg(&row[q + 1]) : 0u;
  uint32_t v = sh ? (lo >> sh) | (hi << (32 - sh)) : lo;
  if (x0 < 0) v &= ~0u << (-x0);
  if (x0 + 32 > W) v &= (1u << (W - x0)) - 1u;
  return v;
}

// Bits i with lo <= i < hi of a 32-bit word (lo, hi clamped to [0, 32]).
__device__ __forceinline__ uint32_t bit_range(int lo, int hi) {
  lo = max(lo, 0);
  hi = min(hi, 32);
  if (hi <= lo) return 0u;
  const uint32_t upto_hi = hi >= 32 ? ~0u : ((1u << hi) - 1u);
  return upto_hi & (~0u << lo);
}

// occupied() for the 32 points (x0 + i, y), i = 0..31, as a word.
__device__ __forceinline__ uint32_t window_word(const SessionDev &s, int x0, int y) {
  const int W = (int)s.W, H = (int)s.H;
  if ((unsigned)y < s.H) {
    uint32_t v = row_bits(s.occ + (size_t)y * s.wpr, x0, s);
    if (s.tiling) {
      const uint32_t *mr = s.mir + (size_t)y * s.wpr;
      // x >= W: mirror of xs = x - W when xs < x_l
      v |= row_bits(mr, x0 - W, s) & bit_range(0, s.x_l - (x0 - W));
      // x < 0: mirror of xs = x + W when xs > x_r
      v |= row_bits(mr, x0 + W, s) & bit_range(s.x_r + 1 - (x0 + W), 32);
    }
    return v;
  }
  if (!s.tiling) return 0u;
  if (y >= H) {
    const int ys = y - H;
    return ys < s.y_b ? row_bits(s.mir + (size_t)ys * s.wpr, x0, s) : 0u;
  }
  const int ys = y + H;
  return (ys >= 0 && ys > s.y_t) ? row_bits(s.mir + (size_t)ys * s.wpr, x0, s) : 0u;
}

// kWin: small (latency-bound) steps, whose sparse items switch to a
// window in dynamic shared memory (kWalkWinBytes) once the hits so far say
// more than two further rounds are needed.
template <bool kWin>
__device__ __forceinline__ void knn_walk_body(const SessionDev &s, const StageDev &st, const BatchDev &b, uint32_t vb,
                                              uint32_t vg) {
  const int lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t nb = b.i1 - b.i0;
  for (uint32_t local = vb * kWalkWarps + (threadIdx.x >> 5); local < nb; local += vg * kWalkWarps) {
    const uint32_t pixel = st.items[b.i0 + local];
    const int px = (int)(pixel % s.W), py = (int)(pixel / s.W);
    int32_t *nbo = b.nbuf + (size_t)local * s.k;
    const uint32_t n_tree = item_nres(b, b.i0 + local);
    uint32_t count = 0;
    const uint32_t tab_n = b.grid_first ? 0u : s.knn_tab_n;
    // 64 table entries per round, two per lane, both looked up before either
    // is used; `hit` answers membership for an offset
    auto round = [&](uint32_t c, auto &&hit) {
      const uint32_t i0 = c + lane, i1 = c + kWarp + lane;
      const int32_t o0 = i0 < tab_n ? __ldg(&s.knn_tab[i0]) : 0;
      const int32_t o1 = i1 < tab_n ? __ldg(&s.knn_tab[i1]) : 0;
      const bool h0 = i0 < tab_n && hit(off_dx(o0), off_dy(o0));
      const bool h1 = i1 < tab_n && hit(off_dx(o1), off_dy(o1));
      const uint32_t b0 = __ballot_sync(0xffffffffu, h0);
      const uint32_t b1 = __ballot_sync(0xffffffffu, h1);
      const uint32_t r0 = count + __popc(b0 & lt), r1 = count + __popc(b0) + __popc(b1 & lt);
      if (h0 && r0 < s.k) nbo[r0] = o0;
      if (h1 && r1 < s.k) nbo[r1] = o1;
      count += __popc(b0) + __popc(b1);
    };
    // rounds look the bitmap up directly while the hits so far say that
    // two more rounds or fewer will do (dense steps end here)
    uint32_t c = 0;
    while (c < tab_n) {
      round(c, [&](int dx, int dy) { return occupied_n(s, px + dx, py + dy, n_tree); });
      c += 2 * kWarp;
      if (count >= s.k) break;
      if (kWin && (count == 0 || (uint64_t)(s.k - count) * c > (uint64_t)count * kWalkDirect)) break;
    }
    if (kWin && count < s.k && c < tab_n) {
      // sparse: the membership bits of the whole table's square, built in
      // one pass of independent loads, then the rest of the walk from
      // shared memory
      extern __shared__ uint32_t walk_win[];
      uint32_t *win = walk_win + (threadIdx.x >> 5) * (kWinRows * kWinWords);
      for (uint32_t wi = lane; wi < kWinRows * kWinWords; wi += kWarp) {
        const int row = (int)(wi / kWinWords), word = (int)(wi - row * kWinWords);
        win[wi] = window_word(s, px - kKnnTabRadius + 32 * word, py - kKnnTabRadius + row);
      }
      __syncwarp();
      for (; c < tab_n; c += 2 * kWarp) {
        round(c, [&](int dx, int dy) {
          const int i = dx + kKnnTabRadius;
          // (a set bit of a later point fails its tree check)
          return ((win[(dy + kKnnTabRadius) * kWinWords + (i >> 5)] >> (i & 31)) & 1u) != 0u &&
                 (!s.rank || occupied_n(s, px + dx, py + dy, n_tree));
        });
        if (count >= s.k) break;
      }
      __syncwarp();  // the window is rebuilt for the warp's next item
    }
    if (count >= s.k) {
      // the distances once the k offsets are known, 32 per f64 warp
      // instruction (an f64 instruction costs the same whatever its active
      // lanes, and GB300's f64 pipe is narrow)
      __syncwarp();
      // (sessions with exact sums store no distances: the resolve derives
      // each one from its offset, exact_dist)
      unsigned long long part = 0;
      for (uint32_t j = lane; j < s.k; j += kWarp) {
        const int32_t o = nbo[j];
        if (s.exact_sum)
          part += exact_units(s, off_dx(o), off_dy(o));
        else
          b.dist[(size_t)j * nb + local] = neighbour_dist_near(s, px, py, off_dx(o), off_dy(o));
      }
      if (s.exact_sum) {
        part = warp_sum_units(part);
        if (lane == 0) b.mean[local] = exact_mean(s, part, s.k);
      }
    }
    if (lane == 0) {
      if (count >= s.k) {
        b.ncnt[local] = s.k;
      } else {
        const uint32_t slot = atomicAdd(b.fb_count, 1u);
        b.fb_list[slot] = local;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Exhaustive k-NN (one CTA per item): radix-select the k-th smallest d2 over
// every resolved point and its mirrors, keep the points at or below it, sort
// them by (d2, y, x) and emit the first k.
// ---------------------------------------------------------------------------
// The mean of a neighbour distance list on one thread (ms.rs:417-423, as
// k_mean_staged computes it): the 4n-long chain of f64 adds in order, then
// / (4n).  Where one thread runs it alone this is shorter than the integer
// form of the four adds (ts_add4_fast): 14.1k against 16.8k cycles for
// n = 50 on GB300.
__device__ __forceinline__ double mean_chain(const double *d, uint32_t n) {
  double sum = 0.0;
  for (uint32_t i = 0; i < n; ++i) {
    const double v = d[i];
    sum = __dadd_rn(sum, v);
    sum = __dadd_rn(sum, v);
    sum = __dadd_rn(sum, v);
    sum = __dadd_rn(sum, v);
  }
  return __ddiv_rn(sum, (double)(n * 4u));
}

struct ExhShared {
  double dist[256];  // the item's neighbour distances, when the kernel also computes the mean
  unsigned long long wsum[16];  // per-warp distance sums in units (SessionDev::exact_sum), up to 512 threads
  int32_t nbo[256];  // and their offsets
  uint32_t hist[256];
  unsigned long long keys[kExhCap];
  uint32_t nkeys;
  uint32_t total;
  uint32_t prefix;
  uint32_t rank;
  int overflow;
  uint32_t flag, cnt;  // cell-grid search: a ring cell lies in the grid; keys below the bound
  uint32_t below, le;  // select: keys below the selected digit's range; at or below it
};

constexpr uint32_t kExhGridFrom = 4096;  // resolved points from which the cell grid is searched

__device__ __forceinline__ void ring_cell(int r, int i, int &dx, int &dy) {
  if (r == 0) {
    dx = dy = 0;
  } else if (i < 2 * r + 1) {
    dx = -r + i;
    dy = -r;
  } else if (i < 4 * r + 2) {
    dx = -r + (i - (2 * r + 1));
    dy = r;
  } else if (i < 6 * r + 1) {
    dx = -r;
    dy = -r + 1 + (i - (4 * r + 2));
  } else {
    dx = r;
    dy = -r + 1 + (i - (6 * r + 1));
  }
}

template <typename F>
__device__ __forceinline__ void for_points(const SessionDev &s, uint32_t n_res, F &&f) {
  for (uint32_t e = threadIdx.x; e < n_res; e += blockDim.x) {
    const uint32_t p = s.resolved[e];
    const int x = (int)(p % s.W), y = (int)(p / s.W);
    f(x, y);
    if (s.tiling && mir_bit(s, (uint32_t)x, (uint32_t)y)) {
      if (x < s.x_l)
        f(x + (int)s.W, y);
      else if (x > s.x_r)
        f(x - (int)s.W, y);
      if (y < s.y_b)
        f(x, y + (int)s.H);
      else if (y > s.y_t)
        f(x, y - (int)s.H);
    }
  }
}

__device__ uint32_t knn_exhaustive_item(const SessionDev &s, const StageDev &st, const BatchDev &b, uint32_t local,
                                        ExhShared &sh, unsigned long long *all, uint32_t cap, bool with_mean,
                                        bool use_grid = true, bool mean_here = true);

// One CTA per item.  `all` (dynamic shared memory, kExhAllKeys entries)
// receives every point's key in one pass over the resolved list; when they
// fit, a bitonic sort of them gives the answer directly, otherwise a
// radix select over further passes finds the cut distance first.
__device__ __forceinline__ void knn_exhaustive_body(const SessionDev &s, const StageDev &st, const BatchDev &b,
                                                    int all_items, uint32_t cap, uint32_t vb, uint32_t vg,
                                                    bool use_grid = true) {
  __shared__ ExhShared sh;
  extern __shared__ unsigned long long all_keys[];
  const uint32_t n = all_items ? b.i1 - b.i0 : *b.fb_count;
  for (uint32_t e = vb; e < n; e += vg) {
    const uint32_t local = all_items ? e : b.fb_list[e];
    knn_exhaustive_item(s, st, b, local, sh, all_keys, cap, all_items != 0, use_grid);
    __syncthreads();
  }
}

// Bitonic sort of keys[0, np2) ascending (np2 a power of two), whole CTA.
__device__ __forceinline__ void block_bitonic(unsigned long long *keys, uint32_t np2) {
  for (uint32_t size = 2; size <= np2; size <<= 1) {
    for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
      for (uint32_t i = threadIdx.x; i < np2; i += blockDim.x) {
        const uint32_t j = i ^ stride;
        if (j > i) {
          const bool up = (i & size) == 0;
          const unsigned long long a = keys[i], c = keys[j];
          if ((a > c) == up) {
            keys[i] = c;
            keys[j] = a;
          }
        }
      }
      __syncthreads();
    }
  }
}

// The first `nout` of the n distinct keys in keys[] in ascending order.
// Up to kExhRankSort keys: each key's rank is the count of smaller keys (all
// threads read the same key at a time), and the key lands at out[rank] when
// the rank is below nout; more keys: a bitonic sort in place.  Returns the
// sorted array.
constexpr uint32_t kExhRankSort = 512;
__device__ __forceinline__ const unsigned long long *sort_first(unsigned long long *keys, uint32_t n, uint32_t nout,
                                                                unsigned long long *out) {
  if (n <= kExhRankSort) {
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
      const unsigned long long key = keys[i];
      uint32_t r = 0;
#pragma unroll 8
      for (uint32_t q = 0; q < n; ++q) r += keys[q] < key ? 1u : 0u;
      if (r < nout) out[r] = key;
    }
    __syncthreads();
    return out;
  }
  uint32_t np2 = 1;
  while (np2 < n) np2 <<= 1;
  for (uint32_t i = n + threadIdx.x; i < np2; i += blockDim.x) keys[i] = ~0ull;
  __syncthreads();
  block_bitonic(keys, np2);
  return keys;
}

// The points of the cells in rings around the item's cell, as keys in
// all[], until k keys lie below the rings' reach: after rings 0..r every
// point with d2 < (r * kCell + 1)^2 has been seen (the cells beyond are that
// far away in x or y), so the k smallest collected keys are then the k
// nearest points under the tie rule; a ring wholly outside the grid means
// every point has been seen.  The cells of consecutive rings are numbered
// 0, 1.. (ring r starts at 4r(r-1) + 1) and taken blockDim.x at a time; the
// bound is tested after each such round for the last ring it completed.
// Leaves the count in sh.total (above kExhAllKeys: the buffer overflowed)
// and the OR of the d2 in sh.prefix.
__device__ __forceinline__ uint32_t ring_base(uint32_t r) { return r == 0 ? 0u : 4u * r * (r - 1u) + 1u; }

__device__ void grid_collect(const SessionDev &s, int px, int py, uint32_t k, uint32_t n_tree, ExhShared &sh,
                             unsigned long long *all, uint32_t cap) {
  if (threadIdx.x == 0) {
    sh.total = 0;
    sh.prefix = 0;
    sh.flag = 0;
    sh.cnt = 0;
  }
  __syncthreads();
  const int qcx = (px - s.cox) / kCell, qcy = (py - s.coy) / kCell;
  // rings wholly outside the grid start beyond the farthest grid edge
  const uint32_t r_max = (uint32_t)max(max(qcx, (int)s.cgw - 1 - qcx), max(qcy, (int)s.cgh - 1 - qcy));
  const uint32_t f_end_all = ring_base(r_max + 1);
  for (uint32_t f0 = 0; f0 < f_end_all; f0 += blockDim.x) {
    const uint32_t f = f0 + threadIdx.x;
    uint32_t dor = 0;
    if (f < f_end_all) {
      // ring r of cell number f: 4r(r-1) + 1 <= f < 4r(r+1) + 1
      uint32_t r = f == 0 ? 0u : (uint32_t)(sqrtf((float)(f - 1) * 0.25f + 0.25f) + 0.5f);
      while (r > 0 && ring_base(r) > f) --r;
      while (ring_base(r + 1) <= f) ++r;
      int gx, gy;
      ring_cell((int)r, (int)(f - ring_base(r)), gx, gy);
      gx += qcx;
      gy += qcy;
      const uint32_t cnt =
          ((unsigned)gx < s.cgw && (unsigned)gy < s.cgh) ? __ldg(&s.cells[(size_t)gy * s.cgw + gx]) : 0u;
      if (cnt) {
        const int x0 = s.cox + gx * kCell, y0 = s.coy + gy * kCell;
        uint32_t found = 0;
        for (int yy = 0; yy < kCell && found < cnt; ++yy) {
          const int y = y0 + yy, dy = y - py;
          uint32_t bits;
          if ((unsigned)y < s.H && x0 >= 0 && x0 + kCell <= (int)s.W) {
            const uint32_t wi = (uint32_t)x0 >> 5, sh5 = (uint32_t)x0 & 31u;
            const uint32_t *row = s.occ + (size_t)y * s.wpr;
            uint64_t wv = __ldg(&row[wi]);
            if (sh5 + kCell > 32) wv |= (uint64_t)__ldg(&row[wi + 1]) << 32;
            bits = (uint32_t)(wv >> sh5) & ((1u << kCell) - 1u);
            if (s.rank)  // set bits of later points (k-NN made ahead) do not count
              for (uint32_t t = bits; t;) {
                const int bp = __ffs(t) - 1;
                t &= t - 1u;
                if (!in_tree(s, (uint32_t)y * s.W + (uint32_t)(x0 + bp), n_tree)) bits &= ~(1u << bp);
              }
          } else {
            bits = 0;
            for (int xx = 0; xx < kCell; ++xx)
              if (occupied_n(s, x0 + xx, y, n_tree)) bits |= 1u << xx;
          }
          while (bits) {
            const int bp = __ffs(bits) - 1;
            bits &= bits - 1u;
            const int x = x0 + bp, dx = x - px;
            const uint32_t d2 = (uint32_t)(dx * dx + dy * dy);
            dor |= d2;
            const uint32_t slot = atomicAdd(&sh.total, 1u);
            if (slot < cap) all[slot] = nb_key(d2, x, y);
            ++found;
          }
        }
      }
    }
    if (dor) atomicOr(&sh.prefix, dor);
    __syncthreads();
    const uint32_t n = sh.total;
    if (n > cap) break;
    // the last ring this round completed
    const uint32_t f_done = min(f0 + blockDim.x, f_end_all);
    uint32_t r_done = 0;
    while (ring_base(r_done + 2) <= f_done) ++r_done;
    if (ring_base(r_done + 1) > f_done) continue;  // not even ring 0 complete (cannot happen)
    const uint32_t lim = (uint32_t)(r_done * kCell + 1) * (uint32_t)(r_done * kCell + 1);
    uint32_t c = 0;
    for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) c += (uint32_t)(all[e] >> 32) < lim ? 1u : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(&sh.cnt, c);
    __syncthreads();
    const uint32_t lt = sh.cnt;
    __syncthreads();  // every thread has read cnt
    if (lt >= k) break;
    if (threadIdx.x == 0) sh.cnt = 0;
    __syncthreads();
  }
}

__device__ uint32_t knn_exhaustive_item(const SessionDev &s, const StageDev &st, const BatchDev &b, uint32_t local,
                                        ExhShared &sh, unsigned long long *all, uint32_t cap, bool with_mean,
                                        bool use_grid, bool mean_here) {
  const uint32_t pixel = st.items[b.i0 + local];
  const int px = (int)(pixel % s.W), py = (int)(pixel / s.W);
  const uint32_t k = s.k;
  const uint32_t n_res = item_nres(b, b.i0 + local);
  auto d2of = [&](int x, int y) -> uint32_t {
    const int dx = x - px, dy = y - py;
    return (uint32_t)(dx * dx + dy * dy);
  };
  if (threadIdx.x == 0) {
    sh.nkeys = 0;
    sh.total = 0;
    sh.prefix = 0;
    sh.rank = k;
    sh.overflow = 0;
  }
  __syncthreads();
  // pass 1: every key into shared memory while it fits, and the count; one
  // shared atomic per warp and round.  Many points: the cell grid's rings
  // instead, which hold the k nearest.
  const int lane = threadIdx.x & 31;
  const bool grid = use_grid && s.cells != nullptr && n_res > kExhGridFrom;
  if (grid) grid_collect(s, px, py, k, n_res, sh, all, cap);
  // kPts points per thread and round: their loads (the point, then its
  // mirror bit) are all in flight together
  constexpr int kPts = 4;
  for (uint32_t e0 = 0; e0 < (grid ? 0u : n_res); e0 += kPts * blockDim.x) {
    uint32_t pt[kPts];
#pragma unroll
    for (int u = 0; u < kPts; ++u) {
      const uint32_t e = e0 + (uint32_t)u * blockDim.x + threadIdx.x;
      pt[u] = e < n_res ? __ldg(&s.resolved[e]) : 0xffffffffu;
    }
    // up to three keys per point in fixed slots (the point, its mirror
    // across x, its mirror across y), compacted through a bit mask
    int xs[3 * kPts], ys[3 * kPts];
    uint32_t vm = 0;
#pragma unroll
    for (int u = 0; u < kPts; ++u) {
      const int x = (int)(pt[u] % s.W), y = (int)(pt[u] / s.W);
      const bool mb = pt[u] != 0xffffffffu && s.tiling && mir_bit(s, (uint32_t)x, (uint32_t)y);
      xs[3 * u] = x;
      ys[3 * u] = y;
      xs[3 * u + 1] = x < s.x_l ? x + (int)s.W : x - (int)s.W;
      ys[3 * u + 1] = y;
      xs[3 * u + 2] = x;
      ys[3 * u + 2] = y < s.y_b ? y + (int)s.H : y - (int)s.H;
      if (pt[u] != 0xffffffffu) vm |= 1u << (3 * u);
      if (mb && (x < s.x_l || x > s.x_r)) vm |= 2u << (3 * u);
      if (mb && (y < s.y_b || y > s.y_t)) vm |= 4u << (3 * u);
    }
    const uint32_t cnt = (uint32_t)__popc(vm);
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    uint32_t base = 0;
    if (lane == 31) base = atomicAdd(&sh.total, incl);
    base = __shfl_sync(0xffffffffu, base, 31) + incl - cnt;
    uint32_t dor = 0;
#pragma unroll
    for (int i = 0; i < 3 * kPts; ++i) {
      if ((vm >> i) & 1u) {
        const uint32_t d2 = d2of(xs[i], ys[i]);
        dor |= d2;
        const uint32_t slot = base + (uint32_t)__popc(vm & ((1u << i) - 1u));
        if (slot < cap) all[slot] = nb_key(d2, xs[i], ys[i]);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dor |= __shfl_xor_sync(0xffffffffu, dor, o);
    if (lane == 0 && dor) atomicOr(&sh.prefix, dor);  // prefix holds the OR of all d2 until the select
  }
  __syncthreads();
  uint32_t total = sh.total;
  if (use_grid && !grid && total > cap && s.cells != nullptr) {
    __syncthreads();
    grid_collect(s, px, py, k, n_res, sh, all, cap);
    total = sh.total;
  }
  const unsigned long long *sorted;
  uint32_t n;
  if (total <= k || total <= cap) {
    // radix select over the shared keys, digits of up to 8 bits from the
    // highest significant bit of any d2 down, until the keys at or below the
    // selected digit's range fit the sort buffer (for points spread over an
    // area d2 is near uniform, so the first digit usually suffices); few
    // keys are sorted whole
    const uint32_t dor_all = sh.prefix;
    const int bits = dor_all ? 32 - __clz(dor_all) : 1;
    uint32_t D = 0xffffffffu;
    if (total > k && total > (uint32_t)kExhSortAll) {
      __syncthreads();
      if (threadIdx.x == 0) {
        sh.prefix = 0;
        sh.rank = k;
        sh.below = 0;
      }
      int hi = bits;  // the bits at and above hi are fixed by the prefix
      for (;;) {
        const int lo = max(hi - 8, 0);
        const uint32_t dmask = (1u << (hi - lo)) - 1u;
        for (int i = threadIdx.x; i < 256; i += blockDim.x) sh.hist[i] = 0;
        __syncthreads();
        const uint32_t prefix = sh.prefix;
        for (uint32_t i0 = 0; i0 < total; i0 += blockDim.x) {
          const uint32_t i = i0 + threadIdx.x;
          uint32_t bin = 0xffffffffu;
          if (i < total) {
            const uint32_t d2 = (uint32_t)(all[i] >> 32);
            if (hi >= 32 || (d2 >> hi) == (prefix >> hi)) bin = (d2 >> lo) & dmask;
          }
          // one shared atomic per distinct digit of the warp
          const uint32_t peers = __match_any_sync(0xffffffffu, bin);
          if (bin != 0xffffffffu && lane == __ffs(peers) - 1) atomicAdd(&sh.hist[bin], (uint32_t)__popc(peers));
        }
        __syncthreads();
        if (threadIdx.x < 32) {
          // warp 0: inclusive scan of 256 bins, 8 per lane
          uint32_t v[8], acc = 0;
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            acc += sh.hist[lane * 8 + q];
            v[q] = acc;
          }
          uint32_t off = acc;
#pragma unroll
          for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, off, o);
            if (lane >= o) off += t;
          }
          off -= acc;  // exclusive prefix of this lane's 8 bins
          const uint32_t rank = sh.rank, below = sh.below;
          __syncwarp();
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const uint32_t lo_c = off + (q ? v[q - 1] : 0u), hi_c = off + v[q];
            if (lo_c < rank && rank <= hi_c) {
              sh.prefix = prefix | ((uint32_t)(lane * 8 + q) << lo);
              sh.rank = rank - lo_c;
              sh.le = below + hi_c;  // keys at or below the digit's range
              sh.below = below + lo_c;
            }
          }
        }
        __syncthreads();
        if (lo == 0 || sh.le <= (uint32_t)kExhCap) {
          D = sh.prefix | ((1u << lo) - 1u);
          break;
        }
        hi = lo;
      }
      // keys at or below the cut, into the small buffer
      if (threadIdx.x == 0) sh.nkeys = 0;
      __syncthreads();
      for (uint32_t i = threadIdx.x; i < total; i += blockDim.x) {
        const unsigned long long key = all[i];
        if ((uint32_t)(key >> 32) <= D) {
          const uint32_t slot = atomicAdd(&sh.nkeys, 1u);
          if (slot < (uint32_t)kExhCap)
            sh.keys[slot] = key;
          else
            sh.overflow = 1;
        }
      }
    } else {
      if (threadIdx.x == 0) sh.nkeys = total;
      for (uint32_t i = threadIdx.x; i < total; i += blockDim.x) sh.keys[i] = all[i];
    }
    __syncthreads();
    if (sh.overflow) {
      if (threadIdx.x == 0) {
        set_err(s.err, kDevErrLimit);
        b.ncnt[local] = 0;
      }
      return 0;
    }
    n = sh.nkeys;
    sorted = sort_first(sh.keys, n, n < k ? n : k, all);
  } else {
    if (threadIdx.x == 0) {
      sh.prefix = 0;
      sh.rank = k;
    }
    __syncthreads();
    // radix select of the k-th smallest d2 over further passes
    for (int pass = 0; pass < 4; ++pass) {
      const int shift = 24 - 8 * pass;
      for (int i = threadIdx.x; i < 256; i += blockDim.x) sh.hist[i] = 0;
      __syncthreads();
      const uint32_t prefix = sh.prefix;
      for_points(s, n_res, [&](int x, int y) {
        const uint32_t d2 = d2of(x, y);
        const bool match = pass == 0 || ((d2 ^ prefix) >> (shift + 8)) == 0;
        if (match) atomicAdd(&sh.hist[(d2 >> shift) & 255u], 1u);
      });
      __syncthreads();
      if (threadIdx.x == 0) {
        uint32_t cum = 0, rank = sh.rank;
        for (int bk = 0; bk < 256; ++bk) {
          const uint32_t h = sh.hist[bk];
          if (cum + h >= rank) {
            sh.prefix = prefix | ((uint32_t)bk << shift);
            sh.rank = rank - cum;
            break;
          }
          cum += h;
        }
      }
      __syncthreads();
    }
    const uint32_t D = sh.prefix;
    for_points(s, n_res, [&](int x, int y) {
      const uint32_t d2 = d2of(x, y);
      if (d2 <= D) {
        const uint32_t slot = atomicAdd(&sh.nkeys, 1u);
        if (slot < (uint32_t)kExhCap)
          sh.keys[slot] = nb_key(d2, x, y);
        else
          sh.overflow = 1;
      }
    });
    __syncthreads();
    if (sh.overflow) {
      if (threadIdx.x == 0) {
        set_err(s.err, kDevErrLimit);
        b.ncnt[local] = 0;
      }
      return 0;
    }
    n = sh.nkeys;
    sorted = sort_first(sh.keys, n, n < k ? n : k, all);
  }
  const uint32_t nout = n < k ? n : k;
  int32_t *nbo = b.nbuf + (size_t)local * k;
  const uint32_t nb = b.i1 - b.i0;
  // the f64 distances from the coordinate tables, where something reads
  // them: every list of an inexact session, and the caller's weights when the
  // mean is not made here (exact sums derive the rest from the offsets; runs
  // with the k-NN made ahead have no coordinate tables)
  const bool want_d = !s.exact_sum || (with_mean && !mean_here);
  double x2 = 0.0, y2 = 0.0;
  if (want_d) {
    x2 = s.xdiv[px + s.xdiv_off];
    y2 = s.ydiv[py + s.ydiv_off];
  }
  unsigned long long part = 0;
  for (uint32_t i = threadIdx.x; i < nout; i += blockDim.x) {
    const unsigned long long key = sorted[i];
    const int x = (int)(key & 0xffffu) - 32768, y = (int)((key >> 16) & 0xffffu) - 32768;
    nbo[i] = pack_off(x - px, y - py);
    const double d = want_d ? neighbour_dist(s, px, py, x - px, y - py, x2, y2) : 0.0;
    if (s.exact_sum)
      part += exact_units(s, x - px, y - py);
    else
      b.dist[(size_t)i * nb + local] = d;
    if (with_mean) {
      sh.dist[i] = d;
      sh.nbo[i] = pack_off(x - px, y - py);
    }
  }
  if (s.exact_sum && mean_here) {
    // every item of the launch, fallback items included, gets its mean here
    part = warp_sum_units(part);
    if ((threadIdx.x & 31) == 0) sh.wsum[threadIdx.x >> 5] = part;
    __syncthreads();
    if (threadIdx.x == 0 && nout > 0) {
      unsigned long long sum = 0;
      for (uint32_t w = 0; w < blockDim.x / 32; ++w) sum += sh.wsum[w];
      b.mean[local] = exact_mean(s, sum, nout);
    }
  } else if (with_mean && mean_here) {
    __syncthreads();
    if (threadIdx.x == 0 && nout > 0) b.mean[local] = mean_chain(sh.dist, nout);
  }
  if (threadIdx.x == 0) b.ncnt[local] = nout;
  return nout;
}

// ---------------------------------------------------------------------------
// mean: thread per item (get_distances_to_k_neighs, ms.rs:417-423): the sum
// of the 4x-duplicated distance list in order, then / (4k).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mean_body(const SessionDev &s, const BatchDev &b, uint32_t vb) {
  const uint32_t nb = b.i1 - b.i0;
  const uint32_t local = vb * blockDim.x + threadIdx.x;
  if (local >= nb) return;
  const uint32_t nk = b.ncnt[local];
  if (nk == 0) return;
  // one item per lane: 32 chains share each f64 warp instruction, which on
  // GB300 costs the same whatever its active-lane count
  double sum = 0.0;
#pragma unroll 8
  for (uint32_t j = 0; j < nk; ++j) {
    const double d = b.dist[(size_t)j * nb + local];
    sum = __dadd_rn(sum, d);
    sum = __dadd_rn(sum, d);
    sum = __dadd_rn(sum, d);
    sum = __dadd_rn(sum, d);
  }
  b.mean[local] = __ddiv_rn(sum, (double)(nk * 4u));
}

// ---------------------------------------------------------------------------
// resolve: warp per item.
// ---------------------------------------------------------------------------
// Per-warp shared memory: one 16-byte record per neighbour
// {offset, own pattern texel, target-guide texel, weight bits}, then the
// candidates {x | y<<16} and {map | neg flag | source index << 16}.
struct WarpSmem {
  uint4 *nbr;
  uint32_t *cxy, *caux;
  float *term;   // candidate 0's neighbour terms
  int32_t *lin;  // neighbour offsets as texel offsets on the padded planes (dy * ppitch + dx)
};

__device__ __forceinline__ size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }

__host__ __device__ __forceinline__ size_t warp_smem_bytes(uint32_t k, uint32_t m) {
  const size_t kk = k ? k : 1;
  size_t b = kk * 16;                            // nbr
  b += (((kk + m) * 4 + 15) & ~(size_t)15) * 2;  // cxy, caux
  b += (kk * 4 + 15) & ~(size_t)15;              // term
  b += (kk * 4 + 15) & ~(size_t)15;              // lin
  return b;
}

__device__ __forceinline__ WarpSmem carve(unsigned char *base, uint32_t k, uint32_t m) {
  const size_t kk = k ? k : 1;
  WarpSmem w;
  unsigned char *p = base;
  w.nbr = (uint4 *)p;
  p += kk * 16;
  w.cxy = (uint32_t *)p;
  p += align16((kk + m) * 4);
  w.caux = (uint32_t *)p;
  p += align16((kk + m) * 4);
  w.term = (float *)p;
  p += align16(kk * 4);
  w.lin = (int32_t *)p;
  return w;
}

constexpr uint32_t kAuxNeg = 0x8000u;  // random candidate: neighbourhood c + (p - n)

__device__ __forceinline__ uint32_t texel(const uint32_t *lv, const MapDesc &md, int x, int y) {
  if ((unsigned)x < md.w && (unsigned)y < md.h) return __ldg(&lv[(size_t)y * md.w + x]);
  return kOutside;
}

// Sum of the four channel LUT terms in channel order, starting from acc.
// The byte offsets of the four entries come straight from the packed
// differences (d >> (8c - 2)) & 0x3fc.  kOpaque (StageDev::opaque): the
// alpha difference is always 0 and its term +-0, which leaves the sum as it
// is, so only the colour channels are looked up.
template <bool kOpaque = false>
__device__ __forceinline__ float lut4(const float *lut, uint32_t d, float acc) {
  const char *lb = (const char *)lut;
  acc = __fadd_rn(acc, *(const float *)(lb + ((d << 2) & 0x3fcu)));
  acc = __fadd_rn(acc, *(const float *)(lb + ((d >> 6) & 0x3fcu)));
  acc = __fadd_rn(acc, *(const float *)(lb + ((d >> 14) & 0x3fcu)));
  if (!kOpaque) acc = __fadd_rn(acc, *(const float *)(lb + ((d >> 22) & 0x3fcu)));
  return acc;
}
// The same with the stage's flag at run time (the alpha lookup predicated).
__device__ __forceinline__ float lut4r(const float *lut, uint32_t d, float acc, int opaque) {
  const char *lb = (const char *)lut;
  acc = __fadd_rn(acc, *(const float *)(lb + ((d << 2) & 0x3fcu)));
  acc = __fadd_rn(acc, *(const float *)(lb + ((d >> 6) & 0x3fcu)));
  acc = __fadd_rn(acc, *(const float *)(lb + ((d >> 14) & 0x3fcu)));
  if (!opaque) acc = __fadd_rn(acc, *(const float *)(lb + ((d >> 22) & 0x3fcu)));
  return acc;
}

// Cost of candidate c (better_match, ms.rs:1225-1288), abandoning once the
// partial sum reaches `bound`; bounds-checked gathers (out-of-bounds texels
// read Rgba(0,0,0,255)), issued four neighbours ahead.  Returns false when
// abandoned.  The terms are never negative, so partial sums never decrease
// and testing every fourth one, and the total, decides as the reference's
// test after every term does.
// kG = false compiles the guide terms out (sessions without guides).
template <bool kG = true>
__device__ __forceinline__ bool candidate_cost(const SessionDev &s, const StageDev &st, const WarpSmem &w,
                                               const float *lc, const float *lg, uint32_t nk, uint32_t cxy,
                                               uint32_t aux, float bound, float &out) {
  const uint32_t map = aux & 0x7fffu;
  const int sg = (aux & kAuxNeg) ? -1 : 1;
  const MapDesc md = s.maps[map];
  const uint32_t *lv = s.levels + md.off + (size_t)st.level * md.w * md.h;
  const int cx = (int)(cxy & 0xffffu), cy = (int)(cxy >> 16);
  const uint32_t *gv = nullptr;
  GuideDesc gd;
  if (kG && s.guided) {
    gd = s.gdesc[map];
    gv = s.guides + gd.off + (size_t)st.level * gd.w * gd.h;
  }
  float score = 0.0f;
  for (uint32_t j0 = 0; j0 < nk; j0 += 4) {
    uint4 nr[4];
    uint32_t t[4], gt[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      t[u] = kOutside;
      gt[u] = kOutside;
      if (j0 + u < nk) {
        nr[u] = w.nbr[j0 + u];
        const int qx = cx + sg * off_dx((int32_t)nr[u].x), qy = cy + sg * off_dy((int32_t)nr[u].x);
        if ((unsigned)qx < md.w && (unsigned)qy < md.h) t[u] = __ldg(&lv[(size_t)qy * md.w + qx]);
        if (kG && s.guided && (unsigned)qx < gd.w && (unsigned)qy < gd.h) gt[u] = __ldg(&gv[(size_t)qy * gd.w + qx]);
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (j0 + u >= nk) break;
      float nps = lut4(lc, __vabsdiffu4(nr[u].y, t[u]), 0.0f);
      if (kG && s.guided) nps = lut4(lg, __vabsdiffu4(nr[u].z, gt[u]), nps);
      score = __fadd_rn(score, __fmul_rn(nps, __uint_as_float(nr[u].w)));
    }
    if (score >= bound) return false;
  }
  out = score;
  return true;
}

// The same on the padded images, for items whose neighbour offsets all lie
// within kPad: no bounds checks, gathers issued four neighbours ahead.
template <bool kGuided, bool kOpaque>
__device__ __forceinline__ bool candidate_cost_padded_v(const SessionDev &s, const StageDev &st, const WarpSmem &w,
                                                      const float *lc, const float *lg, uint32_t nk, uint32_t cxy,
                                                      uint32_t aux, float bound, float &out) {
  const uint32_t map = aux & 0x7fffu;
  const int sg = (aux & kAuxNeg) ? -1 : 1;
  const MapDesc md = s.maps[map];
  const int cx = (int)(cxy & 0xffffu), cy = (int)(cxy >> 16);
  const size_t poff = md.poff + (size_t)st.level * md.pw * md.ph + (size_t)(cy + kPad) * md.pw + (cx + kPad);
  const uint32_t *base = s.plevels + poff;
  const uint32_t *gbase = kGuided ? s.pguides + poff : nullptr;
  float score = 0.0f;
  uint32_t j = 0;
  for (; j + 4 <= nk; j += 4) {
    uint4 nr[4];
    uint32_t t[4], gt[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      nr[u] = w.nbr[j + u];
      const int lin = sg * w.lin[j + u];
      t[u] = __ldg(base + lin);
      if (kGuided) gt[u] = __ldg(gbase + lin);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      float nps = lut4<kOpaque>(lc, __vabsdiffu4(nr[u].y, t[u]), 0.0f);
      if (kGuided) nps = lut4<kOpaque>(lg, __vabsdiffu4(nr[u].z, gt[u]), nps);
      score = __fadd_rn(score, __fmul_rn(nps, __uint_as_float(nr[u].w)));
    }
    if (score >= bound) return false;
  }
  for (; j < nk; ++j) {
    const uint4 nr = w.nbr[j];
    const int lin = sg * w.lin[j];
    float nps = lut4<kOpaque>(lc, __vabsdiffu4(nr.y, __ldg(base + lin)), 0.0f);
    if (kGuided) nps = lut4<kOpaque>(lg, __vabsdiffu4(nr.z, __ldg(gbase + lin)), nps);
    score = __fadd_rn(score, __fmul_rn(nps, __uint_as_float(nr.w)));
  }
  if (score >= bound) return false;
  out = score;
  return true;
}

// The loop in two versions, chosen per stage (a uniform branch).
template <bool kGuided>
__device__ __forceinline__ bool candidate_cost_padded(const SessionDev &s, const StageDev &st, const WarpSmem &w,
                                                      const float *lc, const float *lg, uint32_t nk, uint32_t cxy,
                                                      uint32_t aux, float bound, float &out) {
  if (st.opaque) return candidate_cost_padded_v<kGuided, true>(s, st, w, lc, lg, nk, cxy, aux, bound, out);
  return candidate_cost_padded_v<kGuided, false>(s, st, w, lc, lg, nk, cxy, aux, bound, out);
}

// Per-neighbour set-up of an item: weight (find_best_match, ms.rs:1198-1203,
// w = (f32) exp(-(d / mean))), own pattern texel and target-guide texel
// (ms.rs:1151-1181, wrapped when tiling), the record in shared memory, and
// the neighbour's coherence candidate (ms.rs:497-547): its source plus the
// shift to the centre, kept if valid.  Returns true for a valid candidate.
// The weight alone, w = (f32) exp(-(d / mean)) (find_best_match,
// ms.rs:1198-1203): the double-f32 path when it decides, else the exact f64
// one.
__device__ __forceinline__ float neighbour_weight(double dj, double avg, const double *tab, const float *tab_ff) {
  float wv;
  if (!ts_weight_ff(dj, avg, tab_ff, wv))
    wv = __double2float_rn(ts_exp64(-1.0 * ts_div_markstein(dj, avg, __drcp_rn(avg)), tab));
  return wv;
}

// Batch-start colour and state of output pixel p: the image, unless the
// previous batch step left its commit to this launch (BatchDev::prev_tag)
// and p is one of its pixels, whose values the shadow holds.  All loads are
// issued together.  Tags of this launch's own deferred pixels never equal
// prev_tag.
__device__ __forceinline__ void start_pixel(const SessionDev &s, const BatchDev &b, uint32_t p, bool want_colour,
                                            uint32_t &colour, uint4 &state) {
  colour = want_colour ? s.color[p] : 0u;
  state = s.state[p];
  if (b.prev_tag) {
    const uint4 h0 = s.shadow[2 * (size_t)p], h1 = s.shadow[2 * (size_t)p + 1];
    if (h0.x == b.prev_tag) {
      colour = want_colour ? h0.y : 0u;
      state = h1;
    }
  }
}

// Everything of neighbour_setup but the weight, which the record gets as wv.
template <bool kG = true>
__device__ __forceinline__ bool neighbour_records(const SessionDev &s, const StageDev &st, const BatchDev &b, int px,
                                                  int py, uint32_t j, int32_t off, float wv, const WarpSmem &w,
                                                  uint32_t &cxy, uint32_t &aux, int &maxoff, bool &bad_map) {
  const int W = (int)s.W, H = (int)s.H;
  maxoff = max(maxoff, max(abs(off_dx(off)), abs(off_dy(off))));
  const int nx = px + off_dx(off), ny = py + off_dy(off);
  int qx = nx, qy = ny;
  if (s.tiling) {
    qx = modi(nx, W);
    qy = modi(ny, H);
  }
  const bool inb = (unsigned)qx < s.W && (unsigned)qy < s.H;
  // colour and state of the neighbour (inb: (qx, qy) is its wrapped point)
  const int wx = modi(nx, W), wy = modi(ny, H);
  uint32_t pat;
  uint4 sv;
  start_pixel(s, b, (uint32_t)wy * s.W + (uint32_t)wx, inb, pat, sv);
  if (!inb) pat = kOutside;
  uint32_t gpat = 0;
  if (kG && s.guided) gpat = inb ? __ldg(&s.tguide[(size_t)st.level * s.W * s.H + (size_t)qy * s.W + qx]) : kOutside;
  w.nbr[j] = make_uint4((uint32_t)off, pat, gpat, __float_as_uint(wv));
  w.lin[j] = off_dy(off) * (int)s.ppitch + off_dx(off);
  const uint32_t map = sv.z;
  if (map >= s.n_maps) {
    bad_map = true;
    return false;
  }
  const int ccx = (int)(sv.x & 0xffffu) + (px - nx);
  const int ccy = (int)(sv.x >> 16) + (py - ny);
  if (!coord_valid(s, s.maps[map], ccx, ccy)) return false;
  cxy = (uint32_t)ccx | ((uint32_t)ccy << 16);
  aux = map | (j << 16);
  return true;
}

template <bool kG = true>
__device__ __forceinline__ bool neighbour_setup(const SessionDev &s, const StageDev &st, const BatchDev &b,
                                                uint32_t local, uint32_t nb, int px, int py, uint32_t j, int32_t off,
                                                double avg, const double *tab, const float *tab_ff,
                                                const WarpSmem &w, uint32_t &cxy, uint32_t &aux, bool &nan_w,
                                                int &maxoff, bool &bad_map) {
  const double d = s.exact_sum ? exact_dist(s, off) : b.dist[(size_t)j * nb + local];
  const float wv = neighbour_weight(d, avg, tab, tab_ff);
  nan_w |= (wv != wv);
  return neighbour_records<kG>(s, st, b, px, py, j, off, wv, w, cxy, aux, maxoff, bad_map);
}

// Candidate 0's exact score (better_match, ms.rs:1225-1288, with no bound):
// lane j of a group of G lanes (a warp, or a CTA's warp) computes the terms
// nps_j * w_j of neighbours j, j + G, ..., lane 0 sums them in order; every
// lane returns the sum.
template <int G, bool kG = true>
__device__ __forceinline__ float candidate0_score(const SessionDev &s, const StageDev &st, const WarpSmem &w,
                                                  const float *lc, const float *lg, uint32_t nk, int gl,
                                                  uint32_t gmask) {
  const uint32_t cxy0 = w.cxy[0], aux0 = w.caux[0];
  const uint32_t map = aux0 & 0x7fffu;
  const bool neg = (aux0 & kAuxNeg) != 0;
  const MapDesc md = s.maps[map];
  const uint32_t *lv = s.levels + md.off + (size_t)st.level * md.w * md.h;
  const int cx = (int)(cxy0 & 0xffffu), cy = (int)(cxy0 >> 16);
  for (uint32_t j = gl; j < nk; j += G) {
    const uint4 nr = w.nbr[j];
    int dx = off_dx((int32_t)nr.x), dy = off_dy((int32_t)nr.x);
    if (neg) {
      dx = -dx;
      dy = -dy;
    }
    const int qx = cx + dx, qy = cy + dy;
    float nps = lut4(lc, __vabsdiffu4(nr.y, texel(lv, md, qx, qy)), 0.0f);
    if (kG && s.guided) {
      const GuideDesc gd = s.gdesc[map];
      const uint32_t *gv = s.guides + gd.off + (size_t)st.level * gd.w * gd.h;
      uint32_t gt = kOutside;
      if ((unsigned)qx < gd.w && (unsigned)qy < gd.h) gt = __ldg(&gv[(size_t)qy * gd.w + qx]);
      nps = lut4(lg, __vabsdiffu4(nr.z, gt), nps);
    }
    w.term[j] = __fmul_rn(nps, __uint_as_float(nr.w));
  }
  __syncwarp(gmask);
  float sc = 0.0f;
  if (gl == 0)
    for (uint32_t j = 0; j < nk; ++j) sc = __fadd_rn(sc, w.term[j]);
  return __shfl_sync(gmask, sc, 0, G);
}

// The reference's sequential find_best_match (ms.rs:1184-1221), for stages or
// items with non-finite costs, where early exit and argmin need its exact
// comparison sequence.  One thread.
template <bool kG = true>
__device__ void sequential_best(const SessionDev &s, const StageDev &st, const WarpSmem &w, const float *lc,
                                const float *lg, uint32_t nk, uint32_t nc, float &best_s, uint32_t &best_i) {
  best_s = FLT_MAX;
  best_i = 0;
  for (uint32_t c = 0; c < nc; ++c) {
    const uint32_t aux = w.caux[c];
    const uint32_t map = aux & 0x7fffu;
    const bool neg = (aux & kAuxNeg) != 0;
    const MapDesc md = s.maps[map];
    const uint32_t *lv = s.levels + md.off + (size_t)st.level * md.w * md.h;
    const int cx = (int)(w.cxy[c] & 0xffffu), cy = (int)(w.cxy[c] >> 16);
    float score = 0.0f;
    bool better = true;
    for (uint32_t j = 0; j < nk; ++j) {
      const uint4 nr = w.nbr[j];
      int dx = off_dx((int32_t)nr.x), dy = off_dy((int32_t)nr.x);
      if (neg) {
        dx = -dx;
        dy = -dy;
      }
      const int qx = cx + dx, qy = cy + dy;
      float nps = lut4(lc, __vabsdiffu4(nr.y, texel(lv, md, qx, qy)), 0.0f);
      if (kG && s.guided) {
        const GuideDesc gd = s.gdesc[map];
        const uint32_t *gv = s.guides + gd.off + (size_t)st.level * gd.w * gd.h;
        uint32_t gt = kOutside;
        if ((unsigned)qx < gd.w && (unsigned)qy < gd.h) gt = gv[(size_t)qy * gd.w + qx];
        nps = lut4(lg, __vabsdiffu4(nr.z, gt), nps);
      }
      score = __fadd_rn(score, __fmul_rn(nps, __uint_as_float(nr.w)));
      if (score >= best_s) {
        better = false;
        break;
      }
    }
    if (better) {
      best_s = score;
      best_i = c;
    }
  }
}

__device__ __forceinline__ void add_cell_point(const SessionDev &s, int x, int y) {
  atomicAdd(&s.cells[(size_t)((y - s.coy) / kCell) * s.cgw + (x - s.cox) / kCell], 1u);
}

// update + flush_resolved of one item (ms.rs:296-377): its colour and state,
// its place in the resolved list, the bitmap, mirrors and cell counts.
__device__ __forceinline__ void commit_item(const SessionDev &s, const StageDev &st, const BatchDev &b, uint32_t local,
                                            const Result &r, bool count_evals = true) {
  const uint32_t p = r.pixel;
  if (r.cmap >= s.n_maps || p >= s.W * s.H) {
    set_err(s.err, kDevErrIndex);
    return;
  }
  const MapDesc md = s.maps[r.cmap];
  const uint32_t sx = r.srcxy & 0xffffu, sy = r.srcxy >> 16;
  if (sx >= md.w || sy >= md.h) {
    set_err(s.err, kDevErrIndex);
    return;
  }
  s.state[p] = make_uint4(r.srcxy, r.idp, r.idm, r.cmap);
  s.color[p] = s.levels[md.off + (size_t)st.level * md.w * md.h + (size_t)sy * md.w + sx];
  if (count_evals && r.ncand) atomicAdd(s.evals, (unsigned long long)r.ncand);
  if (r.flags & kResAppend) {
    const uint32_t item = b.i0 + local;
    const uint32_t pos = b.n_res + (item - b.append_from);
    s.rscore[pos] = r.score;
    if (s.rank) return;  // k-NN made ahead: k_tree_append entered the point already
    s.resolved[pos] = p;
    const uint32_t x = p % s.W, y = p / s.W;
    atomicOr(&s.occ[(size_t)y * s.wpr + (x >> 5)], 1u << (x & 31));
    add_cell_point(s, (int)x, (int)y);
    if (s.tiling && (r.flags & kResMirrors)) {
      atomicOr(&s.mir[(size_t)y * s.wpr + (x >> 5)], 1u << (x & 31));
      // the tree's mirror copies (flush_resolved, ms.rs:306-328)
      if ((int)x < s.x_l)
        add_cell_point(s, (int)x + (int)s.W, (int)y);
      else if ((int)x > s.x_r)
        add_cell_point(s, (int)x - (int)s.W, (int)y);
      if ((int)y < s.y_b)
        add_cell_point(s, (int)x, (int)y + (int)s.H);
      else if ((int)y > s.y_t)
        add_cell_point(s, (int)x, (int)y - (int)s.H);
    }
  }
}

// An item's result: committed at once when the batch holds only new items
// (b.fused_commit: no item of the batch is in the tree, so no other item
// reads its pixel, state or bit during the batch), else kept for k_commit.
__device__ __forceinline__ void emit_result(const SessionDev &s, const StageDev &st, const BatchDev &b, uint32_t local,
                                            const Result &r) {
  if (b.fused_commit) {
    commit_item(s, st, b, local, r);
  } else {
    b.res[local] = r;
    if (b.defer_tag && r.cmap < s.n_maps && r.pixel < s.W * s.H) {
      // what the commit will write, for the next step's readers (start_pixel)
      const MapDesc md = s.maps[r.cmap];
      const uint32_t sx = r.srcxy & 0xffffu, sy = r.srcxy >> 16;
      if (sx < md.w && sy < md.h) {
        const uint32_t col = s.levels[md.off + (size_t)st.level * md.w * md.h + (size_t)sy * md.w + sx];
        s.shadow[2 * (size_t)r.pixel] = make_uint4(b.defer_tag, col, 0u, 0u);
        s.shadow[2 * (size_t)r.pixel + 1] = make_uint4(r.srcxy, r.idp, r.idm, r.cmap);
      }
    }
  }
}

// The winning candidate as an update (ms.rs:976-1001): source coordinate and
// map, patch id (the neighbour's for coherence candidates, the example flat
// index for random ones), score.
__device__ void write_result(const SessionDev &s, const StageDev &st, const WarpSmem &w, const BatchDev &b,
                             uint32_t local, uint32_t pixel, int px, int py, bool is_new, uint32_t nc, float best_s,
                             uint32_t best_i) {
  const uint32_t aux = w.caux[best_i];
  const uint32_t map = aux & 0x7fffu;
  const uint32_t cxy = w.cxy[best_i];
  uint32_t idp;
  if (aux & kAuxNeg) {
    idp = (cxy >> 16) * s.maps[map].w + (cxy & 0xffffu);
  } else {
    const uint32_t j = aux >> 16;
    const int32_t off = (int32_t)w.nbr[j].x;
    const int wx = modi(px + off_dx(off), (int)s.W), wy = modi(py + off_dy(off), (int)s.H);
    uint32_t unused;
    uint4 sv;
    start_pixel(s, b, (uint32_t)wy * s.W + (uint32_t)wx, false, unused, sv);
    idp = sv.y;
  }
  Result r;
  r.pixel = pixel;
  r.srcxy = cxy;
  r.idp = idp;
  r.idm = map;
  r.cmap = map;
  r.flags = (is_new ? kResAppend : 0u) | kResMirrors;
  r.score = best_s;
  r.ncand = nc;
  emit_result(s, st, b, local, r);
}

// Result for an item with no resolved neighbour: resolve_at_random with the
// stage seed, appended without tiling mirrors (ms.rs:1002-1010, 473).
__device__ void write_random_result(const SessionDev &s, const StageDev &st, const BatchDev &b, uint32_t local,
                                    uint32_t pixel) {
  Pcg32 g = pcg_from_u64(st.stage_seed);
  uint64_t map64 = 0;
  uint32_t x = 0, y = 0;
  bool ok = gen_range_u64_bounded(g, s.n_maps, 256, map64);
  const uint32_t map = ok ? (uint32_t)map64 : 0u;
  const MapDesc md = s.maps[map];
  g = pcg_from_u64(st.stage_seed);
  ok = ok && gen_range_u32_bounded(g, md.w, 256, x);
  g = pcg_from_u64(st.stage_seed);
  ok = ok && gen_range_u32_bounded(g, md.h, 256, y);
  if (!ok) set_err(s.err, kDevErrNoSample);
  Result r;
  r.pixel = pixel;
  r.srcxy = x | (y << 16);
  r.idp = pixel;
  r.idm = map;
  r.cmap = map;
  r.flags = kResAppend;
  r.score = 0.0f;
  r.ncand = 0;
  emit_result(s, st, b, local, r);
}

// A result that commit skips (an invalid map id was met; the reference
// panics there).
__device__ void write_bad_result(const SessionDev &s, const StageDev &st, const BatchDev &b, uint32_t local,
                                 uint32_t pixel) {
  set_err(s.err, kDevErrIndex);
  Result r;
  r.pixel = pixel;
  r.srcxy = 0;
  r.idp = 0;
  r.idm = 0;
  r.cmap = 0xffffffffu;
  r.flags = 0;
  r.score = 0.0f;
  r.ncand = 0;
  emit_result(s, st, b, local, r);
}

// kLean: sessions without guides only (the guide terms compiled out, which
// lets the multi-session kernel run more blocks per SM).
template <bool kLean>
__device__ __forceinline__ void resolve_body(const SessionDev &s, const StageDev &st, const BatchDev &b, uint32_t vb,
                                             uint32_t vg) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double tab[64];
  __shared__ float tab_ff[128];
  float *lc = (float *)smem;
  float *lg = lc + 256;
  for (int i = threadIdx.x; i < 512; i += blockDim.x) lc[i] = st.lut[i];
  if (threadIdx.x < 64) tab[threadIdx.x] = g_exp2_64[threadIdx.x];
  tab_ff[threadIdx.x] = g_exp2_ff[threadIdx.x];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  const WarpSmem w = carve(smem + 2048 + (size_t)warp * warp_smem_bytes(s.k, s.m), s.k, s.m);
  __syncthreads();
  const uint32_t nb = b.i1 - b.i0;
  const uint32_t grid_warps = vg * kResolveWarps;
  // the next item of this warp: the grid stride, or (BatchDev::work_ctr)
  // the next one nobody has taken once every warp has had its first
  auto next_item = [&](uint32_t cur) -> uint32_t {
    if (!b.work_ctr) return cur + grid_warps;
    uint32_t v = 0;
    if (lane == 0) v = atomicAdd(b.work_ctr, 1u) + grid_warps;
    return __shfl_sync(0xffffffffu, v, 0);
  };
  for (uint32_t local = vb * kResolveWarps + warp; local < nb; local = next_item(local)) {
    const uint32_t item = b.i0 + local;
    const uint32_t pixel = st.items[item];
    const int px = (int)(pixel % s.W), py = (int)(pixel / s.W);
    const bool is_new = item >= st.redo;
    const uint32_t nk = s.k ? b.ncnt[local] : 0u;
    Result r;
    r.pixel = pixel;
    r.ncand = 0;
    if (nk == 0) {
      // no resolved neighbours: resolve_at_random with the stage seed, kept
      // in the resolved list without tiling mirrors (ms.rs:1002-1010, 473)
      if (lane == 0) write_random_result(s, st, b, local, pixel);
      continue;
    }
    const int32_t *nbo = b.nbuf + (size_t)local * s.k;
    const double avg = b.mean[local];
    // neighbours: offsets, weights, own pattern, coherence candidates.
    // With `dedupe`, a coherence candidate equal to an earlier one (same
    // source and map) is left out: its cost equals the earlier one's, so it
    // can neither beat it nor tie it with a lower index, and the reference's
    // winner is the same without it.  The exact sequential form for
    // non-finite costs keeps every candidate.
    bool nan_w = false;
    int maxoff = 0;
    uint32_t ncoh = 0, ncoh_all = 0;
    bool bad_map = false;
    auto coherence = [&](bool dedupe) {
      ncoh = ncoh_all = 0;
      for (uint32_t j0 = 0; j0 < nk; j0 += kWarp) {
        const uint32_t j = j0 + lane;
        bool valid = false;
        uint32_t cxy = 0, aux = 0;
        if (j < nk)
          valid = neighbour_setup<!kLean>(s, st, b, local, nb, px, py, j, nbo[j], avg, tab, tab_ff, w, cxy, aux, nan_w,
                                  maxoff, bad_map);
        bool keep = valid;
        if (dedupe) {
          const unsigned long long key =
              valid ? (((unsigned long long)(aux & 0x7fffu) << 32) | cxy) : ((1ull << 63) | (unsigned long long)lane);
          if (__match_any_sync(0xffffffffu, key) & lt) keep = false;  // a lower lane holds it
          for (uint32_t i = 0; keep && i < ncoh; ++i)
            if (w.cxy[i] == cxy && (w.caux[i] & 0x7fffu) == (aux & 0x7fffu)) keep = false;
        }
        ncoh_all += __popc(__ballot_sync(0xffffffffu, valid));
        const uint32_t bal = __ballot_sync(0xffffffffu, keep);
        if (keep) {
          const uint32_t slot = ncoh + __popc(bal & lt);
          w.cxy[slot] = cxy;
          w.caux[slot] = aux;
        }
        ncoh += __popc(bal);
        __syncwarp();
      }
    };
    coherence(!st.slow_lut);
    if (!st.slow_lut && __any_sync(0xffffffffu, nan_w)) coherence(false);
    if (__any_sync(0xffffffffu, bad_map)) {
      // the reference panics on this index; record the error and leave the
      // pixel untouched (commit skips results with an invalid map)
      if (lane == 0) write_bad_result(s, st, b, local, pixel);
      continue;
    }
    // random candidates after the coherence ones
    const uint2 *rc = st.rcand + (size_t)item * s.m;
    for (uint32_t t = lane; t < s.m; t += kWarp) {
      const uint2 v = use_rcand(s, rc[t]);
      w.cxy[ncoh + t] = v.x;
      w.caux[ncoh + t] = v.y | kAuxNeg | (t << 16);
    }
    const bool slow = st.slow_lut || __any_sync(0xffffffffu, nan_w);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) maxoff = max(maxoff, __shfl_xor_sync(0xffffffffu, maxoff, o));
    const bool padded = maxoff <= kPad && !s.guide_dims_differ;
    __syncwarp();
    const uint32_t nc = ncoh + s.m;
    float best_s = FLT_MAX;
    uint32_t best_i = 0;
    if (!slow) {
      // candidate 0 first: its terms on all lanes, their in-order sum on
      // lane 0; it wins ties with every later candidate, so the rest run
      // against min(S_0, f32::MAX) from the start
      {
        const float s0 = candidate0_score<kWarp, !kLean>(s, st, w, lc, lg, nk, lane, 0xffffffffu);
        if (s0 < best_s) best_s = s0;
      }
      for (uint32_t base = 1; base < nc; base += kWarp) {
        const uint32_t c = base + lane;
        float sc = 0.0f;
        bool alive = false;
        if (c < nc) {
          if (!padded)
            alive = candidate_cost<!kLean>(s, st, w, lc, lg, nk, w.cxy[c], w.caux[c], best_s, sc);
          else if (!kLean && s.guided)
            alive = candidate_cost_padded<true>(s, st, w, lc, lg, nk, w.cxy[c], w.caux[c], best_s, sc);
          else
            alive = candidate_cost_padded<false>(s, st, w, lc, lg, nk, w.cxy[c], w.caux[c], best_s, sc);
        }
        float v = alive ? sc : __int_as_float(0x7f800000);
        uint32_t idx = alive ? c : 0xffffffffu;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const float ov = __shfl_xor_sync(0xffffffffu, v, o);
          const uint32_t oi = __shfl_xor_sync(0xffffffffu, idx, o);
          if (ov < v || (ov == v && oi < idx)) {
            v = ov;
            idx = oi;
          }
        }
        if (idx != 0xffffffffu && v < best_s) {
          best_s = v;
          best_i = idx;
        }
      }
    } else if (lane == 0) {
      sequential_best<!kLean>(s, st, w, lc, lg, nk, nc, best_s, best_i);
    }
    if (lane == 0) write_result(s, st, w, b, local, pixel, px, py, is_new, ncoh_all + s.m, best_s, best_i);
  }
}


// ---------------------------------------------------------------------------
// resolve, team form: one CTA of T threads per item, one candidate per
// thread.  Candidate 0's exact score is computed first (its neighbour terms
// in parallel, their in-order sum on one thread); every other candidate then
// runs against min(S_0, its thread's earlier results) and stops as soon as
// its partial sum reaches that bound; a block-wide first-index argmin picks
// the winner.  The first strict minimum of the reference never stops early
// (every bound it meets is larger, or equal with a later index), so the
// result is the reference's.  Latency per item is about one candidate's
// evaluation, which suits batches too small to fill the GPU with warps.
// ---------------------------------------------------------------------------
template <int T, bool kFull>
__device__ __forceinline__ void resolve_team_body(const SessionDev &s, const StageDev &st, const BatchDev &b,
                                                  uint32_t vb, uint32_t vg) {
  constexpr int NW = T / 32;
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double tab[64];
  __shared__ float tab_ff[128];
  __shared__ uint32_t wcnt[NW];
  __shared__ float red_s[NW];
  __shared__ uint32_t red_i[NW];
  __shared__ int sh_flags, sh_maxoff;
  __shared__ float sh_s0;
  float *lc = (float *)smem;
  float *lg = lc + 256;
  for (int i = threadIdx.x; i < 512; i += T) lc[i] = st.lut[i];
  for (int i = threadIdx.x; i < 64; i += T) tab[i] = g_exp2_64[i];
  for (int i = threadIdx.x; i < 128; i += T) tab_ff[i] = g_exp2_ff[i];
  const WarpSmem w = carve(smem + 2048, s.k, s.m);
  float *term = (float *)(smem + 2048 + warp_smem_bytes(s.k, s.m));
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t nb = b.i1 - b.i0;
  __syncthreads();
  for (uint32_t local = vb; local < nb; local += vg) {
    const uint32_t item = b.i0 + local;
    const uint32_t pixel = st.items[item];
    const int px = (int)(pixel % s.W), py = (int)(pixel / s.W);
    const bool is_new = item >= st.redo;
    const uint32_t nk = s.k ? b.ncnt[local] : 0u;
    if (nk == 0) {
      if (tid == 0) write_random_result(s, st, b, local, pixel);
      continue;
    }
    if (tid == 0) {
      sh_flags = 0;
      sh_maxoff = 0;
    }
    __syncthreads();
    const int32_t *nbo = b.nbuf + (size_t)local * s.k;
    const double avg = b.mean[local];
    bool nan_w = false, bad_map = false;
    int maxoff = 0;
    uint32_t ncoh = 0;
    for (uint32_t j0 = 0; j0 < nk; j0 += T) {
      const uint32_t j = j0 + tid;
      bool valid = false;
      uint32_t cxy = 0, aux = 0;
      if (j < nk)
        valid = neighbour_setup(s, st, b, local, nb, px, py, j, nbo[j], avg, tab, tab_ff, w, cxy, aux, nan_w,
                                maxoff, bad_map);
      // order-preserving compaction of the valid coherence candidates
      const uint32_t bal = __ballot_sync(0xffffffffu, valid);
      if (lane == 0) wcnt[warp] = __popc(bal);
      __syncthreads();
      uint32_t base = ncoh, total = 0;
#pragma unroll
      for (int i = 0; i < NW; ++i) {
        if (i < warp) base += wcnt[i];
        total += wcnt[i];
      }
      if (valid) {
        const uint32_t slot = base + __popc(bal & lt);
        w.cxy[slot] = cxy;
        w.caux[slot] = aux;
      }
      ncoh += total;
      __syncthreads();
    }
    if (nan_w) atomicOr(&sh_flags, 1);
    if (bad_map) atomicOr(&sh_flags, 2);
    if (maxoff) atomicMax(&sh_maxoff, maxoff);
    const uint2 *rc = st.rcand + (size_t)item * s.m;
    for (uint32_t t = tid; t < s.m; t += T) {
      const uint2 v = use_rcand(s, rc[t]);
      w.cxy[ncoh + t] = v.x;
      w.caux[ncoh + t] = v.y | kAuxNeg | (t << 16);
    }
    __syncthreads();
    if (sh_flags & 2) {
      if (tid == 0) write_bad_result(s, st, b, local, pixel);
      __syncthreads();
      continue;
    }
    const bool slow = st.slow_lut || (sh_flags & 1);
    const bool padded = sh_maxoff <= kPad && !s.guide_dims_differ;
    const uint32_t nc = ncoh + s.m;
    float best_s = FLT_MAX;
    uint32_t best_i = 0;
    if (!slow && kFull && padded) {
      // every term nps(c, j) * w_j in parallel, then each candidate's
      // in-order sum on one thread: the reference's scores, all of them.
      // Padded planes: each candidate's plane offset once, then eight texel
      // loads in flight per thread before their terms are formed.
      unsigned long long *cb = (unsigned long long *)(term + (((size_t)nk * nc + 1) & ~(size_t)1));
      for (uint32_t c = tid; c < nc; c += T) {
        const uint32_t cxy = w.cxy[c], aux = w.caux[c];
        const MapDesc md = s.maps[aux & 0x7fffu];
        const unsigned long long off = md.poff + (unsigned long long)st.level * md.pw * md.ph +
                                       (unsigned long long)((cxy >> 16) + kPad) * md.pw + ((cxy & 0xffffu) + kPad);
        cb[c] = off | ((aux & kAuxNeg) ? (1ull << 63) : 0ull);
      }
      __syncthreads();
      const uint32_t total = nc * nk;
      for (uint32_t i0 = tid; i0 < total; i0 += 8 * T) {
        uint32_t tx[8], gx[8], ii[8], jj[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const uint32_t i = i0 + (uint32_t)u * T;
          ii[u] = i;
          if (i < total) {
            const uint32_t c = i / nk;
            jj[u] = i - c * nk;
            const unsigned long long v = cb[c];
            const int lin = (v >> 63) ? -w.lin[jj[u]] : w.lin[jj[u]];
            const size_t off = (size_t)(v & 0x7fffffffffffffffull) + lin;
            tx[u] = __ldg(s.plevels + off);
            if (s.guided) gx[u] = __ldg(s.pguides + off);
          }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          if (ii[u] < total) {
            const uint4 nr = w.nbr[jj[u]];
            float nps = lut4r(lc, __vabsdiffu4(nr.y, tx[u]), 0.0f, st.opaque);
            if (s.guided) nps = lut4r(lg, __vabsdiffu4(nr.z, gx[u]), nps, st.opaque);
            term[ii[u]] = __fmul_rn(nps, __uint_as_float(nr.w));
          }
        }
      }
    }
    if (!slow && kFull && !padded) {
      // the same with bounds-checked gathers (far neighbours or guides of
      // other sizes); consecutive threads take consecutive neighbours of one
      // candidate
      uint32_t c = tid / nk, j = tid - c * nk;
      const uint32_t dc = T / nk, dj = T - dc * nk;
      for (uint32_t i = tid; i < nc * nk; i += T) {
        const uint32_t cxy = w.cxy[c], aux = w.caux[c];
        const uint32_t map = aux & 0x7fffu;
        const int sg = (aux & kAuxNeg) ? -1 : 1;
        const MapDesc md = s.maps[map];
        const uint4 nr = w.nbr[j];
        const int qx = (int)(cxy & 0xffffu) + sg * off_dx((int32_t)nr.x);
        const int qy = (int)(cxy >> 16) + sg * off_dy((int32_t)nr.x);
        uint32_t t = kOutside;
        if ((unsigned)qx < md.w && (unsigned)qy < md.h)
          t = __ldg(&s.levels[md.off + (size_t)st.level * md.w * md.h + (size_t)qy * md.w + qx]);
        float nps = lut4(lc, __vabsdiffu4(nr.y, t), 0.0f);
        if (s.guided) {
          const GuideDesc gd = s.gdesc[map];
          uint32_t gt = kOutside;
          if ((unsigned)qx < gd.w && (unsigned)qy < gd.h)
            gt = __ldg(&s.guides[gd.off + (size_t)st.level * gd.w * gd.h + (size_t)qy * gd.w + qx]);
          nps = lut4(lg, __vabsdiffu4(nr.z, gt), nps);
        }
        term[i] = __fmul_rn(nps, __uint_as_float(nr.w));
        c += dc;
        j += dj;
        if (j >= nk) {
          j -= nk;
          ++c;
        }
      }
    }
    if (!slow && kFull) {
      __syncthreads();
      float my_s = FLT_MAX;
      uint32_t my_i = 0xffffffffu;
      for (uint32_t cc = tid; cc < nc; cc += T) {
        float sc = 0.0f;
        const float *tc = term + (size_t)cc * nk;
        for (uint32_t jj = 0; jj < nk; ++jj) sc = __fadd_rn(sc, tc[jj]);
        if (sc < my_s) {  // first strict minimum among this thread's candidates
          my_s = sc;
          my_i = cc;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, my_s, o);
        const uint32_t oi = __shfl_xor_sync(0xffffffffu, my_i, o);
        if (ov < my_s || (ov == my_s && oi < my_i)) {
          my_s = ov;
          my_i = oi;
        }
      }
      if (lane == 0) {
        red_s[warp] = my_s;
        red_i[warp] = my_i;
      }
      __syncthreads();
      best_s = red_s[0];
      best_i = red_i[0];
      for (int i = 1; i < NW; ++i) {
        if (red_s[i] < best_s || (red_s[i] == best_s && red_i[i] < best_i)) {
          best_s = red_s[i];
          best_i = red_i[i];
        }
      }
      if (best_i == 0xffffffffu) {  // no score below f32::MAX: the reference keeps candidate 0
        best_s = FLT_MAX;
        best_i = 0;
      }
    } else if (!slow) {
      // S_0: candidate 0's terms nps_j * w_j in parallel, summed in order
      {
        const uint32_t cxy0 = w.cxy[0], aux0 = w.caux[0];
        const uint32_t map = aux0 & 0x7fffu;
        const bool neg = (aux0 & kAuxNeg) != 0;
        const MapDesc md = s.maps[map];
        const uint32_t *lv = s.levels + md.off + (size_t)st.level * md.w * md.h;
        const int cx = (int)(cxy0 & 0xffffu), cy = (int)(cxy0 >> 16);
        for (uint32_t j = tid; j < nk; j += T) {
          const uint4 nr = w.nbr[j];
          int dx = off_dx((int32_t)nr.x), dy = off_dy((int32_t)nr.x);
          if (neg) {
            dx = -dx;
            dy = -dy;
          }
          const int qx = cx + dx, qy = cy + dy;
          float nps = lut4(lc, __vabsdiffu4(nr.y, texel(lv, md, qx, qy)), 0.0f);
          if (s.guided) {
            const GuideDesc gd = s.gdesc[map];
            const uint32_t *gv = s.guides + gd.off + (size_t)st.level * gd.w * gd.h;
            uint32_t gt = kOutside;
            if ((unsigned)qx < gd.w && (unsigned)qy < gd.h) gt = __ldg(&gv[(size_t)qy * gd.w + qx]);
            nps = lut4(lg, __vabsdiffu4(nr.z, gt), nps);
          }
          term[j] = __fmul_rn(nps, __uint_as_float(nr.w));
        }
        __syncthreads();
        if (tid == 0) {
          float sc = 0.0f;
          for (uint32_t j = 0; j < nk; ++j) sc = __fadd_rn(sc, term[j]);
          sh_s0 = sc;
        }
        __syncthreads();
      }
      float my_s = sh_s0;
      uint32_t my_i = 0;
      for (uint32_t c = 1 + tid; c < nc; c += T) {
        float sc;
        bool alive;
        if (!padded)
          alive = candidate_cost(s, st, w, lc, lg, nk, w.cxy[c], w.caux[c], my_s, sc);
        else if (s.guided)
          alive = candidate_cost_padded<true>(s, st, w, lc, lg, nk, w.cxy[c], w.caux[c], my_s, sc);
        else
          alive = candidate_cost_padded<false>(s, st, w, lc, lg, nk, w.cxy[c], w.caux[c], my_s, sc);
        if (alive) {
          my_s = sc;
          my_i = c;
        }
      }
      // first index of the minimum over the block
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, my_s, o);
        const uint32_t oi = __shfl_xor_sync(0xffffffffu, my_i, o);
        if (ov < my_s || (ov == my_s && oi < my_i)) {
          my_s = ov;
          my_i = oi;
        }
      }
      if (lane == 0) {
        red_s[warp] = my_s;
        red_i[warp] = my_i;
      }
      __syncthreads();
      best_s = red_s[0];
      best_i = red_i[0];
      for (int i = 1; i < NW; ++i) {
        if (red_s[i] < best_s || (red_s[i] == best_s && red_i[i] < best_i)) {
          best_s = red_s[i];
          best_i = red_i[i];
        }
      }
    } else if (tid == 0) {
      sequential_best(s, st, w, lc, lg, nk, nc, best_s, best_i);
    }
    if (tid == 0) write_result(s, st, w, b, local, pixel, px, py, is_new, nc, best_s, best_i);
    __syncthreads();
  }
}

// update + flush_resolved for a batch (ms.rs:296-377): one thread per item.

__device__ __forceinline__ void commit_body(const SessionDev &s, const StageDev &st, const BatchDev &b, uint32_t vb) {
  const uint32_t local = vb * blockDim.x + threadIdx.x;
  const uint32_t nb = b.i1 - b.i0;
  if (local >= nb) return;
  commit_item(s, st, b, local, b.res[local]);
}

// next_pyramid_level (ms.rs:687-700)
__device__ __forceinline__ void level_switch_body(const SessionDev &s, uint32_t level, uint32_t n_res, uint32_t vb) {
  const uint32_t e = vb * blockDim.x + threadIdx.x;
  if (e >= n_res) return;
  const uint32_t p = s.resolved[e];
  const uint4 sv = s.state[p];
  if (sv.w >= s.n_maps) {
    set_err(s.err, kDevErrIndex);
    return;
  }
  const MapDesc md = s.maps[sv.w];
  const uint32_t x = sv.x & 0xffffu, y = sv.x >> 16;
  if (x >= md.w || y >= md.h) {  // a coordinate drawn for another example (the reference panics)
    set_err(s.err, kDevErrIndex);
    return;
  }
  s.color[p] = s.levels[md.off + (size_t)level * md.w * md.h + (size_t)y * md.w + x];
}

// Initial state of the random-init pixels (Generator::new, ms.rs:427-475):
// list[6i..6i+6] = {pixel, colour, state.x, state.y, state.z, state.w}.
__global__ void k_scatter_init(const uint32_t *list, uint32_t n, uint32_t *color, uint4 *state, uint32_t *res) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t *e = list + (size_t)i * 6;
  color[e[0]] = e[1];
  state[e[0]] = make_uint4(e[2], e[3], e[4], e[5]);
  res[i] = e[0];
}

// CoordinateTransform::apply (lib.rs:176-212): output pixel i takes texel
// (x, y) of source map `map`, (x, y, map) = buf[3i..3i+3].  maps[m] =
// {texel offset low, high, width, height}.  An entry outside the maps (the
// reference panics in get_pixel) writes 0 and sets *err.
__global__ void k_transform_apply(const uint32_t *buf, size_t n, const uint32_t *texels, const uint4 *maps,
                                  uint32_t n_maps, uint32_t *out, int *err) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t x = buf[3 * i], y = buf[3 * i + 1], m = buf[3 * i + 2];
    uint32_t v = 0;
    if (m < n_maps) {
      const uint4 md = maps[m];
      if (x < md.z && y < md.w)
        v = texels[(((size_t)md.y << 32) | md.x) + (size_t)y * md.z + x];
      else
        set_err(err, 1);
    } else {
      set_err(err, 1);
    }
    out[i] = v;
  }
}

// Debug maps (ms.rs:604-653): the patch-id and map-id colours of every
// pixel, and the uncertainty colour of every resolved pixel (the others
// stay 0).  Ids combine in u32 arithmetic, which wraps as the reference's
// release build does.
__global__ void k_id_maps(const uint32_t *ids, size_t n, uint32_t *patch_rgba, uint32_t *map_rgba) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t p = ids[2 * i], m = ids[2 * i + 1];
    patch_rgba[i] = (uint32_t)id_colour(p) | ((uint32_t)id_colour(p * 5u + 21u) << 8) |
                    ((uint32_t)id_colour(p / 4u + 12u) << 16) | 0xff000000u;
    map_rgba[i] = (uint32_t)id_colour((uint64_t)m * 200u) | ((uint32_t)id_colour(m * 5u + 341u) << 8) |
                  ((uint32_t)id_colour(m * 1200u - 35412u) << 16) | 0xff000000u;
  }
}

__global__ void k_uncertainty(const uint32_t *flat, const float *score, size_t n_res, size_t n_px, uint32_t *out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n_res; i += (size_t)gridDim.x * blockDim.x) {
    // (score.min(1.0) * 255.0) as u8: f32::min returns the other operand
    // for NaN, and `as` truncates and saturates
    const float v = __fmul_rn(fminf(score[i], 1.0f), 255.0f);
    const uint32_t ns = v >= 255.0f ? 255u : (v > 0.0f ? (uint32_t)v : 0u);
    if (flat[i] < n_px) out[flat[i]] = ns | ((255u - ns) << 8) | 0xff000000u;
  }
}

// Automatic guide maps (utils.rs:101-183).  DynamicImage::grayscale of RGBA8
// (image 0.23 rgb_to_luma): l = 0.2126 R + 0.7152 G + 0.0722 B in f32, left
// to right, truncated to u8 (NumCast), with the histogram of l; the
// histogram of channel 0 of an RGBA8 image; and the histogram-matching map
// applied as (n, n, n, 255).
__global__ void k_luma_hist(const uint32_t *src, size_t n, uint8_t *luma, uint32_t *hist) {
  __shared__ uint32_t h[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
  __syncthreads();
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t p = src[i];
    float l = __fmul_rn(0.2126f, (float)(p & 0xffu));
    l = __fadd_rn(l, __fmul_rn(0.7152f, (float)((p >> 8) & 0xffu)));
    l = __fadd_rn(l, __fmul_rn(0.0722f, (float)((p >> 16) & 0xffu)));
    const uint32_t v = l >= 255.0f ? 255u : (uint32_t)l;
    luma[i] = (uint8_t)v;
    atomicAdd(&h[v], 1u);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 256; i += blockDim.x)
    if (h[i]) atomicAdd(&hist[i], h[i]);
}

__global__ void k_hist_r(const uint32_t *src, size_t n, uint32_t *hist) {
  __shared__ uint32_t h[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
  __syncthreads();
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    atomicAdd(&h[src[i] & 0xffu], 1u);
  __syncthreads();
  for (int i = threadIdx.x; i < 256; i += blockDim.x)
    if (h[i]) atomicAdd(&hist[i], h[i]);
}

__global__ void k_apply_map(const uint8_t *luma, size_t n, const uint8_t *map, uint32_t *out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const uint32_t v = map[luma[i]];
    out[i] = v | (v << 8) | (v << 16) | 0xff000000u;
  }
}

// vertical_sample: u8 RGBA -> f32 RGBA, new height nh.
__global__ void k_resize_v(const uint8_t *src, uint32_t w, uint32_t h, float *tmp, uint32_t nh, const uint4 *taps,
                           const float *wts) {
  const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t oy = blockIdx.y;
  if (x >= w || oy >= nh) return;
  const uint4 t = taps[oy];
  float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
  for (uint32_t i = 0; i < t.y; ++i) {
    const uchar4 p = *(const uchar4 *)(src + ((size_t)(t.x + i) * w + x) * 4);
    const float wt = wts[t.z + i];
    a0 = __fadd_rn(a0, __fmul_rn((float)p.x, wt));
    a1 = __fadd_rn(a1, __fmul_rn((float)p.y, wt));
    a2 = __fadd_rn(a2, __fmul_rn((float)p.z, wt));
    a3 = __fadd_rn(a3, __fmul_rn((float)p.w, wt));
  }
  *(float4 *)(tmp + ((size_t)oy * w + x) * 4) = make_float4(a0, a1, a2, a3);
}

__device__ __forceinline__ uint8_t to_u8(float v) {
  v = v < 0.0f ? 0.0f : v;
  v = v > 255.0f ? 255.0f : v;
  return (uint8_t)roundf(v);
}

// horizontal_sample: f32 RGBA -> u8 RGBA (clamped, rounded half away from 0).
__global__ void k_resize_h(const float *tmp, uint32_t w, uint32_t nh, uint8_t *dst, uint32_t nw, const uint4 *taps,
                           const float *wts) {
  const uint32_t ox = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t y = blockIdx.y;
  if (ox >= nw || y >= nh) return;
  const uint4 t = taps[ox];
  float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
  for (uint32_t i = 0; i < t.y; ++i) {
    const float4 p = *(const float4 *)(tmp + ((size_t)y * w + t.x + i) * 4);
    const float wt = wts[t.z + i];
    a0 = __fadd_rn(a0, __fmul_rn(p.x, wt));
    a1 = __fadd_rn(a1, __fmul_rn(p.y, wt));
    a2 = __fadd_rn(a2, __fmul_rn(p.z, wt));
    a3 = __fadd_rn(a3, __fmul_rn(p.w, wt));
  }
  uchar4 o;
  o.x = to_u8(a0);
  o.y = to_u8(a1);
  o.z = to_u8(a2);
  o.w = to_u8(a3);
  *(uchar4 *)(dst + ((size_t)y * nw + ox) * 4) = o;
}

// The job owning block b of a pass: jobs sorted by first block, one ballot
// per 32 (block0 selects the pass's column).
template <bool kV>
__device__ __forceinline__ uint32_t find_job(const ResizeJob *jobs, uint32_t n, uint32_t b) {
  const int lane = threadIdx.x & 31;
  uint32_t j = 0;
  for (uint32_t c = 0; c < n; c += 32) {
    const uint32_t i = c + lane;
    const bool le = i < n && (kV ? jobs[i].block0_v : jobs[i].block0_h) <= b;
    const uint32_t bal = __ballot_sync(0xffffffffu, le);
    j = c + __popc(bal) - 1;
    if (bal != 0xffffffffu) break;
  }
  return j;
}

// k_resize_v over many jobs: job blocks laid out as cdiv(w, 128) x nh.
__global__ void k_resize_v_jobs(const ResizeJob *jobs, uint32_t n) {
  const uint32_t j = find_job<true>(jobs, n, blockIdx.x);
  const ResizeJob jb = jobs[j];
  const uint32_t lb = blockIdx.x - jb.block0_v, bx = (jb.w + 127) / 128;
  const uint32_t x = (lb % bx) * 128 + threadIdx.x, oy = lb / bx;
  if (x >= jb.w || oy >= jb.nh) return;
  const uint4 t = jb.tv[oy];
  float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
  for (uint32_t i = 0; i < t.y; ++i) {
    const uchar4 p = *(const uchar4 *)(jb.src + ((size_t)(t.x + i) * jb.w + x) * 4);
    const float wt = jb.wv[t.z + i];
    a0 = __fadd_rn(a0, __fmul_rn((float)p.x, wt));
    a1 = __fadd_rn(a1, __fmul_rn((float)p.y, wt));
    a2 = __fadd_rn(a2, __fmul_rn((float)p.z, wt));
    a3 = __fadd_rn(a3, __fmul_rn((float)p.w, wt));
  }
  *(float4 *)(jb.tmp + ((size_t)oy * jb.w + x) * 4) = make_float4(a0, a1, a2, a3);
}

// k_resize_h over many jobs: job blocks laid out as cdiv(nw, 128) x nh.
__global__ void k_resize_h_jobs(const ResizeJob *jobs, uint32_t n) {
  const uint32_t j = find_job<false>(jobs, n, blockIdx.x);
  const ResizeJob jb = jobs[j];
  const uint32_t lb = blockIdx.x - jb.block0_h, bx = (jb.nw + 127) / 128;
  const uint32_t ox = (lb % bx) * 128 + threadIdx.x, y = lb / bx;
  if (ox >= jb.nw || y >= jb.nh) return;
  const uint4 t = jb.th[ox];
  float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
  for (uint32_t i = 0; i < t.y; ++i) {
    const float4 p = *(const float4 *)(jb.tmp + ((size_t)y * jb.w + t.x + i) * 4);
    const float wt = jb.wh[t.z + i];
    a0 = __fadd_rn(a0, __fmul_rn(p.x, wt));
    a1 = __fadd_rn(a1, __fmul_rn(p.y, wt));
    a2 = __fadd_rn(a2, __fmul_rn(p.z, wt));
    a3 = __fadd_rn(a3, __fmul_rn(p.w, wt));
  }
  uchar4 o;
  o.x = to_u8(a0);
  o.y = to_u8(a1);
  o.z = to_u8(a2);
  o.w = to_u8(a3);
  *(uchar4 *)(jb.dst + ((size_t)y * jb.nw + ox) * 4) = o;
}

// Padded copy: dst[l][y + kPad][x + kPad] = src[l][y][x], border = kOutside.
__global__ void k_pad(const uint32_t *src, uint32_t w, uint32_t h, uint32_t levels, uint32_t pw, uint32_t *dst) {
  const uint32_t ph = h + 2 * kPad;
  const size_t n = (size_t)pw * ph * levels;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t l = i / ((size_t)pw * ph);
    const uint32_t r = (uint32_t)(i - l * pw * ph);
    const int y = (int)(r / pw) - kPad, x = (int)(r % pw) - kPad;
    dst[i] = ((unsigned)x < w && (unsigned)y < h) ? src[l * w * h + (size_t)y * w + x] : kOutside;
  }
}

// Programmatic dependent launch: every hot-loop kernel first waits for the
// kernel before it in the stream to complete (its memory is then visible),
// then lets the next one launch, whose blocks start and wait in turn while
// this one's last wave runs.  Kernels launched without the attribute pass
// both instructions at once.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// ---------------------------------------------------------------------------
// Kernels.  The plain form takes one session's descriptors as parameters;
// the multi form runs one phase of one batch step for many sessions, each
// segment of its grid belonging to one (session, step).
// ---------------------------------------------------------------------------
struct SegView {
  const SessionDev *s;
  const StepDev *d;
  uint32_t vb, vg;
};

// The segment owning this block: segments are sorted by first block, so the
// ones starting at or before blockIdx.x form a prefix; one ballot per 32.
__device__ __forceinline__ SegView find_segment(const MultiLaunch &ml) {
  const uint32_t bx = blockIdx.x + ml.block_base;
  const int lane = threadIdx.x & 31;
  uint32_t j = 0;
  for (uint32_t c = 0; c < ml.n_segs; c += kWarp) {
    const uint32_t i = c + lane;
    const bool le = i < ml.n_segs && __ldg(&ml.segs[i].block0) <= bx;
    const uint32_t bal = __ballot_sync(0xffffffffu, le);
    j = c + __popc(bal) - 1;
    if (bal != 0xffffffffu) break;
  }
  const Segment g = ml.segs[j];
  SegView v;
  v.s = ml.sessions + g.session;
  v.d = ml.step_tabs[g.session] + g.step;
  v.vb = bx - g.block0;
  v.vg = g.nblocks;
  return v;
}

// The tree entries of a chunk of appended stage items, for k-NN made ahead
// of the resolves (SessionDev::rank): what the commits of those items
// enter in flush_resolved (ms.rs:296-331), the resolved-list slot, bitmap
// and mirror bits and cell counts, plus the tree position.  The appended
// pixels and their order come from the pick chain alone, so this runs
// before their resolves; the k-NN kernels check every set bit against the
// item's own tree length.
__global__ void k_tree_append(SessionDev s, StageDev st, uint32_t a0, uint32_t a1, uint32_t pos0, uint32_t nomir_end) {
  pdl_enter();
  const uint32_t i = a0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a1) return;
  const uint32_t p = st.items[i];
  if (p >= s.W * s.H) {
    set_err(s.err, kDevErrIndex);
    return;
  }
  const uint32_t pos = pos0 + (i - a0);
  s.resolved[pos] = p;
  s.rank[p] = pos + 1u;
  const uint32_t x = p % s.W, y = p / s.W;
  atomicOr(&s.occ[(size_t)y * s.wpr + (x >> 5)], 1u << (x & 31));
  add_cell_point(s, (int)x, (int)y);
  if (s.tiling && i >= nomir_end) {
    atomicOr(&s.mir[(size_t)y * s.wpr + (x >> 5)], 1u << (x & 31));
    if ((int)x < s.x_l)
      add_cell_point(s, (int)x + (int)s.W, (int)y);
    else if ((int)x > s.x_r)
      add_cell_point(s, (int)x - (int)s.W, (int)y);
    if ((int)y < s.y_b)
      add_cell_point(s, (int)x, (int)y + (int)s.H);
    else if ((int)y > s.y_t)
      add_cell_point(s, (int)x, (int)y - (int)s.H);
  }
}

// Tree positions of the initial tree (random-init or locked pixels).
__global__ void k_rank_init(SessionDev s, uint32_t n) {
  const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const uint32_t p = s.resolved[e];
  if (p < s.W * s.H) s.rank[p] = e + 1u;
}

__global__ void k_random_candidates(SessionDev s, StageDev st) {
  pdl_enter(); random_candidates_body(s, st, blockIdx.x); }
__global__ void k_random_candidates_multi(MultiLaunch ml) {
  pdl_enter();
  const SegView v = find_segment(ml);
  random_candidates_body(*v.s, v.d->rc, v.vb);
}

// The commit of a pending batch of redo items, spread over the launch's
// threads (PendingCommit).
__device__ __forceinline__ void pending_commit(const SessionDev &s, const PendingCommit &pc) {
  uint32_t evals = 0;  // one atomic per warp instead of one per item
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < pc.n; i += gridDim.x * blockDim.x) {
    const Result r = pc.b.res[i];
    evals += r.ncand;
    commit_item(s, pc.st, pc.b, i, r, false);
  }
  evals = __reduce_add_sync(0xffffffffu, evals);
  if ((threadIdx.x & 31) == 0 && evals) atomicAdd(s.evals, (unsigned long long)evals);
}

template <bool kWin>
__global__ void __launch_bounds__(kWalkWarps *kWarp, 4)
    k_knn_walk(SessionDev s, StageDev st, BatchDev b, const __grid_constant__ PendingCommit pc) {
  pdl_enter();
  if (pc.n) pending_commit(s, pc);
  knn_walk_body<kWin>(s, st, b, blockIdx.x, gridDim.x);
}
__global__ void __launch_bounds__(kWalkWarps *kWarp, 4) k_knn_walk_multi(MultiLaunch ml) {
  pdl_enter();
  const SegView v = find_segment(ml);
  knn_walk_body<false>(*v.s, v.d->st, v.d->b, v.vb, v.vg);
}

__global__ void __launch_bounds__(kExhThreads) k_knn_exhaustive(SessionDev s, StageDev st, BatchDev b, uint32_t cap,
                                                                 int all_items,
                                                                 const __grid_constant__ PendingCommit pc) {
  pdl_enter();
  if (pc.n) pending_commit(s, pc);
  knn_exhaustive_body(s, st, b, all_items, cap, blockIdx.x, gridDim.x);
}
__global__ void __launch_bounds__(kExhThreads) k_knn_exhaustive_multi(MultiLaunch ml) {
  pdl_enter();
  __shared__ ExhShared sh;
  extern __shared__ unsigned long long all_keys[];
  if (blockIdx.x < ml.pool_block0) {  // whole batches of sparse steps
    const SegView v = find_segment(ml);
    const StepDev &d = *v.d;
    const uint32_t n = d.b.i1 - d.b.i0;
    for (uint32_t e = v.vb; e < n; e += v.vg) {
      knn_exhaustive_item(*v.s, d.st, d.b, e, sh, all_keys, ml.key_cap, true);
      __syncthreads();
    }
    return;
  }
  // the pool: the fallback lists of all walk steps, concatenated, in turn;
  // their lengths are read in parallel, kExhThreads at a time
  __shared__ uint32_t fb_cnt[kExhThreads];
  const uint32_t vb = blockIdx.x - ml.pool_block0, vg = gridDim.x - ml.pool_block0;
  uint32_t base = 0;
  for (uint32_t c0 = 0; c0 < ml.n_fb; c0 += kExhThreads) {
    const uint32_t nc = min((uint32_t)kExhThreads, ml.n_fb - c0);
    __syncthreads();
    if (threadIdx.x < nc) {
      const Segment g = ml.fb[c0 + threadIdx.x];
      fb_cnt[threadIdx.x] = *ml.step_tabs[g.session][g.step].b.fb_count;
    }
    __syncthreads();
    for (uint32_t j = 0; j < nc; ++j) {
      const uint32_t cnt = fb_cnt[j];
      uint32_t v = base + (vb + vg - base % vg) % vg;
      if (v < base + cnt) {
        const Segment g = ml.fb[c0 + j];
        const StepDev &d = ml.step_tabs[g.session][g.step];
        for (; v < base + cnt; v += vg) {
          knn_exhaustive_item(ml.sessions[g.session], d.st, d.b, d.b.fb_list[v - base], sh, all_keys, ml.key_cap,
                              false);
          __syncthreads();
        }
      }
      base += cnt;
    }
  }
}

// The single-session mean: each thread first copies its item's distances
// into its own column of shared memory with asynchronous copies (all in
// flight at once), so that only the f64 chain itself stays on the
// critical path of these mostly latency-bound launches.
constexpr uint32_t kMeanThreads = 64;
__device__ __forceinline__ void mean_body_staged(const BatchDev &b, uint32_t vb) {
  extern __shared__ double md[];  // [k][kMeanThreads]
  const uint32_t nb = b.i1 - b.i0;
  const uint32_t local = vb * kMeanThreads + threadIdx.x;
  if (local >= nb) return;
  const uint32_t nk = b.ncnt[local];
  if (nk == 0) return;
  double *col = md + threadIdx.x;
  for (uint32_t j = 0; j < nk; ++j) __pipeline_memcpy_async(col + j * kMeanThreads, b.dist + (size_t)j * nb + local, 8);
  __pipeline_commit();
  __pipeline_wait_prior(0);
  double sum = 0.0;
  for (uint32_t j = 0; j < nk; ++j) {
    const double d = col[j * kMeanThreads];
    sum = __dadd_rn(sum, d);
    sum = __dadd_rn(sum, d);
    sum = __dadd_rn(sum, d);
    sum = __dadd_rn(sum, d);
  }
  b.mean[local] = __ddiv_rn(sum, (double)(nk * 4u));
}

__global__ void __launch_bounds__(kMeanThreads) k_mean_staged(SessionDev s, StageDev st, BatchDev b) {
  pdl_enter();
  mean_body_staged(b, blockIdx.x);
}

__global__ void __launch_bounds__(128) k_mean_multi(MultiLaunch ml) {
  pdl_enter();
  const SegView v = find_segment(ml);
  mean_body(*v.s, v.d->b, v.vb);
}

// pc: the previous batch step's deferred commit (BatchDev::prev_tag), made
// here by every thread of the grid before its own item; this launch's
// readers of those pixels take their values from pc.b.res instead.
__global__ void __launch_bounds__(kResolveWarps *kWarp, 8)
    k_resolve(SessionDev s, StageDev st, BatchDev b, const __grid_constant__ PendingCommit pc) {
  pdl_enter();
  if (pc.n) pending_commit(s, pc);
  resolve_body<false>(s, st, b, blockIdx.x, gridDim.x);
}
// Sessions without guides (the guide terms compiled out).
__global__ void __launch_bounds__(kResolveWarps *kWarp, 9)
    k_resolve_lean(SessionDev s, StageDev st, BatchDev b, const __grid_constant__ PendingCommit pc) {
  pdl_enter();
  if (pc.n) pending_commit(s, pc);
  resolve_body<true>(s, st, b, blockIdx.x, gridDim.x);
}
__global__ void __launch_bounds__(kResolveWarps *kWarp, 8) k_resolve_multi(MultiLaunch ml) {
  pdl_enter();
  const SegView v = find_segment(ml);
  resolve_body<false>(*v.s, v.d->st, v.d->b, v.vb, v.vg);
}
// Segments of sessions without guides: 56 registers, nine blocks per SM.
__global__ void __launch_bounds__(kResolveWarps *kWarp, 9) k_resolve_multi_lean(MultiLaunch ml) {
  pdl_enter();
  const SegView v = find_segment(ml);
  resolve_body<true>(*v.s, v.d->st, v.d->b, v.vb, v.vg);
}

template <int T, bool kFull>
__global__ void __launch_bounds__(T)
    k_resolve_team(SessionDev s, StageDev st, BatchDev b, const __grid_constant__ PendingCommit pc) {
  pdl_enter();
  if (pc.n) pending_commit(s, pc);
  resolve_team_body<T, kFull>(s, st, b, blockIdx.x, gridDim.x);
}
template <int T, bool kFull>
__global__ void __launch_bounds__(T) k_resolve_team_multi(MultiLaunch ml) {
  pdl_enter();
  const SegView v = find_segment(ml);
  resolve_team_body<T, kFull>(*v.s, v.d->st, v.d->b, v.vb, v.vg);
}

// One step of a batch of new items whose neighbours the exhaustive k-NN
// finds, one item per CTA at a time (256 threads): the item's k-NN, then its
// full-evaluation resolve (every candidate scored completely, as the team
// form does), in one launch.  The mean's chain of 4k dependent f64 adds
// (ms.rs:417-423) runs on warp 0's first lane while warps 1-7 set up the
// neighbour records and candidates and gather every (candidate, neighbour)
// LUT sum, none of which needs the mean; the weights and each candidate's
// in-order sum of nps_j * w_j follow on all warps.  The other CTAs' commits
// change only their own pixels, the resolved list beyond n_res and the
// occupancy, mirror and cell records of those pixels; this k-NN reads the
// first n_res points and their mirror bits only (the cell grid is not
// searched here; a key buffer overflow rescans the points).
// Barrier of the set-up warps (all but warp 0): TS threads.
template <int TS>
__device__ __forceinline__ void setup_bar() {
  asm volatile("bar.sync 1, %0;" ::"n"(TS) : "memory");
}

// T = 256, or 512 for steps of at most one item per SM, where the extra
// warps shorten each item's latency-bound k-NN and gathers.
template <int T>
__global__ void __launch_bounds__(T) k_step_team_full(SessionDev s, StageDev st, BatchDev b, uint32_t cap) {
  constexpr int NW = T / kWarp, TS = T - kWarp;
  __shared__ ExhShared sh;
  __shared__ double tab[64];
  __shared__ float tab_ff[128];
  __shared__ uint32_t wcnt[NW];
  __shared__ float red_s[NW];
  __shared__ uint32_t red_i[NW];
  __shared__ int sh_flags, sh_maxoff;
  __shared__ uint32_t sh_ncoh;
  __shared__ double sh_mean;
  extern __shared__ __align__(16) unsigned char smem[];
  pdl_enter();
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t nb = b.i1 - b.i0;
  float *lc = (float *)smem;
  float *lg = lc + 256;
  const WarpSmem w = carve(smem + 2048, s.k, s.m);
  float *term = (float *)(smem + 2048 + warp_smem_bytes(s.k, s.m));
  for (uint32_t local = blockIdx.x; local < nb; local += gridDim.x) {
    const uint32_t nk = knn_exhaustive_item(s, st, b, local, sh, (unsigned long long *)smem, cap, true, false, false);
    __syncthreads();  // sh.dist, sh.nbo; the key buffer is free again
    const uint32_t item = b.i0 + local;
    const uint32_t pixel = st.items[item];
    const int px = (int)(pixel % s.W), py = (int)(pixel / s.W);
    const bool is_new = item >= st.redo;
    if (nk == 0) {
      if (tid == 0) write_random_result(s, st, b, local, pixel);
      __syncthreads();
      continue;
    }
    if (warp == 0) {
      if (s.exact_sum) {
        unsigned long long part = 0;
        for (uint32_t j = lane; j < nk; j += kWarp) part += exact_units(s, off_dx(sh.nbo[j]), off_dy(sh.nbo[j]));
        part = warp_sum_units(part);
        if (lane == 0) {
          const double mean = exact_mean(s, part, nk);
          sh_mean = mean;
          b.mean[local] = mean;
        }
      } else if (lane == 0) {
        const double mean = mean_chain(sh.dist, nk);
        sh_mean = mean;
        b.mean[local] = mean;
      }
    } else {
      const int t = tid - kWarp;
      // the LUTs, the exp tables and the first random candidates go into
      // registers first, so that their loads are in flight together with
      // the neighbour records' loads; they reach shared memory after the
      // records (the records loop's barriers order the flags' reset before
      // their first update)
      constexpr int kLutPer = (512 + TS - 1) / TS;
      float lreg[kLutPer];
#pragma unroll
      for (int u = 0; u < kLutPer; ++u) {
        const int i = t + u * TS;
        lreg[u] = i < 512 ? st.lut[i] : 0.0f;
      }
      const double treg = t < 64 ? g_exp2_64[t] : 0.0;
      const float freg = t < 128 ? g_exp2_ff[t] : 0.0f;
      const uint2 *rc = st.rcand + (size_t)item * s.m;
      const uint2 rv0 = (uint32_t)t < s.m ? rc[t] : make_uint2(0u, 0u);
      if (t == 0) {
        sh_flags = 0;
        sh_maxoff = 0;
      }
      // neighbour records and coherence candidates, compacted in order
      bool bad_map = false;
      int maxoff = 0;
      uint32_t ncoh = 0;
      for (uint32_t j0 = 0; j0 < nk; j0 += TS) {
        const uint32_t j = j0 + t;
        bool valid = false;
        uint32_t cxy = 0, aux = 0;
        if (j < nk) valid = neighbour_records(s, st, b, px, py, j, sh.nbo[j], 0.0f, w, cxy, aux, maxoff, bad_map);
        const uint32_t bal = __ballot_sync(0xffffffffu, valid);
        if (lane == 0) wcnt[warp] = __popc(bal);
        setup_bar<TS>();
        uint32_t base = ncoh, total = 0;
#pragma unroll
        for (int i = 1; i < NW; ++i) {
          if (i < warp) base += wcnt[i];
          total += wcnt[i];
        }
        if (valid) {
          const uint32_t slot = base + __popc(bal & lt);
          w.cxy[slot] = cxy;
          w.caux[slot] = aux;
        }
        ncoh += total;
        setup_bar<TS>();
      }
#pragma unroll
      for (int u = 0; u < kLutPer; ++u) {
        const int i = t + u * TS;
        if (i < 512) lc[i] = lreg[u];
      }
      if (t < 64) tab[t] = treg;
      if (t < 128) tab_ff[t] = freg;
      if (bad_map) atomicOr(&sh_flags, 2);
      if (maxoff) atomicMax(&sh_maxoff, maxoff);
      for (uint32_t q = t; q < s.m; q += TS) {
        const uint2 v = use_rcand(s, q == (uint32_t)t ? rv0 : rc[q]);
        w.cxy[ncoh + q] = v.x;
        w.caux[ncoh + q] = v.y | kAuxNeg | (q << 16);
      }
      if (t == 0) sh_ncoh = ncoh;
      setup_bar<TS>();
      if (!(sh_flags & 2) && !st.slow_lut) {
        // every candidate's LUT sums nps(c, j), before the weights exist
        const uint32_t nc = ncoh + s.m, total = nc * nk;
        if (sh_maxoff <= kPad && !s.guide_dims_differ) {
          unsigned long long *cb = (unsigned long long *)(term + (((size_t)nk * nc + 1) & ~(size_t)1));
          for (uint32_t c = t; c < nc; c += TS) {
            const uint32_t cxy = w.cxy[c], aux = w.caux[c];
            const MapDesc md = s.maps[aux & 0x7fffu];
            const unsigned long long off = md.poff + (unsigned long long)st.level * md.pw * md.ph +
                                           (unsigned long long)((cxy >> 16) + kPad) * md.pw + ((cxy & 0xffffu) + kPad);
            cb[c] = off | ((aux & kAuxNeg) ? (1ull << 63) : 0ull);
          }
          setup_bar<TS>();
          constexpr int kRound = 16;  // gathers in flight per thread
          for (uint32_t i0 = t; i0 < total; i0 += kRound * TS) {
            uint32_t tx[kRound], gx[kRound], ii[kRound], jj[kRound];
#pragma unroll
            for (int u = 0; u < kRound; ++u) {
              const uint32_t i = i0 + (uint32_t)u * TS;
              ii[u] = i;
              if (i < total) {
                const uint32_t c = i / nk;
                jj[u] = i - c * nk;
                const unsigned long long v = cb[c];
                const int lin = (v >> 63) ? -w.lin[jj[u]] : w.lin[jj[u]];
                const size_t off = (size_t)(v & 0x7fffffffffffffffull) + lin;
                tx[u] = __ldg(s.plevels + off);
                if (s.guided) gx[u] = __ldg(s.pguides + off);
              }
            }
#pragma unroll
            for (int u = 0; u < kRound; ++u) {
              if (ii[u] < total) {
                const uint4 nr = w.nbr[jj[u]];
                float nps = lut4r(lc, __vabsdiffu4(nr.y, tx[u]), 0.0f, st.opaque);
                if (s.guided) nps = lut4r(lg, __vabsdiffu4(nr.z, gx[u]), nps, st.opaque);
                term[ii[u]] = nps;
              }
            }
          }
        } else {
          // bounds-checked gathers (far neighbours or guides of other sizes)
          uint32_t c = (uint32_t)t / nk, j = (uint32_t)t - c * nk;
          const uint32_t dc = (uint32_t)TS / nk, dj = (uint32_t)TS - dc * nk;
          for (uint32_t i = t; i < total; i += TS) {
            const uint32_t cxy = w.cxy[c], aux = w.caux[c];
            const uint32_t map = aux & 0x7fffu;
            const int sg = (aux & kAuxNeg) ? -1 : 1;
            const MapDesc md = s.maps[map];
            const uint4 nr = w.nbr[j];
            const int qx = (int)(cxy & 0xffffu) + sg * off_dx((int32_t)nr.x);
            const int qy = (int)(cxy >> 16) + sg * off_dy((int32_t)nr.x);
            uint32_t tt = kOutside;
            if ((unsigned)qx < md.w && (unsigned)qy < md.h)
              tt = __ldg(&s.levels[md.off + (size_t)st.level * md.w * md.h + (size_t)qy * md.w + qx]);
            float nps = lut4(lc, __vabsdiffu4(nr.y, tt), 0.0f);
            if (s.guided) {
              const GuideDesc gd = s.gdesc[map];
              uint32_t gt = kOutside;
              if ((unsigned)qx < gd.w && (unsigned)qy < gd.h)
                gt = __ldg(&s.guides[gd.off + (size_t)st.level * gd.w * gd.h + (size_t)qy * gd.w + qx]);
              nps = lut4(lg, __vabsdiffu4(nr.z, gt), nps);
            }
            term[i] = nps;
            c += dc;
            j += dj;
            if (j >= nk) {
              j -= nk;
              ++c;
            }
          }
        }
      }
    }
    __syncthreads();  // the mean, the records, the candidates and the LUT sums
    const uint32_t ncoh = sh_ncoh, nc = ncoh + s.m;
    if (sh_flags & 2) {
      if (tid == 0) write_bad_result(s, st, b, local, pixel);
      __syncthreads();
      continue;
    }
    // the weights: into the records (for the sequential form) and, as
    // floats, into w.term
    {
      const double avg = sh_mean;
      bool nan_w = false;
      for (uint32_t j = tid; j < nk; j += T) {
        const float wv = neighbour_weight(sh.dist[j], avg, tab, tab_ff);
        nan_w |= (wv != wv);
        w.nbr[j].w = __float_as_uint(wv);
        w.term[j] = wv;
      }
      if (nan_w) atomicOr(&sh_flags, 1);
    }
    __syncthreads();
    float best_s = FLT_MAX;
    uint32_t best_i = 0;
    if (!st.slow_lut && !(sh_flags & 1)) {
      float my_s = FLT_MAX;
      uint32_t my_i = 0xffffffffu;
      for (uint32_t cc = tid; cc < nc; cc += T) {
        float sc = 0.0f;
        const float *tc = term + (size_t)cc * nk;
        for (uint32_t jj = 0; jj < nk; ++jj) sc = __fadd_rn(sc, __fmul_rn(tc[jj], w.term[jj]));
        if (sc < my_s) {  // first strict minimum among this thread's candidates
          my_s = sc;
          my_i = cc;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, my_s, o);
        const uint32_t oi = __shfl_xor_sync(0xffffffffu, my_i, o);
        if (ov < my_s || (ov == my_s && oi < my_i)) {
          my_s = ov;
          my_i = oi;
        }
      }
      if (lane == 0) {
        red_s[warp] = my_s;
        red_i[warp] = my_i;
      }
      __syncthreads();
      best_s = red_s[0];
      best_i = red_i[0];
      for (int i = 1; i < NW; ++i) {
        if (red_s[i] < best_s || (red_s[i] == best_s && red_i[i] < best_i)) {
          best_s = red_s[i];
          best_i = red_i[i];
        }
      }
      if (best_i == 0xffffffffu) {  // no score below f32::MAX: the reference keeps candidate 0
        best_s = FLT_MAX;
        best_i = 0;
      }
    } else if (tid == 0) {
      sequential_best(s, st, w, lc, lg, nk, nc, best_s, best_i);
    }
    if (tid == 0) write_result(s, st, w, b, local, pixel, px, py, is_new, nc, best_s, best_i);
    __syncthreads();
  }
}

__global__ void k_commit(SessionDev s, StageDev st, BatchDev b) {
  pdl_enter(); commit_body(s, st, b, blockIdx.x); }
__global__ void k_commit_multi(MultiLaunch ml) {
  pdl_enter();
  const SegView v = find_segment(ml);
  commit_body(*v.s, v.d->st, v.d->b, v.vb);
}

__global__ void k_level_switch(SessionDev s, uint32_t level, uint32_t n_res) {
  pdl_enter();
  level_switch_body(s, level, n_res, blockIdx.x);
}
__global__ void k_level_switch_multi(MultiLaunch ml) {
  pdl_enter();
  const SegView v = find_segment(ml);
  level_switch_body(*v.s, v.d->level, v.d->ls_n_res, v.vb);
}

inline uint32_t cdiv(uint64_t a, uint64_t b) { return (uint32_t)((a + b - 1) / b); }

template <typename... KArgs, typename... Args>
void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

}  // namespace

size_t resolve_smem_bytes(uint32_t k, uint32_t m, int) { return 2048 + (size_t)kResolveWarps * warp_smem_bytes(k, m); }
static size_t team_smem_bytes(uint32_t k, uint32_t m) { return 2048 + warp_smem_bytes(k, m) + (size_t)(k ? k : 1) * 4; }
// the full-evaluation team form keeps every (candidate, neighbour) term
static size_t team_full_smem_bytes(uint32_t k, uint32_t m) {
  const size_t kk = k ? k : 1;
  return 2048 + warp_smem_bytes(k, m) + ((kk * (k + m) * 4 + 7) & ~(size_t)7) + (size_t)(k + m) * 8;
}
constexpr size_t kTeamFullMaxSmem = 96 * 1024;

// Raises (never lowers) a kernel's dynamic shared-memory limit on the
// current device, so that sessions with different (k, m) can be built in
// any order and run later.
template <typename K>
static cudaError_t raise_smem(K *kernel, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, size_t> cur;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(mu);
  auto it = cur.find({dev, (const void *)kernel});
  if (it == cur.end()) {
    // without the opt-in, static plus dynamic shared memory stays within 48 KB
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess) return e;
    it = cur.emplace(std::make_pair(dev, (const void *)kernel),
                     fa.sharedSizeBytes < 48 * 1024 ? 48 * 1024 - fa.sharedSizeBytes : 0)
             .first;
  }
  size_t &c = it->second;
  if (bytes <= c) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) c = bytes;
  return e;
}

cudaError_t configure_kernels(uint32_t k, uint32_t m) {
  cudaError_t e = raise_smem(k_resolve, resolve_smem_bytes(k, m, 0));
  if (e != cudaSuccess) return e;
  e = raise_smem(k_resolve_lean, resolve_smem_bytes(k, m, 0));
  if (e != cudaSuccess) return e;
  e = raise_smem(k_knn_exhaustive, kExhAllKeys * 8);
  if (e != cudaSuccess) return e;
  e = raise_smem(k_mean_staged, (size_t)k * kMeanThreads * 8);
  if (e != cudaSuccess) return e;
  e = raise_smem(k_resolve_team<kTeamThreads, false>, team_smem_bytes(k, m));
  if (e != cudaSuccess) return e;
  const size_t fsm = team_full_smem_bytes(k, m);
  if (fsm <= kTeamFullMaxSmem) {
    e = raise_smem(k_resolve_team<kTeamFullThreads, true>, fsm);
    if (e != cudaSuccess) return e;
    e = raise_smem(k_resolve_team<kStepWideThreads, true>, fsm);
    if (e != cudaSuccess) return e;
    e = raise_smem(k_step_team_full<kTeamFullThreads>, std::max<size_t>(fsm, (size_t)kExhAllKeys * 8));
    if (e != cudaSuccess) return e;
    return raise_smem(k_step_team_full<kStepWideThreads>, std::max<size_t>(fsm, (size_t)kExhAllKeys * 8));
  }
  return cudaSuccess;
}

cudaError_t set_multi_smem(int phase, size_t bytes) {
  switch (phase) {
    case kPhaseExhaustive: return raise_smem(k_knn_exhaustive_multi, bytes);
    case kPhaseResolve: {
      const cudaError_t e = raise_smem(k_resolve_multi, bytes);
      return e != cudaSuccess ? e : raise_smem(k_resolve_multi_lean, bytes);
    }
    case kPhaseTeamPart: return raise_smem(k_resolve_team_multi<kTeamThreads, false>, bytes);
    case kPhaseTeamFull: return raise_smem(k_resolve_team_multi<kTeamFullThreads, true>, bytes);
    default: return cudaSuccess;
  }
}

bool team_full_fits(uint32_t k, uint32_t m) { return team_full_smem_bytes(k, m) <= kTeamFullMaxSmem; }


uint32_t multi_threads(int phase) {
  switch (phase) {
    case kPhaseLevelSwitch: return 256;
    case kPhaseRandom: return 128;
    case kPhaseWalk: return kWalkWarps * kWarp;
    case kPhaseExhaustive: return kExhThreads;
    case kPhaseMean: return 128;
    case kPhaseResolve: return kResolveWarps * kWarp;
    case kPhaseTeamPart: return kTeamThreads;
    case kPhaseTeamFull: return kTeamFullThreads;
    default: return 256;
  }
}

uint32_t multi_blocks(int phase, uint32_t n, uint32_t cap) {
  if (n == 0) return 0;
  uint32_t b = 0;
  switch (phase) {
    case kPhaseLevelSwitch: b = cdiv(n, 256); break;
    case kPhaseRandom: b = cdiv(n, 128); break;
    case kPhaseWalk: b = cdiv(n, kWalkWarps); break;
    case kPhaseExhaustive: b = n; break;
    case kPhaseMean: b = cdiv(n, 128); break;
    case kPhaseResolve: b = cdiv(n, kResolveWarps); break;
    case kPhaseTeamPart:
    case kPhaseTeamFull: b = n; break;
    default: b = cdiv(n, 256); break;
  }
  // only the grid-stride phases may take fewer blocks than items need
  const bool strided = phase == kPhaseWalk || phase == kPhaseExhaustive || phase == kPhaseResolve ||
                       phase == kPhaseTeamPart || phase == kPhaseTeamFull;
  if (strided && cap && b > cap) b = cap;
  return b;
}

size_t multi_smem_bytes(int phase, uint32_t k, uint32_t m) {
  switch (phase) {
    case kPhaseExhaustive: return (size_t)kExhAllKeys * 8;
    case kPhaseResolve: return resolve_smem_bytes(k, m, 0);
    case kPhaseTeamPart: return team_smem_bytes(k, m);
    case kPhaseTeamFull: return team_full_smem_bytes(k, m);
    default: return 0;
  }
}

void launch_multi(int phase, const MultiLaunch &ml, uint32_t blocks, size_t smem, cudaStream_t stream) {
  if (blocks == 0) return;  // a launch may carry only the exhaustive k-NN's fallback pool (no segments)
  const uint32_t t = multi_threads(phase);
  switch (phase) {
    case kPhaseLevelSwitch: launch_pdl(k_level_switch_multi, blocks, t, 0, stream, ml); break;
    case kPhaseRandom: launch_pdl(k_random_candidates_multi, blocks, t, 0, stream, ml); break;
    case kPhaseWalk: launch_pdl(k_knn_walk_multi, blocks, t, 0, stream, ml); break;
    case kPhaseExhaustive: launch_pdl(k_knn_exhaustive_multi, blocks, t, smem, stream, ml); break;
    case kPhaseMean: launch_pdl(k_mean_multi, blocks, t, 0, stream, ml); break;
    case kPhaseResolve: {
      // segments [0, n_lean) belong to sessions without guides (lean kernel,
      // blocks [0, lean_blocks)); the rest run the general kernel
      MultiLaunch a = ml, g = ml;
      a.n_segs = ml.n_lean;
      g.segs = ml.segs + ml.n_lean;
      g.n_segs = ml.n_segs - ml.n_lean;
      g.block_base = ml.block_base + ml.lean_blocks;
      if (a.n_segs) launch_pdl(k_resolve_multi_lean, ml.lean_blocks, t, smem, stream, a);
      if (g.n_segs) launch_pdl(k_resolve_multi, blocks - ml.lean_blocks, t, smem, stream, g);
      break;
    }
    case kPhaseTeamPart: launch_pdl(k_resolve_team_multi<kTeamThreads, false>, blocks, t, smem, stream, ml); break;
    case kPhaseTeamFull: launch_pdl(k_resolve_team_multi<kTeamFullThreads, true>, blocks, t, smem, stream, ml); break;
    case kPhaseCommit: launch_pdl(k_commit_multi, blocks, t, 0, stream, ml); break;
    default: break;
  }
}

void launch_random_candidates(const SessionDev &s, const StageDev &st, cudaStream_t stream) {
  if (st.n_items == 0 || s.m == 0) return;
  launch_pdl(k_random_candidates, cdiv(st.n_items, 128), 128, 0, stream, s, st);
}

void launch_knn_walk(const SessionDev &s, const StageDev &st, const BatchDev &b, cudaStream_t stream,
                     const PendingCommit &pc) {
  const uint32_t n = b.i1 - b.i0;
  if (n == 0 && pc.n == 0) return;
  const uint32_t grid = std::max(cdiv(n, kWalkWarps), cdiv(pc.n, kWalkWarps * kWarp));
  if (b.walk_window)
    launch_pdl(k_knn_walk<true>, grid, kWalkWarps * kWarp, kWalkWinBytes, stream, s, st, b, pc);
  else
    launch_pdl(k_knn_walk<false>, grid, kWalkWarps * kWarp, 0, stream, s, st, b, pc);
}

uint32_t exh_key_cap(const SessionDev &s, const BatchDev &b) {
  // every point and its (at most two) tiling mirrors while they fit, else
  // the cell grid's rings (a few times k keys; an overflow falls back to
  // rescanning the points, exactly)
  const uint64_t want = b.n_res <= kExhGridFrom ? (uint64_t)b.n_res * (s.tiling ? 3 : 1) + 64 : 2048;
  return (uint32_t)std::min<uint64_t>(kExhAllKeys, std::max<uint64_t>(want, 4u * std::max<uint32_t>(s.k, 64u)));
}

void launch_knn_exhaustive(const SessionDev &s, const StageDev &st, const BatchDev &b, bool all_items,
                           cudaStream_t stream, const PendingCommit &pc) {
  const uint32_t n = b.i1 - b.i0;
  if (n == 0 && pc.n == 0) return;
  uint32_t grid = n < 608u ? n : 608u;  // 152 SMs x 4 CTAs, grid-stride beyond
  grid = std::max(grid, std::min(608u, cdiv(pc.n, kExhThreads)));
  const uint32_t cap = exh_key_cap(s, b);
  launch_pdl(k_knn_exhaustive, grid, kExhThreads, (size_t)cap * 8, stream, s, st, b, cap, all_items ? 1 : 0, pc);
}

void launch_mean(const SessionDev &s, const StageDev &st, const BatchDev &b, cudaStream_t stream) {
  const uint32_t n = b.i1 - b.i0;
  if (n == 0 || s.k == 0) return;
  launch_pdl(k_mean_staged, cdiv(n, kMeanThreads), kMeanThreads, (size_t)s.k * kMeanThreads * 8, stream, s, st, b);
}

// Resident blocks of a kernel on the current device (cached per kernel and
// dynamic shared-memory size).
template <typename K>
static uint32_t resident_blocks(K *kernel, int threads, size_t smem) {
  static std::mutex mu;
  static std::map<std::pair<const void *, size_t>, uint32_t> cache;
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find({(const void *)kernel, smem});
  if (it != cache.end()) return it->second;
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm <= 0)
    return 0;  // unknown: the caller keeps a full grid
  const uint32_t n = (uint32_t)sms * (uint32_t)per_sm;
  cache[{(const void *)kernel, smem}] = n;
  return n;
}

void launch_resolve(const SessionDev &s, const StageDev &st, const BatchDev &b, cudaStream_t stream,
                    const PendingCommit &pc) {
  const uint32_t n = b.i1 - b.i0;
  if (n == 0 && pc.n == 0) return;
  const size_t smem = resolve_smem_bytes(s.k, s.m, s.guided);
  uint32_t grid = cdiv(n, kResolveWarps);
  if (b.work_ctr) {
    // a resident grid whose warps take further items from the counter
    const uint32_t cap = s.guided ? resident_blocks(k_resolve, kResolveWarps * kWarp, smem)
                                  : resident_blocks(k_resolve_lean, kResolveWarps * kWarp, smem);
    if (cap) grid = std::min(grid, cap);
  }
  grid = std::max(grid, cdiv(pc.n, kResolveWarps * kWarp));
  if (s.guided)
    launch_pdl(k_resolve, grid, kResolveWarps * kWarp, smem, stream, s, st, b, pc);
  else
    launch_pdl(k_resolve_lean, grid, kResolveWarps * kWarp, smem, stream, s, st, b, pc);
}

void launch_resolve_team(const SessionDev &s, const StageDev &st, const BatchDev &b, bool full,
                         cudaStream_t stream, const PendingCommit &pc) {
  const uint32_t n = b.i1 - b.i0;
  if (n == 0 && pc.n == 0) return;
  uint32_t grid = n < 152u * 16u ? n : 152u * 16u;
  grid = std::max(grid, std::min(152u * 16u, cdiv(pc.n, kTeamThreads)));
  if (full && team_full_smem_bytes(s.k, s.m) <= kTeamFullMaxSmem && n <= 152u && pc.n == 0)
    // at most one item per SM of a GB300: twice the threads per item
    launch_pdl(k_resolve_team<kStepWideThreads, true>, grid, kStepWideThreads, team_full_smem_bytes(s.k, s.m), stream,
               s, st, b, pc);
  else if (full && team_full_smem_bytes(s.k, s.m) <= kTeamFullMaxSmem)
    launch_pdl(k_resolve_team<kTeamFullThreads, true>, grid, kTeamFullThreads, team_full_smem_bytes(s.k, s.m), stream, s,
               st, b, pc);
  else
    launch_pdl(k_resolve_team<kTeamThreads, false>, grid, kTeamThreads, team_smem_bytes(s.k, s.m), stream, s, st, b,
               pc);
}

void launch_step_team_full(const SessionDev &s, const StageDev &st, const BatchDev &b, cudaStream_t stream) {
  const uint32_t n = b.i1 - b.i0;
  if (n == 0) return;
  const uint32_t grid = n < 608u ? n : 608u;
  const uint32_t cap = exh_key_cap(s, b);
  const size_t smem = std::max<size_t>((size_t)cap * 8, team_full_smem_bytes(s.k, s.m));
  if (n <= 152u)  // at most one item per SM of a GB300
    launch_pdl(k_step_team_full<kStepWideThreads>, grid, kStepWideThreads, smem, stream, s, st, b, cap);
  else
    launch_pdl(k_step_team_full<kTeamFullThreads>, grid, kTeamFullThreads, smem, stream, s, st, b, cap);
}

void launch_commit(const SessionDev &s, const StageDev &st, const BatchDev &b, cudaStream_t stream) {
  const uint32_t n = b.i1 - b.i0;
  if (n == 0) return;
  launch_pdl(k_commit, cdiv(n, 256), 256, 0, stream, s, st, b);
}

void launch_level_switch(const SessionDev &s, uint32_t level, uint32_t n_res, cudaStream_t stream) {
  if (n_res == 0) return;
  launch_pdl(k_level_switch, cdiv(n_res, 256), 256, 0, stream, s, level, n_res);
}

void launch_pad(const uint32_t *src, uint32_t w, uint32_t h, uint32_t levels, uint32_t pitch, uint32_t *dst,
                cudaStream_t stream) {
  const size_t n = (size_t)pitch * (h + 2 * kPad) * levels;
  if (n == 0) return;
  k_pad<<<(uint32_t)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, stream>>>(src, w, h, levels, pitch, dst);
}

void launch_tree_append(const SessionDev &s, const StageDev &st, uint32_t a0, uint32_t a1, uint32_t pos0,
                        uint32_t nomir_end, cudaStream_t stream) {
  if (a1 <= a0) return;
  launch_pdl(k_tree_append, cdiv(a1 - a0, 256), 256, 0, stream, s, st, a0, a1, pos0, nomir_end);
}

void launch_rank_init(const SessionDev &s, uint32_t n, cudaStream_t stream) {
  if (n == 0) return;
  k_rank_init<<<cdiv(n, 256), 256, 0, stream>>>(s, n);
}

void launch_scatter_init(const uint32_t *list, uint32_t n, uint32_t *color, uint4 *state, uint32_t *res,
                         cudaStream_t stream) {
  if (n == 0) return;
  k_scatter_init<<<(n + 127) / 128, 128, 0, stream>>>(list, n, color, state, res);
}

void launch_transform_apply(const uint32_t *buf, size_t n, const uint32_t *texels, const uint4 *maps,
                            uint32_t n_maps, uint32_t *out, int *err, cudaStream_t stream) {
  if (n == 0) return;
  k_transform_apply<<<(uint32_t)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, stream>>>(buf, n, texels, maps,
                                                                                                n_maps, out, err);
}

void launch_debug_maps(const uint32_t *ids, size_t n, const uint32_t *flat, const float *score, size_t n_res,
                       uint32_t *patch_rgba, uint32_t *map_rgba, uint32_t *unc_rgba, cudaStream_t stream) {
  if (n > 0)
    k_id_maps<<<(uint32_t)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, stream>>>(ids, n, patch_rgba, map_rgba);
  if (n_res > 0)
    k_uncertainty<<<(uint32_t)std::min<size_t>((n_res + 255) / 256, 152 * 16), 256, 0, stream>>>(flat, score, n_res, n,
                                                                                                  unc_rgba);
}

void launch_luma_hist(const uint32_t *src, size_t n, uint8_t *luma, uint32_t *hist, cudaStream_t stream) {
  if (n == 0) return;
  k_luma_hist<<<(uint32_t)std::min<size_t>((n + 255) / 256, 152 * 4), 256, 0, stream>>>(src, n, luma, hist);
}

void launch_hist_r(const uint32_t *src, size_t n, uint32_t *hist, cudaStream_t stream) {
  if (n == 0) return;
  k_hist_r<<<(uint32_t)std::min<size_t>((n + 255) / 256, 152 * 4), 256, 0, stream>>>(src, n, hist);
}

void launch_apply_map(const uint8_t *luma, size_t n, const uint8_t *map, uint32_t *out, cudaStream_t stream) {
  if (n == 0) return;
  k_apply_map<<<(uint32_t)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, stream>>>(luma, n, map, out);
}

void launch_resize_v(const uint8_t *src, uint32_t w, uint32_t h, float *tmp, uint32_t nh, const uint4 *taps,
                     const float *wts, cudaStream_t stream) {
  if (w == 0 || nh == 0) return;
  dim3 grid(cdiv(w, 128), nh);
  k_resize_v<<<grid, 128, 0, stream>>>(src, w, h, tmp, nh, taps, wts);
}

void launch_resize_v_jobs(const ResizeJob *jobs, uint32_t n, uint32_t blocks, cudaStream_t stream) {
  if (n == 0 || blocks == 0) return;
  k_resize_v_jobs<<<blocks, 128, 0, stream>>>(jobs, n);
}

void launch_resize_h_jobs(const ResizeJob *jobs, uint32_t n, uint32_t blocks, cudaStream_t stream) {
  if (n == 0 || blocks == 0) return;
  k_resize_h_jobs<<<blocks, 128, 0, stream>>>(jobs, n);
}

void launch_resize_h(const float *tmp, uint32_t w, uint32_t nh, uint8_t *dst, uint32_t nw, const uint4 *taps,
                     const float *wts, cudaStream_t stream) {
  if (nw == 0 || nh == 0) return;
  dim3 grid(cdiv(nw, 128), nh);
  k_resize_h<<<grid, 128, 0, stream>>>(tmp, w, nh, dst, nw, taps, wts);
}

}  // namespace ts
