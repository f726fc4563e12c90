// ts_kernels.cuh — device data layout and kernel launchers of the synthesis
// hot loop (the internal interface between ts_session.cpp and ts_kernels.cu).
//
// Layout in device memory (one session):
//   levels  u32[ ]   every non-ignored example's pyramid, packed RGBA8
//                    (byte 0 = R); map f, level l at maps[f].off + l*w*h
//   masks   u8[ ]    sample-mask bytes (1 = may be sampled), maps[f].mask_off
//   guides  u32[ ]   example-guide pyramids, indexed by the unfiltered
//                    example index (the reference indexes its guide list with
//                    the filtered map id, ms.rs:1261-1266)
//   tguide  u32[levels][W*H]  target-guide pyramid
//   color   u32[W*H] output colour map
//   state   uint4[W*H] {src x | y<<16, patch id, id-map id, coord-map id}
//   occ/mir u32[H][ceil(W/32)] resolved-point bitmap / "has tiling mirrors"
//   resolved u32[], rscore f32[]  the resolved list and first-resolve scores
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

namespace ts {

// Padded level images: each level is also stored with a border of
// kPad texels of the out-of-bounds colour Rgba(0,0,0,255) (ms.rs:1139-1148),
// pitch pw = w + 2 kPad, so that a neighbourhood within kPad of an in-bounds
// centre reads the same values without bounds checks.
constexpr int kPad = 32;

struct MapDesc {
  uint32_t w, h;
  uint64_t off;      // texel offset of level 0
  int64_t mask_off;  // byte offset in the mask buffer, -1 = every texel valid
  uint64_t poff;     // texel offset of level 0's padded image (its (-kPad, -kPad) corner)
  uint32_t pw, ph;   // padded pitch (the session's common one) and height
};

struct GuideDesc {
  uint32_t w, h;
  uint64_t off;
};

enum : uint32_t { kResAppend = 1u, kResMirrors = 2u };

struct Result {
  uint32_t pixel, srcxy, idp, idm;
  uint32_t cmap, flags;
  float score;
  uint32_t ncand;
};

// Device status word values (0 = fine).
enum : int { kDevOk = 0, kDevErrIndex = 1, kDevErrNoSample = 2, kDevErrLimit = 3 };

struct SessionDev {
  const uint32_t *levels;
  const uint32_t *plevels;  // padded copies of levels, row pitch ppitch
  const uint32_t *pguides;  // padded guide of map f at maps[f].poff (when sizes agree)
  uint32_t ppitch;
  const uint8_t *masks;
  const MapDesc *maps;
  uint32_t n_maps;
  uint32_t n_levels;
  const uint32_t *guides;
  const GuideDesc *gdesc;
  uint32_t n_guides;
  int guided;
  const uint32_t *tguide;
  const double *xdiv;  // xdiv[x + xdiv_off] == (double)x / W
  const double *ydiv;
  int32_t xdiv_off, ydiv_off;
  // dxt[px * (2R+1) + dx + R] == xdiv[px + dx] - xdiv[px] and
  // dy2t[py * (2R+1) + dy + R] == dy * dy (dy likewise), for |dx|, |dy| <= R
  const double *dxt;
  const double *dy2t;
  int32_t dtab_r;
  uint32_t *color;
  uint4 *state;
  uint32_t *occ;
  uint32_t *mir;
  uint32_t *resolved;
  float *rscore;
  const int32_t *knn_tab;  // offsets (dx & 0xffff) | (dy << 16), sorted by (d2, dy, dx)
  uint32_t knn_tab_n;
  int *err;
  unsigned long long *evals;  // candidate-cost evaluations, summed by commit
  int guide_dims_differ;  // some example guide differs in size from its map
  // W and H are powers of two: every neighbour distance is an integer
  // multiple of 1/max(W,H)^2 and every partial sum of a distance list stays
  // below 2^53 such units, so the in-order f64 sum (ms.rs:417-421) is exact
  // and any order of exact adds gives its bits (exact_sum_ok on the host)
  int exact_sum;
  // with exact_sum: a neighbour at integer offset (dx, dy) lies at distance
  // ((dx^2 << exact_sx) + (dy^2 << exact_sy)) * exact_q, exact_q =
  // 1 / max(W, H)^2, exact_sx = 2 log2(max(W, H) / W), exact_sy likewise
  uint32_t exact_sx, exact_sy;
  double exact_q;
  int32_t exact_qe;  // exact_q = 2^exact_qe
  uint32_t W, H, wpr;  // wpr: 32-bit words per bitmap row
  int tiling;
  int32_t x_l, x_r, y_b, y_t;
  uint32_t k, m;
  // resolved points per kCell x kCell cell of the plane the tree spans
  // (the image plus the tiling bands), origin (cox, coy): cells[gy * cgw + gx]
  uint32_t *cells;
  int32_t cox, coy;
  uint32_t cgw, cgh;
  // Tree positions, for k-NN made ahead of the resolves (plain path,
  // k_tree_append): rank[p] = 1 + p's index in the resolved list, 0 while p
  // has none.  The bitmap, mirror bits, cell counts and resolved list then
  // already hold the points of whole chunks of later batches; a point is in
  // an item's tree when its index is below the item's batch-start length.
  // Null: the bitmap is the tree itself (commits grow it).
  uint32_t *rank;
  // k-NN ahead: for the pixels whose commit a batch step left to the next
  // step's resolve launch (BatchDev::defer_tag), the colour and state that
  // commit writes: shadow[2p] = {tag, colour, 0, 0}, shadow[2p + 1] = state;
  // zeroed at the start
  uint4 *shadow;
};

constexpr int kCell = 8;

// Radius of the sorted k-NN offset table: every lattice offset with
// dx^2 + dy^2 <= kKnnTabRadius^2.
constexpr int kKnnTabRadius = 36;

struct StageDev {
  uint32_t level;
  int slow_lut;            // LUT holds a non-finite value: exact sequential argmin
  // Every texel the cost loop can compare has alpha 255 and both LUTs hold
  // +-0 at |a - b| = 0: the alpha channel's term adds +-0 to a partial sum,
  // which leaves it unchanged, so the fast cost loops skip it
  int opaque;
  const float *lut;        // [2][256]: content, guide
  uint64_t stage_seed;
  const uint32_t *items;   // item -> pixel for this stage
  uint32_t n_items;
  uint32_t redo;
  uint2 *rcand;            // [n_items][m] random candidates {x | y<<16, map}
};

struct BatchDev {
  uint32_t i0, i1;       // stage items [i0, i1)
  uint32_t n_res;        // resolved-list length at batch start
  uint32_t append_from;  // items >= append_from append to the resolved list
  int32_t *nbuf;         // [batch][k] neighbour offsets
  uint32_t *ncnt;        // [batch] neighbour counts
  uint32_t *fb_list;     // items needing the exhaustive k-NN
  uint32_t *fb_count;
  double *dist;          // [k][batch] squared normalised distances
  double *mean;          // [batch] mean of the 4x-duplicated distance list
  Result *res;           // [batch]
  int grid_first;        // sparse step: search the cell grid without walking the offset table first
  int walk_window;       // small step (latency-bound): the single-session walk lets sparse items walk a shared-memory bitmap window
  int fused_commit;      // only new items: the resolve kernels commit each item themselves (no k_commit)
  // k-NN made ahead over several batches (SessionDev::rank): btab[j] =
  // {first stage item, resolved-list length at the start} of the j-th batch
  // the launch covers, ascending; null: every item's tree has n_res points
  const uint2 *btab;
  uint32_t nbt;
  // Commit of a batch left to the next step (k-NN ahead): a launch with
  // defer_tag != 0 keeps its results in res and their colour and state in
  // SessionDev::shadow under that tag; the next batch step (prev_tag == the
  // tag) commits them while it runs (PendingCommit) and reads a tagged
  // pixel's batch-start colour and state from the shadow instead of the image
  uint32_t defer_tag, prev_tag;
  // warp resolve of the plain path: a counter (zeroed) from which the warps
  // of a resident grid take items after their first, so that no warp waits
  // for its block's slowest item; null: one item per warp of a full grid
  uint32_t *work_ctr;
};

// One batch step of one session as the multi-session kernels read it.
struct StepDev {
  StageDev st;         // stage view of the step's random-candidate chunk
  StageDev rc;         // the same chunk as random_candidates sees it (its own seed)
  BatchDev b;
  uint32_t level;      // level switch: new level and resolved-list length
  uint32_t ls_n_res;
  int all_items;       // exhaustive k-NN over every item of the batch
  int pad;
};

// A run of `nblocks` blocks, from block0 on, working on step `step` of
// session slot `session`.
struct Segment {
  uint32_t block0, nblocks, session, step;
};

// Parameters of one multi-session launch: segments sorted by block0;
// sessions[slot] and step_tabs[slot][step] describe a segment's work.  The
// exhaustive k-NN also drains the walk's fallback lists of the steps in
// `fb` with the blocks from pool_block0 on (whose count is known only on
// the device).
struct MultiLaunch {
  const Segment *segs;
  uint32_t n_segs;
  const SessionDev *sessions;
  const StepDev *const *step_tabs;
  const Segment *fb;
  uint32_t n_fb;
  uint32_t pool_block0;
  uint32_t block_base = 0;  // block index of this launch's first block in the segment numbering
  // resolve phase: the first n_lean segments (lean_blocks blocks) belong to
  // sessions without guides
  uint32_t n_lean = 0, lean_blocks = 0;
  // exhaustive phase: keys held in dynamic shared memory (exh_key_cap, the
  // largest over the launch's steps)
  uint32_t key_cap = 8192;
};

// Phases of a batch step, in launch order.
enum : int {
  kPhaseLevelSwitch = 0,
  kPhaseRandom,
  kPhaseWalk,
  kPhaseExhaustive,
  kPhaseMean,
  kPhaseResolve,
  kPhaseTeamPart,
  kPhaseTeamFull,
  kPhaseCommit,
  kPhases
};

// Threads per block, blocks for a segment of n units (items, or resolved
// points for the level switch; `cap` bounds the grid-stride phases, 0 = no
// bound) and dynamic shared memory of each phase's multi-session kernel.
uint32_t multi_threads(int phase);
uint32_t multi_blocks(int phase, uint32_t n, uint32_t cap);
size_t multi_smem_bytes(int phase, uint32_t k, uint32_t m);
void launch_multi(int phase, const MultiLaunch &ml, uint32_t blocks, size_t smem, cudaStream_t stream);
// Lets a phase's multi-session kernel use `bytes` of dynamic shared memory
// (current device).
cudaError_t set_multi_smem(int phase, size_t bytes);
// Keys the exhaustive k-NN holds in shared memory for a step (8 bytes each).
uint32_t exh_key_cap(const SessionDev &s, const BatchDev &b);
// Whether the full-evaluation team form has room for (k, m).
bool team_full_fits(uint32_t k, uint32_t m);

// Launchers (stream-ordered, no synchronisation).
void launch_random_candidates(const SessionDev &s, const StageDev &st, cudaStream_t stream);
// The commit of an earlier step that a k-NN launch makes before its own
// work (n = 0: none).  Only for batches of redo items: their commit writes
// colour, state and the eval count, which the k-NN kernels never read, and
// appends nothing to the resolved list, bitmap or cell counts, which they
// do read.
struct PendingCommit {
  StageDev st;
  BatchDev b;
  uint32_t n;
};

void launch_knn_walk(const SessionDev &s, const StageDev &st, const BatchDev &b, cudaStream_t stream,
                     const PendingCommit &pc = PendingCommit{});
// all_items: every item of the batch (and the mean too); otherwise the items
// the walk left in fb_list.
void launch_knn_exhaustive(const SessionDev &s, const StageDev &st, const BatchDev &b, bool all_items,
                           cudaStream_t stream, const PendingCommit &pc = PendingCommit{});
void launch_mean(const SessionDev &s, const StageDev &st, const BatchDev &b, cudaStream_t stream);
void launch_resolve(const SessionDev &s, const StageDev &st, const BatchDev &b, cudaStream_t stream,
                    const PendingCommit &pc = PendingCommit{});
// One CTA per item; `full` scores every candidate completely (lowest latency,
// for batches far too small to fill the GPU), otherwise candidate 0 first
// and the rest with early exit.
void launch_resolve_team(const SessionDev &s, const StageDev &st, const BatchDev &b, bool full, cudaStream_t stream,
                         const PendingCommit &pc = PendingCommit{});
// One step of a batch whose neighbours the exhaustive k-NN finds, resolved
// in the full-evaluation team form (when team_full_fits): both in one
// launch, one CTA per item.
void launch_step_team_full(const SessionDev &s, const StageDev &st, const BatchDev &b, cudaStream_t stream);
void launch_commit(const SessionDev &s, const StageDev &st, const BatchDev &b, cudaStream_t stream);
void launch_level_switch(const SessionDev &s, uint32_t level, uint32_t n_res, cudaStream_t stream);

// Initial state of the pixels set before the first stage (random init):
// list[6i..6i+6] = {pixel, colour, state.x, state.y, state.z, state.w};
// res[i] = pixel (the resolved list starts with them, in list order).
// k-NN ahead (SessionDev::rank): the tree entries of stage items [a0, a1),
// every one appended at resolved-list index pos0 + (i - a0); items below
// nomir_end (a batch that met an empty tree) get no tiling mirrors.
void launch_tree_append(const SessionDev &s, const StageDev &st, uint32_t a0, uint32_t a1, uint32_t pos0,
                        uint32_t nomir_end, cudaStream_t stream);
// rank of the first n resolved-list entries (the initial tree).
void launch_rank_init(const SessionDev &s, uint32_t n, cudaStream_t stream);
void launch_scatter_init(const uint32_t *list, uint32_t n, uint32_t *color, uint4 *state, uint32_t *res,
                         cudaStream_t stream);

// CoordinateTransform::apply: out[i] = texel buf[3i..3i+3] = (x, y, map) of
// the maps {offset low, offset high, w, h}; *err set for entries outside.
void launch_transform_apply(const uint32_t *buf, size_t n, const uint32_t *texels, const uint4 *maps,
                            uint32_t n_maps, uint32_t *out, int *err, cudaStream_t stream);
// Debug maps: patch-id and map-id colours of the n pixels' (patch, map) ids,
// and the uncertainty colours of the n_res resolved entries (unc_rgba must
// start zeroed).
void launch_debug_maps(const uint32_t *ids, size_t n, const uint32_t *flat, const float *score, size_t n_res,
                       uint32_t *patch_rgba, uint32_t *map_rgba, uint32_t *unc_rgba, cudaStream_t stream);

// Automatic guide maps: luma of RGBA8 with its histogram (hist: 256 zeroed
// counters), the histogram of channel 0, and map[luma] as (n, n, n, 255).
void launch_luma_hist(const uint32_t *src, size_t n, uint8_t *luma, uint32_t *hist, cudaStream_t stream);
void launch_hist_r(const uint32_t *src, size_t n, uint32_t *hist, cudaStream_t stream);
void launch_apply_map(const uint8_t *luma, size_t n, const uint8_t *map, uint32_t *out, cudaStream_t stream);

// Separable resize (image 0.23 imageops::resize): taps[o] = {left, count,
// weight offset}; vertical pass u8 -> f32, horizontal pass f32 -> u8.
void launch_resize_v(const uint8_t *src, uint32_t w, uint32_t h, float *tmp, uint32_t nh, const uint4 *taps,
                     const float *wts, cudaStream_t stream);
void launch_resize_h(const float *tmp, uint32_t w, uint32_t nh, uint8_t *dst, uint32_t nw, const uint4 *taps,
                     const float *wts, cudaStream_t stream);

// Many resizes in one launch per pass: job j resizes src (w x h) to dst
// (nw x nh) through tmp (w x nh floats), the taps as above; block0 is the
// job's first block of the pass (jobs sorted by it, the last entry the total).
struct ResizeJob {
  const uint8_t *src;
  uint8_t *dst;
  float *tmp;
  const uint4 *tv, *th;
  const float *wv, *wh;
  uint32_t w, h, nw, nh;
  uint32_t block0_v, block0_h;
};
// Vertical passes of jobs [0, n) (blocks: jobs[n].block0_v in total) and
// horizontal passes (jobs[n].block0_h); jobs in device memory.
void launch_resize_v_jobs(const ResizeJob *jobs, uint32_t n, uint32_t blocks, cudaStream_t stream);
void launch_resize_h_jobs(const ResizeJob *jobs, uint32_t n, uint32_t blocks, cudaStream_t stream);

// Padded copy of `levels` images of w x h texels (see kPad) with row pitch
// `pitch` >= w + 2 kPad.
void launch_pad(const uint32_t *src, uint32_t w, uint32_t h, uint32_t levels, uint32_t pitch, uint32_t *dst,
                cudaStream_t stream);

// Bytes of dynamic shared memory the resolve kernel needs per CTA.
size_t resolve_smem_bytes(uint32_t k, uint32_t m, int guided);
// Per-device kernel attributes for a (k, m) session (current device).
cudaError_t configure_kernels(uint32_t k, uint32_t m);

}  // namespace ts
