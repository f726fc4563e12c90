// ts_session.cpp — the C ABI (include/tsgpu.h): session builder, build() and
// run() of the synthesis hot loop on one CUDA device.
//
// build() mirrors SessionBuilder::build (session.rs:336-448): parameter and
// image validation, input resizes, example / guide pyramids (built on the
// device), generator initialisation.  run() mirrors Session::run
// (session.rs:37-66) and Generator::resolve (ms.rs:702-1051): the host lays
// out the whole data-independent schedule (stage seeds and sizes, the order
// in which unresolved pixels are picked, the batch steps, the cost tables),
// uploads it once and enqueues every kernel on one stream; the only
// synchronisation is at the end (and once per stage when a progress callback
// is given).
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <cmath>

#include <algorithm>
#include <chrono>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/tsgpu.h"
#include "ts_common.h"
#include "ts_kernels.cuh"
#include "ts_resample.h"

using namespace ts;

namespace {

constexpr uint32_t kMaxK = 256;
constexpr uint32_t kMaxM = 1024;
constexpr uint32_t kMaxExamples = 256;
constexpr uint32_t kMaxSide = 16384;
constexpr float kTilingBoundary = 0.05f;  // TILING_BOUNDARY_PERCENTAGE, ms.rs:15
constexpr int kKnnTabRadius = 36;
constexpr int kDistTabRadius = 64;  // offsets the weight tables cover
constexpr uint64_t kRcandBudget = 64ull << 20;  // random-candidate entries held at once

struct Image {
  std::vector<uint8_t> px;  // RGBA8
  uint32_t w = 0, h = 0;
  bool empty() const { return w == 0 && h == 0 && px.empty(); }
};

struct ExampleIn {
  Image img;
  bool has_guide = false;
  Image guide;
  int method = TS_SAMPLE_ALL;
  Image mask;
};

struct InpaintIn {
  bool channel = false;
  int ch = 0;
  Image mask;
  uint32_t example_index = 0;
  uint32_t w = 0, h = 0;
};

struct Params {
  bool tiling = false;
  uint32_t k = 50;
  uint64_t m = 50;
  float cauchy = 1.0f;
  float backtrack_percent = 0.5f;
  uint32_t backtrack_stages = 5;
  bool has_resize_input = false;
  uint32_t resize_w = 0, resize_h = 0;
  uint32_t out_w = 500, out_h = 500;
  float alpha = 0.8f;
  bool has_random_init = false;
  uint64_t random_init = 0;
  bool has_max_threads = false;
  uint64_t max_threads = 0;
  uint64_t seed = 0;
  uint32_t batch_divisor = 8;
  uint32_t max_batch = 0;
  int device = 0;
  bool profile = false;
  uint32_t team_max_batch = 8192;
  uint32_t team_full_max_batch = 1024;
};

std::string fmt_float(float v) {
  char buf[64];
  snprintf(buf, sizeof(buf), "%g", (double)v);
  return buf;
}

template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { reset(); }
  void reset() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t count) {
    reset();
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)&p, count * sizeof(T));
    if (e == cudaSuccess) n = count;
    return e;
  }
};

struct Failure {
  int status;
  std::string msg;
};

#define CUDA_TRY(expr)                                                                      \
  do {                                                                                     \
    cudaError_t _e = (expr);                                                               \
    if (_e != cudaSuccess) throw Failure{_e == cudaErrorMemoryAllocation ? TS_ERR_OUT_OF_MEMORY : TS_ERR_CUDA, \
                                         std::string(#expr) + ": " + cudaGetErrorString(_e)}; \
  } while (0)

bool check_image(const uint8_t *p, uint32_t w, uint32_t h) { return p != nullptr && w > 0 && h > 0; }

Image copy_image(const uint8_t *p, uint32_t w, uint32_t h) {
  Image im;
  im.w = w;
  im.h = h;
  im.px.assign(p, p + (size_t)w * h * 4);
  return im;
}

// Upload taps of one axis: {left, count, offset} per output + weights.
struct DevTaps {
  DevBuf<uint4> taps;
  DevBuf<float> wts;
};
void upload_taps(const Taps &t, DevTaps &d, cudaStream_t st) {
  std::vector<uint4> v(t.left.size());
  for (size_t i = 0; i < v.size(); ++i) v[i] = make_uint4(t.left[i], t.count[i], t.offset[i], 0);
  CUDA_TRY(d.taps.alloc(v.size()));
  CUDA_TRY(d.wts.alloc(t.weights.size()));
  if (!v.empty()) CUDA_TRY(cudaMemcpyAsync(d.taps.p, v.data(), v.size() * sizeof(uint4), cudaMemcpyHostToDevice, st));
  if (!t.weights.empty())
    CUDA_TRY(cudaMemcpyAsync(d.wts.p, t.weights.data(), t.weights.size() * 4, cudaMemcpyHostToDevice, st));
}

// imageops::resize on the device: src (device u8, w x h) -> dst (device u8,
// nw x nh).  Synchronises the stream before returning (the taps are freed).
void device_resize(const uint8_t *src, uint32_t w, uint32_t h, uint8_t *dst, uint32_t nw, uint32_t nh, Filter f,
                   cudaStream_t st) {
  if (nw == 0 || nh == 0) return;
  DevTaps tv, th;
  upload_taps(axis_taps(f, h, nh), tv, st);
  upload_taps(axis_taps(f, w, nw), th, st);
  DevBuf<float> tmp;
  CUDA_TRY(tmp.alloc((size_t)w * nh * 4));
  CUDA_TRY(cudaMemsetAsync(tmp.p, 0, (size_t)w * nh * 4 * sizeof(float), st));
  if (h > 0) launch_resize_v(src, w, h, tmp.p, nh, tv.taps.p, tv.wts.p, st);
  if (w > 0) {
    launch_resize_h(tmp.p, w, nh, dst, nw, th.taps.p, th.wts.p, st);
  } else {
    CUDA_TRY(cudaMemsetAsync(dst, 0, (size_t)nw * nh * 4, st));
  }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(st));
}

// load_image (utils.rs:55-80): resize with CatmullRom when a size is given
// and differs.  Runs on the device; returns the host image.
Image load_image(const Image &in, bool has_size, uint32_t w, uint32_t h, cudaStream_t st) {
  if (!has_size || (in.w == w && in.h == h)) return in;
  DevBuf<uint8_t> a, b;
  CUDA_TRY(a.alloc(in.px.size()));
  CUDA_TRY(b.alloc((size_t)w * h * 4));
  CUDA_TRY(cudaMemcpyAsync(a.p, in.px.data(), in.px.size(), cudaMemcpyHostToDevice, st));
  device_resize(a.p, in.w, in.h, b.p, w, h, kCatmullRom, st);
  Image out;
  out.w = w;
  out.h = h;
  out.px.resize((size_t)w * h * 4);
  CUDA_TRY(cudaMemcpy(out.px.data(), b.p, out.px.size(), cudaMemcpyDeviceToHost));
  return out;
}

// ImagePyramid::new(img, Some(levels)) (img_pyramid.rs:7-37) written into
// dst (device, max(levels,1) images of w*h texels).
void device_pyramid(const Image &img, uint32_t levels, uint32_t *dst, cudaStream_t st) {
  const uint32_t nl = levels == 0 ? 1 : levels;
  const size_t sz = (size_t)img.w * img.h;
  uint8_t *base = (uint8_t *)dst;
  CUDA_TRY(cudaMemcpyAsync(base + (size_t)(nl - 1) * sz * 4, img.px.data(), sz * 4, cudaMemcpyHostToDevice, st));
  const uint8_t *orig = base + (size_t)(nl - 1) * sz * 4;
  for (uint32_t l = 0; l + 1 < nl; ++l) {
    const uint32_t i = nl - 1 - l;
    const uint32_t p = 1u << i;
    const uint32_t sw = img.w / p, sh = img.h / p;
    DevBuf<uint8_t> small;
    CUDA_TRY(small.alloc((size_t)sw * sh * 4));
    if (sw == 0 || sh == 0) {
      // a zero-sized intermediate makes the crate return a zero image
      CUDA_TRY(cudaMemsetAsync(base + (size_t)l * sz * 4, 0, sz * 4, st));
      continue;
    }
    device_resize(orig, img.w, img.h, small.p, sw, sh, kGaussian, st);
    device_resize(small.p, sw, sh, base + (size_t)l * sz * 4, img.w, img.h, kGaussian, st);
  }
}

inline uint32_t pcg_stage_seed(uint64_t seed) {
  Pcg32 g = pcg_from_u64(seed);
  return pcg_u32(g);
}

}  // namespace

// ---------------------------------------------------------------------------
// Objects behind the opaque handles.
// ---------------------------------------------------------------------------
struct ts_builder {
  Params prm;
  std::vector<ExampleIn> examples;
  bool has_target = false;
  Image target;
  bool has_inpaint = false;
  InpaintIn inpaint;
  bool consumed = false;
  std::string err;
};

struct ts_session {
  Params prm;
  uint32_t W = 0, H = 0;
  uint32_t n_ex = 0, n_maps = 0, n_levels = 1;
  bool guided = false;
  std::vector<uint32_t> filtered;            // filtered map -> unfiltered example index
  std::vector<MapDesc> maps;
  std::vector<Image> bottoms;                // every example at its loaded size (random init)
  bool inpaint = false;
  uint32_t inpaint_index = 0;
  Image inpaint_colors;
  std::vector<uint8_t> inpaint_mask;         // W*H: 1 = to synthesise
  DevBuf<uint32_t> levels, guides, tguide, plevels, pguides;
  bool guide_dims_differ = false;
  DevBuf<uint8_t> masks;
  DevBuf<MapDesc> d_maps;
  DevBuf<GuideDesc> d_gdesc;
  bool consumed = false;
  std::string err;
};

struct ts_generated {
  uint32_t W = 0, H = 0;
  std::vector<uint8_t> image;
  std::vector<uint32_t> coord;  // 3 per pixel
  std::vector<uint32_t> ids;    // 2 per pixel
  std::vector<uint32_t> resolved;
  std::vector<float> scores;
  ts_run_stats stats{};
  std::vector<ts_launch_record> launches;
};

extern "C" {

const char *ts_status_str(int s) {
  switch (s) {
    case TS_OK: return "ok";
    case TS_ERR_INVALID_RANGE: return "invalid range";
    case TS_ERR_SIZE_MISMATCH: return "size mismatch";
    case TS_ERR_EXAMPLE_GUIDE_MISMATCH: return "example guide mismatch";
    case TS_ERR_NO_EXAMPLES: return "no examples";
    case TS_ERR_MAPS_COUNT_MISMATCH: return "maps count mismatch";
    case TS_ERR_IMAGE: return "image";
    case TS_ERR_UNSUPPORTED: return "unsupported";
    case TS_ERR_NO_VALID_SAMPLE: return "no valid sample";
    case TS_ERR_INDEX: return "index out of range";
    case TS_ERR_CUDA: return "cuda";
    case TS_ERR_STATE: return "invalid state";
    case TS_ERR_LIMIT: return "limit exceeded";
    case TS_ERR_OUT_OF_MEMORY: return "out of memory";
    case TS_ERR_NULL: return "null argument";
    default: return "unknown";
  }
}

void ts_get_limits(ts_limits *out) {
  if (!out) return;
  out->max_nearest_neighbors = kMaxK;
  out->max_random_sample_locations = kMaxM;
  out->max_examples = kMaxExamples;
  out->max_image_side = kMaxSide;
}

int ts_image_pyramid(const uint8_t *rgba, uint32_t w, uint32_t h, uint32_t levels, uint8_t *out, int32_t device) {
  if (!rgba || !out) return TS_ERR_NULL;
  if (w == 0 || h == 0) return TS_ERR_IMAGE;
  if (w > kMaxSide || h > kMaxSide || levels > 30) return TS_ERR_LIMIT;
  try {
    CUDA_TRY(cudaSetDevice(device));
    const uint32_t nl = levels == 0 ? 1 : levels;
    Image img = copy_image(rgba, w, h);
    DevBuf<uint32_t> d;
    CUDA_TRY(d.alloc((size_t)w * h * nl));
    device_pyramid(img, levels, d.p, 0);
    CUDA_TRY(cudaMemcpy(out, d.p, (size_t)w * h * nl * 4, cudaMemcpyDeviceToHost));
  } catch (const Failure &f) {
    return f.status;
  }
  return TS_OK;
}

ts_builder *ts_builder_new(void) { return new (std::nothrow) ts_builder(); }
void ts_builder_free(ts_builder *b) { delete b; }
const char *ts_builder_last_error(const ts_builder *b) { return b ? b->err.c_str() : "null builder"; }

#define BUILDER_GUARD(b)                    \
  if (!(b)) return TS_ERR_NULL;             \
  if ((b)->consumed) {                      \
    (b)->err = "builder already consumed";  \
    return TS_ERR_STATE;                    \
  }

static int read_example(ts_builder *b, const ts_example_desc *ex, ExampleIn &out) {
  if (!ex || !check_image(ex->rgba, ex->width, ex->height)) {
    b->err = "example image buffer is empty";
    return TS_ERR_IMAGE;
  }
  out.img = copy_image(ex->rgba, ex->width, ex->height);
  if (ex->guide_rgba) {
    if (!check_image(ex->guide_rgba, ex->guide_width, ex->guide_height)) {
      b->err = "example guide buffer is empty";
      return TS_ERR_IMAGE;
    }
    out.has_guide = true;
    out.guide = copy_image(ex->guide_rgba, ex->guide_width, ex->guide_height);
  }
  if (ex->sample_method < TS_SAMPLE_ALL || ex->sample_method > TS_SAMPLE_IMAGE) {
    b->err = "unknown sample method";
    return TS_ERR_INVALID_RANGE;
  }
  out.method = ex->sample_method;
  if (out.method == TS_SAMPLE_IMAGE) {
    if (!check_image(ex->mask_rgba, ex->mask_width, ex->mask_height)) {
      b->err = "sample mask buffer is empty";
      return TS_ERR_IMAGE;
    }
    out.mask = copy_image(ex->mask_rgba, ex->mask_width, ex->mask_height);
  }
  return TS_OK;
}

int ts_builder_add_example(ts_builder *b, const ts_example_desc *ex) {
  BUILDER_GUARD(b);
  ExampleIn e;
  int rc = read_example(b, ex, e);
  if (rc) return rc;
  b->examples.push_back(std::move(e));
  return TS_OK;
}

int ts_builder_inpaint_example(ts_builder *b, const uint8_t *mask_rgba, uint32_t mw, uint32_t mh,
                               const ts_example_desc *ex, uint32_t w, uint32_t h) {
  BUILDER_GUARD(b);
  if (!check_image(mask_rgba, mw, mh)) {
    b->err = "inpaint mask buffer is empty";
    return TS_ERR_IMAGE;
  }
  ExampleIn e;
  int rc = read_example(b, ex, e);
  if (rc) return rc;
  b->has_inpaint = true;
  b->inpaint = InpaintIn();
  b->inpaint.mask = copy_image(mask_rgba, mw, mh);
  b->inpaint.example_index = (uint32_t)b->examples.size();
  b->inpaint.w = w;
  b->inpaint.h = h;
  b->examples.push_back(std::move(e));
  return TS_OK;
}

int ts_builder_inpaint_example_channel(ts_builder *b, int32_t channel, const ts_example_desc *ex, uint32_t w,
                                       uint32_t h) {
  BUILDER_GUARD(b);
  if (channel < 0 || channel > 3) {
    b->err = "channel must be 0..3 (R, G, B, A)";
    return TS_ERR_INVALID_RANGE;
  }
  ExampleIn e;
  int rc = read_example(b, ex, e);
  if (rc) return rc;
  b->has_inpaint = true;
  b->inpaint = InpaintIn();
  b->inpaint.channel = true;
  b->inpaint.ch = channel;
  b->inpaint.example_index = (uint32_t)b->examples.size();
  b->inpaint.w = w;
  b->inpaint.h = h;
  b->examples.push_back(std::move(e));
  return TS_OK;
}

int ts_builder_load_target_guide(ts_builder *b, const uint8_t *rgba, uint32_t w, uint32_t h) {
  BUILDER_GUARD(b);
  if (!check_image(rgba, w, h)) {
    b->err = "target guide buffer is empty";
    return TS_ERR_IMAGE;
  }
  b->has_target = true;
  b->target = copy_image(rgba, w, h);
  return TS_OK;
}

int ts_builder_resize_input(ts_builder *b, uint32_t w, uint32_t h) {
  BUILDER_GUARD(b);
  b->prm.has_resize_input = true;
  b->prm.resize_w = w;
  b->prm.resize_h = h;
  return TS_OK;
}
int ts_builder_seed(ts_builder *b, uint64_t seed) {
  BUILDER_GUARD(b);
  b->prm.seed = seed;
  return TS_OK;
}
int ts_builder_tiling_mode(ts_builder *b, int32_t tiling) {
  BUILDER_GUARD(b);
  b->prm.tiling = tiling != 0;
  return TS_OK;
}
int ts_builder_nearest_neighbors(ts_builder *b, uint32_t count) {
  BUILDER_GUARD(b);
  b->prm.k = count;
  return TS_OK;
}
int ts_builder_random_sample_locations(ts_builder *b, uint64_t count) {
  BUILDER_GUARD(b);
  b->prm.m = count;
  return TS_OK;
}
int ts_builder_random_init(ts_builder *b, uint64_t count) {
  BUILDER_GUARD(b);
  b->prm.has_random_init = true;
  b->prm.random_init = count;
  return TS_OK;
}
int ts_builder_cauchy_dispersion(ts_builder *b, float v) {
  BUILDER_GUARD(b);
  b->prm.cauchy = v;
  return TS_OK;
}
int ts_builder_guide_alpha(ts_builder *b, float v) {
  BUILDER_GUARD(b);
  b->prm.alpha = v;
  return TS_OK;
}
int ts_builder_backtrack_percent(ts_builder *b, float v) {
  BUILDER_GUARD(b);
  b->prm.backtrack_percent = v;
  return TS_OK;
}
int ts_builder_backtrack_stages(ts_builder *b, uint32_t stages) {
  BUILDER_GUARD(b);
  b->prm.backtrack_stages = stages;
  return TS_OK;
}
int ts_builder_output_size(ts_builder *b, uint32_t w, uint32_t h) {
  BUILDER_GUARD(b);
  b->prm.out_w = w;
  b->prm.out_h = h;
  return TS_OK;
}
int ts_builder_max_thread_count(ts_builder *b, uint64_t count) {
  BUILDER_GUARD(b);
  b->prm.has_max_threads = true;
  b->prm.max_threads = count;
  return TS_OK;
}
int ts_builder_batch_schedule(ts_builder *b, uint32_t divisor, uint32_t max_batch) {
  BUILDER_GUARD(b);
  b->prm.batch_divisor = divisor;
  b->prm.max_batch = max_batch;
  return TS_OK;
}
int ts_builder_device(ts_builder *b, int32_t device) {
  BUILDER_GUARD(b);
  b->prm.device = device;
  return TS_OK;
}
int ts_builder_resolve_team(ts_builder *b, uint32_t team_max_batch, uint32_t full_max_batch) {
  BUILDER_GUARD(b);
  b->prm.team_max_batch = team_max_batch;
  b->prm.team_full_max_batch = full_max_batch;
  return TS_OK;
}
int ts_builder_profile_kernels(ts_builder *b, int32_t on) {
  BUILDER_GUARD(b);
  b->prm.profile = on != 0;
  return TS_OK;
}

}  // extern "C"

namespace {

// check_parameters_validity (session.rs:450-499); NaN passes, as there.
int check_parameters(const Params &p, std::string &err) {
  auto range = [&](float v, const char *name) {
    err = std::string("parameter '") + name + "' - value '" + fmt_float(v) + "' is outside the range of 0-1";
    return TS_ERR_INVALID_RANGE;
  };
  if (p.cauchy < 0.0f || p.cauchy > 1.0f) return range(p.cauchy, "cauchy-dispersion");
  if (p.backtrack_percent < 0.0f || p.backtrack_percent > 1.0f) return range(p.backtrack_percent, "backtrack-percent");
  if (p.alpha < 0.0f || p.alpha > 1.0f) return range(p.alpha, "guide-alpha");
  if (p.has_max_threads && p.max_threads == 0) {
    err = "parameter 'max-thread-count' - value '0' is outside the range of 1-1024";
    return TS_ERR_INVALID_RANGE;
  }
  if (p.m == 0) {
    err = "parameter 'm-rand' - value '0' is outside the range of 1-1024";
    return TS_ERR_INVALID_RANGE;
  }
  return TS_OK;
}

int check_limits(const ts_builder &b, uint32_t W, uint32_t H, std::string &err) {
  const Params &p = b.prm;
  if (p.k > kMaxK) {
    err = "nearest_neighbors " + std::to_string(p.k) + " exceeds this library's limit of " + std::to_string(kMaxK);
    return TS_ERR_LIMIT;
  }
  if (p.m > kMaxM) {
    err = "random_sample_locations " + std::to_string(p.m) + " exceeds this library's limit of " +
          std::to_string(kMaxM);
    return TS_ERR_LIMIT;
  }
  if (b.examples.size() > kMaxExamples) {
    err = "more than " + std::to_string(kMaxExamples) + " examples";
    return TS_ERR_LIMIT;
  }
  if (W == 0 || H == 0) {
    err = "output size must be non-zero";
    return TS_ERR_IMAGE;
  }
  if (W > kMaxSide || H > kMaxSide) {
    err = "output side exceeds " + std::to_string(kMaxSide);
    return TS_ERR_LIMIT;
  }
  return TS_OK;
}

}  // namespace

extern "C" int ts_builder_build(ts_builder *b, ts_session **out) {
  BUILDER_GUARD(b);
  if (!out) return TS_ERR_NULL;
  *out = nullptr;
  b->consumed = true;
  const Params &p = b->prm;
  int rc = check_parameters(p, b->err);
  if (rc) return rc;
  // check_images_validity (session.rs:501-524)
  size_t input_count = 0, num_guides = 0;
  for (auto &e : b->examples) {
    if (e.method != TS_SAMPLE_IGNORE) ++input_count;
    if (e.has_guide) ++num_guides;
  }
  if (input_count == 0) {
    b->err = "at least 1 example must be available as a sampling source";
    return TS_ERR_NO_EXAMPLES;
  }
  if (num_guides != 0 && b->examples.size() != num_guides) {
    const size_t ne = b->examples.size();
    b->err = std::to_string(ne) + " examples were provided, but " + (ne > num_guides ? "only " : "") +
             std::to_string(num_guides) + " guides were";
    return TS_ERR_EXAMPLE_GUIDE_MISMATCH;
  }
  uint32_t W, H;
  bool has_in = p.has_resize_input;
  uint32_t in_w = p.resize_w, in_h = p.resize_h;
  if (b->has_inpaint) {
    W = b->inpaint.w;
    H = b->inpaint.h;
    has_in = true;
    in_w = W;
    in_h = H;
  } else {
    W = p.out_w;
    H = p.out_h;
  }
  rc = check_limits(*b, W, H, b->err);
  if (rc) return rc;
  if (b->has_target && num_guides == 0) {
    b->err = "style transfer (a target guide without example guides) needs automatic guide maps, which this "
             "library does not build; pass example guides";
    return TS_ERR_UNSUPPORTED;
  }
  std::unique_ptr<ts_session> s(new (std::nothrow) ts_session());
  if (!s) return TS_ERR_OUT_OF_MEMORY;
  s->prm = p;
  s->W = W;
  s->H = H;
  s->n_ex = (uint32_t)b->examples.size();
  s->n_levels = p.backtrack_stages == 0 ? 1 : p.backtrack_stages;
  s->guided = b->has_target;
  try {
    CUDA_TRY(cudaSetDevice(p.device));
    cudaStream_t st = 0;
    CUDA_TRY(configure_kernels(p.k, (uint32_t)p.m));
    // inputs at their final sizes (Example::resolve, lib.rs:564-603)
    std::vector<Image> imgs(s->n_ex), guides(s->n_ex), masks(s->n_ex);
    for (uint32_t e = 0; e < s->n_ex; ++e) {
      const ExampleIn &ex = b->examples[e];
      imgs[e] = load_image(ex.img, has_in, in_w, in_h, st);
      if (imgs[e].w > kMaxSide || imgs[e].h > kMaxSide) throw Failure{TS_ERR_LIMIT, "example side exceeds limit"};
      if (s->guided) {
        guides[e] = load_image(ex.guide, has_in, in_w, in_h, st);
        if (guides[e].w > kMaxSide || guides[e].h > kMaxSide) throw Failure{TS_ERR_LIMIT, "guide side exceeds limit"};
      }
      if (ex.method == TS_SAMPLE_IMAGE) {
        masks[e] = load_image(ex.mask, has_in, in_w, in_h, st);
        if (masks[e].w != imgs[e].w || masks[e].h != imgs[e].h)
          throw Failure{TS_ERR_SIZE_MISMATCH, "sample mask size differs from its example"};
      }
    }
    // inpaint mask and colour map (session.rs:346-382, ms.rs:236-293)
    if (b->has_inpaint) {
      s->inpaint = true;
      s->inpaint_index = b->inpaint.example_index;
      Image mask;
      if (b->inpaint.channel) {
        mask = load_image(b->examples[s->inpaint_index].img, true, W, H, st);
        const int c = b->inpaint.ch;
        for (size_t i = 0; i < (size_t)W * H; ++i) {
          uint8_t v = mask.px[4 * i + c];
          mask.px[4 * i] = v;
          mask.px[4 * i + 1] = v;
          mask.px[4 * i + 2] = v;
          mask.px[4 * i + 3] = 255;
        }
      } else {
        mask = load_image(b->inpaint.mask, true, W, H, st);
      }
      s->inpaint_mask.resize((size_t)W * H);
      for (size_t i = 0; i < (size_t)W * H; ++i) s->inpaint_mask[i] = mask.px[4 * i] < 255 ? 1 : 0;
      s->inpaint_colors = imgs[s->inpaint_index];
    }
    // filtered maps and their device pyramids
    uint64_t texels = 0, ptexels = 0, mask_bytes = 0;
    for (uint32_t e = 0; e < s->n_ex; ++e) {
      if (b->examples[e].method == TS_SAMPLE_IGNORE) continue;
      MapDesc md;
      md.w = imgs[e].w;
      md.h = imgs[e].h;
      md.off = texels;
      md.mask_off = -1;
      md.pw = md.w + 2 * kPad;
      md.ph = md.h + 2 * kPad;
      md.poff = ptexels;
      texels += (uint64_t)md.w * md.h * s->n_levels;
      ptexels += (uint64_t)md.pw * md.ph * s->n_levels;
      if (b->examples[e].method == TS_SAMPLE_IMAGE) {
        bool any = false;
        for (size_t i = 0; i < (size_t)md.w * md.h && !any; ++i) any = masks[e].px[4 * i] != 0;
        if (!any) throw Failure{TS_ERR_NO_VALID_SAMPLE, "a sample mask has no texel to sample from"};
        md.mask_off = (int64_t)mask_bytes;
        mask_bytes += (uint64_t)md.w * md.h;
      }
      s->maps.push_back(md);
      s->filtered.push_back(e);
    }
    s->n_maps = (uint32_t)s->maps.size();
    CUDA_TRY(s->levels.alloc(texels));
    CUDA_TRY(s->masks.alloc(mask_bytes));
    for (uint32_t f = 0; f < s->n_maps; ++f) {
      const uint32_t e = s->filtered[f];
      device_pyramid(imgs[e], p.backtrack_stages, s->levels.p + s->maps[f].off, st);
      if (s->maps[f].mask_off >= 0) {
        std::vector<uint8_t> mb((size_t)s->maps[f].w * s->maps[f].h);
        for (size_t i = 0; i < mb.size(); ++i) mb[i] = masks[e].px[4 * i] != 0 ? 1 : 0;
        CUDA_TRY(cudaMemcpy(s->masks.p + s->maps[f].mask_off, mb.data(), mb.size(), cudaMemcpyHostToDevice));
      }
    }
    CUDA_TRY(s->plevels.alloc(ptexels));
    for (uint32_t f = 0; f < s->n_maps; ++f)
      launch_pad(s->levels.p + s->maps[f].off, s->maps[f].w, s->maps[f].h, s->n_levels,
                 s->plevels.p + s->maps[f].poff, st);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(s->d_maps.alloc(s->n_maps));
    CUDA_TRY(cudaMemcpy(s->d_maps.p, s->maps.data(), s->n_maps * sizeof(MapDesc), cudaMemcpyHostToDevice));
    // guides: every example (unfiltered order) plus the target guide
    std::vector<GuideDesc> gd(std::max<uint32_t>(s->n_ex, 1));
    if (s->guided) {
      uint64_t gtex = 0, pgtex = 0;
      for (uint32_t e = 0; e < s->n_ex; ++e) {
        gd[e].w = guides[e].w;
        gd[e].h = guides[e].h;
        gd[e].off = gtex;
        gd[e].pw = gd[e].w + 2 * kPad;
        gd[e].ph = gd[e].h + 2 * kPad;
        gd[e].poff = pgtex;
        gtex += (uint64_t)guides[e].w * guides[e].h * s->n_levels;
        pgtex += (uint64_t)gd[e].pw * gd[e].ph * s->n_levels;
      }
      // the guide of map f is example f's guide (unfiltered index); the
      // padded fast path needs its size to equal the map's
      for (uint32_t f = 0; f < s->n_maps; ++f)
        if (f >= s->n_ex || gd[f].w != s->maps[f].w || gd[f].h != s->maps[f].h) s->guide_dims_differ = true;
      CUDA_TRY(s->guides.alloc(gtex));
      CUDA_TRY(s->pguides.alloc(pgtex));
      for (uint32_t e = 0; e < s->n_ex; ++e) {
        device_pyramid(guides[e], p.backtrack_stages, s->guides.p + gd[e].off, st);
        launch_pad(s->guides.p + gd[e].off, gd[e].w, gd[e].h, s->n_levels, s->pguides.p + gd[e].poff, st);
      }
      CUDA_TRY(cudaGetLastError());
      Image tg = load_image(b->target, true, W, H, st);
      CUDA_TRY(s->tguide.alloc((size_t)W * H * s->n_levels));
      device_pyramid(tg, p.backtrack_stages, s->tguide.p, st);
    }
    CUDA_TRY(s->d_gdesc.alloc(gd.size()));
    CUDA_TRY(cudaMemcpy(s->d_gdesc.p, gd.data(), gd.size() * sizeof(GuideDesc), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaDeviceSynchronize());
    s->bottoms = std::move(imgs);
  } catch (const Failure &f) {
    b->err = f.msg;
    return f.status;
  }
  *out = s.release();
  return TS_OK;
}

// ---------------------------------------------------------------------------
// run
// ---------------------------------------------------------------------------
namespace {

struct BatchPlan {
  uint32_t i0, i1, n_res, append_from;
  bool exhaustive;
};

struct StagePlan {
  int32_t p_stage;
  uint32_t level;
  bool level_switch;
  uint32_t n_res_start;
  uint64_t seed;
  uint32_t items_off, n_items, redo;
  bool slow_lut;
  std::vector<BatchPlan> batches;
};

std::vector<int32_t> knn_table(int radius) {
  struct E {
    int d2, dy, dx;
  };
  std::vector<E> v;
  for (int dy = -radius; dy <= radius; ++dy)
    for (int dx = -radius; dx <= radius; ++dx) {
      const int d2 = dx * dx + dy * dy;
      if (d2 <= radius * radius) v.push_back({d2, dy, dx});
    }
  std::sort(v.begin(), v.end(), [](const E &a, const E &b) {
    if (a.d2 != b.d2) return a.d2 < b.d2;
    if (a.dy != b.dy) return a.dy < b.dy;
    return a.dx < b.dx;
  });
  std::vector<int32_t> out(v.size());
  for (size_t i = 0; i < v.size(); ++i)
    out[i] = (int32_t)((uint32_t)(v[i].dx & 0xffff) | ((uint32_t)v[i].dy << 16));
  return out;
}

}  // namespace

namespace {

// Per-launch CUDA event pairs, recorded only when profiling is on.
struct LaunchTimer {
  struct Rec {
    int kind, stage;
    uint32_t items;
    cudaEvent_t a, b;
  };
  bool on = false;
  cudaStream_t st = 0;
  int stage = -1;
  uint32_t items = 0;
  std::vector<Rec> ev;
  ~LaunchTimer() {
    for (auto &e : ev) {
      cudaEventDestroy(e.a);
      cudaEventDestroy(e.b);
    }
  }
  template <typename F>
  void run(int kind, F &&f) {
    if (!on) {
      f();
      return;
    }
    Rec r{kind, stage, items, nullptr, nullptr};
    CUDA_TRY(cudaEventCreate(&r.a));
    CUDA_TRY(cudaEventCreate(&r.b));
    CUDA_TRY(cudaEventRecord(r.a, st));
    f();
    CUDA_TRY(cudaEventRecord(r.b, st));
    ev.push_back(r);
  }
  void collect(ts_run_stats &out, std::vector<ts_launch_record> &recs) {
    for (auto &e : ev) {
      float ms = 0.0f;
      CUDA_TRY(cudaEventElapsedTime(&ms, e.a, e.b));
      out.kernel_count[e.kind] += 1;
      out.kernel_ms[e.kind] += ms;
      recs.push_back(ts_launch_record{e.kind, e.stage, e.items, ms});
    }
  }
};

}  // namespace

extern "C" int ts_session_run(ts_session *s, ts_progress_fn progress, void *user, ts_generated **out) {
  if (!s || !out) return TS_ERR_NULL;
  *out = nullptr;
  if (s->consumed) {
    s->err = "session already consumed";
    return TS_ERR_STATE;
  }
  s->consumed = true;
  const auto t_wall0 = std::chrono::steady_clock::now();
  const Params &p = s->prm;
  const uint32_t W = s->W, H = s->H;
  const size_t N = (size_t)W * H;
  const uint32_t k = p.k, m = (uint32_t)p.m;
  const uint32_t stages = p.backtrack_stages;
  std::unique_ptr<ts_generated> g(new (std::nothrow) ts_generated());
  if (!g) return TS_ERR_OUT_OF_MEMORY;
  try {
    CUDA_TRY(cudaSetDevice(p.device));
    cudaStream_t st;
    CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    struct StreamGuard {
      cudaStream_t s;
      ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{st};
    // ---- initial state (Generator::new / new_from_inpaint) ----
    std::vector<uint32_t> color(N, 0);
    std::vector<uint4> state(N, make_uint4(0, 0, 0, 0));
    std::vector<uint32_t> resolved;
    std::vector<float> rscore;
    std::vector<uint32_t> unresolved;
    std::vector<uint8_t> mirf;  // per resolved entry: insert with mirrors
    size_t locked = 0;
    if (s->inpaint) {
      for (size_t i = 0; i < N; ++i) {
        const uint8_t *c = &s->inpaint_colors.px[4 * i];
        color[i] = (uint32_t)c[0] | ((uint32_t)c[1] << 8) | ((uint32_t)c[2] << 16) | ((uint32_t)c[3] << 24);
        if (s->inpaint_mask[i]) {
          unresolved.push_back((uint32_t)i);
        } else {
          resolved.push_back((uint32_t)i);
          rscore.push_back(0.0f);
          state[i] = make_uint4((uint32_t)(i % W) | ((uint32_t)(i / W) << 16), 0, 0, s->inpaint_index);
        }
      }
      locked = resolved.size();
    } else {
      unresolved.resize(N);
      for (size_t i = 0; i < N; ++i) unresolved[i] = (uint32_t)i;
    }
    auto pick = [&](uint64_t seed) -> uint32_t {
      Pcg32 r = pcg_from_u64(seed);
      const uint64_t idx = gen_range_u64(r, unresolved.size());
      const uint32_t v = unresolved[idx];
      unresolved[idx] = unresolved.back();
      unresolved.pop_back();
      return v;
    };
    // ---- random init (session.rs:42-52, ms.rs:427-475): all examples ----
    if (p.has_random_init) {
      if (p.random_init > unresolved.size())
        throw Failure{TS_ERR_INVALID_RANGE, "random_init exceeds the number of pixels to synthesise"};
      for (uint64_t i = 0; i < p.random_init; ++i) {
        const uint32_t px = pick(p.seed + i);
        const uint64_t sd = p.seed + i + (uint64_t)px;
        Pcg32 r = pcg_from_u64(sd);
        const uint32_t map = (uint32_t)gen_range_u64(r, s->n_ex);
        const Image &im = s->bottoms[map];
        r = pcg_from_u64(sd);
        const uint32_t x = gen_range_u32(r, im.w);
        r = pcg_from_u64(sd);
        const uint32_t y = gen_range_u32(r, im.h);
        if (x > 0xffffu || y > 0xffffu) throw Failure{TS_ERR_LIMIT, "example side exceeds limit"};
        state[px] = make_uint4(x | (y << 16), px, map, map);
        const uint8_t *c = &im.px[((size_t)y * im.w + x) * 4];
        color[px] = (uint32_t)c[0] | ((uint32_t)c[1] << 8) | ((uint32_t)c[2] << 16) | ((uint32_t)c[3] << 24);
        resolved.push_back(px);
        rscore.push_back(0.0f);
      }
      locked += p.random_init;
    }
    const size_t total = unresolved.size();
    // ---- the schedule of Generator::resolve ----
    const int32_t x_l = (int32_t)((float)W * kTilingBoundary), y_b = (int32_t)((float)H * kTilingBoundary);
    const float sig2 = p.cauchy * p.cauchy;
    float cauchy[256], l2[256];
    for (int d = 0; d < 256; ++d) {
      const float x = ((float)d - 0.0f) / 255.0f;
      const float x2 = x * x;
      cauchy[d] = log1pf(x2 / sig2);
      l2[d] = x2;
    }
    std::vector<StagePlan> plan;
    std::vector<uint32_t> items;
    std::vector<float> luts;
    size_t n_res = resolved.size();
    int32_t pyramid_level = 0;
    uint32_t max_batch_items = 1, max_stage_items = 1;
    const std::vector<int32_t> tab = knn_table(kKnnTabRadius);
    for (int32_t ps = (int32_t)stages; ps >= 0; --ps) {
      StagePlan sp;
      sp.p_stage = ps;
      sp.level = (uint32_t)pyramid_level;
      sp.level_switch = pyramid_level > 0;
      pyramid_level += 1;
      if (pyramid_level > (int32_t)stages - 1) pyramid_level = (int32_t)stages - 1;
      sp.seed = pcg_stage_seed(p.seed + (uint64_t)ps);
      const float fp = powf(p.backtrack_percent, (float)ps) * (float)total;
      size_t P = fp >= 0.0f ? (size_t)fp : 0;  // `as usize` saturates NaN and negatives to 0
      const size_t redo = n_res - locked;
      float adaptive = 0.0f;
      if (s->guided && ps > 0) {
        const float a = p.alpha * (1.0f - ((float)n_res / (float)total));
        adaptive = (a * a) * a;
      }
      // stage LUTs (ms.rs:853-858): content = (1 - a) * cauchy when guided
      bool slow = false;
      for (int d = 0; d < 256; ++d) {
        const float c = s->guided ? (1.0f - adaptive) * cauchy[d] : cauchy[d];
        luts.push_back(c);
        slow |= !std::isfinite(c);
      }
      for (int d = 0; d < 256; ++d) {
        const float gv = s->guided ? adaptive * l2[d] : 0.0f;
        luts.push_back(gv);
        slow |= !std::isfinite(gv);
      }
      sp.slow_lut = slow;
      const size_t P_eff = std::min(P, redo + unresolved.size());
      sp.items_off = (uint32_t)items.size();
      sp.n_items = (uint32_t)P_eff;
      sp.redo = (uint32_t)redo;
      sp.n_res_start = (uint32_t)n_res;
      for (size_t i = 0; i < P_eff; ++i) {
        if (i < redo)
          items.push_back(resolved[i + locked]);
        else
          items.push_back(pick(sp.seed + (uint64_t)i));
      }
      size_t i = 0, R = n_res;
      while (i < P_eff) {
        size_t bsz = 1;
        if (p.batch_divisor) {
          bsz = R / p.batch_divisor;
          if (bsz < 1) bsz = 1;
          if (p.max_batch && bsz > p.max_batch) bsz = p.max_batch;
        }
        if (bsz > P_eff - i) bsz = P_eff - i;
        BatchPlan bp;
        bp.i0 = (uint32_t)i;
        bp.i1 = (uint32_t)(i + bsz);
        bp.n_res = (uint32_t)R;
        bp.append_from = k == 0 ? bp.i0 : std::max<uint32_t>(bp.i0, (uint32_t)std::min(redo, (size_t)bp.i1));
        // exhaustive k-NN when the table walk is unlikely to find k points
        bp.exhaustive = k > 0 && (R <= 4096 && (double)R * tab.size() < 2.0 * k * (double)N);
        const size_t appended = bp.i1 - bp.append_from;
        for (size_t t = bp.append_from; t < bp.i1; ++t) {
          resolved.push_back(items[sp.items_off + t]);
          rscore.push_back(0.0f);
        }
        R += appended;
        sp.batches.push_back(bp);
        max_batch_items = std::max<uint32_t>(max_batch_items, (uint32_t)bsz);
        i += bsz;
      }
      n_res = R;
      max_stage_items = std::max<uint32_t>(max_stage_items, (uint32_t)P_eff);
      plan.push_back(std::move(sp));
    }
    // ---- device state and schedule ----
    DevBuf<uint32_t> d_color, d_occ, d_mir, d_res, d_items, d_ncnt, d_fbl, d_fbc;
    DevBuf<uint4> d_state;
    DevBuf<float> d_rscore, d_lut;
    DevBuf<double> d_xdiv, d_ydiv, d_dist, d_dxt, d_dy2t, d_mean;
    DevBuf<int32_t> d_tab, d_nbuf;
    DevBuf<uint2> d_rcand;
    DevBuf<Result> d_result;
    DevBuf<int> d_err;
    DevBuf<unsigned long long> d_evals;
    const uint32_t wpr = (W + 31) / 32;
    size_t n_batches = 0;
    for (auto &sp : plan) n_batches += sp.batches.size();
    CUDA_TRY(d_color.alloc(N));
    CUDA_TRY(d_state.alloc(N));
    CUDA_TRY(d_occ.alloc((size_t)wpr * H));
    CUDA_TRY(d_mir.alloc((size_t)wpr * H));
    CUDA_TRY(d_res.alloc(resolved.size()));
    CUDA_TRY(d_rscore.alloc(resolved.size()));
    CUDA_TRY(d_items.alloc(items.size()));
    CUDA_TRY(d_lut.alloc(luts.size()));
    CUDA_TRY(d_tab.alloc(tab.size()));
    CUDA_TRY(d_nbuf.alloc((size_t)max_batch_items * std::max<uint32_t>(k, 1)));
    CUDA_TRY(d_ncnt.alloc(max_batch_items));
    CUDA_TRY(d_dist.alloc((size_t)max_batch_items * std::max<uint32_t>(k, 1)));
    CUDA_TRY(d_mean.alloc(max_batch_items));
    CUDA_TRY(d_fbl.alloc(max_batch_items));
    CUDA_TRY(d_fbc.alloc(n_batches));
    CUDA_TRY(d_result.alloc(max_batch_items));
    CUDA_TRY(d_err.alloc(1));
    CUDA_TRY(d_evals.alloc(1));
    const uint64_t rc_items = std::max<uint64_t>(1, std::min<uint64_t>(max_stage_items, kRcandBudget / std::max(m, 1u)));
    CUDA_TRY(d_rcand.alloc((size_t)std::max<uint64_t>(rc_items, max_batch_items) * m));
    const int32_t xo = x_l + 2, yo = y_b + 2;
    std::vector<double> xdiv(W + 2 * (size_t)xo + 1), ydiv(H + 2 * (size_t)yo + 1);
    for (size_t i = 0; i < xdiv.size(); ++i) xdiv[i] = (double)((int64_t)i - xo) / (double)W;
    for (size_t i = 0; i < ydiv.size(); ++i) ydiv[i] = (double)((int64_t)i - yo) / (double)H;
    CUDA_TRY(d_xdiv.alloc(xdiv.size()));
    CUDA_TRY(d_ydiv.alloc(ydiv.size()));
    // per-pixel tables of the normalised offsets the weights use: dx and
    // dy * dy for |offset| <= kDistTabRadius, the same IEEE operations as
    // get_distances_to_k_neighs (ms.rs:410-415)
    const int32_t R = kDistTabRadius;
    std::vector<double> dxt((size_t)W * (2 * R + 1)), dy2t((size_t)H * (2 * R + 1));
    for (uint32_t x = 0; x < W; ++x)
      for (int32_t o = -R; o <= R; ++o)
        dxt[(size_t)x * (2 * R + 1) + o + R] = (double)((int64_t)x + o) / (double)W - (double)x / (double)W;
    for (uint32_t y = 0; y < H; ++y)
      for (int32_t o = -R; o <= R; ++o) {
        const double dy = (double)((int64_t)y + o) / (double)H - (double)y / (double)H;
        dy2t[(size_t)y * (2 * R + 1) + o + R] = dy * dy;
      }
    CUDA_TRY(d_dxt.alloc(dxt.size()));
    CUDA_TRY(d_dy2t.alloc(dy2t.size()));
    // the tree is rebuilt from the resolved list, mirrors included (ms.rs:747-779)
    std::vector<uint32_t> occ((size_t)wpr * H, 0), mir((size_t)wpr * H, 0);
    for (size_t i = 0; i < locked; ++i) {
      const uint32_t q = resolved[i];
      occ[(size_t)(q / W) * wpr + (q % W) / 32] |= 1u << ((q % W) & 31);
      if (p.tiling) mir[(size_t)(q / W) * wpr + (q % W) / 32] |= 1u << ((q % W) & 31);
    }
    cudaEvent_t ev0, ev1;
    CUDA_TRY(cudaEventCreate(&ev0));
    CUDA_TRY(cudaEventCreate(&ev1));
    struct EvGuard {
      cudaEvent_t a, b;
      ~EvGuard() {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
      }
    } eg{ev0, ev1};
    CUDA_TRY(cudaEventRecord(ev0, st));
    CUDA_TRY(cudaMemcpyAsync(d_color.p, color.data(), N * 4, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_state.p, state.data(), N * sizeof(uint4), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_occ.p, occ.data(), occ.size() * 4, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_mir.p, mir.data(), mir.size() * 4, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_res.p, resolved.data(), locked * 4, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemsetAsync(d_rscore.p, 0, resolved.size() * 4, st));
    if (!items.empty())
      CUDA_TRY(cudaMemcpyAsync(d_items.p, items.data(), items.size() * 4, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_lut.p, luts.data(), luts.size() * 4, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_tab.p, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_xdiv.p, xdiv.data(), xdiv.size() * 8, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_ydiv.p, ydiv.data(), ydiv.size() * 8, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_dxt.p, dxt.data(), dxt.size() * 8, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_dy2t.p, dy2t.data(), dy2t.size() * 8, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemsetAsync(d_fbc.p, 0, n_batches * 4, st));
    CUDA_TRY(cudaMemsetAsync(d_err.p, 0, sizeof(int), st));
    CUDA_TRY(cudaMemsetAsync(d_evals.p, 0, sizeof(unsigned long long), st));

    SessionDev sd{};
    sd.levels = s->levels.p;
    sd.plevels = s->plevels.p;
    sd.pguides = s->pguides.p;
    sd.guide_dims_differ = s->guide_dims_differ ? 1 : 0;
    sd.masks = s->masks.p;
    sd.maps = s->d_maps.p;
    sd.n_maps = s->n_maps;
    sd.n_levels = s->n_levels;
    sd.guides = s->guides.p;
    sd.gdesc = s->d_gdesc.p;
    sd.n_guides = s->guided ? s->n_ex : 0;
    sd.guided = s->guided ? 1 : 0;
    sd.tguide = s->tguide.p;
    sd.xdiv = d_xdiv.p;
    sd.ydiv = d_ydiv.p;
    sd.xdiv_off = xo;
    sd.ydiv_off = yo;
    sd.dxt = d_dxt.p;
    sd.dy2t = d_dy2t.p;
    sd.dtab_r = R;
    sd.color = d_color.p;
    sd.state = d_state.p;
    sd.occ = d_occ.p;
    sd.mir = d_mir.p;
    sd.resolved = d_res.p;
    sd.rscore = d_rscore.p;
    sd.knn_tab = d_tab.p;
    sd.knn_tab_n = (uint32_t)tab.size();
    sd.err = d_err.p;
    sd.evals = d_evals.p;
    sd.W = W;
    sd.H = H;
    sd.wpr = wpr;
    sd.tiling = p.tiling ? 1 : 0;
    sd.x_l = x_l;
    sd.x_r = (int32_t)W - x_l;
    sd.y_b = y_b;
    sd.y_t = (int32_t)H - y_b;
    sd.k = k;
    sd.m = m;
    uint64_t launches = 0, batches = 0, resolves = 0;
    LaunchTimer lt;
    lt.on = p.profile;
    lt.st = st;
    size_t fb_index = 0;
    uint64_t overall_total = 0, overall_current = 0;
    for (auto &sp : plan) overall_total += sp.n_items;
    std::vector<uint8_t> prog_img;
    for (size_t si = 0; si < plan.size(); ++si) {
      const StagePlan &sp = plan[si];
      lt.stage = sp.p_stage;
      lt.items = sp.n_items;
      if (sp.level_switch) {
        lt.run(TS_KERNEL_LEVEL_SWITCH, [&] { launch_level_switch(sd, sp.level, sp.n_res_start, st); });
        ++launches;
      }
      StageDev sdv{};
      sdv.level = sp.level;
      sdv.slow_lut = sp.slow_lut ? 1 : 0;
      sdv.lut = d_lut.p + si * 512;
      sdv.stage_seed = sp.seed;
      sdv.items = d_items.p + sp.items_off;
      sdv.redo = sp.redo;
      // random candidates in chunks of whole batches that fit the buffer
      size_t bi = 0;
      while (bi < sp.batches.size()) {
        size_t bj = bi;
        const uint32_t c0 = sp.batches[bi].i0;
        while (bj < sp.batches.size() && (bj == bi || sp.batches[bj].i1 - c0 <= rc_items)) ++bj;
        const uint32_t c1 = sp.batches[bj - 1].i1;
        StageDev chunk = sdv;
        chunk.items = sdv.items + c0;
        chunk.n_items = c1 - c0;
        chunk.stage_seed = sp.seed + c0;  // item i's stream is seeded with stage_seed + i + 1
        chunk.rcand = d_rcand.p;
        chunk.redo = sp.redo > c0 ? sp.redo - c0 : 0;
        lt.run(TS_KERNEL_RANDOM_CANDIDATES, [&] { launch_random_candidates(sd, chunk, st); });
        ++launches;
        chunk.stage_seed = sp.seed;  // resolve_at_random uses the stage seed itself
        for (size_t bk = bi; bk < bj; ++bk) {
          const BatchPlan &bp = sp.batches[bk];
          lt.items = bp.i1 - bp.i0;
          BatchDev bd{};
          bd.i0 = bp.i0 - c0;
          bd.i1 = bp.i1 - c0;
          bd.n_res = bp.n_res;
          bd.append_from = bp.append_from - c0;
          bd.nbuf = d_nbuf.p;
          bd.ncnt = d_ncnt.p;
          bd.fb_list = d_fbl.p;
          bd.fb_count = d_fbc.p + fb_index++;
          bd.dist = d_dist.p;
          bd.mean = d_mean.p;
          bd.res = d_result.p;
          if (k > 0) {
            if (bp.exhaustive) {
              lt.run(TS_KERNEL_KNN_EXHAUSTIVE, [&] { launch_knn_exhaustive(sd, chunk, bd, true, st); });
              ++launches;
            } else {
              lt.run(TS_KERNEL_KNN_WALK, [&] { launch_knn_walk(sd, chunk, bd, st); });
              lt.run(TS_KERNEL_KNN_EXHAUSTIVE, [&] { launch_knn_exhaustive(sd, chunk, bd, false, st); });
              launches += 2;
            }
          }
          if (k > 0 && !bp.exhaustive) {  // the exhaustive k-NN over a whole batch computes the mean itself
            lt.run(TS_KERNEL_MEAN, [&] { launch_mean(sd, chunk, bd, st); });
            ++launches;
          }
          if (bp.i1 - bp.i0 <= p.team_max_batch)
            lt.run(TS_KERNEL_RESOLVE,
                   [&] { launch_resolve_team(sd, chunk, bd, bp.i1 - bp.i0 <= p.team_full_max_batch, st); });
          else
            lt.run(TS_KERNEL_RESOLVE, [&] { launch_resolve(sd, chunk, bd, st); });
          lt.run(TS_KERNEL_COMMIT, [&] { launch_commit(sd, chunk, bd, st); });
          launches += 2;
          ++batches;
          resolves += bp.i1 - bp.i0;
        }
        bi = bj;
      }
      CUDA_TRY(cudaGetLastError());
      overall_current += sp.n_items;
      if (progress) {
        prog_img.resize(N * 4);
        CUDA_TRY(cudaMemcpyAsync(prog_img.data(), d_color.p, N * 4, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        ts_progress up;
        up.image = prog_img.data();
        up.width = W;
        up.height = H;
        up.total_current = overall_current;
        up.total_total = overall_total;
        up.stage_current = sp.n_items;
        up.stage_total = sp.n_items;
        progress(&up, user);
      }
    }
    // ---- results ----
    g->W = W;
    g->H = H;
    std::vector<uint32_t> col(N);
    std::vector<uint4> stv(N);
    g->resolved.resize(resolved.size());
    g->scores.resize(resolved.size());
    int derr = 0;
    unsigned long long evals = 0;
    CUDA_TRY(cudaMemcpyAsync(&evals, d_evals.p, sizeof(evals), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(col.data(), d_color.p, N * 4, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(stv.data(), d_state.p, N * sizeof(uint4), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(g->resolved.data(), d_res.p, resolved.size() * 4, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(g->scores.data(), d_rscore.p, resolved.size() * 4, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(&derr, d_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaEventRecord(ev1, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (derr == kDevErrIndex) throw Failure{TS_ERR_INDEX, "a map id points past the non-ignored examples"};
    if (derr == kDevErrNoSample) throw Failure{TS_ERR_NO_VALID_SAMPLE, "no valid sample location found"};
    if (derr == kDevErrLimit) throw Failure{TS_ERR_LIMIT, "too many equidistant neighbours for the k-NN buffer"};
    if (derr) throw Failure{TS_ERR_CUDA, "device reported error " + std::to_string(derr)};
    float ms = 0.0f;
    CUDA_TRY(cudaEventElapsedTime(&ms, ev0, ev1));
    g->image.resize(N * 4);
    memcpy(g->image.data(), col.data(), N * 4);
    g->coord.resize(N * 3);
    g->ids.resize(N * 2);
    for (size_t i = 0; i < N; ++i) {
      g->coord[3 * i] = stv[i].x & 0xffffu;
      g->coord[3 * i + 1] = stv[i].x >> 16;
      g->coord[3 * i + 2] = stv[i].w;
      g->ids[2 * i] = stv[i].y;
      g->ids[2 * i + 1] = stv[i].z;
    }
    g->stats.resolves = resolves;
    g->stats.batches = batches;
    g->stats.stages = plan.size();
    g->stats.kernel_launches = launches;
    g->stats.gpu_ms = ms;
    lt.collect(g->stats, g->launches);
    g->stats.cost_evals = evals;
  } catch (const Failure &f) {
    s->err = f.msg;
    return f.status;
  }
  g->stats.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_wall0).count();
  *out = g.release();
  return TS_OK;
}

extern "C" {

void ts_session_free(ts_session *s) { delete s; }
const char *ts_session_last_error(const ts_session *s) { return s ? s->err.c_str() : "null session"; }

void ts_generated_dims(const ts_generated *g, uint32_t *w, uint32_t *h) {
  if (!g) return;
  if (w) *w = g->W;
  if (h) *h = g->H;
}
int ts_generated_image(const ts_generated *g, uint8_t *out) {
  if (!g || !out) return TS_ERR_NULL;
  memcpy(out, g->image.data(), g->image.size());
  return TS_OK;
}
int ts_generated_coord_map(const ts_generated *g, uint32_t *out) {
  if (!g || !out) return TS_ERR_NULL;
  memcpy(out, g->coord.data(), g->coord.size() * 4);
  return TS_OK;
}
int ts_generated_id_map(const ts_generated *g, uint32_t *out) {
  if (!g || !out) return TS_ERR_NULL;
  memcpy(out, g->ids.data(), g->ids.size() * 4);
  return TS_OK;
}
uint64_t ts_generated_resolved_count(const ts_generated *g) { return g ? g->resolved.size() : 0; }
int ts_generated_resolved(const ts_generated *g, uint32_t *flat, float *score) {
  if (!g) return TS_ERR_NULL;
  if (flat) memcpy(flat, g->resolved.data(), g->resolved.size() * 4);
  if (score) memcpy(score, g->scores.data(), g->scores.size() * 4);
  return TS_OK;
}
void ts_generated_stats(const ts_generated *g, ts_run_stats *out) {
  if (g && out) *out = g->stats;
}
uint64_t ts_generated_launch_count(const ts_generated *g) { return g ? g->launches.size() : 0; }
int ts_generated_launches(const ts_generated *g, ts_launch_record *out) {
  if (!g || !out) return TS_ERR_NULL;
  if (!g->launches.empty()) memcpy(out, g->launches.data(), g->launches.size() * sizeof(ts_launch_record));
  return TS_OK;
}
void ts_generated_free(ts_generated *g) { delete g; }

}  // extern "C"
