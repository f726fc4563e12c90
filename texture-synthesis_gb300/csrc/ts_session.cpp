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
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <unordered_map>
#include <string>
#include <thread>
#include <vector>

#include <cuda.h>  // green-context types (entry points through cudaGetDriverEntryPointByVersion)
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
constexpr int kDistTabRadius = 64;  // offsets the weight tables cover
static_assert(kDistTabRadius >= kKnnTabRadius, "the walk's distances come from the tables alone");
constexpr uint64_t kRcandBudget = 64ull << 20;  // random-candidate entries held at once
// Walk steps of at most this many items are latency-bound: their sparse items
// build a bitmap window instead of more rounds of bitmap loads (the default;
// ts_builder_tuning sets it per session).
constexpr uint32_t kWalkWindowItems = 4096;
// Runs whose random candidates for every stage fit this many entries make
// them all ahead, on a side stream, while the first stages run.
constexpr uint64_t kRcandWhole = 256ull << 20;

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
  uint32_t team_max_batch = 2048;
  uint32_t team_full_max_batch = 256;
  uint32_t walk_window_max = kWalkWindowItems;
};

std::string fmt_float(float v) {
  char buf[64];
  snprintf(buf, sizeof(buf), "%g", (double)v);
  return buf;
}

// A device array.  alloc() uses cudaMalloc (freed with cudaFree, which
// waits for the device); alloc_on(stream) takes stream-ordered pool memory,
// freed with cudaFreeAsync on the stream set by free_on (at first the
// allocating one), so that freeing never stalls the device.  view() makes
// it a non-owning window into another array.
template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  bool pooled = false;
  bool owned = true;
  cudaStream_t fs = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n), pooled(o.pooled), owned(o.owned), fs(o.fs) {
    o.p = nullptr;
    o.n = 0;
  }
  DevBuf &operator=(DevBuf &&o) noexcept {
    if (this != &o) {
      reset();
      p = o.p;
      n = o.n;
      pooled = o.pooled;
      owned = o.owned;
      fs = o.fs;
      o.p = nullptr;
      o.n = 0;
    }
    return *this;
  }
  ~DevBuf() { reset(); }
  void reset() {
    if (p && owned) {
      if (pooled)
        cudaFreeAsync(p, fs);
      else
        cudaFree(p);
    }
    p = nullptr;
    n = 0;
    pooled = false;
    owned = true;
  }
  void view(void *base, size_t count) {
    reset();
    p = (T *)base;
    n = count;
    owned = false;
  }
  cudaError_t alloc(size_t count) {
    reset();
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)&p, count * sizeof(T));
    if (e == cudaSuccess)
      n = count;
    else
      p = nullptr;
    return e;
  }
  cudaError_t alloc_on(size_t count, cudaStream_t st) {
    reset();
    if (count == 0) count = 1;
    cudaError_t e = cudaMallocAsync((void **)&p, count * sizeof(T), st);
    if (e == cudaSuccess) {
      n = count;
      pooled = true;
      fs = st;
    } else {
      p = nullptr;
    }
    return e;
  }
  // Stream-ordered pool memory that outlives the stream it was made on: it
  // is freed on the legacy stream, for buffers whose users have all
  // finished when they go (a session's pyramids and tables).
  cudaError_t alloc_kept(size_t count, cudaStream_t st) {
    const cudaError_t e = alloc_on(count, st);
    fs = nullptr;
    return e;
  }
  void free_on(cudaStream_t st) { fs = st; }
  size_t bytes() const { return p ? n * sizeof(T) : 0; }
};

// Process-wide cache of page-locked host blocks: cudaMallocHost costs about
// as much host time as the copies it speeds up, so blocks are kept and
// reused (at most kKeep bytes idle; sizes rounded up to 2 MiB).  Never
// destroyed: the CUDA context may be gone at process exit.
class PinnedPool {
 public:
  static PinnedPool &get() {
    static PinnedPool *pool = new PinnedPool();
    return *pool;
  }
  cudaError_t take(size_t bytes, void **p, size_t *got) {
    bytes = (std::max<size_t>(bytes, 1) + kRound - 1) / kRound * kRound;
    {
      std::lock_guard<std::mutex> lk(mu_);
      size_t best = idle_.size();
      for (size_t i = 0; i < idle_.size(); ++i)
        if (idle_[i].second >= bytes && (best == idle_.size() || idle_[i].second < idle_[best].second)) best = i;
      if (best < idle_.size() && idle_[best].second <= 2 * bytes) {
        *p = idle_[best].first;
        *got = idle_[best].second;
        idle_bytes_ -= *got;
        idle_.erase(idle_.begin() + best);
        return cudaSuccess;
      }
    }
    *got = bytes;
    return cudaMallocHost(p, bytes);
  }
  void give(void *p, size_t bytes) {
    {
      std::lock_guard<std::mutex> lk(mu_);
      if (idle_bytes_ + bytes <= kKeep) {
        idle_.emplace_back(p, bytes);
        idle_bytes_ += bytes;
        return;
      }
    }
    cudaFreeHost(p);
  }

 private:
  static constexpr size_t kRound = 2u << 20;
  static constexpr size_t kKeep = 1ull << 30;
  std::mutex mu_;
  std::vector<std::pair<void *, size_t>> idle_;
  size_t idle_bytes_ = 0;
};

// Page-locked host memory from the pool, for copies that must not wait.
// The owner makes sure no copy from it is in flight when it goes.
template <typename T>
struct PinnedBuf {
  T *p = nullptr;
  size_t got = 0;
  PinnedBuf() = default;
  PinnedBuf(const PinnedBuf &) = delete;
  PinnedBuf &operator=(const PinnedBuf &) = delete;
  PinnedBuf(PinnedBuf &&o) noexcept : p(o.p), got(o.got) { o.p = nullptr; }
  PinnedBuf &operator=(PinnedBuf &&o) noexcept {
    if (this != &o) {
      reset();
      p = o.p;
      got = o.got;
      o.p = nullptr;
    }
    return *this;
  }
  ~PinnedBuf() { reset(); }
  void reset() {
    if (p) PinnedPool::get().give(p, got);
    p = nullptr;
  }
  cudaError_t alloc(size_t count) {
    reset();
    void *v = nullptr;
    const cudaError_t e = PinnedPool::get().take((count ? count : 1) * sizeof(T), &v, &got);
    p = e == cudaSuccess ? (T *)v : nullptr;
    return e;
  }
};

// An owned CUDA event (movable).
struct EventHandle {
  cudaEvent_t e = nullptr;
  EventHandle() = default;
  EventHandle(const EventHandle &) = delete;
  EventHandle &operator=(const EventHandle &) = delete;
  EventHandle(EventHandle &&o) noexcept : e(o.e) { o.e = nullptr; }
  EventHandle &operator=(EventHandle &&o) noexcept {
    if (this != &o) {
      if (e) cudaEventDestroy(e);
      e = o.e;
      o.e = nullptr;
    }
    return *this;
  }
  ~EventHandle() {
    if (e) cudaEventDestroy(e);
  }
};

struct StreamGuard {
  cudaStream_t s = nullptr;
  ~StreamGuard() {
    if (s) cudaStreamDestroy(s);
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

// Device copies of filter taps, kept per (device, filter, sigma, lengths)
// for the life of the process: the same resizes recur for every example of
// a size and every level of a pyramid.  kBlurFilter marks imageops::blur's
// Gaussian of standard deviation sigma.
constexpr int kBlurFilter = -1;

struct DevTapsRef {
  const uint4 *taps;
  const float *wts;
};

DevTapsRef cached_taps(int filter, float sigma, uint32_t in_len, uint32_t out_len) {
  static std::mutex mu;
  static std::unordered_map<std::string, DevTapsRef> cache;
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  uint32_t sb = 0;
  memcpy(&sb, &sigma, 4);
  const std::string key = std::to_string(dev) + "/" + std::to_string(filter) + "/" + std::to_string(sb) + "/" +
                          std::to_string(in_len) + "/" + std::to_string(out_len);
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  const Taps t = filter == kBlurFilter ? blur_taps(in_len, sigma) : axis_taps((Filter)filter, in_len, out_len);
  std::vector<uint4> v(t.left.size());
  for (size_t i = 0; i < v.size(); ++i) v[i] = make_uint4(t.left[i], t.count[i], t.offset[i], 0);
  uint4 *dt = nullptr;
  float *dw = nullptr;
  CUDA_TRY(cudaMalloc((void **)&dt, std::max<size_t>(1, v.size()) * sizeof(uint4)));
  CUDA_TRY(cudaMalloc((void **)&dw, std::max<size_t>(1, t.weights.size()) * sizeof(float)));
  if (!v.empty()) CUDA_TRY(cudaMemcpy(dt, v.data(), v.size() * sizeof(uint4), cudaMemcpyHostToDevice));
  if (!t.weights.empty())
    CUDA_TRY(cudaMemcpy(dw, t.weights.data(), t.weights.size() * sizeof(float), cudaMemcpyHostToDevice));
  if (cache.size() > 4096) cache.clear();  // bounded; the dropped device copies stay allocated
  return cache[key] = DevTapsRef{dt, dw};
}

void device_resample(const uint8_t *src, uint32_t w, uint32_t h, uint8_t *dst, uint32_t nw, uint32_t nh, int filter,
                     float sigma, cudaStream_t st) {
  if (nw == 0 || nh == 0) return;
  const DevTapsRef tv = cached_taps(filter, sigma, h, nh);
  const DevTapsRef th = cached_taps(filter, sigma, w, nw);
  DevBuf<float> tmp;
  CUDA_TRY(tmp.alloc_on((size_t)w * nh * 4, st));
  CUDA_TRY(cudaMemsetAsync(tmp.p, 0, (size_t)w * nh * 4 * sizeof(float), st));
  if (h > 0) launch_resize_v(src, w, h, tmp.p, nh, tv.taps, tv.wts, st);
  if (w > 0) {
    launch_resize_h(tmp.p, w, nh, dst, nw, th.taps, th.wts, st);
  } else {
    CUDA_TRY(cudaMemsetAsync(dst, 0, (size_t)nw * nh * 4, st));
  }
  CUDA_TRY(cudaGetLastError());
}

void device_resize(const uint8_t *src, uint32_t w, uint32_t h, uint8_t *dst, uint32_t nw, uint32_t nh, Filter f,
                   cudaStream_t st) {
  device_resample(src, w, h, dst, nw, nh, (int)f, 0.0f, st);
}

// transform_to_guide_map + match_histograms (utils.rs:101-183) on the device:
// imageops::blur with sigma 2 (the resize passes at the same size),
// grayscale, then the luma histogram matched to channel 0 of `target`.  The
// transform's own resize discards its result (utils.rs:110-114) and is left
// out.  The 256-entry map comes from the two histograms in the reference's
// f32 arithmetic: v -> (first index whose target cdf exceeds cdf_src[v],
// else v + 1 in u8) as u8 minus 1, wrapping as the reference's release
// build does.
Image device_guide_map(const Image &img, const Image &target, cudaStream_t st) {
  const size_t n = (size_t)img.w * img.h, nt = (size_t)target.w * target.h;
  DevBuf<uint8_t> d_src, d_blur, d_luma, d_map;
  DevBuf<uint32_t> d_tgt, d_hist, d_out;
  CUDA_TRY(d_src.alloc_on(n * 4, st));
  CUDA_TRY(d_blur.alloc_on(n * 4, st));
  CUDA_TRY(d_luma.alloc_on(n, st));
  CUDA_TRY(d_map.alloc_on(256, st));
  CUDA_TRY(d_tgt.alloc_on(nt, st));
  CUDA_TRY(d_hist.alloc_on(512, st));
  CUDA_TRY(d_out.alloc_on(n, st));
  CUDA_TRY(cudaMemcpyAsync(d_src.p, img.px.data(), n * 4, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(d_tgt.p, target.px.data(), nt * 4, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemsetAsync(d_hist.p, 0, 512 * 4, st));
  device_resample(d_src.p, img.w, img.h, d_blur.p, img.w, img.h, kBlurFilter, 2.0f, st);
  launch_luma_hist((const uint32_t *)d_blur.p, n, d_luma.p, d_hist.p, st);
  launch_hist_r(d_tgt.p, nt, d_hist.p + 256, st);
  uint32_t hist[512];
  CUDA_TRY(cudaMemcpyAsync(hist, d_hist.p, sizeof(hist), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  float cs[256], ct[256];
  cs[0] = (float)hist[0];
  ct[0] = (float)hist[256];
  for (int i = 1; i < 256; ++i) {
    cs[i] = cs[i - 1] + (float)hist[i];
    ct[i] = ct[i - 1] + (float)hist[256 + i];
  }
  const float ms = cs[255], mt = ct[255];
  for (int i = 0; i < 256; ++i) {
    cs[i] /= ms;
    ct[i] /= mt;
  }
  uint8_t map[256];
  for (int v = 0; v < 256; ++v) {
    int pos = -1;
    for (int i = 0; i < 256 && pos < 0; ++i)
      if (ct[i] > cs[v]) pos = i;
    const uint32_t idx = pos >= 0 ? (uint32_t)pos : (uint32_t)(uint8_t)(v + 1);
    map[v] = (uint8_t)((uint8_t)idx - 1u);
  }
  CUDA_TRY(cudaMemcpyAsync(d_map.p, map, 256, cudaMemcpyHostToDevice, st));
  launch_apply_map(d_luma.p, n, d_map.p, d_out.p, st);
  CUDA_TRY(cudaGetLastError());
  Image out;
  out.w = img.w;
  out.h = img.h;
  out.px.resize(n * 4);
  CUDA_TRY(cudaMemcpyAsync(out.px.data(), d_out.p, n * 4, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return out;
}

// load_image (utils.rs:55-80): resize with CatmullRom when a size is given
// and differs.  Runs on the device; returns the host image.  This form
// takes over an input nothing reads afterwards (a consumed builder's): an
// image already at its size is moved, not copied.
Image load_image(Image &&in, bool has_size, uint32_t w, uint32_t h, cudaStream_t st) {
  if (!has_size || (in.w == w && in.h == h)) return std::move(in);
  DevBuf<uint8_t> a, b;
  CUDA_TRY(a.alloc_on(in.px.size(), st));
  CUDA_TRY(b.alloc_on((size_t)w * h * 4, st));
  CUDA_TRY(cudaMemcpyAsync(a.p, in.px.data(), in.px.size(), cudaMemcpyHostToDevice, st));
  device_resize(a.p, in.w, in.h, b.p, w, h, kCatmullRom, st);
  Image out;
  out.w = w;
  out.h = h;
  out.px.resize((size_t)w * h * 4);
  CUDA_TRY(cudaMemcpyAsync(out.px.data(), b.p, out.px.size(), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return out;
}

// The same for an input that stays with its owner.
Image load_image(const Image &in, bool has_size, uint32_t w, uint32_t h, cudaStream_t st) {
  if (!has_size || (in.w == w && in.h == h)) return in;
  return load_image(Image(in), has_size, w, h, st);
}


inline uint32_t cdiv_u32(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

// ImagePyramid::new (img_pyramid.rs:7-37) for many images at once: every
// level of every image is a Gaussian resize of the original down by 2^i and
// back up, so all images' levels go through four launches (down vertical,
// down horizontal, up vertical, up horizontal) instead of four per level.
// The originals are copied from pageable host memory (staged before the
// call returns); the scratch is stream-ordered pool memory.
struct PyramidJob {
  const Image *img;
  uint32_t levels;
  uint32_t *dst;  // max(levels, 1) images of w*h texels
};

void device_pyramids(const std::vector<PyramidJob> &pj, cudaStream_t st) {
  std::vector<ResizeJob> down, up;
  size_t small_bytes = 0, tmp_floats = 0;
  struct Lvl {
    size_t job;
    uint32_t l, sw, sh;
    size_t small_off, tmp_down, tmp_up;
  };
  std::vector<Lvl> lv;
  for (size_t q = 0; q < pj.size(); ++q) {
    const Image &img = *pj[q].img;
    const uint32_t nl = pj[q].levels == 0 ? 1 : pj[q].levels;
    const size_t sz = (size_t)img.w * img.h;
    uint8_t *base = (uint8_t *)pj[q].dst;
    CUDA_TRY(cudaMemcpyAsync(base + (size_t)(nl - 1) * sz * 4, img.px.data(), sz * 4, cudaMemcpyHostToDevice, st));
    for (uint32_t l = 0; l + 1 < nl; ++l) {
      const uint32_t i = nl - 1 - l;
      const uint32_t sw = img.w >> std::min(i, 31u), sh = img.h >> std::min(i, 31u);
      if (sw == 0 || sh == 0) {
        // a zero-sized intermediate makes the crate return a zero image
        CUDA_TRY(cudaMemsetAsync(base + (size_t)l * sz * 4, 0, sz * 4, st));
        continue;
      }
      Lvl v{q, l, sw, sh, small_bytes, tmp_floats, 0};
      small_bytes += ((size_t)sw * sh * 4 + 255) & ~(size_t)255;
      tmp_floats += (size_t)img.w * sh * 4;
      v.tmp_up = tmp_floats;
      tmp_floats += (size_t)sw * img.h * 4;
      lv.push_back(v);
    }
  }
  if (lv.empty()) return;
  DevBuf<uint8_t> d_small;
  DevBuf<float> d_tmp;
  DevBuf<ResizeJob> d_jobs;
  CUDA_TRY(d_small.alloc_on(small_bytes, st));
  CUDA_TRY(d_tmp.alloc_on(tmp_floats, st));
  uint32_t bdv = 0, bdh = 0, buv = 0, buh = 0;
  for (const Lvl &v : lv) {
    const Image &img = *pj[v.job].img;
    const uint32_t nl = pj[v.job].levels == 0 ? 1 : pj[v.job].levels;
    const size_t sz = (size_t)img.w * img.h;
    uint8_t *base = (uint8_t *)pj[v.job].dst;
    uint8_t *small = d_small.p + v.small_off;
    ResizeJob d{};
    d.src = base + (size_t)(nl - 1) * sz * 4;
    d.dst = small;
    d.tmp = d_tmp.p + v.tmp_down;
    d.w = img.w;
    d.h = img.h;
    d.nw = v.sw;
    d.nh = v.sh;
    const DevTapsRef dv = cached_taps(kGaussian, 0.0f, img.h, v.sh), dh = cached_taps(kGaussian, 0.0f, img.w, v.sw);
    d.tv = dv.taps;
    d.wv = dv.wts;
    d.th = dh.taps;
    d.wh = dh.wts;
    d.block0_v = bdv;
    d.block0_h = bdh;
    bdv += cdiv_u32(img.w, 128) * v.sh;
    bdh += cdiv_u32(v.sw, 128) * v.sh;
    down.push_back(d);
    ResizeJob u{};
    u.src = small;
    u.dst = base + (size_t)v.l * sz * 4;
    u.tmp = d_tmp.p + v.tmp_up;
    u.w = v.sw;
    u.h = v.sh;
    u.nw = img.w;
    u.nh = img.h;
    const DevTapsRef uv = cached_taps(kGaussian, 0.0f, v.sh, img.h), uh = cached_taps(kGaussian, 0.0f, v.sw, img.w);
    u.tv = uv.taps;
    u.wv = uv.wts;
    u.th = uh.taps;
    u.wh = uh.wts;
    u.block0_v = buv;
    u.block0_h = buh;
    buv += cdiv_u32(v.sw, 128) * img.h;
    buh += cdiv_u32(img.w, 128) * img.h;
    up.push_back(u);
  }
  const size_t nj = lv.size();
  std::vector<ResizeJob> all(down);
  all.insert(all.end(), up.begin(), up.end());
  CUDA_TRY(d_jobs.alloc_on(all.size(), st));
  CUDA_TRY(cudaMemcpyAsync(d_jobs.p, all.data(), all.size() * sizeof(ResizeJob), cudaMemcpyHostToDevice, st));
  launch_resize_v_jobs(d_jobs.p, (uint32_t)nj, bdv, st);
  launch_resize_h_jobs(d_jobs.p, (uint32_t)nj, bdh, st);
  launch_resize_v_jobs(d_jobs.p + nj, (uint32_t)nj, buv, st);
  launch_resize_h_jobs(d_jobs.p + nj, (uint32_t)nj, buh, st);
  CUDA_TRY(cudaGetLastError());
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
  uint32_t ppitch = 0;  // row pitch of the padded levels
  uint64_t dev_bytes = 0;  // device memory the session holds
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
  // every texel a run can compare has alpha 255: all examples (ignored ones
  // too, random init copies them), guides and the target guide are opaque,
  // and no pyramid level is a zero image (a downscale with a zero side)
  bool opaque = false;
  EventHandle ready;  // recorded after build()'s device work; runs wait for it
  bool consumed = false;
  std::string err;
  // The pyramids are stream-ordered pool memory freed on the legacy stream:
  // wait for build()'s own work first (a run waits for its work itself).
  ~ts_session() {
    if (ready.e) cudaEventSynchronize(ready.e);
  }
  ts_session() = default;
  ts_session(ts_session &&) = default;
  ts_session &operator=(ts_session &&) = default;
};

struct ts_generated {
  uint32_t W = 0, H = 0;
  std::vector<uint32_t> in_dims;  // (w, h) of every example at its loaded size
  std::vector<uint4> state;       // per pixel, until the maps below are first asked for
  void ensure_maps() {
    if (state.empty()) return;
    const size_t N = state.size();
    coord.resize(N * 3);
    ids.resize(N * 2);
    for (size_t i = 0; i < N; ++i) {
      coord[3 * i] = state[i].x & 0xffffu;
      coord[3 * i + 1] = state[i].x >> 16;
      coord[3 * i + 2] = state[i].w;
      ids[2 * i] = state[i].y;
      ids[2 * i + 1] = state[i].z;
    }
    std::vector<uint4>().swap(state);
  }
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
    device_pyramids({PyramidJob{&img, levels, d.p}}, 0);
    CUDA_TRY(cudaMemcpy(out, d.p, (size_t)w * h * nl * 4, cudaMemcpyDeviceToHost));
  } catch (const Failure &f) {
    return f.status;
  }
  return TS_OK;
}

int ts_guide_map(const uint8_t *rgba, uint32_t w, uint32_t h, const uint8_t *target_rgba, uint32_t tw, uint32_t th,
                 uint8_t *out_rgba, int32_t device) {
  if (!rgba || !target_rgba || !out_rgba) return TS_ERR_NULL;
  if (w == 0 || h == 0 || tw == 0 || th == 0) return TS_ERR_IMAGE;
  if (w > kMaxSide || h > kMaxSide || tw > kMaxSide || th > kMaxSide) return TS_ERR_LIMIT;
  try {
    CUDA_TRY(cudaSetDevice(device));
    StreamGuard sg;
    CUDA_TRY(cudaStreamCreateWithFlags(&sg.s, cudaStreamNonBlocking));
    const Image g = device_guide_map(copy_image(rgba, w, h), copy_image(target_rgba, tw, th), sg.s);
    memcpy(out_rgba, g.px.data(), g.px.size());
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
int ts_builder_tuning(ts_builder *b, const ts_tuning *t) {
  BUILDER_GUARD(b);
  if (!t) return TS_ERR_NULL;
  b->prm.team_max_batch = t->team_max_items;
  b->prm.team_full_max_batch = t->team_full_max_items;
  b->prm.walk_window_max = t->walk_window_max_items;
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

namespace {
void keep_pool(int dev);
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
    keep_pool(p.device);
    StreamGuard sg;
    CUDA_TRY(cudaStreamCreateWithFlags(&sg.s, cudaStreamNonBlocking));
    const cudaStream_t st = sg.s;
    CUDA_TRY(configure_kernels(p.k, (uint32_t)p.m));
    // the target guide at the output size (session.rs:258-266), then the
    // inputs at their final sizes (Example::resolve, lib.rs:564-603);
    // examples without a guide get the automatic one (lib.rs:575-582)
    // (the builder is consumed: its images are taken over, except an
    // inpainting example whose channel the mask is made from below)
    Image tg;
    if (s->guided) tg = load_image(std::move(b->target), true, W, H, st);
    std::vector<Image> imgs(s->n_ex), guides(s->n_ex), masks(s->n_ex);
    for (uint32_t e = 0; e < s->n_ex; ++e) {
      ExampleIn &ex = b->examples[e];
      const bool reread = b->has_inpaint && b->inpaint.channel && e == b->inpaint.example_index;
      imgs[e] = reread ? load_image(ex.img, has_in, in_w, in_h, st) : load_image(std::move(ex.img), has_in, in_w, in_h, st);
      if (imgs[e].w > kMaxSide || imgs[e].h > kMaxSide) throw Failure{TS_ERR_LIMIT, "example side exceeds limit"};
      if (s->guided) {
        guides[e] = ex.has_guide ? load_image(std::move(ex.guide), has_in, in_w, in_h, st)
                                 : device_guide_map(imgs[e], tg, st);
        if (guides[e].w > kMaxSide || guides[e].h > kMaxSide) throw Failure{TS_ERR_LIMIT, "guide side exceeds limit"};
      }
      if (ex.method == TS_SAMPLE_IMAGE) {
        masks[e] = load_image(std::move(ex.mask), has_in, in_w, in_h, st);
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
      texels += (uint64_t)md.w * md.h * s->n_levels;
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
    {
      // constant alpha 255 stays 255 through the pyramid's resizes (their
      // weights are normalised, and the u8 result is rounded), unless a
      // level's downscale has a zero side
      const uint32_t sh = s->n_levels - 1;
      auto opaque = [&](const Image &im) {
        if (sh < 32 && ((im.w >> sh) == 0 || (im.h >> sh) == 0)) return false;
        for (size_t i = 0; i < (size_t)im.w * im.h; ++i)
          if (im.px[4 * i + 3] != 255) return false;
        return true;
      };
      bool op = sh < 32;
      for (uint32_t e = 0; op && e < s->n_ex; ++e) op = opaque(imgs[e]) && (!s->guided || opaque(guides[e]));
      if (op && s->guided) op = opaque(tg);
      s->opaque = op;
    }
    // padded copies share one row pitch, the widest map's, so that a
    // neighbour offset is one texel offset on every map
    uint32_t pitch = 0;
    for (const MapDesc &md : s->maps) pitch = std::max(pitch, md.w + 2 * kPad);
    s->ppitch = pitch;
    for (MapDesc &md : s->maps) {
      md.pw = pitch;
      md.ph = md.h + 2 * kPad;
      md.poff = ptexels;
      ptexels += (uint64_t)md.pw * md.ph * s->n_levels;
    }
    CUDA_TRY(s->levels.alloc_kept(texels, st));
    CUDA_TRY(s->masks.alloc_kept(mask_bytes, st));
    std::vector<PyramidJob> pyr;  // every pyramid of the session, built together below
    for (uint32_t f = 0; f < s->n_maps; ++f) {
      const uint32_t e = s->filtered[f];
      pyr.push_back(PyramidJob{&imgs[e], p.backtrack_stages, s->levels.p + s->maps[f].off});
      if (s->maps[f].mask_off >= 0) {
        std::vector<uint8_t> mb((size_t)s->maps[f].w * s->maps[f].h);
        for (size_t i = 0; i < mb.size(); ++i) mb[i] = masks[e].px[4 * i] != 0 ? 1 : 0;
        CUDA_TRY(cudaMemcpyAsync(s->masks.p + s->maps[f].mask_off, mb.data(), mb.size(), cudaMemcpyHostToDevice, st));
      }
    }
    CUDA_TRY(s->plevels.alloc_kept(ptexels, st));
    CUDA_TRY(s->d_maps.alloc_kept(s->n_maps, st));
    CUDA_TRY(cudaMemcpyAsync(s->d_maps.p, s->maps.data(), s->n_maps * sizeof(MapDesc), cudaMemcpyHostToDevice, st));
    // guides: every example (unfiltered order) plus the target guide
    std::vector<GuideDesc> gd(std::max<uint32_t>(s->n_ex, 1));
    if (s->guided) {
      uint64_t gtex = 0;
      for (uint32_t e = 0; e < s->n_ex; ++e) {
        gd[e].w = guides[e].w;
        gd[e].h = guides[e].h;
        gd[e].off = gtex;
        gtex += (uint64_t)guides[e].w * guides[e].h * s->n_levels;
      }
      // the guide of map f is example f's guide (unfiltered index); the
      // padded fast path needs its size to equal the map's
      for (uint32_t f = 0; f < s->n_maps; ++f)
        if (f >= s->n_ex || gd[f].w != s->maps[f].w || gd[f].h != s->maps[f].h) s->guide_dims_differ = true;
      CUDA_TRY(s->guides.alloc_kept(gtex, st));
      for (uint32_t e = 0; e < s->n_ex; ++e)
        pyr.push_back(PyramidJob{&guides[e], p.backtrack_stages, s->guides.p + gd[e].off});
      if (!s->guide_dims_differ) CUDA_TRY(s->pguides.alloc_kept(ptexels, st));
      CUDA_TRY(s->tguide.alloc_kept((size_t)W * H * s->n_levels, st));
      pyr.push_back(PyramidJob{&tg, p.backtrack_stages, s->tguide.p});
    }
    device_pyramids(pyr, st);
    for (uint32_t f = 0; f < s->n_maps; ++f)
      launch_pad(s->levels.p + s->maps[f].off, s->maps[f].w, s->maps[f].h, s->n_levels, pitch,
                 s->plevels.p + s->maps[f].poff, st);
    // padded guides per map, at the map's own padded offsets (same size:
    // only then are they read)
    if (s->guided && !s->guide_dims_differ)
      for (uint32_t f = 0; f < s->n_maps; ++f)
        launch_pad(s->guides.p + gd[f].off, gd[f].w, gd[f].h, s->n_levels, pitch, s->pguides.p + s->maps[f].poff, st);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(s->d_gdesc.alloc_kept(gd.size(), st));
    CUDA_TRY(cudaMemcpyAsync(s->d_gdesc.p, gd.data(), gd.size() * sizeof(GuideDesc), cudaMemcpyHostToDevice, st));
    // the pyramids are still being built: run() waits for this event on the
    // device, so its host planning overlaps them
    CUDA_TRY(cudaEventCreateWithFlags(&s->ready.e, cudaEventDisableTiming));
    CUDA_TRY(cudaEventRecord(s->ready.e, st));
    s->dev_bytes = s->levels.bytes() + s->plevels.bytes() + s->guides.bytes() + s->pguides.bytes() +
                   s->tguide.bytes() + s->masks.bytes() + s->d_maps.bytes() + s->d_gdesc.bytes();
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
  bool grid_first;
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

namespace {

// One batch step of a session's run, with the launches it needs; the plain
// path issues them one session at a time, the batched path one phase of many
// sessions' steps per launch.
struct Step {
  int stage = 0;                 // index into the stage plan
  bool stage_end = false;        // last step of its stage (progress point)
  bool ls = false;               // level switch before the step
  uint32_t ls_level = 0, ls_n_res = 0;
  bool rc = false;               // random candidates of a new chunk
  StageDev rc_st{};
  bool batch = false;
  StageDev st{};
  BatchDev bd{};
  bool exhaustive = false;       // exhaustive k-NN over the whole batch
  int resolve = kPhaseResolve;   // kPhaseResolve, kPhaseTeamPart or kPhaseTeamFull
  uint32_t n = 0;                // items of the batch
  uint32_t stage_i0 = 0;         // the batch's first item within its stage
  uint32_t bidx = 0;             // index of the batch in the run (RunCtx::btab)
  int knn_wait = -1;             // k-NN ahead: the chunk whose k-NN this step waits for first
};

// k-NN made ahead of the resolves (RunCtx::knn_ahead): consecutive batch
// steps of one stage whose neighbour lists one launch (or a walk and its
// fallback launch) computes on the k-NN stream.
struct KnnChunk {
  int stage = 0;
  StageDev st{};                // the stage's items
  BatchDev b{};                 // stage items [b.i0, b.i1); each item's tree length from b.btab
  bool all_exhaustive = false;  // exhaustive k-NN for every item (else the walk, then its fallbacks)
  // tree entries of the chunk's appended items, made just before its k-NN:
  // items [a0, a1) at resolved-list index pos0 on; none below nomir_end
  // gets tiling mirrors
  uint32_t a0 = 0, a1 = 0, pos0 = 0, nomir_end = 0;
};

// Everything one run holds between planning and reading back.
struct RunCtx {
  ts_session *s = nullptr;
  uint32_t W = 0, H = 0, k = 0, m = 0;
  size_t N = 0;
  size_t locked = 0;
  std::vector<StagePlan> plan;
  std::vector<Step> steps;
  // host data uploaded at the start of the run
  std::vector<uint32_t> color, resolved, items, occ, mir, cells;
  int32_t cox = 0, coy = 0;
  uint32_t cgw = 0, cgh = 0;
  std::vector<uint4> state;
  // dense_init: colour and state are uploaded whole (inpainting); otherwise
  // both start zeroed on the device and init_list holds the few set pixels
  // as {pixel, colour, state.x, state.y, state.z, state.w}
  bool dense_init = false;
  std::vector<uint32_t> init_list;
  // items_async: the caller uploads the items from pitems itself
  bool items_async = false;
  PinnedBuf<uint32_t> pitems;
  std::vector<float> luts;
  std::vector<int32_t> tab;
  std::vector<double> xdiv, ydiv, dxt, dy2t;
  size_t n_batches = 0;
  uint64_t overall_total = 0;
  uint32_t max_batch_items = 1;
  uint64_t rc_items = 1;
  // rc_ahead: every stage's random candidates are made on a side stream at
  // the start (stage q's launch carried by step rc_step[q]); the main
  // stream waits for rc_ev[q] instead of launching them itself
  bool want_rc_ahead = false, rc_ahead = false;
  std::vector<int> rc_step;
  std::vector<EventHandle> rc_ev;
  // knn_ahead: the neighbour lists and means of every batch are made on a
  // k-NN stream, chunk by chunk, as soon as a stage's items are up (they
  // depend on the pick chain's order only: which pixels are in the tree at
  // each batch start); the resolves wait for their chunk's event.  Plain
  // path, k > 0, exact distance sums.
  bool want_knn_ahead = false, knn_ahead = false;
  std::vector<KnnChunk> knn_chunks;
  std::vector<EventHandle> knn_ev;  // per chunk: its k-NN is done
  std::vector<EventHandle> items_ev;  // per stage: its items are on the device
  std::vector<uint2> btab;          // every batch: {first stage item, tree length at its start}
  // knn_ahead: a batch step whose commit the next step's resolve launch
  // makes (its results in one of two result buffers, alternating)
  bool pend = false;
  int pend_stage = -1;
  StageDev pend_st{};
  BatchDev pend_bd{};
  uint32_t pend_n = 0, defer_parity = 0;
  size_t res_total = 0;                // resolved-list length at the end of the run
  std::vector<uint32_t> unresolved;    // pixels not yet picked (the pick chain's state)
  size_t picked_stages = 0;            // stages whose items are known
  bool parallel_picks = false;         // draws of large stages on the shared host pool (single-session runs)
  std::vector<uint64_t> draws;         // a stage's random indices, before the swap-removes
  int32_t x_l = 0, y_b = 0;
  uint64_t dev_bytes = 0;  // device memory run_alloc takes
  // device state
  // three allocations: zeroed at the start (zero), uploaded from the pinned
  // block ptab (tabs) and scratch (work); the arrays below are views
  DevBuf<uint8_t> d_zero, d_tabs, d_work;
  size_t zero_bytes = 0, tabs_bytes = 0;
  struct TabPart {
    size_t off;
    const void *src;
    size_t bytes;
  };
  std::vector<TabPart> tab_parts;
  PinnedBuf<uint8_t> ptab;
  DevBuf<uint32_t> d_color, d_occ, d_mir, d_res, d_items, d_ncnt, d_fbl, d_fbc, d_cells, d_init;
  DevBuf<uint32_t> d_rank, d_kncnt, d_kfbl, d_kfbc;  // knn_ahead
  DevBuf<uint32_t> d_wctr;  // per batch: the warp resolve's item counter (BatchDev::work_ctr)
  DevBuf<int32_t> d_knbuf;
  DevBuf<double> d_kmean;
  DevBuf<uint2> d_btab;
  DevBuf<uint4> d_shadow;
  DevBuf<uint4> d_state;
  DevBuf<float> d_rscore, d_lut;
  DevBuf<double> d_xdiv, d_ydiv, d_dist, d_dxt, d_dy2t, d_mean;
  DevBuf<int32_t> d_tab, d_nbuf;
  DevBuf<uint2> d_rcand;
  DevBuf<Result> d_result;
  DevBuf<int> d_err;
  DevBuf<unsigned long long> d_evals;
  SessionDev sd{};
  // read back
  std::vector<uint32_t> col;
  std::vector<uint4> stv;
  int derr = 0;
  unsigned long long evals = 0;
  std::unique_ptr<ts_generated> g;
  uint64_t launches = 0, batches = 0, resolves = 0;
};

bool exact_sum_ok(uint32_t W, uint32_t H, uint32_t k);

// Whether a run makes its k-NN ahead (RunCtx::knn_ahead): asked for, k > 0,
// exact sums, and the lists of every item of the run, held at once, within
// kKnnAheadMaxBytes (larger runs keep the per-step form's scratch).  run_plan
// leaves out the coordinate tables of such runs, so it decides the same way.
bool knn_ahead_fits(const RunCtx &c, uint32_t W, uint32_t H, uint32_t k) {
  constexpr uint64_t kKnnAheadMaxBytes = 16ull << 30;
  return c.want_knn_ahead && k > 0 && exact_sum_ok(W, H, k) &&
         (uint64_t)c.items.size() * ((uint64_t)k * 4 + 16) <= kKnnAheadMaxBytes;
}

// Host schedule of Generator::resolve (ms.rs:702-1051) and the device
// buffers of the run; nothing is enqueued yet.
void run_plan(ts_session *s, RunCtx &c) {
  const Params &p = s->prm;
  c.s = s;
  const uint32_t W = c.W = s->W, H = c.H = s->H;
  const size_t N = c.N = (size_t)W * H;
  const uint32_t k = c.k = p.k, m = c.m = (uint32_t)p.m;
  const uint32_t stages = p.backtrack_stages;
  c.g.reset(new (std::nothrow) ts_generated());
  if (!c.g) throw Failure{TS_ERR_OUT_OF_MEMORY, "out of host memory"};
  // ---- initial state (Generator::new / new_from_inpaint) ----
  std::vector<uint32_t> &color = c.color;
  std::vector<uint4> &state = c.state;
  std::vector<uint32_t> &resolved = c.resolved;
  c.dense_init = s->inpaint;
  c.init_list.clear();
  if (c.dense_init) {
    color.assign(N, 0);
    state.assign(N, make_uint4(0, 0, 0, 0));
  }
  auto put = [&](uint32_t px, uint32_t col, uint4 sv) {
    if (c.dense_init) {
      color[px] = col;
      state[px] = sv;
    } else {
      c.init_list.insert(c.init_list.end(), {px, col, sv.x, sv.y, sv.z, sv.w});
    }
  };
  std::vector<uint32_t> &unresolved = c.unresolved;
  unresolved.clear();
  size_t locked = 0;
  if (s->inpaint) {
    for (size_t i = 0; i < N; ++i) {
      const uint8_t *cc = &s->inpaint_colors.px[4 * i];
      color[i] = (uint32_t)cc[0] | ((uint32_t)cc[1] << 8) | ((uint32_t)cc[2] << 16) | ((uint32_t)cc[3] << 24);
      if (s->inpaint_mask[i]) {
        unresolved.push_back((uint32_t)i);
      } else {
        resolved.push_back((uint32_t)i);
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
      const uint8_t *cc = &im.px[((size_t)y * im.w + x) * 4];
      put(px, (uint32_t)cc[0] | ((uint32_t)cc[1] << 8) | ((uint32_t)cc[2] << 16) | ((uint32_t)cc[3] << 24),
          make_uint4(x | (y << 16), px, map, map));
      resolved.push_back(px);
    }
    locked += p.random_init;
  }
  c.locked = locked;
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
  std::vector<StagePlan> &plan = c.plan;
  std::vector<uint32_t> &items = c.items;
  std::vector<float> &luts = c.luts;
  size_t n_res = resolved.size();
  size_t n_unresolved = unresolved.size();
  size_t n_items_total = 0;
  int32_t pyramid_level = 0;
  uint32_t max_batch_items = 1, max_stage_items = 1;
  static const std::vector<int32_t> kTab = knn_table(kKnnTabRadius);  // built once per process
  c.tab = kTab;
  const std::vector<int32_t> &tab = c.tab;
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
      const float cv = s->guided ? (1.0f - adaptive) * cauchy[d] : cauchy[d];
      luts.push_back(cv);
      slow |= !std::isfinite(cv);
    }
    for (int d = 0; d < 256; ++d) {
      const float gv = s->guided ? adaptive * l2[d] : 0.0f;
      luts.push_back(gv);
      slow |= !std::isfinite(gv);
    }
    sp.slow_lut = slow;
    const size_t P_eff = std::min(P, redo + n_unresolved);
    sp.items_off = (uint32_t)n_items_total;
    sp.n_items = (uint32_t)P_eff;
    sp.redo = (uint32_t)redo;
    sp.n_res_start = (uint32_t)n_res;
    n_items_total += P_eff;
    n_unresolved -= P_eff > redo ? P_eff - redo : 0;
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
      // fewer than k points expected within the offset table: straight to
      // the cell grid
      bp.grid_first = k > 0 && !bp.exhaustive && (double)R * tab.size() < (double)k * (double)N;
      R += bp.i1 - bp.append_from;
      sp.batches.push_back(bp);
      max_batch_items = std::max<uint32_t>(max_batch_items, (uint32_t)bsz);
      i += bsz;
    }
    n_res = R;
    max_stage_items = std::max<uint32_t>(max_stage_items, (uint32_t)P_eff);
    plan.push_back(std::move(sp));
  }
  // the items themselves come from the pick chain, stage by stage (run_pick)
  items.assign(n_items_total, 0);
  c.res_total = n_res;
  resolved.reserve(n_res);  // the picks append without moving the locked entries
  c.picked_stages = 0;
  // ---- host tables ----
  const uint32_t wpr = (W + 31) / 32;
  for (auto &sp : plan) c.n_batches += sp.batches.size();
  c.max_batch_items = max_batch_items;
  c.rc_items = std::max<uint64_t>(1, std::min<uint64_t>(max_stage_items, kRcandBudget / std::max(m, 1u)));
  c.rc_ahead = c.want_rc_ahead && m > 0 && (uint64_t)n_items_total * m <= kRcandWhole;
  c.x_l = x_l;
  c.y_b = y_b;
  const int32_t xo = x_l + 2, yo = y_b + 2;
  // The coordinate tables below serve the f64 distances of inexact sessions
  // and of the fused small-step kernel; a run whose k-NN is made ahead
  // (exact sums) derives every distance from its offset and needs none.
  const bool no_dist_tables = knn_ahead_fits(c, W, H, k);
  c.xdiv.resize(no_dist_tables ? 0 : W + 2 * (size_t)xo + 1);
  c.ydiv.resize(no_dist_tables ? 0 : H + 2 * (size_t)yo + 1);
  for (size_t i = 0; i < c.xdiv.size(); ++i) c.xdiv[i] = (double)((int64_t)i - xo) / (double)W;
  for (size_t i = 0; i < c.ydiv.size(); ++i) c.ydiv[i] = (double)((int64_t)i - yo) / (double)H;
  // per-pixel tables of the normalised offsets the weights use: dx and
  // dy * dy for |offset| <= kDistTabRadius, the same IEEE operations as
  // get_distances_to_k_neighs (ms.rs:410-415)
  const int32_t R = kDistTabRadius;
  c.dxt.resize(no_dist_tables ? 0 : (size_t)W * (2 * R + 1));
  c.dy2t.resize(no_dist_tables ? 0 : (size_t)H * (2 * R + 1));
  for (uint32_t x = 0; x < W && !no_dist_tables; ++x)
    for (int32_t o = -R; o <= R; ++o)
      c.dxt[(size_t)x * (2 * R + 1) + o + R] = (double)((int64_t)x + o) / (double)W - (double)x / (double)W;
  for (uint32_t y = 0; y < H && !no_dist_tables; ++y)
    for (int32_t o = -R; o <= R; ++o) {
      const double dy = (double)((int64_t)y + o) / (double)H - (double)y / (double)H;
      c.dy2t[(size_t)y * (2 * R + 1) + o + R] = dy * dy;
    }
  // the tree is rebuilt from the resolved list, mirrors included (ms.rs:747-779)
  c.occ.assign((size_t)wpr * H, 0);
  c.mir.assign((size_t)wpr * H, 0);
  for (size_t i = 0; i < locked; ++i) {
    const uint32_t q = resolved[i];
    c.occ[(size_t)(q / W) * wpr + (q % W) / 32] |= 1u << ((q % W) & 31);
    if (p.tiling) c.mir[(size_t)(q / W) * wpr + (q % W) / 32] |= 1u << ((q % W) & 31);
  }
  // resolved points per cell of the plane the tree spans (the image and,
  // when tiling, its mirror bands)
  c.cox = p.tiling ? -x_l : 0;
  c.coy = p.tiling ? -y_b : 0;
  c.cgw = (W + (p.tiling ? 2 * (uint32_t)x_l : 0) + kCell - 1) / kCell;
  c.cgh = (H + (p.tiling ? 2 * (uint32_t)y_b : 0) + kCell - 1) / kCell;
  c.cells.assign((size_t)c.cgw * c.cgh, 0);
  auto add_cell = [&](int x, int y) { c.cells[(size_t)((y - c.coy) / kCell) * c.cgw + (x - c.cox) / kCell] += 1; };
  for (size_t i = 0; i < locked; ++i) {
    const int x = (int)(resolved[i] % W), y = (int)(resolved[i] / W);
    add_cell(x, y);
    if (!p.tiling || !((c.mir[(size_t)y * wpr + x / 32] >> (x & 31)) & 1u)) continue;
    if (x < x_l)
      add_cell(x + (int)W, y);
    else if (x > (int)W - x_l)
      add_cell(x - (int)W, y);
    if (y < y_b)
      add_cell(x, y + (int)H);
    else if (y > (int)H - y_b)
      add_cell(x, y - (int)H);
  }
  // device memory the run will hold (run_alloc), for admission control
  const size_t kk = std::max<uint32_t>(k, 1), mb = max_batch_items;
  uint64_t steps_est = 0;
  for (auto &sp : plan) steps_est += sp.batches.size() + 1;
  c.dev_bytes = N * 4 + N * sizeof(uint4) + 2 * (uint64_t)wpr * H * 4 + c.res_total * 8 + items.size() * 4 +
                c.luts.size() * 4 + c.tab.size() * 4 + mb * kk * 12 + mb * (4 + 8 + 4 + sizeof(Result)) +
                c.n_batches * 4 + (c.rc_ahead ? (uint64_t)items.size() : std::max<uint64_t>(c.rc_items, mb)) * m * 8 +
                (c.xdiv.size() + c.ydiv.size() + c.dxt.size() + c.dy2t.size()) * 8 + steps_est * sizeof(StepDev) +
                c.cells.size() * 4 + c.init_list.size() * 4;
}

// A small pool of host threads shared by every single-session run: it
// computes the random draws of the large stages of the pick chain.  One job
// at a time (runs that find it busy compute their draws themselves).
class DrawPool {
 public:
  static DrawPool &get() {
    static DrawPool *pool = new DrawPool();  // never destroyed: its threads sleep on it until exit
    return *pool;
  }
  // fn(a, b) over [0, n) in chunks of `grain`, on the pool and the caller;
  // false (nothing done) when another run holds the pool
  bool run(size_t n, size_t grain, const std::function<void(size_t, size_t)> &fn) {
    std::unique_lock<std::mutex> job(job_mu_, std::try_to_lock);
    if (!job.owns_lock() || workers_.empty()) return false;
    {
      std::lock_guard<std::mutex> lk(mu_);
      fn_ = &fn;
      n_ = n;
      grain_ = grain;
      next_ = 0;
      left_ = (n + grain - 1) / grain;
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return left_ == 0; });
    fn_ = nullptr;
    return true;
  }

 private:
  DrawPool() {
    const unsigned hc = std::max(1u, std::thread::hardware_concurrency());
    const unsigned nw = std::min(7u, hc > 2 ? hc - 2 : 0u);
    for (unsigned i = 0; i < nw; ++i) workers_.emplace_back([this] { loop(); });
    for (auto &t : workers_) t.detach();  // they sleep until the process exits
  }
  void loop() {
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return fn_ != nullptr && next_ * grain_ < n_; });
      }
      work();
    }
  }
  // Chunks are claimed under the mutex, so a claim always belongs to the
  // job that is current when it is made.
  void work() {
    for (;;) {
      const std::function<void(size_t, size_t)> *fn;
      size_t a, b;
      {
        std::lock_guard<std::mutex> lk(mu_);
        if (!fn_ || next_ * grain_ >= n_) return;
        fn = fn_;
        a = next_ * grain_;
        b = std::min(n_, a + grain_);
        ++next_;
      }
      (*fn)(a, b);
      std::lock_guard<std::mutex> lk(mu_);
      if (--left_ == 0) done_cv_.notify_all();
    }
  }
  std::mutex job_mu_, mu_;
  std::condition_variable cv_, done_cv_;
  std::vector<std::thread> workers_;
  const std::function<void(size_t, size_t)> *fn_ = nullptr;
  size_t n_ = 0, grain_ = 1, next_ = 0, left_ = 0;
};

// pick_random_unresolved (ms.rs:380-389) for a stage's items: redo item i
// is resolved[i + locked]; new item i swap-removes
// Pcg32::seed_from_u64(seed + i).gen_range(0..len) from the unresolved list.
// len is known in advance (the list shrinks by one per new item), so the
// draws are independent of one another and of the list; only the
// swap-removes that consume them run in order.
void run_pick(RunCtx &c) {
  const StagePlan &sp = c.plan[c.picked_stages++];
  std::vector<uint32_t> &unresolved = c.unresolved;
  uint32_t *it = c.items.data() + sp.items_off;
  const uint32_t redo = std::min(sp.redo, sp.n_items);
  for (uint32_t i = 0; i < redo; ++i) it[i] = c.resolved[i + c.locked];
  const size_t n_new = sp.n_items - redo, len0 = unresolved.size();
  if (n_new > len0) throw Failure{TS_ERR_INVALID_RANGE, "more new items than unresolved pixels"};
  c.draws.resize(n_new);
  uint64_t *dr = c.draws.data();
  const std::function<void(size_t, size_t)> draw = [&](size_t a, size_t b) {
    for (size_t q = a; q < b; ++q) {
      Pcg32 r = pcg_from_u64(sp.seed + (uint64_t)(redo + q));
      dr[q] = gen_range_u64(r, len0 - q);
    }
  };
  constexpr size_t kGrain = 8192;
  if (!(c.parallel_picks && n_new >= 4 * kGrain && DrawPool::get().run(n_new, kGrain, draw))) draw(0, n_new);
  uint32_t *un = unresolved.data();
  size_t len = len0;
  for (size_t q = 0; q < n_new; ++q) {
    const uint64_t idx = dr[q];
    it[redo + q] = un[idx];
    un[idx] = un[--len];
  }
  unresolved.resize(len);
  for (const BatchPlan &bp : sp.batches)
    for (uint32_t t = bp.append_from; t < bp.i1; ++t) c.resolved.push_back(it[t]);
}

void run_pick_all(RunCtx &c) {
  while (c.picked_stages < c.plan.size()) run_pick(c);
}

// Let the device's default stream-ordered pool keep freed memory (by
// default it returns it at every synchronisation), so that each run's
// buffers come from the pool without device calls.  Once per device.
void keep_pool(int dev) {
  static std::mutex mu;
  static std::vector<int> done;
  std::lock_guard<std::mutex> lk(mu);
  if (std::find(done.begin(), done.end(), dev) != done.end()) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  done.push_back(dev);
}

// Whether a session's neighbour-distance sums (get_distances_to_k_neighs,
// ms.rs:405-425) are exact.  With W and H powers of two, x / W and y / H are
// exact, so every distance fma(dx, dx, dy * dy) is an integer multiple of
// q = 1 / max(W, H)^2 below 8 max(W, H)^2 q (tiling mirrors included), and a
// list of 4k such values sums below 32 k max(W, H)^2 q.  When that is below
// 2^53 q every partial sum is representable, so the reference's in-order f64
// adds never round and any order of exact adds yields the same double.
bool exact_sum_ok(uint32_t W, uint32_t H, uint32_t k) {
  auto pow2 = [](uint32_t v) { return v != 0 && (v & (v - 1)) == 0; };
  if (!pow2(W) || !pow2(H)) return false;
  const uint64_t M = std::max(W, H);
  return M <= (1u << 16) && 32ull * std::max<uint32_t>(k, 1) * M * M < (1ull << 53);
}

// Side streams of a run (the k-NN and random candidates made ahead) run on a
// green context that holds all SMs but kReservedSms.  A running block cannot
// be preempted, so side blocks on every SM would hold up each launch of the
// resolve chain, which in the first stage is a long chain of small
// latency-bound launches; the reserved SMs take those at once.  Created once
// per device and kept; where the driver offers no green contexts the side
// streams are ordinary (low-priority) streams.
constexpr unsigned kReservedSms = 8;

struct GreenSide {
  bool ok = false;
  CUgreenCtx g = nullptr;
  CUresult (*stream_create)(CUstream *, CUgreenCtx, unsigned, int) = nullptr;
};

template <typename F>
bool driver_entry(const char *name, F &fn) {
  void *v = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion(name, &v, 13000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !v)
    return false;
  fn = (F)v;
  return true;
}

const GreenSide &green_side(int dev) {
  static std::mutex mu;
  static std::map<int, GreenSide> sides;
  std::lock_guard<std::mutex> lk(mu);
  auto it = sides.find(dev);
  if (it != sides.end()) return it->second;
  GreenSide &gs = sides[dev];
  CUresult (*device_get)(CUdevice *, int) = nullptr;
  CUresult (*get_resource)(CUdevice, CUdevResource *, CUdevResourceType) = nullptr;
  CUresult (*split)(CUdevResource *, unsigned *, const CUdevResource *, CUdevResource *, unsigned, unsigned) = nullptr;
  CUresult (*make_desc)(CUdevResourceDesc *, CUdevResource *, unsigned) = nullptr;
  CUresult (*create)(CUgreenCtx *, CUdevResourceDesc, CUdevice, unsigned) = nullptr;
  if (!driver_entry("cuDeviceGet", device_get) || !driver_entry("cuDeviceGetDevResource", get_resource) ||
      !driver_entry("cuDevSmResourceSplitByCount", split) || !driver_entry("cuDevResourceGenerateDesc", make_desc) ||
      !driver_entry("cuGreenCtxCreate", create) || !driver_entry("cuGreenCtxStreamCreate", gs.stream_create))
    return gs;
  CUdevice cd;
  CUdevResource all{}, part{}, rest{};
  unsigned groups = 1;
  CUdevResourceDesc desc;
  if (device_get(&cd, dev) != CUDA_SUCCESS || get_resource(cd, &all, CU_DEV_RESOURCE_TYPE_SM) != CUDA_SUCCESS ||
      all.sm.smCount <= kReservedSms + all.sm.minSmPartitionSize)
    return gs;
  if (split(&part, &groups, &all, &rest, 0, all.sm.smCount - kReservedSms) != CUDA_SUCCESS || groups != 1 ||
      part.sm.smCount >= all.sm.smCount || make_desc(&desc, &part, 1) != CUDA_SUCCESS ||
      create(&gs.g, desc, cd, CU_GREEN_CTX_DEFAULT_STREAM) != CUDA_SUCCESS)
    return gs;
  gs.ok = true;
  return gs;
}

// A side stream of priority prio on the device's green context (green_side),
// else an ordinary one.
cudaError_t side_stream(int dev, int prio, cudaStream_t *out) {
  const GreenSide &gs = green_side(dev);
  CUstream cs = nullptr;
  if (gs.ok && gs.stream_create(&cs, gs.g, CU_STREAM_NON_BLOCKING, prio) == CUDA_SUCCESS) {
    *out = (cudaStream_t)cs;
    return cudaSuccess;
  }
  return cudaStreamCreateWithPriority(out, cudaStreamNonBlocking, prio);
}

// Device buffers of a run and the step descriptors that point into them.
// With a pool stream, the buffers are stream-ordered pool memory (freed
// without waiting for the device); otherwise plain cudaMalloc.
void run_alloc(RunCtx &c, cudaStream_t pool) {
  ts_session *s = c.s;
  const Params &p = s->prm;
  const uint32_t W = c.W, H = c.H;
  const size_t N = c.N;
  const uint32_t k = c.k, m = c.m;
  const std::vector<StagePlan> &plan = c.plan;
  const uint32_t max_batch_items = c.max_batch_items;
  const uint64_t rc_items = c.rc_items;
  const int32_t x_l = c.x_l, y_b = c.y_b;
  const int32_t xo = x_l + 2, yo = y_b + 2;
  const int32_t R = kDistTabRadius;
  const uint32_t wpr = (W + 31) / 32;
  auto A = [&](auto &buf, size_t n) { return pool ? buf.alloc_on(n, pool) : buf.alloc(n); };
  struct Layout {
    size_t off = 0;
    size_t add(size_t bytes) {
      const size_t o = off;
      off += (std::max<size_t>(bytes, 1) + 255) / 256 * 256;
      return o;
    }
  } zl, tl, wl;
  const size_t kk = std::max<uint32_t>(k, 1), mb = max_batch_items;
  const size_t rc_n = c.rc_ahead ? c.items.size() * m : (size_t)std::max<uint64_t>(rc_items, mb) * m;
  // k-NN ahead: the batch table and the chunks (consecutive batches of a
  // stage with one k-NN form, each at least as large as the stage's items
  // before it, so that a chunk's k-NN overlaps the resolves of the ones
  // before)
  c.knn_ahead = knn_ahead_fits(c, W, H, k);
  c.btab.clear();
  c.knn_chunks.clear();
  std::vector<std::pair<uint32_t, uint32_t>> chunk_batches;  // [first, last) batch of each chunk
  std::vector<uint32_t> stage_bt_base(plan.size(), 0);        // each stage's first batch
  if (c.knn_ahead) {
    constexpr uint32_t kChunkMinItems = 64;
    for (size_t si = 0; si < plan.size(); ++si) {
      const StagePlan &sp = plan[si];
      const uint32_t bt_base = stage_bt_base[si] = (uint32_t)c.btab.size();
      for (const BatchPlan &bp : sp.batches) c.btab.push_back(make_uint2(bp.i0, bp.n_res));
      auto form = [&](const BatchPlan &bp) {
        return (bp.exhaustive ? 1 : 0) | (bp.grid_first ? 2 : 0) | ((bp.i1 - bp.i0) <= p.walk_window_max ? 4 : 0);
      };
      uint32_t covered = 0;
      size_t j = 0;
      while (j < sp.batches.size()) {
        const size_t j0 = j;
        uint32_t items = 0;
        while (j < sp.batches.size() && form(sp.batches[j]) == form(sp.batches[j0]) &&
               (j == j0 || items < std::max(kChunkMinItems, covered))) {
          items += sp.batches[j].i1 - sp.batches[j].i0;
          ++j;
        }
        chunk_batches.push_back({bt_base + (uint32_t)j0, bt_base + (uint32_t)j});
        KnnChunk ch;
        ch.stage = (int)si;
        c.knn_chunks.push_back(ch);
        covered += items;
      }
    }
  }
  const size_t n_chunks = c.knn_chunks.size(), n_kitems = c.knn_ahead ? c.items.size() : 0;
  // zeroed: colour and state first (uploaded instead when dense_init)
  const size_t z_color = zl.add(N * 4), z_state = zl.add(N * sizeof(uint4)), z_rscore = zl.add(c.res_total * 4),
               z_fbc = zl.add(c.n_batches * 4), z_err = zl.add(sizeof(int)), z_evals = zl.add(8),
               z_rank = zl.add(c.knn_ahead ? N * 4 : 0), z_kfbc = zl.add(n_chunks * 4),
               z_shadow = zl.add(c.knn_ahead ? 2 * N * sizeof(uint4) : 0), z_wctr = zl.add(c.n_batches * 4);
  // uploaded tables
  c.tab_parts.clear();
  auto T = [&](const auto &v) {
    const size_t bytes = v.size() * sizeof(v[0]);
    const size_t o = tl.add(bytes);
    c.tab_parts.push_back(RunCtx::TabPart{o, v.data(), bytes});
    return o;
  };
  const size_t t_lut = T(c.luts), t_tab = T(c.tab), t_xdiv = T(c.xdiv), t_ydiv = T(c.ydiv), t_dxt = T(c.dxt),
               t_dy2t = T(c.dy2t), t_cells = T(c.cells), t_occ = T(c.occ), t_mir = T(c.mir), t_init = T(c.init_list),
               t_btab = T(c.btab);
  // scratch
  const size_t w_res = wl.add(c.res_total * 4), w_items = wl.add(c.items.size() * 4), w_nbuf = wl.add(mb * kk * 4),
               w_ncnt = wl.add(mb * 4), w_dist = wl.add(mb * kk * 8), w_mean = wl.add(mb * 8), w_fbl = wl.add(mb * 4),
               w_result = wl.add((c.knn_ahead ? 2 : 1) * mb * sizeof(Result)), w_rcand = wl.add(rc_n * 8),
               w_knbuf = wl.add(n_kitems * kk * 4), w_kncnt = wl.add(n_kitems * 4), w_kmean = wl.add(n_kitems * 8),
               w_kfbl = wl.add(n_kitems * 4);
  CUDA_TRY(A(c.d_zero, zl.off));
  CUDA_TRY(A(c.d_tabs, tl.off));
  CUDA_TRY(A(c.d_work, wl.off));
  c.zero_bytes = zl.off;
  c.tabs_bytes = tl.off;
  uint8_t *z = c.d_zero.p, *tb = c.d_tabs.p, *wk = c.d_work.p;
  c.d_color.view(z + z_color, N);
  c.d_state.view(z + z_state, N);
  c.d_rscore.view(z + z_rscore, c.res_total);
  c.d_fbc.view(z + z_fbc, c.n_batches);
  c.d_err.view(z + z_err, 1);
  c.d_evals.view(z + z_evals, 1);
  c.d_lut.view(tb + t_lut, c.luts.size());
  c.d_tab.view(tb + t_tab, c.tab.size());
  c.d_xdiv.view(tb + t_xdiv, c.xdiv.size());
  c.d_ydiv.view(tb + t_ydiv, c.ydiv.size());
  c.d_dxt.view(tb + t_dxt, c.dxt.size());
  c.d_dy2t.view(tb + t_dy2t, c.dy2t.size());
  c.d_cells.view(tb + t_cells, c.cells.size());
  c.d_occ.view(tb + t_occ, c.occ.size());
  c.d_mir.view(tb + t_mir, c.mir.size());
  c.d_init.view(tb + t_init, c.init_list.size());
  c.d_btab.view(tb + t_btab, c.btab.size());
  c.d_rank.view(z + z_rank, c.knn_ahead ? N : 0);
  c.d_shadow.view(z + z_shadow, c.knn_ahead ? 2 * N : 0);
  c.d_wctr.view(z + z_wctr, c.n_batches);
  c.d_kfbc.view(z + z_kfbc, n_chunks);
  c.d_knbuf.view(wk + w_knbuf, n_kitems * kk);
  c.d_kncnt.view(wk + w_kncnt, n_kitems);
  c.d_kmean.view(wk + w_kmean, n_kitems);
  c.d_kfbl.view(wk + w_kfbl, n_kitems);
  c.d_res.view(wk + w_res, c.res_total);
  c.d_items.view(wk + w_items, c.items.size());
  c.d_nbuf.view(wk + w_nbuf, mb * kk);
  c.d_ncnt.view(wk + w_ncnt, mb);
  c.d_dist.view(wk + w_dist, mb * kk);
  c.d_mean.view(wk + w_mean, mb);
  c.d_fbl.view(wk + w_fbl, mb);
  c.d_result.view(wk + w_result, (c.knn_ahead ? 2 : 1) * mb);
  c.d_rcand.view(wk + w_rcand, rc_n);
  const std::vector<int32_t> &tab = c.tab;

  SessionDev &sd = c.sd;
  sd = SessionDev{};
  sd.levels = s->levels.p;
  sd.plevels = s->plevels.p;
  sd.pguides = s->pguides.p;
  sd.ppitch = s->ppitch;
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
  sd.xdiv = c.d_xdiv.p;
  sd.ydiv = c.d_ydiv.p;
  sd.xdiv_off = xo;
  sd.ydiv_off = yo;
  sd.dxt = c.d_dxt.p;
  sd.dy2t = c.d_dy2t.p;
  sd.dtab_r = R;
  sd.color = c.d_color.p;
  sd.state = c.d_state.p;
  sd.occ = c.d_occ.p;
  sd.mir = c.d_mir.p;
  sd.resolved = c.d_res.p;
  sd.rscore = c.d_rscore.p;
  sd.knn_tab = c.d_tab.p;
  sd.knn_tab_n = (uint32_t)tab.size();
  sd.err = c.d_err.p;
  sd.evals = c.d_evals.p;
  sd.W = W;
  sd.H = H;
  sd.exact_sum = exact_sum_ok(W, H, k) ? 1 : 0;
  if (sd.exact_sum) {
    const uint32_t M = std::max(W, H);
    auto lg2 = [](uint32_t v) {
      uint32_t l = 0;
      while ((1u << l) < v) ++l;
      return l;
    };
    sd.exact_sx = 2 * (lg2(M) - lg2(W));
    sd.exact_sy = 2 * (lg2(M) - lg2(H));
    sd.exact_qe = -2 * (int32_t)lg2(M);
    sd.exact_q = std::ldexp(1.0, sd.exact_qe);
  }
  sd.wpr = wpr;
  sd.tiling = p.tiling ? 1 : 0;
  sd.x_l = x_l;
  sd.x_r = (int32_t)W - x_l;
  sd.y_b = y_b;
  sd.y_t = (int32_t)H - y_b;
  sd.k = k;
  sd.m = m;
  sd.cells = c.d_cells.p;
  sd.cox = c.cox;
  sd.coy = c.coy;
  sd.cgw = c.cgw;
  sd.cgh = c.cgh;
  sd.rank = c.knn_ahead ? c.d_rank.p : nullptr;
  sd.shadow = c.knn_ahead ? c.d_shadow.p : nullptr;
  c.pend = false;

  // ---- the steps ----
  size_t fb_index = 0;
  uint32_t bidx = 0;
  c.rc_step.assign(plan.size(), -1);
  for (size_t si = 0; si < plan.size(); ++si) {
    const StagePlan &sp = plan[si];
    c.overall_total += sp.n_items;
    const size_t first = c.steps.size();
    if (c.rc_ahead && !sp.batches.empty()) c.rc_step[si] = (int)first;
    Step pending;
    pending.stage = (int)si;
    if (sp.level_switch) {
      pending.ls = true;
      pending.ls_level = sp.level;
      pending.ls_n_res = sp.n_res_start;
    }
    StageDev sdv{};
    sdv.level = sp.level;
    sdv.slow_lut = sp.slow_lut ? 1 : 0;
    sdv.lut = c.d_lut.p + si * 512;
    sdv.opaque = (s->opaque && !sp.slow_lut && c.luts[si * 512] == 0.0f && c.luts[si * 512 + 256] == 0.0f) ? 1 : 0;
    sdv.stage_seed = sp.seed;
    sdv.items = c.d_items.p + sp.items_off;
    sdv.redo = sp.redo;
    // random candidates in chunks of whole batches that fit the buffer
    size_t bi = 0;
    while (bi < sp.batches.size()) {
      size_t bj = bi;
      const uint32_t c0 = sp.batches[bi].i0;
      while (bj < sp.batches.size() && (bj == bi || c.rc_ahead || sp.batches[bj].i1 - c0 <= rc_items)) ++bj;
      const uint32_t c1 = sp.batches[bj - 1].i1;
      StageDev chunk = sdv;
      chunk.items = sdv.items + c0;
      chunk.n_items = c1 - c0;
      chunk.stage_seed = sp.seed + c0;  // item i's stream is seeded with stage_seed + i + 1
      chunk.rcand = c.d_rcand.p + (c.rc_ahead ? (size_t)sp.items_off * m : 0);
      chunk.redo = sp.redo > c0 ? sp.redo - c0 : 0;
      pending.rc = true;
      pending.rc_st = chunk;
      chunk.stage_seed = sp.seed;  // resolve_at_random uses the stage seed itself
      for (size_t bk = bi; bk < bj; ++bk) {
        const BatchPlan &bp = sp.batches[bk];
        Step stp = pending;
        pending = Step{};
        pending.stage = (int)si;
        stp.batch = true;
        stp.st = chunk;
        BatchDev &bd = stp.bd;
        bd.i0 = bp.i0 - c0;
        bd.i1 = bp.i1 - c0;
        bd.n_res = bp.n_res;
        bd.append_from = bp.append_from - c0;
        bd.nbuf = c.d_nbuf.p;
        bd.ncnt = c.d_ncnt.p;
        bd.fb_list = c.d_fbl.p;
        bd.fb_count = c.d_fbc.p + fb_index++;
        bd.dist = c.d_dist.p;
        bd.mean = c.d_mean.p;
        bd.res = c.d_result.p;
        stp.n = bp.i1 - bp.i0;
        stp.stage_i0 = bp.i0;
        if (c.want_knn_ahead) bd.work_ctr = c.d_wctr.p + bidx;  // plain runs (ts_session_run) only
        stp.bidx = bidx++;
        if (c.knn_ahead) {  // the chunk's lists, made ahead on the k-NN stream
          const size_t g0 = (size_t)sp.items_off + bp.i0;
          bd.nbuf = c.d_knbuf.p + g0 * kk;
          bd.ncnt = c.d_kncnt.p + g0;
          bd.mean = c.d_kmean.p + g0;
        }
        stp.exhaustive = bp.exhaustive;
        bd.grid_first = bp.grid_first ? 1 : 0;
        bd.walk_window = (bp.i1 - bp.i0) <= p.walk_window_max ? 1 : 0;
        // a batch of new items only: none of them is in the tree, so no item
        // reads another's pixel, state or bit, and each commits as it resolves
        bd.fused_commit = bp.i0 >= sp.redo ? 1 : 0;
        if (stp.n <= p.team_max_batch)
          stp.resolve = (stp.n <= p.team_full_max_batch && team_full_fits(k, m)) ? kPhaseTeamFull : kPhaseTeamPart;
        else
          stp.resolve = kPhaseResolve;
        c.steps.push_back(stp);
      }
      bi = bj;
    }
    if (c.steps.size() == first) c.steps.push_back(pending);  // a stage without batches
    c.steps.back().stage_end = true;
  }
  // ---- the k-NN chunks ----
  if (c.knn_ahead) {
    std::vector<size_t> step_of(c.btab.size(), 0);
    for (size_t t = 0; t < c.steps.size(); ++t)
      if (c.steps[t].batch) step_of[c.steps[t].bidx] = t;
    for (size_t q = 0; q < c.knn_chunks.size(); ++q) {
      KnnChunk &ch = c.knn_chunks[q];
      const StagePlan &sp = plan[ch.stage];
      const uint32_t bt0 = chunk_batches[q].first, bt1 = chunk_batches[q].second;
      c.steps[step_of[bt0]].knn_wait = (int)q;
      // the chunk's batches as indices into the stage's list
      const size_t sb0 = bt0 - stage_bt_base[ch.stage], sb1 = bt1 - stage_bt_base[ch.stage];
      const BatchPlan &b0 = sp.batches[sb0], &bl = sp.batches[sb1 - 1];
      ch.st = StageDev{};
      ch.st.level = sp.level;
      ch.st.stage_seed = sp.seed;
      ch.st.items = c.d_items.p + sp.items_off;
      ch.st.n_items = sp.n_items;
      ch.st.redo = sp.redo;
      BatchDev &kb = ch.b;
      kb = BatchDev{};
      kb.i0 = b0.i0;
      kb.i1 = bl.i1;
      kb.n_res = bl.n_res;  // the largest tree of the chunk (sizes the exhaustive key buffer)
      kb.append_from = kb.i1;
      const size_t g0 = (size_t)sp.items_off + kb.i0;
      kb.nbuf = c.d_knbuf.p + g0 * kk;
      kb.ncnt = c.d_kncnt.p + g0;
      kb.mean = c.d_kmean.p + g0;
      kb.fb_list = c.d_kfbl.p + g0;
      kb.fb_count = c.d_kfbc.p + q;
      kb.grid_first = b0.grid_first ? 1 : 0;
      kb.walk_window = (b0.i1 - b0.i0) <= p.walk_window_max ? 1 : 0;
      kb.btab = c.d_btab.p + bt0;
      kb.nbt = bt1 - bt0;
      ch.all_exhaustive = b0.exhaustive;
      ch.a0 = std::max(kb.i0, sp.redo);
      ch.a1 = std::max(kb.i1, sp.redo);
      ch.pos0 = sp.n_res_start + (ch.a0 - sp.redo);
      for (size_t j = sb0; j < sb1; ++j)
        if (sp.batches[j].n_res == 0) ch.nomir_end = std::max(ch.nomir_end, sp.batches[j].i1);
    }
  }
}

// Uploads of the initial state, enqueued on st.
// The session's tables in a pinned block laid out as the device's table
// arena (ready for one copy); the batched form makes it on its planning
// threads, the other paths in run_upload.
void run_stage_tables(RunCtx &c) {
  if (c.ptab.p) return;
  CUDA_TRY(c.ptab.alloc(c.tabs_bytes));
  for (const RunCtx::TabPart &t : c.tab_parts)
    if (t.bytes) memcpy(c.ptab.p + t.off, t.src, t.bytes);
}

// Uploads of the initial state, enqueued on st: one zero fill, one copy of
// the tables (colour and state too when dense_init), the random-init
// pixels; the items unless the caller sends them (items_async).
void run_upload(RunCtx &c, cudaStream_t st) {
  run_stage_tables(c);
  if (c.dense_init) {
    const size_t cs = (size_t)((uint8_t *)c.d_rscore.p - c.d_zero.p);
    CUDA_TRY(cudaMemcpyAsync(c.d_color.p, c.color.data(), c.N * 4, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(c.d_state.p, c.state.data(), c.N * sizeof(uint4), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemsetAsync(c.d_zero.p + cs, 0, c.zero_bytes - cs, st));
  } else {
    CUDA_TRY(cudaMemsetAsync(c.d_zero.p, 0, c.zero_bytes, st));
  }
  CUDA_TRY(cudaMemcpyAsync(c.d_tabs.p, c.ptab.p, c.tabs_bytes, cudaMemcpyHostToDevice, st));
  if (c.dense_init) {
    if (c.locked) CUDA_TRY(cudaMemcpyAsync(c.d_res.p, c.resolved.data(), c.locked * 4, cudaMemcpyHostToDevice, st));
  } else if (!c.init_list.empty()) {
    // the resolved list starts with the random-init pixels, in list order
    launch_scatter_init(c.d_init.p, (uint32_t)(c.init_list.size() / 6), c.d_color.p, c.d_state.p, c.d_res.p, st);
    ++c.launches;
  }
  if (!c.items_async && !c.items.empty() && c.picked_stages == c.plan.size())
    CUDA_TRY(cudaMemcpyAsync(c.d_items.p, c.items.data(), c.items.size() * 4, cudaMemcpyHostToDevice, st));
}

// Whether the commit of step `stp` can be left to the first k-NN launch of
// `next`, the following step of the same stage: stp holds only redo items
// (nothing is appended to the resolved list, the bitmap or the cell
// counts), and next starts with a walk or an exhaustive k-NN launch, not
// the fused small-step kernel, which reads colours.
bool can_defer_commit(const RunCtx &c, const Step &stp, const Step *next) {
  if (!stp.batch || stp.bd.fused_commit || c.k == 0 || stp.bd.append_from < stp.bd.i1) return false;
  if (!next || !next->batch || next->ls || next->stage != stp.stage) return false;
  return !(next->exhaustive && next->resolve == kPhaseTeamFull && team_full_fits(c.sd.k, c.sd.m));
}

// k-NN ahead: the chunks of stage `stage` on the k-NN stream kst, once its
// items are up: each chunk's tree entries, then its neighbour lists and
// means, then its event.
void run_enqueue_knn(RunCtx &c, cudaStream_t kst, LaunchTimer &lt, int stage) {
  const SessionDev &sd = c.sd;
  const cudaStream_t main_st = lt.st;
  lt.st = kst;
  for (size_t q = 0; q < c.knn_chunks.size(); ++q) {
    const KnnChunk &ch = c.knn_chunks[q];
    if (ch.stage != stage) continue;
    lt.items = ch.b.i1 - ch.b.i0;
    if (ch.a1 > ch.a0) {
      lt.run(TS_KERNEL_COMMIT, [&] { launch_tree_append(sd, ch.st, ch.a0, ch.a1, ch.pos0, ch.nomir_end, kst); });
      ++c.launches;
    }
    if (ch.all_exhaustive) {
      lt.run(TS_KERNEL_KNN_EXHAUSTIVE, [&] { launch_knn_exhaustive(sd, ch.st, ch.b, true, kst, PendingCommit{}); });
      ++c.launches;
    } else {
      lt.run(TS_KERNEL_KNN_WALK, [&] { launch_knn_walk(sd, ch.st, ch.b, kst, PendingCommit{}); });
      lt.run(TS_KERNEL_KNN_EXHAUSTIVE, [&] { launch_knn_exhaustive(sd, ch.st, ch.b, false, kst, PendingCommit{}); });
      c.launches += 2;
    }
    CUDA_TRY(cudaEventCreateWithFlags(&c.knn_ev[q].e, cudaEventDisableTiming));
    CUDA_TRY(cudaEventRecord(c.knn_ev[q].e, kst));
  }
  lt.st = main_st;
}

// k-NN ahead: the commit a batch step left to the next step, as its own
// launch (before a level switch, at a stage's end).
void commit_pending(RunCtx &c, cudaStream_t st, LaunchTimer &lt) {
  if (!c.pend) return;
  lt.items = c.pend_n;
  lt.run(TS_KERNEL_COMMIT, [&] { launch_commit(c.sd, c.pend_st, c.pend_bd, st); });
  ++c.launches;
  c.pend = false;
}

// k-NN ahead: step t on the main stream.  Its neighbour lists come from the
// k-NN stream (the step waits for its chunk's event first), so a batch step
// is its resolve launch alone: a batch of new items commits inside it; any
// other batch keeps its results and tags their pixels, and the next batch
// step's launch commits them while it runs, its readers taking those pixels'
// batch-start values from the kept results.
void enqueue_step_ahead(RunCtx &c, size_t t, cudaStream_t st, LaunchTimer &lt) {
  const SessionDev &sd = c.sd;
  const Step &stp = c.steps[t];
  if (c.pend && (stp.ls || !stp.batch || stp.stage != c.pend_stage)) commit_pending(c, st, lt);
  if (stp.knn_wait >= 0) {
    const uint32_t items = lt.items;
    lt.items = stp.n;
    lt.run(TS_KERNEL_KNN_WAIT, [&] { CUDA_TRY(cudaStreamWaitEvent(st, c.knn_ev[stp.knn_wait].e, 0)); });
    lt.items = items;
  }
  if (stp.ls) {
    lt.run(TS_KERNEL_LEVEL_SWITCH, [&] { launch_level_switch(sd, stp.ls_level, stp.ls_n_res, st); });
    ++c.launches;
  }
  if (stp.rc) {
    if (c.rc_ahead) {
      CUDA_TRY(cudaStreamWaitEvent(st, c.rc_ev[stp.stage].e, 0));
    } else {
      lt.run(TS_KERNEL_RANDOM_CANDIDATES, [&] { launch_random_candidates(sd, stp.rc_st, st); });
      ++c.launches;
    }
  }
  if (!stp.batch) return;
  BatchDev bd = stp.bd;
  PendingCommit pc{};
  if (c.pend) {
    pc.st = c.pend_st;
    pc.b = c.pend_bd;
    pc.n = c.pend_n;
    bd.prev_tag = c.pend_bd.defer_tag;
  }
  if (!bd.fused_commit) {
    bd.defer_tag = (uint32_t)t + 1;
    bd.res = c.d_result.p + (c.defer_parity ? c.max_batch_items : 0);
    c.defer_parity ^= 1u;
  }
  lt.items = stp.n;
  if (stp.resolve == kPhaseResolve)
    lt.run(TS_KERNEL_RESOLVE, [&] { launch_resolve(sd, stp.st, bd, st, pc); });
  else
    lt.run(TS_KERNEL_RESOLVE, [&] { launch_resolve_team(sd, stp.st, bd, stp.resolve == kPhaseTeamFull, st, pc); });
  c.launches += 1;
  c.pend = !bd.fused_commit;
  if (c.pend) {
    c.pend_st = stp.st;
    c.pend_bd = bd;
    c.pend_bd.prev_tag = 0;
    c.pend_n = stp.n;
    c.pend_stage = stp.stage;
  }
}

// The launches of one step of one session, with the single-session
// kernels (parameters by value).  pending: an earlier step whose commit
// this step's first k-NN launch makes; defer: leave this step's commit to
// the next step (can_defer_commit).
void enqueue_step(RunCtx &c, const Step &stp, cudaStream_t st, LaunchTimer &lt, const Step *pending = nullptr,
                  bool defer = false) {
  const SessionDev &sd = c.sd;
  PendingCommit pc{};
  if (pending) {
    pc.st = pending->st;
    pc.b = pending->bd;
    pc.n = pending->bd.i1 - pending->bd.i0;
  }
  if (stp.ls) {
    lt.run(TS_KERNEL_LEVEL_SWITCH, [&] { launch_level_switch(sd, stp.ls_level, stp.ls_n_res, st); });
    ++c.launches;
  }
  if (stp.rc) {
    if (c.rc_ahead) {
      CUDA_TRY(cudaStreamWaitEvent(st, c.rc_ev[stp.stage].e, 0));
    } else {
      lt.run(TS_KERNEL_RANDOM_CANDIDATES, [&] { launch_random_candidates(sd, stp.rc_st, st); });
      ++c.launches;
    }
  }
  if (stp.batch) {
    lt.items = stp.n;
    if (c.k > 0 && stp.exhaustive && stp.resolve == kPhaseTeamFull && team_full_fits(sd.k, sd.m)) {
      // small batch, exhaustive k-NN: neighbours, mean and resolve in one launch
      lt.run(TS_KERNEL_RESOLVE, [&] { launch_step_team_full(sd, stp.st, stp.bd, st); });
      c.launches += 1;
      if (!stp.bd.fused_commit) {
        lt.run(TS_KERNEL_COMMIT, [&] { launch_commit(sd, stp.st, stp.bd, st); });
        c.launches += 1;
      }
      return;
    }
    if (c.k > 0) {
      if (stp.exhaustive) {
        lt.run(TS_KERNEL_KNN_EXHAUSTIVE, [&] { launch_knn_exhaustive(sd, stp.st, stp.bd, true, st, pc); });
        ++c.launches;
      } else {
        lt.run(TS_KERNEL_KNN_WALK, [&] { launch_knn_walk(sd, stp.st, stp.bd, st, pc); });
        lt.run(TS_KERNEL_KNN_EXHAUSTIVE, [&] { launch_knn_exhaustive(sd, stp.st, stp.bd, false, st); });
        c.launches += 2;
      }
    }
    // the exhaustive k-NN over a whole batch computes the mean itself, and so
    // do the walk and the fallback k-NN for sessions whose sums are exact
    if (c.k > 0 && !stp.exhaustive && !sd.exact_sum) {
      lt.run(TS_KERNEL_MEAN, [&] { launch_mean(sd, stp.st, stp.bd, st); });
      ++c.launches;
    }
    if (stp.resolve == kPhaseResolve)
      lt.run(TS_KERNEL_RESOLVE, [&] { launch_resolve(sd, stp.st, stp.bd, st); });
    else
      lt.run(TS_KERNEL_RESOLVE, [&] { launch_resolve_team(sd, stp.st, stp.bd, stp.resolve == kPhaseTeamFull, st); });
    c.launches += 1;
    if (!stp.bd.fused_commit && !defer) {
      lt.run(TS_KERNEL_COMMIT, [&] { launch_commit(sd, stp.st, stp.bd, st); });
      c.launches += 1;
    }
  }
}

// The plain path: one session's launches, step by step (only those of
// stage `stage` when it is not negative).
void run_enqueue_plain(RunCtx &c, cudaStream_t st, LaunchTimer &lt, ts_progress_fn progress, void *user,
                       int stage = -1) {
  uint64_t overall_current = 0;
  for (const StagePlan &sp : c.plan)
    if (stage >= 0 && (&sp - c.plan.data()) < stage) overall_current += sp.n_items;
  std::vector<uint8_t> prog_img;
  const Step *pending = nullptr;  // a step whose commit the next step's k-NN launch makes
  for (size_t i = 0; i < c.steps.size(); ++i) {
    const Step &stp = c.steps[i];
    if (stage >= 0 && stp.stage != stage) continue;
    const StagePlan &sp = c.plan[stp.stage];
    lt.stage = sp.p_stage;
    lt.items = sp.n_items;
    if (c.knn_ahead) {
      enqueue_step_ahead(c, i, st, lt);
      if (stp.stage_end) commit_pending(c, st, lt);  // nothing waits across a stage's end
    } else {
      const bool defer = can_defer_commit(c, stp, i + 1 < c.steps.size() ? &c.steps[i + 1] : nullptr);
      enqueue_step(c, stp, st, lt, pending, defer);
      pending = defer ? &stp : nullptr;
    }
    if (stp.batch) {
      ++c.batches;
      c.resolves += stp.n;
    }
    if (stp.stage_end) {
      CUDA_TRY(cudaGetLastError());
      overall_current += sp.n_items;
      if (progress) {
        prog_img.resize(c.N * 4);
        CUDA_TRY(cudaMemcpyAsync(prog_img.data(), c.d_color.p, c.N * 4, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        ts_progress up;
        up.image = prog_img.data();
        up.width = c.W;
        up.height = c.H;
        up.total_current = overall_current;
        up.total_total = c.overall_total;
        up.stage_current = sp.n_items;
        up.stage_total = sp.n_items;
        progress(&up, user);
      }
    }
  }
}

// Device-to-host copies of the results, enqueued on st.
void run_readback(RunCtx &c, cudaStream_t st) {
  ts_generated *g = c.g.get();
  c.col.resize(c.N);
  c.stv.resize(c.N);
  g->resolved.resize(c.res_total);
  g->scores.resize(c.res_total);
  CUDA_TRY(cudaMemcpyAsync(&c.evals, c.d_evals.p, sizeof(c.evals), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(c.col.data(), c.d_color.p, c.N * 4, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(c.stv.data(), c.d_state.p, c.N * sizeof(uint4), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(g->resolved.data(), c.d_res.p, c.res_total * 4, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(g->scores.data(), c.d_rscore.p, c.res_total * 4, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(&c.derr, c.d_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
}

// After the stream has drained: device errors and the host-side result.
void run_finish(RunCtx &c) {
  if (c.derr == kDevErrIndex) throw Failure{TS_ERR_INDEX, "a map id points past the non-ignored examples"};
  if (c.derr == kDevErrNoSample) throw Failure{TS_ERR_NO_VALID_SAMPLE, "no valid sample location found"};
  if (c.derr == kDevErrLimit) throw Failure{TS_ERR_LIMIT, "too many equidistant neighbours for the k-NN buffer"};
  if (c.derr) throw Failure{TS_ERR_CUDA, "device reported error " + std::to_string(c.derr)};
  ts_generated *g = c.g.get();
  const size_t N = c.N;
  g->W = c.W;
  g->H = c.H;
  g->image.resize(N * 4);
  memcpy(g->image.data(), c.col.data(), N * 4);
  g->state = std::move(c.stv);  // the coordinate and id maps are made on first use
  g->in_dims.clear();
  for (const Image &im : c.s->bottoms) {
    g->in_dims.push_back(im.w);
    g->in_dims.push_back(im.h);
  }
  g->stats.resolves = c.resolves;
  g->stats.batches = c.batches;
  g->stats.stages = c.plan.size();
  g->stats.kernel_launches = c.launches;
  g->stats.cost_evals = c.evals;
}

struct EventPair {
  cudaEvent_t a = nullptr, b = nullptr;
  ~EventPair() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
  void create() {
    CUDA_TRY(cudaEventCreate(&a));
    CUDA_TRY(cudaEventCreate(&b));
  }
  float ms() const {
    float v = 0.0f;
    CUDA_TRY(cudaEventElapsedTime(&v, a, b));
    return v;
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
  StreamGuard sg;  // declared first: the run's pool buffers are freed on it before it goes
  StreamGuard rg;  // side stream of the random candidates made ahead
  StreamGuard kg;  // k-NN stream (knn_ahead)
  // the items go up stage by stage from pinned memory, so that the device
  // runs a stage while the host picks the next one
  PinnedBuf<uint32_t> pitems;
  RunCtx c;
  // The pick chain (pick_random_unresolved, ms.rs:380-389) on its own host
  // thread from the plan on, stage after stage, so that a stage's picks
  // never wait behind the launches of the one before; the launching thread
  // takes each stage once it is picked.  Declared after c: it is joined
  // before c goes.
  struct PickThread {
    std::thread th;
    std::mutex mu;
    std::condition_variable cv;
    size_t done = 0;  // stages picked
    bool failed = false;
    Failure fail{};
    std::atomic<bool> stop{false};
    ~PickThread() {
      stop = true;
      if (th.joinable()) th.join();
    }
  } pk;
  try {
    CUDA_TRY(cudaSetDevice(s->prm.device));
    keep_pool(s->prm.device);
    // the resolve chain on the highest priority, the work made ahead on the
    // side streams on the lowest: blocks of the chain's next launch take the
    // first free SMs
    int prio_low = 0, prio_high = 0;
    CUDA_TRY(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
    CUDA_TRY(cudaStreamCreateWithPriority(&sg.s, cudaStreamNonBlocking, prio_high));
    const cudaStream_t st = sg.s;
    if (s->ready.e) CUDA_TRY(cudaStreamWaitEvent(st, s->ready.e, 0));
    auto t = std::chrono::steady_clock::now();
    auto lap = [&]() {
      const auto n = std::chrono::steady_clock::now();
      const double ms = std::chrono::duration<double, std::milli>(n - t).count();
      t = n;
      return ms;
    };
    c.want_rc_ahead = true;
    c.want_knn_ahead = true;
    c.parallel_picks = true;
    run_plan(s, c);
    c.items_async = true;  // each stage's items go up once the pick thread has them
    pk.th = std::thread([&c, &pk] {
      try {
        for (size_t q = 0; q < c.plan.size() && !pk.stop; ++q) {
          run_pick(c);
          std::lock_guard<std::mutex> lk(pk.mu);
          pk.done = q + 1;
          pk.cv.notify_one();
        }
      } catch (const Failure &f) {
        std::lock_guard<std::mutex> lk(pk.mu);
        pk.failed = true;
        pk.fail = f;
        pk.cv.notify_one();
      } catch (...) {
        std::lock_guard<std::mutex> lk(pk.mu);
        pk.failed = true;
        pk.fail = Failure{TS_ERR_OUT_OF_MEMORY, "out of host memory"};
        pk.cv.notify_one();
      }
    });
    const double plan_ms = lap();
    run_alloc(c, st);
    CUDA_TRY(pitems.alloc(c.items.size()));
    run_stage_tables(c);  // its pinned block too, before the device clock starts
    const double alloc_ms = lap();
    EventPair ev, ev_up, ev_rb;
    ev.create();
    ev_up.create();
    ev_rb.create();
    CUDA_TRY(cudaEventRecord(ev.a, st));
    run_upload(c, st);
    if (c.knn_ahead) {
      // the initial tree's positions; the k-NN stream starts after them
      launch_rank_init(c.sd, (uint32_t)c.locked, st);
      if (c.locked) ++c.launches;
      CUDA_TRY(side_stream(s->prm.device, prio_low, &kg.s));
      c.knn_ev.resize(c.knn_chunks.size());
      c.items_ev.resize(c.plan.size());
    }
    CUDA_TRY(cudaEventRecord(ev_up.a, st));
    LaunchTimer lt;
    lt.on = s->prm.profile;
    if (c.rc_ahead) {
      // every stage's random candidates depend on the examples and the
      // stage plan only: a side stream makes them while the first stages run
      if (c.knn_ahead)
        CUDA_TRY(side_stream(s->prm.device, prio_low, &rg.s));
      else
        CUDA_TRY(cudaStreamCreateWithPriority(&rg.s, cudaStreamNonBlocking, prio_low));
      EventHandle fork;
      CUDA_TRY(cudaEventCreateWithFlags(&fork.e, cudaEventDisableTiming));
      CUDA_TRY(cudaEventRecord(fork.e, st));
      CUDA_TRY(cudaStreamWaitEvent(rg.s, fork.e, 0));
      c.rc_ev.resize(c.plan.size());
      lt.st = rg.s;
      for (size_t q = 0; q < c.plan.size(); ++q) {
        if (c.rc_step[q] < 0) continue;
        const Step &stp = c.steps[c.rc_step[q]];
        lt.stage = c.plan[q].p_stage;
        lt.items = stp.rc_st.n_items;
        lt.run(TS_KERNEL_RANDOM_CANDIDATES, [&] { launch_random_candidates(c.sd, stp.rc_st, rg.s); });
        ++c.launches;
        CUDA_TRY(cudaEventCreateWithFlags(&c.rc_ev[q].e, cudaEventDisableTiming));
        CUDA_TRY(cudaEventRecord(c.rc_ev[q].e, rg.s));
      }
    }
    lt.st = st;
    double pick_ms = 0.0;
    for (size_t si = 0; si < c.plan.size(); ++si) {
      const auto p0 = std::chrono::steady_clock::now();
      {
        std::unique_lock<std::mutex> lk(pk.mu);
        pk.cv.wait(lk, [&] { return pk.done > si || pk.failed; });
        if (pk.done <= si) throw pk.fail;
      }
      pick_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - p0).count();
      const StagePlan &sp = c.plan[si];
      if (sp.n_items) {
        memcpy(pitems.p + sp.items_off, c.items.data() + sp.items_off, (size_t)sp.n_items * 4);
        CUDA_TRY(cudaMemcpyAsync(c.d_items.p + sp.items_off, pitems.p + sp.items_off, (size_t)sp.n_items * 4,
                                 cudaMemcpyHostToDevice, st));
      }
      if (c.knn_ahead) {
        // the stage's neighbour lists on the k-NN stream, from its items on
        CUDA_TRY(cudaEventCreateWithFlags(&c.items_ev[si].e, cudaEventDisableTiming));
        CUDA_TRY(cudaEventRecord(c.items_ev[si].e, st));
        CUDA_TRY(cudaStreamWaitEvent(kg.s, c.items_ev[si].e, 0));
        lt.stage = sp.p_stage;
        run_enqueue_knn(c, kg.s, lt, (int)si);
      }
      run_enqueue_plain(c, st, lt, progress, user, (int)si);
    }
    CUDA_TRY(cudaEventRecord(ev_rb.a, st));
    run_readback(c, st);
    CUDA_TRY(cudaEventRecord(ev.b, st));
    const double enqueue_ms = lap();
    CUDA_TRY(cudaStreamSynchronize(st));
    const double wait_ms = lap();
    run_finish(c);
    c.g->stats.host_plan_ms = plan_ms;
    c.g->stats.host_alloc_ms = alloc_ms;
    c.g->stats.host_enqueue_ms = enqueue_ms;
    c.g->stats.host_pick_ms = pick_ms;
    c.g->stats.host_launch_ms = enqueue_ms - pick_ms;
    c.g->stats.knn_chunks = c.knn_chunks.size();
    c.g->stats.host_wait_ms = wait_ms;
    c.g->stats.host_finish_ms = lap();
    c.g->stats.gpu_ms = ev.ms();
    {
      float up = 0.0f, rb = 0.0f;
      CUDA_TRY(cudaEventElapsedTime(&up, ev.a, ev_up.a));
      CUDA_TRY(cudaEventElapsedTime(&rb, ev_rb.a, ev.b));
      c.g->stats.upload_ms = up;
      c.g->stats.readback_ms = rb;
    }
    lt.collect(c.g->stats, c.g->launches);
  } catch (const Failure &f) {
    // nothing of the run may be in flight when its buffers go
    if (kg.s) cudaStreamSynchronize(kg.s);
    if (rg.s) cudaStreamSynchronize(rg.s);
    if (sg.s) cudaStreamSynchronize(sg.s);
    s->err = f.msg;
    return f.status;
  }
  c.g->stats.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_wall0).count();
  *out = c.g.release();
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
  const_cast<ts_generated *>(g)->ensure_maps();  // made on first use (the object is not shared between threads)
  memcpy(out, g->coord.data(), g->coord.size() * 4);
  return TS_OK;
}
int ts_generated_id_map(const ts_generated *g, uint32_t *out) {
  if (!g || !out) return TS_ERR_NULL;
  const_cast<ts_generated *>(g)->ensure_maps();
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

// ---------------------------------------------------------------------------
// Batched form: every session's steps advance together, one launch per phase
// of a global step carrying one segment per session that has work in it.
// ---------------------------------------------------------------------------
struct ts_batch {
  int device = 0;
  std::vector<ts_session *> sessions;
  bool graph = false;
  bool profile = false;
  uint32_t plan_threads = 0;
  uint32_t team_max_items = 2048, team_full_max_items = 256;
  ts_batch_stats stats{};
  std::string err;
};

namespace {

// Units a session's step hands to a phase (0 = no segment).
uint32_t phase_units(const Step &stp, const RunCtx &c, int phase) {
  const bool knn = stp.batch && c.k > 0;
  switch (phase) {
    case kPhaseLevelSwitch: return stp.ls ? stp.ls_n_res : 0;
    case kPhaseRandom: return (stp.rc && c.m > 0 && !c.rc_ahead) ? stp.rc_st.n_items : 0;
    case kPhaseWalk: return (knn && !stp.exhaustive) ? stp.n : 0;
    case kPhaseExhaustive: return (knn && stp.exhaustive) ? stp.n : 0;
    case kPhaseMean: return (knn && !stp.exhaustive && !c.sd.exact_sum) ? stp.n : 0;
    case kPhaseResolve:
    case kPhaseTeamPart:
    case kPhaseTeamFull: return (stp.batch && stp.resolve == phase) ? stp.n : 0;
    case kPhaseCommit: return (stp.batch && !stp.bd.fused_commit) ? stp.n : 0;
    default: return 0;
  }
}

// Grid bound per segment of the grid-stride phases: the exhaustive k-NN's
// fallback segments usually hold few items (the walk finds k points for
// most), so they get few blocks.
uint32_t phase_cap(const Step &stp, int phase) {
  switch (phase) {
    case kPhaseExhaustive: return 608u;
    case kPhaseTeamPart:
    case kPhaseTeamFull: return 152u * 16u;
    default: return 0;
  }
}

struct PlannedLaunch {
  int phase;
  uint32_t seg0, n_segs, blocks;
  size_t smem;
  uint32_t fb0 = 0, n_fb = 0, pool_block0 = 0;  // exhaustive k-NN: fallback lists drained by a block pool
  uint32_t n_lean = 0, lean_blocks = 0;  // resolve: leading segments of sessions without guides
  uint32_t key_cap = 0;                  // exhaustive: keys in shared memory (largest over the steps)
  int wait_rc = -1;  // first wait for the side stream's random candidates up to this launch of them
  int wait_items = -1;  // first wait for the side stream's item uploads up to this part
};

// Blocks of the exhaustive k-NN's fallback pool (three 64 KB CTAs per SM).
constexpr uint32_t kFallbackPool = 152u * 3u;

}  // namespace

extern "C" {

ts_batch *ts_batch_new(int32_t device) {
  ts_batch *b = new (std::nothrow) ts_batch();
  if (b) b->device = device;
  return b;
}
void ts_batch_free(ts_batch *b) {
  if (!b) return;
  for (ts_session *s : b->sessions) delete s;
  delete b;
}
const char *ts_batch_last_error(const ts_batch *b) { return b ? b->err.c_str() : "null batch"; }
uint64_t ts_batch_size(const ts_batch *b) { return b ? b->sessions.size() : 0; }
int ts_batch_use_graph(ts_batch *b, int32_t on) {
  if (!b) return TS_ERR_NULL;
  b->graph = on != 0;
  return TS_OK;
}
int ts_batch_profile(ts_batch *b, int32_t on) {
  if (!b) return TS_ERR_NULL;
  b->profile = on != 0;
  return TS_OK;
}
int ts_batch_resolve_team(ts_batch *b, uint32_t team_max_items, uint32_t full_max_items) {
  if (!b) return TS_ERR_NULL;
  b->team_max_items = team_max_items;
  b->team_full_max_items = full_max_items;
  return TS_OK;
}
int ts_batch_tuning(ts_batch *b, const ts_tuning *t) {
  if (!b || !t) return TS_ERR_NULL;
  b->team_max_items = t->team_max_items;
  b->team_full_max_items = t->team_full_max_items;
  return TS_OK;
}
int ts_batch_plan_threads(ts_batch *b, uint32_t n) {
  if (!b) return TS_ERR_NULL;
  b->plan_threads = n;
  return TS_OK;
}
void ts_batch_stats_get(const ts_batch *b, ts_batch_stats *out) {
  if (b && out) *out = b->stats;
}

int ts_batch_add(ts_batch *b, ts_session *s) {
  if (!b || !s) return TS_ERR_NULL;
  if (s->consumed) {
    b->err = "session already consumed";
    return TS_ERR_STATE;
  }
  if (s->prm.device != b->device) {
    b->err = "session device " + std::to_string(s->prm.device) + " differs from the batch's " +
             std::to_string(b->device);
    return TS_ERR_STATE;
  }
  // the batch owns the session's device data from here on; the caller's
  // handle stays valid but consumed
  ts_session *own = new (std::nothrow) ts_session();
  if (!own) return TS_ERR_OUT_OF_MEMORY;
  *own = std::move(*s);
  s->consumed = true;
  s->err = "session handed to a batch";
  b->sessions.push_back(own);
  return TS_OK;
}

int ts_batch_run(ts_batch *b, ts_generated **out) {
  if (!b || !out) return TS_ERR_NULL;
  const size_t n = b->sessions.size();
  if (n == 0) {
    b->err = "empty batch";
    return TS_ERR_STATE;
  }
  for (size_t i = 0; i < n; ++i) out[i] = nullptr;
  const auto t_wall0 = std::chrono::steady_clock::now();
  std::vector<ts_session *> sessions;
  sessions.swap(b->sessions);
  struct Owned {
    std::vector<ts_session *> &v;
    ~Owned() {
      for (ts_session *s : v) delete s;
    }
  } owned{sessions};
  // main stream, side stream (item uploads, random candidates made ahead)
  // and copy stream (read-backs); outside the try so that a failure can
  // drain them before the sessions' buffers go
  StreamGuard sg, rg, cg;
  std::vector<std::unique_ptr<RunCtx>> ctx(n);
  size_t current = 0;
  try {
    CUDA_TRY(cudaSetDevice(b->device));
    // the step chain on the highest priority, the side stream's work on the
    // lowest and (unless the launches are captured into a graph) on the
    // green context that leaves SMs to the chain (side_stream)
    int prio_low = 0, prio_high = 0;
    CUDA_TRY(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
    CUDA_TRY(cudaStreamCreateWithPriority(&sg.s, cudaStreamNonBlocking, prio_high));
    const cudaStream_t st = sg.s;
    size_t max_steps = 0;
    const auto t_plan0 = std::chrono::steady_clock::now();
    {
      // sessions plan independently: host threads take them in turn
      unsigned nt = b->plan_threads ? b->plan_threads : std::min(32u, std::max(1u, std::thread::hardware_concurrency()));
      nt = (unsigned)std::min<size_t>(nt, n);
      std::atomic<size_t> next{0};
      std::vector<Failure> fails(n, Failure{TS_OK, ""});
      auto work = [&] {
        if (cudaSetDevice(b->device) != cudaSuccess) return;
        for (size_t j = next++; j < n; j = next++) {
          try {
            ctx[j].reset(new RunCtx());
            ctx[j]->want_rc_ahead = true;
            run_plan(sessions[j], *ctx[j]);
            run_pick_all(*ctx[j]);
            run_alloc(*ctx[j], nullptr);
            RunCtx &c = *ctx[j];
            run_stage_tables(c);
            // touch the read-back destinations here, in parallel, rather
            // than in the copies at the end of the run
            c.col.resize(c.N);
            c.stv.resize(c.N);
            c.g->resolved.resize(c.res_total);
            c.g->scores.resize(c.res_total);
            if (cudaSuccess != c.pitems.alloc(c.items.size())) throw Failure{TS_ERR_CUDA, "pinned host memory"};
            memcpy(c.pitems.p, c.items.data(), c.items.size() * 4);
            c.items_async = true;
          } catch (const Failure &f) {
            fails[j] = f;
          } catch (const std::bad_alloc &) {
            fails[j] = Failure{TS_ERR_OUT_OF_MEMORY, "out of host memory"};
          }
        }
      };
      std::vector<std::thread> pool;
      for (unsigned i = 1; i < nt; ++i) pool.emplace_back(work);
      work();
      for (auto &t : pool) t.join();
      for (current = 0; current < n; ++current) {
        if (fails[current].status != TS_OK) throw fails[current];
        if (!ctx[current]) throw Failure{TS_ERR_CUDA, "cannot select the device"};
        max_steps = std::max(max_steps, ctx[current]->steps.size());
      }
    }
    const double plan_ms =
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_plan0).count();
    // ---- the launch plan: per global step and phase, one segment per session ----
    std::vector<SessionDev> h_sess(n);
    std::vector<size_t> step_base(n);
    size_t n_steps = 0;
    for (size_t j = 0; j < n; ++j) {
      h_sess[j] = ctx[j]->sd;
      step_base[j] = n_steps;
      n_steps += ctx[j]->steps.size();
    }
    std::vector<StepDev> h_steps(n_steps);
    for (size_t j = 0; j < n; ++j)
      for (size_t t = 0; t < ctx[j]->steps.size(); ++t) {
        const Step &stp = ctx[j]->steps[t];
        StepDev &d = h_steps[step_base[j] + t];
        d = StepDev{};
        d.st = stp.st;
        d.rc = stp.rc_st;
        d.b = stp.bd;
        d.level = stp.ls_level;
        d.ls_n_res = stp.ls_n_res;
        d.all_items = stp.exhaustive ? 1 : 0;
      }
    std::vector<Segment> h_segs, h_fb;
    std::vector<PlannedLaunch> launches;
    std::vector<size_t> last_launch(n, 0);  // a session's results are final after this launch
    size_t phase_smem[kPhases] = {};
    // segments of a launch go heaviest session first (per-item resolve work
    // grows with k (k + m), doubled by a guide), so that the blocks left for
    // the end of a launch are the light ones
    std::vector<size_t> heavy(n);
    for (size_t j = 0; j < n; ++j) heavy[j] = j;
    auto weight = [&](size_t j) {
      const RunCtx &c = *ctx[j];
      return (uint64_t)std::max<uint32_t>(c.k, 1) * (c.k + c.m) * (sessions[j]->guided ? 2 : 1);
    };
    std::stable_sort(heavy.begin(), heavy.end(), [&](size_t x, size_t y) { return weight(x) > weight(y); });
    // random candidates made ahead on a side stream: launch q holds stage q
    // of every session that makes them so (rc_pos[q] indexes rc_launches)
    size_t max_stages = 0;
    for (size_t j = 0; j < n; ++j) max_stages = std::max(max_stages, ctx[j]->plan.size());
    std::vector<PlannedLaunch> rc_launches;
    std::vector<int> rc_pos(max_stages, -1);
    for (size_t q = 0; q < max_stages; ++q) {
      PlannedLaunch pl;
      pl.phase = kPhaseRandom;
      pl.seg0 = (uint32_t)h_segs.size();
      pl.n_segs = pl.blocks = 0;
      pl.smem = 0;
      for (size_t j : heavy) {
        const RunCtx &c = *ctx[j];
        if (!c.rc_ahead || q >= c.rc_step.size() || c.rc_step[q] < 0) continue;
        const uint32_t t = (uint32_t)c.rc_step[q];
        const uint32_t nb = multi_blocks(kPhaseRandom, c.steps[t].rc_st.n_items, 0);
        if (nb == 0) continue;
        h_segs.push_back(Segment{pl.blocks, nb, (uint32_t)j, t});
        pl.blocks += nb;
        pl.n_segs += 1;
        pl.smem = std::max(pl.smem, multi_smem_bytes(kPhaseRandom, c.k, c.m));
      }
      pl.pool_block0 = pl.blocks;
      if (pl.n_segs) {
        phase_smem[kPhaseRandom] = std::max(phase_smem[kPhaseRandom], pl.smem);
        rc_pos[q] = (int)rc_launches.size();
        rc_launches.push_back(pl);
      }
    }
    int rc_waited = -1, items_waited = -1;
    for (size_t t = 0; t < max_steps; ++t) {
      // a session starting stage q at this step needs rc launch q done
      int rc_need = -1;
      for (size_t j = 0; j < n; ++j) {
        const RunCtx &c = *ctx[j];
        if (c.rc_ahead && t < c.steps.size() && c.steps[t].rc) rc_need = std::max(rc_need, rc_pos[c.steps[t].stage]);
      }
      const size_t launches_before = launches.size();
      // the resolve form follows the step's items over all sessions: the
      // team forms only pay while the whole launch is too small to fill
      // the GPU with warps
      uint64_t step_items = 0;
      bool all_team_full = true;
      for (size_t j = 0; j < n; ++j)
        if (t < ctx[j]->steps.size() && ctx[j]->steps[t].batch) {
          step_items += ctx[j]->steps[t].n;
          all_team_full &= team_full_fits(ctx[j]->k, ctx[j]->m);
        }
      const int form = step_items > b->team_max_items ? kPhaseResolve
                       : (step_items <= b->team_full_max_items && all_team_full) ? kPhaseTeamFull
                                                                                 : kPhaseTeamPart;
      for (size_t j = 0; j < n; ++j)
        if (t < ctx[j]->steps.size()) ctx[j]->steps[t].resolve = form;
      for (int ph = 0; ph < kPhases; ++ph) {
        PlannedLaunch pl;
        pl.phase = ph;
        pl.seg0 = (uint32_t)h_segs.size();
        pl.n_segs = pl.blocks = 0;
        pl.smem = 0;
        pl.fb0 = (uint32_t)h_fb.size();
        // resolve: sessions without guides first (the lean kernel), then the rest
        for (int pass = 0; pass < (ph == kPhaseResolve ? 2 : 1); ++pass) {
          for (size_t j : heavy) {
            const RunCtx &c = *ctx[j];
            if (t >= c.steps.size()) continue;
            if (ph == kPhaseResolve && sessions[j]->guided != (pass == 1)) continue;
            const Step &stp = c.steps[t];
            if (ph == kPhaseExhaustive && stp.batch && c.k > 0 && !stp.exhaustive) {
              h_fb.push_back(Segment{0, 0, (uint32_t)j, (uint32_t)t});
              pl.n_fb += 1;
              pl.key_cap = std::max(pl.key_cap, exh_key_cap(c.sd, stp.bd));
            }
            const uint32_t units = phase_units(stp, c, ph);
            const uint32_t nb = multi_blocks(ph, units, phase_cap(stp, ph));
            if (nb == 0) continue;
            h_segs.push_back(Segment{pl.blocks, nb, (uint32_t)j, (uint32_t)t});
            pl.blocks += nb;
            pl.n_segs += 1;
            if (ph == kPhaseExhaustive)
              pl.key_cap = std::max(pl.key_cap, exh_key_cap(c.sd, stp.bd));
            else
              pl.smem = std::max(pl.smem, multi_smem_bytes(ph, c.k, c.m));
          }
          if (ph == kPhaseResolve && pass == 0) {
            pl.n_lean = pl.n_segs;
            pl.lean_blocks = pl.blocks;
          }
        }
        pl.pool_block0 = pl.blocks;
        if (pl.n_fb) pl.blocks += kFallbackPool;
        if (ph == kPhaseExhaustive) pl.smem = (size_t)pl.key_cap * 8;
        if (pl.n_segs || pl.n_fb) {
          phase_smem[ph] = std::max(phase_smem[ph], pl.smem);
          launches.push_back(pl);
          for (uint32_t q = pl.seg0; q < pl.seg0 + pl.n_segs; ++q) last_launch[h_segs[q].session] = launches.size() - 1;
          for (uint32_t q = pl.fb0; q < pl.fb0 + pl.n_fb; ++q) last_launch[h_fb[q].session] = launches.size() - 1;
        }
      }
      if (rc_need > rc_waited && launches.size() > launches_before) {
        launches[launches_before].wait_rc = rc_need;
        rc_waited = rc_need;
      }
      // stage 0 items before the first launch, the rest before any session
      // gets past stage 0
      int items_need = t == 0 ? 0 : -1;
      for (size_t j = 0; j < n; ++j)
        if (t < ctx[j]->steps.size() && ctx[j]->steps[t].stage >= 1) items_need = 1;
      if (items_need > items_waited && launches.size() > launches_before) {
        launches[launches_before].wait_items = items_need;
        items_waited = items_need;
      }
    }
    for (int ph = 0; ph < kPhases; ++ph) CUDA_TRY(set_multi_smem(ph, phase_smem[ph]));
    DevBuf<SessionDev> d_sess;
    DevBuf<StepDev> d_steps;
    DevBuf<Segment> d_segs, d_fb;
    DevBuf<const StepDev *> d_tabs;
    CUDA_TRY(d_tabs.alloc(n));
    CUDA_TRY(d_sess.alloc(n));
    CUDA_TRY(d_steps.alloc(n_steps));
    CUDA_TRY(d_segs.alloc(h_segs.size()));
    CUDA_TRY(d_fb.alloc(h_fb.size()));
    EventPair ev, ev_io;
    ev.create();
    ev_io.create();
    CUDA_TRY(cudaEventRecord(ev.a, st));
    for (current = 0; current < n; ++current) {
      if (sessions[current]->ready.e) CUDA_TRY(cudaStreamWaitEvent(st, sessions[current]->ready.e, 0));
      run_upload(*ctx[current], st);
    }
    CUDA_TRY(cudaMemcpyAsync(d_sess.p, h_sess.data(), n * sizeof(SessionDev), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_steps.p, h_steps.data(), n_steps * sizeof(StepDev), cudaMemcpyHostToDevice, st));
    std::vector<const StepDev *> h_tabs(n);
    for (size_t j = 0; j < n; ++j) h_tabs[j] = d_steps.p + step_base[j];
    CUDA_TRY(cudaMemcpyAsync(d_tabs.p, h_tabs.data(), n * sizeof(const StepDev *), cudaMemcpyHostToDevice, st));
    if (!h_segs.empty())
      CUDA_TRY(cudaMemcpyAsync(d_segs.p, h_segs.data(), h_segs.size() * sizeof(Segment), cudaMemcpyHostToDevice,
                               st));
    if (!h_fb.empty())
      CUDA_TRY(cudaMemcpyAsync(d_fb.p, h_fb.data(), h_fb.size() * sizeof(Segment), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaEventRecord(ev_io.a, st));
    std::vector<EventPair> pev(b->profile && !b->graph ? launches.size() : 0);
    for (auto &e : pev) e.create();
    // sessions are read back on a copy stream as soon as their last launch
    // is done, while the longer sessions still run
    std::vector<size_t> order(n);
    for (size_t j = 0; j < n; ++j) order[j] = j;
    std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return last_launch[x] < last_launch[y]; });
    std::vector<EventHandle> done_ev(launches.size());
    for (size_t j = 0; j < n; ++j)
      if (!done_ev[last_launch[j]].e) CUDA_TRY(cudaEventCreateWithFlags(&done_ev[last_launch[j]].e, cudaEventDisableTiming));
    CUDA_TRY(cudaStreamCreateWithFlags(&cg.s, cudaStreamNonBlocking));
    EventHandle copies_done;
    CUDA_TRY(cudaEventCreateWithFlags(&copies_done.e, cudaEventDisableTiming));
    auto readbacks = [&] {
      for (size_t q = 0; q < n; ++q) {
        current = order[q];
        if (q == 0 || last_launch[order[q - 1]] != last_launch[current])
          CUDA_TRY(cudaStreamWaitEvent(cg.s, done_ev[last_launch[current]].e, 0));
        run_readback(*ctx[current], cg.s);
      }
      CUDA_TRY(cudaEventRecord(copies_done.e, cg.s));
      CUDA_TRY(cudaStreamWaitEvent(st, copies_done.e, 0));
    };
    std::vector<EventHandle> rc_ev(rc_launches.size());
    if (b->graph)
      CUDA_TRY(cudaStreamCreateWithPriority(&rg.s, cudaStreamNonBlocking, prio_low));
    else
      CUDA_TRY(side_stream(b->device, prio_low, &rg.s));
    for (auto &e : rc_ev) CUDA_TRY(cudaEventCreateWithFlags(&e.e, cudaEventDisableTiming));
    EventHandle fork, side_done, items_ev[2];
    CUDA_TRY(cudaEventCreateWithFlags(&fork.e, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&side_done.e, cudaEventDisableTiming));
    for (auto &e : items_ev) CUDA_TRY(cudaEventCreateWithFlags(&e.e, cudaEventDisableTiming));
    // the items of stage 0 (part 0) and of the later stages (part 1), every
    // session's, from its pinned copy
    auto upload_items = [&](int part) {
      for (size_t j = 0; j < n; ++j) {
        RunCtx &c = *ctx[j];
        if (c.items.empty()) continue;
        const size_t split = c.plan.size() > 1 ? c.plan[1].items_off : c.items.size();
        const size_t a = part == 0 ? 0 : split, e = part == 0 ? split : c.items.size();
        if (e > a)
          CUDA_TRY(cudaMemcpyAsync(c.d_items.p + a, c.pitems.p + a, (e - a) * 4, cudaMemcpyHostToDevice, rg.s));
      }
      CUDA_TRY(cudaEventRecord(items_ev[part].e, rg.s));
    };
    auto launch_rc = [&](size_t i) {
      const PlannedLaunch &pl = rc_launches[i];
      MultiLaunch ml;
      ml.segs = d_segs.p + pl.seg0;
      ml.n_segs = pl.n_segs;
      ml.sessions = d_sess.p;
      ml.step_tabs = d_tabs.p;
      ml.fb = d_fb.p;
      ml.n_fb = 0;
      ml.pool_block0 = pl.blocks;
      launch_multi(kPhaseRandom, ml, pl.blocks, pl.smem, rg.s);
      CUDA_TRY(cudaEventRecord(rc_ev[i].e, rg.s));
    };
    auto enqueue = [&](cudaStream_t s) {
      // side stream: stage 0's items and random candidates first (the
      // first steps wait for them), then the later stages' while those
      // first steps run
      CUDA_TRY(cudaEventRecord(fork.e, s));
      CUDA_TRY(cudaStreamWaitEvent(rg.s, fork.e, 0));
      upload_items(0);
      size_t rci = 0;
      if (!rc_launches.empty() && rc_pos[0] == 0) launch_rc(rci++);
      upload_items(1);
      for (; rci < rc_launches.size(); ++rci) launch_rc(rci);
      CUDA_TRY(cudaEventRecord(side_done.e, rg.s));
      for (size_t li = 0; li < launches.size(); ++li) {
        const PlannedLaunch &pl = launches[li];
        if (pl.wait_items >= 0) CUDA_TRY(cudaStreamWaitEvent(s, items_ev[pl.wait_items].e, 0));
        if (pl.wait_rc >= 0) CUDA_TRY(cudaStreamWaitEvent(s, rc_ev[pl.wait_rc].e, 0));
        MultiLaunch ml;
        ml.segs = d_segs.p + pl.seg0;
        ml.n_segs = pl.n_segs;
        ml.sessions = d_sess.p;
        ml.step_tabs = d_tabs.p;
        ml.fb = d_fb.p + pl.fb0;
        ml.n_fb = pl.n_fb;
        ml.pool_block0 = pl.n_fb ? pl.pool_block0 : pl.blocks;
        ml.n_lean = pl.n_lean;
        ml.lean_blocks = pl.lean_blocks;
        ml.key_cap = pl.key_cap;
        if (!pev.empty()) CUDA_TRY(cudaEventRecord(pev[li].a, s));
        launch_multi(pl.phase, ml, pl.blocks, pl.smem, s);
        if (!pev.empty()) CUDA_TRY(cudaEventRecord(pev[li].b, s));
        if (done_ev[li].e)
          CUDA_TRY(cudaEventRecordWithFlags(done_ev[li].e, s, b->graph ? cudaEventRecordExternal : cudaEventRecordDefault));
      }
      CUDA_TRY(cudaStreamWaitEvent(s, side_done.e, 0));  // joins the side stream
      CUDA_TRY(cudaGetLastError());
    };
    if (b->graph) {
      cudaGraph_t graph = nullptr;
      cudaGraphExec_t exec = nullptr;
      CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      try {
        enqueue(st);
      } catch (...) {
        cudaStreamEndCapture(st, &graph);
        if (graph) cudaGraphDestroy(graph);
        throw;
      }
      CUDA_TRY(cudaStreamEndCapture(st, &graph));
      struct GraphGuard {
        cudaGraph_t g;
        cudaGraphExec_t &e;
        ~GraphGuard() {
          if (e) cudaGraphExecDestroy(e);
          if (g) cudaGraphDestroy(g);
        }
      } gg{graph, exec};
      CUDA_TRY(cudaGraphInstantiate(&exec, graph, 0));
      CUDA_TRY(cudaGraphLaunch(exec, st));
      CUDA_TRY(cudaEventRecord(ev_io.b, st));
      readbacks();
      CUDA_TRY(cudaEventRecord(ev.b, st));
      CUDA_TRY(cudaStreamSynchronize(st));
    } else {
      enqueue(st);
      CUDA_TRY(cudaEventRecord(ev_io.b, st));
      readbacks();
      CUDA_TRY(cudaEventRecord(ev.b, st));
      CUDA_TRY(cudaStreamSynchronize(st));
    }
    const double gpu_ms = ev.ms();
    ts_batch_stats bs{};
    bs.sessions = n;
    bs.steps = max_steps;
    bs.launches = launches.size() + rc_launches.size();
    for (const PlannedLaunch &pl : launches)
      if (pl.phase == kPhaseResolve && pl.n_lean && pl.n_lean < pl.n_segs) bs.launches += 1;  // two kernels
    bs.phase_launches[kPhaseRandom] += rc_launches.size();
    bs.plan_ms = plan_ms;
    {
      float up = 0.0f, rb = 0.0f;
      CUDA_TRY(cudaEventElapsedTime(&up, ev.a, ev_io.a));
      CUDA_TRY(cudaEventElapsedTime(&rb, ev_io.b, ev.b));
      bs.upload_ms = up;
      bs.readback_ms = rb;
    }
    for (size_t li = 0; li < pev.size(); ++li) {
      bs.phase_launches[launches[li].phase] += 1;
      bs.phase_ms[launches[li].phase] += pev[li].ms();
    }
    for (current = 0; current < n; ++current) {
      RunCtx &c = *ctx[current];
      for (const Step &stp : c.steps)
        if (stp.batch) {
          ++c.batches;
          c.resolves += stp.n;
        }
      run_finish(c);
      c.g->stats.gpu_ms = gpu_ms;
      c.g->stats.kernel_launches = launches.size();
      bs.output_pixels += c.N;
      bs.resolves += c.resolves;
      bs.cost_evals += c.evals;
    }
    bs.gpu_ms = gpu_ms;
    bs.wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_wall0).count();
    b->stats = bs;
  } catch (const Failure &f) {
    // nothing may be in flight when the sessions' buffers go
    for (cudaStream_t q : {sg.s, rg.s, cg.s})
      if (q) cudaStreamSynchronize(q);
    b->err = "session " + std::to_string(current < n ? current : 0) + ": " + f.msg;
    return f.status;
  }
  for (size_t i = 0; i < n; ++i) {
    ctx[i]->g->stats.wall_ms = b->stats.wall_ms;
    out[i] = ctx[i]->g.release();
  }
  return TS_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Served form: continuous batching.  Requests (built sessions) are planned
// on the submitting thread and queued; a driver thread admits them into
// session slots while the device-memory budget allows and then runs ticks:
// one tick is one batch step of every admitted session, issued as the
// multi-session launches of the batched form, so a request that arrives
// while others run joins them at the next tick.  A completion thread reads
// finished sessions back and releases their memory and slot.
// ---------------------------------------------------------------------------
namespace {

double host_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct ServerReq {
  uint64_t ticket = 0;
  ts_session *s = nullptr;  // owned
  std::unique_ptr<RunCtx> c;
  DevBuf<StepDev> d_steps;
  uint32_t slot = 0;
  bool slotted = false;  // holds a slot and its budget charge
  size_t cursor = 0;
  uint64_t bytes = 0;  // admission charge: the run's buffers plus the session's pyramids
  double t_submit = 0, t_admit = 0, t_done = 0;
  int status = TS_OK;
  std::string err;
  ts_generated *result = nullptr;
  bool done = false;
  // The pick chain runs ahead of the device: stage 0 on the submitting
  // thread, the rest on a picker thread, into c->pitems; `picked` counts the
  // stages whose items are there, `uploaded` those the driver has copied
  // to the device (driver only), `picks_done` guards c against the picker.
  std::atomic<uint32_t> picked{0};
  uint32_t uploaded = 0;
  bool picks_done = false;  // under the server mutex
  cudaEvent_t up_ev = nullptr, ev = nullptr;  // uploads done; last kernels done
  ~ServerReq() {
    if (up_ev) cudaEventDestroy(up_ev);
    if (ev) cudaEventDestroy(ev);
    delete result;
    delete s;
  }
};

constexpr uint32_t kServerRing = 8;  // ticks in flight
constexpr size_t kLoneSteps = 16;    // steps of a tick that holds a single request

}  // namespace

struct ts_server {
  int device = 0;
  uint64_t budget = 0;
  uint32_t max_active = 0;
  uint32_t team_max_items = 2048, team_full_max_items = 256;
  double t0 = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_complete, cv_pick, cv_picked;
  std::deque<ServerReq *> to_pick;  // requests whose later stages are still to be picked
  std::deque<ServerReq *> pending;
  std::atomic<uint32_t> n_pending{0};  // pending.size(), read by the driver without the mutex
  std::unordered_map<uint64_t, ServerReq *> reqs;  // submitted, not yet collected
  std::deque<ServerReq *> completing;              // steps done, waiting for read-back
  std::vector<uint32_t> free_slots;
  uint64_t used = 0;
  uint64_t next_ticket = 1;
  bool stop = false, stop_completer = false, stop_pickers = false;
  int fatal = TS_OK;
  std::string err;
  std::vector<ServerReq *> active;  // driver thread only
  std::thread driver, completer;
  std::vector<std::thread> pickers;
  cudaStream_t st = nullptr, ust = nullptr, cst = nullptr;  // compute, upload, completion
  DevBuf<SessionDev> d_sess;
  DevBuf<const StepDev *> d_tabs;
  struct Ring {
    Segment *h = nullptr;  // pinned, read by the tick's kernels
    cudaEvent_t ev = nullptr;
    bool used = false;
  };
  Ring ring[kServerRing];
  uint32_t seg_cap = 0;
  ts_server_stats stats{};
};

namespace {

void server_fail(ts_server *S, ServerReq *r, const Failure &f) {
  r->status = f.status;
  r->err = f.msg;
}

// The next stage of a request's pick chain, into its pinned items.
void server_pick_stage(ServerReq &r) {
  RunCtx &c = *r.c;
  const size_t q = c.picked_stages;
  run_pick(c);
  const StagePlan &sp = c.plan[q];
  if (sp.n_items) memcpy(c.pitems.p + sp.items_off, c.items.data() + sp.items_off, (size_t)sp.n_items * 4);
  r.picked.store((uint32_t)q + 1, std::memory_order_release);
}

void server_picker(ts_server *S) {
  for (;;) {
    ServerReq *r = nullptr;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_pick.wait(lk, [&] { return S->stop_pickers || !S->to_pick.empty(); });
      if (S->to_pick.empty()) return;
      r = S->to_pick.front();
      S->to_pick.pop_front();
    }
    while (r->picked.load(std::memory_order_relaxed) < r->c->plan.size()) {
      server_pick_stage(*r);
      std::lock_guard<std::mutex> lk(S->mu);  // the driver may be waiting for this stage
      S->cv_picked.notify_all();
    }
    std::lock_guard<std::mutex> lk(S->mu);
    r->picks_done = true;
    S->cv_picked.notify_all();
  }
}

// Device buffers, uploads and slot entries of an admitted request, on the
// upload stream; the compute stream waits for them before its next tick.
void server_admit(ts_server *S, ServerReq *r) {
  RunCtx &c = *r->c;
  if (r->s->ready.e) CUDA_TRY(cudaStreamWaitEvent(S->ust, r->s->ready.e, 0));
  run_alloc(c, S->ust);
  run_upload(c, S->ust);
  std::vector<StepDev> h(c.steps.size());
  for (size_t t = 0; t < c.steps.size(); ++t) {
    const Step &stp = c.steps[t];
    StepDev &d = h[t];
    d = StepDev{};
    d.st = stp.st;
    d.rc = stp.rc_st;
    d.b = stp.bd;
    d.level = stp.ls_level;
    d.ls_n_res = stp.ls_n_res;
    d.all_items = stp.exhaustive ? 1 : 0;
  }
  CUDA_TRY(r->d_steps.alloc_on(h.size(), S->ust));
  CUDA_TRY(cudaMemcpyAsync(r->d_steps.p, h.data(), h.size() * sizeof(StepDev), cudaMemcpyHostToDevice, S->ust));
  const StepDev *tab = r->d_steps.p;
  CUDA_TRY(cudaMemcpyAsync(S->d_sess.p + r->slot, &c.sd, sizeof(SessionDev), cudaMemcpyHostToDevice, S->ust));
  CUDA_TRY(cudaMemcpyAsync(S->d_tabs.p + r->slot, &tab, sizeof(tab), cudaMemcpyHostToDevice, S->ust));
  CUDA_TRY(cudaEventCreateWithFlags(&r->up_ev, cudaEventDisableTiming));
  // the completion thread sleeps on this one instead of spinning beside the driver
  CUDA_TRY(cudaEventCreateWithFlags(&r->ev, cudaEventDisableTiming | cudaEventBlockingSync));
  CUDA_TRY(cudaEventRecord(r->up_ev, S->ust));
  CUDA_TRY(cudaStreamWaitEvent(S->st, r->up_ev, 0));
}

void server_driver(ts_server *S) {
  if (cudaSetDevice(S->device) != cudaSuccess) return;
  std::vector<ServerReq *> ready_buf;
  std::vector<Segment> segs, fb;
  std::vector<PlannedLaunch> launches;
  size_t phase_smem[kPhases] = {};
  uint32_t ri = 0;
  for (;;) {
    // ---- admission ----
    {
      std::unique_lock<std::mutex> lk(S->mu);
      if (S->active.empty()) {
        S->cv_work.wait(lk, [&] { return S->stop || !S->pending.empty(); });
        if (S->pending.empty()) break;  // stopping, nothing left
      }
      while (!S->pending.empty() && !S->free_slots.empty()) {
        ServerReq *r = S->pending.front();
        // within the budget, or alone on the device
        if (!S->active.empty() && S->used + r->bytes > S->budget) break;
        S->pending.pop_front();
        S->n_pending.store((uint32_t)S->pending.size(), std::memory_order_relaxed);
        r->slot = S->free_slots.back();
        S->free_slots.pop_back();
        r->slotted = true;
        S->used += r->bytes;
        S->stats.peak_bytes = std::max(S->stats.peak_bytes, S->used);
        lk.unlock();
        r->t_admit = host_ms() - S->t0;
        bool ok = true;
        try {
          server_admit(S, r);
        } catch (const Failure &f) {
          server_fail(S, r, f);
          ok = false;
        }
        lk.lock();
        if (ok) {
          S->active.push_back(r);
          S->stats.admitted += 1;
        } else {
          S->completing.push_back(r);
          S->cv_complete.notify_one();
        }
      }
      S->stats.peak_active = std::max<uint64_t>(S->stats.peak_active, S->active.size());
    }
    if (S->active.empty()) continue;
    // ---- one tick: the next step of every active session whose items are
    // picked (the others wait for their picker) ----
    std::vector<ServerReq *> &ready = ready_buf;
    ready.clear();
    for (ServerReq *r : S->active)
      if (r->c->steps[r->cursor].stage < (int)r->picked.load(std::memory_order_acquire)) ready.push_back(r);
    if (ready.empty()) {
      const double w0 = host_ms();
      // Wait for a picker (or a new request), re-checking under the mutex:
      // a picker publishes `picked` before it takes the mutex to notify, so
      // no wake-up is lost between the check above and the wait.
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_picked.wait_for(lk, std::chrono::microseconds(500), [&] {
        if (S->stop || (!S->pending.empty() && !S->free_slots.empty())) return true;
        for (ServerReq *r : S->active)
          if (r->c->steps[r->cursor].stage < (int)r->picked.load(std::memory_order_acquire)) return true;
        return false;
      });
      S->stats.driver_pick_wait_us += (uint64_t)((host_ms() - w0) * 1e3);
      continue;
    }
    const double t_tick0 = host_ms();
    try {
      ts_server::Ring &R = S->ring[ri];
      double ring_wait = 0.0, launch_ms = 0.0;
      if (R.used) {  // the slot's previous tick is done
        const double w0 = host_ms();
        CUDA_TRY(cudaEventSynchronize(R.ev));
        ring_wait = host_ms() - w0;
      }
      for (ServerReq *r : ready) {
        // items of the stages picked so far, in stream order before the launches
        RunCtx &c = *r->c;
        const uint32_t upto = r->picked.load(std::memory_order_acquire);
        for (; r->uploaded < upto; ++r->uploaded) {
          const StagePlan &sp = c.plan[r->uploaded];
          if (sp.n_items)
            CUDA_TRY(cudaMemcpyAsync(c.d_items.p + sp.items_off, c.pitems.p + sp.items_off,
                                     (size_t)sp.n_items * 4, cudaMemcpyHostToDevice, S->st));
        }
      }
      uint64_t step_items = 0;
      bool all_team_full = true;
      for (ServerReq *r : ready) {
        const Step &stp = r->c->steps[r->cursor];
        if (stp.batch) {
          step_items += stp.n;
          all_team_full &= team_full_fits(r->c->k, r->c->m);
        }
      }
      const int form = step_items > S->team_max_items                              ? kPhaseResolve
                       : (step_items <= S->team_full_max_items && all_team_full) ? kPhaseTeamFull
                                                                                 : kPhaseTeamPart;
      segs.clear();
      fb.clear();
      launches.clear();
      for (ServerReq *r : ready) r->c->steps[r->cursor].resolve = form;
      uint64_t tick_launches = 0;
      size_t lone_steps = 1;  // steps the tick advances a lone session by
      if (ready.size() == 1) {
        // one session in the tick: its steps with the single-session kernels
        // (no segment lookups at the start of every block).  While nothing
        // waits for admission it takes up to kLoneSteps consecutive steps
        // whose items are picked, as the plain path would (a redo-only
        // batch's commit then rides in the next step's first k-NN launch),
        // so that the host's per-tick work does not pace a lone request; a
        // request that arrives meanwhile joins at the next tick.
        ServerReq *r0 = ready[0];
        RunCtx &c = *r0->c;
        const uint64_t before = c.launches;
        LaunchTimer lt;
        const double l0 = host_ms();
        // only stages whose items went up above: a picker may have
        // published more since
        const uint32_t uploaded = r0->uploaded;
        const size_t limit = S->n_pending.load(std::memory_order_relaxed) ? 1 : kLoneSteps;
        auto usable = [&](size_t t) { return t < c.steps.size() && c.steps[t].stage < (int)uploaded; };
        const Step *pending = nullptr;
        size_t n = 0;
        while (n < limit && usable(r0->cursor + n)) {
          Step &stp = c.steps[r0->cursor + n];
          if (n > 0)
            stp.resolve = stp.n > S->team_max_items                                        ? kPhaseResolve
                          : (stp.n <= S->team_full_max_items && team_full_fits(c.k, c.m)) ? kPhaseTeamFull
                                                                                           : kPhaseTeamPart;
          const bool more = n + 1 < limit && usable(r0->cursor + n + 1);
          if (more) {
            Step &nx = c.steps[r0->cursor + n + 1];
            nx.resolve = nx.n > S->team_max_items                                        ? kPhaseResolve
                         : (nx.n <= S->team_full_max_items && team_full_fits(c.k, c.m)) ? kPhaseTeamFull
                                                                                         : kPhaseTeamPart;
          }
          const bool defer = more && can_defer_commit(c, stp, &c.steps[r0->cursor + n + 1]);
          enqueue_step(c, stp, S->st, lt, pending, defer);
          pending = defer ? &stp : nullptr;
          ++n;
        }
        lone_steps = n;
        launch_ms += host_ms() - l0;
        tick_launches = c.launches - before;
      } else {
        for (int ph = 0; ph < kPhases; ++ph) {
          PlannedLaunch pl;
          pl.phase = ph;
          pl.seg0 = (uint32_t)segs.size();
          pl.n_segs = pl.blocks = 0;
          pl.smem = 0;
          pl.fb0 = (uint32_t)fb.size();
          // resolve: sessions without guides first (the lean kernel), then the rest
          for (int pass = 0; pass < (ph == kPhaseResolve ? 2 : 1); ++pass) {
            for (ServerReq *r : ready) {
              const RunCtx &c = *r->c;
              if (ph == kPhaseResolve && r->s->guided != (pass == 1)) continue;
              const Step &stp = c.steps[r->cursor];
              if (ph == kPhaseExhaustive && stp.batch && c.k > 0 && !stp.exhaustive) {
                fb.push_back(Segment{0, 0, r->slot, (uint32_t)r->cursor});
                pl.n_fb += 1;
                pl.key_cap = std::max(pl.key_cap, exh_key_cap(c.sd, stp.bd));
              }
              const uint32_t nb = multi_blocks(ph, phase_units(stp, c, ph), phase_cap(stp, ph));
              if (nb == 0) continue;
              segs.push_back(Segment{pl.blocks, nb, r->slot, (uint32_t)r->cursor});
              pl.blocks += nb;
              pl.n_segs += 1;
              if (ph == kPhaseExhaustive)
                pl.key_cap = std::max(pl.key_cap, exh_key_cap(c.sd, stp.bd));
              else
                pl.smem = std::max(pl.smem, multi_smem_bytes(ph, c.k, c.m));
            }
            if (ph == kPhaseResolve && pass == 0) {
              pl.n_lean = pl.n_segs;
              pl.lean_blocks = pl.blocks;
            }
          }
          pl.pool_block0 = pl.blocks;
          if (pl.n_fb) pl.blocks += kFallbackPool;
          if (ph == kPhaseExhaustive) pl.smem = (size_t)pl.key_cap * 8;
          if (pl.n_segs || pl.n_fb) {
            if (pl.smem > phase_smem[ph]) {
              CUDA_TRY(set_multi_smem(ph, pl.smem));
              phase_smem[ph] = pl.smem;
            }
            launches.push_back(pl);
          }
        }
        const size_t nseg = segs.size() + fb.size();
        if (nseg > S->seg_cap) throw Failure{TS_ERR_LIMIT, "segment table overflow"};
        // the kernels read the tick's segment table straight from pinned host
        // memory (no copy in the stream between ticks)
        std::copy(segs.begin(), segs.end(), R.h);
        std::copy(fb.begin(), fb.end(), R.h + segs.size());
        for (const PlannedLaunch &pl : launches) {
          MultiLaunch ml;
          ml.segs = R.h + pl.seg0;
          ml.n_segs = pl.n_segs;
          ml.sessions = S->d_sess.p;
          ml.step_tabs = S->d_tabs.p;
          ml.fb = R.h + segs.size() + pl.fb0;
          ml.n_fb = pl.n_fb;
          ml.pool_block0 = pl.n_fb ? pl.pool_block0 : pl.blocks;
          ml.n_lean = pl.n_lean;
          ml.lean_blocks = pl.lean_blocks;
          ml.key_cap = pl.key_cap;
          const double l0 = host_ms();
          launch_multi(pl.phase, ml, pl.blocks, pl.smem, S->st);
          launch_ms += host_ms() - l0;
        }
        tick_launches = launches.size();
        for (const PlannedLaunch &pl : launches)
          if (pl.phase == kPhaseResolve && pl.n_lean && pl.n_lean < pl.n_segs) tick_launches += 1;
      }
      CUDA_TRY(cudaGetLastError());
      CUDA_TRY(cudaEventRecord(R.ev, S->st));
      R.used = true;
      ri = (ri + 1) % kServerRing;
      // advance; finished sessions go to the completion thread
      std::vector<ServerReq *> still;
      std::vector<ServerReq *> finished;
      for (ServerReq *r : S->active) {
        if (std::find(ready.begin(), ready.end(), r) == ready.end()) {
          still.push_back(r);
          continue;
        }
        RunCtx &c = *r->c;
        for (size_t q = 0; q < lone_steps; ++q) {
          const Step &stp = c.steps[r->cursor];
          if (stp.batch) {
            ++c.batches;
            c.resolves += stp.n;
          }
          ++r->cursor;
        }
        if (r->cursor == c.steps.size()) {
          CUDA_TRY(cudaEventRecord(r->ev, S->st));
          finished.push_back(r);
        } else {
          still.push_back(r);
        }
      }
      S->active.swap(still);
      {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stats.ticks += 1;
        S->stats.launches += tick_launches;
        S->stats.driver_ring_wait_us += (uint64_t)(ring_wait * 1e3);
        S->stats.driver_launch_us += (uint64_t)(launch_ms * 1e3);
        S->stats.driver_tick_us += (uint64_t)((host_ms() - t_tick0 - ring_wait) * 1e3);
        for (ServerReq *r : finished) S->completing.push_back(r);
        if (!finished.empty()) S->cv_complete.notify_one();
      }
    } catch (const Failure &f) {
      // the device is unusable for this server: fail everything in flight
      std::lock_guard<std::mutex> lk(S->mu);
      S->fatal = f.status;
      S->err = f.msg;
      for (ServerReq *r : S->active) {
        server_fail(S, r, f);
        S->completing.push_back(r);
      }
      S->active.clear();
      for (ServerReq *r : S->pending) {
        server_fail(S, r, f);
        S->completing.push_back(r);
      }
      S->pending.clear();
      S->n_pending.store(0, std::memory_order_relaxed);
      S->cv_complete.notify_one();
    }
  }
}

void server_completer(ts_server *S) {
  if (cudaSetDevice(S->device) != cudaSuccess) return;
  EventHandle copied;  // the read-back copies' end, waited on without spinning
  if (cudaEventCreateWithFlags(&copied.e, cudaEventDisableTiming | cudaEventBlockingSync) != cudaSuccess) return;
  for (;;) {
    ServerReq *r = nullptr;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_complete.wait(lk, [&] { return S->stop_completer || !S->completing.empty(); });
      if (S->completing.empty()) break;
      r = S->completing.front();
      S->completing.pop_front();
    }
    if (r->status == TS_OK) {
      try {
        CUDA_TRY(cudaEventSynchronize(r->ev));
        run_readback(*r->c, S->cst);
        CUDA_TRY(cudaEventRecord(copied.e, S->cst));
        CUDA_TRY(cudaEventSynchronize(copied.e));
        run_finish(*r->c);
        r->result = r->c->g.release();
      } catch (const Failure &f) {
        server_fail(S, r, f);
      }
    }
    const bool admitted = r->slotted;
    if (r->ev) cudaEventSynchronize(r->ev);  // no kernel of the request is left
    {
      std::unique_lock<std::mutex> lk(S->mu);  // nor is its picker (after a failure)
      S->cv_picked.wait(lk, [&] { return r->picks_done; });
    }
    // the run's buffers are pool memory (freed in stream order, no device
    // wait); the session's pyramids are freed with it
    r->c.reset();
    r->d_steps.reset();
    delete r->s;
    r->s = nullptr;
    {
      std::lock_guard<std::mutex> lk(S->mu);
      r->t_done = host_ms() - S->t0;
      if (admitted) {
        S->used -= r->bytes;
        S->free_slots.push_back(r->slot);
      }
      if (r->result) {
        S->stats.completed += 1;
        S->stats.output_pixels += (uint64_t)r->result->W * r->result->H;
        S->stats.cost_evals += r->result->stats.cost_evals;
        r->result->stats.wall_ms = r->t_done - r->t_submit;
        r->result->stats.kernel_launches = 0;
      } else {
        S->stats.failed += 1;
      }
      r->done = true;
      S->cv_done.notify_all();
      S->cv_work.notify_one();
    }
  }
}

}  // namespace

extern "C" {

ts_server *ts_server_new(int32_t device, uint64_t hbm_budget_bytes, uint32_t max_active) {
  std::unique_ptr<ts_server> S(new (std::nothrow) ts_server());
  if (!S) return nullptr;
  S->device = device;
  S->max_active = max_active ? max_active : 64;
  try {
    CUDA_TRY(cudaSetDevice(device));
    size_t free_b = 0, total_b = 0;
    CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    S->budget = hbm_budget_bytes ? hbm_budget_bytes : (uint64_t)(free_b / 2);
    CUDA_TRY(cudaStreamCreateWithFlags(&S->st, cudaStreamNonBlocking));
    CUDA_TRY(cudaStreamCreateWithFlags(&S->ust, cudaStreamNonBlocking));
    CUDA_TRY(cudaStreamCreateWithFlags(&S->cst, cudaStreamNonBlocking));
    CUDA_TRY(S->d_sess.alloc(S->max_active));
    CUDA_TRY(S->d_tabs.alloc(S->max_active));
    S->seg_cap = S->max_active * (kPhases + 1);
    for (auto &R : S->ring) {
      CUDA_TRY(cudaMallocHost((void **)&R.h, S->seg_cap * sizeof(Segment)));
      CUDA_TRY(cudaEventCreateWithFlags(&R.ev, cudaEventDisableTiming));
    }
  } catch (const Failure &) {
    ts_server_free(S.release());
    return nullptr;
  }
  for (uint32_t i = 0; i < S->max_active; ++i) S->free_slots.push_back(S->max_active - 1 - i);
  S->t0 = host_ms();
  S->driver = std::thread(server_driver, S.get());
  S->completer = std::thread(server_completer, S.get());
  const unsigned hc = std::max(1u, std::thread::hardware_concurrency());
  // half the host threads (at most eight) run pick chains: with many
  // requests waiting they, not the device, bound the server's throughput
  for (unsigned i = 0; i < std::min(8u, std::max(1u, hc / 2)); ++i) S->pickers.emplace_back(server_picker, S.get());
  return S.release();
}

void ts_server_free(ts_server *S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    S->cv_work.notify_all();
  }
  if (S->driver.joinable()) S->driver.join();  // drains every submitted request first
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop_completer = true;
    S->cv_complete.notify_all();
  }
  if (S->completer.joinable()) S->completer.join();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop_pickers = true;
    S->cv_pick.notify_all();
  }
  for (auto &t : S->pickers)
    if (t.joinable()) t.join();
  for (auto &kv : S->reqs) delete kv.second;
  if (S->st) cudaStreamSynchronize(S->st);
  for (auto &R : S->ring) {
    if (R.h) cudaFreeHost(R.h);
    if (R.ev) cudaEventDestroy(R.ev);
  }
  S->d_sess.reset();
  S->d_tabs.reset();
  if (S->st) cudaStreamDestroy(S->st);
  if (S->ust) cudaStreamDestroy(S->ust);
  if (S->cst) cudaStreamDestroy(S->cst);
  delete S;
}

const char *ts_server_last_error(const ts_server *S) { return S ? S->err.c_str() : "null server"; }

int ts_server_resolve_team(ts_server *S, uint32_t team_max_items, uint32_t full_max_items) {
  if (!S) return TS_ERR_NULL;
  std::lock_guard<std::mutex> lk(S->mu);
  S->team_max_items = team_max_items;
  S->team_full_max_items = full_max_items;
  return TS_OK;
}
int ts_server_tuning(ts_server *S, const ts_tuning *t) {
  if (!S || !t) return TS_ERR_NULL;
  return ts_server_resolve_team(S, t->team_max_items, t->team_full_max_items);
}

int ts_server_submit(ts_server *S, ts_session *s, uint64_t *ticket) {
  if (!S || !s || !ticket) return TS_ERR_NULL;
  if (s->consumed) {
    S->err = "session already consumed";
    return TS_ERR_STATE;
  }
  if (s->prm.device != S->device) {
    S->err = "session device differs from the server's";
    return TS_ERR_STATE;
  }
  std::unique_ptr<ServerReq> r(new (std::nothrow) ServerReq());
  if (!r) return TS_ERR_OUT_OF_MEMORY;
  r->s = new (std::nothrow) ts_session();
  if (!r->s) return TS_ERR_OUT_OF_MEMORY;
  *r->s = std::move(*s);
  s->consumed = true;
  s->err = "session handed to a server";
  r->t_submit = host_ms() - S->t0;
  r->c.reset(new RunCtx());
  try {
    RunCtx &c = *r->c;
    run_plan(r->s, c);  // host schedule, on the caller's thread
    c.items_async = true;
    if (cudaSuccess != c.pitems.alloc(c.items.size())) throw Failure{TS_ERR_CUDA, "pinned host memory"};
    if (!c.plan.empty()) server_pick_stage(*r);  // stage 0 here, the rest on a picker thread
  } catch (const Failure &f) {
    S->err = f.msg;
    return f.status;
  }
  r->bytes = r->c->dev_bytes + r->s->dev_bytes;
  const bool more = r->picked.load() < r->c->plan.size();
  r->picks_done = !more;
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->fatal) {
    S->err = "server stopped after a device error";
    return S->fatal;
  }
  r->ticket = S->next_ticket++;
  *ticket = r->ticket;
  S->reqs[r->ticket] = r.get();
  if (more) {
    S->to_pick.push_back(r.get());
    S->cv_pick.notify_one();
  }
  S->pending.push_back(r.release());
  S->n_pending.store((uint32_t)S->pending.size(), std::memory_order_relaxed);
  S->stats.submitted += 1;
  S->cv_work.notify_one();
  S->cv_picked.notify_all();  // a driver waiting on pickers admits it at once
  return TS_OK;
}

int ts_server_wait(ts_server *S, uint64_t ticket, ts_generated **out, ts_request_times *times) {
  if (!S || !out) return TS_ERR_NULL;
  *out = nullptr;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) {
    S->err = "unknown ticket";
    return TS_ERR_STATE;
  }
  ServerReq *r = it->second;
  S->cv_done.wait(lk, [&] { return r->done; });
  S->reqs.erase(it);
  lk.unlock();
  if (times) {
    times->submit_ms = r->t_submit;
    times->admit_ms = r->t_admit;
    times->done_ms = r->t_done;
  }
  const int status = r->status;
  if (status == TS_OK) {
    *out = r->result;
    r->result = nullptr;
  } else {
    std::lock_guard<std::mutex> lk2(S->mu);
    S->err = r->err;
  }
  delete r;
  return status;
}

int ts_server_done(ts_server *S, uint64_t ticket) {
  if (!S) return -1;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->reqs.find(ticket);
  if (it == S->reqs.end()) return -1;
  return it->second->done ? 1 : 0;
}

void ts_server_stats_get(ts_server *S, ts_server_stats *out) {
  if (!S || !out) return;
  std::lock_guard<std::mutex> lk(S->mu);
  *out = S->stats;
  out->budget_bytes = S->budget;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// CoordinateTransform (lib.rs:162-325) and the debug maps (ms.rs:604-653).
// ---------------------------------------------------------------------------
struct ts_transform {
  uint32_t W = 0, H = 0;
  std::vector<uint32_t> maps;  // (w, h) per original example
  std::vector<uint32_t> buf;   // (x, y, map) per output pixel
};

namespace {
constexpr uint32_t kTransformMagic = 0x12340001u;  // TRANSFORM_MAGIC, lib.rs:168
}

extern "C" {

ts_transform *ts_generated_coord_transform(const ts_generated *g) {
  if (!g) return nullptr;
  const_cast<ts_generated *>(g)->ensure_maps();
  ts_transform *t = new (std::nothrow) ts_transform();
  if (!t) return nullptr;
  t->W = g->W;
  t->H = g->H;
  t->maps = g->in_dims;
  t->buf = g->coord;
  return t;
}

void ts_transform_free(ts_transform *t) { delete t; }

void ts_transform_dims(const ts_transform *t, uint32_t *width, uint32_t *height, uint32_t *n_maps) {
  if (!t) return;
  if (width) *width = t->W;
  if (height) *height = t->H;
  if (n_maps) *n_maps = (uint32_t)(t->maps.size() / 2);
}

int ts_transform_map_dims(const ts_transform *t, uint32_t i, uint32_t *width, uint32_t *height) {
  if (!t || !width || !height) return TS_ERR_NULL;
  if ((size_t)i * 2 >= t->maps.size()) return TS_ERR_INDEX;
  *width = t->maps[2 * (size_t)i];
  *height = t->maps[2 * (size_t)i + 1];
  return TS_OK;
}

int ts_transform_write(const ts_transform *t, uint8_t *out, size_t capacity, size_t *written) {
  if (!t || !written) return TS_ERR_NULL;
  if (t->buf.size() != (size_t)t->W * t->H * 3) return TS_ERR_SIZE_MISMATCH;
  std::vector<uint32_t> words;
  words.reserve(4 + t->maps.size() + t->buf.size());
  words.push_back(kTransformMagic);
  words.push_back(t->W);
  words.push_back(t->H);
  words.push_back((uint32_t)(t->maps.size() / 2));
  words.insert(words.end(), t->maps.begin(), t->maps.end());
  words.insert(words.end(), t->buf.begin(), t->buf.end());
  *written = words.size() * 4;
  if (!out) return TS_OK;  // size query
  if (capacity < words.size() * 4) return TS_ERR_LIMIT;
  for (size_t i = 0; i < words.size(); ++i) {  // little-endian u32, as the reference writes on its targets
    out[4 * i] = (uint8_t)words[i];
    out[4 * i + 1] = (uint8_t)(words[i] >> 8);
    out[4 * i + 2] = (uint8_t)(words[i] >> 16);
    out[4 * i + 3] = (uint8_t)(words[i] >> 24);
  }
  return TS_OK;
}

int ts_transform_read(const uint8_t *data, size_t len, ts_transform **out) {
  if (!data || !out) return TS_ERR_NULL;
  *out = nullptr;
  size_t pos = 0;
  auto word = [&](uint32_t &v) {
    if (pos + 4 > len) return false;
    v = (uint32_t)data[pos] | ((uint32_t)data[pos + 1] << 8) | ((uint32_t)data[pos + 2] << 16) |
        ((uint32_t)data[pos + 3] << 24);
    pos += 4;
    return true;
  };
  uint32_t magic = 0, w = 0, h = 0, n = 0;
  if (!word(magic) || (magic >> 16) != 0x1234u || (magic & 0xffffu) != 0x1u) return TS_ERR_INVALID_RANGE;
  if (!word(w) || !word(h) || !word(n)) return TS_ERR_INVALID_RANGE;
  if ((uint64_t)n * 8 > len || (uint64_t)w * h * 12 > len) return TS_ERR_INVALID_RANGE;
  std::unique_ptr<ts_transform> t(new (std::nothrow) ts_transform());
  if (!t) return TS_ERR_OUT_OF_MEMORY;
  t->W = w;
  t->H = h;
  t->maps.resize((size_t)n * 2);
  for (auto &v : t->maps)
    if (!word(v)) return TS_ERR_INVALID_RANGE;
  t->buf.resize((size_t)w * h * 3);
  for (auto &v : t->buf)
    if (!word(v)) return TS_ERR_INVALID_RANGE;
  *out = t.release();
  return TS_OK;
}

int ts_transform_apply(const ts_transform *t, const ts_image_desc *sources, uint32_t n_sources, uint8_t *out_rgba,
                       int32_t device) {
  if (!t || !out_rgba || (n_sources && !sources)) return TS_ERR_NULL;
  const uint32_t n_maps = (uint32_t)(t->maps.size() / 2);
  // the sources pair with the original maps; extra sources are dropped, too
  // few are an error (lib.rs:183-198)
  if (std::min(n_sources, n_maps) != n_maps) return TS_ERR_MAPS_COUNT_MISMATCH;
  try {
    CUDA_TRY(cudaSetDevice(device));
    StreamGuard sg;
    CUDA_TRY(cudaStreamCreateWithFlags(&sg.s, cudaStreamNonBlocking));
    const cudaStream_t st = sg.s;
    std::vector<Image> maps(n_maps);
    std::vector<uint4> desc(std::max<uint32_t>(n_maps, 1));
    uint64_t texels = 0;
    for (uint32_t i = 0; i < n_maps; ++i) {
      if (!check_image(sources[i].rgba, sources[i].width, sources[i].height)) return TS_ERR_IMAGE;
      // load_image with the original size: CatmullRom resize if it differs
      maps[i] = load_image(copy_image(sources[i].rgba, sources[i].width, sources[i].height), true, t->maps[2 * i],
                           t->maps[2 * i + 1], st);
      desc[i] = make_uint4((uint32_t)texels, (uint32_t)(texels >> 32), maps[i].w, maps[i].h);
      texels += (uint64_t)maps[i].w * maps[i].h;
    }
    const size_t n = (size_t)t->W * t->H;
    DevBuf<uint32_t> d_tex, d_buf, d_out;
    DevBuf<uint4> d_desc;
    DevBuf<int> d_err;
    CUDA_TRY(d_tex.alloc_on(texels, st));
    CUDA_TRY(d_buf.alloc_on(t->buf.size(), st));
    CUDA_TRY(d_out.alloc_on(n, st));
    CUDA_TRY(d_desc.alloc_on(desc.size(), st));
    CUDA_TRY(d_err.alloc_on(1, st));
    for (uint32_t i = 0; i < n_maps; ++i)
      CUDA_TRY(cudaMemcpyAsync(d_tex.p + ((uint64_t)desc[i].y << 32 | desc[i].x), maps[i].px.data(),
                               maps[i].px.size(), cudaMemcpyHostToDevice, st));
    if (!t->buf.empty())
      CUDA_TRY(cudaMemcpyAsync(d_buf.p, t->buf.data(), t->buf.size() * 4, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_desc.p, desc.data(), desc.size() * sizeof(uint4), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemsetAsync(d_err.p, 0, sizeof(int), st));
    launch_transform_apply(d_buf.p, n, d_tex.p, d_desc.p, n_maps, d_out.p, d_err.p, st);
    CUDA_TRY(cudaGetLastError());
    int err = 0;
    if (n) CUDA_TRY(cudaMemcpyAsync(out_rgba, d_out.p, n * 4, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(&err, d_err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (err) return TS_ERR_INDEX;
  } catch (const Failure &f) {
    return f.status;
  }
  return TS_OK;
}

int ts_generated_debug_maps(const ts_generated *g, uint8_t *patch_id_rgba, uint8_t *map_id_rgba,
                            uint8_t *uncertainty_rgba, int32_t device) {
  if (!g || !patch_id_rgba || !map_id_rgba || !uncertainty_rgba) return TS_ERR_NULL;
  const_cast<ts_generated *>(g)->ensure_maps();
  try {
    CUDA_TRY(cudaSetDevice(device));
    StreamGuard sg;
    CUDA_TRY(cudaStreamCreateWithFlags(&sg.s, cudaStreamNonBlocking));
    const cudaStream_t st = sg.s;
    const size_t n = (size_t)g->W * g->H, nr = g->resolved.size();
    DevBuf<uint32_t> d_ids, d_flat, d_patch, d_map, d_unc;
    DevBuf<float> d_score;
    CUDA_TRY(d_ids.alloc_on(n * 2, st));
    CUDA_TRY(d_flat.alloc_on(nr, st));
    CUDA_TRY(d_score.alloc_on(nr, st));
    CUDA_TRY(d_patch.alloc_on(n, st));
    CUDA_TRY(d_map.alloc_on(n, st));
    CUDA_TRY(d_unc.alloc_on(n, st));
    if (n) CUDA_TRY(cudaMemcpyAsync(d_ids.p, g->ids.data(), n * 8, cudaMemcpyHostToDevice, st));
    if (nr) {
      CUDA_TRY(cudaMemcpyAsync(d_flat.p, g->resolved.data(), nr * 4, cudaMemcpyHostToDevice, st));
      CUDA_TRY(cudaMemcpyAsync(d_score.p, g->scores.data(), nr * 4, cudaMemcpyHostToDevice, st));
    }
    CUDA_TRY(cudaMemsetAsync(d_unc.p, 0, n * 4, st));
    launch_debug_maps(d_ids.p, n, d_flat.p, d_score.p, nr, d_patch.p, d_map.p, d_unc.p, st);
    CUDA_TRY(cudaGetLastError());
    if (n) {
      CUDA_TRY(cudaMemcpyAsync(patch_id_rgba, d_patch.p, n * 4, cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaMemcpyAsync(map_id_rgba, d_map.p, n * 4, cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaMemcpyAsync(uncertainty_rgba, d_unc.p, n * 4, cudaMemcpyDeviceToHost, st));
    }
    CUDA_TRY(cudaStreamSynchronize(st));
  } catch (const Failure &f) {
    return f.status;
  }
  return TS_OK;
}

}  // extern "C"
