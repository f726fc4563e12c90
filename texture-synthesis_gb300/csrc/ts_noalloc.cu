// ts_noalloc.cu — ts_image_pyramid_noalloc: the image pyramid of
// ts_image_pyramid for callers that cannot allocate device memory.
//
// Who needs it: code that must not call cudaMalloc / cudaFree while it runs
// -- a renderer or game engine that owns a fixed device-memory budget and
// hands every byte to its own allocator, a framework whose caching
// allocator has reserved the device, or code on a latency-critical path
// where an allocation may synchronise the device.  Such a caller passes its
// own input and output buffers; the intermediate data of the resize passes
// (an f32 image, the downscaled image, the filter taps) lives in one
// file-scope device array of fixed size, kNoAllocScratchBytes, which every
// GPU that loads the library holds until the process exits.  The call copies
// nothing from host memory with cudaMemcpy: the taps travel as kernel
// parameters, so enqueueing never waits for the caller's stream.
#include <string.h>

#include <algorithm>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/tsgpu.h"
#include "ts_kernels.cuh"
#include "ts_resample.h"

namespace {

// Largest image: width * height <= 1024 * 1024 and each side <= 4096.
constexpr uint64_t kMaxPixels = TS_NOALLOC_MAX_PIXELS;
constexpr uint32_t kMaxSideNoAlloc = TS_NOALLOC_MAX_SIDE;
constexpr uint32_t kMaxLevels = TS_NOALLOC_MAX_LEVELS;
// One axis of one resize: at most kMaxSideNoAlloc outputs, and at most
// 8 weights per output when upscaling (Gaussian support 3) or
// (len / p) * (6p + 2) <= 7 * len when downscaling by p >= 2.
constexpr size_t kTapsEntries = kMaxSideNoAlloc;  // {left, count, offset, 0}
constexpr size_t kWeightCap = 8 * kMaxSideNoAlloc;
// The f32 RGBA intermediate holds w x (h/p) or (w/p) x h texels (p >= 2),
// the downscaled RGBA8 image (w/p) x (h/p) texels.
constexpr size_t kTmpBytes = kMaxPixels / 2 * 16;
constexpr size_t kSmallBytes = kMaxPixels / 4 * 4;
constexpr size_t kTapsBytes = kTapsEntries * 16;   // one axis
constexpr size_t kWeightBytes = kWeightCap * 4;    // one axis
constexpr size_t kNoAllocScratchBytes = kTmpBytes + kSmallBytes + 2 * (kTapsBytes + kWeightBytes);
static_assert(kNoAllocScratchBytes == 9830400, "scratch size as documented in tsgpu.h (9.4 MiB)");

// The scratch.  In host code this name is a host-side stand-in, not a
// device address: host code passes the address cudaGetSymbolAddress returns.
static __device__ __align__(256) unsigned char g_pyramid_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;              // guards the set-up and the host tap buffers
unsigned char *g_scratch[kMaxDevices] = {};
uint32_t g_host_taps[2][kTapsEntries * 4];
float g_host_weights[2][kWeightCap];

// The filter taps reach the device inside kernel parameters, which a launch
// copies when it is made: no host-to-device copy from pageable memory (such
// a copy may wait for the stream), and the host buffers above are free for
// the next resize as soon as the launch returns.  32,004 bytes of
// parameters, within the 32,764 bytes a launch may carry.
constexpr uint32_t kPutWords = 8000;
struct PutWords {
  uint32_t n;
  uint32_t w[kPutWords];
};
PutWords g_put;  // guarded by g_mutex

__global__ void k_put_words(uint32_t *dst, const __grid_constant__ PutWords p) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += gridDim.x * blockDim.x) dst[i] = p.w[i];
}

// Stores n words from host memory at dst (device) in launches of at most
// kPutWords words each.
cudaError_t put_words(uint32_t *dst, const void *src, size_t n, cudaStream_t st) {
  const uint32_t *w = (const uint32_t *)src;
  for (size_t i = 0; i < n; i += kPutWords) {
    const uint32_t c = (uint32_t)std::min<size_t>(kPutWords, n - i);
    g_put.n = c;
    memcpy(g_put.w, w + i, (size_t)c * 4);
    k_put_words<<<(c + 255) / 256, 256, 0, st>>>(dst + i, g_put);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Scratch regions, offsets from the start of the array.
constexpr size_t kOffTmp = 0;
constexpr size_t kOffSmall = kOffTmp + kTmpBytes;
constexpr size_t kOffTaps0 = kOffSmall + kSmallBytes;
constexpr size_t kOffWeights0 = kOffTaps0 + kTapsBytes;
constexpr size_t kOffTaps1 = kOffWeights0 + kWeightBytes;
constexpr size_t kOffWeights1 = kOffTaps1 + kTapsBytes;

// imageops::resize of src (w x h) into dst (nw x nh), both device RGBA8,
// with the scratch at `base`; enqueued on `st`.  Returns a ts_status.
int resize_noalloc(unsigned char *base, const uint8_t *src, uint32_t w, uint32_t h, uint8_t *dst, uint32_t nw,
                   uint32_t nh, ts::Filter f, cudaStream_t st) {
  if (nw == 0 || nh == 0) return TS_OK;
  if (nw > kTapsEntries || nh > kTapsEntries) return TS_ERR_LIMIT;
  if ((uint64_t)w * nh * 16 > kTmpBytes) return TS_ERR_LIMIT;
  const long wv = ts::axis_taps_into(f, h, nh, g_host_taps[0], g_host_weights[0], kWeightCap);
  const long wh = ts::axis_taps_into(f, w, nw, g_host_taps[1], g_host_weights[1], kWeightCap);
  if (wv < 0 || wh < 0) return TS_ERR_LIMIT;
  if (put_words((uint32_t *)(base + kOffTaps0), g_host_taps[0], (size_t)nh * 4, st) != cudaSuccess ||
      put_words((uint32_t *)(base + kOffTaps1), g_host_taps[1], (size_t)nw * 4, st) != cudaSuccess ||
      put_words((uint32_t *)(base + kOffWeights0), g_host_weights[0], (size_t)wv, st) != cudaSuccess ||
      put_words((uint32_t *)(base + kOffWeights1), g_host_weights[1], (size_t)wh, st) != cudaSuccess)
    return TS_ERR_CUDA;
  float *tmp = (float *)(base + kOffTmp);
  // the f32 image starts at zero, as a fresh buffer does in ts_image_pyramid
  if (cudaMemsetAsync(tmp, 0, (size_t)w * nh * 16, st) != cudaSuccess) return TS_ERR_CUDA;
  if (h > 0)
    ts::launch_resize_v(src, w, h, tmp, nh, (const uint4 *)(base + kOffTaps0), (const float *)(base + kOffWeights0),
                        st);
  if (w > 0) {
    ts::launch_resize_h(tmp, w, nh, dst, nw, (const uint4 *)(base + kOffTaps1),
                        (const float *)(base + kOffWeights1), st);
  } else if (cudaMemsetAsync(dst, 0, (size_t)nw * nh * 4, st) != cudaSuccess) {
    return TS_ERR_CUDA;
  }
  // no error was pending when the call began, so this one is the resize's
  return cudaGetLastError() == cudaSuccess ? TS_OK : TS_ERR_CUDA;
}

}  // namespace

extern "C" int ts_image_pyramid_noalloc(const uint8_t *d_rgba, uint32_t width, uint32_t height, uint32_t levels,
                                        uint8_t *d_out, void *stream) {
  if (!d_rgba || !d_out) return TS_ERR_NULL;
  if (width == 0 || height == 0) return TS_ERR_IMAGE;
  if (width > kMaxSideNoAlloc || height > kMaxSideNoAlloc || (uint64_t)width * height > kMaxPixels ||
      levels > kMaxLevels)
    return TS_ERR_LIMIT;
  // An error left by the caller's own work stays theirs: report it without
  // clearing it, and enqueue nothing.
  if (cudaPeekAtLastError() != cudaSuccess) return TS_ERR_CUDA;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return TS_ERR_CUDA;
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch[dev]) {
    // once per device, with that device current: the device address of the
    // scratch array (the first call on a device must precede stream capture)
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_pyramid_scratch) != cudaSuccess || !p) return TS_ERR_CUDA;
    g_scratch[dev] = (unsigned char *)p;
  }
  unsigned char *base = g_scratch[dev];
  const uint32_t nl = levels == 0 ? 1 : levels;
  const size_t sz = (size_t)width * height * 4;
  // the last level is the image itself
  if (cudaMemcpyAsync(d_out + (size_t)(nl - 1) * sz, d_rgba, sz, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return TS_ERR_CUDA;
  const uint8_t *orig = d_out + (size_t)(nl - 1) * sz;
  uint8_t *small = base + kOffSmall;
  for (uint32_t l = 0; l + 1 < nl; ++l) {
    const uint32_t p = 1u << (nl - 1 - l);
    const uint32_t sw = width / p, sh = height / p;
    uint8_t *lev = d_out + (size_t)l * sz;
    if (sw == 0 || sh == 0) {  // a zero-sized intermediate gives a zero level
      if (cudaMemsetAsync(lev, 0, sz, st) != cudaSuccess) return TS_ERR_CUDA;
      continue;
    }
    int rc = resize_noalloc(base, orig, width, height, small, sw, sh, ts::kGaussian, st);
    if (rc == TS_OK) rc = resize_noalloc(base, small, sw, sh, lev, width, height, ts::kGaussian, st);
    if (rc != TS_OK) return rc;
  }
  return TS_OK;
}
