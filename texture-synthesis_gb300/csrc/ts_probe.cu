// ts_probe.cu — the gather ceiling that the cost kernels are measured against.
//
// The cost loop (better_match, ms.rs:1225-1288) reads, for every candidate,
// the k example texels at the candidate's source plus the item's neighbour
// offsets: 32-bit gathers from an example level that stays in L2.  Neither
// the HBM copy bandwidth nor a dense-GEMM rate bounds that; what does is how
// many such gathers the SMs' load path (L1, then L2) can serve.  This file
// measures it with kernels that do nothing but those gathers, at full
// occupancy:
//
//   patch   each thread takes a pseudo-random centre in the table and reads
//           the texels at centre + offset_j for the k offsets nearest the
//           origin, (d^2, dy, dx) order, four or eight loads in flight
//           (the cost loop's access shape, without its LUT work and early
//           exit);
//   random  each thread reads independent pseudo-random texels, four or
//           eight in flight (no spatial locality: the L2 gather rate).
// Each is timed at both depths and the faster is kept.
//
// The table is allocated and filled here, sized by the caller (the example
// level of the workload being measured).  Measurement only: no counterpart
// in the reference.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "tsgpu.h"

namespace {

constexpr int kProbeThreads = 256;
constexpr int kProbeMaxK = 256;
constexpr int kProbeRadius = 12;  // the table keeps this border around every centre

__device__ __forceinline__ uint32_t mix32(uint32_t v) {
  v ^= v >> 16;
  v *= 0x7feb352du;
  v ^= v >> 15;
  v *= 0x846ca68bu;
  v ^= v >> 16;
  return v;
}

template <int ILP>
__global__ void __launch_bounds__(kProbeThreads) k_gather_patch(const uint32_t *table, uint32_t pitch, uint32_t cw,
                                                                uint32_t ch, const int32_t *lin_g, uint32_t k,
                                                                uint32_t iters, uint32_t *sink) {
  __shared__ int32_t lin[kProbeMaxK];
  for (uint32_t i = threadIdx.x; i < k; i += blockDim.x) lin[i] = lin_g[i];
  __syncthreads();
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t acc = 0;
  for (uint32_t it = 0; it < iters; ++it) {
    const uint32_t h = mix32(tid * 0x9e3779b9u + it * 0x85ebca6bu + 0x632be5abu);
    const uint32_t cx = kProbeRadius + (h & 0xffffu) % cw, cy = kProbeRadius + (h >> 16) % ch;
    const uint32_t *base = table + (size_t)cy * pitch + cx;
    uint32_t j = 0;
    for (; j + ILP <= k; j += ILP) {
      uint32_t t[ILP];
#pragma unroll
      for (int u = 0; u < ILP; ++u) t[u] = __ldg(base + lin[j + u]);
#pragma unroll
      for (int u = 0; u < ILP; ++u) acc += t[u];
    }
    for (; j < k; ++j) acc += __ldg(base + lin[j]);
  }
  sink[tid] = acc;
}

template <int ILP>
__global__ void __launch_bounds__(kProbeThreads) k_gather_random(const uint32_t *table, uint32_t words,
                                                                 uint32_t loads, uint32_t *sink) {
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t acc = 0, h = mix32(tid + 0x51ed270bu);
  for (uint32_t i = 0; i < loads; i += ILP) {
    uint32_t t[ILP];
#pragma unroll
    for (int u = 0; u < ILP; ++u) {
      h = mix32(h + (uint32_t)u);
      t[u] = __ldg(table + h % words);
    }
#pragma unroll
    for (int u = 0; u < ILP; ++u) acc += t[u];
  }
  sink[tid] = acc;
}

__global__ void k_fill(uint32_t *p, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    p[i] = (uint32_t)i * 2654435761u;
}

// Best of `reps` timed launches (after one warm-up), in ms.
template <typename F>
cudaError_t best_ms(F &&launch, int reps, cudaStream_t st, float &best) {
  cudaEvent_t e0, e1;
  cudaError_t err = cudaEventCreate(&e0);
  if (err != cudaSuccess) return err;
  err = cudaEventCreate(&e1);
  if (err != cudaSuccess) {
    cudaEventDestroy(e0);
    return err;
  }
  best = 1e30f;
  launch();
  for (int r = 0; r < reps && err == cudaSuccess; ++r) {
    cudaEventRecord(e0, st);
    launch();
    cudaEventRecord(e1, st);
    err = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    if (err == cudaSuccess) best = std::min(best, ms);
  }
  if (err == cudaSuccess) err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return err;
}

}  // namespace

extern "C" int ts_measure_gather_peak(int32_t device, uint32_t width, uint32_t height, uint32_t k, int32_t reps,
                                      ts_gather_peak *out) {
  if (!out) return TS_ERR_NULL;
  if (width == 0 || height == 0 || k == 0 || k > kProbeMaxK || width > 16384 || height > 16384)
    return TS_ERR_INVALID_RANGE;
  if (cudaSetDevice(device) != cudaSuccess) return TS_ERR_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return TS_ERR_CUDA;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gather_patch<8>, kProbeThreads, 0) != cudaSuccess)
    return TS_ERR_CUDA;
  const uint32_t blocks = (uint32_t)(sms * std::max(per_sm, 1));
  const uint32_t threads = blocks * kProbeThreads;
  // the nearest k offsets, (d^2, dy, dx) ascending, as texel offsets
  const uint32_t pitch = width + 2 * kProbeRadius;
  const size_t words = (size_t)pitch * (height + 2 * kProbeRadius);
  std::vector<int32_t> offs;
  std::vector<std::pair<int, std::pair<int, int>>> all;
  for (int dy = -kProbeRadius; dy <= kProbeRadius; ++dy)
    for (int dx = -kProbeRadius; dx <= kProbeRadius; ++dx) all.push_back({dx * dx + dy * dy, {dy, dx}});
  std::sort(all.begin(), all.end());
  for (uint32_t j = 0; j < k; ++j) offs.push_back(all[j].second.first * (int32_t)pitch + all[j].second.second);

  uint32_t *table = nullptr, *sink = nullptr;
  int32_t *lin = nullptr;
  cudaStream_t st = nullptr;
  int rc = TS_OK;
  float patch_ms = 0.0f, rand_ms = 0.0f;
  // a launch reads about 2 GB of texels: long enough to time, short enough to repeat
  const uint32_t iters = std::max(1u, (uint32_t)(2e9 / 4.0 / k / threads));
  const uint32_t loads = std::max(8u, (uint32_t)(1e9 / 4.0 / threads) & ~7u);
  do {
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&table, words * 4) != cudaSuccess || cudaMalloc(&sink, (size_t)threads * 4) != cudaSuccess ||
        cudaMalloc(&lin, k * 4) != cudaSuccess) {
      rc = TS_ERR_CUDA;
      break;
    }
    k_fill<<<sms * 4, 256, 0, st>>>(table, words);
    if (cudaMemcpyAsync(lin, offs.data(), k * 4, cudaMemcpyHostToDevice, st) != cudaSuccess) {
      rc = TS_ERR_CUDA;
      break;
    }
    // four and eight loads in flight per thread; the faster of the two
    auto patch4 = [&] { k_gather_patch<4><<<blocks, kProbeThreads, 0, st>>>(table, pitch, width, height, lin, k, iters, sink); };
    auto patch8 = [&] { k_gather_patch<8><<<blocks, kProbeThreads, 0, st>>>(table, pitch, width, height, lin, k, iters, sink); };
    auto rnd4 = [&] { k_gather_random<4><<<blocks, kProbeThreads, 0, st>>>(table, (uint32_t)words, loads, sink); };
    auto rnd8 = [&] { k_gather_random<8><<<blocks, kProbeThreads, 0, st>>>(table, (uint32_t)words, loads, sink); };
    float p4 = 0, p8 = 0, r4 = 0, r8 = 0;
    if (best_ms(patch4, std::max(1, reps), st, p4) != cudaSuccess ||
        best_ms(patch8, std::max(1, reps), st, p8) != cudaSuccess ||
        best_ms(rnd4, std::max(1, reps), st, r4) != cudaSuccess ||
        best_ms(rnd8, std::max(1, reps), st, r8) != cudaSuccess) {
      rc = TS_ERR_CUDA;
      break;
    }
    patch_ms = std::min(p4, p8);
    rand_ms = std::min(r4, r8);
    out->patch_ilp = p8 < p4 ? 8 : 4;
    out->random_ilp = r8 < r4 ? 8 : 4;
  } while (false);
  if (st) cudaStreamSynchronize(st);
  cudaFree(table);
  cudaFree(sink);
  cudaFree(lin);
  if (st) cudaStreamDestroy(st);
  if (rc != TS_OK) return rc;
  out->patch_gbs = (double)threads * iters * k * 4.0 / (patch_ms * 1e-3) / 1e9;
  out->random_gbs = (double)threads * loads * 4.0 / (rand_ms * 1e-3) / 1e9;
  out->table_bytes = (double)words * 4.0;
  out->threads = threads;
  out->patch_ms = patch_ms;
  out->random_ms = rand_ms;
  return TS_OK;
}
