// Checks of the f64 primitives the neighbour weights use (ts_common.h):
//  - ts_div_markstein(a, b, __drcp_rn(b)) equals __ddiv_rn(a, b)
//  - ts_exp64 on the device equals ts_exp64 compiled for the host
//  - ts_exp64 stays within 2 ulp of CUDA's exp()
//  - the double-f32 weight (ts_weight_ff), when it decides, equals the
//    exact f64 weight, and decides for almost every input
//  - the integer mean (ts_add4_rn chain, ts_div_int_rn) of a 50-entry
//    distance list equals the __dadd_rn chain divided by __ddiv_rn
// Prints one JSON line of mismatch counts; exit status 0.
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <cmath>
#include <vector>
#include "ts_common.h"

__device__ const double g_tab[64] = {TS_EXP2_TABLE_VALUES};
__device__ const float g_tab_ff[128] = {TS_EXP2_FF_TABLE_VALUES};
static const double h_tab[64] = {TS_EXP2_TABLE_VALUES};

// weights of (a[i], b[i]) treated as (distance, mean): fast and exact
__global__ void k_weight(const double *a, const double *b, size_t n, float *w_fast, int *decided, float *w_exact) {
  __shared__ double tab[64];
  __shared__ float tab_ff[128];
  if (threadIdx.x < 64) tab[threadIdx.x] = g_tab[threadIdx.x];
  if (threadIdx.x < 128) tab_ff[threadIdx.x] = g_tab_ff[threadIdx.x];
  __syncthreads();
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float w = 0.0f;
    decided[i] = ts::ts_weight_ff(a[i], b[i], tab_ff, w) ? 1 : 0;
    w_fast[i] = w;
    const double q = ts::ts_div_markstein(a[i], b[i], __drcp_rn(b[i]));
    w_exact[i] = __double2float_rn(ts::ts_exp64(-1.0 * q, tab));
  }
}

__global__ void k_check(const double *a, const double *b, const double *x, size_t n, double *q_fast, double *q_ref,
                        double *e_dev, double *e_cuda) {
  __shared__ double tab[64];
  if (threadIdx.x < 64) tab[threadIdx.x] = g_tab[threadIdx.x];
  __syncthreads();
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    q_fast[i] = ts::ts_div_markstein(a[i], b[i], __drcp_rn(b[i]));
    q_ref[i] = __ddiv_rn(a[i], b[i]);
    e_dev[i] = ts::ts_exp64(x[i], tab);
    e_cuda[i] = exp(x[i]);
  }
}

// means of 50-entry lists: integer chain vs f64 chain
__global__ void k_mean_check(const double *d, size_t lists, double *m_int, double *m_ref) {
  for (size_t l = blockIdx.x * (size_t)blockDim.x + threadIdx.x; l < lists; l += (size_t)gridDim.x * blockDim.x) {
    uint64_t acc = 0;
    double ref = 0.0;
    for (int j = 0; j < 50; ++j) {
      const double v = d[l * 50 + j];
      acc = ts::ts_add4_rn(acc, ts::dbl_bits(v));
      for (int r = 0; r < 4; ++r) ref = __dadd_rn(ref, v);
    }
    m_int[l] = ts::bits_dbl(ts::ts_div_int_rn(acc, 200u));
    m_ref[l] = __ddiv_rn(ref, 200.0);
  }
}

static uint64_t bits(double v) { uint64_t u; memcpy(&u, &v, 8); return u; }

int main() {
  const size_t n = 1 << 22;
  std::vector<double> a(n), b(n), x(n);
  uint64_t s = 0x9e3779b97f4a7c15ULL;
  auto rnd = [&]() { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; };
  auto unif = [&]() { return (double)(rnd() >> 11) * (1.0 / 9007199254740992.0); };
  for (size_t i = 0; i < n; ++i) {
    // distances and means as the weights see them: lattice offsets over a
    // W x H plane, plus raw random operands
    if (i % 4 == 0) {
      const double W = 64 + (double)(rnd() % 4000), H = 64 + (double)(rnd() % 4000);
      const double dx = ((double)(int)(rnd() % 161) - 80) / W, dy = ((double)(int)(rnd() % 161) - 80) / H;
      a[i] = fma(dx, dx, dy * dy);
      b[i] = a[i] * (0.1 + 3.0 * unif()) + 1e-9;
    } else {
      a[i] = unif() * 8.0;
      b[i] = unif() * 2.0 + 1e-12;
    }
    x[i] = (i % 8 == 0) ? -700.0 * unif() : -16.0 * unif() * unif();
  }
  x[0] = 0.0; x[1] = -0.0; x[2] = -700.0; x[3] = -1e-300; x[4] = NAN;
  a[5] = 0.0; b[5] = 0.5;
  double *da, *db, *dx, *q1, *q2, *e1, *e2;
  cudaMalloc(&da, n * 8); cudaMalloc(&db, n * 8); cudaMalloc(&dx, n * 8);
  cudaMalloc(&q1, n * 8); cudaMalloc(&q2, n * 8); cudaMalloc(&e1, n * 8); cudaMalloc(&e2, n * 8);
  cudaMemcpy(da, a.data(), n * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(db, b.data(), n * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(dx, x.data(), n * 8, cudaMemcpyHostToDevice);
  k_check<<<1216, 256>>>(da, db, dx, n, q1, q2, e1, e2);
  cudaError_t err = cudaDeviceSynchronize();
  if (err != cudaSuccess) { printf("{\"cuda_error\": \"%s\"}\n", cudaGetErrorString(err)); return 1; }
  std::vector<double> hq1(n), hq2(n), he1(n), he2(n);
  cudaMemcpy(hq1.data(), q1, n * 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(hq2.data(), q2, n * 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(he1.data(), e1, n * 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(he2.data(), e2, n * 8, cudaMemcpyDeviceToHost);
  size_t div_bad = 0, host_div_bad = 0, exp_host_bad = 0, exp_ulp_bad = 0, f32_bad = 0;
  double max_ulp = 0;
  for (size_t i = 0; i < n; ++i) {
    if (bits(hq1[i]) != bits(hq2[i])) ++div_bad;
    if (bits(hq2[i]) != bits(a[i] / b[i])) ++host_div_bad;
    const double eh = ts::ts_exp64(x[i], h_tab);
    if (bits(eh) != bits(he1[i]) && !(eh != eh && he1[i] != he1[i])) ++exp_host_bad;
    if (he2[i] > 1e-300 && std::isfinite(he2[i])) {
      const double ulp = fabs(he1[i] - he2[i]) / (nextafter(he2[i], INFINITY) - he2[i]);
      if (ulp > max_ulp) max_ulp = ulp;
      if (ulp > 2.0) ++exp_ulp_bad;
      if ((float)he1[i] != (float)he2[i]) ++f32_bad;
    }
  }
  // weights: distance / mean pairs from lattice geometry
  std::vector<double> wd(n), wm(n);
  for (size_t i = 0; i < n; i += 50) {
    const double W = 16 + (double)(rnd() % 4096), H = 16 + (double)(rnd() % 4096);
    const int px = (int)(rnd() % (uint64_t)W), py = (int)(rnd() % (uint64_t)H);
    double sum = 0.0;
    const size_t m = (i + 50 <= n) ? 50 : n - i;
    for (size_t j = 0; j < m; ++j) {
      const int ox = (int)(rnd() % 81) - 40, oy = (int)(rnd() % 81) - 40;
      const double dx = (double)(px + ox) / W - (double)px / W, dy = (double)(py + oy) / H - (double)py / H;
      wd[i + j] = fma(dx, dx, dy * dy);
      for (int r = 0; r < 4; ++r) sum += wd[i + j];
    }
    for (size_t j = 0; j < m; ++j) wm[i + j] = sum / (double)(4 * m);
  }
  float *wf, *we;
  int *dec;
  cudaMalloc(&wf, n * 4); cudaMalloc(&we, n * 4); cudaMalloc(&dec, n * 4);
  cudaMemcpy(da, wd.data(), n * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(db, wm.data(), n * 8, cudaMemcpyHostToDevice);
  k_weight<<<1216, 256>>>(da, db, n, wf, dec, we);
  const size_t lists = n / 50;
  k_mean_check<<<1216, 256>>>(da, lists, q1, q2);
  err = cudaDeviceSynchronize();
  if (err != cudaSuccess) { printf("{\"cuda_error\": \"%s\"}\n", cudaGetErrorString(err)); return 1; }
  std::vector<float> hwf(n), hwe(n);
  std::vector<int> hdec(n);
  cudaMemcpy(hwf.data(), wf, n * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(hwe.data(), we, n * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(hdec.data(), dec, n * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(hq1.data(), q1, lists * 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(hq2.data(), q2, lists * 8, cudaMemcpyDeviceToHost);
  size_t mean_bad = 0;
  for (size_t l = 0; l < lists; ++l)
    if (bits(hq1[l]) != bits(hq2[l])) ++mean_bad;
  size_t w_bad = 0, w_undecided = 0;
  for (size_t i = 0; i < n; ++i) {
    if (!hdec[i]) { ++w_undecided; continue; }
    uint32_t a, b;
    memcpy(&a, &hwf[i], 4); memcpy(&b, &hwe[i], 4);
    if (a != b) ++w_bad;
  }
  printf("{\"n\": %zu, \"div_mismatch\": %zu, \"host_div_mismatch\": %zu, \"exp_host_device_mismatch\": %zu, "
         "\"exp_over_2ulp\": %zu, \"exp_max_ulp\": %.3f, \"exp_f32_differs_from_cuda\": %zu, "
         "\"weight_mismatch\": %zu, \"weight_undecided\": %zu, \"mean_mismatch\": %zu}\n",
         n, div_bad, host_div_bad, exp_host_bad, exp_ulp_bad, max_ulp, f32_bad, w_bad, w_undecided, mean_bad);
  return 0;
}
