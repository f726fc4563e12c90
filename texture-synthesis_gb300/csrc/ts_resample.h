// ts_resample.h — filter taps of the image crate's separable resize
// (image 0.23.12 imageops::sample::{resize, vertical_sample,
// horizontal_sample}), which the reference calls to build its pyramids
// (img_pyramid.rs:27-32) and to resize inputs (utils.rs:67-72).
//
// For every output index the crate takes the input interval
// [floor(c - s), ceil(c + s)) around the centre c = (o + 0.5) * ratio, with
// s = support * max(ratio, 1), clamped to the image, evaluates the kernel at
// (i - (c - 0.5)) / max(ratio, 1) and normalises the weights by their sum.
// All arithmetic is f32, evaluated in that order.
#pragma once
#include <math.h>
#include <stdint.h>

#include <vector>

namespace ts {

enum Filter { kNearest = 0, kTriangle = 1, kCatmullRom = 2, kGaussian = 3 };

inline float filter_support(Filter f) {
  switch (f) {
    case kTriangle: return 1.0f;
    case kCatmullRom: return 2.0f;
    case kGaussian: return 3.0f;
    default: return 0.0f;
  }
}

// gaussian_kernel: the Gaussian with standard deviation 0.5.
inline float gaussian_kernel(float x) {
  const float r = 0.5f;
  const float norm = 1.0f / (sqrtf(2.0f * 3.14159265358979323846f) * r);
  return norm * expf(-(x * x) / (2.0f * (r * r)));
}

inline float triangle_kernel(float x) {
  const float a = fabsf(x);
  return a < 1.0f ? 1.0f - a : 0.0f;
}

// catmullrom_kernel = cubic_bc(b = 0, c = 0.5, x).
inline float catmullrom_kernel(float x) {
  const float b = 0.0f, c = 0.5f;
  const float a = fabsf(x);
  float k;
  if (a < 1.0f) {
    k = (12.0f - 9.0f * b - 6.0f * c) * (a * a * a) + (-18.0f + 12.0f * b + 6.0f * c) * (a * a) + (6.0f - 2.0f * b);
  } else if (a < 2.0f) {
    k = (-b - 6.0f * c) * (a * a * a) + (6.0f * b + 30.0f * c) * (a * a) + (-12.0f * b - 48.0f * c) * a +
        (8.0f * b + 24.0f * c);
  } else {
    k = 0.0f;
  }
  return k / 6.0f;
}

inline float box_kernel(float x) { return (x >= -0.5f && x < 0.5f) ? 1.0f : 0.0f; }

inline float filter_eval(Filter f, float x) {
  switch (f) {
    case kTriangle: return triangle_kernel(x);
    case kCatmullRom: return catmullrom_kernel(x);
    case kGaussian: return gaussian_kernel(x);
    default: return box_kernel(x);
  }
}

struct Taps {
  std::vector<uint32_t> left, count, offset;  // per output index
  std::vector<float> weights;
};

// imageops::blur's kernel (image 0.23.12 sample.rs gaussian): the Gaussian
// with standard deviation r, support 2r.
inline float gaussian_sigma(float x, float r) {
  const float norm = 1.0f / (sqrtf(2.0f * 3.14159265358979323846f) * r);
  return norm * expf(-(x * x) / (2.0f * (r * r)));
}

// Taps along one axis of length in_len resampled to out_len with kernel k of
// the given support.
template <typename K>
inline Taps axis_taps_k(float support, K k, uint32_t in_len, uint32_t out_len) {
  Taps t;
  t.left.resize(out_len);
  t.count.resize(out_len);
  t.offset.resize(out_len);
  if (in_len == 0) return t;  // every output is zero: no taps
  const float ratio = (float)in_len / (float)out_len;
  const float sratio = ratio < 1.0f ? 1.0f : ratio;
  const float src_support = support * sratio;
  for (uint32_t o = 0; o < out_len; ++o) {
    float c = ((float)o + 0.5f) * ratio;
    int64_t left = (int64_t)floorf(c - src_support);
    if (left < 0) left = 0;
    if (left > (int64_t)in_len - 1) left = (int64_t)in_len - 1;
    int64_t right = (int64_t)ceilf(c + src_support);
    if (right < left + 1) right = left + 1;
    if (right > (int64_t)in_len) right = (int64_t)in_len;
    c = c - 0.5f;
    const size_t base = t.weights.size();
    float sum = 0.0f;
    for (int64_t i = left; i < right; ++i) {
      const float w = k(((float)i - c) / sratio);
      t.weights.push_back(w);
      sum += w;
    }
    for (size_t i = base; i < t.weights.size(); ++i) t.weights[i] /= sum;
    t.left[o] = (uint32_t)left;
    t.count[o] = (uint32_t)(right - left);
    t.offset[o] = (uint32_t)base;
  }
  return t;
}

inline Taps axis_taps(Filter f, uint32_t in_len, uint32_t out_len) {
  return axis_taps_k(filter_support(f), [f](float x) { return filter_eval(f, x); }, in_len, out_len);
}

// imageops::blur (sigma <= 0 means 1): the resize passes at the same size.
inline Taps blur_taps(uint32_t len, float sigma) {
  const float r = sigma <= 0.0f ? 1.0f : sigma;
  return axis_taps_k(2.0f * r, [r](float x) { return gaussian_sigma(x, r); }, len, len);
}

// axis_taps written into caller storage: left/count/offset per output index
// packed as {left, count, offset, 0} in `taps4` (out_len entries) and the
// weights in `weights`.  Returns the weight count, or -1 if more than
// `weight_cap` weights would be needed.  Same values as axis_taps.
inline long axis_taps_into(Filter f, uint32_t in_len, uint32_t out_len, uint32_t *taps4, float *weights,
                           size_t weight_cap) {
  for (uint32_t o = 0; o < out_len; ++o) {
    taps4[4 * o] = 0;
    taps4[4 * o + 1] = 0;
    taps4[4 * o + 2] = 0;
    taps4[4 * o + 3] = 0;
  }
  if (in_len == 0) return 0;
  const float ratio = (float)in_len / (float)out_len;
  const float sratio = ratio < 1.0f ? 1.0f : ratio;
  const float src_support = filter_support(f) * sratio;
  size_t nw = 0;
  for (uint32_t o = 0; o < out_len; ++o) {
    float c = ((float)o + 0.5f) * ratio;
    int64_t left = (int64_t)floorf(c - src_support);
    if (left < 0) left = 0;
    if (left > (int64_t)in_len - 1) left = (int64_t)in_len - 1;
    int64_t right = (int64_t)ceilf(c + src_support);
    if (right < left + 1) right = left + 1;
    if (right > (int64_t)in_len) right = (int64_t)in_len;
    c = c - 0.5f;
    if (nw + (size_t)(right - left) > weight_cap) return -1;
    const size_t base = nw;
    float sum = 0.0f;
    for (int64_t i = left; i < right; ++i) {
      const float w = filter_eval(f, ((float)i - c) / sratio);
      weights[nw++] = w;
      sum += w;
    }
    for (size_t i = base; i < nw; ++i) weights[i] /= sum;
    taps4[4 * o] = (uint32_t)left;
    taps4[4 * o + 1] = (uint32_t)(right - left);
    taps4[4 * o + 2] = (uint32_t)base;
  }
  return (long)nw;
}

}  // namespace ts
