// cplx.h -- complex helpers for double2 / float2 amplitudes.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace qvmg {

template <typename T>
struct CT;
template <>
struct CT<double> {
  using C = double2;
  static __host__ __device__ __forceinline__ C make(double x, double y) {
    return make_double2(x, y);
  }
};
template <>
struct CT<float> {
  using C = float2;
  static __host__ __device__ __forceinline__ C make(float x, float y) {
    return make_float2(x, y);
  }
};

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// acc += a * b
__device__ __forceinline__ void cmac(double2 &acc, double2 a, double2 b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
__device__ __forceinline__ void cmac(float2 &acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
}
// acc += r * b with a real coefficient r
__device__ __forceinline__ void rmac(double2 &acc, double r, double2 b) {
  acc.x = fma(r, b.x, acc.x);
  acc.y = fma(r, b.y, acc.y);
}
__device__ __forceinline__ void rmac(float2 &acc, float r, float2 b) {
  acc.x = fmaf(r, b.x, acc.x);
  acc.y = fmaf(r, b.y, acc.y);
}

// inject-bit (src/utilities.lisp:243-255): insert a 0 at bit position q.
__host__ __device__ __forceinline__ uint64_t inject0(uint64_t x, int q) {
  uint64_t lo = x & ((1ull << q) - 1ull);
  return ((x >> q) << (q + 1)) | lo;
}

// ---- FP64-accurate probabilities of FP32 amplitudes --------------------------
__device__ __forceinline__ double amp_prob(double2 v) { return fma(v.x, v.x, v.y * v.y); }

// Two-sum of a float into (hi, lo).
__device__ __forceinline__ void df_add(float &hi, float &lo, float x) {
  float s = hi + x;
  float bp = s - hi;
  float e = (hi - (s - bp)) + (x - bp);
  hi = s;
  lo += e;
}

// Add |v|^2 of an FP32 amplitude into (hi, lo) without rounding the
// squares: x*x = p + e exactly with e = fma(x, x, -p).  The error terms of
// the squares and of the two-sums are gathered in lo.
__device__ __forceinline__ void df_add_prob(float &hi, float &lo, float2 v) {
  float pr = v.x * v.x, er = fmaf(v.x, v.x, -pr);
  float pi = v.y * v.y, ei = fmaf(v.y, v.y, -pi);
  float s = pr + pi;
  float bp = s - pr;
  float es = (pr - (s - bp)) + (pi - bp);
  df_add(hi, lo, s);
  lo += (er + ei) + es;
}

// |v|^2 as a double for an FP32 amplitude: exact squares, rounded once.
__device__ __forceinline__ double prob_f64(float2 v) {
  float hi = 0.f, lo = 0.f;
  df_add_prob(hi, lo, v);
  return (double)hi + (double)lo;
}
__device__ __forceinline__ double prob_f64(double2 v) { return fma(v.x, v.x, v.y * v.y); }


}  // namespace qvmg
