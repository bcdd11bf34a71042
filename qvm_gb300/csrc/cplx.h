// cplx.h -- complex helpers for double2 / float2 amplitudes.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

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

// ---- double-float (FP32 pairs) complex arithmetic ------------------------------
//
// On this part the FP64 pipe runs at 1/64 of the FP32 rate.  Fused FP64 tile
// passes therefore hold their tile as double-float complex numbers (each
// component an unevaluated sum hi + lo of two floats, ~47 significant bits)
// and do the arithmetic on the FP32 pipe with error-free transformations
// (two-sum; two-product through fma), converting from and to the FP64 state
// at the tile's load and store.  `dfloat` tags that arithmetic; the state in
// HBM stays complex FP64.
struct dfloat {};
struct __align__(16) dfc {
  float rh, rl, ih, il;
};
template <>
struct CT<dfloat> {
  using C = dfc;
};

// float bits -> double bits of the same value (exact for normal floats and
// zero; float subnormals, below 1.2e-38, come out within 1.2e-38).
__device__ __forceinline__ unsigned long long df_f2d_bits(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
  const unsigned mag = u & 0x7FFFFFFFu;
  if (mag == 0) return sign;
  return sign | (((unsigned long long)mag + (896ull << 23)) << 29);
}
// Bit moves that compile for the host as well (the integer split below is
// checked against FP64 arithmetic on the CPU).
__host__ __device__ __forceinline__ unsigned df_fbits(float f) {
  unsigned u;
  memcpy(&u, &f, 4);
  return u;
}
__host__ __device__ __forceinline__ float df_bitsf(unsigned u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}
__host__ __device__ __forceinline__ unsigned long long df_dbits(double d) {
  unsigned long long u;
  memcpy(&u, &d, 8);
  return u;
}

// hi + lo as a double: both convert exactly by bit moves, then one FP64 add
// (an exact integer form of the rounded sum costs more ALU instructions than
// the add costs on the 1/64-rate FP64 pipe).
__device__ __forceinline__ double df_to_double(float hi, float lo) {
  return __longlong_as_double(df_f2d_bits(hi)) + __longlong_as_double(df_f2d_bits(lo));
}

// x -> (hi, lo) for 2^-74 <= |x| < 2^128 by integer operations and one
// int -> float conversion: hi is x truncated to 24 bits, lo = RN(x - hi) =
// RN(r) * 2^(e - 1075) with r the 29 low significand bits (the scale is a
// normal float in this range, so the product is exact).  Equal bit for bit to
// the FP64 form below; false outside the range.
__host__ __device__ __forceinline__ bool df_split_int(double x, float &hi, float &lo) {
  const unsigned long long u = df_dbits(x);
  const unsigned long long mag = u & 0x7FFFFFFFFFFFFFFFull;
  if (mag < (949ull << 52) || mag >= (1151ull << 52)) return false;
  const unsigned sign = (unsigned)(u >> 32) & 0x80000000u;
  hi = df_bitsf((unsigned)((mag >> 29) - (896ull << 23)) | sign);
  const unsigned r = (unsigned)(mag & ((1ull << 29) - 1ull));
  const unsigned e = (unsigned)(mag >> 52);
  const float scale = df_bitsf((e - 948u) << 23);  // 2^(e - 1075)
#ifdef __CUDA_ARCH__
  const float rf = __uint2float_rn(r);
#else
  const float rf = (float)r;  // round to nearest (the host's default mode)
#endif
  lo = r ? df_bitsf(df_fbits(rf * scale) | sign) : 0.f;
  return true;
}

// x -> (hi, lo): hi is x truncated to 24 bits by integer operations, lo the
// rounded remainder (one FP64 subtraction, exact, and one conversion) where
// the integer form does not apply.  |x| below 2^-126 goes entirely to lo.
// |x| must be below 2^128.
__device__ __forceinline__ void df_split(double x, float &hi, float &lo) {
  if (df_split_int(x, hi, lo)) return;
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned long long mag = u & 0x7FFFFFFFFFFFFFFFull;
  if (mag < (897ull << 52)) {
    hi = 0.f;
    lo = __double2float_rn(x);
    return;
  }
  const unsigned hb = (unsigned)((mag >> 29) - (896ull << 23)) | (unsigned)((u >> 32) & 0x80000000u);
  hi = __uint_as_float(hb);
  lo = __double2float_rn(x - __longlong_as_double(df_f2d_bits(hi)));
}
__device__ __forceinline__ dfc df_from_double2(double2 v) {
  dfc r;
  df_split(v.x, r.rh, r.rl);
  df_split(v.y, r.ih, r.il);
  return r;
}
// Exact-range conversion for op data (matrices, phase tables).
__device__ __forceinline__ dfc df_from_double2_any(double2 v) {
  dfc r;
  r.rh = __double2float_rn(v.x);
  r.rl = __double2float_rn(v.x - (double)r.rh);
  r.ih = __double2float_rn(v.y);
  r.il = __double2float_rn(v.y - (double)r.ih);
  return r;
}
__device__ __forceinline__ double2 df_to_double2(const dfc &v) {
  return make_double2(df_to_double(v.rh, v.rl), df_to_double(v.ih, v.il));
}

// Running double-float sums of complex products: (s, e) per component, s
// the exact two-sum of the leading product terms, e the low-order terms.
struct dfacc {
  float sr, er, si, ei;
};
__device__ __forceinline__ void df_acc_term(float &s, float &e, float ah, float al, float bh,
                                            float bl, bool neg) {
  float p = ah * bh;
  float q = fmaf(ah, bh, -p);
  q = fmaf(ah, bl, q);
  q = fmaf(al, bh, q);
  if (neg) {
    p = -p;
    q = -q;
  }
  const float t = s + p;
  const float bb = t - s;
  const float err = (s - (t - bb)) + (p - bb);
  s = t;
  e += err + q;
}
// acc += a * b
__device__ __forceinline__ void df_cmac(dfacc &acc, const dfc &a, const dfc &b) {
  df_acc_term(acc.sr, acc.er, a.rh, a.rl, b.rh, b.rl, false);
  df_acc_term(acc.sr, acc.er, a.ih, a.il, b.ih, b.il, true);
  df_acc_term(acc.si, acc.ei, a.rh, a.rl, b.ih, b.il, false);
  df_acc_term(acc.si, acc.ei, a.ih, a.il, b.rh, b.rl, false);
}
__device__ __forceinline__ dfc df_result(const dfacc &acc) {
  dfc r;
  r.rh = acc.sr + acc.er;
  r.rl = acc.er - (r.rh - acc.sr);
  r.ih = acc.si + acc.ei;
  r.il = acc.ei - (r.ih - acc.si);
  return r;
}
__device__ __forceinline__ dfc df_cmul(const dfc &a, const dfc &b) {
  dfacc acc{0.f, 0.f, 0.f, 0.f};
  df_cmac(acc, a, b);
  return df_result(acc);
}

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

// 16-byte asynchronous global -> shared copy (LDGSTS): every load of a tile
// is in flight at once without holding registers; wait_all completes them.
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

}  // namespace qvmg
