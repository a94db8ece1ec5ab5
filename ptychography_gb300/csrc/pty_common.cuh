// Common device helpers for the GB300 ptychography engine.
//
// Complex numbers are float2 (interleaved re/im, the layout of NumPy
// complex64 and torch.complex64).  Accumulations that the reference performs
// over many frames (the overlap denominators, the modulus / convergence error
// sums) use a float-float pair ("ff": hi + lo, about 48 significand bits).
// GB300's FP64 pipe runs at roughly 1/60 of its FP32 rate, so an FP64 add per
// (pixel, frame) term would dominate the iteration; the pair keeps FP64-class
// accuracy at FP32 throughput and is converted to IEEE double once per output.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define PTY_DEV __device__ __forceinline__
#define PTY_HD __host__ __device__ __forceinline__

// ---------------------------------------------------------------- complex
// Complex additions, subtractions and real scalings issue as one packed
// FP32x2 instruction (add / sub / mul .rn.f32x2, sm_100 and later) instead of
// two scalar ones: the FFT butterflies are mostly such operations and the
// frame kernels are bound by instruction issue (measured on the 256^2 Pmod_7
// kernel: 18 % fewer warp instructions, 4 % less time).  Each lane rounds as
// the scalar add.rn / sub.rn / mul.rn does; the compiler can no longer
// contract a packed product into a following addition (one FMA), so results
// may differ from the scalar forms (PTY_PACKED_F32X2=0) in the last bit.
#ifndef PTY_PACKED_F32X2
#define PTY_PACKED_F32X2 1
#endif
#if PTY_PACKED_F32X2
PTY_DEV unsigned long long f2_pack(float2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
PTY_DEV float2 f2_unpack(unsigned long long r) {
  float2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}
PTY_DEV float2 cadd(float2 a, float2 b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(r);
}
PTY_DEV float2 csub(float2 a, float2 b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(r);
}
#else
PTY_DEV float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
PTY_DEV float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
#endif
PTY_DEV float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
PTY_DEV float2 cmulc(float2 a, float2 b) {
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
#if PTY_PACKED_F32X2
PTY_DEV float2 cscale(float2 a, float s) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(make_float2(s, s))));
  return f2_unpack(r);
}
#else
PTY_DEV float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
#endif
PTY_DEV float cabs2(float2 a) { return a.x * a.x + a.y * a.y; }
// multiply by W or conj(W) depending on the transform direction
template <int DIR>
PTY_DEV float2 ctw(float2 a, float2 w) {
  if constexpr (DIR < 0) return cmul(a, w);
  else return cmulc(a, w);
}

// ---------------------------------------------------------------- float-float
struct ff {
  float hi, lo;
};
PTY_DEV ff ff_zero() { return ff{0.f, 0.f}; }
// Knuth two-sum of the pair and one float; renormalised.
PTY_DEV ff ff_add(ff a, float b) {
  float s = a.hi + b;
  float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b - bb);
  e += a.lo;
  float hi = s + e;
  float lo = e - (hi - s);
  return ff{hi, lo};
}
PTY_DEV ff ff_add(ff a, ff b) {
  float s = a.hi + b.hi;
  float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);
  e += a.lo + b.lo;
  float hi = s + e;
  float lo = e - (hi - s);
  return ff{hi, lo};
}
PTY_DEV double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }

// A byte as a float without an int-to-float conversion instruction (those
// issue through the shared MIO path, where the frame kernels' exchanges
// already queue): the byte placed in the low mantissa bits of 2^23 gives the
// float 2^23 + b exactly, and subtracting 2^23 leaves b (exact for b < 2^23).
PTY_DEV float byte_to_float(unsigned b) { return __int_as_float(0x4B000000u | b) - 8388608.0f; }

// ---------------------------------------------------------------- reductions
PTY_DEV double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of one double per thread; fixed tree order (deterministic).
// `red` must hold 32 doubles.  Result valid in thread 0.
PTY_DEV double block_sum_d(double v, double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum_d(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    s = lane < nw ? red[lane] : 0.0;
    s = warp_sum_d(s);
  }
  return s;
}

// ---------------------------------------------------------------- compile-time trig
// Twiddles are compile-time constants evaluated from the Taylor series of
// sin/cos in double precision, then rounded once to float.
namespace ctrig {
constexpr double kPi = 3.14159265358979323846264338327950288;
__host__ __device__ constexpr double sin_series(double x) {
  double term = x, sum = x;
  for (int n = 1; n < 40; ++n) {
    term *= -x * x / ((2.0 * n) * (2.0 * n + 1.0));
    sum += term;
  }
  return sum;
}
__host__ __device__ constexpr double cos_series(double x) {
  double term = 1.0, sum = 1.0;
  for (int n = 1; n < 40; ++n) {
    term *= -x * x / ((2.0 * n - 1.0) * (2.0 * n));
    sum += term;
  }
  return sum;
}
// exp(-2 pi i k / n): angle reduced into (-pi, pi]
__host__ __device__ constexpr double wre(int k, int n) {
  k %= n;
  if (k < 0) k += n;
  double th = 2.0 * kPi * (double)k / (double)n;
  if (th > kPi) th -= 2.0 * kPi;
  return cos_series(th);
}
__host__ __device__ constexpr double wim(int k, int n) {
  k %= n;
  if (k < 0) k += n;
  double th = 2.0 * kPi * (double)k / (double)n;
  if (th > kPi) th -= 2.0 * kPi;
  return -sin_series(th);
}
}  // namespace ctrig

template <int I>
struct IC {
  static constexpr int value = I;
};
template <int B, int E, class F>
PTY_DEV void sfor(F&& f) {
  if constexpr (B < E) {
    f(IC<B>{});
    sfor<B + 1, E>(f);
  }
}

// status codes (PTY_OK, PTY_ERR_*) come from the public header
#include "../../include/ptycho_gb300.h"
