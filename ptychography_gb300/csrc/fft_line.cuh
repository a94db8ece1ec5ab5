// Register/shared-memory FFT building blocks.
//
// dft<R, DIR>(x): in-register DFT of R complex values (R a power of two, or 3
// times one, <= 64), natural order in and out, DIR = -1 forward
// (exp(-2 pi i/R)), +1 inverse (unnormalised).  Radix-4 / radix-2 / radix-3
// decimation in time with compile-time twiddles.
//
// Line FFT of length L = A * B (B a multiple of A), split over A threads:
//   * thread t holds v[j] = x[t + A j], j < B            ("stride-A" layout)
//   * B-point DFT in registers, twiddle by W_L^(t k1)
//   * one exchange through shared memory (slot (t, k1))
//   * B/A A-point DFTs in registers
//   * thread t ends with v[j] = X[t + A j]               (same layout)
// The exchange slots are supplied by the caller as accessors so the same code
// runs in place along frame rows and frame columns.
#pragma once
#include "pty_common.cuh"

// x * W^E with W = exp(-2 pi i / R) (forward) or its conjugate (inverse).
// Multiples of R/8 reduce to swaps, negations and one scale by sqrt(1/2), so
// no multiply is spent on +-1 or +-i (whose float constants would not be exact).
template <int E, int R, int DIR>
PTY_DEV float2 tw_mul(float2 x) {
  constexpr int e0 = ((E % R) + R) % R;
  constexpr int e = (DIR < 0) ? e0 : (R - e0) % R;   // inverse: conj(W^e) = W^(R-e)
  constexpr float h = 0.70710678118654752440f;       // sqrt(1/2)
  if constexpr (e == 0) {
    return x;
  } else if constexpr (4 * e == R) {                  // -i
    return make_float2(x.y, -x.x);
  } else if constexpr (2 * e == R) {                  // -1
    return make_float2(-x.x, -x.y);
  } else if constexpr (4 * e == 3 * R) {              // +i
    return make_float2(-x.y, x.x);
  } else if constexpr (8 * e == R) {                  // h - h i
    return make_float2(h * (x.x + x.y), h * (x.y - x.x));
  } else if constexpr (8 * e == 3 * R) {              // -h - h i
    return make_float2(h * (x.y - x.x), -h * (x.x + x.y));
  } else if constexpr (8 * e == 5 * R) {              // -h + h i
    return make_float2(-h * (x.x + x.y), h * (x.x - x.y));
  } else if constexpr (8 * e == 7 * R) {              // h + h i
    return make_float2(h * (x.x - x.y), h * (x.x + x.y));
  } else {
    constexpr float wr = (float)ctrig::wre(e, R), wi = (float)ctrig::wim(e, R);
    return cmul(x, make_float2(wr, wi));
  }
}

template <int DIR>
PTY_DEV void bfly4(float2& a, float2& b, float2& c, float2& d) {
  // X0 = a+b+c+d, X2 = a-b+c-d, X1/X3 = (a-c) -/+ i (b-d) (forward)
  float2 t0 = cadd(a, c), t1 = csub(a, c), t2 = cadd(b, d), t3 = csub(b, d);
  float2 j3 = (DIR < 0) ? make_float2(t3.y, -t3.x) : make_float2(-t3.y, t3.x);  // -+ i t3
  a = cadd(t0, t2);
  c = csub(t0, t2);
  b = cadd(t1, j3);
  d = csub(t1, j3);
}

// 3-point DFT in place: X0 = a+b+c, X1/X2 = (a - (b+c)/2) -/+ i sqrt(3)/2 (b-c) (forward)
template <int DIR>
PTY_DEV void bfly3(float2& a, float2& b, float2& c) {
  constexpr float s3 = 0.86602540378443864676f;   // sqrt(3) / 2
  const float2 t1 = cadd(b, c);
  const float2 t2 = make_float2(a.x - 0.5f * t1.x, a.y - 0.5f * t1.y);
  const float2 t3 = make_float2(s3 * (b.x - c.x), s3 * (b.y - c.y));
  // -i t3 = (t3.y, -t3.x); +i t3 = (-t3.y, t3.x)
  const float2 m = (DIR < 0) ? make_float2(t3.y, -t3.x) : make_float2(-t3.y, t3.x);
  a = cadd(a, t1);
  b = cadd(t2, m);
  c = csub(t2, m);
}

template <int R, int DIR>
PTY_DEV void dft(float2 (&x)[R]) {
  static_assert(R <= 64 && ((R & (R - 1)) == 0 || (R % 3 == 0 && ((R / 3) & (R / 3 - 1)) == 0)),
                "codelet sizes: powers of two and 3 x powers of two");
  if constexpr (R == 1) {
    return;
  } else if constexpr (R == 2) {
    float2 a = x[0], b = x[1];
    x[0] = cadd(a, b);
    x[1] = csub(a, b);
  } else if constexpr (R == 3) {
    bfly3<DIR>(x[0], x[1], x[2]);
  } else if constexpr (R == 4) {
    bfly4<DIR>(x[0], x[1], x[2], x[3]);
  } else if constexpr (R % 3 == 0) {
    // radix-3 decimation in time over three power-of-two sub-DFTs
    constexpr int M = R / 3;
    float2 s0[M], s1[M], s2[M];
#pragma unroll
    for (int m = 0; m < M; ++m) {
      s0[m] = x[3 * m + 0];
      s1[m] = x[3 * m + 1];
      s2[m] = x[3 * m + 2];
    }
    dft<M, DIR>(s0);
    dft<M, DIR>(s1);
    dft<M, DIR>(s2);
    sfor<0, M>([&](auto ik) {
      constexpr int k = decltype(ik)::value;
      float2 a = s0[k];
      float2 b = tw_mul<k, R, DIR>(s1[k]);
      float2 c = tw_mul<2 * k, R, DIR>(s2[k]);
      bfly3<DIR>(a, b, c);
      x[k] = a;
      x[k + M] = b;
      x[k + 2 * M] = c;
    });
  } else if constexpr (R % 4 == 0) {
    constexpr int M = R / 4;
    float2 s0[M], s1[M], s2[M], s3[M];
#pragma unroll
    for (int m = 0; m < M; ++m) {
      s0[m] = x[4 * m + 0];
      s1[m] = x[4 * m + 1];
      s2[m] = x[4 * m + 2];
      s3[m] = x[4 * m + 3];
    }
    dft<M, DIR>(s0);
    dft<M, DIR>(s1);
    dft<M, DIR>(s2);
    dft<M, DIR>(s3);
    sfor<0, M>([&](auto ik) {
      constexpr int k = decltype(ik)::value;
      float2 a = s0[k];
      float2 b = tw_mul<k, R, DIR>(s1[k]);
      float2 c = tw_mul<2 * k, R, DIR>(s2[k]);
      float2 d = tw_mul<3 * k, R, DIR>(s3[k]);
      bfly4<DIR>(a, b, c, d);
      x[k] = a;
      x[k + M] = b;
      x[k + 2 * M] = c;
      x[k + 3 * M] = d;
    });
  } else {  // R = 2 * (power of 4)
    constexpr int M = R / 2;
    float2 s0[M], s1[M];
#pragma unroll
    for (int m = 0; m < M; ++m) {
      s0[m] = x[2 * m];
      s1[m] = x[2 * m + 1];
    }
    dft<M, DIR>(s0);
    dft<M, DIR>(s1);
    sfor<0, M>([&](auto ik) {
      constexpr int k = decltype(ik)::value;
      float2 a = s0[k];
      float2 b = tw_mul<k, R, DIR>(s1[k]);
      x[k] = cadd(a, b);
      x[k + M] = csub(a, b);
    });
  }
}

// Geometry of a line transform of length L handled by A threads holding B values.
template <int L>
struct LineGeom;
template <> struct LineGeom<16>  { static constexpr int A = 4,  B = 4;  };
template <> struct LineGeom<32>  { static constexpr int A = 4,  B = 8;  };
template <> struct LineGeom<64>  { static constexpr int A = 8,  B = 8;  };
template <> struct LineGeom<128> { static constexpr int A = 8,  B = 16; };
template <> struct LineGeom<192> { static constexpr int A = 8,  B = 24; };
template <> struct LineGeom<256> { static constexpr int A = 16, B = 16; };
template <> struct LineGeom<512> { static constexpr int A = 16, B = 32; };

// First half of the line transform: B-point DFT and inter-step twiddle.
// tw[k1 * A + t] = exp(-2 pi i t k1 / L) (forward table; inverse conjugates).
template <int L, int DIR>
PTY_DEV void line_stage1(float2 (&v)[LineGeom<L>::B], int t, const float2* __restrict__ tw) {
  constexpr int A = LineGeom<L>::A, B = LineGeom<L>::B;
  dft<B, DIR>(v);
#pragma unroll
  for (int k1 = 1; k1 < B; ++k1) v[k1] = ctw<DIR>(v[k1], tw[k1 * A + t]);
}

// Second half: read the exchange slots, A-point DFTs, leave X[t + A j] in v[j].
// rd(tt, k1) returns slot (tt, k1) written by stage 1 of thread tt.
template <int L, int DIR, class RD>
PTY_DEV void line_stage2(float2 (&v)[LineGeom<L>::B], int t, RD rd) {
  constexpr int A = LineGeom<L>::A, B = LineGeom<L>::B, m = B / A;
#pragma unroll
  for (int q = 0; q < m; ++q) {
    float2 u[A];
#pragma unroll
    for (int tt = 0; tt < A; ++tt) u[tt] = rd(tt, t + A * q);
    dft<A, DIR>(u);
#pragma unroll
    for (int k2 = 0; k2 < A; ++k2) v[q + m * k2] = u[k2];
  }
}
