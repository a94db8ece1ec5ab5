// Three-stage line transforms over 32 threads: 256 points (8 values per
// thread, 8 x 8 x 4) and 512 points (16 values per thread, 16 x 8 x 4).
//
// 256 points:
// Layout in and out: thread t (t < 32) of the line holds v[j] = x[t + 32 j]
// (j < 8); after the transform v[j] = X[t + 32 j].  With 256 = 8 x 32 and
// 32 = 8 x 4:
//   1. DFT-8 over j, twiddle W256^(t k1)             (thread t, register k1)
//   2. exchange E1; thread t = k1 + 8 t1 takes Y'[t1 + 4 t2][k1], t2 < 8;
//      DFT-8 over t2, twiddle W32^(t1 m1)            (register m1)
//   3. exchange E2; thread t = k1 + 8 q takes Z'[k1][t1][m1], t1 < 4, for
//      m1 = q and q + 4; two DFT-4 over t1 give X[k1 + 8 m1 + 64 m2] =
//      X[t + 32 (h + 2 m2)], stored in v[h + 2 m2].
// The caller supplies the exchange storage (e1 / e2: slot -> float2&), the
// slot layouts (s1(t, k1) and s2(k1, t1, m1)) and the barrier that orders
// writes before reads (sync).  E1 and E2 may be the same storage when
// SAME_STORAGE, which adds the write-after-read barrier between them.
#pragma once
#include "fft_line.cuh"

namespace pty {

template <int DIR, bool SAME_STORAGE, class E1, class E2, class S1, class S2, class SYNC>
PTY_DEV void line3_fft256(float2 (&v)[8], int t, E1 e1, E2 e2, S1 s1, S2 s2, SYNC sync,
                          const float2* __restrict__ tw1, const float2* __restrict__ twf) {
  // tw1[k1 * 32 + t] = W256^(t k1), twf[e] = W256^e (forward; the inverse conjugates)
  dft<8, DIR>(v);
#pragma unroll
  for (int k1 = 1; k1 < 8; ++k1) v[k1] = ctw<DIR>(v[k1], tw1[k1 * 32 + t]);
#pragma unroll
  for (int k1 = 0; k1 < 8; ++k1) e1(s1(t, k1)) = v[k1];
  sync();
  const int k1 = t & 7, t1 = t >> 3;
#pragma unroll
  for (int t2 = 0; t2 < 8; ++t2) v[t2] = e1(s1(t1 + 4 * t2, k1));
  dft<8, DIR>(v);
#pragma unroll
  for (int m1 = 1; m1 < 8; ++m1) v[m1] = ctw<DIR>(v[m1], twf[(8 * t1 * m1) & 255]);
  if constexpr (SAME_STORAGE) sync();   // every E1 read done before E2 overwrites it
#pragma unroll
  for (int m1 = 0; m1 < 8; ++m1) e2(s2(k1, t1, m1)) = v[m1];
  sync();
  const int q = t >> 3;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float2 u[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) u[s] = e2(s2(k1, s, q + 4 * h));
    dft<4, DIR>(u);
#pragma unroll
    for (int m2 = 0; m2 < 4; ++m2) v[h + 2 * m2] = u[m2];
  }
}

// 512 points over 32 threads x 16 values, 512 = 16 x 32 with 32 = 8 x 4.
// Layout in and out: thread t holds v[j] = x[t + 32 j] (j < 16); after the
// transform v[j] = X[t + 32 j].
//   1. DFT-16 over j, twiddle W512^(t k1)                (thread t, register k1)
//   2. exchange E1; thread t = kl + 8 t1 (kl < 8, t1 < 4) takes Y'[t1 + 4 t2][k1]
//      (t2 < 8) for k1 = kl and kl + 8; DFT-8 over t2, twiddle W32^(t1 m1)
//   3. exchange E2; thread t = k1 + 16 q takes Z'[k1][s][m1], s < 4, for
//      m1 = q + 2 h (h < 4); DFT-4 over s gives X[k1 + 16 m1 + 128 m2] =
//      X[t + 32 (h + 4 m2)], stored in v[h + 4 m2].
// Same caller-supplied storage, slot layouts and barrier as line3_fft256;
// tw2[m1 * 4 + t1] = W32^(t1 m1).
template <int DIR, bool SAME_STORAGE, class E1, class E2, class S1, class S2, class SYNC>
PTY_DEV void line3_fft512(float2 (&v)[16], int t, E1 e1, E2 e2, S1 s1, S2 s2, SYNC sync,
                          const float2* __restrict__ tw1, const float2* __restrict__ tw2) {
  // tw1[k1 * 32 + t] = W512^(t k1) (forward; the inverse conjugates)
  dft<16, DIR>(v);
#pragma unroll
  for (int k1 = 1; k1 < 16; ++k1) v[k1] = ctw<DIR>(v[k1], tw1[k1 * 32 + t]);
#pragma unroll
  for (int k1 = 0; k1 < 16; ++k1) e1(s1(t, k1)) = v[k1];
  sync();
  const int kl = t & 7, t1 = t >> 3;
#pragma unroll
  for (int kh = 0; kh < 2; ++kh) {
    float2 u[8];
#pragma unroll
    for (int t2 = 0; t2 < 8; ++t2) u[t2] = e1(s1(t1 + 4 * t2, kl + 8 * kh));
    dft<8, DIR>(u);
    v[8 * kh] = u[0];
#pragma unroll
    for (int m1 = 1; m1 < 8; ++m1) v[8 * kh + m1] = ctw<DIR>(u[m1], tw2[m1 * 4 + t1]);
  }
  if constexpr (SAME_STORAGE) sync();   // every E1 read done before E2 overwrites it
#pragma unroll
  for (int kh = 0; kh < 2; ++kh)
#pragma unroll
    for (int m1 = 0; m1 < 8; ++m1) e2(s2(kl + 8 * kh, t1, m1)) = v[8 * kh + m1];
  sync();
  const int k1 = t & 15, q = t >> 4;
#pragma unroll
  for (int h = 0; h < 4; ++h) {
    float2 u[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) u[s] = e2(s2(k1, s, q + 2 * h));
    dft<4, DIR>(u);
#pragma unroll
    for (int m2 = 0; m2 < 4; ++m2) v[h + 4 * m2] = u[m2];
  }
}

}  // namespace pty
