// Per-pixel pieces of the fused frame kernels, shared by the one-CTA-per-frame
// kernel (frame_kernels.cu) and the cluster-per-frame kernel (cluster_frame.cuh):
//   frame_input   -- the wave entering the forward FFT at detector pixel (a, b)
//   frame_modulus -- the constraint applied to F at frequency (kr, kc)
//   frame_output  -- what is written back after the inverse FFT
#pragma once
#include "engine.h"

namespace pty {

template <int OP>
struct OpTraits {
  static constexpr bool IN_EXIT = (OP == OP_EXIT1 || OP == OP_EXIT7 || OP == OP_MERR || OP == OP_INTENS);
  static constexpr bool IN_DM = (OP == OP_DM1 || OP == OP_DM7);
  // a second (inverse) half after the column constraint
  static constexpr bool INVERSE = !(OP == OP_MERR || OP == OP_MERR_PSI || OP == OP_INTENS || OP == OP_BP);
  // direction of the first half: OP_BP is a single inverse transform
  static constexpr int FIRST_DIR = (OP == OP_BP) ? +1 : -1;
};

// exit wave P * O[window] (era.py:426-433) at frame pixel (a, b).  Plan
// creation guarantees every window lies inside the object, so the periodic
// wrap of the reference's roll never triggers and is not evaluated.
template <int N1>
PTY_DEV float2 exit_wave(const FrameArgs& g, int r0, int r1, int a, int b) {
  return cmul(__ldg(&g.O[(size_t)(a - r0) * g.V + (b - r1)]), __ldg(&g.P[a * N1 + b]));
}

template <int N1, int OP>
PTY_DEV float2 frame_input(const FrameArgs& g, int f, int r0, int r1, float2* psi, int a, int b) {
  if constexpr (OpTraits<OP>::IN_EXIT) {
    return exit_wave<N1>(g, r0, r1, a, b);
  } else if constexpr (OpTraits<OP>::IN_DM) {
    // dm.py:94-95: e1 = psi - ex0 ; x = ex0 - e1  (= 2 ex0 - psi, rounded as the reference).
    // e1 replaces psi at this pixel: the output stage (frame_output_line)
    // needs exactly e1, and one load of it is cheaper there than re-reading
    // psi and forming the exit wave again; no other thread reads the pixel.
    const float2 ex0 = exit_wave<N1>(g, r0, r1, a, b);
    const float2 e1 = csub(psi[a * N1 + b], ex0);
    psi[a * N1 + b] = e1;
    return csub(ex0, e1);
  } else if constexpr (OP == OP_BP) {
    // back_projection.py:74-77: mask * sqrt(I) * exp(i angle(fftn(P))), with the
    // reference's centred-order amp and mask taken from the engine's unshifted
    // buffers (ifftshift of an even length is a half-length roll), and g.P
    // holding the unit phasors of fftn(P) in natural order
    const int pa = (a + g.N0h) % (2 * g.N0h), pb = (b + g.N1h) % (2 * g.N1h);
    const int pix = pa * N1 + pb;
    const float m = g.mask ? byte_to_float(g.mask[pix]) : 1.0f;
    return cscale(__ldg(&g.P[a * N1 + b]), m * g.amp[(size_t)g.amp_stride * f + pix]);
  } else {
    return psi[a * N1 + b];
  }
}

// The modulus constraint on one column line: v[j] = F[t + A j][kc], in two
// parts so a kernel can issue the line's global loads early and overlap
// their latency with the forward transform:
//   modulus_load      -- amp, mask and background of the line into registers
//   modulus_load_late -- DM7's background state and mean, just before use
//   modulus_apply     -- the constraint on v, the error sum, the background store
// All loads of a line precede its stores (the output pointers may alias the
// inputs, which would otherwise serialise every load behind the previous
// element's store).
template <int OP, int B>
struct ModIn {
  static constexpr bool BG_IN = (OP == OP_EXIT7 || OP == OP_PSI7 || OP == OP_MERR || OP == OP_MERR_PSI);
  static constexpr bool BG_OUT = (OP == OP_EXIT7 || OP == OP_PSI7 || OP == OP_DM7);
  static constexpr bool NEEDS = !(OP == OP_INTENS || OP == OP_BP);
  float am[B], mk[B], bb[B], b0v[B];
};

template <int N0, int N1, int OP, int A, int B>
PTY_DEV void modulus_load(const FrameArgs& g, int f, size_t fbase, int t, int kc, ModIn<OP, B>& m) {
  if constexpr (ModIn<OP, B>::NEEDS) {
    const float* amp = g.amp + (size_t)g.amp_stride * f;
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const int pix = (t + A * j) * N1 + kc;
      m.am[j] = __ldg(&amp[pix]);
      m.mk[j] = g.mask ? byte_to_float(__ldg(&g.mask[pix])) : 1.0f;
      if constexpr (ModIn<OP, B>::BG_IN) m.bb[j] = g.bg_in ? g.bg_in[(size_t)g.bg_stride * f + pix] : 0.0f;
    }
  }
}

// The DM7 background state and mean, loaded just before the constraint: with
// amp and mask already in flight, two more arrays across the forward
// transform would not fit the register budget.
template <int N0, int N1, int OP, int A, int B>
PTY_DEV void modulus_load_late(const FrameArgs& g, size_t fbase, int t, int kc, ModIn<OP, B>& m) {
  if constexpr (OP == OP_DM7) {
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const int pix = (t + A * j) * N1 + kc;
      m.bb[j] = g.bg_out[fbase + pix];
      m.b0v[j] = __ldg(&g.b0[pix]);
    }
  }
}

template <int OP, int B>
PTY_DEV void modulus_compute(const FrameArgs& g, float2 (&v)[B], ModIn<OP, B>& m, ff& err);

template <int N0, int N1, int OP, int A, int B>
PTY_DEV void modulus_apply(const FrameArgs& g, size_t fbase, int t, int kc, float2 (&v)[B],
                           ModIn<OP, B>& m, ff& err) {
  if constexpr (OP == OP_INTENS) {
    const int sc = (kc + N1 / 2) % N1;   // fftshift, era.py:295
#pragma unroll
    for (int j = 0; j < B; ++j) {
      const int sr = (t + A * j + N0 / 2) % N0;
      g.out_real[fbase + (size_t)sr * N1 + sc] = cabs2(v[j]);
    }
    return;
  } else if constexpr (OP == OP_BP) {
    // the inverse transform is complete: write psi, scaled 1 / (N0 N1) as ifftn
    constexpr float kInv = 1.0f / (float)(N0 * N1);
#pragma unroll
    for (int j = 0; j < B; ++j) g.psi[fbase + (size_t)(t + A * j) * N1 + kc] = cscale(v[j], kInv);
    return;
  } else {
    modulus_compute<OP, B>(g, v, m, err);
    if constexpr (ModIn<OP, B>::BG_OUT) {
#pragma unroll
      for (int j = 0; j < B; ++j) g.bg_out[fbase + (size_t)(t + A * j) * N1 + kc] = m.bb[j];
    }
  }
}

// The constraint on one pixel (EXIT / PSI / DM / MERR forms): F at the
// pixel's frequency, its amplitude am and mask value mk; bb is the pixel's
// background (updated in place by the background forms), b0 the DM mean
// background.  Returns the new F and adds the pixel's error term to line_err.
template <int OP>
PTY_DEV float2 modulus_pixel(const FrameArgs& g, float2 F, float am, float mk, float& bb,
                             const float& b0, float& line_err) {
  // square roots and quotients use the hardware reciprocal square root
  // (a few ulp; the engine's tolerances are 1e-5 relative)
  if constexpr (OP == OP_EXIT1 || OP == OP_PSI1 || OP == OP_DM1) {
    // era.py:561-571: |F| + alpha, masked pixels keep F
    const float x2 = cabs2(F);
    const float mag = (x2 > 0.f ? x2 * rsqrtf(x2) : 0.f) + g.alpha;
    const float d = mag - am;
    line_err += d * d * mk;
    const float fac = (mk != 0.f) ? __fdividef(am, mag) : 1.0f;
    return cscale(F, fac);
  } else if constexpr (OP == OP_EXIT7 || OP == OP_PSI7) {
    // era.py:584-594: sqrt(|F|^2 + b^2 + alpha), masked pixels zeroed
    const float x2 = cabs2(F) + bb * bb + g.alpha;
    const float rs = rsqrtf(x2);
    const float d = x2 * rs - am;
    line_err += d * d * mk;
    const float fac = mk * am * rs;
    bb *= fac;
    return cscale(F, fac);
  } else if constexpr (OP == OP_DM7) {
    // dm.py:219-224 on the background: g1 = g - b0 ; tb = b0 - g1 ; g = g1 + Pmod7(tb)
    const float g1 = bb - b0;
    const float tb = b0 - g1;
    const float fac = mk * am * rsqrtf(cabs2(F) + tb * tb + g.alpha);
    bb = g1 + tb * fac;
    return cscale(F, fac);
  } else if constexpr (OP == OP_MERR || OP == OP_MERR_PSI) {
    // dm.py:338-340, no alpha
    const float x2 = cabs2(F) + bb * bb;
    const float d = (x2 > 0.f ? x2 * rsqrtf(x2) : 0.f) - am;
    line_err += mk * (d * d);
    return F;
  } else {
    return F;
  }
}

// The constraint on a line held in registers: updates v and, for the
// background forms, m.bb; adds the line's error terms to err.
template <int OP, int B>
PTY_DEV void modulus_compute(const FrameArgs& g, float2 (&v)[B], ModIn<OP, B>& m, ff& err) {
  float line_err = 0.f;   // FP32 over one line (B terms), folded into err once
#pragma unroll
  for (int j = 0; j < B; ++j) v[j] = modulus_pixel<OP>(g, v[j], m.am[j], m.mk[j], m.bb[j], m.b0v[j], line_err);
  err = ff_add(err, line_err);
}

template <int N0, int N1, int OP, int A, int B>
PTY_DEV void frame_modulus_line(const FrameArgs& g, int f, size_t fbase, int t, int kc,
                                float2 (&v)[B], ff& err) {
  ModIn<OP, B> m;
  modulus_load<N0, N1, OP, A, B>(g, f, fbase, t, kc, m);
  modulus_load_late<N0, N1, OP, A, B>(g, fbase, t, kc, m);
  modulus_apply<N0, N1, OP, A, B>(g, fbase, t, kc, v, m, err);
}

// The result of the inverse transform for one row line (v[j] at column
// t + A j, already scaled): loads first, then stores (see frame_modulus_line).
template <int N1, int OP, int A, int B>
PTY_DEV void frame_output_line(const FrameArgs& g, int r0, int r1, float2* psi, int a, int t,
                               float2 (&v)[B]) {
  if constexpr (OpTraits<OP>::IN_DM) {
#pragma unroll
    for (int j = 0; j < B; ++j) {
      // dm.py:94-97: psi_new = (psi - ex0) + Pmod(2 ex0 - psi), with psi - ex0
      // (e1) left in psi by frame_input
      v[j] = cadd(psi[a * N1 + t + A * j], v[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < B; ++j) psi[a * N1 + t + A * j] = v[j];
}

}  // namespace pty
