// Overlap (consistency) projections and small reductions.
//
// Every cross-frame sum is a gather in a fixed order, never a float atomic:
// an object tile walks its own ascending list of overlapping frames, and the
// probe / background reductions split the frames into K fixed chunks whose
// partials are combined in chunk order.  Two runs on the same inputs therefore
// produce identical bits.
#include "engine.h"

namespace pty {

constexpr int kTile = kGatherTileCols;      // tile width (columns) of the object / probe gathers
constexpr int kTileRows = kGatherTileRows;  // tile height (rows)
constexpr int kRowStep = kTileRows / 2;     // a thread's two pixels are kRowStep rows apart
constexpr int kGatherNT = 256; // threads per tile, 2 pixels each
static_assert(kGatherNT * 2 == kTile * kTileRows && kTileRows % 2 == 0, "gather tile split");
#ifndef PTY_GATHER_PREFETCH
#define PTY_GATHER_PREFETCH 4
#endif
constexpr int kPrefetch = PTY_GATHER_PREFETCH;   // frames whose loads are issued together (object gather)
constexpr int kPrefetchP = 4;  // the same for the probe gather

// acc += conj(p) x as four FMAs
PTY_DEV void cmac_conj(float2& acc, float2 x, float2 p) {
  acc.x = fmaf(p.x, x.x, fmaf(p.y, x.y, acc.x));
  acc.y = fmaf(p.x, x.y, fmaf(-p.y, x.x, acc.y));
}

// ------------------------------------------------------------------ psup_O
// era.py:336-369: O = sum_i psi_i * conj(P) placed at window i, / (heat + alpha),
// with heat = sum_i |P|^2 (era.py:402-410) recomputed in the same pass when HEAT.
// A thread owns 2 pixels (rows ty, ty + kRowStep) of an object tile; the tile's
// frames are visited in ascending order, kPrefetch at a time with all their
// loads issued first.  Out-of-window pixels contribute an exact zero.
template <bool HEAT>
__global__ void __launch_bounds__(kGatherNT) psup_O_kernel(
    TileLists tl, int N0, int N1, int U, int V, const int* __restrict__ R,
    const float2* __restrict__ psi, const float2* __restrict__ P, double* __restrict__ heat,
    float alpha, float2* __restrict__ O) {
  const int tile = blockIdx.x;
  const int tu = tile / tl.ntv, tv = tile % tl.ntv;
  const int tx = threadIdx.x % kTile, ty = threadIdx.x / kTile;
  const int v = tv * kTile + tx;
  const int u0 = tu * kTileRows + ty;
  float2 acc[2];
  ff h[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    acc[k] = make_float2(0.f, 0.f);
    h[k] = ff_zero();
  }
  const int beg = tl.ptr[tile], end = tl.ptr[tile + 1];
  auto fetch = [&](int e, float2 (&x)[2], float2 (&p)[2]) {
    const int f = tl.frames[e];
    const int r0 = R[2 * f], r1 = R[2 * f + 1];
    const int b = v + r1;
    const bool bok = b >= 0 && b < N1;
    const float2* pf = psi + (size_t)f * N0 * N1;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int a = u0 + kRowStep * k + r0;
      const bool ok = bok && a >= 0 && a < N0;
      x[k] = ok ? pf[a * N1 + b] : make_float2(0.f, 0.f);
      p[k] = ok ? P[a * N1 + b] : make_float2(0.f, 0.f);
    }
  };
  // The heat terms of a prefetch group are summed in FP32 (at most kPrefetch
  // terms of one sign, relative error < 2e-7) and the group sum is added to
  // the float-float total, so the total's error does not grow with the frame
  // count; the numerators accumulate with fused multiply-adds.
  int e = beg;
  for (; e + kPrefetch <= end; e += kPrefetch) {
    float2 x[kPrefetch][2], p[kPrefetch][2];
#pragma unroll
    for (int q = 0; q < kPrefetch; ++q) fetch(e + q, x[q], p[q]);
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      float hs = 0.f;
#pragma unroll
      for (int q = 0; q < kPrefetch; ++q) {
        cmac_conj(acc[k], x[q][k], p[q][k]);
        if (HEAT) hs += cabs2(p[q][k]);
      }
      if (HEAT) h[k] = ff_add(h[k], hs);
    }
  }
  for (; e < end; ++e) {
    float2 x[2], p[2];
    fetch(e, x, p);
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      cmac_conj(acc[k], x[k], p[k]);
      if (HEAT) h[k] = ff_add(h[k], cabs2(p[k]));
    }
  }
  if (v < V) {
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int uu = u0 + kRowStep * k;
      if (uu < U) {
        const size_t o = (size_t)uu * V + v;
        double hd;
        if (HEAT) {
          hd = ff_to_double(h[k]);
          heat[o] = hd;
        } else {
          hd = heat[o];
        }
        const float den = (float)(hd + (double)alpha);
        O[o] = make_float2(acc[k].x / den, acc[k].y / den);
      }
    }
  }
}

// era.py:402-410: heat = sum_i |P|^2 at window i (float-float, written as double)
__global__ void __launch_bounds__(kGatherNT) heat_P_kernel(
    TileLists tl, int N0, int N1, int U, int V, const int* __restrict__ R,
    const float2* __restrict__ P, double* __restrict__ heat) {
  const int tile = blockIdx.x;
  const int tu = tile / tl.ntv, tv = tile % tl.ntv;
  const int tx = threadIdx.x % kTile, ty = threadIdx.x / kTile;
  const int v = tv * kTile + tx;
  ff acc[2];
#pragma unroll
  for (int k = 0; k < 2; ++k) acc[k] = ff_zero();
  const int beg = tl.ptr[tile], end = tl.ptr[tile + 1];
  // |P|^2 at window pixel of list entry e, or an exact zero outside the window
  auto term = [&](int e, int k) -> float {
    const int f = tl.frames[e];
    const int r0 = R[2 * f], r1 = R[2 * f + 1];
    const int b = v + r1, a = tu * kTileRows + ty + kRowStep * k + r0;
    return (b >= 0 && b < N1 && a >= 0 && a < N0) ? cabs2(__ldg(&P[a * N1 + b])) : 0.f;
  };
  // the same grouping as psup_O_kernel<true>: FP32 sums of kPrefetch entries,
  // each added to the float-float total, then the remaining entries one by one
  // (adding an exact zero leaves a normalised pair unchanged), so both kernels
  // produce the same bits
  int e = beg;
  for (; e + kPrefetch <= end; e += kPrefetch) {
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      float hs = 0.f;
#pragma unroll
      for (int q = 0; q < kPrefetch; ++q) hs += term(e + q, k);
      acc[k] = ff_add(acc[k], hs);
    }
  }
  for (; e < end; ++e) {
#pragma unroll
    for (int k = 0; k < 2; ++k) acc[k] = ff_add(acc[k], term(e, k));
  }
  if (v < V) {
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int uu = tu * kTileRows + ty + kRowStep * k;
      if (uu < U) heat[(size_t)uu * V + v] = ff_to_double(acc[k]);
    }
  }
}

int launch_psup_O(const TileLists& tl, int n, int N0, int N1, int U, int V, const int* R,
                  const float2* psi, const float2* P, double* heat, bool compute_heat, float alpha,
                  float2* O, cudaStream_t st) {
  (void)n;
  if (compute_heat)
    psup_O_kernel<true><<<tl.ntu * tl.ntv, kGatherNT, 0, st>>>(tl, N0, N1, U, V, R, psi, P, heat, alpha, O);
  else
    psup_O_kernel<false><<<tl.ntu * tl.ntv, kGatherNT, 0, st>>>(tl, N0, N1, U, V, R, psi, P, heat, alpha, O);
  return check_launch("psup_O_kernel");
}

int launch_heat_P(const TileLists& tl, int n, int N0, int N1, int U, int V, const int* R,
                  const float2* P, double* heat, cudaStream_t st) {
  (void)n;
  heat_P_kernel<<<tl.ntu * tl.ntv, kGatherNT, 0, st>>>(tl, N0, N1, U, V, R, P, heat);
  return check_launch("heat_P_kernel");
}

// ------------------------------------------------------------------ psup_P
// era.py:371-400 (+ make_O_heatmap era.py:412-417): per probe pixel, sum over
// frames of psi_i * conj(O_i) and |O_i|^2.  Grid: kTileRows x kTile probe tiles x K
// frame chunks; a thread owns 2 pixels (rows ty, ty + kRowStep) and issues the loads of
// kPrefetch frames together.
__global__ void __launch_bounds__(kGatherNT) psup_P_partial_kernel(
    int n, int N0, int N1, int U, int V, const int* __restrict__ R, const float2* __restrict__ psi,
    const float2* __restrict__ O, int K, bool want_den, float2* __restrict__ part_num,
    float2* __restrict__ part_den) {
  const int ntv = (N1 + kTile - 1) / kTile;
  const int tile = blockIdx.x, k = blockIdx.y;
  const int tu = tile / ntv, tv = tile % ntv;
  const int tx = threadIdx.x % kTile, ty = threadIdx.x / kTile;
  const int b = tv * kTile + tx;
  const int f0 = (int)(((long long)n * k) / K), f1 = (int)(((long long)n * (k + 1)) / K);
  float2 num[2];
  ff den[2];
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    num[q] = make_float2(0.f, 0.f);
    den[q] = ff_zero();
  }
  if (b < N1) {
    auto fetch = [&](int f, float2 (&x)[2], float2 (&o)[2]) {
      const int r0 = R[2 * f], r1 = R[2 * f + 1];
      const float2* pf = psi + (size_t)f * N0 * N1;
      const int vv = b - r1;
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int a = tu * kTileRows + ty + kRowStep * q;
        if (a < N0) {
          o[q] = __ldg(&O[(size_t)(a - r0) * V + vv]);
          x[q] = pf[a * N1 + b];
        } else {
          o[q] = x[q] = make_float2(0.f, 0.f);
        }
      }
    };
    // as in psup_O: FMA numerators, |O|^2 group sums added to a float-float total
    int f = f0;
    for (; f + kPrefetchP <= f1; f += kPrefetchP) {
      float2 x[kPrefetchP][2], o[kPrefetchP][2];
#pragma unroll
      for (int j = 0; j < kPrefetchP; ++j) fetch(f + j, x[j], o[j]);
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        float ds = 0.f;
#pragma unroll
        for (int j = 0; j < kPrefetchP; ++j) {
          cmac_conj(num[q], x[j][q], o[j][q]);
          ds += cabs2(o[j][q]);
        }
        if (want_den) den[q] = ff_add(den[q], ds);
      }
    }
    for (; f < f1; ++f) {
      float2 x[2], o[2];
      fetch(f, x, o);
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        cmac_conj(num[q], x[q], o[q]);
        if (want_den) den[q] = ff_add(den[q], cabs2(o[q]));
      }
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int a = tu * kTileRows + ty + kRowStep * q;
      if (a < N0) {
        const size_t o = (size_t)k * N0 * N1 + (size_t)a * N1 + b;
        part_num[o] = num[q];
        if (want_den) part_den[o] = make_float2(den[q].hi, den[q].lo);
      }
    }
  }
}

__global__ void psup_P_reduce_kernel(int npix, int K, const float2* __restrict__ part_num,
                                     const float2* __restrict__ part_den, bool recompute,
                                     double* __restrict__ heatO, float alpha, float2* __restrict__ P) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npix) return;
  ff nr = ff_zero(), ni = ff_zero();
  for (int k = 0; k < K; ++k) {
    const float2 x = part_num[(size_t)k * npix + i];
    nr = ff_add(nr, x.x);
    ni = ff_add(ni, x.y);
  }
  double h;
  if (recompute) {
    ff d = ff_zero();
    for (int k = 0; k < K; ++k) {
      const float2 x = part_den[(size_t)k * npix + i];
      d = ff_add(d, ff{x.x, x.y});
    }
    h = ff_to_double(d);
    heatO[i] = h;
  } else {
    h = heatO[i];
  }
  const float den = (float)(h + (double)alpha);
  P[i] = make_float2(nr.hi / den, ni.hi / den);
}

// The same partial sums for frames whose rows are a multiple of 256 wide: a
// block takes whole frame rows -- 1024 / N1 rows x N1 columns, 4 pixels per
// thread (CPT columns of 1024 / (256 CPT) rows) -- so each psi load of a warp
// reads a contiguous row segment and a block's reads of one frame are
// consecutive rows (better DRAM page locality than small 2-D tiles).
template <int CPT>
__global__ void __launch_bounds__(kGatherNT) psup_P_rows_kernel(
    int n, int N0, int N1, int U, int V, const int* __restrict__ R, const float2* __restrict__ psi,
    const float2* __restrict__ O, int K, bool want_den, float2* __restrict__ part_num,
    float2* __restrict__ part_den) {
  constexpr int TR = 4 / CPT;               // rows per block
  constexpr int PF = 2;                     // frames whose loads are issued together
  const int k = blockIdx.y;
  const int a0 = blockIdx.x * TR;
  const int f0 = (int)(((long long)n * k) / K), f1 = (int)(((long long)n * (k + 1)) / K);
  int pa[4], pc[4];
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    pa[p] = a0 + p / CPT;
    pc[p] = threadIdx.x + kGatherNT * (p % CPT);
  }
  float2 num[4];
  ff den[4];
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    num[p] = make_float2(0.f, 0.f);
    den[p] = ff_zero();
  }
  auto fetch = [&](int f, float2 (&x)[4], float2 (&o)[4]) {
    const int r0 = R[2 * f], r1 = R[2 * f + 1];
    const float2* pf = psi + (size_t)f * N0 * N1;
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      x[p] = pf[pa[p] * N1 + pc[p]];
      o[p] = __ldg(&O[(size_t)(pa[p] - r0) * V + (pc[p] - r1)]);
    }
  };
  int f = f0;
  for (; f + PF <= f1; f += PF) {
    float2 x[PF][4], o[PF][4];
#pragma unroll
    for (int j = 0; j < PF; ++j) fetch(f + j, x[j], o[j]);
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      float ds = 0.f;
#pragma unroll
      for (int j = 0; j < PF; ++j) {
        cmac_conj(num[p], x[j][p], o[j][p]);
        ds += cabs2(o[j][p]);
      }
      if (want_den) den[p] = ff_add(den[p], ds);
    }
  }
  for (; f < f1; ++f) {
    float2 x[4], o[4];
    fetch(f, x, o);
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      cmac_conj(num[p], x[p], o[p]);
      if (want_den) den[p] = ff_add(den[p], cabs2(o[p]));
    }
  }
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const size_t idx = (size_t)k * N0 * N1 + (size_t)pa[p] * N1 + pc[p];
    part_num[idx] = num[p];
    if (want_den) part_den[idx] = make_float2(den[p].hi, den[p].lo);
  }
}

bool psup_P_by_rows(int N0, int N1) {
  return (N1 == 256 && N0 % 4 == 0) || (N1 == 512 && N0 % 2 == 0);
}

int psup_P_tiles(int N0, int N1) {
  if (psup_P_by_rows(N0, N1)) return N0 / (1024 / N1);
  return ((N0 + kTileRows - 1) / kTileRows) * ((N1 + kTile - 1) / kTile);
}

int launch_psup_P(int n, int N0, int N1, int U, int V, const int* R, const float2* psi,
                  const float2* O, float2* part_num, float2* part_den, int K, double* heatO,
                  bool recompute_heat, float alpha, float2* P, cudaStream_t st) {
  const int ntiles = psup_P_tiles(N0, N1);
  if (N1 == 256 && psup_P_by_rows(N0, N1))
    psup_P_rows_kernel<1><<<dim3(ntiles, K), kGatherNT, 0, st>>>(n, N0, N1, U, V, R, psi, O, K,
                                                                 recompute_heat, part_num, part_den);
  else if (N1 == 512 && psup_P_by_rows(N0, N1))
    psup_P_rows_kernel<2><<<dim3(ntiles, K), kGatherNT, 0, st>>>(n, N0, N1, U, V, R, psi, O, K,
                                                                 recompute_heat, part_num, part_den);
  else
    psup_P_partial_kernel<<<dim3(ntiles, K), kGatherNT, 0, st>>>(n, N0, N1, U, V, R, psi, O, K,
                                                                 recompute_heat, part_num, part_den);
  int rc = check_launch("psup_P_partial_kernel");
  if (rc) return rc;
  const int npix = N0 * N1;
  psup_P_reduce_kernel<<<(npix + 255) / 256, 256, 0, st>>>(npix, K, part_num, part_den,
                                                           recompute_heat, heatO, alpha, P);
  return check_launch("psup_P_reduce_kernel");
}

// make_O_heatmap alone (era.py:412-417), used by the standalone C-ABI op
__global__ void heat_O_partial_kernel(int n, int N0, int N1, int U, int V, const int* __restrict__ R,
                                      const float2* __restrict__ O, int K, float2* __restrict__ part) {
  const int npix = N0 * N1;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  if (i >= npix) return;
  const int a = i / N1, b = i % N1;
  const int f0 = (int)(((long long)n * k) / K), f1 = (int)(((long long)n * (k + 1)) / K);
  ff d = ff_zero();
  for (int f = f0; f < f1; ++f) {
    int uu = a - R[2 * f], vv = b - R[2 * f + 1];
    if (uu >= U) uu -= U;
    if (vv >= V) vv -= V;
    d = ff_add(d, cabs2(__ldg(&O[(size_t)uu * V + vv])));
  }
  part[(size_t)k * npix + i] = make_float2(d.hi, d.lo);
}

__global__ void heat_O_reduce_kernel(int npix, int K, const float2* __restrict__ part,
                                     double* __restrict__ heatO) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npix) return;
  ff d = ff_zero();
  for (int k = 0; k < K; ++k) {
    const float2 x = part[(size_t)k * npix + i];
    d = ff_add(d, ff{x.x, x.y});
  }
  heatO[i] = ff_to_double(d);
}

int launch_heat_O(int n, int N0, int N1, int U, int V, const int* R, const float2* O, float2* part,
                  int K, double* heatO, cudaStream_t st) {
  const int npix = N0 * N1;
  heat_O_partial_kernel<<<dim3((npix + 255) / 256, K), 256, 0, st>>>(n, N0, N1, U, V, R, O, K, part);
  int rc = check_launch("heat_O_partial_kernel");
  if (rc) return rc;
  heat_O_reduce_kernel<<<(npix + 255) / 256, 256, 0, st>>>(npix, K, part, heatO);
  return check_launch("heat_O_reduce_kernel");
}

// ------------------------------------------------------------------ frame mean
// era.py:265-270 / dm.py:208-213: b = mean over frames, per detector pixel
__global__ void frame_mean_partial_kernel(int n, int npix, const float* __restrict__ x, int K,
                                          float2* __restrict__ part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  if (i >= npix) return;
  const int f0 = (int)(((long long)n * k) / K), f1 = (int)(((long long)n * (k + 1)) / K);
  ff s = ff_zero();
  for (int f = f0; f < f1; ++f) s = ff_add(s, x[(size_t)f * npix + i]);
  part[(size_t)k * npix + i] = make_float2(s.hi, s.lo);
}

__global__ void frame_mean_reduce_kernel(int n, int npix, int K, const float2* __restrict__ part,
                                         float* __restrict__ mean) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npix) return;
  ff s = ff_zero();
  for (int k = 0; k < K; ++k) {
    const float2 x = part[(size_t)k * npix + i];
    s = ff_add(s, ff{x.x, x.y});
  }
  mean[i] = (float)(ff_to_double(s) / (double)n);
}

int launch_frame_mean(int n, int npix, const float* x, float2* part, int K, float* mean,
                      cudaStream_t st) {
  frame_mean_partial_kernel<<<dim3((npix + 255) / 256, K), 256, 0, st>>>(n, npix, x, K, part);
  int rc = check_launch("frame_mean_partial_kernel");
  if (rc) return rc;
  frame_mean_reduce_kernel<<<(npix + 255) / 256, 256, 0, st>>>(n, npix, K, part, mean);
  return check_launch("frame_mean_reduce_kernel");
}

// ------------------------------------------------------------------ metrics
// eCon numerator / denominator partials: sum |a-b|^2, sum |b|^2 (era.py:206-207)
__global__ void diffnorm_kernel(const float2* __restrict__ a, const float2* __restrict__ b,
                                long long count, double* __restrict__ part) {
  __shared__ double red[32];
  ff d = ff_zero(), c = ff_zero();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const float2 x = a[i], y = b[i];
    d = ff_add(d, cabs2(csub(x, y)));
    c = ff_add(c, cabs2(y));
  }
  const double sd = block_sum_d(ff_to_double(d), red);
  const double sc = block_sum_d(ff_to_double(c), red);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = sd;
    part[2 * blockIdx.x + 1] = sc;
  }
}

int launch_diffnorm(const float2* a, const float2* b, long long count, double* part, int nblocks,
                    cudaStream_t st) {
  diffnorm_kernel<<<nblocks, 256, 0, st>>>(a, b, count, part);
  return check_launch("diffnorm_kernel");
}

// eMod = sqrt(sum err / I_norm) (era.py:210), eCon = sqrt(d / c) (era.py:207-208)
__global__ void finalize_kernel(const double* __restrict__ err_part, int n,
                                const double* __restrict__ dn_part, int ndn, double I_norm,
                                double* hist_emod, double* hist_econ, int it) {
  __shared__ double red[32];
  double d = 0.0, c = 0.0;
  // four independent running sums per thread keep four loads in flight
  double e4[4] = {0.0, 0.0, 0.0, 0.0};
  const int stride = 4 * blockDim.x;
  int i0 = threadIdx.x;
  for (; i0 + 3 * (int)blockDim.x < n; i0 += stride)
#pragma unroll
    for (int k = 0; k < 4; ++k) e4[k] += err_part[i0 + k * blockDim.x];
  for (int k = 0; k < 4; ++k)
    if (i0 + k * (int)blockDim.x < n) e4[k] += err_part[i0 + k * blockDim.x];
  double e = (e4[0] + e4[1]) + (e4[2] + e4[3]);
  for (int i = threadIdx.x; i < ndn; i += blockDim.x) {
    d += dn_part[2 * i];
    c += dn_part[2 * i + 1];
  }
  e = block_sum_d(e, red);
  d = block_sum_d(d, red);
  c = block_sum_d(c, red);
  if (threadIdx.x == 0) {
    if (hist_emod) hist_emod[it] = sqrt(e / I_norm);
    if (hist_econ) hist_econ[it] = sqrt(d / c);
  }
}

int launch_finalize(const double* err_part, int n, const double* dn_part, int ndn, double I_norm,
                    double* hist_emod, double* hist_econ, int it, cudaStream_t st) {
  finalize_kernel<<<1, 1024, 0, st>>>(err_part, n, dn_part, ndn, I_norm, hist_emod, hist_econ, it);
  return check_launch("finalize_kernel");
}

// ------------------------------------------------------------------ centring
// era.py:172-186: cm = rint(centre_of_mass(|P|^2)) - shape // 2
__global__ void probe_shift_kernel(const float2* __restrict__ P, int N0, int N1, int* shift) {
  __shared__ double red[32];
  ff s = ff_zero(), sa = ff_zero(), sb = ff_zero();
  for (int i = threadIdx.x; i < N0 * N1; i += blockDim.x) {
    const float w = cabs2(P[i]);
    s = ff_add(s, w);
    sa = ff_add(sa, w * (float)(i / N1));
    sb = ff_add(sb, w * (float)(i % N1));
  }
  const double S = block_sum_d(ff_to_double(s), red);
  const double SA = block_sum_d(ff_to_double(sa), red);
  const double SB = block_sum_d(ff_to_double(sb), red);
  if (threadIdx.x == 0) {
    shift[0] = (int)rint(SA / S) - N0 / 2;
    shift[1] = (int)rint(SB / S) - N1 / 2;
  }
}

int launch_probe_shift(const float2* P, int N0, int N1, int* shift, cudaStream_t st) {
  probe_shift_kernel<<<1, 1024, 0, st>>>(P, N0, N1, shift);
  return check_launch("probe_shift_kernel");
}

// multiroll(x, -cm) (era.py:631-740) per image: dst[r][c] = src[(r + s0) mod H][(c + s1) mod W].
// Grid: (blocks over one image's rows, images); 32-bit index math inside an
// image, threads along a row (coalesced writes, reads coalesced up to the one
// wrap point of the row).
__global__ void roll_kernel(const float2* __restrict__ src, float2* __restrict__ dst, int nimg,
                            int H, int W, const int* __restrict__ shift) {
  const int s0 = shift[0], s1 = shift[1];
  const size_t npix = (size_t)H * W;
  for (int img = blockIdx.y; img < nimg; img += gridDim.y) {
    const float2* s = src + (size_t)img * npix;
    float2* d = dst + (size_t)img * npix;
    for (int r = blockIdx.x; r < H; r += gridDim.x) {
      int rr = (r + s0) % H;
      if (rr < 0) rr += H;
      const float2* srow = s + (size_t)rr * W;
      float2* drow = d + (size_t)r * W;
      for (int c = threadIdx.x; c < W; c += blockDim.x) {
        int cc = (c + s1) % W;
        if (cc < 0) cc += W;
        drow[c] = srow[cc];
      }
    }
  }
}

int launch_roll(const float2* src, float2* dst, int nimg, int H, int W, const int* shift,
                cudaStream_t st) {
  // about 16 CTAs per SM in all: rows split further when there are few images
  const int gy = nimg < 65535 ? nimg : 65535;
  int gx = (152 * 16 + gy - 1) / gy;
  gx = gx < 1 ? 1 : (gx > H ? H : gx);
  roll_kernel<<<dim3(gx, gy), 256, 0, st>>>(src, dst, nimg, H, W, shift);
  return check_launch("roll_kernel");
}

// make_exits (era.py:426-433): grid (8-row band, frame), threads along a row.
// Plan creation guarantees every window lies inside the object.
__global__ void make_exits_kernel(int N0, int N1, int U, int V, const int* __restrict__ R,
                                  const float2* __restrict__ O, const float2* __restrict__ P,
                                  float2* __restrict__ psi) {
  const int f = blockIdx.y;
  const int r0 = R[2 * f], r1 = R[2 * f + 1];
  const int npix = 8 * N1;
  const int a0 = blockIdx.x * 8;
  float2* out = psi + ((size_t)f * N0 + a0) * N1;
  for (int i = threadIdx.x; i < npix; i += blockDim.x) {
    const int a = a0 + i / N1, b = i % N1;
    if (a < N0) out[i] = cmul(__ldg(&O[(size_t)(a - r0) * V + (b - r1)]), __ldg(&P[a * N1 + b]));
  }
}

int launch_make_exits(int n, int N0, int N1, int U, int V, const int* R, const float2* O,
                      const float2* P, float2* psi, cudaStream_t st) {
  make_exits_kernel<<<dim3((N0 + 7) / 8, n), 256, 0, st>>>(N0, N1, U, V, R, O, P, psi);
  return check_launch("make_exits_kernel");
}

}  // namespace pty
