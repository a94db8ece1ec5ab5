// The learned warm start's network: 3 x 3 convolutions as im2col + BF16
// tensor-core GEMMs with FP32 accumulation, and the element-wise pieces of
// its forward pass, backward pass and Adam step.  No reference counterpart:
// the reference starts ERA from ones (ptychography/era.py:480-486); the warm
// start replaces that initial object by one stitched from per-frame phases
// this network predicts from each frame's back-projection.
//
// Layout: activations NHWC (pixel-major, channels contiguous), BF16 between
// layers; GEMM outputs FP32.  A convolution with C_in inputs is
//   forward  Y[p][co] = sum_k col[p][k] W[co][k],     col = im2col(X), k = (ky*3 + kx) C_in + ci
//   dgrad    dcol[p][k] = sum_co dY[p][co] W[co][k],  dX = col2im(dcol)
//   wgrad    dW[co][k] = sum_p dY[p][co] col[p][k]    (split over p, partials summed in order)
// all three by one GEMM kernel with strided operands.
//
// The GEMM: mma.sync.m16n8k16 (BF16 in, FP32 accumulate), 64 x 64 output
// tiles, 4 warps of 32 x 32, K in steps of 32 staged through shared memory
// ([m][k] and [n][k], 40-element rows: the fragment loads of a warp hit 32
// distinct banks).  Fragment layout of m16n8k16 (PTX ISA): lane = 4 g + t;
// A: a0 = (g, 2t..2t+1), a1 = (g+8, 2t..), a2 = (g, 2t+8..), a3 = (g+8, 2t+8..);
// B (k x n, column-major): b0 = (2t..2t+1, g), b1 = (2t+8.., g);
// C: c0, c1 = (g, 2t..2t+1), c2, c3 = (g+8, 2t..2t+1).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/ptycho_gb300.h"
#include "engine.h"

namespace pty {

namespace {

constexpr int kTM = 64, kTN = 64, kTK = 32, kPad = 40, kGemmThreads = 128;

struct GemmArgs {
  int M, N, K;
  const __nv_bfloat16* A;
  long long sam, sak;        // A(m, k) = A[m sam + k sak]
  const __nv_bfloat16* B;
  long long sbk, sbn;        // B(k, n) = B[k sbk + n sbn]
  float* C;                  // C(m, n) = C[m scm + n scn] (+ split * M * N for partials)
  long long scm, scn;
  int k_per_split;           // K range of one blockIdx.z
  int a_vec, b_vec;          // 16-byte loads: 1 along k, 2 along m (A) / n (B), 0 none
};

// Stage an R x 32 operand tile (R = 64 rows of m or n) into s[row][k].
// vec 1: k contiguous (8 k per 16-byte load); vec 2: rows contiguous (8 rows
// per load, scattered); chunks crossing the operand's edge load element-wise.
__device__ __forceinline__ void stage_tile(__nv_bfloat16 (*s)[kPad], const __nv_bfloat16* __restrict__ src,
                                           long long s_row, long long s_k, int rows, int row0, int k0,
                                           int kend, int vec) {
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  const int tid = threadIdx.x;
  if (vec == 1) {
    for (int c = tid; c < kTM * (kTK / 8); c += kGemmThreads) {
      const int r = c >> 2, kc = (c & 3) * 8;
      const int row = row0 + r, k = k0 + kc;
      if (row < rows && k + 8 <= kend) {
        // asynchronous 16-byte copy: lands while the other buffer is computed
        const unsigned sa = (unsigned)__cvta_generic_to_shared(&s[r][kc]);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa),
                     "l"(src + (long long)row * s_row + k)
                     : "memory");
      } else {
#pragma unroll
        for (int j = 0; j < 8; ++j)
          s[r][kc + j] = (row < rows && k + j < kend) ? src[(long long)row * s_row + k + j] : zero;
      }
    }
  } else if (vec == 2) {
    for (int c = tid; c < (kTM / 8) * kTK; c += kGemmThreads) {
      const int kk = c >> 3, rc = (c & 7) * 8;
      const int row = row0 + rc, k = k0 + kk;
      if (row + 8 <= rows && k < kend) {
        const uint4 v = __ldg(reinterpret_cast<const uint4*>(src + row + (long long)k * s_k));
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int j = 0; j < 8; ++j)
          s[rc + j][kk] = __ushort_as_bfloat16((unsigned short)((w[j >> 1] >> (16 * (j & 1))) & 0xffffu));
      } else {
#pragma unroll
        for (int j = 0; j < 8; ++j)
          s[rc + j][kk] = (row + j < rows && k < kend) ? src[(long long)(row + j) + (long long)k * s_k] : zero;
      }
    }
  } else {
    for (int i = tid; i < kTM * kTK; i += kGemmThreads) {
      const int r = i / kTK, c = i % kTK;
      const int row = row0 + r, k = k0 + c;
      s[r][c] = (row < rows && k < kend) ? src[(long long)row * s_row + (long long)k * s_k] : zero;
    }
  }
}

__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16* p) {
  return *reinterpret_cast<const uint32_t*>(p);
}

__global__ void __launch_bounds__(kGemmThreads) ws_gemm_kernel(GemmArgs g) {
  __shared__ __align__(16) __nv_bfloat16 sa[2][kTM][kPad];
  __shared__ __align__(16) __nv_bfloat16 sb[2][kTN][kPad];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int m0 = blockIdx.y * kTM, n0 = blockIdx.x * kTN;
  const int kbeg = blockIdx.z * g.k_per_split;
  const int kend = min(g.K, kbeg + g.k_per_split);
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;   // warp's 32 x 32 sub-tile
  const int gq = lane >> 2, tq = lane & 3;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
  // double buffering: the tile of step k0 + 32 is staged (asynchronously for
  // k-contiguous operands) while step k0 is multiplied
  int buf = 0;
  if (kbeg < kend) {
    stage_tile(sa[0], g.A, g.sam, g.sak, g.M, m0, kbeg, kend, g.a_vec);
    stage_tile(sb[0], g.B, g.sbn, g.sbk, g.N, n0, kbeg, kend, g.b_vec);
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
  for (int k0 = kbeg; k0 < kend; k0 += kTK, buf ^= 1) {
    if (k0 + kTK < kend) {
      stage_tile(sa[buf ^ 1], g.A, g.sam, g.sak, g.M, m0, k0 + kTK, kend, g.a_vec);
      stage_tile(sb[buf ^ 1], g.B, g.sbn, g.sbk, g.N, n0, k0 + kTK, kend, g.b_vec);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 1;" ::: "memory");   // this step's copies landed
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kTK; kk += 16) {
      uint32_t af[2][4], bf[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = wm + 16 * i + gq;
        af[i][0] = ld_pair(&sa[buf][r][kk + 2 * tq]);
        af[i][1] = ld_pair(&sa[buf][r + 8][kk + 2 * tq]);
        af[i][2] = ld_pair(&sa[buf][r][kk + 2 * tq + 8]);
        af[i][3] = ld_pair(&sa[buf][r + 8][kk + 2 * tq + 8]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = wn + 8 * j + gq;
        bf[j][0] = ld_pair(&sb[buf][c][kk + 2 * tq]);
        bf[j][1] = ld_pair(&sb[buf][c][kk + 2 * tq + 8]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
          asm volatile(
              "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
              "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};"
              : "+f"(acc[i][j][0]), "+f"(acc[i][j][1]), "+f"(acc[i][j][2]), "+f"(acc[i][j][3])
              : "r"(af[i][0]), "r"(af[i][1]), "r"(af[i][2]), "r"(af[i][3]), "r"(bf[j][0]), "r"(bf[j][1]));
    }
    __syncthreads();
  }
  float* C = g.C + (size_t)blockIdx.z * g.M * g.N;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int m = m0 + wm + 16 * i + gq + (r >= 2 ? 8 : 0);
        const int n = n0 + wn + 8 * j + 2 * tq + (r & 1);
        if (m < g.M && n < g.N) C[(long long)m * g.scm + (long long)n * g.scn] = acc[i][j][r];
      }
}

// out[i] = sum over s < splits of part[s][i], in split order (deterministic)
__global__ void ws_sum_splits_kernel(const float* __restrict__ part, int splits, long long n,
                                     float* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int k = 0; k < splits; ++k) s += part[(size_t)k * n + i];
    out[i] = s;
  }
}

#define WS_LOOP(i, n) \
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (n); i += (long long)gridDim.x * blockDim.x)

// col[p][(ky*3 + kx) C + c] = X[b][y + ky - 1][x + kx - 1][c] (zero outside), p = (b, y, x)
__global__ void ws_im2col_kernel(int Bt, int H, int W, int C, const __nv_bfloat16* __restrict__ X,
                                 __nv_bfloat16* __restrict__ col) {
  const long long K = 9ll * C, n = (long long)Bt * H * W * K;
  WS_LOOP(i, n) {
    const long long p = i / K;
    const int k = (int)(i % K), tap = k / C, c = k % C;
    const int x = (int)(p % W), y = (int)((p / W) % H), b = (int)(p / ((long long)W * H));
    const int yy = y + tap / 3 - 1, xx = x + tap % 3 - 1;
    col[i] = (yy >= 0 && yy < H && xx >= 0 && xx < W)
                 ? X[(((long long)b * H + yy) * W + xx) * C + c]
                 : __float2bfloat16(0.f);
  }
}

// The same with 8 channels per thread (C a multiple of 8): thread = (pixel,
// channel chunk), grid row = tap; 16-byte copies, 32-bit index arithmetic
// (pixels x C / 8 < 2^31).
__global__ void ws_im2col8_kernel(int Bt, int H, int W, int C, const __nv_bfloat16* __restrict__ X,
                                  __nv_bfloat16* __restrict__ col) {
  const int chunks = C >> 3, tap = blockIdx.y;
  const int n = Bt * H * W * chunks;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int p = i / chunks, ch = i - p * chunks;
  const int x = p % W, t = p / W, y = t % H, b = t / H;
  const int yy = y + tap / 3 - 1, xx = x + tap % 3 - 1;
  uint4 v = make_uint4(0u, 0u, 0u, 0u);
  if (yy >= 0 && yy < H && xx >= 0 && xx < W)
    v = __ldg(reinterpret_cast<const uint4*>(X + ((size_t)(b * H + yy) * W + xx) * C + ch * 8));
  *reinterpret_cast<uint4*>(col + (size_t)p * 9 * C + tap * C + ch * 8) = v;
}

// col2im with 4 channels per thread (C a multiple of 4), float4 reads
__global__ void ws_col2im4_kernel(int Bt, int H, int W, int C, const float* __restrict__ dcol,
                                  float* __restrict__ dX) {
  const int chunks = C >> 2;
  const int n = Bt * H * W * chunks;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int p = i / chunks, ch = i - p * chunks;
  const int x = p % W, t = p / W, y = t % H, b = t / H;
  float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
  for (int tap = 0; tap < 9; ++tap) {
    const int yy = y - tap / 3 + 1, xx = x - tap % 3 + 1;
    if (yy >= 0 && yy < H && xx >= 0 && xx < W) {
      const float4 v = __ldg(reinterpret_cast<const float4*>(
          dcol + ((size_t)(b * H + yy) * W + xx) * 9 * C + tap * C + ch * 4));
      s.x += v.x;
      s.y += v.y;
      s.z += v.z;
      s.w += v.w;
    }
  }
  *reinterpret_cast<float4*>(dX + (size_t)p * C + ch * 4) = s;
}

// dX[b][y][x][c] = sum over taps of dcol[(b, y - ky + 1, x - kx + 1)][(ky*3 + kx) C + c]
__global__ void ws_col2im_kernel(int Bt, int H, int W, int C, const float* __restrict__ dcol,
                                 float* __restrict__ dX) {
  const long long n = (long long)Bt * H * W * C, K = 9ll * C;
  WS_LOOP(i, n) {
    const int c = (int)(i % C);
    const long long p = i / C;
    const int x = (int)(p % W), y = (int)((p / W) % H), b = (int)(p / ((long long)W * H));
    float s = 0.f;
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
      const int yy = y - tap / 3 + 1, xx = x - tap % 3 + 1;
      if (yy >= 0 && yy < H && xx >= 0 && xx < W)
        s += dcol[(((long long)b * H + yy) * W + xx) * K + tap * C + c];
    }
    dX[i] = s;
  }
}

// 2 x 2 average pooling (NHWC) and its adjoint
__global__ void ws_pool2_kernel(int Bt, int H, int W, int C, const __nv_bfloat16* __restrict__ X,
                                __nv_bfloat16* __restrict__ Y) {
  const int h = H / 2, w = W / 2;
  const long long n = (long long)Bt * h * w * C;
  WS_LOOP(i, n) {
    const int c = (int)(i % C);
    const long long p = i / C;
    const int x = (int)(p % w), y = (int)((p / w) % h), b = (int)(p / ((long long)w * h));
    const long long base = (((long long)b * H + 2 * y) * W + 2 * x) * C + c;
    const float s = __bfloat162float(X[base]) + __bfloat162float(X[base + C]) +
                    __bfloat162float(X[base + (long long)W * C]) + __bfloat162float(X[base + (long long)W * C + C]);
    Y[i] = __float2bfloat16(0.25f * s);
  }
}
__global__ void ws_pool2_bwd_kernel(int Bt, int H, int W, int C, const float* __restrict__ dY,
                                    float* __restrict__ dX) {
  const long long n = (long long)Bt * H * W * C;
  WS_LOOP(i, n) {
    const int c = (int)(i % C);
    const long long p = i / C;
    const int x = (int)(p % W), y = (int)((p / W) % H), b = (int)(p / ((long long)W * H));
    dX[i] = 0.25f * dY[(((long long)b * (H / 2) + y / 2) * (W / 2) + x / 2) * C + c];
  }
}

// The same with 8 channels per thread (C a multiple of 8, 16-byte aligned
// arrays, outputs x C / 8 < 2^31): 16-byte loads and stores, 32-bit indices
__global__ void ws_pool2_v8_kernel(int Bt, int H, int W, int C, const __nv_bfloat16* __restrict__ X,
                                   __nv_bfloat16* __restrict__ Y) {
  const int h = H / 2, w = W / 2, chunks = C >> 3;
  const int n = Bt * h * w * chunks;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int ch = i % chunks, p = i / chunks;
    const int x = p % w, t = p / w, y = t % h, b = t / h;
    const size_t base = ((size_t)(b * H + 2 * y) * W + 2 * x) * C + 8 * ch;
    const size_t off[4] = {0, (size_t)C, (size_t)W * C, (size_t)W * C + C};
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint4 u = __ldg(reinterpret_cast<const uint4*>(X + base + off[q]));
      const __nv_bfloat162* hv = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float2 f = __bfloat1622float2(hv[k]);
        acc[2 * k] += f.x;
        acc[2 * k + 1] += f.y;
      }
    }
    uint4 r;
    __nv_bfloat162* rv = reinterpret_cast<__nv_bfloat162*>(&r);
#pragma unroll
    for (int k = 0; k < 4; ++k) rv[k] = __floats2bfloat162_rn(0.25f * acc[2 * k], 0.25f * acc[2 * k + 1]);
    *reinterpret_cast<uint4*>(Y + (size_t)i * 8) = r;
  }
}

// nearest 2 x upsampling (h x w -> 2h x 2w, NHWC) and its adjoint
__global__ void ws_up2_kernel(int Bt, int h, int w, int C, const __nv_bfloat16* __restrict__ X,
                              __nv_bfloat16* __restrict__ Y) {
  const long long n = (long long)Bt * 4 * h * w * C;
  WS_LOOP(i, n) {
    const int c = (int)(i % C);
    const long long p = i / C;
    const int x = (int)(p % (2 * w)), y = (int)((p / (2 * w)) % (2 * h)), b = (int)(p / (4ll * w * h));
    Y[i] = X[(((long long)b * h + y / 2) * w + x / 2) * C + c];
  }
}
// 8 channels per thread (conditions as ws_pool2_v8_kernel)
__global__ void ws_up2_v8_kernel(int Bt, int h, int w, int C, const __nv_bfloat16* __restrict__ X,
                                 __nv_bfloat16* __restrict__ Y) {
  const int chunks = C >> 3;
  const int n = Bt * 4 * h * w * chunks;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int ch = i % chunks, p = i / chunks;
    const int x = p % (2 * w), t = p / (2 * w), y = t % (2 * h), b = t / (2 * h);
    *reinterpret_cast<uint4*>(Y + (size_t)i * 8) =
        __ldg(reinterpret_cast<const uint4*>(X + ((size_t)(b * h + y / 2) * w + x / 2) * C + 8 * ch));
  }
}
__global__ void ws_up2_bwd_kernel(int Bt, int h, int w, int C, const float* __restrict__ dY,
                                  float* __restrict__ dX) {
  const long long n = (long long)Bt * h * w * C;
  WS_LOOP(i, n) {
    const int c = (int)(i % C);
    const long long p = i / C;
    const int x = (int)(p % w), y = (int)((p / w) % h), b = (int)(p / ((long long)w * h));
    const long long W2 = 2ll * w;
    const long long base = (((long long)b * 2 * h + 2 * y) * W2 + 2 * x) * C + c;
    dX[i] = dY[base] + dY[base + C] + dY[base + W2 * C] + dY[base + W2 * C + C];
  }
}

// a = act(Z + bias) (relu when relu != 0); out = a + skip (skip may be null).
// a and out as BF16; a32 (optional) as FP32 (the network's final output).
__global__ void ws_bias_act_kernel(long long P, int C, const float* __restrict__ Z, const float* __restrict__ bias,
                                   int relu, const __nv_bfloat16* __restrict__ skip,
                                   __nv_bfloat16* __restrict__ a, __nv_bfloat16* __restrict__ out,
                                   float* __restrict__ a32) {
  const long long n = P * C;
  WS_LOOP(i, n) {
    float v = Z[i] + bias[i % C];
    if (relu) v = fmaxf(v, 0.f);
    const __nv_bfloat16 vb = __float2bfloat16(v);
    if (a) a[i] = vb;
    if (a32) a32[i] = v;
    if (out) out[i] = skip ? __float2bfloat16(__bfloat162float(vb) + __bfloat162float(skip[i])) : vb;
  }
}

// dZ = dA * (a > 0) (relu) or dA; as BF16 for the GEMMs; per-block partial
// sums of dZ per channel into part[blockIdx.x][C] (bias gradient, summed in
// block order by ws_sum_rows_kernel)
__global__ void ws_act_bwd_kernel(long long P, int C, const float* __restrict__ dA,
                                  const __nv_bfloat16* __restrict__ a, int relu,
                                  __nv_bfloat16* __restrict__ dZ, float* __restrict__ part,
                                  long long rows_per_block) {
  const long long r0 = blockIdx.x * rows_per_block;
  const long long r1 = min(P, r0 + rows_per_block);
  for (int c0 = 0; c0 < C; c0 += blockDim.x) {
    const int c = c0 + threadIdx.x;
    float s = 0.f;
    if (c < C) {
      for (long long r = r0; r < r1; ++r) {
        const long long i = r * C + c;
        float g = dA[i];
        if (relu && !(__bfloat162float(a[i]) > 0.f)) g = 0.f;
        dZ[i] = __float2bfloat16(g);
        s += g;
      }
      part[(size_t)blockIdx.x * C + c] = s;
    }
  }
}

// out[c] = sum over r < rows of part[r][c]: one block per channel, each
// thread a fixed stride of rows, then a fixed tree (deterministic)
__global__ void __launch_bounds__(256) ws_sum_rows_kernel(const float* __restrict__ part, int rows, int C,
                                                          float* __restrict__ out) {
  __shared__ float red[256];
  const int c = blockIdx.x;
  float s = 0.f;
  for (int r = threadIdx.x; r < rows; r += blockDim.x) s += part[(size_t)r * C + c];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[c] = red[0];
}

// weighted squared error of Y [P][2] against T [P][2] with per-pixel weights
// w [P] (already normalised to sum 1): dY = 2 w (Y - T); per-block partial
// losses into lpart[blockIdx.x]
__global__ void ws_loss_kernel(long long P, const float* __restrict__ Y, const float* __restrict__ T,
                               const float* __restrict__ w, float* __restrict__ dY, float* __restrict__ lpart) {
  __shared__ float red[256];
  float s = 0.f;
  WS_LOOP(p, P) {
    const float w0 = w[p];
    const float e0 = Y[2 * p] - T[2 * p], e1 = Y[2 * p + 1] - T[2 * p + 1];
    dY[2 * p] = 2.f * w0 * e0;
    dY[2 * p + 1] = 2.f * w0 * e1;
    s += w0 * (e0 * e0 + e1 * e1);
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) lpart[blockIdx.x] = red[0];
}

// Adam (Kingma and Ba, 2015) on FP32 master weights, with a BF16 copy
__global__ void ws_adam_kernel(long long n, float* __restrict__ w, __nv_bfloat16* __restrict__ wb,
                               const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                               float lr, float b1, float b2, float eps, float c1, float c2) {
  WS_LOOP(i, n) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
  }
}

__global__ void ws_to_bf16_kernel(long long n, const float* __restrict__ x, __nv_bfloat16* __restrict__ y) {
  WS_LOOP(i, n) y[i] = __float2bfloat16(x[i]);
}

// out = a + b (FP32), for gradients meeting at a skip connection
__global__ void ws_add_kernel(long long n, const float* __restrict__ a, const float* __restrict__ b,
                              float* __restrict__ out) {
  WS_LOOP(i, n) out[i] = a[i] + b[i];
}

// The input-gradient convolution's weights: Wf[ci][t C_out + co] = W[co][(8 - t) C_in + ci],
// the forward weights with C_in and C_out exchanged and the 3 x 3 taps turned
// by 180 degrees, so that dX = conv3x3(dZ, Wf) in the forward layout
__global__ void ws_flip_weights_kernel(int cin, int cout, const __nv_bfloat16* __restrict__ w,
                                       __nv_bfloat16* __restrict__ wf) {
  const long long n = 9LL * cin * cout;
  WS_LOOP(i, n) {
    const int ci = (int)(i / (9 * cout)), r = (int)(i % (9 * cout));
    const int t = r / cout, co = r % cout;
    wf[i] = w[(size_t)co * 9 * cin + (size_t)(8 - t) * cin + ci];
  }
}

inline unsigned grid_for(long long n) {
  long long g = (n + 255) / 256;
  if (g > 8 * 152) g = 8 * 152;
  return (unsigned)(g < 1 ? 1 : g);
}

}  // namespace

}  // namespace pty

using namespace pty;

namespace {
typedef __nv_bfloat16 bf16;
constexpr long long kActRows = 256;   // pixels per block of ws_act_bwd_kernel
constexpr int kLossBlocks = 256;
int ws_launched(const char* where) { return check_launch(where); }
}  // namespace

extern "C" int pty_ws_gemm(int32_t M, int32_t N, int32_t K, const void* A, int64_t sam, int64_t sak,
                           const void* B, int64_t sbk, int64_t sbn, float* C, int64_t scm, int64_t scn,
                           int32_t splits, float* partial, void* stream) {
  if (M < 1 || N < 1 || K < 1 || !A || !B || !C) return set_error(PTY_ERR_ARG, "bad GEMM arguments");
  if (splits < 1) splits = 1;
  if (splits > 1 && (!partial || scm != N || scn != 1))
    return set_error(PTY_ERR_ARG, "split GEMM needs partials and a contiguous M x N output");
  GemmArgs g;
  g.M = M;
  g.N = N;
  g.K = K;
  g.A = (const bf16*)A;
  g.sam = sam;
  g.sak = sak;
  g.B = (const bf16*)B;
  g.sbk = sbk;
  g.sbn = sbn;
  g.C = splits > 1 ? partial : C;
  g.scm = scm;
  g.scn = scn;
  // K per split a multiple of the K step, so only the last split is ragged
  int kps = (K + splits - 1) / splits;
  kps = ((kps + kTK - 1) / kTK) * kTK;
  splits = (K + kps - 1) / kps;
  g.k_per_split = kps;
  // 16-byte loads where the operand has a contiguous dimension, 16-byte
  // aligned rows and a base aligned to 16 bytes
  auto vec_of = [](const void* ptr, long long s_row, long long s_k) {
    if (((uintptr_t)ptr & 15u) != 0) return 0;
    if (s_k == 1 && s_row % 8 == 0) return 1;
    if (s_row == 1 && s_k % 8 == 0) return 2;
    return 0;
  };
  g.a_vec = vec_of(A, sam, sak);
  g.b_vec = vec_of(B, sbn, sbk);
  cudaStream_t st = (cudaStream_t)stream;
  dim3 grid((N + kTN - 1) / kTN, (M + kTM - 1) / kTM, splits);
  ws_gemm_kernel<<<grid, kGemmThreads, 0, st>>>(g);
  PTY_TRY(ws_launched("ws_gemm_kernel"));
  if (g.C != C) {
    const long long n = (long long)M * N;
    ws_sum_splits_kernel<<<grid_for(n), 256, 0, st>>>(partial, splits, n, C);
    PTY_TRY(ws_launched("ws_sum_splits_kernel"));
  }
  return PTY_OK;
}

extern "C" int pty_ws_im2col(int32_t B, int32_t H, int32_t W, int32_t C, const void* X, void* col,
                             void* stream) {
  if (B < 1 || H < 1 || W < 1 || C < 1 || !X || !col) return set_error(PTY_ERR_ARG, "bad im2col arguments");
  const long long n = 9ll * B * H * W * C;
  const long long n8 = (long long)B * H * W * (C / 8);
  const bool vec = C % 8 == 0 && n8 < (1ll << 31) && ((uintptr_t)X & 15u) == 0 && ((uintptr_t)col & 15u) == 0;
  if (vec) {
    const dim3 grid((unsigned)((n8 + 255) / 256), 9);
    ws_im2col8_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(B, H, W, C, (const bf16*)X, (bf16*)col);
    return ws_launched("ws_im2col8_kernel");
  }
  ws_im2col_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(B, H, W, C, (const bf16*)X, (bf16*)col);
  return ws_launched("ws_im2col_kernel");
}

extern "C" int pty_ws_col2im(int32_t B, int32_t H, int32_t W, int32_t C, const float* dcol, float* dX,
                             void* stream) {
  if (B < 1 || H < 1 || W < 1 || C < 1 || !dcol || !dX) return set_error(PTY_ERR_ARG, "bad col2im arguments");
  const long long n = (long long)B * H * W * C;
  const long long n4 = n / 4;
  const bool vec = C % 4 == 0 && n4 < (1ll << 31) && ((uintptr_t)dcol & 15u) == 0 && ((uintptr_t)dX & 15u) == 0;
  if (vec) {
    ws_col2im4_kernel<<<(unsigned)((n4 + 255) / 256), 256, 0, (cudaStream_t)stream>>>(B, H, W, C, dcol, dX);
    return ws_launched("ws_col2im4_kernel");
  }
  ws_col2im_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(B, H, W, C, dcol, dX);
  return ws_launched("ws_col2im_kernel");
}

extern "C" int pty_ws_pool2(int32_t B, int32_t H, int32_t W, int32_t C, const void* X, void* Y, void* stream) {
  if (B < 1 || H < 2 || W < 2 || (H | W) & 1 || C < 1 || !X || !Y) return set_error(PTY_ERR_ARG, "bad pool arguments");
  const long long n = (long long)B * (H / 2) * (W / 2) * C;
  if (C % 8 == 0 && n / 8 < (1ll << 31) && (long long)B * H * W * C < (1ll << 40) &&
      (((uintptr_t)X | (uintptr_t)Y) & 15u) == 0) {
    ws_pool2_v8_kernel<<<grid_for(n / 8), 256, 0, (cudaStream_t)stream>>>(B, H, W, C, (const bf16*)X, (bf16*)Y);
    return ws_launched("ws_pool2_v8_kernel");
  }
  ws_pool2_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(B, H, W, C, (const bf16*)X, (bf16*)Y);
  return ws_launched("ws_pool2_kernel");
}

extern "C" int pty_ws_pool2_bwd(int32_t B, int32_t H, int32_t W, int32_t C, const float* dY, float* dX,
                                void* stream) {
  if (B < 1 || H < 2 || W < 2 || (H | W) & 1 || C < 1 || !dY || !dX) return set_error(PTY_ERR_ARG, "bad pool arguments");
  const long long n = (long long)B * H * W * C;
  ws_pool2_bwd_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(B, H, W, C, dY, dX);
  return ws_launched("ws_pool2_bwd_kernel");
}

extern "C" int pty_ws_up2(int32_t B, int32_t h, int32_t w, int32_t C, const void* X, void* Y, void* stream) {
  if (B < 1 || h < 1 || w < 1 || C < 1 || !X || !Y) return set_error(PTY_ERR_ARG, "bad upsample arguments");
  const long long n = 4ll * B * h * w * C;
  if (C % 8 == 0 && n / 8 < (1ll << 31) && (((uintptr_t)X | (uintptr_t)Y) & 15u) == 0) {
    ws_up2_v8_kernel<<<grid_for(n / 8), 256, 0, (cudaStream_t)stream>>>(B, h, w, C, (const bf16*)X, (bf16*)Y);
    return ws_launched("ws_up2_v8_kernel");
  }
  ws_up2_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(B, h, w, C, (const bf16*)X, (bf16*)Y);
  return ws_launched("ws_up2_kernel");
}

extern "C" int pty_ws_up2_bwd(int32_t B, int32_t h, int32_t w, int32_t C, const float* dY, float* dX,
                              void* stream) {
  if (B < 1 || h < 1 || w < 1 || C < 1 || !dY || !dX) return set_error(PTY_ERR_ARG, "bad upsample arguments");
  const long long n = (long long)B * h * w * C;
  ws_up2_bwd_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(B, h, w, C, dY, dX);
  return ws_launched("ws_up2_bwd_kernel");
}

extern "C" int pty_ws_bias_act(int64_t P, int32_t C, const float* Z, const float* bias, int32_t relu,
                               const void* skip, void* a, void* out, float* a32, void* stream) {
  if (P < 1 || C < 1 || !Z || !bias) return set_error(PTY_ERR_ARG, "bad activation arguments");
  const long long n = P * C;
  ws_bias_act_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(P, C, Z, bias, relu, (const bf16*)skip,
                                                                    (bf16*)a, (bf16*)out, a32);
  return ws_launched("ws_bias_act_kernel");
}

extern "C" int64_t pty_ws_act_bwd_scratch(int64_t P, int32_t C) {
  if (P < 1 || C < 1) return -1;
  return ((P + kActRows - 1) / kActRows) * C;
}

extern "C" int pty_ws_act_bwd(int64_t P, int32_t C, const float* dA, const void* a, int32_t relu, void* dZ,
                              float* dbias, float* scratch, void* stream) {
  if (P < 1 || C < 1 || C > 1024 || !dA || !dZ || !dbias || !scratch || (relu && !a))
    return set_error(PTY_ERR_ARG, "bad activation-gradient arguments");
  const long long blocks = (P + kActRows - 1) / kActRows;
  if (blocks > 2147483647ll) return set_error(PTY_ERR_RANGE, "too many pixels");
  cudaStream_t st = (cudaStream_t)stream;
  const int threads = C < 32 ? 32 : (C > 256 ? 256 : ((C + 31) / 32) * 32);
  ws_act_bwd_kernel<<<(unsigned)blocks, threads, 0, st>>>(P, C, dA, (const bf16*)a, relu, (bf16*)dZ, scratch,
                                                          kActRows);
  PTY_TRY(ws_launched("ws_act_bwd_kernel"));
  ws_sum_rows_kernel<<<C, 256, 0, st>>>(scratch, (int)blocks, C, dbias);
  return ws_launched("ws_sum_rows_kernel");
}

extern "C" int pty_ws_loss(int64_t P, const float* Y, const float* T, const float* w, float* dY,
                           float* loss_parts, void* stream) {
  if (P < 1 || !Y || !T || !w || !dY || !loss_parts) return set_error(PTY_ERR_ARG, "bad loss arguments");
  ws_loss_kernel<<<kLossBlocks, 256, 0, (cudaStream_t)stream>>>(P, Y, T, w, dY, loss_parts);
  return ws_launched("ws_loss_kernel");
}

extern "C" int pty_ws_adam(int64_t n, float* w, void* wb, const float* g, float* m, float* v, float lr,
                           float b1, float b2, float eps, int32_t step, void* stream) {
  if (n < 1 || !w || !g || !m || !v || step < 1) return set_error(PTY_ERR_ARG, "bad Adam arguments");
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  ws_adam_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(n, w, (bf16*)wb, g, m, v, lr, b1, b2, eps, c1, c2);
  return ws_launched("ws_adam_kernel");
}

extern "C" int pty_ws_to_bf16(int64_t n, const float* x, void* y, void* stream) {
  if (n < 1 || !x || !y) return set_error(PTY_ERR_ARG, "bad conversion arguments");
  ws_to_bf16_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(n, x, (bf16*)y);
  return ws_launched("ws_to_bf16_kernel");
}

extern "C" int pty_ws_flip_weights(int32_t Cin, int32_t Cout, const void* W, void* Wf, void* stream) {
  if (Cin < 1 || Cout < 1 || !W || !Wf) return set_error(PTY_ERR_ARG, "bad weight-flip arguments");
  ws_flip_weights_kernel<<<grid_for(9LL * Cin * Cout), 256, 0, (cudaStream_t)stream>>>(Cin, Cout, (const bf16*)W,
                                                                                      (bf16*)Wf);
  return ws_launched("ws_flip_weights_kernel");
}

extern "C" int pty_ws_add(int64_t n, const float* a, const float* b, float* out, void* stream) {
  if (n < 1 || !a || !b || !out) return set_error(PTY_ERR_ARG, "bad add arguments");
  ws_add_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(n, a, b, out);
  return ws_launched("ws_add_kernel");
}

// ---------------------------------------------------------------- data
namespace pty {
namespace {

// The network's input from back-projected exit waves bp (one block per frame):
// z = s bp conj(P) / (max|P|^2 r), r = sqrt(sum |bp|^2 / sum |P|^2) the frame's
// RMS object amplitude, s = (-1)^(row + col) when `checker` (undoing the
// modulation that a half-period shift of the far-field product leaves in bp),
// else 1; x[f][p] = bf16(Re z, Im z).  Inside the probe z is the object up to
// its scale r; outside it fades with |P|^2.
__global__ void __launch_bounds__(1024) ws_prep_bp_kernel(int N1, long long npix, const float2* __restrict__ bp,
                                                          const float2* __restrict__ P, int checker,
                                                          __nv_bfloat16* __restrict__ x) {
  __shared__ float red[3][1024];
  const float2* bf = bp + (size_t)blockIdx.x * npix;
  __nv_bfloat16* xf = x + (size_t)blockIdx.x * npix * 2;
  float sb = 0.f, sp = 0.f, mp = 0.f;
  for (long long p = threadIdx.x; p < npix; p += blockDim.x) {
    const float2 v = bf[p], q = P[p];
    const float a = q.x * q.x + q.y * q.y;
    sb += v.x * v.x + v.y * v.y;
    sp += a;
    mp = fmaxf(mp, a);
  }
  red[0][threadIdx.x] = sb;
  red[1][threadIdx.x] = sp;
  red[2][threadIdx.x] = mp;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      red[0][threadIdx.x] += red[0][threadIdx.x + o];
      red[1][threadIdx.x] += red[1][threadIdx.x + o];
      red[2][threadIdx.x] = fmaxf(red[2][threadIdx.x], red[2][threadIdx.x + o]);
    }
    __syncthreads();
  }
  const float r = (red[0][0] > 0.f && red[1][0] > 0.f) ? sqrtf(red[0][0] / red[1][0]) : 1.f;
  const float scale = red[2][0] > 0.f ? 1.f / (red[2][0] * r) : 0.f;
  for (long long p = threadIdx.x; p < npix; p += blockDim.x) {
    const long long row = p / N1, col = p - row * N1;
    const float s = (checker && ((row + col) & 1)) ? -scale : scale;
    const float2 v = bf[p], q = P[p];
    xf[2 * p] = __float2bfloat16((v.x * q.x + v.y * q.y) * s);
    xf[2 * p + 1] = __float2bfloat16((v.y * q.x - v.x * q.y) * s);
  }
}

// target[f][p] = (cos, sin) of arg psi[f][p] (object_phase: of arg psi conj(P),
// the object's phase under the probe); weight[f][p] = |P[p]|^2 * wscale
__global__ void ws_targets_kernel(long long nf, long long npix, const float2* __restrict__ psi,
                                  const float2* __restrict__ P, int object_phase, float wscale,
                                  float* __restrict__ target, float* __restrict__ weight) {
  const long long n = nf * npix;
  WS_LOOP(i, n) {
    float2 v = psi[i];
    if (object_phase) {
      const float2 q = P[i % npix];
      v = make_float2(v.x * q.x + v.y * q.y, v.y * q.x - v.x * q.y);
    }
    const float r = sqrtf(v.x * v.x + v.y * v.y);
    target[2 * i] = r > 0.f ? v.x / r : 1.f;
    target[2 * i + 1] = r > 0.f ? v.y / r : 0.f;
    const float2 q = P[i % npix];
    weight[i] = (q.x * q.x + q.y * q.y) * wscale;
  }
}

// psi[f][p] = |P[p]| (y0 + i y1) / |y|, the exit wave with the predicted phase
// (object_phase: P[p] (y0 + i y1) / |y|, the probe's phase added back)
__global__ void ws_exits_kernel(long long nf, long long npix, const float* __restrict__ y,
                                const float2* __restrict__ P, int object_phase, float2* __restrict__ psi) {
  const long long n = nf * npix;
  WS_LOOP(i, n) {
    const float a = y[2 * i], b = y[2 * i + 1];
    const float r = sqrtf(a * a + b * b);
    const float ca = r > 0.f ? a / r : 1.f, sa = r > 0.f ? b / r : 0.f;
    const float2 q = P[i % npix];
    if (object_phase) {
      psi[i] = make_float2(q.x * ca - q.y * sa, q.x * sa + q.y * ca);
    } else {
      const float m = sqrtf(q.x * q.x + q.y * q.y);
      psi[i] = make_float2(m * ca, m * sa);
    }
  }
}

}  // namespace
}  // namespace pty

extern "C" int pty_ws_prep_bp(int32_t nf, int32_t N0, int32_t N1, const void* bp, const void* P,
                              int32_t checker, void* x, void* stream) {
  if (nf < 1 || N0 < 1 || N1 < 1 || !bp || !P || !x)
    return set_error(PTY_ERR_ARG, "bad back-projection input arguments");
  // the (-1)^(row + col) correction is the half-period shift only for even sides
  if (checker && ((N0 | N1) & 1)) return set_error(PTY_ERR_SHAPE, "checker sign needs even frame sides");
  ws_prep_bp_kernel<<<nf, 1024, 0, (cudaStream_t)stream>>>(N1, (long long)N0 * N1, (const float2*)bp,
                                                           (const float2*)P, checker, (bf16*)x);
  return ws_launched("ws_prep_bp_kernel");
}

extern "C" int pty_ws_targets(int32_t nf, int64_t npix, const void* psi, const void* P, int32_t object_phase,
                              float wscale, float* target, float* weight, void* stream) {
  if (nf < 1 || npix < 1 || !psi || !P || !target || !weight) return set_error(PTY_ERR_ARG, "bad target arguments");
  const long long n = (long long)nf * npix;
  ws_targets_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(nf, npix, (const float2*)psi, (const float2*)P,
                                                                   object_phase, wscale, target, weight);
  return ws_launched("ws_targets_kernel");
}

extern "C" int pty_ws_exits(int32_t nf, int64_t npix, const float* y, const void* P, int32_t object_phase,
                            void* psi, void* stream) {
  if (nf < 1 || npix < 1 || !y || !P || !psi) return set_error(PTY_ERR_ARG, "bad exit-wave arguments");
  const long long n = (long long)nf * npix;
  ws_exits_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(nf, npix, y, (const float2*)P, object_phase,
                                                                 (float2*)psi);
  return ws_launched("ws_exits_kernel");
}

// ---------------------------------------------------------------- direct convolution
namespace pty {
namespace {

constexpr int kDirThreads = 128;

// A 3 x 3 convolution (zero padding) for layers with few channels, one thread
// per output pixel holding all COUT sums: Z[p][co] = sum over taps and input
// channels of X[p + tap][ci] W[co][tap C_in + ci], in that order, FP32.  Then
// v = Z + bias (relu when asked), a = bf16(v), out = a (+ skip, rounded to
// bf16 as ws_bias_act_kernel does) and out32 = v.  The weights sit in shared
// memory transposed to [k][COUT], so every thread reads the same words.
// Inputs are read VEC channels at a time (8: 16-byte loads, C_in a multiple
// of 8; 2: 4-byte loads), outputs written as whole 16-, 8- or 4-byte pieces.
template <int VEC>
struct BfVec;
template <>
struct BfVec<8> {
  static PTY_DEV void load(const __nv_bfloat16* p, float* f) {
    const uint4 u = __ldg(reinterpret_cast<const uint4*>(p));
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float2 t = __bfloat1622float2(h[i]);
      f[2 * i] = t.x;
      f[2 * i + 1] = t.y;
    }
  }
};
template <>
struct BfVec<2> {
  static PTY_DEV void load(const __nv_bfloat16* p, float* f) {
    const float2 t = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(p));
    f[0] = t.x;
    f[1] = t.y;
  }
};

template <int COUT, int VEC, int PX, int CIN>
__global__ void __launch_bounds__(kDirThreads) ws_conv_direct_kernel(int Bt, int H, int W, int Cin_rt,
                                                                     const __nv_bfloat16* __restrict__ X,
                                                                     const __nv_bfloat16* __restrict__ Wt,
                                                                     const float* __restrict__ bias, int relu,
                                                                     const __nv_bfloat16* __restrict__ skip,
                                                                     __nv_bfloat16* __restrict__ out,
                                                                     float* __restrict__ out32) {
  // a thread owns PX pixels of a row, 32 apart (W a multiple of 32 PX when
  // PX > 1), so that every weight read from shared memory feeds PX
  // multiply-adds while the lanes of a warp still read neighbouring pixels.
  // CIN > 0 fixes C_in at compile time (the network's 2- and 32-channel
  // inputs): the channel loop unrolls and a tap's loads issue together.
  const int Cin = CIN > 0 ? CIN : Cin_rt;
  extern __shared__ __align__(16) float wsm[];   // [9 Cin][COUT]
  const int K = 9 * Cin;
  for (int i = threadIdx.x; i < K * COUT; i += blockDim.x) {
    const int co = i / K, k = i - co * K;
    wsm[k * COUT + co] = __bfloat162float(Wt[i]);
  }
  __syncthreads();
  const int Wq = W / PX;
  const int Q = Bt * H * Wq;                     // pixel groups (< 2^31, checked on the host)
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < Q; q += gridDim.x * blockDim.x) {
    const int xi = q % Wq, t = q / Wq, y = t % H, b = t / H;
    const int x0 = PX > 1 ? (xi >> 5) * 32 * PX + (xi & 31) : xi;   // pixel u at x0 + 32 u
    float acc[PX][COUT];
#pragma unroll
    for (int u = 0; u < PX; ++u)
#pragma unroll
      for (int c = 0; c < COUT; ++c) acc[u][c] = 0.f;
#pragma unroll (CIN > 0 && CIN <= 8 ? 9 : 1)
    for (int tap = 0; tap < 9; ++tap) {
      const int yy = y + tap / 3 - 1;
      if (yy < 0 || yy >= H) continue;
      const int dx = tap % 3 - 1;
      const __nv_bfloat16* xrow = X + (size_t)(b * H + yy) * W * Cin;
      const float* wk = wsm + tap * Cin * COUT;
      for (int ci = 0; ci < Cin; ci += VEC) {
        float v[PX][VEC];
#pragma unroll
        for (int u = 0; u < PX; ++u) {
          const int xx = x0 + 32 * u + dx;
          if (xx >= 0 && xx < W) {
            BfVec<VEC>::load(xrow + (size_t)xx * Cin + ci, v[u]);
          } else {
#pragma unroll
            for (int j = 0; j < VEC; ++j) v[u][j] = 0.f;
          }
        }
#pragma unroll
        for (int j = 0; j < VEC; ++j)
#pragma unroll
          for (int c = 0; c < COUT; ++c) {
            const float wv = wk[(ci + j) * COUT + c];
#pragma unroll
            for (int u = 0; u < PX; ++u) acc[u][c] = fmaf(v[u][j], wv, acc[u][c]);
          }
      }
    }
#pragma unroll
    for (int u = 0; u < PX; ++u) {
#pragma unroll
      for (int c = 0; c < COUT; ++c) {
        acc[u][c] += bias[c];
        if (relu) acc[u][c] = fmaxf(acc[u][c], 0.f);
      }
      const size_t o = ((size_t)(b * H + y) * W + x0 + 32 * u) * COUT;
      if (out32) {
        if constexpr (COUT % 4 == 0) {
#pragma unroll
          for (int c = 0; c < COUT; c += 4)
            *reinterpret_cast<float4*>(out32 + o + c) =
                make_float4(acc[u][c], acc[u][c + 1], acc[u][c + 2], acc[u][c + 3]);
        } else {
#pragma unroll
          for (int c = 0; c < COUT; c += 2)
            *reinterpret_cast<float2*>(out32 + o + c) = make_float2(acc[u][c], acc[u][c + 1]);
        }
      }
      if (out) {
        __nv_bfloat162 hv[COUT / 2];
#pragma unroll
        for (int c = 0; c < COUT; c += 2) {
          __nv_bfloat162 a2 = __floats2bfloat162_rn(acc[u][c], acc[u][c + 1]);
          if (skip) {
            const float2 af = __bfloat1622float2(a2);
            const float2 sf = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(skip + o + c));
            a2 = __floats2bfloat162_rn(af.x + sf.x, af.y + sf.y);
          }
          hv[c / 2] = a2;
        }
        if constexpr (COUT % 8 == 0) {
#pragma unroll
          for (int c = 0; c < COUT; c += 8)
            *reinterpret_cast<uint4*>(out + o + c) = *reinterpret_cast<const uint4*>(&hv[c / 2]);
        } else {
#pragma unroll
          for (int c = 0; c < COUT; c += 2) *reinterpret_cast<__nv_bfloat162*>(out + o + c) = hv[c / 2];
        }
      }
    }
  }
}

// out[f][a][b] = scale I[g][a + (N0 - M0) / 2][b + (N1 - M1) / 2], g = frames[f]
// (or f): the central M0 x M1 of each (chosen) centred pattern
__global__ void ws_crop_center_kernel(long long nf, int N0, int N1, int M0, int M1, const float* __restrict__ I,
                                      const int* __restrict__ frames, float scale, float* __restrict__ out) {
  const long long n = nf * M0 * M1;
  const int o0 = (N0 - M0) / 2, o1 = (N1 - M1) / 2;
  WS_LOOP(i, n) {
    const long long f = i / ((long long)M0 * M1);
    const int r = (int)(i % ((long long)M0 * M1));
    const int a = r / M1, b = r - a * M1;
    const long long g = frames ? (long long)frames[f] : f;
    out[i] = scale * I[(g * N0 + a + o0) * N1 + b + o1];
  }
}

// O[u][v] = bilinear sample of Oh at (u / f, v / f), clamped to Oh's edges
__global__ void ws_upsample_kernel(int Uh, int Vh, const float2* __restrict__ Oh, int U, int V, int f,
                                   float2* __restrict__ O) {
  const long long n = (long long)U * V;
  const float inv = 1.f / (float)f;
  WS_LOOP(i, n) {
    const int u = (int)(i / V), v = (int)(i % V);
    const float su = fminf(u * inv, (float)(Uh - 1)), sv = fminf(v * inv, (float)(Vh - 1));
    const int u0 = (int)su, v0 = (int)sv;
    const int u1 = u0 + 1 < Uh ? u0 + 1 : u0, v1 = v0 + 1 < Vh ? v0 + 1 : v0;
    const float du = su - u0, dv = sv - v0;
    const float2 a = Oh[(size_t)u0 * Vh + v0], b = Oh[(size_t)u0 * Vh + v1];
    const float2 c = Oh[(size_t)u1 * Vh + v0], d = Oh[(size_t)u1 * Vh + v1];
    const float w00 = (1.f - du) * (1.f - dv), w01 = (1.f - du) * dv, w10 = du * (1.f - dv), w11 = du * dv;
    O[i] = make_float2(w00 * a.x + w01 * b.x + w10 * c.x + w11 * d.x, w00 * a.y + w01 * b.y + w10 * c.y + w11 * d.y);
  }
}


// The network's last layer, 32 -> 2 channels with an FP32 output, on the CUDA
// cores.  Four lanes share a pixel, each summing 8 of its 32 input channels:
// a warp load then covers 8 pixels' 64 contiguous bytes (4 cache lines), where
// one lane per pixel reading 16 of them touches 16 lines per load and the L1
// wavefronts bound the kernel.  A lane owns 4 pixels 8 apart (a warp: 32
// consecutive pixels of a row) and accumulates channel pairs in packed FP32x2
// FMAs (even and odd channels in the two halves); the halves and then the four
// lanes' sums are added at the end.
constexpr int kC2Threads = 256;

PTY_DEV unsigned long long fma2(unsigned long long a, unsigned long long b, unsigned long long c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
PTY_DEV unsigned long long pack2(float lo, float hi) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
PTY_DEV float2 unpack2(unsigned long long r) {
  float2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}

__global__ void __launch_bounds__(kC2Threads) ws_conv_c32o2_kernel(int Bt, int H, int W,
                                                                  const __nv_bfloat16* __restrict__ X,
                                                                  const __nv_bfloat16* __restrict__ Wt,
                                                                  const float* __restrict__ bias, int relu,
                                                                  float* __restrict__ out32) {
  __shared__ __align__(16) float wsm[9][2][32];             // [tap][co][ci]
  for (int i = threadIdx.x; i < 2 * 9 * 32; i += blockDim.x) {
    const int co = i / 288, k = i % 288;                    // Wt[co][tap 32 + ci]
    wsm[k / 32][co][k % 32] = __bfloat162float(Wt[i]);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, q = lane & 3, pc = lane >> 2;
  const int wpb = blockDim.x >> 5;
  const long long xblocks = W / 32, units = (long long)Bt * H * xblocks;
  const float b0 = bias[0], b1 = bias[1];
  for (long long u0 = (long long)blockIdx.x * wpb + (threadIdx.x >> 5); u0 < units;
       u0 += (long long)gridDim.x * wpb) {
    const int xb = (int)(u0 % xblocks) * 32;
    const long long t = u0 / xblocks;
    const int y = (int)(t % H), b = (int)(t / H);
    unsigned long long acc[4][2];
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[u][0] = acc[u][1] = 0ull;
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
      const int yy = y + tap / 3 - 1, dx = tap % 3 - 1;
      if (yy < 0 || yy >= H) continue;                      // the same for the whole warp
      const float4* wp = reinterpret_cast<const float4*>(&wsm[tap][0][8 * q]);
      const float4 w00 = wp[0], w01 = wp[1];                // co 0, channels 8q .. 8q + 7
      const float4 w10 = wp[8], w11 = wp[9];                // co 1 (32 floats further)
      const unsigned long long wc0[4] = {pack2(w00.x, w00.y), pack2(w00.z, w00.w), pack2(w01.x, w01.y),
                                         pack2(w01.z, w01.w)};
      const unsigned long long wc1[4] = {pack2(w10.x, w10.y), pack2(w10.z, w10.w), pack2(w11.x, w11.y),
                                         pack2(w11.z, w11.w)};
      const __nv_bfloat16* xrow = X + ((size_t)(b * H + yy) * W) * 32 + 8 * q;
      uint4 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int x = xb + pc + 8 * u + dx;
        v[u] = (x >= 0 && x < W) ? __ldg(reinterpret_cast<const uint4*>(xrow + (size_t)x * 32))
                                 : make_uint4(0u, 0u, 0u, 0u);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const unsigned int wd[4] = {v[u].x, v[u].y, v[u].z, v[u].w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          // a bf16 pair (channels 2e, 2e + 1 of the chunk) as two floats
          const unsigned long long xe = pack2(__uint_as_float(wd[e] << 16), __uint_as_float(wd[e] & 0xffff0000u));
          acc[u][0] = fma2(xe, wc0[e], acc[u][0]);
          acc[u][1] = fma2(xe, wc1[e], acc[u][1]);
        }
      }
    }
    float r[4][2];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const float2 h = unpack2(acc[u][c]);
        float sum = h.x + h.y;
        sum += __shfl_xor_sync(0xffffffffu, sum, 1);
        sum += __shfl_xor_sync(0xffffffffu, sum, 2);
        r[u][c] = sum;
      }
    }
    // lane q writes pixel u = q of its column: a warp stores 32 consecutive pixels
    float o0 = r[0][0], o1 = r[0][1];
#pragma unroll
    for (int u = 1; u < 4; ++u)
      if (q == u) {
        o0 = r[u][0];
        o1 = r[u][1];
      }
    o0 += b0;
    o1 += b1;
    if (relu) {
      o0 = fmaxf(o0, 0.f);
      o1 = fmaxf(o1, 0.f);
    }
    const int x = xb + pc + 8 * q;
    *reinterpret_cast<float2*>(out32 + ((size_t)(b * H + y) * W + x) * 2) = make_float2(o0, o1);
  }
}

template <int COUT, int VEC, int PX, int CIN>
void direct_grid(int B, int H, int W, int Cin, const void* X, const void* Wt, const float* bias, int relu,
                 const void* skip, void* out, float* out32, size_t smem, cudaStream_t st) {
  const long long Q = (long long)B * H * (W / PX);
  long long g = (Q + kDirThreads - 1) / kDirThreads;
  if (g > 32 * 152) g = 32 * 152;
  ws_conv_direct_kernel<COUT, VEC, PX, CIN><<<(unsigned)g, kDirThreads, smem, st>>>(
      B, H, W, Cin, (const __nv_bfloat16*)X, (const __nv_bfloat16*)Wt, bias, relu, (const __nv_bfloat16*)skip,
      (__nv_bfloat16*)out, out32);
}

template <int COUT>
int launch_direct(int B, int H, int W, int Cin, const void* X, const void* Wt, const float* bias, int relu,
                  const void* skip, void* out, float* out32, cudaStream_t st) {
  const size_t smem = (size_t)9 * Cin * COUT * sizeof(float);
  const bool v8 = Cin % 8 == 0 && ((uintptr_t)X & 15u) == 0;
  // pixels per thread: more for narrow outputs (fewer accumulators)
  constexpr int PXW = COUT <= 4 ? 4 : 2;
  if (W % (32 * PXW) == 0) {
    // the network's shapes with C_in fixed at compile time: 2 -> 32 and 32 -> 2
    if (COUT == 32 && Cin == 2)
      direct_grid<COUT, 2, PXW, 2>(B, H, W, Cin, X, Wt, bias, relu, skip, out, out32, smem, st);
    else if (COUT == 2 && Cin == 32 && v8)
      direct_grid<COUT, 8, PXW, 32>(B, H, W, Cin, X, Wt, bias, relu, skip, out, out32, smem, st);
    else if (v8)
      direct_grid<COUT, 8, PXW, 0>(B, H, W, Cin, X, Wt, bias, relu, skip, out, out32, smem, st);
    else
      direct_grid<COUT, 2, PXW, 0>(B, H, W, Cin, X, Wt, bias, relu, skip, out, out32, smem, st);
  } else {
    if (v8) direct_grid<COUT, 8, 1, 0>(B, H, W, Cin, X, Wt, bias, relu, skip, out, out32, smem, st);
    else direct_grid<COUT, 2, 1, 0>(B, H, W, Cin, X, Wt, bias, relu, skip, out, out32, smem, st);
  }
  return check_launch("ws_conv_direct_kernel");
}

}  // namespace
}  // namespace pty

extern "C" int pty_ws_conv3x3_direct(int32_t B, int32_t H, int32_t W, int32_t Cin, int32_t Cout, const void* X,
                                     const void* Wt, const float* bias, int32_t relu, const void* skip, void* out,
                                     float* out32, void* stream) {
  if (B < 1 || H < 1 || W < 1 || !X || !Wt || !bias || (!out && !out32))
    return set_error(PTY_ERR_ARG, "pty_ws_conv3x3_direct: bad arguments");
  if (Cin < 2 || Cin > 32 || (Cin & 1)) return set_error(PTY_ERR_UNSUPPORTED, "pty_ws_conv3x3_direct: C_in must be even, 2..32");
  if (((uintptr_t)X & 3) || ((uintptr_t)Wt & 1) || ((uintptr_t)skip & 3) || ((uintptr_t)out & 15) ||
      ((uintptr_t)out32 & 15))
    return set_error(PTY_ERR_ARG, "pty_ws_conv3x3_direct: X and skip must be 4-byte, out and out32 16-byte aligned");
  if ((long long)B * H * W >= (1ll << 31)) return set_error(PTY_ERR_ARG, "pty_ws_conv3x3_direct: too many pixels");
  cudaStream_t st = (cudaStream_t)stream;
  if (Cin == 32 && Cout == 2 && !out && !skip && W % 32 == 0 && ((uintptr_t)X & 15) == 0) {
    const long long units = (long long)B * H * (W / 32);
    const long long wpb = kC2Threads / 32;
    long long g = (units + wpb - 1) / wpb;
    if (g > 16 * 152) g = 16 * 152;
    ws_conv_c32o2_kernel<<<(unsigned)g, kC2Threads, 0, st>>>(B, H, W, (const __nv_bfloat16*)X,
                                                            (const __nv_bfloat16*)Wt, bias, relu, out32);
    return check_launch("ws_conv_c32o2_kernel");
  }
  switch (Cout) {
    case 2: return launch_direct<2>(B, H, W, Cin, X, Wt, bias, relu, skip, out, out32, st);
    case 4: return launch_direct<4>(B, H, W, Cin, X, Wt, bias, relu, skip, out, out32, st);
    case 8: return launch_direct<8>(B, H, W, Cin, X, Wt, bias, relu, skip, out, out32, st);
    case 16: return launch_direct<16>(B, H, W, Cin, X, Wt, bias, relu, skip, out, out32, st);
    case 32: return launch_direct<32>(B, H, W, Cin, X, Wt, bias, relu, skip, out, out32, st);
  }
  return set_error(PTY_ERR_UNSUPPORTED, "pty_ws_conv3x3_direct: C_out must be 2, 4, 8, 16 or 32");
}

extern "C" int pty_ws_crop_center(int32_t nf, int32_t N0, int32_t N1, int32_t M0, int32_t M1, const float* I,
                                  const int32_t* frames, float scale, float* out, void* stream) {
  if (nf < 1 || M0 < 1 || M1 < 1 || M0 > N0 || M1 > N1 || !I || !out)
    return set_error(PTY_ERR_ARG, "pty_ws_crop_center: bad arguments");
  const long long n = (long long)nf * M0 * M1;
  ws_crop_center_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(nf, N0, N1, M0, M1, I, frames, scale, out);
  return ws_launched("ws_crop_center_kernel");
}

namespace pty {
namespace {

// Per-frame phase alignment of predicted exit waves before they are stitched
// again: a frame's far-field data fix its object phase only up to a constant,
// so the network's frames disagree by per-frame offsets.  For frame f with
// object window starting at (a_f, b_f):
//   z_f = sum_r psi_f(r) conj(P(r) O(a_f + r0, b_f + r1)),  psi_f *= conj(z_f) / |z_f|
// (one block per frame, a fixed-order block sum: deterministic).
constexpr int kAlignThreads = 256;
__global__ void __launch_bounds__(kAlignThreads) ws_align_phase_kernel(int M0, int M1, const int* __restrict__ win,
                                                                       int U, int V, const float2* __restrict__ O,
                                                                       const float2* __restrict__ P,
                                                                       float2* __restrict__ psi) {
  __shared__ float2 red[kAlignThreads];
  const int f = blockIdx.x;
  const int a = win[2 * f], b = win[2 * f + 1];
  if (a < 0 || b < 0 || a > U - M0 || b > V - M1) return;   // a window outside the object: frame left as is
  const int npix = M0 * M1;
  float2* fr = psi + (size_t)f * npix;
  float2 acc = make_float2(0.f, 0.f);
  for (int pix = threadIdx.x; pix < npix; pix += blockDim.x) {
    const int r0 = pix / M1, r1 = pix - r0 * M1;
    const float2 po = cmul(P[pix], O[(size_t)(a + r0) * V + b + r1]);
    acc = cadd(acc, cmulc(fr[pix], po));
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = cadd(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  const float2 z = red[0];
  const float m = sqrtf(z.x * z.x + z.y * z.y);
  const float2 rot = m > 0.f ? make_float2(z.x / m, -z.y / m) : make_float2(1.f, 0.f);
  for (int pix = threadIdx.x; pix < npix; pix += blockDim.x) fr[pix] = cmul(fr[pix], rot);
}

}  // namespace
}  // namespace pty

extern "C" int pty_ws_align_phase(int32_t nf, int32_t M0, int32_t M1, const int32_t* win, int32_t U, int32_t V,
                                  const void* O, const void* P, void* psi, void* stream) {
  if (nf < 1 || M0 < 1 || M1 < 1 || U < M0 || V < M1 || !win || !O || !P || !psi)
    return set_error(PTY_ERR_ARG, "pty_ws_align_phase: bad arguments");
  if ((long long)M0 * M1 >= (1ll << 31)) return set_error(PTY_ERR_ARG, "pty_ws_align_phase: frame too large");
  ws_align_phase_kernel<<<(unsigned)nf, kAlignThreads, 0, (cudaStream_t)stream>>>(
      M0, M1, win, U, V, (const float2*)O, (const float2*)P, (float2*)psi);
  return ws_launched("ws_align_phase_kernel");
}

extern "C" int pty_ws_upsample_object(int32_t Uh, int32_t Vh, const void* Oh, int32_t U, int32_t V, int32_t f,
                                      void* O, void* stream) {
  if (Uh < 1 || Vh < 1 || U < 1 || V < 1 || f < 1 || !Oh || !O)
    return set_error(PTY_ERR_ARG, "pty_ws_upsample_object: bad arguments");
  const long long n = (long long)U * V;
  ws_upsample_kernel<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(Uh, Vh, (const float2*)Oh, U, V, f, (float2*)O);
  return ws_launched("ws_upsample_kernel");
}
