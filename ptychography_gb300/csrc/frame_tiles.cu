// Frame tiles and the tile autotuner.
//
// A frame tile is the number of CTAs that transform one frame: tile 1 is the
// single-CTA kernel (whole frame in one CTA's shared memory, frame_kernels.cu),
// tile C > 1 the cluster kernel with C CTAs per frame (cluster_frame.cuh).
// Several tiles are built for some shapes because which one is fastest
// depends on the GPU's shared memory, register file and cluster scheduling:
//
//   128^2: 1 CTA of 512 threads (one per SM) or 2-CTA clusters of 256 (two per SM)
//   256^2: 8-CTA clusters of 256 threads (two CTAs per SM), 4-CTA clusters
//          of 512 (one per SM), or (tile id 108) 8-CTA clusters of 512 threads
//          with three-stage line transforms (two CTAs, 32 warps per SM)
//   512^2: (tile id 264, the default) the staged row / column / row launches
//          through a frame scratch (staged_512.cu), or 16-CTA clusters of 512
//          threads with three-stage line transforms (tile 116, 16 values per
//          thread, 16 warps per SM) or of 256 threads (tile 16, 32 values per
//          thread); one cluster CTA per SM
//
// Tiles are chosen per op family: the background (Pmod_7) forms move more
// bytes and hold more registers than the plain ones, and the fastest tile
// differs between them.  The first plan created for a shape on a device times
// every candidate on a scratch batch of frames (about 256 MiB of waves) --
// OP_PSI1 for the plain family, OP_PSI7 for the background family; five timed
// launches each after a warm-up, fastest kept -- and keeps the winners for the
// process; a candidate replaces the first-listed default only when at least
// 3 % faster.  A plan with fewer frames than the GPU has SMs launches less
// than one wave, where per-frame latency rather than throughput decides; such
// frame counts are tuned on exactly that many frames, each count once.
// PTY_AUTOTUNE=0 in the environment skips the timing and takes the first
// candidate listed; pty_set_frame_tile forces a tile for every frame count.
// Tiles with the same line transforms give the same exit waves, object and
// probe; only the summation order of the per-frame error partials (one per
// CTA) differs.  The three-stage transforms of tiles 108 and 116 agree with
// the others to FP32 rounding.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "../../include/ptycho_gb300.h"
#include "engine.h"

namespace pty {

namespace {

struct ShapeTiles {
  int N0, N1, count;
  int tiles[4];   // first = default without autotuning
};

constexpr ShapeTiles kShapes[] = {
    {32, 32, 1, {1, 0, 0, 0}},   {64, 64, 1, {1, 0, 0, 0}},   {32, 64, 1, {1, 0, 0, 0}},
    {128, 128, 2, {1, 2, 0, 0}}, {192, 192, 1, {2, 0, 0, 0}}, {256, 256, 3, {8, 4, 108, 0}},
    {512, 512, 3, {264, 116, 16, 0}},
};

const ShapeTiles* find_shape(int N0, int N1) {
  for (const ShapeTiles& s : kShapes)
    if (s.N0 == N0 && s.N1 == N1) return &s;
  return nullptr;
}

bool tile_listed(const ShapeTiles* s, int tile) {
  for (int i = 0; i < s->count; ++i)
    if (s->tiles[i] == tile) return true;
  return false;
}

int prepare_tile(int N0, int N1, int tile) {
  if (tile == 1) return prepare_single_cta(N0, N1);
  if (N0 == 128 && N1 == 128 && tile == 2) return prepare_cluster_128x2();
  if (N0 == 192 && N1 == 192 && tile == 2) return prepare_cluster_192x2();
  if (N0 == 256 && N1 == 256 && tile == 4) return prepare_cluster_256x4();
  if (N0 == 256 && N1 == 256 && tile == 8) return prepare_cluster_256x8();
  if (N0 == 256 && N1 == 256 && tile == 108) return prepare_cluster_256x8l();
  if (N0 == 512 && N1 == 512 && tile == 16) return prepare_cluster_512x16();
  if (N0 == 512 && N1 == 512 && tile == 116) return prepare_cluster_512x16l();
  if (N0 == 512 && N1 == 512 && tile == 264) return prepare_staged_512();
  return set_error(PTY_ERR_UNSUPPORTED, "frame tile not built for this shape");
}

using Key = std::tuple<int, int, int, int, int>;   // device, N0, N1, family, frames class
std::mutex g_mu;
std::map<Key, int> g_tile;               // tuned tile per device, shape, family, frames class
std::map<Key, int> g_forced;             // tiles forced by pty_set_frame_tile

bool autotune_enabled() {
  const char* v = std::getenv("PTY_AUTOTUNE");
  return !(v && std::strcmp(v, "0") == 0);
}

// Times the family's op (OP_PSI1 / OP_PSI7) with each candidate tile on F
// scratch frames; *best = fastest.
int tune(const ShapeTiles* s, int family, int small_frames, int* best) {
  const int N0 = s->N0, N1 = s->N1;
  const size_t npix = (size_t)N0 * N1;
  // about 256 MiB of exit waves (several waves of CTAs, larger than L2), or the
  // plan's own frame count for launches too small to fill the GPU, where the
  // per-frame latency decides
  size_t F = ((size_t)256 << 20) / (npix * sizeof(float2));
  if (F < 64) F = 64;
  if (F > 8192) F = 8192;
  if (small_frames > 0) F = (size_t)small_frames;
  float2 *psi = nullptr, *tw0 = nullptr, *tw1 = nullptr, *twf = nullptr, *stage = nullptr;
  bool staged = false;
  for (int i = 0; i < s->count; ++i) staged = staged || tile_staged(s->tiles[i]);
  int stage_frames = staged_group_frames(N0, N1);
  if (stage_frames > (int)F) stage_frames = (int)F;
  float *amp = nullptr, *bg = nullptr;
  double* err = nullptr;
  const int op = family == FAM_BG ? OP_PSI7 : OP_PSI1;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = PTY_OK;
  cudaError_t e = cudaMalloc(&psi, F * npix * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&amp, F * npix * sizeof(float));
  if (e == cudaSuccess && family == FAM_BG) e = cudaMalloc(&bg, F * npix * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&err, F * 64 * sizeof(double));
  if (e == cudaSuccess && staged) e = cudaMalloc(&stage, (size_t)stage_frames * npix * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&tw0, N0 * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&tw1, N1 * sizeof(float2));
  if (e == cudaSuccess) e = cudaMalloc(&twf, N1 * sizeof(float2));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) {
    std::vector<float2> h0(N0), h1(N1), hf(N1);
    make_twiddles(N0, h0.data());
    make_twiddles(N1, h1.data());
    make_full_twiddles(N1, hf.data());
    e = cudaMemcpyAsync(tw0, h0.data(), N0 * sizeof(float2), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(tw1, h1.data(), N1 * sizeof(float2), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(twf, hf.data(), N1 * sizeof(float2), cudaMemcpyHostToDevice, st);
    // finite positive values (every byte 0x3c) in the waves and amplitudes
    if (e == cudaSuccess) e = cudaMemsetAsync(psi, 0x3c, F * npix * sizeof(float2), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(amp, 0x3c, F * npix * sizeof(float), st);
    if (e == cudaSuccess && bg) e = cudaMemsetAsync(bg, 0x3c, F * npix * sizeof(float), st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  if (e != cudaSuccess) rc = set_cuda_error(e, "frame tile autotuner set-up");
  float best_ms = INFINITY;
  *best = s->tiles[0];
  for (int i = 0; rc == PTY_OK && i < s->count; ++i) {
    const int tile = s->tiles[i];
    FrameArgs a{};
    a.psi = psi;
    a.amp = amp;
    a.amp_stride = (long long)npix;
    a.err_part = err;
    a.err_stride = 64;
    a.stage = stage;
    a.stage_frames = stage_frames;
    a.bg_in = bg;
    a.bg_out = bg;
    a.bg_stride = (long long)npix;
    a.alpha = 1e-10f;
    a.tw0 = tw0;
    a.tw1 = tw1;
    a.twf = twf;
    a.N0h = N0 / 2;
    a.N1h = N1 / 2;
    if ((rc = prepare_tile(N0, N1, tile))) break;
    if ((rc = launch_frame_op(op, N0, N1, tile, a, (int)F, st))) break;
    float ms_min = INFINITY;
    for (int r = 0; r < 5 && rc == PTY_OK; ++r) {
      e = cudaEventRecord(e0, st);
      if (e == cudaSuccess && (rc = launch_frame_op(op, N0, N1, tile, a, (int)F, st))) break;
      if (e == cudaSuccess) e = cudaEventRecord(e1, st);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e != cudaSuccess) rc = set_cuda_error(e, "frame tile autotuner timing");
      else if (ms < ms_min) ms_min = ms;
    }
    // another tile replaces the default only when at least 3 % faster, so
    // timing noise between near-equal tiles does not flip the choice
    if (rc == PTY_OK && (i == 0 || ms_min < 0.97f * best_ms)) {
      best_ms = ms_min;
      *best = tile;
    }
  }
  if (st) cudaStreamSynchronize(st);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  cudaFree(psi);
  cudaFree(amp);
  cudaFree(bg);
  cudaFree(err);
  cudaFree(tw0);
  cudaFree(tw1);
  cudaFree(twf);
  cudaFree(stage);
  return rc;
}

int current_device(int* dev) {
  cudaError_t e = cudaGetDevice(dev);
  if (e != cudaSuccess) return set_cuda_error(e, "cudaGetDevice");
  return PTY_OK;
}

}  // namespace

bool frame_shape_supported(int N0, int N1) { return find_shape(N0, N1) != nullptr; }

int staged_group_frames(int N0, int N1) {
  // about 2 GiB of scratch: launches large enough that their tails and the
  // gaps between the three launches of a group cost little (measured: groups
  // of 1024 512^2 frames ran Pmod_7 3 % faster than groups of 256, 17 %
  // faster than groups of 64, whose scratch mostly stays in L2)
  const long long per = (long long)N0 * N1 * (long long)sizeof(float2);
  const long long g = ((long long)1 << 31) / per;
  return g < 1 ? 1 : (int)g;
}

int frame_tile_candidates(int N0, int N1, int* tiles, int cap) {
  const ShapeTiles* s = find_shape(N0, N1);
  if (!s) return 0;
  for (int i = 0; i < s->count && i < cap; ++i) tiles[i] = s->tiles[i];
  return s->count;
}

int max_frame_tile(int N0, int N1) {
  const ShapeTiles* s = find_shape(N0, N1);
  int m = 1;
  for (int i = 0; s && i < s->count; ++i) m = tile_ctas(s->tiles[i]) > m ? tile_ctas(s->tiles[i]) : m;
  return m;
}

// Frame counts below this many per SM form their own tuning class, tuned on
// exactly that many frames (one class per count, the counts being small).
constexpr int kSmallFramesPerSM = 1;

int choose_frame_tile(int N0, int N1, int family, int nframes, int* tile) {
  const ShapeTiles* s = find_shape(N0, N1);
  if (!s) return set_error(PTY_ERR_SHAPE, "frame shape not supported by the fused FFT kernels");
  if (family != FAM_PLAIN && family != FAM_BG) return set_error(PTY_ERR_ARG, "unknown op family");
  int dev = 0;
  PTY_TRY(current_device(&dev));
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    sms = 0;
  }
  const int small = (nframes > 0 && nframes < kSmallFramesPerSM * sms) ? nframes : 0;
  std::lock_guard<std::mutex> lock(g_mu);
  // a forced tile (pty_set_frame_tile, class 0) applies to every frame count
  auto forced = g_forced.find(Key{dev, N0, N1, family, 0});
  const Key key{dev, N0, N1, family, small};
  auto it = g_tile.find(key);
  int t = s->tiles[0];
  if (forced != g_forced.end()) {
    t = forced->second;
  } else if (it != g_tile.end()) {
    t = it->second;
  } else {
    if (s->count > 1 && autotune_enabled()) PTY_TRY(tune(s, family, small, &t));
    g_tile[key] = t;
  }
  PTY_TRY(prepare_tile(N0, N1, t));
  *tile = t;
  return PTY_OK;
}

int launch_frame_op(int op, int N0, int N1, int tile, const FrameArgs& a, int nframes,
                    cudaStream_t st) {
  if (nframes <= 0) return PTY_OK;
  if (tile == 1) return launch_single_cta_op(op, N0, N1, a, nframes, st);
  if (N0 == N1) {
    if (N0 == 128 && tile == 2) return launch_cluster_128x2(op, a, nframes, st);
    if (N0 == 192 && tile == 2) return launch_cluster_192x2(op, a, nframes, st);
    if (N0 == 256 && tile == 4) return launch_cluster_256x4(op, a, nframes, st);
    if (N0 == 256 && tile == 8) return launch_cluster_256x8(op, a, nframes, st);
    if (N0 == 256 && tile == 108) return launch_cluster_256x8l(op, a, nframes, st);
    if (N0 == 512 && tile == 16) return launch_cluster_512x16(op, a, nframes, st);
    if (N0 == 512 && tile == 116) return launch_cluster_512x16l(op, a, nframes, st);
    if (N0 == 512 && tile == 264) return launch_staged_512(op, a, nframes, st);
  }
  return set_error(PTY_ERR_UNSUPPORTED, "frame tile not built for this shape");
}

// Inter-step twiddles of the two-step line transform of length L = A * B
// (A threads x B values, fft_line.cuh): tw[k1 * A + t] = exp(-2 pi i t k1 / L),
// evaluated in double and rounded once.
void make_twiddles(int L, float2* out) {
  int A = 16, B = L / 16;
  switch (L) {
    case 16: A = 4; B = 4; break;
    case 32: A = 4; B = 8; break;
    case 64: A = 8; B = 8; break;
    case 128: A = 8; B = 16; break;
    case 192: A = 8; B = 24; break;
    case 256: A = 16; B = 16; break;
    case 512: A = 16; B = 32; break;
  }
  for (int i = 0; i < L; ++i) out[i] = make_float2(1.f, 0.f);
  const double pi = 3.14159265358979323846;
  for (int k1 = 0; k1 < B; ++k1)
    for (int t = 0; t < A; ++t) {
      const double th = -2.0 * pi * (double)((long long)t * k1 % L) / (double)L;
      out[k1 * A + t] = make_float2((float)std::cos(th), (float)std::sin(th));
    }
}

// twf[e] = exp(-2 pi i e / L), e < L, evaluated in double and rounded once.
void make_full_twiddles(int L, float2* out) {
  const double pi = 3.14159265358979323846;
  for (int e = 0; e < L; ++e) {
    const double th = -2.0 * pi * (double)e / (double)L;
    out[e] = make_float2((float)std::cos(th), (float)std::sin(th));
  }
}

}  // namespace pty

using namespace pty;

extern "C" int pty_frame_tile_candidates(int32_t N0, int32_t N1, int32_t* tiles, int32_t cap,
                                         int32_t* count) {
  if (!count || (cap > 0 && !tiles)) return set_error(PTY_ERR_ARG, "null argument");
  int buf[4] = {0, 0, 0, 0};
  const int n = frame_tile_candidates(N0, N1, buf, 4);
  if (n == 0) return set_error(PTY_ERR_SHAPE, "frame shape not supported by the fused FFT kernels");
  for (int i = 0; i < n && i < cap; ++i) tiles[i] = buf[i];
  *count = n;
  return PTY_OK;
}

extern "C" int pty_get_frame_tile(int32_t N0, int32_t N1, int32_t family, int32_t* tile) {
  if (!tile) return set_error(PTY_ERR_ARG, "null argument");
  int t = 0;
  PTY_TRY(choose_frame_tile(N0, N1, family, 0, &t));
  *tile = t;
  return PTY_OK;
}

extern "C" int pty_set_frame_tile(int32_t N0, int32_t N1, int32_t family, int32_t tile) {
  const ShapeTiles* s = find_shape(N0, N1);
  if (!s) return set_error(PTY_ERR_SHAPE, "frame shape not supported by the fused FFT kernels");
  if (family != FAM_PLAIN && family != FAM_BG) return set_error(PTY_ERR_ARG, "unknown op family");
  if (tile != 0 && !tile_listed(s, tile))
    return set_error(PTY_ERR_ARG, "tile not built for this frame shape");
  int dev = 0;
  PTY_TRY(current_device(&dev));
  std::lock_guard<std::mutex> lock(g_mu);
  const Key key{dev, (int)N0, (int)N1, (int)family, 0};
  if (tile == 0) {   // forget the forced tile and every tuned choice for the shape
    g_forced.erase(key);
    for (auto it = g_tile.begin(); it != g_tile.end();) {
      const Key& k = it->first;
      if (std::get<0>(k) == dev && std::get<1>(k) == N0 && std::get<2>(k) == N1 &&
          std::get<3>(k) == family)
        it = g_tile.erase(it);
      else
        ++it;
    }
    return PTY_OK;
  }
  PTY_TRY(prepare_tile(N0, N1, tile));
  g_forced[key] = tile;
  return PTY_OK;
}
