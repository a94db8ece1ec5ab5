// Probe update without any device allocation: pty_psup_P_noalloc.
//
// Some callers cannot allocate device memory at all: code embedded in a host
// application that owns the whole device budget, a framework whose allocator
// forbids foreign cudaMalloc calls, or a real-time loop where an allocation
// could block.  They cannot create a plan (a plan allocates its scratch with
// cudaMalloc), so this entry point takes every input and output from the
// caller and keeps what it needs besides -- the frame chunks' partial sums and
// a device copy of the scan offsets -- in fixed arrays compiled into the
// library.
//
// Those arrays live on every GPU that loads the library, for the life of the
// process: 8 MiB of partial sums (8 chunks x 65536 pixels x 2 float2) plus
// 128 KiB of scan offsets (16384 frames x 2 int32).
//
// The offsets reach the device as kernel parameters (batches of
// kOffsetsPerLaunch frames, copied by a small kernel into g_noalloc_R): the
// launch copies its parameters when it is enqueued, so the call needs no host
// staging buffer, no pageable memcpy and no host synchronisation.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/ptycho_gb300.h"
#include "engine.h"

namespace pty {

constexpr int kNoAllocMaxPixels = 256 * 256;  // largest probe (N0 * N1) accepted
constexpr int kNoAllocMaxFrames = 16384;      // most scan positions accepted
constexpr int kNoAllocChunks = 8;             // frame chunks of the split reduction
constexpr size_t kNoAllocElems = (size_t)2 * kNoAllocChunks * kNoAllocMaxPixels;

// Partial numerators (first half) and float-float denominators (second half).
// Each call writes every slot it later reads, so nothing needs clearing.
static __device__ __align__(256) float2 g_noalloc_scratch[kNoAllocElems];
// Scan offsets of the current call, int32 [n][2].
static __device__ __align__(256) int g_noalloc_R[2 * kNoAllocMaxFrames];

// One launch's share of the offsets, passed by value (16 KiB of parameters,
// inside the 32 KiB kernel-parameter limit of sm_70 and later).
constexpr int kOffsetsPerLaunch = 2048;
struct OffsetsBatch {
  int first;                       // first frame of the batch
  int count;                       // frames in the batch
  int r[2 * kOffsetsPerLaunch];    // (r0, r1) per frame
};

__global__ void noalloc_stage_offsets_kernel(const OffsetsBatch b) {
  for (int i = threadIdx.x; i < 2 * b.count; i += blockDim.x)
    g_noalloc_R[2 * b.first + i] = b.r[i];
}

constexpr int kMaxDevices = 64;
struct NoAllocSymbols {
  float2* scratch = nullptr;
  int* R = nullptr;
};
static NoAllocSymbols g_symbols[kMaxDevices];
static std::mutex g_symbols_mutex;

// Addresses of the fixed arrays on the current device, looked up once per
// device (under a lock, so host threads driving different GPUs may call at
// the same time).  In host code the arrays' names are host-side stand-ins,
// not device addresses: only these looked-up pointers may go to a kernel.
static int symbols_on_current_device(NoAllocSymbols* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_cuda_error(e, "pty_psup_P_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices)
    return set_error(PTY_ERR_ARG, "pty_psup_P_noalloc: device index too large");
  std::lock_guard<std::mutex> lock(g_symbols_mutex);
  NoAllocSymbols& s = g_symbols[dev];
  if (!s.scratch || !s.R) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return set_cuda_error(e, "pty_psup_P_noalloc: cudaGetSymbolAddress");
    void* q = nullptr;
    e = cudaGetSymbolAddress(&q, g_noalloc_R);
    if (e != cudaSuccess) return set_cuda_error(e, "pty_psup_P_noalloc: cudaGetSymbolAddress");
    s.scratch = static_cast<float2*>(p);
    s.R = static_cast<int*>(q);
  }
  *out = s;
  return PTY_OK;
}

}  // namespace pty

using namespace pty;

extern "C" int pty_psup_P_noalloc(const pty_geometry* geom, const int64_t* R_host, const void* psi,
                                  const void* O, double* O_heatmap, int32_t recompute_heatmap,
                                  double alpha, void* P_out, void* stream) {
  if (!geom || !R_host || !psi || !O || !O_heatmap || !P_out)
    return set_error(PTY_ERR_ARG, "pty_psup_P_noalloc: null argument");
  const int n = geom->n_frames, N0 = geom->N0, N1 = geom->N1, U = geom->U, V = geom->V;
  if (n < 1 || N0 < 1 || N1 < 1 || U < 1 || V < 1)
    return set_error(PTY_ERR_ARG, "pty_psup_P_noalloc: empty geometry");
  if ((long long)N0 * N1 > kNoAllocMaxPixels)
    return set_error(PTY_ERR_RANGE,
                     "pty_psup_P_noalloc: probe larger than its fixed scratch (N0 * N1 > 65536)");
  if (n > kNoAllocMaxFrames)
    return set_error(PTY_ERR_RANGE,
                     "pty_psup_P_noalloc: more frames than its fixed scratch (n_frames > 16384)");
  for (int f = 0; f < n; ++f) {
    const long long r0 = R_host[2 * f], r1 = R_host[2 * f + 1];
    if (r0 > 0 || r1 > 0 || -r0 + N0 > U || -r1 + N1 > V)
      return set_error(PTY_ERR_RANGE,
                       "pty_psup_P_noalloc: scan position places the probe window outside the object");
  }
  NoAllocSymbols sym;
  int rc = symbols_on_current_device(&sym);
  if (rc != PTY_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  OffsetsBatch b;
  for (int f0 = 0; f0 < n; f0 += kOffsetsPerLaunch) {
    b.first = f0;
    b.count = n - f0 < kOffsetsPerLaunch ? n - f0 : kOffsetsPerLaunch;
    for (int i = 0; i < 2 * b.count; ++i) b.r[i] = (int)R_host[2 * f0 + i];
    noalloc_stage_offsets_kernel<<<1, 256, 0, st>>>(b);
    rc = check_launch("noalloc_stage_offsets_kernel");
    if (rc != PTY_OK) return rc;
  }
  const int K = n < kNoAllocChunks ? n : kNoAllocChunks;
  float2* part_num = sym.scratch;
  float2* part_den = sym.scratch + (size_t)kNoAllocChunks * kNoAllocMaxPixels;
  return launch_psup_P(n, N0, N1, U, V, sym.R, (const float2*)psi, (const float2*)O, part_num,
                       part_den, K, O_heatmap, recompute_heatmap != 0, (float)alpha,
                       (float2*)P_out, st);
}
