// Plan, iteration drivers and the extern "C" surface of libptycho_gb300.
//
// The ERA and DM loops below follow the control flow of the reference
// (ptychography/era.py:13-332, ptychography/dm.py:13-333) operation for
// operation, with every array resident on the device: the per-iteration
// numerator/denominator all-reduces of the MPI version become the fixed-order
// gathers of overlap_kernels.cu, and the modulus projection is the fused frame
// kernel.  Nothing is copied to the host inside the loop; the error histories
// are written to device arrays.
#include <atomic>
#include <cmath>
#include <mutex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ptycho_gb300.h"
#include "engine.h"

namespace pty {

static thread_local std::string g_last_error;

int set_error(int code, const char* msg) {
  g_last_error = msg;
  return code;
}
int set_cuda_error(cudaError_t e, const char* where) {
  g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
  return PTY_ERR_CUDA;
}
static std::atomic<long long> g_launches{0};
void count_launches(long long k) { g_launches += k; }
long long launch_total() { return g_launches.load(); }

// One int per GPU, set by a kernel whose bounded wait ran out (the TMA-staged
// and tensor-core kernels).  Allocated before any stream capture: by
// pty_plan_create, or by the first call of an entry point that uses it.
static int* g_timeout_flag[64] = {};
static std::mutex g_timeout_mutex;
int device_timeout_flag(int** out) {
  int dev = 0;
  PTY_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(PTY_ERR_ARG, "device index too large");
  std::lock_guard<std::mutex> lock(g_timeout_mutex);
  if (!g_timeout_flag[dev]) {
    void* q = nullptr;
    PTY_CUDA(cudaMalloc(&q, sizeof(int)));
    PTY_CUDA(cudaMemset(q, 0, sizeof(int)));
    g_timeout_flag[dev] = static_cast<int*>(q);
  }
  *out = g_timeout_flag[dev];
  return PTY_OK;
}

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::once_flag g_encode_once;
int tensor_map_encoder(PFN_cuTensorMapEncodeTiled_v12000* out) {
  std::call_once(g_encode_once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  });
  if (!g_encode) return set_error(PTY_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  *out = g_encode;
  return PTY_OK;
}

int check_launch(const char* where) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_cuda_error(e, where);
  g_launches += 1;
  return PTY_OK;
}

}  // namespace pty

using namespace pty;

struct pty_plan {
  int n = 0, N0 = 0, N1 = 0, U = 0, V = 0;
  int* d_R = nullptr;
  int* d_tile_ptr = nullptr;
  int* d_tile_frames = nullptr;
  TileLists tl{};
  float2* d_tw0 = nullptr;
  float2* d_tw1 = nullptr;
  float2* d_twf = nullptr;       // W_N1^e, e < N1
  double* d_heatP = nullptr;     // P_heatmap cache
  double* d_heatP2 = nullptr;    // DM metric-branch heatmap
  double* d_heatO = nullptr;     // O_heatmap cache
  double* d_heatO2 = nullptr;
  int K = 1;                     // psup_P frame chunks
  float2* d_part_num = nullptr;
  float2* d_part_den = nullptr;
  int Km = 1;                    // background-mean frame chunks
  float2* d_mean_part = nullptr;
  double* d_err_part = nullptr;  // [n * eslots]
  float2* d_stage = nullptr;     // frame scratch of a staged tile
  uint8_t* d_mask_blk = nullptr; // the mask in the staged tile's column-block order
  int stage_frames = 0;
  int* d_timeout = nullptr;      // the device's timeout flag (not owned)
  int tile[2] = {1, 1};          // CTAs per frame of the fused frame kernels, per op family
  int eslots = 1;                // error-partial slots per frame (the larger family tile)
  int ndn = 304;                 // diffnorm blocks per array (two per SM)
  double* d_dn_part = nullptr;   // [2 arrays][ndn][2]
  int* d_shift = nullptr;
  float2* d_bakO = nullptr;
  float2* d_bakP = nullptr;
  float2* d_Os = nullptr;
  float2* d_Ps = nullptr;
  float2* d_tmpO = nullptr;
  float2* d_tmpP = nullptr;
  float* d_bgf = nullptr;        // [n][N0][N1] per-frame background after Pmod_7
  float* d_b0 = nullptr;         // [N0][N1]
  float2* d_psi_tmp = nullptr;   // DM centring roll scratch (lazy)
  double* d_sum = nullptr;
  cudaStream_t cap = nullptr;    // capture stream
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  // last captured loop of each kind (ERA, DM): replayed when a call repeats it
  struct CachedGraph {
    std::string key;
    cudaGraphExec_t exec = nullptr;
    int heat_valid = 0;
    long long kernels = 0;
  } graphs[2];
  // last batch graph launched with this plan first (pty_run_batch)
  cudaGraphExec_t batch_exec = nullptr;
  std::string batch_key;
  std::vector<char> batch_heat;
  long long batch_kernels = 0;
  long long serial = 0;          // unique per plan in the process (batch keys)
  std::vector<void*> allocs;
};

static int dalloc(pty_plan* p, void** ptr, size_t bytes) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(ptr, bytes);
  if (e != cudaSuccess) {
    *ptr = nullptr;
    cudaGetLastError();
    return set_error(PTY_ERR_NOMEM, "device scratch allocation failed");
  }
  p->allocs.push_back(*ptr);
  return PTY_OK;
}
template <class T>
static int dalloc_t(pty_plan* p, T** ptr, size_t count) {
  return dalloc(p, reinterpret_cast<void**>(ptr), count * sizeof(T));
}



extern "C" int pty_shape_supported(int32_t N0, int32_t N1) {
  return frame_shape_supported(N0, N1) ? 1 : 0;
}

extern "C" int pty_version(void) { return 100; }

extern "C" int64_t pty_launch_count(void) { return (int64_t)launch_total(); }

extern "C" const char* pty_last_error(void) { return g_last_error.c_str(); }

extern "C" int pty_timeout_status(int32_t* timed_out) {
  if (!timed_out) return set_error(PTY_ERR_ARG, "pty_timeout_status: null argument");
  int* flag = nullptr;
  PTY_TRY(device_timeout_flag(&flag));
  int h = 0;
  PTY_CUDA(cudaMemcpy(&h, flag, sizeof(int), cudaMemcpyDeviceToHost));
  if (h) PTY_CUDA(cudaMemset(flag, 0, sizeof(int)));
  *timed_out = h;
  return PTY_OK;
}

extern "C" int pty_plan_destroy(pty_plan* p) {
  if (!p) return PTY_OK;
  for (void* a : p->allocs) cudaFree(a);
  if (p->d_psi_tmp) cudaFree(p->d_psi_tmp);
  for (auto& cg : p->graphs)
    if (cg.exec) cudaGraphExecDestroy(cg.exec);
  if (p->batch_exec) cudaGraphExecDestroy(p->batch_exec);
  if (p->cap) cudaStreamDestroy(p->cap);
  if (p->ev_in) cudaEventDestroy(p->ev_in);
  if (p->ev_out) cudaEventDestroy(p->ev_out);
  delete p;
  return PTY_OK;
}

extern "C" int pty_plan_geometry(const pty_plan* p, pty_geometry* g) {
  if (!p || !g) return set_error(PTY_ERR_ARG, "pty_plan_geometry: null argument");
  g->n_frames = p->n;
  g->N0 = p->N0;
  g->N1 = p->N1;
  g->U = p->U;
  g->V = p->V;
  return PTY_OK;
}

extern "C" int pty_plan_create(const pty_geometry* g, const int64_t* R_host, pty_plan** out) {
  if (!g || !R_host || !out) return set_error(PTY_ERR_ARG, "null argument");
  *out = nullptr;
  const int n = g->n_frames, N0 = g->N0, N1 = g->N1, U = g->U, V = g->V;
  if (n < 1 || N0 < 1 || N1 < 1 || U < 1 || V < 1) return set_error(PTY_ERR_ARG, "empty geometry");
  if (!frame_shape_supported(N0, N1))
    return set_error(PTY_ERR_SHAPE, "frame shape not supported by the fused FFT kernels");
  std::vector<int> R(2 * (size_t)n);
  for (int f = 0; f < n; ++f) {
    const long long r0 = R_host[2 * f], r1 = R_host[2 * f + 1];
    if (r0 > 0 || r1 > 0 || -r0 + N0 > U || -r1 + N1 > V)
      return set_error(PTY_ERR_RANGE, "scan position places the probe window outside the object");
    R[2 * f] = (int)r0;
    R[2 * f + 1] = (int)r1;
  }
  int* timeout_flag = nullptr;
  PTY_TRY(device_timeout_flag(&timeout_flag));
  pty_plan* p = new pty_plan();
  p->n = n; p->N0 = N0; p->N1 = N1; p->U = U; p->V = V;
  p->d_timeout = timeout_flag;
  static std::atomic<long long> next_serial{1};
  p->serial = next_serial++;
  int rc = PTY_OK;
  auto fail = [&](int code) { pty_plan_destroy(p); return code; };

  // per-tile ascending frame lists for the object gathers
  const int T = kGatherTileCols, TR = kGatherTileRows;
  const int ntu = (U + TR - 1) / TR, ntv = (V + T - 1) / T;
  std::vector<int> ptr((size_t)ntu * ntv + 1, 0), frames;
  {
    std::vector<std::vector<int>> lists((size_t)ntu * ntv);
    for (int f = 0; f < n; ++f) {
      const int u0 = -R[2 * f], v0 = -R[2 * f + 1];
      const int tu0 = u0 / TR, tu1 = (u0 + N0 - 1) / TR, tv0 = v0 / T, tv1 = (v0 + N1 - 1) / T;
      for (int tu = tu0; tu <= tu1 && tu < ntu; ++tu)
        for (int tv = tv0; tv <= tv1 && tv < ntv; ++tv) lists[(size_t)tu * ntv + tv].push_back(f);
    }
    for (size_t t = 0; t < lists.size(); ++t) {
      ptr[t + 1] = ptr[t] + (int)lists[t].size();
      frames.insert(frames.end(), lists[t].begin(), lists[t].end());
    }
  }
  const size_t npix = (size_t)N0 * N1, nobj = (size_t)U * V;
  if ((rc = dalloc_t(p, &p->d_R, R.size()))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_tile_ptr, ptr.size()))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_tile_frames, frames.size() + 1))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_tw0, (size_t)N0))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_tw1, (size_t)N1))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_twf, (size_t)N1))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_heatP, nobj))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_heatP2, nobj))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_heatO, npix))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_heatO2, npix))) return fail(rc);
  {
    // enough frame chunks for about four waves of probe-gather blocks
    const int ntiles = psup_P_tiles(N0, N1);
    int K = (2432 + ntiles - 1) / ntiles;
    if (K > 64) K = 64;
    if (K > n) K = n;
    if (K < 1) K = 1;
    p->K = K;
    const int pblocks = (int)((npix + 255) / 256);
    int Km = (608 + pblocks - 1) / pblocks;
    if (Km > 64) Km = 64;
    if (Km > n) Km = n;
    if (Km < 1) Km = 1;
    p->Km = Km;
  }
  if ((rc = dalloc_t(p, &p->d_part_num, (size_t)p->K * npix))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_part_den, (size_t)p->K * npix))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_mean_part, (size_t)(p->Km > p->K ? p->Km : p->K) * npix))) return fail(rc);
  if ((rc = choose_frame_tile(N0, N1, FAM_PLAIN, n, &p->tile[FAM_PLAIN]))) return fail(rc);
  if ((rc = choose_frame_tile(N0, N1, FAM_BG, n, &p->tile[FAM_BG]))) return fail(rc);
  p->eslots = tile_ctas(p->tile[0]) > tile_ctas(p->tile[1]) ? tile_ctas(p->tile[0])
                                                             : tile_ctas(p->tile[1]);
  if ((rc = dalloc_t(p, &p->d_err_part, (size_t)n * p->eslots))) return fail(rc);
  if (tile_staged(p->tile[0]) || tile_staged(p->tile[1])) {
    p->stage_frames = staged_group_frames(N0, N1) < n ? staged_group_frames(N0, N1) : n;
    if ((rc = dalloc_t(p, &p->d_stage, (size_t)p->stage_frames * npix))) return fail(rc);
    if ((rc = dalloc_t(p, &p->d_mask_blk, npix))) return fail(rc);
  }
  if ((rc = dalloc_t(p, &p->d_dn_part, (size_t)4 * p->ndn))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_shift, 2))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_bakO, nobj))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_bakP, npix))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_Os, nobj))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_Ps, npix))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_tmpO, nobj))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_tmpP, npix))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_b0, npix))) return fail(rc);
  if ((rc = dalloc_t(p, &p->d_sum, 4))) return fail(rc);

  std::vector<float2> tw0(N0), tw1(N1);
  make_twiddles(N0, tw0.data());
  make_twiddles(N1, tw1.data());
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = cudaMemcpy(p->d_R, R.data(), R.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p->d_tile_ptr, ptr.data(), ptr.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !frames.empty())
    e = cudaMemcpy(p->d_tile_frames, frames.data(), frames.size() * sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p->d_tw0, tw0.data(), N0 * sizeof(float2), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p->d_tw1, tw1.data(), N1 * sizeof(float2), cudaMemcpyHostToDevice);
  {
    std::vector<float2> twf(N1);
    make_full_twiddles(N1, twf.data());
    if (e == cudaSuccess) e = cudaMemcpy(p->d_twf, twf.data(), N1 * sizeof(float2), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_in, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_out, cudaEventDisableTiming);
  if (e != cudaSuccess) return fail(set_cuda_error(e, "pty_plan_create"));
  p->tl = TileLists{TR, T, ntu, ntv, p->d_tile_ptr, p->d_tile_frames};
  *out = p;
  return PTY_OK;
}

// ------------------------------------------------------------------ helpers
static FrameArgs base_args(const pty_plan* p) {
  FrameArgs a{};
  a.U = p->U;
  a.V = p->V;
  a.R = p->d_R;
  a.tw0 = p->d_tw0;
  a.tw1 = p->d_tw1;
  a.twf = p->d_twf;
  a.amp_stride = (long long)p->N0 * p->N1;
  a.N0h = p->N0 / 2;
  a.N1h = p->N1 / 2;
  a.err_stride = p->eslots;
  a.stage = p->d_stage;
  a.stage_frames = p->stage_frames;
  a.mask_blk = p->d_mask_blk;
  a.timeout = p->d_timeout;
  return a;
}

static int frame_op(const pty_plan* p, int op, const FrameArgs& a, int nframes, cudaStream_t st) {
  return launch_frame_op(op, p->N0, p->N1, p->tile[frame_family(op)], a, nframes, st);
}

// Pmod_P (era.py:597-610): the probe as a single frame through the Pmod_1 path
static int pmod_probe(pty_plan* p, float2* P, const float* Pamp, const uint8_t* mask, float alpha,
                      cudaStream_t st) {
  FrameArgs a = base_args(p);
  a.psi = P;
  a.amp = Pamp;
  a.amp_stride = 0;
  a.mask = mask;
  a.alpha = alpha;
  return frame_op(p, OP_PSI1, a, 1, st);
}

static int copy_d2d(void* dst, const void* src, size_t bytes, cudaStream_t st) {
  PTY_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st));
  return PTY_OK;
}

// eCon partials for the quantity the update method tracks (era.py:202-208)
static int econ_partials(pty_plan* p, int upd, const float2* bakO, const float2* O,
                         const float2* bakP, const float2* P, cudaStream_t st, int* ndn_total) {
  const size_t nobj = (size_t)p->U * p->V, npix = (size_t)p->N0 * p->N1;
  int used = 0;
  if (upd & 1) {
    PTY_TRY(launch_diffnorm(bakO, O, (long long)nobj, p->d_dn_part, p->ndn, st));
    used += p->ndn;
  }
  if (upd & 2) {
    PTY_TRY(launch_diffnorm(bakP, P, (long long)npix, p->d_dn_part + 2 * used, p->ndn, st));
    used += p->ndn;
  }
  *ndn_total = used;
  return PTY_OK;
}

// centre |P|^2 and shift O (and psi) with it (era.py:172-186, dm.py:65-82)
static int centre(pty_plan* p, float2* P, float2* O, float2* psi, cudaStream_t st) {
  const size_t nobj = (size_t)p->U * p->V, npix = (size_t)p->N0 * p->N1;
  PTY_TRY(launch_probe_shift(P, p->N0, p->N1, p->d_shift, st));
  PTY_TRY(launch_roll(P, p->d_tmpP, 1, p->N0, p->N1, p->d_shift, st));
  PTY_TRY(copy_d2d(P, p->d_tmpP, npix * sizeof(float2), st));
  PTY_TRY(launch_roll(O, p->d_tmpO, 1, p->U, p->V, p->d_shift, st));
  PTY_TRY(copy_d2d(O, p->d_tmpO, nobj * sizeof(float2), st));
  if (psi) {
    PTY_TRY(launch_roll(psi, p->d_psi_tmp, p->n, p->N0, p->N1, p->d_shift, st));
    PTY_TRY(copy_d2d(psi, p->d_psi_tmp, (size_t)p->n * npix * sizeof(float2), st));
  }
  return PTY_OK;
}

static int validate_run(pty_plan* p, const pty_buffers* b, const pty_options* o, int iters) {
  if (!p || !b || !o) return set_error(PTY_ERR_ARG, "null argument");
  if (o->method < 1 || o->method > 6) return set_error(PTY_ERR_ARG, "method must be 1..6");
  if (iters < 0) return set_error(PTY_ERR_ARG, "iters must be >= 0");
  if (!b->O || !b->P || !b->psi || !b->amp) return set_error(PTY_ERR_ARG, "missing O, P, psi or amp");
  if (o->method >= 4 && !b->background) return set_error(PTY_ERR_ARG, "methods 4-6 need a background buffer");
  if (o->Pmod_probe > 0 && !b->Pamp) return set_error(PTY_ERR_ARG, "Pmod_probe needs Pamp");
  if (o->OP_iters0 < 1 || o->OP_iters1 < 1) return set_error(PTY_ERR_ARG, "OP_iters must be >= 1");
  return PTY_OK;
}

// Identity of a whole-loop request: the kind, every buffer pointer, every
// option and the iteration count.  Equal keys launch identical work.
static std::string request_key(char kind, const pty_buffers* b, const pty_options* o, int iters) {
  std::string k(1, kind);
  k.append(reinterpret_cast<const char*>(b), sizeof(*b));
  k.append(reinterpret_cast<const char*>(o), sizeof(*o));
  k.append(reinterpret_cast<const char*>(&iters), sizeof(iters));
  return k;
}

// Run `body` on the plan's stream, joined to the caller's stream by events.
// With `graph`, the whole loop is captured once as a CUDA graph and kept in the
// plan; a later call with the same key replays it without re-capturing.
// `heat_valid` is the host-side heatmap state the body leaves behind.
template <class F>
static int run_on_stream(pty_plan* p, cudaStream_t user, bool graph, const std::string& key,
                         F body, bool& heat_valid) {
  PTY_CUDA(cudaEventRecord(p->ev_in, user));
  PTY_CUDA(cudaStreamWaitEvent(p->cap, p->ev_in, 0));
  int rc = PTY_OK;
  auto& slot = p->graphs[key[0] == 'D' ? 1 : 0];
  if (graph && slot.exec && slot.key == key) {
    cudaError_t e = cudaGraphLaunch(slot.exec, p->cap);
    if (e != cudaSuccess) rc = set_cuda_error(e, "graph replay");
    else count_launches(slot.kernels);
    heat_valid = slot.heat_valid != 0;
  } else if (graph) {
    PTY_CUDA(cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal));
    const long long before = launch_total();
    rc = body(p->cap);
    const long long nkern = launch_total() - before;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(p->cap, &g);
    if (rc == PTY_OK && e != cudaSuccess) rc = set_cuda_error(e, "cudaStreamEndCapture");
    if (rc == PTY_OK) {
      cudaGraphExec_t ge = nullptr;
      e = cudaGraphInstantiate(&ge, g, 0);
      if (e == cudaSuccess) e = cudaGraphLaunch(ge, p->cap);
      if (e != cudaSuccess) {
        rc = set_cuda_error(e, "graph launch");
        if (ge) cudaGraphExecDestroy(ge);
      } else {
        if (slot.exec) cudaGraphExecDestroy(slot.exec);
        slot.exec = ge;
        slot.key = key;
        slot.heat_valid = heat_valid ? 1 : 0;
        slot.kernels = nkern;
      }
    }
    if (g) cudaGraphDestroy(g);
  } else {
    rc = body(p->cap);
  }
  PTY_CUDA(cudaEventRecord(p->ev_out, p->cap));
  PTY_CUDA(cudaStreamWaitEvent(user, p->ev_out, 0));
  return rc;
}

static int update_mask(int method) {  // 1 = O, 2 = P, 3 = OP
  switch (method) {
    case 1: case 4: return 1;
    case 2: case 5: return 2;
    default: return 3;
  }
}

// ------------------------------------------------------------------ ERA
static int era_prepare(pty_plan* p, const pty_buffers* b, const pty_options* o, int iters) {
  PTY_TRY(validate_run(p, b, o, iters));
  const size_t npix = (size_t)p->N0 * p->N1;
  if (o->method >= 4 && !p->d_bgf) PTY_TRY(dalloc_t(p, &p->d_bgf, (size_t)p->n * npix));
  return PTY_OK;
}

// The ERA loop (era.py:13-332) on stream st.  heatP_valid ends as the state of
// the reference's P_heatmap (false where it would be None).
static int era_body(pty_plan* p, const pty_buffers* b, const pty_options* o, int iters,
                    bool& heatP_valid, cudaStream_t st) {
  const int upd = update_mask(o->method);
  const bool use_bg = o->method >= 4;
  const size_t nobj = (size_t)p->U * p->V, npix = (size_t)p->N0 * p->N1;
  const float alpha = (float)o->alpha;
  float2* O = (float2*)b->O;
  float2* P = (float2*)b->P;
  float2* psi = (float2*)b->psi;
  heatP_valid = false;
  bool heatO_valid = false;

    for (int i = 0; i < iters; ++i) {
      if (upd & 1) PTY_TRY(copy_d2d(p->d_bakO, O, nobj * sizeof(float2), st));
      if (upd & 2) PTY_TRY(copy_d2d(p->d_bakP, P, npix * sizeof(float2), st));
      // modulus projection on exits = P * O[R] (era.py:160 / 230, exits from era.py:196 / 272)
      FrameArgs a = base_args(p);
      a.O = O;
      a.P = P;
      a.psi = psi;
      a.amp = b->amp;
      a.mask = b->mask;
      a.alpha = alpha;
      a.err_part = p->d_err_part;
      if (use_bg) {
        a.bg_in = (i == 0) ? b->background : p->d_b0;
        a.bg_stride = (i == 0) ? (long long)npix : 0;
        a.bg_out = p->d_bgf;
        PTY_TRY(frame_op(p, OP_EXIT7, a, p->n, st));
      } else {
        PTY_TRY(frame_op(p, OP_EXIT1, a, p->n, st));
      }
      // consistency projection (era.py:163-189)
      if (upd == 1) {
        PTY_TRY(launch_psup_O(p->tl, p->n, p->N0, p->N1, p->U, p->V, p->d_R, psi, P, p->d_heatP, !heatP_valid, alpha, O, st));
        heatP_valid = true;
      } else if (upd == 2) {
        PTY_TRY(launch_psup_P(p->n, p->N0, p->N1, p->U, p->V, p->d_R, psi, O, p->d_part_num,
                              p->d_part_den, p->K, p->d_heatO, !heatO_valid, alpha, P, st));
        heatO_valid = true;
      } else if (i % o->OP_iters1 == 0) {
        for (int j = 0; j < o->OP_iters0; ++j) {
          PTY_TRY(launch_psup_O(p->tl, p->n, p->N0, p->N1, p->U, p->V, p->d_R, psi, P, p->d_heatP, true, alpha, O, st));
          PTY_TRY(launch_psup_P(p->n, p->N0, p->N1, p->U, p->V, p->d_R, psi, O, p->d_part_num,
                                p->d_part_den, p->K, p->d_heatO, true, alpha, P, st));
        }
        heatP_valid = heatO_valid = true;
        if (o->probe_centering) {
          PTY_TRY(centre(p, P, O, nullptr, st));
          heatP_valid = heatO_valid = false;
        }
      } else {
        PTY_TRY(launch_psup_O(p->tl, p->n, p->N0, p->N1, p->U, p->V, p->d_R, psi, P, p->d_heatP, !heatP_valid, alpha, O, st));
        heatP_valid = true;
      }
      if (i < o->Pmod_probe) PTY_TRY(pmod_probe(p, P, b->Pamp, b->mask, alpha, st));  // era.py:193-194
      if (use_bg) PTY_TRY(launch_frame_mean(p->n, (int)npix, p->d_bgf, p->d_mean_part, p->Km, p->d_b0, st));
      int ndn = 0;
      PTY_TRY(econ_partials(p, upd, p->d_bakO, O, p->d_bakP, P, st, &ndn));
      PTY_TRY(launch_finalize(p->d_err_part, p->n * p->eslots, p->d_dn_part, ndn, o->I_norm, b->eMod, b->eCon, i, st));
    }
    if (b->intensities) {  // era.py:295
      FrameArgs a = base_args(p);
      a.O = O;
      a.P = P;
      a.out_real = b->intensities;
      PTY_TRY(frame_op(p, OP_INTENS, a, p->n, st));
    }
    if (b->heatmap && heatP_valid) PTY_TRY(copy_d2d(b->heatmap, p->d_heatP, nobj * sizeof(double), st));
    if (use_bg && b->background_mean) {
      // after the loop the background is the frame mean (era.py:270, 311-314)
      const float* src = iters > 0 ? p->d_b0 : b->background;
      PTY_TRY(copy_d2d(b->background_mean, src, npix * sizeof(float), st));
    }
    return PTY_OK;
}

extern "C" int pty_era(pty_plan* p, const pty_buffers* b, const pty_options* o, int32_t iters,
                       int32_t* heatmap_valid, void* stream) {
  PTY_TRY(era_prepare(p, b, o, iters));
  bool heatP_valid = false;
  auto body = [&](cudaStream_t st) -> int { return era_body(p, b, o, iters, heatP_valid, st); };
  int rc = run_on_stream(p, (cudaStream_t)stream, o->use_graph != 0, request_key('E', b, o, iters),
                         body, heatP_valid);
  if (heatmap_valid) *heatmap_valid = heatP_valid ? 1 : 0;
  return rc;
}

// ------------------------------------------------------------------ DM
static int dm_prepare(pty_plan* p, const pty_buffers* b, const pty_options* o, int iters) {
  PTY_TRY(validate_run(p, b, o, iters));
  const size_t npix = (size_t)p->N0 * p->N1;
  if (o->probe_centering && update_mask(o->method) == 3 && !p->d_psi_tmp) {
    cudaError_t e = cudaMalloc(&p->d_psi_tmp, (size_t)p->n * npix * sizeof(float2));
    if (e != cudaSuccess) {
      cudaGetLastError();
      p->d_psi_tmp = nullptr;
      return set_error(PTY_ERR_NOMEM, "DM centring scratch allocation failed");
    }
  }
  return PTY_OK;
}

// The DM loop (dm.py:13-333) on stream st.
static int dm_body(pty_plan* p, const pty_buffers* b, const pty_options* o, int iters,
                   bool& heatP_valid, cudaStream_t st) {
  const int upd = update_mask(o->method);
  const bool use_bg = o->method >= 4;
  const size_t nobj = (size_t)p->U * p->V, npix = (size_t)p->N0 * p->N1;
  const float alpha = (float)o->alpha;
  float2* O = (float2*)b->O;
  float2* P = (float2*)b->P;
  float2* psi = (float2*)b->psi;
  float* bg = b->background;
  heatP_valid = false;
  bool heatO_valid = false;
  const int n = p->n, N0 = p->N0, N1 = p->N1, U = p->U, V = p->V;
  const int* R = p->d_R;

    // Iteration j's main projection (dm.py:56-85) equals iteration j-1's
    // metric projection (dm.py:104-134): both project the same exits from the
    // same O, P (the metric starts from copies), with the same branch.  That
    // holds for methods 1-3 only (methods 4-6 project pmod_7(exits) in the
    // main branch, dm.py:171), and needs the same OP branch in both
    // iterations and no Pmod_P after the metric projection (dm.py:136-137).
    // Probe centring rolls the metric's Os, Ps by the shift the main branch
    // then applies to the exits as well (dm.py:68-82, 118-127).
    auto foldable = [&](int j) -> bool {
      if (use_bg || j <= 0 || j >= iters) return false;
      if (j - 1 < o->Pmod_probe) return false;
      if (upd == 3 && ((j - 1) % o->OP_iters1 == 0) != (j % o->OP_iters1 == 0)) return false;
      return true;
    };
    bool main_done = false;
    // era.py:536: psi = P * O[R]; methods 4-6 form it inside their first Pmod_7 pass
    if (!use_bg || iters == 0) PTY_TRY(launch_make_exits(n, N0, N1, U, V, R, O, P, psi, st));
    if (upd & 1) PTY_TRY(copy_d2d(p->d_bakO, O, nobj * sizeof(float2), st));  // dm.py:35-38
    if (upd & 2) PTY_TRY(copy_d2d(p->d_bakP, P, npix * sizeof(float2), st));
    for (int i = 0; i < iters; ++i) {
      FrameArgs a = base_args(p);
      a.amp = b->amp;
      a.mask = b->mask;
      a.alpha = alpha;
      if (use_bg) {  // dm.py:171
        a.psi = psi;
        a.bg_in = bg;
        a.bg_stride = (long long)npix;
        a.bg_out = bg;
        if (i == 0) {  // exits straight from P * O[R] (era.py:536), same values
          a.O = O;
          a.P = P;
          PTY_TRY(frame_op(p, OP_EXIT7, a, n, st));
        } else {
          PTY_TRY(frame_op(p, OP_PSI7, a, n, st));
        }
      }
      // main consistency projection (dm.py:56-85)
      if (main_done) {
        // O and P (and the heatmaps) already hold it: the previous iteration's
        // metric projection was computed into them (see `foldable`).  Only
        // the centring's roll of the exit waves (dm.py:81-82) remains.
        if (upd == 3 && i % o->OP_iters1 == 0) {
          heatP_valid = heatO_valid = true;
          if (o->probe_centering) {
            PTY_TRY(launch_roll(psi, p->d_psi_tmp, n, N0, N1, p->d_shift, st));
            PTY_TRY(copy_d2d(psi, p->d_psi_tmp, (size_t)n * npix * sizeof(float2), st));
            heatP_valid = heatO_valid = false;
          }
        }
      } else if (upd == 1) {
        PTY_TRY(launch_psup_O(p->tl, n, N0, N1, U, V, R, psi, P, p->d_heatP, !heatP_valid, alpha, O, st));
        heatP_valid = true;
      } else if (upd == 2) {
        PTY_TRY(launch_psup_P(n, N0, N1, U, V, R, psi, O, p->d_part_num, p->d_part_den, p->K,
                              p->d_heatO, !heatO_valid, alpha, P, st));
        heatO_valid = true;
      } else if (i % o->OP_iters1 == 0) {
        for (int j = 0; j < o->OP_iters0; ++j) {
          PTY_TRY(launch_psup_O(p->tl, n, N0, N1, U, V, R, psi, P, p->d_heatP, true, alpha, O, st));
          PTY_TRY(launch_psup_P(n, N0, N1, U, V, R, psi, O, p->d_part_num, p->d_part_den, p->K,
                                p->d_heatO, true, alpha, P, st));
        }
        heatP_valid = heatO_valid = true;
        if (o->probe_centering) {
          PTY_TRY(centre(p, P, O, psi, st));
          heatP_valid = heatO_valid = false;
        }
      } else {
        PTY_TRY(launch_psup_O(p->tl, n, N0, N1, U, V, R, psi, P, p->d_heatP, !heatP_valid, alpha, O, st));
        heatP_valid = true;
      }
      if (i < o->Pmod_probe) PTY_TRY(pmod_probe(p, P, b->Pamp, b->mask, alpha, st));  // dm.py:88-89
      // difference-map update (dm.py:91-97 / 208-224)
      if (use_bg) PTY_TRY(launch_frame_mean(n, (int)npix, bg, p->d_mean_part, p->Km, p->d_b0, st));
      {
        FrameArgs d = base_args(p);
        d.O = O;
        d.P = P;
        d.psi = psi;
        d.amp = b->amp;
        d.mask = b->mask;
        d.alpha = alpha;
        if (use_bg) {
          d.bg_out = bg;
          d.b0 = p->d_b0;
          PTY_TRY(frame_op(p, OP_DM7, d, n, st));
        } else {
          PTY_TRY(frame_op(p, OP_DM1, d, n, st));
        }
      }
      // metric projection (dm.py:104-137 / 231-271).  When the next
      // iteration's main projection equals it, it is computed straight into
      // O and P (the main branch's values are not needed again) and the next
      // iteration skips its own; otherwise into the scratch Os, Ps.
      const bool direct = foldable(i + 1);
      float2* Os = direct ? O : p->d_Os;
      float2* Ps = direct ? P : p->d_Ps;
      double* hP2 = direct ? p->d_heatP : p->d_heatP2;
      double* hO2 = direct ? p->d_heatO : p->d_heatO2;
      if (!direct) {
        PTY_TRY(copy_d2d(Os, O, nobj * sizeof(float2), st));
        PTY_TRY(copy_d2d(Ps, P, npix * sizeof(float2), st));
      }
      if (upd == 1) {
        PTY_TRY(launch_psup_O(p->tl, n, N0, N1, U, V, R, psi, Ps, p->d_heatP, !heatP_valid, alpha, Os, st));
        heatP_valid = true;
      } else if (upd == 2) {
        PTY_TRY(launch_psup_P(n, N0, N1, U, V, R, psi, Os, p->d_part_num, p->d_part_den, p->K,
                              p->d_heatO, !heatO_valid, alpha, Ps, st));
        heatO_valid = true;
      } else if (i % o->OP_iters1 == 0) {
        for (int j = 0; j < o->OP_iters0; ++j) {
          PTY_TRY(launch_psup_O(p->tl, n, N0, N1, U, V, R, psi, Ps, hP2, true, alpha, Os, st));
          PTY_TRY(launch_psup_P(n, N0, N1, U, V, R, psi, Os, p->d_part_num, p->d_part_den, p->K,
                                hO2, true, alpha, Ps, st));
        }
        if (o->probe_centering) PTY_TRY(centre(p, Ps, Os, nullptr, st));
      } else {
        PTY_TRY(launch_psup_O(p->tl, n, N0, N1, U, V, R, psi, P, p->d_heatP, !heatP_valid, alpha, Os, st));
        heatP_valid = true;
      }
      if (i < o->Pmod_probe) PTY_TRY(pmod_probe(p, Ps, b->Pamp, b->mask, alpha, st));
      if (use_bg) PTY_TRY(launch_frame_mean(n, (int)npix, bg, p->d_mean_part, p->Km, p->d_b0, st));
      {
        FrameArgs m = base_args(p);
        m.O = Os;
        m.P = Ps;
        m.amp = b->amp;
        m.mask = b->mask;
        m.bg_in = use_bg ? p->d_b0 : nullptr;
        m.bg_stride = 0;
        m.err_part = p->d_err_part;
        PTY_TRY(frame_op(p, OP_MERR, m, n, st));
      }
      int ndn = 0;
      PTY_TRY(econ_partials(p, upd, p->d_bakO, Os, p->d_bakP, Ps, st, &ndn));
      PTY_TRY(launch_finalize(p->d_err_part, n * p->eslots, p->d_dn_part, ndn, o->I_norm, b->eMod, b->eCon, i, st));
      if (upd & 1) PTY_TRY(copy_d2d(p->d_bakO, Os, nobj * sizeof(float2), st));
      if (upd & 2) PTY_TRY(copy_d2d(p->d_bakP, Ps, npix * sizeof(float2), st));
      main_done = direct;
    }
    if (b->intensities && iters > 0) {  // dm.py:298-299
      FrameArgs a = base_args(p);
      a.O = p->d_Os;
      a.P = p->d_Ps;
      a.out_real = b->intensities;
      PTY_TRY(frame_op(p, OP_INTENS, a, n, st));
    }
    if (b->heatmap && heatP_valid) PTY_TRY(copy_d2d(b->heatmap, p->d_heatP, nobj * sizeof(double), st));
    if (use_bg && b->background_mean && iters > 0)
      PTY_TRY(copy_d2d(b->background_mean, p->d_b0, npix * sizeof(float), st));
    return PTY_OK;
}

extern "C" int pty_dm(pty_plan* p, const pty_buffers* b, const pty_options* o, int32_t iters,
                      int32_t* heatmap_valid, void* stream) {
  PTY_TRY(dm_prepare(p, b, o, iters));
  bool heatP_valid = false;
  auto body = [&](cudaStream_t st) -> int { return dm_body(p, b, o, iters, heatP_valid, st); };
  int rc = run_on_stream(p, (cudaStream_t)stream, o->use_graph != 0, request_key('D', b, o, iters),
                         body, heatP_valid);
  if (heatmap_valid) *heatmap_valid = heatP_valid ? 1 : 0;
  return rc;
}

// ------------------------------------------------------------------ batches
// Independent reconstructions in one CUDA graph: each plan's loop is captured
// on that plan's own stream, forked from and joined to the first plan's
// stream, so the graph holds one branch per reconstruction and the GPU runs
// the branches concurrently.
extern "C" int pty_run_batch(int32_t kind, pty_plan* const* plans, const pty_buffers* bufs,
                             const pty_options* opts, int32_t nrec, int32_t iters,
                             int32_t* heatmap_valid, void* stream) {
  if (!plans || !bufs || !opts || nrec < 1) return set_error(PTY_ERR_ARG, "empty batch");
  if (kind != 0 && kind != 1) return set_error(PTY_ERR_ARG, "kind must be 0 (ERA) or 1 (DM)");
  for (int r = 0; r < nrec; ++r) {
    for (int q = 0; q < r; ++q)
      if (plans[q] == plans[r]) return set_error(PTY_ERR_ARG, "a plan appears twice in the batch");
    PTY_TRY(kind == 0 ? era_prepare(plans[r], &bufs[r], &opts[r], iters)
                      : dm_prepare(plans[r], &bufs[r], &opts[r], iters));
  }
  pty_plan* p0 = plans[0];
  cudaStream_t master = p0->cap, user = (cudaStream_t)stream;
  // a batch with the same plans (by serial, so a freed and re-created plan
  // never matches), buffers, options and iteration count replays its graph
  std::string key;
  for (int r = 0; r < nrec; ++r) {
    key.append(reinterpret_cast<const char*>(&plans[r]->serial), sizeof(long long));
    key += request_key(kind == 0 ? 'E' : 'D', &bufs[r], &opts[r], iters);
  }
  std::vector<bool> hv(nrec, false);
  PTY_CUDA(cudaEventRecord(p0->ev_in, user));
  PTY_CUDA(cudaStreamWaitEvent(master, p0->ev_in, 0));
  int rc = PTY_OK;
  if (p0->batch_exec && p0->batch_key == key) {
    cudaError_t e = cudaGraphLaunch(p0->batch_exec, master);
    if (e != cudaSuccess) rc = set_cuda_error(e, "batch graph replay");
    else count_launches(p0->batch_kernels);
    for (int r = 0; r < nrec; ++r) hv[r] = p0->batch_heat[r] != 0;
  } else {
    cudaEvent_t fork = nullptr;
    PTY_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    cudaGraph_t g = nullptr;
    const long long before = launch_total();
    cudaError_t e = cudaStreamBeginCapture(master, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) rc = set_cuda_error(e, "batch capture");
    const bool capturing = (rc == PTY_OK);
    if (rc == PTY_OK) {
      e = cudaEventRecord(fork, master);
      if (e != cudaSuccess) rc = set_cuda_error(e, "batch fork");
    }
    for (int r = 0; rc == PTY_OK && r < nrec; ++r) {
      cudaStream_t st = (r == 0) ? master : plans[r]->cap;
      if (r > 0 && (e = cudaStreamWaitEvent(st, fork, 0)) != cudaSuccess) {
        rc = set_cuda_error(e, "batch fork wait");
        break;
      }
      bool h = false;
      rc = kind == 0 ? era_body(plans[r], &bufs[r], &opts[r], iters, h, st)
                     : dm_body(plans[r], &bufs[r], &opts[r], iters, h, st);
      hv[r] = h;
      if (rc == PTY_OK && r > 0) {
        e = cudaEventRecord(plans[r]->ev_out, st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(master, plans[r]->ev_out, 0);
        if (e != cudaSuccess) rc = set_cuda_error(e, "batch join");
      }
    }
    const long long nkern = launch_total() - before;
    if (capturing) {
      e = cudaStreamEndCapture(master, &g);
      if (rc == PTY_OK && e != cudaSuccess) rc = set_cuda_error(e, "batch end capture");
    }
    if (rc == PTY_OK) {
      cudaGraphExec_t ge = nullptr;
      e = cudaGraphInstantiate(&ge, g, 0);
      if (e == cudaSuccess) e = cudaGraphLaunch(ge, master);
      if (e != cudaSuccess) {
        rc = set_cuda_error(e, "batch graph launch");
        if (ge) cudaGraphExecDestroy(ge);
      } else {
        // kept until the plan is destroyed or launches another batch
        if (p0->batch_exec) cudaGraphExecDestroy(p0->batch_exec);
        p0->batch_exec = ge;
        p0->batch_key = key;
        p0->batch_heat.assign(hv.begin(), hv.end());
        p0->batch_kernels = nkern;
      }
    }
    if (g) cudaGraphDestroy(g);
    cudaEventDestroy(fork);
  }
  cudaEventRecord(p0->ev_out, master);
  cudaStreamWaitEvent(user, p0->ev_out, 0);
  if (heatmap_valid)
    for (int r = 0; r < nrec; ++r) heatmap_valid[r] = hv[r] ? 1 : 0;
  return rc;
}

// ------------------------------------------------------------------ single operators
static __global__ void sum_kernel(const double* x, int n, double* out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += x[i];
  s = block_sum_d(s, red);
  if (threadIdx.x == 0) *out = s;
}

static int sum_partials(pty_plan* p, double* out, cudaStream_t st) {
  sum_kernel<<<1, 256, 0, st>>>(p->d_err_part, p->n * p->eslots, out);
  return check_launch("sum_kernel");
}

extern "C" int pty_make_exits(pty_plan* p, const void* O, const void* P, void* psi, void* stream) {
  if (!p || !O || !P || !psi) return set_error(PTY_ERR_ARG, "null argument");
  return launch_make_exits(p->n, p->N0, p->N1, p->U, p->V, p->d_R, (const float2*)O,
                           (const float2*)P, (float2*)psi, (cudaStream_t)stream);
}

extern "C" int pty_pmod_1(pty_plan* p, const float* amp, void* psi, const uint8_t* mask,
                          double alpha, double* eMod_dev, void* stream) {
  if (!p || !amp || !psi) return set_error(PTY_ERR_ARG, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  FrameArgs a = base_args(p);
  a.psi = (float2*)psi;
  a.amp = amp;
  a.mask = mask;
  a.alpha = (float)alpha;
  a.err_part = eMod_dev ? p->d_err_part : nullptr;
  PTY_TRY(frame_op(p, OP_PSI1, a, p->n, st));
  if (eMod_dev) PTY_TRY(sum_partials(p, eMod_dev, st));
  return PTY_OK;
}

extern "C" int pty_pmod_7(pty_plan* p, const float* amp, float* background, void* psi,
                          const uint8_t* mask, double alpha, double* eMod_dev, void* stream) {
  if (!p || !amp || !psi || !background) return set_error(PTY_ERR_ARG, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  FrameArgs a = base_args(p);
  a.psi = (float2*)psi;
  a.amp = amp;
  a.mask = mask;
  a.alpha = (float)alpha;
  a.bg_in = background;
  a.bg_stride = (long long)p->N0 * p->N1;
  a.bg_out = background;
  a.err_part = eMod_dev ? p->d_err_part : nullptr;
  PTY_TRY(frame_op(p, OP_PSI7, a, p->n, st));
  if (eMod_dev) PTY_TRY(sum_partials(p, eMod_dev, st));
  return PTY_OK;
}

extern "C" int pty_Pmod_P(pty_plan* p, const float* Pamp, void* P, const uint8_t* mask,
                          double alpha, void* stream) {
  if (!p || !Pamp || !P) return set_error(PTY_ERR_ARG, "null argument");
  return pmod_probe(p, (float2*)P, Pamp, mask, (float)alpha, (cudaStream_t)stream);
}

extern "C" int pty_psup_O(pty_plan* p, const void* psi, const void* P, double* heat,
                          int32_t recompute, double alpha, void* O_out, void* stream) {
  if (!p || !psi || !P || !heat || !O_out) return set_error(PTY_ERR_ARG, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  return launch_psup_O(p->tl, p->n, p->N0, p->N1, p->U, p->V, p->d_R, (const float2*)psi,
                       (const float2*)P, heat, recompute != 0, (float)alpha, (float2*)O_out, st);
}

extern "C" int pty_psup_P(pty_plan* p, const void* psi, const void* O, double* heat,
                          int32_t recompute, double alpha, void* P_out, void* stream) {
  if (!p || !psi || !O || !heat || !P_out) return set_error(PTY_ERR_ARG, "null argument");
  return launch_psup_P(p->n, p->N0, p->N1, p->U, p->V, p->d_R, (const float2*)psi,
                       (const float2*)O, p->d_part_num, p->d_part_den, p->K, heat, recompute != 0,
                       (float)alpha, (float2*)P_out, (cudaStream_t)stream);
}

extern "C" int pty_make_P_heatmap(pty_plan* p, const void* P, double* heat, void* stream) {
  if (!p || !P || !heat) return set_error(PTY_ERR_ARG, "null argument");
  return launch_heat_P(p->tl, p->n, p->N0, p->N1, p->U, p->V, p->d_R, (const float2*)P, heat,
                       (cudaStream_t)stream);
}

extern "C" int pty_make_O_heatmap(pty_plan* p, const void* O, double* heat, void* stream) {
  if (!p || !O || !heat) return set_error(PTY_ERR_ARG, "null argument");
  return launch_heat_O(p->n, p->N0, p->N1, p->U, p->V, p->d_R, (const float2*)O, p->d_part_den,
                       p->K, heat, (cudaStream_t)stream);
}

extern "C" int pty_model_error_1(pty_plan* p, const float* amp, const void* psi,
                                 const uint8_t* mask, const float* background,
                                 int32_t background_per_frame, double* err_dev, void* stream) {
  if (!p || !amp || !psi || !err_dev) return set_error(PTY_ERR_ARG, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  FrameArgs a = base_args(p);
  a.psi = (float2*)psi;
  a.amp = amp;
  a.mask = mask;
  a.bg_in = background;
  a.bg_stride = background_per_frame ? (long long)p->N0 * p->N1 : 0;
  a.err_part = p->d_err_part;
  PTY_TRY(frame_op(p, OP_MERR_PSI, a, p->n, st));
  return sum_partials(p, err_dev, st);
}

extern "C" int pty_intensities(pty_plan* p, const void* O, const void* P, float* I_out,
                               void* stream) {
  if (!p || !O || !P || !I_out) return set_error(PTY_ERR_ARG, "null argument");
  FrameArgs a = base_args(p);
  a.O = (const float2*)O;
  a.P = (const float2*)P;
  a.out_real = I_out;
  return frame_op(p, OP_INTENS, a, p->n, (cudaStream_t)stream);
}

extern "C" int pty_back_project(pty_plan* p, const float* amp, const uint8_t* mask,
                                const void* phase, void* exits, void* stream) {
  if (!p || !amp || !phase || !exits) return set_error(PTY_ERR_ARG, "null argument");
  if ((p->N0 & 1) || (p->N1 & 1)) return set_error(PTY_ERR_SHAPE, "back projection needs even frame sizes");
  FrameArgs a = base_args(p);
  a.amp = amp;
  a.mask = mask;
  a.P = (const float2*)phase;
  a.psi = (float2*)exits;
  return frame_op(p, OP_BP, a, p->n, (cudaStream_t)stream);
}

extern "C" int pty_background_mean(pty_plan* p, const float* background, float* mean_out,
                                   void* stream) {
  if (!p || !background || !mean_out) return set_error(PTY_ERR_ARG, "null argument");
  return launch_frame_mean(p->n, p->N0 * p->N1, background, p->d_mean_part, p->Km, mean_out,
                           (cudaStream_t)stream);
}

static __global__ void amp_kernel(const void* I, int is_double, int n, int N0, int N1, float* amp) {
  const long long tot = (long long)n * N0 * N1;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot;
       i += (long long)gridDim.x * blockDim.x) {
    const long long f = i / ((long long)N0 * N1);
    const int k0 = (int)((i / N1) % N0), k1 = (int)(i % N1);
    const long long src = f * N0 * N1 + (long long)((k0 + N0 / 2) % N0) * N1 + (k1 + N1 / 2) % N1;
    if (is_double) amp[i] = (float)sqrt(((const double*)I)[src]);
    else amp[i] = sqrtf(((const float*)I)[src]);
  }
}

// amp as above, plus per-block partial sums of mask * I (era.py:495, I_norm)
// in double; the mask is in unshifted order, like amp.
static __global__ void amp_norm_kernel(const void* I, int is_double, int n, int N0, int N1,
                                       const uint8_t* mask, float* amp, double* part) {
  __shared__ double red[32];
  const long long tot = (long long)n * N0 * N1;
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot;
       i += (long long)gridDim.x * blockDim.x) {
    const long long f = i / ((long long)N0 * N1);
    const int k0 = (int)((i / N1) % N0), k1 = (int)(i % N1);
    const long long src = f * N0 * N1 + (long long)((k0 + N0 / 2) % N0) * N1 + (k1 + N1 / 2) % N1;
    const double m = mask ? (double)mask[(long long)k0 * N1 + k1] : 1.0;
    if (is_double) {
      const double v = ((const double*)I)[src];
      amp[i] = (float)sqrt(v);
      acc += m * v;
    } else {
      const float v = ((const float*)I)[src];
      amp[i] = sqrtf(v);
      acc += m * (double)v;
    }
  }
  acc = block_sum_d(acc, red);
  if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

static __global__ void sum_parts_kernel(const double* part, int nparts, double* out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += part[i];
  s = block_sum_d(s, red);
  if (threadIdx.x == 0) *out = s;
}

extern "C" int pty_amp_and_norm(pty_plan* p, const void* I, int32_t is_double, const uint8_t* mask,
                                float* amp, double* norm, void* stream) {
  if (!p || !I || !amp || !norm) return set_error(PTY_ERR_ARG, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  constexpr int kBlocks = 152 * 8;
  double* part = nullptr;
  PTY_CUDA(cudaMallocAsync(&part, kBlocks * sizeof(double), st));
  amp_norm_kernel<<<kBlocks, 256, 0, st>>>(I, is_double, p->n, p->N0, p->N1, mask, amp, part);
  int rc = check_launch("amp_norm_kernel");
  if (rc == PTY_OK) {
    sum_parts_kernel<<<1, 256, 0, st>>>(part, kBlocks, norm);
    rc = check_launch("sum_parts_kernel");
  }
  cudaFreeAsync(part, st);
  return rc;
}

extern "C" int pty_amp_from_intensity(pty_plan* p, const void* I, int32_t is_double, float* amp,
                                      void* stream) {
  if (!p || !I || !amp) return set_error(PTY_ERR_ARG, "null argument");
  const long long tot = (long long)p->n * p->N0 * p->N1;
  int blocks = (int)((tot + 255) / 256);
  if (blocks > 152 * 32) blocks = 152 * 32;
  amp_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(I, is_double, p->n, p->N0, p->N1, amp);
  return check_launch("amp_kernel");
}

