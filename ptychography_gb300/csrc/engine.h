// Internal declarations shared by the CUDA translation units of libptycho_gb300.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include "pty_common.cuh"

namespace pty {

// operations of the fused frame kernel
enum FrameOp {
  OP_EXIT1 = 0,  // P*O[R] -> FFT -> Pmod_1 (+eMod) -> IFFT -> psi          (ERA m1-3)
  OP_EXIT7 = 1,  // P*O[R] -> FFT -> Pmod_7 (+eMod, bg*f out) -> IFFT -> psi (ERA m4-6)
  OP_PSI1 = 2,   // psi -> FFT -> Pmod_1 -> IFFT -> psi                     (pmod_1, Pmod_P)
  OP_PSI7 = 3,   // psi -> FFT -> Pmod_7 (bg in/out) -> IFFT -> psi          (pmod_7, DM m4-6)
  OP_DM1 = 4,    // psi <- psi - ex0 + Pmod_1(2 ex0 - psi)                    (DM m1-3)
  OP_DM7 = 5,    // same with the background recursion                        (DM m4-6)
  OP_MERR = 6,   // P*O[R] -> FFT -> model error (no alpha)                    (model_error_1)
  OP_INTENS = 7, // P*O[R] -> FFT -> fftshift |F|^2                            (info['I'])
  OP_MERR_PSI = 8, // psi -> FFT -> model error                                (model_error_1)
  OP_BP = 9,     // mask * sqrt(I) * exp(i arg FFT(P)) -> IFFT -> psi           (Back_projection)
};

struct FrameArgs {
  int U, V;                  // object shape
  const int* R;              // [n][2] scan offsets (<= 0), int32
  const float2* O;           // [U][V]
  const float2* P;           // [N0][N1]
  float2* psi;               // [n][N0][N1] exit waves, in/out
  const float* amp;          // [n][N0][N1] sqrt(I), unshifted order
  long long amp_stride;      // elements between frames of amp (0: shared)
  const uint8_t* mask;       // [N0][N1] 1 = valid, or nullptr
  const float* bg_in;        // background read by Pmod_7
  long long bg_stride;       // 0: shared pattern, N0*N1: per frame
  float* bg_out;             // [n][N0][N1] per-frame background written (or DM state)
  const float* b0;           // [N0][N1] mean background (DM m4-6, model error)
  float* out_real;           // [n][N0][N1] intensities (OP_INTENS)
  double* err_part;          // [n][err_stride] per-frame error partials, or nullptr
  int err_stride;            // partial slots per frame (>= CTAs per frame; the rest zeroed)
  float alpha;
  int N0h, N1h;              // N0 / 2, N1 / 2 (back-projection index roll)
  const float2* tw0;         // twiddles of the column transform (length N0)
  const float2* tw1;         // twiddles of the row transform (length N1)
  const float2* twf;         // W_N1^e, e < N1 (three-stage line transforms)
  float2* stage;             // [stage_frames][N0][N1] frame scratch of the staged tiles
  int stage_frames;          // frames the scratch holds (launches run in groups of it)
  uint8_t* mask_blk;         // [N0 * N1] mask in column-block order (staged tiles)
  int* timeout;              // set when a bounded wait of a kernel runs out
};

// Frame tiles: how many CTAs transform one frame.  Tile 1 is the single-CTA
// kernel (frame_kernels.cu), tile C > 1 the C-CTA cluster kernel
// (cluster_frame.cuh).  frame_tiles.cu lists the tiles built per shape and
// picks one per shape and device (autotuned, or forced by the caller).
// Op families tuned separately: the background forms (Pmod_7: EXIT7, PSI7,
// DM7) move 28 N^2 bytes per frame and hold more registers than the rest.
enum FrameFamily { FAM_PLAIN = 0, FAM_BG = 1 };
inline int frame_family(int op) {
  return (op == OP_EXIT7 || op == OP_PSI7 || op == OP_DM7) ? FAM_BG : FAM_PLAIN;
}
// Tile ids: C = C CTAs per frame with the two-stage line transforms;
// 100 + C = C CTAs with three-stage transforms (32 threads per line);
// 200 + C = staged: row, column and row launches through a frame scratch, C
// column CTAs per frame.  tile_ctas = the error-partial slots a frame needs.
inline int tile_ctas(int tile) { return tile % 100; }
inline bool tile_staged(int tile) { return tile >= 200; }
// frames of scratch a staged tile works through at a time
int staged_group_frames(int N0, int N1);
bool frame_shape_supported(int N0, int N1);
int frame_tile_candidates(int N0, int N1, int* tiles, int cap);   // returns the count
int max_frame_tile(int N0, int N1);
// nframes: the plan's frame count (0: a large launch); prepares the kernels too
int choose_frame_tile(int N0, int N1, int family, int nframes, int* tile);
int launch_frame_op(int op, int N0, int N1, int tile, const FrameArgs& a, int nframes,
                    cudaStream_t st);
void make_twiddles(int L, float2* out);   // host table tw[k1 * A + t], length L
void make_full_twiddles(int L, float2* out);   // host table W_L^e, e < L

int prepare_single_cta(int N0, int N1);
int launch_single_cta_op(int op, int N0, int N1, const FrameArgs& a, int nframes, cudaStream_t st);
#define PTY_DECLARE_CLUSTER_TILE(N, C)                                                    \
  int prepare_cluster_##N##x##C();                                                        \
  int launch_cluster_##N##x##C(int op, const FrameArgs& a, int nframes, cudaStream_t st);
PTY_DECLARE_CLUSTER_TILE(128, 2)
PTY_DECLARE_CLUSTER_TILE(192, 2)
PTY_DECLARE_CLUSTER_TILE(256, 4)
PTY_DECLARE_CLUSTER_TILE(256, 8)
int prepare_cluster_256x8l();
int launch_cluster_256x8l(int op, const FrameArgs& a, int nframes, cudaStream_t st);
PTY_DECLARE_CLUSTER_TILE(512, 16)
int prepare_cluster_512x16l();
int launch_cluster_512x16l(int op, const FrameArgs& a, int nframes, cudaStream_t st);
int prepare_staged_512();
int launch_staged_512(int op, const FrameArgs& a, int nframes, cudaStream_t st);
#undef PTY_DECLARE_CLUSTER_TILE

// error reporting (engine.cu)
int set_error(int code, const char* msg);
int set_cuda_error(cudaError_t e, const char* where);
// return early with the status of a failing call
#define PTY_TRY(x)                   \
  do {                               \
    int _rc = (x);                   \
    if (_rc != PTY_OK) return _rc;   \
  } while (0)
#define PTY_CUDA(x)                                          \
  do {                                                       \
    cudaError_t _e = (x);                                    \
    if (_e != cudaSuccess) return pty::set_cuda_error(_e, #x); \
  } while (0)
int check_launch(const char* where);  // also counts the launch
// the device's timeout flag (allocated on first use; see pty_timeout_status)
int device_timeout_flag(int** out);
// cuTensorMapEncodeTiled from the driver (TMA tensor maps)
int tensor_map_encoder(PFN_cuTensorMapEncodeTiled_v12000* out);
void count_launches(long long k);
long long launch_total();

// ------------------------------------------------------------ overlap kernels
// object / probe gather tiles: kGatherTileRows x kGatherTileCols pixels, one
// block of 256 threads (two pixels each) per tile.  (8 x 64 tiles, with wider
// contiguous row segments, measured slower: more frames overlap a tile only
// partially.)
constexpr int kGatherTileRows = 16;
constexpr int kGatherTileCols = 32;
struct TileLists {
  int TU, TV, ntu, ntv;      // object tiles
  const int* ptr;            // [ntu*ntv + 1]
  const int* frames;         // concatenated frame indices, ascending per tile
};

// O = sum conj(P) psi / (heat + alpha)   (era.py:336-369); heat in double
// (compute_heat: heat is recomputed from P in the same pass and written out)
int launch_psup_O(const TileLists& tl, int n, int N0, int N1, int U, int V, const int* R,
                  const float2* psi, const float2* P, double* heat, bool compute_heat, float alpha,
                  float2* O, cudaStream_t st);
// heat = sum |P|^2 over windows (era.py:402-410)
int launch_heat_P(const TileLists& tl, int n, int N0, int N1, int U, int V, const int* R,
                  const float2* P, double* heat, cudaStream_t st);
// P = sum conj(O_i) psi_i / (sum |O_i|^2 + alpha) (era.py:371-400, 412-417)
// blocks per frame chunk of the probe gather (sets the plan's chunk count)
int psup_P_tiles(int N0, int N1);
int launch_psup_P(int n, int N0, int N1, int U, int V, const int* R, const float2* psi,
                  const float2* O, float2* part_num, float2* part_den, int K, double* heatO,
                  bool recompute_heat, float alpha, float2* P, cudaStream_t st);
// mean over frames of a per-frame real pattern (era.py:265-270)
int launch_frame_mean(int n, int npix, const float* x, float2* part, int K, float* mean,
                      cudaStream_t st);
// partial sums of |a-b|^2 and |b|^2 (eCon, era.py:206-208)
int launch_diffnorm(const float2* a, const float2* b, long long count, double* part, int nblocks,
                    cudaStream_t st);
// final per-iteration metrics
int launch_finalize(const double* err_part, int n, const double* dn_part, int ndn, double I_norm,
                    double* hist_emod, double* hist_econ, int it, cudaStream_t st);
// probe centring (era.py:172-186)
int launch_probe_shift(const float2* P, int N0, int N1, int* shift, cudaStream_t st);
int launch_roll(const float2* src, float2* dst, int nimg, int H, int W, const int* shift,
                cudaStream_t st);
int launch_make_exits(int n, int N0, int N1, int U, int V, const int* R, const float2* O,
                      const float2* P, float2* psi, cudaStream_t st);
int launch_heat_O(int n, int N0, int N1, int U, int V, const int* R, const float2* O,
                  float2* part, int K, double* heatO, cudaStream_t st);

}  // namespace pty
