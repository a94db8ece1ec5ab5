/*
 * ptycho_gb300.h -- C ABI of the GB300 ptychography engine (libptycho_gb300.so).
 *
 * The reference (andyofmelbourne/Ptychography) is a Python/NumPy package with
 * no native interface; each entry point below replaces the reference function
 * it cites (file:line within that project), and takes plain device pointers,
 * sizes and a cudaStream_t passed as void*.  The Python drop-in
 * (ptychography_gb300.ERA / DM) binds these through ctypes.
 *
 * Conventions
 *   - complex arrays are interleaved complex64 (NumPy/torch complex64 layout);
 *   - detector-plane arrays (amp, mask, background, Pamp) are in unshifted FFT
 *     order, i.e. already ifftshift-ed as the reference's preamble does
 *     (ptychography/era.py:497-499, 543);
 *   - scan offsets R are int64 [n][2], every entry <= 0 (the preamble's shift,
 *     era.py:504-505), and each probe window must lie inside the object;
 *   - all buffers belong to the caller; the library never frees them.  A plan
 *     owns its own device scratch (tile lists, partial sums);
 *   - every call is stream-ordered; none synchronises the host;
 *   - return value: PTY_OK (0) or an error code; pty_last_error() describes
 *     the most recent error on the calling thread.
 * Calls on one plan are not thread-safe; distinct plans are independent.
 */
#ifndef PTYCHO_GB300_H
#define PTYCHO_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PTY_OK 0
#define PTY_ERR_ARG 1         /* null pointer, bad method or option */
#define PTY_ERR_SHAPE 2       /* frame shape has no kernel */
#define PTY_ERR_RANGE 3       /* a scan window falls outside the object */
#define PTY_ERR_CUDA 4        /* a CUDA runtime call failed */
#define PTY_ERR_NOMEM 5       /* device scratch allocation failed */
#define PTY_ERR_UNSUPPORTED 6 /* valid request the engine does not implement */

typedef struct pty_plan pty_plan;

/* n frames of N0 x N1 detector pixels; object U x V. */
typedef struct {
  int32_t n_frames, N0, N1, U, V;
} pty_geometry;

/* Device buffers of one reconstruction (all device pointers). */
typedef struct {
  void* O;                  /* complex64 [U][V] object, in/out */
  void* P;                  /* complex64 [N0][N1] probe, in/out */
  void* psi;                /* complex64 [n][N0][N1] exit waves: DM state, ERA scratch */
  const float* amp;         /* float32 [n][N0][N1] sqrt(I) */
  const uint8_t* mask;      /* uint8 [N0][N1], 1 = valid pixel; NULL = all valid */
  float* background;        /* float32 [n][N0][N1] sqrt-background state (methods 4-6) */
  const float* Pamp;        /* float32 [N0][N1] |FFT(P0)| for Pmod_probe; NULL if unused */
  float* background_mean;   /* float32 [N0][N1] out: final frame-mean sqrt-background */
  double* heatmap;          /* float64 [U][V] out: P_heatmap, or NULL */
  float* intensities;       /* float32 [n][N0][N1] out: fftshift |FFT psi|^2, or NULL */
  double* eMod;             /* float64 [iters] out: modulus error history */
  double* eCon;             /* float64 [iters] out: convergence error history */
} pty_buffers;

typedef struct {
  int32_t method;           /* 1..6, ptychography/era.py:61-78 */
  int32_t OP_iters0;        /* OP rounds per update, era.py:49-55 */
  int32_t OP_iters1;        /* update the probe every OP_iters1 iterations */
  int64_t Pmod_probe;       /* apply Pmod_P while iteration < Pmod_probe */
  int32_t probe_centering;  /* era.py:171-186 */
  int32_t use_graph;        /* capture the whole loop in one CUDA graph */
  double alpha;             /* regulariser, era.py:90-91 */
  double I_norm;            /* sum(mask * I), era.py:495 */
} pty_options;

/* Plan for one scan geometry: uploads R, builds the per-tile frame lists of
 * the overlap gathers and the FFT twiddles.  Replaces the set-up half of
 * preamble(), ptychography/era.py:435-548 (R must already be shifted). */
int pty_plan_create(const pty_geometry* geom, const int64_t* R_host, pty_plan** plan_out);
int pty_plan_destroy(pty_plan* plan);
/* The geometry a plan was created with (host memory out; no device work).
 * No reference counterpart: callers that size buffers for a plan's entry
 * points (which write n_frames frames) check their arrays against it. */
int pty_plan_geometry(const pty_plan* plan, pty_geometry* geom_out);

/* Whole reconstructions.  pty_era replaces ERA, ptychography/era.py:13-332;
 * pty_dm replaces DM, ptychography/dm.py:13-333.  *heatmap_valid (host) is
 * set to 0 when the reference would report info['heatmap'] = None. */
int pty_era(pty_plan* plan, const pty_buffers* buf, const pty_options* opt, int32_t iters,
            int32_t* heatmap_valid, void* stream);
int pty_dm(pty_plan* plan, const pty_buffers* buf, const pty_options* opt, int32_t iters,
           int32_t* heatmap_valid, void* stream);

/* Many independent reconstructions at once: the batched form of pty_era
 * (kind 0) or pty_dm (kind 1), for nrec distinct plans with their own buffers
 * and options.  No reference counterpart (the reference runs one
 * reconstruction per call).  All loops are captured into one CUDA graph with
 * one branch per reconstruction, launched once; heatmap_valid (host, nrec
 * entries) as in pty_era. */
int pty_run_batch(int32_t kind, pty_plan* const* plans, const pty_buffers* bufs,
                  const pty_options* opts, int32_t nrec, int32_t iters, int32_t* heatmap_valid,
                  void* stream);

/* Single operators (each replaces the reference function it names). */
/* make_exits, era.py:426-433 */
int pty_make_exits(pty_plan* plan, const void* O, const void* P, void* psi, void* stream);
/* pmod_1 + Pmod_1, era.py:550-572: psi in place; *eMod_dev = sum mask (|F|+a - amp)^2 */
int pty_pmod_1(pty_plan* plan, const float* amp, void* psi, const uint8_t* mask, double alpha,
               double* eMod_dev, void* stream);
/* pmod_7 + Pmod_7, era.py:574-595: psi and background (per frame) in place */
int pty_pmod_7(pty_plan* plan, const float* amp, float* background, void* psi,
               const uint8_t* mask, double alpha, double* eMod_dev, void* stream);
/* Pmod_P, era.py:597-610: P in place */
int pty_Pmod_P(pty_plan* plan, const float* Pamp, void* P, const uint8_t* mask, double alpha,
               void* stream);
/* psup_O, era.py:336-369; P_heatmap recomputed when recompute_heatmap != 0 */
int pty_psup_O(pty_plan* plan, const void* psi, const void* P, double* P_heatmap,
               int32_t recompute_heatmap, double alpha, void* O_out, void* stream);
/* psup_P, era.py:371-400; O_heatmap recomputed when recompute_heatmap != 0 */
int pty_psup_P(pty_plan* plan, const void* psi, const void* O, double* O_heatmap,
               int32_t recompute_heatmap, double alpha, void* P_out, void* stream);
/* make_P_heatmap, era.py:402-410 */
int pty_make_P_heatmap(pty_plan* plan, const void* P, double* heat, void* stream);
/* make_O_heatmap, era.py:412-417 */
int pty_make_O_heatmap(pty_plan* plan, const void* O, double* heat, void* stream);
/* model_error_1, dm.py:337-341.  background: NULL (= 0), one [N0][N1] pattern,
 * or [n][N0][N1] when background_per_frame != 0. */
int pty_model_error_1(pty_plan* plan, const float* amp, const void* psi, const uint8_t* mask,
                      const float* background, int32_t background_per_frame, double* err_dev,
                      void* stream);
/* info['I'] = fftshift |FFT(P * O[R])|^2, era.py:295 */
int pty_intensities(pty_plan* plan, const void* O, const void* P, float* I_out, void* stream);
/* Exit waves of Back_projection, back_projection.py:74-78: for every frame,
 * exits = ifftn(mask_c * sqrt(I)_c * exp(i angle(fftn(P)))), where amp and mask
 * are given in the engine's unshifted order (as for pty_pmod_1) and are used in
 * the reference's centred order, and phase holds the unit phasors
 * exp(i angle(fftn(P))) (complex64 [N0][N1], natural FFT order).  Even sizes. */
int pty_back_project(pty_plan* plan, const float* amp, const uint8_t* mask, const void* phase,
                     void* exits, void* stream);
/* Per-frame mean of a background stack, era.py:265-270 */
int pty_background_mean(pty_plan* plan, const float* background, float* mean_out, void* stream);

/* amp = ifftshift(sqrt(I)) per frame, the preamble's era.py:497-498.
 * I is float32 (is_double = 0) or float64 (is_double = 1), centred order. */
int pty_amp_from_intensity(pty_plan* plan, const void* I, int32_t is_double, float* amp,
                           void* stream);
/* pty_amp_from_intensity plus I_norm = sum(mask * I) over all frames
 * (era.py:495) into the device double *norm, summed in double in a fixed
 * order (a deterministic value, within rounding of the reference's sum in I's
 * dtype).  mask: the device uint8 mask in unshifted order (as pty_era takes
 * it), or NULL for all pixels. */
int pty_amp_and_norm(pty_plan* plan, const void* I, int32_t is_double, const uint8_t* mask,
                     float* amp, double* norm, void* stream);
/* Probe update for callers that cannot allocate device memory.  No
 * counterpart in the reference: it computes what pty_psup_P computes
 * (psup_P, era.py:371-400) without a plan, for code that must not call
 * cudaMalloc -- an application that owns the whole device budget, an
 * allocator that forbids foreign allocations, or a loop that must not block
 * on one.  Every input and output is the caller's: R_host is the int64
 * [n][2] scan offsets on the host (validated like pty_plan_create); psi,
 * O, O_heatmap (float64 [N0][N1], recomputed when recompute_heatmap != 0)
 * and P_out are device pointers.  The partial sums and the device copy of R
 * live in fixed arrays compiled into the library (8 MiB + 128 KiB on every
 * GPU that loads it, until the process exits); sizes beyond them --
 * N0 * N1 > 65536 or n_frames > 16384 -- are rejected with PTY_ERR_RANGE.
 * The offsets go to the device as kernel parameters of small copy launches
 * (one per 2048 frames), so the call makes no memcpy and does not
 * synchronise the host.  The first call on a device looks up that device's
 * copies of the arrays (cudaGetSymbolAddress, serialised across host
 * threads); make that first call on each device before any stream capture
 * begins.  All calls on one GPU share its arrays, so calls whose GPU work
 * overlaps (other streams, other host threads on the same GPU) race; nothing
 * in them needs clearing between calls, as each call writes every slot it
 * reads. */
int pty_psup_P_noalloc(const pty_geometry* geom, const int64_t* R_host, const void* psi,
                       const void* O, double* O_heatmap, int32_t recompute_heatmap, double alpha,
                       void* P_out, void* stream);
/* The random initial background of methods 4-6 (era.py:539-540:
 * np.random.random((n, N0, N1)).astype(dtype) + 0.1) drawn on the device from
 * NumPy's legacy global generator.  key[624] / pos: the MT19937 state as
 * np.random.get_state() returns it (host memory); count doubles are drawn
 * (n * N0 * N1), out[i] = float32(dtype(u_i) + 0.1) with dtype float64 when
 * rdt_double, else float32 (device memory); scratch: device memory of
 * pty_legacy_random_scratch_words(pos, count) uint32 words, or NULL to have
 * the call allocate it; key_out[624] / *pos_out: the state after the draw, to
 * be handed back with np.random.set_state.  Synchronises the stream. */
int pty_legacy_random_background(const uint32_t* key, int32_t pos, int64_t count,
                                 int32_t rdt_double, float* out, uint32_t* scratch,
                                 uint32_t* key_out, int32_t* pos_out, void* stream);
/* The same without synchronising: the draw and the copy of the state into
 * key_out are stream-ordered, so key_out must be page-locked host memory and
 * is valid once the stream has reached that point (*pos_out is set at once).
 * The public ERA / DM calls use it to overlap the draw with their uploads.
 * No reference counterpart beyond the draw itself. */
int pty_legacy_random_background_async(const uint32_t* key, int32_t pos, int64_t count,
                                       int32_t rdt_double, float* out, uint32_t* scratch,
                                       uint32_t* key_out, int32_t* pos_out, void* stream);
/* Scratch words pty_legacy_random_background needs (-1 for invalid input). */
int64_t pty_legacy_random_scratch_words(int32_t pos, int64_t count);
/* Host-side jump-ahead of the same generator (no reference counterpart; it
 * checks the jump-ahead that lets the device draw run in parallel segments):
 * window_out[624] = the 624 raw (untempered) words at offset `words` of the
 * sequence whose first 624 words are key (a state as np.random.get_state()
 * returns it right after a twist), from x^words mod phi, phi the generator's
 * characteristic polynomial.  The low 31 bits of window_out[0] are not the
 * sequence's (the generator never reads them). */
int pty_legacy_random_jump(const uint32_t* key, int64_t words, uint32_t* window_out);

/* ---- Learned warm start (no reference counterpart: the reference starts
 * ERA from an object of ones, era.py:480-486).  The network that maps sqrt(I)
 * frames to exit-wave phases (ptychography_gb300/warmstart.py) runs on these
 * device-memory building blocks; activations NHWC, "bf16" = bfloat16 arrays,
 * everything stream-ordered on `stream`, no host synchronisation.
 *   pty_ws_gemm: C(m, n) = sum_k A(m, k) B(k, n), A, B bf16 with element
 *     strides (A(m, k) = A[m sam + k sak], B(k, n) = B[k sbk + n sbn]), C float
 *     (C[m scm + n scn]); BF16 tensor-core products, FP32 accumulation.
 *     splits > 1 splits K (deterministic: partial[splits][M][N] summed in
 *     order) and needs C contiguous (scm = N, scn = 1).
 *   pty_ws_im2col: col[p][(ky*3 + kx) C + c] = X[b][y+ky-1][x+kx-1][c] (3 x 3,
 *     zero padding; X and col bf16); pty_ws_col2im: its adjoint (float).
 *   pty_ws_pool2 / pty_ws_up2: 2 x 2 average pooling / nearest 2 x
 *     upsampling (bf16), and their adjoints _bwd (float).
 *   pty_ws_bias_act: a = act(Z + bias) (relu if relu), out = a + skip (skip
 *     optional); a, out bf16 (optional), a32 float (optional).
 *   pty_ws_act_bwd: dZ = dA (relu: where a > 0), bf16; dbias[c] = sum_p dZ;
 *     scratch of pty_ws_act_bwd_scratch(P, C) floats.
 *   pty_ws_loss: weighted squared error of Y[P][2] against T[P][2], weights
 *     w[P] summing to 1: dY = 2 w (Y - T); loss_parts[256] partial sums.
 *   pty_ws_adam: one Adam step (Kingma and Ba) on float weights w with
 *     moments m, v (step counts from 1); wb (optional) gets a bf16 copy.
 *   pty_ws_to_bf16, pty_ws_add: element-wise conversion and sum;
 *   pty_ws_flip_weights: Wf[ci][t C_out + co] = W[co][(8 - t) C_in + ci] (bf16),
 *     the weights of the input-gradient convolution dX = conv3x3(dZ, Wf). */
int pty_ws_gemm(int32_t M, int32_t N, int32_t K, const void* A, int64_t sam, int64_t sak,
                const void* B, int64_t sbk, int64_t sbn, float* C, int64_t scm, int64_t scn,
                int32_t splits, float* partial, void* stream);
int pty_ws_im2col(int32_t B, int32_t H, int32_t W, int32_t C, const void* X, void* col, void* stream);
int pty_ws_col2im(int32_t B, int32_t H, int32_t W, int32_t C, const float* dcol, float* dX, void* stream);
int pty_ws_pool2(int32_t B, int32_t H, int32_t W, int32_t C, const void* X, void* Y, void* stream);
int pty_ws_pool2_bwd(int32_t B, int32_t H, int32_t W, int32_t C, const float* dY, float* dX, void* stream);
int pty_ws_up2(int32_t B, int32_t h, int32_t w, int32_t C, const void* X, void* Y, void* stream);
int pty_ws_up2_bwd(int32_t B, int32_t h, int32_t w, int32_t C, const float* dY, float* dX, void* stream);
int pty_ws_bias_act(int64_t P, int32_t C, const float* Z, const float* bias, int32_t relu,
                    const void* skip, void* a, void* out, float* a32, void* stream);
int64_t pty_ws_act_bwd_scratch(int64_t P, int32_t C);
int pty_ws_act_bwd(int64_t P, int32_t C, const float* dA, const void* a, int32_t relu, void* dZ,
                   float* dbias, float* scratch, void* stream);
int pty_ws_loss(int64_t P, const float* Y, const float* T, const float* w, float* dY,
                float* loss_parts, void* stream);
int pty_ws_adam(int64_t n, float* w, void* wb, const float* g, float* m, float* v, float lr,
                float b1, float b2, float eps, int32_t step, void* stream);
int pty_ws_to_bf16(int64_t n, const float* x, void* y, void* stream);
int pty_ws_add(int64_t n, const float* a, const float* b, float* out, void* stream);
int pty_ws_flip_weights(int32_t Cin, int32_t Cout, const void* W, void* Wf, void* stream);
/* Data for the network, nf frames of npix pixels:
 *   pty_ws_prep_bp: the network's input from back-projected exit waves bp
 *     (complex64 [nf][N0][N1]) under the probe P (complex64 [N0][N1]):
 *     x[f][p] = bf16 of (Re, Im) of s bp conj(P) / (max|P|^2 r), with
 *     r = sqrt(sum |bp|^2 / sum |P|^2) per frame and s = (-1)^(row + col)
 *     when checker != 0 (bp made by pty_back_project from the engine-order
 *     amplitudes and the fftshifted phasors fftshift(exp(i angle(fftn P))),
 *     which is the back-projection ifftn(sqrt(I) exp(i angle(fftn P))) in
 *     natural order times (-1)^(row + col); even sides only, else
 *     PTY_ERR_SHAPE), else 1.  x: bf16 [nf][N0][N1][2];
 *   pty_ws_targets: target[2 i .. 2 i + 1] = (cos, sin) of arg psi[i] (psi
 *     complex64), or with object_phase of arg psi[i] conj(P[i mod npix]);
 *     weight[i] = |P[i mod npix]|^2 wscale;
 *   pty_ws_exits: psi[i] = |P[i mod npix]| (y0 + i y1) / |(y0, y1)|, or with
 *     object_phase P[i mod npix] (y0 + i y1) / |(y0, y1)|: the exit waves with
 *     the predicted phases (y float pairs). */
int pty_ws_prep_bp(int32_t nf, int32_t N0, int32_t N1, const void* bp, const void* P, int32_t checker,
                   void* x, void* stream);
int pty_ws_targets(int32_t nf, int64_t npix, const void* psi, const void* P, int32_t object_phase,
                   float wscale, float* target, float* weight, void* stream);
int pty_ws_exits(int32_t nf, int64_t npix, const float* y, const void* P, int32_t object_phase,
                 void* psi, void* stream);
/* The same convolution on the CUDA cores for layers with few channels
 * (C_in even, 2..32; C_out 2, 4, 8, 16 or 32: the network's 2-channel first
 * and last layers), one thread per output pixel, no im2col buffer: out (bf16,
 * skip added when given) and/or out32 (float, no skip) may be NULL. */
int pty_ws_conv3x3_direct(int32_t B, int32_t H, int32_t W, int32_t Cin, int32_t Cout, const void* X,
                          const void* Wt, const float* bias, int32_t relu, const void* skip, void* out,
                          float* out32, void* stream);
/* Pieces of the warm start for frames larger than the network's (the frame
 * at a coarser real-space sampling):
 *   pty_ws_crop_center: out[f][a][b] = scale * I[g][a + (N0 - M0) / 2][b + (N1 - M1) / 2],
 *     g = frames[f] (a device int32 list, each entry a frame of I) or f when
 *     frames is NULL: the central M0 x M1 of each chosen centred pattern
 *     (float, device);
 *   pty_ws_upsample_object: O[u][v] = bilinear sample of Oh (Uh x Vh) at
 *     (u / f, v / f), clamped at the edges (complex64, device). */
int pty_ws_crop_center(int32_t nf, int32_t N0, int32_t N1, int32_t M0, int32_t M1, const float* I,
                       const int32_t* frames, float scale, float* out, void* stream);
int pty_ws_upsample_object(int32_t Uh, int32_t Vh, const void* Oh, int32_t U, int32_t V, int32_t f,
                           void* O, void* stream);
/* Per-frame phase alignment of predicted exit waves before they are stitched
 * again (a frame's far-field data fix its object phase only up to a
 * constant): for frame f with object window starting at win[f] = (a, b)
 * (device int32 [nf][2], the negated scan offsets of a plan),
 *   z_f = sum_r psi_f(r) conj(P(r) O(a + r0, b + r1)),  psi_f *= conj(z_f) / |z_f|;
 * psi complex64 [nf][M0][M1] in place, P complex64 [M0][M1], O complex64
 * [U][V] (the current stitched object).  A frame whose window is not inside
 * the object is left unchanged. */
int pty_ws_align_phase(int32_t nf, int32_t M0, int32_t M1, const int32_t* win, int32_t U, int32_t V,
                       const void* O, const void* P, void* psi, void* stream);
/* The network's forward 3 x 3 convolution (zero padding) on the tensor cores
 * (tcgen05, accumulators in tensor memory, operands staged by TMA), with the
 * bias, activation and skip of pty_ws_bias_act fused:
 *   out[p][co] = act(sum_{tap, ci} X[p shifted by tap][ci] Wt[co][tap C_in + ci]
 *                    + bias[co]) (+ skip[p][co]),
 * X, out, skip NHWC bf16 [B][H][W][C] (skip optional), Wt bf16 [C_out][9 C_in]
 * (the im2col path's layout), bias float [C_out], relu != 0 for ReLU.  The
 * same result as pty_ws_im2col + pty_ws_gemm + pty_ws_bias_act up to the FP32
 * summation order.  C_in = 32 or a multiple of 64, C_out a multiple of 32 up
 * to 128, W dividing 128 (H a multiple of 128 / W) or a multiple of 128;
 * arrays 16-byte aligned; others are PTY_ERR_UNSUPPORTED.  act, when not
 * NULL, also receives act(sum + bias) before the skip is added (bf16, as out):
 * the activation a training pass's backward reads.  Its mbarrier waits are
 * bounded (see pty_timeout_status). */
int pty_ws_conv3x3_tc(int32_t B, int32_t H, int32_t W, int32_t Cin, int32_t Cout, const void* X,
                      const void* Wt, const float* bias, int32_t relu, const void* skip, void* out,
                      void* act, void* stream);
/* The same convolution without bias, activation or skip, FP32 output out32
 * [B][H][W][C_out] (16-byte aligned): a training pass's input gradient,
 * conv3x3(dZ, Wf) with Wf from pty_ws_flip_weights.  Same shape rules. */
int pty_ws_conv3x3_tc_f32(int32_t B, int32_t H, int32_t W, int32_t Cin, int32_t Cout, const void* X,
                          const void* Wt, float* out32, void* stream);
/* The weight gradient of that convolution on the tensor cores:
 *   dW[co][tap C_in + ci] = sum_p dZ[p][co] X[p shifted by tap][ci]
 * (dW float [C_out][9 C_in], the im2col path's layout), from XS, the layer
 * input in three x-shifted channel-major copies, and dZT, the gradient at the
 * pre-activation sums channel-major, both made by pty_ws_shift_transpose:
 *   pty_ws_shift_transpose: XS[s][c][p] = X[p shifted by s - 1 along x][c]
 *     (zero past the row ends) for S = 3; XS[0][c][p] = X[p][c] for S = 1;
 *     X bf16 [P][C] (P = B H W, W even, C <= 128), XS bf16 [S][C][P];
 *   pty_ws_wgrad_tc: XS [3][C_in][P], dZT [C_out][P], C_in 32, 64 or 128,
 *     C_out 1..128, W 32 or a multiple of 64; scratch of at least
 *     pty_ws_wgrad_tc_scratch(...) floats (-1: shape unsupported) holds the
 *     per-split partial sums, added in split order (deterministic); arrays
 *     16-byte aligned.  Its mbarrier waits are bounded (pty_timeout_status). */
int pty_ws_shift_transpose(int32_t B, int32_t H, int32_t W, int32_t C, int32_t S, const void* X, void* XS,
                           void* stream);
int64_t pty_ws_wgrad_tc_scratch(int32_t B, int32_t H, int32_t W, int32_t Cin, int32_t Cout);
int pty_ws_wgrad_tc(int32_t B, int32_t H, int32_t W, int32_t Cin, int32_t Cout, const void* XS,
                    const void* dZT, float* dW, float* scratch, int64_t scratch_floats, void* stream);

/* 1 if the frame shape N0 x N1 has a fused FFT kernel. */
int pty_shape_supported(int32_t N0, int32_t N1);

/* Frame tiles (no reference counterpart): the number of CTAs that transform
 * one frame, 1 = one CTA per frame, C > 1 = a cluster of C CTAs; 100 + C = a
 * cluster of C CTAs whose line transforms run in three stages over 32
 * threads (8 values per thread at 256 points, 16 at 512: more threads per
 * CTA at fewer registers); 200 + C = staged: a row launch, a column launch
 * (C CTAs per frame) and an inverse row launch through a frame scratch of
 * about 2 GiB held by the plan, without clusters (512 x 512: tile 264).
 * Tiles are chosen per op family: family 0 = the
 * plain forms (Pmod_1, model error, intensities, back projection), family 1
 * = the background forms (Pmod_7 and the DM background recursion).  Shapes
 * with more than one tile built (128 x 128: 1 or 2; 256 x 256: 8, 4 or 108;
 * 512 x 512: 16, 116 or 264) get theirs from an autotuner run
 * by the first plan created for the shape on a device (disabled by
 * PTY_AUTOTUNE=0 in the environment: first candidate).  A plan keeps the
 * tiles chosen when it was created.
 *   pty_frame_tile_candidates: the tiles built for the shape (up to cap
 *     written to tiles[], their number to *count);
 *   pty_get_frame_tile: the tile new plans with at least one frame per SM
 *     get for the family (tunes now if not yet done); plans with fewer frames
 *     are tuned on their own frame count;
 *   pty_set_frame_tile: force a listed tile for the family in plans created
 *     afterwards on the current device, whatever their frame count; tile 0
 *     forgets forced and tuned choices (tuned again next time). */
int pty_frame_tile_candidates(int32_t N0, int32_t N1, int32_t* tiles, int32_t cap, int32_t* count);
int pty_get_frame_tile(int32_t N0, int32_t N1, int32_t family, int32_t* tile);
int pty_set_frame_tile(int32_t N0, int32_t N1, int32_t family, int32_t tile);
const char* pty_last_error(void);
/* Kernels that wait on TMA copies or tensor-core work through mbarriers
 * (pty_ws_conv3x3_tc, the staged 512 x 512 frame tile) bound every wait; one
 * that runs out sets a per-device flag, finishes its copies in flight and
 * returns, leaving its outputs invalid.  This reads the flag of the current
 * device into *timed_out (1: a wait ran out since the last call) and clears
 * it; it synchronises the calling thread with the device.  No reference
 * counterpart. */
int pty_timeout_status(int32_t* timed_out);
int pty_version(void);
/* Kernels this library has launched in the process so far (direct launches
 * plus the kernel nodes of replayed CUDA graphs).  No reference counterpart:
 * it lets a caller confirm the GPU path ran. */
int64_t pty_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* PTYCHO_GB300_H */
