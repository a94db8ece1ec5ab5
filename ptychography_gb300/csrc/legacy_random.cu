// NumPy's legacy global generator continued on the device.
//
// The reference draws the initial background of methods 4-6 from NumPy's
// global RandomState (ptychography/era.py:539-540,
// np.random.random((n, N0, N1)).astype(dtype) + 0.1): at 1024 x 256^2 that is
// 67 M doubles, a quarter of a second of single-core Mersenne Twister on the
// host, then two dtype passes and an upload.  pty_legacy_random_background
// produces the same numbers on the GPU from the generator's state and returns
// the state the host generator would have afterwards, so the caller can hand
// it back to NumPy and every later draw is unchanged.
//
// The generator is MT19937 (M. Matsumoto and T. Nishimura, "Mersenne Twister:
// a 623-dimensionally equidistributed uniform pseudo-random number generator",
// ACM TOMACS 8(1), 1998).  Written as a sequence, with x[0..623] the state
// array as last twisted:
//   x[m] = x[m - 227] ^ ((y >> 1) ^ (y & 1 ? 0x9908b0df : 0)),
//   y    = (x[m - 624] & 0x80000000) | (x[m - 623] & 0x7fffffff),   m >= 624,
// and the k-th output is temper(x[pos + k]).  Each word depends on words at
// least 227 back, so one CTA computes 227 words per step and writes them out
// (the only serial part, ~0.6 M steps at 1024 x 256^2); a second, fully
// parallel kernel tempers them and forms the doubles: a double takes two
// consecutive outputs a, b,
// ((a >> 5) 2^26 + (b >> 6)) 2^-53 (53 random bits, NumPy's legacy conversion).
#include <cuda_runtime.h>

#include <cstring>

#include "../../include/ptycho_gb300.h"
#include "engine.h"

namespace pty {

namespace {

constexpr int kMtN = 624;
constexpr int kMtLag = 227;          // 624 - 397
constexpr int kThreads = 256;

struct MtState {
  uint32_t key[kMtN];
};

__device__ __forceinline__ uint32_t mt_temper(uint32_t y) {
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

__device__ __forceinline__ uint32_t mt_next_word(uint32_t lag, uint32_t lo, uint32_t hi) {
  const uint32_t y = (lo & 0x80000000u) | (hi & 0x7fffffffu);
  return lag ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}

// Words x[0, total) of the sequence into x (x[0..623] = the state array); the
// last 624 computed words, the state after the draw, into key_out.  One CTA:
// step s computes words m = 624 + 227 s + t (thread t < 227).  Word m needs
// x[m - 227] -- the same thread's word of step s - 1, kept in a register --
// and x[m - 624], x[m - 623], words of steps s - 2 and s - 3 read from a
// shared ring of the last 2048 words.  So one barrier after every second
// step makes every read word visible, and a slot is overwritten only ~9 steps
// after it was written, long after its last reader passed a barrier.
__global__ void __launch_bounds__(kThreads, 1)
    legacy_words_kernel(MtState st, long long total, uint32_t* x, uint32_t* key_out) {
  constexpr int kRingW = 2048;
  __shared__ uint32_t ring[kRingW];
  const int tid = threadIdx.x;
  for (int i = tid; i < kMtN; i += kThreads) {
    ring[i] = st.key[i];
    x[i] = st.key[i];
  }
  __syncthreads();
  uint32_t prev = tid < kMtLag ? ring[kMtN - kMtLag + tid] : 0u;   // x[m - 227] of step 0
  int step = 0;
  for (long long m0 = kMtN; m0 < total; m0 += kMtLag, ++step) {
    if (tid < kMtLag && m0 + tid < total) {
      const int s = (int)((m0 + tid) & (kRingW - 1));
      const uint32_t v = mt_next_word(prev, ring[(s - kMtN) & (kRingW - 1)],
                                      ring[(s - kMtN + 1) & (kRingW - 1)]);
      ring[s] = v;
      x[m0 + tid] = v;
      prev = v;
    }
    if (step & 1) __syncthreads();
  }
  __syncthreads();
  for (int i = tid; i < kMtN; i += kThreads)
    key_out[i] = ring[(int)((total - kMtN + i) & (kRingW - 1))];
}

// out[i] = float32(dtype(u_i) + 0.1), u_i the double from outputs pos + 2 i and
// pos + 2 i + 1 (NumPy's legacy 53-bit conversion).
__global__ void legacy_uniform_kernel(const uint32_t* __restrict__ x, int pos, long long count,
                                      int rdt_double, float* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const long long w = pos + 2 * i;
    const uint32_t a = mt_temper(x[w]) >> 5;
    const uint32_t b = mt_temper(x[w + 1]) >> 6;
    const unsigned long long v = ((unsigned long long)a << 26) | b;   // < 2^53
    float r;
    if (rdt_double) {
      r = __double2float_rn(__dadd_rn(__ull2double_rn(v) * 0x1p-53, 0.1));
    } else {
      // float32(v 2^-53): v rounds once to float32, the power-of-two scale is exact
      r = __fadd_rn(__ull2float_rn(v) * 0x1p-53f, 0.1f);
    }
    out[i] = r;
  }
}

}  // namespace

}  // namespace pty

using namespace pty;

extern "C" int64_t pty_legacy_random_scratch_words(int32_t pos, int64_t count) {
  if (pos < 0 || pos > kMtN || count < 1) return -1;
  const long long end = (long long)pos + 2 * (long long)count;
  return ((end - 1) / kMtN + 1) * kMtN + kMtN;
}

extern "C" int pty_legacy_random_background(const uint32_t* key, int32_t pos, int64_t count,
                                            int32_t rdt_double, float* out, uint32_t* scratch,
                                            uint32_t* key_out, int32_t* pos_out, void* stream) {
  if (!key || !out || !key_out || !pos_out) return set_error(PTY_ERR_ARG, "null argument");
  if (pos < 0 || pos > kMtN) return set_error(PTY_ERR_ARG, "generator position outside 0..624");
  if (count < 1) return set_error(PTY_ERR_ARG, "count must be positive");
  cudaStream_t st = (cudaStream_t)stream;
  MtState s;
  std::memcpy(s.key, key, sizeof(s.key));
  const long long end = (long long)pos + 2 * (long long)count;   // one past the last word drawn
  const long long total = ((end - 1) / kMtN + 1) * kMtN;          // through the block holding it
  // raw words plus the final state: the caller's scratch, else stream-ordered
  uint32_t* d_x = scratch;
  cudaError_t e = cudaSuccess;
  if (!d_x) {
    e = cudaMallocAsync(&d_x, (size_t)(total + kMtN) * sizeof(uint32_t), st);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return set_error(PTY_ERR_NOMEM, "generator scratch allocation failed");
    }
  }
  uint32_t* d_key = d_x + total;
  legacy_words_kernel<<<1, kThreads, 0, st>>>(s, total, d_x, d_key);
  int rc = check_launch("legacy_words_kernel");
  if (rc == PTY_OK) {
    legacy_uniform_kernel<<<4 * 152, 256, 0, st>>>(d_x, pos, count, rdt_double != 0, out);
    rc = check_launch("legacy_uniform_kernel");
  }
  if (rc == PTY_OK) {
    e = cudaMemcpyAsync(key_out, d_key, kMtN * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) rc = set_cuda_error(e, "generator state copy");
  }
  if (!scratch) cudaFreeAsync(d_x, st);
  if (rc == PTY_OK) {
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = set_cuda_error(e, "generator state copy");
  }
  if (rc == PTY_OK) *pos_out = (int32_t)((end - 1) % kMtN + 1);
  return rc;
}
