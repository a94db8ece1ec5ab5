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
// least 227 back, so a CTA computes 227 words per step.  A long draw is cut
// into segments of 2^17 words generated by separate CTAs, each started from
// the 624-word window at its offset, which a jump-ahead computes (below); a
// last, fully parallel kernel tempers the words and forms the doubles: a
// double takes two consecutive outputs a, b,
// ((a >> 5) 2^26 + (b >> 6)) 2^-53 (53 random bits, NumPy's legacy conversion).
//
// Jump-ahead: the window at offset J is T^J applied to the first window, T the
// one-word advance of the generator's 19937-bit state (the top bit of the
// window's first word and its other 623 words).  T^J = g(T) with
// g(x) = x^J mod phi(x), phi the characteristic polynomial of T (degree
// 19937), after H. Haramoto, M. Matsumoto, T. Nishimura, F. Panneton and
// P. L'Ecuyer, "Efficient jump ahead for F2-linear random number generators",
// INFORMS J. Computing 20(3), 2008.  phi comes from the Berlekamp-Massey
// algorithm run on 2 x 19937 output bits of the generator itself, the jump
// polynomials x^(2^e) mod phi from repeated squaring; both once per process
// on the host.  Windows of segments [4^l, 4^(l+1)) are jumps of 1, 2 or 3 x
// 4^l segments from windows [0, 4^l), so a draw of S segments needs
// ceil(log4 S) rounds of jumps, each a launch of independent CTAs.  The low
// 31 bits of a jumped window's first word are not the sequence's (T ignores
// them): a segment uses only that word's top bit and writes only the words
// after its window.
#include <cuda_runtime.h>

#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/ptycho_gb300.h"
#include "engine.h"

namespace pty {

namespace {

constexpr int kMtN = 624;
constexpr int kMtLag = 227;                          // 624 - 397
constexpr int kThreads = 256;
constexpr int kMtDeg = 19937;                        // bits of generator state
constexpr int kPolyW = (kMtDeg + 63) / 64;           // 312 64-bit words
constexpr int kSegLog = 17;                          // segment: 2^17 words
constexpr long long kSegWords = 1ll << kSegLog;
constexpr int kMaxRounds = 24;                       // x^(2^(17 + r)), r < 24
constexpr int kLevels = kMaxRounds / 2;              // radix-4 rounds: up to 4^12 segments
constexpr int kJumpThreads = 640;
constexpr int kChunks = (kMtDeg + kMtLag - 1) / kMtLag;   // 88 chunks of 227 coefficients

__device__ __forceinline__ uint32_t mt_temper(uint32_t y) {
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

__host__ __device__ __forceinline__ uint32_t mt_next_word(uint32_t lag, uint32_t lo, uint32_t hi) {
  const uint32_t y = (lo & 0x80000000u) | (hi & 0x7fffffffu);
  return lag ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}

// Segment k writes words [624 + k L, 624 + (k+1) L) (clipped to total; L =
// 2^17) from win[k], the window of words [k L, k L + 624); segment 0 also
// copies the initial state to x[0, 624).  Step s computes words
// m = m0 + t (thread t < 227).  Word m needs x[m - 227] -- the same thread's
// word of the previous step, kept in a register -- and x[m - 624],
// x[m - 623], words of steps s - 2 and s - 3 read from a shared ring of the
// last 2048 words.  So one barrier after every second step makes every read
// word visible, and a slot is overwritten only ~9 steps after it was written,
// long after its last reader passed a barrier.
__global__ void __launch_bounds__(kThreads)
    legacy_segments_kernel(const uint32_t* __restrict__ win, long long total, uint32_t* __restrict__ x) {
  constexpr int kRingW = 2048;
  __shared__ uint32_t ring[kRingW];
  const int tid = threadIdx.x;
  const long long start = kMtN + (long long)blockIdx.x * kSegWords;
  const long long stop = start + kSegWords < total ? start + kSegWords : total;
  const uint32_t* w = win + (size_t)blockIdx.x * kMtN;
  for (int i = tid; i < kMtN; i += kThreads) {
    ring[(int)((start - kMtN + i) & (kRingW - 1))] = w[i];
    if (blockIdx.x == 0) x[i] = w[i];
  }
  __syncthreads();
  uint32_t prev = tid < kMtLag ? w[kMtN - kMtLag + tid] : 0u;   // x[m - 227] of the first step
  int step = 0;
  for (long long m0 = start; m0 < stop; m0 += kMtLag, ++step) {
    if (tid < kMtLag && m0 + tid < stop) {
      const int s = (int)((m0 + tid) & (kRingW - 1));
      const uint32_t v = mt_next_word(prev, ring[(s - kMtN) & (kRingW - 1)],
                                      ring[(s - kMtN + 1) & (kRingW - 1)]);
      ring[s] = v;
      x[m0 + tid] = v;
      prev = v;
    }
    if (step & 1) __syncthreads();
  }
}

// One radix-4 round of jumps: windows [0, nsrc) are the sources; block b
// computes window (j + 1) nsrc + i = g_j(T) window i, j = b / nsrc,
// i = b mod nsrc, with g_j = polys[j] = x^((j + 1) nsrc L) mod phi (windows
// at or past segs are skipped).  g as 19968 bits (624 32-bit words, degree
// < 19937).  Horner's rule 227 coefficients at a time:
// with S the source window extended by 227 words (sx[0, 851)),
//   R <- T^227 R  xor  sum_{j < 227} g_(hi - j) T^(226 - j) S,
// where T^227 R is 227 new words that each depend on R alone and T^k S is
// the window sx[k, k + 624).  88 chunks cover the coefficients (the highest
// chunk padded with zeros).
__global__ void __launch_bounds__(kJumpThreads)
    legacy_jump_kernel(const uint32_t* __restrict__ polys, uint32_t* win, int nsrc, long long segs) {
  constexpr int kR = 1024;                   // R as a ring: window at [base, base + 624)
  __shared__ uint32_t sx[kMtN + kMtLag];
  __shared__ uint32_t r[kR];
  __shared__ uint32_t gb[kMtN + 8];          // coefficients, zero above bit 19967
  const int tid = threadIdx.x;
  const int jj = blockIdx.x / nsrc, i0 = blockIdx.x % nsrc;
  const long long d = (long long)(jj + 1) * nsrc + i0;
  if (d >= segs) return;                     // whole block: no barrier skipped
  const uint32_t* g = polys + (size_t)jj * kMtN;
  const uint32_t* src = win + (size_t)i0 * kMtN;
  uint32_t* dst = win + (size_t)d * kMtN;
  for (int i = tid; i < kR; i += kJumpThreads) r[i] = 0u;
  for (int i = tid; i < kMtN + 8; i += kJumpThreads) gb[i] = i < kMtN ? g[i] : 0u;
  for (int i = tid; i < kMtN; i += kJumpThreads) sx[i] = src[i];
  __syncthreads();
  if (tid < kMtLag) sx[kMtN + tid] = mt_next_word(sx[tid + kMtN - kMtLag], sx[tid], sx[tid + 1]);
  __syncthreads();
  int base = 0;
  for (int c = 0; c < kChunks; ++c) {
    if (tid < kMtLag)
      r[(base + kMtN + tid) & (kR - 1)] = mt_next_word(r[(base + tid + kMtN - kMtLag) & (kR - 1)],
                                                      r[(base + tid) & (kR - 1)],
                                                      r[(base + tid + 1) & (kR - 1)]);
    __syncthreads();
    base += kMtLag;
    if (tid < kMtN) {
      const int hi = kChunks * kMtLag - 1 - kMtLag * c;   // this chunk's top coefficient
      uint32_t acc[4] = {0u, 0u, 0u, 0u};      // independent XOR chains
#pragma unroll
      for (int j = 0; j < kMtLag; j += 32) {
        // coefficients hi - j - k (k < 32) as bit k (the same for every
        // thread of the warp), applied as masks: no data-dependent loop
        const int top = hi - j, lo = top - 31;
        uint32_t bits;
        if (lo >= 0) {
          const int sh = lo & 31;
          const uint32_t a = gb[lo >> 5], b = gb[(lo >> 5) + 1];
          bits = sh ? (a >> sh) | (b << (32 - sh)) : a;     // bit k = coefficient lo + k
        } else {
          bits = gb[0] << (-lo);                             // no coefficients below 0
        }
        bits = __brev(bits);                                 // bit k = coefficient top - k
        const uint32_t* sp = sx + (kMtLag - 1 - j) + tid;    // sp[-k] = sx[226 - (j + k) + tid]
#pragma unroll
        for (int k = 0; k < 32; ++k)
          if (j + k < kMtLag) acc[k & 3] ^= sp[-k] & (0u - ((bits >> k) & 1u));
      }
      r[(base + tid) & (kR - 1)] ^= (acc[0] ^ acc[1]) ^ (acc[2] ^ acc[3]);
    }
    __syncthreads();
  }
  for (int i = tid; i < kMtN; i += kJumpThreads) dst[i] = r[(base + i) & (kR - 1)];
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

// ------------------------------------------------------------ host side
// GF(2) polynomials as little-endian bit vectors of 64-bit words.
using Bits = std::vector<uint64_t>;

inline int bit_of(const Bits& v, long long i) { return (int)((v[(size_t)(i >> 6)] >> (i & 63)) & 1u); }

// v ^= u << sh, for the first nu words of u (bits beyond v's end dropped)
void xor_shl(Bits& v, const Bits& u, int nu, long long sh) {
  const size_t ws = (size_t)(sh >> 6);
  const int bs = (int)(sh & 63);
  for (int i = 0; i < nu && ws + i < v.size(); ++i) {
    const uint64_t w = u[(size_t)i];
    if (!w) continue;
    v[ws + i] ^= w << bs;
    if (bs && ws + i + 1 < v.size()) v[ws + i + 1] ^= w >> (64 - bs);
  }
}

inline int parity64(uint64_t x) {
  x ^= x >> 32;
  x ^= x >> 16;
  x ^= x >> 8;
  x ^= x >> 4;
  x ^= x >> 2;
  x ^= x >> 1;
  return (int)(x & 1u);
}

// phi by Berlekamp-Massey over GF(2) on the top bits of 2 x 19937 words of
// the sequence from init_genrand(5489) (Matsumoto and Nishimura's reference
// initialisation); any non-zero output bit sequence of the generator has
// phi (primitive) as its minimal polynomial.  Returns phi as 312 words, or
// nothing if the sequence's linear complexity is not 19937.
Bits charpoly_phi() {
  constexpr int N = 2 * kMtDeg;
  std::vector<uint32_t> x(kMtN + N);
  x[0] = 5489u;
  for (int i = 1; i < kMtN; ++i) x[i] = 1812433253u * (x[i - 1] ^ (x[i - 1] >> 30)) + (uint32_t)i;
  for (int m = kMtN; m < kMtN + N; ++m) x[m] = mt_next_word(x[m - kMtLag], x[m - kMtN], x[m - kMtN + 1]);
  const int W = N / 64 + 2;
  Bits C(W, 0), B(W, 0), V(W, 0);   // connection polynomial, its last copy, s reversed
  C[0] = B[0] = 1;
  int L = 0, m = 1;
  for (int n = 0; n < N; ++n) {
    // V bit i = s[n - i], s[n] the top bit of word 624 + n
    for (int i = W - 1; i > 0; --i) V[i] = (V[i] << 1) | (V[i - 1] >> 63);
    V[0] = (V[0] << 1) | (x[kMtN + n] >> 31);
    uint64_t acc = 0;
    for (int i = 0; i <= L / 64; ++i) acc ^= C[i] & V[i];
    if (!parity64(acc)) {              // no discrepancy
      ++m;
      continue;
    }
    if (2 * L <= n) {
      Bits Cprev = C;
      xor_shl(C, B, W, m);
      L = n + 1 - L;
      B = Cprev;
      m = 1;
    } else {
      xor_shl(C, B, W, m);
      ++m;
    }
  }
  if (L != kMtDeg) return Bits();
  Bits phi(kPolyW, 0);
  for (int i = 0; i <= L; ++i)         // phi_i = C_(L - i)
    if (bit_of(C, L - i)) phi[(size_t)(i >> 6)] ^= 1ull << (i & 63);
  return phi;
}

// q reduced modulo phi to 312 words
Bits reduce_phi(Bits q, const Bits& phi) {
  for (long long b = (long long)q.size() * 64 - 1; b >= kMtDeg; --b)
    if (bit_of(q, b)) xor_shl(q, phi, kPolyW, b - kMtDeg);
  q.resize(kPolyW);
  return q;
}

inline uint64_t spread32(uint32_t v) {     // bit i -> bit 2 i
  uint64_t x = v;
  x = (x | (x << 16)) & 0x0000ffff0000ffffull;
  x = (x | (x << 8)) & 0x00ff00ff00ff00ffull;
  x = (x | (x << 4)) & 0x0f0f0f0f0f0f0f0full;
  x = (x | (x << 2)) & 0x3333333333333333ull;
  x = (x | (x << 1)) & 0x5555555555555555ull;
  return x;
}

Bits sqr_mod(const Bits& p, const Bits& phi) {   // squaring in GF(2): bit i -> bit 2 i
  Bits q(2 * kPolyW, 0);
  for (int i = 0; i < kPolyW; ++i) {
    q[(size_t)(2 * i)] = spread32((uint32_t)p[(size_t)i]);
    q[(size_t)(2 * i + 1)] = spread32((uint32_t)(p[(size_t)i] >> 32));
  }
  return reduce_phi(std::move(q), phi);
}

Bits mul_mod(const Bits& a, const Bits& b, const Bits& phi) {
  Bits q(2 * kPolyW + 1, 0);
  for (long long i = 0; i < kMtDeg; ++i)
    if (bit_of(a, i)) xor_shl(q, b, kPolyW, i);
  return reduce_phi(std::move(q), phi);
}

struct JumpTable {
  Bits phi;
  std::vector<Bits> pow2;      // pow2[r] = x^(2^(17 + r)) mod phi
  std::vector<Bits> pow3;      // pow3[l] = x^(3 4^l 2^17) mod phi
  bool ok = false;
};

const JumpTable& jump_table() {
  static JumpTable t;
  static std::once_flag once;
  std::call_once(once, [] {
    t.phi = charpoly_phi();
    if (t.phi.empty()) return;
    Bits p(kPolyW, 0);
    p[0] = 2;                    // x
    for (int e = 0; e < kSegLog; ++e) p = sqr_mod(p, t.phi);
    for (int r = 0; r < kMaxRounds; ++r) {
      t.pow2.push_back(p);
      p = sqr_mod(p, t.phi);
    }
    for (int l = 0; l < kLevels; ++l) t.pow3.push_back(mul_mod(t.pow2[2 * l], t.pow2[2 * l + 1], t.phi));
    t.ok = true;
  });
  return t;
}

// g(T) applied to a 624-word window on the host: Horner's rule one
// coefficient at a time, R kept as a growing sequence (window at offset t)
void host_apply_poly(const Bits& g, const uint32_t* src, uint32_t* dst) {
  std::vector<uint32_t> r((size_t)kMtN + kMtDeg + 1, 0u);
  long long t = 0;
  for (long long i = kMtDeg - 1; i >= 0; --i) {
    r[(size_t)(t + kMtN)] = mt_next_word(r[(size_t)(t + kMtN - kMtLag)], r[(size_t)t], r[(size_t)(t + 1)]);
    ++t;
    if (bit_of(g, i))
      for (int p = 0; p < kMtN; ++p) r[(size_t)(t + p)] ^= src[p];
  }
  for (int p = 0; p < kMtN; ++p) dst[p] = r[(size_t)(t + p)];
}

// words of the draw's sequence (through the 624-word block holding its last
// word) and its segments
struct DrawSize {
  long long total, segs;
};
DrawSize draw_size(int pos, long long count) {
  const long long end = (long long)pos + 2 * count;           // one past the last word drawn
  const long long total = ((end - 1) / kMtN + 1) * kMtN;
  const long long gen = total - kMtN;
  return {total, gen > 0 ? (gen + kSegWords - 1) / kSegWords : 1};
}

// the jump polynomials x^(2^(17 + r)) mod phi on the device (once per device)
int device_jump_polys(const uint32_t** out) {
  static std::mutex mu;
  static std::map<int, uint32_t*> per_dev;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_cuda_error(e, "cudaGetDevice");
  std::lock_guard<std::mutex> lk(mu);
  auto it = per_dev.find(dev);
  if (it != per_dev.end()) {
    *out = it->second;
    return PTY_OK;
  }
  const JumpTable& jt = jump_table();
  if (!jt.ok) return set_error(PTY_ERR_CUDA, "MT19937 characteristic polynomial not found");
  // level l: x^(j 4^l 2^17) for j = 1, 2, 3 (pow2[2 l], pow2[2 l + 1], pow3[l])
  std::vector<uint32_t> h((size_t)kLevels * 3 * kMtN, 0u);
  for (int l = 0; l < kLevels; ++l)
    for (int j = 0; j < 3; ++j) {
      const Bits& q = j == 0 ? jt.pow2[(size_t)(2 * l)] : j == 1 ? jt.pow2[(size_t)(2 * l + 1)] : jt.pow3[(size_t)l];
      uint32_t* o = &h[((size_t)l * 3 + j) * kMtN];
      for (int i = 0; i < kPolyW; ++i) {
        o[2 * i] = (uint32_t)q[(size_t)i];
        o[2 * i + 1] = (uint32_t)(q[(size_t)i] >> 32);
      }
    }
  uint32_t* d = nullptr;
  e = cudaMalloc(&d, h.size() * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemcpy(d, h.data(), h.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    if (d) cudaFree(d);
    return set_cuda_error(e, "jump polynomial upload");
  }
  per_dev[dev] = d;
  *out = d;
  return PTY_OK;
}

}  // namespace

}  // namespace pty

using namespace pty;

extern "C" int64_t pty_legacy_random_scratch_words(int32_t pos, int64_t count) {
  if (pos < 0 || pos > kMtN || count < 1) return -1;
  const DrawSize d = draw_size(pos, count);
  // the sequence, 624 spare words, one 624-word window per segment
  return d.total + kMtN + d.segs * kMtN;
}

static int random_background(const uint32_t* key, int32_t pos, int64_t count, int32_t rdt_double, float* out,
                             uint32_t* scratch, uint32_t* key_out, int32_t* pos_out, void* stream, bool sync) {
  if (!key || !out || !key_out || !pos_out) return set_error(PTY_ERR_ARG, "null argument");
  if (pos < 0 || pos > kMtN) return set_error(PTY_ERR_ARG, "generator position outside 0..624");
  if (count < 1) return set_error(PTY_ERR_ARG, "count must be positive");
  cudaStream_t st = (cudaStream_t)stream;
  const DrawSize d = draw_size(pos, count);
  const long long total = d.total, segs = d.segs;
  if (segs > (1ll << (2 * kLevels))) return set_error(PTY_ERR_RANGE, "draw too large");
  const uint32_t* polys = nullptr;
  if (segs > 1) PTY_TRY(device_jump_polys(&polys));
  // the sequence x[0, total), 624 spare words, the segment windows: the
  // caller's scratch, else stream-ordered
  uint32_t* d_x = scratch;
  cudaError_t e = cudaSuccess;
  const size_t words = (size_t)(total + kMtN + segs * kMtN);
  if (!d_x) {
    e = cudaMallocAsync(&d_x, words * sizeof(uint32_t), st);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return set_error(PTY_ERR_NOMEM, "generator scratch allocation failed");
    }
  }
  uint32_t* d_win = d_x + total + kMtN;
  int rc = PTY_OK;
  e = cudaMemcpyAsync(d_win, key, kMtN * sizeof(uint32_t), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) rc = set_cuda_error(e, "generator state upload");
  // radix-4 rounds: windows of segments [4^l, 4^(l+1)) jump 1, 2 or 3 x 4^l
  // segments from windows [0, 4^l)
  int level = 0;
  for (long long nsrc = 1; rc == PTY_OK && nsrc < segs; nsrc *= 4, ++level) {
    const long long want = segs - nsrc < 3 * nsrc ? segs - nsrc : 3 * nsrc;
    const long long blocks = ((want + nsrc - 1) / nsrc) * nsrc;       // whole j groups
    legacy_jump_kernel<<<(unsigned)blocks, kJumpThreads, 0, st>>>(polys + (size_t)level * 3 * kMtN, d_win,
                                                                 (int)nsrc, segs);
    rc = check_launch("legacy_jump_kernel");
  }
  if (rc == PTY_OK) {
    legacy_segments_kernel<<<(unsigned)segs, kThreads, 0, st>>>(d_win, total, d_x);
    rc = check_launch("legacy_segments_kernel");
  }
  if (rc == PTY_OK) {
    legacy_uniform_kernel<<<4 * 152, 256, 0, st>>>(d_x, pos, count, rdt_double != 0, out);
    rc = check_launch("legacy_uniform_kernel");
  }
  if (rc == PTY_OK) {
    // the state after the draw: the last 624 words
    e = cudaMemcpyAsync(key_out, d_x + (total - kMtN), kMtN * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) rc = set_cuda_error(e, "generator state copy");
  }
  if (!scratch) cudaFreeAsync(d_x, st);
  if (rc == PTY_OK && sync) {
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = set_cuda_error(e, "generator state copy");
  }
  if (rc == PTY_OK) {
    const long long end = (long long)pos + 2 * count;
    *pos_out = (int32_t)((end - 1) % kMtN + 1);
  }
  return rc;
}

extern "C" int pty_legacy_random_background(const uint32_t* key, int32_t pos, int64_t count,
                                            int32_t rdt_double, float* out, uint32_t* scratch,
                                            uint32_t* key_out, int32_t* pos_out, void* stream) {
  return random_background(key, pos, count, rdt_double, out, scratch, key_out, pos_out, stream, true);
}

extern "C" int pty_legacy_random_background_async(const uint32_t* key, int32_t pos, int64_t count,
                                                  int32_t rdt_double, float* out, uint32_t* scratch,
                                                  uint32_t* key_out, int32_t* pos_out, void* stream) {
  return random_background(key, pos, count, rdt_double, out, scratch, key_out, pos_out, stream, false);
}

// The window of 624 words at offset `words` of the raw sequence whose first
// window is key (key as np.random.get_state() returns it, a freshly twisted
// state), computed on the host with the jump-ahead polynomial x^words mod phi;
// the first word's low 31 bits are not the sequence's.  For tests of the
// jump-ahead.
extern "C" int pty_legacy_random_jump(const uint32_t* key, int64_t words, uint32_t* window_out) {
  if (!key || !window_out) return set_error(PTY_ERR_ARG, "null argument");
  if (words < 0) return set_error(PTY_ERR_ARG, "negative jump");
  const JumpTable& jt = jump_table();
  if (!jt.ok) return set_error(PTY_ERR_CUDA, "MT19937 characteristic polynomial not found");
  Bits g(kPolyW, 0), base(kPolyW, 0);    // x^words by square-and-multiply
  g[0] = 1;
  base[0] = 2;
  for (int64_t e = words; e > 0; e >>= 1) {
    if (e & 1) g = mul_mod(g, base, jt.phi);
    if (e > 1) base = sqr_mod(base, jt.phi);
  }
  host_apply_poly(g, key, window_out);
  return PTY_OK;
}
