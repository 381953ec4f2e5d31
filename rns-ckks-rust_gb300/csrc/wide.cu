// Exact integer key product ("wide-CRT") for the hybrid and Q-only keyswitch.
//
// The reference forms sum_i d_i * k_ij mod q_j for every limb j of the key
// (src/rns/keyswitching.rs:130-194): D digit polynomials times D key
// polynomials per limb.  Because the balanced digits satisfy |d_i| <= 2^29 and
// the key residues 0 <= k_ij < q_j, the negacyclic convolution
// S_j = sum_i d_i * k_ij has integer coefficients bounded by
// D * N * 2^29 * (q_j - 1).  Here S_j is computed exactly under four internal
// primes w0..w3 < 2^29 (A = w0 w1 w2 w3 > 4 * bound, checked on the host) and
// turned back into S_j mod q_j by CRT in the finalize pass, which gives the
// reference's residues bit for bit.  The digits are transformed once per
// internal prime (4 D transforms instead of D (l + K)), and the key product is
// one 32 x 32 -> 64-bit multiply-add per term.
//
// The primes are handled in pairs (w0, w1), (w2, w3): an element is a uint2
// of its two residues, which keeps the 8-byte element layouts and swizzles of
// the 64-bit transforms (nttcore.cuh).  Layouts (uint2 elements):
//   digit transforms, tiled:  dtt[job][pair][x/32][digit][32]
//   key, tiled:               kwt[limb][pair][x/32][digit][c][32]
//   products:                 acc[job][c][limb][pair][N]
#include <mutex>

#include "kernels.cuh"
#include "nttcore.cuh"
#include "wide.cuh"
#include "nttr16.cuh"

namespace rc {
namespace {

constexpr int W_ROW_WARPS = 4;
// warps per key-product CTA: 8 for job groups (two CTAs per SM); one job per CTA (the per-op path, bound by the
// key stream) takes 13, more loads in flight per SM
template <int BC>
__host__ __device__ constexpr int w_mac_warps() {
  return BC == 1 ? 13 : 8;
}

// entry 2 * pair + k of a four-entry table in the kernel parameter, picked by a select: a dynamic index
// would copy the whole parameter struct to local memory
template <class T>
__device__ __forceinline__ T pick(const T (&a)[4], int pair, int k) {
  return pair ? a[2 + k] : a[k];
}

template <int M>
struct WColTile {
  static constexpr int COLS = (8 * core::Geo<M>::SUBS) > 16 ? 8 * core::Geo<M>::SUBS : 16;
};

__device__ __forceinline__ uint2 reduce4(uint2 v, uint32_t q0, uint32_t q1) {
  uint32_t a = v.x >= 2 * q0 ? v.x - 2 * q0 : v.x;
  uint32_t b = v.y >= 2 * q1 ? v.y - 2 * q1 : v.y;
  return make_uint2(fold32(a, q0), fold32(b, q1));
}

// Forward column phase of polynomial p0 + blockIdx.z under pair blockIdx.y.
// SRC 0: int32 digits[poly][N], taken as d + 2q (in [0, 4q) since 2q > 2^29);
// SRC 1: residues src[poly][pair][N].  Output out[poly][pair][N].
template <int M1, int M2, int SRC>
__global__ __launch_bounds__(256, 2) void k_w_cols_fwd(WidePrimes w, const void* src, uint2* out, int p0) {
  using G = core::Geo<M1>;
  constexpr int COLS = WColTile<M1>::COLS, N1 = 1 << M1, N2 = 1 << M2, N = N1 * N2;
  __shared__ uint2 tile[COLS * G::STRIDE];
  __shared__ __align__(16) Tw2 twl[N1];
  const int c0 = blockIdx.x * COLS;
  const int pair = blockIdx.y;
  const size_t poly = (size_t)p0 + blockIdx.z;
  const uint32_t q0 = pick(w.q, pair, 0), q1 = pick(w.q, pair, 1);
  // tile (digits: the int32 into the element's first word, converted at first use) and twiddles by
  // asynchronous copies, all in flight together; thread t copies column t mod COLS of rows it R + t / COLS
  // from one per-thread base (the swizzled row it R + (r0 ^ swz_h(it R / 16)), as in k_cols_f)
  constexpr int R = 256 / COLS, ROUNDS = N1 * COLS / 256;
  static_assert(R * COLS == 256, "tile rounds");
  const int r0 = threadIdx.x / COLS, cc = threadIdx.x % COLS;
  uint2* tc = tile + cc * G::STRIDE;
  const size_t goff = (size_t)r0 * N2 + c0 + cc;
#pragma unroll
  for (int it = 0; it < ROUNDS; ++it) {
    uint2* s = tc + it * R + (r0 ^ core::swz_h<M1>((it * R) >> 4));
    if (SRC == 0)
      core::cp_async4(&s->x, static_cast<const int32_t*>(src) + poly * N + goff + (size_t)it * R * N2);
    else
      core::cp_async8(s, static_cast<const uint2*>(src) + (poly * 2 + pair) * N + goff + (size_t)it * R * N2);
  }
  core::stage_twiddles_async<M1>(twl, w.tw_fwd + (size_t)pair * N, 1, threadIdx.x, 256);
  core::cp_async_wait_all();
  __syncthreads();
  const int warp = threadIdx.x >> 5;
#pragma unroll 1
  for (int cb = warp * G::SUBS; cb < COLS; cb += 8 * G::SUBS) {
    const int lv = core::lane_id_volatile();
    const int sub = lv / G::LANES, l = lv % G::LANES;
    uint2* buf = tile + (cb + sub) * G::STRIDE;
    uint2 v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      v[k] = buf[core::swz<M1>(core::first_idx<M1>(l, k))];
      if (SRC == 0) {  // digit d as d + 2q, in [0, 4q) since 2q > 2^29 >= |d|
        const int32_t d = (int32_t)v[k].x;
        v[k] = make_uint2((uint32_t)(d + (int32_t)(2 * q0)), (uint32_t)(d + (int32_t)(2 * q1)));
      }
    }
    __syncwarp();
    core::fwd_sub2<M1>(v, buf, l, twl, q0, q1);
#pragma unroll
    for (int k = 0; k < 8; ++k) buf[core::swz<M1>(core::last_idx<M1>(l, k))] = v[k];
  }
  __syncthreads();
  uint2* o = out + (poly * 2 + pair) * N + goff;
#pragma unroll
  for (int it = 0; it < ROUNDS; ++it) o[(size_t)it * R * N2] = tc[it * R + (r0 ^ core::swz_h<M1>((it * R) >> 4))];
}

// Row kernels: a block transforms the same ROWS rows of W_ROW_POLYS consecutive polynomials, so each row's
// twiddles (as many bytes as two rows of data) are staged once for all of them; the next polynomial's rows
// are loaded while the current one is transformed.
constexpr int W_ROW_POLYS = 16;

// Where digit polynomial `poly` of a batch goes in the tiled layout: its job's first digit polynomial, its
// digit index and its job's digit count.  UniDig: D digits per job (poly = job * D + digit); MlDig: job j's
// digits are polynomials [dig[j], dig[j+1]), found by a binary search for a block's first polynomial and
// then followed forward (`job` carries the position between calls).
struct UniDig {
  int D;
  __device__ __forceinline__ void locate(int poly, int& job, int& first, int& digit, int& d) const {
    job = poly / D;
    first = job * D;
    digit = poly - first;
    d = D;
  }
};
struct MlDig {
  int J;
  int dig[ML_MAXJ + 1];
  __device__ __forceinline__ void locate(int poly, int& job, int& first, int& digit, int& d) const {
    if (job < 0) {  // first call: the last job whose first digit is at or below poly
      int lo = 0, hi = J - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (dig[mid] <= poly) lo = mid;
        else hi = mid - 1;
      }
      job = lo;
    }
    while (poly >= dig[job + 1]) ++job;
    first = dig[job];
    digit = poly - first;
    d = dig[job + 1] - first;
  }
};

// Forward row phase of data[poly][pair][N] (polys p0 + blockIdx.z * W_ROW_POLYS .. below p0 + cnt), outputs
// reduced to [0, q).  TILED: written as dtt[job][pair][x/32][digit][32] (job j's tiles from 2 N first(j),
// DM maps a polynomial to its job); otherwise in place.
template <int M1, int M2, bool TILED, class DM>
__global__ __launch_bounds__(32 * W_ROW_WARPS) void k_w_rows_fwd(WidePrimes w, uint2* data, uint2* dtt, int p0,
                                                                 int cnt, DM dm) {
  using G = core::Geo<M2>;
  constexpr int N1 = 1 << M1, N2 = 1 << M2, N = N1 * N2, ROWS = W_ROW_WARPS * G::SUBS;
  __shared__ uint2 bufs[ROWS * G::STRIDE];
  __shared__ __align__(16) Tw2 twl[ROWS][N2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane / G::LANES, l = lane % G::LANES;
  const int row0 = blockIdx.x * ROWS;
  const int pair = blockIdx.y;
  const int first = blockIdx.z * W_ROW_POLYS, count = min(W_ROW_POLYS, cnt - first);
  const uint32_t q0 = pick(w.q, pair, 0), q1 = pick(w.q, pair, 1);
  const Tw2* twg = w.tw_fwd + (size_t)pair * N;
  const int rl = warp * G::SUBS + sub, row = row0 + rl;
  auto row_ptr = [&](int t) { return data + (((size_t)p0 + first + t) * 2 + pair) * N + (size_t)row * N2; };
  uint2* buf = bufs + rl * G::STRIDE;
  int job = -1;  // the digit map's position (TILED)
  uint2 v[8], vn[8];  // requested before the twiddle tables, so both latencies overlap
  {
    const uint2* in = row_ptr(0);
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = in[core::first_idx<M2>(l, k)];
  }
#pragma unroll 1
  for (int rr = 0; rr < ROWS; ++rr)
    core::stage_twiddles_async<M2>(twl[rr], twg, (u64)(N1 + row0 + rr), threadIdx.x, 32 * W_ROW_WARPS);
  core::cp_async_wait_all();
  __syncthreads();
#pragma unroll 1
  for (int t = 0; t < count; ++t) {
    if (t + 1 < count) {
      const uint2* in = row_ptr(t + 1);
#pragma unroll
      for (int k = 0; k < 8; ++k) vn[k] = in[core::first_idx<M2>(l, k)];
    }
    core::fwd_sub2<M2>(v, buf, l, twl[rl], q0, q1);
    if (TILED) {
      int jfirst, digit, D;
      dm.locate(p0 + first + t, job, jfirst, digit, D);
      uint2* o = dtt + (size_t)jfirst * 2 * N + (size_t)pair * N * D + (size_t)digit * 32;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int x = row * N2 + core::last_idx<M2>(l, k);
        o[(size_t)(x >> 5) * (D * 32) + (x & 31)] = reduce4(v[k], q0, q1);
      }
    } else {
      uint2* out = row_ptr(t);
#pragma unroll
      for (int k = 0; k < 8; ++k) out[core::last_idx<M2>(l, k)] = reduce4(v[k], q0, q1);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = vn[k];
    __syncwarp();  // the warp's buffer is reused by the next polynomial
  }
}

// Inverse row phase, in place on data[poly][pair][N] (polys blockIdx.z * W_ROW_POLYS .. below cnt); inputs in
// [0, 2q).
template <int M1, int M2>
__global__ __launch_bounds__(32 * W_ROW_WARPS) void k_w_rows_inv(WidePrimes w, uint2* data, int cnt) {
  using G = core::Geo<M2>;
  constexpr int N1 = 1 << M1, N2 = 1 << M2, N = N1 * N2, ROWS = W_ROW_WARPS * G::SUBS;
  __shared__ uint2 bufs[ROWS * G::STRIDE];
  __shared__ __align__(16) Tw2 twl[ROWS][N2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane / G::LANES, l = lane % G::LANES;
  const int row0 = blockIdx.x * ROWS;
  const int pair = blockIdx.y;
  const int first = blockIdx.z * W_ROW_POLYS, count = min(W_ROW_POLYS, cnt - first);
  const uint32_t q0 = pick(w.q, pair, 0), q1 = pick(w.q, pair, 1);
  const Tw2* twg = w.tw_inv + (size_t)pair * N;
  const int rl = warp * G::SUBS + sub, row = row0 + rl;
  auto row_ptr = [&](int t) { return data + (((size_t)first + t) * 2 + pair) * N + (size_t)row * N2; };
  uint2* buf = bufs + rl * G::STRIDE;
  uint2 v[8], vn[8];  // requested before the twiddle tables, so both latencies overlap
  {
    const uint2* in = row_ptr(0);
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = in[core::last_idx<M2>(l, k)];
  }
#pragma unroll 1
  for (int rr = 0; rr < ROWS; ++rr)
    core::stage_twiddles_async<M2>(twl[rr], twg, (u64)(N1 + row0 + rr), threadIdx.x, 32 * W_ROW_WARPS);
  core::cp_async_wait_all();
  __syncthreads();
#pragma unroll 1
  for (int t = 0; t < count; ++t) {
    if (t + 1 < count) {
      const uint2* in = row_ptr(t + 1);
#pragma unroll
      for (int k = 0; k < 8; ++k) vn[k] = in[core::last_idx<M2>(l, k)];
    }
    core::inv_sub2<M2>(v, buf, l, twl[rl], q0, q1);
    uint2* out = row_ptr(t);
#pragma unroll
    for (int k = 0; k < 8; ++k) out[core::first_idx<M2>(l, k)] = v[k];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = vn[k];
    __syncwarp();  // the warp's buffer is reused by the next polynomial
  }
}

// Inverse column phase, in place, times N^-1 (folded into the last stage, InvScale2): outputs in [0, q).
template <int M1, int M2>
__global__ __launch_bounds__(256, 3) void k_w_cols_inv(WidePrimes w, uint2* data) {
  using G = core::Geo<M1>;
  constexpr int COLS = WColTile<M1>::COLS, N1 = 1 << M1, N2 = 1 << M2, N = N1 * N2;
  __shared__ uint2 tile[COLS * G::STRIDE];
  __shared__ __align__(16) Tw2 twl[N1];
  const int c0 = blockIdx.x * COLS;
  const int pair = blockIdx.y;
  const size_t poly = blockIdx.z;
  const uint32_t q0 = pick(w.q, pair, 0), q1 = pick(w.q, pair, 1);
  const InvScale2 sc{pick(w.n_inv, pair, 0), pick(w.n_inv_s, pair, 0), pick(w.w1n, pair, 0), pick(w.w1n_s, pair, 0),
                     pick(w.n_inv, pair, 1), pick(w.n_inv_s, pair, 1), pick(w.w1n, pair, 1), pick(w.w1n_s, pair, 1)};
  // thread t copies column t mod COLS of rows it R + t / COLS from one per-thread base (as in k_cols_f)
  constexpr int R = 256 / COLS, ROUNDS = N1 * COLS / 256;
  static_assert(R * COLS == 256, "tile rounds");
  const int r0 = threadIdx.x / COLS, cc = threadIdx.x % COLS;
  uint2* tc = tile + cc * G::STRIDE;
  uint2* io = data + (poly * 2 + pair) * N + (size_t)r0 * N2 + c0 + cc;
#pragma unroll
  for (int it = 0; it < ROUNDS; ++it)
    core::cp_async8(tc + it * R + (r0 ^ core::swz_h<M1>((it * R) >> 4)), io + (size_t)it * R * N2);
  core::stage_twiddles_async<M1>(twl, w.tw_inv + (size_t)pair * N, 1, threadIdx.x, 256);
  core::cp_async_wait_all();
  __syncthreads();
  const int warp = threadIdx.x >> 5;
#pragma unroll 1
  for (int cb = warp * G::SUBS; cb < COLS; cb += 8 * G::SUBS) {
    const int lv = core::lane_id_volatile();
    const int sub = lv / G::LANES, l = lv % G::LANES;
    uint2* buf = tile + (cb + sub) * G::STRIDE;
    uint2 v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = buf[core::swz<M1>(core::last_idx<M1>(l, k))];
    __syncwarp();
    core::inv_sub2<M1, true>(v, buf, l, twl, q0, q1, sc);
#pragma unroll
    for (int k = 0; k < 8; ++k) buf[core::swz<M1>(core::first_idx<M1>(l, k))] = v[k];
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < ROUNDS; ++it) io[(size_t)it * R * N2] = tc[it * R + (r0 ^ core::swz_h<M1>((it * R) >> 4))];
}

// acc[b][c][j][pair][x] = sum_i DT[b][pair][x][i] * KW[j][pair][x][i][c] for
// BC jobs sharing a key.  CTA = one 32-position tile x one pair x up to BC
// jobs: the jobs' digit transforms for the tile sit in shared memory, each warp
// sweeps limbs j and streams the key tile (one contiguous run per limb and
// pair) once for all BC jobs, the next digit's key words loaded ahead.  Terms
// are < 2^58, so 64 of them fit a 64-bit sum; longer sums (FOLD, D > 64) are
// folded every 64 terms.
constexpr int W_PF = 8;  // digits of key words in flight per warp (asynchronous copies into a ring)

__device__ __forceinline__ void cp_async8(uint32_t dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// 8 bytes from global address g + OFF to shared address s + OFF: the offset is an immediate of the instruction,
// so copies at constant distances from one base need no address arithmetic of their own
template <int OFF>
__device__ __forceinline__ void cp_async8_at(uint32_t s, const void* g) {
  asm volatile("cp.async.ca.shared.global [%0+%2], [%1+%2], 8;" ::"r"(s), "l"(g), "n"(OFF) : "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Set by a key-product CTA whose bulk copies did not complete within the wait limit (read and cleared by
// rc_kernel_errors).  The decision is taken for the whole CTA at once: no thread of such a CTA computes or
// writes its outputs, so every result of the launch (and of whatever consumed it) must be discarded.
__device__ int g_wide_errors = 0;

// polls of the drain wait after a timed-out first wait: long enough for any copy to land
constexpr uint32_t W_DRAIN_POLLS = 1u << 22;

// Waits for phase `parity` of the mbarrier at shared address bar, at most `polls` polls; false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, uint32_t polls) {
  for (uint32_t it = 0; it < polls; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Hoisted rotations: the digit transforms of sigma_g(d) are those of d permuted, NTT(sigma_g d) at evaluation
// index k = NTT(d) at k' with 2k'+1 = g (2k+1) mod 2N.  In the bit-reversed storage order the 32 positions of
// one tile all come from one source tile, permuted among its lanes (the top five bits of k' depend on the
// lane, the rest on the tile only): src(x) = bitrev(k'(bitrev(x))).
__device__ __forceinline__ uint32_t galois_source(uint32_t x, uint32_t g, int log_n) {
  const uint32_t k = __brev(x) >> (32 - log_n);
  const uint32_t mask2 = (2u << log_n) - 1;  // mod 2N
  const uint32_t kk = (((g * (2 * k + 1)) & mask2) - 1) >> 1;
  return __brev(kk) >> (32 - log_n);
}

// One limb j of the key product for up to BC jobs whose digit transforms sit in shared memory at dsm
// ([BC][D][32], job b at b * run): the warp streams limb j's key words of tile xb under pair `pair` through its
// ring (this lane's slots at ring / shared address rs) and writes the nloc jobs' sums, job b's products from
// limb polynomial acc_first(bstart + b) on.
template <int BC, bool FOLD, class KT>
__device__ __forceinline__ void w_mac_unit(const KT& kt, const uint2* __restrict__ kwt, const uint2* dsm, int run,
                                           uint2* ring, uint32_t rs, int D, int key_digits, int total, int j,
                                           int pair, int xb, int log_n, int slane, int bstart, int nloc,
                                           uint32_t q0, uint32_t q1, u64 bar0, u64 bar1, uint32_t qn0, uint32_t qn1,
                                           uint32_t kq0, uint32_t kq1, uint2* acc) {
  const int lane = threadIdx.x & 31, N = 1 << log_n, tiles = N >> 5;
  const size_t krun = (size_t)key_digits * 2 * 32;
  const uint2* kp = kwt + (((size_t)j * 2 + pair) * tiles + xb) * krun + lane;
  u64 a0[BC], a1[BC], c0[BC], c1[BC];
#pragma unroll
  for (int b = 0; b < BC; ++b) a0[b] = a1[b] = c0[b] = c1[b] = 0;
  // this lane's digit word of job b at the current group's first digit, advanced once per group of W_PF digits,
  // so that the loads inside a group take compile-time offsets (no per-job address arithmetic per digit)
  const uint2* dj[BC];
#pragma unroll
  for (int b = 0; b < BC; ++b) dj[b] = dsm + (size_t)b * run + slane;
  // each lane copies and later reads only its own words, so the waits need no warp barrier
#pragma unroll
  for (int u = 0; u < W_PF; ++u) {
    if (u < D) {
      cp_async8(rs + 8u * (64 * u), kp + (size_t)u * 64);
      cp_async8(rs + 8u * (64 * u + 32), kp + (size_t)u * 64 + 32);
    }
    cp_async_commit();
  }
  const uint2* kn = kp + (size_t)W_PF * 64;  // the key words of the digit W_PF past the group's first
#pragma unroll 1
  for (int i0 = 0; i0 < D; i0 += W_PF) {
    if (FOLD && i0 > 0 && (i0 & 63) == 0) {  // fold: the next 64 terms then stay below 2^64
#pragma unroll
      for (int b = 0; b < BC; ++b) {
        a0[b] = reduce64_32(a0[b], q0, bar0);
        a1[b] = reduce64_32(a1[b], q1, bar1);
        c0[b] = reduce64_32(c0[b], q0, bar0);
        c1[b] = reduce64_32(c1[b], q1, bar1);
      }
    }
#pragma unroll
    for (int u = 0; u < W_PF; ++u) {
      const int i = i0 + u;
      if (i < D) {
        cp_async_wait<W_PF - 1>();  // digit i's group has landed
        const uint2 k0 = ring[64 * u], k1 = ring[64 * u + 32];
#pragma unroll
        for (int b = 0; b < BC; ++b) {
          const uint2 d = dj[b][32 * u];
          a0[b] += (u64)d.x * k0.x;
          a1[b] += (u64)d.y * k0.y;
          c0[b] += (u64)d.x * k1.x;
          c1[b] += (u64)d.y * k1.y;
        }
        // refill the slot with digit i + W_PF once its words have been used: words k0 and k1 of slot u sit
        // 512 u and 512 u + 256 bytes past rs, and digit i + W_PF's words the same distances past kn (the
        // switch on the unrolled, hence constant, u selects one pair of immediate-offset copies)
        if (i + W_PF < D) {
          static_assert(W_PF == 8, "one case per ring slot");
          switch (u) {
#define RC_REFILL(U)                          \
  case U:                                     \
    cp_async8_at<512 * U>(rs, kn);            \
    cp_async8_at<512 * U + 256>(rs, kn);      \
    break;
            RC_REFILL(0) RC_REFILL(1) RC_REFILL(2) RC_REFILL(3) RC_REFILL(4) RC_REFILL(5) RC_REFILL(6) RC_REFILL(7)
#undef RC_REFILL
          }
        }
        cp_async_commit();
      }
    }
#pragma unroll
    for (int b = 0; b < BC; ++b) dj[b] += 32 * W_PF;
    kn += (size_t)W_PF * 64;
  }
  cp_async_wait<0>();
  const int x = xb * 32 + lane;
#pragma unroll
  for (int b = 0; b < BC; ++b) {
    if (b < nloc) {
      const size_t ab = kt.acc_first(bstart + b, total);
      // the sums times 2^-32 (Montgomery), taken out by the inverse transform's scale (WidePrimes::n_inv)
      acc[((ab + j) * 2 + pair) * N + x] =
          make_uint2(mont64_32(a0[b], q0, qn0, kq0), mont64_32(a1[b], q1, qn1, kq1));
      acc[((ab + total + j) * 2 + pair) * N + x] =
          make_uint2(mont64_32(c0[b], q0, qn0, kq0), mont64_32(c1[b], q1, qn1, kq1));
    }
  }
}

// Job tables of the key product.  A CTA (blockIdx.x) covers up to BC consecutive jobs that share one key;
// cta() gives that key (tiled wide form, digits used and stored, limbs + K) and the jobs; dt_first(job) is
// where the job's digit transforms start (in uint2 words), acc_first(job, total) where its products start
// (in [pair][N] limb polynomials).  UniMac: nb jobs from b0 sharing one key, D digits each; MlMac: CTA x
// covers jobs [ch_first[x], + ch_n[x]) of key ch_key[x], jobs laid out by the mixed-level table.
struct UniMac {
  const uint2* kwt;
  int D, key_digits, total, b0, nb;
  template <int BC>
  __device__ __forceinline__ void cta(int x, const uint2*& k, int& d, int& kd, int& tot, int& bstart,
                                      int& nloc) const {
    k = kwt, d = D, kd = key_digits, tot = total;
    bstart = b0 + x * BC;
    nloc = min(BC, b0 + nb - bstart);
  }
  __device__ __forceinline__ size_t dt_first(int job, int N) const { return (size_t)job * 2 * N * D; }
  __device__ __forceinline__ size_t acc_first(int job, int tot) const { return (size_t)job * 2 * tot; }
};
struct MlMac {
  MlKeys keys;
  int dig[ML_MAXJ + 1], acc[ML_MAXJ + 1];
  unsigned char ch_key[ML_MAXJ], ch_n[ML_MAXJ];
  short ch_first[ML_MAXJ];
  template <int BC>
  __device__ __forceinline__ void cta(int x, const uint2*& k, int& d, int& kd, int& tot, int& bstart,
                                      int& nloc) const {
    const MlKey& key = keys.k[ch_key[x]];
    k = key.kwt, d = key.D, kd = key.key_digits, tot = key.total;
    bstart = ch_first[x];
    nloc = ch_n[x];
  }
  __device__ __forceinline__ size_t dt_first(int job, int N) const { return (size_t)dig[job] * 2 * N; }
  __device__ __forceinline__ size_t acc_first(int job, int) const { return (size_t)acc[job]; }
};

template <int BC, bool FOLD, class KT>
__global__ __launch_bounds__(32 * w_mac_warps<BC>(), BC >= 8 ? 2 : (BC >= 4 ? 3 : (BC >= 2 ? 4 : 3))) void k_w_mac(
    WidePrimes w, KT kt, const uint2* __restrict__ dtt, uint2* acc, uint32_t gal) {
  extern __shared__ __align__(128) uint2 dsm[];  // [BC][D][32] digit transforms, then [warps][W_PF][2][32] key ring
  const int N = 1 << w.log_n, tiles = N >> 5;
  // job groups vary fastest, so the CTAs that stream the same key tile run together and share it in L2
  const int pair = blockIdx.y, xb = blockIdx.z;
  const uint2* key;
  int D, key_digits, total, bstart, nloc;
  kt.template cta<BC>(blockIdx.x, key, D, key_digits, total, bstart, nloc);
  const uint2* __restrict__ kwt = key;
  const int run = D * 32;
  // gal > 1: the digits are those of sigma_gal of the decomposed polynomial (one source tile, lanes permuted)
  const uint32_t src0 = gal > 1 ? galois_source((uint32_t)xb * 32, gal, w.log_n) : (uint32_t)xb * 32;
  const int stile = (int)(src0 >> 5);
  const int slane = gal > 1 ? (int)(galois_source((uint32_t)xb * 32 + (threadIdx.x & 31), gal, w.log_n) & 31)
                            : (int)(threadIdx.x & 31);
  // the jobs' digit-transform runs (D * 256 bytes each, contiguous, 256-byte aligned) go to shared memory as
  // one bulk copy per job through the tensor memory accelerator, completing on an mbarrier; jobs past nloc
  // read as zero.  The wait is bounded: on timeout the kernel records it in g_wide_errors and returns.
  {
    __shared__ __align__(8) uint64_t mbar;
    const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&mbar);
    const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(dsm);
    const uint32_t run_bytes = (uint32_t)run * 8u;
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int e = nloc * run + threadIdx.x; e < BC * run; e += 32 * w_mac_warps<BC>()) dsm[e] = make_uint2(0, 0);
    __syncthreads();
    if (threadIdx.x == 0) {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(run_bytes * (uint32_t)nloc)
                   : "memory");
      for (int b = 0; b < nloc; ++b) {
        const uint2* src = dtt + kt.dt_first(bstart + b, N) + ((size_t)pair * tiles + stile) * run;
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                sbase + (uint32_t)b * run_bytes),
            "l"(src), "r"(run_bytes), "r"(bar)
            : "memory");
      }
    }
    // one decision for the whole CTA: either every thread saw the copies land, or none computes
    if (!__syncthreads_and(mbar_wait_bounded(bar, 0, w.first_wait_polls))) {
      if (threadIdx.x == 0) atomicOr(&g_wide_errors, 1);
      // drain: the bulk copies still in flight target this CTA's shared memory, so wait for them (again
      // bounded) before the CTA exits and the shared memory passes to another CTA
      __syncthreads_and(mbar_wait_bounded(bar, 0, W_DRAIN_POLLS));
      return;
    }
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t q0 = pick(w.q, pair, 0), q1 = pick(w.q, pair, 1);
  const u64 bar0 = pick(w.bar, pair, 0), bar1 = pick(w.bar, pair, 1);
  const uint32_t qn0 = pick(w.qinv_neg, pair, 0), qn1 = pick(w.qinv_neg, pair, 1);
  const uint32_t kq0 = pick(w.kq, pair, 0), kq1 = pick(w.kq, pair, 1);
  // this lane's slots of the warp's key ring: slot u holds (k0, k1) of one digit at ring[u][0|1][lane]
  uint2* ring = dsm + (size_t)BC * run + (size_t)warp * W_PF * 64 + lane;
  const uint32_t rs = (uint32_t)__cvta_generic_to_shared(ring);
#pragma unroll 1
  for (int j = warp; j < total; j += w_mac_warps<BC>())
    w_mac_unit<BC, FOLD>(kt, kwt, dsm, run, ring, rs, D, key_digits, total, j, pair, xb, w.log_n, slane, bstart,
                         nloc, q0, q1, bar0, bar1, qn0, qn1, kq0, kq1, acc);
}

// D: the largest digit count of the launch (sizes the shared memory); ctas: grid.x
template <int BC, bool FOLD, class KT>
void launch_w_mac(const WidePrimes& w, const KT& kt, int D, int ctas, const uint2* dtt, uint2* acc, uint32_t gal,
                  cudaStream_t s) {
  const size_t smem = ((size_t)BC * D * 32 + (size_t)w_mac_warps<BC>() * W_PF * 64) * sizeof(uint2);
  // the opt-in limit is set once per instance, before any launch of it (callers on several host threads)
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0, optin = 48 * 1024;
    if (cudaGetDevice(&dev) == cudaSuccess)
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, k_w_mac<BC, FOLD, KT>);  // the static part (the mbarrier) counts against the limit
    cudaFuncSetAttribute(k_w_mac<BC, FOLD, KT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         optin - (int)fa.sharedSizeBytes);
  });
  dim3 g(ctas, 2, (1 << w.log_n) / 32);
  k_w_mac<BC, FOLD, KT><<<g, 32 * w_mac_warps<BC>(), smem, s>>>(w, kt, dtt, acc, gal);
}

template <int BC, bool FOLD>
void launch_w_mac_uni(const WidePrimes& w, int D, int key_digits, int total, const uint2* kwt, const uint2* dtt,
                      uint2* acc, int b0, int nb, uint32_t gal, cudaStream_t s) {
  const UniMac kt{kwt, D, key_digits, total, b0, nb};
  launch_w_mac<BC, FOLD>(w, kt, D, (nb + BC - 1) / BC, dtt, acc, gal, s);
}

// Persistent form of the key product for a uniform batch (BC jobs per tile, sums of at most 64 terms): one
// CTA of WP_WARPS warps per SM walks the tiles blockIdx.x, + gridDim.x, ... (a tile = one job group x one pair
// x 32 positions; job groups vary fastest, so the CTAs streaming the same key tile run side by side and share
// it in L2).  The (tile, limb) units of the CTA's tiles are taken in order from a shared counter, so no warp
// waits at a tile's end for another warp's last limb; the digit tiles are double-buffered: the last unit of
// tile i to finish starts the bulk copy of tile i + 2 into the buffer tile i used.  Every wait is bounded; a
// wait that runs out records g_wide_errors and stops the CTA, which still waits (bounded) for its copies in
// flight before it exits.
constexpr int WP_WARPS = 16;

struct WPersist {
  uint64_t full[2];  // per buffer: completes when a tile's bulk copies have landed
  int next;          // next unit to take
  int done[2];       // units of the buffer's current tile finished
  int tile_in[2];    // local tile whose copies were last issued into the buffer (-1: none)
  int abort;
};

template <int BC>
__global__ __launch_bounds__(32 * WP_WARPS, 1) void k_w_mac_p(WidePrimes w, UniMac kt, const uint2* __restrict__ dtt,
                                                              uint2* acc, uint32_t gal, int groups) {
  extern __shared__ __align__(128) uint2 dsm[];  // [2][BC][D][32] digit tiles, then [warps][W_PF][2][32] key ring
  __shared__ WPersist st;
  const int N = 1 << w.log_n, tiles = N >> 5;
  const int D = kt.D, total = kt.total, run = D * 32;
  const int ntiles = groups * 2 * tiles;
  const int count = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  const int units = count * total;
  const uint32_t full0 = (uint32_t)__cvta_generic_to_shared(&st.full[0]);
  const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(dsm);
  const uint32_t run_bytes = (uint32_t)run * 8u, tile_bytes = (uint32_t)BC * run_bytes;
  auto tile_of = [&](int i, int& g, int& pair, int& xb) {
    int t = (int)blockIdx.x + i * (int)gridDim.x;
    g = t % groups;
    t /= groups;
    pair = t & 1;
    xb = t >> 1;
  };
  // one thread: the bulk copies of local tile i's digit transforms into buffer i & 1
  auto issue = [&](int i) {
    int g, pair, xb;
    tile_of(i, g, pair, xb);
    const int bstart = kt.b0 + g * BC, nloc = min(BC, kt.b0 + kt.nb - bstart);
    const uint32_t src0 = gal > 1 ? galois_source((uint32_t)xb * 32, gal, w.log_n) : (uint32_t)xb * 32;
    const int stile = (int)(src0 >> 5);
    const uint32_t bar = full0 + 8u * (uint32_t)(i & 1);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(run_bytes * (uint32_t)nloc)
                 : "memory");
    for (int b = 0; b < nloc; ++b) {
      const uint2* src = dtt + kt.dt_first(bstart + b, N) + ((size_t)pair * tiles + stile) * run;
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
              sbase + (uint32_t)(i & 1) * tile_bytes + (uint32_t)b * run_bytes),
          "l"(src), "r"(run_bytes), "r"(bar)
          : "memory");
    }
    atomicExch(&st.tile_in[i & 1], i);
  };
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(full0) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(full0 + 8u) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    st.next = 0;
    st.done[0] = st.done[1] = 0;
    st.tile_in[0] = st.tile_in[1] = -1;
    st.abort = 0;
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int i = 0; i < 2 && i < count; ++i) issue(i);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint2* ring = dsm + 2 * (size_t)BC * run + (size_t)warp * W_PF * 64 + lane;
  const uint32_t rs = (uint32_t)__cvta_generic_to_shared(ring);
  volatile int* vst = &st.abort;
  volatile int* vtile = st.tile_in;
#pragma unroll 1
  for (;;) {
    int u = 0;
    if (lane == 0) u = atomicAdd(&st.next, 1);
    u = __shfl_sync(0xffffffffu, u, 0);
    if (u >= units || *vst) break;
    const int i = u / total, j = u - i * total, buf = i & 1;
    // the buffer's mbarrier phase parity names tile i only once tile i's copies have been issued into it
    bool ok = true;
    for (uint32_t it = 0; vtile[buf] != i; ++it)
      if (*vst || it >= w.first_wait_polls) {
        ok = false;
        break;
      }
    ok = __all_sync(0xffffffffu, ok && mbar_wait_bounded(full0 + 8u * (uint32_t)buf, (uint32_t)(i >> 1) & 1u,
                                                         w.first_wait_polls));
    if (!ok) {
      if (lane == 0) {
        atomicOr(&g_wide_errors, 1);
        atomicExch(&st.abort, 1);
      }
      break;
    }
    int g, pair, xb;
    tile_of(i, g, pair, xb);
    const int bstart = kt.b0 + g * BC, nloc = min(BC, kt.b0 + kt.nb - bstart);
    const int slane = gal > 1 ? (int)(galois_source((uint32_t)xb * 32 + (uint32_t)lane, gal, w.log_n) & 31) : lane;
    w_mac_unit<BC, false>(kt, kt.kwt, dsm + (size_t)buf * BC * run, run, ring, rs, D, kt.key_digits, total, j, pair,
                          xb, w.log_n, slane, bstart, nloc, pick(w.q, pair, 0), pick(w.q, pair, 1),
                          pick(w.bar, pair, 0), pick(w.bar, pair, 1), pick(w.qinv_neg, pair, 0),
                          pick(w.qinv_neg, pair, 1), pick(w.kq, pair, 0), pick(w.kq, pair, 1), acc);
    // every lane's reads of the buffer are done (ordered by the warp barrier and the fence) before the unit
    // counts; the tile's last unit hands the buffer to the bulk copies of tile i + 2
    __syncwarp();
    if (lane == 0) {
      __threadfence_block();
      if (atomicAdd(&st.done[buf], 1) == total - 1) {
        __threadfence_block();
        atomicExch(&st.done[buf], 0);
        if (i + 2 < count && !*vst) {
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          issue(i + 2);
        }
      }
    }
  }
  __syncthreads();
  // drain: the copies last issued into each buffer have landed before the shared memory is released
  if (threadIdx.x == 0)
    for (int b = 0; b < 2; ++b)
      if (st.tile_in[b] >= 0 &&
          !mbar_wait_bounded(full0 + 8u * (uint32_t)b, (uint32_t)(st.tile_in[b] >> 1) & 1u, W_DRAIN_POLLS))
        atomicOr(&g_wide_errors, 1);
}

// Launches the persistent key product when its two digit tiles and the rings fit the shared memory of one
// CTA; false (nothing launched) otherwise.
template <int BC>
bool launch_w_mac_persistent(const WidePrimes& w, int D, int key_digits, int total, const uint2* kwt,
                             const uint2* dtt, uint2* acc, int b0, int nb, uint32_t gal, cudaStream_t s) {
  struct Limits {
    int smem = 0, sms = 0;
  };
  static Limits lim;
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0, optin = 48 * 1024, sms = 1;
    if (cudaGetDevice(&dev) == cudaSuccess) {
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    }
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, k_w_mac_p<BC>);
    lim.smem = optin - (int)fa.sharedSizeBytes;
    lim.sms = sms;
    cudaFuncSetAttribute(k_w_mac_p<BC>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim.smem);
  });
  const size_t smem = (2 * (size_t)BC * D * 32 + (size_t)WP_WARPS * W_PF * 64) * sizeof(uint2);
  if (D > 64 || smem > (size_t)lim.smem) return false;
  const int groups = (nb + BC - 1) / BC;
  const int ntiles = groups * 2 * ((1 << w.log_n) / 32);
  const int grid = ntiles < lim.sms ? ntiles : lim.sms;
  const UniMac kt{kwt, D, key_digits, total, b0, nb};
  k_w_mac_p<BC><<<grid, 32 * WP_WARPS, smem, s>>>(w, kt, dtt, acc, gal, groups);
  return true;
}

// coefficient-form key [digits][2][limbs][N] -> kw[((j * digits + i) * 2 + c)][pair][N]
__global__ void k_w_key_prep(WidePrimes w, const u64* src, uint2* dst, int digits, int limbs) {
  const u64 N = 1ull << w.log_n;
  const size_t total = (size_t)digits * 2 * limbs * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const u64 x = e & (N - 1);
    size_t r = e >> w.log_n;
    const int j = (int)(r % limbs);
    r /= limbs;
    const int c = (int)(r % 2);
    const int i = (int)(r / 2);
    const u64 v = src[e];
    const size_t poly = ((size_t)j * digits + i) * 2 + c;
#pragma unroll
    for (int p = 0; p < 2; ++p)
      dst[(poly * 2 + p) * N + x] =
          make_uint2(reduce64_32(v, w.q[2 * p], w.bar[2 * p]), reduce64_32(v, w.q[2 * p + 1], w.bar[2 * p + 1]));
  }
}

// transformed kw[((j * digits + i) * 2 + c)][pair][N] -> kwt[j][pair][x/32][i][c][32]
__global__ void k_w_key_tile(const uint2* src, uint2* dst, int digits, int limbs, int log_n) {
  const size_t N = (size_t)1 << log_n;
  const size_t total = (size_t)limbs * 2 * digits * 2 * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const size_t lanei = e & 31;
    size_t r = e >> 5;
    const int c = (int)(r % 2);
    r /= 2;
    const int i = (int)(r % digits);
    r /= digits;
    const size_t xb = r % (N >> 5);
    r /= (N >> 5);
    const int p = (int)(r % 2);
    const int j = (int)(r / 2);
    dst[e] = src[((((size_t)j * digits + i) * 2 + c) * 2 + p) * N + xb * 32 + lanei];
  }
}

int grid_for_elems(size_t total) {
  size_t g = (total + 255) / 256;
  return (int)(g > 65535 * 8 ? 65535 * 8 : g);
}

// forward transforms of polys [p0, p0 + count) of data[poly][pair][N]; SRC as in k_w_cols_fwd, DM as in
// k_w_rows_fwd
template <int M1, int M2, int SRC, bool TILED, class DM>
void w_forward(const WidePrimes& w, const void* src, uint2* work, uint2* dtt, int polys, const DM& dm,
               cudaStream_t s) {
  constexpr int N1 = 1 << M1, N2 = 1 << M2;
  // N = 2^16: the 16-residue passes (nttr16.cuh) on 16-byte aligned buffers
  const bool n16 = M1 == 8 && M2 == 8 && r16::aligned(src) && r16::aligned(work) && (!TILED || r16::aligned(dtt));
  const bool cols16 = n16 && (w.r16 & r16::R16_WCOLS), rows16 = n16 && (w.r16 & r16::R16_WROWS);
  for (int p0 = 0; p0 < polys; p0 += 65535) {
    const int cnt = polys - p0 < 65535 ? polys - p0 : 65535;
    if (cols16) {
      const int nt = 16 * 2 * cnt;
      r16::smem_optin<k16_w_cols_fwd<SRC>, r16::COL_SMEM>();
      k16_w_cols_fwd<SRC><<<r16::col_grid(nt), 256, r16::COL_SMEM, s>>>(w, src, work, p0, nt);
    } else {
      k_w_cols_fwd<M1, M2, SRC><<<dim3(N2 / WColTile<M1>::COLS, 2, cnt), 256, 0, s>>>(w, src, work, p0);
    }
    if (rows16) {
      k16_w_rows_fwd<TILED, DM, W_ROW_POLYS>
          <<<dim3(256 / (2 * r16::RW), 2, (cnt + W_ROW_POLYS - 1) / W_ROW_POLYS), 32 * r16::RW, 0, s>>>(w, work, dtt, p0,
                                                                                                     cnt, dm);
    } else {
      k_w_rows_fwd<M1, M2, TILED, DM><<<dim3(N1 / (W_ROW_WARPS * core::Geo<M2>::SUBS), 2,
                                             (cnt + W_ROW_POLYS - 1) / W_ROW_POLYS),
                                        32 * W_ROW_WARPS, 0, s>>>(w, work, dtt, p0, cnt, dm);
    }
  }
}

template <int SRC, bool TILED, class DM>
bool w_forward_dispatch(const WidePrimes& w, const void* src, uint2* work, uint2* dtt, int polys, const DM& dm,
                        cudaStream_t s) {
  switch (w.log_n) {
    case 12: w_forward<6, 6, SRC, TILED>(w, src, work, dtt, polys, dm, s); return true;
    case 13: w_forward<6, 7, SRC, TILED>(w, src, work, dtt, polys, dm, s); return true;
    case 14: w_forward<7, 7, SRC, TILED>(w, src, work, dtt, polys, dm, s); return true;
    case 15: w_forward<7, 8, SRC, TILED>(w, src, work, dtt, polys, dm, s); return true;
    case 16: w_forward<8, 8, SRC, TILED>(w, src, work, dtt, polys, dm, s); return true;
    default: return false;
  }
}

template <int M1, int M2>
void w_inverse(const WidePrimes& w, uint2* data, int polys, cudaStream_t s) {
  constexpr int N1 = 1 << M1, N2 = 1 << M2;
  for (int p0 = 0; p0 < polys; p0 += 65535) {
    const int cnt = polys - p0 < 65535 ? polys - p0 : 65535;
    uint2* d = data + (size_t)p0 * 2 * (N1 * N2);
    // N = 2^16: the 16-residue passes (nttr16.cuh) where their bits of WidePrimes::r16 are set
    const bool n16 = M1 == 8 && M2 == 8 && r16::aligned(d);
    if (n16 && (w.r16 & r16::R16_WROWS)) {
      ProfScope p("wide_inv_rows", s);
      k16_w_rows_inv<W_ROW_POLYS>
          <<<dim3(256 / (2 * r16::RW), 2, (cnt + W_ROW_POLYS - 1) / W_ROW_POLYS), 32 * r16::RW, 0, s>>>(w, d, cnt);
    } else {
      ProfScope p("wide_inv_rows", s);
      k_w_rows_inv<M1, M2><<<dim3(N1 / (W_ROW_WARPS * core::Geo<M2>::SUBS), 2,
                                  (cnt + W_ROW_POLYS - 1) / W_ROW_POLYS),
                             32 * W_ROW_WARPS, 0, s>>>(w, d, cnt);
    }
    if (n16 && (w.r16 & r16::R16_WCOLS)) {
      const int nt = 16 * 2 * cnt;
      r16::smem_optin<k16_w_cols_inv<>, r16::COL_SMEM>();
      ProfScope p("wide_inv_cols", s);
      k16_w_cols_inv<><<<r16::col_grid(nt), 256, r16::COL_SMEM, s>>>(w, d, nt);
    } else {
      ProfScope p("wide_inv_cols", s);
      k_w_cols_inv<M1, M2><<<dim3(N2 / WColTile<M1>::COLS, 2, cnt), 256, 0, s>>>(w, d);
    }
  }
}

}  // namespace

bool wide_digit_transforms(const WidePrimes& w, int D, int jobs, const int32_t* digits, uint2* work, uint2* dtt,
                           cudaStream_t s) {
  ProfScope p("wide_digit_ntt", s);
  return w_forward_dispatch<0, true>(w, digits, work, dtt, jobs * D, UniDig{D}, s);
}

bool wide_digit_transforms_ml(const WidePrimes& w, const MlTab& t, const int32_t* digits, uint2* work, uint2* dtt,
                              cudaStream_t s) {
  if (t.J <= 0) return true;
  ProfScope p("wide_digit_ntt", s);
  MlDig dm;
  dm.J = t.J;
  for (int j = 0; j <= t.J; ++j) dm.dig[j] = t.dig[j];
  return w_forward_dispatch<0, true>(w, digits, work, dtt, t.dig[t.J], dm, s);
}

void wide_mac(const WidePrimes& w, int D, int key_digits, int total, const uint2* kwt, const uint2* dtt, uint2* acc,
              int b0, int nb, int bc_max, cudaStream_t s, uint32_t gal) {
  ProfScope p("wide_mac", s);
  const int want = nb < bc_max ? nb : bc_max;  // jobs per CTA: the group size, at most bc_max
  if (D > 64) {  // folded sums; at most 4 jobs per CTA keep the fold within the register budget
    if (want <= 1) launch_w_mac_uni<1, true>(w, D, key_digits, total, kwt, dtt, acc, b0, nb, gal, s);
    else if (want <= 2) launch_w_mac_uni<2, true>(w, D, key_digits, total, kwt, dtt, acc, b0, nb, gal, s);
    else launch_w_mac_uni<4, true>(w, D, key_digits, total, kwt, dtt, acc, b0, nb, gal, s);
    return;
  }
  if (w.persistent && want > 4 && launch_w_mac_persistent<8>(w, D, key_digits, total, kwt, dtt, acc, b0, nb, gal, s))
    return;
  if (w.persistent && want > 2 && want <= 4 &&
      launch_w_mac_persistent<4>(w, D, key_digits, total, kwt, dtt, acc, b0, nb, gal, s))
    return;
  if (want <= 1) launch_w_mac_uni<1, false>(w, D, key_digits, total, kwt, dtt, acc, b0, nb, gal, s);
  else if (want <= 2) launch_w_mac_uni<2, false>(w, D, key_digits, total, kwt, dtt, acc, b0, nb, gal, s);
  else if (want <= 4) launch_w_mac_uni<4, false>(w, D, key_digits, total, kwt, dtt, acc, b0, nb, gal, s);
  else launch_w_mac_uni<8, false>(w, D, key_digits, total, kwt, dtt, acc, b0, nb, gal, s);
}

namespace {
// CTAs of BC jobs, each within one key's consecutive jobs
template <int BC, bool FOLD>
void launch_w_mac_ml(const WidePrimes& w, const MlTab& t, const MlKeys& keys, const uint2* dtt, uint2* acc,
                     cudaStream_t s) {
  MlMac kt;
  kt.keys = keys;
  for (int j = 0; j <= t.J; ++j) kt.dig[j] = t.dig[j], kt.acc[j] = t.acc[j];
  int ctas = 0, D = 0;
  for (int k = 0; k < keys.n; ++k) {
    D = keys.k[k].D > D ? keys.k[k].D : D;
    for (int b = 0; b < keys.k[k].count; b += BC) {
      kt.ch_key[ctas] = (unsigned char)k;
      kt.ch_first[ctas] = (short)(keys.k[k].first + b);
      kt.ch_n[ctas] = (unsigned char)(keys.k[k].count - b < BC ? keys.k[k].count - b : BC);
      ++ctas;
    }
  }
  launch_w_mac<BC, FOLD>(w, kt, D, ctas, dtt, acc, 0, s);
}
}  // namespace

void wide_mac_ml(const WidePrimes& w, const MlTab& t, const MlKeys& keys, const uint2* dtt, uint2* acc, int bc_max,
                 cudaStream_t s) {
  if (t.J <= 0 || keys.n <= 0) return;
  ProfScope p("wide_mac", s);
  int most = 0, D = 0;
  for (int k = 0; k < keys.n; ++k) {
    most = keys.k[k].count > most ? keys.k[k].count : most;
    D = keys.k[k].D > D ? keys.k[k].D : D;
  }
  const int want = most < bc_max ? most : bc_max;
  if (D > 64) {
    if (want <= 1) launch_w_mac_ml<1, true>(w, t, keys, dtt, acc, s);
    else if (want <= 2) launch_w_mac_ml<2, true>(w, t, keys, dtt, acc, s);
    else launch_w_mac_ml<4, true>(w, t, keys, dtt, acc, s);
    return;
  }
  if (want <= 1) launch_w_mac_ml<1, false>(w, t, keys, dtt, acc, s);
  else if (want <= 2) launch_w_mac_ml<2, false>(w, t, keys, dtt, acc, s);
  else if (want <= 4) launch_w_mac_ml<4, false>(w, t, keys, dtt, acc, s);
  else launch_w_mac_ml<8, false>(w, t, keys, dtt, acc, s);
}

int wide_kernel_errors(bool clear) {
  int v = 0;
  // a failed read (e.g. a sticky error after a fault) is an error, never a clean flag
  cuda_check(cudaMemcpyFromSymbol(&v, g_wide_errors, sizeof(int)), "reading the key-product error flag");
  if (clear && v) {
    const int zero = 0;
    cuda_check(cudaMemcpyToSymbol(g_wide_errors, &zero, sizeof(int)), "clearing the key-product error flag");
  }
  return v;
}

bool wide_inverse(const WidePrimes& w, uint2* data, int polys, cudaStream_t s) {
  switch (w.log_n) {
    case 12: w_inverse<6, 6>(w, data, polys, s); return true;
    case 13: w_inverse<6, 7>(w, data, polys, s); return true;
    case 14: w_inverse<7, 7>(w, data, polys, s); return true;
    case 15: w_inverse<7, 8>(w, data, polys, s); return true;
    case 16: w_inverse<8, 8>(w, data, polys, s); return true;
    default: return false;
  }
}

bool wide_key_build(const WidePrimes& w, const u64* key, int digits, int limbs, uint2* tmp, uint2* kwt,
                    cudaStream_t s) {
  const size_t N = (size_t)1 << w.log_n;
  const int polys = digits * 2 * limbs;
  k_w_key_prep<<<grid_for_elems((size_t)polys * N), 256, 0, s>>>(w, key, tmp, digits, limbs);
  // forward transforms in place (the column phase reads tmp and writes tmp)
  if (!w_forward_dispatch<1, false>(w, tmp, tmp, nullptr, polys, UniDig{1}, s)) return false;
  k_w_key_tile<<<grid_for_elems((size_t)polys * 2 * N), 256, 0, s>>>(tmp, kwt, digits, limbs, w.log_n);
  return true;
}

}  // namespace rc
