// Kernel templates of the negacyclic NTT shared by the forward (ntt.cu) and inverse (ntt_inv.cu) translation
// units: the generic shared-memory passes for any ring size and the fast register-blocked column and row
// passes for log N in 12..16 with their launch-shape dispatch (four-step split, CTAs per SM of the column
// pass, polynomials per row block).
//
// Negacyclic NTT / INTT over RNS limbs, split four-step into a column phase
// and a row phase.
//
// The reference multiplies polynomials by twisting with psi^i, running a
// radix-2 cyclic NTT (bit reversal + DIT with recurrence twiddles,
// src/math/ntt.rs:92-130) and untwisting afterwards (src/poly/mod.rs:134-175).
// Here the twist is merged into the twiddles (psi^bitrev(k) tables) and the
// transform is a Cooley-Tukey pass from natural to bit-reversed order; the
// inverse is the matching Gentleman-Sande pass with psi^-bitrev(k) and N^-1.
// Evaluation at psi^(2k+1) lands at bit-reversed index k, so the
// coefficient-domain results of every product equal the reference's exactly.
//
// N = N1 * N2 (N1 = 2^n1).  Stages 0..n1-1 only pair elements in the same
// column (index mod N2), stages n1..log N-1 only pair elements in the same row
// (index div N2): the column kernel stages a tile of columns in shared memory,
// the row kernel a tile of rows.  Arithmetic is Harvey's lazy Shoup butterfly
// (values in [0, 4q) forward, [0, 2q) inverse; q < 2^61).
#pragma once
#include <type_traits>

#include "kernels.cuh"
#include "nttcore.cuh"

namespace rc {
namespace {

__host__ __device__ __forceinline__ int cols_per_cta(int n2) { return n2 < 16 ? n2 : 16; }
__host__ __device__ __forceinline__ int rows_per_cta(int n1, int n2) {
  int r = 2048 / n2;
  if (r < 1) r = 1;
  return r < n1 ? r : n1;
}


// ---------------------------------------------------------------------------
// fast path, log N in 12..16: warp-level register-blocked sub-transforms
// ---------------------------------------------------------------------------
template <int M>
struct ColTile {
  static constexpr int COLS = (8 * core::Geo<M>::SUBS) > 16 ? 8 * core::Geo<M>::SUBS : 16;
};

// x < 65q (lazy) or < 4q -> [0, q)
template <bool LAZY>
__device__ __forceinline__ u64 reduce_out(u64 x, const PrimeConst& c) {
  if (LAZY) {
    x = mul_shoup_lazy(x, 1, c.one_s, c.q);
    return x >= c.q ? x - c.q : x;
  }
  return reduce_4q(x, c.q);
}

// Column phase: the CTA stages a tile of COLS columns (2^M1 rows each) and the
// column twiddle table in shared memory; each warp transforms SUBS columns at
// a time in registers.  LAZY: forward, unreduced butterflies; inverse, butterflies without reductions
// (inputs below 2q, primes below 2^55).  Inverse: the N^-1 (or N^-1 2^64) scale is folded into the last stage
// (InvScale), whose products leave canonical outputs.
template <int M1, int M2, bool LAZY, bool FWD, int CC>
__global__ __launch_bounds__(256, CC) void k_cols_f(NttArgs a, PtrTab src, PtrTab dst, LimbMap map) {
  using G = core::Geo<M1>;
  constexpr int COLS = ColTile<M1>::COLS, N1 = 1 << M1, N2 = 1 << M2, N = N1 * N2;
  __shared__ u64 tile[COLS * G::STRIDE];
  __shared__ __align__(16) Twiddle twl[N1];
  const int c0 = blockIdx.x * COLS;
  const int limb = blockIdx.y, poly = blockIdx.z;
  const int prime = map.prime(limb);
  const PrimeConst& pc = a.pc[prime];
  const u64 q = pc.q;
  const InvScale sc = a.mont_out ? InvScale{pc.n_inv_r, pc.n_inv_r_s, pc.w1nr, pc.w1nr_s}
                                  : InvScale{pc.n_inv, pc.n_inv_s, pc.w1n, pc.w1n_s};
  // thread t copies column t mod COLS of rows it R + t / COLS (R = 256 / COLS rows per round): a per-thread
  // base plus constant offsets, the swizzled row being it R + (r0 ^ swz_h(it R / 16)) with r0 = t / COLS < R
  constexpr int R = 256 / COLS, ROUNDS = N1 * COLS / 256;
  static_assert(R * COLS == 256, "tile rounds");  // and swz_h < R: below 16 = R (M1 7, 8), at most 2 < R = 8 (M1 6)
  const int r0 = threadIdx.x / COLS, cc = threadIdx.x % COLS;
  const u64* in = src.p[poly] + (size_t)limb * N + (size_t)r0 * N2 + c0 + cc;
  u64* out = dst.p[poly] + (size_t)limb * N + (size_t)r0 * N2 + c0 + cc;
  u64* tc = tile + cc * G::STRIDE;
  // tile and twiddles by asynchronous copies, all in flight together
#pragma unroll
  for (int it = 0; it < ROUNDS; ++it)
    core::cp_async8(tc + it * R + (r0 ^ core::swz_h<M1>((it * R) >> 4)), in + (size_t)it * R * N2);
  core::stage_twiddles_async<M1>(twl, (FWD ? a.tw_fwd : a.tw_inv) + (size_t)prime * N, 1, threadIdx.x, 256);
  core::cp_async_wait_all();
  __syncthreads();
  const int warp = threadIdx.x >> 5;
#pragma unroll 1
  for (int cb = warp * G::SUBS; cb < COLS; cb += 8 * G::SUBS) {
    const int lv = core::lane_id_volatile();
    const int sub = lv / G::LANES, l = lv % G::LANES;
    u64* buf = tile + (cb + sub) * G::STRIDE;
    u64 v[8];
    if (FWD) {
#pragma unroll
      for (int k = 0; k < 8; ++k) v[k] = buf[core::swz<M1>(core::first_idx<M1>(l, k))];
      __syncwarp();
      core::fwd_sub<M1, LAZY>(v, buf, l, twl, q);
#pragma unroll
      for (int k = 0; k < 8; ++k) buf[core::swz<M1>(core::last_idx<M1>(l, k))] = v[k];
    } else {
#pragma unroll
      for (int k = 0; k < 8; ++k) v[k] = buf[core::swz<M1>(core::last_idx<M1>(l, k))];
      __syncwarp();
      core::inv_sub<M1, LAZY, true>(v, buf, l, twl, q, sc);
#pragma unroll
      for (int k = 0; k < 8; ++k) buf[core::swz<M1>(core::first_idx<M1>(l, k))] = v[k];
    }
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < ROUNDS; ++it) out[(size_t)it * R * N2] = tc[it * R + (r0 ^ core::swz_h<M1>((it * R) >> 4))];
}

constexpr int ROW_WARPS = 4;
// polynomials per row block (RP, 8 or 16, tunable "row_polys"): the same rows (and limb) of RP polynomials
// share one staging of the rows' twiddles, which take as many bytes as two rows of data

// Row phase: each warp transforms SUBS rows of 2^M2 contiguous residues of polynomials
// blockIdx.z * RP .. below `polys`, loading the next polynomial's rows while transforming the current
// one; the CTA stages the rows' twiddle tables in shared memory once.  Forward outputs in [0, q), or (RAW,
// for the tensor: NttArgs::raw_out) left below (4 log N + 1) q (LAZY) or 4q.
template <int M1, int M2, bool LAZY, bool FWD, int RP, bool RAW = false>
__global__ __launch_bounds__(32 * ROW_WARPS) void k_rows_f(NttArgs a, PtrTab src, PtrTab dst, LimbMap map,
                                                           int polys) {
  using G = core::Geo<M2>;
  constexpr int N1 = 1 << M1, N2 = 1 << M2, N = N1 * N2, ROWS = ROW_WARPS * G::SUBS;
  __shared__ u64 bufs[ROWS * G::STRIDE];
  __shared__ __align__(16) Twiddle twl[ROWS][N2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane / G::LANES, l = lane % G::LANES;
  const int row0 = blockIdx.x * ROWS;
  const int limb = blockIdx.y, first = blockIdx.z * RP, count = min(RP, polys - first);
  const int prime = map.prime(limb);
  const PrimeConst& pc = a.pc[prime];
  const Twiddle* twg = (FWD ? a.tw_fwd : a.tw_inv) + (size_t)prime * N;
  const int rl = warp * G::SUBS + sub, row = row0 + rl;
  const size_t off = (size_t)limb * N + (size_t)row * N2;
  u64* buf = bufs + rl * G::STRIDE;
  // the first polynomial's values are requested before the twiddle tables, so both latencies overlap
  u64 v[8], vn[8];
  {
    const u64* in = src.p[first] + off;
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = in[FWD ? core::first_idx<M2>(l, k) : core::last_idx<M2>(l, k)];
  }
#pragma unroll 1
  for (int rr = 0; rr < ROWS; ++rr)
    core::stage_twiddles_async<M2>(twl[rr], twg, (u64)(N1 + row0 + rr), threadIdx.x, 32 * ROW_WARPS);
  core::cp_async_wait_all();
  __syncthreads();
#pragma unroll 1
  for (int t = 0; t < count; ++t) {
    if (t + 1 < count) {
      const u64* in = src.p[first + t + 1] + off;
#pragma unroll
      for (int k = 0; k < 8; ++k) vn[k] = in[FWD ? core::first_idx<M2>(l, k) : core::last_idx<M2>(l, k)];
    }
    u64* out = dst.p[first + t] + off;
    if (FWD) {
      core::fwd_sub<M2, LAZY>(v, buf, l, twl[rl], pc.q);
#pragma unroll
      for (int k = 0; k < 8; ++k) out[core::last_idx<M2>(l, k)] = RAW ? v[k] : reduce_out<LAZY>(v[k], pc);
    } else {
      core::inv_sub<M2>(v, buf, l, twl[rl], pc.q);
#pragma unroll
      for (int k = 0; k < 8; ++k) out[core::first_idx<M2>(l, k)] = v[k];
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = vn[k];
    __syncwarp();  // the warp's buffer is reused by the next polynomial
  }
}

// the launch shapes the column and row passes take from NttArgs (tunables "col_ctas", "row_polys")

template <class F>
void with_cc(int cc, F&& f) {
  if (cc == 2) f(std::integral_constant<int, 2>{});
  else f(std::integral_constant<int, 3>{});
}
template <class F>
void with_rp(int rp, F&& f) {
  if (rp == 8) f(std::integral_constant<int, 8>{});
  else f(std::integral_constant<int, 16>{});
}


template <class F>
bool with_split(int log_n, int n1, F&& f) {
  const int n2 = log_n - n1;
#define RC_SPLIT(A, B)                                                    \
  if (n1 == A && n2 == B) {                                                \
    f(std::integral_constant<int, A>{}, std::integral_constant<int, B>{}); \
    return true;                                                           \
  }
  RC_SPLIT(6, 6)
  RC_SPLIT(6, 7)
  RC_SPLIT(7, 6)
  RC_SPLIT(6, 8)
  RC_SPLIT(7, 7)
  RC_SPLIT(8, 6)
  RC_SPLIT(7, 8)
  RC_SPLIT(8, 7)
  RC_SPLIT(8, 8)
#undef RC_SPLIT
  return false;
}


inline int threads_for(int work) {
  int t = 32;
  while (t < 256 && t < work) t <<= 1;
  return t;
}


}  // namespace
}  // namespace rc
