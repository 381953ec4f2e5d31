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

__global__ void k_fwd_cols(NttArgs a, PtrTab src, PtrTab dst, LimbMap map) {
  extern __shared__ u64 sm[];
  const int log_n = a.log_n, n1 = a.n1;
  const int N = 1 << log_n, N1 = 1 << n1, N2 = N >> n1;
  const int COLS = cols_per_cta(N2);
  const int c0 = blockIdx.x * COLS;
  const int limb = blockIdx.y, poly = blockIdx.z;
  const int prime = map.prime(limb);
  const u64 q = a.pc[prime].q, two_q = q << 1;
  const Twiddle* tw = a.tw_fwd + (size_t)prime * N;
  const u64* in = src.p[poly] + (size_t)limb * N;
  u64* out = dst.p[poly] + (size_t)limb * N;

  for (int idx = threadIdx.x; idx < N1 * COLS; idx += blockDim.x) {
    int r = idx / COLS, c = idx % COLS;
    sm[idx] = in[(size_t)r * N2 + c0 + c];
  }
  __syncthreads();
  for (int s = 0; s < n1; ++s) {
    const int t = N1 >> (s + 1);
    for (int idx = threadIdx.x; idx < (N1 / 2) * COLS; idx += blockDim.x) {
      int p = idx / COLS, c = idx % COLS;
      int r = (p / t) * 2 * t + (p % t);
      Twiddle w = tw[(1 << s) + (r >> (n1 - s))];
      u64 x = sm[r * COLS + c], y = sm[(r + t) * COLS + c];
      x = x >= two_q ? x - two_q : x;
      u64 v = mul_shoup_lazy(y, w.w, w.ws, q);
      sm[r * COLS + c] = x + v;
      sm[(r + t) * COLS + c] = x - v + two_q;
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < N1 * COLS; idx += blockDim.x) {
    int r = idx / COLS, c = idx % COLS;
    out[(size_t)r * N2 + c0 + c] = sm[idx];
  }
}

__global__ void k_fwd_rows(NttArgs a, PtrTab src, PtrTab dst, LimbMap map) {
  extern __shared__ u64 sm[];
  const int log_n = a.log_n, n1 = a.n1;
  const int N = 1 << log_n, N1 = 1 << n1, N2 = N >> n1;
  const int ROWS = rows_per_cta(N1, N2);
  const int r0 = blockIdx.x * ROWS;
  const int limb = blockIdx.y, poly = blockIdx.z;
  const int prime = map.prime(limb);
  const u64 q = a.pc[prime].q, two_q = q << 1;
  const Twiddle* tw = a.tw_fwd + (size_t)prime * N;
  const u64* in = src.p[poly] + (size_t)limb * N + (size_t)r0 * N2;
  u64* out = dst.p[poly] + (size_t)limb * N + (size_t)r0 * N2;
  const int tile = ROWS * N2;

  for (int idx = threadIdx.x; idx < tile; idx += blockDim.x) sm[idx] = in[idx];
  __syncthreads();
  const int half = N2 / 2;
  for (int s = n1; s < log_n; ++s) {
    const int t = N2 >> (s - n1 + 1);
    for (int idx = threadIdx.x; idx < tile / 2; idx += blockDim.x) {
      int rl = idx / half, p = idx % half;
      int c = (p / t) * 2 * t + (p % t);
      int j = (r0 + rl) * N2 + c;
      Twiddle w = tw[(1 << s) + (j >> (log_n - s))];
      u64* base = sm + rl * N2;
      u64 x = base[c], y = base[c + t];
      x = x >= two_q ? x - two_q : x;
      u64 v = mul_shoup_lazy(y, w.w, w.ws, q);
      base[c] = x + v;
      base[c + t] = x - v + two_q;
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < tile; idx += blockDim.x) out[idx] = reduce_4q(sm[idx], q);
}

__global__ void k_inv_rows(NttArgs a, PtrTab src, PtrTab dst, LimbMap map) {
  extern __shared__ u64 sm[];
  const int log_n = a.log_n, n1 = a.n1;
  const int N = 1 << log_n, N1 = 1 << n1, N2 = N >> n1;
  const int ROWS = rows_per_cta(N1, N2);
  const int r0 = blockIdx.x * ROWS;
  const int limb = blockIdx.y, poly = blockIdx.z;
  const int prime = map.prime(limb);
  const u64 q = a.pc[prime].q, two_q = q << 1;
  const Twiddle* tw = a.tw_inv + (size_t)prime * N;
  const u64* in = src.p[poly] + (size_t)limb * N + (size_t)r0 * N2;
  u64* out = dst.p[poly] + (size_t)limb * N + (size_t)r0 * N2;
  const int tile = ROWS * N2;

  for (int idx = threadIdx.x; idx < tile; idx += blockDim.x) sm[idx] = in[idx];
  __syncthreads();
  const int half = N2 / 2;
  for (int s = log_n - 1; s >= n1; --s) {
    const int t = N2 >> (s - n1 + 1);
    for (int idx = threadIdx.x; idx < tile / 2; idx += blockDim.x) {
      int rl = idx / half, p = idx % half;
      int c = (p / t) * 2 * t + (p % t);
      int j = (r0 + rl) * N2 + c;
      Twiddle w = tw[(1 << s) + (j >> (log_n - s))];
      u64* base = sm + rl * N2;
      u64 x = base[c], y = base[c + t];
      u64 u = x + y;
      u = u >= two_q ? u - two_q : u;
      base[c] = u;
      base[c + t] = mul_shoup_lazy(x - y + two_q, w.w, w.ws, q);
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < tile; idx += blockDim.x) out[idx] = sm[idx];
}

__global__ void k_inv_cols(NttArgs a, PtrTab src, PtrTab dst, LimbMap map) {
  extern __shared__ u64 sm[];
  const int log_n = a.log_n, n1 = a.n1;
  const int N = 1 << log_n, N1 = 1 << n1, N2 = N >> n1;
  const int COLS = cols_per_cta(N2);
  const int c0 = blockIdx.x * COLS;
  const int limb = blockIdx.y, poly = blockIdx.z;
  const int prime = map.prime(limb);
  const PrimeConst& pc = a.pc[prime];
  const u64 q = pc.q, two_q = q << 1;
  const Twiddle* tw = a.tw_inv + (size_t)prime * N;
  const u64* in = src.p[poly] + (size_t)limb * N;
  u64* out = dst.p[poly] + (size_t)limb * N;

  for (int idx = threadIdx.x; idx < N1 * COLS; idx += blockDim.x) {
    int r = idx / COLS, c = idx % COLS;
    sm[idx] = in[(size_t)r * N2 + c0 + c];
  }
  __syncthreads();
  for (int s = n1 - 1; s >= 0; --s) {
    const int t = N1 >> (s + 1);
    for (int idx = threadIdx.x; idx < (N1 / 2) * COLS; idx += blockDim.x) {
      int p = idx / COLS, c = idx % COLS;
      int r = (p / t) * 2 * t + (p % t);
      Twiddle w = tw[(1 << s) + (r >> (n1 - s))];
      u64 x = sm[r * COLS + c], y = sm[(r + t) * COLS + c];
      u64 u = x + y;
      u = u >= two_q ? u - two_q : u;
      sm[r * COLS + c] = u;
      sm[(r + t) * COLS + c] = mul_shoup_lazy(x - y + two_q, w.w, w.ws, q);
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < N1 * COLS; idx += blockDim.x) {
    int r = idx / COLS, c = idx % COLS;
    out[(size_t)r * N2 + c0 + c] =
        a.mont_out ? mul_shoup(sm[idx], pc.n_inv_r, pc.n_inv_r_s, q) : mul_shoup(sm[idx], pc.n_inv, pc.n_inv_s, q);
  }
}

// ---------------------------------------------------------------------------
// fast path, log N in 12..16: warp-level register-blocked sub-transforms
// ---------------------------------------------------------------------------
template <int M>
struct ColTile {
  static constexpr int COLS = (8 * core::Geo<M>::SUBS) > 16 ? 8 * core::Geo<M>::SUBS : 16;
};

// x < 33q (lazy) or < 4q -> [0, q)
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
// (inputs below 2q, primes below 2^55), the final N^-1 product reducing every output.
template <int M1, int M2, bool LAZY, bool FWD>
__global__ __launch_bounds__(256, 3) void k_cols_f(NttArgs a, PtrTab src, PtrTab dst, LimbMap map) {
  using G = core::Geo<M1>;
  constexpr int COLS = ColTile<M1>::COLS, N1 = 1 << M1, N2 = 1 << M2, N = N1 * N2;
  __shared__ u64 tile[COLS * G::STRIDE];
  __shared__ __align__(16) Twiddle twl[N1];
  const int c0 = blockIdx.x * COLS;
  const int limb = blockIdx.y, poly = blockIdx.z;
  const int prime = map.prime(limb);
  const PrimeConst& pc = a.pc[prime];
  const u64 q = pc.q;
  const u64 ninv = a.mont_out ? pc.n_inv_r : pc.n_inv, ninv_s = a.mont_out ? pc.n_inv_r_s : pc.n_inv_s;
  const u64* in = src.p[poly] + (size_t)limb * N;
  u64* out = dst.p[poly] + (size_t)limb * N;
  // tile and twiddles by asynchronous copies, all in flight together
#pragma unroll 4
  for (int it = 0; it < N1 * COLS / 256; ++it) {
    const int idx = it * 256 + threadIdx.x;
    const int r = idx / COLS, c = idx % COLS;
    core::cp_async8(&tile[c * G::STRIDE + core::swz<M1>(r)], &in[(size_t)r * N2 + c0 + c]);
  }
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
      core::inv_sub<M1, LAZY>(v, buf, l, twl, q);
#pragma unroll
      for (int k = 0; k < 8; ++k) buf[core::swz<M1>(core::first_idx<M1>(l, k))] = v[k];
    }
  }
  __syncthreads();
#pragma unroll 4
  for (int it = 0; it < N1 * COLS / 256; ++it) {
    const int idx = it * 256 + threadIdx.x;
    const int r = idx / COLS, c = idx % COLS;
    const u64 x = tile[c * G::STRIDE + core::swz<M1>(r)];
    out[(size_t)r * N2 + c0 + c] = FWD ? x : mul_shoup(x, ninv, ninv_s, q);
  }
}

constexpr int ROW_WARPS = 4;
// polynomials per row block: the same rows (and limb) of ROW_POLYS polynomials share one staging of the rows'
// twiddles, which take as many bytes as two rows of data
constexpr int ROW_POLYS = 16;

// Row phase: each warp transforms SUBS rows of 2^M2 contiguous residues of polynomials
// blockIdx.z * ROW_POLYS .. below `polys`, loading the next polynomial's rows while transforming the current
// one; the CTA stages the rows' twiddle tables in shared memory once.
template <int M1, int M2, bool LAZY, bool FWD>
__global__ __launch_bounds__(32 * ROW_WARPS) void k_rows_f(NttArgs a, PtrTab src, PtrTab dst, LimbMap map,
                                                           int polys) {
  using G = core::Geo<M2>;
  constexpr int N1 = 1 << M1, N2 = 1 << M2, N = N1 * N2, ROWS = ROW_WARPS * G::SUBS;
  __shared__ u64 bufs[ROWS * G::STRIDE];
  __shared__ __align__(16) Twiddle twl[ROWS][N2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane / G::LANES, l = lane % G::LANES;
  const int row0 = blockIdx.x * ROWS;
  const int limb = blockIdx.y, first = blockIdx.z * ROW_POLYS, count = min(ROW_POLYS, polys - first);
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
      for (int k = 0; k < 8; ++k) out[core::last_idx<M2>(l, k)] = reduce_out<LAZY>(v[k], pc);
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

template <int M1, int M2, bool LAZY>
void fwd_fast(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
              cudaStream_t s) {
  constexpr int N2 = 1 << M2, N1 = 1 << M1;
  dim3 g1(N2 / ColTile<M1>::COLS, limbs, polys),
      g2(N1 / (ROW_WARPS * core::Geo<M2>::SUBS), limbs, (polys + ROW_POLYS - 1) / ROW_POLYS);
  {
    ProfScope p("ntt_fwd_cols", s);
    k_cols_f<M1, M2, LAZY, true><<<g1, 256, 0, s>>>(a, src, dst, map);
  }
  {
    ProfScope p("ntt_fwd_rows", s);
    k_rows_f<M1, M2, LAZY, true><<<g2, 32 * ROW_WARPS, 0, s>>>(a, dst, dst, map, polys);
  }
}

template <int M1, int M2>
void inv_fast(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
              cudaStream_t s) {
  constexpr int N2 = 1 << M2, N1 = 1 << M1;
  dim3 g1(N2 / ColTile<M1>::COLS, limbs, polys),
      g2(N1 / (ROW_WARPS * core::Geo<M2>::SUBS), limbs, (polys + ROW_POLYS - 1) / ROW_POLYS);
  {
    ProfScope p("ntt_inv_rows", s);
    k_rows_f<M1, M2, false, false><<<g2, 32 * ROW_WARPS, 0, s>>>(a, src, dst, map, polys);
  }
  {
    ProfScope p("ntt_inv_cols", s);
    if (a.lazy_inv) k_cols_f<M1, M2, true, false><<<g1, 256, 0, s>>>(a, dst, dst, map);
    else k_cols_f<M1, M2, false, false><<<g1, 256, 0, s>>>(a, dst, dst, map);
  }
}

// The tensor and the inverse row phase in one pass: for each job of the block, d0 = a0 b0, d1 = a0 b1 + a1 b0
// and d2 = a1 b1 (Montgomery products of the forward transforms in4[4j..4j+3]; the inverse column pass's scale
// takes out their 2^-64) go straight into the inverse row transform, so the quadratic NTT-domain values never
// reach HBM.  A block transforms the same rows of TENSOR_ROW_JOBS jobs (three outputs each) with one twiddle
// staging.
constexpr int TENSOR_ROW_JOBS = 4;

template <int M1, int M2>
__global__ __launch_bounds__(32 * ROW_WARPS) void k_tensor_inv_rows(NttArgs a, PtrTab in4, PtrTab out3, LimbMap map,
                                                                    int jobs) {
  using G = core::Geo<M2>;
  constexpr int N1 = 1 << M1, N2 = 1 << M2, N = N1 * N2, ROWS = ROW_WARPS * G::SUBS;
  __shared__ u64 bufs[ROWS * G::STRIDE];
  __shared__ __align__(16) Twiddle twl[ROWS][N2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane / G::LANES, l = lane % G::LANES;
  const int row0 = blockIdx.x * ROWS;
  const int limb = blockIdx.y, first = blockIdx.z * TENSOR_ROW_JOBS, count = min(TENSOR_ROW_JOBS, jobs - first);
  const int prime = map.prime(limb);
  const PrimeConst& pc = a.pc[prime];
  const Twiddle* twg = a.tw_inv + (size_t)prime * N;
  const int rl = warp * G::SUBS + sub, row = row0 + rl;
  const size_t off = (size_t)limb * N + (size_t)row * N2;
  u64* buf = bufs + rl * G::STRIDE;
  // the first job's products are formed before the twiddle tables land, so both latencies overlap
  u64 d[3][8];
  auto products = [&](int j) {
    const u64 *x0 = in4.p[4 * j] + off, *x1 = in4.p[4 * j + 1] + off;
    const u64 *y0 = in4.p[4 * j + 2] + off, *y1 = in4.p[4 * j + 3] + off;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int x = core::last_idx<M2>(l, k);
      const u64 a0 = x0[x], a1 = x1[x], b0 = y0[x], b1 = y1[x];
      d[0][k] = mont_reduce(mul_wide(a0, b0), pc);
      U128 m = mul_wide(a0, b1);
      add_to(m, mul_wide(a1, b0));
      d[1][k] = mont_reduce(m, pc);
      d[2][k] = mont_reduce(mul_wide(a1, b1), pc);
    }
  };
  products(first);
#pragma unroll 1
  for (int rr = 0; rr < ROWS; ++rr)
    core::stage_twiddles_async<M2>(twl[rr], twg, (u64)(N1 + row0 + rr), threadIdx.x, 32 * ROW_WARPS);
  core::cp_async_wait_all();
  __syncthreads();
#pragma unroll 1
  for (int t = 0; t < count; ++t) {
    const int j = first + t;
    if (t > 0) products(j);
#pragma unroll
    for (int o = 0; o < 3; ++o) {
      core::inv_sub<M2>(d[o], buf, l, twl[rl], pc.q);
      u64* out = out3.p[3 * j + o] + off;
#pragma unroll
      for (int k = 0; k < 8; ++k) out[core::first_idx<M2>(l, k)] = d[o][k];
      __syncwarp();  // the warp's buffer is reused by the next transform
    }
  }
}

template <int M1, int M2>
void tensor_inv_rows_fast(const NttArgs& a, const PtrTab& in4, const PtrTab& out3, int jobs, int limbs, LimbMap map,
                          cudaStream_t s) {
  constexpr int N1 = 1 << M1;
  dim3 g(N1 / (ROW_WARPS * core::Geo<M2>::SUBS), limbs, (jobs + TENSOR_ROW_JOBS - 1) / TENSOR_ROW_JOBS);
  ProfScope p("tensor_inv_rows", s);
  k_tensor_inv_rows<M1, M2><<<g, 32 * ROW_WARPS, 0, s>>>(a, in4, out3, map, jobs);
}

template <int M1, int M2>
void inv_cols_fast(const NttArgs& a, const PtrTab& data, int polys, int limbs, LimbMap map, cudaStream_t s) {
  constexpr int N2 = 1 << M2;
  dim3 g1(N2 / ColTile<M1>::COLS, limbs, polys);
  ProfScope p("ntt_inv_cols", s);
  if (a.lazy_inv) k_cols_f<M1, M2, true, false><<<g1, 256, 0, s>>>(a, data, data, map);
  else k_cols_f<M1, M2, false, false><<<g1, 256, 0, s>>>(a, data, data, map);
}

template <bool LAZY>
bool fwd_dispatch(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
                  cudaStream_t s) {
  switch (a.log_n) {
    case 12: fwd_fast<6, 6, LAZY>(a, src, dst, polys, limbs, map, s); return true;
    case 13: fwd_fast<6, 7, LAZY>(a, src, dst, polys, limbs, map, s); return true;
    case 14: fwd_fast<7, 7, LAZY>(a, src, dst, polys, limbs, map, s); return true;
    case 15: fwd_fast<7, 8, LAZY>(a, src, dst, polys, limbs, map, s); return true;
    case 16: fwd_fast<8, 8, LAZY>(a, src, dst, polys, limbs, map, s); return true;
    default: return false;
  }
}

bool inv_dispatch(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
                  cudaStream_t s) {
  switch (a.log_n) {
    case 12: inv_fast<6, 6>(a, src, dst, polys, limbs, map, s); return true;
    case 13: inv_fast<6, 7>(a, src, dst, polys, limbs, map, s); return true;
    case 14: inv_fast<7, 7>(a, src, dst, polys, limbs, map, s); return true;
    case 15: inv_fast<7, 8>(a, src, dst, polys, limbs, map, s); return true;
    case 16: inv_fast<8, 8>(a, src, dst, polys, limbs, map, s); return true;
    default: return false;
  }
}

inline int threads_for(int work) {
  int t = 32;
  while (t < 256 && t < work) t <<= 1;
  return t;
}

}  // namespace

namespace {

// Tensor product between the two phases of the transforms: for job blockIdx.z and limb blockIdx.y, each warp
// takes a row of the column-phase outputs of (a0, a1, b0, b1), finishes their forward transforms (row
// phase), forms d0 = a0 b0, d1 = a0 b1 + a1 b0, d2 = a1 b1 in the NTT domain and runs the row phase of the
// inverse transforms of d0, d1, d2, so the NTT-domain values never leave the SM.  in4.p[4j..4j+3] ->
// out3.p[3j..3j+2]; the inverse column phase follows.
template <int M1, int M2, bool LAZY>
__global__ __launch_bounds__(32 * ROW_WARPS, 3) void k_tensor_rows(NttArgs a, PtrTab in4, PtrTab out3,
                                                                     LimbMap map) {
  using G = core::Geo<M2>;
  constexpr int N1 = 1 << M1, N2 = 1 << M2, N = N1 * N2, ROWS = ROW_WARPS * G::SUBS;
  __shared__ u64 bufs[ROWS * G::STRIDE];
  __shared__ __align__(16) Twiddle twf[ROWS][N2];
  __shared__ __align__(16) Twiddle twi[ROWS][N2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane / G::LANES, l = lane % G::LANES;
  const int row0 = blockIdx.x * ROWS;
  const int limb = blockIdx.y, job = blockIdx.z;
  const int prime = map.prime(limb);
  const PrimeConst& pc = a.pc[prime];
  const u64 q = pc.q;
  const int rl = warp * G::SUBS + sub, row = row0 + rl;
  const size_t off = (size_t)limb * N + (size_t)row * N2;
  const u64* a0p = in4.p[4 * job + 0] + off;
  const u64* a1p = in4.p[4 * job + 1] + off;
  const u64* b0p = in4.p[4 * job + 2] + off;
  const u64* b1p = in4.p[4 * job + 3] + off;
  // a0 and b0 are requested before the twiddle tables, so both latencies overlap
  u64 x[8], y[8], z[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    x[k] = a0p[core::first_idx<M2>(l, k)];
    y[k] = b0p[core::first_idx<M2>(l, k)];
  }
  const Twiddle* tf = a.tw_fwd + (size_t)prime * N;
  const Twiddle* ti = a.tw_inv + (size_t)prime * N;
#pragma unroll 1
  for (int rr = 0; rr < ROWS; ++rr) {
    core::stage_twiddles_async<M2>(twf[rr], tf, (u64)(N1 + row0 + rr), threadIdx.x, 32 * ROW_WARPS);
    core::stage_twiddles_async<M2>(twi[rr], ti, (u64)(N1 + row0 + rr), threadIdx.x, 32 * ROW_WARPS);
  }
  core::cp_async_wait_all();
  __syncthreads();
  u64* buf = bufs + rl * G::STRIDE;
  auto fwd = [&](u64(&v)[8]) {
    core::fwd_sub<M2, LAZY>(v, buf, l, twf[rl], q);
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = reduce_out<LAZY>(v[k], pc);
  };
  auto inv_store = [&](u64(&v)[8], int d) {
    core::inv_sub<M2>(v, buf, l, twi[rl], q);
    u64* o = out3.p[3 * job + d] + off;
#pragma unroll
    for (int k = 0; k < 8; ++k) o[core::first_idx<M2>(l, k)] = v[k];
  };
  // three rows live at a time: (a0, b0) -> d0; b1 -> a0 b1; a1 -> d1 = a0 b1 + a1 b0 and d2 = a1 b1
  fwd(x);
  fwd(y);
#pragma unroll
  for (int k = 0; k < 8; ++k) z[k] = mul_mod(x[k], y[k], pc);  // d0
  u64 w[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) w[k] = b1p[core::first_idx<M2>(l, k)];  // b1, in flight during d0's inverse
  inv_store(z, 0);
  fwd(w);
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = mul_mod(x[k], w[k], pc);  // a0 b1
#pragma unroll
  for (int k = 0; k < 8; ++k) z[k] = a1p[core::first_idx<M2>(l, k)];  // a1
  fwd(z);
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    U128 t = mul_wide(z[k], y[k]);  // a1 b0
    t.lo += x[k];
    t.hi += t.lo < x[k] ? 1ull : 0ull;
    x[k] = barrett_reduce(t, pc);  // d1
    y[k] = mul_mod(z[k], w[k], pc);  // d2
  }
  inv_store(x, 1);
  inv_store(y, 2);
}

}  // namespace

bool tensor_fused(const NttArgs& a, const PrimeConst* pc, const PtrTab& in4, const PtrTab& work4,
                  const PtrTab& out3, int jobs, int limbs, LimbMap map, cudaStream_t s) {
  if (jobs <= 0) return true;
  switch (a.log_n) {
#define RC_TENSOR(LN, A, B)                                                                                   \
  case LN: {                                                                                                  \
    constexpr int N2 = 1 << B, N1 = 1 << A;                                                                   \
    dim3 g1(N2 / ColTile<A>::COLS, limbs, 4 * jobs), g2(N1 / (ROW_WARPS * core::Geo<B>::SUBS), limbs, jobs);    \
    dim3 g3(N2 / ColTile<A>::COLS, limbs, 3 * jobs);                                                          \
    {                                                                                                         \
      ProfScope p("ntt_fwd_cols", s);                                                                         \
      if (a.lazy) k_cols_f<A, B, true, true><<<g1, 256, 0, s>>>(a, in4, work4, map);                          \
      else k_cols_f<A, B, false, true><<<g1, 256, 0, s>>>(a, in4, work4, map);                                \
    }                                                                                                         \
    {                                                                                                         \
      ProfScope p("tensor_rows", s);                                                                          \
      if (a.lazy) k_tensor_rows<A, B, true><<<g2, 32 * ROW_WARPS, 0, s>>>(a, work4, out3, map);               \
      else k_tensor_rows<A, B, false><<<g2, 32 * ROW_WARPS, 0, s>>>(a, work4, out3, map);                     \
    }                                                                                                         \
    {                                                                                                         \
      ProfScope p("ntt_inv_cols", s);                                                                         \
      k_cols_f<A, B, false, false><<<g3, 256, 0, s>>>(a, out3, out3, map);                                    \
    }                                                                                                         \
    return true;                                                                                              \
  }
    RC_TENSOR(12, 6, 6)
    RC_TENSOR(13, 6, 7)
    RC_TENSOR(14, 7, 7)
    RC_TENSOR(15, 7, 8)
    RC_TENSOR(16, 8, 8)
#undef RC_TENSOR
    default:
      return false;
  }
}

void ntt_forward(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
                 cudaStream_t s) {
  if (polys <= 0 || limbs <= 0) return;
  if (a.lazy ? fwd_dispatch<true>(a, src, dst, polys, limbs, map, s)
             : fwd_dispatch<false>(a, src, dst, polys, limbs, map, s))
    return;
  const int N = 1 << a.log_n, N1 = 1 << a.n1, N2 = N >> a.n1;
  const int COLS = cols_per_cta(N2), ROWS = rows_per_cta(N1, N2);
  dim3 g1(N2 / COLS, limbs, polys), g2(N1 / ROWS, limbs, polys);
  {
    ProfScope p("ntt_fwd_cols", s);
    k_fwd_cols<<<g1, threads_for(N1 * COLS / 2), N1 * COLS * sizeof(u64), s>>>(a, src, dst, map);
  }
  {
    ProfScope p("ntt_fwd_rows", s);
    k_fwd_rows<<<g2, threads_for(ROWS * N2 / 2), ROWS * N2 * sizeof(u64), s>>>(a, dst, dst, map);
  }
}

void ntt_inverse(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
                 cudaStream_t s) {
  if (polys <= 0 || limbs <= 0) return;
  if (inv_dispatch(a, src, dst, polys, limbs, map, s)) return;
  const int N = 1 << a.log_n, N1 = 1 << a.n1, N2 = N >> a.n1;
  const int COLS = cols_per_cta(N2), ROWS = rows_per_cta(N1, N2);
  dim3 g1(N2 / COLS, limbs, polys), g2(N1 / ROWS, limbs, polys);
  {
    ProfScope p("ntt_inv_rows", s);
    k_inv_rows<<<g2, threads_for(ROWS * N2 / 2), ROWS * N2 * sizeof(u64), s>>>(a, src, dst, map);
  }
  {
    ProfScope p("ntt_inv_cols", s);
    k_inv_cols<<<g1, threads_for(N1 * COLS / 2), N1 * COLS * sizeof(u64), s>>>(a, dst, dst, map);
  }
}

bool tensor_inverse_rows(const NttArgs& a, const PtrTab& in4, const PtrTab& out3, int jobs, int limbs, LimbMap map,
                         cudaStream_t s) {
  switch (a.log_n) {
    case 12: tensor_inv_rows_fast<6, 6>(a, in4, out3, jobs, limbs, map, s); return true;
    case 13: tensor_inv_rows_fast<6, 7>(a, in4, out3, jobs, limbs, map, s); return true;
    case 14: tensor_inv_rows_fast<7, 7>(a, in4, out3, jobs, limbs, map, s); return true;
    case 15: tensor_inv_rows_fast<7, 8>(a, in4, out3, jobs, limbs, map, s); return true;
    case 16: tensor_inv_rows_fast<8, 8>(a, in4, out3, jobs, limbs, map, s); return true;
    default: return false;
  }
}

bool ntt_inverse_cols(const NttArgs& a, const PtrTab& data, int polys, int limbs, LimbMap map, cudaStream_t s) {
  switch (a.log_n) {
    case 12: inv_cols_fast<6, 6>(a, data, polys, limbs, map, s); return true;
    case 13: inv_cols_fast<6, 7>(a, data, polys, limbs, map, s); return true;
    case 14: inv_cols_fast<7, 7>(a, data, polys, limbs, map, s); return true;
    case 15: inv_cols_fast<7, 8>(a, data, polys, limbs, map, s); return true;
    case 16: inv_cols_fast<8, 8>(a, data, polys, limbs, map, s); return true;
    default: return false;
  }
}

}  // namespace rc
