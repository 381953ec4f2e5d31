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
    out[(size_t)r * N2 + c0 + c] = mul_shoup(sm[idx], pc.n_inv, pc.n_inv_s, q);
  }
}

inline int threads_for(int work) {
  int t = 32;
  while (t < 256 && t < work) t <<= 1;
  return t;
}

}  // namespace

void ntt_forward(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
                 cudaStream_t s) {
  if (polys <= 0 || limbs <= 0) return;
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

}  // namespace rc
