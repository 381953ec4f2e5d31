// Inverse negacyclic NTT over RNS limbs (the kernels are in ntt_kernels.cuh), the tensor products fused into
// the inverse row pass, and the inverse column pass alone.
#include "ntt_kernels.cuh"
#include "nttr16.cuh"

namespace rc {

namespace {

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


template <int M1, int M2>
void inv_cols_fast(const NttArgs& a, const PtrTab& data, int polys, int limbs, LimbMap map, cudaStream_t s) {
  constexpr int N2 = 1 << M2;
  dim3 g1(N2 / ColTile<M1>::COLS, limbs, polys);
  ProfScope p("ntt_inv_cols", s);
  with_cc(a.col_ctas, [&](auto cc) {
    if (a.lazy_inv) k_cols_f<M1, M2, true, false, cc.value><<<g1, 256, 0, s>>>(a, data, data, map);
    else k_cols_f<M1, M2, false, false, cc.value><<<g1, 256, 0, s>>>(a, data, data, map);
  });
}


template <int M1, int M2>
void inv_fast(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
              cudaStream_t s) {
  constexpr int N1 = 1 << M1;
  {
    ProfScope p("ntt_inv_rows", s);
    with_rp(a.row_polys, [&](auto rp) {
      dim3 g2(N1 / (ROW_WARPS * core::Geo<M2>::SUBS), limbs, (polys + rp.value - 1) / rp.value);
      k_rows_f<M1, M2, false, false, rp.value><<<g2, 32 * ROW_WARPS, 0, s>>>(a, src, dst, map, polys);
    });
  }
  inv_cols_fast<M1, M2>(a, dst, polys, limbs, map, s);
}

// The tensor and the inverse row phase in one pass: for each job of the block, d0 = a0 b0, d1 = a0 b1 + a1 b0
// and d2 = a1 b1 (Montgomery products of the forward transforms in4[4j..4j+3], left in [0, 2q) as the inverse
// butterflies accept; the inverse column pass's scale takes out their 2^-64) go straight into the inverse row
// transform, so the quadratic NTT-domain values never
// reach HBM.  A block transforms the same rows of NttArgs::tensor_jobs jobs (three outputs each) with one twiddle
// staging.


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
  const int tj = a.tensor_jobs;
  const int limb = blockIdx.y, first = blockIdx.z * tj, count = min(tj, jobs - first);
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
      // a0 b1 + a1 b0 = (a0 + a1)(b0 + b1) - a0 b0 - a1 b1 exactly (inputs below q < 2^61): three 128-bit
      // products instead of four, the same integer into the same Montgomery reduction
      const U128 p0 = mul_wide(a0, b0), p2 = mul_wide(a1, b1);
      U128 m = mul_wide(a0 + a1, b0 + b1);
      sub_from(m, p0);
      sub_from(m, p2);
      d[0][k] = mont_reduce_lazy(p0, pc);
      d[1][k] = mont_reduce_lazy(m, pc);
      d[2][k] = mont_reduce_lazy(p2, pc);
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
    // one copy of the sub-transform for the three outputs (selected into v): the unrolled form stalled on
    // instruction fetch and ran 7 % slower
#pragma unroll 1
    for (int o = 0; o < 3; ++o) {
      u64 v[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) v[k] = o == 0 ? d[0][k] : (o == 1 ? d[1][k] : d[2][k]);
      core::inv_sub<M2>(v, buf, l, twl[rl], pc.q);
      u64* out = out3.p[3 * j + o] + off;
#pragma unroll
      for (int k = 0; k < 8; ++k) out[core::first_idx<M2>(l, k)] = v[k];
      __syncwarp();  // the warp's buffer is reused by the next transform
    }
  }
}

template <int M1, int M2>
void tensor_inv_rows_fast(const NttArgs& a, const PtrTab& in4, const PtrTab& out3, int jobs, int limbs, LimbMap map,
                          cudaStream_t s) {
  constexpr int N1 = 1 << M1;
  dim3 g(N1 / (ROW_WARPS * core::Geo<M2>::SUBS), limbs, (jobs + a.tensor_jobs - 1) / a.tensor_jobs);
  ProfScope p("tensor_inv_rows", s);
  k_tensor_inv_rows<M1, M2><<<g, 32 * ROW_WARPS, 0, s>>>(a, in4, out3, map, jobs);
}


// N = 2^16: the 16-residue passes (nttr16.cuh), each pass taken when its bit of NttArgs::r16 is set and its
// polynomials are 16-byte aligned
bool r16_inv_cols(const NttArgs& a, const PtrTab& data, int polys, int limbs, LimbMap map, cudaStream_t s) {
  if (!r16::applies(a, r16::R16_ICOLS) || !r16::aligned(data, polys)) return false;
  const int nt = 16 * limbs * polys;
  ProfScope p("ntt_inv_cols", s);
  if (a.lazy_inv) {
    r16::smem_optin<k16_cols<true, false>, r16::COL_SMEM>();
    k16_cols<true, false><<<r16::col_grid(nt), 256, r16::COL_SMEM, s>>>(a, data, data, map, limbs, nt);
  } else {
    r16::smem_optin<k16_cols<false, false>, r16::COL_SMEM>();
    k16_cols<false, false><<<r16::col_grid(nt), 256, r16::COL_SMEM, s>>>(a, data, data, map, limbs, nt);
  }
  return true;
}
bool r16_inverse(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
                 cudaStream_t s) {
  if (!a.r16 || a.log_n != 16 || a.n1 != 8) return false;
  if (r16::applies(a, r16::R16_ROWS) && r16::aligned(src, polys) && r16::aligned(dst, polys)) {
    ProfScope p("ntt_inv_rows", s);
    with_rp(a.row_polys, [&](auto rp) {
      k16_rows<false, false, rp.value>
          <<<dim3(256 / (2 * r16::RW), limbs, (polys + rp.value - 1) / rp.value), 32 * r16::RW, 0, s>>>(a, src, dst, map,
                                                                                                     polys);
    });
  } else {
    ProfScope p("ntt_inv_rows", s);
    with_rp(a.row_polys, [&](auto rp) {
      dim3 g2(256 / (ROW_WARPS * core::Geo<8>::SUBS), limbs, (polys + rp.value - 1) / rp.value);
      k_rows_f<8, 8, false, false, rp.value><<<g2, 32 * ROW_WARPS, 0, s>>>(a, src, dst, map, polys);
    });
  }
  if (!r16_inv_cols(a, dst, polys, limbs, map, s)) inv_cols_fast<8, 8>(a, dst, polys, limbs, map, s);
  return true;
}

// calls f(integral_constant<M1>, integral_constant<M2>) for the fast path's four-step split of 2^log_n
// points with a column phase of 2^n1 (both phases 2^6..2^8); false when there is none

bool inv_dispatch(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
                  cudaStream_t s) {
  return with_split(a.log_n, a.n1, [&](auto m1, auto m2) {
    inv_fast<m1.value, m2.value>(a, src, dst, polys, limbs, map, s);
  });
}

}  // namespace

void ntt_inverse(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
                 cudaStream_t s) {
  if (polys <= 0 || limbs <= 0) return;
  if (r16_inverse(a, src, dst, polys, limbs, map, s)) return;
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
  if (r16::applies(a, r16::R16_TENSOR) && r16::aligned(in4, 4 * jobs) && r16::aligned(out3, 3 * jobs)) {
    ProfScope p("tensor_inv_rows", s);
    k16_tensor_inv_rows<4>
        <<<dim3(256 / (2 * r16::RW), limbs, (jobs + 4 - 1) / 4), 32 * r16::RW, 0, s>>>(a, in4, out3, map,
                                                                                                jobs);
    return true;
  }
  return with_split(a.log_n, a.n1, [&](auto m1, auto m2) {
    tensor_inv_rows_fast<m1.value, m2.value>(a, in4, out3, jobs, limbs, map, s);
  });
}


bool ntt_inverse_cols(const NttArgs& a, const PtrTab& data, int polys, int limbs, LimbMap map, cudaStream_t s) {
  if (r16_inv_cols(a, data, polys, limbs, map, s)) return true;
  return with_split(a.log_n, a.n1, [&](auto m1, auto m2) {
    inv_cols_fast<m1.value, m2.value>(a, data, polys, limbs, map, s);
  });
}

}  // namespace rc
