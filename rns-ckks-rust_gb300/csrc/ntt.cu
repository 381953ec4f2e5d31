// Forward negacyclic NTT over RNS limbs (the kernels are in ntt_kernels.cuh) and the fused tensor pass.
#include "ntt_kernels.cuh"
#include "nttr16.cuh"

namespace rc {

namespace {

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


template <int M1, int M2, bool LAZY>
void fwd_fast(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
              cudaStream_t s) {
  constexpr int N2 = 1 << M2, N1 = 1 << M1;
  dim3 g1(N2 / ColTile<M1>::COLS, limbs, polys);
  {
    ProfScope p("ntt_fwd_cols", s);
    with_cc(a.col_ctas, [&](auto cc) { k_cols_f<M1, M2, LAZY, true, cc.value><<<g1, 256, 0, s>>>(a, src, dst, map); });
  }
  {
    ProfScope p("ntt_fwd_rows", s);
    with_rp(a.row_polys, [&](auto rp) {
      dim3 g2(N1 / (ROW_WARPS * core::Geo<M2>::SUBS), limbs, (polys + rp.value - 1) / rp.value);
      if constexpr (M1 == 8 && M2 == 8) {  // unreduced outputs for the tensor at N = 2^16 (NttArgs::raw_out)
        if (a.raw_out) {
          k_rows_f<M1, M2, LAZY, true, rp.value, true><<<g2, 32 * ROW_WARPS, 0, s>>>(a, dst, dst, map, polys);
          return;
        }
      }
      k_rows_f<M1, M2, LAZY, true, rp.value><<<g2, 32 * ROW_WARPS, 0, s>>>(a, dst, dst, map, polys);
    });
  }
}

// the inverse column pass, in place (lazy for primes below 2^55)

// N = 2^16: the 16-residue passes (nttr16.cuh), each pass taken when its bit of NttArgs::r16 is set and its
// polynomials are 16-byte aligned (the passes read and write natural order, so they mix with the others)
template <bool LAZY>
bool r16_fwd_cols(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
                  cudaStream_t s) {
  if (!r16::applies(a, r16::R16_COLS) || !r16::aligned(src, polys) || !r16::aligned(dst, polys)) return false;
  const int nt = 16 * limbs * polys;
  r16::smem_optin<k16_cols<LAZY, true>, r16::COL_SMEM>();
  ProfScope p("ntt_fwd_cols", s);
  k16_cols<LAZY, true><<<r16::col_grid(nt), 256, r16::COL_SMEM, s>>>(a, src, dst, map, limbs, nt);
  return true;
}
template <bool LAZY>
bool r16_fwd_rows(const NttArgs& a, const PtrTab& data, int polys, int limbs, LimbMap map, cudaStream_t s) {
  if (!r16::applies(a, r16::R16_ROWS) || !r16::aligned(data, polys)) return false;
  ProfScope p("ntt_fwd_rows", s);
  with_rp(a.row_polys, [&](auto rp) {
    const dim3 g(256 / (2 * r16::RW), limbs, (polys + rp.value - 1) / rp.value);
    if (a.raw_out) k16_rows<LAZY, true, rp.value, true><<<g, 32 * r16::RW, 0, s>>>(a, data, data, map, polys);
    else k16_rows<LAZY, true, rp.value><<<g, 32 * r16::RW, 0, s>>>(a, data, data, map, polys);
  });
  return true;
}
template <bool LAZY>
bool r16_forward(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
                 cudaStream_t s) {
  if (a.log_n != 16 || a.n1 != 8) return false;
  if (!r16_fwd_cols<LAZY>(a, src, dst, polys, limbs, map, s)) {
    ProfScope p("ntt_fwd_cols", s);
    with_cc(a.col_ctas, [&](auto cc) {
      k_cols_f<8, 8, LAZY, true, cc.value><<<dim3(256 / ColTile<8>::COLS, limbs, polys), 256, 0, s>>>(a, src, dst, map);
    });
  }
  if (!r16_fwd_rows<LAZY>(a, dst, polys, limbs, map, s)) {
    ProfScope p("ntt_fwd_rows", s);
    with_rp(a.row_polys, [&](auto rp) {
      dim3 g2(256 / (ROW_WARPS * core::Geo<8>::SUBS), limbs, (polys + rp.value - 1) / rp.value);
      if (a.raw_out) k_rows_f<8, 8, LAZY, true, rp.value, true><<<g2, 32 * ROW_WARPS, 0, s>>>(a, dst, dst, map, polys);
      else k_rows_f<8, 8, LAZY, true, rp.value><<<g2, 32 * ROW_WARPS, 0, s>>>(a, dst, dst, map, polys);
    });
  }
  return true;
}

template <bool LAZY>
bool fwd_dispatch(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
                  cudaStream_t s) {
  return with_split(a.log_n, a.n1, [&](auto m1, auto m2) {
    fwd_fast<m1.value, m2.value, LAZY>(a, src, dst, polys, limbs, map, s);
  });
}



}  // namespace

bool ntt_forward_cols(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
                      cudaStream_t s) {
  if (a.lazy ? r16_fwd_cols<true>(a, src, dst, polys, limbs, map, s)
             : r16_fwd_cols<false>(a, src, dst, polys, limbs, map, s))
    return true;
  return with_split(a.log_n, a.n1, [&](auto m1, auto m2) {
    constexpr int A = m1.value, B = m2.value;
    dim3 g1((1 << B) / ColTile<A>::COLS, limbs, polys);
    ProfScope p("ntt_fwd_cols", s);
    with_cc(a.col_ctas, [&](auto cc) {
      if (a.lazy) k_cols_f<A, B, true, true, cc.value><<<g1, 256, 0, s>>>(a, src, dst, map);
      else k_cols_f<A, B, false, true, cc.value><<<g1, 256, 0, s>>>(a, src, dst, map);
    });
  });
}

void ntt_forward(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
                 cudaStream_t s) {
  if (polys <= 0 || limbs <= 0) return;
  if (a.r16 && (a.lazy ? r16_forward<true>(a, src, dst, polys, limbs, map, s)
                       : r16_forward<false>(a, src, dst, polys, limbs, map, s)))
    return;
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

}  // namespace rc
