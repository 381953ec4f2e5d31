// The fused tensor pass (tunable "fuse_tensor"): the forward column phase, then one kernel for the forward
// row phase, the NTT-domain tensor and the inverse row phase, then the inverse column phase (the kernels
// shared with the transforms are in ntt_kernels.cuh).
#include "ntt_kernels.cuh"

namespace rc {

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
  return with_split(a.log_n, a.n1, [&](auto m1, auto m2) {
    constexpr int A = m1.value, B = m2.value;
    constexpr int N1 = 1 << A;
    dim3 g2(N1 / (ROW_WARPS * core::Geo<B>::SUBS), limbs, jobs);
    ntt_forward_cols(a, in4, work4, 4 * jobs, limbs, map, s);
    {
      ProfScope p("tensor_rows", s);
      if (a.lazy) k_tensor_rows<A, B, true><<<g2, 32 * ROW_WARPS, 0, s>>>(a, work4, out3, map);
      else k_tensor_rows<A, B, false><<<g2, 32 * ROW_WARPS, 0, s>>>(a, work4, out3, map);
    }
    ntt_inverse_cols(a, out3, 3 * jobs, limbs, map, s);
  });
}


}  // namespace rc
