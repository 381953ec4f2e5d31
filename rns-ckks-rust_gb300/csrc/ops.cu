// Limbwise elementwise kernels: add/sub/pointwise multiply, the NTT-domain
// tensor product, the coefficient-domain Galois automorphism and rescale.
#include "kernels.cuh"

namespace rc {

namespace {

// A value v < q_src reduced modulo q (q may be smaller than q_src): exact.
__device__ __forceinline__ u64 reduce_any(u64 v, const PrimeConst& c) {
  if (v < c.q) return v;
  U128 t;
  t.lo = v;
  t.hi = 0;
  return barrett_reduce(t, c);
}

__global__ void k_ew_binary(int op, const PrimeConst* pc, PtrTab a, PtrTab b, int b_shared, PtrTab out, int limbs,
                            LimbMap map, int log_n) {
  const size_t total = (size_t)limbs << log_n;
  const int poly = blockIdx.y;
  const u64* pa = a.p[poly];
  const u64* pb = b.p[b_shared ? 0 : poly];
  u64* po = out.p[poly];
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int limb = (int)(e >> log_n);
    const PrimeConst& c = pc[map.prime(limb)];
    u64 x = pa[e], y = pb[e];
    u64 r;
    if (op == 0) r = add_mod(x, y, c.q);
    else if (op == 1) r = sub_mod(x, y, c.q);
    else if (op == 2) r = mul_mod(x, y, c);
    else r = mont_reduce(mul_wide(x, y), c);
    po[e] = r;
  }
}

__global__ void k_plain_mac(const PrimeConst* pc, PtrTab ct, PtrTab pt, int count, u64* acc, int accumulate,
                            int limbs, LimbMap map, int log_n) {
  const size_t total = (size_t)limbs << log_n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const PrimeConst& c = pc[map.prime((int)(e >> log_n))];
    u64 s0 = accumulate ? acc[e] : 0, s1 = accumulate ? acc[total + e] : 0;
    if ((c.q >> 59) == 0 && count <= 16) {
      // 128-bit sums (below (count + 1) q^2 < q 2^64), one Barrett reduction per output
      U128 t0{s0, 0}, t1{s1, 0};
      for (int k = 0; k < count; ++k) {
        const u64 p = pt.p[k][e];
        add_to(t0, mul_wide(ct.p[k][e], p));
        add_to(t1, mul_wide(ct.p[k][total + e], p));
      }
      s0 = barrett_reduce(t0, c);
      s1 = barrett_reduce(t1, c);
    } else {
      for (int k = 0; k < count; ++k) {
        const u64 p = pt.p[k][e];
        s0 = add_mod(s0, mul_mod(ct.p[k][e], p, c), c.q);
        s1 = add_mod(s1, mul_mod(ct.p[k][total + e], p, c), c.q);
      }
    }
    acc[e] = s0;
    acc[total + e] = s1;
  }
}

__global__ void k_tensor(const PrimeConst* pc, PtrTab in4, PtrTab out3, int limbs, int log_n) {
  const size_t total = (size_t)limbs << log_n;
  const int job = blockIdx.y;
  const u64* a0 = in4.p[4 * job + 0];
  const u64* a1 = in4.p[4 * job + 1];
  const u64* b0 = in4.p[4 * job + 2];
  const u64* b1 = in4.p[4 * job + 3];
  u64* d0 = out3.p[3 * job + 0];
  u64* d1 = out3.p[3 * job + 1];
  u64* d2 = out3.p[3 * job + 2];
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const PrimeConst& c = pc[(int)(e >> log_n)];
    u64 x0 = a0[e], x1 = a1[e], y0 = b0[e], y1 = b1[e];
    // Montgomery products (x y 2^-64 mod q; the sum of two stays below q 2^64): one low and one high
    // 64-bit product per reduction against Barrett's five
    d0[e] = mont_reduce(mul_wide(x0, y0), c);
    U128 m = mul_wide(x0, y1);
    add_to(m, mul_wide(x1, y0));
    d1[e] = mont_reduce(m, c);
    d2[e] = mont_reduce(mul_wide(x1, y1), c);
  }
}

// out[m] = sigma_g(in)[m]: the source index is m * g^-1 mod 2N; a source index
// in [N, 2N) means the coefficient wrapped past X^N and is negated
// (src/poly/mod.rs:110-131 states the same map from the source side).
__global__ void k_automorphism(const PrimeConst* pc, PtrTab in, PtrTab out, int limbs, u64 g_inv, int log_n) {
  const u64 N = 1ull << log_n, mask2 = 2 * N - 1;
  const size_t total = (size_t)limbs << log_n;
  const int poly = blockIdx.y;
  const u64* src = in.p[poly];
  u64* dst = out.p[poly];
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int limb = (int)(e >> log_n);
    const u64 m = e & (N - 1);
    u64 i = (m * g_inv) & mask2;
    const bool neg = i >= N;
    if (neg) i -= N;
    u64 v = src[((size_t)limb << log_n) + i];
    if (neg && v) v = pc[limb].q - v;
    dst[e] = v;
  }
}

// rescale_poly_rns (src/rns/ops.rs:135-186): drop prime l-1; for i < l-1,
// out_i = (c_i - centred(c_{l-1}) mod q_i) * q_{l-1}^-1 mod q_i, where values
// <= floor(q_{l-1}/2) count as positive.
__global__ void k_rescale(const PrimeConst* pc, RescaleTab rt, int L, PtrTab in, PtrTab out, int limbs, int log_n) {
  const size_t N = 1ull << log_n;
  const size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (x >= N) return;
  const int poly = blockIdx.y;
  const u64* src = in.p[poly];
  u64* dst = out.p[poly];
  const int last = limbs - 1;
  const u64 ql = pc[last].q, half = ql >> 1;
  const u64 v = src[(size_t)last * N + x];
  const bool pos = v <= half;
  const u64 dist = pos ? v : ql - v;
  for (int i = 0; i < last; ++i) {
    const PrimeConst& c = pc[i];
    u64 d = reduce_any(dist, c);
    u64 cd = pos ? d : (d == 0 ? 0 : c.q - d);
    u64 num = sub_mod(src[(size_t)i * N + x], cd, c.q);
    size_t k = (size_t)last * L + i;
    dst[(size_t)i * N + x] = mul_shoup(num, rt.inv[k], rt.inv_s[k], c.q);
  }
}

__global__ void k_mul_scalar(const PrimeConst* pc, const u64* a, ScalarTab v, u64* out, int limbs, LimbMap map,
                             int log_n) {
  const size_t total = (size_t)limbs << log_n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const int limb = (int)(e >> log_n);
    out[e] = mul_mod(a[e], v.v[limb], pc[map.prime(limb)]);
  }
}

inline int grid_for(size_t total, int threads) {
  size_t g = (total + threads - 1) / threads;
  if (g > 65535 * 4) g = 65535 * 4;
  if (g > 2147483647ull) g = 2147483647ull;
  return (int)(g == 0 ? 1 : g);
}

}  // namespace

void ew_binary(EwOp op, const PrimeConst* pc, const PtrTab& a, const PtrTab& b, int b_shared, const PtrTab& out,
               int polys, int limbs, LimbMap map, int n, cudaStream_t s) {
  if (polys <= 0) return;
  int log_n = __builtin_ctz(n);
  dim3 g(grid_for((size_t)limbs * n, 256), polys);
  ProfScope p("elementwise", s);
  k_ew_binary<<<g, 256, 0, s>>>(op == EwOp::Add ? 0 : op == EwOp::Sub ? 1 : op == EwOp::Mul ? 2 : 3, pc, a, b,
                                b_shared, out, limbs, map, log_n);
}

void plain_mac(const PrimeConst* pc, const PtrTab& ct, const PtrTab& pt, int count, u64* acc, int accumulate,
               int limbs, LimbMap map, int n, cudaStream_t s) {
  if (count <= 0) return;
  ProfScope p("plain_mac", s);
  k_plain_mac<<<grid_for((size_t)limbs * n, 256), 256, 0, s>>>(pc, ct, pt, count, acc, accumulate, limbs, map,
                                                              __builtin_ctz(n));
}

void mul_scalar(const PrimeConst* pc, const u64* a, const ScalarTab& v, u64* out, int limbs, LimbMap map, int n,
                cudaStream_t s) {
  k_mul_scalar<<<grid_for((size_t)limbs * n, 256), 256, 0, s>>>(pc, a, v, out, limbs, map, __builtin_ctz(n));
}

void tensor_ntt(const PrimeConst* pc, const PtrTab& in4, const PtrTab& out3, int jobs, int limbs, int n,
                cudaStream_t s) {
  if (jobs <= 0) return;
  dim3 g(grid_for((size_t)limbs * n, 256), jobs);
  ProfScope p("tensor", s);
  k_tensor<<<g, 256, 0, s>>>(pc, in4, out3, limbs, __builtin_ctz(n));
}

void automorphism(const PrimeConst* pc, const PtrTab& in, const PtrTab& out, int polys, int limbs, uint64_t g_inv,
                  int log_n, cudaStream_t s) {
  if (polys <= 0) return;
  dim3 g(grid_for((size_t)limbs << log_n, 256), polys);
  ProfScope p("automorphism", s);
  k_automorphism<<<g, 256, 0, s>>>(pc, in, out, limbs, g_inv, log_n);
}

void rescale(const PrimeConst* pc, const RescaleTab& rt, int L, const PtrTab& in, const PtrTab& out, int polys,
             int limbs, int n, cudaStream_t s) {
  if (polys <= 0) return;
  dim3 g((n + 255) / 256, polys);
  ProfScope p("rescale", s);
  k_rescale<<<g, 256, 0, s>>>(pc, rt, L, in, out, limbs, __builtin_ctz(n));
}

}  // namespace rc
