// RNS-hybrid key switching ("dnum" gadget; no counterpart in the reference, whose only gadget is balanced
// base-2^30 digits, src/rns/keyswitching.rs:238-240).  The active chain Q_l is cut into dnum groups of alpha
// consecutive limbs; group b's part of the polynomial, [c]_{Q_b}, is extended to Q_l u P by a fast basis
// conversion (ModUp: sum_i [c_i (Q_b/q_i)^-1]_{q_i} (Q_b/q_i) mod t, exact up to a multiple of Q_b that the key
// annihilates), multiplied in the NTT domain by key b and summed; ModDown by P (the exact centred conversion
// of k_finalize) brings it back to Q_l.  Key b encrypts [i in group b] (P mod q_i) s^2, so the result
// decrypts to c s^2 plus the keys' noise divided by P.  Results are not the reference's residues (a different
// gadget); they decrypt to the same values.
#include "kernels.cuh"

namespace rc {

namespace {

// D[job][b][limb][N] for limb in 0..total-1 (Q limbs then aux limbs) from the job's coefficient-form
// polynomial src.p[job] ([qlimbs][N]).  tab holds, per group b: (Q_b/q_i)^-1 mod q_i and its Shoup companion
// for the group's limbs, then (Q_b/q_i) mod t for every target limb t: [dnum][alpha][2 + total].
__global__ void k_dnum_modup(const PrimeConst* pc, PtrTab src, const u64* tab, u64* D, int qlimbs, int total,
                             int alpha, int dnum, LimbMap map, int log_n) {
  extern __shared__ u64 st[];  // group b's [alpha][2 + total] table
  const int b = blockIdx.y, job = blockIdx.z;
  const int row = 2 + total;
  const u64* tb = tab + (size_t)b * alpha * row;
  for (int e = threadIdx.x; e < alpha * row; e += blockDim.x) st[e] = tb[e];
  __syncthreads();
  const u64 N = 1ull << log_n;
  const u64 x = blockIdx.x * (u64)blockDim.x + threadIdx.x;
  if (x >= N) return;
  const int i0 = b * alpha, i1 = min(i0 + alpha, qlimbs);
  const u64* in = src.p[job];
  u64* out = D + ((size_t)job * dnum + b) * total * N + x;
  u64 y[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    if (k < i1 - i0) {
      const int i = i0 + k;
      const u64 c = in[(size_t)i * N + x];
      out[(size_t)i * N] = c;  // the group's own limbs are the polynomial's residues
      y[k] = mul_shoup(c, st[k * row], st[k * row + 1], pc[i].q);
    }
  }
  for (int t = 0; t < total; ++t) {
    if (t >= i0 && t < i1) continue;
    const PrimeConst& pt = pc[map.prime(t)];
    U128 acc{0, 0};
#pragma unroll
    for (int k = 0; k < 16; ++k)
      if (k < i1 - i0) add_to(acc, mul_wide(y[k], st[k * row + 2 + t]));
    out[(size_t)t * N] = barrett_reduce(acc, pt);
  }
}

// acc[job][c][limb] = sum_b D[job][b][limb] * key[b][c][limb] mod t, NTT domain (dnum <= 16 terms: 128-bit sums
// below q 2^64, one Barrett reduction)
__global__ void k_dnum_mac(const PrimeConst* pc, const u64* D, const u64* key, u64* acc, int total, int dnum,
                           LimbMap map, int log_n) {
  const size_t per = (size_t)total << log_n;
  const int job = blockIdx.y;
  const u64* d = D + (size_t)job * dnum * per;
  u64* a = acc + (size_t)job * 2 * per;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < per; e += (size_t)gridDim.x * blockDim.x) {
    const PrimeConst& c = pc[map.prime((int)(e >> log_n))];
    U128 t0{0, 0}, t1{0, 0};
    for (int b = 0; b < dnum; ++b) {
      const u64 v = d[(size_t)b * per + e];
      add_to(t0, mul_wide(v, key[(size_t)b * 2 * per + e]));
      add_to(t1, mul_wide(v, key[((size_t)b * 2 + 1) * per + e]));
    }
    a[e] = barrett_reduce(t0, c);
    a[per + e] = barrett_reduce(t1, c);
  }
}

}  // namespace

void dnum_modup(const PrimeConst* pc, const PtrTab& src, int jobs, const u64* tab, u64* D, int qlimbs, int total,
                int alpha, int dnum, LimbMap map, int log_n, cudaStream_t s) {
  if (jobs <= 0) return;
  const int N = 1 << log_n;
  const int threads = N < 128 ? N : 128;
  dim3 g((N + threads - 1) / threads, dnum, jobs);
  ProfScope p("dnum_modup", s);
  k_dnum_modup<<<g, threads, (size_t)alpha * (2 + total) * 8, s>>>(pc, src, tab, D, qlimbs, total, alpha, dnum, map,
                                                                    log_n);
}

void dnum_mac(const PrimeConst* pc, const u64* D, const u64* key, u64* acc, int jobs, int total, int dnum,
              LimbMap map, int log_n, cudaStream_t s) {
  if (jobs <= 0) return;
  const size_t per = (size_t)total << log_n;
  size_t blocks = (per + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  ProfScope p("dnum_mac", s);
  k_dnum_mac<<<dim3((unsigned)blocks, jobs), 256, 0, s>>>(pc, D, key, acc, total, dnum, map, log_n);
}

}  // namespace rc
