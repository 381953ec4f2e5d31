// RNS-hybrid key switching ("dnum" gadget; no counterpart in the reference, whose only gadget is balanced
// base-2^30 digits, src/rns/keyswitching.rs:238-240).  The active chain Q_l is cut into dnum groups of alpha
// consecutive limbs; group b's part of the polynomial, [c]_{Q_b}, is extended to Q_l u P by a fast basis
// conversion (ModUp: sum_i [c_i (Q_b/q_i)^-1]_{q_i} (Q_b/q_i) mod t, exact up to a multiple of Q_b that the key
// annihilates), multiplied in the NTT domain by key b and summed; ModDown by P (the exact centred conversion
// of k_finalize) brings it back to Q_l.  Key b encrypts [i in group b] (P mod q_i) s^2, so the result
// decrypts to c s^2 plus the keys' noise divided by P.  Results are not the reference's residues (a different
// gadget); they decrypt to the same values.
#include <stdexcept>
#include <type_traits>

#include "kernels.cuh"

namespace rc {

namespace {

// D[job][b][limb][N] for limb in 0..total-1 (Q limbs then aux limbs) from the job's coefficient-form
// polynomial src.p[job] ([qlimbs][N]).  tab holds, per group b: (Q_b/q_i)^-1 mod q_i and its Shoup companion
// for the group's limbs, then (Q_b/q_i) mod t for every target limb t: [dnum][alpha][2 + total].  A = alpha
// (the last group may hold fewer limbs).
template <int A>
__global__ void k_dnum_modup(const PrimeConst* pc, PtrTab src, const u64* tab, u64* D, int qlimbs, int total,
                             int dnum, LimbMap map, int log_n) {
  extern __shared__ u64 st[];  // group b's [A][2 + total] table
  const int b = blockIdx.y, job = blockIdx.z;
  const int row = 2 + total;
  const u64* tb = tab + (size_t)b * A * row;
  for (int e = threadIdx.x; e < A * row; e += blockDim.x) st[e] = tb[e];
  __syncthreads();
  const u64 N = 1ull << log_n;
  const u64 x = blockIdx.x * (u64)blockDim.x + threadIdx.x;
  if (x >= N) return;
  const int i0 = b * A, n = min(A, qlimbs - i0);
  const u64* in = src.p[job];
  u64* out = D + ((size_t)job * dnum + b) * total * N + x;
  u64 y[A];
#pragma unroll
  for (int k = 0; k < A; ++k) {
    y[k] = 0;  // a short last group contributes nothing past its limbs
    if (k < n) {
      const int i = i0 + k;
      const u64 c = in[(size_t)i * N + x];
      out[(size_t)i * N] = c;  // the group's own limbs are the polynomial's residues
      y[k] = mul_shoup(c, st[k * row], st[k * row + 1], pc[i].q);
    }
  }
  for (int t = 0; t < total; ++t) {
    if (t >= i0 && t < i0 + n) continue;
    const PrimeConst& pt = pc[map.prime(t)];
    U128 acc{0, 0};
#pragma unroll
    for (int k = 0; k < A; ++k) add_to(acc, mul_wide(y[k], st[k * row + 2 + t]));
    out[(size_t)t * N] = barrett_reduce(acc, pt);
  }
}

// acc[job][c][limb] = sum_b D[job][b][limb] * key[b][c][limb] mod t, NTT domain, for the jobs of one run
// sharing the key: a thread keeps its element's 2 DN key words in registers and sweeps the jobs, so the key
// is read once per launch (sums of DN <= 16 terms below q 2^64 in 128 bits, one Barrett reduction each)
template <int DN>
__global__ void k_dnum_mac(const PrimeConst* pc, const u64* D, const u64* key, u64* acc, int jobs, int total,
                           LimbMap map, int log_n) {
  const size_t per = (size_t)total << log_n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < per; e += (size_t)gridDim.x * blockDim.x) {
    const PrimeConst& c = pc[map.prime((int)(e >> log_n))];
    u64 k0[DN], k1[DN];
#pragma unroll
    for (int b = 0; b < DN; ++b) {
      k0[b] = key[(size_t)b * 2 * per + e];
      k1[b] = key[((size_t)b * 2 + 1) * per + e];
    }
    for (int j = 0; j < jobs; ++j) {
      const u64* d = D + (size_t)j * DN * per + e;
      U128 t0{0, 0}, t1{0, 0};
#pragma unroll
      for (int b = 0; b < DN; ++b) {
        const u64 v = d[(size_t)b * per];
        add_to(t0, mul_wide(v, k0[b]));
        add_to(t1, mul_wide(v, k1[b]));
      }
      u64* a = acc + (size_t)j * 2 * per + e;
      a[0] = barrett_reduce(t0, c);
      a[per] = barrett_reduce(t1, c);
    }
  }
}

template <int... V>
struct IntList {};

// calls f(std::integral_constant<int, v>) for the v of the list equal to x; false if none is
template <class F, int V0, int... V>
bool dispatch_int(int x, IntList<V0, V...>, F&& f) {
  if (x == V0) {
    f(std::integral_constant<int, V0>{});
    return true;
  }
  if constexpr (sizeof...(V) > 0) return dispatch_int(x, IntList<V...>{}, f);
  return false;
}

}  // namespace

void dnum_modup(const PrimeConst* pc, const PtrTab& src, int jobs, const u64* tab, u64* D, int qlimbs, int total,
                int alpha, int dnum, LimbMap map, int log_n, cudaStream_t s) {
  if (jobs <= 0) return;
  const int N = 1 << log_n;
  const int threads = N < 128 ? N : 128;
  dim3 g((N + threads - 1) / threads, dnum, jobs);
  ProfScope p("dnum_modup", s);
  const size_t smem = (size_t)alpha * (2 + total) * 8;
  const bool ok = dispatch_int(alpha, IntList<1, 2, 3, 4, 5, 6, 7, 8>{}, [&](auto a) {
    k_dnum_modup<decltype(a)::value><<<g, threads, smem, s>>>(pc, src, tab, D, qlimbs, total, dnum, map, log_n);
  });
  if (!ok) throw std::runtime_error("internal: RNS-hybrid group size outside 1..8");
}

void dnum_mac(const PrimeConst* pc, const u64* D, const u64* key, u64* acc, int jobs, int total, int dnum,
              LimbMap map, int log_n, cudaStream_t s) {
  if (jobs <= 0) return;
  const size_t per = (size_t)total << log_n;
  size_t blocks = (per + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  ProfScope p("dnum_mac", s);
  const bool ok = dispatch_int(dnum, IntList<1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16>{}, [&](auto d) {
    k_dnum_mac<decltype(d)::value><<<(unsigned)blocks, 256, 0, s>>>(pc, D, key, acc, jobs, total, map, log_n);
  });
  if (!ok) throw std::runtime_error("internal: RNS-hybrid group count outside 1..16");
}

}  // namespace rc
