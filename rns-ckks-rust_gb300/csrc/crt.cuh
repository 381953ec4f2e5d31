// Centred CRT reconstruction of one coefficient from its residues, shared by the decomposition, the lift to
// the aux basis and the device decoder: the value X in (-Q/2, Q/2] (the tie X == floor(Q/2) stays positive,
// keyswitching.rs:397-454 and polynomial.rs:162-201) as a W-word two's complement number.
#pragma once
#include "kernels.cuh"
#include "modarith.cuh"

namespace rc {

// The CRT tables every thread of a decomposition or lift walks (words of Q/q_l, (Q/q_l)^-1, q_l, 1/q_l,
// Q, floor(Q/2)), staged in shared memory by all threads of the block; the caller synchronises.
struct CrtSmem {
  const u64 *qhat, *q, *hinv, *hinv_s;
  const u64* invq;  // fixed-point 1/q_l (DecompTab::inv_q)
  const u64 *Q, *half;
};

__device__ __forceinline__ CrtSmem stage_crt_tables(const PrimeConst* pc, const DecompTab& dt, int limbs) {
  extern __shared__ u64 dsm_tab[];
  const int W = dt.W;
  u64* s_qhat = dsm_tab;                       // [limbs][W]
  u64* s_q = s_qhat + (size_t)limbs * W;       // [limbs]
  u64* s_hinv = s_q + limbs;                   // [limbs]
  u64* s_hinv_s = s_hinv + limbs;              // [limbs]
  u64* s_invq = s_hinv_s + limbs;              // [limbs]
  u64* s_Q = s_invq + limbs;                   // [W]
  u64* s_half = s_Q + W;                       // [W]
  for (int e = threadIdx.x; e < limbs * W; e += blockDim.x) s_qhat[e] = dt.qhat[e];
  for (int e = threadIdx.x; e < limbs; e += blockDim.x) {
    s_q[e] = pc[e].q;
    s_hinv[e] = dt.qhat_inv[e];
    s_hinv_s[e] = dt.qhat_inv_s[e];
    s_invq[e] = dt.inv_q[e];
  }
  for (int e = threadIdx.x; e < W; e += blockDim.x) {
    s_Q[e] = dt.Q[e];
    s_half[e] = dt.halfQ[e];
  }
  return CrtSmem{s_qhat, s_q, s_hinv, s_hinv_s, s_invq, s_Q, s_half};
}

inline size_t crt_smem_bytes(int limbs, int W) { return ((size_t)limbs * W + 4 * (size_t)limbs + 2 * (size_t)W) * 8; }

// The centred CRT value of one coefficient: X in (-Q/2, Q/2] as a W-word two's complement number in X[0..W)
// (keyswitching.rs:397-454 up to the digit split; the tie X == floor(Q/2) stays positive).  `in` points at
// limb 0 of the coefficient, limbs N apart; neg negates every residue first (a negacyclic automorphism
// source).  Returns the sign extension word (all ones when X < 0).
template <int WM>
__device__ __forceinline__ u64 centred_crt(const CrtSmem& t, int W, int limbs, const u64* in, u64 N, bool neg,
                                           u64 (&X)[WM]) {
#pragma unroll
  for (int w = 0; w < WM; ++w) X[w] = 0;
  u64 fsum = 0;  // sum of y_l / q_l in units of 2^-31 (each term within 3 units below its value)
  for (int l = 0; l < limbs; ++l) {
    const u64 q = t.q[l];
    u64 r = in[(u64)l * N];
    if (neg && r) r = q - r;
    const u64 y = mul_shoup(r, t.hinv[l], t.hinv_s[l], q);
    const u64 fx = t.invq[l];
    fsum += __umulhi((uint32_t)((y << (uint32_t)(fx >> 32)) >> 32), (uint32_t)fx);
    const u64* qh = t.qhat + (size_t)l * W;
    u64 carry = 0;
#pragma unroll
    for (int w = 0; w < WM; ++w) {
      if (w < W) {
        U128 p = mul_wide(y, qh[w]);
        u64 lo = p.lo + X[w];
        u64 c1 = lo < X[w] ? 1ull : 0ull;
        u64 lo2 = lo + carry;
        u64 c2 = lo2 < carry ? 1ull : 0ull;
        X[w] = lo2;
        carry = p.hi + c1 + c2;
      }
    }
  }
  // X' = X - k*Q with k = floor(sum y_i / q_i) (exact up to +-1, fixed below).  `top` follows the
  // word W-1 as each pass writes it: reading X[W-1] afterwards would index X dynamically and move it to
  // local memory.
  u64 k = fsum >> 31;
  u64 top = 0;
  {
    u64 borrow = 0, carry = 0;
#pragma unroll
    for (int w = 0; w < WM; ++w) {
      if (w < W) {
        U128 p = mul_wide(k, t.Q[w]);
        u64 sub = p.lo + carry;
        carry = p.hi + (sub < carry ? 1ull : 0ull);
        u64 xw = X[w];
        u64 d = xw - sub;
        u64 b1 = xw < sub ? 1ull : 0ull;
        u64 d2 = d - borrow;
        u64 b2 = d < borrow ? 1ull : 0ull;
        X[w] = d2;
        top = d2;
        borrow = b1 + b2;
      }
    }
  }
  // X is now in [-Q, 2Q) as a W-word two's complement value
  auto top_neg = [&]() -> bool { return (top >> 63) != 0; };
  auto add_Q = [&](bool subtract) {
    u64 c = 0;
#pragma unroll
    for (int w = 0; w < WM; ++w) {
      if (w < W) {
        u64 qw = t.Q[w];
        if (!subtract) {
          u64 s = X[w] + qw;
          u64 c1 = s < qw ? 1ull : 0ull;
          u64 s2 = s + c;
          u64 c2 = s2 < c ? 1ull : 0ull;
          X[w] = s2;
          top = s2;
          c = c1 + c2;
        } else {
          u64 d = X[w] - qw;
          u64 b1 = X[w] < qw ? 1ull : 0ull;
          u64 d2 = d - c;
          u64 b2 = d < c ? 1ull : 0ull;
          X[w] = d2;
          top = d2;
          c = b1 + b2;
        }
      }
    }
  };
  // compare X (non-negative) with a W-word constant: returns X > C
  auto greater_than = [&](const u64* C, bool or_equal) -> bool {
    int res = 0;  // 0 equal so far, 1 greater, -1 less (from the top)
#pragma unroll
    for (int w = WM - 1; w >= 0; --w) {
      if (w < W && res == 0) {
        if (X[w] > C[w]) res = 1;
        else if (X[w] < C[w]) res = -1;
      }
    }
    return res > 0 || (or_equal && res == 0);
  };
  if (top_neg()) add_Q(false);
  else if (greater_than(t.Q, true)) add_Q(true);
  // centre: X > floor(Q/2) -> X - Q
  if (greater_than(t.half, false)) add_Q(true);
  return top_neg() ? ~0ull : 0ull;
}

}  // namespace rc
