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

// x[0..8) += lo (HI = false) or hi (HI = true) of a * b[j] at word j, a carry chain of 32-bit multiply-adds with
// carry in cin (0 or 1); returns the carry out of x[7]
template <bool HI>
__device__ __forceinline__ uint32_t mac_chain8(uint32_t* x, uint32_t a, const uint32_t* b, uint32_t cin) {
  uint32_t cout;
  if (HI)
    asm("{\n\t.reg .u32 t;\n\t"
        "add.cc.u32 t, %9, 0xffffffff;\n\t"  // carry flag = (cin != 0)
        "madc.hi.cc.u32 %0, %10, %11, %0;\n\tmadc.hi.cc.u32 %1, %10, %12, %1;\n\t"
        "madc.hi.cc.u32 %2, %10, %13, %2;\n\tmadc.hi.cc.u32 %3, %10, %14, %3;\n\t"
        "madc.hi.cc.u32 %4, %10, %15, %4;\n\tmadc.hi.cc.u32 %5, %10, %16, %5;\n\t"
        "madc.hi.cc.u32 %6, %10, %17, %6;\n\tmadc.hi.cc.u32 %7, %10, %18, %7;\n\t"
        "addc.u32 %8, 0, 0;\n\t}"
        : "+r"(x[0]), "+r"(x[1]), "+r"(x[2]), "+r"(x[3]), "+r"(x[4]), "+r"(x[5]), "+r"(x[6]), "+r"(x[7]),
          "=r"(cout)
        : "r"(cin), "r"(a), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]),
          "r"(b[7]));
  else
    asm("{\n\t.reg .u32 t;\n\t"
        "add.cc.u32 t, %9, 0xffffffff;\n\t"
        "madc.lo.cc.u32 %0, %10, %11, %0;\n\tmadc.lo.cc.u32 %1, %10, %12, %1;\n\t"
        "madc.lo.cc.u32 %2, %10, %13, %2;\n\tmadc.lo.cc.u32 %3, %10, %14, %3;\n\t"
        "madc.lo.cc.u32 %4, %10, %15, %4;\n\tmadc.lo.cc.u32 %5, %10, %16, %5;\n\t"
        "madc.lo.cc.u32 %6, %10, %17, %6;\n\tmadc.lo.cc.u32 %7, %10, %18, %7;\n\t"
        "addc.u32 %8, 0, 0;\n\t}"
        : "+r"(x[0]), "+r"(x[1]), "+r"(x[2]), "+r"(x[3]), "+r"(x[4]), "+r"(x[5]), "+r"(x[6]), "+r"(x[7]),
          "=r"(cout)
        : "r"(cin), "r"(a), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]),
          "r"(b[7]));
  return cout;
}

// X (32-bit words x[0..2WM+2)) += y * (W 64-bit words qh): four carry chains of 32-bit multiply-adds (lo and hi
// halves of y_lo * qh and y_hi * qh) over blocks of eight words, each block's words loaded once for the four
// chains.  Every partial sum stays below 2^(64 W) (W has 8 bits of headroom over Q and the sum is below
// limbs * Q), so no chain carries out of word 2W - 1 and the carries out of the last block are zero.
template <int WM>
__device__ __forceinline__ void crt_mac32(uint32_t (&x)[2 * WM + 2], u64 y, const u64* qh, int W) {
  const uint32_t y0 = (uint32_t)y, y1 = (uint32_t)(y >> 32);
  uint32_t ca = 0, cb = 0, cc = 0, cd = 0;
#pragma unroll
  for (int k = 0; k < WM / 4; ++k) {
    if (4 * k < W) {
      uint32_t b[8];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const u64 v = 4 * k + i < W ? qh[4 * k + i] : 0ull;
        b[2 * i] = (uint32_t)v;
        b[2 * i + 1] = (uint32_t)(v >> 32);
      }
      ca = mac_chain8<false>(x + 8 * k, y0, b, ca);
      cb = mac_chain8<true>(x + 8 * k + 1, y0, b, cb);
      cc = mac_chain8<false>(x + 8 * k + 1, y1, b, cc);
      cd = mac_chain8<true>(x + 8 * k + 2, y1, b, cd);
    }
  }
}

// X (32-bit words) += k * (2^(64 W) - Q) = X - k Q mod 2^(64 W): two carry chains (lo and hi halves) of k times
// the words of 2^(64 W) - Q = ~Q + 1 (Q is odd, so the +1 never carries out of word 0).  Words at 2W and
// above take the carries past 2^(64 W) and are not read.
template <int WM>
__device__ __forceinline__ void crt_sub_kq32(uint32_t (&x)[2 * WM + 2], uint32_t k, const u64* Q, int W) {
  uint32_t ca = 0, cb = 0;
#pragma unroll
  for (int blk = 0; blk < WM / 4; ++blk) {
    if (4 * blk < W) {
      uint32_t b[8];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int w = 4 * blk + i;
        const u64 v = w < W ? (w == 0 ? ~Q[0] + 1 : ~Q[w]) : 0ull;
        b[2 * i] = (uint32_t)v;
        b[2 * i + 1] = (uint32_t)(v >> 32);
      }
      ca = mac_chain8<false>(x + 8 * blk, k, b, ca);
      cb = mac_chain8<true>(x + 8 * blk + 1, k, b, cb);
    }
  }
}

// The centred CRT value of one coefficient: X in (-Q/2, Q/2] as a W-word two's complement number in X[0..W)
// (keyswitching.rs:397-454 up to the digit split; the tie X == floor(Q/2) stays positive).  `in` points at
// limb 0 of the coefficient, limbs N apart; neg negates every residue first (a negacyclic automorphism
// source).  Returns the sign extension word (all ones when X < 0).
template <int WM>
__device__ __forceinline__ u64 centred_crt(const CrtSmem& t, int W, int limbs, const u64* in, u64 N, bool neg,
                                           u64 (&X)[WM]) {
  uint32_t X32[2 * WM + 2];
#pragma unroll
  for (int w = 0; w < 2 * WM + 2; ++w) X32[w] = 0;
  u64 fsum = 0;  // sum of y_l / q_l in units of 2^-31 (each term within 3 units below its value)
  // limb l + 1's residue is requested before limb l's multiply-add chains, so its latency is covered
  u64 rnext = limbs > 0 ? in[0] : 0;
  for (int l = 0; l < limbs; ++l) {
    const u64 q = t.q[l];
    u64 r = rnext;
    if (l + 1 < limbs) rnext = in[(u64)(l + 1) * N];
    if (neg && r) r = q - r;
    const u64 y = mul_shoup(r, t.hinv[l], t.hinv_s[l], q);
    const u64 fx = t.invq[l];
    fsum += __umulhi((uint32_t)((y << (uint32_t)(fx >> 32)) >> 32), (uint32_t)fx);
    crt_mac32<WM>(X32, y, t.qhat + (size_t)l * W, W);  // X += y * (Q / q_l)
  }
  crt_sub_kq32<WM>(X32, (uint32_t)(fsum >> 31), t.Q, W);
#pragma unroll
  for (int w = 0; w < WM; ++w) X[w] = (u64)X32[2 * w] | ((u64)X32[2 * w + 1] << 32);
  u64 top = 0;
#pragma unroll
  for (int w = 0; w < WM; ++w)
    if (w < W) top = X[w];
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
