// Device-side 64-bit modular arithmetic for RNS primes q < 2^61.
//
// The reference computes every product as `(a as u128 * b as u128) % q`
// (src/math/ntt.rs:149-151).  On the GPU a 128-bit division per product is far
// too slow, so this header provides exact replacements that return the same
// canonical residues:
//   * Shoup multiplication by a precomputed constant w (w' = floor(w 2^64 / q)),
//     result in [0, 2q) for any 64-bit input (Harvey's lazy butterflies);
//   * Barrett reduction of a 128-bit value with mu = floor(2^128 / q);
//   * Montgomery reduction (R = 2^64) for the keyswitch inner product, whose
//     key operand is stored premultiplied by R.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>  // defines __device__/__host__ for host-only compilers too

namespace rc {

typedef uint64_t u64;
typedef uint32_t u32;

struct Twiddle {
  u64 w;   // twiddle value in [0, q)
  u64 ws;  // floor(w * 2^64 / q)
};

// twiddles of a pair of 32-bit primes (q0, q1) at one index, with Shoup companions floor(w * 2^32 / q)
struct Tw2 {
  uint32_t w0, w1, s0, s1;
};

// Per-prime constants; one entry per prime of the Q u P chain.
struct PrimeConst {
  u64 q;
  u64 two_q;
  u64 mu_hi, mu_lo;   // floor(2^128 / q) = mu_hi * 2^64 + mu_lo
  u64 qinv_neg;       // -q^-1 mod 2^64
  u64 n_inv, n_inv_s; // N^-1 mod q and its Shoup companion
  u64 r2;             // 2^128 mod q (R^2 for Montgomery conversion)
  u64 mac_chunk;      // products of a lazy NTT output and a key word that sum below q * 2^64
  u64 one_s;          // floor(2^64 / q): Shoup companion of 1 (reduces x < 2^64 to [0, 2q))
  u64 mac_chunk64;    // per-term Montgomery values (< 2q each) that sum below 2^64
  u64 n_inv_r, n_inv_r_s;  // N^-1 2^64 mod q (+ Shoup): the inverse transform's scale after Montgomery products
  // the inverse transform's last stage (global stage 0, one twiddle w1 = psi^-bitrev(1)) times the scale:
  // w1 N^-1 and w1 N^-1 2^64 mod q (+ Shoup)
  u64 w1n, w1n_s, w1nr, w1nr_s;
  u64 pad[3];
};

// The inverse transform's scale folded into its last stage: every butterfly of global stage 0 shares the
// twiddle w1, so its outputs are (x + y) n and (x - y) (w1 n), canonical, and no separate pass multiplies every
// output by n (N^-1 or N^-1 2^64): one Shoup product fewer per stage-0 butterfly
struct InvScale {
  u64 n, n_s, wn, wn_s;
};
// the same for two 29-bit primes (the wide key product's internal primes), 32-bit Shoup companions
struct InvScale2 {
  uint32_t n0, n0s, wn0, wn0s, n1, n1s, wn1, wn1s;
};

#ifdef __CUDACC__
__device__ __forceinline__ u64 mulhi(u64 a, u64 b) { return __umul64hi(a, b); }
__device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b) { return __umulhi(a, b); }
#else
inline u64 mulhi(u64 a, u64 b) { return (u64)(((unsigned __int128)a * b) >> 64); }
inline uint32_t mulhi32(uint32_t a, uint32_t b) { return (uint32_t)(((u64)a * b) >> 32); }
#endif

// a * w mod q lazily: result in [0, 2q) for any a < 2^64 (requires q < 2^63).
__device__ __forceinline__ u64 mul_shoup_lazy(u64 a, u64 w, u64 ws, u64 q) {
  u64 hi = mulhi(a, ws);
  return a * w - hi * q;
}
// a * w mod q in [0, 4q) for any a < 2^64 (q < 2^62).  Shoup's quotient estimated from three of the four
// 32 x 32-bit partial products of a * ws: a1 s1 whole and the high halves of a1 s0 and a0 s1 (their low halves and
// a0 s0 dropped).  The estimate is an integer at most P / 2^64 and above P / 2^64 - 3 (P = a ws), so it is at
// most 2 below the exact floor(P / 2^64) and the remainder is below 2q + 2q.  One 32 x 32 -> 64-bit product and
// two high halves instead of the exact quotient's three and one.
__device__ __forceinline__ u64 mul_shoup_apx(u64 a, u64 w, u64 ws, u64 q) {
  const uint32_t a0 = (uint32_t)a, a1 = (uint32_t)(a >> 32), s0 = (uint32_t)ws, s1 = (uint32_t)(ws >> 32);
  const u64 qh = (u64)a1 * s1 + mulhi32(a1, s0) + mulhi32(a0, s1);
  return a * w - qh * q;
}
__device__ __forceinline__ u64 reduce_2q(u64 x, u64 q) { return x >= q ? x - q : x; }
__device__ __forceinline__ u64 reduce_4q(u64 x, u64 q) {
  u64 two_q = q << 1;
  x = x >= two_q ? x - two_q : x;
  return x >= q ? x - q : x;
}
__device__ __forceinline__ u64 mul_shoup(u64 a, u64 w, u64 ws, u64 q) {
  return reduce_2q(mul_shoup_lazy(a, w, ws, q), q);
}
__device__ __forceinline__ u64 add_mod(u64 a, u64 b, u64 q) {
  u64 s = a + b;
  return s >= q ? s - q : s;
}
__device__ __forceinline__ u64 sub_mod(u64 a, u64 b, u64 q) { return a >= b ? a - b : a + q - b; }

// 128-bit helpers -------------------------------------------------------------
struct U128 {
  u64 lo, hi;
};
__device__ __forceinline__ U128 mul_wide(u64 a, u64 b) {
  U128 r;
  r.lo = a * b;
  r.hi = mulhi(a, b);
  return r;
}
__device__ __forceinline__ void add_to(U128& acc, const U128& x) {
  u64 lo = acc.lo + x.lo;
  acc.hi += x.hi + (lo < x.lo ? 1ull : 0ull);
  acc.lo = lo;
}
// acc -= x (x <= acc)
__device__ __forceinline__ void sub_from(U128& acc, const U128& x) {
  const u64 borrow = acc.lo < x.lo ? 1ull : 0ull;
  acc.lo -= x.lo;
  acc.hi -= x.hi + borrow;
}

// Barrett: t mod q for t < q * 2^64, q < 2^61.  The quotient estimate keeps the
// middle-word carries, so it is at most 2 below the true quotient.
__device__ __forceinline__ u64 barrett_reduce(U128 t, const PrimeConst& c) {
  u64 a = mulhi(t.lo, c.mu_lo);
  u64 b_lo = t.lo * c.mu_hi, b_hi = mulhi(t.lo, c.mu_hi);
  u64 c_lo = t.hi * c.mu_lo, c_hi = mulhi(t.hi, c.mu_lo);
  u64 s = a + b_lo;
  u64 carry = s < a ? 1ull : 0ull;
  u64 s2 = s + c_lo;
  carry += s2 < s ? 1ull : 0ull;
  u64 qhat = t.hi * c.mu_hi + b_hi + c_hi + carry;
  u64 r = t.lo - qhat * c.q;
  r = r >= c.q ? r - c.q : r;
  r = r >= c.q ? r - c.q : r;
  return r;
}
__device__ __forceinline__ u64 mul_mod(u64 a, u64 b, const PrimeConst& c) { return barrett_reduce(mul_wide(a, b), c); }

// Montgomery: t * 2^-64 mod q for t < q * 2^64, before its final conditional subtraction: in [0, 2q)
__device__ __forceinline__ u64 mont_reduce_lazy(U128 t, const PrimeConst& c) {
  u64 m = t.lo * c.qinv_neg;
  U128 mq = mul_wide(m, c.q);
  return t.hi + mq.hi + (t.lo != 0 ? 1ull : 0ull);
}
// Montgomery: t * 2^-64 mod q for t < q * 2^64; result in [0, q).
__device__ __forceinline__ u64 mont_reduce(U128 t, const PrimeConst& c) {
  u64 m = t.lo * c.qinv_neg;
  U128 mq = mul_wide(m, c.q);
  // t + m*q is divisible by 2^64; its low word is zero, carry out iff t.lo != 0
  u64 hi = t.hi + mq.hi + (t.lo != 0 ? 1ull : 0ull);
  return hi >= c.q ? hi - c.q : hi;
}

}  // namespace rc
