// Device helpers of the exact integer key product ("wide-CRT") under the four
// internal primes w0..w3 < 2^29 (see wide.cu).
#pragma once
#include "kernels.cuh"

namespace rc {

__device__ __forceinline__ uint32_t mul_shoup32(uint32_t x, uint32_t w, uint32_t ws, uint32_t q) {
  const uint32_t r = x * w - __umulhi(x, ws) * q;
  return min(r, r - q);  // r - q wraps above r when r < q
}

// x mod q for any 64-bit x (bar = floor(2^64 / q))
__device__ __forceinline__ uint32_t reduce64_32(u64 x, uint32_t q, u64 bar) {
  const u64 r = x - __umul64hi(x, bar) * q;
  return (uint32_t)(r >= q ? r - q : r);
}

// x 2^-32 mod q in [0, q) for any 64-bit x, q < 2^29 (qn = -q^-1 mod 2^32, kq = floor(2^31 / q) q): one 32-bit
// and one 32 x 32 -> 64-bit multiply instead of reduce64_32's 64 x 64 high product.  An x at or above 2^63 first
// loses kq 2^32 (a multiple of q, at most 2^63 and above 2^63 - q 2^32), so x + m q stays below 2^63 + 2^62;
// the quotient by 2^32 is then below 3 2^30 < 8q, and three conditional subtractions finish it
__device__ __forceinline__ uint32_t mont64_32(u64 x, uint32_t q, uint32_t qn, uint32_t kq) {
  if (x >> 63) x -= (u64)kq << 32;
  const uint32_t m = (uint32_t)x * qn;
  uint32_t t = (uint32_t)((x + (u64)m * q) >> 32);
  t = t >= 4 * q ? t - 4 * q : t;
  t = t >= 2 * q ? t - 2 * q : t;
  return t >= q ? t - q : t;
}

// a - b mod q for a, b < q
__device__ __forceinline__ uint32_t sub32(uint32_t a, uint32_t b, uint32_t q) { return a >= b ? a - b : a + q - b; }

// v < 2q -> v mod q
__device__ __forceinline__ uint32_t fold32(uint32_t v, uint32_t q) { return min(v, v - q); }

// wide_crt_mod with the per-prime constants passed in: S * F mod q for a factor F given as
// (F mod q + Shoup) = (lo_w, lo_ws), (w0 w1 F) mod q + Shoup = (c01, c01_s) and (A F) mod q = a_mod
// (F = 1: lo_w = 1, lo_ws = floor(2^64 / q))
__device__ __forceinline__ u64 wide_crt_mod_c(uint2 p01, uint2 p23, const WideTab& W, u64 q, u64 lo_w, u64 lo_ws,
                                              u64 c01, u64 c01_s, u64 a_mod) {
  const uint32_t w1 = W.w[1], w2 = W.w[2], w3 = W.w[3];
  const uint32_t v0 = p01.x;
  const uint32_t v1 = mul_shoup32(sub32(p01.y, fold32(v0, w1), w1), W.g01, W.g01s, w1);
  uint32_t a = mul_shoup32(sub32(p23.x, fold32(v0, w2), w2), W.g02, W.g02s, w2);
  const uint32_t v2 = mul_shoup32(sub32(a, fold32(v1, w2), w2), W.g12, W.g12s, w2);
  uint32_t b = mul_shoup32(sub32(p23.y, fold32(v0, w3), w3), W.g03, W.g03s, w3);
  b = mul_shoup32(sub32(b, fold32(v1, w3), w3), W.g13, W.g13s, w3);
  const uint32_t v3 = mul_shoup32(sub32(b, fold32(v2, w3), w3), W.g23, W.g23s, w3);
  const u64 lo = (u64)v0 + (u64)W.w[0] * v1;
  const u64 hi = (u64)v2 + (u64)w2 * v3;
  u64 r = reduce_4q(mul_shoup_lazy(lo, lo_w, lo_ws, q) + mul_shoup_lazy(hi, c01, c01_s, q), q);
  if (v3 >= W.half3) r = sub_mod(r, a_mod, q);
  return r;
}

// wide_crt_mod_c before its reduction, for a caller that sums further lazy terms: a value below 9q congruent
// to S * F mod q (its two 64-bit products are approximate Shoup products, below 4q each), where
// namod = (q - (A F mod q)) mod q is what a negative S adds
__device__ __forceinline__ u64 wide_crt_lazy(uint2 p01, uint2 p23, const WideTab& W, u64 q, u64 lo_w, u64 lo_ws,
                                            u64 c01, u64 c01_s, u64 namod) {
  const uint32_t w1 = W.w[1], w2 = W.w[2], w3 = W.w[3];
  const uint32_t v0 = p01.x;
  const uint32_t v1 = mul_shoup32(sub32(p01.y, fold32(v0, w1), w1), W.g01, W.g01s, w1);
  uint32_t a = mul_shoup32(sub32(p23.x, fold32(v0, w2), w2), W.g02, W.g02s, w2);
  const uint32_t v2 = mul_shoup32(sub32(a, fold32(v1, w2), w2), W.g12, W.g12s, w2);
  uint32_t b = mul_shoup32(sub32(p23.y, fold32(v0, w3), w3), W.g03, W.g03s, w3);
  b = mul_shoup32(sub32(b, fold32(v1, w3), w3), W.g13, W.g13s, w3);
  const uint32_t v3 = mul_shoup32(sub32(b, fold32(v2, w3), w3), W.g23, W.g23s, w3);
  const u64 lo = (u64)v0 + (u64)W.w[0] * v1;
  const u64 hi = (u64)v2 + (u64)w2 * v3;
  u64 r = mul_shoup_apx(lo, lo_w, lo_ws, q) + mul_shoup_apx(hi, c01, c01_s, q);
  return v3 >= W.half3 ? r + namod : r;
}

// Centred S from (S mod w0, S mod w1) = p01 and (S mod w2, S mod w3) = p23,
// reduced mod the scheme prime t.  Garner: S = v0 + w0 v1 + w0 w1 v2 + w0 w1 w2 v3
// with v_i < w_i; with |S| < A/4 the sign of the centred value is v3 >= (w3+1)/2.
// S mod t = (v0 + w0 v1) + (w0 w1 mod t) (v2 + w2 v3): both halves are < 2^58.
__device__ __forceinline__ u64 wide_crt_mod(uint2 p01, uint2 p23, const WideTab& W, int t, const PrimeConst& c) {
  const uint32_t w1 = W.w[1], w2 = W.w[2], w3 = W.w[3];
  const uint32_t v0 = p01.x;
  const uint32_t v1 = mul_shoup32(sub32(p01.y, fold32(v0, w1), w1), W.g01, W.g01s, w1);
  uint32_t a = mul_shoup32(sub32(p23.x, fold32(v0, w2), w2), W.g02, W.g02s, w2);
  const uint32_t v2 = mul_shoup32(sub32(a, fold32(v1, w2), w2), W.g12, W.g12s, w2);
  uint32_t b = mul_shoup32(sub32(p23.y, fold32(v0, w3), w3), W.g03, W.g03s, w3);
  b = mul_shoup32(sub32(b, fold32(v1, w3), w3), W.g13, W.g13s, w3);
  const uint32_t v3 = mul_shoup32(sub32(b, fold32(v2, w3), w3), W.g23, W.g23s, w3);
  const u64 lo = (u64)v0 + (u64)W.w[0] * v1;
  const u64 hi = (u64)v2 + (u64)w2 * v3;
  // two lazy Shoup products in [0, 2q) each, one reduction of their sum from [0, 4q)
  u64 r = reduce_4q(mul_shoup_lazy(lo, 1, c.one_s, c.q) + mul_shoup_lazy(hi, W.c01_mod_t[t], W.c01_mod_t_s[t], c.q),
                    c.q);
  if (v3 >= W.half3) r = sub_mod(r, W.A_mod_t[t], c.q);
  return r;
}

}  // namespace rc
