// Minimal unsigned multiprecision integers for host-side precomputation
// (products of RNS primes, CRT constants, centring thresholds).  Little-endian
// 64-bit words.  Only what the context set-up needs; no GMP dependency.
#pragma once
#include <algorithm>
#include <cstdint>
#include <vector>

namespace rc {

typedef unsigned __int128 u128h;

struct BigU {
  std::vector<uint64_t> w;  // little-endian, no trailing zero words (zero = empty)

  BigU() {}
  explicit BigU(uint64_t v) {
    if (v) w.push_back(v);
  }
  void trim() {
    while (!w.empty() && w.back() == 0) w.pop_back();
  }
  bool is_zero() const { return w.empty(); }
  size_t bits() const {
    if (w.empty()) return 0;
    return (w.size() - 1) * 64 + (64 - __builtin_clzll(w.back()));
  }
  BigU mul_u64(uint64_t m) const {
    BigU r;
    u128h carry = 0;
    for (uint64_t x : w) {
      u128h p = (u128h)x * m + carry;
      r.w.push_back((uint64_t)p);
      carry = p >> 64;
    }
    if (carry) r.w.push_back((uint64_t)carry);
    r.trim();
    return r;
  }
  BigU add(const BigU& o) const {
    BigU r;
    size_t n = std::max(w.size(), o.w.size());
    uint64_t carry = 0;
    for (size_t i = 0; i < n; ++i) {
      uint64_t a = i < w.size() ? w[i] : 0, b = i < o.w.size() ? o.w[i] : 0;
      u128h s = (u128h)a + b + carry;
      r.w.push_back((uint64_t)s);
      carry = (uint64_t)(s >> 64);
    }
    if (carry) r.w.push_back(carry);
    r.trim();
    return r;
  }
  // requires *this >= o
  BigU sub(const BigU& o) const {
    BigU r;
    uint64_t borrow = 0;
    for (size_t i = 0; i < w.size(); ++i) {
      uint64_t a = w[i], b = i < o.w.size() ? o.w[i] : 0;
      u128h need = (u128h)b + borrow;
      r.w.push_back(a - (uint64_t)need);
      borrow = need > (u128h)a ? 1 : 0;
    }
    r.trim();
    return r;
  }
  int cmp(const BigU& o) const {
    if (w.size() != o.w.size()) return w.size() < o.w.size() ? -1 : 1;
    for (size_t i = w.size(); i-- > 0;)
      if (w[i] != o.w[i]) return w[i] < o.w[i] ? -1 : 1;
    return 0;
  }
  BigU shr1() const {
    BigU r;
    r.w.resize(w.size());
    for (size_t i = 0; i < w.size(); ++i) {
      uint64_t hi = i + 1 < w.size() ? w[i + 1] : 0;
      r.w[i] = (w[i] >> 1) | (hi << 63);
    }
    r.trim();
    return r;
  }
  uint64_t mod_u64(uint64_t m) const {
    u128h r = 0;
    for (size_t i = w.size(); i-- > 0;) r = ((r << 64) | w[i]) % m;
    return (uint64_t)r;
  }
  // exact division by a u64 that divides *this
  BigU div_u64(uint64_t m) const {
    BigU r;
    r.w.resize(w.size());
    u128h rem = 0;
    for (size_t i = w.size(); i-- > 0;) {
      u128h cur = (rem << 64) | w[i];
      r.w[i] = (uint64_t)(cur / m);
      rem = cur % m;
    }
    r.trim();
    return r;
  }
  std::vector<uint64_t> words(size_t n) const {
    std::vector<uint64_t> out(n, 0);
    for (size_t i = 0; i < w.size() && i < n; ++i) out[i] = w[i];
    return out;
  }
};

inline BigU product(const std::vector<uint64_t>& m, size_t begin, size_t end) {
  BigU r(1);
  for (size_t i = begin; i < end; ++i) r = r.mul_u64(m[i]);
  return r;
}

inline uint64_t mulmod_h(uint64_t a, uint64_t b, uint64_t m) { return (uint64_t)(((u128h)a * b) % m); }
inline uint64_t powmod_h(uint64_t b, uint64_t e, uint64_t m) {
  uint64_t r = 1 % m;
  b %= m;
  while (e) {
    if (e & 1) r = mulmod_h(r, b, m);
    b = mulmod_h(b, b, m);
    e >>= 1;
  }
  return r;
}
// modular inverse by extended Euclid (0 when not invertible)
inline uint64_t invmod_h(uint64_t v, uint64_t m) {
  __int128 t = 0, nt = 1, r = m, nr = v % m;
  while (nr) {
    __int128 q = r / nr, tmp;
    tmp = t - q * nt; t = nt; nt = tmp;
    tmp = r - q * nr; r = nr; nr = tmp;
  }
  if (r != 1) return 0;
  if (t < 0) t += m;
  return (uint64_t)t;
}
inline uint64_t shoup_h(uint64_t w, uint64_t q) { return (uint64_t)(((u128h)w << 64) / q); }

// deterministic Miller-Rabin for 64-bit integers
inline bool is_prime_u64(uint64_t n) {
  if (n < 2) return false;
  static const uint64_t small[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
  for (uint64_t p : small)
    if (n % p == 0) return n == p;
  uint64_t d = n - 1;
  int s = 0;
  while ((d & 1) == 0) {
    d >>= 1;
    ++s;
  }
  for (uint64_t a : small) {
    uint64_t x = powmod_h(a, d, n);
    if (x == 1 || x == n - 1) continue;
    bool comp = true;
    for (int r = 1; r < s; ++r) {
      x = mulmod_h(x, x, n);
      if (x == n - 1) {
        comp = false;
        break;
      }
    }
    if (comp) return false;
  }
  return true;
}

}  // namespace rc
