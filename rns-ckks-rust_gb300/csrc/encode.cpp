// Host FP64 CKKS encode/decode (the reference keeps these on the CPU in FP64:
// src/rns/encoding.rs:9-88, src/math/canonical_embedding.rs:21-79).
//
// Same operation order as the reference: bit reversal + radix-2 DIT FFT whose
// twiddle advances by recurrence (w *= w_len), xi^(+-i) by exponentiation by
// squaring, complex products (ac - bd, ad + bc), rounding half away from zero.
// Built with -ffp-contract=off so no multiply-add is fused.
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "context.hpp"

using namespace rc;

namespace {

struct C {
  double re, im;
};
inline C cmul(C a, C b) { return C{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline C cadd(C a, C b) { return C{a.re + b.re, a.im + b.im}; }
inline C csub(C a, C b) { return C{a.re - b.re, a.im - b.im}; }
inline C polar(double theta) { return C{1.0 * std::cos(theta), 1.0 * std::sin(theta)}; }

// num-complex powi: inverse for negative exponents, then exponentiation by
// squaring in num-traits' order
C cpowi(C z, long e) {
  if (e < 0) {
    double d = z.re * z.re + z.im * z.im;
    z = C{z.re / d, 0.0 - z.im / d};
    e = -e;
  }
  if (e == 0) return C{1.0, 0.0};
  C base = z;
  while ((e & 1) == 0) {
    base = cmul(base, base);
    e >>= 1;
  }
  if (e == 1) return base;
  C acc = base;
  while (e > 1) {
    e >>= 1;
    base = cmul(base, base);
    if (e & 1) acc = cmul(acc, base);
  }
  return acc;
}

// fft_in_place, canonical_embedding.rs:44-79
void fft_in_place(std::vector<C>& v, bool inverse) {
  const size_t n = v.size();
  size_t j = 0;
  for (size_t i = 1; i < n; ++i) {
    size_t bit = n >> 1;
    while (j & bit) {
      j ^= bit;
      bit >>= 1;
    }
    j ^= bit;
    if (i < j) std::swap(v[i], v[j]);
  }
  for (size_t len = 2; len <= n; len <<= 1) {
    const double angle = inverse ? -2.0 * M_PI / (double)len : 2.0 * M_PI / (double)len;
    const C w_len = polar(angle);
    for (size_t c = 0; c < n; c += len) {
      C w{1.0, 0.0};
      for (size_t i = 0; i < len / 2; ++i) {
        C u = v[c + i];
        C t = cmul(v[c + i + len / 2], w);
        v[c + i] = cadd(u, t);
        v[c + i + len / 2] = csub(u, t);
        w = cmul(w, w_len);
      }
    }
  }
  if (inverse) {
    const double s = 1.0 / (double)n;
    for (auto& x : v) x = C{x.re * s, x.im * s};
  }
}

std::vector<size_t> slot_exponents(size_t n) {
  std::vector<size_t> e(n / 2);
  size_t cur = 1;
  for (size_t i = 0; i < n / 2; ++i) {
    e[i] = cur;
    cur = cur * 5 % (2 * n);
  }
  return e;
}

// f64::round then `as i128` (saturating)
__int128 round_to_i128(double x) {
  double r = std::round(x);  // half away from zero, like Rust's f64::round
  if (std::isnan(r)) return 0;
  const double lim = 1.7014118346046923e38;  // 2^127
  if (r >= lim) return (__int128)(((unsigned __int128)1 << 127) - 1);
  if (r <= -lim) return -(__int128)(((unsigned __int128)1 << 127) - 1) - 1;
  return (__int128)r;
}

uint64_t mod_i128(__int128 v, uint64_t q) {
  __int128 r = v % (__int128)q;
  if (r < 0) r += q;
  return (uint64_t)r;
}

// correctly rounded conversion of a multiword magnitude to double
double words_to_double(const std::vector<uint64_t>& w) {
  size_t top = w.size();
  while (top > 0 && w[top - 1] == 0) --top;
  if (top == 0) return 0.0;
  const int lz = __builtin_clzll(w[top - 1]);
  const size_t bits = top * 64 - lz;
  if (bits <= 64) return (double)w[0];
  // top 64 bits with a sticky bit for everything below
  const size_t shift = bits - 64;
  const size_t ws = shift / 64, bs = shift % 64;
  uint64_t m = w[ws] >> bs;
  if (bs && ws + 1 < w.size()) m |= w[ws + 1] << (64 - bs);
  bool sticky = (bs && (w[ws] & ((1ull << bs) - 1))) != 0;
  for (size_t i = 0; i < ws && !sticky; ++i) sticky = w[i] != 0;
  if (sticky) m |= 1;
  return std::ldexp((double)m, (int)shift);
}

}  // namespace

extern "C" int rc_encode(const rc_context* c, const double* slots, int32_t level, uint32_t scale_bits,
                         uint64_t* out) {
  try {
    if (!c || !slots || !out) return RC_ERR_INVALID_ARGUMENT;
    if (level < 0 || level >= c->L) return RC_ERR_INVALID_ARGUMENT;
    const size_t n = (size_t)c->N;
    std::vector<C> evals(n, C{0.0, 0.0});
    auto ex = slot_exponents(n);
    for (size_t k = 0; k < n / 2; ++k) {
      const C v{slots[2 * k], slots[2 * k + 1]};
      const size_t e = ex[k];
      evals[(e - 1) / 2] = v;
      evals[(((2 * n - e) % (2 * n)) - 1) / 2] = C{v.re, -v.im};
    }
    fft_in_place(evals, true);
    const C xi = polar(M_PI / (double)n);
    const double scale = std::pow(2.0, (double)scale_bits);  // 2f64.powi(scale_bits)
    const int limbs = level + 1;
    for (size_t i = 0; i < n; ++i) {
      const C tw = cmul(evals[i], cpowi(xi, -(long)i));
      const __int128 v = round_to_i128(tw.re * scale);
      for (int l = 0; l < limbs; ++l) out[(size_t)l * n + i] = mod_i128(v, c->mod[l]);
    }
    return RC_OK;
  } catch (...) {
    return RC_ERR_CUDA;
  }
}

extern "C" int rc_decode(const rc_context* c, const uint64_t* poly, int32_t level, uint32_t scale_bits,
                         double* slots_out) {
  try {
    if (!c || !poly || !slots_out) return RC_ERR_INVALID_ARGUMENT;
    if (level < 0 || level >= c->L) return RC_ERR_INVALID_ARGUMENT;
    const size_t n = (size_t)c->N;
    const int limbs = level + 1;
    const std::vector<uint64_t>& m = c->mod;
    BigU Q = product(m, 0, limbs);
    BigU half = Q.shr1();
    // Garner constants
    std::vector<uint64_t> inv((size_t)limbs * limbs, 0);
    for (int i = 0; i < limbs; ++i)
      for (int j = 0; j < i; ++j) inv[(size_t)i * limbs + j] = invmod_h(m[j] % m[i], m[i]);
    const double inv_delta = 1.0 / std::pow(2.0, (double)scale_bits);
    const C xi = polar(M_PI / (double)n);
    std::vector<C> b(n);
    std::vector<uint64_t> v(limbs);
    for (size_t x = 0; x < n; ++x) {
      for (int i = 0; i < limbs; ++i) {
        uint64_t val = poly[(size_t)i * n + x] % m[i];
        for (int j = 0; j < i; ++j) {
          uint64_t vj = v[j] % m[i];
          val = val >= vj ? val - vj : val + m[i] - vj;
          val = mulmod_h(val, inv[(size_t)i * limbs + j], m[i]);
        }
        v[i] = val;
      }
      BigU X(v[limbs - 1]);
      for (int i = limbs - 2; i >= 0; --i) X = X.mul_u64(m[i]).add(BigU(v[i]));
      double d;
      if (X.cmp(half) <= 0) d = words_to_double(X.w);
      else d = -words_to_double(Q.sub(X).w);
      b[x] = cmul(C{d * inv_delta, 0.0}, cpowi(xi, (long)x));
    }
    fft_in_place(b, false);
    auto ex = slot_exponents(n);
    for (size_t k = 0; k < n / 2; ++k) {
      const C s = b[(ex[k] - 1) / 2];
      slots_out[2 * k] = s.re;
      slots_out[2 * k + 1] = s.im;
    }
    return RC_OK;
  } catch (...) {
    return RC_ERR_CUDA;
  }
}

// dense_slots_to_real_coeffs (src/ckks/bootstrapping/exact_transforms.rs:180-200): conjugate-symmetric
// evaluations at the 5^j exponents, canonical_embedding_backward, times xi^-i, real part.  Needs no context.
extern "C" int rc_slots_to_real_coeffs(uint64_t n, const double* slots, double* coeffs_out) {
  try {
    if (!slots || !coeffs_out || n < 2 || (n & (n - 1))) return RC_ERR_INVALID_ARGUMENT;
    std::vector<C> evals(n, C{0.0, 0.0});
    auto ex = slot_exponents(n);
    for (size_t k = 0; k < n / 2; ++k) {
      const C v{slots[2 * k], slots[2 * k + 1]};
      const size_t e = ex[k];
      evals[(e - 1) / 2] = v;
      evals[(((2 * n - e) % (2 * n)) - 1) / 2] = C{v.re, -v.im};
    }
    fft_in_place(evals, true);
    const C xi = polar(M_PI / (double)n);
    for (size_t i = 0; i < n; ++i) coeffs_out[i] = cmul(evals[i], cpowi(xi, -(long)i)).re;
    return RC_OK;
  } catch (...) {
    return RC_ERR_OUT_OF_MEMORY;
  }
}

// dense_complex_coeffs_to_slots (exact_transforms.rs:210-229): coefficients times xi^i,
// canonical_embedding_forward, the evaluations at the 5^j exponents.  Needs no context.
extern "C" int rc_complex_coeffs_to_slots(uint64_t n, const double* coeffs, double* slots_out) {
  try {
    if (!coeffs || !slots_out || n < 2 || (n & (n - 1))) return RC_ERR_INVALID_ARGUMENT;
    const C xi = polar(M_PI / (double)n);
    std::vector<C> v(n);
    for (size_t i = 0; i < n; ++i) v[i] = cmul(C{coeffs[2 * i], coeffs[2 * i + 1]}, cpowi(xi, (long)i));
    fft_in_place(v, false);
    auto ex = slot_exponents(n);
    for (size_t k = 0; k < n / 2; ++k) {
      const C s = v[(ex[k] - 1) / 2];
      slots_out[2 * k] = s.re;
      slots_out[2 * k + 1] = s.im;
    }
    return RC_OK;
  } catch (...) {
    return RC_ERR_OUT_OF_MEMORY;
  }
}

// The values the host FFT uses, for the device encoder/decoder to reproduce it bit for bit: per stage
// len = 2, 4, ..., n the twiddles w_i (i < len/2) by fft_in_place's recurrence w *= w_len, stored from
// complex offset len/2 - 1 (n - 1 entries per direction), and the twists xi^-i (encode) and xi^i (decode).
// Interleaved (re, im).
void rc::fft_tables(size_t n, std::vector<double>& tw_inv, std::vector<double>& tw_fwd, std::vector<double>& xi_neg,
                    std::vector<double>& xi_pos) {
  tw_inv.assign(2 * (n - 1), 0.0);
  tw_fwd.assign(2 * (n - 1), 0.0);
  for (int dir = 0; dir < 2; ++dir) {
    std::vector<double>& t = dir ? tw_inv : tw_fwd;
    for (size_t len = 2; len <= n; len <<= 1) {
      const double angle = dir ? -2.0 * M_PI / (double)len : 2.0 * M_PI / (double)len;
      const C w_len = polar(angle);
      C w{1.0, 0.0};
      for (size_t i = 0; i < len / 2; ++i) {
        t[2 * (len / 2 - 1 + i)] = w.re;
        t[2 * (len / 2 - 1 + i) + 1] = w.im;
        w = cmul(w, w_len);
      }
    }
  }
  const C xi = polar(M_PI / (double)n);
  xi_neg.resize(2 * n);
  xi_pos.resize(2 * n);
  for (size_t i = 0; i < n; ++i) {
    const C a = cpowi(xi, -(long)i), b = cpowi(xi, (long)i);
    xi_neg[2 * i] = a.re;
    xi_neg[2 * i + 1] = a.im;
    xi_pos[2 * i] = b.re;
    xi_pos[2 * i + 1] = b.im;
  }
}
