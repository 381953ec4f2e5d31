// FP64 CKKS encode/decode on the GPU, bit for bit the host encoder (csrc/encode.cpp, which follows
// src/rns/encoding.rs:9-66 and src/math/canonical_embedding.rs:44-79): the same radix-2 DIT FFT with the
// same twiddle values (the host's recurrence w *= w_len, tabulated on the host), the same twists xi^(-+i),
// the same complex products (ac - bd, ad + bc) with every multiply and add rounded separately (__dmul_rn /
// __dadd_rn / __dsub_rn, never fused), rounding half away from zero, the same saturating i128 conversion and
// centred CRT with correctly rounded multiword-to-double conversion.  Many plaintexts per call: inputs and
// outputs stay on the device.
//
// FFT layout: after the bit-reversal scatter, stages len = 2 .. 2048 run inside one CTA per 2048-element
// block in shared memory; the remaining stages (N = 2^12 .. 2^17) are one launch each, a thread per butterfly.
#include <cmath>
#include <mutex>

#include "context.hpp"
#include "crt.cuh"

using namespace rc;

namespace {

struct Cd {
  double re, im;
};

__device__ __forceinline__ Cd cmul(Cd a, Cd b) {
  return Cd{__dsub_rn(__dmul_rn(a.re, b.re), __dmul_rn(a.im, b.im)),
            __dadd_rn(__dmul_rn(a.re, b.im), __dmul_rn(a.im, b.re))};
}
__device__ __forceinline__ Cd cadd(Cd a, Cd b) { return Cd{__dadd_rn(a.re, b.re), __dadd_rn(a.im, b.im)}; }
__device__ __forceinline__ Cd csub(Cd a, Cd b) { return Cd{__dsub_rn(a.re, b.re), __dsub_rn(a.im, b.im)}; }

__device__ __forceinline__ uint32_t brev(uint32_t i, int bits) { return __brev(i) >> (32 - bits); }

constexpr int FFT_BLOCK_LOG = 11;  // 2048 complex doubles = 32 KB of shared memory per CTA

struct FftTabs {
  const Cd* tw_inv;   // [n - 1]: stage len at offset len/2 - 1
  const Cd* tw_fwd;   // [n - 1]
  const Cd* xi_neg;   // [n]
  const Cd* xi_pos;   // [n]
  const uint2* slot;  // [n/2]: evaluation index of slot k and of its conjugate
};

// encode step 1: evaluations (slot k at (5^k - 1)/2, its conjugate at (2N - 5^k - 1)/2) written straight to
// their bit-reversed positions
__global__ void k_enc_scatter(const double* slots, Cd* work, FftTabs t, int log_n, uint32_t count) {
  const size_t half = (size_t)1 << (log_n - 1), total = half * count;
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < total; g += (size_t)gridDim.x * blockDim.x) {
    const size_t p = g / half, k = g % half;
    const double re = slots[2 * g], im = slots[2 * g + 1];
    const uint2 ab = t.slot[k];
    Cd* w = work + (p << log_n);
    w[brev(ab.x, log_n)] = Cd{re, im};
    w[brev(ab.y, log_n)] = Cd{re, -im};
  }
}

// stages len = 2 .. 2^lb of every 2^lb-element block in shared memory
__global__ void k_fft_block(Cd* work, const Cd* tw, int lb) {
  extern __shared__ Cd sm[];
  const int B = 1 << lb;
  Cd* base = work + (size_t)blockIdx.x * B;
  for (int i = threadIdx.x; i < B; i += blockDim.x) sm[i] = base[i];
  __syncthreads();
  for (int len = 2; len <= B; len <<= 1) {
    const int h = len >> 1;
    for (int b = threadIdx.x; b < B / 2; b += blockDim.x) {
      const int c = (b / h) * len, i = b % h;
      const Cd u = sm[c + i];
      const Cd v = cmul(sm[c + i + h], tw[h - 1 + i]);
      sm[c + i] = cadd(u, v);
      sm[c + i + h] = csub(u, v);
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < B; i += blockDim.x) base[i] = sm[i];
}

// one stage of length len over all polynomials, a thread per butterfly
__global__ void k_fft_stage(Cd* work, const Cd* tw, int log_n, int len, uint32_t count) {
  const size_t half = (size_t)1 << (log_n - 1), total = half * count;
  const int h = len >> 1;
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < total; g += (size_t)gridDim.x * blockDim.x) {
    const size_t p = g / half, b = g % half;
    Cd* w = work + (p << log_n);
    const size_t c = (b / h) * len, i = b % h;
    const Cd u = w[c + i];
    const Cd v = cmul(w[c + i + h], tw[h - 1 + i]);
    w[c + i] = cadd(u, v);
    w[c + i + h] = csub(u, v);
  }
}

// magnitude (< 2^128) of a rounded, saturated value mod q, then the sign: mod_i128 of the host
__device__ __forceinline__ u64 signed_mod(bool neg, u64 hi, u64 lo, const PrimeConst& p) {
  const u64 q = p.q;
  auto red = [&](u64 x) {  // x mod q for any x < 2^64
    const u64 t = x - __umul64hi(x, p.one_s) * q;
    return t >= q ? t - q : t;
  };
  u64 r = red(lo);
  if (hi) {
    const u64 two64 = 0ull - p.one_s * q;  // 2^64 mod q
    r = add_mod(r, mul_mod(red(hi), two64, p), q);
  }
  return (neg && r) ? q - r : r;
}

// encode step 3: x / n, times xi^-i, real part times 2^scale_bits, f64::round, saturating i128, residues
__global__ void k_enc_finish(const Cd* work, FftTabs t, const PrimeConst* pc, int limbs, int log_n, double inv_n,
                             double scale, uint32_t count, u64* out) {
  const size_t n = (size_t)1 << log_n, total = n * count;
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < total; g += (size_t)gridDim.x * blockDim.x) {
    const size_t p = g >> log_n, i = g & (n - 1);
    const Cd x = work[g];
    const Cd s{__dmul_rn(x.re, inv_n), __dmul_rn(x.im, inv_n)};
    const Cd xi = t.xi_neg[i];
    const double re = __dsub_rn(__dmul_rn(s.re, xi.re), __dmul_rn(s.im, xi.im));
    const double r = round(__dmul_rn(re, scale));
    bool neg = false;
    u64 hi = 0, lo = 0;
    if (!isnan(r)) {
      const double lim = 1.7014118346046923e38;  // 2^127
      double m = fabs(r);
      neg = r < 0;
      if (r >= lim) {
        hi = 0x7FFFFFFFFFFFFFFFull;
        lo = ~0ull;  // 2^127 - 1
      } else if (r <= -lim) {
        hi = 0x8000000000000000ull;  // |-2^127|
      } else if (m < 18446744073709551616.0) {
        lo = __double2ull_rz(m);
      } else {
        const double h = floor(m * 0x1.0p-64);  // exact: m is an integer-valued double
        hi = __double2ull_rz(h);
        lo = __double2ull_rz(m - h * 0x1.0p64);
      }
    }
    u64* o = out + p * limbs * n + i;
    for (int j = 0; j < limbs; ++j) o[(size_t)j * n] = signed_mod(neg, hi, lo, pc[j]);
  }
}

// correctly rounded double of a W-word magnitude (the host's words_to_double): the top 64 significant bits with
// a sticky bit for everything below, converted to nearest, scaled by 2^shift
template <int WM>
__device__ __forceinline__ double words_to_double(const u64 (&X)[WM], int W) {
  bool found = false, sticky = false;
  int top = 0, lz = 0;
  u64 hiw = 0, next = 0;
#pragma unroll
  for (int w = WM - 1; w >= 0; --w) {
    if (w < W) {
      if (!found) {
        if (X[w]) {
          found = true;
          top = w;
          hiw = X[w];
          lz = __clzll(hiw);
        }
      } else if (w == top - 1) {
        next = X[w];
      } else {
        sticky |= X[w] != 0;
      }
    }
  }
  if (!found) return 0.0;
  if (top == 0) return __ull2double_rn(hiw);
  u64 m;
  if (lz == 0) {
    m = hiw;
    sticky |= next != 0;
  } else {
    m = (hiw << lz) | (next >> (64 - lz));
    sticky |= (next << lz) != 0;
  }
  if (sticky) m |= 1;
  return scalbn(__ull2double_rn(m), top * 64 - lz);
}

// decode step 1: centred CRT value, to double, times 2^-scale_bits, times xi^i, to the bit-reversed position
template <int WM>
__global__ void k_dec_crt(const PrimeConst* pc, DecompTab dt, const u64* polys, Cd* work, FftTabs t, int limbs,
                          int log_n, double inv_delta, uint32_t count) {
  const CrtSmem tabs = stage_crt_tables(pc, dt, limbs);
  __syncthreads();
  const size_t n = (size_t)1 << log_n;
  const size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const size_t p = blockIdx.y;
  if (x >= n || p >= count) return;
  u64 X[WM];
  const u64 ext = centred_crt<WM>(tabs, dt.W, limbs, polys + p * limbs * n + x, n, false, X);
  if (ext) {  // magnitude of a negative value: two's complement negation over W words
    u64 carry = 1;
#pragma unroll
    for (int w = 0; w < WM; ++w) {
      if (w < dt.W) {
        const u64 v = ~X[w] + carry;
        carry = (carry && v == 0) ? 1 : 0;
        X[w] = v;
      }
    }
  }
  double d = words_to_double<WM>(X, dt.W);
  if (ext) d = -d;
  const Cd a{__dmul_rn(d, inv_delta), 0.0};
  work[(p << log_n) + brev((uint32_t)x, log_n)] = cmul(a, t.xi_pos[x]);
}

// decode step 3: slot k = evaluation (5^k - 1)/2
__global__ void k_dec_gather(const Cd* work, FftTabs t, int log_n, uint32_t count, double* slots) {
  const size_t half = (size_t)1 << (log_n - 1), total = half * count;
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < total; g += (size_t)gridDim.x * blockDim.x) {
    const size_t p = g / half, k = g % half;
    const Cd v = work[(p << log_n) + t.slot[k].x];
    slots[2 * g] = v.re;
    slots[2 * g + 1] = v.im;
  }
}

int grid_for(size_t items) {
  const size_t g = (items + 255) / 256;
  return (int)(g < 1 ? 1 : (g > 152 * 64 ? 152 * 64 : g));
}

FftTabs fft_tabs(rc_context* c) {
  std::lock_guard<std::mutex> lk(c->mu);
  const size_t n = (size_t)c->N;
  if (!c->fft_buf) {
    std::vector<double> ti, tf, xn, xp;
    fft_tables(n, ti, tf, xn, xp);
    std::vector<uint32_t> slot(n);
    size_t e = 1;
    for (size_t k = 0; k < n / 2; ++k) {  // slot exponents 5^k mod 2N (encoding.rs:68-79)
      slot[2 * k] = (uint32_t)((e - 1) / 2);
      slot[2 * k + 1] = (uint32_t)(((2 * n - e) % (2 * n) - 1) / 2);
      e = e * 5 % (2 * n);
    }
    const size_t doubles = ti.size() + tf.size() + xn.size() + xp.size();
    c->fft_buf.reset(new DevBuf(doubles * 8 + slot.size() * 4));
    double* d = (double*)c->fft_buf->p;
    size_t off = 0;
    for (auto* v : {&ti, &tf, &xn, &xp}) {
      cuda_check(cudaMemcpy(d + off, v->data(), v->size() * 8, cudaMemcpyHostToDevice), "encoder tables");
      off += v->size();
    }
    cuda_check(cudaMemcpy(d + off, slot.data(), slot.size() * 4, cudaMemcpyHostToDevice), "encoder tables");
  }
  const Cd* base = (const Cd*)c->fft_buf->p;
  FftTabs t;
  t.tw_inv = base;
  t.tw_fwd = base + (n - 1);
  t.xi_neg = base + 2 * (n - 1);
  t.xi_pos = t.xi_neg + n;
  t.slot = (const uint2*)(t.xi_pos + n);
  return t;
}

void fft(Cd* work, const Cd* tw, int log_n, uint32_t count, cudaStream_t s) {
  const int lb = log_n < FFT_BLOCK_LOG ? log_n : FFT_BLOCK_LOG;
  const size_t blocks = ((size_t)count << log_n) >> lb;
  const int threads = (1 << lb) / 2 < 256 ? ((1 << lb) / 2 < 32 ? 32 : (1 << lb) / 2) : 256;
  for (size_t b0 = 0; b0 < blocks; b0 += 65535 * 16) {
    const size_t nb = blocks - b0 < 65535 * 16 ? blocks - b0 : 65535 * 16;
    k_fft_block<<<(unsigned)nb, threads, (sizeof(Cd) << lb), s>>>(work + (b0 << lb), tw, lb);
  }
  for (int len = 2 << lb; len <= (1 << log_n); len <<= 1)
    k_fft_stage<<<grid_for(((size_t)count << log_n) / 2), 256, 0, s>>>(work, tw, log_n, len, count);
}

}  // namespace

extern "C" int rc_encode_device(rc_context* c, const double* slots, uint32_t count, int32_t level,
                                uint32_t scale_bits, uint64_t* out, void* stream) {
  return guarded("rc_encode_device", [&] {
    require(c && slots && out, "arguments must not be null");
    require(level >= 0 && level < c->L, "level out of range for this context");
    if (count == 0) return;
    cudaStream_t s = (cudaStream_t)stream;
    const FftTabs t = fft_tabs(c);
    const size_t n = (size_t)c->N;
    Cd* work = (Cd*)context_workspace(c, s, (size_t)count * n * sizeof(Cd));
    k_enc_scatter<<<grid_for(count * n / 2), 256, 0, s>>>(slots, work, t, c->log_n, count);
    fft(work, t.tw_inv, c->log_n, count, s);
    const double scale = std::pow(2.0, (double)scale_bits);  // 2f64.powi(scale_bits)
    k_enc_finish<<<grid_for(count * n), 256, 0, s>>>(work, t, c->d_pc, level + 1, c->log_n, 1.0 / (double)n, scale,
                                                    count, out);
    cuda_check(cudaGetLastError(), "encode");
  });
}

extern "C" int rc_decode_device(rc_context* c, const uint64_t* polys, uint32_t count, int32_t level,
                                uint32_t scale_bits, double* slots_out, void* stream) {
  return guarded("rc_decode_device", [&] {
    require(c && polys && slots_out, "arguments must not be null");
    require(level >= 0 && level < c->L, "level out of range for this context");
    if (count == 0) return;
    require(count <= 65535, "at most 65535 polynomials per decode call");
    cudaStream_t s = (cudaStream_t)stream;
    const FftTabs t = fft_tabs(c);
    const size_t n = (size_t)c->N;
    const int limbs = level + 1;
    const DecompTab& dt = context_level(c, limbs).dt;
    Cd* work = (Cd*)context_workspace(c, s, (size_t)count * n * sizeof(Cd));
    const int threads = n < 128 ? (int)n : 128;
    const dim3 g((unsigned)((n + threads - 1) / threads), count);
    const size_t smem = crt_smem_bytes(limbs, dt.W);
    const double inv_delta = 1.0 / std::pow(2.0, (double)scale_bits);
    const int W = dt.W;
#define RC_DEC(WMV) k_dec_crt<WMV><<<g, threads, smem, s>>>(c->d_pc, dt, polys, work, t, limbs, c->log_n, inv_delta, count)
    if (W <= 4) RC_DEC(4);
    else if (W <= 8) RC_DEC(8);
    else if (W <= 16) RC_DEC(16);
    else if (W <= 24) RC_DEC(24);
    else if (W <= 32) RC_DEC(32);
    else RC_DEC(64);
#undef RC_DEC
    fft(work, t.tw_fwd, c->log_n, count, s);
    k_dec_gather<<<grid_for(count * n / 2), 256, 0, s>>>(work, t, c->log_n, count, slots_out);
    cuda_check(cudaGetLastError(), "decode");
  });
}
