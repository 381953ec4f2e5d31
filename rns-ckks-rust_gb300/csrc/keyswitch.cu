// Keyswitching with the reference's gadget: balanced base-2^30 digits of the
// centred CRT value (src/rns/keyswitching.rs:130-236, 381-467), ModUp of the
// digits to the aux basis (lift_poly_to_context, 242-276), the key inner
// product, and ModDown (mod_down_eval_to_q, 278-322).
//
// GPU formulation (exact, same residues as the reference):
//  * decompose: one thread per coefficient builds X = sum_i y_i * (Q/q_i) with
//    y_i = c_i * (Q/q_i)^-1 mod q_i in 64-bit words, removes floor(sum y_i/q_i)
//    multiples of Q (exact fix-up), centres it, and emits the balanced digits
//    of its two's complement: identical to the reference's Garner +
//    sign-magnitude digits + carry normalisation (including the dropped final
//    carry when the digits run out).
//  * digit NTT + key product: a digit d in [-2^29, 2^29) has residue d (or
//    d + q) in every limb, so ModUp of a digit polynomial is just that residue
//    in each aux prime.  Each digit is NTT'd per limb (column pass to scratch,
//    row pass fused with the multiply-accumulate against the key, which lives
//    in the NTT domain and Montgomery form), so neither the lifted digits nor
//    the per-digit products ever reach HBM.
//  * finalize: ModDown by exact centred Garner over the aux primes, optional
//    addend (relinearize / rotate) and optional rescale in one pass.
#include "kernels.cuh"
#include "nttcore.cuh"
#include "wide.cuh"
#include "crt.cuh"

namespace rc {

namespace {

// ---------------------------------------------------------------------------
// decomposition
// ---------------------------------------------------------------------------
// Job tables of the decomposition: where job j's input, tables and digits are.  UniDecomp: one level for
// every job (digits [job][D][N]); MlDecomp: each job at its own level (tables from the per-level array,
// digits of job j from polynomial dig[j] on).
struct UniDecomp {
  DecompTab dt;
  PtrTab src;
  int limbs, D;
  __device__ __forceinline__ const DecompTab& tab(int) const { return dt; }
  __device__ __forceinline__ int nlimbs(int) const { return limbs; }
  __device__ __forceinline__ int digits(int) const { return D; }
  __device__ __forceinline__ size_t first_digit(int job) const { return (size_t)job * D; }
  __device__ __forceinline__ const u64* in(int job) const { return src.p[job]; }
};
struct MlDecomp {
  const DecompTab* dts;  // [limbs] (device)
  MlTab t;
  MlPtrTab src;
  __device__ __forceinline__ const DecompTab& tab(int job) const { return dts[t.limbs[job]]; }
  __device__ __forceinline__ int nlimbs(int job) const { return t.limbs[job]; }
  __device__ __forceinline__ int digits(int job) const { return t.dig[job + 1] - t.dig[job]; }
  __device__ __forceinline__ size_t first_digit(int job) const { return (size_t)t.dig[job]; }
  __device__ __forceinline__ const u64* in(int job) const { return src.p[job]; }
};

template <int WM, bool TIES, class JT>
__global__ void k_decompose(const PrimeConst* pc, JT jt, int32_t* digits, u64 g_inv, int log_n, int* tie_flags) {
  const int job = blockIdx.y;
  const DecompTab& dt = jt.tab(job);
  const int limbs = jt.nlimbs(job), D = jt.digits(job);
  const CrtSmem tabs = stage_crt_tables(pc, dt, limbs);
  __syncthreads();
  const int W = dt.W;
  const u64 N = 1ull << log_n;
  const u64 x = blockIdx.x * (u64)blockDim.x + threadIdx.x;
  if (x >= N) return;
  const u64* in = jt.in(job);

  u64 sidx = x;
  bool neg = false;
  if (g_inv > 1) {
    sidx = (x * g_inv) & (2 * N - 1);
    neg = sidx >= N;
    if (neg) sidx -= N;
  }
  u64 X[WM];
  const u64 ext = centred_crt<WM>(tabs, W, limbs, in + sidx, N, neg, X);

  // balanced base-2^30 digits of the two's complement value
  int32_t* out = digits + jt.first_digit(job) * N + x;
  u64 carry = 0;
  bool tie = false;  // a digit at -2^29
  constexpr int DMAX = (64 * WM) / 30 + 2;
#pragma unroll
  for (int d = 0; d < DMAX; ++d) {
    if (d < D) {
      const int bit = 30 * d;
      const int w0 = bit / 64, sh = bit % 64;
      u64 lo = (w0 < WM) ? (w0 < W ? X[w0 < WM ? w0 : 0] : ext) : ext;
      u64 chunk = lo >> sh;
      if (sh > 34) {
        const int w1 = w0 + 1;
        u64 hi = (w1 < WM) ? (w1 < W ? X[w1 < WM ? w1 : 0] : ext) : ext;
        chunk |= hi << (64 - sh);
      }
      chunk &= (1ull << 30) - 1;
      u64 v = chunk + carry;
      int64_t dig;
      if (v >= (1ull << 29)) {
        dig = (int64_t)v - (1ll << 30);
        carry = 1;
      } else {
        dig = (int64_t)v;
        carry = 0;
      }
      if (TIES) tie |= dig == -(1ll << 29);
      out[(size_t)d * N] = (int32_t)dig;
    }
  }
  // digits beyond DMAX (only for keys with far more digits than the modulus
  // needs) are pure sign extension
  for (int d = DMAX; d < D; ++d) {
    u64 chunk = ext & ((1ull << 30) - 1);
    u64 v = chunk + carry;
    int64_t dig;
    if (v >= (1ull << 29)) {
      dig = (int64_t)v - (1ll << 30);
      carry = 1;
    } else {
      dig = (int64_t)v;
      carry = 0;
    }
    if (TIES) tie |= dig == -(1ll << 29);
    out[(size_t)d * N] = (int32_t)dig;
  }
  if (TIES && tie) atomicOr(&tie_flags[job], 1);
}

// lift_poly_to_context (keyswitching.rs:242-276) for polynomial blockIdx.y: the Q limbs are copied and limb
// limbs + k is the centred CRT value mod p_k (convert_centered_residues_to_target, 365-379):
// sum_w X[w] * (2^(64 w) mod p_k) minus 2^(64 W) mod p_k when X < 0.
template <int WM>
__global__ void k_lift(const PrimeConst* pc, const PrimeConst* ppc, DecompTab dt, const u64* src, u64* dst,
                       int limbs, int K, int log_n) {
  const CrtSmem tabs = stage_crt_tables(pc, dt, limbs);
  __syncthreads();
  const int W = dt.W;
  const u64 N = 1ull << log_n;
  const u64 x = blockIdx.x * (u64)blockDim.x + threadIdx.x;
  if (x >= N) return;
  const u64* in = src + (size_t)blockIdx.y * limbs * N + x;
  u64* out = dst + (size_t)blockIdx.y * (limbs + K) * N + x;
  for (int l = 0; l < limbs; ++l) out[(size_t)l * N] = in[(size_t)l * N];
  u64 X[WM];
  const u64 ext = centred_crt<WM>(tabs, W, limbs, in, N, false, X);
  for (int k = 0; k < K; ++k) {
    const u64 p = ppc[k].q, one_s = ppc[k].one_s;
    const u64* pw = dt.lift_pw + (size_t)k * (W + 1);
    const u64* pws = dt.lift_pw_s + (size_t)k * (W + 1);
    u64 acc = 0;
#pragma unroll
    for (int w = 0; w < WM; ++w) {
      if (w < W) {
        const u64 r = reduce_2q(mul_shoup_lazy(X[w], 1, one_s, p), p);  // X[w] mod p
        acc = add_mod(acc, mul_shoup(r, pw[w], pws[w], p), p);
      }
    }
    if (ext) acc = sub_mod(acc, pw[W], p);
    out[(size_t)(limbs + k) * N] = acc;
  }
}

// signed_digit_mod_q (keyswitching.rs:456-467) for |d| <= 2^29
__device__ __forceinline__ u64 digit_residue(int32_t d, u64 q) {
  if (q > (1ull << 29)) return d >= 0 ? (u64)d : q - (u64)(-(int64_t)d);
  u64 m = (u64)(d >= 0 ? (int64_t)d : -(int64_t)d) % q;
  return d >= 0 ? m : (m ? q - m : 0);
}

// Residue of the lifted digit in aux prime p: the centred representative of
// (d mod Q) reduced mod p (convert_centered_residues_to_target).  For Q > 2^30
// that representative is d itself.
__device__ __forceinline__ u64 lifted_residue(int32_t d, u64 p, const DecompTab& dt) {
  if (!dt.small_q) return digit_residue(d, p);
  const int64_t Qs = (int64_t)dt.Qsmall;
  int64_t x = (int64_t)d % Qs;
  if (x < 0) x += Qs;
  if ((u64)x > (dt.Qsmall >> 1)) x -= Qs;
  int64_t r = x % (int64_t)p;
  if (r < 0) r += (int64_t)p;
  return (u64)r;
}

// ---------------------------------------------------------------------------
// digit NTT: column pass (digit -> residue -> stages 0..n1-1 -> scratch)
// ---------------------------------------------------------------------------
__global__ void k_digit_cols(KsArgs a, DecompTab dt, const int32_t* digits, u64* scratch, int p0, int pc_count) {
  extern __shared__ u64 sm[];
  const int log_n = a.ntt.log_n, n1 = a.ntt.n1;
  const int N = 1 << log_n, N1 = 1 << n1, N2 = N >> n1;
  const int COLS = N2 < 16 ? N2 : 16;
  const int c0 = blockIdx.x * COLS;
  const int digit = blockIdx.y / pc_count, pl = blockIdx.y % pc_count;
  const int total = a.qlimbs + a.K;
  const int pair = p0 + pl;
  const int job = pair / total, limb = pair % total;
  const LimbMap map{a.qlimbs, a.L};
  const int prime = map.prime(limb);
  const u64 q = a.pc[prime].q, two_q = q << 1;
  const bool aux = limb >= a.qlimbs;
  const Twiddle* tw = a.ntt.tw_fwd + (size_t)prime * N;
  const int32_t* in = digits + ((size_t)job * a.D + digit) * N;
  u64* out = scratch + ((size_t)pl * a.D + digit) * N;

  for (int idx = threadIdx.x; idx < N1 * COLS; idx += blockDim.x) {
    int r = idx / COLS, c = idx % COLS;
    int32_t d = in[(size_t)r * N2 + c0 + c];
    sm[idx] = aux ? lifted_residue(d, q, dt) : digit_residue(d, q);
  }
  __syncthreads();
  for (int s = 0; s < n1; ++s) {
    const int t = N1 >> (s + 1);
    for (int idx = threadIdx.x; idx < (N1 / 2) * COLS; idx += blockDim.x) {
      int p = idx / COLS, c = idx % COLS;
      int r = (p / t) * 2 * t + (p % t);
      Twiddle w = tw[(1 << s) + (r >> (n1 - s))];
      u64 x = sm[r * COLS + c], y = sm[(r + t) * COLS + c];
      x = x >= two_q ? x - two_q : x;
      u64 v = mul_shoup_lazy(y, w.w, w.ws, q);
      sm[r * COLS + c] = x + v;
      sm[(r + t) * COLS + c] = x - v + two_q;
    }
    __syncthreads();
  }
  for (int idx = threadIdx.x; idx < N1 * COLS; idx += blockDim.x) {
    int r = idx / COLS, c = idx % COLS;
    out[(size_t)r * N2 + c0 + c] = sm[idx];
  }
}

// ---------------------------------------------------------------------------
// digit NTT row pass fused with the key multiply-accumulate
// ---------------------------------------------------------------------------
constexpr int MAC_E = 4;  // elements per thread

struct KeyTab {
  const u64* k[MAXP];
};

__global__ void k_digit_rows_mac(KsArgs a, const u64* scratch, KeyTab keys, u64* acc, int p0) {
  extern __shared__ u64 sm[];
  const int log_n = a.ntt.log_n, n1 = a.ntt.n1;
  const int N = 1 << log_n, N2 = N >> n1;
  const int tile = blockDim.x * MAC_E;  // ROWS * N2
  const int ROWS = tile / N2;
  const int r0 = blockIdx.x * ROWS;
  const int pl = blockIdx.y;
  const int limbs_total = a.qlimbs + a.K;
  const int pair = p0 + pl;
  const int job = pair / limbs_total, limb = pair % limbs_total;
  const LimbMap map{a.qlimbs, a.L};
  const int prime = map.prime(limb);
  const PrimeConst& pc = a.pc[prime];
  const u64 q = pc.q, two_q = q << 1;
  const Twiddle* tw = a.ntt.tw_fwd + (size_t)prime * N;
  // key layout [limb][key_digits][2][N]
  const u64* key = keys.k[job] + (size_t)limb * a.key_digits * 2 * N + (size_t)r0 * N2;

  U128 acc0[MAC_E], acc1[MAC_E];
  u64 red0[MAC_E], red1[MAC_E];
#pragma unroll
  for (int e = 0; e < MAC_E; ++e) {
    acc0[e].lo = acc0[e].hi = acc1[e].lo = acc1[e].hi = 0;
    red0[e] = red1[e] = 0;
  }
  const int half = N2 / 2;
  const u64 chunk = pc.mac_chunk;
  u64 since = 0;
  for (int digit = 0; digit < a.D; ++digit) {
    const u64* in = scratch + ((size_t)pl * a.D + digit) * N + (size_t)r0 * N2;
    for (int idx = threadIdx.x; idx < tile; idx += blockDim.x) sm[idx] = in[idx];
    __syncthreads();
    for (int s = n1; s < log_n; ++s) {
      const int t = N2 >> (s - n1 + 1);
      for (int idx = threadIdx.x; idx < tile / 2; idx += blockDim.x) {
        int rl = idx / half, p = idx % half;
        int c = (p / t) * 2 * t + (p % t);
        int j = (r0 + rl) * N2 + c;
        Twiddle w = tw[(1 << s) + (j >> (log_n - s))];
        u64* base = sm + rl * N2;
        u64 x = base[c], y = base[c + t];
        x = x >= two_q ? x - two_q : x;
        u64 v = mul_shoup_lazy(y, w.w, w.ws, q);
        base[c] = x + v;
        base[c + t] = x - v + two_q;
      }
      __syncthreads();
    }
    const u64* k0 = key + (size_t)digit * 2 * N;
    const u64* k1 = k0 + N;
#pragma unroll
    for (int e = 0; e < MAC_E; ++e) {
      const int idx = threadIdx.x + e * blockDim.x;
      const u64 v = reduce_4q(sm[idx], q);
      add_to(acc0[e], mul_wide(v, k0[idx]));
      add_to(acc1[e], mul_wide(v, k1[idx]));
    }
    if (++since == chunk) {
#pragma unroll
      for (int e = 0; e < MAC_E; ++e) {
        red0[e] = add_mod(red0[e], mont_reduce(acc0[e], pc), q);
        red1[e] = add_mod(red1[e], mont_reduce(acc1[e], pc), q);
        acc0[e].lo = acc0[e].hi = acc1[e].lo = acc1[e].hi = 0;
      }
      since = 0;
    }
    __syncthreads();
  }
  u64* out0 = acc + ((size_t)job * 2 * limbs_total + limb) * N + (size_t)r0 * N2;
  u64* out1 = out0 + (size_t)limbs_total * N;
#pragma unroll
  for (int e = 0; e < MAC_E; ++e) {
    const int idx = threadIdx.x + e * blockDim.x;
    out0[idx] = add_mod(red0[e], mont_reduce(acc0[e], pc), q);
    out1[idx] = add_mod(red1[e], mont_reduce(acc1[e], pc), q);
  }
}

// ---------------------------------------------------------------------------
// fast path (log N in 12..16): warp-level register-blocked digit transforms
// ---------------------------------------------------------------------------
template <int M>
struct DigitColTile {
  static constexpr int COLS = (8 * core::Geo<M>::SUBS) > 16 ? 8 * core::Geo<M>::SUBS : 16;
};

template <int M1, int M2, bool LAZY>
__global__ __launch_bounds__(256, 2) void k_digit_cols_f(KsArgs a, DecompTab dt, const int32_t* digits, u64* scratch,
                                                         int p0, int pc_count) {
  using G = core::Geo<M1>;
  constexpr int COLS = DigitColTile<M1>::COLS, N1 = 1 << M1, N2 = 1 << M2, N = N1 * N2;
  __shared__ u64 tile[COLS * G::STRIDE];
  __shared__ Twiddle twl[N1];
  const int c0 = blockIdx.x * COLS;
  const int digit = blockIdx.y / pc_count, pl = blockIdx.y % pc_count;
  const int total = a.qlimbs + a.K;
  const int pair = p0 + pl;
  const int job = pair / total, limb = pair % total;
  const LimbMap map{a.qlimbs, a.L};
  const int prime = map.prime(limb);
  const u64 q = a.pc[prime].q;
  const bool aux = limb >= a.qlimbs;
  core::stage_twiddles<M1>(twl, a.ntt.tw_fwd + (size_t)prime * N, 1, threadIdx.x, 256);
  const int32_t* in = digits + ((size_t)job * a.D + digit) * N;
  u64* out = scratch + ((size_t)pl * a.D + digit) * N;
#pragma unroll 4
  for (int it = 0; it < N1 * COLS / 256; ++it) {
    const int idx = it * 256 + threadIdx.x;
    const int r = idx / COLS, c = idx % COLS;
    const int32_t d = in[(size_t)r * N2 + c0 + c];
    tile[c * G::STRIDE + core::swz<M1>(r)] = aux ? lifted_residue(d, q, dt) : digit_residue(d, q);
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5;
#pragma unroll 1
  for (int cb = warp * G::SUBS; cb < COLS; cb += 8 * G::SUBS) {
    const int lv = core::lane_id_volatile();
    const int sub = lv / G::LANES, l = lv % G::LANES;
    u64* buf = tile + (cb + sub) * G::STRIDE;
    u64 v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = buf[core::swz<M1>(core::first_idx<M1>(l, k))];
    __syncwarp();
    core::fwd_sub<M1, LAZY>(v, buf, l, twl, q);
#pragma unroll
    for (int k = 0; k < 8; ++k) buf[core::swz<M1>(core::last_idx<M1>(l, k))] = v[k];
  }
  __syncthreads();
#pragma unroll 4
  for (int it = 0; it < N1 * COLS / 256; ++it) {
    const int idx = it * 256 + threadIdx.x;
    const int r = idx / COLS, c = idx % COLS;
    out[(size_t)r * N2 + c0 + c] = tile[c * G::STRIDE + core::swz<M1>(r)];
  }
}

constexpr int MAC_WARPS = 4;

// Row pass of every digit transform of one (job, limb) and the key product.
// The rows' twiddle tables are staged once and reused for all digits; the next
// digit's row is prefetched while the current one is transformed.  ACC64:
// 64-bit accumulators with per-term Montgomery reduction (each term < 2q)
// instead of 128-bit lazy sums.
template <int M1, int M2, bool LAZY, bool ACC64>
__global__ __launch_bounds__(32 * MAC_WARPS, ACC64 ? 4 : 3) void k_digit_rows_mac_f(KsArgs a, const u64* scratch,
                                                                                     KeyTab keys, u64* acc, int p0) {
  using G = core::Geo<M2>;
  constexpr int N1 = 1 << M1, N2 = 1 << M2, N = N1 * N2, ROWS = MAC_WARPS * G::SUBS;
  __shared__ u64 bufs[ROWS * G::STRIDE];
  __shared__ Twiddle twl[ROWS][N2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane / G::LANES;
  const int row0 = blockIdx.x * ROWS;
  const int rl = warp * G::SUBS + sub, row = row0 + rl;
  const int pl = blockIdx.y;
  const int total = a.qlimbs + a.K;
  const int pair = p0 + pl;
  const int job = pair / total, limb = pair % total;
  const LimbMap map{a.qlimbs, a.L};
  const int prime = map.prime(limb);
  const PrimeConst& pc = a.pc[prime];
  const u64 q = pc.q, qn = pc.qinv_neg;
  const Twiddle* twg = a.ntt.tw_fwd + (size_t)prime * N;
#pragma unroll 1
  for (int rr = 0; rr < ROWS; ++rr)
    core::stage_twiddles<M2>(twl[rr], twg, (u64)(N1 + row0 + rr), threadIdx.x, 32 * MAC_WARPS);
  __syncthreads();
  const u64* key = keys.k[job] + (size_t)limb * a.key_digits * 2 * N + (size_t)row * N2;
  u64* buf = bufs + rl * G::STRIDE;
  const u64* rowin = scratch + (size_t)pl * a.D * N + (size_t)row * N2;

  U128 acc0[8], acc1[8];  // ACC64 uses only .lo
#pragma unroll
  for (int k = 0; k < 8; ++k) acc0[k].lo = acc0[k].hi = acc1[k].lo = acc1[k].hi = 0;
  const u64 chunk = ACC64 ? pc.mac_chunk64 : pc.mac_chunk;
  u64 since = 0;
  auto term = [&](u64 x, u64 y) -> u64 {  // (x*y + m*q) / 2^64, m = -(x*y) q^-1 mod 2^64: < 2q
    const u64 lo = x * y, hi = mulhi(x, y);
    const u64 m = lo * qn;
    return hi + mulhi(m, q) + (lo != 0 ? 1ull : 0ull);
  };
  u64 nxt[8];
  {
    const int l = lane % G::LANES;
#pragma unroll
    for (int k = 0; k < 8; ++k) nxt[k] = rowin[core::first_idx<M2>(l, k)];
  }
#pragma unroll 1
  for (int digit = 0; digit < a.D; ++digit) {
    const int l = core::lane_id_volatile() % G::LANES;
    u64 v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = nxt[k];
    if (digit + 1 < a.D) {
      const u64* in = rowin + (size_t)(digit + 1) * N;
#pragma unroll
      for (int k = 0; k < 8; ++k) nxt[k] = in[core::first_idx<M2>(l, k)];
    }
    core::fwd_sub<M2, LAZY>(v, buf, l, twl[rl], q);
    const u64* k0 = key + (size_t)digit * 2 * N;
    const u64* k1 = k0 + N;
#pragma unroll
    for (int k = 0; k < 8; k += 2) {
      const int pos = core::last_idx<M2>(l, k);  // pos, pos+1 hold elements k, k+1
      const ulonglong2 w0 = *reinterpret_cast<const ulonglong2*>(k0 + pos);
      const ulonglong2 w1 = *reinterpret_cast<const ulonglong2*>(k1 + pos);
      if (ACC64) {
        acc0[k].lo += term(v[k], w0.x);
        acc0[k + 1].lo += term(v[k + 1], w0.y);
        acc1[k].lo += term(v[k], w1.x);
        acc1[k + 1].lo += term(v[k + 1], w1.y);
      } else {
        add_to(acc0[k], mul_wide(v[k], w0.x));
        add_to(acc0[k + 1], mul_wide(v[k + 1], w0.y));
        add_to(acc1[k], mul_wide(v[k], w1.x));
        add_to(acc1[k + 1], mul_wide(v[k + 1], w1.y));
      }
    }
    if (++since == chunk) {  // fold: keep the sums congruent mod q and small
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        acc0[k].lo = barrett_reduce(acc0[k], pc);
        acc0[k].hi = 0;
        acc1[k].lo = barrett_reduce(acc1[k], pc);
        acc1[k].hi = 0;
      }
      since = 1;
    }
  }
  const int l = lane % G::LANES;
  u64* out0 = acc + ((size_t)job * 2 * total + limb) * N + (size_t)row * N2;
  u64* out1 = out0 + (size_t)total * N;
#pragma unroll
  for (int k = 0; k < 8; k += 2) {
    const int pos = core::last_idx<M2>(l, k);
    ulonglong2 o0, o1;
    if (ACC64) {
      o0.x = barrett_reduce(acc0[k], pc);
      o0.y = barrett_reduce(acc0[k + 1], pc);
      o1.x = barrett_reduce(acc1[k], pc);
      o1.y = barrett_reduce(acc1[k + 1], pc);
    } else {
      o0.x = mont_reduce(acc0[k], pc);
      o0.y = mont_reduce(acc0[k + 1], pc);
      o1.x = mont_reduce(acc1[k], pc);
      o1.y = mont_reduce(acc1[k + 1], pc);
    }
    *reinterpret_cast<ulonglong2*>(out0 + pos) = o0;
    *reinterpret_cast<ulonglong2*>(out1 + pos) = o1;
  }
}

template <int M1, int M2, bool LAZY>
void digit_fast(const KsArgs& a, const int32_t* digits, const KeyTab& kt, u64* acc, u64* scratch, int p0, int pcc,
                cudaStream_t s) {
  {
    ProfScope p("digit_cols", s);
    dim3 g1((1 << M2) / DigitColTile<M1>::COLS, a.D * pcc);
    k_digit_cols_f<M1, M2, LAZY><<<g1, 256, 0, s>>>(a, *a.dt, digits, scratch, p0, pcc);
  }
  {
    ProfScope p("digit_rows_mac", s);
    dim3 g2((1 << M1) / (MAC_WARPS * core::Geo<M2>::SUBS), pcc);
    if (a.mac64) k_digit_rows_mac_f<M1, M2, LAZY, true><<<g2, 32 * MAC_WARPS, 0, s>>>(a, scratch, kt, acc, p0);
    else k_digit_rows_mac_f<M1, M2, LAZY, false><<<g2, 32 * MAC_WARPS, 0, s>>>(a, scratch, kt, acc, p0);
  }
}

template <bool LAZY>
bool digit_dispatch(const KsArgs& a, const int32_t* digits, const KeyTab& kt, u64* acc, u64* scratch, int p0,
                    int pcc, cudaStream_t s) {
  switch (a.ntt.log_n) {
    case 12: digit_fast<6, 6, LAZY>(a, digits, kt, acc, scratch, p0, pcc, s); return true;
    case 13: digit_fast<6, 7, LAZY>(a, digits, kt, acc, scratch, p0, pcc, s); return true;
    case 14: digit_fast<7, 7, LAZY>(a, digits, kt, acc, scratch, p0, pcc, s); return true;
    case 15: digit_fast<7, 8, LAZY>(a, digits, kt, acc, scratch, p0, pcc, s); return true;
    case 16: digit_fast<8, 8, LAZY>(a, digits, kt, acc, scratch, p0, pcc, s); return true;
    default: return false;
  }
}

// ---------------------------------------------------------------------------
// finalize: ModDown + addend + rescale
// ---------------------------------------------------------------------------
constexpr int KMAX = 8;

// Per-limb constants of k_finalize, staged once per CTA in shared memory (every thread of a CTA walks the
// same limbs): FT fields per limb, then K Montgomery weights and their Shoup companions.
enum FT { FT_Q, FT_ONE_S, FT_LO, FT_LO_S, FT_C01, FT_C01_S, FT_AMOD, FT_PINV, FT_PINV_S, FT_PMOD, FT_RINV,
          FT_RINV_S, FT_N };
__host__ __device__ __forceinline__ int ft_stride(int K) { return FT_N + 2 * K; }

// Job tables of the finalize pass: job j's Q limb count, where its products start in acc (in limb
// polynomials of N words), its addends and outputs.  UniFin: every job at f.qlimbs, acc [job][2][lq + K];
// MlFin: each job at its own level, products from limb polynomial 2 acc[j] on.
struct UniFin {
  PtrTab addend, out;
  int lq, K;
  __device__ __forceinline__ int limbs(int) const { return lq; }
  __device__ __forceinline__ size_t first_poly(int job) const { return (size_t)job * 2 * (lq + K); }
  __device__ __forceinline__ const u64* add(int job, int comp) const { return addend.p[2 * job + comp]; }
  __device__ __forceinline__ u64* dst(int job, int comp) const { return out.p[2 * job + comp]; }
};
struct MlFin {
  MlTab t;
  MlPtrTab addend, out;
  __device__ __forceinline__ int limbs(int job) const { return t.limbs[job]; }
  __device__ __forceinline__ size_t first_poly(int job) const { return (size_t)t.acc[job]; }
  __device__ __forceinline__ const u64* add(int job, int comp) const { return addend.p[2 * job + comp]; }
  __device__ __forceinline__ u64* dst(int job, int comp) const { return out.p[2 * job + comp]; }
};

// KC: the aux limb count K when it is a compile-time constant (0, 1, 2), -1 for any K up to KMAX (loops over the
// aux limbs then run to KMAX under predicates).  FAST: the lazy wide path (f.wide && f.lazy), so each instance
// carries only its own path's code
template <class JT, int KC, bool FAST>
__global__ void k_finalize(FinalizeArgs f, const u64* acc, JT jt) {
  constexpr int KB = KC > 0 ? KC : (KC == 0 ? 1 : KMAX);  // bound of the loops over aux limbs and words of P
  extern __shared__ u64 tab[];  // [lq + K][FT_N + 2K]
  const u64 N = 1ull << f.log_n;
  const int comp = blockIdx.y & 1, job = blockIdx.y >> 1;
  const int lq = jt.limbs(job), K = KC >= 0 ? KC : f.K;
  const LimbMap fmap{lq, f.L};
  const int st = ft_stride(K);
  // with the wide CRT and an aux basis, a Q limb's constants carry the factor P^-1 (`fold`): the CRT then
  // yields S * P^-1, the P-part conversion (M_k P^-1) and its sign correction (P P^-1 = 1) match it, and
  // ModDown's own multiply by P^-1 disappears
  const bool fold = f.wide && K > 0;
  // lazy wide path: each Q limb's terms are summed unreduced and reduced once, so its subtracted constants
  // are staged negated: q - A F (added when S < 0) and q - M_k F with Shoup companion ~(M_k F)_s (for
  // 0 < w < q, floor((q - w) 2^64 / q) = 2^64 - 1 - floor(w 2^64 / q))
  const bool fast = FAST;  // = f.wide && f.lazy (the launch picks the instance)
  for (int e = threadIdx.x; e < (lq + K) * st; e += blockDim.x) {
    const int i = e / st, fld = e - i * st;
    const int t = fmap.prime(i);
    const bool q_limb = i < lq;
    const bool fq = fold && q_limb;
    u64 v = 0;
    switch (fld) {
      case FT_Q: v = f.pc[t].q; break;
      case FT_ONE_S: v = f.pc[t].one_s; break;
      case FT_LO: v = fq ? f.md.pinv[i] : 1; break;
      case FT_LO_S: v = fq ? f.md.pinv_s[i] : f.pc[t].one_s; break;
      case FT_C01: v = !f.wide ? 0 : (fq ? f.wt.c01p[i] : f.wt.c01_mod_t[t]); break;
      case FT_C01_S: v = !f.wide ? 0 : (fq ? f.wt.c01p_s[i] : f.wt.c01_mod_t_s[t]); break;
      case FT_AMOD: v = !f.wide ? 0 : (fq ? f.wt.ap[i] : f.wt.A_mod_t[t]); break;
      case FT_PINV: v = (K && q_limb) ? f.md.pinv[i] : 0; break;
      case FT_PINV_S: v = (K && q_limb) ? f.md.pinv_s[i] : 0; break;
      case FT_PMOD: v = (K && q_limb) ? (fq ? 1 : f.md.pmod[i]) : 0; break;
      case FT_RINV: v = (f.rescale && i < lq - 1) ? f.rt.inv[(size_t)(lq - 1) * f.L + i] : 0; break;
      case FT_RINV_S: v = (f.rescale && i < lq - 1) ? f.rt.inv_s[(size_t)(lq - 1) * f.L + i] : 0; break;
      default: {
        const int k = fld - FT_N;
        if (q_limb && k < K) v = fq ? f.wt.mkp[(size_t)i * K + k] : f.md.mk[(size_t)i * K + k];
        else if (q_limb) v = fq ? f.wt.mkp_s[(size_t)i * K + (k - K)] : f.md.mk_s[(size_t)i * K + (k - K)];
      }
    }
    if (fast) {
      const u64 q = f.pc[t].q;
      if (q_limb && fld == FT_AMOD) v = v ? q - v : 0;  // the aux limbs' Garner keeps A F
      if (q_limb && fld >= FT_N && fld < FT_N + K) {
        const int k = fld - FT_N;
        const u64 w = fq ? f.wt.mkp[(size_t)i * K + k] : f.md.mk[(size_t)i * K + k];
        v = w ? q - w : 0;
      }
      if (q_limb && fld >= FT_N + K) {
        const int k = fld - FT_N - K;
        const u64 w = fq ? f.wt.mkp[(size_t)i * K + k] : f.md.mk[(size_t)i * K + k];
        v = w ? ~v : 0;
      }
    }
    tab[e] = v;
  }
  __syncthreads();
  const u64 x = blockIdx.x * (u64)blockDim.x + threadIdx.x;
  if (x >= N) return;
  const int wf = f.wide ? 2 : 1;  // 8-byte words per limb and coefficient in acc
  const u64* a = acc + (jt.first_poly(job) + (size_t)comp * (lq + K)) * N * wf;
  const uint2* a2 = reinterpret_cast<const uint2*>(a);
  auto T = [&](int i, int fld) -> u64 { return tab[i * st + fld]; };
  auto accv = [&](int j) -> u64 {  // value of limb j at x
    if (!f.wide) return a[(size_t)j * N + x];
    return wide_crt_mod_c(a2[(size_t)j * 2 * N + x], a2[((size_t)j * 2 + 1) * N + x], f.wt, T(j, FT_Q),
                          T(j, FT_LO), T(j, FT_LO_S), T(j, FT_C01), T(j, FT_C01_S), T(j, FT_AMOD));
  };
  const u64* add = jt.add(job, comp);
  u64* dst = jt.dst(job, comp);

  u64 addsrc = x;
  bool addneg = false;
  if (add && f.add_g_inv > 1) {
    addsrc = (x * f.add_g_inv) & (2 * N - 1);
    addneg = addsrc >= N;
    if (addneg) addsrc -= N;
  }

  // Garner over the aux primes: mixed-radix digits v_k of [x]_P
  u64 v[KB];
  bool pneg = false;
  if (K > 0) {
#pragma unroll
    for (int k = 0; k < KB; ++k) {
      if (k < K) {
        const u64 pq = T(lq + k, FT_Q), pone = T(lq + k, FT_ONE_S);
        u64 val = accv(lq + k);
#pragma unroll
        for (int t = 0; t < KB; ++t) {
          if (t < k) {
            const u64 vr = v[t] < pq ? v[t] : mul_shoup(v[t], 1, pone, pq);
            val = sub_mod(val, vr, pq);
            val = mul_shoup(val, f.md.p_garner[k * K + t], f.md.p_garner_s[k * K + t], pq);
          }
        }
        v[k] = val;
      }
    }
    // X_P = sum v_k M_k by Horner (K words max); compare with floor(P/2)
    u64 X[KB];
#pragma unroll
    for (int w = 0; w < KB; ++w) X[w] = 0;
#pragma unroll
    for (int k = KB - 1; k >= 0; --k) {
      if (k < K) {
        const u64 pk = T(lq + k, FT_Q);
        u64 carry = v[k];
#pragma unroll
        for (int w = 0; w < KB; ++w) {
          U128 p = mul_wide(X[w], pk);
          u64 lo = p.lo + carry;
          carry = p.hi + (lo < carry ? 1ull : 0ull);
          X[w] = lo;
        }
      }
    }
    int res = 0;
#pragma unroll
    for (int w = KB - 1; w >= 0; --w) {
      if (res == 0) {
        u64 h = w < f.md.KW ? f.md.halfP[w < KB ? w : 0] : 0ull;
        if (X[w] > h) res = 1;
        else if (X[w] < h) res = -1;
      }
    }
    pneg = res > 0;
  }

  // one limb's inputs (wide products and addend) and the value computed from them; the limb loops below
  // request limb i+2's inputs before computing limb i, so each thread has several limbs' loads in flight
  struct LimbIn {
    uint2 p01, p23;
    u64 av;
  };
  auto load = [&](int j) -> LimbIn {
    LimbIn r;
    r.p01 = a2[(size_t)j * 2 * N + x];
    r.p23 = a2[((size_t)j * 2 + 1) * N + x];
    r.av = add ? add[(size_t)j * N + addsrc] : 0;
    return r;
  };

  if (fast) {
    // S F + [S < 0] (q - A F) + sum_k v_k (q - M_k F) + [X_P > P/2] P F + addend (+ the rescale term): the
    // CRT's two products and the K conversion terms are approximate Shoup products below 4q, the rest below q:
    // at most (12 + 4K) q < 2^64, reduced once by the final (exact) Shoup product
    auto lazy_value = [&](int i, const LimbIn& in) -> u64 {
      const u64 q = T(i, FT_Q);
      u64 s = wide_crt_lazy(in.p01, in.p23, f.wt, q, T(i, FT_LO), T(i, FT_LO_S), T(i, FT_C01), T(i, FT_C01_S),
                            T(i, FT_AMOD));
#pragma unroll
      for (int k = 0; k < KB; ++k)
        if (k < K) s += mul_shoup_apx(v[k], T(i, FT_N + k), T(i, FT_N + K + k), q);
      if (pneg) s += T(i, FT_PMOD);
      if (add) s += (addneg && in.av) ? q - in.av : in.av;
      return s;
    };
    if (!f.rescale) {
      LimbIn cur = load(0), nxt;
      if (lq > 1) nxt = load(1);
#pragma unroll 1
      for (int i = 0; i < lq; ++i) {
        LimbIn far;
        if (i + 2 < lq) far = load(i + 2);
        const u64 q = T(i, FT_Q);
        dst[(size_t)i * N + x] = reduce_2q(mul_shoup_lazy(lazy_value(i, cur), 1, T(i, FT_ONE_S), q), q);
        cur = nxt;
        nxt = far;
      }
      return;
    }
    const int last = lq - 1;
    const u64 ql = T(last, FT_Q), half = ql >> 1;
    const u64 vl = reduce_2q(mul_shoup_lazy(lazy_value(last, load(last)), 1, T(last, FT_ONE_S), ql), ql);
    const bool pos = vl <= half;
    const u64 dist = pos ? vl : ql - vl;
    if (last == 0) return;
    LimbIn cur = load(0), nxt;
    if (last > 1) nxt = load(1);
#pragma unroll 1
    for (int i = 0; i < last; ++i) {
      LimbIn far;
      if (i + 2 < last) far = load(i + 2);
      const u64 q = T(i, FT_Q);
      // (value - centred last limb) * q_last^-1: the centred value's negation enters the sum lazily
      const u64 d = dist < q ? dist : mul_shoup(dist, 1, T(i, FT_ONE_S), q);
      const u64 s = lazy_value(i, cur) + (pos ? q - d : d);
      dst[(size_t)i * N + x] = reduce_2q(mul_shoup_lazy(s, T(i, FT_RINV), T(i, FT_RINV_S), q), q);
      cur = nxt;
      nxt = far;
    }
    return;
  }
  auto finish_value = [&](int i, u64 val, u64 av) -> u64 {
    const u64 q = T(i, FT_Q);
    if (K > 0) {
      u64 conv = 0;
#pragma unroll
      for (int k = 0; k < KB; ++k) {
        if (k < K) conv = add_mod(conv, mul_shoup(v[k], T(i, FT_N + k), T(i, FT_N + K + k), q), q);
      }
      if (pneg) conv = sub_mod(conv, T(i, FT_PMOD), q);
      val = sub_mod(val, conv, q);
      if (!fold) val = mul_shoup(val, T(i, FT_PINV), T(i, FT_PINV_S), q);
    }
    if (add) {
      if (addneg && av) av = q - av;
      val = add_mod(val, av, q);
    }
    return val;
  };
  auto wide_value = [&](int i, const LimbIn& in) -> u64 {
    const u64 val = wide_crt_mod_c(in.p01, in.p23, f.wt, T(i, FT_Q), T(i, FT_LO), T(i, FT_LO_S), T(i, FT_C01),
                                   T(i, FT_C01_S), T(i, FT_AMOD));
    return finish_value(i, val, in.av);
  };

  auto limb_value = [&](int i) -> u64 {
    const u64 q = T(i, FT_Q);
    u64 val = accv(i);
    if (K > 0) {
      // centred [x]_P mod q_i; Shoup's product is exact for any 64-bit multiplicand, so v[k] (< p_k) needs
      // no reduction mod q_i
      u64 conv = 0;
#pragma unroll
      for (int k = 0; k < KB; ++k) {
        if (k < K) conv = add_mod(conv, mul_shoup(v[k], T(i, FT_N + k), T(i, FT_N + K + k), q), q);
      }
      if (pneg) conv = sub_mod(conv, T(i, FT_PMOD), q);
      val = sub_mod(val, conv, q);
      if (!fold) val = mul_shoup(val, T(i, FT_PINV), T(i, FT_PINV_S), q);
    }
    if (add) {
      u64 av = add[(size_t)i * N + addsrc];
      if (addneg && av) av = q - av;
      val = add_mod(val, av, q);
    }
    return val;
  };

  if (!f.rescale) {
    for (int i = 0; i < lq; ++i) dst[(size_t)i * N + x] = limb_value(i);
    return;
  }
  const int last = lq - 1;
  const u64 vl = limb_value(last);
  const u64 ql = T(last, FT_Q), half = ql >> 1;
  const bool pos = vl <= half;
  const u64 dist = pos ? vl : ql - vl;
  auto rescaled = [&](int i, u64 value) {
    const u64 q = T(i, FT_Q);
    const u64 d = dist < q ? dist : mul_shoup(dist, 1, T(i, FT_ONE_S), q);
    const u64 cd = pos ? d : (d == 0 ? 0 : q - d);
    const u64 num = sub_mod(value, cd, q);
    dst[(size_t)i * N + x] = mul_shoup(num, T(i, FT_RINV), T(i, FT_RINV_S), q);
  };
  if (f.wide && last > 0) {
    LimbIn cur = load(0), nxt;
    if (last > 1) nxt = load(1);
#pragma unroll 1
    for (int i = 0; i < last; ++i) {
      LimbIn far;
      if (i + 2 < last) far = load(i + 2);
      rescaled(i, wide_value(i, cur));
      cur = nxt;
      nxt = far;
    }
    return;
  }
  for (int i = 0; i < last; ++i) rescaled(i, limb_value(i));
}

// key relayout [digits][2][limbs][N] (NTT domain) -> [limbs][digits][2][N] in Montgomery form
__global__ void k_key_relayout(const PrimeConst* pc, const u64* src, u64* dst, int digits, int limbs, LimbMap map,
                               int log_n) {
  const u64 N = 1ull << log_n;
  const size_t total = (size_t)digits * 2 * limbs * N;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const u64 x = e & (N - 1);
    size_t r = e >> log_n;
    const int j = (int)(r % limbs);
    r /= limbs;
    const int c = (int)(r % 2);
    const int i = (int)(r / 2);
    const PrimeConst& p = pc[map.prime(j)];
    U128 t;
    t.lo = 0;
    t.hi = src[e];  // v * 2^64 mod q = Montgomery form of v
    dst[(((size_t)j * digits + i) * 2 + c) * N + x] = barrett_reduce(t, p);
  }
}

}  // namespace

template <int WM, class JT>
void launch_decompose(dim3 g, int threads, size_t smem, cudaStream_t s, const PrimeConst* pc, const JT& jt,
                      int32_t* digits, uint64_t g_inv, int log_n, int* tie_flags) {
  if (tie_flags) k_decompose<WM, true, JT><<<g, threads, smem, s>>>(pc, jt, digits, g_inv, log_n, tie_flags);
  else k_decompose<WM, false, JT><<<g, threads, smem, s>>>(pc, jt, digits, g_inv, log_n, nullptr);
}

// the word count is a template parameter (register-resident value); the closest instance at or above W runs
template <class JT>
void decompose_dispatch(int W, dim3 g, int threads, size_t smem, cudaStream_t s, const PrimeConst* pc, const JT& jt,
                        int32_t* digits, uint64_t g_inv, int log_n, int* tie_flags) {
  if (W <= 4) launch_decompose<4>(g, threads, smem, s, pc, jt, digits, g_inv, log_n, tie_flags);
  else if (W <= 8) launch_decompose<8>(g, threads, smem, s, pc, jt, digits, g_inv, log_n, tie_flags);
  else if (W <= 12) launch_decompose<12>(g, threads, smem, s, pc, jt, digits, g_inv, log_n, tie_flags);
  else if (W <= 16) launch_decompose<16>(g, threads, smem, s, pc, jt, digits, g_inv, log_n, tie_flags);
  else if (W <= 20) launch_decompose<20>(g, threads, smem, s, pc, jt, digits, g_inv, log_n, tie_flags);
  else if (W <= 24) launch_decompose<24>(g, threads, smem, s, pc, jt, digits, g_inv, log_n, tie_flags);
  else if (W <= 32) launch_decompose<32>(g, threads, smem, s, pc, jt, digits, g_inv, log_n, tie_flags);
  else launch_decompose<64>(g, threads, smem, s, pc, jt, digits, g_inv, log_n, tie_flags);
}

void decompose(const PrimeConst* pc, const DecompTab& dt, const PtrTab& src, int jobs, int limbs, int D,
               int32_t* digits, uint64_t g_inv, int log_n, cudaStream_t s, int* tie_flags) {
  if (jobs <= 0) return;
  const int N = 1 << log_n;
  const int threads = N < 128 ? N : 128;
  dim3 g((N + threads - 1) / threads, jobs);
  ProfScope p("decompose", s);
  const UniDecomp jt{dt, src, limbs, D};
  decompose_dispatch(dt.W, g, threads, crt_smem_bytes(limbs, dt.W), s, pc, jt, digits, g_inv, log_n, tie_flags);
}

void decompose_ml(const PrimeConst* pc, const DecompTab* d_dts, const MlTab& t, const MlPtrTab& src, int max_limbs,
                  int max_W, int32_t* digits, int log_n, cudaStream_t s) {
  if (t.J <= 0) return;
  const int N = 1 << log_n;
  const int threads = N < 128 ? N : 128;
  dim3 g((N + threads - 1) / threads, t.J);
  ProfScope p("decompose", s);
  const MlDecomp jt{d_dts, t, src};
  decompose_dispatch(max_W, g, threads, crt_smem_bytes(max_limbs, max_W), s, pc, jt, digits, 0, log_n, nullptr);
}

void lift_to_aux(const PrimeConst* pc, const PrimeConst* ppc, const DecompTab& dt, const u64* src, u64* dst,
                 int polys, int limbs, int K, int log_n, cudaStream_t s) {
  if (polys <= 0) return;
  const int N = 1 << log_n;
  const int threads = N < 128 ? N : 128;
  dim3 g((N + threads - 1) / threads, polys);
  const int W = dt.W;
  ProfScope p("lift", s);
  const size_t smem = crt_smem_bytes(limbs, W);
  if (W <= 4) k_lift<4><<<g, threads, smem, s>>>(pc, ppc, dt, src, dst, limbs, K, log_n);
  else if (W <= 8) k_lift<8><<<g, threads, smem, s>>>(pc, ppc, dt, src, dst, limbs, K, log_n);
  else if (W <= 16) k_lift<16><<<g, threads, smem, s>>>(pc, ppc, dt, src, dst, limbs, K, log_n);
  else if (W <= 24) k_lift<24><<<g, threads, smem, s>>>(pc, ppc, dt, src, dst, limbs, K, log_n);
  else if (W <= 32) k_lift<32><<<g, threads, smem, s>>>(pc, ppc, dt, src, dst, limbs, K, log_n);
  else k_lift<64><<<g, threads, smem, s>>>(pc, ppc, dt, src, dst, limbs, K, log_n);
}

void digit_ntt_mac(const KsArgs& a, const int32_t* digits, const u64* const* keys, int jobs, u64* acc,
                   u64* scratch, size_t scratch_elems, cudaStream_t s) {
  if (jobs <= 0) return;
  const int N = a.n, N1 = 1 << a.ntt.n1, N2 = N >> a.ntt.n1;
  const int total = a.qlimbs + a.K;
  const int pairs = jobs * total;
  int chunk = (int)(scratch_elems / ((size_t)a.D * N));
  if (chunk < 1) chunk = 1;
  if (chunk > pairs) chunk = pairs;
  if (chunk > 65535 / a.D) chunk = 65535 / a.D;
  KeyTab kt;
  for (int j = 0; j < jobs && j < MAXP; ++j) kt.k[j] = keys[j];
  const int COLS = N2 < 16 ? N2 : 16;
  int threads_c = 32;
  while (threads_c < 256 && threads_c < N1 * COLS / 2) threads_c <<= 1;
  // row pass: tile = threads * MAC_E elements, whole rows
  int tile = N < 1024 ? N : 1024;
  if (tile < N2) tile = N2;
  int threads_r = tile / MAC_E;
  if (threads_r < 1) threads_r = 1;
  tile = threads_r * MAC_E;
  const int rows = tile / N2;
  for (int p0 = 0; p0 < pairs; p0 += chunk) {
    const int pc_count = (pairs - p0) < chunk ? (pairs - p0) : chunk;
    if (a.ntt.lazy ? digit_dispatch<true>(a, digits, kt, acc, scratch, p0, pc_count, s)
                   : digit_dispatch<false>(a, digits, kt, acc, scratch, p0, pc_count, s))
      continue;
    dim3 g1(N2 / COLS, a.D * pc_count);
    {
      ProfScope p("digit_cols", s);
      k_digit_cols<<<g1, threads_c, N1 * COLS * sizeof(u64), s>>>(a, *a.dt, digits, scratch, p0, pc_count);
    }
    dim3 g2(N1 / rows, pc_count);
    {
      ProfScope p("digit_rows_mac", s);
      k_digit_rows_mac<<<g2, threads_r, tile * sizeof(u64), s>>>(a, scratch, kt, acc, p0);
    }
  }
}

void finalize(const FinalizeArgs& f, const u64* acc, const PtrTab& addend, const PtrTab& out, int jobs,
              cudaStream_t s) {
  if (jobs <= 0) return;
  const int N = f.n;
  // batches: one staging of the limb constants per 256 coefficients; a few jobs: smaller blocks fill the SMs
  const int tpb = jobs >= 8 ? 256 : 128;
  const int threads = N < tpb ? N : tpb;
  dim3 g((N + threads - 1) / threads, 2 * jobs);
  ProfScope p("finalize", s);
  const size_t smem = (size_t)(f.qlimbs + f.K) * ft_stride(f.K) * sizeof(u64);
  const UniFin jt{addend, out, f.qlimbs, f.K};
  auto launch = [&](auto fast) {
    switch (f.K) {
      case 0: k_finalize<UniFin, 0, fast.value><<<g, threads, smem, s>>>(f, acc, jt); break;
      case 1: k_finalize<UniFin, 1, fast.value><<<g, threads, smem, s>>>(f, acc, jt); break;
      case 2: k_finalize<UniFin, 2, fast.value><<<g, threads, smem, s>>>(f, acc, jt); break;
      default: k_finalize<UniFin, -1, fast.value><<<g, threads, smem, s>>>(f, acc, jt);
    }
  };
  if (f.wide && f.lazy) launch(std::true_type{});
  else launch(std::false_type{});
}

void finalize_ml(const FinalizeArgs& f, const MlTab& t, const u64* acc, const MlPtrTab& addend, const MlPtrTab& out,
                 cudaStream_t s) {
  if (t.J <= 0) return;
  const int N = f.n;
  const int tpb = t.J >= 8 ? 256 : 128;
  const int threads = N < tpb ? N : tpb;
  dim3 g((N + threads - 1) / threads, 2 * t.J);
  int max_lq = 0;
  for (int j = 0; j < t.J; ++j) max_lq = t.limbs[j] > max_lq ? t.limbs[j] : max_lq;
  ProfScope p("finalize", s);
  const size_t smem = (size_t)(max_lq + f.K) * ft_stride(f.K) * sizeof(u64);
  const MlFin jt{t, addend, out};
  auto launch = [&](auto fast) {
    switch (f.K) {
      case 0: k_finalize<MlFin, 0, fast.value><<<g, threads, smem, s>>>(f, acc, jt); break;
      case 1: k_finalize<MlFin, 1, fast.value><<<g, threads, smem, s>>>(f, acc, jt); break;
      case 2: k_finalize<MlFin, 2, fast.value><<<g, threads, smem, s>>>(f, acc, jt); break;
      default: k_finalize<MlFin, -1, fast.value><<<g, threads, smem, s>>>(f, acc, jt);
    }
  };
  if (f.wide && f.lazy) launch(std::true_type{});
  else launch(std::false_type{});
}

void key_to_device_form(const NttArgs& a, const PrimeConst* pc, const u64* src, u64* dst, int digits, int limbs,
                        LimbMap map, int n, cudaStream_t s) {
  const size_t total = (size_t)digits * 2 * limbs * n;
  int g = (int)((total + 255) / 256);
  if (g > 65535 * 8) g = 65535 * 8;
  k_key_relayout<<<g, 256, 0, s>>>(pc, src, dst, digits, limbs, map, a.log_n);
}

}  // namespace rc
