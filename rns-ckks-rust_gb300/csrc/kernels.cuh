// Internal interfaces between the C ABI layer and the CUDA kernels.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "modarith.cuh"

namespace rc {

// throws (RC_ERR_CUDA) on a CUDA error; defined with the C ABI
void cuda_check(cudaError_t e, const char* what);

// per-kernel event timing and NVTX ranges (profile.cu); no-ops unless rc_profile_enable turned them on
bool prof_enabled();
bool nvtx_enabled();
void nvtx_push(const char* name);
void nvtx_pop();
void prof_begin(const char* name, cudaStream_t s);
void prof_end(const char* name, cudaStream_t s);
struct ProfScope {
  const char* n;
  cudaStream_t s;
  ProfScope(const char* name, cudaStream_t st) : n(name), s(st) { prof_begin(n, s); }
  ~ProfScope() { prof_end(n, s); }
};

// Up to MAXP polynomials per launch, addressed through a by-value pointer table
// (kernel parameters, so launches need no extra upload and can be captured in
// CUDA graphs).  Limb j of polynomial k lives at p[k] + j * N.
constexpr int MAXP = 128;
struct PtrTab {
  u64* p[MAXP];
};

// Mixed-level batches: up to ML_MAXJ jobs of different levels in one launch per pass.  Job j has
// limbs[j] Q limbs; its digit polynomials are [dig[j], dig[j+1]) of the batch's digit array and its key
// products the limb polynomials [acc[j], acc[j+1]) (2 (limbs[j] + K) of them) of the product array.
constexpr int ML_MAXJ = 128;
struct MlTab {
  int J;
  int limbs[ML_MAXJ];
  int dig[ML_MAXJ + 1];
  int acc[ML_MAXJ + 1];
};
struct MlPtrTab {
  u64* p[2 * ML_MAXJ];
};

// Limb j of a polynomial uses prime prime(j) of the context's Q u P list:
// the first `qcount` limbs are Q primes 0..qcount-1, the rest are the aux
// primes L, L+1, ...
struct LimbMap {
  int qcount;
  int L;
  __host__ __device__ __forceinline__ int prime(int j) const { return j < qcount ? j : L + (j - qcount); }
};

namespace r16 {
// passes of the N = 2^16 transforms that take the 16-residues-per-lane form of nttr16.cuh (bits of NttArgs::r16
// and WidePrimes::r16, tunable "ntt_r16"): 64-bit forward column passes, 64-bit row passes, the tensor's inverse
// rows, the wide key product's column and row passes, 64-bit inverse column passes
enum : int { R16_COLS = 1, R16_ROWS = 2, R16_TENSOR = 4, R16_WCOLS = 8, R16_WROWS = 16, R16_ICOLS = 32, R16_ALL = 63 };
constexpr int R16_DEFAULT = R16_COLS | R16_WCOLS;
}  // namespace r16

struct NttArgs {
  const PrimeConst* pc;
  const Twiddle* tw_fwd;  // [primes][N]: psi^bitrev(k)
  const Twiddle* tw_inv;  // [primes][N]: psi^-bitrev(k)
  int log_n;
  int n1;    // column-phase size 2^n1; row-phase size 2^(log_n - n1) (tunable "ntt_split" for log N 12..16)
  int lazy;  // all primes < 2^57: forward butterflies skip the [0,4q) correction (approximate Shoup products)
  int mont_out = 0;  // inverse: scale by N^-1 2^64 instead of N^-1 (inputs are Montgomery products)
  int lazy_inv = 0;  // all primes < 2^55: the inverse column pass runs without reductions
  int col_ctas = 3;  // column passes: CTAs per SM the kernel is compiled for (2 or 3; more registers at 2)
  int row_polys = 16;  // row passes: polynomials per block sharing one twiddle staging (8 or 16)
  int tensor_jobs = 4;  // tensor + inverse row pass: jobs per block sharing one twiddle staging (tunable)
  int r16 = r16::R16_DEFAULT;  // N = 2^16 split 2^8 x 2^8: passes in the 16-residues-per-lane form (bits above)
  // forward row passes at N = 2^16 (2^8 x 2^8): outputs left unreduced, below (4 log N + 1) q (lazy) or 4q, for
  // the tensor, whose Montgomery products reduce them (set only when those bounds keep its 128-bit sums below
  // q 2^64); other ring sizes and passes, and every caller that did not set it, write outputs in [0, q)
  int raw_out = 0;
};

// Negacyclic NTT over `polys` x `limbs` limbs, src -> dst (may alias).
// Forward: canonical coefficients -> canonical evaluations in bit-reversed order.
// Inverse: the reverse, including the N^-1 scaling.
void ntt_forward(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
                 cudaStream_t s);
void ntt_inverse(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
                 cudaStream_t s);

// NTT-domain (a0, a1, b0, b1) = in4.p[4j..4j+3] -> out3.p[3j..3j+2] = the inverse row phase of (a0 b0,
// a0 b1 + a1 b0, a1 b1) as Montgomery products; ntt_inverse_cols with NttArgs::mont_out then completes the
// inverse transform.  False (nothing launched) if N is not supported (log N outside 12..16).
bool tensor_inverse_rows(const NttArgs& a, const PtrTab& in4, const PtrTab& out3, int jobs, int limbs, LimbMap map,
                         cudaStream_t s);
// the forward transform's column phase alone (src -> dst; the row phase is done elsewhere); false (nothing
// launched) if N is not supported (log N outside 12..16)
bool ntt_forward_cols(const NttArgs& a, const PtrTab& src, const PtrTab& dst, int polys, int limbs, LimbMap map,
                      cudaStream_t s);
// the inverse transform's column phase alone (in place, times N^-1), after a row phase done elsewhere
bool ntt_inverse_cols(const NttArgs& a, const PtrTab& data, int polys, int limbs, LimbMap map, cudaStream_t s);

// Coefficient-form ciphertext pairs in4.p[4j..4j+3] = (a0, a1, b0, b1) -> coefficient-form
// out3.p[3j..3j+2] = (a0 b0, a0 b1 + a1 b0, a1 b1): forward column phase into work4, one fused kernel for the
// forward row phase, the NTT-domain tensor and the inverse row phase, then the inverse column phase in place.
// False (nothing launched) if N is not supported (log N outside 12..16).
bool tensor_fused(const NttArgs& a, const PrimeConst* pc, const PtrTab& in4, const PtrTab& work4,
                  const PtrTab& out3, int jobs, int limbs, LimbMap map, cudaStream_t s);

// ---- elementwise / scheme kernels (ops.cu) ----
// MulMont: x y 2^-64 mod q (Montgomery), for products an inverse transform with NttArgs::mont_out follows
enum class EwOp { Add, Sub, Mul, MulMont };
// out[k] = a[k] (op) b[k] over `polys` polys of `limbs` limbs; b may be shared
// across polys (b_shared != 0 uses b.p[0] for every poly).
void ew_binary(EwOp op, const PrimeConst* pc, const PtrTab& a, const PtrTab& b, int b_shared, const PtrTab& out,
               int polys, int limbs, LimbMap map, int n, cudaStream_t s);
// acc[c] (+)= sum_k ct[k][c] * pt[k] mod q for c in {0,1}: NTT-domain plaintext products summed over `count`
// terms (ct.p[k] -> component 0 of term k, component 1 at +limbs*n); accumulate != 0 adds to acc
void plain_mac(const PrimeConst* pc, const PtrTab& ct, const PtrTab& pt, int count, u64* acc, int accumulate,
               int limbs, LimbMap map, int n, cudaStream_t s);
// out_j = a_j * v[j] mod q_j
struct ScalarTab {
  u64 v[80];
};
void mul_scalar(const PrimeConst* pc, const u64* a, const ScalarTab& v, u64* out, int limbs, LimbMap map, int n,
                cudaStream_t s);
// NTT-domain tensor: for each job j, in = [a0,a1,b0,b1] (4 polys) -> out = [d0,d1,d2] * 2^-64 (Montgomery
// products; an inverse transform with NttArgs::mont_out takes the factor out)
void tensor_ntt(const PrimeConst* pc, const PtrTab& in4, const PtrTab& out3, int jobs, int limbs, int n,
                cudaStream_t s);
// coefficient-domain Galois automorphism X -> X^g (signed permutation), g given by its inverse mod 2N
void automorphism(const PrimeConst* pc, const PtrTab& in, const PtrTab& out, int polys, int limbs, uint64_t g_inv,
                  int log_n, cudaStream_t s);

struct RescaleTab {
  const u64* inv;    // [L][L]: inv[(l-1)*L + i] = q_{l-1}^-1 mod q_i
  const u64* inv_s;  // Shoup companions
};
// rescale_poly_rns for `polys` polys at `limbs` limbs -> limbs-1
void rescale(const PrimeConst* pc, const RescaleTab& rt, int L, const PtrTab& in, const PtrTab& out, int polys,
             int limbs, int n, cudaStream_t s);

// ---- keyswitch (keyswitch.cu) ----
struct DecompTab {
  const u64* qhat;       // [limbs][W] words of Q/q_i
  const u64* qhat_inv;   // [limbs] (Q/q_i)^-1 mod q_i
  const u64* qhat_inv_s; // Shoup companions
  const u64* inv_q;      // [limbs] 1/q_i in fixed point: (n << 32) | floor(2^95 / (q_i << n)), n = 64 - bits(q_i)
  const u64* Q;          // [W]
  const u64* halfQ;      // [W]
  int W;                 // words for Q (with headroom for the CRT sum)
  int small_q;           // Q <= 2^30: digits need the general centred lift
  u64 Qsmall;            // Q when small_q
  const u64* lift_pw;    // [K][W+1]: 2^(64 w) mod p_k (the aux primes), w = 0..W
  const u64* lift_pw_s;  // Shoup companions
};

struct ModDownTab {
  // aux basis P (K primes): Garner inverses and mixed-radix weights
  const u64* p_garner;    // [K][K]: p_garner[k*K + t] = p_t^-1 mod p_k (t < k)
  const u64* p_garner_s;
  const u64* halfP;       // [KW]
  int KW;                 // words of P
  // per Q prime i: P^-1 mod q_i, P mod q_i, M_k mod q_i (M_k = p_0..p_{k-1})
  const u64* pinv;        // [L]
  const u64* pinv_s;
  const u64* pmod;        // [L]
  const u64* mk;          // [L][K]
  const u64* mk_s;
};

// lift_poly_to_context (keyswitching.rs:242-276): polys polynomials over Q_limbs ([polys][limbs][N]) to
// Q_limbs u P ([polys][limbs + K][N]); ppc = the aux primes' constants.
void lift_to_aux(const PrimeConst* pc, const PrimeConst* ppc, const DecompTab& dt, const u64* src, u64* dst,
                 int polys, int limbs, int K, int log_n, cudaStream_t s);
// digits[job][d][x] (int32) of the centred CRT value of src (optionally read
// through the automorphism with inverse element g_inv; 0/1 = none).  tie_flags (optional, [jobs], zeroed by
// the caller) get 1 where a digit equals -2^29: only then can the digits of -X differ from the negated
// digits of X (the balanced rule sends both +2^29 and -2^29 to -2^29)
void decompose(const PrimeConst* pc, const DecompTab& dt, const PtrTab& src, int jobs, int limbs, int D,
               int32_t* digits, uint64_t g_inv, int log_n, cudaStream_t s, int* tie_flags = nullptr);

// Exact integer key product ("wide-CRT"): S = sum_i d_i * k_i is carried under
// four internal primes w0..w3 < 2^29 (product A), handled as two pairs
// (w0, w1), (w2, w3) whose residues sit side by side in a uint2.
struct WidePrimes {
  uint32_t q[4];
  // the inverse transform's scale: N^-1 2^32 mod q (+ Shoup), since the key product's outputs, the only values
  // it transforms, carry the factor 2^-32 of their Montgomery reduction (mont64_32)
  uint32_t n_inv[4], n_inv_s[4];
  uint32_t w1n[4], w1n_s[4];      // the inverse transform's stage-0 twiddle times that scale (+ Shoup), InvScale2
  u64 bar[4];                     // floor(2^64 / q): 64-bit -> residue reduction
  uint32_t qinv_neg[4];           // -q^-1 mod 2^32
  uint32_t kq[4];                 // floor(2^31 / q) q
  const Tw2* tw_fwd;              // [2 pairs][N]: psi^bitrev(k)
  const Tw2* tw_inv;              // [2 pairs][N]: psi^-bitrev(k)
  int log_n;
  // polls of the key product's first wait for its staged digit transforms (tunable "mac_wait_polls"; a
  // limit of 0 makes every CTA time out, which tests the error path without a fault)
  uint32_t first_wait_polls = 1u << 22;
  // uniform batches of more than two jobs per CTA take the persistent key product (tunable "mac_persistent")
  int persistent = 1;
  // N = 2^16: transform passes in the 16-residues-per-lane form (bits of r16::R16_*)
  int r16 = r16::R16_DEFAULT;
};
// Garner CRT of (S mod w0..w3) to the centred integer S (|S| < A/4), reduced mod
// each scheme prime t.
struct WideTab {
  uint32_t w[4];
  uint32_t g01, g01s, g02, g02s, g12, g12s;  // w0^-1 mod w1, w0^-1 mod w2, w1^-1 mod w2 (+ Shoup)
  uint32_t g03, g03s, g13, g13s, g23, g23s;  // w0^-1, w1^-1, w2^-1 mod w3 (+ Shoup)
  uint32_t half3;                            // top mixed-radix digit >= half3 <=> S >= A/2
  const u64* c01_mod_t;                      // [Q u P] (w0 w1) mod t and its Shoup companion
  const u64* c01_mod_t_s;
  const u64* A_mod_t;                        // [Q u P] A mod t
  // with an aux basis P, the same constants times P^-1 mod q_i for the Q primes, so the CRT lands directly on
  // S * P^-1 and ModDown needs no separate multiply: [L] (w0 w1 P^-1) mod q_i (+ Shoup), (A P^-1) mod q_i,
  // and [L][K] (M_k P^-1) mod q_i (+ Shoup)
  const u64* c01p;
  const u64* c01p_s;
  const u64* ap;
  const u64* mkp;
  const u64* mkp_s;
};

struct KsArgs {
  const PrimeConst* pc;
  NttArgs ntt;
  int n;
  int L;          // Q chain length (for the limb map)
  int qlimbs;     // active Q limbs
  int K;          // aux limbs used (0 = Q-only)
  int D;          // digits decomposed (and used from the key)
  int key_digits; // digits stored per key limb
  int mac64;      // key product with 64-bit per-term Montgomery accumulators
  const DecompTab* dt;
};

// For each job: NTT every digit into each extended-basis limb and accumulate
// against the key -> acc[job][2][qlimbs+K][N] (NTT domain, canonical).
// scratch must hold jobs * chunk * D * N u64 (chunk = limbs per pass).
void digit_ntt_mac(const KsArgs& a, const int32_t* digits, const u64* const* keys, int jobs, u64* acc,
                   u64* scratch, size_t scratch_elems, cudaStream_t s);

// ModDown (if K>0) + optional addend (optionally through an automorphism) +
// optional rescale; acc in coefficient form [job][2][qlimbs+K][N].
// addend.p[2*job + c] (null = none); out.p[2*job + c].
struct FinalizeArgs {
  const PrimeConst* pc;
  ModDownTab md;
  RescaleTab rt;
  int L, n, log_n;
  int qlimbs, K;
  int rescale;
  uint64_t add_g_inv;  // automorphism applied to the addend (0/1 = none)
  int wide;            // acc holds [job][2][limbs][2 pairs][N] uint2 residues mod w0..w3 to CRT-combine
  WideTab wt;
  int lazy;            // every prime below 2^64 / (8 + 2K): a limb's terms are summed unreduced
};
void finalize(const FinalizeArgs& f, const u64* acc, const PtrTab& addend, const PtrTab& out, int jobs,
              cudaStream_t s);

// ---- mixed-level forms (one launch per pass; f.qlimbs unused) ----
// digits of job j (src.p[j], limbs[j] Q limbs) from polynomial dig[j] of `digits`; d_dts[limbs] are the
// per-level tables, max_limbs / max_W the largest job's
void decompose_ml(const PrimeConst* pc, const DecompTab* d_dts, const MlTab& t, const MlPtrTab& src, int max_limbs,
                  int max_W, int32_t* digits, int log_n, cudaStream_t s);
// finalize of wide products acc (job j's 2 (limbs[j] + K) limb polynomials from acc[j] on)
void finalize_ml(const FinalizeArgs& f, const MlTab& t, const u64* acc, const MlPtrTab& addend, const MlPtrTab& out,
                 cudaStream_t s);
// the jobs of one key in a mixed-level key product: jobs [first, first + count) (consecutive), the key's
// tiled wide form, its digits used (D) and stored (key_digits), limbs + K of the level
struct MlKey {
  const uint2* kwt;
  int D, key_digits, total, first, count;
};
constexpr int ML_MAXK = 64;
struct MlKeys {
  int n;
  MlKey k[ML_MAXK];
};
// digit transforms of every job (dig[J] digit polynomials), tiled per job: job j's tiles from 2 N dig[j]
bool wide_digit_transforms_ml(const WidePrimes& w, const MlTab& t, const int32_t* digits, uint2* work, uint2* dtt,
                              cudaStream_t s);
// key products of every job into acc (job j's [c][limb][pair][N] from 2 N acc[j]), one launch
void wide_mac_ml(const WidePrimes& w, const MlTab& t, const MlKeys& keys, const uint2* dtt, uint2* acc, int bc_max,
                 cudaStream_t s);

// ---- RNS-hybrid ("dnum") key switching (dnum.cu) ----
// ModUp of each job's coefficient-form polynomial src.p[job] ([qlimbs][N]) group by group:
// D[job][b][limb][N] over the qlimbs Q limbs and the aux limbs (total), tab = [dnum][alpha][2 + total]
// ((Q_b/q_i)^-1 mod q_i, its Shoup companion, then (Q_b/q_i) mod every target prime); alpha <= 8
void dnum_modup(const PrimeConst* pc, const PtrTab& src, int jobs, const u64* tab, u64* D, int qlimbs, int total,
                int alpha, int dnum, LimbMap map, int log_n, cudaStream_t s);
// acc[job][c][limb][N] = sum_b D[job][b] * key[b][c] (NTT domain; key [dnum][2][total][N]; dnum <= 16)
void dnum_mac(const PrimeConst* pc, const u64* D, const u64* key, u64* acc, int jobs, int total, int dnum,
              LimbMap map, int log_n, cudaStream_t s);

// ---- wide-CRT key product (wide.cu) ----
// digits [job][digit][N] -> transforms under w0..w3, written tiled:
// dtt[job][pair][x/32][digit][32].  `work` holds jobs*D*2*N uint2.  False if N
// is unsupported (log N outside 12..16).
bool wide_digit_transforms(const WidePrimes& w, int D, int jobs, const int32_t* digits, uint2* work, uint2* dtt,
                           cudaStream_t s);
// acc[b][c][j][pair][N] (NTT domain, reduced) for jobs b0..b0+nb-1 sharing the
// tiled key kwt[j][pair][x/32][digit][c][32]; gal > 1 reads the digit transforms through the automorphism
// X -> X^gal (their NTT-domain permutation: hoisted rotations of one decomposition)
void wide_mac(const WidePrimes& w, int D, int key_digits, int total, const uint2* kwt, const uint2* dtt, uint2* acc,
              int b0, int nb, int bc_max, cudaStream_t s, uint32_t gal = 0);
// nonzero if a key-product launch timed out waiting for its bulk copies (then its outputs are not valid);
// reads the device flag (synchronising) and optionally clears it
int wide_kernel_errors(bool clear);
// inverse transforms of `polys` consecutive [pair][N] polynomials, in place
bool wide_inverse(const WidePrimes& w, uint2* data, int polys, cudaStream_t s);
// coefficient-form key [digits][2][limbs][N] (residues mod the scheme primes) ->
// tiled wide key kwt; `tmp` holds digits*2*limbs*2*N uint2
bool wide_key_build(const WidePrimes& w, const u64* key, int digits, int limbs, uint2* tmp, uint2* kwt,
                    cudaStream_t s);

// key upload: coefficient-form key [digits][2][limbs][N] (device) ->
// [limbs][digits][2][N] NTT domain, Montgomery form
void key_to_device_form(const NttArgs& a, const PrimeConst* pc, const u64* src, u64* dst, int digits, int limbs,
                        LimbMap map, int n, cudaStream_t s);

}  // namespace rc
