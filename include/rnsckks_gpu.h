/*
 * rnsckks_gpu.h — C ABI of the GB300 (sm_103a) RNS-CKKS ciphertext-arithmetic
 * library.  It is the drop-in boundary for the hot path of the Rust crate
 * Akram275/rns-ckks-rust: each entry point names the reference function it
 * replaces (paths relative to that crate).
 *
 * Conventions
 *  - Every function returns an int status (RC_OK = 0).  On failure the message
 *    is available from rc_last_error(ctx); nothing aborts.  Where the
 *    reference panics on a precondition (level/scale/shape mismatch) the
 *    library returns RC_ERR_INVALID_ARGUMENT with the reference's message.
 *  - Polynomials are u64 residues in [0, q_i), limb-major [limbs][N], in
 *    coefficient form (the reference's representation).  Ciphertext data is
 *    [components][limbs][N] contiguous: 2 components for RnsCiphertext, 3 for
 *    RnsQuadraticCiphertext.  `level` = limbs - 1, as in the reference.
 *  - Ops on rc_ciphertext take DEVICE pointers and run on the given CUDA
 *    stream (`void*` holding a cudaStream_t; NULL = legacy default stream).
 *    Functions with the suffix _host take HOST pointers and include the
 *    host<->device copies.
 *  - Keys are uploaded once (coefficient form, reference layout) and kept
 *    device-resident in the NTT domain.
 *  - One context may be used from several host threads on distinct streams.
 *    Calls on the same stream are ordered; the library's scratch memory is per
 *    stream.
 */
#ifndef RNSCKKS_GPU_H
#define RNSCKKS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RC_OK 0
#define RC_ERR_INVALID_ARGUMENT 1
#define RC_ERR_CUDA 2
#define RC_ERR_OUT_OF_MEMORY 3
#define RC_ERR_UNSUPPORTED 4

typedef struct rc_context rc_context;
typedef struct rc_ksk rc_ksk;
typedef struct rc_graph rc_graph;

/* RnsPrime{modulus, primitive_root}: src/rns/basis.rs:8-22 */
typedef struct {
  uint64_t modulus;
  uint64_t primitive_root;
} rc_prime;

/* RnsCkksParams{poly_degree, primes, aux_primes, scale_bits}: src/rns/context.rs:16-21 */
typedef struct {
  uint64_t poly_degree;
  const rc_prime* primes;
  uint32_t prime_count;
  const rc_prime* aux_primes;
  uint32_t aux_count;
  uint32_t scale_bits;
} rc_params;

/* RnsCiphertext / RnsQuadraticCiphertext {c0, c1[, c2], scale_bits, level}:
 * src/rns/ciphertexts.rs:4-18.  `data` is a device pointer to
 * [components][level+1][N] residues. */
typedef struct {
  uint64_t* data;
  int32_t level;
  int32_t scale_bits;
} rc_ciphertext;

/* ---- context: RnsCkksContext::new, src/rns/context/construction.rs:9-31,
 *      with RnsCkksParams::validate, src/rns/context/params.rs:48-73 ---- */
int rc_context_create(const rc_params* params, rc_context** out);
void rc_context_destroy(rc_context* ctx);
const char* rc_last_error(const rc_context* ctx);
/* Device-side error flags of the library's kernels (no reference counterpart): nonzero when a key-product
 * launch gave up waiting for its bulk copies.  Such a CTA drains its copies and writes nothing, so the
 * results of every operation issued since the flag was last clear are invalid and must be discarded.
 * Synchronises the device; clear != 0 resets the flags.  A failed read of the flag returns RC_ERR_CUDA. */
int rc_kernel_errors(int32_t* flags, int32_t clear);
/* levels(), num_slots(), poly_degree, aux count: context.rs:57-95 */
int rc_context_info(const rc_context* ctx, uint64_t* poly_degree, uint32_t* levels, uint32_t* aux_count,
                    uint32_t* scale_bits);
/* num_decomp_digits(bits(Q_level), 30): src/rns/keyswitching.rs:238-240 */
int rc_decomp_digits(const rc_context* ctx, int32_t level, uint32_t* digits);
/* Pre-size the per-stream scratch for ops on `max_batch` ciphertexts at
 * `max_level` (so later calls, e.g. under CUDA graph capture, allocate nothing). */
int rc_reserve(rc_context* ctx, int32_t max_level, uint32_t max_batch, void* stream);

/* Tunables (no reference counterpart; results never depend on them): "ks_jobs" (jobs per key-switch
 * launch, 1..64, default 32), "mac_bc" (most jobs per CTA of the key product: 1, 2, 4, 8), "host_chunk" (jobs
 * per stage of the pipelined host-buffer entry, default 8), "host_edge" (its first and last stages have
 * host_chunk / host_edge jobs, default 2), "lazy_ntt" (unreduced forward butterflies, only
 * when every prime is below 2^58), "fuse_tensor" (forward row phase + tensor + inverse row phase of a
 * ciphertext product in one kernel, default 1), "host_phased" (host-buffer batches of up to ks_jobs same-level
 * jobs: 1 = one key read for the batch, copies overlapped chunk by chunk; 2 = two such groups on two compute
 * streams, the second's copy-in and preparation overlapping the first's key product; 0 = independent
 * stages; default 1), "mixed_levels" (relinearize batches
 * whose jobs are at different levels: one launch per pass over all levels instead of one per level, default
 * 1), "ml_jobs" (jobs per such launch, 1..128, default 128), "mac_wait_polls" (polls of
 * the key product's first wait for its staged digit transforms, 0..2^22, default 2^22; 0 makes every CTA
 * time out and raise the rc_kernel_errors flag, for testing that path), "mac_persistent" (key products of
 * more than two jobs per CTA in one persistent CTA per SM taking (tile, limb) units, the next tile's digit
 * transforms copied while the current one is used; default 1), "ntt_split" (log size of the four-step
 * column phase, both phases 2^6..2^8 points), "col_ctas" (CTAs per SM of the column pass: 2 or 3),
 * "row_polys" (polynomials per row block: 8 or 16).  Set them between calls, not while calls on the context
 * are in flight. */
int rc_tune_set(rc_context* ctx, const char* name, int32_t value);
int rc_tune_get(const rc_context* ctx, const char* name, int32_t* value);

/* ---- keys ---- */
/* RnsKeySwitchingKey{ksk, decomp_bits, level, aux_level_count}:
 * src/rns/keyswitching.rs:13-18.  `host_key` = [digits][2][level+1+aux_count][N]
 * coefficient-form residues (ksk[i].c0, ksk[i].c1), aux_count = 0 (Q-only key)
 * or the context's aux prime count (hybrid key).  The key is transformed once
 * on upload.  galois_element = 0 for a relinearisation key, otherwise the
 * RnsRotationKey's element (src/rns/rotation.rs:9-12). */
int rc_ksk_upload(rc_context* ctx, const uint64_t* host_key, uint32_t digits, int32_t level, uint32_t aux_count,
                  uint64_t galois_element, rc_ksk** out);
/* Same as rc_ksk_upload with the coefficient-form key already in device memory
 * (e.g. generated on the GPU); the source buffer is not modified. */
int rc_ksk_upload_device(rc_context* ctx, const uint64_t* device_key, uint32_t digits, int32_t level,
                         uint32_t aux_count, uint64_t galois_element, rc_ksk** out);
/* RNS-hybrid ("dnum") relinearization key at `level` (no reference counterpart: the reference's only gadget
 * is balanced base-2^30 digits, keyswitching.rs:238-240).  The active chain is cut into dnum = ceil((level+1)
 * / alpha) groups of alpha consecutive limbs (1 <= alpha <= aux count, at most 8; every prime below 2^60);
 * key = [dnum][2][level + 1 + aux][N] coefficient-form residues over Q_level u P (host memory, or device memory
 * with key_on_device != 0), group b's pair encrypting [i in group b] (P mod q_i) s^2 as (e - a s + that, a).
 * Relinearization and mult_relinearized with such a key extend each group of c2 to Q u P by a fast basis
 * conversion, multiply by the key in the NTT domain and ModDown by P: the results decrypt to the same values
 * as with the reference's gadget but are not its residues.  Relinearization only; not serialisable. */
int rc_ksk_upload_dnum(rc_context* ctx, const uint64_t* key, int32_t key_on_device, uint32_t alpha, int32_t level,
                       rc_ksk** out);
/* RnsKeySwitchingKey::truncate_levels (Q-only keys): keyswitching.rs:32-41 */
int rc_ksk_truncate(rc_context* ctx, const rc_ksk* key, int32_t level, rc_ksk** out);
int rc_ksk_info(const rc_ksk* key, uint32_t* digits, int32_t* level, uint32_t* aux_count, uint64_t* galois_element);
void rc_ksk_destroy(rc_ksk* key);
/* Serialised keys (no counterpart in the reference, which has none): a 96-byte header (magic "RCKSKEY1",
 * version, form, N, digits, level, aux_count, galois element, payload bytes, fingerprint of the modulus chain,
 * payload checksum) followed by the key exactly as it is resident (NTT domain, the library's layout), so
 * reloading is one host->device copy.  A record loads only into a context with the same ring degree and
 * modulus chain; a truncated Q-only key serialises its prefix of limbs.  rc_ksk_serialize writes into a
 * caller buffer of at least rc_ksk_serialized_size bytes and returns when the buffer is filled. */
int rc_ksk_serialized_size(const rc_ksk* key, uint64_t* bytes);
int rc_ksk_serialize(rc_context* ctx, const rc_ksk* key, void* host_buf, uint64_t buf_bytes, void* stream);
int rc_ksk_deserialize(rc_context* ctx, const void* host_buf, uint64_t buf_bytes, rc_ksk** out);

/* ---- polynomial-level ops (device pointers, limb-major) ---- */
/* NttPlan::forward/inverse composed with the negacyclic twist
 * (src/math/ntt.rs:78-89, src/poly/mod.rs:134-175): for `polys` polynomials of
 * `limbs` limbs laid out [polys][limbs][N], limb j using prime j of the chain
 * (limbs <= levels) or, when with_aux != 0, primes 0..limbs-aux-1 followed by
 * the aux primes.  Output order: evaluation at psi^(2k+1) stored at
 * bit-reversed index k. */
int rc_ntt_forward(rc_context* ctx, uint64_t* data, uint32_t polys, uint32_t limbs, int32_t with_aux, void* stream);
int rc_ntt_inverse(rc_context* ctx, uint64_t* data, uint32_t polys, uint32_t limbs, int32_t with_aux, void* stream);
/* RnsPolynomial::multiply_ntt: src/rns/polynomial.rs:121-136.  with_aux != 0:
 * the polynomial is over Q_(limbs-aux) followed by the aux primes (the
 * eval-key basis, context.rs:104-118). */
int rc_poly_multiply(rc_context* ctx, const uint64_t* a, const uint64_t* b, uint64_t* out, uint32_t limbs,
                     int32_t with_aux, void* stream);
/* RnsPolynomial::add / sub: polynomial.rs:99-119 */
int rc_poly_add(rc_context* ctx, const uint64_t* a, const uint64_t* b, uint64_t* out, uint32_t limbs,
                int32_t with_aux, void* stream);
int rc_poly_sub(rc_context* ctx, const uint64_t* a, const uint64_t* b, uint64_t* out, uint32_t limbs,
                int32_t with_aux, void* stream);
/* Allocation-free form of rc_poly_multiply for callers that may not allocate
 * device memory through this library (a host that owns the whole GPU pool, or
 * a latency-critical loop that cannot take cudaMalloc's device-wide
 * synchronisation).  No counterpart in the reference (which has no device
 * memory at all).  Scratch is a fixed 16 MiB array inside the library, so
 * limbs * N must not exceed 2^20 (RC_ERR_INVALID_ARGUMENT otherwise).  The
 * first call on a device looks the array up and should precede any CUDA graph
 * capture; all calls share the array, so calls that overlap on the GPU race. */
int rc_poly_multiply_noalloc(rc_context* ctx, const uint64_t* a, const uint64_t* b, uint64_t* out, uint32_t limbs,
                             int32_t with_aux, void* stream);
/* out_j = a_j * scalars[j] mod q_j (scalars: host array, one per limb): the
 * per-prime reduction of (coefficient * B^i [* P]) in key generation,
 * src/rns/keyswitching.rs:64-68,108-112 */
int rc_poly_mul_scalar(rc_context* ctx, const uint64_t* a, const uint64_t* scalars, uint64_t* out, uint32_t limbs,
                       int32_t with_aux, void* stream);
/* RnsCkksContext::apply_galois_automorphism: src/rns/context/rotation.rs:6-10,
 * src/poly/mod.rs:110-131 */
int rc_poly_automorphism(rc_context* ctx, const uint64_t* a, uint64_t* out, uint32_t limbs, uint64_t galois_element,
                         void* stream);

/* ---- seeded samplers on the device (key generation and encryption inputs) ----
 * The distributions of src/rns/keys.rs, written as residues over `limbs` limbs (with_aux as for
 * rc_poly_multiply) into out[limbs][N]: rc_sample_uniform = 64 random bits mod q_j per residue
 * (sample_uniform_poly, keys.rs:87-99); rc_sample_error = round(N(0, 3.19)) per coefficient, the same integer
 * in every limb (sample_gaussian_i64 / sample_error_poly, keys.rs:82-85,101-121); rc_sample_ternary = uniform
 * {0, 1, -1} per coefficient (sample_ternary_poly, keys.rs:123-147).  Every value is a function of
 * (seed, stream_id, index) through Philox4x32-10, so a (seed, stream_id) pair names one reproducible sample;
 * callers use a distinct stream_id for each polynomial they draw.  The reference seeds from the OS, so its
 * samples are not reproducible and are not compared value for value. */
int rc_sample_uniform(rc_context* ctx, uint64_t seed, uint64_t stream_id, uint64_t* out, uint32_t limbs,
                      int32_t with_aux, void* stream);
int rc_sample_error(rc_context* ctx, uint64_t seed, uint64_t stream_id, uint64_t* out, uint32_t limbs,
                    int32_t with_aux, void* stream);
int rc_sample_ternary(rc_context* ctx, uint64_t seed, uint64_t stream_id, uint64_t* out, uint32_t limbs,
                      int32_t with_aux, void* stream);

/* ---- ciphertext ops (RnsCkksContext, src/rns/context/ops.rs) ---- */
/* RnsCiphertext::add: src/rns/ciphertexts.rs:60-69 */
int rc_add(rc_context* ctx, const rc_ciphertext* lhs, const rc_ciphertext* rhs, rc_ciphertext* out, void* stream);
/* mult_plain: context/ops.rs:20-30 (scale doubles) */
int rc_mult_plain(rc_context* ctx, const rc_ciphertext* ct, const uint64_t* plain, rc_ciphertext* out, void* stream);
/* multiply_plain_rns: src/rns/ops.rs:54-66 (scale unchanged) */
int rc_multiply_plain_rns(rc_context* ctx, const rc_ciphertext* ct, const uint64_t* plain, rc_ciphertext* out,
                          void* stream);
/* `count` independent RnsCiphertext::add / multiply_plain_rns jobs in one call (same rules and messages as
 * the single forms; jobs may mix levels). */
int rc_add_batch(rc_context* ctx, uint32_t count, const rc_ciphertext* lhs, const rc_ciphertext* rhs,
                 rc_ciphertext* out, void* stream);
int rc_multiply_plain_rns_batch(rc_context* ctx, uint32_t count, const rc_ciphertext* ct,
                                const uint64_t* const* plains, rc_ciphertext* out, void* stream);
/* `count` independent rescales (context/ops.rs:32-37) in one call */
int rc_rescale_batch(rc_context* ctx, uint32_t count, const rc_ciphertext* ct, rc_ciphertext* out, void* stream);
/* Serialised ciphertexts: a 64-byte header (magic "RCCTXT01", version, components (2 or 3), N, level,
 * scale_bits, payload bytes, modulus-chain fingerprint, checksum) followed by the [components][level+1][N]
 * coefficient-form residues.  rc_ct_header reads the header of a record (no context needed) so the caller can
 * allocate the device buffer rc_ct_deserialize fills; out->level and out->scale_bits are set from the record.
 * out_bytes is the capacity of out->data: a record whose payload is larger is refused, nothing is written. */
int rc_ct_serialized_size(const rc_context* ctx, int32_t level, uint32_t components, uint64_t* bytes);
int rc_ct_serialize(rc_context* ctx, const rc_ciphertext* ct, uint32_t components, void* host_buf,
                    uint64_t buf_bytes, void* stream);
int rc_ct_header(const void* host_buf, uint64_t buf_bytes, uint64_t* poly_degree, int32_t* level,
                 int32_t* scale_bits, uint32_t* components);
int rc_ct_deserialize(rc_context* ctx, const void* host_buf, uint64_t buf_bytes, rc_ciphertext* out,
                      uint64_t out_bytes, void* stream);
/* lift_poly_to_context: src/rns/keyswitching.rs:242-276 (convert_centered_residues_to_target, 365-379).
 * `polys` polynomials over Q_limbs ([polys][limbs][N]) -> over Q_limbs followed by the aux primes
 * ([polys][limbs + aux_count][N]): the Q limbs are copied, each aux limb is the centred CRT value (the tie
 * X == floor(Q/2) stays positive) mod that prime.  Requires an aux basis. */
int rc_lift_to_aux(rc_context* ctx, const uint64_t* a, uint64_t* out, uint32_t polys, uint32_t limbs,
                   void* stream);
/* mod_raise: src/ckks/bootstrapping/mod_raise.rs:29-45.  out->data holds [2][level + 1 + aux_count][N]
 * (c0 then c1 over the eval-key basis); out->level = ct->level + aux_count (the eval-key context's level),
 * scale unchanged.  The first level + 1 limbs of each component are the input's. */
int rc_mod_raise(rc_context* ctx, const rc_ciphertext* ct, rc_ciphertext* out, void* stream);
/* Sum over k of mult_plain(cts[k], plains[k]), the inner sum of the BSGS linear transform
 * (apply_giant_step_terms, src/ckks/bootstrapping/linear_transform.rs:234-252: mult_plain, context/ops.rs:20-30,
 * folded with RnsCiphertext::add, ciphertexts.rs:60-69).  All cts share level and scale; out gets the level and
 * twice the scale.  cts_ntt / plains_ntt = 1 when those inputs are already in the NTT domain (as written by
 * rc_ntt_forward), so a caller can transform baby-step rotations and diagonals once and reuse them; the
 * products are summed in the NTT domain and transformed back once.  Output in coefficient form. */
int rc_mult_plain_accumulate(rc_context* ctx, uint32_t count, const rc_ciphertext* cts, int32_t cts_ntt,
                             const uint64_t* const* plains, int32_t plains_ntt, rc_ciphertext* out, void* stream);
/* mult: context/ops.rs:63-70 -> multiply_ciphertexts_rns, src/rns/ops.rs:84-100 */
int rc_mult(rc_context* ctx, const rc_ciphertext* lhs, const rc_ciphertext* rhs, rc_ciphertext* out_quadratic,
            void* stream);
/* rescale: context/ops.rs:32-37 -> rescale_ciphertext_rns, src/rns/ops.rs:68-82 */
int rc_rescale(rc_context* ctx, const rc_ciphertext* ct, rc_ciphertext* out, void* stream);
/* rescale_quadratic: context/ops.rs:85-90 -> src/rns/ops.rs:115-133 */
int rc_rescale_quadratic(rc_context* ctx, const rc_ciphertext* ct, rc_ciphertext* out, void* stream);
/* keyswitch: context/ops.rs:97-109 -> keyswitch_rns / keyswitch_rns_hybrid,
 * src/rns/keyswitching.rs:130-194.  `poly` holds level+1 limbs. */
int rc_keyswitch(rc_context* ctx, const uint64_t* poly, int32_t level, const rc_ksk* key, rc_ciphertext* out,
                 void* stream);
/* relinearize: context/ops.rs:111-122 */
int rc_relinearize(rc_context* ctx, const rc_ciphertext* quadratic, const rc_ksk* key, rc_ciphertext* out,
                   void* stream);
/* mult_relinearized: context/ops.rs:124-133 (tensor, relinearize, rescale) */
int rc_mult_relinearized(rc_context* ctx, const rc_ciphertext* lhs, const rc_ciphertext* rhs, const rc_ksk* key,
                         rc_ciphertext* out, void* stream);
/* rotate / conjugate: context/rotation.rs:104-135 (the key carries the Galois element) */
int rc_rotate(rc_context* ctx, const rc_ciphertext* ct, const rc_ksk* rotation_key, rc_ciphertext* out, void* stream);
/* rotate_raw / conjugate_raw / apply_galois_automorphism on a ciphertext:
 * src/rns/ciphertexts.rs:36-46,71-78 */
int rc_automorphism(rc_context* ctx, const rc_ciphertext* ct, uint64_t galois_element, rc_ciphertext* out,
                    void* stream);

/* ---- batched forms: `count` independent jobs in as few launches as the
 * (level, key) grouping allows; jobs may mix levels. ---- */
int rc_mult_relinearized_batch(rc_context* ctx, uint32_t count, const rc_ciphertext* lhs, const rc_ciphertext* rhs,
                               const rc_ksk* const* keys, rc_ciphertext* out, void* stream);
int rc_relinearize_batch(rc_context* ctx, uint32_t count, const rc_ciphertext* quadratic, const rc_ksk* const* keys,
                         rc_ciphertext* out, void* stream);
int rc_rotate_batch(rc_context* ctx, uint32_t count, const rc_ciphertext* ct, const rc_ksk* const* keys,
                    rc_ciphertext* out, void* stream);
/* rotate (context/rotation.rs:104-127) of each of `count` same-level ciphertexts by each of `nrot` rotation
 * keys, out[i * nrot + r] = rotate(ct[i], keys[r]), with one decomposition of each c1 shared by its rotations
 * ("hoisted"; the baby steps of linear_transform.rs:213-232 rotate one input by 1..b-1).  Results equal
 * rc_rotate's residue for residue: an input whose decomposition holds a digit at -2^29 (where the digits of a
 * negated coefficient are not the negated digits) is rotated the ordinary way.  Mixed levels or key shapes
 * run as rc_rotate_batch.  Reading those flags synchronises the stream once per 32 inputs, so the call is not
 * capturable in a CUDA graph (neither is rc_bsgs_apply_batch, which uses it for its baby steps). */
int rc_rotate_hoisted(rc_context* ctx, uint32_t count, const rc_ciphertext* ct, uint32_t nrot,
                      const rc_ksk* const* keys, rc_ciphertext* out, void* stream);
/* relinearize then rescale (context/ops.rs:111-122 followed by context/ops.rs:32-37) for `count`
 * quadratic ciphertexts of any mix of levels; the rescale is fused into the keyswitch's last pass.  out[i]
 * gets level - 1 and the rescaled scale.  A batch of several levels whose keys all take the wide key product
 * runs as one launch per pass (decompose, digit transforms, key product, inverse transforms, finalize) over
 * all its levels, in chunks of up to 128 jobs (tunable "ml_jobs"); other batches run level by level.  Both
 * rc_relinearize_batch and this call do so.  After rc_reserve(ctx, top level, batch size, stream) the call
 * allocates nothing and can be captured in a CUDA graph. */
int rc_relinearize_rescale_batch(rc_context* ctx, uint32_t count, const rc_ciphertext* quadratic,
                                 const rc_ksk* const* keys, rc_ciphertext* out, void* stream);

/* ---- the crate's src/algorithms routines as whole schedules over a batch (one call, no per-step host
 * glue; the crate's schedules, scale/level rules and messages, so residues equal the crate's) ----
 * rc_total_sum_batch: total_sum.rs:45-60 for `count` ciphertexts; step_keys[t] is the rotation key of fold
 *   step 2^t (t < key_count), out[i] receives the result (level and scale of the input).
 * rc_halevi_shoup_batch: halevi_shoup.rs:46-71; plain = [count][plain_len] real slot values (zero-padded to
 *   N/2 and encoded at each ciphertext's level and scale on the GPU), mult_plain_slots_real then the fold
 *   over next_power_of_two(plain_len); out[i] is one level down.
 * rc_paterson_stockmeyer_batch: paterson_stockmeyer.rs:28-108 (helpers 146-349) of one polynomial
 *   (coefficients[terms], lowest degree first) on ciphertexts sharing level and scale; relin_keys[l] is the
 *   relinearization key at level l (null where absent, key_levels entries). */
int rc_total_sum_batch(rc_context* ctx, uint32_t count, const rc_ciphertext* cts, uint32_t active_slots,
                       const rc_ksk* const* step_keys, uint32_t key_count, rc_ciphertext* out, void* stream);
int rc_halevi_shoup_batch(rc_context* ctx, uint32_t count, const rc_ciphertext* cts, const double* plain,
                          uint32_t plain_len, const rc_ksk* const* step_keys, uint32_t key_count, rc_ciphertext* out,
                          void* stream);
int rc_paterson_stockmeyer_batch(rc_context* ctx, uint32_t count, const rc_ciphertext* cts,
                                 const double* coefficients, uint32_t terms, const rc_ksk* const* relin_keys,
                                 uint32_t key_levels, rc_ciphertext* out, void* stream);
/* apply_diagonal_linear_transform (src/ckks/bootstrapping/linear_transform.rs:109-150, 213-252) for `count`
 * ciphertexts at (diag_level, diag_scale_bits) sharing one set of packed BSGS diagonals: diag_ntt[g *
 * baby_step + j] is diagonal g*b+j pre-rotated by the giant shift g*b, encoded at the ciphertexts' level and
 * scale and in the NTT domain (rc_ntt_forward), null past the dimension; baby_keys[s-1] rotates by s
 * (s < min(baby_step, dimension)), giant_keys[g-1] by g*baby_step.  out[i] is one level down. */
int rc_bsgs_apply_batch(rc_context* ctx, uint32_t count, const rc_ciphertext* cts, uint32_t dimension,
                        uint32_t baby_step, const uint64_t* const* diag_ntt, uint32_t giants, int32_t diag_level,
                        int32_t diag_scale_bits, const rc_ksk* const* baby_keys, const rc_ksk* const* giant_keys,
                        rc_ciphertext* out, void* stream);

/* ---- CUDA graphs of library calls (no reference counterpart: the crate is CPU-only).  Capture every
 * call made on `stream` between begin and end (thread-local capture mode) into an executable graph;
 * rc_reserve the scratch first (capture refuses to grow it).  Pointers and sizes are baked in: replay
 * with rc_graph_launch on the same buffers. ---- */
int rc_graph_begin(rc_context* ctx, void* stream);
int rc_graph_end(rc_context* ctx, void* stream, rc_graph** out);
int rc_graph_launch(rc_graph* graph, void* stream);
void rc_graph_destroy(rc_graph* graph);

/* ---- host-buffer entry points (what a CPU-side caller such as the Rust crate
 * binds): host [2][level+1][N] inputs, host [2][level][N] output, copies
 * included.  scale bookkeeping as in mult_relinearized. ---- */
int rc_mult_relinearized_host(rc_context* ctx, const uint64_t* lhs, const uint64_t* rhs, int32_t level,
                              int32_t scale_bits, const rc_ksk* key, uint64_t* out, int32_t* out_scale_bits,
                              void* stream);
int rc_mult_relinearized_batch_host(rc_context* ctx, uint32_t count, const uint64_t* const* lhs,
                                    const uint64_t* const* rhs, const int32_t* levels, const int32_t* scale_bits,
                                    const rc_ksk* const* keys, uint64_t* const* out, int32_t* out_scale_bits,
                                    void* stream);
/* The same batch without waiting for it (context/ops.rs:124-133 per job, as above): returns once the copies
 * and kernels are enqueued, so a caller streaming batches overlaps one batch's copies with the previous one's
 * arithmetic.  out_scale_bits is filled before the call returns; the residues reach `out` later: after
 * rc_host_join(ctx, stream) and a synchronisation of `stream` (e.g. cudaStreamSynchronize) every earlier
 * asynchronous batch of that stream has its results in `out`, and only then may the caller change or free
 * the `lhs`/`rhs` host buffers or read `out`.  Host buffers should be pinned (page-locked) memory. */
int rc_mult_relinearized_batch_host_async(rc_context* ctx, uint32_t count, const uint64_t* const* lhs,
                                          const uint64_t* const* rhs, const int32_t* levels,
                                          const int32_t* scale_bits, const rc_ksk* const* keys,
                                          uint64_t* const* out, int32_t* out_scale_bits, void* stream);
/* Orders later work on `stream` after every asynchronous host-buffer batch issued on it (no host wait). */
int rc_host_join(rc_context* ctx, void* stream);

/* ---- host FP64 helpers (src/rns/encoding.rs, src/math/canonical_embedding.rs) ---- */
/* encode_integer_coeffs + poly_from_bigint_coeffs: encoding.rs:9-31,
 * polynomial.rs:78-85.  slots: N/2 complex values as interleaved (re, im). */
int rc_encode(const rc_context* ctx, const double* slots, int32_t level, uint32_t scale_bits, uint64_t* out_host);
/* reconstruct_coefficients + decode_integer_coeffs: polynomial.rs:162-201, encoding.rs:33-66 */
int rc_decode(const rc_context* ctx, const uint64_t* poly_host, int32_t level, uint32_t scale_bits,
              double* slots_out);
/* The same encode and decode on the GPU, bit for bit (same FFT twiddles and order, every product and sum
 * rounded separately, same rounding and CRT): `count` plaintexts per call, device buffers.  Encode: slots
 * [count][N/2] complex as interleaved (re, im) doubles -> out [count][level+1][N] residues.  Decode: polys
 * [count][level+1][N] -> slots [count][N/2] interleaved (count <= 65535). */
int rc_encode_device(rc_context* ctx, const double* slots, uint32_t count, int32_t level, uint32_t scale_bits,
                     uint64_t* out, void* stream);
int rc_decode_device(rc_context* ctx, const uint64_t* polys, uint32_t count, int32_t level, uint32_t scale_bits,
                     double* slots_out, void* stream);
/* The two slot/coefficient maps the exact bootstrapping transforms are built from, in FP64 with the
 * reference's operation order; they need no context (n = ring degree).
 * dense_slots_to_real_coeffs (src/ckks/bootstrapping/exact_transforms.rs:180-200): n/2 complex slots
 * (interleaved) -> n real coefficients.
 * dense_complex_coeffs_to_slots (exact_transforms.rs:210-229): n complex coefficients (interleaved) -> n/2
 * complex slots (interleaved). */
int rc_slots_to_real_coeffs(uint64_t n, const double* slots, double* coeffs_out);
int rc_complex_coeffs_to_slots(uint64_t n, const double* coeffs, double* slots_out);

/* ---- instrumentation (no reference counterpart: the reference only has
 * std::time::Instant around whole ops, examples/operations/timings.rs:282-308) ----
 * rc_profile_enable(flags), flags a combination of:
 *   RC_PROFILE_EVENTS: every kernel launch is bracketed by CUDA events on its stream (not for launches
 *     recorded into a CUDA graph); rc_profile_report synchronizes the device and writes a JSON object
 *     {"kernel": {"launches": n, "ms": total}, ...} into buf, then resets;
 *   RC_PROFILE_NVTX: NVTX ranges on the calling host thread, one per public entry point (named after it,
 *     e.g. "rc_mult_relinearized_batch") and one per kernel launch inside it (the names the event report
 *     uses), for a timeline tool; no cost when no tool is attached.
 * 0 turns both off (the default). */
#define RC_PROFILE_EVENTS 1
#define RC_PROFILE_NVTX 2
int rc_profile_enable(int flags);
int rc_profile_report(char* buf, size_t len);

#ifdef __cplusplus
}
#endif
#endif /* RNSCKKS_GPU_H */
