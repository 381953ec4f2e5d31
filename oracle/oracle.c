/*
 * CPU ORACLE — test infrastructure only.
 *
 * A plain-C restatement of the reference crate's (Akram275/rns-ckks-rust) CPU
 * arithmetic for the ciphertext hot path.  It is the checker for the CUDA path
 * and the timed CPU baseline; nothing in the product links or calls it.  Every
 * function names the reference file:line it follows and keeps the reference's
 * algorithm: radix-2 cyclic NTT with recurrence twiddles and u128 `%` modular
 * multiplication, twist/untwist around every polynomial product, Garner mixed
 * radix + base-2^30 multi-precision digits for the keyswitch gadget, exact
 * centred basis conversion for ModUp/ModDown, exact centred rescale.
 *
 * Parallelism mirrors the reference's rayon splits (limbs, coefficients,
 * keyswitch digits) with a pthread pool; the arithmetic is identical whatever
 * the thread count.
 *
 * Layout: an RNS polynomial with L limbs of degree N is uint64_t[L][N]
 * (limb-major, one contiguous Vec<u64> per limb as in
 * src/rns/polynomial.rs:9-11 / src/poly/mod.rs:7-10).
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

typedef uint64_t u64;
typedef int64_t i64;
typedef unsigned __int128 u128;
typedef __int128 i128;

/* ------------------------------------------------------------------------- */
/* thread pool: a dynamic-chunk parallel-for (stands in for rayon par_iter)   */
/* ------------------------------------------------------------------------- */
static int g_threads = 0;

void orc_set_threads(int n) { g_threads = n; }
int orc_get_threads(void) {
    if (g_threads <= 0) {
        long c = sysconf(_SC_NPROCESSORS_ONLN);
        g_threads = c > 0 ? (int)c : 1;
    }
    return g_threads;
}

typedef void (*pf_fn)(size_t index, void* arg);
typedef struct {
    size_t n;
    size_t next;
    pthread_mutex_t mu;
    pf_fn fn;
    void* arg;
} pf_state;

static void* pf_worker(void* p) {
    pf_state* s = (pf_state*)p;
    for (;;) {
        pthread_mutex_lock(&s->mu);
        size_t i = s->next++;
        pthread_mutex_unlock(&s->mu);
        if (i >= s->n) break;
        s->fn(i, s->arg);
    }
    return NULL;
}

static void parallel_for(size_t n, pf_fn fn, void* arg) {
    int t = orc_get_threads();
    if (t <= 1 || n <= 1) {
        for (size_t i = 0; i < n; ++i) fn(i, arg);
        return;
    }
    if ((size_t)t > n) t = (int)n;
    pf_state s;
    s.n = n;
    s.next = 0;
    s.fn = fn;
    s.arg = arg;
    pthread_mutex_init(&s.mu, NULL);
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)t);
    char* ok = (char*)calloc((size_t)t, 1);
    for (int k = 1; k < t; ++k) ok[k] = pthread_create(&th[k], NULL, pf_worker, &s) == 0;
    pf_worker(&s);
    for (int k = 1; k < t; ++k)
        if (ok[k]) pthread_join(th[k], NULL);
    free(ok);
    pthread_mutex_destroy(&s.mu);
    free(th);
}

/* ------------------------------------------------------------------------- */
/* src/math/ntt.rs                                                           */
/* ------------------------------------------------------------------------- */
typedef struct {
    u64 modulus;
    u64 size;
    u64 root;
    u64 root_inv;
    u64 negacyclic_twiddle;
    u64 negacyclic_twiddle_inv;
    u64 size_inv;
} orc_plan;

/* ntt.rs:149-151 */
static inline u64 mod_mul(u64 a, u64 b, u64 m) { return (u64)(((u128)a * (u128)b) % (u128)m); }
/* ntt.rs:132-139 */
static inline u64 mod_add(u64 a, u64 b, u64 m) {
    u128 s = (u128)a + (u128)b;
    return s >= (u128)m ? (u64)(s - m) : (u64)s;
}
/* ntt.rs:141-147 */
static inline u64 mod_sub(u64 a, u64 b, u64 m) { return a >= b ? a - b : m - (b - a); }
/* ntt.rs:153-163 */
static u64 mod_pow(u64 base, u64 exp, u64 m) {
    u64 r = 1;
    while (exp > 0) {
        if (exp & 1) r = mod_mul(r, base, m);
        base = mod_mul(base, base, m);
        exp >>= 1;
    }
    return r;
}
/* ntt.rs:165-188 and basis.rs:114-137 (identical extended Euclid); returns 0 when not invertible */
static int mod_inv(u64 value, u64 m, u64* out) {
    if (value == 0) return 0;
    i128 t = 0, nt = 1, r = (i128)m, nr = (i128)value;
    while (nr != 0) {
        i128 q = r / nr, tmp;
        tmp = t - q * nt; t = nt; nt = tmp;
        tmp = r - q * nr; r = nr; nr = tmp;
    }
    if (r != 1) return 0;
    if (t < 0) t += (i128)m;
    *out = (u64)(t % (i128)m);
    return 1;
}

/* NttPlan::new, ntt.rs:17-60.  Returns 0 on success, otherwise the index of the
 * failed check in source order (1: size, 2: modulus, 3: size|q-1, 4: 2size|q-1,
 * 5: root order, 6: root primitive, 7: root inverse, 8: size inverse,
 * 9: negacyclic twiddle, 10: twiddle inverse). */
int orc_ntt_plan_new(u64 size, u64 modulus, u64 primitive_root, orc_plan* out) {
    if (size == 0 || (size & (size - 1))) return 1;
    if (modulus < 3) return 2;
    if ((modulus - 1) % size != 0) return 3;
    if ((modulus - 1) % (2 * size) != 0) return 4;
    u64 exponent = (modulus - 1) / size;
    u64 root = mod_pow(primitive_root % modulus, exponent, modulus);
    if (mod_pow(root, size, modulus) != 1) return 5;
    if (size > 1 && mod_pow(root, size / 2, modulus) == 1) return 6;
    u64 root_inv, size_inv, tw_inv;
    if (!mod_inv(root, modulus, &root_inv)) return 7;
    if (!mod_inv(size % modulus, modulus, &size_inv)) return 8;
    u64 tw = mod_pow(primitive_root % modulus, (modulus - 1) / (2 * size), modulus);
    if (mod_pow(tw, 2 * size, modulus) != 1 || mod_pow(tw, size, modulus) != modulus - 1) return 9;
    if (!mod_inv(tw, modulus, &tw_inv)) return 10;
    out->modulus = modulus;
    out->size = size;
    out->root = root;
    out->root_inv = root_inv;
    out->negacyclic_twiddle = tw;
    out->negacyclic_twiddle_inv = tw_inv;
    out->size_inv = size_inv;
    return 0;
}

/* bit_reverse_permute, ntt.rs:116-130 */
static void bit_reverse_permute(u64* v, size_t n) {
    size_t j = 0;
    for (size_t i = 1; i < n; ++i) {
        size_t bit = n >> 1;
        while (j & bit) {
            j ^= bit;
            bit >>= 1;
        }
        j ^= bit;
        if (i < j) {
            u64 t = v[i];
            v[i] = v[j];
            v[j] = t;
        }
    }
}

/* ntt_in_place, ntt.rs:92-114: bit reversal then iterative DIT, twiddle by recurrence */
static void ntt_in_place(u64* v, size_t n, u64 m, u64 root) {
    bit_reverse_permute(v, n);
    for (size_t len = 2; len <= n; len <<= 1) {
        size_t step = n / len;
        u64 w_len = mod_pow(root, (u64)step, m);
        for (size_t c = 0; c < n; c += len) {
            u64 w = 1;
            for (size_t i = 0; i < len / 2; ++i) {
                u64 u = v[c + i];
                u64 x = mod_mul(v[c + i + len / 2], w, m);
                v[c + i] = mod_add(u, x, m);
                v[c + i + len / 2] = mod_sub(u, x, m);
                w = mod_mul(w, w_len, m);
            }
        }
    }
}

/* NttPlan::forward / inverse, ntt.rs:78-89 */
void orc_ntt_forward(const orc_plan* p, u64* v) { ntt_in_place(v, p->size, p->modulus, p->root); }
void orc_ntt_inverse(const orc_plan* p, u64* v) {
    ntt_in_place(v, p->size, p->modulus, p->root_inv);
    for (size_t i = 0; i < p->size; ++i) v[i] = mod_mul(v[i], p->size_inv, p->modulus);
}

/* ------------------------------------------------------------------------- */
/* src/poly/mod.rs                                                           */
/* ------------------------------------------------------------------------- */
/* ModularPolynomial::add / sub, poly/mod.rs:37-59 (add_mod/sub_mod 177-192) */
void orc_poly_add(const u64* a, const u64* b, u64* out, size_t n, u64 m) {
    for (size_t i = 0; i < n; ++i) out[i] = mod_add(a[i], b[i], m);
}
void orc_poly_sub(const u64* a, const u64* b, u64* out, size_t n, u64 m) {
    for (size_t i = 0; i < n; ++i) out[i] = mod_sub(a[i], b[i], m);
}

/* multiply_naive, poly/mod.rs:62-107 (schoolbook, x^n = -1) */
void orc_poly_mul_naive(const u64* a, const u64* b, u64* out, size_t n, u64 m) {
    u64* r = (u64*)calloc(n, sizeof(u64));
    for (size_t i = 0; i < n; ++i) {
        if (a[i] == 0) continue;
        for (size_t j = 0; j < n; ++j) {
            if (b[j] == 0) continue;
            u64 prod = mod_mul(a[i], b[j], m);
            size_t k = i + j;
            if (k < n) r[k] = mod_add(r[k], prod, m);
            else r[k - n] = mod_sub(r[k - n], prod, m);
        }
    }
    memcpy(out, r, n * sizeof(u64));
    free(r);
}

/* apply_galois_automorphism, poly/mod.rs:110-131 */
void orc_poly_automorphism(const u64* a, u64* out, size_t n, u64 m, u64 g) {
    u64* r = (u64*)calloc(n, sizeof(u64));
    size_t two_n = 2 * n;
    for (size_t i = 0; i < n; ++i) {
        if (a[i] == 0) continue;
        size_t mapped = (size_t)(((u128)i * g) % two_n);
        if (mapped < n) r[mapped] = mod_add(r[mapped], a[i], m);
        else r[mapped - n] = mod_sub(r[mapped - n], a[i], m);
    }
    memcpy(out, r, n * sizeof(u64));
    free(r);
}

/* twist_in_place, poly/mod.rs:169-175 */
static void twist_in_place(u64* c, size_t n, u64 tw, u64 m) {
    u64 power = 1;
    for (size_t i = 0; i < n; ++i) {
        c[i] = mod_mul(c[i], power, m);
        power = mod_mul(power, tw, m);
    }
}

/* multiply_ntt, poly/mod.rs:134-161: twist both, forward both, pointwise,
 * inverse, untwist.  `out` may alias `a` or `b`. */
void orc_poly_mul_ntt(const orc_plan* p, const u64* a, const u64* b, u64* out) {
    size_t n = p->size;
    u64 m = p->modulus;
    u64* lhs = (u64*)malloc(n * sizeof(u64));
    u64* rhs = (u64*)malloc(n * sizeof(u64));
    memcpy(lhs, a, n * sizeof(u64));
    memcpy(rhs, b, n * sizeof(u64));
    twist_in_place(lhs, n, p->negacyclic_twiddle, m);
    twist_in_place(rhs, n, p->negacyclic_twiddle, m);
    orc_ntt_forward(p, lhs);
    orc_ntt_forward(p, rhs);
    for (size_t i = 0; i < n; ++i) lhs[i] = mod_mul(lhs[i], rhs[i], m);
    orc_ntt_inverse(p, lhs);
    twist_in_place(lhs, n, p->negacyclic_twiddle_inv, m);
    memcpy(out, lhs, n * sizeof(u64));
    free(lhs);
    free(rhs);
}

/* ------------------------------------------------------------------------- */
/* src/rns/polynomial.rs: limb-parallel wrappers (rayon over limbs)          */
/* ------------------------------------------------------------------------- */
typedef struct {
    const orc_plan* plans;
    const u64* a;
    const u64* b;
    u64* out;
    u64 g;
} limb_job;

static void job_mul_ntt(size_t l, void* arg) {
    limb_job* j = (limb_job*)arg;
    size_t n = j->plans[0].size;
    orc_poly_mul_ntt(&j->plans[l], j->a + l * n, j->b + l * n, j->out + l * n);
}
static void job_add(size_t l, void* arg) {
    limb_job* j = (limb_job*)arg;
    size_t n = j->plans[0].size;
    orc_poly_add(j->a + l * n, j->b + l * n, j->out + l * n, n, j->plans[l].modulus);
}
static void job_sub(size_t l, void* arg) {
    limb_job* j = (limb_job*)arg;
    size_t n = j->plans[0].size;
    orc_poly_sub(j->a + l * n, j->b + l * n, j->out + l * n, n, j->plans[l].modulus);
}
static void job_aut(size_t l, void* arg) {
    limb_job* j = (limb_job*)arg;
    size_t n = j->plans[0].size;
    orc_poly_automorphism(j->a + l * n, j->out + l * n, n, j->plans[l].modulus, j->g);
}

/* RnsPolynomial::multiply_ntt, polynomial.rs:121-136 */
void orc_rns_mul_ntt(const orc_plan* plans, size_t limbs, const u64* a, const u64* b, u64* out) {
    limb_job j = {plans, a, b, out, 0};
    parallel_for(limbs, job_mul_ntt, &j);
}
/* RnsPolynomial::add / sub, polynomial.rs:99-119 */
void orc_rns_add(const orc_plan* plans, size_t limbs, const u64* a, const u64* b, u64* out) {
    limb_job j = {plans, a, b, out, 0};
    parallel_for(limbs, job_add, &j);
}
void orc_rns_sub(const orc_plan* plans, size_t limbs, const u64* a, const u64* b, u64* out) {
    limb_job j = {plans, a, b, out, 0};
    parallel_for(limbs, job_sub, &j);
}
/* RnsPolynomial::apply_galois_automorphism, polynomial.rs:138-145 */
void orc_rns_automorphism(const orc_plan* plans, size_t limbs, const u64* a, u64* out, u64 g) {
    limb_job j = {plans, a, NULL, out, g};
    parallel_for(limbs, job_aut, &j);
}

/* ------------------------------------------------------------------------- */
/* src/rns/ops.rs: tensor, rescale                                           */
/* ------------------------------------------------------------------------- */
/* multiply_ciphertexts_rns, ops.rs:84-100: (a0b0, a0b1 + a1b0, a1b1) */
void orc_tensor(const orc_plan* plans, size_t limbs, const u64* a0, const u64* a1, const u64* b0,
                const u64* b1, u64* c0, u64* c1, u64* c2) {
    size_t n = plans[0].size;
    u64* t = (u64*)malloc(limbs * n * sizeof(u64));
    orc_rns_mul_ntt(plans, limbs, a0, b0, c0);
    orc_rns_mul_ntt(plans, limbs, a0, b1, c1);
    orc_rns_mul_ntt(plans, limbs, a1, b0, t);
    orc_rns_add(plans, limbs, c1, t, c1);
    orc_rns_mul_ntt(plans, limbs, a1, b1, c2);
    free(t);
}

/* centered_residue_mod_prime, ops.rs:175-186 */
static inline u64 centered_residue_mod_prime(u64 value, u64 modulus, u64 half, u64 target) {
    if (value <= half) return value % target;
    u64 distance = (modulus - value) % target;
    return distance == 0 ? 0 : target - distance;
}

typedef struct {
    const orc_plan* plans;
    const u64* in;
    u64* out;
    size_t limbs_in;
} rescale_job;

static void job_rescale(size_t l, void* arg) {
    rescale_job* r = (rescale_job*)arg;
    size_t n = r->plans[0].size;
    u64 dropped = r->plans[r->limbs_in - 1].modulus;
    u64 half = dropped >> 1;
    const u64* dc = r->in + (r->limbs_in - 1) * n;
    u64 qi = r->plans[l].modulus;
    u64 inv = 0;
    mod_inv(dropped % qi, qi, &inv);
    const u64* c = r->in + l * n;
    u64* o = r->out + l * n;
    for (size_t i = 0; i < n; ++i) {
        u64 cd = centered_residue_mod_prime(dc[i], dropped, half, qi);
        u64 num = mod_sub(c[i], cd, qi); /* ops.rs:188-193 sub_mod_u64 (no pre-reduction) */
        o[i] = (u64)(((u128)num * inv) % qi);
    }
}

/* rescale_poly_rns, ops.rs:135-173: limbs_in -> limbs_in-1 limbs (rayon over limbs) */
void orc_rescale_poly(const orc_plan* plans, size_t limbs_in, const u64* in, u64* out) {
    rescale_job r = {plans, in, out, limbs_in};
    parallel_for(limbs_in - 1, job_rescale, &r);
}

/* ------------------------------------------------------------------------- */
/* src/rns/keyswitching.rs: base-2^30 gadget, basis conversion               */
/* ------------------------------------------------------------------------- */
#define MAXD 512 /* base digits of a modulus product: 64 limbs * 62 bits / 30 < 140 */

typedef struct {
    size_t count;
    const u64* moduli;
    u64* inverses; /* [count][count], inverses[i*count+j] = moduli[j]^-1 mod moduli[i], j < i */
    u64 modulus_digits[MAXD];
    size_t modulus_len;
    u64 half_digits[MAXD];
    size_t half_len;
    u64 base;
} bc_precomp;

/* mul_add_small_base, keyswitching.rs:469-480 */
static void mul_add_small_base(u64* d, size_t* len, u64 mul, u64 add, u64 base) {
    u128 carry = add;
    for (size_t i = 0; i < *len; ++i) {
        u128 v = (u128)d[i] * mul + carry;
        d[i] = (u64)(v % base);
        carry = v / base;
    }
    while (carry > 0) {
        d[(*len)++] = (u64)(carry % base);
        carry /= base;
    }
}
/* div2_base_digits, keyswitching.rs:482-489 */
static void div2_base_digits(u64* d, size_t len, u64 base) {
    u64 carry = 0;
    for (size_t k = len; k-- > 0;) {
        u128 v = (u128)carry * base + d[k];
        d[k] = (u64)(v / 2);
        carry = (u64)(v % 2);
    }
}
/* trim_base_digits, keyswitching.rs:491-495 */
static void trim_base_digits(u64* d, size_t* len) {
    while (*len > 1 && d[*len - 1] == 0) (*len)--;
}
/* cmp_base_digits, keyswitching.rs:497-509 */
static int cmp_base_digits(const u64* a, size_t la, const u64* b, size_t lb) {
    size_t ra = la, rb = lb;
    while (ra > 0 && a[ra - 1] == 0) ra--;
    while (rb > 0 && b[rb - 1] == 0) rb--;
    if (ra != rb) return ra < rb ? -1 : 1;
    for (size_t k = ra; k-- > 0;)
        if (a[k] != b[k]) return a[k] < b[k] ? -1 : 1;
    return 0;
}
/* sub_base_digits, keyswitching.rs:511-529 */
static void sub_base_digits(const u64* a, size_t la, const u64* b, size_t lb, u64 base, u64* out,
                            size_t* lo) {
    i128 borrow = 0;
    for (size_t k = 0; k < la; ++k) {
        i128 v = (i128)a[k] - (i128)(k < lb ? b[k] : 0) - borrow;
        if (v < 0) {
            v += (i128)base;
            borrow = 1;
        } else {
            borrow = 0;
        }
        out[k] = (u64)v;
    }
    *lo = la;
    trim_base_digits(out, lo);
}
/* keyswitching.rs:549-557 sub_mod_u64 (reduces both operands first) */
static inline u64 sub_mod_u64(u64 a, u64 b, u64 m) {
    a %= m;
    b %= m;
    return a >= b ? a - b : m - (b - a);
}
/* keyswitching.rs:540-547 */
static inline u64 add_mod_u64(u64 a, u64 b, u64 m) { return mod_add(a, b, m); }
/* keyswitching.rs:559-561 */
static inline u64 mul_mod_u64(u64 a, u64 b, u64 m) { return mod_mul(a, b, m); }

/* BasisConversionPrecomp::new, keyswitching.rs:333-363 */
static void bc_init(bc_precomp* p, const u64* moduli, size_t count, u64 base) {
    p->count = count;
    p->moduli = moduli;
    p->base = base;
    p->inverses = (u64*)calloc(count * count + 1, sizeof(u64));
    for (size_t i = 0; i < count; ++i)
        for (size_t j = 0; j < i; ++j) mod_inv(moduli[j] % moduli[i], moduli[i], &p->inverses[i * count + j]);
    p->modulus_digits[0] = 1;
    p->modulus_len = 1;
    for (size_t i = 0; i < count; ++i) mul_add_small_base(p->modulus_digits, &p->modulus_len, moduli[i], 0, base);
    trim_base_digits(p->modulus_digits, &p->modulus_len);
    memcpy(p->half_digits, p->modulus_digits, sizeof(u64) * p->modulus_len);
    p->half_len = p->modulus_len;
    div2_base_digits(p->half_digits, p->half_len, base);
    trim_base_digits(p->half_digits, &p->half_len);
}
static void bc_free(bc_precomp* p) { free(p->inverses); }

/* mixed_radix_digits, keyswitching.rs:397-410 (Garner) */
static void mixed_radix_digits(const u64* residues, const bc_precomp* p, u64* digits) {
    size_t c = p->count;
    for (size_t i = 0; i < c; ++i) digits[i] = residues[i];
    for (size_t i = 1; i < c; ++i) {
        u64 m = p->moduli[i];
        u64 v = digits[i];
        for (size_t j = 0; j < i; ++j) {
            v = sub_mod_u64(v, digits[j] % m, m);
            v = mul_mod_u64(v, p->inverses[i * c + j], m);
        }
        digits[i] = v;
    }
}
/* evaluate_mixed_radix_mod, keyswitching.rs:412-423 */
static u64 evaluate_mixed_radix_mod(const u64* mixed, const u64* moduli, size_t c, u64 t) {
    if (c == 0) return 0;
    u64 acc = mixed[c - 1] % t;
    for (size_t k = c - 1; k-- > 0;) {
        acc = (u64)(((u128)acc * (moduli[k] % t)) % t);
        acc = add_mod_u64(acc, mixed[k] % t, t);
    }
    return acc;
}
/* canonical_digits_from_mixed_radix, keyswitching.rs:425-432 */
static void canonical_digits(const u64* mixed, const u64* moduli, size_t c, u64 base, u64* d, size_t* len) {
    d[0] = 0;
    *len = 1;
    for (size_t k = c; k-- > 0;) mul_add_small_base(d, len, moduli[k], mixed[k], base);
    trim_base_digits(d, len);
}
/* base_digits_mod_modulus, keyswitching.rs:531-538 */
static u64 base_digits_mod_modulus(const u64* d, size_t len, u64 base, u64 m) {
    u64 acc = 0;
    for (size_t k = len; k-- > 0;) {
        acc = (u64)(((u128)acc * (base % m)) % m);
        acc = add_mod_u64(acc, d[k] % m, m);
    }
    return acc;
}
/* convert_centered_residues_to_target, keyswitching.rs:365-379 */
static u64 convert_centered(const u64* residues, const bc_precomp* p, u64 target) {
    u64 mixed[256];
    u64 canon[MAXD];
    size_t clen;
    mixed_radix_digits(residues, p, mixed);
    canonical_digits(mixed, p->moduli, p->count, p->base, canon, &clen);
    u64 cm = evaluate_mixed_radix_mod(mixed, p->moduli, p->count, target);
    if (cmp_base_digits(canon, clen, p->half_digits, p->half_len) > 0) {
        u64 mm = base_digits_mod_modulus(p->modulus_digits, p->modulus_len, p->base, target);
        return sub_mod_u64(cm, mm, target);
    }
    return cm;
}
/* normalize_balanced_digits, keyswitching.rs:434-454 (release build: final carry dropped) */
static void normalize_balanced(i64* digits, size_t have, size_t levels, i64 base, i64* out) {
    i64 half = base >> 1;
    i64 carry = 0;
    for (size_t k = 0; k < levels; ++k) {
        i64 value = (k < have ? digits[k] : 0) + carry;
        i64 d = value % base; /* Rust `%` on i64 truncates toward zero like C */
        if (d >= half) d -= base;
        else if (d < -half) d += base;
        carry = (value - d) / base;
        out[k] = d;
    }
}
/* decompose_residues_balanced, keyswitching.rs:381-395 */
static void decompose_residues_balanced(const u64* residues, const bc_precomp* p, size_t levels, i64* out) {
    u64 mixed[256];
    u64 canon[MAXD];
    size_t clen;
    i64 signed_digits[MAXD];
    mixed_radix_digits(residues, p, mixed);
    canonical_digits(mixed, p->moduli, p->count, p->base, canon, &clen);
    size_t have;
    if (cmp_base_digits(canon, clen, p->half_digits, p->half_len) > 0) {
        u64 mag[MAXD];
        size_t mlen;
        sub_base_digits(p->modulus_digits, p->modulus_len, canon, clen, p->base, mag, &mlen);
        for (size_t k = 0; k < mlen; ++k) signed_digits[k] = -(i64)mag[k];
        have = mlen;
    } else {
        for (size_t k = 0; k < clen; ++k) signed_digits[k] = (i64)canon[k];
        have = clen;
    }
    /* digits.resize(levels + 1, 0): truncation beyond levels+1 never affects the
     * first `levels` outputs, which only read digits[0..levels). */
    normalize_balanced(signed_digits, have, levels, (i64)p->base, out);
}
/* signed_digit_mod_q, keyswitching.rs:456-467 */
static inline u64 signed_digit_mod_q(i64 d, u64 m) {
    if (d >= 0) return (u64)d % m;
    u64 mag = ((u64)(-d)) % m;
    return mag == 0 ? 0 : m - mag;
}

typedef struct {
    const orc_plan* plans;
    size_t limbs;
    const u64* poly;
    const bc_precomp* pc;
    size_t levels;
    i64* digits; /* [levels][n] */
} decomp_job;

static void job_decomp(size_t i, void* arg) {
    decomp_job* d = (decomp_job*)arg;
    size_t n = d->plans[0].size;
    u64 res[256];
    i64 out[MAXD];
    for (size_t l = 0; l < d->limbs; ++l) res[l] = d->poly[l * n + i];
    decompose_residues_balanced(res, d->pc, d->levels, out);
    for (size_t k = 0; k < d->levels; ++k) d->digits[k * n + i] = out[k];
}

/* decompose_poly_rns_with_levels, keyswitching.rs:196-236, split in two: the signed
 * digits per coefficient (rayon over coefficients), then signed_digit_mod_q into
 * every limb.  `digits_out` = i64[levels][n]; `residues_out` (optional) =
 * u64[levels][limbs][n]. */
void orc_decompose(const orc_plan* plans, size_t limbs, const u64* poly, size_t decomp_bits, size_t levels,
                   i64* digits_out, u64* residues_out) {
    size_t n = plans[0].size;
    u64 moduli[256];
    for (size_t l = 0; l < limbs; ++l) moduli[l] = plans[l].modulus;
    bc_precomp pc;
    bc_init(&pc, moduli, limbs, (u64)1 << decomp_bits);
    decomp_job d = {plans, limbs, poly, &pc, levels, digits_out};
    parallel_for(n, job_decomp, &d);
    bc_free(&pc);
    if (residues_out)
        for (size_t k = 0; k < levels; ++k)
            for (size_t l = 0; l < limbs; ++l)
                for (size_t i = 0; i < n; ++i)
                    residues_out[(k * limbs + l) * n + i] = signed_digit_mod_q(digits_out[k * n + i], moduli[l]);
}

typedef struct {
    const orc_plan* src;
    size_t ls;
    const orc_plan* tgt;
    size_t lt;
    const u64* poly;
    const bc_precomp* pc;
    u64* out; /* [ls + lt][n] */
} lift_job;

static void job_lift(size_t i, void* arg) {
    lift_job* j = (lift_job*)arg;
    size_t n = j->src[0].size;
    u64 res[256];
    for (size_t l = 0; l < j->ls; ++l) res[l] = j->poly[l * n + i];
    for (size_t t = 0; t < j->lt; ++t) j->out[(j->ls + t) * n + i] = convert_centered(res, j->pc, j->tgt[t].modulus);
}

/* lift_poly_to_context, keyswitching.rs:242-276: appends the centred conversion of
 * each coefficient to every target (aux) prime. */
void orc_lift(const orc_plan* src, size_t ls, const orc_plan* tgt, size_t lt, const u64* poly, u64* out) {
    size_t n = src[0].size;
    memmove(out, poly, ls * n * sizeof(u64));
    if (lt == 0) return;
    u64 moduli[256];
    for (size_t l = 0; l < ls; ++l) moduli[l] = src[l].modulus;
    bc_precomp pc;
    bc_init(&pc, moduli, ls, (u64)1 << 30);
    lift_job j = {src, ls, tgt, lt, out, &pc, out};
    parallel_for(n, job_lift, &j);
    bc_free(&pc);
}

typedef struct {
    const orc_plan* q;
    size_t lq;
    const orc_plan* p;
    size_t lp;
    const u64* poly;
    const bc_precomp* pc;
    u64* out;
    size_t prime_index;
    u64 p_inv;
} moddown_job;

static void job_moddown(size_t i, void* arg) {
    moddown_job* j = (moddown_job*)arg;
    size_t n = j->q[0].size;
    u64 aux[256];
    for (size_t k = 0; k < j->lp; ++k) aux[k] = j->poly[(j->lq + k) * n + i];
    u64 qi = j->q[j->prime_index].modulus;
    u64 c = convert_centered(aux, j->pc, qi);
    u64 num = sub_mod_u64(j->poly[j->prime_index * n + i], c, qi);
    j->out[j->prime_index * n + i] = (u64)(((u128)num * j->p_inv) % qi);
}

/* mod_down_eval_to_q, keyswitching.rs:278-322: for each q_i (sequential), rayon over
 * coefficients: (x_i - centred([x]_P) mod q_i) * P^-1 mod q_i. */
void orc_mod_down(const orc_plan* q, size_t lq, const orc_plan* p, size_t lp, const u64* poly, u64* out) {
    u64 moduli[256];
    for (size_t k = 0; k < lp; ++k) moduli[k] = p[k].modulus;
    bc_precomp pc;
    bc_init(&pc, moduli, lp, (u64)1 << 30);
    for (size_t i = 0; i < lq; ++i) {
        u64 qi = q[i].modulus;
        /* P mod q_i via the product of residues (equals the BigUint remainder) */
        u64 pm = 1;
        for (size_t k = 0; k < lp; ++k) pm = mod_mul(pm, moduli[k] % qi, qi);
        u64 pinv = 0;
        mod_inv(pm, qi, &pinv);
        moddown_job j = {q, lq, p, lp, poly, &pc, out, i, pinv};
        parallel_for(q[0].size, job_moddown, &j);
    }
    bc_free(&pc);
}

/* num_decomp_digits, keyswitching.rs:238-240 */
size_t orc_num_decomp_digits(size_t total_bits, size_t decomp_bits) { return (total_bits + decomp_bits - 1) / decomp_bits; }

/* bit length of the product of the moduli (BigUint::bits) */
size_t orc_modulus_bits(const u64* moduli, size_t count) {
    u64 d[MAXD];
    size_t len = 1;
    d[0] = 1;
    for (size_t i = 0; i < count; ++i) mul_add_small_base(d, &len, moduli[i], 0, (u64)1 << 30);
    trim_base_digits(d, &len);
    if (d[len - 1] == 0) return 0;
    return (len - 1) * 30 + (size_t)(64 - __builtin_clzll(d[len - 1]));
}

typedef struct {
    const orc_plan* plans; /* the multiplication basis (Q or Q u P) */
    size_t limbs;
    const u64* digit_res; /* [digits][limbs][n] */
    const u64* ksk;       /* [digits][2][limbs][n] */
    u64* contrib;         /* [digits][2][limbs][n] */
} ks_job;

static void job_ks(size_t t, void* arg) {
    ks_job* k = (ks_job*)arg;
    size_t n = k->plans[0].size;
    size_t L = k->limbs;
    size_t digit = t / (2 * L);
    size_t comp = (t / L) % 2;
    size_t l = t % L;
    orc_poly_mul_ntt(&k->plans[l], k->digit_res + (digit * L + l) * n, k->ksk + ((digit * 2 + comp) * L + l) * n,
                     k->contrib + ((digit * 2 + comp) * L + l) * n);
}

/* keyswitch_rns, keyswitching.rs:130-157 (Q-only) when lp == 0, otherwise
 * keyswitch_rns_hybrid, keyswitching.rs:159-194.  `decomp_levels` is the number of
 * gadget digits the reference decomposes into: ksk.ksk.len() for Q-only (138),
 * active digits for hybrid (167-170).  The key is [ksk_digits][2][lq+lp][n] in
 * coefficient form; the digit products run in parallel (rayon over digits and
 * limbs), then are summed serially. */
void orc_keyswitch(const orc_plan* q, size_t lq, const orc_plan* p, size_t lp, const u64* poly, const u64* ksk,
                   size_t decomp_levels, u64* out_c0, u64* out_c1) {
    size_t n = q[0].size;
    size_t L = lq + lp;
    orc_plan* all = (orc_plan*)malloc(sizeof(orc_plan) * L);
    memcpy(all, q, sizeof(orc_plan) * lq);
    if (lp) memcpy(all + lq, p, sizeof(orc_plan) * lp);
    i64* digits = (i64*)malloc(sizeof(i64) * decomp_levels * n);
    u64* qres = (u64*)malloc(sizeof(u64) * decomp_levels * lq * n);
    orc_decompose(q, lq, poly, 30, decomp_levels, digits, qres);
    u64* dres = qres;
    if (lp) {
        dres = (u64*)malloc(sizeof(u64) * decomp_levels * L * n);
        for (size_t d = 0; d < decomp_levels; ++d) orc_lift(q, lq, p, lp, qres + d * lq * n, dres + d * L * n);
    }
    u64* contrib = (u64*)malloc(sizeof(u64) * decomp_levels * 2 * L * n);
    ks_job kj = {all, L, dres, ksk, contrib};
    parallel_for(decomp_levels * 2 * L, job_ks, &kj);
    u64* acc0 = (u64*)calloc(L * n, sizeof(u64));
    u64* acc1 = (u64*)calloc(L * n, sizeof(u64));
    for (size_t d = 0; d < decomp_levels; ++d) {
        orc_rns_add(all, L, acc0, contrib + (d * 2 + 0) * L * n, acc0);
        orc_rns_add(all, L, acc1, contrib + (d * 2 + 1) * L * n, acc1);
    }
    if (lp) {
        orc_mod_down(q, lq, p, lp, acc0, out_c0);
        orc_mod_down(q, lq, p, lp, acc1, out_c1);
    } else {
        memcpy(out_c0, acc0, sizeof(u64) * lq * n);
        memcpy(out_c1, acc1, sizeof(u64) * lq * n);
    }
    free(acc0);
    free(acc1);
    free(contrib);
    if (dres != qres) free(dres);
    free(qres);
    free(digits);
    free(all);
}

/* RnsCkksContext::relinearize, context/ops.rs:111-122 followed by rescale
 * (context/ops.rs:32-37), i.e. the tail of mult_relinearized (124-133).
 * Input: quadratic ciphertext c0,c1,c2 at lq limbs; output: ct at lq-1 limbs. */
void orc_relinearize(const orc_plan* q, size_t lq, const orc_plan* p, size_t lp, const u64* c0, const u64* c1,
                     const u64* c2, const u64* ksk, size_t decomp_levels, u64* out0, u64* out1) {
    size_t n = q[0].size;
    u64* k0 = (u64*)malloc(sizeof(u64) * lq * n);
    u64* k1 = (u64*)malloc(sizeof(u64) * lq * n);
    orc_keyswitch(q, lq, p, lp, c2, ksk, decomp_levels, k0, k1);
    orc_rns_add(q, lq, c0, k0, out0);
    orc_rns_add(q, lq, c1, k1, out1);
    free(k0);
    free(k1);
}

/* RnsCkksContext::mult_relinearized, context/ops.rs:124-133: tensor, relinearize,
 * rescale.  a = (a0,a1), b = (b0,b1) at lq limbs -> out (lq-1 limbs each). */
void orc_mult_relinearized(const orc_plan* q, size_t lq, const orc_plan* p, size_t lp, const u64* a0, const u64* a1,
                           const u64* b0, const u64* b1, const u64* ksk, size_t decomp_levels, u64* out0, u64* out1) {
    size_t n = q[0].size;
    u64* c0 = (u64*)malloc(sizeof(u64) * lq * n);
    u64* c1 = (u64*)malloc(sizeof(u64) * lq * n);
    u64* c2 = (u64*)malloc(sizeof(u64) * lq * n);
    orc_tensor(q, lq, a0, a1, b0, b1, c0, c1, c2);
    orc_relinearize(q, lq, p, lp, c0, c1, c2, ksk, decomp_levels, c0, c1);
    orc_rescale_poly(q, lq, c0, out0);
    orc_rescale_poly(q, lq, c1, out1);
    free(c0);
    free(c1);
    free(c2);
}

/* RnsCkksContext::rotate, context/rotation.rs:104-127: automorphism on (c0, c1),
 * keyswitch of the rotated c1, result (c0' + ks.c0, ks.c1). */
void orc_rotate(const orc_plan* q, size_t lq, const orc_plan* p, size_t lp, const u64* c0, const u64* c1, u64 g,
                const u64* ksk, size_t decomp_levels, u64* out0, u64* out1) {
    size_t n = q[0].size;
    u64* r0 = (u64*)malloc(sizeof(u64) * lq * n);
    u64* r1 = (u64*)malloc(sizeof(u64) * lq * n);
    u64* k0 = (u64*)malloc(sizeof(u64) * lq * n);
    orc_rns_automorphism(q, lq, c0, r0, g);
    orc_rns_automorphism(q, lq, c1, r1, g);
    orc_keyswitch(q, lq, p, lp, r1, ksk, decomp_levels, k0, out1);
    orc_rns_add(q, lq, r0, k0, out0);
    free(r0);
    free(r1);
    free(k0);
}

/* out[i] = a[i] * f mod m (u128 %), the per-limb scalar products used when the
 * reference reduces (coefficient * B^i [* P]) into each RNS prime
 * (keyswitching.rs:64-68, 108-112). */
void orc_mul_scalar(const u64* a, u64* out, size_t n, u64 f, u64 m) {
    f %= m;
    for (size_t i = 0; i < n; ++i) out[i] = mod_mul(a[i] % m, f, m);
}
