// C ABI (include/rnsckks_gpu.h): context creation with all precomputed tables,
// device-resident keys, per-stream scratch and the per-op / batched entry
// points.  Preconditions that the reference asserts (and panics on) become
// RC_ERR_INVALID_ARGUMENT with the reference's message.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>

#include "context.hpp"

using namespace rc;

namespace rc {

static thread_local std::string g_err;

void set_last_error(const std::string& m) { g_err = m; }

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    if (e == cudaErrorMemoryAllocation) fail(RC_ERR_OUT_OF_MEMORY, std::string(what) + ": " + cudaGetErrorString(e));
    fail(RC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  }
}

DevBuf::DevBuf(size_t b) : bytes(b) {
  if (b) cuda_check(cudaMalloc(&p, b), "cudaMalloc");
}
DevBuf::~DevBuf() {
  if (p) cudaFree(p);
}
Workspace::~Workspace() {
  if (host_pinned) cudaFreeHost(host_pinned);
}

cudaEvent_t HostPipe::event() {
  if (next == events.size()) {
    cudaEvent_t e;
    cuda_check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
    events.push_back(e);
  }
  return events[next++];
}

HostPipe::~HostPipe() {
  for (cudaEvent_t e : events) cudaEventDestroy(e);
  for (int i = 0; i < 4; ++i) {
    if (consumed[i]) cudaEventDestroy(consumed[i]);
    if (drained[i]) cudaEventDestroy(drained[i]);
  }
  if (last) cudaEventDestroy(last);
  for (cudaStream_t st : {in, comp, out, comp2})
    if (st) cudaStreamDestroy(st);
}

}  // namespace rc

namespace {

typedef unsigned __int128 u128h;

const char* plan_error(uint64_t size, uint64_t q, uint64_t g) {
  // NttPlan::new checks, src/math/ntt.rs:17-60
  if (size == 0 || (size & (size - 1))) return "NTT size must be a non-zero power of two";
  if (q < 3) return "modulus must be an odd prime larger than 2";
  if ((q - 1) % size) return "size must divide modulus - 1";
  if ((q - 1) % (2 * size)) return "2 * size must divide modulus - 1 for negacyclic NTTs";
  uint64_t w = powmod_h(g % q, (q - 1) / size, q);
  if (powmod_h(w, size, q) != 1) return "primitive_root does not generate a size-th root of unity";
  if (size > 1 && powmod_h(w, size / 2, q) == 1) return "root is not primitive for the requested size";
  uint64_t psi = powmod_h(g % q, (q - 1) / (2 * size), q);
  if (powmod_h(psi, 2 * size, q) != 1 || powmod_h(psi, size, q) != q - 1)
    return "primitive_root does not generate a valid negacyclic twiddle";
  return nullptr;
}

void validate_chain(uint64_t n, const std::vector<uint64_t>& m, const std::vector<uint64_t>& g) {
  // RnsContext::new, src/rns/basis.rs:32-59
  require(n != 0 && !(n & (n - 1)), "poly_degree must be a non-zero power of two");
  require(!m.empty(), "RNS basis must contain at least one prime");
  for (size_t i = 0; i < m.size(); ++i) {
    for (size_t j = 0; j < i; ++j) require(m[j] != m[i], "duplicate RNS modulus " + std::to_string(m[i]));
    const char* e = plan_error(n, m[i], g[i]);
    if (e) fail(RC_ERR_INVALID_ARGUMENT, "invalid RNS prime " + std::to_string(m[i]) + ": " + e);
  }
}

int bitrev(int x, int bits) {
  int r = 0;
  for (int i = 0; i < bits; ++i) r |= ((x >> i) & 1) << (bits - 1 - i);
  return r;
}

cudaStream_t S(void* s) { return (cudaStream_t)s; }

Workspace& workspace(rc_context* ctx, cudaStream_t s) {
  std::lock_guard<std::mutex> lk(ctx->mu);
  auto& w = ctx->ws[s];
  if (!w) w.reset(new Workspace());
  return *w;
}

void* ws_device(rc_context* ctx, cudaStream_t s, size_t bytes) {
  Workspace& w = workspace(ctx, s);
  if (!w.dev || w.dev->bytes < bytes) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    cuda_check(cudaStreamIsCapturing(s, &st), "cudaStreamIsCapturing");
    if (st != cudaStreamCaptureStatusNone)
      fail(RC_ERR_INVALID_ARGUMENT, "scratch must be reserved (rc_reserve) before CUDA graph capture");
    cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    w.dev.reset();
    w.dev.reset(new DevBuf(bytes + (bytes >> 3)));
  }
  return w.dev->p;
}

void launch_check(const char* what) { cuda_check(cudaGetLastError(), what); }

LimbMap qmap(const rc_context* c, int limbs) { return LimbMap{limbs, c->L}; }

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

struct Arena {
  char* base;
  size_t off = 0;
  explicit Arena(void* b) : base((char*)b) {}
  template <class T>
  T* take(size_t count) {
    off = align_up(off, 256);
    T* p = (T*)(base + off);
    off += count * sizeof(T);
    return p;
  }
};

size_t arena_size_u64(size_t count) { return align_up(count * 8, 256); }

const LevelInfo& level_info(const rc_context* c, int limbs) {
  require(limbs >= 1 && limbs <= c->L, "level out of range for this context");
  return c->levels[limbs];
}

int floor_log2(uint64_t q) { return 63 - __builtin_clzll(q); }

// ------------------------------------------------------------------------
// keyswitch core shared by keyswitch / relinearize / mult_relinearized / rotate
// ------------------------------------------------------------------------
struct KsJob {
  const uint64_t* poly;  // c2 or c1 (device), qlimbs limbs
  const rc_ksk* key;
  const uint64_t* add0;  // addend for component 0 (null: none)
  const uint64_t* add1;
  uint64_t* out0;
  uint64_t* out1;
};

// batches group their jobs by (level, key kind, digits); the kind separates Q-only, gadget hybrid and
// RNS-hybrid keys
int key_kind(const rc_ksk* k) { return (int)(k->aux | (k->alpha << 16)); }

void check_key_for(const rc_context* c, const rc_ksk* key, int qlimbs) {
  require(key != nullptr, "keyswitch key must not be null");
  require(key->ctx == c, "keyswitch key belongs to another context");
  const LevelInfo& li = level_info(c, qlimbs);
  if (key->alpha) {  // RNS-hybrid key: one per level, over the active chain and P
    require(key->level == qlimbs - 1, "keyswitch key level must match the active Q chain");
    require((int)key->aux == c->K, "eval-key context must match the keyswitch key auxiliary basis");
    return;
  }
  if (key->aux == 0) {
    // keyswitch_rns, keyswitching.rs:135-137
    require(key->level == qlimbs - 1, "keyswitch key level must match the active modulus chain");
    require((int)key->digits >= li.digits, "keyswitch key must cover the active modulus chain");
  } else {
    // keyswitch_rns_hybrid, keyswitching.rs:165-168
    require(c->K > 0, "hybrid keyswitching requires an eval-key level context");
    require(key->level == qlimbs - 1, "keyswitch key level must match the active Q chain");
    require((int)key->aux == c->K, "eval-key context must match the keyswitch key auxiliary basis");
    require((int)key->digits >= li.digits, "keyswitch key must cover the active modulus chain");
  }
}

int ks_digits(const rc_context* c, const rc_ksk* k0, int qlimbs) {
  // Q-only: the reference decomposes into ksk.ksk.len() digits (keyswitching.rs:138);
  // hybrid: into the active digit count (167-170)
  const LevelInfo& li = level_info(c, qlimbs);
  if (k0 && k0->alpha) return (int)k0->digits;  // RNS-hybrid: the key's groups
  return (k0 && k0->aux) ? li.digits : (k0 ? std::max((int)k0->digits, 1) : li.digits);
}

size_t ks_scratch_elems(const rc_context* c, int J, int total, int D) {
  size_t pairs = (size_t)J * total;
  size_t chunk = c->scratch_budget / ((size_t)D * c->N * 8);
  if (chunk < 1) chunk = 1;
  if (chunk > pairs) chunk = pairs;
  return chunk * D * c->N;
}

size_t ks_ws_bytes(const rc_context* c, int J, int qlimbs, int K, int D) {
  const int total = qlimbs + K;
  const size_t standard = align_up((size_t)J * D * c->N * 4, 256) + arena_size_u64((size_t)J * 2 * total * c->N) +
                          arena_size_u64(ks_scratch_elems(c, J, total, D)) + 1024;
  const size_t wide = align_up((size_t)J * D * c->N * 4, 256) + 2 * arena_size_u64((size_t)J * D * 2 * c->N) +
                      arena_size_u64((size_t)J * 2 * total * 2 * c->N) + 1024;
  return std::max(standard, c->wide_ok ? wide : 0);
}

// scratch of the RNS-hybrid key switch: ModUp outputs [J][dnum][total][N] and products [J][2][total][N]
size_t dnum_ws_bytes(const rc_context* c, int J, int qlimbs, int dnum) {
  const size_t total = (size_t)qlimbs + c->K;
  return arena_size_u64((size_t)J * dnum * total * c->N) + arena_size_u64((size_t)J * 2 * total * c->N) + 1024;
}

// scratch of a key switch of J jobs at qlimbs with keys like k0
size_t ks_bytes_for(const rc_context* c, int J, int qlimbs, const rc_ksk* k0) {
  if (k0 && k0->alpha) return dnum_ws_bytes(c, J, qlimbs, (int)k0->digits);
  const int K = k0 && k0->aux ? c->K : 0;
  return ks_ws_bytes(c, J, qlimbs, K, ks_digits(c, k0, qlimbs));
}

// The exact integer key product applies when the internal primes' product A
// exceeds four times the largest possible |sum_i d_i k_ij| = D * N * 2^29 * (q_max - 1)
// (the CRT recovers the centred value from the top mixed-radix digit) and every
// digit is its own residue in each limb (no prime below 2^29 in Q_l).
bool wide_applies(const rc_context* c, int qlimbs, int K, int D) {
  if (!c->wide_ok || D > 200) return false;  // the key product keeps D digit words per job in shared memory
  if (level_info(c, qlimbs).dt.small_q) return false;
  uint64_t qmax = 0;
  for (int i = 0; i < qlimbs; ++i) qmax = std::max(qmax, c->mod[i]);
  for (int k = 0; k < K; ++k) qmax = std::max(qmax, c->mod[c->L + k]);
  const u128h bound = (u128h)D * (u128h)c->N * ((u128h)1 << 29) * (u128h)(qmax - 1);
  if (bound >= ((u128h)1 << 124)) return false;
  u128h A = 1;
  for (int i = 0; i < 4; ++i) A *= c->wp.q[i];
  return 4 * bound < A;
}

bool use_wide(const rc_context* c, const std::vector<KsJob>& jobs, int qlimbs, int K, int D) {
  for (auto& j : jobs)
    if (!j.key->wdata) return false;
  return wide_applies(c, qlimbs, K, D);
}

// ---- the wide key switch in phases, for pipelines that interleave other work between them ----
// Per-batch device buffers of the wide path: int32 digits, digit transforms and products of J jobs, plus a
// column-phase work area for up to `chunk` jobs at a time.
struct WideKs {
  int J = 0, D = 0, total = 0, qlimbs = 0, K = 0, chunk = 0;
  int32_t* digits = nullptr;
  uint2 *work = nullptr, *dt = nullptr, *acc = nullptr;
};

size_t wide_ks_bytes(const rc_context* c, int J, int chunk, int qlimbs, int K, int D) {
  const size_t N = c->N;
  return align_up((size_t)J * D * N * 4, 256) + arena_size_u64((size_t)chunk * D * 2 * N) +
         arena_size_u64((size_t)J * D * 2 * N) + arena_size_u64((size_t)J * 2 * (qlimbs + K) * 2 * N) + 1024;
}

WideKs wide_ks_layout(rc_context* c, Arena& ar, int J, int chunk, int qlimbs, int K, int D) {
  WideKs w;
  w.J = J, w.D = D, w.qlimbs = qlimbs, w.K = K, w.total = qlimbs + K, w.chunk = chunk;
  const size_t N = c->N;
  w.digits = ar.take<int32_t>((size_t)J * D * N);
  w.work = ar.take<uint2>((size_t)chunk * D * 2 * N);
  w.dt = ar.take<uint2>((size_t)J * D * 2 * N);
  w.acc = ar.take<uint2>((size_t)J * 2 * w.total * 2 * N);
  return w;
}

// decomposition and digit transforms of jobs [b0, b0 + n) (n <= chunk)
void wide_ks_prepare(rc_context* c, const WideKs& w, const std::vector<KsJob>& jobs, int b0, int n, uint64_t g_inv,
                     cudaStream_t s) {
  const size_t N = c->N;
  PtrTab src{};
  for (int j = 0; j < n; ++j) src.p[j] = const_cast<uint64_t*>(jobs[b0 + j].poly);
  decompose(c->d_pc, level_info(c, w.qlimbs).dt, src, n, w.qlimbs, w.D, w.digits + (size_t)b0 * w.D * N, g_inv,
            c->log_n, s);
  launch_check("decompose");
  require(wide_digit_transforms(c->wp, w.D, n, w.digits + (size_t)b0 * w.D * N, w.work,
                                w.dt + (size_t)b0 * 2 * w.D * N, s),
          "internal: wide transforms unsupported");
  launch_check("wide digit transforms");
}

// key products of all jobs, one launch per run of jobs sharing a key
void wide_ks_mac(rc_context* c, const WideKs& w, const std::vector<KsJob>& jobs, cudaStream_t s) {
  int b = 0;
  while (b < w.J) {
    int e = b + 1;
    while (e < w.J && jobs[e].key->wdata == jobs[b].key->wdata) ++e;
    wide_mac(c->wp, w.D, (int)jobs[b].key->digits, w.total, (const uint2*)jobs[b].key->wdata, w.dt, w.acc, b, e - b,
             c->mac_bc, s);
    launch_check("wide mac");
    b = e;
  }
}

// inverse transforms and finalize (ModDown, addends, optional rescale) of jobs [b0, b0 + n)
void wide_ks_finish(rc_context* c, const WideKs& w, const std::vector<KsJob>& jobs, int b0, int n, uint64_t g_inv,
                    bool rescale, cudaStream_t s) {
  const size_t N = c->N;
  uint2* acc = w.acc + (size_t)b0 * 2 * w.total * 2 * N;
  require(wide_inverse(c->wp, acc, n * 2 * w.total, s), "internal: wide transforms unsupported");
  launch_check("wide inverse transforms");
  FinalizeArgs f;
  f.pc = c->d_pc;
  f.md = c->md;
  f.rt = c->rt;
  f.L = c->L;
  f.n = c->N;
  f.log_n = c->log_n;
  f.qlimbs = w.qlimbs;
  f.K = w.K;
  f.rescale = rescale ? 1 : 0;
  f.add_g_inv = g_inv;
  f.wide = 1;
  f.wt = c->wide;
  // the lazy finalize sums per limb terms below (12 + 4K) q in all: every prime below 2^64 / (12 + 4K)
  f.lazy = 1;
  for (uint64_t m : c->mod)
    if (m >= UINT64_MAX / (uint64_t)(12 + 4 * w.K)) f.lazy = 0;
  PtrTab add{}, out{};
  for (int j = 0; j < n; ++j) {
    add.p[2 * j] = const_cast<uint64_t*>(jobs[b0 + j].add0);
    add.p[2 * j + 1] = const_cast<uint64_t*>(jobs[b0 + j].add1);
    out.p[2 * j] = jobs[b0 + j].out0;
    out.p[2 * j + 1] = jobs[b0 + j].out1;
  }
  finalize(f, (const uint64_t*)acc, add, out, n, s);
  launch_check("finalize");
}

// ---- mixed-level wide key switch: every pass is one launch over jobs of different levels ----
// Job j is at qlimbs[j] Q limbs; jobs sharing a key are consecutive.  Buffers: int32 digits [sum D][N],
// column-phase work and tiled digit transforms [sum D][2][N], products [sum 2 (limbs + K)][2][N] (uint2).
size_t ml_ks_bytes(const rc_context* c, const std::vector<KsJob>& jobs, const std::vector<int>& qlimbs, int K) {
  size_t dig = 0, acc = 0;
  for (size_t j = 0; j < jobs.size(); ++j) {
    dig += (size_t)ks_digits(c, jobs[j].key, qlimbs[j]);
    acc += (size_t)2 * (qlimbs[j] + K);
  }
  const size_t N = c->N;
  return align_up(dig * N * 4, 256) + 2 * arena_size_u64(dig * 2 * N) + arena_size_u64(acc * 2 * N) + 1024;
}

// a job fits the mixed-level path: a wide key of the batch's kind whose level passes the wide product's bound
bool ml_job_ok(const rc_context* c, const rc_ksk* key, int qlimbs, int K) {
  if (!key || !key->wdata || (key->aux ? c->K : 0) != K) return false;
  return wide_applies(c, qlimbs, K, ks_digits(c, key, qlimbs));
}

void keyswitch_ml(rc_context* c, const std::vector<KsJob>& jobs, const std::vector<int>& qlimbs, bool rescale,
                  void* ws, cudaStream_t s) {
  const int J = (int)jobs.size();
  if (!J) return;
  require(J <= ML_MAXJ, "internal: mixed-level chunk too large");
  const int K = jobs[0].key->aux ? c->K : 0;
  const size_t N = c->N;
  MlTab t{};
  MlPtrTab src{}, add{}, out{};
  MlKeys keys{};
  t.J = J;
  int max_limbs = 0, max_W = 0;
  for (int j = 0; j < J; ++j) {
    check_key_for(c, jobs[j].key, qlimbs[j]);
    require(ml_job_ok(c, jobs[j].key, qlimbs[j], K), "internal: job outside the mixed-level key switch");
    const int D = ks_digits(c, jobs[j].key, qlimbs[j]);
    t.limbs[j] = qlimbs[j];
    t.dig[j + 1] = t.dig[j] + D;
    t.acc[j + 1] = t.acc[j] + 2 * (qlimbs[j] + K);
    src.p[j] = const_cast<uint64_t*>(jobs[j].poly);
    add.p[2 * j] = const_cast<uint64_t*>(jobs[j].add0);
    add.p[2 * j + 1] = const_cast<uint64_t*>(jobs[j].add1);
    out.p[2 * j] = jobs[j].out0;
    out.p[2 * j + 1] = jobs[j].out1;
    max_limbs = std::max(max_limbs, qlimbs[j]);
    max_W = std::max(max_W, level_info(c, qlimbs[j]).dt.W);
    if (j == 0 || jobs[j].key->wdata != jobs[j - 1].key->wdata) {
      require(keys.n < ML_MAXK, "internal: too many keys in a mixed-level chunk");
      keys.k[keys.n++] = MlKey{(const uint2*)jobs[j].key->wdata, D, (int)jobs[j].key->digits, qlimbs[j] + K, j, 0};
    }
    require(keys.k[keys.n - 1].total == qlimbs[j] + K, "internal: one key at two levels");
    keys.k[keys.n - 1].count++;
  }
  Arena ar(ws);
  int32_t* digits = ar.take<int32_t>((size_t)t.dig[J] * N);
  uint2* work = ar.take<uint2>((size_t)t.dig[J] * 2 * N);
  uint2* dt = ar.take<uint2>((size_t)t.dig[J] * 2 * N);
  uint2* acc = ar.take<uint2>((size_t)t.acc[J] * 2 * N);
  decompose_ml(c->d_pc, c->d_dts, t, src, max_limbs, max_W, digits, c->log_n, s);
  launch_check("decompose (mixed levels)");
  require(wide_digit_transforms_ml(c->wp, t, digits, work, dt, s), "internal: wide transforms unsupported");
  launch_check("wide digit transforms (mixed levels)");
  wide_mac_ml(c->wp, t, keys, dt, acc, c->mac_bc, s);
  launch_check("wide mac (mixed levels)");
  require(wide_inverse(c->wp, acc, t.acc[J], s), "internal: wide transforms unsupported");
  launch_check("wide inverse transforms (mixed levels)");
  FinalizeArgs f;
  f.pc = c->d_pc;
  f.md = c->md;
  f.rt = c->rt;
  f.L = c->L;
  f.n = c->N;
  f.log_n = c->log_n;
  f.qlimbs = max_limbs;
  f.K = K;
  f.rescale = rescale ? 1 : 0;
  f.add_g_inv = 0;
  f.wide = 1;
  f.wt = c->wide;
  f.lazy = 1;  // as in keyswitch_wide: per-limb terms below (12 + 4K) q in all
  for (uint64_t m : c->mod)
    if (m >= UINT64_MAX / (uint64_t)(12 + 4 * K)) f.lazy = 0;
  finalize_ml(f, t, (const uint64_t*)acc, add, out, s);
  launch_check("finalize (mixed levels)");
}

// Key switch + add (+ rescale) of a batch of any levels: when every job fits the mixed-level path, the jobs
// (highest level first, jobs of one key together) run in chunks of up to ml_jobs jobs, each chunk one
// launch per pass; otherwise false (the caller groups by level).
bool keyswitch_mixed_batch(rc_context* c, const rc_ciphertext* qct, const rc_ksk* const* keys, rc_ciphertext* out,
                           uint32_t count, bool rescale, cudaStream_t s) {
  if (!c->mixed_levels || !c->wide_ok || count < 2) return false;
  const int K = keys[0]->aux ? c->K : 0;
  bool mixed = false;
  for (uint32_t i = 0; i < count; ++i) {
    if (!ml_job_ok(c, keys[i], qct[i].level + 1, K)) return false;
    mixed = mixed || qct[i].level != qct[0].level;
  }
  if (!mixed) return false;  // one level: the uniform path
  std::vector<int> order(count);
  for (uint32_t i = 0; i < count; ++i) order[i] = (int)i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    if (qct[a].level != qct[b].level) return qct[a].level > qct[b].level;
    return keys[a]->wdata < keys[b]->wdata;
  });
  size_t b = 0;
  while (b < order.size()) {
    std::vector<KsJob> jobs;
    std::vector<int> ql;
    int nkeys = 0;
    for (size_t k = b; k < order.size() && (int)jobs.size() < c->ml_jobs; ++k) {
      const int i = order[k];
      const bool new_key = jobs.empty() || keys[i]->wdata != jobs.back().key->wdata;
      if (new_key && nkeys == ML_MAXK) break;
      nkeys += new_key ? 1 : 0;
      const int limbs = qct[i].level + 1;
      const size_t pl = (size_t)limbs * c->N;
      const size_t po = (size_t)(rescale ? limbs - 1 : limbs) * c->N;
      jobs.push_back(KsJob{qct[i].data + 2 * pl, keys[i], qct[i].data, qct[i].data + pl, out[i].data,
                           out[i].data + po});
      ql.push_back(limbs);
    }
    void* ws = ws_device(c, s, ml_ks_bytes(c, jobs, ql, K));
    keyswitch_ml(c, jobs, ql, rescale, ws, s);
    b += jobs.size();
  }
  return true;
}

// The RNS-hybrid key switch of `jobs` (keys from rc_ksk_upload_dnum at this level): ModUp of each job's
// polynomial group by group, forward transforms over Q_l u P, the key product, inverse transforms, and the
// exact ModDown with addends and optional rescale of k_finalize.  Relinearization only (no automorphism).
void keyswitch_dnum(rc_context* c, const std::vector<KsJob>& jobs, int qlimbs, uint64_t g_inv, bool rescale,
                    void* ws, cudaStream_t s) {
  require(g_inv <= 1, "RNS-hybrid keys serve relinearization only");
  const int J = (int)jobs.size();
  const rc_ksk* k0 = jobs[0].key;
  const int dnum = (int)k0->digits, alpha = (int)k0->alpha, K = c->K, total = qlimbs + K;
  for (auto& j : jobs) require((int)j.key->digits == dnum, "internal: mixed key shapes in one keyswitch batch");
  const size_t N = c->N, per = (size_t)total * N;
  const LimbMap map{qlimbs, c->L};
  Arena ar(ws);
  uint64_t* D = ar.take<uint64_t>((size_t)J * dnum * per);
  uint64_t* acc = ar.take<uint64_t>((size_t)J * 2 * per);
  int b = 0;
  while (b < J) {  // runs of jobs sharing a key
    int e = b + 1;
    while (e < J && jobs[e].key == jobs[b].key) ++e;
    PtrTab src{};
    for (int j = b; j < e; ++j) src.p[j - b] = const_cast<uint64_t*>(jobs[j].poly);
    dnum_modup(c->d_pc, src, e - b, (const uint64_t*)jobs[b].key->mbuf->p, D + (size_t)b * dnum * per, qlimbs, total,
               alpha, dnum, map, c->log_n, s);
    launch_check("dnum modup");
    const int polys = (e - b) * dnum;
    for (int p0 = 0; p0 < polys; p0 += MAXP) {
      PtrTab t{};
      const int cnt = std::min(MAXP, polys - p0);
      for (int k = 0; k < cnt; ++k) t.p[k] = D + ((size_t)b * dnum + p0 + k) * per;
      ntt_forward(c->ntt(), t, t, cnt, total, map, s);
      launch_check("dnum ntt");
    }
    dnum_mac(c->d_pc, D + (size_t)b * dnum * per, jobs[b].key->data, acc + (size_t)b * 2 * per, e - b, total, dnum,
             map, c->log_n, s);
    launch_check("dnum mac");
    b = e;
  }
  for (int p0 = 0; p0 < 2 * J; p0 += MAXP) {
    PtrTab t{};
    const int cnt = std::min(MAXP, 2 * J - p0);
    for (int k = 0; k < cnt; ++k) t.p[k] = acc + (size_t)(p0 + k) * per;
    ntt_inverse(c->ntt(), t, t, cnt, total, map, s);
    launch_check("dnum inverse ntt");
  }
  FinalizeArgs f;
  f.pc = c->d_pc;
  f.md = c->md;
  f.rt = c->rt;
  f.L = c->L;
  f.n = c->N;
  f.log_n = c->log_n;
  f.qlimbs = qlimbs;
  f.K = K;
  f.rescale = rescale ? 1 : 0;
  f.add_g_inv = 0;
  f.wide = 0;
  f.wt = c->wide;
  f.lazy = 0;
  PtrTab add{}, out{};
  for (int j = 0; j < J; ++j) {
    add.p[2 * j] = const_cast<uint64_t*>(jobs[j].add0);
    add.p[2 * j + 1] = const_cast<uint64_t*>(jobs[j].add1);
    out.p[2 * j] = jobs[j].out0;
    out.p[2 * j + 1] = jobs[j].out1;
  }
  finalize(f, acc, add, out, J, s);
  launch_check("finalize");
}

// Runs keyswitch for `jobs` jobs at `qlimbs` limbs (all keys of the same kind);
// the result is finalized with addends, optional automorphism on the addend and
// optional rescale.  g_inv: automorphism applied to the keyswitched polynomial
// and to addend 0 (rotation), 0 = none.  `ws` holds ks_ws_bytes().
void keyswitch_core(rc_context* c, const std::vector<KsJob>& jobs, int qlimbs, uint64_t g_inv, bool rescale,
                    void* ws, cudaStream_t s) {
  if (jobs.empty()) return;
  const int J = (int)jobs.size();
  require(J <= MAXP / 2, "internal: keyswitch chunk too large");
  const rc_ksk* k0 = jobs[0].key;
  for (auto& j : jobs) check_key_for(c, j.key, qlimbs);
  for (auto& j : jobs) require(j.key->alpha == k0->alpha, "internal: mixed key kinds in one keyswitch batch");
  if (k0->alpha) {
    keyswitch_dnum(c, jobs, qlimbs, g_inv, rescale, ws, s);
    return;
  }
  const int K = k0->aux ? c->K : 0;
  const LevelInfo& li = level_info(c, qlimbs);
  const int D = ks_digits(c, k0, qlimbs);
  for (auto& j : jobs) {
    require((j.key->aux ? c->K : 0) == K, "internal: mixed key kinds in one keyswitch batch");
    if (!K) require((int)j.key->digits == D, "internal: mixed digit counts in one keyswitch batch");
  }
  const int N = c->N, total = qlimbs + K;
  if (use_wide(c, jobs, qlimbs, K, D)) {
    Arena aw(ws);
    const WideKs w = wide_ks_layout(c, aw, J, J, qlimbs, K, D);
    wide_ks_prepare(c, w, jobs, 0, J, g_inv, s);
    wide_ks_mac(c, w, jobs, s);
    wide_ks_finish(c, w, jobs, 0, J, g_inv, rescale, s);
    return;
  }
  const size_t scratch_elems = ks_scratch_elems(c, J, total, D);
  Arena ar(ws);
  int32_t* digits = ar.take<int32_t>((size_t)J * D * N);
  PtrTab src{};
  for (int j = 0; j < J; ++j) src.p[j] = const_cast<uint64_t*>(jobs[j].poly);
  decompose(c->d_pc, li.dt, src, J, qlimbs, D, digits, g_inv, c->log_n, s);
  launch_check("decompose");

  FinalizeArgs f;
  f.pc = c->d_pc;
  f.md = c->md;
  f.rt = c->rt;
  f.L = c->L;
  f.n = N;
  f.log_n = c->log_n;
  f.qlimbs = qlimbs;
  f.K = K;
  f.rescale = rescale ? 1 : 0;
  f.add_g_inv = g_inv;
  f.wide = 0;
  f.wt = c->wide;
  f.lazy = 0;
  PtrTab add{}, out{};
  for (int j = 0; j < J; ++j) {
    add.p[2 * j] = const_cast<uint64_t*>(jobs[j].add0);
    add.p[2 * j + 1] = const_cast<uint64_t*>(jobs[j].add1);
    out.p[2 * j] = jobs[j].out0;
    out.p[2 * j + 1] = jobs[j].out1;
  }

  for (auto& j : jobs) require(j.key->data != nullptr, "internal: keyswitch key has no per-limb form");
  uint64_t* acc = ar.take<uint64_t>((size_t)J * 2 * total * N);
  uint64_t* scratch = ar.take<uint64_t>(scratch_elems);

  KsArgs ka;
  ka.pc = c->d_pc;
  ka.ntt = c->ntt();
  ka.n = N;
  ka.L = c->L;
  ka.qlimbs = qlimbs;
  ka.K = K;
  ka.D = D;
  ka.key_digits = (int)k0->digits;
  ka.mac64 = c->mac64 ? 1 : 0;
  ka.dt = &li.dt;
  std::vector<const uint64_t*> keys(J);
  for (int j = 0; j < J; ++j) keys[j] = jobs[j].key->data;
  digit_ntt_mac(ka, digits, keys.data(), J, acc, scratch, scratch_elems, s);
  launch_check("digit_ntt_mac");

  // back to coefficient form: 2*J polys of `total` limbs
  PtrTab t{};
  for (int p = 0; p < 2 * J; ++p) t.p[p] = acc + (size_t)p * total * N;
  ntt_inverse(c->ntt(), t, t, 2 * J, total, LimbMap{qlimbs, c->L}, s);
  launch_check("ntt_inverse(acc)");
  finalize(f, acc, add, out, J, s);
  launch_check("finalize");
}

// single-call keyswitch with its own workspace
void keyswitch_run(rc_context* c, const std::vector<KsJob>& jobs, int qlimbs, uint64_t g_inv, bool rescale,
                   cudaStream_t s) {
  if (jobs.empty()) return;
  const rc_ksk* k0 = jobs[0].key;
  check_key_for(c, k0, qlimbs);
  const int K = k0->aux ? c->K : 0;
  (void)K;
  void* ws = ws_device(c, s, ks_bytes_for(c, (int)jobs.size(), qlimbs, k0));
  keyswitch_core(c, jobs, qlimbs, g_inv, rescale, ws, s);
}

size_t tensor_ws_bytes(const rc_context* c, int J, int limbs) {
  return arena_size_u64((size_t)4 * J * limbs * c->N) + 512;
}

// tensor for J jobs at `limbs` limbs; writes coefficient-form (d0,d1,d2) to
// quad[j] (3 polys contiguous).  `ws` holds tensor_ws_bytes().
void tensor_core(rc_context* c, const std::vector<const uint64_t*>& lhs, const std::vector<const uint64_t*>& rhs,
                 const std::vector<uint64_t*>& quad, int limbs, void* ws, cudaStream_t s) {
  const int J = (int)lhs.size();
  if (!J) return;
  require(4 * J <= MAXP, "internal: tensor chunk too large");
  const size_t pl = (size_t)limbs * c->N;
  Arena ar(ws);
  uint64_t* fw = ar.take<uint64_t>(4 * J * pl);
  PtrTab src{}, dst{};
  for (int j = 0; j < J; ++j) {
    src.p[4 * j + 0] = const_cast<uint64_t*>(lhs[j]);
    src.p[4 * j + 1] = const_cast<uint64_t*>(lhs[j]) + pl;
    src.p[4 * j + 2] = const_cast<uint64_t*>(rhs[j]);
    src.p[4 * j + 3] = const_cast<uint64_t*>(rhs[j]) + pl;
    for (int k = 0; k < 4; ++k) dst.p[4 * j + k] = fw + (4 * j + k) * pl;
  }
  PtrTab o3{};
  for (int j = 0; j < J; ++j)
    for (int k = 0; k < 3; ++k) o3.p[3 * j + k] = quad[j] + k * pl;
  if (c->fuse_tensor && tensor_fused(c->ntt(), c->d_pc, src, dst, o3, J, limbs, qmap(c, limbs), s)) {
    launch_check("tensor (fused)");
    return;
  }
  // the forward outputs go only to the tensor's Montgomery products: left unreduced (below B q, B = 4 log N + 1
  // lazy, else 4) when every prime keeps a0 b1 + a1 b0 < 2 B^2 q^2 below q 2^64, the bound of its reduction;
  // the products' residues, and so the canonical outputs of the inverse transform, are the same
  NttArgs fwd = c->ntt();
  {
    const uint64_t B = fwd.lazy ? 4 * (uint64_t)c->log_n + 1 : 4;
    bool ok = true;
    for (int i = 0; i < limbs; ++i) ok = ok && (u128h)2 * B * B * c->mod[i] < ((u128h)1 << 64);
    fwd.raw_out = ok ? 1 : 0;
  }
  ntt_forward(fwd, src, dst, 4 * J, limbs, qmap(c, limbs), s);
  launch_check("ntt_forward(tensor)");
  // the tensor's Montgomery products carry a factor 2^-64, taken out by the inverse transform's scale
  NttArgs inv = c->ntt();
  inv.mont_out = 1;
  if (tensor_inverse_rows(inv, dst, o3, J, limbs, qmap(c, limbs), s)) {
    launch_check("tensor + inverse rows");
    require(ntt_inverse_cols(inv, o3, 3 * J, limbs, qmap(c, limbs), s), "internal: inverse columns unsupported");
    launch_check("ntt_inverse(tensor) columns");
    return;
  }
  tensor_ntt(c->d_pc, dst, o3, J, limbs, c->N, s);
  launch_check("tensor");
  ntt_inverse(inv, o3, o3, 3 * J, limbs, qmap(c, limbs), s);
  launch_check("ntt_inverse(tensor)");
}

void check_ct(const rc_context* c, const rc_ciphertext* ct, const char* name) {
  require(ct != nullptr && ct->data != nullptr, std::string(name) + " must not be null");
  require(ct->level >= 0 && ct->level < c->L, std::string(name) + " level out of range for this context");
}

uint64_t galois_inverse(const rc_context* c, uint64_t g) {
  const uint64_t m = 2ull * c->N;
  require(g % 2 == 1, "galois automorphisms require an odd exponent");
  return invmod_h(g % m, m);
}

// mult_relinearized on J jobs: the tensor runs in chunks of MAXP/4 jobs (four pointer-table entries each),
// the keyswitch on all J <= MAXP/2 jobs at once so that one key read serves them all
size_t mult_relin_ws_bytes(const rc_context* c, int J, int limbs, const rc_ksk* k0) {
  const size_t pl = (size_t)limbs * c->N;
  return align_up(std::max(ks_bytes_for(c, J, limbs, k0),
                           tensor_ws_bytes(c, std::min(J, MAXP / 4), limbs)),
                  256) +
         arena_size_u64((size_t)3 * J * pl) + 256;
}

// mult_relinearized for a same-level, same-key-kind group (chunked to fit the
// pointer tables): tensor into quads at the end of the workspace, then
// keyswitch(c2) + add (c0, c1) + rescale in the fused finalize.
void mult_relin_group(rc_context* c, const std::vector<int>& idx, const rc_ciphertext* lhs, const rc_ciphertext* rhs,
                      const rc_ksk* const* keys, rc_ciphertext* out, cudaStream_t s) {
  const int limbs = lhs[idx[0]].level + 1;
  require(limbs > 1, "rescale requires at least two levels");
  const size_t pl = (size_t)limbs * c->N;
  const int CH = c->ks_jobs;
  for (size_t b = 0; b < idx.size(); b += CH) {
    const int J = (int)std::min<size_t>(CH, idx.size() - b);
    std::vector<KsJob> jobs(J);
    for (int j = 0; j < J; ++j) {
      require(keys[idx[b + j]] != nullptr, "keyswitch key must not be null");
      check_key_for(c, keys[idx[b + j]], limbs);
    }
    const rc_ksk* k0 = keys[idx[b]];
    const size_t head = align_up(std::max(ks_bytes_for(c, J, limbs, k0),
                                          tensor_ws_bytes(c, std::min(J, MAXP / 4), limbs)),
                                 256);
    char* ws = (char*)ws_device(c, s, mult_relin_ws_bytes(c, J, limbs, k0));
    uint64_t* quad = (uint64_t*)(ws + head);
    std::vector<uint64_t*> Q(J);
    for (int j = 0; j < J; ++j) Q[j] = quad + (size_t)j * 3 * pl;
    for (int t0 = 0; t0 < J; t0 += MAXP / 4) {
      const int T = std::min(J - t0, MAXP / 4);
      std::vector<const uint64_t*> Lp(T), Rp(T);
      std::vector<uint64_t*> Qt(T);
      for (int j = 0; j < T; ++j) {
        Lp[j] = lhs[idx[b + t0 + j]].data;
        Rp[j] = rhs[idx[b + t0 + j]].data;
        Qt[j] = Q[t0 + j];
      }
      tensor_core(c, Lp, Rp, Qt, limbs, ws, s);
    }
    for (int j = 0; j < J; ++j) {
      const int i = idx[b + j];
      jobs[j].poly = Q[j] + 2 * pl;
      jobs[j].key = keys[i];
      jobs[j].add0 = Q[j];
      jobs[j].add1 = Q[j] + pl;
      jobs[j].out0 = out[i].data;
      jobs[j].out1 = out[i].data + (size_t)(limbs - 1) * c->N;
    }
    keyswitch_core(c, jobs, limbs, 0, true, ws, s);
    for (int j = 0; j < J; ++j) {
      const int i = idx[b + j];
      const int sb = lhs[i].scale_bits + rhs[i].scale_bits - floor_log2(c->mod[limbs - 1]);
      out[i].level = lhs[i].level - 1;
      out[i].scale_bits = sb < 0 ? 0 : sb;
    }
  }
}

void check_mult_pair(const rc_context* c, const rc_ciphertext* a, const rc_ciphertext* b) {
  check_ct(c, a, "lhs");
  check_ct(c, b, "rhs");
  // RnsCkksContext::mult, context/ops.rs:64-65
  require(a->level == b->level, "ciphertexts must be at the same level to multiply");
  require(a->scale_bits == b->scale_bits, "ciphertexts must share the same scale to multiply");
}

}  // namespace

namespace rc {
const LevelInfo& context_level(const rc_context* c, int limbs) { return level_info(c, limbs); }
bool context_wide_applies(const rc_context* c, int qlimbs, int K, int D) { return wide_applies(c, qlimbs, K, D); }
void context_check_ct(const rc_context* c, const rc_ciphertext* ct, const char* name) { check_ct(c, ct, name); }
uint64_t context_galois_inverse(const rc_context* c, uint64_t g) { return galois_inverse(c, g); }
}  // namespace rc

// =========================================================================
// context
// =========================================================================
extern "C" int rc_context_create(const rc_params* p, rc_context** out) {
  return guarded("rc_context_create", [&] {
    require(p != nullptr && out != nullptr, "params and out must not be null");
    *out = nullptr;
    // RnsCkksParams::validate, src/rns/context/params.rs:48-73
    require(p->scale_bits != 0, "scale_bits must be greater than zero");
    require(p->scale_bits < 60, "scale_bits must stay below 60 bits per rescale step in this RNS scaffold");
    std::vector<uint64_t> qm, qg, pm, pg;
    for (uint32_t i = 0; i < p->prime_count; ++i) {
      qm.push_back(p->primes[i].modulus);
      qg.push_back(p->primes[i].primitive_root);
    }
    for (uint32_t i = 0; i < p->aux_count; ++i) {
      pm.push_back(p->aux_primes[i].modulus);
      pg.push_back(p->aux_primes[i].primitive_root);
    }
    for (uint64_t a : pm)
      for (uint64_t q : qm)
        require(a != q, "auxiliary eval-key modulus " + std::to_string(a) +
                            " must be distinct from the ciphertext modulus chain");
    validate_chain(p->poly_degree, qm, qg);
    if (!pm.empty()) {
      validate_chain(p->poly_degree, pm, pg);
      std::vector<uint64_t> all = qm, allg = qg;
      all.insert(all.end(), pm.begin(), pm.end());
      allg.insert(allg.end(), pg.begin(), pg.end());
      validate_chain(p->poly_degree, all, allg);
    }
    // limits of this implementation
    const uint64_t N = p->poly_degree;
    if (N < 2 || N > (1u << 17)) fail(RC_ERR_UNSUPPORTED, "poly_degree must be in 2..=131072 on the GPU path");
    if (qm.size() > 64) fail(RC_ERR_UNSUPPORTED, "at most 64 ciphertext primes on the GPU path");
    if (pm.size() > 8) fail(RC_ERR_UNSUPPORTED, "at most 8 auxiliary primes on the GPU path");
    for (uint64_t q : qm)
      if (q >= (1ull << 61)) fail(RC_ERR_UNSUPPORTED, "primes must be below 2^61 on the GPU path");
    for (uint64_t q : pm)
      if (q >= (1ull << 61)) fail(RC_ERR_UNSUPPORTED, "primes must be below 2^61 on the GPU path");

    std::unique_ptr<rc_context> c(new rc_context());
    cuda_check(cudaGetDevice(&c->device), "cudaGetDevice");
    c->N = (int)N;
    c->log_n = __builtin_ctzll(N);
    c->n1 = c->log_n / 2;
    c->L = (int)qm.size();
    c->K = (int)pm.size();
    c->scale_bits = (int)p->scale_bits;
    c->mod = qm;
    c->mod.insert(c->mod.end(), pm.begin(), pm.end());
    c->root = qg;
    c->root.insert(c->root.end(), pg.begin(), pg.end());
    const int P = (int)c->mod.size();
    // Lazy (unreduced) forward butterflies with approximate Shoup products need every prime < 2^57
    // ((4 log N + 1) q < 2^64)
    c->lazy = true;
    if (const char* e = getenv("RNSCKKS_LAZY_NTT")) c->lazy = atoi(e) != 0;
    for (uint64_t q : c->mod) c->lazy = c->lazy && q < (1ull << 57);
    c->lazy_inv = true;
    for (uint64_t q : c->mod) c->lazy_inv = c->lazy_inv && q < (1ull << 55);
    if (const char* e = getenv("RNSCKKS_MAC64")) c->mac64 = atoi(e) != 0;

    // ---- per-prime constants and twiddles
    std::vector<PrimeConst> pcs(P);
    // bound (in multiples of q) of a forward-NTT output fed to the key product: 4q per stage above q when lazy
    // (approximate Shoup products), 4q otherwise; for either butterfly mode (the mode can be changed later with
    // rc_tune_set), so the key-product chunk below stays valid
    const uint64_t out_bound = std::max<uint64_t>(4 * c->log_n + 1, 4);
    std::vector<Twiddle> twf((size_t)P * N), twi((size_t)P * N);
    for (int i = 0; i < P; ++i) {
      const uint64_t q = c->mod[i];
      PrimeConst& k = pcs[i];
      memset(&k, 0, sizeof(k));
      k.q = q;
      k.two_q = 2 * q;
      u128h mu = (~(u128h)0) / q;
      k.mu_hi = (uint64_t)(mu >> 64);
      k.mu_lo = (uint64_t)mu;
      uint64_t inv = q;  // Newton iteration for q^-1 mod 2^64
      for (int it = 0; it < 6; ++it) inv *= 2 - q * inv;
      k.qinv_neg = (uint64_t)0 - inv;
      k.n_inv = invmod_h(N % q, q);
      k.n_inv_s = shoup_h(k.n_inv, q);
      k.r2 = (uint64_t)((((u128h)1 << 64) % q) * (((u128h)1 << 64) % q) % q);
      k.n_inv_r = (uint64_t)((u128h)k.n_inv * (uint64_t)(((u128h)1 << 64) % q) % q);
      k.n_inv_r_s = shoup_h(k.n_inv_r, q);
      k.one_s = shoup_h(1, q);
      // key words are < q: sum of chunk products stays below q * 2^64
      k.mac_chunk = (uint64_t)((~0ull) / (out_bound * q));
      k.mac_chunk64 = (uint64_t)((~0ull) / (2 * q));
      // psi = g^((q-1)/2N) (NttPlan::new, ntt.rs:42)
      const uint64_t psi = powmod_h(c->root[i] % q, (q - 1) / (2 * N), q);
      const uint64_t psi_inv = invmod_h(psi, q);
      std::vector<uint64_t> pw(N), pwi(N);
      pw[0] = pwi[0] = 1;
      for (uint64_t e = 1; e < N; ++e) {
        pw[e] = mulmod_h(pw[e - 1], psi, q);
        pwi[e] = mulmod_h(pwi[e - 1], psi_inv, q);
      }
      for (uint64_t kk = 0; kk < N; ++kk) {
        int e = bitrev((int)kk, c->log_n);
        Twiddle& f = twf[(size_t)i * N + kk];
        f.w = pw[e];
        f.ws = shoup_h(f.w, q);
        Twiddle& g = twi[(size_t)i * N + kk];
        g.w = pwi[e];
        g.ws = shoup_h(g.w, q);
      }
      // the inverse transform's last stage (its one twiddle, index 1 of the table) times the scale (InvScale)
      const uint64_t w1 = N > 1 ? twi[(size_t)i * N + 1].w : 1;
      k.w1n = mulmod_h(w1, k.n_inv, q);
      k.w1n_s = shoup_h(k.w1n, q);
      k.w1nr = mulmod_h(w1, k.n_inv_r, q);
      k.w1nr_s = shoup_h(k.w1nr, q);
    }
    c->pc_buf.reset(new DevBuf(sizeof(PrimeConst) * P));
    c->d_pc = (PrimeConst*)c->pc_buf->p;
    cuda_check(cudaMemcpy(c->d_pc, pcs.data(), sizeof(PrimeConst) * P, cudaMemcpyHostToDevice), "upload consts");
    c->tw_buf.reset(new DevBuf(sizeof(Twiddle) * 2 * P * N));
    c->d_twf = (Twiddle*)c->tw_buf->p;
    c->d_twi = c->d_twf + (size_t)P * N;
    cuda_check(cudaMemcpy(c->d_twf, twf.data(), sizeof(Twiddle) * P * N, cudaMemcpyHostToDevice), "upload tw");
    cuda_check(cudaMemcpy(c->d_twi, twi.data(), sizeof(Twiddle) * P * N, cudaMemcpyHostToDevice), "upload tw");

    // ---- per-level decomposition tables
    c->levels.resize(c->L + 1);
    for (int l = 1; l <= c->L; ++l) {
      LevelInfo& li = c->levels[l];
      li.limbs = l;
      BigU Q = product(qm, 0, l);
      li.bits = Q.bits();
      li.digits = (int)((li.bits + 29) / 30);
      const int W = (int)((li.bits + 8 + 63) / 64);
      std::vector<uint64_t> blob;  // [qhat l*W][qinv l][qinv_s l][invq l][Q W][halfQ W]
      blob.reserve((size_t)l * W + 3 * l + 2 * W);
      for (int i = 0; i < l; ++i) {
        auto w = Q.div_u64(qm[i]).words(W);
        blob.insert(blob.end(), w.begin(), w.end());
      }
      size_t o_qinv = blob.size();
      for (int i = 0; i < l; ++i) blob.push_back(invmod_h(Q.div_u64(qm[i]).mod_u64(qm[i]), qm[i]));
      size_t o_qinv_s = blob.size();
      for (int i = 0; i < l; ++i) blob.push_back(shoup_h(blob[o_qinv + i], qm[i]));
      size_t o_invq = blob.size();
      for (int i = 0; i < l; ++i) {
        int bits = 0;
        while (bits < 64 && (qm[i] >> bits)) ++bits;
        const uint32_t n = (uint32_t)(64 - bits);
        const unsigned __int128 qn = (unsigned __int128)(qm[i] << n);
        const uint64_t r = (uint64_t)((((unsigned __int128)1) << 95) / qn);  // < 2^32: qn > 2^63
        blob.push_back(((uint64_t)n << 32) | r);
      }
      size_t o_Q = blob.size();
      auto qw = Q.words(W);
      blob.insert(blob.end(), qw.begin(), qw.end());
      size_t o_hQ = blob.size();
      auto hw = Q.shr1().words(W);
      blob.insert(blob.end(), hw.begin(), hw.end());
      // lift to the aux primes: 2^(64 w) mod p_k for w = 0..W, then their Shoup companions
      size_t o_pw = blob.size();
      for (size_t k = 0; k < pm.size(); ++k) {
        const uint64_t two64 = mulmod_h(powmod_h(2, 32, pm[k]), powmod_h(2, 32, pm[k]), pm[k]);
        for (int w = 0; w <= W; ++w) blob.push_back(powmod_h(two64, (uint64_t)w, pm[k]));
      }
      size_t o_pws = blob.size();
      for (size_t k = 0; k < pm.size(); ++k)
        for (int w = 0; w <= W; ++w) blob.push_back(shoup_h(blob[o_pw + k * (W + 1) + w], pm[k]));
      li.buf.reset(new DevBuf(blob.size() * 8));
      uint64_t* d = (uint64_t*)li.buf->p;
      cuda_check(cudaMemcpy(d, blob.data(), blob.size() * 8, cudaMemcpyHostToDevice), "upload level tables");
      li.dt.qhat = d;
      li.dt.qhat_inv = d + o_qinv;
      li.dt.qhat_inv_s = d + o_qinv_s;
      li.dt.inv_q = d + o_invq;
      li.dt.Q = d + o_Q;
      li.dt.halfQ = d + o_hQ;
      li.dt.lift_pw = pm.empty() ? nullptr : d + o_pw;
      li.dt.lift_pw_s = pm.empty() ? nullptr : d + o_pws;
      li.dt.W = W;
      li.dt.small_q = li.bits <= 30 ? 1 : 0;
      li.dt.Qsmall = li.bits <= 63 ? Q.words(1)[0] : 0;
    }
    // the same tables as one device array indexed by limb count, for launches that mix levels
    {
      std::vector<DecompTab> dts(c->L + 1);
      for (int l = 1; l <= c->L; ++l) dts[l] = c->levels[l].dt;
      c->dt_buf.reset(new DevBuf(dts.size() * sizeof(DecompTab)));
      c->d_dts = (DecompTab*)c->dt_buf->p;
      cuda_check(cudaMemcpy(c->d_dts, dts.data(), dts.size() * sizeof(DecompTab), cudaMemcpyHostToDevice),
                 "upload level tables");
    }

    // ---- ModDown tables (aux basis)
    {
      const int K = c->K, L = c->L;
      std::vector<uint64_t> blob;
      size_t o_pg = 0, o_pgs, o_half, o_pinv, o_pinvs, o_pmod, o_mk, o_mks;
      int KW = 0;
      if (K > 0) {
        for (int k = 0; k < K; ++k)
          for (int t = 0; t < K; ++t) blob.push_back(t < k ? invmod_h(pm[t] % pm[k], pm[k]) : 0);
        o_pgs = blob.size();
        for (int k = 0; k < K; ++k)
          for (int t = 0; t < K; ++t) blob.push_back(shoup_h(blob[k * K + t], pm[k]));
        BigU Pb = product(pm, 0, K);
        KW = (int)Pb.w.size();
        o_half = blob.size();
        auto hw = Pb.shr1().words(8);
        blob.insert(blob.end(), hw.begin(), hw.end());
        o_pinv = blob.size();
        for (int i = 0; i < L; ++i) blob.push_back(invmod_h(Pb.mod_u64(qm[i]), qm[i]));
        o_pinvs = blob.size();
        for (int i = 0; i < L; ++i) blob.push_back(shoup_h(blob[o_pinv + i], qm[i]));
        o_pmod = blob.size();
        for (int i = 0; i < L; ++i) blob.push_back(Pb.mod_u64(qm[i]));
        o_mk = blob.size();
        for (int i = 0; i < L; ++i)
          for (int k = 0; k < K; ++k) blob.push_back(product(pm, 0, k).mod_u64(qm[i]));
        o_mks = blob.size();
        for (int i = 0; i < L; ++i)
          for (int k = 0; k < K; ++k) blob.push_back(shoup_h(blob[o_mk + (size_t)i * K + k], qm[i]));
        c->md_buf.reset(new DevBuf(blob.size() * 8));
        uint64_t* d = (uint64_t*)c->md_buf->p;
        cuda_check(cudaMemcpy(d, blob.data(), blob.size() * 8, cudaMemcpyHostToDevice), "upload moddown tables");
        c->md.p_garner = d + o_pg;
        c->md.p_garner_s = d + o_pgs;
        c->md.halfP = d + o_half;
        c->md.KW = KW;
        c->md.pinv = d + o_pinv;
        c->md.pinv_s = d + o_pinvs;
        c->md.pmod = d + o_pmod;
        c->md.mk = d + o_mk;
        c->md.mk_s = d + o_mks;
      }
    }
    // ---- rescale tables: inv[l*L + i] = q_l^-1 mod q_i (i < l)
    {
      const int L = c->L;
      std::vector<uint64_t> blob((size_t)2 * L * L, 0);
      for (int l = 0; l < L; ++l)
        for (int i = 0; i < l; ++i) {
          uint64_t v = invmod_h(qm[l] % qm[i], qm[i]);
          blob[(size_t)l * L + i] = v;
          blob[(size_t)L * L + (size_t)l * L + i] = shoup_h(v, qm[i]);
        }
      c->rt_buf.reset(new DevBuf(blob.size() * 8));
      uint64_t* d = (uint64_t*)c->rt_buf->p;
      cuda_check(cudaMemcpy(d, blob.data(), blob.size() * 8, cudaMemcpyHostToDevice), "upload rescale tables");
      c->rt.inv = d;
      c->rt.inv_s = d + (size_t)L * L;
    }
    // ---- internal primes of the exact key product: the four largest w = k * 2^17 + 1 < 2^29
    // (w = 1 mod 2N for every N <= 2^16), with twiddle tables for the pairs (w0, w1), (w2, w3)
    {
      std::vector<uint64_t> w;
      for (uint64_t k = ((1ull << 29) - 2) >> 17; k > 0 && w.size() < 4; --k)
        if (is_prime_u64((k << 17) + 1)) w.push_back((k << 17) + 1);
      c->wide_ok = w.size() == 4 && c->log_n >= 12 && c->log_n <= 16;
      if (const char* e = getenv("RNSCKKS_WIDE")) c->wide_ok = c->wide_ok && atoi(e) != 0;
      if (c->wide_ok) {
        WidePrimes& wp = c->wp;
        wp.log_n = c->log_n;
        auto shoup32 = [](uint64_t x, uint64_t q) { return (uint32_t)((x << 32) / q); };
        std::vector<Tw2> tf((size_t)2 * N), ti((size_t)2 * N);
        for (int i = 0; i < 4; ++i) {
          const uint64_t q = w[i];
          wp.q[i] = (uint32_t)q;
          // N^-1 2^32: the key product's Montgomery outputs carry 2^-32 (WidePrimes)
          wp.n_inv[i] = (uint32_t)mulmod_h(invmod_h(N % q, q), (1ull << 32) % q, q);
          wp.n_inv_s[i] = shoup32(wp.n_inv[i], q);
          wp.bar[i] = (~0ull) / q;
          uint32_t qi = (uint32_t)q;  // Newton iteration for q^-1 mod 2^32
          for (int it = 0; it < 5; ++it) qi *= 2u - (uint32_t)q * qi;
          wp.qinv_neg[i] = 0u - qi;
          wp.kq[i] = (uint32_t)(((1ull << 31) / q) * q);
          uint64_t psi = 0;  // any primitive 2N-th root of unity (these primes never meet user data)
          for (uint64_t x = 2; x < 100000 && !psi; ++x) {
            const uint64_t cand = powmod_h(x, (q - 1) / (2 * N), q);
            if (powmod_h(cand, N, q) == q - 1) psi = cand;
          }
          require(psi != 0, "internal: no root of unity for an internal prime");
          const uint64_t psi_inv = invmod_h(psi, q);
          std::vector<uint64_t> pw(N), pwi(N);
          pw[0] = pwi[0] = 1;
          for (uint64_t e = 1; e < N; ++e) {
            pw[e] = mulmod_h(pw[e - 1], psi, q);
            pwi[e] = mulmod_h(pwi[e - 1], psi_inv, q);
          }
          const int pair = i >> 1, half = i & 1;
          // the inverse transform's last stage (its one twiddle, psi^-bitrev(1)) times N^-1 (InvScale2)
          wp.w1n[i] = (uint32_t)mulmod_h(pwi[bitrev(1, c->log_n)], wp.n_inv[i], q);
          wp.w1n_s[i] = shoup32(wp.w1n[i], q);
          for (uint64_t kk = 0; kk < N; ++kk) {
            const int e = bitrev((int)kk, c->log_n);
            Tw2& f = tf[(size_t)pair * N + kk];
            Tw2& g = ti[(size_t)pair * N + kk];
            (half ? f.w1 : f.w0) = (uint32_t)pw[e];
            (half ? f.s1 : f.s0) = shoup32(pw[e], q);
            (half ? g.w1 : g.w0) = (uint32_t)pwi[e];
            (half ? g.s1 : g.s0) = shoup32(pwi[e], q);
          }
        }
        c->wide_tw.reset(new DevBuf(sizeof(Tw2) * 4 * N));
        Tw2* dtw = (Tw2*)c->wide_tw->p;
        cuda_check(cudaMemcpy(dtw, tf.data(), sizeof(Tw2) * 2 * N, cudaMemcpyHostToDevice), "upload wide tw");
        cuda_check(cudaMemcpy(dtw + 2 * N, ti.data(), sizeof(Tw2) * 2 * N, cudaMemcpyHostToDevice), "upload wide tw");
        wp.tw_fwd = dtw;
        wp.tw_inv = dtw + 2 * N;
        // Garner constants and, per scheme prime t, (w0 w1) mod t and A mod t
        WideTab& W = c->wide;
        for (int i = 0; i < 4; ++i) W.w[i] = (uint32_t)w[i];
        auto inv_pair = [&](int a, int m, uint32_t& g, uint32_t& gs) {
          g = (uint32_t)invmod_h(w[a] % w[m], w[m]);
          gs = shoup32(g, w[m]);
        };
        inv_pair(0, 1, W.g01, W.g01s);
        inv_pair(0, 2, W.g02, W.g02s);
        inv_pair(1, 2, W.g12, W.g12s);
        inv_pair(0, 3, W.g03, W.g03s);
        inv_pair(1, 3, W.g13, W.g13s);
        inv_pair(2, 3, W.g23, W.g23s);
        W.half3 = (uint32_t)((w[3] + 1) / 2);
        const int QP = c->L + c->K;
        const u128h A = (u128h)w[0] * w[1] * w[2] * w[3];
        std::vector<uint64_t> blob((size_t)3 * QP);
        for (int t = 0; t < QP; ++t) {
          const uint64_t m = c->mod[t];
          const uint64_t c01 = (uint64_t)(((u128h)w[0] * w[1]) % m);
          blob[t] = c01;
          blob[QP + t] = shoup_h(c01, m);
          blob[2 * QP + t] = (uint64_t)(A % m);
        }
        // the Q primes' constants times P^-1 (ModDown folded into the CRT): c01p[L], c01p_s[L], ap[L],
        // mkp[L][K], mkp_s[L][K]
        const size_t o_fold = blob.size();
        const int L = c->L, K = c->K;
        if (K > 0) {
          std::vector<uint64_t> pinv(L), c01p(L), c01ps(L), ap(L), mkp((size_t)L * K), mkps((size_t)L * K);
          for (int i = 0; i < L; ++i) {
            const uint64_t m = c->mod[i];
            uint64_t pm = 1 % m;
            for (int k = 0; k < K; ++k) pm = mulmod_h(pm, c->mod[L + k] % m, m);
            pinv[i] = invmod_h(pm, m);
            c01p[i] = mulmod_h(blob[i], pinv[i], m);
            c01ps[i] = shoup_h(c01p[i], m);
            ap[i] = mulmod_h(blob[2 * QP + i], pinv[i], m);
            uint64_t mk = 1 % m;  // M_k = p_0 ... p_{k-1}
            for (int k = 0; k < K; ++k) {
              mkp[(size_t)i * K + k] = mulmod_h(mk, pinv[i], m);
              mkps[(size_t)i * K + k] = shoup_h(mkp[(size_t)i * K + k], m);
              mk = mulmod_h(mk, c->mod[L + k] % m, m);
            }
          }
          for (auto* v : {&c01p, &c01ps, &ap, &mkp, &mkps}) blob.insert(blob.end(), v->begin(), v->end());
        }
        c->wide_buf.reset(new DevBuf(blob.size() * 8));
        uint64_t* d = (uint64_t*)c->wide_buf->p;
        cuda_check(cudaMemcpy(d, blob.data(), blob.size() * 8, cudaMemcpyHostToDevice), "upload wide tables");
        W.c01_mod_t = d;
        W.c01_mod_t_s = d + QP;
        W.A_mod_t = d + 2 * QP;
        if (K > 0) {
          W.c01p = d + o_fold;
          W.c01p_s = W.c01p + L;
          W.ap = W.c01p_s + L;
          W.mkp = W.ap + L;
          W.mkp_s = W.mkp + (size_t)L * K;
        } else {
          W.c01p = W.c01p_s = W.ap = W.mkp = W.mkp_s = nullptr;
        }
      }
    }
    cuda_check(cudaDeviceSynchronize(), "context setup");
    *out = c.release();
  });
}

extern "C" void rc_context_destroy(rc_context* ctx) {
  if (!ctx) return;
  cudaDeviceSynchronize();
  delete ctx;
}

extern "C" const char* rc_last_error(const rc_context*) { return g_err.c_str(); }

extern "C" int rc_kernel_errors(int32_t* flags, int32_t clear) {
  return guarded("rc_kernel_errors", [&] {
    require(flags != nullptr, "arguments must not be null");
    *flags = wide_kernel_errors(clear != 0);
  });
}

extern "C" int rc_context_info(const rc_context* c, uint64_t* n, uint32_t* levels, uint32_t* aux, uint32_t* sb) {
  return guarded("rc_context_info", [&] {
    require(c != nullptr, "context must not be null");
    if (n) *n = (uint64_t)c->N;
    if (levels) *levels = (uint32_t)c->L;
    if (aux) *aux = (uint32_t)c->K;
    if (sb) *sb = (uint32_t)c->scale_bits;
  });
}

extern "C" int rc_decomp_digits(const rc_context* c, int32_t level, uint32_t* digits) {
  return guarded("rc_decomp_digits", [&] {
    require(c != nullptr && digits != nullptr, "arguments must not be null");
    *digits = (uint32_t)level_info(c, level + 1).digits;
  });
}

extern "C" int rc_tune_set(rc_context* c, const char* name, int32_t value) {
  return guarded("rc_tune_set", [&] {
    require(c && name, "arguments must not be null");
    const std::string n(name);
    if (n == "ks_jobs") {
      require(value >= 1 && value <= MAXP / 2, "ks_jobs must be in 1.." + std::to_string(MAXP / 2));
      c->ks_jobs = value;
    } else if (n == "mac_bc") {
      require(value == 1 || value == 2 || value == 4 || value == 8, "mac_bc must be 1, 2, 4 or 8");
      c->mac_bc = value;
    } else if (n == "host_chunk") {
      require(value >= 1, "host_chunk must be positive");
      c->host_chunk = value;
    } else if (n == "host_edge") {
      require(value >= 1, "host_edge must be positive");
      c->host_edge = value;
    } else if (n == "fuse_tensor") {
      c->fuse_tensor = value != 0;
    } else if (n == "host_phased") {
      require(value >= 0 && value <= 2, "host_phased must be 0, 1 or 2");
      c->host_phased = value;
    } else if (n == "ntt_split") {
      const int n2 = c->log_n - value;
      require(c->log_n >= 12 && c->log_n <= 16 && value >= 6 && value <= 8 && n2 >= 6 && n2 <= 8,
              "ntt_split must leave both four-step phases between 2^6 and 2^8 points (log N 12..16)");
      c->n1 = value;
    } else if (n == "col_ctas") {
      require(value == 2 || value == 3, "col_ctas must be 2 or 3");
      c->col_ctas = value;
    } else if (n == "tensor_jobs") {
      require(value >= 1 && value <= 16, "tensor_jobs must be in 1..16");
      c->tensor_jobs = value;
    } else if (n == "row_polys") {
      require(value == 8 || value == 16, "row_polys must be 8 or 16");
      c->row_polys = value;
    } else if (n == "mixed_levels") {
      c->mixed_levels = value != 0;
    } else if (n == "ml_jobs") {
      require(value >= 1 && value <= ML_MAXJ, "ml_jobs must be in 1.." + std::to_string(ML_MAXJ));
      c->ml_jobs = value;
    } else if (n == "mac_wait_polls") {
      require(value >= 0 && value <= (1 << 22), "mac_wait_polls must be in 0..4194304");
      c->wp.first_wait_polls = (uint32_t)value;
    } else if (n == "mac_persistent") {
      c->wp.persistent = value != 0;
    } else if (n == "ntt_r16") {
      require(value >= 0 && value <= r16::R16_ALL, "ntt_r16 must be a set of pass bits in 0..63");
      c->r16 = value;
      c->wp.r16 = value;
    } else if (n == "lazy_ntt") {
      bool ok = true;
      for (uint64_t q : c->mod) ok = ok && q < (1ull << 57);
      require(!value || ok, "lazy_ntt needs every prime below 2^57");
      c->lazy = value != 0;
    } else {
      fail(RC_ERR_INVALID_ARGUMENT, "unknown tunable " + n);
    }
  });
}

extern "C" int rc_tune_get(const rc_context* c, const char* name, int32_t* value) {
  return guarded("rc_tune_get", [&] {
    require(c && name && value, "arguments must not be null");
    const std::string n(name);
    if (n == "ks_jobs") *value = c->ks_jobs;
    else if (n == "mac_bc") *value = c->mac_bc;
    else if (n == "host_chunk") *value = c->host_chunk;
    else if (n == "host_edge") *value = c->host_edge;
    else if (n == "lazy_ntt") *value = c->lazy ? 1 : 0;
    else if (n == "fuse_tensor") *value = c->fuse_tensor ? 1 : 0;
    else if (n == "host_phased") *value = c->host_phased;
    else if (n == "mac_wait_polls") *value = (int32_t)c->wp.first_wait_polls;
    else if (n == "mac_persistent") *value = c->wp.persistent ? 1 : 0;
    else if (n == "mixed_levels") *value = c->mixed_levels ? 1 : 0;
    else if (n == "ntt_split") *value = c->n1;
    else if (n == "col_ctas") *value = c->col_ctas;
    else if (n == "row_polys") *value = c->row_polys;
    else if (n == "tensor_jobs") *value = c->tensor_jobs;
    else if (n == "ntt_r16") *value = c->r16;
    else if (n == "ml_jobs") *value = c->ml_jobs;
    else fail(RC_ERR_INVALID_ARGUMENT, "unknown tunable " + n);
  });
}

extern "C" int rc_reserve(rc_context* c, int32_t max_level, uint32_t max_batch, void* stream) {
  return guarded("rc_reserve", [&] {
    require(c != nullptr, "context must not be null");
    const int limbs = max_level + 1;
    const LevelInfo& li = level_info(c, limbs);
    const int J = (int)std::min<uint32_t>(max_batch ? max_batch : 1, (uint32_t)c->ks_jobs);
    const int D = li.digits + 4;
    const size_t pl = (size_t)limbs * c->N;
    size_t need = align_up(std::max(ks_ws_bytes(c, J, limbs, c->K, D), tensor_ws_bytes(c, std::min(J, MAXP / 4), limbs)),
                           256) +
                  arena_size_u64((size_t)3 * J * pl) + 256;
    // a mixed-level chunk of up to ml_jobs jobs, each at most at max_level (digits with the same headroom)
    if (c->wide_ok) {
      const int JM = (int)std::min<uint32_t>(max_batch ? max_batch : 1, (uint32_t)c->ml_jobs);
      const size_t N = c->N;
      const size_t dig = (size_t)JM * D, acc = (size_t)JM * 2 * (limbs + c->K);
      need = std::max(need, align_up(dig * N * 4, 256) + 2 * arena_size_u64(dig * 2 * N) +
                                arena_size_u64(acc * 2 * N) + 1024);
    }
    ws_device(c, S(stream), need);
  });
}

// =========================================================================
// keys
// =========================================================================
static int ksk_upload_impl(rc_context* c, const uint64_t* key, bool on_device, uint32_t digits, int32_t level,
                           uint32_t aux_count, uint64_t galois_element, rc_ksk** out) {
  return guarded([&] {
    require(c && key && out, "arguments must not be null");
    *out = nullptr;
    require(level >= 0 && level < c->L, "keyswitch key level out of range for this context");
    require(aux_count == 0 || (int)aux_count == c->K, "eval-key context must match the keyswitch key auxiliary basis");
    require(digits >= 1, "keyswitch key must have at least one digit");
    if (galois_element) galois_inverse(c, galois_element);
    const int limbs = level + 1 + (int)aux_count;
    const size_t elems = (size_t)digits * 2 * limbs * c->N;
    DevBuf tmp(elems * 8);
    cuda_check(cudaMemcpy(tmp.p, key, elems * 8, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice),
               "key upload");
    const LimbMap map{level + 1, c->L};
    uint64_t* t = (uint64_t*)tmp.p;
    // wide form (exact integer key product) when it applies at the key's level: the same integers under
    // the internal primes, transformed and tiled; it then replaces the per-limb form, which is built
    // otherwise.  Q-only keys truncated to fewer levels keep qualifying (smaller q_max, same digits).
    const int Kk = aux_count ? c->K : 0;
    const int Dk = aux_count ? level_info(c, level + 1).digits : (int)digits;
    std::shared_ptr<DevBuf> wide, fin;
    if (wide_applies(c, level + 1, Kk, Dk)) {
      const size_t welems = elems * 2;  // two uint2 pairs per coefficient
      DevBuf wtmp(welems * 8);
      wide.reset(new DevBuf(welems * 8));
      require(wide_key_build(c->wp, t, (int)digits, limbs, (uint2*)wtmp.p, (uint2*)wide->p, 0),
              "internal: wide transforms unsupported");
      launch_check("wide key");
      cuda_check(cudaDeviceSynchronize(), "wide key");
    } else {
      fin.reset(new DevBuf(elems * 8));
      const int polys = (int)digits * 2;
      for (int p0 = 0; p0 < polys; p0 += MAXP) {
        PtrTab tab{};
        const int cnt = std::min(MAXP, polys - p0);
        for (int k = 0; k < cnt; ++k) tab.p[k] = t + (size_t)(p0 + k) * limbs * c->N;
        ntt_forward(c->ntt(), tab, tab, cnt, limbs, map, 0);
        launch_check("key ntt");
      }
      key_to_device_form(c->ntt(), c->d_pc, t, (uint64_t*)fin->p, (int)digits, limbs, map, c->N, 0);
      launch_check("key relayout");
      cuda_check(cudaDeviceSynchronize(), "key upload");
    }
    rc_ksk* k = new rc_ksk();
    k->ctx = c;
    k->buf = fin;
    k->data = fin ? (uint64_t*)fin->p : nullptr;
    k->wbuf = wide;
    k->wdata = wide ? (uint64_t*)wide->p : nullptr;
    k->digits = digits;
    k->level = level;
    k->aux = aux_count;
    k->galois = galois_element;
    *out = k;
  });
}

extern "C" int rc_ksk_upload(rc_context* c, const uint64_t* host_key, uint32_t digits, int32_t level,
                             uint32_t aux_count, uint64_t galois_element, rc_ksk** out) {
  OpRange op_range("rc_ksk_upload");
  return ksk_upload_impl(c, host_key, false, digits, level, aux_count, galois_element, out);
}

extern "C" int rc_ksk_upload_device(rc_context* c, const uint64_t* dev_key, uint32_t digits, int32_t level,
                                    uint32_t aux_count, uint64_t galois_element, rc_ksk** out) {
  OpRange op_range("rc_ksk_upload_device");
  return ksk_upload_impl(c, dev_key, true, digits, level, aux_count, galois_element, out);
}

// RNS-hybrid ("dnum") relinearization key: no counterpart in the reference (its gadget is base 2^30 digits).
extern "C" int rc_ksk_upload_dnum(rc_context* c, const uint64_t* key, int32_t key_on_device, uint32_t alpha,
                                  int32_t level, rc_ksk** out) {
  return guarded("rc_ksk_upload_dnum", [&] {
    require(c && key && out, "arguments must not be null");
    *out = nullptr;
    require(c->K > 0, "RNS-hybrid keys need an auxiliary basis");
    require(level >= 0 && level < c->L, "keyswitch key level out of range for this context");
    require(alpha >= 1 && (int)alpha <= std::min(c->K, 8),
            "alpha must be between 1 and the number of aux primes (at most 8)");
    for (uint64_t m : c->mod) require(m < (1ull << 60), "RNS-hybrid keys need every prime below 2^60");
    const int qlimbs = level + 1, K = c->K, total = qlimbs + K;
    const int dnum = (qlimbs + (int)alpha - 1) / (int)alpha;
    require(dnum <= 16, "RNS-hybrid keys take at most 16 groups");
    const size_t N = c->N, per = (size_t)total * N;
    std::shared_ptr<DevBuf> kb(new DevBuf((size_t)dnum * 2 * per * 8));
    uint64_t* kd = (uint64_t*)kb->p;
    cuda_check(cudaMemcpy(kd, key, (size_t)dnum * 2 * per * 8,
                          key_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice),
               "key upload");
    const LimbMap map{qlimbs, c->L};
    for (int p0 = 0; p0 < 2 * dnum; p0 += MAXP) {
      PtrTab t{};
      const int cnt = std::min(MAXP, 2 * dnum - p0);
      for (int k = 0; k < cnt; ++k) t.p[k] = kd + (size_t)(p0 + k) * per;
      ntt_forward(c->ntt(), t, t, cnt, total, map, 0);
      launch_check("key ntt");
    }
    // ModUp tables per group b: (Q_b/q_i)^-1 mod q_i (+ Shoup), then (Q_b/q_i) mod every target prime
    const int row = 2 + total;
    std::vector<uint64_t> tab((size_t)dnum * alpha * row, 0);
    for (int b = 0; b < dnum; ++b) {
      const int i0 = b * (int)alpha, i1 = std::min(i0 + (int)alpha, qlimbs);
      const BigU Qb = product(c->mod, (size_t)i0, (size_t)i1);
      for (int i = i0; i < i1; ++i) {
        const uint64_t q = c->mod[i];
        const BigU hat = Qb.div_u64(q);
        uint64_t* r = tab.data() + ((size_t)b * alpha + (i - i0)) * row;
        r[0] = invmod_h(hat.mod_u64(q), q);
        r[1] = shoup_h(r[0], q);
        for (int t = 0; t < total; ++t) r[2 + t] = hat.mod_u64(c->mod[map.prime(t)]);
      }
    }
    std::shared_ptr<DevBuf> mb(new DevBuf(tab.size() * 8));
    cuda_check(cudaMemcpy(mb->p, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice), "key tables");
    cuda_check(cudaDeviceSynchronize(), "key upload");
    rc_ksk* k = new rc_ksk();
    k->ctx = c;
    k->buf = kb;
    k->data = kd;
    k->digits = (uint32_t)dnum;
    k->level = level;
    k->aux = (uint32_t)K;
    k->galois = 0;
    k->alpha = alpha;
    k->mbuf = mb;
    *out = k;
  });
}

extern "C" int rc_ksk_truncate(rc_context* c, const rc_ksk* key, int32_t level, rc_ksk** out) {
  return guarded("rc_ksk_truncate", [&] {
    require(c && key && out, "arguments must not be null");
    // RnsKeySwitchingKey::truncate_levels / drop_last_level, keyswitching.rs:21-41
    require(level + 1 > 0, "level_count must be positive");
    require(level <= key->level, "level_count cannot exceed keyswitch levels");
    require(level == key->level || key->aux == 0, "dropping levels is only supported for Q-only keyswitch keys");
    rc_ksk* k = new rc_ksk(*key);
    k->level = level;  // limb-major layout: the first level+1 limbs are the truncated key
    *out = k;
  });
}

extern "C" int rc_ksk_info(const rc_ksk* k, uint32_t* digits, int32_t* level, uint32_t* aux, uint64_t* g) {
  if (!k) return RC_ERR_INVALID_ARGUMENT;
  if (digits) *digits = k->digits;
  if (level) *level = k->level;
  if (aux) *aux = k->aux;
  if (g) *g = k->galois;
  return RC_OK;
}

extern "C" void rc_ksk_destroy(rc_ksk* k) { delete k; }

// =========================================================================
// polynomial ops
// =========================================================================
static int ntt_entry(rc_context* c, uint64_t* data, uint32_t polys, uint32_t limbs, int32_t with_aux, void* stream,
                     bool forward) {
  return guarded([&] {
    require(c && data, "arguments must not be null");
    LimbMap map{(int)limbs, c->L};
    if (with_aux) {
      require((int)limbs > c->K && (int)limbs - c->K <= c->L, "limb count out of range for the extended basis");
      map.qcount = (int)limbs - c->K;
    } else {
      require(limbs >= 1 && (int)limbs <= c->L, "limb count out of range for this context");
    }
    for (uint32_t p0 = 0; p0 < polys; p0 += MAXP) {
      const int cnt = (int)std::min<uint32_t>(MAXP, polys - p0);
      PtrTab t{};
      for (int k = 0; k < cnt; ++k) t.p[k] = data + (size_t)(p0 + k) * limbs * c->N;
      if (forward) ntt_forward(c->ntt(), t, t, cnt, (int)limbs, map, S(stream));
      else ntt_inverse(c->ntt(), t, t, cnt, (int)limbs, map, S(stream));
      launch_check("ntt");
    }
  });
}

extern "C" int rc_ntt_forward(rc_context* c, uint64_t* d, uint32_t polys, uint32_t limbs, int32_t aux, void* s) {
  OpRange op_range("rc_ntt_forward");
  return ntt_entry(c, d, polys, limbs, aux, s, true);
}
extern "C" int rc_ntt_inverse(rc_context* c, uint64_t* d, uint32_t polys, uint32_t limbs, int32_t aux, void* s) {
  OpRange op_range("rc_ntt_inverse");
  return ntt_entry(c, d, polys, limbs, aux, s, false);
}

static LimbMap basis_map(const rc_context* c, uint32_t limbs, int32_t with_aux) {
  if (with_aux) {
    require(c->K > 0, "eval-key level context requires an auxiliary basis");
    require((int)limbs > c->K && (int)limbs - c->K <= c->L, "limb count out of range for the extended basis");
    return LimbMap{(int)limbs - c->K, c->L};
  }
  require(limbs >= 1 && (int)limbs <= c->L, "context level count must match polynomial levels");
  return LimbMap{(int)limbs, c->L};
}

LimbMap rc::context_basis_map(const rc_context* c, uint32_t limbs, int32_t with_aux) {
  return basis_map(c, limbs, with_aux);
}

void* rc::context_workspace(rc_context* c, cudaStream_t s, size_t bytes) { return ws_device(c, s, bytes); }

extern "C" int rc_poly_multiply(rc_context* c, const uint64_t* a, const uint64_t* b, uint64_t* out, uint32_t limbs,
                                int32_t with_aux, void* stream) {
  return guarded("rc_poly_multiply", [&] {
    require(c && a && b && out, "arguments must not be null");
    const LimbMap map = basis_map(c, limbs, with_aux);
    cudaStream_t s = S(stream);
    const size_t pl = (size_t)limbs * c->N;
    Arena ar(ws_device(c, s, 2 * arena_size_u64(pl) + 512));
    uint64_t* ta = ar.take<uint64_t>(pl);
    uint64_t* tb = ar.take<uint64_t>(pl);
    PtrTab src{}, dst{};
    src.p[0] = const_cast<uint64_t*>(a);
    src.p[1] = const_cast<uint64_t*>(b);
    dst.p[0] = ta;
    dst.p[1] = tb;
    ntt_forward(c->ntt(), src, dst, 2, (int)limbs, map, s);
    PtrTab x{}, y{};
    x.p[0] = ta;
    y.p[0] = tb;
    ew_binary(EwOp::MulMont, c->d_pc, x, y, 0, x, 1, (int)limbs, map, c->N, s);
    PtrTab o{};
    o.p[0] = out;
    NttArgs inv = c->ntt();
    inv.mont_out = 1;  // takes out the Montgomery products' 2^-64
    ntt_inverse(inv, x, o, 1, (int)limbs, map, s);
    launch_check("poly_multiply");
  });
}

static int poly_binary(rc_context* c, const uint64_t* a, const uint64_t* b, uint64_t* out, uint32_t limbs,
                       int32_t with_aux, void* stream, EwOp op) {
  return guarded([&] {
    require(c && a && b && out, "arguments must not be null");
    const LimbMap map = basis_map(c, limbs, with_aux);
    PtrTab x{}, y{}, o{};
    x.p[0] = const_cast<uint64_t*>(a);
    y.p[0] = const_cast<uint64_t*>(b);
    o.p[0] = out;
    ew_binary(op, c->d_pc, x, y, 0, o, 1, (int)limbs, map, c->N, S(stream));
    launch_check("poly add/sub");
  });
}
extern "C" int rc_poly_add(rc_context* c, const uint64_t* a, const uint64_t* b, uint64_t* o, uint32_t l,
                           int32_t aux, void* s) {
  OpRange op_range("rc_poly_add");
  return poly_binary(c, a, b, o, l, aux, s, EwOp::Add);
}
extern "C" int rc_poly_sub(rc_context* c, const uint64_t* a, const uint64_t* b, uint64_t* o, uint32_t l,
                           int32_t aux, void* s) {
  OpRange op_range("rc_poly_sub");
  return poly_binary(c, a, b, o, l, aux, s, EwOp::Sub);
}

extern "C" int rc_poly_mul_scalar(rc_context* c, const uint64_t* a, const uint64_t* scalars, uint64_t* out,
                                  uint32_t limbs, int32_t with_aux, void* stream) {
  return guarded("rc_poly_mul_scalar", [&] {
    require(c && a && scalars && out, "arguments must not be null");
    const LimbMap map = basis_map(c, limbs, with_aux);
    ScalarTab st{};
    require(limbs <= (uint32_t)(sizeof(st.v) / sizeof(st.v[0])), "too many limbs for a scalar product");
    for (uint32_t j = 0; j < limbs; ++j) st.v[j] = scalars[j] % c->mod[map.prime((int)j)];
    mul_scalar(c->d_pc, a, st, out, (int)limbs, map, c->N, S(stream));
    launch_check("poly_mul_scalar");
  });
}

extern "C" int rc_poly_automorphism(rc_context* c, const uint64_t* a, uint64_t* out, uint32_t limbs, uint64_t g,
                                    void* stream) {
  return guarded("rc_poly_automorphism", [&] {
    require(c && a && out, "arguments must not be null");
    require(limbs >= 1 && (int)limbs <= c->L, "limb count out of range for this context");
    require(a != out, "automorphism output must not alias its input");
    require(g < 2ull * c->N, "galois element must be reduced modulo 2N");
    const uint64_t gi = galois_inverse(c, g);
    PtrTab x{}, o{};
    x.p[0] = const_cast<uint64_t*>(a);
    o.p[0] = out;
    automorphism(c->d_pc, x, o, 1, (int)limbs, gi, c->log_n, S(stream));
    launch_check("automorphism");
  });
}

// =========================================================================
// ciphertext ops
// =========================================================================
extern "C" int rc_add(rc_context* c, const rc_ciphertext* a, const rc_ciphertext* b, rc_ciphertext* out,
                      void* stream) {
  return guarded("rc_add", [&] {
    require(c && out && out->data, "arguments must not be null");
    check_ct(c, a, "lhs");
    check_ct(c, b, "rhs");
    // RnsCiphertext::add, ciphertexts.rs:60-62
    require(a->scale_bits == b->scale_bits, "ciphertexts must share the same scale to add");
    require(a->level == b->level, "ciphertexts must be at the same level to add");
    const int limbs = a->level + 1;
    const size_t pl = (size_t)limbs * c->N;
    PtrTab x{}, y{}, o{};
    for (int k = 0; k < 2; ++k) {
      x.p[k] = a->data + k * pl;
      y.p[k] = b->data + k * pl;
      o.p[k] = out->data + k * pl;
    }
    ew_binary(EwOp::Add, c->d_pc, x, y, 0, o, 2, limbs, qmap(c, limbs), c->N, S(stream));
    launch_check("add");
    out->level = a->level;
    out->scale_bits = a->scale_bits;
  });
}

// Batched forms of add and multiply_plain_rns: `count` independent jobs in one call (the Python-side
// algorithms and the server issue one call per step of a batch instead of one per job).
extern "C" int rc_add_batch(rc_context* c, uint32_t count, const rc_ciphertext* a, const rc_ciphertext* b,
                            rc_ciphertext* out, void* stream) {
  return guarded("rc_add_batch", [&] {
    require(c && a && b && out, "arguments must not be null");
    // jobs of one level go out in launches of up to MAXP/2 ciphertexts (two components each)
    std::map<int, std::vector<uint32_t>> by_level;
    for (uint32_t i = 0; i < count; ++i) {
      require(out[i].data != nullptr, "arguments must not be null");
      check_ct(c, &a[i], "lhs");
      check_ct(c, &b[i], "rhs");
      require(a[i].scale_bits == b[i].scale_bits, "ciphertexts must share the same scale to add");
      require(a[i].level == b[i].level, "ciphertexts must be at the same level to add");
      by_level[a[i].level].push_back(i);
    }
    for (auto& g : by_level) {
      const int limbs = g.first + 1;
      const size_t pl = (size_t)limbs * c->N;
      for (size_t b0 = 0; b0 < g.second.size(); b0 += MAXP / 2) {
        PtrTab x{}, y{}, o{};
        int polys = 0;
        for (size_t k = b0; k < g.second.size() && k < b0 + MAXP / 2; ++k) {
          const uint32_t i = g.second[k];
          for (int comp = 0; comp < 2; ++comp, ++polys) {
            x.p[polys] = a[i].data + comp * pl;
            y.p[polys] = b[i].data + comp * pl;
            o.p[polys] = out[i].data + comp * pl;
          }
          out[i].level = a[i].level;
          out[i].scale_bits = a[i].scale_bits;
        }
        ew_binary(EwOp::Add, c->d_pc, x, y, 0, o, polys, limbs, qmap(c, limbs), c->N, S(stream));
        launch_check("add_batch");
      }
    }
  });
}

static void mult_plain_impl(rc_context* c, const rc_ciphertext* ct, const uint64_t* plain, rc_ciphertext* out,
                            cudaStream_t s) {
  require(c && out && out->data && plain, "arguments must not be null");
  check_ct(c, ct, "ciphertext");
  const int limbs = ct->level + 1;
  const size_t pl = (size_t)limbs * c->N;
  Arena ar(ws_device(c, s, 3 * arena_size_u64(pl) + 1024));
  uint64_t* f = ar.take<uint64_t>(3 * pl);
  PtrTab src{}, dst{};
  src.p[0] = ct->data;
  src.p[1] = ct->data + pl;
  src.p[2] = const_cast<uint64_t*>(plain);
  for (int k = 0; k < 3; ++k) dst.p[k] = f + k * pl;
  ntt_forward(c->ntt(), src, dst, 3, limbs, qmap(c, limbs), s);
  PtrTab a{}, b{};
  a.p[0] = f;
  a.p[1] = f + pl;
  b.p[0] = f + 2 * pl;
  ew_binary(EwOp::MulMont, c->d_pc, a, b, 1, a, 2, limbs, qmap(c, limbs), c->N, s);
  PtrTab o{};
  o.p[0] = out->data;
  o.p[1] = out->data + pl;
  NttArgs inv = c->ntt();
  inv.mont_out = 1;  // takes out the Montgomery products' 2^-64
  ntt_inverse(inv, a, o, 2, limbs, qmap(c, limbs), s);
  launch_check("mult_plain");
  out->level = ct->level;
}

extern "C" int rc_mult_plain(rc_context* c, const rc_ciphertext* ct, const uint64_t* plain, rc_ciphertext* out,
                             void* stream) {
  return guarded("rc_mult_plain", [&] {
    const int sb = ct ? ct->scale_bits : 0;
    mult_plain_impl(c, ct, plain, out, S(stream));
    out->scale_bits = sb + sb;  // context/ops.rs:24-29
  });
}

extern "C" int rc_multiply_plain_rns_batch(rc_context* c, uint32_t count, const rc_ciphertext* ct,
                                           const uint64_t* const* plains, rc_ciphertext* out, void* stream) {
  return guarded("rc_multiply_plain_rns_batch", [&] {
    require(c && ct && plains && out, "arguments must not be null");
    for (uint32_t i = 0; i < count; ++i) {
      const int sb = ct[i].scale_bits;
      mult_plain_impl(c, &ct[i], plains[i], &out[i], S(stream));
      out[i].scale_bits = sb;
    }
  });
}

extern "C" int rc_multiply_plain_rns(rc_context* c, const rc_ciphertext* ct, const uint64_t* plain,
                                     rc_ciphertext* out, void* stream) {
  return guarded("rc_multiply_plain_rns", [&] {
    const int sb = ct ? ct->scale_bits : 0;
    mult_plain_impl(c, ct, plain, out, S(stream));
    out->scale_bits = sb;
  });
}

extern "C" int rc_mult_plain_accumulate(rc_context* c, uint32_t count, const rc_ciphertext* cts, int32_t cts_ntt,
                                        const uint64_t* const* plains, int32_t plains_ntt, rc_ciphertext* out,
                                        void* stream) {
  return guarded("rc_mult_plain_accumulate", [&] {
    require(c && cts && plains && out && out->data, "arguments must not be null");
    require(count >= 1, "the inner sum needs at least one term");
    for (uint32_t k = 0; k < count; ++k) {
      check_ct(c, &cts[k], "ciphertext");
      require(plains[k] != nullptr, "arguments must not be null");
      require(cts[k].scale_bits == cts[0].scale_bits, "ciphertexts must share the same scale to add");
      require(cts[k].level == cts[0].level, "ciphertexts must be at the same level to add");
    }
    cudaStream_t s = S(stream);
    const int limbs = cts[0].level + 1;
    const size_t pl = (size_t)limbs * c->N;
    const LimbMap map = qmap(c, limbs);
    constexpr int CH = 16;  // terms per pass: bounds the scratch for coefficient-form inputs
    const int ct_buf = cts_ntt ? 0 : 2 * CH, pt_buf = plains_ntt ? 0 : CH;
    Arena ar(ws_device(c, s, arena_size_u64(2 * pl) + arena_size_u64((size_t)(ct_buf + pt_buf) * pl) + 1024));
    uint64_t* acc = ar.take<uint64_t>(2 * pl);
    uint64_t* tmp = (ct_buf + pt_buf) ? ar.take<uint64_t>((size_t)(ct_buf + pt_buf) * pl) : nullptr;
    for (uint32_t b = 0; b < count; b += CH) {
      const int J = (int)std::min<uint32_t>(CH, count - b);
      PtrTab ctab{}, ptab{};
      if (cts_ntt) {
        for (int j = 0; j < J; ++j) ctab.p[j] = cts[b + j].data;
      } else {
        PtrTab src{}, dst{};
        for (int j = 0; j < J; ++j) {
          src.p[2 * j] = cts[b + j].data;
          src.p[2 * j + 1] = cts[b + j].data + pl;
          dst.p[2 * j] = tmp + (size_t)2 * j * pl;
          dst.p[2 * j + 1] = tmp + (size_t)(2 * j + 1) * pl;
          ctab.p[j] = dst.p[2 * j];
        }
        ntt_forward(c->ntt(), src, dst, 2 * J, limbs, map, s);
      }
      if (plains_ntt) {
        for (int j = 0; j < J; ++j) ptab.p[j] = const_cast<uint64_t*>(plains[b + j]);
      } else {
        PtrTab src{}, dst{};
        for (int j = 0; j < J; ++j) {
          src.p[j] = const_cast<uint64_t*>(plains[b + j]);
          dst.p[j] = tmp + (size_t)(ct_buf + j) * pl;
          ptab.p[j] = dst.p[j];
        }
        ntt_forward(c->ntt(), src, dst, J, limbs, map, s);
      }
      plain_mac(c->d_pc, ctab, ptab, J, acc, b > 0, limbs, map, c->N, s);
    }
    PtrTab a{}, o{};
    a.p[0] = acc;
    a.p[1] = acc + pl;
    o.p[0] = out->data;
    o.p[1] = out->data + pl;
    ntt_inverse(c->ntt(), a, o, 2, limbs, map, s);
    launch_check("mult_plain_accumulate");
    out->level = cts[0].level;
    out->scale_bits = cts[0].scale_bits + cts[0].scale_bits;  // mult_plain, context/ops.rs:24-29
  });
}

extern "C" int rc_mult(rc_context* c, const rc_ciphertext* a, const rc_ciphertext* b, rc_ciphertext* out,
                       void* stream) {
  return guarded("rc_mult", [&] {
    require(c && out && out->data, "arguments must not be null");
    check_mult_pair(c, a, b);
    const int limbs = a->level + 1;
    void* ws = ws_device(c, S(stream), tensor_ws_bytes(c, 1, limbs));
    tensor_core(c, {a->data}, {b->data}, {out->data}, limbs, ws, S(stream));
    out->level = a->level;
    out->scale_bits = a->scale_bits + b->scale_bits;
  });
}

static void rescale_impl(rc_context* c, const rc_ciphertext* ct, rc_ciphertext* out, int comps, cudaStream_t s) {
  require(c && out && out->data, "arguments must not be null");
  check_ct(c, ct, "ciphertext");
  const int limbs = ct->level + 1;
  require(limbs > 1, comps == 3 ? "quadratic rescale requires at least two levels"
                                : "rescale requires at least two levels");
  require(out->data != ct->data, "rescale output must not alias its input");
  const size_t pl = (size_t)limbs * c->N, po = (size_t)(limbs - 1) * c->N;
  PtrTab in{}, o{};
  for (int k = 0; k < comps; ++k) {
    in.p[k] = ct->data + k * pl;
    o.p[k] = out->data + k * po;
  }
  rescale(c->d_pc, c->rt, c->L, in, o, comps, limbs, c->N, s);
  launch_check("rescale");
  const int sb = ct->scale_bits - floor_log2(c->mod[limbs - 1]);
  out->scale_bits = sb < 0 ? 0 : sb;  // saturating_sub, ops.rs:79
  out->level = ct->level - 1;
}

extern "C" int rc_rescale(rc_context* c, const rc_ciphertext* ct, rc_ciphertext* out, void* stream) {
  return guarded("rc_rescale", [&] { rescale_impl(c, ct, out, 2, S(stream)); });
}
extern "C" int rc_rescale_quadratic(rc_context* c, const rc_ciphertext* ct, rc_ciphertext* out, void* stream) {
  return guarded("rc_rescale_quadratic", [&] { rescale_impl(c, ct, out, 3, S(stream)); });
}
extern "C" int rc_rescale_batch(rc_context* c, uint32_t count, const rc_ciphertext* ct, rc_ciphertext* out,
                                void* stream) {
  return guarded("rc_rescale_batch", [&] {
    require(c && ct && out, "arguments must not be null");
    for (uint32_t i = 0; i < count; ++i) rescale_impl(c, &ct[i], &out[i], 2, S(stream));
  });
}

// lift_poly_to_context (keyswitching.rs:242-276) from Q_limbs to Q_limbs u P
static void lift_impl(rc_context* c, const uint64_t* a, uint64_t* out, uint32_t polys, uint32_t limbs,
                      cudaStream_t s) {
  require(c && a && out, "arguments must not be null");
  require(c->K > 0, "lifting requires an auxiliary evaluation basis");
  require(limbs >= 1 && (int)limbs <= c->L, "limb count out of range for this context");
  require(a != out, "lift output must not alias its input");
  lift_to_aux(c->d_pc, c->d_pc + c->L, level_info(c, (int)limbs).dt, a, out, (int)polys, (int)limbs, c->K,
              c->log_n, s);
  launch_check("lift");
}

extern "C" int rc_lift_to_aux(rc_context* c, const uint64_t* a, uint64_t* out, uint32_t polys, uint32_t limbs,
                              void* stream) {
  return guarded("rc_lift_to_aux", [&] { lift_impl(c, a, out, polys, limbs, S(stream)); });
}

extern "C" int rc_mod_raise(rc_context* c, const rc_ciphertext* ct, rc_ciphertext* out, void* stream) {
  return guarded("rc_mod_raise", [&] {
    require(c && out && out->data, "arguments must not be null");
    check_ct(c, ct, "ciphertext");
    lift_impl(c, ct->data, out->data, 2, (uint32_t)ct->level + 1, S(stream));
    out->level = ct->level + c->K;  // the eval-key context's levels - 1 (mod_raise.rs:40-44)
    out->scale_bits = ct->scale_bits;
  });
}

extern "C" int rc_keyswitch(rc_context* c, const uint64_t* poly, int32_t level, const rc_ksk* key,
                            rc_ciphertext* out, void* stream) {
  return guarded("rc_keyswitch", [&] {
    require(c && poly && out && out->data, "arguments must not be null");
    require(level >= 0 && level < c->L, "keyswitch level context must exist");
    const int limbs = level + 1;
    KsJob j{poly, key, nullptr, nullptr, out->data, out->data + (size_t)limbs * c->N};
    keyswitch_run(c, {j}, limbs, 0, false, S(stream));
    out->level = level;
    out->scale_bits = limbs;  // RnsCiphertext::new(c0, c1, poly.levels()), keyswitching.rs:156,193
  });
}

extern "C" int rc_relinearize(rc_context* c, const rc_ciphertext* qct, const rc_ksk* key, rc_ciphertext* out,
                              void* stream) {
  return guarded("rc_relinearize", [&] {
    require(c && out && out->data, "arguments must not be null");
    check_ct(c, qct, "quadratic ciphertext");
    const int limbs = qct->level + 1;
    const size_t pl = (size_t)limbs * c->N;
    KsJob j{qct->data + 2 * pl, key, qct->data, qct->data + pl, out->data, out->data + pl};
    keyswitch_run(c, {j}, limbs, 0, false, S(stream));
    out->level = qct->level;
    out->scale_bits = qct->scale_bits;
  });
}

extern "C" int rc_mult_relinearized(rc_context* c, const rc_ciphertext* a, const rc_ciphertext* b,
                                    const rc_ksk* key, rc_ciphertext* out, void* stream) {
  return guarded("rc_mult_relinearized", [&] {
    require(c && out && out->data, "arguments must not be null");
    check_mult_pair(c, a, b);
    std::vector<int> idx{0};
    mult_relin_group(c, idx, a, b, &key, out, S(stream));
  });
}

extern "C" int rc_rotate(rc_context* c, const rc_ciphertext* ct, const rc_ksk* key, rc_ciphertext* out,
                         void* stream) {
  return guarded("rc_rotate", [&] {
    require(c && out && out->data && key, "arguments must not be null");
    check_ct(c, ct, "ciphertext");
    // context/rotation.rs:106
    require(key->level == ct->level, "rotation key level must match the ciphertext level");
    require(key->galois != 0, "rotation key carries no Galois element");
    const uint64_t gi = galois_inverse(c, key->galois);
    const int limbs = ct->level + 1;
    const size_t pl = (size_t)limbs * c->N;
    require(out->data != ct->data, "rotate output must not alias its input");
    KsJob j{ct->data + pl, key, ct->data, nullptr, out->data, out->data + pl};
    keyswitch_run(c, {j}, limbs, gi, false, S(stream));
    out->level = ct->level;
    out->scale_bits = ct->scale_bits;
  });
}

extern "C" int rc_automorphism(rc_context* c, const rc_ciphertext* ct, uint64_t g, rc_ciphertext* out,
                               void* stream) {
  return guarded("rc_automorphism", [&] {
    require(c && out && out->data, "arguments must not be null");
    check_ct(c, ct, "ciphertext");
    require(out->data != ct->data, "automorphism output must not alias its input");
    const uint64_t gi = galois_inverse(c, g);
    const int limbs = ct->level + 1;
    const size_t pl = (size_t)limbs * c->N;
    PtrTab x{}, o{};
    x.p[0] = ct->data;
    x.p[1] = ct->data + pl;
    o.p[0] = out->data;
    o.p[1] = out->data + pl;
    automorphism(c->d_pc, x, o, 2, limbs, gi, c->log_n, S(stream));
    launch_check("automorphism");
    out->level = ct->level;
    out->scale_bits = ct->scale_bits;
  });
}

// =========================================================================
// batched forms
// =========================================================================
extern "C" int rc_mult_relinearized_batch(rc_context* c, uint32_t count, const rc_ciphertext* lhs,
                                          const rc_ciphertext* rhs, const rc_ksk* const* keys, rc_ciphertext* out,
                                          void* stream) {
  return guarded("rc_mult_relinearized_batch", [&] {
    require(c && lhs && rhs && keys && out, "arguments must not be null");
    std::map<std::pair<int, std::pair<int, int>>, std::vector<int>> groups;
    for (uint32_t i = 0; i < count; ++i) {
      check_mult_pair(c, &lhs[i], &rhs[i]);
      require(out[i].data != nullptr, "output must not be null");
      const rc_ksk* k = keys[i];
      require(k != nullptr, "keyswitch key must not be null");
      groups[{lhs[i].level, {key_kind(k), (int)k->digits}}].push_back((int)i);
    }
    for (auto& g : groups) mult_relin_group(c, g.second, lhs, rhs, keys, out, S(stream));
  });
}

extern "C" int rc_relinearize_batch(rc_context* c, uint32_t count, const rc_ciphertext* qct,
                                    const rc_ksk* const* keys, rc_ciphertext* out, void* stream) {
  return guarded("rc_relinearize_batch", [&] {
    require(c && qct && keys && out, "arguments must not be null");
    std::map<std::pair<int, std::pair<int, int>>, std::vector<int>> groups;
    for (uint32_t i = 0; i < count; ++i) {
      check_ct(c, &qct[i], "quadratic ciphertext");
      require(keys[i] != nullptr, "keyswitch key must not be null");
      check_key_for(c, keys[i], qct[i].level + 1);
      groups[{qct[i].level, {key_kind(keys[i]), (int)keys[i]->digits}}].push_back((int)i);
    }
    if (keyswitch_mixed_batch(c, qct, keys, out, count, false, S(stream))) {
      for (uint32_t i = 0; i < count; ++i) {
        out[i].level = qct[i].level;
        out[i].scale_bits = qct[i].scale_bits;
      }
      return;
    }
    for (auto& g : groups) {
      const int limbs = g.first.first + 1;
      const size_t pl = (size_t)limbs * c->N;
      for (size_t b = 0; b < g.second.size(); b += c->ks_jobs) {
        std::vector<KsJob> jobs;
        for (size_t k = b; k < g.second.size() && k < b + c->ks_jobs; ++k) {
          const int i = g.second[k];
          jobs.push_back(KsJob{qct[i].data + 2 * pl, keys[i], qct[i].data, qct[i].data + pl, out[i].data,
                               out[i].data + pl});
          out[i].level = qct[i].level;
          out[i].scale_bits = qct[i].scale_bits;
        }
        keyswitch_run(c, jobs, limbs, 0, false, S(stream));
      }
    }
  });
}

extern "C" int rc_relinearize_rescale_batch(rc_context* c, uint32_t count, const rc_ciphertext* qct,
                                            const rc_ksk* const* keys, rc_ciphertext* out, void* stream) {
  return guarded("rc_relinearize_rescale_batch", [&] {
    require(c && qct && keys && out, "arguments must not be null");
    std::map<std::pair<int, std::pair<int, int>>, std::vector<int>> groups;
    for (uint32_t i = 0; i < count; ++i) {
      check_ct(c, &qct[i], "quadratic ciphertext");
      require(out[i].data != nullptr, "arguments must not be null");
      require(out[i].data != qct[i].data, "rescale output must not alias its input");
      require(qct[i].level >= 1, "rescale requires at least two levels");
      require(keys[i] != nullptr, "keyswitch key must not be null");
      check_key_for(c, keys[i], qct[i].level + 1);
      groups[{qct[i].level, {key_kind(keys[i]), (int)keys[i]->digits}}].push_back((int)i);
    }
    if (keyswitch_mixed_batch(c, qct, keys, out, count, true, S(stream))) {
      for (uint32_t i = 0; i < count; ++i) {
        out[i].level = qct[i].level - 1;
        const int sb = qct[i].scale_bits - floor_log2(c->mod[qct[i].level]);  // rescale_ciphertext_rns
        out[i].scale_bits = sb < 0 ? 0 : sb;
      }
      return;
    }
    // groups run from the highest level down, each in chunks of at most MAXP/2 jobs (the size rc_reserve
    // provisions), so one reserve of the top level covers a whole mixed-level batch under graph capture
    for (auto g = groups.rbegin(); g != groups.rend(); ++g) {
      const int limbs = g->first.first + 1;
      const size_t pl = (size_t)limbs * c->N, po = (size_t)(limbs - 1) * c->N;
      const int drop = floor_log2(c->mod[limbs - 1]);
      for (size_t b = 0; b < g->second.size(); b += c->ks_jobs) {
        std::vector<KsJob> jobs;
        for (size_t k = b; k < g->second.size() && k < b + c->ks_jobs; ++k) {
          const int i = g->second[k];
          jobs.push_back(KsJob{qct[i].data + 2 * pl, keys[i], qct[i].data, qct[i].data + pl, out[i].data,
                               out[i].data + po});
          out[i].level = qct[i].level - 1;
          const int sb = qct[i].scale_bits - drop;  // rescale_ciphertext_rns, ops.rs:68-82
          out[i].scale_bits = sb < 0 ? 0 : sb;
        }
        keyswitch_run(c, jobs, limbs, 0, true, S(stream));
      }
    }
  });
}

// ---- CUDA graphs of library calls ----
struct rc_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

extern "C" int rc_graph_begin(rc_context* c, void* stream) {
  return guarded("rc_graph_begin", [&] {
    require(c != nullptr, "context must not be null");
    require(stream != nullptr, "CUDA graph capture needs a non-default stream");
    cuda_check(cudaStreamBeginCapture(S(stream), cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
  });
}

extern "C" int rc_graph_end(rc_context* c, void* stream, rc_graph** out) {
  return guarded("rc_graph_end", [&] {
    require(c && out && stream, "arguments must not be null");
    *out = nullptr;
    std::unique_ptr<rc_graph> g(new rc_graph());
    cuda_check(cudaStreamEndCapture(S(stream), &g->graph), "cudaStreamEndCapture");
    cuda_check(cudaGraphInstantiate(&g->exec, g->graph, 0), "cudaGraphInstantiate");
    *out = g.release();
  });
}

extern "C" int rc_graph_launch(rc_graph* g, void* stream) {
  OpRange op_range("rc_graph_launch");
  if (!g || !g->exec) {
    set_last_error("graph must not be null");
    return RC_ERR_INVALID_ARGUMENT;
  }
  const cudaError_t e = cudaGraphLaunch(g->exec, S(stream));
  if (e != cudaSuccess) {
    set_last_error(std::string("cudaGraphLaunch: ") + cudaGetErrorString(e));
    return RC_ERR_CUDA;
  }
  return RC_OK;
}

extern "C" void rc_graph_destroy(rc_graph* g) {
  if (!g) return;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
}

extern "C" int rc_rotate_batch(rc_context* c, uint32_t count, const rc_ciphertext* ct, const rc_ksk* const* keys,
                               rc_ciphertext* out, void* stream) {
  return guarded("rc_rotate_batch", [&] {
    require(c && ct && keys && out, "arguments must not be null");
    // group by (level, key kind, galois element): the gather is per launch
    std::map<std::pair<std::pair<int, uint64_t>, std::pair<int, int>>, std::vector<int>> groups;
    for (uint32_t i = 0; i < count; ++i) {
      check_ct(c, &ct[i], "ciphertext");
      const rc_ksk* k = keys[i];
      require(k != nullptr, "rotation key must not be null");
      require(k->level == ct[i].level, "rotation key level must match the ciphertext level");
      require(k->galois != 0, "rotation key carries no Galois element");
      groups[{{ct[i].level, k->galois}, {(int)k->aux, (int)k->digits}}].push_back((int)i);
    }
    for (auto& g : groups) {
      const int limbs = g.first.first.first + 1;
      const uint64_t gi = galois_inverse(c, g.first.first.second);
      const size_t pl = (size_t)limbs * c->N;
      for (size_t b = 0; b < g.second.size(); b += c->ks_jobs) {
        std::vector<KsJob> jobs;
        for (size_t k = b; k < g.second.size() && k < b + c->ks_jobs; ++k) {
          const int i = g.second[k];
          require(out[i].data != ct[i].data, "rotate output must not alias its input");
          jobs.push_back(KsJob{ct[i].data + pl, keys[i], ct[i].data, nullptr, out[i].data, out[i].data + pl});
          out[i].level = ct[i].level;
          out[i].scale_bits = ct[i].scale_bits;
        }
        keyswitch_run(c, jobs, limbs, gi, false, S(stream));
      }
    }
  });
}

// Rotations of every ciphertext by each of several keys from one decomposition ("hoisted"): c1 is decomposed
// and its digits transformed once, and each rotation's key product reads those transforms through the
// automorphism's NTT-domain permutation; the addend is sigma(c0) as in rc_rotate.  The digits of sigma(c1)
// are sigma of the digits of c1 -- the automorphism moves coefficients and flips signs, and the balanced
// digits of -X are the negated digits of X -- except where a digit of X is -2^29 (the balanced rule sends
// both +2^29 and -2^29 there).  A ciphertext with such a digit is rotated again the ordinary way, so every
// result equals rc_rotate's for the same (ciphertext, key).  Mixed levels, keys of different shapes or a
// chain outside the wide key product run as rc_rotate_batch.
extern "C" int rc_rotate_hoisted(rc_context* c, uint32_t count, const rc_ciphertext* cts, uint32_t nrot,
                                 const rc_ksk* const* keys, rc_ciphertext* out, void* stream) {
  return guarded("rc_rotate_hoisted", [&] {
    require(c && cts && keys && out, "arguments must not be null");
    if (count == 0 || nrot == 0) return;
    cudaStream_t s = S(stream);
    const int level = cts[0].level;
    bool hoist = true;
    for (uint32_t i = 0; i < count; ++i) {
      check_ct(c, &cts[i], "ciphertext");
      hoist = hoist && cts[i].level == level;
      for (uint32_t r = 0; r < nrot; ++r)
        require(out[(size_t)i * nrot + r].data != nullptr && out[(size_t)i * nrot + r].data != cts[i].data,
                "rotate output must not alias its input");
    }
    for (uint32_t r = 0; r < nrot; ++r) {
      require(keys[r] != nullptr, "rotation key must not be null");
      hoist = hoist && keys[r]->aux == keys[0]->aux && keys[r]->digits == keys[0]->digits && keys[r]->wdata &&
              keys[r]->galois > 1 && keys[r]->level == level;
    }
    auto ordinary = [&](const std::vector<std::pair<uint32_t, uint32_t>>& pairs) {
      std::vector<rc_ciphertext> in, o;
      std::vector<const rc_ksk*> ks;
      for (auto& p : pairs) {
        in.push_back(cts[p.first]);
        ks.push_back(keys[p.second]);
        o.push_back(out[(size_t)p.first * nrot + p.second]);
      }
      const int rc = rc_rotate_batch(c, (uint32_t)in.size(), in.data(), ks.data(), o.data(), stream);
      if (rc != RC_OK) fail(rc, g_err);
      for (size_t k = 0; k < pairs.size(); ++k) out[(size_t)pairs[k].first * nrot + pairs[k].second] = o[k];
    };
    const int limbs = level + 1;
    const int K = keys[0]->aux ? c->K : 0;
    const int D = ks_digits(c, keys[0], limbs);
    if (hoist) {
      for (uint32_t r = 0; r < nrot; ++r) check_key_for(c, keys[r], limbs);
      hoist = wide_applies(c, limbs, K, D) && c->log_n >= 5;
    }
    if (!hoist) {
      std::vector<std::pair<uint32_t, uint32_t>> all;
      for (uint32_t i = 0; i < count; ++i)
        for (uint32_t r = 0; r < nrot; ++r) all.emplace_back(i, r);
      ordinary(all);
      return;
    }
    const size_t N = c->N, pl = (size_t)limbs * N;
    for (uint32_t b0 = 0; b0 < count; b0 += (uint32_t)c->ks_jobs) {
      const int n = (int)std::min<uint32_t>((uint32_t)c->ks_jobs, count - b0);
      Arena ar(ws_device(c, s, wide_ks_bytes(c, n, n, limbs, K, D) + 2048));
      const WideKs w = wide_ks_layout(c, ar, n, n, limbs, K, D);
      int* flags = ar.take<int>((size_t)n);
      cuda_check(cudaMemsetAsync(flags, 0, (size_t)n * sizeof(int), s), "cudaMemsetAsync");
      PtrTab src{};
      for (int j = 0; j < n; ++j) src.p[j] = cts[b0 + j].data + pl;
      decompose(c->d_pc, level_info(c, limbs).dt, src, n, limbs, D, w.digits, 1, c->log_n, s, flags);
      launch_check("decompose");
      require(wide_digit_transforms(c->wp, D, n, w.digits, w.work, w.dt, s), "internal: wide transforms unsupported");
      launch_check("wide digit transforms");
      std::vector<int> tie((size_t)n);
      cuda_check(cudaMemcpyAsync(tie.data(), flags, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, s), "D2H");
      for (uint32_t r = 0; r < nrot; ++r) {
        const rc_ksk* k = keys[r];
        wide_mac(c->wp, D, (int)k->digits, w.total, (const uint2*)k->wdata, w.dt, w.acc, 0, n, c->mac_bc, s,
                 (uint32_t)k->galois);
        launch_check("wide mac");
        std::vector<KsJob> fin((size_t)n);
        for (int j = 0; j < n; ++j) {
          rc_ciphertext& o = out[(size_t)(b0 + j) * nrot + r];
          fin[(size_t)j] = KsJob{nullptr, k, cts[b0 + j].data, nullptr, o.data, o.data + pl};
          o.level = level;
          o.scale_bits = cts[b0 + j].scale_bits;
        }
        wide_ks_finish(c, w, fin, 0, n, galois_inverse(c, k->galois), false, s);
      }
      cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize");  // the tie flags
      std::vector<std::pair<uint32_t, uint32_t>> redo;
      for (int j = 0; j < n; ++j)
        if (tie[(size_t)j])
          for (uint32_t r = 0; r < nrot; ++r) redo.emplace_back(b0 + (uint32_t)j, r);
      if (!redo.empty()) ordinary(redo);
    }
  });
}

// =========================================================================
// host-buffer entry points
// =========================================================================
// Stage boundaries of a pipelined host-buffer batch.  Only the first stage's copy-in and the last stage's
// copy-out are not overlapped with arithmetic, so those two stages get chunk / edge jobs and the others
// chunk: [e, c, c, ..., c, rest - e, e].
static std::vector<uint32_t> stage_bounds(uint32_t count, uint32_t chunk, uint32_t edge) {
  const uint32_t e = std::max<uint32_t>(1, chunk / std::max<uint32_t>(1, edge));
  std::vector<uint32_t> b{0};
  uint32_t at = std::min(count, e);
  b.push_back(at);
  while (count - at > chunk + e) {
    at += chunk;
    b.push_back(at);
  }
  if (count - at > e) {
    at = count - e;
    b.push_back(at);
  }
  if (at < count) b.push_back(count);
  return b;
}

// One key-product group of a phased host-buffer batch: jobs [j0, j1) of the call, computed on `cs` with
// staging slot `sl`; inputs go through hp->in in job order, outputs through hp->out.  Returns the event of
// its last copy out.
static cudaEvent_t host_phased_group(rc_context* c, HostPipe* hp, uint32_t j0, uint32_t j1,
                                     const uint64_t* const* lhs, const uint64_t* const* rhs, const int32_t* levels,
                                     const int32_t* scale_bits, const rc_ksk* const* keys, uint64_t* const* out,
                                     int32_t* out_scale_bits, cudaStream_t cs, int sl, int chunk, int K, int D) {
  const int limbs = levels[j0] + 1;
  const int J = (int)(j1 - j0);
  const size_t N = c->N, pl = (size_t)limbs * N, po = (size_t)(limbs - 1) * N;
  // staging: inputs [J][lhs, rhs][2][limbs][N], outputs [J][2][limbs-1][N]
  const size_t stage = ((size_t)J * 4 * pl + (size_t)J * 2 * po) * 8;
  if (!hp->slot[sl] || hp->slot[sl]->bytes < stage) {
    for (cudaStream_t st : {hp->in, hp->comp, hp->out, hp->comp2})
      cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
    hp->slot[sl].reset();
    hp->slot[sl].reset(new DevBuf(stage));
  }
  if (!hp->consumed[sl]) {
    cuda_check(cudaEventCreateWithFlags(&hp->consumed[sl], cudaEventDisableTiming), "cudaEventCreate");
    cuda_check(cudaEventCreateWithFlags(&hp->drained[sl], cudaEventDisableTiming), "cudaEventCreate");
  }
  // an earlier call's work on this slot: its inputs read before new copies in, its outputs copied out before
  // new results
  if (hp->used[sl]) {
    cuda_check(cudaStreamWaitEvent(hp->in, hp->consumed[sl], 0), "wait");
    cuda_check(cudaStreamWaitEvent(cs, hp->drained[sl], 0), "wait");
  }
  hp->used[sl] = true;
  uint64_t* in_dev = (uint64_t*)hp->slot[sl]->p;
  uint64_t* out_dev = in_dev + (size_t)J * 4 * pl;
  const size_t tbytes = tensor_ws_bytes(c, chunk, limbs);
  char* ws = (char*)ws_device(c, cs, arena_size_u64((size_t)3 * J * pl) + align_up(tbytes, 256) +
                                         wide_ks_bytes(c, J, chunk, limbs, K, D) + 1024);
  Arena ar(ws);
  uint64_t* quads = ar.take<uint64_t>((size_t)3 * J * pl);
  char* tscr = ar.take<char>(tbytes);
  const WideKs w = wide_ks_layout(c, ar, J, chunk, limbs, K, D);

  const std::vector<uint32_t> bounds = stage_bounds((uint32_t)J, (uint32_t)chunk, (uint32_t)c->host_edge);
  const int nchunks = (int)bounds.size() - 1;
  std::vector<cudaEvent_t> in_done(nchunks), comp_done(nchunks);
  for (int k = 0; k < nchunks; ++k) {  // every chunk's inputs, back to back in job order
    for (int j = (int)bounds[k]; j < (int)bounds[k + 1]; ++j) {
      cuda_check(cudaMemcpyAsync(in_dev + (size_t)j * 4 * pl, lhs[j0 + j], 2 * pl * 8, cudaMemcpyHostToDevice,
                                 hp->in),
                 "H2D");
      cuda_check(cudaMemcpyAsync(in_dev + (size_t)j * 4 * pl + 2 * pl, rhs[j0 + j], 2 * pl * 8,
                                 cudaMemcpyHostToDevice, hp->in),
                 "H2D");
    }
    in_done[k] = hp->event();
    cuda_check(cudaEventRecord(in_done[k], hp->in), "cudaEventRecord");
  }
  std::vector<KsJob> jobs(J);
  for (int j = 0; j < J; ++j) {
    uint64_t* qd = quads + (size_t)j * 3 * pl;
    jobs[j] = KsJob{qd + 2 * pl, keys[j0 + j], qd, qd + pl, out_dev + (size_t)j * 2 * po,
                    out_dev + (size_t)j * 2 * po + po};
  }
  for (int k = 0; k < nchunks; ++k) {
    const int b0 = (int)bounds[k], n = (int)bounds[k + 1] - b0;
    cuda_check(cudaStreamWaitEvent(cs, in_done[k], 0), "wait");
    std::vector<const uint64_t*> Lp(n), Rp(n);
    std::vector<uint64_t*> Q(n);
    for (int j = 0; j < n; ++j) {
      Lp[j] = in_dev + (size_t)(b0 + j) * 4 * pl;
      Rp[j] = Lp[j] + 2 * pl;
      Q[j] = quads + (size_t)(b0 + j) * 3 * pl;
    }
    tensor_core(c, Lp, Rp, Q, limbs, tscr, cs);
    wide_ks_prepare(c, w, jobs, b0, n, 0, cs);
  }
  cuda_check(cudaEventRecord(hp->consumed[sl], cs), "cudaEventRecord");  // the slot's inputs are read
  wide_ks_mac(c, w, jobs, cs);
  const int drop = floor_log2(c->mod[limbs - 1]);
  for (int k = 0; k < nchunks; ++k) {
    const int b0 = (int)bounds[k], n = (int)bounds[k + 1] - b0;
    wide_ks_finish(c, w, jobs, b0, n, 0, true, cs);
    comp_done[k] = hp->event();
    cuda_check(cudaEventRecord(comp_done[k], cs), "cudaEventRecord");
    cuda_check(cudaStreamWaitEvent(hp->out, comp_done[k], 0), "wait");
    for (int j = b0; j < b0 + n; ++j) {
      cuda_check(cudaMemcpyAsync(out[j0 + j], out_dev + (size_t)j * 2 * po, 2 * po * 8, cudaMemcpyDeviceToHost,
                                 hp->out),
                 "D2H");
      if (out_scale_bits) {
        const int sb = scale_bits[j0 + j] + scale_bits[j0 + j] - drop;  // mult_relinearized, context/ops.rs:124-133
        out_scale_bits[j0 + j] = sb < 0 ? 0 : sb;
      }
    }
  }
  cuda_check(cudaEventRecord(hp->drained[sl], hp->out), "cudaEventRecord");
  cudaEvent_t fin = hp->event();
  cuda_check(cudaEventRecord(fin, hp->out), "cudaEventRecord");
  return fin;
}

// Host-buffer batch of up to ks_jobs same-level jobs on the wide key-switch path in `groups` key-product
// groups (1 or 2).  Each group is phased: its inputs are copied in back to back, each chunk's tensor,
// decomposition and digit transforms start as soon as the chunk's inputs have landed, one key-product pass
// covers the group, then each chunk's inverse transforms and finalize run and its results are copied out
// while the next chunk finishes.  With two groups the second computes on its own stream and staging slot,
// so its copy-in and preparation overlap the first group's key product and the first group's copy-out
// overlaps the second's arithmetic (one more key read).  Returns false (nothing done) when the batch does
// not fit this form.
static bool mult_relin_host_phased(rc_context* c, HostPipe* hp, uint32_t count, const uint64_t* const* lhs,
                                   const uint64_t* const* rhs, const int32_t* levels, const int32_t* scale_bits,
                                   const rc_ksk* const* keys, uint64_t* const* out, int32_t* out_scale_bits,
                                   cudaStream_t s, int chunk, int groups, bool async) {
  const int level = levels[0];
  if (count > (uint32_t)c->ks_jobs) return false;
  for (uint32_t i = 0; i < count; ++i)
    if (levels[i] != level) return false;
  const int limbs = level + 1;
  if (limbs < 2) return false;
  const rc_ksk* k0 = keys[0];
  for (uint32_t i = 0; i < count; ++i) {
    require(keys[i] != nullptr, "keyswitch key must not be null");
    check_key_for(c, keys[i], limbs);
    if ((keys[i]->aux != 0) != (k0->aux != 0) || !keys[i]->wdata) return false;
  }
  const int K = k0->aux ? c->K : 0;
  const int D = ks_digits(c, k0, limbs);
  for (uint32_t i = 0; i < count; ++i)
    if (!K && (int)keys[i]->digits != D) return false;
  if (!wide_applies(c, limbs, K, D)) return false;
  chunk = std::max(1, std::min(chunk, MAXP / 4));
  groups = std::max(1, std::min(groups, 2));
  if (count < 2) groups = 1;
  cudaEvent_t start = hp->event();
  cuda_check(cudaEventRecord(start, s), "cudaEventRecord");
  for (cudaStream_t st : {hp->in, hp->comp, hp->out, hp->comp2})
    cuda_check(cudaStreamWaitEvent(st, start, 0), "cudaStreamWaitEvent");
  const uint32_t split = groups == 2 ? (count + 1) / 2 : count;
  const int set = 2 * hp->ring;  // staging slots of this call (alternating sets, see HostPipe)
  hp->ring ^= 1;
  cudaEvent_t fin = host_phased_group(c, hp, 0, split, lhs, rhs, levels, scale_bits, keys, out, out_scale_bits,
                                      hp->comp, set, chunk, K, D);
  if (split < count)
    fin = host_phased_group(c, hp, split, count, lhs, rhs, levels, scale_bits, keys, out, out_scale_bits, hp->comp2,
                            set + 1, chunk, K, D);
  cuda_check(cudaEventRecord(hp->last, hp->out), "cudaEventRecord");  // the copies out are in order on hp->out
  if (async) {
    hp->pending = true;
    return true;
  }
  cuda_check(cudaStreamWaitEvent(s, fin, 0), "wait");
  cuda_check(cudaStreamSynchronize(hp->out), "cudaStreamSynchronize");
  hp->pending = false;  // the copies out of earlier asynchronous calls precede these on hp->out
  return true;
}

// Host-buffer batch: the jobs run in chunks through a three-stage pipeline on internal streams (copy in
// on two streams, compute, copy out) with two device staging slots, so that transfers overlap the
// arithmetic.  The whole call is ordered after earlier work on `stream` and returns when the results are
// in host memory.
// the host pipeline of caller stream s (created on first use)
static HostPipe* host_pipe(rc_context* c, cudaStream_t s) {
  std::lock_guard<std::mutex> lk(c->mu);
  auto& p = c->pipes[s];
  if (!p) {
    p.reset(new HostPipe());
    for (cudaStream_t* st : {&p->in, &p->comp, &p->out, &p->comp2})
      cuda_check(cudaStreamCreateWithFlags(st, cudaStreamNonBlocking), "cudaStreamCreate");
    cuda_check(cudaEventCreateWithFlags(&p->last, cudaEventDisableTiming), "cudaEventCreate");
  }
  return p.get();
}

// The host-buffer batch (see rc_mult_relinearized_batch_host); async: return once enqueued (phased form).
static void mult_relin_batch_host(rc_context* c, uint32_t count, const uint64_t* const* lhs,
                                  const uint64_t* const* rhs, const int32_t* levels, const int32_t* scale_bits,
                                  const rc_ksk* const* keys, uint64_t* const* out, int32_t* out_scale_bits,
                                  cudaStream_t s, bool async) {
    require(c && lhs && rhs && levels && scale_bits && keys && out, "arguments must not be null");
    for (uint32_t i = 0; i < count; ++i)
      require(levels[i] >= 1 && levels[i] < c->L, "ciphertext level context must exist");
    if (count == 0) return;
    HostPipe* hp = host_pipe(c, s);
    hp->next = 0;
    int chunk = c->host_chunk;  // jobs per pipeline stage
    if (const char* e = getenv("RNSCKKS_HOST_CHUNK")) chunk = std::max(1, atoi(e));
    if (c->host_phased && mult_relin_host_phased(c, hp, count, lhs, rhs, levels, scale_bits, keys, out,
                                                 out_scale_bits, s, chunk, c->host_phased, async))
      return;
    // the staged form below is synchronous: earlier asynchronous calls finish first
    if (hp->pending) {
      cuda_check(cudaStreamSynchronize(hp->out), "cudaStreamSynchronize");
      hp->pending = false;
    }
    const std::vector<uint32_t> bounds = stage_bounds(count, (uint32_t)chunk, (uint32_t)c->host_edge);
    const uint32_t nchunks = (uint32_t)bounds.size() - 1;
    auto in_elems = [&](uint32_t i) { return (size_t)2 * (levels[i] + 1) * c->N; };
    auto out_elems = [&](uint32_t i) { return (size_t)2 * levels[i] * c->N; };
    size_t need = 0;
    for (uint32_t k = 0; k < nchunks; ++k) {
      size_t b = 0;
      for (uint32_t i = bounds[k]; i < bounds[k + 1]; ++i)
        b += 2 * in_elems(i) + out_elems(i);
      need = std::max(need, b * 8);
    }
    for (int sl = 0; sl < 2; ++sl) {
      if (!hp->slot[sl] || hp->slot[sl]->bytes < need) {
        for (cudaStream_t st : {hp->in, hp->comp, hp->out, hp->comp2})
          cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
        hp->slot[sl].reset();
        hp->slot[sl].reset(new DevBuf(need));
      }
    }
    cudaEvent_t start = hp->event();
    cuda_check(cudaEventRecord(start, s), "cudaEventRecord");
    for (cudaStream_t st : {hp->in, hp->comp, hp->out, hp->comp2})
      cuda_check(cudaStreamWaitEvent(st, start, 0), "cudaStreamWaitEvent");
    std::vector<cudaEvent_t> comp_done(nchunks), out_done(nchunks);
    for (uint32_t k = 0; k < nchunks; ++k) {
      const uint32_t i0 = bounds[k], i1 = bounds[k + 1], n = i1 - i0;
      uint64_t* dev = (uint64_t*)hp->slot[k & 1]->p;
      if (k >= 2) {  // the slot's inputs were consumed by chunk k-2's compute
        cuda_check(cudaStreamWaitEvent(hp->in, comp_done[k - 2], 0), "wait");
      }
      std::vector<rc_ciphertext> L(n), R(n), O(n);
      size_t off = 0;
      for (uint32_t j = 0; j < n; ++j) {
        const uint32_t i = i0 + j;
        L[j] = rc_ciphertext{dev + off, levels[i], scale_bits[i]};
        cuda_check(cudaMemcpyAsync(dev + off, lhs[i], in_elems(i) * 8, cudaMemcpyHostToDevice, hp->in), "H2D");
        off += in_elems(i);
        R[j] = rc_ciphertext{dev + off, levels[i], scale_bits[i]};
        cuda_check(cudaMemcpyAsync(dev + off, rhs[i], in_elems(i) * 8, cudaMemcpyHostToDevice, hp->in), "H2D");
        off += in_elems(i);
      }
      for (uint32_t j = 0; j < n; ++j) {
        O[j] = rc_ciphertext{dev + off, 0, 0};
        off += out_elems(i0 + j);
      }
      cudaStream_t cs = (k & 1) ? hp->comp2 : hp->comp;
      {
        cudaEvent_t e = hp->event();
        cuda_check(cudaEventRecord(e, hp->in), "cudaEventRecord");
        cuda_check(cudaStreamWaitEvent(cs, e, 0), "wait");
      }
      if (k >= 2) cuda_check(cudaStreamWaitEvent(cs, out_done[k - 2], 0), "wait");  // slot outputs read
      int rc = rc_mult_relinearized_batch(c, n, L.data(), R.data(), keys + i0, O.data(), cs);
      if (rc != RC_OK) fail(rc, g_err);
      comp_done[k] = hp->event();
      cuda_check(cudaEventRecord(comp_done[k], cs), "cudaEventRecord");
      cuda_check(cudaStreamWaitEvent(hp->out, comp_done[k], 0), "wait");
      for (uint32_t j = 0; j < n; ++j) {
        const uint32_t i = i0 + j;
        cuda_check(cudaMemcpyAsync(out[i], O[j].data, out_elems(i) * 8, cudaMemcpyDeviceToHost, hp->out), "D2H");
        if (out_scale_bits) out_scale_bits[i] = O[j].scale_bits;
      }
      out_done[k] = hp->event();
      cuda_check(cudaEventRecord(out_done[k], hp->out), "cudaEventRecord");
    }
    // later work on the caller's stream is ordered after the whole call
    cuda_check(cudaEventRecord(hp->last, hp->out), "cudaEventRecord");
    cuda_check(cudaStreamWaitEvent(s, out_done[nchunks - 1], 0), "wait");
    cuda_check(cudaStreamSynchronize(hp->out), "cudaStreamSynchronize");
}

extern "C" int rc_mult_relinearized_batch_host(rc_context* c, uint32_t count, const uint64_t* const* lhs,
                                               const uint64_t* const* rhs, const int32_t* levels,
                                               const int32_t* scale_bits, const rc_ksk* const* keys,
                                               uint64_t* const* out, int32_t* out_scale_bits, void* stream) {
  return guarded("rc_mult_relinearized_batch_host", [&] {
    mult_relin_batch_host(c, count, lhs, rhs, levels, scale_bits, keys, out, out_scale_bits, S(stream), false);
  });
}

extern "C" int rc_mult_relinearized_batch_host_async(rc_context* c, uint32_t count, const uint64_t* const* lhs,
                                                     const uint64_t* const* rhs, const int32_t* levels,
                                                     const int32_t* scale_bits, const rc_ksk* const* keys,
                                                     uint64_t* const* out, int32_t* out_scale_bits, void* stream) {
  OpRange op_range("rc_mult_relinearized_batch_host_async");
  return guarded("rc_mult_relinearized_batch_host_async", [&] {
    mult_relin_batch_host(c, count, lhs, rhs, levels, scale_bits, keys, out, out_scale_bits, S(stream), true);
  });
}

extern "C" int rc_host_join(rc_context* c, void* stream) {
  return guarded("rc_host_join", [&] {
    require(c != nullptr, "context must not be null");
    const cudaStream_t s = S(stream);
    HostPipe* hp = nullptr;
    {
      std::lock_guard<std::mutex> lk(c->mu);
      auto it = c->pipes.find(s);
      if (it != c->pipes.end()) hp = it->second.get();
    }
    if (!hp) return;
    cuda_check(cudaStreamWaitEvent(s, hp->last, 0), "wait");
    hp->pending = false;
  });
}


extern "C" int rc_mult_relinearized_host(rc_context* c, const uint64_t* lhs, const uint64_t* rhs, int32_t level,
                                         int32_t scale_bits, const rc_ksk* key, uint64_t* out,
                                         int32_t* out_scale_bits, void* stream) {
  OpRange op_range("rc_mult_relinearized_host");
  const uint64_t* l[1] = {lhs};
  const uint64_t* r[1] = {rhs};
  uint64_t* o[1] = {out};
  const rc_ksk* k[1] = {key};
  return rc_mult_relinearized_batch_host(c, 1, l, r, &level, &scale_bits, k, o, out_scale_bits, stream);
}
