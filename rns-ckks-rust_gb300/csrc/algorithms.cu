// The crate's src/algorithms routines (total sum, Halevi-Shoup dot product, Paterson-Stockmeyer) as C ABI
// entry points over the library's own batched ops, so a caller runs a whole schedule for a batch of
// ciphertexts in one call with no per-step host glue.  Each routine keeps the crate's schedule, scale and
// level bookkeeping and panic messages (returned as RC_ERR_INVALID_ARGUMENT with the message), so the
// residues equal the crate's for the same keys and inputs:
//   total_sum.rs:45-60, halevi_shoup.rs:46-71 (with context/ops.rs:39-48), paterson_stockmeyer.rs:28-349.
// Intermediates live in stream-ordered device allocations (cudaMallocAsync) released at the end of the call.
#include <cmath>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "context.hpp"

using namespace rc;

namespace {

// N/2 complex slots all equal to (value, 0), interleaved
__global__ void k_fill_const(double* slots, double value, size_t half) {
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < half; k += (size_t)gridDim.x * blockDim.x) {
    slots[2 * k] = value;
    slots[2 * k + 1] = 0.0;
  }
}

void ok(int status) {
  if (status != RC_OK) fail(status, rc_last_error(nullptr));
}

// ---- BSGS inner sums of a batch in one launch (apply_giant_step_terms, linear_transform.rs:234-252) ----
// inner[i][g][c] = sum_j baby[i][j][c] * diag[g][j] mod q over the NTT domain, for every ciphertext i, giant
// g and component c.  A thread owns one coefficient of one ciphertext and keeps its b babies in registers
// across the giants; the warps of a block share coefficients (ciphertexts differ), so each diagonal word is
// fetched from memory once per block.  On a limb whose prime is below 2^52 a residue x splits as
// x1 * 2^26 + x0 (both < 2^26) and a product as x0 y0 + ((x0 + x1)(y0 + y1) - x0 y0 - x1 y1) 2^26 + x1 y1 2^52:
// three 32 x 32 -> 64-bit multiply-adds per term, summed exactly in 64-bit columns (each column below
// 16 * 2^54) and reduced once per output.  A limb with a larger prime (a 60-bit base prime) sums full
// 128-bit products (one Barrett reduction per output; per term above 2^60); a block's 32 coefficients
// share one limb for N >= 32, so the branch is uniform there.
constexpr int BSGS_MAX_TABLE = 256;
struct DiagTab {
  const u64* p[BSGS_MAX_TABLE];  // [g * b + j], null past the dimension
};

__device__ __forceinline__ uint32_t lo26(u64 x) { return (uint32_t)x & ((1u << 26) - 1); }
__device__ __forceinline__ uint32_t hi26(u64 x) { return (uint32_t)(x >> 26); }
__device__ __forceinline__ u64 mad_wide(uint32_t a, uint32_t b, u64 acc) { return acc + (u64)a * b; }

template <int BM>
__global__ void __launch_bounds__(256, 2) k_bsgs_inner(const PrimeConst* pc, const u64* __restrict__ babies,
                                                       DiagTab diag, u64* __restrict__ out, int count, int b,
                                                       int giants, int limbs, int log_n) {
  extern __shared__ u64 dsm[];  // [giants * BM][32]: this block's 32 words of every diagonal
  const size_t pl = (size_t)limbs << log_n;
  const size_t e0 = (size_t)blockIdx.x * 32, e = e0 + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  const int tid = threadIdx.y * 32 + threadIdx.x, slots = giants * BM;
  // every diagonal word of the block in flight at once (one 256-byte row per diagonal), stored as the two
  // 26-bit halves (low word, high word) when the word's prime is split (a block's 32 coefficients share one
  // limb unless N < 32)
  for (int k = tid; k < slots * 32; k += 256) {
    const int slot = k >> 5, lane = k & 31;
    const size_t ek = e0 + lane;
    const u64 y = ek < pl ? __ldg(diag.p[slot] + ek) : 0;
    const bool sk = ek < pl && (pc[(int)(ek >> log_n)].q >> 52) == 0;
    dsm[k] = sk ? ((u64)hi26(y) << 32 | lo26(y)) : y;
  }
  const bool active = e < pl && i < count;
  const PrimeConst& c = pc[(int)((active ? e : e0) >> log_n)];
  const bool split = (c.q >> 52) == 0;
  // babies: (x0, x1) = the 26-bit halves when split, else the 32-bit words; zero past the baby step (their
  // diagonals are the zero polynomial)
  uint32_t x0[2][BM], x1[2][BM];
#pragma unroll
  for (int j = 0; j < BM; ++j) {
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const u64 v = active && j < b ? babies[(((size_t)i * b + j) * 2 + k) * pl + e] : 0;
      x0[k][j] = split ? lo26(v) : (uint32_t)v;
      x1[k][j] = split ? hi26(v) : (uint32_t)(v >> 32);
    }
  }
  __syncthreads();
  if (!active) return;
  for (int g = 0; g < giants; ++g) {
    const u64* y = dsm + (size_t)g * BM * 32 + threadIdx.x;
    u64* o = out + ((size_t)i * giants + g) * 2 * pl + e;
    if (split) {
      u64 p00[2] = {0, 0}, p11[2] = {0, 0}, pk[2] = {0, 0};
#pragma unroll
      for (int j = 0; j < BM; ++j) {
        const u64 yj = y[j * 32];
        const uint32_t y0 = (uint32_t)yj, y1 = (uint32_t)(yj >> 32), ys = y0 + y1;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          p00[k] = mad_wide(x0[k][j], y0, p00[k]);
          p11[k] = mad_wide(x1[k][j], y1, p11[k]);
          pk[k] = mad_wide(x0[k][j] + x1[k][j], ys, pk[k]);
        }
      }
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const u64 cross = pk[k] - p00[k] - p11[k];
        // p00 + cross * 2^26 + p11 * 2^52 as 128 bits (below 16 q^2 < q * 2^64)
        U128 t;
        const u64 c_lo = cross << 26, p_lo = p11[k] << 52;
        t.lo = p00[k] + c_lo;
        t.hi = (cross >> 38) + (t.lo < c_lo ? 1ull : 0ull);
        t.lo += p_lo;
        t.hi += (p11[k] >> 12) + (t.lo < p_lo ? 1ull : 0ull);
        o[(size_t)k * pl] = barrett_reduce(t, c);
      }
    } else if ((c.q >> 60) == 0) {
      // 128-bit sums of at most 16 products, below 16 q^2 < q * 2^64: one reduction per output
      U128 acc[2] = {{0, 0}, {0, 0}};
#pragma unroll
      for (int j = 0; j < BM; ++j) {
        const u64 yj = y[j * 32];
#pragma unroll
        for (int k = 0; k < 2; ++k) add_to(acc[k], mul_wide((u64)x1[k][j] << 32 | x0[k][j], yj));
      }
      o[0] = barrett_reduce(acc[0], c);
      o[pl] = barrett_reduce(acc[1], c);
    } else {
      u64 acc[2] = {0, 0};
#pragma unroll
      for (int j = 0; j < BM; ++j) {
        const u64 yj = y[j * 32];
#pragma unroll
        for (int k = 0; k < 2; ++k)
          acc[k] = add_mod(acc[k], mul_mod((u64)x1[k][j] << 32 | x0[k][j], yj, c), c.q);
      }
      o[0] = acc[0];
      o[pl] = acc[1];
    }
  }
}

template <int BM>
void launch_bsgs_inner(const rc_context* c, dim3 grid, dim3 block, const u64* babies, const DiagTab& diag, u64* out,
                       int count, int b, int giants, int limbs, cudaStream_t s) {
  const size_t smem = (size_t)giants * BM * 32 * 8;
  static std::once_flag once;
  std::call_once(once, [] {
    cudaFuncSetAttribute(k_bsgs_inner<BM>, cudaFuncAttributeMaxDynamicSharedMemorySize, BSGS_MAX_TABLE * 32 * 8);
  });
  k_bsgs_inner<BM><<<grid, block, smem, s>>>(c->d_pc, babies, diag, out, count, b, giants, limbs, c->log_n);
}

// register tile (babies per thread) for a baby step b <= 16
int bsgs_tile(uint32_t b) { return b <= 4 ? 4 : b <= 8 ? 8 : b <= 12 ? 12 : 16; }

// true when the fused kernel applies: baby step within the register budget and the padded diagonal table
// within the launch parameter block
bool bsgs_inner_applies(uint32_t b, uint32_t giants) {
  return b <= 16 && (size_t)bsgs_tile(b) * giants <= (size_t)BSGS_MAX_TABLE;
}

// diag: [giants][bsgs_tile(b)] NTT-domain diagonals, the zero polynomial where the transform has none
void bsgs_inner(const rc_context* c, const u64* babies, const DiagTab& diag, u64* out, int count, int b, int giants,
                int limbs, cudaStream_t s) {
  ProfScope p("bsgs_inner", s);
  const size_t pl = (size_t)limbs * c->N;
  const dim3 block(32, 8), grid((unsigned)((pl + 31) / 32), (unsigned)((count + 7) / 8));
  switch (bsgs_tile((uint32_t)b)) {
    case 4: launch_bsgs_inner<4>(c, grid, block, babies, diag, out, count, b, giants, limbs, s); break;
    case 8: launch_bsgs_inner<8>(c, grid, block, babies, diag, out, count, b, giants, limbs, s); break;
    case 12: launch_bsgs_inner<12>(c, grid, block, babies, diag, out, count, b, giants, limbs, s); break;
    default: launch_bsgs_inner<16>(c, grid, block, babies, diag, out, count, b, giants, limbs, s);
  }
  cuda_check(cudaGetLastError(), "bsgs inner sums");
}

// stream-ordered scratch of one call
struct Pool {
  cudaStream_t s;
  std::vector<void*> ptrs;
  explicit Pool(cudaStream_t st) : s(st) {}
  ~Pool() {
    for (void* p : ptrs) cudaFreeAsync(p, s);
  }
  uint64_t* take(size_t words) {
    void* p = nullptr;
    cuda_check(cudaMallocAsync(&p, words * 8, s), "cudaMallocAsync");
    ptrs.push_back(p);
    return (uint64_t*)p;
  }
};

struct Algo {
  rc_context* c;
  cudaStream_t s;
  Pool pool;
  size_t N;
  std::map<std::tuple<double, int, int>, uint64_t*> consts;  // encoded constants by (value, level, scale)

  Algo(rc_context* ctx, void* stream) : c(ctx), s((cudaStream_t)stream), pool((cudaStream_t)stream), N(ctx->N) {
    // keep freed blocks in the device's stream-ordered pool between calls (a setting of this process's pool)
    static std::once_flag once;
    std::call_once(once, [] {
      int dev = 0;
      cudaMemPool_t mp;
      if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&mp, dev) == cudaSuccess) {
        uint64_t keep = ~0ull;
        cudaMemPoolSetAttribute(mp, cudaMemPoolAttrReleaseThreshold, &keep);
      }
    });
  }

  rc_ciphertext fresh(int level, int scale) { return rc_ciphertext{pool.take(2 * (size_t)(level + 1) * N), level, scale}; }

  // the first `level + 1` limbs of each component (truncate_levels): a copy, components are [2][limbs][N]
  rc_ciphertext truncate(const rc_ciphertext& ct, int level) {
    if (level == ct.level) return ct;
    rc_ciphertext o = fresh(level, ct.scale_bits);
    const size_t bytes = (size_t)(level + 1) * N * 8;
    for (int k = 0; k < 2; ++k)
      cuda_check(cudaMemcpyAsync(o.data + k * (level + 1) * N, ct.data + k * (size_t)(ct.level + 1) * N, bytes,
                                 cudaMemcpyDeviceToDevice, s),
                 "truncate");
    return o;
  }

  // encode of N/2 slots all equal to `value` at (level, scale), on the GPU, kept in the context's cache (the
  // same constants recur across calls: PS coefficients, plaintext ones of the scale lifts); past the cache's
  // cap a constant lives in this call's stream-ordered scratch
  uint64_t* constant(double value, int level, int scale) {
    auto key = std::make_tuple(value, level, scale);
    auto it = consts.find(key);
    if (it != consts.end()) return it->second;
    const size_t words = (size_t)(level + 1) * N;
    std::unique_ptr<DevBuf> buf;
    {
      std::lock_guard<std::mutex> lk(c->mu);
      auto ct = c->const_cache.find(key);
      if (ct != c->const_cache.end()) return consts[key] = (uint64_t*)ct->second->p;
      if (c->const_cache.size() < 1024) buf.reset(new DevBuf(words * 8));
    }
    uint64_t* out = buf ? (uint64_t*)buf->p : pool.take(words);
    double* dslots = (double*)pool.take(N);
    const size_t half = N / 2;
    k_fill_const<<<(unsigned)std::min<size_t>((half + 255) / 256, 1024), 256, 0, s>>>(dslots, value, half);
    cuda_check(cudaGetLastError(), "constant slots");
    ok(rc_encode_device(c, dslots, 1, level, (uint32_t)scale, out, s));
    if (buf) {
      cuda_check(cudaStreamSynchronize(s), "constant encode");  // complete before another stream may read it
      std::lock_guard<std::mutex> lk(c->mu);
      auto& slot = c->const_cache[key];
      if (!slot) slot = std::move(buf);  // another thread may have cached the same constant meanwhile
      out = (uint64_t*)slot->p;
    }
    return consts[key] = out;
  }

  std::vector<rc_ciphertext> add(const std::vector<rc_ciphertext>& a, const std::vector<rc_ciphertext>& b,
                                 rc_ciphertext* into = nullptr) {
    std::vector<rc_ciphertext> o(a.size());
    for (size_t i = 0; i < a.size(); ++i) o[i] = into ? into[i] : fresh(a[i].level, a[i].scale_bits);
    ok(rc_add_batch(c, (uint32_t)a.size(), a.data(), b.data(), o.data(), s));
    if (into)
      for (size_t i = 0; i < a.size(); ++i) into[i] = o[i];  // level and scale of the caller's outputs
    return o;
  }

  std::vector<rc_ciphertext> rotate(const std::vector<rc_ciphertext>& a, const rc_ksk* key) {
    std::vector<rc_ciphertext> o(a.size());
    std::vector<const rc_ksk*> ks(a.size(), key);
    for (size_t i = 0; i < a.size(); ++i) o[i] = fresh(a[i].level, a[i].scale_bits);
    ok(rc_rotate_batch(c, (uint32_t)a.size(), a.data(), ks.data(), o.data(), s));
    return o;
  }

  // multiply_plain_rns of every ciphertext by the same plaintext, then scale_bits set to `scale`
  std::vector<rc_ciphertext> mul_plain(const std::vector<rc_ciphertext>& a, const uint64_t* plain, int scale) {
    std::vector<rc_ciphertext> o(a.size());
    std::vector<const uint64_t*> ps(a.size(), plain);
    for (size_t i = 0; i < a.size(); ++i) o[i] = fresh(a[i].level, a[i].scale_bits);
    ok(rc_multiply_plain_rns_batch(c, (uint32_t)a.size(), a.data(), ps.data(), o.data(), s));
    for (auto& x : o) x.scale_bits = scale;
    return o;
  }
};

// fold steps 1, 2, 4, ... below next_power_of_two(active_slots) (halevi_shoup.rs:15-26, total_sum.rs:14-25)
std::vector<uint32_t> fold_steps(uint32_t active_slots) {
  require(active_slots > 0, "active_slots must be positive");
  uint32_t width = 1;
  while (width < active_slots) width <<= 1;
  std::vector<uint32_t> steps;
  for (uint32_t st = 1; st < width; st <<= 1) steps.push_back(st);
  return steps;
}

// rotate-and-add over the fold steps; the last add writes into `out`
void fold(Algo& A, std::vector<rc_ciphertext> accs, uint32_t active_slots, const rc_ksk* const* keys,
          uint32_t key_count, const char* missing, rc_ciphertext* out) {
  const std::vector<uint32_t> steps = fold_steps(active_slots);
  for (size_t t = 0; t < steps.size(); ++t) {
    if (t >= key_count || !keys[t]) fail(RC_ERR_INVALID_ARGUMENT, missing + std::to_string(steps[t]));
    const std::vector<rc_ciphertext> rotated = A.rotate(accs, keys[t]);
    accs = A.add(accs, rotated, t + 1 == steps.size() ? out : nullptr);
  }
  if (steps.empty()) {  // nothing to fold: the input itself
    for (size_t i = 0; i < accs.size(); ++i) {
      cuda_check(cudaMemcpyAsync(out[i].data, accs[i].data, 2 * (size_t)(accs[i].level + 1) * A.N * 8,
                                 cudaMemcpyDeviceToDevice, A.s),
                 "copy");
      out[i].level = accs[i].level;
      out[i].scale_bits = accs[i].scale_bits;
    }
  }
}

// paterson_stockmeyer.rs:18-26 and 110-126
uint32_t ps_block_size(uint32_t terms) {
  require(terms > 0, "term_count must be positive");
  uint32_t b = 1;
  while (b * b < terms) ++b;
  return b;
}

std::vector<int> ps_required_levels(int level, uint32_t terms) {
  require(terms > 0, "term_count must be positive");
  if (terms == 1) return {};
  const int b = (int)ps_block_size(terms), blocks = (int)((terms + b - 1) / b);
  const int top = level - (b - 1);
  require(top >= 0, "polynomial degree is too large for the available CKKS level budget");
  const int fin = top - (blocks - 1);
  require(fin >= 0, "polynomial degree is too large for the available CKKS level budget");
  std::vector<int> out;
  for (int l = level; l > fin; --l) out.push_back(l);
  return out;
}

int floor_log2_u64(uint64_t q) { return 63 - __builtin_clzll(q); }

}  // namespace

extern "C" int rc_total_sum_batch(rc_context* c, uint32_t count, const rc_ciphertext* cts, uint32_t active_slots,
                                  const rc_ksk* const* step_keys, uint32_t key_count, rc_ciphertext* out,
                                  void* stream) {
  return guarded("rc_total_sum_batch", [&] {
    require(c && cts && out, "arguments must not be null");
    if (count == 0) return;
    Algo A(c, stream);
    fold(A, std::vector<rc_ciphertext>(cts, cts + count), active_slots, step_keys, key_count,
         "missing total-sum rotation key for step ", out);
  });
}

extern "C" int rc_halevi_shoup_batch(rc_context* c, uint32_t count, const rc_ciphertext* cts, const double* plain,
                                     uint32_t plain_len, const rc_ksk* const* step_keys, uint32_t key_count,
                                     rc_ciphertext* out, void* stream) {
  return guarded("rc_halevi_shoup_batch", [&] {
    require(c && cts && plain && out, "arguments must not be null");
    if (count == 0) return;
    Algo A(c, stream);
    const size_t half = A.N / 2;
    require(plain_len <= half, "plaintext slot vector cannot exceed the CKKS slot count");
    require(plain_len > 0, "plaintext slot vector cannot be empty");
    // mult_plain_slots_real (context/ops.rs:39-48): encode at the ciphertext's level and scale, mult_plain
    // (scale doubles), rescale
    std::vector<rc_ciphertext> in(cts, cts + count), prods(count), accs(count);
    std::vector<double> slots((size_t)count * 2 * half, 0.0);
    for (uint32_t i = 0; i < count; ++i)
      for (uint32_t k = 0; k < plain_len; ++k) slots[(size_t)i * 2 * half + 2 * k] = plain[(size_t)i * plain_len + k];
    double* dslots = (double*)A.pool.take(slots.size());
    // a copy from pageable memory returns once the source has been staged, so `slots` may go at return
    cuda_check(cudaMemcpyAsync(dslots, slots.data(), slots.size() * 8, cudaMemcpyHostToDevice, A.s), "slots");
    std::vector<const uint64_t*> plains(count);
    bool uniform = true;
    for (uint32_t i = 0; i < count; ++i)
      uniform = uniform && in[i].level == in[0].level && in[i].scale_bits == in[0].scale_bits;
    if (uniform) {  // one batched encode
      const size_t pl = (size_t)(in[0].level + 1) * A.N;
      uint64_t* p = A.pool.take(pl * count);
      ok(rc_encode_device(c, dslots, count, in[0].level, (uint32_t)in[0].scale_bits, p, A.s));
      for (uint32_t i = 0; i < count; ++i) plains[i] = p + i * pl;
    } else {
      for (uint32_t i = 0; i < count; ++i) {
        uint64_t* p = A.pool.take((size_t)(in[i].level + 1) * A.N);
        ok(rc_encode_device(c, dslots + (size_t)i * 2 * half, 1, in[i].level, (uint32_t)in[i].scale_bits, p, A.s));
        plains[i] = p;
      }
    }
    for (uint32_t i = 0; i < count; ++i) {
      prods[i] = A.fresh(in[i].level, in[i].scale_bits);
      accs[i] = A.fresh(in[i].level > 0 ? in[i].level - 1 : 0, 0);
    }
    ok(rc_multiply_plain_rns_batch(c, count, in.data(), plains.data(), prods.data(), A.s));
    for (uint32_t i = 0; i < count; ++i) prods[i].scale_bits = in[i].scale_bits + in[i].scale_bits;
    ok(rc_rescale_batch(c, count, prods.data(), accs.data(), A.s));
    fold(A, accs, plain_len, step_keys, key_count, "missing rotation key for step ", out);
  });
}

extern "C" int rc_paterson_stockmeyer_batch(rc_context* c, uint32_t count, const rc_ciphertext* cts,
                                            const double* coefficients, uint32_t terms,
                                            const rc_ksk* const* relin_keys, uint32_t key_levels,
                                            rc_ciphertext* out, void* stream) {
  return guarded("rc_paterson_stockmeyer_batch", [&] {
    require(c && cts && out && (terms == 0 || coefficients), "arguments must not be null");
    require(terms > 0, "polynomial must contain at least one coefficient");
    if (count == 0) return;
    Algo A(c, stream);
    // floor(log2 q_level) of the context's chain (the crate's scale rule)
    auto qbits = [&](int level) -> int { return floor_log2_u64(c->mod[level]); };
    std::vector<rc_ciphertext> in(cts, cts + count);
    const int level = in[0].level, in_scale = in[0].scale_bits;
    for (const auto& ct : in)
      require(ct.level == level && ct.scale_bits == in_scale, "a batch must share level and scale");

    auto constant_ct = [&](int lv, int scale, double value) {  // paterson_stockmeyer.rs:311-336
      rc_ciphertext z = A.fresh(lv, scale);
      cuda_check(cudaMemsetAsync(z.data, 0, 2 * (size_t)(lv + 1) * A.N * 8, A.s), "zero");
      if (value != 0.0) ok(rc_poly_add(c, z.data, A.constant(value, lv, scale), z.data, lv + 1, 0, A.s));
      return z;
    };
    auto write_out = [&](const std::vector<rc_ciphertext>& r) {
      for (uint32_t i = 0; i < count; ++i) {
        cuda_check(cudaMemcpyAsync(out[i].data, r[i].data, 2 * (size_t)(r[i].level + 1) * A.N * 8,
                                   cudaMemcpyDeviceToDevice, A.s),
                   "copy");
        out[i].level = r[i].level;
        out[i].scale_bits = r[i].scale_bits;
      }
    };
    if (terms == 1) {
      std::vector<rc_ciphertext> r(count);
      for (auto& x : r) x = constant_ct(level, in_scale, coefficients[0]);
      write_out(r);
      return;
    }
    const int b = (int)ps_block_size(terms), blocks = (int)((terms + b - 1) / b);
    const std::vector<int> req = ps_required_levels(level, terms);
    require(!req.empty(), "Paterson-Stockmeyer multiplication levels must be non-empty");
    int working = 1 << 30;
    for (int lv : req) working = std::min(working, qbits(lv));
    const int coeff_scale = working - in_scale;
    require(coeff_scale >= 0, "Paterson-Stockmeyer working scale must dominate the input ciphertext scale");

    auto lift_all = [&](const std::vector<rc_ciphertext>& cs, int target) {  // paterson_stockmeyer.rs:230-254
      require(cs[0].scale_bits <= target, "cannot lower ciphertext scale with a plaintext-one lift");
      if (cs[0].scale_bits == target) return cs;
      return A.mul_plain(cs, A.constant(1.0, cs[0].level, target - cs[0].scale_bits), target);
    };
    auto truncate_all = [&](const std::vector<rc_ciphertext>& cs, int lv) {  // paterson_stockmeyer.rs:221-228
      require(lv <= cs[0].level, "target level cannot exceed ciphertext level");
      std::vector<rc_ciphertext> o(cs.size());
      for (size_t i = 0; i < cs.size(); ++i) o[i] = A.truncate(cs[i], lv);
      return o;
    };
    auto mult_relin = [&](const std::vector<rc_ciphertext>& lhs, const std::vector<rc_ciphertext>& rhs) {
      const int lv = lhs[0].level;
      if (lv < 0 || (uint32_t)lv >= key_levels || !relin_keys[lv])
        fail(RC_ERR_INVALID_ARGUMENT, "missing Paterson-Stockmeyer relinearization key at level " + std::to_string(lv));
      std::vector<rc_ciphertext> o(lhs.size());
      std::vector<const rc_ksk*> ks(lhs.size(), relin_keys[lv]);
      for (size_t i = 0; i < lhs.size(); ++i) o[i] = A.fresh(lv > 0 ? lv - 1 : 0, 0);
      ok(rc_mult_relinearized_batch(c, (uint32_t)lhs.size(), lhs.data(), rhs.data(), ks.data(), o.data(), A.s));
      return o;
    };

    // baby powers x, x^2, ..., x^b (paterson_stockmeyer.rs:146-173; each lifted to the input scale)
    const std::vector<rc_ciphertext> base = lift_all(in, in_scale);
    std::vector<std::vector<rc_ciphertext>> powers{base};
    for (int e = 2; e <= b; ++e) {
      const std::vector<rc_ciphertext>& prev = powers.back();
      const std::vector<rc_ciphertext> aligned_prev = lift_all(prev, in_scale);
      const std::vector<rc_ciphertext> aligned_base = truncate_all(base, prev[0].level);
      powers.push_back(lift_all(mult_relin(aligned_prev, aligned_base), in_scale));
    }
    const std::vector<rc_ciphertext> giant = powers.back();
    require(giant[0].level + 1 >= blocks, "polynomial degree is too large for the available CKKS level budget");
    const int top = giant[0].level;

    auto evaluate_block = [&](int bi, int target_level) {  // paterson_stockmeyer.rs:175-219
      std::vector<rc_ciphertext> accs(count);
      for (auto& x : accs) x = constant_ct(target_level, working, 0.0);
      for (int off = 0; off < b; ++off) {
        const int k = bi * b + off;
        if (k >= (int)terms) break;
        const double cf = coefficients[k];
        if (cf == 0.0) continue;
        if (off == 0) {
          for (auto& x : accs)
            ok(rc_poly_add(c, x.data, A.constant(cf, x.level, x.scale_bits), x.data, x.level + 1, 0, A.s));
          continue;
        }
        const std::vector<rc_ciphertext>& power = powers[off - 1];
        const std::vector<rc_ciphertext> aligned = lift_all(truncate_all(power, target_level), power[0].scale_bits);
        const std::vector<rc_ciphertext> t =
            A.mul_plain(aligned, A.constant(cf, aligned[0].level, coeff_scale), aligned[0].scale_bits + coeff_scale);
        accs = A.add(accs, t);
      }
      return accs;
    };
    std::vector<std::vector<rc_ciphertext>> block_out;
    for (int bi = 0; bi < blocks; ++bi) block_out.push_back(evaluate_block(bi, top - (blocks - 1 - bi)));
    std::vector<rc_ciphertext> result = block_out.back();
    for (int bi = blocks - 2; bi >= 0; --bi) {
      const std::vector<rc_ciphertext> aligned_giant =
          lift_all(truncate_all(giant, result[0].level), result[0].scale_bits);
      const std::vector<rc_ciphertext> multiplied = mult_relin(result, aligned_giant);
      result = A.add(lift_all(multiplied, result[0].scale_bits), block_out[bi]);
    }
    write_out(result);
  });
}

// apply_diagonal_linear_transform (src/ckks/bootstrapping/linear_transform.rs:109-150, 213-252) for a batch
// sharing one set of packed diagonals: baby-step rotations of every ciphertext in one call, all babies to the
// NTT domain in one call, each inner sum as one NTT-domain multiply-accumulate, the giant-step rotations of all
// inner sums in one call, the adds in the crate's giant order, one rescale.  diag_ntt[g * baby_step + j] is
// the NTT-domain diagonal g*b+j pre-rotated by g*b (null past the dimension); baby_keys[s-1] rotates by s,
// giant_keys[g-1] by g*b.
extern "C" int rc_bsgs_apply_batch(rc_context* c, uint32_t count, const rc_ciphertext* cts, uint32_t dimension,
                                   uint32_t baby_step, const uint64_t* const* diag_ntt, uint32_t giants,
                                   int32_t diag_level, int32_t diag_scale_bits, const rc_ksk* const* baby_keys,
                                   const rc_ksk* const* giant_keys, rc_ciphertext* out, void* stream) {
  return guarded("rc_bsgs_apply_batch", [&] {
    require(c && cts && diag_ntt && out, "arguments must not be null");
    if (count == 0) return;
    for (uint32_t i = 0; i < count; ++i) {
      require(cts[i].level == diag_level, "packed diagonals must match the ciphertext level");
      require(cts[i].scale_bits == diag_scale_bits, "packed diagonals must match the ciphertext scale");
    }
    Algo A(c, stream);
    const int lv = diag_level, limbs = lv + 1;
    const uint32_t b = std::min(baby_step, dimension);
    const size_t ct_words = 2 * (size_t)limbs * A.N;
    // precompute_baby_rotations (213-232): rotations by 1 .. b-1 of every ciphertext, hoisted (one
    // decomposition of each ciphertext serves its b-1 rotations)
    std::vector<rc_ciphertext> jobs, rot;
    std::vector<const rc_ksk*> keys;
    for (uint32_t st = 1; st < b; ++st) {
      if (!baby_keys || !baby_keys[st - 1])
        fail(RC_ERR_INVALID_ARGUMENT, "missing input rotation key for BSGS baby step " + std::to_string(st));
      keys.push_back(baby_keys[st - 1]);
    }
    // the babies of ciphertext i in the NTT domain: babies[(i * b + j)] (j = 0 is the ciphertext itself)
    uint64_t* babies = A.pool.take(ct_words * count * b);
    if (b > 1) {
      rot.resize((size_t)count * (b - 1));
      for (uint32_t i = 0; i < count; ++i)
        for (uint32_t st = 1; st < b; ++st)
          rot[(size_t)i * (b - 1) + st - 1] = rc_ciphertext{babies + ((size_t)i * b + st) * ct_words, lv, diag_scale_bits};
      ok(rc_rotate_hoisted(c, count, cts, b - 1, keys.data(), rot.data(), A.s));
    }
    for (uint32_t i = 0; i < count; ++i)
      cuda_check(cudaMemcpyAsync(babies + (size_t)i * b * ct_words, cts[i].data, ct_words * 8,
                                 cudaMemcpyDeviceToDevice, A.s),
                 "copy");
    ok(rc_ntt_forward(c, babies, count * b * 2, (uint32_t)limbs, 0, A.s));
    // apply_giant_step_terms (234-252): inner[i][g] = sum_j mult_plain(baby_j, diag_{g,j})
    std::vector<std::vector<rc_ciphertext>> inner(count, std::vector<rc_ciphertext>(giants));
    std::vector<std::vector<bool>> present(count, std::vector<bool>(giants, false));
    const bool fused = b == baby_step && bsgs_inner_applies(b, giants);
    if (fused) {
      // every inner sum of the batch in one launch, then one batched inverse NTT
      const uint32_t tile = (uint32_t)bsgs_tile(b);
      const size_t pl = (size_t)limbs * A.N;
      uint64_t* zero = A.pool.take(pl);
      cuda_check(cudaMemsetAsync(zero, 0, pl * 8, A.s), "zero diagonal");
      DiagTab tab{};
      std::vector<bool> row(giants, false);
      for (uint32_t g = 0; g < giants; ++g)
        for (uint32_t j = 0; j < tile; ++j) {
          const uint64_t* d = j < b ? diag_ntt[(size_t)g * b + j] : nullptr;
          tab.p[g * tile + j] = d ? d : zero;
          if (d) row[g] = true;
        }
      uint64_t* sums = A.pool.take(ct_words * count * giants);
      bsgs_inner(c, babies, tab, sums, (int)count, (int)b, (int)giants, limbs, A.s);
      ok(rc_ntt_inverse(c, sums, count * giants * 2, (uint32_t)limbs, 0, A.s));
      for (uint32_t i = 0; i < count; ++i)
        for (uint32_t g = 0; g < giants; ++g) {
          inner[i][g] = rc_ciphertext{sums + ((size_t)i * giants + g) * ct_words, lv, diag_scale_bits + diag_scale_bits};
          present[i][g] = row[g];
        }
    }
    for (uint32_t i = 0; i < count && !fused; ++i) {
      for (uint32_t g = 0; g < giants; ++g) {
        std::vector<rc_ciphertext> terms;
        std::vector<const uint64_t*> plains;
        for (uint32_t j = 0; j < baby_step; ++j) {
          const uint64_t* d = diag_ntt[(size_t)g * baby_step + j];
          if (!d) continue;
          require(j < b, "internal: diagonal beyond the baby steps");
          terms.push_back(rc_ciphertext{babies + ((size_t)i * b + j) * ct_words, lv, diag_scale_bits});
          plains.push_back(d);
        }
        if (terms.empty()) continue;
        inner[i][g] = A.fresh(lv, 0);
        ok(rc_mult_plain_accumulate(c, (uint32_t)terms.size(), terms.data(), 1, plains.data(), 1, &inner[i][g], A.s));
        present[i][g] = true;
      }
    }
    // giant-step rotations of the unrescaled inner sums, jobs sharing a key adjacent
    jobs.clear();
    keys.clear();
    std::vector<std::pair<uint32_t, uint32_t>> where;
    for (uint32_t g = 1; g < giants; ++g) {
      for (uint32_t i = 0; i < count; ++i) {
        if (!present[i][g]) continue;
        if (!giant_keys || !giant_keys[g - 1])
          fail(RC_ERR_INVALID_ARGUMENT,
               "missing input rotation key for BSGS giant step " + std::to_string(g * baby_step));
        jobs.push_back(inner[i][g]);
        keys.push_back(giant_keys[g - 1]);
        where.emplace_back(i, g);
      }
    }
    if (!jobs.empty()) {
      rot.assign(jobs.size(), rc_ciphertext{});
      for (size_t k = 0; k < jobs.size(); ++k) rot[k] = A.fresh(lv, jobs[k].scale_bits);
      ok(rc_rotate_batch(c, (uint32_t)jobs.size(), jobs.data(), keys.data(), rot.data(), A.s));
      for (size_t k = 0; k < jobs.size(); ++k) inner[where[k].first][where[k].second] = rot[k];
    }
    // the adds in giant order (one batched call per giant step over all ciphertexts), then one rescale
    std::vector<rc_ciphertext> accs(count);
    std::vector<uint32_t> next(count, 0);
    for (uint32_t i = 0; i < count; ++i) {
      uint32_t g = 0;
      while (g < giants && !present[i][g]) ++g;
      require(g < giants, "diagonal transform must contain at least one non-empty giant-step block");
      accs[i] = inner[i][g];
      next[i] = g + 1;
    }
    for (uint32_t g = 1; g < giants; ++g) {
      std::vector<rc_ciphertext> lhs, rhs;
      std::vector<uint32_t> idx;
      for (uint32_t i = 0; i < count; ++i)
        if (g >= next[i] && present[i][g]) {
          lhs.push_back(accs[i]);
          rhs.push_back(inner[i][g]);
          idx.push_back(i);
        }
      if (lhs.empty()) continue;
      const std::vector<rc_ciphertext> sum = A.add(lhs, rhs);
      for (size_t k = 0; k < idx.size(); ++k) accs[idx[k]] = sum[k];
    }
    ok(rc_rescale_batch(c, count, accs.data(), out, A.s));
  });
}
