// Host-side context of the GPU library: parameters, device-resident tables,
// per-stream scratch.  Internal to the library (the ABI exposes rc_context as
// an opaque handle).
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <tuple>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/rnsckks_gpu.h"
#include "bignum.hpp"
#include "kernels.cuh"

namespace rc {

struct ApiError : std::runtime_error {
  int code;
  ApiError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] inline void fail(int code, const std::string& msg) { throw ApiError(code, msg); }
inline void require(bool cond, const std::string& msg) {
  if (!cond) fail(RC_ERR_INVALID_ARGUMENT, msg);
}
void cuda_check(cudaError_t e, const char* what);
void set_last_error(const std::string& m);

// Runs an entry point's body: an ApiError becomes its status code and rc_last_error message; allocation
// failures and CUDA errors become RC_ERR_OUT_OF_MEMORY / RC_ERR_CUDA.  Nothing escapes the C ABI.
template <class F>
int guarded(F&& f) {
  try {
    f();
    return RC_OK;
  } catch (const ApiError& e) {
    set_last_error(e.what());
    return e.code;
  } catch (const std::bad_alloc&) {
    set_last_error("host allocation failed");
    return RC_ERR_OUT_OF_MEMORY;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return RC_ERR_CUDA;
  }
}

// A public entry point's body inside an NVTX range named after it (when rc_profile_enable turned NVTX on).
struct OpRange {
  bool on;
  explicit OpRange(const char* name) : on(nvtx_enabled()) {
    if (on) nvtx_push(name);
  }
  ~OpRange() {
    if (on) nvtx_pop();
  }
};
template <class F>
int guarded(const char* op, F&& f) {
  OpRange r(op);
  return guarded(std::forward<F>(f));
}

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() {}
  explicit DevBuf(size_t b);
  ~DevBuf();
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
};

struct LevelInfo {
  int limbs = 0;
  size_t bits = 0;     // bits of Q_limbs
  int digits = 0;      // num_decomp_digits(bits, 30)
  DecompTab dt{};
  std::shared_ptr<DevBuf> buf;
};

struct Workspace {
  std::unique_ptr<DevBuf> dev;
  void* host_pinned = nullptr;
  size_t host_bytes = 0;
  ~Workspace();
};

// Streams, events and two device staging slots of the pipelined host-buffer entry points: chunk k's
// inputs are copied in while chunk k-1 computes and chunk k-2's results are copied out.  All inputs go
// through one copy stream in job order: the host link serves one copy at a time, so a second input stream
// would only delay the first chunk's other operand.  Consecutive chunks compute on alternating streams
// (comp, comp2), so one chunk's kernels fill the SMs the other's leave idle.
//
// Asynchronous calls (rc_mult_relinearized_batch_host_async) return once their work is enqueued, so the next
// call's copies in run while the previous call computes.  The phased form then takes its staging slots from
// alternating sets (`ring`), each slot guarded by two persistent events: `consumed` (its inputs were read by
// the last call that used it) before new copies in, `drained` (its outputs were copied out) before new
// results; `last` marks the end of the latest call's copies out (rc_host_join).
struct HostPipe {
  cudaStream_t in = nullptr, comp = nullptr, out = nullptr, comp2 = nullptr;
  std::unique_ptr<DevBuf> slot[4];
  cudaEvent_t consumed[4] = {}, drained[4] = {};
  bool used[4] = {};
  cudaEvent_t last = nullptr;
  bool pending = false;  // asynchronous work issued since the last join
  int ring = 0;
  std::vector<cudaEvent_t> events;
  cudaEvent_t event();  // from the pool, created on first use
  size_t next = 0;      // events handed out in the current call
  ~HostPipe();
};

}  // namespace rc

struct rc_context {
  int N = 0, log_n = 0, n1 = 0;
  int L = 0, K = 0;
  int scale_bits = 0;
  int device = 0;
  bool lazy = false;   // every prime < 2^58
  bool lazy_inv = false;  // every prime < 2^55 (2^9 q < 2^64: an unreduced 8-stage inverse pass)
  bool mac64 = false;  // 64-bit per-term Montgomery accumulation in the key product
  bool wide_ok = false;  // exact integer key product under the four internal primes available
  rc::WidePrimes wp{};    // internal primes, transform constants and twiddle tables (wide_tw)
  rc::WideTab wide{};     // CRT back to the scheme primes (tables in wide_buf)
  std::unique_ptr<rc::DevBuf> wide_buf, wide_tw;
  std::unique_ptr<rc::DevBuf> fft_buf;  // device encoder tables (built on first use, under mu)
  // encoded constant plaintexts (all slots = value) by (value, level, scale_bits) for the native schedules;
  // complete before they are handed out, capped in count (under mu)
  std::map<std::tuple<double, int, int>, std::unique_ptr<rc::DevBuf>> const_cache;
  std::vector<uint64_t> mod, root;  // Q then P
  std::unique_ptr<rc::DevBuf> pc_buf, tw_buf, md_buf, rt_buf;
  rc::PrimeConst* d_pc = nullptr;
  rc::Twiddle* d_twf = nullptr;
  rc::Twiddle* d_twi = nullptr;
  std::vector<rc::LevelInfo> levels;  // index = limb count (1..L)
  std::unique_ptr<rc::DevBuf> dt_buf;
  rc::DecompTab* d_dts = nullptr;     // levels[l].dt for l = 0..L on the device (entry 0 unused)
  rc::ModDownTab md{};
  rc::RescaleTab rt{};
  std::vector<uint64_t> host_halfP;
  std::mutex mu;
  std::map<cudaStream_t, std::unique_ptr<rc::Workspace>> ws;
  std::map<cudaStream_t, std::unique_ptr<rc::HostPipe>> pipes;  // per caller stream
  size_t scratch_budget = size_t(256) << 20;
  // tunables (rc_tune_set): results never depend on them
  int ks_jobs = 32;     // jobs per key-switch launch (one key read serves them), <= MAXP / 2
  int mac_bc = 8;       // most jobs per CTA of the wide key product (1, 2, 4 or 8)
  int host_chunk = 8;   // jobs per stage of the pipelined host-buffer entry
  int host_edge = 2;    // its first and last stages have host_chunk / host_edge jobs
  bool fuse_tensor = true;  // forward rows + tensor + inverse rows in one kernel
  int host_phased = 1;  // host-buffer batches: key-product groups (0 = staged, 1 or 2 phased groups)
  bool mixed_levels = true;  // mixed-level key-switch batches: one launch per pass over all levels
  int ml_jobs = rc::ML_MAXJ;  // jobs per mixed-level chunk (each chunk one launch per pass)
  int col_ctas = 3;           // 64-bit column passes: CTAs per SM (2 or 3)
  int row_polys = 16;         // 64-bit row passes: polynomials per block (8 or 16)
  int tensor_jobs = 4;        // tensor + inverse row pass: jobs per block (1..16)
  int r16 = rc::r16::R16_DEFAULT;  // N = 2^16: passes in the 16-residues-per-lane form (bits; also wp.r16)

  rc::NttArgs ntt() const {
    rc::NttArgs a;
    a.pc = d_pc;
    a.tw_fwd = d_twf;
    a.tw_inv = d_twi;
    a.log_n = log_n;
    a.n1 = n1;
    a.lazy = lazy ? 1 : 0;
    a.lazy_inv = lazy_inv ? 1 : 0;
    a.col_ctas = col_ctas;
    a.row_polys = row_polys;
    a.tensor_jobs = tensor_jobs;
    a.r16 = r16;
    return a;
  }
};

struct rc_ksk {
  rc_context* ctx = nullptr;
  // per-limb form [limbs][digits][2][N], NTT domain, Montgomery form (null when the wide form is kept)
  std::shared_ptr<rc::DevBuf> buf;
  uint64_t* data = nullptr;
  // wide form: uint2 residues mod the internal prime pairs, NTT domain, tiled [limbs][pair][N/32][digits][2][32]
  std::shared_ptr<rc::DevBuf> wbuf;
  uint64_t* wdata = nullptr;
  uint32_t digits = 0;
  int32_t level = 0;
  uint32_t aux = 0;
  uint64_t galois = 0;
  // RNS-hybrid key (rc_ksk_upload_dnum): alpha limbs per group, digits = dnum groups; `data` then holds the
  // key [dnum][2][level + 1 + aux][N] in the NTT domain and mbuf the ModUp tables (0 for gadget keys)
  uint32_t alpha = 0;
  std::shared_ptr<rc::DevBuf> mbuf;
  uint32_t limbs() const { return (uint32_t)level + 1 + aux; }
};

namespace rc {
// context queries shared by the C ABI's translation units (defined in capi.cu)
const LevelInfo& context_level(const rc_context* c, int limbs);
bool context_wide_applies(const rc_context* c, int qlimbs, int K, int D);
void context_check_ct(const rc_context* c, const rc_ciphertext* ct, const char* name);
uint64_t context_galois_inverse(const rc_context* c, uint64_t g);
LimbMap context_basis_map(const rc_context* c, uint32_t limbs, int32_t with_aux);
void* context_workspace(rc_context* c, cudaStream_t s, size_t bytes);
// host FFT values for the device encoder (encode.cpp)
void fft_tables(size_t n, std::vector<double>& tw_inv, std::vector<double>& tw_fwd, std::vector<double>& xi_neg,
                std::vector<double>& xi_pos);
}  // namespace rc
