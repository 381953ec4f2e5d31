// Seeded samplers on the device for key generation and encryption: the distributions of the reference's
// src/rns/keys.rs (uniform residues as 64 random bits mod q, sample_uniform_poly 87-99; rounded normal with
// sigma 3.19, sample_gaussian_i64 82-85 and sample_error_poly 101-121; uniform ternary {0, 1, -1},
// sample_ternary_poly 123-147), drawn from a counter-based generator so every coefficient is an independent
// function of (seed, stream id, index) and a whole polynomial is one launch.  The reference seeds from the
// operating system, so its samples are not reproducible and are not compared value for value; what is fixed
// is the distribution and, here, reproducibility per seed.
//
// Generator: Philox4x32 with 10 rounds (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
// 1, 2, 3", SC 2011): a 128-bit counter and a 64-bit key, each round two 32x32->64 multiplies by the
// published constants and a key bump by the published Weyl increments.
#include <cmath>

#include "context.hpp"

using namespace rc;

namespace {

struct U4 {
  uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
  constexpr uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  constexpr uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return c;
}

__device__ __forceinline__ U4 draw(uint64_t seed, uint64_t stream_id, uint64_t index) {
  return philox4x32_10(U4{(uint32_t)index, (uint32_t)(index >> 32), (uint32_t)stream_id, (uint32_t)(stream_id >> 32)},
                       (uint32_t)seed, (uint32_t)(seed >> 32));
}

// r mod q for any 64-bit r (one_s = floor(2^64 / q)): the Shoup reduction lands in [0, 2q)
__device__ __forceinline__ u64 mod_q(u64 r, u64 q, u64 one_s) {
  const u64 t = r - __umul64hi(r, one_s) * q;
  return t >= q ? t - q : t;
}

__global__ void k_sample_uniform(const PrimeConst* pc, LimbMap map, int limbs, int log_n, uint64_t seed,
                                 uint64_t stream_id, u64* out) {
  const size_t total = (size_t)limbs << log_n;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
    const PrimeConst& p = pc[map.prime((int)(e >> log_n))];
    const U4 r = draw(seed, stream_id, e);
    out[e] = mod_q(((u64)r.y << 32) | r.x, p.q, p.one_s);  // rng.gen::<u64>() % q
  }
}

// round(N(0, sigma)) by Box-Muller on two 53-bit uniforms, rounding half away from zero like f64::round
__global__ void k_sample_error(const PrimeConst* pc, LimbMap map, int limbs, int log_n, uint64_t seed,
                               uint64_t stream_id, double sigma, u64* out) {
  const size_t N = (size_t)1 << log_n;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < N; x += (size_t)gridDim.x * blockDim.x) {
    const U4 r = draw(seed, stream_id, x);
    const double u1 = (double)(((((u64)r.y << 32) | r.x) >> 11) + 1) * 0x1.0p-53;  // (0, 1]
    const double u2 = (double)((((u64)r.w << 32) | r.z) >> 11) * 0x1.0p-53;        // [0, 1)
    const double z = sqrt(-2.0 * log(u1)) * cospi(2.0 * u2) * sigma;
    const int64_t v = (int64_t)round(z);
    for (int j = 0; j < limbs; ++j) {
      const u64 q = pc[map.prime(j)].q;
      out[(size_t)j * N + x] = v >= 0 ? (u64)v : q - (u64)(-v);
    }
  }
}

// uniform {0, 1, -1} (gen_range(0..3): 0 -> 0, 1 -> 1, 2 -> -1) by rejection of the one 32-bit value above
// the largest multiple of 3
__global__ void k_sample_ternary(const PrimeConst* pc, LimbMap map, int limbs, int log_n, uint64_t seed,
                                 uint64_t stream_id, u64* out) {
  const size_t N = (size_t)1 << log_n;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < N; x += (size_t)gridDim.x * blockDim.x) {
    const U4 r = draw(seed, stream_id, x);
    const uint32_t w[4] = {r.x, r.y, r.z, r.w};
    uint32_t v = 0;
#pragma unroll
    for (int i = 3; i >= 0; --i)
      if (w[i] != 0xFFFFFFFFu) v = w[i] % 3;  // the first accepted word wins
    for (int j = 0; j < limbs; ++j) {
      const u64 q = pc[map.prime(j)].q;
      out[(size_t)j * N + x] = v == 0 ? 0 : (v == 1 ? 1 : q - 1);
    }
  }
}

int grid_for(size_t items) {
  const size_t g = (items + 255) / 256;
  return (int)(g < 1 ? 1 : (g > 152 * 32 ? 152 * 32 : g));
}

enum class Dist { uniform, error, ternary };

int sample_entry(rc_context* c, Dist d, uint64_t seed, uint64_t stream_id, uint64_t* out, uint32_t limbs,
                 int32_t with_aux, void* stream) {
  return guarded([&] {
    require(c && out, "arguments must not be null");
    const LimbMap map = context_basis_map(c, limbs, with_aux);
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = (size_t)c->N;
    if (d == Dist::uniform)
      k_sample_uniform<<<grid_for(n * limbs), 256, 0, s>>>(c->d_pc, map, (int)limbs, c->log_n, seed, stream_id, out);
    else if (d == Dist::error)
      k_sample_error<<<grid_for(n), 256, 0, s>>>(c->d_pc, map, (int)limbs, c->log_n, seed, stream_id, 3.19, out);
    else
      k_sample_ternary<<<grid_for(n), 256, 0, s>>>(c->d_pc, map, (int)limbs, c->log_n, seed, stream_id, out);
    cuda_check(cudaGetLastError(), "sample launch");
  });
}

}  // namespace

extern "C" int rc_sample_uniform(rc_context* c, uint64_t seed, uint64_t stream_id, uint64_t* out, uint32_t limbs,
                                 int32_t with_aux, void* stream) {
  OpRange op_range("rc_sample_uniform");
  return sample_entry(c, Dist::uniform, seed, stream_id, out, limbs, with_aux, stream);
}

extern "C" int rc_sample_error(rc_context* c, uint64_t seed, uint64_t stream_id, uint64_t* out, uint32_t limbs,
                               int32_t with_aux, void* stream) {
  OpRange op_range("rc_sample_error");
  return sample_entry(c, Dist::error, seed, stream_id, out, limbs, with_aux, stream);
}

extern "C" int rc_sample_ternary(rc_context* c, uint64_t seed, uint64_t stream_id, uint64_t* out, uint32_t limbs,
                                 int32_t with_aux, void* stream) {
  OpRange op_range("rc_sample_ternary");
  return sample_entry(c, Dist::ternary, seed, stream_id, out, limbs, with_aux, stream);
}
