// Measured throughput of the integer multiply forms the kernels are built from (the roofline that bounds
// every kernel of the HMult+relin step): warp-wide instructions per SM per cycle for 32-bit IMAD, IMAD.HI,
// IMAD.WIDE with a 64-bit addend, 64-bit low product and __umul64hi, each as 8 independent dependency
// chains per thread over 8 CTAs of 256 threads per SM.  Measurement only; no reference counterpart.
#include <cstdint>

#include "context.hpp"

namespace {

constexpr int MR_ITERS = 2048;

template <int OP>
__global__ void k_mulrate(uint32_t* out, uint32_t seed) {
  uint32_t a[8];
  unsigned long long acc[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    a[i] = seed * (threadIdx.x + 7 * i + 1);
    acc[i] = a[i];
  }
  const uint32_t b = seed | 1;
  const unsigned long long b64 = ((unsigned long long)seed << 32) | (seed ^ 0x9e3779b9u);
  for (int it = 0; it < MR_ITERS; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      if (OP == 0) acc[i] = (unsigned long long)(uint32_t)acc[i] * b + acc[i];  // IMAD.WIDE.U32, 64-bit addend
      if (OP == 1) a[i] = a[i] * b + (uint32_t)it;                             // IMAD
      if (OP == 2) a[i] = __umulhi(a[i], b) | 1u;                              // IMAD.HI
      if (OP == 3) acc[i] = acc[i] * b64 + 1;                                  // 64-bit low product
      if (OP == 4) acc[i] = __umul64hi(acc[i], b64) | 1ull;                    // 64-bit high product
    }
  }
  uint32_t r = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) r += a[i] + (uint32_t)acc[i] + (uint32_t)(acc[i] >> 32);
  out[blockIdx.x * blockDim.x + threadIdx.x] = r;
}

}  // namespace

// rates[5]: IMAD.WIDE, IMAD, IMAD.HI, 64-bit low, 64-bit high (warp instructions per SM per SM cycle, using
// the device's reported clock); returns RC_OK or a CUDA error status
extern "C" int rc_measure_multiply_rates(double* rates, void* stream) {
  return rc::guarded([&] {
    rc::require(rates != nullptr, "arguments must not be null");
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, sms = 0, khz = 0;
    rc::cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
    rc::cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "attribute");
    rc::cuda_check(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev), "attribute");
    const int blocks = sms * 8, threads = 256;
    rc::DevBuf out((size_t)blocks * threads * 4);
    cudaEvent_t e0, e1;
    rc::cuda_check(cudaEventCreate(&e0), "cudaEventCreate");
    rc::cuda_check(cudaEventCreate(&e1), "cudaEventCreate");
    for (int op = 0; op < 5; ++op) {
      float ms = 0;
      for (int rep = 0; rep < 2; ++rep) {  // the first launch warms up
        rc::cuda_check(cudaEventRecord(e0, s), "cudaEventRecord");
        uint32_t* o = (uint32_t*)out.p;
        switch (op) {
          case 0: k_mulrate<0><<<blocks, threads, 0, s>>>(o, 12345); break;
          case 1: k_mulrate<1><<<blocks, threads, 0, s>>>(o, 12345); break;
          case 2: k_mulrate<2><<<blocks, threads, 0, s>>>(o, 12345); break;
          case 3: k_mulrate<3><<<blocks, threads, 0, s>>>(o, 12345); break;
          default: k_mulrate<4><<<blocks, threads, 0, s>>>(o, 12345); break;
        }
        rc::cuda_check(cudaEventRecord(e1, s), "cudaEventRecord");
        rc::cuda_check(cudaEventSynchronize(e1), "cudaEventSynchronize");
        rc::cuda_check(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
      }
      const double warp_ops = (double)blocks * threads / 32 * MR_ITERS * 8;
      const double cycles = ms * 1e-3 * khz * 1e3;
      rates[op] = warp_ops / sms / cycles;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  });
}
