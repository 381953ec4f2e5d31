// Measured throughput of the integer multiply forms the kernels are built from (the roofline that bounds
// every kernel of the HMult+relin step): warp-wide instructions per SM per cycle for 32-bit IMAD, IMAD.HI,
// IMAD.WIDE with a 64-bit addend, 64-bit low product and __umul64hi, each as 8 independent dependency
// chains per thread over 8 CTAs of 256 threads per SM.
//
// A measurement probe, not part of the library: it is built into its own shared object
// (librnsckks_probe.so, loaded only by the benchmark and its test) so that librnsckks_gpu.so exports product
// entry points only.  No reference counterpart.
//
//   int rc_measure_multiply_rates(double* rates, void* stream);
//     rates[0] IMAD.WIDE (32x32->64 with a 64-bit addend), [1] 32-bit IMAD, [2] IMAD.HI, [3] 64-bit low
//     product, [4] __umul64hi; runs five short kernels on `stream` (about 30 ms).  Returns 0, or the
//     cudaError_t of the first failing CUDA call.
#include <cuda_runtime.h>

#include <cstdint>

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

extern "C" int rc_measure_multiply_rates(double* rates, void* stream) {
  if (!rates) return (int)cudaErrorInvalidValue;
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, sms = 0, khz = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev);
  if (e != cudaSuccess) return (int)e;
  const int blocks = sms * 8, threads = 256;
  uint32_t* out = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  e = cudaMalloc(&out, (size_t)blocks * threads * 4);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  for (int op = 0; op < 5 && e == cudaSuccess; ++op) {
    float ms = 0;
    for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {  // the first launch warms up
      e = cudaEventRecord(e0, s);
      switch (op) {
        case 0: k_mulrate<0><<<blocks, threads, 0, s>>>(out, 12345); break;
        case 1: k_mulrate<1><<<blocks, threads, 0, s>>>(out, 12345); break;
        case 2: k_mulrate<2><<<blocks, threads, 0, s>>>(out, 12345); break;
        case 3: k_mulrate<3><<<blocks, threads, 0, s>>>(out, 12345); break;
        default: k_mulrate<4><<<blocks, threads, 0, s>>>(out, 12345); break;
      }
      if (e == cudaSuccess) e = cudaGetLastError();
      if (e == cudaSuccess) e = cudaEventRecord(e1, s);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    }
    const double warp_ops = (double)blocks * threads / 32 * MR_ITERS * 8;
    const double cycles = ms * 1e-3 * khz * 1e3;
    rates[op] = warp_ops / sms / cycles;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (out) cudaFree(out);
  return (int)e;
}
