// Allocation-free variant of the RNS polynomial product (rc_poly_multiply).
//
// Who needs it: callers that must not allocate device memory from inside this
// library -- a host that reserves the whole GPU pool up front and forbids
// allocation by plugins, or a latency-critical loop that cannot afford the
// device-wide synchronisation cudaMalloc/cudaFree imply.  This entry point
// takes its scratch from a fixed array compiled into the library instead of
// the per-stream workspace the other entry points grow with cudaMalloc.
//
// Limits and behaviour:
//  * The scratch is a file-scope __device__ array of NOALLOC_SCRATCH_ELEMS
//    64-bit words (16 MiB).  Every GPU that loads the library holds it until
//    the process exits.  A product needs 2 * limbs * N words, so limbs * N
//    may be at most NOALLOC_SCRATCH_ELEMS / 2 (e.g. N = 2^16 with 16 limbs);
//    larger requests are rejected with RC_ERR_INVALID_ARGUMENT.
//  * The array's device address is looked up with cudaGetSymbolAddress on the
//    first call on each device (with that device current), so the first call
//    on a device should come before any CUDA graph capture.
//  * All calls share the one array and it keeps the previous call's contents.
//    Nothing needs to start at zero: both halves are fully written by the
//    forward transforms before they are read.  Calls whose kernels overlap on
//    the GPU (different streams, or different host threads) race on the
//    array; issue them on one stream or serialise them.
#include <mutex>

#include "context.hpp"

namespace rc {
namespace {

constexpr size_t NOALLOC_SCRATCH_ELEMS = size_t(2) << 20;  // 16 MiB of u64
__device__ __align__(256) u64 g_noalloc_scratch[NOALLOC_SCRATCH_ELEMS];

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
u64* g_addr[MAX_DEVICES] = {};

u64* scratch_address(int device) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[device]) {
    void* p = nullptr;
    cuda_check(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(no-alloc scratch)");
    g_addr[device] = (u64*)p;
  }
  return g_addr[device];
}

}  // namespace
}  // namespace rc

using namespace rc;

extern "C" int rc_poly_multiply_noalloc(rc_context* c, const uint64_t* a, const uint64_t* b, uint64_t* out,
                                        uint32_t limbs, int32_t with_aux, void* stream) {
  return guarded("rc_poly_multiply_noalloc", [&] {
    require(c && a && b && out, "arguments must not be null");
    // the same limb and basis checks (and messages) as rc_poly_multiply
    const LimbMap map = context_basis_map(c, limbs, with_aux);
    const size_t pl = (size_t)limbs * c->N;
    if (2 * pl > NOALLOC_SCRATCH_ELEMS)
      fail(RC_ERR_INVALID_ARGUMENT, "rc_poly_multiply_noalloc: limbs * N = " + std::to_string(pl) +
                                        " exceeds the static scratch limit of " +
                                        std::to_string(NOALLOC_SCRATCH_ELEMS / 2));
    int device = 0;
    cuda_check(cudaGetDevice(&device), "cudaGetDevice");
    if (device < 0 || device >= MAX_DEVICES) fail(RC_ERR_UNSUPPORTED, "device index out of range");
    u64* scratch = scratch_address(device);
    cudaStream_t s = (cudaStream_t)stream;
    PtrTab src{}, dst{};
    src.p[0] = const_cast<uint64_t*>(a);
    src.p[1] = const_cast<uint64_t*>(b);
    dst.p[0] = scratch;
    dst.p[1] = scratch + pl;
    ntt_forward(c->ntt(), src, dst, 2, (int)limbs, map, s);
    PtrTab x{}, y{}, o{};
    x.p[0] = scratch;
    y.p[0] = scratch + pl;
    ew_binary(EwOp::MulMont, c->d_pc, x, y, 0, x, 1, (int)limbs, map, c->N, s);
    o.p[0] = out;
    NttArgs inv = c->ntt();
    inv.mont_out = 1;  // takes out the Montgomery products' 2^-64
    ntt_inverse(inv, x, o, 1, (int)limbs, map, s);
    cuda_check(cudaGetLastError(), "rc_poly_multiply_noalloc");
  });
}
