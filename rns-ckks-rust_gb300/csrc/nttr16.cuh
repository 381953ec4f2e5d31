// 2^16-point transforms (four-step split 2^8 x 2^8) whose 256-point sub-transforms are held by 16 lanes with
// 16 residues each, two sub-transforms per warp, in two groups of four butterfly stages:
//   layout A: lane l holds elements l + 16 k (k = 0..15); stages 0..3 pair elements of one lane
//   layout B: lane l holds elements 16 l + k;             stages 4..7 pair elements of one lane
// One exchange through shared memory between the groups (the eight-residue form of nttcore.cuh needs two).
// Every shared-memory layout here is additive over the index bits (address = lane part + element part), so
// each access is a per-lane base register plus an immediate offset, and it is free of bank conflicts in both
// lane layouts:
//   column tile of 16 columns: element (r, c) at 17 (r mod 16) + 273 (r div 16) + c; in layout A the sixteen
//     lanes of a half-warp (one column; 8-byte accesses are served per half-warp) hit u64 banks l + c + const
//     (mod 16), all distinct; layout B the same with the roles of r mod 16 and r div 16 swapped;
//   row exchange buffer: element r of sub-transform s at (r mod 16) + 17 (r div 16) + 272 s.
// Twiddle tables are staged per column phase or row (255 entries), stages 4..7 stored lane-fastest so that the
// sixteen lanes of a sub-transform read sixteen consecutive entries.
//
// The butterflies are those of nttcore.cuh (Harvey's lazy Shoup Cooley-Tukey forward, Gentleman-Sande
// inverse; merged psi^bitrev twiddles, src/math/ntt.rs:92-130 and src/poly/mod.rs:134-175 of the reference for
// what they compute); only the assignment of elements to lanes differs, so every pass here is interchangeable
// with the corresponding pass of the eight-residue form (both read and write natural order).
#pragma once
#include "kernels.cuh"
#include "nttcore.cuh"
#include "wide.cuh"

namespace rc {
namespace r16 {

constexpr int TROW = 17;              // u64 slots between rows r and r+1 of a column tile (16 columns + 1)
constexpr int TBLK = 273;             // slots between rows r and r+16 (16 * 17 + 1)
constexpr int TILE_SLOTS = 16 * TBLK;  // 4368 eight-byte slots
// the persistent column passes: two tiles and two twiddle tables in dynamic shared memory
constexpr int COL_SMEM = 2 * TILE_SLOTS * 8 + 2 * 256 * 16;
__host__ __device__ __forceinline__ constexpr int tile_row(int r) { return TROW * (r & 15) + TBLK * (r >> 4); }
constexpr int XB = 544;               // u64 slots of a warp's row exchange buffer
constexpr int RW = 2;                 // row passes: 2 warps, 4 rows per block (24.6 KB of static shared memory)

// the passes below serve N = 2^16 split 2^8 x 2^8, on polynomials that start on 16-byte boundaries (their row
// loads and stores are 16 bytes wide); NttArgs::r16 / WidePrimes::r16 pick them per pass (bits below)
inline bool applies(const NttArgs& a, int pass) { return (a.r16 & pass) && a.log_n == 16 && a.n1 == 8; }
inline bool aligned(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }
inline bool aligned(const PtrTab& t, int n) {
  for (int i = 0; i < n; ++i)
    if (!aligned(t.p[i])) return false;
  return true;
}

// multiprocessors of the current device (cached per device)
inline int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) dev = 0;
  if (!cached[dev]) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
    cached[dev] = n;
  }
  return cached[dev];
}
// grid of a persistent column pass: two blocks per SM, at most one per tile
inline int col_grid(int ntiles) {
  const int g = 2 * sm_count();
  return ntiles < g ? ntiles : g;
}
// the column passes take more than the 48 KB of shared memory a kernel gets without asking: the attribute is
// set once per kernel and device (on the first launch, before any stream capture that launches it)
template <auto KERNEL, int BYTES>
inline void smem_optin() {
  static unsigned long long done = 0;  // device bits
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
  const unsigned long long bit = 1ull << (dev & 63);
  if (__atomic_load_n(&done, __ATOMIC_ACQUIRE) & bit) return;
  cuda_check(cudaFuncSetAttribute(KERNEL, cudaFuncAttributeMaxDynamicSharedMemorySize, BYTES),
             "raising a column pass's shared-memory limit");
  __atomic_fetch_or(&done, bit, __ATOMIC_ACQ_REL);
}

// stage one local twiddle entry t in [1, 256): global (tb << s) + i, s = floor(log2 t), i = t - 2^s; from
// stage 4 on, i = (l << (s - 4)) + m is stored at 2^s + 16 m + l.  T is a 16-byte entry (Twiddle or Tw2).
template <class T>
__device__ __forceinline__ void stage_tw(T* local, const T* global, u64 tb, int t) {
  const int s = 31 - __clz(t), i = t - (1 << s);
  const int d = s < 4 ? t : (1 << s) + 16 * (i & ((1 << (s - 4)) - 1)) + (i >> (s - 4));
  core::cp_async16(local + d, global + (tb << s) + i);
}
// all 255 entries of `rows` tables (row rr at local + 256 rr, global block tb0 + rr) by `nthreads` threads
template <class T>
__device__ __forceinline__ void stage_tw_rows(T* local, const T* global, u64 tb0, int rows, int tid, int nthreads) {
  for (int e = tid; e < rows * 255; e += nthreads) {
    const int rr = e / 255, t = e - rr * 255 + 1;
    stage_tw(local + 256 * rr, global, tb0 + rr, t);
  }
}

// ---- 64-bit residues (q < 2^61), Shoup twiddles ----

// forward outputs to [0, q): LAZY from below 65q (a Shoup product by 1), otherwise from below 4q
template <bool LAZY>
__device__ __forceinline__ u64 reduce_fwd(u64 x, const PrimeConst& c) {
  if (LAZY) {
    x = mul_shoup_lazy(x, 1, c.one_s, c.q);
    return x >= c.q ? x - c.q : x;
  }
  return reduce_4q(x, c.q);
}

// forward stages 0..3 (layout A); tw: the local table (every lane reads the same entry).  LAZY: unreduced values,
// approximate Shoup products (below 4q; values grow by < 4q per stage), as nttcore.cuh's fwd_group
template <bool LAZY>
__device__ __forceinline__ void fwd_a(u64 (&v)[16], const Twiddle* __restrict__ tw, u64 q) {
  const u64 two_q = q << 1;
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int b = 3 - s;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      if (k & (1 << b)) continue;
      const Twiddle w = tw[(1 << s) + (k >> (4 - s))];
      u64 x = v[k];
      if (!LAZY) x = x >= two_q ? x - two_q : x;
      const u64 t = LAZY ? mul_shoup_apx(v[k | (1 << b)], w.w, w.ws, q) : mul_shoup_lazy(v[k | (1 << b)], w.w, w.ws, q);
      v[k] = x + t;
      v[k | (1 << b)] = x - t + (LAZY ? q << 2 : two_q);
    }
  }
}
// forward stages 4..7 (layout B); twl: the local table plus the lane
template <bool LAZY>
__device__ __forceinline__ void fwd_b(u64 (&v)[16], const Twiddle* __restrict__ twl, u64 q) {
  const u64 two_q = q << 1;
#pragma unroll
  for (int s = 4; s < 8; ++s) {
    const int b = 7 - s;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      if (k & (1 << b)) continue;
      const Twiddle w = twl[(1 << s) + 16 * (k >> (8 - s))];
      u64 x = v[k];
      if (!LAZY) x = x >= two_q ? x - two_q : x;
      const u64 t = LAZY ? mul_shoup_apx(v[k | (1 << b)], w.w, w.ws, q) : mul_shoup_lazy(v[k | (1 << b)], w.w, w.ws, q);
      v[k] = x + t;
      v[k | (1 << b)] = x - t + (LAZY ? q << 2 : two_q);
    }
  }
}

// Gentleman-Sande butterfly of stage s, the pair (k, k | 2^b).  LAZYI (sub-transform inputs below 2q, 2^9 q <
// 2^64): no reductions, approximate Shoup products (below 4q); after c = 7 - s stages values are below
// 2^(c+1) q, which the difference path adds as its offset.  Otherwise values stay in [0, 2q) with exact Shoup
// products (as nttcore.cuh's inv_group).
template <bool LAZYI>
__device__ __forceinline__ void gs(u64& x, u64& y, const Twiddle& w, u64 q, int s) {
  if (LAZYI) {
    const u64 a = x, b = y;
    x = a + b;
    y = mul_shoup_apx(a - b + (q << (8 - s)), w.w, w.ws, q);
  } else {
    const u64 two_q = q << 1;
    const u64 a = x, b = y;
    u64 u = a + b;
    x = u >= two_q ? u - two_q : u;
    y = mul_shoup_lazy(a - b + two_q, w.w, w.ws, q);
  }
}
// inverse stages 7..4 (layout B)
template <bool LAZYI>
__device__ __forceinline__ void inv_b(u64 (&v)[16], const Twiddle* __restrict__ twl, u64 q) {
#pragma unroll
  for (int s = 7; s >= 4; --s) {
    const int b = 7 - s;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      if (k & (1 << b)) continue;
      gs<LAZYI>(v[k], v[k | (1 << b)], twl[(1 << s) + 16 * (k >> (8 - s))], q, s);
    }
  }
}
// inverse stages 3..0 (layout A); SC: the scale folded into stage 0 (the column phase: global stage 0 is the
// transform's last, InvScale), canonical outputs
template <bool LAZYI, bool SC = false>
__device__ __forceinline__ void inv_a(u64 (&v)[16], const Twiddle* __restrict__ tw, u64 q,
                                      const InvScale& sc = InvScale{}) {
#pragma unroll
  for (int s = 3; s >= 0; --s) {
    const int b = 3 - s;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      if (k & (1 << b)) continue;
      if (SC && s == 0) {
        const u64 x = v[k], y = v[k | (1 << b)];
        v[k] = mul_shoup(x + y, sc.n, sc.n_s, q);
        v[k | (1 << b)] = mul_shoup(x - y + (LAZYI ? q << 8 : q << 1), sc.wn, sc.wn_s, q);
        continue;
      }
      gs<LAZYI>(v[k], v[k | (1 << b)], tw[(1 << s) + (k >> (4 - s))], q, s);
    }
  }
}

// ---- two 29-bit primes per 8-byte element (the wide key product's internal primes), 32-bit Shoup ----

__device__ __forceinline__ void ct2(uint2& xr, uint2& yr, const Tw2& w, uint32_t q0, uint32_t q1) {
  const uint32_t t0 = q0 << 1, t1 = q1 << 1;
  uint2 x = xr;
  const uint2 y = yr;
  x.x = min(x.x, x.x - t0);  // x - t0 wraps above x when x < t0
  x.y = min(x.y, x.y - t1);
  const uint32_t u0 = core::mul_shoup32_lazy(y.x, w.w0, w.s0, q0);
  const uint32_t u1 = core::mul_shoup32_lazy(y.y, w.w1, w.s1, q1);
  xr = make_uint2(x.x + u0, x.y + u1);
  yr = make_uint2(x.x - u0 + t0, x.y - u1 + t1);
}
__device__ __forceinline__ void gs2(uint2& xr, uint2& yr, const Tw2& w, uint32_t q0, uint32_t q1) {
  const uint32_t t0 = q0 << 1, t1 = q1 << 1;
  const uint2 x = xr, y = yr;
  uint32_t a0 = x.x + y.x, a1 = x.y + y.y;
  a0 = min(a0, a0 - t0);  // a0 - t0 wraps above a0 when a0 < t0 (a0 < 2 t0 < 2^32)
  a1 = min(a1, a1 - t1);
  xr = make_uint2(a0, a1);
  yr = make_uint2(core::mul_shoup32_lazy(x.x - y.x + t0, w.w0, w.s0, q0),
                  core::mul_shoup32_lazy(x.y - y.y + t1, w.w1, w.s1, q1));
}
__device__ __forceinline__ void fwd_a2(uint2 (&v)[16], const Tw2* __restrict__ tw, uint32_t q0, uint32_t q1) {
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const int b = 3 - s;
#pragma unroll
    for (int k = 0; k < 16; ++k)
      if (!(k & (1 << b))) ct2(v[k], v[k | (1 << b)], tw[(1 << s) + (k >> (4 - s))], q0, q1);
  }
}
__device__ __forceinline__ void fwd_b2(uint2 (&v)[16], const Tw2* __restrict__ twl, uint32_t q0, uint32_t q1) {
#pragma unroll
  for (int s = 4; s < 8; ++s) {
    const int b = 7 - s;
#pragma unroll
    for (int k = 0; k < 16; ++k)
      if (!(k & (1 << b))) ct2(v[k], v[k | (1 << b)], twl[(1 << s) + 16 * (k >> (8 - s))], q0, q1);
  }
}
__device__ __forceinline__ void inv_b2(uint2 (&v)[16], const Tw2* __restrict__ twl, uint32_t q0, uint32_t q1) {
#pragma unroll
  for (int s = 7; s >= 4; --s) {
    const int b = 7 - s;
#pragma unroll
    for (int k = 0; k < 16; ++k)
      if (!(k & (1 << b))) gs2(v[k], v[k | (1 << b)], twl[(1 << s) + 16 * (k >> (8 - s))], q0, q1);
  }
}
template <bool SC = false>
__device__ __forceinline__ void inv_a2(uint2 (&v)[16], const Tw2* __restrict__ tw, uint32_t q0, uint32_t q1,
                                       const InvScale2& sc = InvScale2{}) {
#pragma unroll
  for (int s = 3; s >= 0; --s) {
    const int b = 3 - s;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      if (k & (1 << b)) continue;
      if (SC && s == 0) {  // the scale folded into the last stage (InvScale2), canonical outputs
        const uint2 x = v[k], y = v[k | (1 << b)];
        v[k] = make_uint2(core::mul_shoup32c(x.x + y.x, sc.n0, sc.n0s, q0),
                          core::mul_shoup32c(x.y + y.y, sc.n1, sc.n1s, q1));
        v[k | (1 << b)] = make_uint2(core::mul_shoup32c(x.x - y.x + (q0 << 1), sc.wn0, sc.wn0s, q0),
                                     core::mul_shoup32c(x.y - y.y + (q1 << 1), sc.wn1, sc.wn1s, q1));
        continue;
      }
      gs2(v[k], v[k | (1 << b)], tw[(1 << s) + (k >> (4 - s))], q0, q1);
    }
  }
}

// write the lane's values at w[SW k], read them back from r[SR k] (one warp's region)
template <int SW, int SR, class T>
__device__ __forceinline__ void exchange(T (&v)[16], T* w, const T* r) {
#pragma unroll
  for (int k = 0; k < 16; ++k) w[SW * k] = v[k];
  __syncwarp();
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = r[SR * k];
  __syncwarp();
}

// 16-byte halves of a lane's 16 consecutive 8-byte elements (layout B) from / to global memory
template <class T>
__device__ __forceinline__ void ld16(T (&v)[16], const T* p) {
  static_assert(sizeof(T) == 8, "8-byte elements");
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const uint4 x = *reinterpret_cast<const uint4*>(p + 2 * j);
    v[2 * j] = *reinterpret_cast<const T*>(&x.x);
    v[2 * j + 1] = *reinterpret_cast<const T*>(&x.z);
  }
}

// copies a 16-column tile (256 rows of 16 elements at stride 256) into the tile layout: 16 8-byte asynchronous
// copies per thread of a 256-thread block (one row per sixteen threads, coalesced).  Thread t takes row
// 16 it + t/16 and column t mod 16 at copy it, i.e. a per-thread base plus the constant offsets TBLK it (tile)
// and 4096 it (global), which the copies take as immediates
template <class T>
__device__ __forceinline__ void tile_load(T* tile, const T* in, int t) {
  static_assert(sizeof(T) == 8, "8-byte elements");
  const int r0 = t >> 4, c = t & 15;
  T* s = tile + TROW * r0 + c;
  const T* g = in + r0 * 256 + c;
#pragma unroll
  for (int it = 0; it < 16; ++it) core::cp_async8(s + TBLK * it, g + 4096 * it);
}
// the same for 4-byte words (int32 digits) in the word version of the layout
__device__ __forceinline__ void tile_load_words(int32_t* tile, const int32_t* in, int t) {
  const int r0 = t >> 4, c = t & 15;
  int32_t* s = tile + TROW * r0 + c;
  const int32_t* g = in + r0 * 256 + c;
#pragma unroll
  for (int it = 0; it < 16; ++it) core::cp_async4(s + TBLK * it, g + 4096 * it);
}
template <class T>
__device__ __forceinline__ void tile_store(T* out, const T* tile, int t) {
  const int r0 = t >> 4, c = t & 15;
  const T* s = tile + TROW * r0 + c;
  T* g = out + r0 * 256 + c;
#pragma unroll
  for (int it = 0; it < 16; ++it) g[4096 * it] = s[TBLK * it];
}
// tile index -> (limb, polynomial, first column): 16 column blocks per limb, limbs per polynomial
__device__ __forceinline__ void tile_at(int tile, int limbs, int& limb, int& poly, int& c0) {
  c0 = (tile & 15) * 16;
  const int r = tile >> 4;
  poly = r / limbs;
  limb = r - poly * limbs;
}

}  // namespace r16

namespace {

// ---------------------------------------------------------------------------------------------------------------
// 64-bit passes (N = 2^16)
// ---------------------------------------------------------------------------------------------------------------

// Column phase, persistent: block b takes the tiles (16 columns of one limb of one polynomial) b, b + grid, ...;
// the next tile's copies are in flight while the current one is transformed (two tile buffers).  Forward: LAZY
// as in k_cols_f.  Inverse (in place allowed): LAZY = unreduced butterflies (inputs below 2q, primes below
// 2^55); the N^-1 (or N^-1 2^64) scale is folded into the last stage (InvScale), whose Shoup products reduce
// every output to [0, q).
template <bool LAZY, bool FWD>
__global__ __launch_bounds__(256, 2) void k16_cols(NttArgs a, PtrTab src, PtrTab dst, LimbMap map, int limbs,
                                                   int ntiles) {
  using namespace r16;
  constexpr int N = 1 << 16;
  extern __shared__ __align__(16) u64 dsm16[];
  Twiddle* twb = reinterpret_cast<Twiddle*>(dsm16 + 2 * TILE_SLOTS);  // [2][256]
  const int t = threadIdx.x;
  const Twiddle* twg = FWD ? a.tw_fwd : a.tw_inv;
  // (limb, polynomial, first column) of a tile, found once when its copies are issued and kept for its turn
  int limb = 0, poly = 0, c0 = 0, nlimb = 0, npoly = 0, nc0 = 0;
  auto issue = [&](int tile, int b) {
    tile_at(tile, limbs, nlimb, npoly, nc0);
    tile_load(dsm16 + b * TILE_SLOTS, src.p[npoly] + (size_t)nlimb * N + nc0, t);
    if (t > 0) stage_tw(twb + 256 * b, twg + (size_t)map.prime(nlimb) * N, 1, t);
  };
  int tile = blockIdx.x;
  if (tile < ntiles) issue(tile, 0);
  const int lane = t & 31, lam = lane & 15, col = 2 * (t >> 5) + (lane >> 4);
#pragma unroll 1
  for (int b = 0; tile < ntiles; tile += gridDim.x, b ^= 1) {
    limb = nlimb, poly = npoly, c0 = nc0;
    core::cp_async_wait_all();
    __syncthreads();  // tile landed; every thread is done with the other buffer
    if (tile + (int)gridDim.x < ntiles) issue(tile + gridDim.x, b ^ 1);
    const PrimeConst& pc = a.pc[map.prime(limb)];
    const u64 q = pc.q;
    u64* tl = dsm16 + b * TILE_SLOTS;
    const Twiddle* tw = twb + 256 * b;
    u64* pA = tl + TROW * lam + col;  // element lam + 16 k at pA[TBLK k]
    u64* pB = tl + TBLK * lam + col;  // element 16 lam + k at pB[TROW k]
    u64 v[16];
    if (FWD) {
#pragma unroll
      for (int k = 0; k < 16; ++k) v[k] = pA[TBLK * k];
      fwd_a<LAZY>(v, tw, q);
      exchange<TBLK, TROW>(v, pA, pB);
      fwd_b<LAZY>(v, tw + lam, q);
#pragma unroll
      for (int k = 0; k < 16; ++k) pB[TROW * k] = v[k];
    } else {
#pragma unroll
      for (int k = 0; k < 16; ++k) v[k] = pB[TROW * k];
      inv_b<LAZY>(v, tw + lam, q);
      exchange<TROW, TBLK>(v, pB, pA);
      const InvScale sc = a.mont_out ? InvScale{pc.n_inv_r, pc.n_inv_r_s, pc.w1nr, pc.w1nr_s}
                                     : InvScale{pc.n_inv, pc.n_inv_s, pc.w1n, pc.w1n_s};
      inv_a<LAZY, true>(v, tw, q, sc);
#pragma unroll
      for (int k = 0; k < 16; ++k) pA[TBLK * k] = v[k];
    }
    __syncthreads();
    tile_store(dst.p[poly] + (size_t)limb * N + c0, tl, t);
  }
}

// Row phase: each warp transforms two rows (one per 16-lane half) of the polynomials blockIdx.z * RP .. below
// `polys`, the next polynomial's rows loaded while the current one is transformed; the block stages its 8
// rows' twiddle tables once.  Forward outputs reduced to [0, q) (LAZY: from below 65q by a Shoup product by 1),
// or (RAW, for the tensor: NttArgs::raw_out) left below 65q (LAZY) or 4q; inverse outputs in [0, 2q).
template <bool LAZY, bool FWD, int RP, bool RAW = false>
__global__ __launch_bounds__(32 * r16::RW) void k16_rows(NttArgs a, PtrTab src, PtrTab dst, LimbMap map,
                                                               int polys) {
  using namespace r16;
  constexpr int N = 1 << 16, ROWS = 2 * RW;
  __shared__ __align__(16) u64 xb[RW][XB];
  __shared__ __align__(16) Twiddle twl[ROWS][256];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, lam = lane & 15, sub = lane >> 4;
  const int row0 = blockIdx.x * ROWS, rl = 2 * warp + sub, row = row0 + rl;
  const int limb = blockIdx.y, first = blockIdx.z * RP, count = min(RP, polys - first);
  const int prime = map.prime(limb);
  const PrimeConst& pc = a.pc[prime];
  const u64 q = pc.q;
  const size_t off = (size_t)limb * N + (size_t)row * 256;
  u64* xa = &xb[warp][lam + 272 * sub];       // layout A slot of element lam + 16 k: xa[17 k]
  u64* xbb = &xb[warp][17 * lam + 272 * sub];  // layout B slot of element 16 lam + k: xbb[k]
  u64 v[16], vn[16];
  auto load = [&](const u64* in, u64(&x)[16]) {
    if (FWD) {
#pragma unroll
      for (int k = 0; k < 16; ++k) x[k] = in[lam + 16 * k];
    } else {
      ld16(x, in + 16 * lam);
    }
  };
  load(src.p[first] + off, v);  // requested before the twiddle tables, so both latencies overlap
  stage_tw_rows(&twl[0][0], (FWD ? a.tw_fwd : a.tw_inv) + (size_t)prime * N, (u64)(256 + row0), ROWS, threadIdx.x,
                32 * RW);
  core::cp_async_wait_all();
  __syncthreads();
  const Twiddle* tw = twl[rl];
#pragma unroll 1
  for (int p = 0; p < count; ++p) {
    if (p + 1 < count) load(src.p[first + p + 1] + off, vn);
    u64* out = dst.p[first + p] + off;
    if (FWD) {
      fwd_a<LAZY>(v, tw, q);
      exchange<17, 1>(v, xa, xbb);
      fwd_b<LAZY>(v, tw + lam, q);
#pragma unroll
      for (int j = 0; j < 8; ++j)
        *reinterpret_cast<ulonglong2*>(out + 16 * lam + 2 * j) =
            RAW ? make_ulonglong2(v[2 * j], v[2 * j + 1])
                      : make_ulonglong2(reduce_fwd<LAZY>(v[2 * j], pc), reduce_fwd<LAZY>(v[2 * j + 1], pc));
    } else {
      inv_b<false>(v, tw + lam, q);
      exchange<1, 17>(v, xbb, xa);
      inv_a<false>(v, tw, q);
#pragma unroll
      for (int k = 0; k < 16; ++k) out[lam + 16 * k] = v[k];
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = vn[k];
  }
}

// The tensor and the inverse row phase (as k_tensor_inv_rows): for each job of the block, d0 = a0 b0,
// d1 = a0 b1 + a1 b0, d2 = a1 b1 (Montgomery products of the forward transforms in4[4j..4j+3], left in [0, 2q))
// go straight into the inverse row transform; the inverse column pass with NttArgs::mont_out completes it.
template <int TJ>
__global__ __launch_bounds__(32 * r16::RW) void k16_tensor_inv_rows(NttArgs a, PtrTab in4, PtrTab out3,
                                                                          LimbMap map, int jobs) {
  using namespace r16;
  constexpr int N = 1 << 16, ROWS = 2 * RW;
  __shared__ __align__(16) u64 xb[RW][XB];
  __shared__ __align__(16) Twiddle twl[ROWS][256];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, lam = lane & 15, sub = lane >> 4;
  const int row0 = blockIdx.x * ROWS, rl = 2 * warp + sub, row = row0 + rl;
  const int limb = blockIdx.y, first = blockIdx.z * TJ, count = min(TJ, jobs - first);
  const int prime = map.prime(limb);
  const PrimeConst& pc = a.pc[prime];
  const u64 q = pc.q;
  const size_t off = (size_t)limb * N + (size_t)row * 256 + 16 * lam;
  u64* xa = &xb[warp][lam + 272 * sub];
  u64* xbb = &xb[warp][17 * lam + 272 * sub];
  stage_tw_rows(&twl[0][0], a.tw_inv + (size_t)prime * N, (u64)(256 + row0), ROWS, threadIdx.x, 32 * RW);
  core::cp_async_wait_all();
  __syncthreads();
  const Twiddle* tw = twl[rl];
#pragma unroll 1
  for (int p = 0; p < count; ++p) {
    const int j = first + p;
    // one copy of the sub-transform for the three outputs (selected by o)
#pragma unroll 1
    for (int o = 0; o < 3; ++o) {
      const u64* xp = in4.p[4 * j + (o == 2 ? 1 : 0)] + off;  // a0, a0, a1
      const u64* yp = in4.p[4 * j + (o == 0 ? 2 : 3)] + off;  // b0, b1, b1
      u64 v[16];
      if (o == 1) {
        const u64* x2 = in4.p[4 * j + 1] + off;  // a1
        const u64* y2 = in4.p[4 * j + 2] + off;  // b0
#pragma unroll
        for (int h = 0; h < 8; ++h) {
          const ulonglong2 x = *reinterpret_cast<const ulonglong2*>(xp + 2 * h);
          const ulonglong2 y = *reinterpret_cast<const ulonglong2*>(yp + 2 * h);
          const ulonglong2 x1 = *reinterpret_cast<const ulonglong2*>(x2 + 2 * h);
          const ulonglong2 y1 = *reinterpret_cast<const ulonglong2*>(y2 + 2 * h);
          U128 m = mul_wide(x.x, y.x);
          add_to(m, mul_wide(x1.x, y1.x));
          v[2 * h] = mont_reduce_lazy(m, pc);
          m = mul_wide(x.y, y.y);
          add_to(m, mul_wide(x1.y, y1.y));
          v[2 * h + 1] = mont_reduce_lazy(m, pc);
        }
      } else {
#pragma unroll
        for (int h = 0; h < 8; ++h) {
          const ulonglong2 x = *reinterpret_cast<const ulonglong2*>(xp + 2 * h);
          const ulonglong2 y = *reinterpret_cast<const ulonglong2*>(yp + 2 * h);
          v[2 * h] = mont_reduce_lazy(mul_wide(x.x, y.x), pc);
          v[2 * h + 1] = mont_reduce_lazy(mul_wide(x.y, y.y), pc);
        }
      }
      inv_b<false>(v, tw + lam, q);
      exchange<1, 17>(v, xbb, xa);
      inv_a<false>(v, tw, q);
      u64* out = out3.p[3 * j + o] + (size_t)limb * N + (size_t)row * 256;
#pragma unroll
      for (int k = 0; k < 16; ++k) out[lam + 16 * k] = v[k];
    }
  }
}

// ---------------------------------------------------------------------------------------------------------------
// dual 29-bit-prime passes of the wide key product (N = 2^16; element = uint2 of residues mod (q0, q1) of
// pair blockIdx.y; layouts of wide.cu)
// ---------------------------------------------------------------------------------------------------------------

__device__ __forceinline__ uint2 w16_reduce4(uint2 v, uint32_t q0, uint32_t q1) {
  const uint32_t a = v.x >= 2 * q0 ? v.x - 2 * q0 : v.x;
  const uint32_t b = v.y >= 2 * q1 ? v.y - 2 * q1 : v.y;
  return make_uint2(fold32(a, q0), fold32(b, q1));
}

// Forward column phase, persistent (as k16_cols) over the tiles of polynomials p0 .. p0 + polys - 1 and both
// pairs.  SRC 0: int32 digits[poly][N] taken as d + 2q (in [0, 4q) since 2q > 2^29 >= |d|), copied as words
// into the word version of the tile layout and converted at first use; SRC 1: residues src[poly][pair][N].
// Output out[poly][pair][N].
template <int SRC>
__global__ __launch_bounds__(256, 2) void k16_w_cols_fwd(WidePrimes w, const void* src, uint2* out, int p0,
                                                         int ntiles) {
  using namespace r16;
  constexpr int N = 1 << 16;
  extern __shared__ __align__(16) uint2 dsm16w[];
  Tw2* twb = reinterpret_cast<Tw2*>(dsm16w + 2 * TILE_SLOTS);
  const int t = threadIdx.x;
  auto issue = [&](int tile, int b) {
    int pair, poly, c0;
    tile_at(tile, 2, pair, poly, c0);
    const size_t p = (size_t)p0 + poly;
    if (SRC == 0)
      tile_load_words(reinterpret_cast<int32_t*>(dsm16w + b * TILE_SLOTS),
                      static_cast<const int32_t*>(src) + p * N + c0, t);
    else
      tile_load(dsm16w + b * TILE_SLOTS, static_cast<const uint2*>(src) + (p * 2 + pair) * N + c0, t);
    if (t > 0) stage_tw(twb + 256 * b, w.tw_fwd + (size_t)pair * N, 1, t);
  };
  int tile = blockIdx.x;
  if (tile < ntiles) issue(tile, 0);
  const int lane = t & 31, lam = lane & 15, col = 2 * (t >> 5) + (lane >> 4);
#pragma unroll 1
  for (int b = 0; tile < ntiles; tile += gridDim.x, b ^= 1) {
    core::cp_async_wait_all();
    __syncthreads();
    if (tile + (int)gridDim.x < ntiles) issue(tile + gridDim.x, b ^ 1);
    int pair, poly, c0;
    tile_at(tile, 2, pair, poly, c0);
    const uint32_t q0 = pair ? w.q[2] : w.q[0], q1 = pair ? w.q[3] : w.q[1];
    uint2* tl = dsm16w + b * TILE_SLOTS;
    const Tw2* tw = twb + 256 * b;
    uint2* pA = tl + TROW * lam + col;
    uint2* pB = tl + TBLK * lam + col;
    uint2 v[16];
    if (SRC == 0) {
      const int32_t* dA = reinterpret_cast<const int32_t*>(tl) + TROW * lam + col;
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        const int32_t d = dA[TBLK * k];
        v[k] = make_uint2((uint32_t)(d + (int32_t)(2 * q0)), (uint32_t)(d + (int32_t)(2 * q1)));
      }
      __syncthreads();  // the digit words of other warps' columns share the slots written below
    } else {
#pragma unroll
      for (int k = 0; k < 16; ++k) v[k] = pA[TBLK * k];
    }
    fwd_a2(v, tw, q0, q1);
    exchange<TBLK, TROW>(v, pA, pB);
    fwd_b2(v, tw + lam, q0, q1);
#pragma unroll
    for (int k = 0; k < 16; ++k) pB[TROW * k] = v[k];
    __syncthreads();
    tile_store(out + (((size_t)p0 + poly) * 2 + pair) * N + c0, tl, t);
  }
}

// Forward row phase of data[poly][pair][N] (polys p0 + blockIdx.z * RP .. below p0 + cnt), outputs reduced to
// [0, q).  TILED: written as dtt[job][pair][x/32][digit][32] (DM maps a polynomial to its job, as in
// k_w_rows_fwd); otherwise in place.
template <bool TILED, class DM, int RP>
__global__ __launch_bounds__(32 * r16::RW) void k16_w_rows_fwd(WidePrimes w, uint2* data, uint2* dtt, int p0,
                                                                     int cnt, DM dm) {
  using namespace r16;
  constexpr int N = 1 << 16, ROWS = 2 * RW;
  __shared__ __align__(16) uint2 xb[RW][XB];
  __shared__ __align__(16) Tw2 twl[ROWS][256];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, lam = lane & 15, sub = lane >> 4;
  const int row0 = blockIdx.x * ROWS, rl = 2 * warp + sub, row = row0 + rl;
  const int pair = blockIdx.y;
  const int first = blockIdx.z * RP, count = min(RP, cnt - first);
  const uint32_t q0 = pair ? w.q[2] : w.q[0], q1 = pair ? w.q[3] : w.q[1];
  auto row_ptr = [&](int p) { return data + (((size_t)p0 + first + p) * 2 + pair) * N + (size_t)row * 256; };
  uint2* xa = &xb[warp][lam + 272 * sub];
  uint2* xbb = &xb[warp][17 * lam + 272 * sub];
  int job = -1;  // the digit map's position (TILED)
  uint2 v[16], vn[16];
  {
    const uint2* in = row_ptr(0);
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = in[lam + 16 * k];
  }
  stage_tw_rows(&twl[0][0], w.tw_fwd + (size_t)pair * N, (u64)(256 + row0), ROWS, threadIdx.x, 32 * RW);
  core::cp_async_wait_all();
  __syncthreads();
  const Tw2* tw = twl[rl];
#pragma unroll 1
  for (int p = 0; p < count; ++p) {
    if (p + 1 < count) {
      const uint2* in = row_ptr(p + 1);
#pragma unroll
      for (int k = 0; k < 16; ++k) vn[k] = in[lam + 16 * k];
    }
    fwd_a2(v, tw, q0, q1);
    exchange<17, 1>(v, xa, xbb);
    fwd_b2(v, tw + lam, q0, q1);
    uint2* o;
    if (TILED) {
      int jfirst, digit, D;
      dm.locate(p0 + first + p, job, jfirst, digit, D);
      const int x0 = row * 256 + 16 * lam;  // the lane's 16 consecutive positions: one half of a 32-position tile
      o = dtt + (size_t)jfirst * 2 * N + (size_t)pair * N * D + (size_t)digit * 32 + (size_t)(x0 >> 5) * (D * 32) +
          (x0 & 31);
    } else {
      o = row_ptr(p) + 16 * lam;
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint2 e0 = w16_reduce4(v[2 * j], q0, q1), e1 = w16_reduce4(v[2 * j + 1], q0, q1);
      *reinterpret_cast<uint4*>(o + 2 * j) = make_uint4(e0.x, e0.y, e1.x, e1.y);
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = vn[k];
  }
}

// Inverse row phase, in place on data[poly][pair][N] (polys blockIdx.z * RP .. below cnt); inputs in [0, 2q).
template <int RP>
__global__ __launch_bounds__(32 * r16::RW) void k16_w_rows_inv(WidePrimes w, uint2* data, int cnt) {
  using namespace r16;
  constexpr int N = 1 << 16, ROWS = 2 * RW;
  __shared__ __align__(16) uint2 xb[RW][XB];
  __shared__ __align__(16) Tw2 twl[ROWS][256];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, lam = lane & 15, sub = lane >> 4;
  const int row0 = blockIdx.x * ROWS, rl = 2 * warp + sub, row = row0 + rl;
  const int pair = blockIdx.y;
  const int first = blockIdx.z * RP, count = min(RP, cnt - first);
  const uint32_t q0 = pair ? w.q[2] : w.q[0], q1 = pair ? w.q[3] : w.q[1];
  auto row_ptr = [&](int p) { return data + (((size_t)first + p) * 2 + pair) * N + (size_t)row * 256; };
  uint2* xa = &xb[warp][lam + 272 * sub];
  uint2* xbb = &xb[warp][17 * lam + 272 * sub];
  uint2 v[16], vn[16];
  ld16(v, row_ptr(0) + 16 * lam);
  stage_tw_rows(&twl[0][0], w.tw_inv + (size_t)pair * N, (u64)(256 + row0), ROWS, threadIdx.x, 32 * RW);
  core::cp_async_wait_all();
  __syncthreads();
  const Tw2* tw = twl[rl];
#pragma unroll 1
  for (int p = 0; p < count; ++p) {
    if (p + 1 < count) ld16(vn, row_ptr(p + 1) + 16 * lam);
    inv_b2(v, tw + lam, q0, q1);
    exchange<1, 17>(v, xbb, xa);
    inv_a2(v, tw, q0, q1);
    uint2* out = row_ptr(p);
#pragma unroll
    for (int k = 0; k < 16; ++k) out[lam + 16 * k] = v[k];
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = vn[k];
  }
}

// Inverse column phase, persistent (as k16_cols), in place on data[poly][pair][N], times N^-1 (folded into the
// last stage, InvScale2): outputs in [0, q).  (A template so that translation units that do not launch it do not compile it.)
template <int = 0>
__global__ __launch_bounds__(256, 2) void k16_w_cols_inv(WidePrimes w, uint2* data, int ntiles) {
  using namespace r16;
  constexpr int N = 1 << 16;
  extern __shared__ __align__(16) uint2 dsm16w[];
  Tw2* twb = reinterpret_cast<Tw2*>(dsm16w + 2 * TILE_SLOTS);
  const int t = threadIdx.x;
  auto issue = [&](int tile, int b) {
    int pair, poly, c0;
    tile_at(tile, 2, pair, poly, c0);
    tile_load(dsm16w + b * TILE_SLOTS, data + ((size_t)poly * 2 + pair) * N + c0, t);
    if (t > 0) stage_tw(twb + 256 * b, w.tw_inv + (size_t)pair * N, 1, t);
  };
  int tile = blockIdx.x;
  if (tile < ntiles) issue(tile, 0);
  const int lane = t & 31, lam = lane & 15, col = 2 * (t >> 5) + (lane >> 4);
#pragma unroll 1
  for (int b = 0; tile < ntiles; tile += gridDim.x, b ^= 1) {
    core::cp_async_wait_all();
    __syncthreads();
    if (tile + (int)gridDim.x < ntiles) issue(tile + gridDim.x, b ^ 1);
    int pair, poly, c0;
    tile_at(tile, 2, pair, poly, c0);
    const uint32_t q0 = pair ? w.q[2] : w.q[0], q1 = pair ? w.q[3] : w.q[1];
    uint2* tl = dsm16w + b * TILE_SLOTS;
    const Tw2* tw = twb + 256 * b;
    uint2* pA = tl + TROW * lam + col;
    uint2* pB = tl + TBLK * lam + col;
    uint2 v[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = pB[TROW * k];
    inv_b2(v, tw + lam, q0, q1);
    exchange<TROW, TBLK>(v, pB, pA);
    const int e0 = pair ? 2 : 0, e1 = e0 + 1;
    const InvScale2 sc{w.n_inv[e0], w.n_inv_s[e0], w.w1n[e0], w.w1n_s[e0],
                       w.n_inv[e1], w.n_inv_s[e1], w.w1n[e1], w.w1n_s[e1]};
    inv_a2<true>(v, tw, q0, q1, sc);
#pragma unroll
    for (int k = 0; k < 16; ++k) pA[TBLK * k] = v[k];
    __syncthreads();
    tile_store(data + ((size_t)poly * 2 + pair) * N + c0, tl, t);
  }
}

}  // namespace
}  // namespace rc
