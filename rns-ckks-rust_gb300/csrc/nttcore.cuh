// Warp-level register-blocked sub-NTTs of size 2^M (M = 6, 7, 8), eight
// residues per lane.
//
// A 2^M-point column or row transform is done by 2^(M-3) lanes; a warp holds
// 32 / 2^(M-3) of them side by side.  The M butterfly stages are split into
// groups of up to three stages whose butterflies pair elements held by the
// same lane; between groups the lane's eight values go through a warp-private
// shared-memory buffer (XOR-swizzled so that every access pattern below is
// free of bank conflicts for M = 7, 8) and come back in the next group's
// assignment.  All index arithmetic is resolved at compile time except the
// lane number.
//
// Twiddle index of sub-stage s for the lower element r of a pair:
//   (TB << s) + (r >> (M - s)),   TB = 1 for the column phase, 2^n1 + row for
// the row phase; this is the merged-twiddle Cooley-Tukey / Gentleman-Sande
// index of the full N-point transform restricted to one column or row.
// Kernels stage the 2^M - 1 twiddles a column or row needs into a local
// shared-memory table t[(1 << s) + j] = global[(TB << s) + j] (stage_twiddles)
// and the butterflies read t[(1 << s) + (r >> (M - s))].
#pragma once
#include "modarith.cuh"

namespace rc {
namespace core {

// Twiddle (w, w') pair through the read-only path.  The load is volatile so the
// compiler keeps it at its use: hoisting the ~20 loop-invariant twiddles of a
// sub-transform out of the per-digit loop would pin ~80 registers per thread.
__device__ __forceinline__ Twiddle ldtw(const Twiddle* p) {
  Twiddle t;
  asm volatile("ld.global.nc.v2.u64 {%0, %1}, [%2];" : "=l"(t.w), "=l"(t.ws) : "l"(p));
  return t;
}

// local[t] = global[(TB << s) + (t - 2^s)] for t in [1, 2^M), s = floor(log2 t),
// copied cooperatively by `nthreads` threads starting at thread `tid`
template <int M>
__device__ __forceinline__ void stage_twiddles(Twiddle* local, const Twiddle* global, u64 tb, int tid,
                                               int nthreads) {
  for (int t = 1 + tid; t < (1 << M); t += nthreads) {
    const int s = 31 - __clz(t);
    const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(global + ((tb - 1) << s) + t));
    local[t].w = v.x;
    local[t].ws = v.y;
  }
}

// Asynchronous global -> shared copies (cp.async): a thread issues all of its copies before waiting, so
// the tile and twiddle loads of a kernel are in flight together.  Shared destinations of 16-byte copies
// must be 16-byte aligned.
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
               "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
               "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
               "l"(gmem)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// stage_twiddles with asynchronous copies (completed by cp_async_wait_all); T is Twiddle or Tw2 (16 bytes)
template <int M, class T>
__device__ __forceinline__ void stage_twiddles_async(T* local, const T* global, u64 tb, int tid, int nthreads) {
  static_assert(sizeof(T) == 16, "16-byte twiddle entries");
  for (int t = 1 + tid; t < (1 << M); t += nthreads) {
    const int s = 31 - __clz(t);
    cp_async16(local + t, global + ((tb - 1) << s) + t);
  }
}

// Lane id re-read with a volatile move: used inside long loops so that the
// lane-dependent shared-memory addresses are recomputed per iteration instead
// of being hoisted (and pinned in registers) across the loop.
__device__ __forceinline__ int lane_id_volatile() {
  int l;
  asm volatile("mov.u32 %0, %%laneid;" : "=r"(l));
  return l;
}

template <int M>
struct Geo {
  static constexpr int LB = M - 3;  // lane bits per sub-transform
  static constexpr int LANES = 1 << LB;
  static constexpr int SIZE = 1 << M;
  static constexpr int SUBS = 32 / LANES;  // sub-transforms per warp
  static constexpr int STRIDE = SIZE + 1;  // odd stride between sub-transform buffers
};

// stage groups: {S0, G}
template <int M, int GI>
struct Grp;
template <int M>
struct Grp<M, 0> {
  static constexpr int S0 = 0, G = 3;
};
template <int M>
struct Grp<M, 1> {
  static constexpr int S0 = 3, G = 3;
};
template <>
struct Grp<8, 2> {
  static constexpr int S0 = 6, G = 2;
};
template <>
struct Grp<7, 2> {
  static constexpr int S0 = 6, G = 1;
};
template <int M>
struct NGroups {
  static constexpr int value = M == 6 ? 2 : 3;
};

// index of element k of lane l in group (S0, G): the G butterfly bits come from
// k's low bits, the lane bits fill the lowest remaining positions, the rest of
// k fills the highest remaining positions.
template <int M, int S0, int G>
__device__ __forceinline__ int gidx(int l, int k) {
  constexpr int LB = M - 3;
  constexpr int BLO = M - S0 - G;  // lowest butterfly bit position
  int r = ((k & ((1 << G) - 1)) << BLO);
  int li = 0, xi = 0;
#pragma unroll
  for (int p = 0; p < M; ++p) {
    if (p >= BLO && p < BLO + G) continue;
    if (li < LB) {
      r |= ((l >> li) & 1) << p;
      ++li;
    } else {
      r |= ((k >> (G + xi)) & 1) << p;
      ++xi;
    }
  }
  return r;
}

// conflict-free XOR swizzle (found by exhaustive search over GF(2)-linear maps)
template <int M>
__host__ __device__ __forceinline__ constexpr int swz_h(int v) {
  return M == 8 ? ((v & 1) ? 1 : 0) ^ ((v & 2) ? 6 : 0) ^ ((v & 4) ? 8 : 0)
                : (M == 7 ? ((v & 1) ? 3 : 0) ^ ((v & 2) ? 4 : 0) ^ ((v & 4) ? 8 : 0) : ((v & 2) ? 2 : 0));
}
template <int M>
__device__ __forceinline__ int swz(int r) {
  const int v = r >> 4;
  int h;
  if (M == 8) h = ((v & 1) ? 1 : 0) ^ ((v & 2) ? 6 : 0) ^ ((v & 4) ? 8 : 0);
  else if (M == 7) h = ((v & 1) ? 3 : 0) ^ ((v & 2) ? 4 : 0) ^ ((v & 4) ? 8 : 0);
  else h = (v & 2) ? 2 : 0;
  return r ^ h;  // = r ^ swz_h<M>(r >> 4)
}

// Cooley-Tukey butterflies of one group.  LAZY: inputs are not reduced and the twiddle products take the
// approximate Shoup quotient (values grow by < 4q per stage; valid while they stay below 2^64: (4 log N + 1) q,
// primes below 2^57), otherwise Harvey's [0, 4q) invariant with exact Shoup products.
template <int M, int GI, bool LAZY>
__device__ __forceinline__ void fwd_group(u64 (&v)[8], int l, const Twiddle* __restrict__ tw, u64 q) {
  constexpr int S0 = Grp<M, GI>::S0, G = Grp<M, GI>::G;
  const u64 two_q = q << 1, off = LAZY ? q << 2 : two_q;
#pragma unroll
  for (int j = 0; j < G; ++j) {
    const int s = S0 + j;
    const int b = G - 1 - j;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (k & (1 << b)) continue;
      const int r = gidx<M, S0, G>(l, k);
      const Twiddle w = tw[(1 << s) + (r >> (M - s))];
      u64 x = v[k];
      if (!LAZY) x = x >= two_q ? x - two_q : x;
      const u64 t = LAZY ? mul_shoup_apx(v[k | (1 << b)], w.w, w.ws, q) : mul_shoup_lazy(v[k | (1 << b)], w.w, w.ws, q);
      v[k] = x + t;
      v[k | (1 << b)] = x - t + off;
    }
  }
}

// stages of the inverse sub-transform done before group GI starts (groups run from the last down)
template <int M, int GI>
__host__ __device__ constexpr int inv_done() {
  if constexpr (GI + 1 < NGroups<M>::value) return Grp<M, GI + 1>::G + inv_done<M, GI + 1>();
  else return 0;
}

// Gentleman-Sande butterflies of one group, stages in decreasing order; values stay in [0, 2q) (exact Shoup
// products: an approximate one would need a conditional subtraction more, which measured slower).  LAZYI
// (inputs of the sub-transform below 2q): no reductions, approximate Shoup products (below 4q); after c stages
// of the sub-transform values are below 2^(c+1) q (a product, below 4q, stays within that from c = 1 on), so
// the difference path adds that bound as its offset; valid while 2^(M+1) q < 2^64, and the caller reduces the
// outputs.
// SC (the column phase of the inverse transform, whose stage 0 is the transform's last): that stage takes the
// scale (InvScale) and leaves canonical outputs.
template <int M, int GI, bool LAZYI = false, bool SC = false>
__device__ __forceinline__ void inv_group(u64 (&v)[8], int l, const Twiddle* __restrict__ tw, u64 q,
                                          const InvScale& sc = InvScale{}) {
  constexpr int S0 = Grp<M, GI>::S0, G = Grp<M, GI>::G;
  const u64 two_q = q << 1;
  if constexpr (LAZYI) {
#pragma unroll
    for (int j = G - 1; j >= 0; --j) {
      const int s = S0 + j;
      const int b = G - 1 - j;
      const int c = inv_done<M, GI>() + (G - 1 - j);  // stages done before this one
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        if (k & (1 << b)) continue;
        const u64 x = v[k], y = v[k | (1 << b)];
        if (SC && s == 0) {
          v[k] = mul_shoup(x + y, sc.n, sc.n_s, q);
          v[k | (1 << b)] = mul_shoup(x - y + (q << (c + 1)), sc.wn, sc.wn_s, q);
          continue;
        }
        const int r = gidx<M, S0, G>(l, k);
        const Twiddle w = tw[(1 << s) + (r >> (M - s))];
        v[k] = x + y;
        v[k | (1 << b)] = mul_shoup_apx(x - y + (q << (c + 1)), w.w, w.ws, q);
      }
    }
  } else {
#pragma unroll
    for (int j = G - 1; j >= 0; --j) {
      const int s = S0 + j;
      const int b = G - 1 - j;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        if (k & (1 << b)) continue;
        const u64 x = v[k], y = v[k | (1 << b)];
        if (SC && s == 0) {
          v[k] = mul_shoup(x + y, sc.n, sc.n_s, q);
          v[k | (1 << b)] = mul_shoup(x - y + two_q, sc.wn, sc.wn_s, q);
          continue;
        }
        const int r = gidx<M, S0, G>(l, k);
        const Twiddle w = tw[(1 << s) + (r >> (M - s))];
        u64 u = x + y;
        u = u >= two_q ? u - two_q : u;
        v[k] = u;
        v[k | (1 << b)] = mul_shoup_lazy(x - y + two_q, w.w, w.ws, q);
      }
    }
  }
}

// write the lane's values in group A's layout, read them back in group B's
template <int M, int GA, int GB>
__device__ __forceinline__ void exchange(u64 (&v)[8], u64* buf, int l) {
#pragma unroll
  for (int k = 0; k < 8; ++k) buf[swz<M>(gidx<M, Grp<M, GA>::S0, Grp<M, GA>::G>(l, k))] = v[k];
  __syncwarp();
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = buf[swz<M>(gidx<M, Grp<M, GB>::S0, Grp<M, GB>::G>(l, k))];
  __syncwarp();
}

// full forward sub-transform: v holds group 0's layout on entry, the last
// group's layout on exit
template <int M, bool LAZY>
__device__ __forceinline__ void fwd_sub(u64 (&v)[8], u64* buf, int l, const Twiddle* tw, u64 q) {
  fwd_group<M, 0, LAZY>(v, l, tw, q);
  exchange<M, 0, 1>(v, buf, l);
  fwd_group<M, 1, LAZY>(v, l, tw, q);
  if constexpr (NGroups<M>::value == 3) {
    exchange<M, 1, 2>(v, buf, l);
    fwd_group<M, 2, LAZY>(v, l, tw, q);
  }
}

// full inverse sub-transform: v holds the last group's layout on entry, group 0's on exit; SC: the scale folded
// into stage 0 (column phase)
template <int M, bool LAZYI = false, bool SC = false>
__device__ __forceinline__ void inv_sub(u64 (&v)[8], u64* buf, int l, const Twiddle* tw, u64 q,
                                        const InvScale& sc = InvScale{}) {
  if constexpr (NGroups<M>::value == 3) {
    inv_group<M, 2, LAZYI>(v, l, tw, q);
    exchange<M, 2, 1>(v, buf, l);
  }
  inv_group<M, 1, LAZYI>(v, l, tw, q);
  exchange<M, 1, 0>(v, buf, l);
  inv_group<M, 0, LAZYI, SC>(v, l, tw, q, sc);
}

template <int M>
struct Last {
  static constexpr int GI = NGroups<M>::value - 1;
  static constexpr int S0 = Grp<M, GI>::S0, G = Grp<M, GI>::G;
};

template <int M>
__device__ __forceinline__ int first_idx(int l, int k) {
  return gidx<M, 0, 3>(l, k);
}
template <int M>
__device__ __forceinline__ int last_idx(int l, int k) {
  return gidx<M, Last<M>::S0, Last<M>::G>(l, k);
}

// ---------------------------------------------------------------------------
// Two 32-bit primes side by side.  The internal primes of the wide key product
// are below 2^29 and handled in pairs: an element is a uint2 of its residues
// mod (q0, q1), so a pair occupies the 8 bytes of one 64-bit residue and the
// shared-memory layouts, swizzles and register counts above carry over
// unchanged.  Butterflies use 32-bit Shoup multiplication (values < 4q < 2^31).
// ---------------------------------------------------------------------------
// x * w mod q in [0, 2q) for any 32-bit x
__device__ __forceinline__ uint32_t mul_shoup32_lazy(uint32_t x, uint32_t w, uint32_t ws, uint32_t q) {
  return x * w - __umulhi(x, ws) * q;
}
// x * w mod q in [0, q) for any 32-bit x
__device__ __forceinline__ uint32_t mul_shoup32c(uint32_t x, uint32_t w, uint32_t ws, uint32_t q) {
  const uint32_t r = mul_shoup32_lazy(x, w, ws, q);
  return min(r, r - q);  // r - q wraps above r when r < q
}

template <int M>
__device__ __forceinline__ void stage_twiddles2(Tw2* local, const Tw2* global, u64 tb, int tid, int nthreads) {
  for (int t = 1 + tid; t < (1 << M); t += nthreads) {
    const int s = 31 - __clz(t);
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(global + ((tb - 1) << s) + t));
    local[t] = Tw2{v.x, v.y, v.z, v.w};
  }
}

template <int M, int GI>
__device__ __forceinline__ void fwd_group2(uint2 (&v)[8], int l, const Tw2* __restrict__ tw, uint32_t q0,
                                           uint32_t q1) {
  constexpr int S0 = Grp<M, GI>::S0, G = Grp<M, GI>::G;
  const uint32_t t0 = q0 << 1, t1 = q1 << 1;
#pragma unroll
  for (int j = 0; j < G; ++j) {
    const int s = S0 + j;
    const int b = G - 1 - j;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (k & (1 << b)) continue;
      const int r = gidx<M, S0, G>(l, k);
      const Tw2 w = tw[(1 << s) + (r >> (M - s))];
      uint2 x = v[k];
      const uint2 y = v[k | (1 << b)];
      x.x = min(x.x, x.x - t0);  // x - t0 wraps above x when x < t0
      x.y = min(x.y, x.y - t1);
      const uint32_t u0 = mul_shoup32_lazy(y.x, w.w0, w.s0, q0);
      const uint32_t u1 = mul_shoup32_lazy(y.y, w.w1, w.s1, q1);
      v[k] = make_uint2(x.x + u0, x.y + u1);
      v[k | (1 << b)] = make_uint2(x.x - u0 + t0, x.y - u1 + t1);
    }
  }
}

template <int M, int GI, bool SC = false>
__device__ __forceinline__ void inv_group2(uint2 (&v)[8], int l, const Tw2* __restrict__ tw, uint32_t q0,
                                           uint32_t q1, const InvScale2& sc = InvScale2{}) {
  constexpr int S0 = Grp<M, GI>::S0, G = Grp<M, GI>::G;
  const uint32_t t0 = q0 << 1, t1 = q1 << 1;
#pragma unroll
  for (int j = G - 1; j >= 0; --j) {
    const int s = S0 + j;
    const int b = G - 1 - j;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (k & (1 << b)) continue;
      const uint2 x = v[k], y = v[k | (1 << b)];
      if (SC && s == 0) {  // the scale folded into the last stage, canonical outputs (see InvScale)
        v[k] = make_uint2(mul_shoup32c(x.x + y.x, sc.n0, sc.n0s, q0), mul_shoup32c(x.y + y.y, sc.n1, sc.n1s, q1));
        v[k | (1 << b)] = make_uint2(mul_shoup32c(x.x - y.x + t0, sc.wn0, sc.wn0s, q0),
                                     mul_shoup32c(x.y - y.y + t1, sc.wn1, sc.wn1s, q1));
        continue;
      }
      const int r = gidx<M, S0, G>(l, k);
      const Tw2 w = tw[(1 << s) + (r >> (M - s))];
      uint32_t a0 = x.x + y.x, a1 = x.y + y.y;
      a0 = a0 >= t0 ? a0 - t0 : a0;
      a1 = a1 >= t1 ? a1 - t1 : a1;
      v[k] = make_uint2(a0, a1);
      v[k | (1 << b)] = make_uint2(mul_shoup32_lazy(x.x - y.x + t0, w.w0, w.s0, q0),
                                   mul_shoup32_lazy(x.y - y.y + t1, w.w1, w.s1, q1));
    }
  }
}

template <int M, int GA, int GB>
__device__ __forceinline__ void exchange2(uint2 (&v)[8], uint2* buf, int l) {
#pragma unroll
  for (int k = 0; k < 8; ++k) buf[swz<M>(gidx<M, Grp<M, GA>::S0, Grp<M, GA>::G>(l, k))] = v[k];
  __syncwarp();
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = buf[swz<M>(gidx<M, Grp<M, GB>::S0, Grp<M, GB>::G>(l, k))];
  __syncwarp();
}

template <int M>
__device__ __forceinline__ void fwd_sub2(uint2 (&v)[8], uint2* buf, int l, const Tw2* tw, uint32_t q0, uint32_t q1) {
  fwd_group2<M, 0>(v, l, tw, q0, q1);
  exchange2<M, 0, 1>(v, buf, l);
  fwd_group2<M, 1>(v, l, tw, q0, q1);
  if constexpr (NGroups<M>::value == 3) {
    exchange2<M, 1, 2>(v, buf, l);
    fwd_group2<M, 2>(v, l, tw, q0, q1);
  }
}

template <int M, bool SC = false>
__device__ __forceinline__ void inv_sub2(uint2 (&v)[8], uint2* buf, int l, const Tw2* tw, uint32_t q0, uint32_t q1,
                                         const InvScale2& sc = InvScale2{}) {
  if constexpr (NGroups<M>::value == 3) {
    inv_group2<M, 2>(v, l, tw, q0, q1);
    exchange2<M, 2, 1>(v, buf, l);
  }
  inv_group2<M, 1>(v, l, tw, q0, q1);
  exchange2<M, 1, 0>(v, buf, l);
  inv_group2<M, 0, SC>(v, l, tw, q0, q1, sc);
}

}  // namespace core
}  // namespace rc
