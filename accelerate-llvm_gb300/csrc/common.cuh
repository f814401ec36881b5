// common.cuh -- element types, the fixed associative primitives, accumulator
// policies and sm_103a PTX helpers shared by every skeleton kernel.
//
// Primitive semantics follow accelerate-llvm:
//  * integer + and * wrap (no nsw/nuw flags: LLVM/AST/Type/Instruction.hs:429-473),
//    done here in unsigned arithmetic;
//  * integer min/max are `select` on <= / >= (CodeGen/Arithmetic.hs:456-466);
//  * float min/max are IEEE fmin/fmax (NaN-ignoring), CUDA's fminf/fmaxf/fmin/fmax;
//  * no fast-math: float + and * round to nearest, no contraction (__fadd_rn etc.).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <cuda.h>

#include "../../include/acc_gb300.h"
#include "runtime.h"

namespace accgb {

// ----------------------------------------------------------------- errors
// Every wait on another CTA or on a copy is bounded: it gives up after
// WAIT_LIMIT_NS of wall-clock time (%globaltimer), or after SPIN_LIMIT polls,
// whichever comes first.  The poll count alone is no time bound: a poll may
// suspend for microseconds (mbarrier.try_wait) or sleep longer than asked.
constexpr uint32_t SPIN_LIMIT = 1u << 24;
constexpr uint64_t WAIT_LIMIT_NS = 2000000000ull;  // 2 s

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ----------------------------------------------------------------- ops
template <int OP, class T> struct Prim;

template <class T> struct IntBits;
template <> struct IntBits<int32_t>  { using U = uint32_t; };
template <> struct IntBits<uint32_t> { using U = uint32_t; };
template <> struct IntBits<int64_t>  { using U = uint64_t; };
template <> struct IntBits<uint64_t> { using U = uint64_t; };

template <class T> __host__ __device__ constexpr bool is_float() {
  return sizeof(T) == 4 ? (T(0.5) != T(0)) : (T(0.5) != T(0));
}

template <class T> struct Lim;
template <> struct Lim<int32_t>  { __host__ __device__ static int32_t  lo() { return INT32_MIN; } __host__ __device__ static int32_t  hi() { return INT32_MAX; } };
template <> struct Lim<int64_t>  { __host__ __device__ static int64_t  lo() { return INT64_MIN; } __host__ __device__ static int64_t  hi() { return INT64_MAX; } };
template <> struct Lim<uint32_t> { __host__ __device__ static uint32_t lo() { return 0u; }        __host__ __device__ static uint32_t hi() { return 0xffffffffu; } };

__device__ __forceinline__ float  qnan_f() { return __int_as_float(0x7fc00000); }
__device__ __forceinline__ double qnan_d() { return __longlong_as_double(0x7ff8000000000000ll); }

// Identities: for float min/max the identity is NaN (fmin(NaN, x) = x and
// fmin(NaN, NaN) = NaN), for float + it is -0.0 (x + -0.0 = x for every x,
// signed zeros included).
template <class T> struct Prim<ACC_ADD, T> {
  __device__ __forceinline__ static T id() {
    if constexpr (std::is_same<T, float>::value) return -0.0f;
    else if constexpr (std::is_same<T, double>::value) return -0.0;
    else return T(0);
  }
  __device__ __forceinline__ static T ap(T a, T b) {
    if constexpr (std::is_same<T, float>::value) return __fadd_rn(a, b);
    else if constexpr (std::is_same<T, double>::value) return __dadd_rn(a, b);
    else { using U = typename IntBits<T>::U; return (T)((U)a + (U)b); }
  }
};
template <class T> struct Prim<ACC_MUL, T> {
  __device__ __forceinline__ static T id() { return T(1); }
  __device__ __forceinline__ static T ap(T a, T b) {
    if constexpr (std::is_same<T, float>::value) return __fmul_rn(a, b);
    else if constexpr (std::is_same<T, double>::value) return __dmul_rn(a, b);
    else { using U = typename IntBits<T>::U; return (T)((U)a * (U)b); }
  }
};
template <class T> struct Prim<ACC_MIN, T> {
  __device__ __forceinline__ static T id() {
    if constexpr (std::is_same<T, float>::value) return qnan_f();
    else if constexpr (std::is_same<T, double>::value) return qnan_d();
    else return Lim<T>::hi();
  }
  __device__ __forceinline__ static T ap(T a, T b) {
    if constexpr (std::is_same<T, float>::value) return fminf(a, b);
    else if constexpr (std::is_same<T, double>::value) return fmin(a, b);
    else return a <= b ? a : b;
  }
};
template <class T> struct Prim<ACC_MAX, T> {
  __device__ __forceinline__ static T id() {
    if constexpr (std::is_same<T, float>::value) return qnan_f();
    else if constexpr (std::is_same<T, double>::value) return qnan_d();
    else return Lim<T>::lo();
  }
  __device__ __forceinline__ static T ap(T a, T b) {
    if constexpr (std::is_same<T, float>::value) return fmaxf(a, b);
    else if constexpr (std::is_same<T, double>::value) return fmax(a, b);
    else return a >= b ? a : b;
  }
};
template <class T> struct Prim<ACC_AND, T> {
  __device__ __forceinline__ static T id() { return (T)~(typename IntBits<T>::U)0; }
  __device__ __forceinline__ static T ap(T a, T b) { return a & b; }
};
template <class T> struct Prim<ACC_OR, T> {
  __device__ __forceinline__ static T id() { return T(0); }
  __device__ __forceinline__ static T ap(T a, T b) { return a | b; }
};
template <class T> struct Prim<ACC_XOR, T> {
  __device__ __forceinline__ static T id() { return T(0); }
  __device__ __forceinline__ static T ap(T a, T b) { return a ^ b; }
};

// One element of a fused zipWith producer: g x y for the primitive g = zop,
// in the element type (integers wrap; __fmul_rn / __fadd_rn keep each
// product or sum rounded on its own, never contracted into the consumer's
// accumulation).
template <class T>
__device__ __forceinline__ T zip_elem(int zop, T x, T y) {
  switch (zop) {
    case ACC_ADD: return Prim<ACC_ADD, T>::ap(x, y);
    case ACC_MUL: return Prim<ACC_MUL, T>::ap(x, y);
    case ACC_MIN: return Prim<ACC_MIN, T>::ap(x, y);
    default: return Prim<ACC_MAX, T>::ap(x, y);
  }
}

// ----------------------------------------------------------------- accumulators
// An accumulator policy describes the running state S of a reduction over
// elements of T: lift one element, combine two states (left operand first),
// lower the state to a T.  Every S is at most 8 bytes, so it travels in one
// 64-bit shuffle pair and one look-back status slot.
enum { PREC_PLAIN = 0, PREC_COMP = 1, PREC_F64 = 2 };

struct F2 { float s, c; };  // compensated FP32: value s + error c

__device__ __forceinline__ F2 two_sum(float a, float b) {
  // Knuth's TwoSum: s + e == a + b exactly.
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return F2{s, e};
}

template <int OP, class T, int PREC> struct Acc {
  using S = T;
  __device__ __forceinline__ static S id() { return Prim<OP, T>::id(); }
  __device__ __forceinline__ static S lift(T x) { return x; }
  __device__ __forceinline__ static S comb(S a, S b) { return Prim<OP, T>::ap(a, b); }
  __device__ __forceinline__ static S push(S a, T x) { return Prim<OP, T>::ap(a, x); }
  __device__ __forceinline__ static T lower(S s) { return s; }
};

// Compensated Float32 (+): Neumaier-style pair accumulation.
template <> struct Acc<ACC_ADD, float, PREC_COMP> {
  using S = F2;
  __device__ __forceinline__ static S id() { return F2{-0.0f, 0.0f}; }
  __device__ __forceinline__ static S lift(float x) { return F2{x, 0.0f}; }
  __device__ __forceinline__ static S push(S a, float x) {
    F2 t = two_sum(a.s, x);
    return F2{t.s, __fadd_rn(a.c, t.c)};
  }
  __device__ __forceinline__ static S comb(S a, S b) {
    F2 t = two_sum(a.s, b.s);
    return F2{t.s, __fadd_rn(__fadd_rn(a.c, b.c), t.c)};
  }
  // A zero error term keeps the sign of a zero sum; a non-finite running sum
  // (overflow, inf, NaN) is returned as is, as the plain sum would be.
  __device__ __forceinline__ static float lower(S a) {
    if (a.c == 0.0f || !isfinite(a.s)) return a.s;
    return __fadd_rn(a.s, a.c);
  }
};

// FP64 accumulation of Float32 (+).
template <> struct Acc<ACC_ADD, float, PREC_F64> {
  using S = double;
  __device__ __forceinline__ static S id() { return -0.0; }
  __device__ __forceinline__ static S lift(float x) { return (double)x; }
  __device__ __forceinline__ static S push(S a, float x) { return __dadd_rn(a, (double)x); }
  __device__ __forceinline__ static S comb(S a, S b) { return __dadd_rn(a, b); }
  __device__ __forceinline__ static float lower(S a) { return __double2float_rn(a); }
};

// ----------------------------------------------------------------- bit casts
template <class S> __device__ __forceinline__ uint64_t to_bits(S v) {
  static_assert(sizeof(S) <= 8, "state too large");
  uint64_t r = 0;
  memcpy(&r, &v, sizeof(S));
  return r;
}
template <class S> __device__ __forceinline__ S from_bits(uint64_t b) {
  S v;
  memcpy(&v, &b, sizeof(S));
  return v;
}

// ----------------------------------------------------------------- warp helpers
template <class S> __device__ __forceinline__ S shfl_down(S v, int d) {
  if constexpr (sizeof(S) == 4) {
    uint32_t b; memcpy(&b, &v, 4);
    b = __shfl_down_sync(0xffffffffu, b, d);
    memcpy(&v, &b, 4); return v;
  } else {
    uint64_t b = to_bits(v);
    uint32_t lo = __shfl_down_sync(0xffffffffu, (uint32_t)b, d);
    uint32_t hi = __shfl_down_sync(0xffffffffu, (uint32_t)(b >> 32), d);
    return from_bits<S>(((uint64_t)hi << 32) | lo);
  }
}
template <class S> __device__ __forceinline__ S shfl_up(S v, int d) {
  if constexpr (sizeof(S) == 4) {
    uint32_t b; memcpy(&b, &v, 4);
    b = __shfl_up_sync(0xffffffffu, b, d);
    memcpy(&v, &b, 4); return v;
  } else {
    uint64_t b = to_bits(v);
    uint32_t lo = __shfl_up_sync(0xffffffffu, (uint32_t)b, d);
    uint32_t hi = __shfl_up_sync(0xffffffffu, (uint32_t)(b >> 32), d);
    return from_bits<S>(((uint64_t)hi << 32) | lo);
  }
}
template <class S> __device__ __forceinline__ S shfl_idx(S v, int src) {
  if constexpr (sizeof(S) == 4) {
    uint32_t b; memcpy(&b, &v, 4);
    b = __shfl_sync(0xffffffffu, b, src);
    memcpy(&v, &b, 4); return v;
  } else {
    uint64_t b = to_bits(v);
    uint32_t lo = __shfl_sync(0xffffffffu, (uint32_t)b, src);
    uint32_t hi = __shfl_sync(0xffffffffu, (uint32_t)(b >> 32), src);
    return from_bits<S>(((uint64_t)hi << 32) | lo);
  }
}

// Warp reduction that keeps the left-to-right order of lanes: after the call
// lane 0 holds v[0] `comb` v[1] `comb` ... `comb` v[31].
template <class A> __device__ __forceinline__ typename A::S warp_reduce(typename A::S v) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    typename A::S o = shfl_down(v, d);
    if ((threadIdx.x & 31) + d < 32) v = A::comb(v, o);
  }
  return v;
}

// Warp reduction in reversed lane order: lane 0 gets v[31] `comb` ... `comb` v[0].
template <class A> __device__ __forceinline__ typename A::S warp_reduce_rev(typename A::S v) {
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    typename A::S o = shfl_down(v, d);
    if ((threadIdx.x & 31) + d < 32) v = A::comb(o, v);
  }
  return v;
}

// Inclusive warp scan, left to right over lanes (Kogge-Stone with shfl.up).
template <class A> __device__ __forceinline__ typename A::S warp_scan_incl(typename A::S v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    typename A::S o = shfl_up(v, d);
    if (lane >= d) v = A::comb(o, v);
  }
  return v;
}
// Inclusive warp scan right to left over lanes: lane i gets v[i] `comb` ... `comb` v[31].
template <class A> __device__ __forceinline__ typename A::S warp_scan_incl_rev(typename A::S v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    typename A::S o = shfl_down(v, d);
    if (lane + d < 32) v = A::comb(v, o);
  }
  return v;
}

// ----------------------------------------------------------------- memory helpers
__device__ __forceinline__ uint4 ld_stream16(const void *p) {
  uint4 r;
  asm volatile("ld.global.nc.L1::no_allocate.L2::256B.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w) : "l"(p));
  return r;
}
template <class T> __device__ __forceinline__ T ld_stream(const T *p) {
  if constexpr (sizeof(T) == 4) {
    uint32_t v; asm volatile("ld.global.nc.L1::no_allocate.u32 %0, [%1];" : "=r"(v) : "l"(p));
    T r; memcpy(&r, &v, 4); return r;
  } else {
    uint64_t v; asm volatile("ld.global.nc.L1::no_allocate.u64 %0, [%1];" : "=l"(v) : "l"(p));
    T r; memcpy(&r, &v, 8); return r;
  }
}

__device__ __forceinline__ uint64_t ld_relaxed_u64(const uint64_t *p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(uint64_t *p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" :: "l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Both 64-bit words of a look-back status slot in one 16-byte access (slots
// are 16-byte aligned).  The pair is not read atomically; every word carries
// its own tag, so a reader rejects a pair taken from two publications.
// Loading a slot whole lets a poll issue all of its slot loads back to back
// instead of paying one round trip per word.
struct SlotWords { uint64_t w0, w1; };
__device__ __forceinline__ SlotWords ld_slot(const uint64_t *p) {
  SlotWords s;
  asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(s.w0), "=l"(s.w1) : "l"(p) : "memory");
  return s;
}

// Look-back window bookkeeping (warp-collective).  Lane l holds the slots at
// distances l * LB + i (0 = nearest predecessor) with flags fl: 0 not yet
// published, 1 a partial value, 2 a value the walk stops at (an inclusive
// prefix, or a tile that holds a segment end).
//
// Nearest lane holding a stop slot (32: none): the lanes after it need no
// more polling.
template <int LB>
__device__ __forceinline__ int lb_stop_lane(const uint32_t (&fl)[LB]) {
  bool seen = false;
#pragma unroll
  for (int i = 0; i < LB; ++i) seen = seen || fl[i] == 2u;
  const unsigned pm = __ballot_sync(0xffffffffu, seen);
  return pm ? __ffs(pm) - 1 : 32;
}
// Whether the window can be folded: `resolved` when it holds a stop slot and
// every slot nearer than the nearest one is published (the slots beyond it
// are not waited for), `whole` when it holds no stop slot and every slot is
// published.  Returns the nearest stop lane.
template <int LB>
__device__ __forceinline__ int lb_window(const uint32_t (&fl)[LB], bool &resolved, bool &whole) {
  bool all_ready = true, ready_to_p = true, seen = false;
#pragma unroll
  for (int i = 0; i < LB; ++i) {
    all_ready = all_ready && fl[i] != 0u;
    if (!seen) ready_to_p = ready_to_p && fl[i] != 0u;
    seen = seen || fl[i] == 2u;
  }
  const unsigned pm = __ballot_sync(0xffffffffu, seen);
  const unsigned rm = __ballot_sync(0xffffffffu, all_ready);
  const int kp = pm ? __ffs(pm) - 1 : 32;
  const unsigned below = kp >= 32 ? 0xffffffffu : ((1u << kp) - 1u);
  const bool kp_ready = __shfl_sync(0xffffffffu, ready_to_p, kp & 31);
  resolved = pm != 0u && (rm & below) == below && kp_ready;
  whole = pm == 0u && rm == 0xffffffffu;
  return kp;
}

// Coherent (L1-bypassing) load of a state written by another CTA of this grid.
template <class S> __device__ __forceinline__ S ld_state(const S *p) {
  if constexpr (sizeof(S) == 4) {
    return from_bits<S>(ld_relaxed_u32(reinterpret_cast<const uint32_t *>(p)));
  } else {
    return from_bits<S>(ld_relaxed_u64(reinterpret_cast<const uint64_t *>(p)));
  }
}

__device__ __forceinline__ void raise_error(uint32_t *err, uint32_t bits) {
  if (err) atomicOr(err, bits);
}

// ----------------------------------------------------------------- TMA / mbarrier
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
               :: "r"(smem_addr(bar)), "r"(bytes) : "memory");
}
// Bounded wait on an mbarrier phase.  Returns false if the wait gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t phase) {
  uint32_t addr = smem_addr(bar);
  uint64_t t0 = 0;
  for (uint32_t it = 0; it < SPIN_LIMIT; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done) : "r"(addr), "r"(phase) : "memory");
    if (done) return true;
    // The clock starts only once the wait is a long one: a wait that ends
    // within 64 polls (the usual TMA landing) reads no timer.
    if (it == 64) t0 = global_ns();
    if (it > 64) {
      if ((it & 15u) == 0 && global_ns() - t0 > WAIT_LIMIT_NS) return false;
      __nanosleep(64);
    }
  }
  return false;
}
// Bounded wait for a TMA load's mbarrier phase.  A wait that runs out raises
// DEV_ERR_TIMEOUT and waits once more (again bounded), so that a copy still
// in flight has twice the limit to land.  Returns whether the phase
// completed.  The caller makes the outcome CTA-uniform (__syncthreads_or)
// and, when the load did not land, returns without reading the buffer, without
// storing from it and without issuing another copy into it.
__device__ __forceinline__ bool mbar_wait_flagged(uint64_t *bar, uint32_t phase, uint32_t *err) {
  if (mbar_wait(bar, phase)) return true;
  raise_error(err, DEV_ERR_TIMEOUT);
  return mbar_wait(bar, phase);
}
// Bounded wait on an mbarrier phase that suspends the waiting threads (each
// try may sleep up to 2 us until the phase completes) instead of polling, so
// that waiting warps leave the issue slots to the CTAs that have work.  Gives
// up after WAIT_LIMIT_NS or 2^20 tries.  Returns false if it gave up.
__device__ __forceinline__ bool mbar_wait_sleep(uint64_t *bar, uint32_t phase) {
  uint32_t addr = smem_addr(bar);
  uint64_t t0 = 0;
  for (uint32_t it = 0; it < (1u << 20); ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done) : "r"(addr), "r"(phase), "r"(2000u) : "memory");
    if (done) return true;
    if (it == 0) t0 = global_ns();
    if ((it & 15u) == 15u && global_ns() - t0 > WAIT_LIMIT_NS) return false;
    if (it > 8) __nanosleep(128);  // in case a try returns early
  }
  return false;
}
// 2-D tiled TMA load (global -> shared), completion counted on `bar`.
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      :: "r"(smem_addr(dst)), "l"(map), "r"(x), "r"(y), "r"(smem_addr(bar)) : "memory");
}
// L2 cache policies for the hinted TMA copies below: keep a line (it will be
// read again soon) or let it go first (it will not).
__device__ __forceinline__ uint64_t l2_policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
// tma_load_2d with an L2 cache policy.
__device__ __forceinline__ void tma_load_2d_hint(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar,
                                                 uint64_t policy) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1, {%2, %3}], [%4], %5;"
      :: "r"(smem_addr(dst)), "l"(map), "r"(x), "r"(y), "r"(smem_addr(bar)), "l"(policy) : "memory");
}
// tma_store_2d with an L2 cache policy.
__device__ __forceinline__ void tma_store_2d_hint(const CUtensorMap *map, int x, int y, const void *src,
                                                  uint64_t policy) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group.L2::cache_hint [%0, {%1, %2}], [%3], %4;"
               :: "l"(map), "r"(x), "r"(y), "r"(smem_addr(src)), "l"(policy) : "memory");
}
// 2-D tiled TMA store (shared -> global); out-of-range rows/cols are clipped.
__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, int x, int y, const void *src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];"
               :: "l"(map), "r"(x), "r"(y), "r"(smem_addr(src)) : "memory");
}
__device__ __forceinline__ void tma_store_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void tma_store_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void tma_store_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// Plain arrival on an mbarrier (no transaction bytes).
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(smem_addr(bar)) : "memory");
}
// Barrier among the first THREADS threads of the CTA only (named barrier ID,
// 1..15; 0 is __syncthreads), so that warps with other roles take no part.
template <int ID, int THREADS>
__device__ __forceinline__ void named_bar_sync() {
  asm volatile("bar.sync %0, %1;" :: "n"(ID), "n"(THREADS) : "memory");
}
// The same barrier, returning whether v holds in any of those threads.
template <int ID, int THREADS>
__device__ __forceinline__ bool named_bar_or(bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.or.pred q, %2, %3, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r) : "r"((uint32_t)v), "n"(ID), "n"(THREADS) : "memory");
  return r != 0u;
}
__device__ __forceinline__ void prefetch_tmap(const CUtensorMap *map) {
  asm volatile("prefetch.tensormap [%0];" :: "l"(map) : "memory");
}

// ----------------------------------------------------------------- misc
__host__ __device__ __forceinline__ int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace accgb
