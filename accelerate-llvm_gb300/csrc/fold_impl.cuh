// fold_impl.cuh -- the fold kernels, shared by acc_fold (fold.cu) and the
// fused-producer folds acc_fold_zipwith and acc_fold_map (fold_zip.cu).
//
// The reference reduces a vector with a host-driven chain of launches
// (foldAllM1, then foldAllM2 re-launched until one element is left:
// accelerate-llvm-ptx/src/Data/Array/Accelerate/LLVM/PTX/Execute.hs:267-318,
// PTX/CodeGen/Fold.hs:175-285) and a rank >= 2 array with one CTA per row
// (Fold.hs:296-405).  Here every shape is one launch:
//   * fold_rows_thread  -- inner <= 16: one thread per row;
//   * fold_rows_warp    -- short rows, many of them: one warp per row;
//   * fold_split        -- long rows: a row is cut over G CTAs, each thread
//                          streams 16-byte vectors (4 in flight), the CTA
//                          partial goes to scratch, and the last CTA of the
//                          row (atomic ticket) folds the G partials in order
//                          and applies the seed.
// The seed combines on the left, z `f` (x0 `f` ...), as reduceFromTo does
// (accelerate-llvm-native/.../Native/CodeGen/Fold.hs:248-260).  Float32 (+)
// accumulates with a compensated two-sum by default.
#pragma once
#include "common.cuh"

namespace accgb {


// The folded input: one array (ZOP = NO_ZIP), the fused producer
// `zipWith zop p q` of two arrays of the same shape for a primitive zop
// (ZOP < MAP_BASE), or the fused producer `map (\x -> g x c) p` for a
// primitive g = ZOP - MAP_BASE and a constant c (ZOP >= MAP_BASE).
constexpr int NO_ZIP = -1;
constexpr int MAP_BASE = 16;
template <int ZOP> constexpr bool zips() { return ZOP != NO_ZIP && ZOP < MAP_BASE; }
template <int ZOP> constexpr bool maps() { return ZOP >= MAP_BASE; }

template <int ZOP, class T>
__device__ __forceinline__ T zip_at(const T *p, const T *q, int64_t i, T c) {
  if constexpr (ZOP == NO_ZIP) { (void)q; (void)c; return ld_stream(p + i); }
  else if constexpr (maps<ZOP>()) { (void)q; return Prim<ZOP - MAP_BASE, T>::ap(ld_stream(p + i), c); }
  else { (void)c; return Prim<ZOP, T>::ap(ld_stream(p + i), ld_stream(q + i)); }
}

// Fold the span [0, len) of the input as participant t of nt (16-byte vector
// body, scalar head / tail), returning this participant's partial state.
// Two zipped arrays take the vector body when they share their 16-byte
// alignment phase, and a scalar stride otherwise.
template <class A, class T, int ZOP = NO_ZIP>
__device__ __forceinline__ typename A::S reduce_span(const T *p, int64_t len, int64_t t, int64_t nt,
                                                     const T *q = nullptr, T c = T{}) {
  using S = typename A::S;
  constexpr int VEC = 16 / sizeof(T);
  S acc = A::id();
  const uintptr_t addr = reinterpret_cast<uintptr_t>(p);
  if constexpr (zips<ZOP>()) {
    if (((addr ^ reinterpret_cast<uintptr_t>(q)) & 15u) != 0u) {
      for (int64_t i = t; i < len; i += nt) acc = A::push(acc, zip_at<ZOP, T>(p, q, i, c));
      return acc;
    }
  }
  int64_t head = (int64_t)(((16u - (addr & 15u)) & 15u) / sizeof(T));
  if (head > len) head = len;
  if (t < head) acc = A::push(acc, zip_at<ZOP, T>(p, q, t, c));
  const int64_t nvec = (len - head) / VEC;
  const uint4 *pv = reinterpret_cast<const uint4 *>(p + head);
  const uint4 *qv = reinterpret_cast<const uint4 *>(q + head);
  auto push_vec = [&](const uint4 &v, const uint4 &w) {
    T e[VEC];
    memcpy(e, &v, 16);
    if constexpr (zips<ZOP>()) {
      T f[VEC];
      memcpy(f, &w, 16);
#pragma unroll
      for (int k = 0; k < VEC; ++k) e[k] = Prim<ZOP, T>::ap(e[k], f[k]);
    } else if constexpr (maps<ZOP>()) {
      (void)w;
#pragma unroll
      for (int k = 0; k < VEC; ++k) e[k] = Prim<ZOP - MAP_BASE, T>::ap(e[k], c);
    } else {
      (void)w;
    }
#pragma unroll
    for (int k = 0; k < VEC; ++k) acc = A::push(acc, e[k]);
  };
  int64_t i = t;
  for (; i + 3 * nt < nvec; i += 4 * nt) {
    uint4 v[4], w[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      v[u] = ld_stream16(pv + i + u * nt);
      if constexpr (zips<ZOP>()) w[u] = ld_stream16(qv + i + u * nt);
      else w[u] = v[u];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) push_vec(v[u], w[u]);
  }
  for (; i < nvec; i += nt) {
    const uint4 v = ld_stream16(pv + i);
    uint4 w = v;
    if constexpr (zips<ZOP>()) w = ld_stream16(qv + i);
    push_vec(v, w);
  }
  const int64_t tail0 = head + nvec * VEC;
  if (tail0 + t < len) acc = A::push(acc, zip_at<ZOP, T>(p, q, tail0 + t, c));
  return acc;
}

// CTA-wide ordered reduction; the result is valid in thread 0.
template <class A>
__device__ __forceinline__ typename A::S block_reduce(typename A::S v) {
  using S = typename A::S;
  __shared__ S s_part[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
  v = warp_reduce<A>(v);
  if (lane == 0) s_part[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = lane < nw ? s_part[lane] : A::id();
    v = warp_reduce<A>(v);
  }
  __syncthreads();
  return v;
}

struct FoldArgs {
  const void *in;
  void *out;
  const void *in2;  // second input of a fused zipWith, or null
  int64_t outer, inner;
  uint64_t seed;
  int has_seed;
  uint64_t mapc;    // the constant of a fused map (bits of one element)
};

template <int OP, class T, int PREC, int ZOP = NO_ZIP>
__global__ void __launch_bounds__(256) fold_rows_thread(FoldArgs a) {
  using A = Acc<OP, T, PREC>;
  const T *in = static_cast<const T *>(a.in);
  const T *in2 = static_cast<const T *>(a.in2);
  T *out = static_cast<T *>(a.out);
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < a.outer; r += (int64_t)gridDim.x * blockDim.x) {
    const T *p = in + r * a.inner;
    const T *q = zips<ZOP>() ? in2 + r * a.inner : nullptr;
    const T c = from_bits<T>(a.mapc);
    typename A::S acc = a.has_seed ? A::lift(from_bits<T>(a.seed)) : A::lift(zip_at<ZOP, T>(p, q, 0, c));
    for (int64_t i = a.has_seed ? 0 : 1; i < a.inner; ++i) acc = A::push(acc, zip_at<ZOP, T>(p, q, i, c));
    out[r] = A::lower(acc);
  }
}

template <int OP, class T, int PREC, int ZOP = NO_ZIP>
__global__ void __launch_bounds__(256) fold_rows_warp(FoldArgs a) {
  using A = Acc<OP, T, PREC>;
  const T *in = static_cast<const T *>(a.in);
  const T *in2 = static_cast<const T *>(a.in2);
  T *out = static_cast<T *>(a.out);
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = gw; r < a.outer; r += nw) {
    typename A::S acc = reduce_span<A, T, ZOP>(in + r * a.inner, a.inner, lane, 32,
                                               zips<ZOP>() ? in2 + r * a.inner : nullptr, from_bits<T>(a.mapc));
    acc = warp_reduce<A>(acc);
    if (lane == 0) {
      if (a.has_seed) acc = A::comb(A::lift(from_bits<T>(a.seed)), acc);
      out[r] = A::lower(acc);
    }
  }
}

struct SplitArgs {
  const void *in;
  void *out;
  const void *in2;    // second input of a fused zipWith, or null
  int64_t outer, inner;
  int64_t G;          // CTAs per row
  void *partials;     // outer * G states
  uint32_t *tickets;  // outer counters, zero between launches
  uint64_t seed;
  int has_seed;
  uint64_t mapc;      // the constant of a fused map (bits of one element)
};

template <int OP, class T, int PREC, int ZOP = NO_ZIP>
__global__ void __launch_bounds__(256) fold_split(SplitArgs a) {
  using A = Acc<OP, T, PREC>;
  using S = typename A::S;
  __shared__ bool s_last;
  const int64_t G = a.G;
  S *parts = static_cast<S *>(a.partials);
  for (int64_t job = blockIdx.x; job < a.outer * G; job += gridDim.x) {
    const int64_t r = job / G, g = job % G;
    const T *p = static_cast<const T *>(a.in) + r * a.inner;
    const T *q = zips<ZOP>() ? static_cast<const T *>(a.in2) + r * a.inner : nullptr;
    S acc = reduce_span<A, T, ZOP>(p, a.inner, g * blockDim.x + threadIdx.x, G * blockDim.x, q,
                                   from_bits<T>(a.mapc));
    acc = block_reduce<A>(acc);
    if (threadIdx.x == 0) {
      parts[r * G + g] = acc;
      __threadfence();
      const uint32_t prev = atomicAdd(a.tickets + r, 1u);
      s_last = prev == (uint32_t)(G - 1);
    }
    __syncthreads();
    if (s_last) {
      // Last CTA of this row: fold the G partials in order.
      __threadfence();
      // Each thread folds a contiguous run of partials, so that the CTA-wide
      // ordered reduction keeps the partials in order.
      S v = A::id();
      const int64_t per = (G + blockDim.x - 1) / blockDim.x;
      const int64_t b = threadIdx.x * per, e = b + per < G ? b + per : G;
      for (int64_t i = b; i < e; ++i) v = A::comb(v, ld_state<S>(&parts[r * G + i]));
      v = block_reduce<A>(v);
      if (threadIdx.x == 0) {
        if (a.has_seed) v = A::comb(A::lift(from_bits<T>(a.seed)), v);
        static_cast<T *>(a.out)[r] = A::lower(v);
        a.tickets[r] = 0u;  // re-arm for the next launch
      }
    }
    __syncthreads();
  }
}

// ----------------------------------------------------------------- host side
template <int OP, class T, int PREC, int ZOP = NO_ZIP>
int fold_typed(Workspace *w, const T *in, T *out, int64_t outer, int64_t inner, bool has_seed,
               uint64_t seed, cudaStream_t s, const T *in2 = nullptr, uint64_t mapc = 0) {
  using S = typename Acc<OP, T, PREC>::S;
  const Device &d = device_info();
  FoldArgs fa{in, out, in2, outer, inner, seed, has_seed, mapc};
  if (inner <= 16) {
    int64_t blocks = cdiv_h(outer, 256);
    if (blocks > (int64_t)d.sms * 16) blocks = (int64_t)d.sms * 16;
    fold_rows_thread<OP, T, PREC, ZOP><<<(unsigned)blocks, 256, 0, s>>>(fa);
    return check_launch();
  }
  const int64_t row_bytes = inner * (int64_t)sizeof(T);
  // Enough rows to fill the machine with one warp each, and rows short
  // enough that one warp streams them quickly: a warp per row.
  if (row_bytes <= (32 << 10) && outer >= (int64_t)d.sms * 8) {
    int64_t blocks = cdiv_h(outer, 8);
    if (blocks > (int64_t)d.sms * 32) blocks = (int64_t)d.sms * 32;
    fold_rows_warp<OP, T, PREC, ZOP><<<(unsigned)blocks, 256, 0, s>>>(fa);
    return check_launch();
  }
  // Split each row over G CTAs: aim at ~4 resident CTAs of 256 threads per SM
  // over the whole grid, each thread with at least 4 vectors to stream.
  const int64_t vec_per_row = cdiv_h(row_bytes * (zips<ZOP>() ? 2 : 1), 16);
  int64_t G = cdiv_h((int64_t)d.sms * 4, outer);
  const int64_t gmax = cdiv_h(vec_per_row, 256 * 4);
  if (G > gmax) G = gmax;
  if (G < 1) G = 1;
  const int64_t jobs = outer * G;
  int st = ws_words(w, W_ROWTICKET0 + (size_t)outer);
  if (st) return st;
  st = ws_scratch(w, (size_t)jobs * sizeof(S));
  if (st) return st;
  SplitArgs sa{in, out, in2, outer, inner, G, w->scratch, w->words + W_ROWTICKET0, seed, has_seed, mapc};
  int64_t blocks = jobs;
  if (blocks > (int64_t)d.sms * 8) blocks = (int64_t)d.sms * 8;
  fold_split<OP, T, PREC, ZOP><<<(unsigned)blocks, 256, 0, s>>>(sa);
  return check_launch();
}

}  // namespace accgb
