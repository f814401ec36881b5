// foldseg.cu -- foldSeg f z / fold1Seg f over a segment-offset array.
//
// The reference picks ONE kernel for the whole array from the average
// segment length: a warp per segment or a CTA per segment
// (accelerate-llvm-ptx/src/Data/Array/Accelerate/LLVM/PTX/Execute.hs:343-374,
// PTX/CodeGen/FoldSeg.hs:79-458), so skewed (lognormal) lengths leave most
// lanes idle or most CTAs waiting on a few long segments.  Here each segment
// is dispatched by its own length, in two launches:
//   1. seg_classify lists the segments longer than LONG_SEG (atomic append;
//      the order of the list does not matter, each segment is reduced alone);
//   2. foldseg_main: the first CTAs stream the listed long segments, one CTA
//      per segment with 16-byte vector loads; every other warp owns 32
//      consecutive segments and reduces the short ones (<= SHORT_SEG) one per
//      lane, serially, and the medium ones with the whole warp.
// Per segment the result is z `f` (x_u `f` ... `f` x_(v-1)), as the native
// backend's reduceFromTo over [seg[i], seg[i+1]) (accelerate-llvm-native/src/
// Data/Array/Accelerate/LLVM/Native/CodeGen/FoldSeg.hs:103-141).  An empty
// segment gives z with a seed and is left unwritten without one
// (PTX/CodeGen/FoldSeg.hs:170-178).  Offsets that decrease or run past the
// row are skipped and raise ACC_ERR_INDEX instead of reading out of bounds.
#include "common.cuh"

namespace accgb {

constexpr int SHORT_SEG = 32;
constexpr int64_t LONG_SEG = 2048;

struct SegArgs {
  const void *in;
  const void *off;
  void *out;
  int64_t outer, inner, nseg;
  int off64;
  uint64_t seed;
  int has_seed;
  uint32_t *nlong;     // number of listed long segments
  int64_t *longs;      // listed long segment ids
  int64_t long_ctas;   // CTAs [0, long_ctas) work on the list
  int64_t long_cap;    // capacity of the list
  uint32_t *err;
};

__device__ __forceinline__ int64_t seg_off(const SegArgs &a, int64_t i) {
  return a.off64 ? static_cast<const int64_t *>(a.off)[i] : (int64_t) static_cast<const int32_t *>(a.off)[i];
}

__global__ void seg_classify(SegArgs a) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < a.nseg; s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = seg_off(a, s), v = seg_off(a, s + 1);
    if (v - u > LONG_SEG && u >= 0 && v <= a.inner) {
      const uint32_t k = atomicAdd(a.nlong, 1u);
      // Valid offsets give at most inner / LONG_SEG long segments; overlapping
      // (malformed) offsets could give more: never write past the list.
      if ((int64_t)k >= a.long_cap) { raise_error(a.err, DEV_ERR_INDEX); continue; }
      a.longs[k] = s;
    }
  }
}

// Same vector streaming as the fold kernels, 4 x 16 B in flight per thread.
template <class A, class T>
__device__ __forceinline__ typename A::S seg_span(const T *p, int64_t len, int64_t t, int64_t nt) {
  using S = typename A::S;
  constexpr int VEC = 16 / sizeof(T);
  S acc = A::id();
  const uintptr_t addr = reinterpret_cast<uintptr_t>(p);
  int64_t head = (int64_t)(((16u - (addr & 15u)) & 15u) / sizeof(T));
  if (head > len) head = len;
  if (t < head) acc = A::push(acc, ld_stream(p + t));
  const int64_t nvec = (len - head) / VEC;
  const uint4 *qv = reinterpret_cast<const uint4 *>(p + head);
  int64_t i = t;
  for (; i + 3 * nt < nvec; i += 4 * nt) {
    uint4 v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) v[u] = ld_stream16(qv + i + u * nt);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      T e[VEC];
      memcpy(e, &v[u], 16);
#pragma unroll
      for (int k = 0; k < VEC; ++k) acc = A::push(acc, e[k]);
    }
  }
  for (; i < nvec; i += nt) {
    uint4 v = ld_stream16(qv + i);
    T e[VEC];
    memcpy(e, &v, 16);
#pragma unroll
    for (int k = 0; k < VEC; ++k) acc = A::push(acc, e[k]);
  }
  const int64_t tail0 = head + nvec * VEC;
  if (tail0 + t < len) acc = A::push(acc, ld_stream(p + tail0 + t));
  return acc;
}

template <int OP, class T, int PREC>
__global__ void __launch_bounds__(256) foldseg_main(SegArgs a) {
  using A = Acc<OP, T, PREC>;
  using S = typename A::S;
  const T *in = static_cast<const T *>(a.in);
  T *out = static_cast<T *>(a.out);
  const int lane = threadIdx.x & 31;
  __shared__ S s_part[8];

  if ((int64_t)blockIdx.x < a.long_ctas) {
    // ---- long segments: one CTA per (row, listed segment)
    int64_t nl = (int64_t)ld_relaxed_u32(a.nlong);
    if (nl > a.long_cap) nl = a.long_cap;
    for (int64_t job = blockIdx.x; job < nl * a.outer; job += a.long_ctas) {
      const int64_t r = job / nl, s = a.longs[job % nl];
      const int64_t u = seg_off(a, s), v = seg_off(a, s + 1);
      S acc = seg_span<A, T>(in + r * a.inner + u, v - u, threadIdx.x, blockDim.x);
      acc = warp_reduce<A>(acc);
      if (lane == 0) s_part[threadIdx.x >> 5] = acc;
      __syncthreads();
      if (threadIdx.x == 0) {
        S t = s_part[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) t = A::comb(t, s_part[w]);
        if (a.has_seed) t = A::comb(A::lift(from_bits<T>(a.seed)), t);
        out[r * a.nseg + s] = A::lower(t);
      }
      __syncthreads();
    }
    return;
  }

  // ---- short and medium segments: a warp per group of 32 segments
  const int64_t groups = (a.nseg + 31) / 32;
  const int64_t gw = (((int64_t)blockIdx.x - a.long_ctas) * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = (((int64_t)gridDim.x - a.long_ctas) * blockDim.x) >> 5;
  for (int64_t job = gw; job < groups * a.outer; job += nw) {
    const int64_t r = job / groups, g = job % groups;
    const int64_t s = g * 32 + lane;
    const T *row = in + r * a.inner;
    int64_t u = 0, v = 0;
    bool valid = s < a.nseg;
    if (valid) {
      u = seg_off(a, s);
      v = seg_off(a, s + 1);
      if (u < 0 || v < u || v > a.inner) {
        raise_error(a.err, DEV_ERR_INDEX);
        valid = false;
      }
    }
    const int64_t len = valid ? v - u : 0;
    // short: this lane alone, left to right from the seed
    if (valid && len <= SHORT_SEG) {
      if (len > 0 || a.has_seed) {
        S acc;
        int64_t i = u;
        if (a.has_seed) acc = A::lift(from_bits<T>(a.seed));
        else acc = A::lift(row[i++]);
        for (; i < v; ++i) acc = A::push(acc, row[i]);
        out[r * a.nseg + s] = A::lower(acc);
      }
    }
    // medium: the whole warp, one segment at a time
    unsigned med = __ballot_sync(0xffffffffu, valid && len > SHORT_SEG && len <= LONG_SEG);
    while (med) {
      const int src = __ffs(med) - 1;
      med &= med - 1;
      const int64_t mu = __shfl_sync(0xffffffffu, u, src);
      const int64_t mv = __shfl_sync(0xffffffffu, v, src);
      S acc = seg_span<A, T>(row + mu, mv - mu, lane, 32);
      acc = warp_reduce<A>(acc);
      if (lane == 0) {
        if (a.has_seed) acc = A::comb(A::lift(from_bits<T>(a.seed)), acc);
        out[r * a.nseg + g * 32 + src] = A::lower(acc);
      }
    }
  }
}

// ----------------------------------------------------------------- host side
template <int OP, class T, int PREC>
int foldseg_typed(Workspace *w, const T *in, const void *off, int off64, T *out, int64_t outer,
                  int64_t inner, int64_t nseg, bool has_seed, uint64_t seed, cudaStream_t s) {
  const Device &d = device_info();
  // Scratch: the list of long segments (at most inner / LONG_SEG of them).
  int64_t maxlong = inner / LONG_SEG + 1;
  if (maxlong > nseg) maxlong = nseg;
  int st = ws_scratch(w, (size_t)maxlong * sizeof(int64_t) + 256);
  if (st) return st;
  SegArgs a{};
  a.in = in; a.off = off; a.out = out;
  a.outer = outer; a.inner = inner; a.nseg = nseg; a.off64 = off64;
  a.seed = seed; a.has_seed = has_seed;
  a.nlong = w->words + W_SEGBIG;
  a.longs = static_cast<int64_t *>(w->scratch);
  a.long_cap = maxlong;
  a.err = w->words + W_ERR;
  // Only a row longer than LONG_SEG can hold a long segment.
  a.long_ctas = 0;
  if (inner > LONG_SEG) {
    cudaError_t e = cudaMemsetAsync(a.nlong, 0, sizeof(uint32_t), s);
    if (e != cudaSuccess) return cuda_status(e);
    int64_t cb = cdiv_h(nseg, 256);
    if (cb > (int64_t)d.sms * 8) cb = (int64_t)d.sms * 8;
    seg_classify<<<(unsigned)cb, 256, 0, s>>>(a);
    st = check_launch();
    if (st) return st;
    a.long_ctas = (int64_t)d.sms * 2;
  }
  const int64_t groups = cdiv_h(nseg, 32) * outer;
  int64_t sb = cdiv_h(groups, 8);
  if (sb > (int64_t)d.sms * 64) sb = (int64_t)d.sms * 64;
  if (sb < 1) sb = 1;
  foldseg_main<OP, T, PREC><<<(unsigned)(a.long_ctas + sb), 256, 0, s>>>(a);
  return check_launch();
}

int foldseg_dispatch(Workspace *w, int op, int type, int prec, const void *in, const void *off,
                     int off64, void *out, int64_t outer, int64_t inner, int64_t nseg,
                     const void *seed, cudaStream_t s) {
  return with_type(type, [&](auto tv) -> int {
    using T = decltype(tv);
    const uint64_t sb = seed_bits<T>(seed);
    return with_op<T>(op, [&](auto opc) -> int {
      constexpr int OP = decltype(opc)::value;
      return with_prec<OP, T>(prec, [&](auto pc) -> int {
        constexpr int P = decltype(pc)::value;
        return foldseg_typed<OP, T, P>(w, static_cast<const T *>(in), off, off64, static_cast<T *>(out),
                                       outer, inner, nseg, seed != nullptr, sb, s);
      });
    });
  });
}

}  // namespace accgb

using namespace accgb;

static int fold_seg_check(int type, int offset_type, const void *in, const void *offsets, void *out,
                          int64_t outer, int64_t inner, int64_t nseg) {
  if (outer < 0 || inner < 0 || nseg < 0) return ACC_ERR_INVALID;
  if (offset_type != ACC_I32 && offset_type != ACC_I64) return ACC_ERR_INVALID;
  if (type < ACC_I32 || type > ACC_F64) return ACC_ERR_INVALID;
  if (outer > 0 && nseg > 0 && (!offsets || !out)) return ACC_ERR_INVALID;
  if (outer > 0 && inner > 0 && nseg > 0 && !in) return ACC_ERR_INVALID;
  return ACC_OK;
}

extern "C" int acc_fold_seg(int op, int type, int prec, const void *in, const void *offsets,
                            int offset_type, void *out, int64_t outer, int64_t inner, int64_t nseg,
                            const void *seed, void *stream) {
  int st = fold_seg_check(type, offset_type, in, offsets, out, outer, inner, nseg);
  if (st) return st;
  if (outer == 0 || nseg == 0) return ACC_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Workspace *w = workspace(s, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  return foldseg_dispatch(w, op, type, prec, in, offsets, offset_type == ACC_I64, out, outer, inner, nseg, seed, s);
}

extern "C" int acc_fold_seg_lengths(int op, int type, int prec, const void *in, const void *lengths,
                                    int length_type, void *out, int64_t outer, int64_t inner,
                                    int64_t nseg, const void *seed, void *stream) {
  int st = fold_seg_check(type, length_type, in, lengths, out, outer, inner, nseg);
  if (st) return st;
  if (outer == 0 || nseg == 0) return ACC_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Workspace *w = workspace(s, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  // The offsets live at the END of the scratch area, after the long list.
  const size_t esz = length_type == ACC_I64 ? 8 : 4;
  const size_t list_bytes = (size_t)(inner / LONG_SEG + 2) * sizeof(int64_t) + 256;
  const size_t off_bytes = (size_t)(nseg + 1) * esz;
  st = ws_scratch(w, list_bytes + off_bytes + 256);
  if (st) return st;
  void *offsets = static_cast<char *>(w->scratch) + ((list_bytes + 255) & ~size_t(255));
  st = scan_offsets(w, length_type, lengths, offsets, nseg, s);
  if (st) return st;
  return foldseg_dispatch(w, op, type, prec, in, offsets, length_type == ACC_I64, out, outer, inner, nseg, seed, s);
}
