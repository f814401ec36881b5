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
#include <cstdlib>
#include <cstring>

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

// ----------------------------------------------------------------- segmented single pass
// Rows of 1-D values with 16-byte aligned storage take this path: the values
// are cut into tiles of 256 rows x 128 B (TMA, 128-byte swizzle, as in the
// scan), independent of the segment lengths, so every CTA streams the same
// number of bytes however skewed the segmentation is.
//   pre-pass  seg_tiles_kernel: tile_seg[k] = the segment that contains the
//             first element of tile k; empty segments get their seed here.
//   main      foldseg_scan_kernel: a tile's segment ENDS (off[s+1], tile-
//             relative, 16-bit) go to shared memory; each thread folds its
//             128-byte row, restarting after every end; rows combine with a
//             segmented warp / CTA scan ((f1,v1).(f2,v2) = (f1|f2, f2 ? v2 :
//             v1 `f` v2)); the value carried into the tile comes from a
//             segmented decoupled look-back that stops at the first
//             predecessor holding an end; a second pass over the row writes
//             z `f` (segment) where each segment's last element lies.
constexpr int FS_THREADS = 256;
constexpr int FS_ROW_BYTES = 128;
constexpr int FS_CAP = 2048;  // segment ends per tile held in shared memory

struct SegScanArgs {
  const void *in;
  const void *off;
  void *out;
  int64_t inner, nseg;
  int off64;
  uint64_t seed;
  int has_seed;
  int64_t full_rows, ntiles;
  int64_t *tile_seg;
  uint64_t *status;
  uint32_t *ticket;
  uint32_t *err;
  uint32_t epoch;
};

__device__ __forceinline__ int64_t seg_off2(const SegScanArgs &a, int64_t i) {
  return a.off64 ? static_cast<const int64_t *>(a.off)[i] : (int64_t) static_cast<const int32_t *>(a.off)[i];
}

template <class T>
__global__ void seg_tiles_kernel(SegScanArgs a, int64_t tile_elems) {
  const T z = from_bits<T>(a.seed);
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < a.nseg; s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = seg_off2(a, s), v = seg_off2(a, s + 1);
    if (u < 0 || v < u || v > a.inner) { raise_error(a.err, DEV_ERR_INDEX); continue; }
    if (u == v) {
      if (a.has_seed) static_cast<T *>(a.out)[s] = z;
      continue;
    }
    for (int64_t k = (u + tile_elems - 1) / tile_elems; k * tile_elems < v; ++k) a.tile_seg[k] = s;
  }
}

// Look-back slot of the segmented scan: tag = epoch << 3 | end-seen << 2 | flag.
template <class S>
__device__ __forceinline__ void publish_seg(uint64_t *status, int64_t t, uint32_t epoch, uint32_t flag, bool end, S v) {
  uint64_t b = to_bits(v);
  uint64_t tag = (uint64_t)((epoch << 3) | ((uint32_t)end << 2) | flag) << 32;
  if constexpr (sizeof(S) == 8) st_relaxed_u64(status + 2 * t + 1, tag | (b >> 32));
  st_relaxed_u64(status + 2 * t, tag | (b & 0xffffffffull));
}
template <class S>
__device__ __forceinline__ uint32_t decode_seg(SlotWords s, uint32_t epoch, S &v, bool &end) {
  const uint32_t tag = (uint32_t)(s.w0 >> 32);
  if ((tag >> 3) != epoch) return 0;
  uint64_t b = s.w0 & 0xffffffffull;
  if constexpr (sizeof(S) == 8) {
    if ((uint32_t)(s.w1 >> 32) != tag) return 0;
    b |= (s.w1 & 0xffffffffull) << 32;
  }
  v = from_bits<S>(b);
  end = (tag >> 2) & 1u;
  return tag & 3u;
}

template <int OP, class T, int PREC>
__global__ void __launch_bounds__(FS_THREADS, 3)
foldseg_scan_kernel(const __grid_constant__ CUtensorMap tin, SegScanArgs a) {
  using A = Acc<OP, T, PREC>;
  using S = typename A::S;
  constexpr int ITEMS = FS_ROW_BYTES / sizeof(T);
  constexpr int VEC = 16 / sizeof(T);
  constexpr int TE = FS_THREADS * ITEMS;
  constexpr int NWARP = FS_THREADS / 32;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *buf = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ uint64_t bar;
  __shared__ int64_t s_tile, s_lo, s_cnt, s_off0;
  __shared__ uint16_t s_end[FS_CAP];
  __shared__ S s_warp[NWARP];
  __shared__ int s_wend[NWARP];
  __shared__ S s_carry;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const T idT = Prim<OP, T>::id();

  if (tid == 0) {
    const uint32_t dyn = atomicAdd(a.ticket, 1u);
    if ((int64_t)dyn == a.ntiles - 1) *a.ticket = 0u;
    const int64_t tile = dyn;
    s_tile = tile;
    mbar_init(&bar, 1);
    fence_mbar_init();
    mbar_expect_tx(&bar, FS_THREADS * FS_ROW_BYTES);
    tma_load_2d(buf, &tin, 0, (int)(tile * FS_THREADS), &bar);
    const int64_t b = tile * TE;
    const int64_t off0 = seg_off2(a, 0);
    auto first_seg = [&](int64_t k) -> int64_t {
      if (k >= a.ntiles) return a.nseg;
      const int64_t s = a.tile_seg[k];
      if (s >= 0) return s;
      return k * TE < off0 ? 0 : a.nseg;  // tile starts before the first / after the last segment
    };
    const int64_t lo = first_seg(tile), hi = first_seg(tile + 1);
    s_lo = lo;
    s_cnt = hi > lo ? hi - lo : 0;
    s_off0 = off0 > b ? off0 - b : 0;  // elements of this tile before the first segment
  }
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t b = tile * TE;
  const int64_t lo = s_lo, cnt = s_cnt;
  const int off0 = (int)(s_off0 < TE ? s_off0 : TE);
  const bool in_smem_list = cnt <= FS_CAP;
  // Segment s_lo + i ends at tile-relative position end(i) (exclusive).
  if (in_smem_list) {
    for (int64_t i = tid; i < cnt; i += FS_THREADS) {
      int64_t e = seg_off2(a, lo + 1 + i) - b;
      if (e < 1 || e > TE) { raise_error(a.err, DEV_ERR_INDEX); e = TE + 1; }
      s_end[i] = (uint16_t)(e > TE ? 0xffff : e);
    }
  }
  __syncthreads();
  auto end_at = [&](int64_t i) -> int {
    if (i >= cnt) return 1 << 30;
    if (in_smem_list) return s_end[i];
    const int64_t e = seg_off2(a, lo + 1 + i) - b;
    return (e < 1 || e > TE) ? 1 << 30 : (int)e;
  };
  if (!mbar_wait(&bar, 0)) {
    raise_error(a.err, DEV_ERR_TIMEOUT);
    mbar_wait(&bar, 0);
  }

  const int r0 = tid * ITEMS;
  const int64_t grow = tile * FS_THREADS + tid;
  auto load_row = [&](T (&x)[ITEMS]) {
    if (grow < a.full_rows) {
#pragma unroll
      for (int c = 0; c < ITEMS / VEC; ++c) {
        uint4 v = *reinterpret_cast<const uint4 *>(buf + tid * FS_ROW_BYTES + ((c ^ (tid & 7)) << 4));
        memcpy(&x[c * VEC], &v, 16);
      }
    } else {
      const T *src = static_cast<const T *>(a.in);
#pragma unroll
      for (int j = 0; j < ITEMS; ++j) x[j] = (b + r0 + j < a.inner) ? src[b + r0 + j] : idT;
    }
    if (r0 < off0) {
#pragma unroll
      for (int j = 0; j < ITEMS; ++j)
        if (r0 + j < off0) x[j] = idT;  // not part of any segment
    }
  };
  // First end strictly after this row's start: binary search.
  int64_t i0;
  {
    int64_t l = 0, h = cnt;
    while (l < h) {
      const int64_t m = (l + h) >> 1;
      if (end_at(m) <= r0) l = m + 1; else h = m;
    }
    i0 = l;
  }

  // Ends inside this row as a bit mask: bit j set when a segment ends right
  // after element j (several list entries at one position are the empty
  // segments that follow a non-empty one).
  uint32_t emask = 0;
  {
    int64_t i = i0;
    int e = end_at(i);
    while (e <= r0 + ITEMS) {
      emask |= 1u << (e - r0 - 1);
      e = end_at(++i);
    }
  }

  // ---- pass 1: row value since its last end (branch-free), and whether it holds an end
  S acc = A::id();
  const bool ended = emask != 0u;
  {
    T x[ITEMS];
    load_row(x);
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
      acc = A::push(acc, x[j]);
      if ((emask >> j) & 1u) acc = A::id();
    }
  }
  // Segmented inclusive warp scan: (f1, v1) . (f2, v2) = (f1 | f2, f2 ? v2 : v1 `f` v2).
  S incl = acc;
  bool fin = ended;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const S ov = shfl_up(incl, d);
    const bool of = __shfl_up_sync(0xffffffffu, fin, d);
    if (lane >= d) {
      if (!fin) incl = A::comb(ov, incl);
      fin = fin || of;
    }
  }
  S ex = shfl_up(incl, 1);
  bool exf = __shfl_up_sync(0xffffffffu, fin, 1);
  if (lane == 0) { ex = A::id(); exf = false; }
  if (lane == 31) { s_warp[warp] = incl; s_wend[warp] = fin; }
  __syncthreads();
  S wv = A::id();
  bool wf = false;
  for (int w = 0; w < warp; ++w) {
    wv = s_wend[w] ? s_warp[w] : A::comb(wv, s_warp[w]);
    wf = wf || s_wend[w];
  }

  // ---- segmented look-back (warp 0): the value of the segment open at the tile start
  if (warp == 0) {
    S tv = A::id();
    bool tf = false;
    for (int w = 0; w < NWARP; ++w) {
      tv = s_wend[w] ? s_warp[w] : A::comb(tv, s_warp[w]);
      tf = tf || s_wend[w];
    }
    S carry = A::id();
    if (tile > 0) {
      if (lane == 0) publish_seg<S>(a.status, tile, a.epoch, 1u, tf, tv);
      constexpr int LB = 4;
      int64_t k0 = 0;
      bool gave_up = false;
      while (true) {
        uint32_t fl[LB];
        bool en[LB];
        S v[LB];
#pragma unroll
        for (int i = 0; i < LB; ++i) {
          const int64_t pt = tile - 1 - (k0 + lane * LB + i);
          fl[i] = pt >= 0 ? 0u : 2u;
          en[i] = pt < 0;
          v[i] = A::id();
        }
        uint32_t it = 0;
        while (true) {
          SlotWords sw[LB];
#pragma unroll
          for (int i = 0; i < LB; ++i) {
            sw[i] = SlotWords{0ull, 0ull};
            if (fl[i] == 0) sw[i] = ld_slot(a.status + 2 * (tile - 1 - (k0 + lane * LB + i)));
          }
          bool ready = true;
#pragma unroll
          for (int i = 0; i < LB; ++i) {
            if (fl[i] == 0) fl[i] = decode_seg<S>(sw[i], a.epoch, v[i], en[i]);
            ready = ready && fl[i] != 0;
          }
          if (__all_sync(0xffffffffu, ready)) break;
          ++it;
          const bool stop = gave_up || it > SPIN_LIMIT ||
                            ((it & 63u) == 0 && (ld_relaxed_u32(a.err) & DEV_ERR_TIMEOUT) != 0u);
          if (__any_sync(0xffffffffu, stop)) {
            gave_up = true;
            if (lane == 0) raise_error(a.err, DEV_ERR_TIMEOUT);
#pragma unroll
            for (int i = 0; i < LB; ++i)
              if (fl[i] == 0) { fl[i] = 2u; en[i] = true; }
            break;
          }
          __nanosleep(it < 8 ? 32 : 128);
        }
        // Nearest-first fold, stopping at an inclusive prefix or a tile that
        // holds a segment end (its value already starts after that end).
        bool stop_here = false;
        S lv = A::id();
#pragma unroll
        for (int i = 0; i < LB; ++i) {
          if (!stop_here) lv = A::comb(v[i], lv);
          stop_here = stop_here || fl[i] == 2u || en[i];
        }
        const unsigned pm = __ballot_sync(0xffffffffu, stop_here);
        const int kp = pm ? __ffs(pm) - 1 : 32;
        if (lane > kp) lv = A::id();
        S wr = warp_reduce_rev<A>(lv);
        wr = shfl_idx(wr, 0);
        carry = A::comb(wr, carry);
        if (pm) break;
        k0 += 32 * LB;
      }
      // Inclusive value at the tile end: what the next tile carries in.
      if (lane == 0) publish_seg<S>(a.status, tile, a.epoch, 2u, true, tf ? tv : A::comb(carry, tv));
    } else if (lane == 0) {
      publish_seg<S>(a.status, tile, a.epoch, 2u, true, tv);
    }
    if (lane == 0) s_carry = carry;
  }
  __syncthreads();

  // ---- pass 2: walk the row again from its carried-in value, writing segments
  S run;
  {
    // value carried into this row: (tile carry) . (warps before) . (lanes before)
    S c = s_carry;
    c = wf ? wv : A::comb(c, wv);
    run = exf ? ex : A::comb(c, ex);
  }
  {
    T x[ITEMS];
    load_row(x);
    T *out = static_cast<T *>(a.out);
    const T z = from_bits<T>(a.seed);
    int64_t i = i0;
#pragma unroll
    for (int j = 0; j < ITEMS; ++j) {
      run = A::push(run, x[j]);
      if ((emask >> j) & 1u) {
        // The first end of a run of equal ends closes a non-empty segment,
        // except segment 0 when it is empty (a tile starting before off[0]).
        if (a.has_seed || lo + i != 0 || seg_off2(a, 0) < seg_off2(a, 1))
          out[lo + i] = A::lower(a.has_seed ? A::comb(A::lift(z), run) : run);
        run = A::id();
        const int e = r0 + j + 1;
        do { ++i; } while (end_at(i) == e);
      }
    }
  }
}

template <int OP, class T, int PREC>
int foldseg_scan_typed(Workspace *w, const T *in, const void *off, int off64, T *out, int64_t inner,
                       int64_t nseg, bool has_seed, uint64_t seed, cudaStream_t s, bool *taken) {
  constexpr int ITEMS = FS_ROW_BYTES / sizeof(T);
  constexpr int64_t TE = (int64_t)FS_THREADS * ITEMS;
  *taken = false;
  const int64_t full_rows = inner / ITEMS;
  CUtensorMap tin;
  memset(&tin, 0, sizeof(tin));
  if (full_rows == 0 || !encode_2d(&tin, in, sizeof(T), ITEMS, full_rows, FS_ROW_BYTES, ITEMS, FS_THREADS, true))
    return ACC_OK;  // not describable by TMA: the caller uses the per-segment kernels
  const int64_t ntiles = cdiv_h(inner, TE);
  if (ntiles >= (1ll << 31)) return ACC_OK;
  *taken = true;
  int st = ws_status(w, (size_t)ntiles * 2);
  if (st) return st;
  st = ws_scratch(w, (size_t)ntiles * sizeof(int64_t) + 256);
  if (st) return st;
  SegScanArgs a{};
  a.in = in; a.off = off; a.out = out;
  a.inner = inner; a.nseg = nseg; a.off64 = off64;
  a.seed = seed; a.has_seed = has_seed;
  a.full_rows = full_rows; a.ntiles = ntiles;
  a.tile_seg = static_cast<int64_t *>(w->scratch);
  a.status = w->status;
  a.ticket = w->words + W_TICKET;
  a.err = w->words + W_ERR;
  a.epoch = ws_next_epoch(w, s);
  cudaError_t e = cudaMemsetAsync(a.tile_seg, 0xff, (size_t)ntiles * sizeof(int64_t), s);
  if (e != cudaSuccess) return cuda_status(e);
  const Device &d = device_info();
  int64_t pb = cdiv_h(nseg, 256);
  if (pb > (int64_t)d.sms * 8) pb = (int64_t)d.sms * 8;
  if (pb < 1) pb = 1;
  seg_tiles_kernel<T><<<(unsigned)pb, 256, 0, s>>>(a, TE);
  st = check_launch();
  if (st) return st;
  const size_t smem = (size_t)FS_THREADS * FS_ROW_BYTES + 1024;
  auto kern = foldseg_scan_kernel<OP, T, PREC>;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    attr = true;
  }
  kern<<<(unsigned)ntiles, FS_THREADS, smem, s>>>(tin, a);
  return check_launch();
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
        // The segmented single-pass kernel is opt-in (ACC_GB300_FOLDSEG=scan):
        // on GB300 it is still slower than the per-segment kernels.
        static const bool seg_scan = getenv("ACC_GB300_FOLDSEG") && strcmp(getenv("ACC_GB300_FOLDSEG"), "scan") == 0;
        if (outer == 1 && seg_scan) {
          bool taken = false;
          const int st = foldseg_scan_typed<OP, T, P>(w, static_cast<const T *>(in), off, off64,
                                                      static_cast<T *>(out), inner, nseg, seed != nullptr, sb, s,
                                                      &taken);
          if (taken || st) return st;
        }
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
