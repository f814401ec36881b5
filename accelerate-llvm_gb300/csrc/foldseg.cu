// foldseg.cu -- foldSeg f z / fold1Seg f over a segment-offset array.
//
// The reference picks ONE kernel for the whole array from the average
// segment length: a warp per segment or a CTA per segment
// (accelerate-llvm-ptx/src/Data/Array/Accelerate/LLVM/PTX/Execute.hs:343-374,
// PTX/CodeGen/FoldSeg.hs:79-458), so skewed (lognormal) lengths leave most
// lanes idle or most CTAs waiting on a few long segments.  Here:
//   * a 1-D row with 16-byte aligned values goes through foldseg_tile_kernel,
//     one launch that cuts the VALUES into equal tiles whatever the segment
//     lengths (see "tiled single pass" below);
//   * other shapes (rank >= 2, unaligned values) dispatch each segment by its
//     own length, in two launches:
//       1. seg_classify lists the segments longer than LONG_SEG (atomic
//          append; the order of the list does not matter, each segment is
//          reduced alone);
//       2. foldseg_main: the first CTAs stream the listed long segments, one
//          CTA per segment with 16-byte vector loads; every other warp owns 32
//          consecutive segments and reduces the short ones (<= SHORT_SEG) one
//          per lane, serially, and the medium ones with the whole warp.
// Per segment the result is z `f` (x_u `f` ... `f` x_(v-1)), as the native
// backend's reduceFromTo over [seg[i], seg[i+1]) (accelerate-llvm-native/src/
// Data/Array/Accelerate/LLVM/Native/CodeGen/FoldSeg.hs:103-141).  An empty
// segment gives z with a seed and is left unwritten without one
// (PTX/CodeGen/FoldSeg.hs:170-178).  Offsets that decrease or run past the
// row raise ACC_ERR_INDEX instead of reading out of bounds.
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
  const void *in2;     // ZIP kernels: the folded element i is zop(in[i], in2[i])
  int zop;
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

// seg_span over the fused producer zipWith zop p q: the vector body when p
// and q share their 16-byte alignment phase, a scalar stride otherwise.
template <class A, class T>
__device__ __forceinline__ typename A::S seg_span_zip(const T *p, const T *q, int zop, int64_t len, int64_t t,
                                                      int64_t nt) {
  using S = typename A::S;
  constexpr int VEC = 16 / sizeof(T);
  S acc = A::id();
  const uintptr_t addr = reinterpret_cast<uintptr_t>(p);
  if (((addr ^ reinterpret_cast<uintptr_t>(q)) & 15u) != 0u) {
    for (int64_t i = t; i < len; i += nt) acc = A::push(acc, zip_elem(zop, ld_stream(p + i), ld_stream(q + i)));
    return acc;
  }
  int64_t head = (int64_t)(((16u - (addr & 15u)) & 15u) / sizeof(T));
  if (head > len) head = len;
  if (t < head) acc = A::push(acc, zip_elem(zop, ld_stream(p + t), ld_stream(q + t)));
  const int64_t nvec = (len - head) / VEC;
  const uint4 *pv = reinterpret_cast<const uint4 *>(p + head);
  const uint4 *qv = reinterpret_cast<const uint4 *>(q + head);
  for (int64_t i = t; i < nvec; i += nt) {
    const uint4 v = ld_stream16(pv + i), w = ld_stream16(qv + i);
    T e[VEC], f[VEC];
    memcpy(e, &v, 16);
    memcpy(f, &w, 16);
#pragma unroll
    for (int k = 0; k < VEC; ++k) acc = A::push(acc, zip_elem(zop, e[k], f[k]));
  }
  const int64_t tail0 = head + nvec * VEC;
  if (tail0 + t < len) acc = A::push(acc, zip_elem(zop, ld_stream(p + tail0 + t), ld_stream(q + tail0 + t)));
  return acc;
}

// With ZIP the folded array is the fused producer zipWith zop in in2.
template <int OP, class T, int PREC, bool ZIP = false>
__global__ void __launch_bounds__(256) foldseg_main(SegArgs a) {
  using A = Acc<OP, T, PREC>;
  using S = typename A::S;
  const T *in = static_cast<const T *>(a.in);
  const T *in2 = static_cast<const T *>(a.in2);
  (void)in2;
  // Element i of row r, and the fold of a span of row r.
  auto elem = [&](const T *row, const T *row2, int64_t i) -> T {
    if constexpr (ZIP) return zip_elem(a.zop, row[i], row2[i]);
    else { (void)row2; return row[i]; }
  };
  auto span = [&](const T *row, const T *row2, int64_t len, int64_t t, int64_t nt) -> S {
    if constexpr (ZIP) return seg_span_zip<A, T>(row, row2, a.zop, len, t, nt);
    else { (void)row2; return seg_span<A, T>(row, len, t, nt); }
  };
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
      S acc = span(in + r * a.inner + u, ZIP ? in2 + r * a.inner + u : nullptr, v - u, threadIdx.x, blockDim.x);
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
    const T *row2 = ZIP ? in2 + r * a.inner : nullptr;
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
        else acc = A::lift(elem(row, row2, i++));
        for (; i < v; ++i) acc = A::push(acc, elem(row, row2, i));
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
      S acc = span(row + mu, ZIP ? row2 + mu : nullptr, mv - mu, lane, 32);
      acc = warp_reduce<A>(acc);
      if (lane == 0) {
        if (a.has_seed) acc = A::comb(A::lift(from_bits<T>(a.seed)), acc);
        out[r * a.nseg + g * 32 + src] = A::lower(acc);
      }
    }
  }
}

// ----------------------------------------------------------------- tiled single pass
// 1-D rows with 16-byte aligned values take this path.  The values are cut
// into tiles of 256 or 512 rows x 128 B (one 2-D TMA load per 256 rows,
// 128-byte swizzle, as in the scan; each thread owns one or two adjacent
// rows), independent of the segment lengths, so every CTA streams the
// same number of bytes however skewed the segmentation is.  One launch:
//   * a pre-pass (foldseg_tile_index) records for every tile the index of
//     the first offset at or after its start, so a tile knows its offset
//     range [kf, ks) from two loads; the CTA copies those offsets
//     (tile-relative) to shared memory, writing z for the empty segments on
//     the way;
//   * each thread walks its 256 bytes once: a segment boundary inside them
//     closes the segment that was open, whose state the row parks in shared
//     memory when it also saw that segment start; the value before the row's
//     first boundary and after its last one are carried out;
//   * a segmented CTA scan ((f1,v1).(f2,v2) = (f1|f2, f2 ? v2 : v1 `f` v2))
//     gives every row the value carried in from earlier rows of the tile, and
//     the tile's own carried-out value, which is final at once: the tile
//     publishes it (flag 2 when the tile holds a boundary, 1 when it lies
//     inside one segment) before it looks back;
//   * the parked results are written out in one coalesced pass, except the
//     segment that closes at the tile's first boundary, which needs the
//     value carried in from earlier tiles: a decoupled look-back that stops
//     at the nearest tile holding a boundary (usually the previous one).
// An extra tile past the last value closes the segments that end at the
// very end of the row.  Two launches: the index pre-pass and the tile pass.  Offsets that decrease or leave [0, n] raise
// ACC_ERR_INDEX; the tile then writes nothing but still publishes.
constexpr int FT_THREADS = 256;
constexpr int FT_ROW_BYTES = 128;
constexpr int FT_CAP = 512;   // tile-relative offsets (and their results) held in shared memory
// Adjacent 128-byte rows per thread: two for one-word states (a longer walk
// amortises the per-thread scan and bookkeeping), one for the compensated
// Float32 pair, whose longer walk code does not pay for itself.
template <class S> constexpr int ft_rpt() { return std::is_same<S, F2>::value ? 1 : 2; }

struct SegTileArgs {
  const void *in;
  const void *off;
  void *out;
  int64_t n, nseg;
  int64_t full_rows, ntiles;
  uint64_t seed;
  int has_seed;
  const uint64_t *tidx;  // per tile: epoch tag << 35 | first offset index >= the tile start
  uint64_t *status;
  uint32_t *ticket;
  uint32_t *err;
  uint32_t epoch;
};

constexpr int TIDX_SHIFT = 35;  // offset indices below 2^35; the epoch above

// Pre-pass: tidx[t] = the first k with off[k] >= t * te (t < ntiles), and
// tidx[ntiles] = nseg + 1, each tagged with the call's epoch so that no
// clearing is needed.  Thread k writes the tiles whose start lies in
// (off[k-1], off[k]]; k = nseg + 1 stands for the tiles past the last offset.
// Decreasing offsets leave tiles unwritten (their stale tag is caught later).
template <class OT>
__global__ void foldseg_tile_index(const OT *off, int64_t nseg, int64_t ntiles, int64_t te, uint64_t *tidx,
                                   uint32_t epoch) {
  const uint64_t tag = (uint64_t)epoch << TIDX_SHIFT;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k <= nseg + 1;
       k += (int64_t)gridDim.x * blockDim.x) {
    int64_t t0, t1;  // tiles [t0, t1] get k
    if (k == 0) t0 = 0;
    else {
      const int64_t lo = (int64_t)off[k - 1];
      t0 = lo < 0 ? 0 : lo / te + 1;
    }
    if (k == nseg + 1) t1 = ntiles - 1;
    else {
      const int64_t hi = (int64_t)off[k];
      t1 = hi < 0 ? -1 : hi / te;
    }
    if (t1 > ntiles - 1) t1 = ntiles - 1;
    for (int64_t t = t0; t <= t1; ++t) tidx[t] = tag | (uint64_t)k;
    if (k == nseg + 1) tidx[ntiles] = tag | (uint64_t)k;
  }
}

// Look-back slot of the tiled foldSeg: tag = epoch << 3 | flag.
template <class S>
__device__ __forceinline__ void publish_seg(uint64_t *status, int64_t t, uint32_t epoch, uint32_t flag, S v) {
  uint64_t b = to_bits(v);
  uint64_t tag = (uint64_t)((epoch << 3) | flag) << 32;
  if constexpr (sizeof(S) == 8) st_relaxed_u64(status + 2 * t + 1, tag | (b >> 32));
  st_relaxed_u64(status + 2 * t, tag | (b & 0xffffffffull));
}
template <class S>
__device__ __forceinline__ uint32_t decode_seg(SlotWords s, uint32_t epoch, S &v) {
  const uint32_t tag = (uint32_t)(s.w0 >> 32);
  if ((tag >> 3) != epoch) return 0;
  uint64_t b = s.w0 & 0xffffffffull;
  if constexpr (sizeof(S) == 8) {
    if ((uint32_t)(s.w1 >> 32) != tag) return 0;
    b |= (s.w1 & 0xffffffffull) << 32;
  }
  v = from_bits<S>(b);
  return tag & 3u;
}

template <int OP, class T, int PREC, class OT>
__global__ void __launch_bounds__(FT_THREADS, (ft_rpt<typename Acc<OP, T, PREC>::S>() == 1 ? 5 : 3))
foldseg_tile_kernel(const __grid_constant__ CUtensorMap tin, SegTileArgs a) {
  using A = Acc<OP, T, PREC>;
  using S = typename A::S;
  constexpr int FT_RPT = ft_rpt<S>();
  constexpr int ITEMS = FT_ROW_BYTES / sizeof(T);
  constexpr int VEC = 16 / sizeof(T);
  constexpr int W = FT_RPT * ITEMS;          // values per thread (FT_RPT adjacent rows)
  constexpr int TE = FT_THREADS * W;
  constexpr int SUB_BYTES = FT_THREADS * FT_ROW_BYTES;
  constexpr int NWARP = FT_THREADS / 32;
  constexpr int FAR = 1 << 30;  // beyond every tile-relative position
  extern __shared__ unsigned char smem_raw[];
  unsigned char *buf = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ uint64_t bar;
  __shared__ int64_t s_tile, s_kf, s_cnt, s_lo, s_hi, s_first_id;
  __shared__ int s_offs[FT_CAP];
  __shared__ int s_rowh[FT_THREADS];  // per thread: first offset entry at or after its first value
  __shared__ S s_res[FT_CAP];         // per entry (or, in a slot tile, per boundary): a closed segment's state
  __shared__ S s_wv[NWARP], s_first_v, s_tile_v;
  __shared__ int s_wf[NWARP];
  __shared__ int s_has_first, s_tile_f, s_bad;
  __shared__ uint64_t s_bm[FT_THREADS];  // slot tiles: each thread's boundary positions
  __shared__ int s_base[FT_THREADS];     // slot tiles: each thread's first boundary slot
  __shared__ int s_nbw[NWARP];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const OT *off = static_cast<const OT *>(a.off);
  T *out = static_cast<T *>(a.out);
  const T idT = Prim<OP, T>::id();

  if (tid == 0) {
    const uint32_t dyn = atomicAdd(a.ticket, 1u);
    if ((int64_t)dyn == a.ntiles - 1) *a.ticket = 0u;
    s_tile = dyn;
    s_has_first = 0;
    s_bad = 0;
    mbar_init(&bar, 1);
    fence_mbar_init();
    mbar_expect_tx(&bar, FT_RPT * SUB_BYTES);
#pragma unroll
    for (int u = 0; u < FT_RPT; ++u)
      tma_load_2d(buf + u * SUB_BYTES, &tin, 0, (int)(((int64_t)dyn * FT_RPT + u) * FT_THREADS), &bar);
  }
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t tb = tile * TE;
  const bool last_tile = tile == a.ntiles - 1;
  if (tid < 32) {
    // The offsets inside [tb, te) are [kf, ks); the last tile takes every
    // remaining one (ks = nseg + 1).
    const uint64_t tag = (uint64_t)a.epoch << TIDX_SHIFT, mask = (1ull << TIDX_SHIFT) - 1;
    const uint64_t e0 = a.tidx[tile], e1 = a.tidx[tile + 1];
    const int64_t vstart = (int64_t)off[0], vend = (int64_t)off[a.nseg];
    if (lane == 0) {
      const int64_t kf = (int64_t)(e0 & mask), ks = (int64_t)(e1 & mask);
      s_kf = kf;
      s_cnt = ks - kf;
      // Tile-relative value window of the segments, clamped to the tile.
      int64_t lo = vstart - tb, hi = vend - tb;
      s_lo = lo < 0 ? 0 : (lo > TE ? TE : lo);
      s_hi = hi < 0 ? 0 : (hi > TE ? TE : hi);
      if ((e0 & ~mask) != tag || (e1 & ~mask) != tag || ks < kf || ks > a.nseg + 1 || (tile == 0 && kf != 0) ||
          vstart < 0 || vend > a.n || vend < vstart)
        s_bad = 1;
      if (s_bad) s_cnt = 0;
    }
  }
  __syncthreads();
  const int64_t kf = s_kf, cnt = s_cnt > 0 ? s_cnt : 0;
  const T z = from_bits<T>(a.seed);
  // Tile-relative offsets to shared memory (the first FT_CAP of them), the
  // per-thread first entries, checks, and z for the empty segments that
  // start in this tile.  Entry i+1 is the first entry for the threads whose
  // first value lies in (rel_i, rel_(i+1)]; entry 0 for those at or before rel_0.
  if (cnt == 0) s_rowh[tid] = 0;
  bool bad = false;
  for (int64_t i = tid; i < cnt; i += FT_THREADS) {
    const int64_t k = kf + i;
    const int64_t o = (int64_t)off[k];
    const int64_t rel = o - tb;
    if (rel < 0 || (!last_tile && rel >= TE)) bad = true;
    const int r = (int)(rel < 0 ? 0 : (rel > TE ? TE : rel));
    if (i < FT_CAP) s_offs[i] = (int)(rel < 0 ? -1 : r);
    int rn = FAR;  // the next entry, or past the tile
    if (k < a.nseg) {
      const int64_t o1 = (int64_t)off[k + 1];
      if (o1 < o) bad = true;
      else if (o1 == o && a.has_seed) out[k] = z;
      if (i + 1 < cnt) {
        const int64_t reln = o1 - tb;
        rn = (int)(reln < 0 ? 0 : (reln > TE ? TE : reln));
      }
    }
    if (i == 0)
      for (int t = 0; t <= r / W && t < FT_THREADS; ++t) s_rowh[t] = 0;
    const int t_hi = rn >= TE ? FT_THREADS - 1 : rn / W;
    for (int t = r / W + 1; t <= t_hi && t < FT_THREADS; ++t) s_rowh[t] = (int)(i + 1);
  }
  if (bad) s_bad = 1;
  auto rel_at = [&](int64_t h) -> int {
    if (h >= cnt) return FAR;
    if (h < FT_CAP) return s_offs[h];
    const int64_t rel = (int64_t)off[kf + h] - tb;
    return (int)(rel < 0 ? -1 : (rel > TE ? TE : rel));
  };
  // One warp waits for the tile; the others block at the CTA barrier, which
  // costs no issue slots (several CTAs share an SM and the walk is
  // issue-bound).  The barrier orders every thread after the completed load.
  bool landed = true;
  if (warp == 0 && !mbar_wait_sleep(&bar, 0)) {
    if (lane == 0) raise_error(a.err, DEV_ERR_TIMEOUT);
    landed = mbar_wait_sleep(&bar, 0);
  }
  // A tile whose load never landed is neither read nor published.
  if (__syncthreads_or(!landed)) return;
  const bool ok = s_bad == 0;
  if (!ok && tid == 0) raise_error(a.err, DEV_ERR_INDEX);
  const int lo = (int)s_lo, hi = (int)s_hi;

  // ---- the walk over this thread's FT_RPT adjacent rows
  const int tb0 = tid * W;
  int64_t h = s_rowh[tid];
  if (h < 0 || h > cnt) h = cnt;  // only with malformed offsets (nothing is written then)
  int np = rel_at(h);
  S acc = A::id(), left = A::id();
  bool started = false;
  int64_t first_h = -1;
  // A slot tile (the common case: well-formed offsets, all in shared memory,
  // every value of the tile inside the segments, no partial row) parks the
  // closed states by BOUNDARY: thread t's boundaries take slots s_base[t],
  // s_base[t]+1, ... (an exclusive scan of the threads' boundary counts), so
  // the walk keeps one running slot index and has no branch per value;
  // several offsets at one position (empty segments) are one boundary.  The
  // result pass finds a segment's slot from its position.
  const bool slot_tile = ok && cnt <= FT_CAP && lo == 0 && hi == TE &&
                         (tile + 1) * (int64_t)(FT_RPT * FT_THREADS) <= a.full_rows;
  int pbase = 0;
  if (slot_tile) {
    int64_t he = tid + 1 < FT_THREADS ? (int64_t)s_rowh[tid + 1] : cnt;
    if (he < h || he > cnt) he = cnt;
    uint64_t bm = 0;
    for (int64_t e = h; e < he; ++e) {
      const int r = s_offs[e] - tb0;
      if (r >= 0 && r < W) bm |= 1ull << r;
    }
    const int nb = __popcll(bm);
    int incl = nb;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int o = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= d) incl += o;
    }
    if (lane == 31) s_nbw[warp] = incl;
    __syncthreads();
    int wbase = 0;
    for (int w2 = 0; w2 < warp; ++w2) wbase += s_nbw[w2];
    pbase = wbase + incl - nb;
    s_bm[tid] = bm;
    s_base[tid] = pbase;
    int pk = pbase;
    // fully unrolled: every mask bit is tested at a constant position
    const uint32_t bm_lo = (uint32_t)bm, bm_hi = (uint32_t)(bm >> 32);
    const int r0 = FT_RPT * tid;
#pragma unroll
    for (int c = 0; c < W / VEC; ++c) {
      const int r = r0 + c / (ITEMS / VEC);
      const int cc = c % (ITEMS / VEC);
      const int rr = r % FT_THREADS;
      const uint4 v = *reinterpret_cast<const uint4 *>(buf + (r / FT_THREADS) * SUB_BYTES + rr * FT_ROW_BYTES +
                                                       ((cc ^ (rr & 7)) << 4));
      T x[VEC];
      memcpy(x, &v, 16);
#pragma unroll
      for (int q = 0; q < VEC; ++q) {
        const int bit = c * VEC + q;
        const bool bnd = ((bit < 32 ? bm_lo : bm_hi) >> (bit & 31)) & 1u;
        if (bnd) s_res[pk] = acc;
        pk += bnd ? 1 : 0;
        acc = bnd ? A::id() : acc;
        acc = A::push(acc, x[q]);
      }
    }
    started = nb > 0;
    first_h = h;  // the entry of the thread's first boundary
    if (started) left = s_res[pbase];
  } else {
  // A boundary only parks the closed segment's state (the results leave in
  // one coalesced pass after the scan), so a lane that meets one holds its
  // warp up for a few instructions.
  auto boundary = [&](int p) {
    if (!started) {
      left = acc;
      first_h = h;
      started = true;
    } else if (h < FT_CAP) {
      s_res[h] = acc;
    } else if (ok) {  // long offset lists only: write at once
      const int64_t sid = kf + h - 1;
      if (sid >= 0) out[sid] = A::lower(a.has_seed ? A::comb(A::lift(z), acc) : acc);
    }
    acc = A::id();
    do { ++h; np = rel_at(h); } while (np == p);  // several offsets at p: empty segments
  };
  const bool masked = lo > tb0 || hi < tb0 + W;
  auto load_chunk = [&](int c, T (&x)[VEC]) {
    const int r = FT_RPT * tid + c / (ITEMS / VEC);  // row within the tile
    const int cc = c % (ITEMS / VEC);                // 16-byte chunk within the row
    if (tile * (FT_RPT * FT_THREADS) + r < a.full_rows) {
      const int rr = r % FT_THREADS;
      const uint4 v = *reinterpret_cast<const uint4 *>(buf + (r / FT_THREADS) * SUB_BYTES + rr * FT_ROW_BYTES +
                                                       ((cc ^ (rr & 7)) << 4));
      memcpy(x, &v, 16);
    } else {
      const T *src = static_cast<const T *>(a.in);
#pragma unroll
      for (int q = 0; q < VEC; ++q) {
        const int64_t gi = tb + tb0 + c * VEC + q;
        x[q] = gi < a.n ? src[gi] : idT;
      }
    }
  };
  // Fast walk: when this thread's offsets are in shared memory they become
  // a bit mask of boundary positions (bm) and the boundaries take entries
  // h, h+1, ... in order, so a boundary costs a shared-memory store and no
  // load; only a position that holds several offsets (empty segments
  // follow) skips its extra entries by reading them (dm marks those).
  static_assert(W <= 64, "one 64-bit boundary mask per thread");
  int64_t h_end = tid + 1 < FT_THREADS ? (int64_t)s_rowh[tid + 1] : cnt;
  if (h_end < h || h_end > cnt) h_end = cnt;
  bool fast = !masked && ok && h_end <= FT_CAP;
  uint64_t bm = 0, dm = 0;
  if (fast) {
    for (int64_t e = h; e < h_end; ++e) {
      const int r = s_offs[e] - tb0;
      if (r < 0 || r >= W) fast = false;
      else if ((bm >> r) & 1u) dm |= 1ull << r;
      else bm |= 1ull << r;
    }
  }
  if (fast) {
    // Branch-free walk: every boundary, the row's first included, parks the
    // closed segment's state at its entry; the first one is read back as
    // the value carried out to the left.  Only a boundary followed by empty
    // segments branches (to skip their entries).
    int hh = (int)h;
    const int h0 = hh;
#pragma unroll 1
    for (int c = 0; c < W / VEC; ++c) {
      T x[VEC];
      load_chunk(c, x);
      const uint32_t cb = (uint32_t)(bm >> (c * VEC)) & ((1u << VEC) - 1u);
      const uint32_t cd = (uint32_t)(dm >> (c * VEC)) & ((1u << VEC) - 1u);
#pragma unroll
      for (int q = 0; q < VEC; ++q) {
        const bool bnd = (cb >> q) & 1u;
        if (bnd) s_res[hh] = acc;
        if (bnd && ((cd >> q) & 1u)) {
          const int pos = tb0 + c * VEC + q;
          do { ++hh; } while (hh < h_end && s_offs[hh] == pos);
        } else {
          hh += bnd ? 1 : 0;
        }
        acc = bnd ? A::id() : acc;
        acc = A::push(acc, x[q]);
      }
    }
    started = hh != h0;
    first_h = h0;
    if (started) left = s_res[h0];
  } else {
#pragma unroll 1
    for (int c = 0; c < W / VEC; ++c) {
      T x[VEC];
      load_chunk(c, x);
      const int p0 = tb0 + c * VEC;
      if (masked) {
#pragma unroll
        for (int q = 0; q < VEC; ++q) {
          if (p0 + q == np) boundary(p0 + q);
          acc = A::push(acc, (p0 + q >= lo && p0 + q < hi) ? x[q] : idT);
        }
      } else {
#pragma unroll
        for (int q = 0; q < VEC; ++q) {
          if (p0 + q == np) boundary(p0 + q);
          acc = A::push(acc, x[q]);
        }
      }
    }
  }

  }

  // ---- segmented CTA scan of the rows' carried-out values
  S iv = acc;
  bool ifl = started;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const S ov = shfl_up(iv, d);
    const bool of = __shfl_up_sync(0xffffffffu, ifl, d);
    if (lane >= d) {
      if (!ifl) iv = A::comb(ov, iv);
      ifl = ifl || of;
    }
  }
  S ex = shfl_up(iv, 1);
  bool exf = __shfl_up_sync(0xffffffffu, ifl, 1);
  if (lane == 0) { ex = A::id(); exf = false; }
  if (lane == 31) { s_wv[warp] = iv; s_wf[warp] = ifl; }
  __syncthreads();
  S wv = A::id();
  bool wf = false;
  for (int w = 0; w < warp; ++w) {
    wv = s_wf[w] ? s_wv[w] : A::comb(wv, s_wv[w]);
    wf = wf || s_wf[w];
  }
  const S cin = exf ? ex : A::comb(wv, ex);  // value of the segment open at the row start
  const bool cinf = exf || wf;                // that segment started inside the tile
  if (started) {
    const S v = A::comb(cin, left);
    if (cinf) {
      if (slot_tile) s_res[pbase] = v;
      else if (first_h < FT_CAP) s_res[first_h] = v;
      else if (ok) out[kf + first_h - 1] = A::lower(a.has_seed ? A::comb(A::lift(z), v) : v);
    } else {
      s_first_v = v;  // the tile's first boundary: needs the value from earlier tiles
      s_first_id = kf + first_h - 1;
      s_has_first = 1;
    }
  }
  if (tid == FT_THREADS - 1) {
    s_tile_v = started ? acc : A::comb(cin, acc);
    s_tile_f = started || cinf;
  }
  __syncthreads();

  // ---- publish; the parked results leave; look back for the segment closing
  // at the tile's first boundary (entry 0)
  if (tid == 0) publish_seg<S>(a.status, tile, a.epoch, s_tile_f ? 2u : 1u, s_tile_v);
  if (ok) {
    const int64_t nres = cnt < FT_CAP ? cnt : FT_CAP;
    for (int64_t e = 1 + tid; e < nres; e += FT_THREADS)
      if (s_offs[e] > s_offs[e - 1]) {  // the first entry at its position closes a segment
        int slot = (int)e;
        if (slot_tile) {
          // the boundary at position p is bit p % W of thread p / W
          const int p = s_offs[e], t = p / W, bit = p % W;
          slot = s_base[t] + __popcll(s_bm[t] & ((1ull << bit) - 1ull));
        }
        const S v = s_res[slot];
        out[kf + e - 1] = A::lower(a.has_seed ? A::comb(A::lift(z), v) : v);
      }
  }
  if (warp == 0) {
    if (s_has_first && s_first_id >= 0) {
      constexpr int LB = 4;
      S carry = A::id();
      int64_t k0 = 0;
      bool gave_up = false;
      uint32_t it = 0;
      uint64_t t_wait = 0;
      while (true) {
        uint32_t fl[LB];
        S v[LB];
#pragma unroll
        for (int i = 0; i < LB; ++i) {
          fl[i] = tile - 1 - (k0 + lane * LB + i) >= 0 ? 0u : 2u;
          v[i] = A::id();
        }
        bool resolved = false, whole = false;
        int kp = 32;
        while (true) {
          const int kp0 = lb_stop_lane<LB>(fl);
          SlotWords sw[LB];
#pragma unroll
          for (int i = 0; i < LB; ++i) {
            sw[i] = SlotWords{0ull, 0ull};
            if (fl[i] == 0 && lane <= kp0) sw[i] = ld_slot(a.status + 2 * (tile - 1 - (k0 + lane * LB + i)));
          }
#pragma unroll
          for (int i = 0; i < LB; ++i)
            if (fl[i] == 0 && lane <= kp0) fl[i] = decode_seg<S>(sw[i], a.epoch, v[i]);
          kp = lb_window<LB>(fl, resolved, whole);
          if (resolved || whole) break;
          ++it;
          if (it == 8) t_wait = global_ns();  // first checked at it == 64
          const bool stop = gave_up || it > SPIN_LIMIT ||
                            ((it & 63u) == 0 && ((ld_relaxed_u32(a.err) & DEV_ERR_TIMEOUT) != 0u ||
                                                 global_ns() - t_wait > WAIT_LIMIT_NS));
          if (__any_sync(0xffffffffu, stop)) {
            gave_up = true;
            if (lane == 0) raise_error(a.err, DEV_ERR_TIMEOUT);
#pragma unroll
            for (int i = 0; i < LB; ++i)
              if (fl[i] == 0) fl[i] = 2u;
            kp = lb_window<LB>(fl, resolved, whole);
            break;
          }
          __nanosleep(it < 4 ? 64 : (it < 16 ? 256 : 1024));  // back off: the predecessor is usually close behind
        }
        bool stop_here = false;
        S lv = A::id();
#pragma unroll
        for (int i = 0; i < LB; ++i) {
          if (!stop_here) lv = A::comb(v[i], lv);
          stop_here = stop_here || fl[i] == 2u;
        }
        if (lane > kp) lv = A::id();
        S wr = warp_reduce_rev<A>(lv);
        wr = shfl_idx(wr, 0);
        carry = A::comb(wr, carry);
        if (resolved) break;
        k0 += 32 * LB;
      }
      if (lane == 0 && ok) {
        const S v = A::comb(carry, s_first_v);
        out[s_first_id] = A::lower(a.has_seed ? A::comb(A::lift(z), v) : v);
      }
    }
  }
}

// One launcher per kernel instantiation, so that each gets its own
// shared-memory attribute (the tile needs more than the default 48 KB).
template <int OP, class T, int PREC, class OT>
int launch_foldseg_tile(const CUtensorMap &tin, const SegTileArgs &a, int64_t ntiles, cudaStream_t s) {
  constexpr int FT_RPT = ft_rpt<typename Acc<OP, T, PREC>::S>();
  const size_t smem = (size_t)FT_RPT * FT_THREADS * FT_ROW_BYTES + 1024;
  auto kern = foldseg_tile_kernel<OP, T, PREC, OT>;
  static std::atomic<uint64_t> attr_done{0};
  smem_attrs_once(kern, (int)smem, attr_done);
  kern<<<(unsigned)ntiles, FT_THREADS, smem, s>>>(tin, a);
  return check_launch();
}

template <int OP, class T, int PREC>
int foldseg_tile_typed(Workspace *w, const T *in, const void *off, int off64, T *out, int64_t inner,
                       int64_t nseg, bool has_seed, uint64_t seed, cudaStream_t s, bool *taken) {
  constexpr int ITEMS = FT_ROW_BYTES / sizeof(T);
  constexpr int FT_RPT = ft_rpt<typename Acc<OP, T, PREC>::S>();
  constexpr int64_t TE = (int64_t)FT_THREADS * FT_RPT * ITEMS;
  *taken = false;
  const int64_t full_rows = inner / ITEMS;
  CUtensorMap tin;
  memset(&tin, 0, sizeof(tin));
  if (full_rows == 0 || !encode_2d(&tin, in, sizeof(T), ITEMS, full_rows, FT_ROW_BYTES, ITEMS, FT_THREADS, true))
    return ACC_OK;  // not describable by TMA: the caller uses the per-segment kernels
  // One tile more than the values need when they fill the last tile exactly:
  // that tile holds the boundary at position n.
  const int64_t ntiles = inner / TE + 1;
  if (ntiles * FT_RPT * FT_THREADS >= (1ll << 31)) return ACC_OK;  // TMA row coordinates are 32-bit
  if (nseg + 2 >= (1ll << TIDX_SHIFT)) return ACC_OK;
  *taken = true;
  int st = ws_status(w, (size_t)ntiles * 2);
  if (st) return st;
  st = ws_scratch(w, (size_t)(ntiles + 1) * sizeof(uint64_t));
  if (st) return st;
  SegTileArgs a{};
  a.in = in; a.off = off; a.out = out;
  a.n = inner; a.nseg = nseg;
  a.full_rows = full_rows; a.ntiles = ntiles;
  a.seed = seed; a.has_seed = has_seed;
  a.tidx = static_cast<const uint64_t *>(w->scratch);
  a.status = w->status;
  a.ticket = w->words + W_TICKET;
  a.err = w->words + W_ERR;
  a.epoch = ws_next_epoch(w, s);
  {
    const Device &d = device_info();
    int64_t pb = cdiv_h(nseg + 2, 256);
    if (pb > (int64_t)d.sms * 8) pb = (int64_t)d.sms * 8;
    uint64_t *tidx = static_cast<uint64_t *>(w->scratch);
    if (off64)
      foldseg_tile_index<int64_t><<<(unsigned)pb, 256, 0, s>>>(static_cast<const int64_t *>(off), nseg, ntiles, TE,
                                                                tidx, a.epoch);
    else
      foldseg_tile_index<int32_t><<<(unsigned)pb, 256, 0, s>>>(static_cast<const int32_t *>(off), nseg, ntiles, TE,
                                                                tidx, a.epoch);
    st = check_launch();
    if (st) return st;
  }
  return off64 ? launch_foldseg_tile<OP, T, PREC, int64_t>(tin, a, ntiles, s)
               : launch_foldseg_tile<OP, T, PREC, int32_t>(tin, a, ntiles, s);
}

// ----------------------------------------------------------------- host side
// The per-segment path; with ZIP over the fused producer zipWith zop in in2.
template <int OP, class T, int PREC, bool ZIP = false>
int foldseg_typed(Workspace *w, const T *in, const void *off, int off64, T *out, int64_t outer,
                  int64_t inner, int64_t nseg, bool has_seed, uint64_t seed, cudaStream_t s,
                  const T *in2 = nullptr, int zop = 0) {
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
  a.in2 = in2;
  a.zop = zop;
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
  foldseg_main<OP, T, PREC, ZIP><<<(unsigned)(a.long_ctas + sb), 256, 0, s>>>(a);
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
        // Rows of one segmented vector take the tiled single pass unless
        // ACC_GB300_FOLDSEG=segments asks for the per-segment kernels.
        static const bool per_segment =
            getenv("ACC_GB300_FOLDSEG") && strcmp(getenv("ACC_GB300_FOLDSEG"), "segments") == 0;
        if (outer == 1 && !per_segment) {
          bool taken = false;
          const int st = foldseg_tile_typed<OP, T, P>(w, static_cast<const T *>(in), off, off64,
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
  // The offsets live at the END of the scratch area.  The front part,
  // list_bytes, holds what the fold itself keeps in scratch: the per-segment
  // path's long-segment list (at most inner / LONG_SEG + 1 entries) or the
  // tiled path's tile index (inner / tile + 2 entries, tiles of >= 4096
  // values), both within list_bytes, so neither grows (and moves) the
  // scratch under the offsets.
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

// foldSeg f z (zipWith g xs ys): the reference fuses the producer into the
// segmented fold's kernel (its delayed input, PTX/CodeGen/FoldSeg.hs:56-458
// reading a MIRDelayed array).  Here the per-segment kernels read both arrays
// and zip each element as they load it (the zipped array is never written).
// f in {+, min, max}, g in {+, *, min, max}, Int32 / Int64 / Float32 /
// Float64, as for the fused fold and scans.
extern "C" int acc_fold_seg_zipwith(int op, int zop, int type, int prec, const void *xs, const void *ys,
                                    const void *offsets, int offset_type, void *out, int64_t outer, int64_t inner,
                                    int64_t nseg, const void *seed, void *stream) {
  int st = fold_seg_check(type, offset_type, xs, offsets, out, outer, inner, nseg);
  if (st) return st;
  if (op < ACC_ADD || op > ACC_XOR || zop < ACC_ADD || zop > ACC_XOR) return ACC_ERR_INVALID;
  if (outer > 0 && inner > 0 && nseg > 0 && !ys) return ACC_ERR_INVALID;
  if (op != ACC_ADD && op != ACC_MIN && op != ACC_MAX) return ACC_ERR_UNSUPPORTED;
  if (zop != ACC_ADD && zop != ACC_MUL && zop != ACC_MIN && zop != ACC_MAX) return ACC_ERR_UNSUPPORTED;
  if (type == ACC_U32) return ACC_ERR_UNSUPPORTED;
  if (outer == 0 || nseg == 0) return ACC_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Workspace *w = workspace(s, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  return with_type(type, [&](auto tv) -> int {
    using T = decltype(tv);
    const uint64_t sb = seed_bits<T>(seed);
    return with_op<T>(op, [&](auto opc) -> int {
      constexpr int OP = decltype(opc)::value;
      if constexpr ((OP != ACC_ADD && OP != ACC_MIN && OP != ACC_MAX) || std::is_same<T, uint32_t>::value) {
        return ACC_ERR_UNSUPPORTED;
      } else {
        return with_prec<OP, T>(prec, [&](auto pc) -> int {
          constexpr int P = decltype(pc)::value;
          return foldseg_typed<OP, T, P, true>(w, static_cast<const T *>(xs), offsets, offset_type == ACC_I64,
                                               static_cast<T *>(out), outer, inner, nseg, seed != nullptr, sb, s,
                                               static_cast<const T *>(ys), zop);
        });
      }
    });
  });
}
