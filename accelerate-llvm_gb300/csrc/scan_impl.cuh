// scan_impl.cuh -- the scan kernels and their launchers, shared by scan.cu
// (acc_scan, acc_scan_noalloc) and scan_zip.cu (scans over a fused
// zipWith producer).
//
// scanl / scanl1 / scanr / scanr1 / scanl' / scanr' for the fixed
// primitives.
//
// The reference runs a 1-D scan as three kernels (scanP1 block scans, a
// single-block scanP2 over the block totals, scanP3 adding the carries:
// accelerate-llvm-ptx/src/Data/Array/Accelerate/LLVM/PTX/Execute.hs:422-468,
// PTX/CodeGen/Scan.hs:141-439), about 4n words of traffic.  Here a 1-D scan is
// ONE pass of 2n words: a single-pass scan with decoupled look-back
// (Merrill & Garland 2016).  Each CTA
//   1. takes a tile index from an atomic ticket (tiles are handed out in
//      order, so every tile it may wait on belongs to a CTA that is running),
//   2. pulls its 32 KiB tile into shared memory with one 2-D TMA load of a
//      [rows x 128 B] view of the array, 128-byte swizzled so that the
//      thread-per-row reads below are bank-conflict free,
//   3. reduces each thread's 128-byte row serially, scans the thread totals
//      with warp shuffles, publishes the tile aggregate, and (warp 0) looks
//      back over the predecessors' published aggregates / inclusive prefixes,
//   4. rescans its row from the tile prefix and writes the result back to the
//      same swizzled smem buffer, from which one TMA store writes the tile.
// Element semantics follow accelerate-llvm-native/src/Data/Array/Accelerate/
// LLVM/Native/CodeGen/Scan.hs:136-270: left-to-right combines `f acc x`,
// right-to-left `f x acc`; the seed sits at the far left (L2R) or far right
// (R2L).  The primitives are commutative, so one push() serves both.
//
// Rows of a rank >= 2 array are scanned by scan_rows_kernel: one CTA per row
// with a carried prefix, as the reference's `scan` (multi-dim) kernel does
// (PTX/CodeGen/Scan.hs:746-939); many short rows take scan_rows_warp_kernel,
// one warp per row.
#pragma once

#include <cstdlib>
#include <cstring>

#include "common.cuh"

namespace accgb {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ROW_BYTES = 128;  // one thread row = one 128 B swizzle line
#ifndef SCAN_LOOKBACK
#define SCAN_LOOKBACK 1  // predecessor statuses read per lane per look-back poll (window of 32)
#endif

struct ScanArgs {
  const void *in;
  void *out;
  void *total_out;   // grand total (scanl z -> out+n, scan' -> sums) or null
  void *seed_out;    // where to store the seed (scanr z -> out+n) or null
  int64_t n;
  int64_t full_rows;  // rows of 128 B fully inside the array
  int64_t ntiles;
  uint64_t seed;      // seed bits
  uint64_t *status;
  uint32_t *ticket;
  uint32_t *err;
  uint32_t *done;    // persistent kernels: CTAs finished (the last re-arms the ticket)
  uint32_t epoch;
  int has_seed;
  int exclusive;
  int tma_in;
  int tma_out;
  const void *in2;   // ZIP kernels: the scanned element i is zop(in[i], in2[i])
  int zop;           // ... MAP kernels: it is zop(in[i], c)
  uint64_t mapc;     // MAP kernels: the constant c (bits of one element)
  int64_t seg_len;   // segmented (row) scans: the rows' length; a row restarts the scan
  void *seg_sums;    // ... with a seed (scanl' / scanr'): each row's total, or null
};

__device__ __forceinline__ int swz(int row, int chunk) { return row * SCAN_ROW_BYTES + ((chunk ^ (row & 7)) << 4); }

// Publish a look-back status of tile t: (flag, value), flag 1 = aggregate,
// 2 = inclusive prefix.  Each 64-bit slot word carries the 32-bit tag
// (epoch << 2 | flag) next to 32 bits of the value, so every word is
// self-describing; an 8-byte value uses two words that a reader accepts only
// when both carry the same tag.
template <class S>
__device__ __forceinline__ void publish(uint64_t *status, int64_t t, uint32_t epoch, uint32_t flag, S v) {
  uint64_t b = to_bits(v);
  uint64_t tag = (uint64_t)((epoch << 2) | flag) << 32;
  if constexpr (sizeof(S) == 8) st_relaxed_u64(status + 2 * t + 1, tag | (b >> 32));
  st_relaxed_u64(status + 2 * t, tag | (b & 0xffffffffull));
}

// Decode a status slot read by ld_slot; returns the flag (0 = not yet
// published in this epoch, or torn between two publications).
template <class S>
__device__ __forceinline__ uint32_t decode(SlotWords s, uint32_t epoch, S &v) {
  const uint32_t tag = (uint32_t)(s.w0 >> 32);
  if ((tag >> 2) != epoch) return 0;
  uint64_t b = s.w0 & 0xffffffffull;
  if constexpr (sizeof(S) == 8) {
    if ((uint32_t)(s.w1 >> 32) != tag) return 0;
    b |= (s.w1 & 0xffffffffull) << 32;
  }
  v = from_bits<S>(b);
  return tag & 3u;
}

// Warp-collective decoupled look-back of a tile that is not the first one:
// the combination of every predecessor's value, walking from the nearest
// predecessor outwards in windows of 32 * LB tiles (LB consecutive slots per
// lane, all of a poll's loads issued back to back) up to the nearest
// published inclusive prefix.  Every lane returns the result.  A window that
// is not resolved after WAIT_LIMIT_NS (or SPIN_LIMIT polls, or once another
// CTA has timed out) gives up: its missing slots count as the identity and
// the error word records DEV_ERR_TIMEOUT.
template <class A, bool R2L, int LB>
__device__ __forceinline__ typename A::S lookback_prefix(const ScanArgs &a, int64_t tile) {
  using S = typename A::S;
  const int lane = threadIdx.x & 31;
  S acc = A::id();
  int64_t k0 = 0;
  bool gave_up = false;
  while (true) {
    uint32_t fl[LB];
    S v[LB];
    bool ex[LB];
#pragma unroll
    for (int i = 0; i < LB; ++i) {
      const int64_t d = k0 + lane * LB + i;  // 0 = nearest predecessor
      const int64_t pt = R2L ? tile + 1 + d : tile - 1 - d;
      ex[i] = R2L ? (pt < a.ntiles) : (pt >= 0);
      fl[i] = ex[i] ? 0u : 2u;
      v[i] = A::id();
    }
    uint32_t it = 0;
    uint64_t t_wait = 0;
    bool resolved = false, whole = false;
    int kp = 32;
    while (true) {
      // Issue every pending slot load of this poll first, then decode:
      // one round trip per poll, not one per slot.  Lanes beyond the
      // nearest inclusive prefix seen so far need no more reads.
      const int kp0 = lb_stop_lane<LB>(fl);
      SlotWords sw[LB];
#pragma unroll
      for (int i = 0; i < LB; ++i) {
        sw[i] = SlotWords{0ull, 0ull};
        if (ex[i] && fl[i] == 0 && lane <= kp0) {
          const int64_t d = k0 + lane * LB + i;
          sw[i] = ld_slot(a.status + 2 * (R2L ? tile + 1 + d : tile - 1 - d));
        }
      }
#pragma unroll
      for (int i = 0; i < LB; ++i)
        if (ex[i] && fl[i] == 0 && lane <= kp0) fl[i] = decode<S>(sw[i], a.epoch, v[i]);
      kp = lb_window<LB>(fl, resolved, whole);
      if (resolved || whole) break;
      ++it;
      // Give up (warp-uniformly) after WAIT_LIMIT_NS or SPIN_LIMIT polls, or
      // at once when another CTA on this stream has already timed out.
      if (it == 8) t_wait = global_ns();  // first checked at it == 64
      const bool stop = gave_up || it > SPIN_LIMIT ||
                        ((it & 63u) == 0 && ((ld_relaxed_u32(a.err) & DEV_ERR_TIMEOUT) != 0u ||
                                             global_ns() - t_wait > WAIT_LIMIT_NS));
      if (__any_sync(0xffffffffu, stop)) {
        gave_up = true;
        if (lane == 0) raise_error(a.err, DEV_ERR_TIMEOUT);
#pragma unroll
        for (int i = 0; i < LB; ++i)
          if (fl[i] == 0) fl[i] = 2u;  // treat as identity: the result is flagged as failed
        kp = lb_window<LB>(fl, resolved, whole);
        break;
      }
      __nanosleep(it < 8 ? 32 : 128);
    }
    // Lane-local fold from the nearest predecessor outwards, up to and
    // including the first inclusive prefix.
    bool seen_p = false;
    S lv = A::id();
#pragma unroll
    for (int i = 0; i < LB; ++i) {
      if (!seen_p) lv = R2L ? A::comb(lv, v[i]) : A::comb(v[i], lv);
      seen_p = seen_p || fl[i] == 2u;
    }
    if (lane > kp) lv = A::id();
    S wv = R2L ? warp_reduce<A>(lv) : warp_reduce_rev<A>(lv);
    wv = shfl_idx(wv, 0);
    acc = R2L ? A::comb(acc, wv) : A::comb(wv, acc);
    if (resolved) break;
    k0 += 32 * LB;
  }
  return acc;
}

// One tile = SUB sub-tiles of 256 rows x 128 B; thread t owns row t of every
// sub-tile.  The rows of the array's full 128 B lines are in `buf` (each
// sub-tile 32 KiB, 128-byte swizzled); the last, partial line is read from
// and written to global memory directly.  The row is NOT kept in registers
// across the look-back: pass 1 folds it, pass 2 re-reads it from shared memory
// and rescans it from its prefix, which keeps the register count low enough
// for many tiles per SM to be in flight.  On return the results of the full
// rows are in `buf`.
// `sub_done(u)` runs (in every thread) after sub-tile u has been rescanned
// into `buf`, e.g. to start its store while the next sub-tile is rescanned.
struct NoSubDone {
  __device__ void operator()(int) const {}
};

// With ZIP, the rows read from global memory are zipped as they are read
// (the rows in `buf` arrive zipped).  With MAP, every element is mapped as it
// is read, from `buf` or from global memory (map (\x -> zop x c)).
template <int OP, class T, int PREC, bool R2L, int SUB, bool ZIP = false, bool MAP = false,
          class SubDone = NoSubDone>
__device__ __forceinline__ void scan_tile_body(unsigned char *buf, int64_t tile, const ScanArgs &a,
                                               typename Acc<OP, T, PREC>::S (*s_warp)[SCAN_THREADS / 32],
                                               typename Acc<OP, T, PREC>::S &s_prefix, bool smem_all_rows,
                                               SubDone sub_done = SubDone{}) {
  using A = Acc<OP, T, PREC>;
  using S = typename A::S;
  constexpr int ITEMS = SCAN_ROW_BYTES / sizeof(T);
  constexpr int VEC = 16 / sizeof(T);
  constexpr int NWARP = SCAN_THREADS / 32;
  constexpr int SUB_BYTES = SCAN_THREADS * SCAN_ROW_BYTES;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const T idT = Prim<OP, T>::id();
  const int64_t row0 = tile * (int64_t)(SUB * SCAN_THREADS);

  auto load_row = [&](int u, T (&x)[ITEMS]) {
    const int64_t grow = row0 + u * SCAN_THREADS + tid;
    if (smem_all_rows || grow < a.full_rows) {
#pragma unroll
      for (int c = 0; c < ITEMS / VEC; ++c) {
        uint4 v = *reinterpret_cast<const uint4 *>(buf + u * SUB_BYTES + swz(tid, c));
        memcpy(&x[c * VEC], &v, 16);
      }
      if constexpr (MAP) {
        const T cm = from_bits<T>(a.mapc);
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) x[j] = zip_elem(a.zop, x[j], cm);
      }
    } else {
      const T *src = static_cast<const T *>(a.in);
      const int64_t e0 = grow * ITEMS;
      if constexpr (ZIP) {
        const T *src2 = static_cast<const T *>(a.in2);
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) x[j] = (e0 + j < a.n) ? zip_elem(a.zop, src[e0 + j], src2[e0 + j]) : idT;
      } else if constexpr (MAP) {
        const T cm = from_bits<T>(a.mapc);
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) x[j] = (e0 + j < a.n) ? zip_elem(a.zop, src[e0 + j], cm) : idT;
      } else {
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) x[j] = (e0 + j < a.n) ? src[e0 + j] : idT;
      }
    }
  };

  // ---- pass 1: row totals, warp scans, warp totals
  S excl_lane[SUB];
#pragma unroll
  for (int u = 0; u < SUB; ++u) {
    T x[ITEMS];
    load_row(u, x);
    S agg;
    if (!R2L) {
      agg = A::lift(x[0]);
#pragma unroll
      for (int j = 1; j < ITEMS; ++j) agg = A::push(agg, x[j]);
      S incl = warp_scan_incl<A>(agg);
      S up = shfl_up(incl, 1);
      excl_lane[u] = lane == 0 ? A::id() : up;
      if (lane == 31) s_warp[u][warp] = incl;
    } else {
      agg = A::lift(x[ITEMS - 1]);
#pragma unroll
      for (int j = ITEMS - 2; j >= 0; --j) agg = A::push(agg, x[j]);
      S incl = warp_scan_incl_rev<A>(agg);
      S dn = shfl_down(incl, 1);
      excl_lane[u] = lane == 31 ? A::id() : dn;
      if (lane == 0) s_warp[u][warp] = incl;
    }
  }
  __syncthreads();

  // ---- decoupled look-back (warp 0)
  if (warp == 0) {
    S bagg = s_warp[0][0];
#pragma unroll
    for (int k = 1; k < SUB * NWARP; ++k) bagg = A::comb(bagg, s_warp[k / NWARP][k % NWARP]);
    const bool first = R2L ? (tile == a.ntiles - 1) : (tile == 0);
    S prefix;
    if (first) {
      prefix = a.has_seed ? A::lift(from_bits<T>(a.seed)) : A::id();
    } else {
      if (lane == 0) publish<S>(a.status, tile, a.epoch, 1u, bagg);
      prefix = lookback_prefix<A, R2L, SCAN_LOOKBACK>(a, tile);
    }
    const S inclusive = R2L ? A::comb(bagg, prefix) : A::comb(prefix, bagg);
    if (lane == 0) {
      publish<S>(a.status, tile, a.epoch, 2u, inclusive);
      s_prefix = prefix;
      const bool last = R2L ? (tile == 0) : (tile == a.ntiles - 1);
      if (last && a.total_out) *static_cast<T *>(a.total_out) = A::lower(inclusive);
      if (first && a.seed_out) *static_cast<T *>(a.seed_out) = from_bits<T>(a.seed);
    }
  }
  __syncthreads();

  // ---- pass 2: rescan each row from its prefix, results back to buf / global
  T *dst = static_cast<T *>(a.out);
#pragma unroll
  for (int u = 0; u < SUB; ++u) {
    // Everything before (L2R) / after (R2L) this thread's row within the tile.
    S inner = A::id();
    if (!R2L) {
      for (int k = 0; k < u * NWARP + warp; ++k) inner = A::comb(inner, s_warp[k / NWARP][k % NWARP]);
    } else {
      for (int k = u * NWARP + warp + 1; k < SUB * NWARP; ++k) inner = A::comb(inner, s_warp[k / NWARP][k % NWARP]);
    }
    S run = R2L ? A::comb(A::comb(excl_lane[u], inner), s_prefix) : A::comb(s_prefix, A::comb(inner, excl_lane[u]));
    T x[ITEMS];
    load_row(u, x);
    const int64_t grow = row0 + u * SCAN_THREADS + tid;
    const bool in_smem = smem_all_rows || grow < a.full_rows;
    const int64_t e0 = grow * ITEMS;
#pragma unroll
    for (int cc = 0; cc < ITEMS / VEC; ++cc) {
      const int c = R2L ? ITEMS / VEC - 1 - cc : cc;
      T y[VEC];
#pragma unroll
      for (int kk = 0; kk < VEC; ++kk) {
        const int k = R2L ? VEC - 1 - kk : kk;
        const int j = c * VEC + k;
        if (a.exclusive) { y[k] = A::lower(run); run = A::push(run, x[j]); }
        else { run = A::push(run, x[j]); y[k] = A::lower(run); }
      }
      if (in_smem) {
        uint4 v;
        memcpy(&v, y, 16);
        *reinterpret_cast<uint4 *>(buf + u * SUB_BYTES + swz(tid, c)) = v;
      } else {
#pragma unroll
        for (int k = 0; k < VEC; ++k)
          if (e0 + c * VEC + k < a.n) dst[e0 + c * VEC + k] = y[k];
      }
    }
    sub_done(u);
  }
}

// One tile per CTA, any alignment: coalesced loads / stores through the same
// swizzled smem layout (used when a TMA descriptor cannot describe the array).
template <int OP, class T, int PREC, bool R2L, bool ZIP = false, bool MAP = false>
__global__ void __launch_bounds__(SCAN_THREADS) scan_lookback_kernel(ScanArgs a) {
  using S = typename Acc<OP, T, PREC>::S;
  constexpr int ITEMS = SCAN_ROW_BYTES / sizeof(T);
  constexpr int VEC = 16 / sizeof(T);
  constexpr int TILE = SCAN_THREADS * ITEMS;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *buf = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ int64_t s_tile;
  __shared__ S s_warp[1][SCAN_THREADS / 32];
  __shared__ S s_prefix;
  const int tid = threadIdx.x;
  if (tid == 0) {
    const uint32_t dyn = atomicAdd(a.ticket, 1u);
    // The holder of the last ticket knows every other CTA has taken its
    // ticket: it re-arms the counter for the next launch on this stream.
    if ((int64_t)dyn == a.ntiles - 1) *a.ticket = 0u;
    s_tile = R2L ? a.ntiles - 1 - (int64_t)dyn : (int64_t)dyn;
  }
  __syncthreads();
  const int64_t tile = s_tile;
  const int64_t base = tile * (int64_t)TILE;
  const T idT = Prim<OP, T>::id();
  const T *src = static_cast<const T *>(a.in);
  const T *src2 = static_cast<const T *>(a.in2);
  (void)src2;
  for (int e = tid; e < TILE; e += SCAN_THREADS) {
    const int64_t gi = base + e;
    T v = idT;
    if (gi < a.n) {
      if constexpr (ZIP) v = zip_elem(a.zop, src[gi], src2[gi]);
      else if constexpr (MAP) v = zip_elem(a.zop, src[gi], from_bits<T>(a.mapc));
      else v = src[gi];
    }
    const int r = e / ITEMS, k = e % ITEMS;
    *reinterpret_cast<T *>(buf + swz(r, k / VEC) + (k % VEC) * sizeof(T)) = v;
  }
  __syncthreads();
  scan_tile_body<OP, T, PREC, R2L, 1>(buf, tile, a, s_warp, s_prefix, true);
  __syncthreads();
  T *dst = static_cast<T *>(a.out);
  for (int e = tid; e < TILE; e += SCAN_THREADS) {
    const int64_t gi = base + e;
    if (gi < a.n) {
      const int r = e / ITEMS, k = e % ITEMS;
      dst[gi] = *reinterpret_cast<const T *>(buf + swz(r, k / VEC) + (k % VEC) * sizeof(T));
    }
  }
}

// One tile (SUB x 32 KiB) per CTA through TMA, for 16-byte aligned arrays:
// the tile arrives with SUB 2-D TMA loads of [256 rows x 128 B] on one
// mbarrier, is scanned in shared memory, and leaves with SUB TMA stores.
template <int OP, class T, int PREC, bool R2L, int SUB, bool MAP = false>
__global__ void __launch_bounds__(SCAN_THREADS, SUB == 1 ? 6 : 3)
scan_tma_kernel(const __grid_constant__ CUtensorMap tin, const __grid_constant__ CUtensorMap tout, ScanArgs a) {
  using S = typename Acc<OP, T, PREC>::S;
  constexpr int SUB_BYTES = SCAN_THREADS * SCAN_ROW_BYTES;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *buf = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ uint64_t bar;
  __shared__ int64_t s_tile;
  __shared__ S s_warp[SUB][SCAN_THREADS / 32];
  __shared__ S s_prefix;
  const int tid = threadIdx.x;
  if (tid == 0) {
    const uint32_t dyn = atomicAdd(a.ticket, 1u);
    if ((int64_t)dyn == a.ntiles - 1) *a.ticket = 0u;
    const int64_t tile = R2L ? a.ntiles - 1 - (int64_t)dyn : (int64_t)dyn;
    s_tile = tile;
    mbar_init(&bar, 1);
    fence_mbar_init();
    mbar_expect_tx(&bar, SUB * SUB_BYTES);
#pragma unroll
    for (int u = 0; u < SUB; ++u)
      tma_load_2d(buf + u * SUB_BYTES, &tin, 0, (int)((tile * SUB + u) * SCAN_THREADS), &bar);
  }
  __syncthreads();
  const int64_t tile = s_tile;
  // A tile whose load never landed is neither read nor published: its
  // successors' look-backs give up in turn and the call reports the timeout.
  if (__syncthreads_or(!mbar_wait_flagged(&bar, 0, a.err))) return;
  // Each sub-tile leaves by TMA as soon as it is rescanned, while the next
  // one is rescanned; the CTA waits only for the last store's reads.
  auto store_sub = [&](int u) {
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tma_store_2d(&tout, 0, (int)((tile * SUB + u) * SCAN_THREADS), buf + u * SUB_BYTES);
      tma_store_commit();
    }
  };
  scan_tile_body<OP, T, PREC, R2L, SUB, false, MAP>(buf, tile, a, s_warp, s_prefix, false, store_sub);
  if (tid == 0) tma_store_wait_read();
}

// Zip one thread's 128-byte row of the two swizzled tiles into the first:
// buf[row] = g buf[row] buf2[row], element by element.
template <class T, int Z>
__device__ __forceinline__ void zip_row(unsigned char *buf, const unsigned char *buf2, int row) {
  constexpr int VEC = 16 / sizeof(T);
#pragma unroll
  for (int c = 0; c < SCAN_ROW_BYTES / 16; ++c) {
    uint4 v = *reinterpret_cast<const uint4 *>(buf + swz(row, c));
    const uint4 w = *reinterpret_cast<const uint4 *>(buf2 + swz(row, c));
    T x[VEC], y[VEC];
    memcpy(x, &v, 16);
    memcpy(y, &w, 16);
#pragma unroll
    for (int k = 0; k < VEC; ++k) x[k] = Prim<Z, T>::ap(x[k], y[k]);
    memcpy(&v, x, 16);
    *reinterpret_cast<uint4 *>(buf + swz(row, c)) = v;
  }
}

// --------------------------------------------------------------------------
// Persistent single-pass scan with a re-read from L2, for 16-byte aligned
// 1-D arrays.  A tile (32 KiB: 256 rows x 128 B, thread t owns row t) is
// read from HBM into buffer A and folded (pass 1: row totals, warp scans, the
// tile aggregate, published at once); its buffer is then free and takes the
// CTA's next tile while a look-back warp resolves the tile's exclusive
// prefix from its predecessors' published values.  Pass 2 loads the tile
// again into buffer B -- from L2, where pass 1 left it a few microseconds
// earlier -- rescans it from its prefix and stores it by TMA.  So a tile
// occupies shared memory only while it is worked on, never while its
// look-back waits, and the look-back of tile i overlaps the HBM load and fold
// of tile i+1; DRAM still sees each input byte read once.
// Roles: 256 compute threads (8 warps) and one look-back warp; they hand
// tiles over through mbarriers (aggr: the aggregate of the tile in slot p is
// published; pref: its exclusive prefix is known).  Tiles come from a
// dynamic ticket, so that each tile's predecessors are always claimed by
// running CTAs; the grid is launched cooperatively (every CTA resident), and
// a CTA folds and publishes its next tile before it waits for its current
// tile's prefix, so the lowest unfinished tile can always finish.  Every
// wait is bounded: a wait that runs out stops the CTA (after a bounded wait
// for its copies in flight) and raises DEV_ERR_TIMEOUT.
// PROD selects the scanned array's producer (the reference's delayed scan
// input, PTX/CodeGen/Scan.hs:141-439): 0 = the array itself; 1 = map
// (\x -> g x c), applied as each row is read, in both passes; 2 = zipWith g
// xs ys: pass 1 loads the tiles of both arrays (into A and Y), zips them in
// place in A and, besides folding, stores the zipped tile to its place in the
// output, where pass 2 finds it in L2; the zipped array thus costs no DRAM
// traffic and the CTA needs 96 KiB (two per SM).
// SEG: the array is `n / seg_len` rows of seg_len >= one 128-byte line
// (scanl1 / scanr1 over the innermost dimension of a rank-2 array, the
// reference's scanDim, PTX/CodeGen/Scan.hs:441-611): the scan restarts at
// each row's first element in scan order.  A thread's line holds at most one
// such start; states are (restarted, value) pairs combined so that a later
// part that restarted keeps its own value, so warps, tiles and the look-back
// see segmented combinations.  A tile that holds a row start publishes its
// last row's partial sum as an inclusive prefix at once (its successors need
// nothing before it), and a tile that begins with a row start needs no
// look-back.  SEG 2 (scanl' / scanr' over rows: exclusive, each row's total
// to seg_sums): every row restarts from the seed, and the thread whose line
// holds a row's last element in scan order writes the row's total; SEG 3
// (scanl z / scanr z over rows, whose output rows are one element longer):
// every row restarts from the seed and pass 2 stores each element straight to
// its place in the longer output row (index + row), the row's total (scanl
// z) or the seed (scanr z) going to the row's extra last slot; SEG 1
// (scanl1 / scanr1) carries none of that.
constexpr int L2S_COMPUTE = SCAN_THREADS;
constexpr int L2S_THREADS = L2S_COMPUTE + 32;
constexpr int L2S_TILE = SCAN_THREADS * SCAN_ROW_BYTES;
constexpr int L2S_CTAS_PER_SM = 3;
constexpr bool L2S_HINTS = true;  // L2 policies: keep a tile between its two loads, drop it after

template <int OP, class T, int PREC, bool R2L, int PROD = 0, int SEG = 0>
__global__ void __launch_bounds__(L2S_THREADS, PROD == 2 ? 2 : L2S_CTAS_PER_SM)
scan_l2_kernel(const __grid_constant__ CUtensorMap tin, const __grid_constant__ CUtensorMap tout, ScanArgs a,
               const __grid_constant__ CUtensorMap tin2) {
  using A = Acc<OP, T, PREC>;
  using S = typename A::S;
  constexpr int ITEMS = SCAN_ROW_BYTES / sizeof(T);
  constexpr int VEC = 16 / sizeof(T);
  constexpr int NWARP = L2S_COMPUTE / 32;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *bufA = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char *bufB = bufA + L2S_TILE;
  unsigned char *bufY = bufB + L2S_TILE;  // PROD 2: the tile of the second array
  __shared__ uint64_t fullA, fullB, aggr[2], pref[2];
  __shared__ int64_t s_claim;    // dynamic index of the tile pass 1 takes next
  __shared__ int64_t s_tile[2];  // tile in look-back slot p (-1: stop)
  __shared__ S s_warp[2][NWARP];
  __shared__ S s_agg[2], s_prefix[2];
  __shared__ bool s_wflag[2][NWARP], s_aflag[2];  // SEG: the part holds a row start
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  auto tile_of = [&](int64_t d) { return R2L ? a.ntiles - 1 - d : d; };
  // SEG: part `b` follows part `a` in scan order; the pair's state
  auto seg_then = [&](bool fa, S sa, bool fb, S sb, bool &f) -> S {
    f = fa || fb;
    return fb ? sb : (R2L ? A::comb(sb, sa) : A::comb(sa, sb));
  };
  // pass 1's load of the tile with dynamic index d (thread 0): from HBM, kept in L2
  auto load_a = [&](int64_t d) {
    const int row = (int)(tile_of(d) * SCAN_THREADS);
    mbar_expect_tx(&fullA, PROD == 2 ? 2 * L2S_TILE : L2S_TILE);
    if constexpr (L2S_HINTS) {
      tma_load_2d_hint(bufA, &tin, 0, row, &fullA, l2_policy_evict_last());
      if constexpr (PROD == 2) tma_load_2d_hint(bufY, &tin2, 0, row, &fullA, l2_policy_evict_first());
    } else {
      tma_load_2d(bufA, &tin, 0, row, &fullA);
      if constexpr (PROD == 2) tma_load_2d(bufY, &tin2, 0, row, &fullA);
    }
  };

  if (tid == 0) {
    mbar_init(&fullA, 1);
    mbar_init(&fullB, 1);
    mbar_init(&aggr[0], 1);
    mbar_init(&aggr[1], 1);
    mbar_init(&pref[0], 1);
    mbar_init(&pref[1], 1);
    fence_mbar_init();
    prefetch_tmap(&tin);
    prefetch_tmap(&tout);
    if constexpr (PROD == 2) prefetch_tmap(&tin2);
    const int64_t d = (int64_t)atomicAdd(a.ticket, 1u);
    s_claim = d;
    if (d < a.ntiles) load_a(d);
  }
  __syncthreads();

  if (warp == NWARP) {
    // ---- look-back warp: the exclusive prefix of each tile, in this CTA's order
    for (int64_t k = 0;; ++k) {
      const int p = (int)(k & 1);
      const bool ok = mbar_wait_flagged(&aggr[p], (uint32_t)(k >> 1) & 1u, a.err);
      if (__any_sync(0xffffffffu, !ok)) break;
      const int64_t tile = s_tile[p];
      if (tile < 0) break;
      const bool first = R2L ? (tile == a.ntiles - 1) : (tile == 0);
      // SEG: a tile whose first element in scan order starts a row needs no prefix
      const bool fresh = SEG && (R2L ? ((tile + 1) * (int64_t)L2S_TILE / (int64_t)sizeof(T)) % a.seg_len == 0
                                     : (tile * (int64_t)L2S_TILE / (int64_t)sizeof(T)) % a.seg_len == 0);
      const S prefix = (first || fresh) ? (a.has_seed ? A::lift(from_bits<T>(a.seed)) : A::id())
                                        : lookback_prefix<A, R2L, SCAN_LOOKBACK>(a, tile);
      if (lane == 0) {
        const S bagg = s_agg[p];
        const S inclusive = R2L ? A::comb(bagg, prefix) : A::comb(prefix, bagg);
        if (!(SEG && s_aflag[p])) publish<S>(a.status, tile, a.epoch, 2u, inclusive);
        s_prefix[p] = prefix;
        const bool last = R2L ? (tile == 0) : (tile == a.ntiles - 1);
        if (last && a.total_out) *static_cast<T *>(a.total_out) = A::lower(inclusive);
        if (first && a.seed_out) *static_cast<T *>(a.seed_out) = from_bits<T>(a.seed);
        mbar_arrive(&pref[p]);
      }
      __syncwarp();
    }
    return;
  }

  // ---- compute warps
  const T idT = Prim<OP, T>::id();
  const T *src = static_cast<const T *>(a.in);
  T *dst = static_cast<T *>(a.out);
  const T *src2 = static_cast<const T *>(a.in2);
  const T mapc = from_bits<T>(a.mapc);
  (void)src2;
  (void)mapc;
  // Row `tid` of a tile as the scan sees it: from shared memory for full rows
  // (PROD 2: already zipped there), else produced from global memory.
  auto load_row = [&](const unsigned char *buf, int64_t tile, T (&x)[ITEMS]) {
    const int64_t grow = tile * SCAN_THREADS + tid;
    if (grow < a.full_rows) {
#pragma unroll
      for (int c = 0; c < ITEMS / VEC; ++c) {
        const uint4 v = *reinterpret_cast<const uint4 *>(buf + swz(tid, c));
        memcpy(&x[c * VEC], &v, 16);
      }
      if constexpr (PROD == 1) {
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) x[j] = zip_elem(a.zop, x[j], mapc);
      }
    } else {
      const int64_t e0 = grow * ITEMS;
#pragma unroll
      for (int j = 0; j < ITEMS; ++j) {
        x[j] = idT;
        if (e0 + j < a.n) {
          if constexpr (PROD == 2) x[j] = zip_elem(a.zop, src[e0 + j], src2[e0 + j]);
          else if constexpr (PROD == 1) x[j] = zip_elem(a.zop, src[e0 + j], mapc);
          else x[j] = src[e0 + j];
        }
      }
    }
  };
  // SEG: the offset within this thread's line of the row start (in scan
  // order) of tile t's line, or ITEMS when it has none
  auto seg_start = [&](int64_t t) -> int {
    const int64_t e0 = (t * SCAN_THREADS + tid) * (int64_t)ITEMS;
    const int64_t r0 = e0 % a.seg_len;
    const int64_t jb = R2L ? a.seg_len - 1 - r0 : (r0 == 0 ? 0 : a.seg_len - r0);
    return jb < ITEMS ? (int)jb : ITEMS;
  };
  // SEG: the offset of the last element in scan order of a row in tile t's
  // line, or ITEMS
  auto seg_end = [&](int64_t t) -> int {
    const int64_t e0 = (t * SCAN_THREADS + tid) * (int64_t)ITEMS;
    const int64_t r0 = e0 % a.seg_len;
    const int64_t je = R2L ? (r0 == 0 ? 0 : a.seg_len - r0) : a.seg_len - 1 - r0;
    return je < ITEMS ? (int)je : ITEMS;
  };
  // SEG: the state a row starts from
  const S seg_reset = SEG >= 2 ? A::lift(from_bits<T>(a.seed)) : A::id();
  (void)seg_start;
  (void)seg_end;
  (void)seg_reset;
  int64_t d_new = s_claim;
  int64_t t_cur = -1;
  S excl_cur = A::id();
  bool exf_cur = false;
  int64_t k = 0;  // tiles this CTA has taken
  uint32_t phA = 0, phB = 0;
  bool failed = false, b_loading = false;
  while (true) {
    const bool have_new = d_new < a.ntiles;
    const int pn = (int)(k & 1), pc = pn ^ 1;
    int64_t t_new = -1;
    S excl_new = A::id();
    bool exf_new = false;
    if (t_cur >= 0 && tid == 0) {
      // the current tile's second load (from L2) runs during the next tile's
      // fold; PROD 2 reads the zipped tile that pass 1 stored in the output,
      // once that store is complete
      if constexpr (PROD == 2) tma_store_wait_all();
      else tma_store_wait_read();  // the previous store has read B
      mbar_expect_tx(&fullB, L2S_TILE);
      const CUtensorMap *t2 = PROD == 2 ? &tout : &tin;
      if constexpr (L2S_HINTS) tma_load_2d_hint(bufB, t2, 0, (int)(t_cur * SCAN_THREADS), &fullB, l2_policy_evict_first());
      else tma_load_2d(bufB, t2, 0, (int)(t_cur * SCAN_THREADS), &fullB);
    }
    if (t_cur >= 0) b_loading = true;
    if (have_new) {
      // pass 1 of the new tile (in A)
      t_new = tile_of(d_new);
      if (named_bar_or<1, L2S_COMPUTE>(!mbar_wait_flagged(&fullA, phA, a.err))) { failed = true; break; }
      phA ^= 1u;
      if constexpr (PROD == 2) {
        if (t_new * SCAN_THREADS + tid < a.full_rows) {
          switch (a.zop) {
            case ACC_ADD: zip_row<T, ACC_ADD>(bufA, bufY, tid); break;
            case ACC_MUL: zip_row<T, ACC_MUL>(bufA, bufY, tid); break;
            case ACC_MIN: zip_row<T, ACC_MIN>(bufA, bufY, tid); break;
            default: zip_row<T, ACC_MAX>(bufA, bufY, tid); break;
          }
        }
        fence_proxy_async_smem();  // the zipped rows, for pass 1's store of A
      }
      T x[ITEMS];
      load_row(bufA, t_new, x);
      if constexpr (SEG) {
        // the offset of this line's row start (its last element for R2L), if any
        const int jb = seg_start(t_new);
        S agg = A::id();
        if (!R2L) {
#pragma unroll
          for (int j = 0; j < ITEMS; ++j) {
            if (j == jb) agg = seg_reset;
            agg = A::push(agg, x[j]);
          }
        } else {
#pragma unroll
          for (int j = ITEMS - 1; j >= 0; --j) {
            if (j == jb) agg = seg_reset;
            agg = A::push(agg, x[j]);
          }
        }
        bool f = jb < ITEMS;
#pragma unroll
        for (int dd = 1; dd < 32; dd <<= 1) {
          const S ov = R2L ? shfl_down(agg, dd) : shfl_up(agg, dd);
          const bool of = R2L ? __shfl_down_sync(0xffffffffu, f, dd) : __shfl_up_sync(0xffffffffu, f, dd);
          if (R2L ? lane + dd < 32 : lane >= dd) {
            if (!f) agg = R2L ? A::comb(agg, ov) : A::comb(ov, agg);
            f = f || of;
          }
        }
        const S ev = R2L ? shfl_down(agg, 1) : shfl_up(agg, 1);
        const bool ef = R2L ? __shfl_down_sync(0xffffffffu, f, 1) : __shfl_up_sync(0xffffffffu, f, 1);
        const bool edge = R2L ? lane == 31 : lane == 0;
        excl_new = edge ? A::id() : ev;
        exf_new = edge ? false : ef;
        if (R2L ? lane == 0 : lane == 31) {
          s_warp[pn][warp] = agg;
          s_wflag[pn][warp] = f;
        }
      } else if (!R2L) {
        S agg = A::lift(x[0]);
#pragma unroll
        for (int j = 1; j < ITEMS; ++j) agg = A::push(agg, x[j]);
        const S incl = warp_scan_incl<A>(agg);
        const S up = shfl_up(incl, 1);
        excl_new = lane == 0 ? A::id() : up;
        if (lane == 31) s_warp[pn][warp] = incl;
      } else {
        S agg = A::lift(x[ITEMS - 1]);
#pragma unroll
        for (int j = ITEMS - 2; j >= 0; --j) agg = A::push(agg, x[j]);
        const S incl = warp_scan_incl_rev<A>(agg);
        const S dn = shfl_down(incl, 1);
        excl_new = lane == 31 ? A::id() : dn;
        if (lane == 0) s_warp[pn][warp] = incl;
      }
      named_bar_sync<1, L2S_COMPUTE>();  // A is read; the warp totals are in place
      if (tid == 0) {
        S bagg;
        bool tf = false;
        if constexpr (SEG) {
          bagg = A::id();
#pragma unroll
          for (int i = 0; i < NWARP; ++i) {
            const int w = R2L ? NWARP - 1 - i : i;
            bagg = seg_then(tf, bagg, s_wflag[pn][w], s_warp[pn][w], tf);
          }
        } else {
          bagg = s_warp[pn][0];
#pragma unroll
          for (int w = 1; w < NWARP; ++w) bagg = A::comb(bagg, s_warp[pn][w]);
        }
        s_agg[pn] = bagg;
        s_aflag[pn] = tf;
        s_tile[pn] = t_new;
        const bool first = R2L ? (t_new == a.ntiles - 1) : (t_new == 0);
        // SEG: a tile with a row start knows its inclusive prefix already
        if (tf) publish<S>(a.status, t_new, a.epoch, 2u, bagg);
        else if (!first) publish<S>(a.status, t_new, a.epoch, 1u, bagg);
        mbar_arrive(&aggr[pn]);
        // the CTA's next tile: its HBM load runs during this tile's look-back
        if constexpr (PROD == 2) {
          // the zipped tile goes to its place in the output (for pass 2),
          // and A must be read by that store before the next tile lands in it
          if constexpr (L2S_HINTS) tma_store_2d_hint(&tout, 0, (int)(t_new * SCAN_THREADS), bufA, l2_policy_evict_last());
          else tma_store_2d(&tout, 0, (int)(t_new * SCAN_THREADS), bufA);
          tma_store_commit();
          tma_store_wait_read();
        }
        const int64_t dn = (int64_t)atomicAdd(a.ticket, 1u);
        s_claim = dn;
        if (dn < a.ntiles) load_a(dn);
      }
    } else if (tid == 0) {
      s_tile[pn] = -1;  // no more tiles: the look-back warp stops
      mbar_arrive(&aggr[pn]);
    }
    if (t_cur >= 0) {
      // pass 2 of the current tile (loaded again, from L2, into B): rescan it
      // from its prefix, store it
      const bool okp = mbar_wait_flagged(&pref[pc], (uint32_t)((k - 1) >> 1) & 1u, a.err);
      const bool okb = mbar_wait_flagged(&fullB, phB, a.err);
      if (named_bar_or<1, L2S_COMPUTE>(!(okp && okb))) { failed = true; break; }
      phB ^= 1u;
      b_loading = false;
      S inner = A::id();
      const S pfx = s_prefix[pc];
      S run;
      int jb = ITEMS, je = ITEMS;
      if constexpr (SEG) {
        bool f = false;
        if (!R2L) {
          for (int w = 0; w < warp; ++w) inner = seg_then(f, inner, s_wflag[pc][w], s_warp[pc][w], f);
        } else {
          for (int w = NWARP - 1; w > warp; --w) inner = seg_then(f, inner, s_wflag[pc][w], s_warp[pc][w], f);
        }
        inner = seg_then(f, inner, exf_cur, excl_cur, f);
        run = f ? inner : (R2L ? A::comb(inner, pfx) : A::comb(pfx, inner));
        jb = seg_start(t_cur);
        if constexpr (SEG == 2) je = seg_end(t_cur);
      } else {
        if (!R2L) {
          for (int w = 0; w < warp; ++w) inner = A::comb(inner, s_warp[pc][w]);
        } else {
          for (int w = warp + 1; w < NWARP; ++w) inner = A::comb(inner, s_warp[pc][w]);
        }
        run = R2L ? A::comb(A::comb(excl_cur, inner), pfx) : A::comb(pfx, A::comb(inner, excl_cur));
      }
      T x[ITEMS];
      load_row(bufB, t_cur, x);
      const int64_t grow = t_cur * SCAN_THREADS + tid;
      const bool in_smem = grow < a.full_rows;
      const int64_t e0 = grow * ITEMS;
      // SEG 3: element e0 + j goes to index e0 + j + (its row).  jlast: the
      // offset of the last element of the first element's row, if the line
      // holds it (-1 otherwise); the elements after it lie in the next row.
      int64_t orow = 0;
      int jlast = -1;
      if constexpr (SEG == 3) {
        orow = e0 / a.seg_len;
        const int64_t left = a.seg_len - (e0 - orow * a.seg_len);  // elements of the row from e0 on
        jlast = left <= ITEMS ? (int)(left - 1) : -1;
      }
#pragma unroll
      for (int cc = 0; cc < ITEMS / VEC; ++cc) {
        const int c = R2L ? ITEMS / VEC - 1 - cc : cc;
        T y[VEC];
#pragma unroll
        for (int kk = 0; kk < VEC; ++kk) {
          const int q = R2L ? VEC - 1 - kk : kk;
          const int j = c * VEC + q;
          if (SEG && j == jb) run = seg_reset;
          if (a.exclusive) { y[q] = A::lower(run); run = A::push(run, x[j]); }
          else { run = A::push(run, x[j]); y[q] = A::lower(run); }
          if (SEG == 2 && j == je) static_cast<T *>(a.seg_sums)[(e0 + j) / a.seg_len] = A::lower(run);
          if constexpr (SEG == 3) {
            if (e0 + j < a.n) {
              const int64_t o = e0 + j + orow + ((jlast >= 0 && j > jlast) ? 1 : 0);
              dst[o] = y[q];
              // the row's extra slot follows its last element in memory:
              // the total for scanl z, the seed for scanr z
              if (j == jlast) dst[o + 1] = R2L ? from_bits<T>(a.seed) : A::lower(run);
            }
          }
        }
        if constexpr (SEG == 3) continue;  // stored above, not through shared memory
        if (in_smem) {
          uint4 v;
          memcpy(&v, y, 16);
          *reinterpret_cast<uint4 *>(bufB + swz(tid, c)) = v;
        } else {
#pragma unroll
          for (int q = 0; q < VEC; ++q)
            if (e0 + c * VEC + q < a.n) dst[e0 + c * VEC + q] = y[q];
        }
      }
      fence_proxy_async_smem();
      named_bar_sync<1, L2S_COMPUTE>();
      if (tid == 0 && SEG != 3) {
        if constexpr (L2S_HINTS) tma_store_2d_hint(&tout, 0, (int)(t_cur * SCAN_THREADS), bufB, l2_policy_evict_first());
        else tma_store_2d(&tout, 0, (int)(t_cur * SCAN_THREADS), bufB);
        tma_store_commit();
      }
    }
    named_bar_sync<1, L2S_COMPUTE>();  // s_claim is in place
    if (!have_new) break;
    d_new = s_claim;
    t_cur = t_new;
    excl_cur = excl_new;
    exf_cur = exf_new;
    ++k;
  }
  if (tid == 0) {
    if (failed) {
      raise_error(a.err, DEV_ERR_TIMEOUT);
      // bounded waits for this CTA's loads still in flight
      if (s_claim < a.ntiles) mbar_wait(&fullA, phA);
      if (b_loading) mbar_wait(&fullB, phB);
      s_tile[(int)(k & 1)] = -1;
      mbar_arrive(&aggr[(int)(k & 1)]);
    }
    tma_store_wait_all();
    // The last CTA to finish re-arms the ticket for the next launch.
    __threadfence();
    if (atomicAdd(a.done, 1u) == gridDim.x - 1) {
      *a.ticket = 0u;
      *a.done = 0u;
    }
  }
}

// scan f z (zipWith g xs ys) for 16-byte aligned xs, ys and output (the
// reference's delayed scan input, PTX/CodeGen/Scan.hs:141-439 reading a
// MIRDelayed array): one 32 KiB tile of xs and the same tile of ys arrive by
// two 2-D TMA loads on one mbarrier, each thread zips its own row into the
// xs buffer, and the zipped tile is scanned and stored as scan_tma_kernel
// scans and stores one sub-tile.  The zipped array is never written; 64 KiB
// of shared memory per CTA, three CTAs per SM.
template <int OP, class T, int PREC, bool R2L>
__global__ void __launch_bounds__(SCAN_THREADS, 3)
scan_zip_tma_kernel(const __grid_constant__ CUtensorMap tin, const __grid_constant__ CUtensorMap tin2,
                    const __grid_constant__ CUtensorMap tout, ScanArgs a) {
  using S = typename Acc<OP, T, PREC>::S;
  constexpr int SUB_BYTES = SCAN_THREADS * SCAN_ROW_BYTES;
  extern __shared__ unsigned char smem_raw[];
  unsigned char *buf = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char *buf2 = buf + SUB_BYTES;
  __shared__ uint64_t bar;
  __shared__ int64_t s_tile;
  __shared__ S s_warp[1][SCAN_THREADS / 32];
  __shared__ S s_prefix;
  const int tid = threadIdx.x;
  if (tid == 0) {
    const uint32_t dyn = atomicAdd(a.ticket, 1u);
    if ((int64_t)dyn == a.ntiles - 1) *a.ticket = 0u;
    const int64_t tile = R2L ? a.ntiles - 1 - (int64_t)dyn : (int64_t)dyn;
    s_tile = tile;
    mbar_init(&bar, 1);
    fence_mbar_init();
    mbar_expect_tx(&bar, 2 * SUB_BYTES);
    tma_load_2d(buf, &tin, 0, (int)(tile * SCAN_THREADS), &bar);
    tma_load_2d(buf2, &tin2, 0, (int)(tile * SCAN_THREADS), &bar);
  }
  __syncthreads();
  const int64_t tile = s_tile;
  // A tile whose load never landed is neither read nor published: its
  // successors' look-backs give up in turn and the call reports the timeout.
  if (__syncthreads_or(!mbar_wait_flagged(&bar, 0, a.err))) return;
  // Rows past the array's full 128 B lines are read (and zipped) from global
  // memory by the tile body.
  if (tile * SCAN_THREADS + tid < a.full_rows) {
    switch (a.zop) {
      case ACC_ADD: zip_row<T, ACC_ADD>(buf, buf2, tid); break;
      case ACC_MUL: zip_row<T, ACC_MUL>(buf, buf2, tid); break;
      case ACC_MIN: zip_row<T, ACC_MIN>(buf, buf2, tid); break;
      default: zip_row<T, ACC_MAX>(buf, buf2, tid); break;
    }
  }
  auto store_sub = [&](int u) {
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tma_store_2d(&tout, 0, (int)((tile + u) * SCAN_THREADS), buf + u * SUB_BYTES);
      tma_store_commit();
    }
  };
  scan_tile_body<OP, T, PREC, R2L, 1, true>(buf, tile, a, s_warp, s_prefix, false, store_sub);
  if (tid == 0) tma_store_wait_read();
}

// --------------------------------------------------------------------------
// Row scans (rank >= 2): one CTA per row, chunks of 256 x 4 elements with a
// carried prefix.  in/out rows have pitches in_pitch / out_pitch (elements).
struct RowScanArgs {
  const void *in;
  void *out;
  void *sums;        // per-row totals (scan') or null
  int64_t outer, inner;
  int64_t in_pitch, out_pitch;
  int64_t out_shift; // 1 for scanl z (output index i+1 holds the inclusive prefix of i), else 0
  uint64_t seed;
  int has_seed;
  int exclusive;
  int seed_at_end;   // scanr z: out[row][inner] = z
  int total_at_end;  // scanl z: out[row][inner] = total
  const void *in2;   // ZIP kernels: element e of row r is zop(in[r][e], in2[r][e]) (pitch in_pitch)
  int zop;           // ... MAP kernels: it is zop(in[r][e], c)
  uint64_t mapc;     // MAP kernels: the constant c (bits of one element)
};

template <int OP, class T, int PREC, bool R2L, bool ZIP = false, bool MAP = false>
__global__ void __launch_bounds__(256) scan_rows_kernel(RowScanArgs a) {
  using A = Acc<OP, T, PREC>;
  using S = typename A::S;
  constexpr int K = 4;
  constexpr int CH = 256 * K;
  __shared__ S s_warp[8];
  __shared__ S s_carry;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const T idT = Prim<OP, T>::id();
  for (int64_t r = blockIdx.x; r < a.outer; r += gridDim.x) {
    const T *src = static_cast<const T *>(a.in) + r * a.in_pitch;
    const T *src2 = ZIP ? static_cast<const T *>(a.in2) + r * a.in_pitch : nullptr;
    (void)src2;
    T *dst = static_cast<T *>(a.out) + r * a.out_pitch;
    if (tid == 0) s_carry = a.has_seed ? A::lift(from_bits<T>(a.seed)) : A::id();
    __syncthreads();
    const int64_t nch = (a.inner + CH - 1) / CH;
    for (int64_t ci = 0; ci < nch; ++ci) {
      const int64_t c = R2L ? nch - 1 - ci : ci;
      const int64_t e0 = c * CH + (int64_t)tid * K;
      T x[K];
#pragma unroll
      for (int j = 0; j < K; ++j) {
        x[j] = idT;
        if (e0 + j < a.inner) {
          if constexpr (ZIP) x[j] = zip_elem(a.zop, src[e0 + j], src2[e0 + j]);
          else if constexpr (MAP) x[j] = zip_elem(a.zop, src[e0 + j], from_bits<T>(a.mapc));
          else x[j] = src[e0 + j];
        }
      }
      S agg;
      if (!R2L) { agg = A::lift(x[0]); for (int j = 1; j < K; ++j) agg = A::push(agg, x[j]); }
      else { agg = A::lift(x[K - 1]); for (int j = K - 2; j >= 0; --j) agg = A::push(agg, x[j]); }
      S incl, ex;
      if (!R2L) {
        incl = warp_scan_incl<A>(agg);
        S up = shfl_up(incl, 1);
        ex = lane == 0 ? A::id() : up;
        if (lane == 31) s_warp[warp] = incl;
      } else {
        incl = warp_scan_incl_rev<A>(agg);
        S dn = shfl_down(incl, 1);
        ex = lane == 31 ? A::id() : dn;
        if (lane == 0) s_warp[warp] = incl;
      }
      __syncthreads();
      S wpre = A::id();
      if (!R2L) { for (int w = 0; w < warp; ++w) wpre = A::comb(wpre, s_warp[w]); }
      else { for (int w = warp + 1; w < 8; ++w) wpre = A::comb(wpre, s_warp[w]); }
      S bagg = s_warp[0];
      for (int w = 1; w < 8; ++w) bagg = A::comb(bagg, s_warp[w]);
      const S carry = s_carry;
      S run = R2L ? A::comb(A::comb(ex, wpre), carry) : A::comb(carry, A::comb(wpre, ex));
      if (!R2L) {
#pragma unroll
        for (int j = 0; j < K; ++j) {
          T yv;
          if (a.exclusive) { yv = A::lower(run); run = A::push(run, x[j]); }
          else { run = A::push(run, x[j]); yv = A::lower(run); }
          if (e0 + j < a.inner) dst[e0 + j] = yv;
        }
      } else {
#pragma unroll
        for (int j = K - 1; j >= 0; --j) {
          T yv;
          if (a.exclusive) { yv = A::lower(run); run = A::push(run, x[j]); }
          else { run = A::push(run, x[j]); yv = A::lower(run); }
          if (e0 + j < a.inner) dst[e0 + j] = yv;
        }
      }
      __syncthreads();
      if (tid == 0) s_carry = R2L ? A::comb(bagg, carry) : A::comb(carry, bagg);
      __syncthreads();
    }
    if (tid == 0) {
      const T total = A::lower(s_carry);
      if (a.sums) static_cast<T *>(a.sums)[r] = total;
      if (a.total_at_end) dst[a.inner] = total;
      if (a.seed_at_end) dst[a.inner] = from_bits<T>(a.seed);
    }
    __syncthreads();
  }
}

// ----------------------------------------------------------------- host side
constexpr size_t SCAN_SMEM = SCAN_THREADS * SCAN_ROW_BYTES + 1024;

template <int OP, class T, int PREC, bool R2L, int SUB, bool MAP = false>
int launch_scan_1d_sub(Workspace *w, const T *in, T *out, T *total_out, T *seed_out, int64_t n,
                       bool has_seed, bool exclusive, uint64_t seed, cudaStream_t s, int mop = 0,
                       uint64_t mapc = 0) {
  constexpr int ITEMS = SCAN_ROW_BYTES / sizeof(T);
  CUtensorMap tin, tout;
  memset(&tin, 0, sizeof(tin));
  memset(&tout, 0, sizeof(tout));
  const int64_t full_rows = n / ITEMS;
  const bool tma = full_rows > 0 &&
                   encode_2d(&tin, in, sizeof(T), ITEMS, full_rows, SCAN_ROW_BYTES, ITEMS, SCAN_THREADS, true) &&
                   encode_2d(&tout, out, sizeof(T), ITEMS, full_rows, SCAN_ROW_BYTES, ITEMS, SCAN_THREADS, true);
  const int sub = tma ? SUB : 1;
  const int64_t tile_elems = (int64_t)sub * SCAN_THREADS * ITEMS;
  const int64_t ntiles = cdiv_h(n, tile_elems);
  if (ntiles >= (1ll << 31)) return ACC_ERR_TOO_LARGE;
  int st = ws_status(w, (size_t)ntiles * 2);
  if (st) return st;
  ScanArgs a{};
  a.in = in; a.out = out; a.total_out = total_out; a.seed_out = seed_out;
  a.n = n;
  a.full_rows = full_rows;
  a.ntiles = ntiles;
  a.seed = seed;
  a.status = w->status;
  a.ticket = w->words + W_TICKET;
  a.err = w->words + W_ERR;
  a.epoch = ws_next_epoch(w, s);
  a.has_seed = has_seed;
  a.exclusive = exclusive;
  a.tma_in = a.tma_out = tma;
  a.zop = mop;
  a.mapc = mapc;
  if (tma) {
    const size_t smem = (size_t)SUB * SCAN_THREADS * SCAN_ROW_BYTES + 1024;
    auto kern = scan_tma_kernel<OP, T, PREC, R2L, SUB, MAP>;
    static std::atomic<uint64_t> attr_done{0};
    smem_attrs_once(kern, (int)smem, attr_done);
    kern<<<(unsigned)ntiles, SCAN_THREADS, smem, s>>>(tin, tout, a);
    return check_launch();
  }
  auto kern = scan_lookback_kernel<OP, T, PREC, R2L, false, MAP>;
  static std::atomic<uint64_t> attr_done{0};
  smem_attrs_once(kern, (int)SCAN_SMEM, attr_done);
  kern<<<(unsigned)ntiles, SCAN_THREADS, SCAN_SMEM, s>>>(a);
  return check_launch();
}

// The persistent L2-re-read kernel; *launched false when the array cannot be
// described by a TMA tensor map or the cooperative grid cannot be placed.
template <int OP, class T, int PREC, bool R2L, int PROD = 0, int SEG = 0>
int launch_scan_l2(Workspace *w, const T *in, T *out, T *total_out, T *seed_out, int64_t n, bool has_seed,
                   bool exclusive, uint64_t seed, cudaStream_t s, bool *launched, const T *in2 = nullptr,
                   int zop = 0, uint64_t mapc = 0, int64_t seg_len = 0, T *seg_sums = nullptr) {
  constexpr int ITEMS = SCAN_ROW_BYTES / sizeof(T);
  *launched = false;
  CUtensorMap tin, tout, tin2;
  memset(&tin, 0, sizeof(tin));
  memset(&tout, 0, sizeof(tout));
  memset(&tin2, 0, sizeof(tin2));
  const int64_t full_rows = n / ITEMS;
  if (full_rows == 0 ||
      !encode_2d(&tin, in, sizeof(T), ITEMS, full_rows, SCAN_ROW_BYTES, ITEMS, SCAN_THREADS, true) ||
      !encode_2d(&tout, out, sizeof(T), ITEMS, full_rows, SCAN_ROW_BYTES, ITEMS, SCAN_THREADS, true))
    return ACC_OK;
  if (PROD == 2 && !encode_2d(&tin2, in2, sizeof(T), ITEMS, full_rows, SCAN_ROW_BYTES, ITEMS, SCAN_THREADS, true))
    return ACC_OK;
  const int64_t ntiles = cdiv_h(n, (int64_t)SCAN_THREADS * ITEMS);
  // TMA row coordinates are 32-bit: larger arrays take the other kernels.
  if (ntiles * SCAN_THREADS >= (1ll << 31)) return ACC_OK;
  const size_t smem = (PROD == 2 ? 3 : 2) * (size_t)L2S_TILE + 1024;
  auto kern = scan_l2_kernel<OP, T, PREC, R2L, PROD, SEG>;
  static std::atomic<uint64_t> attr_done{0};
  smem_attrs_once(kern, (int)smem, attr_done);
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, L2S_THREADS, smem) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    return ACC_OK;
  }
  int st = ws_status(w, (size_t)ntiles * 2);
  if (st) return st;
  ScanArgs a{};
  a.in = in; a.out = out; a.total_out = total_out; a.seed_out = seed_out;
  a.n = n;
  a.full_rows = full_rows;
  a.ntiles = ntiles;
  a.seed = seed;
  a.status = w->status;
  a.ticket = w->words + W_TICKET;
  a.done = w->words + W_DONE;
  a.err = w->words + W_ERR;
  a.epoch = ws_next_epoch(w, s);
  a.has_seed = has_seed;
  a.exclusive = exclusive;
  a.tma_in = a.tma_out = 1;
  a.in2 = in2;
  a.zop = zop;
  a.mapc = mapc;
  a.seg_len = SEG ? seg_len : 1;
  a.seg_sums = SEG ? seg_sums : nullptr;
  int64_t grid = (int64_t)device_info().sms * per_sm;
  if (grid > ntiles) grid = ntiles;
  // A cooperative launch places every CTA at once (or fails): the tiles a CTA
  // takes wait on tiles that other CTAs hold, so all of them must run together.
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(L2S_THREADS);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const cudaError_t e = cudaLaunchKernelEx(&cfg, kern, tin, tout, a, tin2);
  *launched = true;
  return cuda_status(e);
}

// Large arrays take the persistent kernel (over a fused map as well).  The
// tile kernel's size below that: 2 sub-tiles (64 KiB, 3 CTAs per SM) by
// default, the faster of the two on GB300 at 2^25..2^28 elements;
// ACC_GB300_SCAN_SUB=1 selects 32 KiB tiles (6 CTAs per SM).  A scan over a
// fused map (MAP: map (\x -> mop x c)) always takes the 64 KiB tiles there.
template <int OP, class T, int PREC, bool R2L, bool MAP = false>
int launch_scan_1d(Workspace *w, const T *in, T *out, T *total_out, T *seed_out, int64_t n,
                   bool has_seed, bool exclusive, uint64_t seed, cudaStream_t s, int mop = 0,
                   uint64_t mapc = 0) {
  // Arrays of at least four 32 KiB tiles per SM take the persistent
  // L2-re-read kernel (ACC_GB300_SCAN_KERNEL=tile keeps the tile kernel).
  static const bool l2k = !(getenv("ACC_GB300_SCAN_KERNEL") && strcmp(getenv("ACC_GB300_SCAN_KERNEL"), "tile") == 0);
  if (l2k && n * (int64_t)sizeof(T) >= (int64_t)device_info().sms * 4 * L2S_TILE) {
    bool launched = false;
    const int st = launch_scan_l2<OP, T, PREC, R2L, MAP ? 1 : 0>(w, in, out, total_out, seed_out, n, has_seed,
                                                                 exclusive, seed, s, &launched, nullptr, mop, mapc);
    if (st || launched) return st;
  }
  if constexpr (MAP)
    return launch_scan_1d_sub<OP, T, PREC, R2L, 2, true>(w, in, out, total_out, seed_out, n, has_seed, exclusive,
                                                          seed, s, mop, mapc);
  static const int sub = getenv("ACC_GB300_SCAN_SUB") ? atoi(getenv("ACC_GB300_SCAN_SUB")) : 2;
  if (sub == 2)
    return launch_scan_1d_sub<OP, T, PREC, R2L, 2>(w, in, out, total_out, seed_out, n, has_seed, exclusive, seed, s);
  return launch_scan_1d_sub<OP, T, PREC, R2L, 1>(w, in, out, total_out, seed_out, n, has_seed, exclusive, seed, s);
}

// Short rows, many of them: one warp per row.  The warp walks the row in
// chunks of 32 elements (one per lane, coalesced), scans each chunk with
// shuffles and carries the prefix in a register; the semantics are those of
// scan_rows_kernel (seed placement, exclusive flavours, totals).
template <int OP, class T, int PREC, bool R2L, bool ZIP = false, bool MAP = false>
__global__ void __launch_bounds__(256) scan_rows_warp_kernel(RowScanArgs a) {
  using A = Acc<OP, T, PREC>;
  using S = typename A::S;
  const int lane = threadIdx.x & 31;
  const T idT = Prim<OP, T>::id();
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = gw; r < a.outer; r += nw) {
    const T *src = static_cast<const T *>(a.in) + r * a.in_pitch;
    const T *src2 = ZIP ? static_cast<const T *>(a.in2) + r * a.in_pitch : nullptr;
    (void)src2;
    T *dst = static_cast<T *>(a.out) + r * a.out_pitch;
    S carry = a.has_seed ? A::lift(from_bits<T>(a.seed)) : A::id();
    const int64_t nch = (a.inner + 31) / 32;
    for (int64_t ci = 0; ci < nch; ++ci) {
      const int64_t c = R2L ? nch - 1 - ci : ci;
      const int64_t e = c * 32 + lane;
      T x = idT;
      if (e < a.inner) {
        if constexpr (ZIP) x = zip_elem(a.zop, src[e], src2[e]);
        else if constexpr (MAP) x = zip_elem(a.zop, src[e], from_bits<T>(a.mapc));
        else x = src[e];
      }
      const S v = A::lift(x);
      S incl, ex, tot;
      if (!R2L) {
        incl = warp_scan_incl<A>(v);
        const S up = shfl_up(incl, 1);
        ex = lane == 0 ? A::id() : up;
        tot = shfl_idx(incl, 31);
      } else {
        incl = warp_scan_incl_rev<A>(v);
        const S dn = shfl_down(incl, 1);
        ex = lane == 31 ? A::id() : dn;
        tot = shfl_idx(incl, 0);
      }
      // Everything before (L2R) / after (R2L) this element within the row.
      const S before = R2L ? A::comb(ex, carry) : A::comb(carry, ex);
      const T yv = a.exclusive ? A::lower(before) : A::lower(A::push(before, x));
      if (e < a.inner) dst[e] = yv;
      carry = R2L ? A::comb(tot, carry) : A::comb(carry, tot);
    }
    if (lane == 0) {
      const T total = A::lower(carry);
      if (a.sums) static_cast<T *>(a.sums)[r] = total;
      if (a.total_at_end) dst[a.inner] = total;
      if (a.seed_at_end) dst[a.inner] = from_bits<T>(a.seed);
    }
  }
}

template <int OP, class T, int PREC, bool R2L, bool ZIP = false, bool MAP = false>
int launch_scan_rows(const RowScanArgs &a, cudaStream_t s) {
  const Device &d = device_info();
  if (a.inner <= 512 && a.outer >= (int64_t)d.sms * 64) {
    // a warp per row: 8 rows per CTA
    int64_t blocks = cdiv_h(a.outer, 8);
    if (blocks > (int64_t)d.sms * 16) blocks = (int64_t)d.sms * 16;
    scan_rows_warp_kernel<OP, T, PREC, R2L, ZIP, MAP><<<(unsigned)blocks, 256, 0, s>>>(a);
    return check_launch();
  }
  int64_t blocks = a.outer;
  if (blocks > (int64_t)d.sms * 8) blocks = (int64_t)d.sms * 8;
  scan_rows_kernel<OP, T, PREC, R2L, ZIP, MAP><<<(unsigned)blocks, 256, 0, s>>>(a);
  return check_launch();
}

// A 1-D scan over zipWith g in in2 (g = zop): the zipped tile kernel when
// the three arrays are 16-byte aligned, else the plain-load look-back kernel
// zipping as it loads.  Tiles of 32 KiB in both cases.
template <int OP, class T, int PREC, bool R2L>
int launch_scan_zip_1d(Workspace *w, const T *in, const T *in2, int zop, T *out, T *total_out, T *seed_out,
                       int64_t n, bool has_seed, bool exclusive, uint64_t seed, cudaStream_t s) {
  constexpr int ITEMS = SCAN_ROW_BYTES / sizeof(T);
  CUtensorMap tin, tin2, tout;
  memset(&tin, 0, sizeof(tin));
  memset(&tin2, 0, sizeof(tin2));
  memset(&tout, 0, sizeof(tout));
  const int64_t full_rows = n / ITEMS;
  const bool tma = full_rows > 0 &&
                   encode_2d(&tin, in, sizeof(T), ITEMS, full_rows, SCAN_ROW_BYTES, ITEMS, SCAN_THREADS, true) &&
                   encode_2d(&tin2, in2, sizeof(T), ITEMS, full_rows, SCAN_ROW_BYTES, ITEMS, SCAN_THREADS, true) &&
                   encode_2d(&tout, out, sizeof(T), ITEMS, full_rows, SCAN_ROW_BYTES, ITEMS, SCAN_THREADS, true);
  const int64_t ntiles = cdiv_h(n, (int64_t)SCAN_THREADS * ITEMS);
  if (ntiles >= (1ll << 31)) return ACC_ERR_TOO_LARGE;
  // Arrays of at least four 32 KiB tiles per SM take the persistent
  // L2-re-read kernel, zipping in its first pass.
  static const bool l2k = !(getenv("ACC_GB300_SCAN_KERNEL") && strcmp(getenv("ACC_GB300_SCAN_KERNEL"), "tile") == 0);
  if (tma && l2k && n * (int64_t)sizeof(T) >= (int64_t)device_info().sms * 4 * L2S_TILE) {
    bool launched = false;
    const int st2 = launch_scan_l2<OP, T, PREC, R2L, 2>(w, in, out, total_out, seed_out, n, has_seed, exclusive, seed,
                                                        s, &launched, in2, zop);
    if (st2 || launched) return st2;
  }
  int st = ws_status(w, (size_t)ntiles * 2);
  if (st) return st;
  ScanArgs a{};
  a.in = in; a.out = out; a.total_out = total_out; a.seed_out = seed_out;
  a.in2 = in2; a.zop = zop;
  a.n = n;
  a.full_rows = full_rows;
  a.ntiles = ntiles;
  a.seed = seed;
  a.status = w->status;
  a.ticket = w->words + W_TICKET;
  a.err = w->words + W_ERR;
  a.epoch = ws_next_epoch(w, s);
  a.has_seed = has_seed;
  a.exclusive = exclusive;
  a.tma_in = a.tma_out = tma;
  if (tma) {
    const size_t smem = 2 * (size_t)SCAN_THREADS * SCAN_ROW_BYTES + 1024;
    auto kern = scan_zip_tma_kernel<OP, T, PREC, R2L>;
    static std::atomic<uint64_t> attr_done{0};
    smem_attrs_once(kern, (int)smem, attr_done);
    kern<<<(unsigned)ntiles, SCAN_THREADS, smem, s>>>(tin, tin2, tout, a);
    return check_launch();
  }
  auto kern = scan_lookback_kernel<OP, T, PREC, R2L, true>;
  static std::atomic<uint64_t> attr_done{0};
  smem_attrs_once(kern, (int)SCAN_SMEM, attr_done);
  kern<<<(unsigned)ntiles, SCAN_THREADS, SCAN_SMEM, s>>>(a);
  return check_launch();
}

// Every scan flavour (kind: ACC_SCAN_INCLUSIVE / SEEDED / PRIME) over the
// rows of a contiguous [outer x inner] array by the
// persistent kernel's segmented form (scan_seg.cu, a translation unit of its
// own); *launched false where it does not apply (operator outside + * min
// max, rows shorter than a 128-byte line, the array not describable by a TMA
// tensor map), and the row kernels take the call.
int scan_rows_seg(Workspace *w, int op, int type, int prec, bool r2l, int kind, const void *in, void *out,
                  void *sums, uint64_t seed, int64_t outer, int64_t inner, cudaStream_t s, bool *launched);
template <class T> constexpr int type_code() {
  return std::is_same<T, int32_t>::value ? ACC_I32 : std::is_same<T, int64_t>::value ? ACC_I64
       : std::is_same<T, uint32_t>::value ? ACC_U32 : std::is_same<T, float>::value ? ACC_F32 : ACC_F64;
}

// Every scan flavour over one array, or (ZIP) over zipWith g in in2 with
// g = zop, both [outer x inner], or (MAP) over map (\x -> g x c) in with
// g = zop and c given by its bits `mapc`.
template <int OP, class T, int PREC, bool ZIP = false, bool MAP = false>
int scan_typed(Workspace *w, int dir, int kind, const T *in, T *out, T *sums, int64_t outer,
               int64_t inner, uint64_t seed, cudaStream_t s, const T *in2 = nullptr, int zop = 0,
               uint64_t mapc = 0) {
  const bool r2l = dir == ACC_R2L;
  const bool seeded = kind != ACC_SCAN_INCLUSIVE;
  // Empty innermost extent: scanl/scanr z give [z]; scanl'/scanr' give
  // ([], z); scanl1/scanr1 give [] (PTX/Execute.hs:386-404,500-512).
  if (inner == 0) {
    if (kind == ACC_SCAN_SEEDED) return launch_fill<T>(out, outer, seed, s);
    if (kind == ACC_SCAN_PRIME) return launch_fill<T>(sums, outer, seed, s);
    return ACC_OK;
  }
  // Output element i lines up with input element i in every flavour:
  //   scanl z  (L2R, exclusive, total -> out[n])
  //   scanr z  (R2L, inclusive with the seed on the right, z -> out[n])
  //   scanl' z (L2R, exclusive, total -> sums), scanr' z (R2L, exclusive, total -> sums)
  const bool exclusive = kind == ACC_SCAN_PRIME || (kind == ACC_SCAN_SEEDED && !r2l);
  if (outer == 1) {
    T *total_out = nullptr, *seed_out = nullptr;
    if (kind == ACC_SCAN_SEEDED && !r2l) total_out = out + inner;
    if (kind == ACC_SCAN_SEEDED && r2l) seed_out = out + inner;
    if (kind == ACC_SCAN_PRIME) total_out = sums;
    if constexpr (ZIP) {
      if (r2l)
        return launch_scan_zip_1d<OP, T, PREC, true>(w, in, in2, zop, out, total_out, seed_out, inner, seeded,
                                                     exclusive, seed, s);
      return launch_scan_zip_1d<OP, T, PREC, false>(w, in, in2, zop, out, total_out, seed_out, inner, seeded,
                                                    exclusive, seed, s);
    } else {
      (void)in2;
      if (r2l)
        return launch_scan_1d<OP, T, PREC, true, MAP>(w, in, out, total_out, seed_out, inner, seeded, exclusive,
                                                      seed, s, zop, mapc);
      return launch_scan_1d<OP, T, PREC, false, MAP>(w, in, out, total_out, seed_out, inner, seeded, exclusive,
                                                     seed, s, zop, mapc);
    }
  }
  if constexpr (!ZIP && !MAP) {
    // Long scanl1 / scanr1 / scanl' / scanr' over rows: one segmented pass
    // over the whole array (at least four 32 KiB tiles per SM).
    if (outer * inner * (int64_t)sizeof(T) >= (int64_t)device_info().sms * 4 * L2S_TILE) {
      bool launched = false;
      const int pc = PREC == 1 ? ACC_PREC_COMPENSATED : (PREC == 2 ? ACC_PREC_FP64ACC : ACC_PREC_PLAIN);
      const int st = scan_rows_seg(w, OP, type_code<T>(), pc, r2l, kind, in, out, kind == ACC_SCAN_PRIME ? sums : nullptr,
                                   seed, outer, inner, s, &launched);
      if (st || launched) return st;
    }
  }
  RowScanArgs a{};
  a.in = in; a.out = out; a.sums = kind == ACC_SCAN_PRIME ? sums : nullptr;
  a.outer = outer; a.inner = inner;
  a.in_pitch = inner;
  a.out_pitch = kind == ACC_SCAN_SEEDED ? inner + 1 : inner;
  a.seed = seed; a.has_seed = seeded; a.exclusive = exclusive;
  a.seed_at_end = kind == ACC_SCAN_SEEDED && r2l;
  a.total_at_end = kind == ACC_SCAN_SEEDED && !r2l;
  a.in2 = in2; a.zop = zop; a.mapc = mapc;
  if (r2l) return launch_scan_rows<OP, T, PREC, true, ZIP, MAP>(a, s);
  return launch_scan_rows<OP, T, PREC, false, ZIP, MAP>(a, s);
}

}  // namespace accgb
