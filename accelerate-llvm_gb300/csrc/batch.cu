// batch.cu -- many independent fold / scanl1 requests in ONE persistent launch,
// replayable as a CUDA graph, with tile sizes from the library's autotuner.
//
// The reference launches every skeleton separately, each with host-side
// set-up (PTX/Execute.hs:835-881); thousands of small and medium requests are
// dominated by launch latency.  Here a plan flattens a batch into work items
// (request, tile), each request cut into tiles of NT x IPT elements; the
// autotuner picks the launch shape (NT threads per CTA: 128, 256 or 512) and
// the tile shape (IPT elements per thread) per (kind, type, size bucket), and
// a batch runs with the NT preferred by most of its bytes.  One persistent
// kernel draws items from an atomic ticket in table order:
//   * fold tiles reduce their chunk (16-byte vector loads); the last tile of
//     a request (per-request atomic ticket) folds the tile partials in order
//     and writes z `f` result;
//   * scan tiles stage their chunk in shared memory, scan it, and take the
//     prefix of the earlier tiles of the same request by decoupled look-back
//     (items are drawn in order, so every predecessor tile belongs to a
//     running CTA).
// All scratch is owned by the plan and allocated when the plan is made; a
// launch allocates nothing and takes its look-back epoch from a device word
// that the last CTA advances, so a captured graph replays unchanged.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "common.cuh"

namespace accgb {

constexpr int BT = 256;                    // threads per CTA of untuned launches and of the serving arena
constexpr int B_MAX_TILE_BYTES = 32768;    // largest tile staged in shared memory

struct BReq {
  const void *in;
  void *out;
  int64_t n;
  uint64_t seed;
  int64_t first_item;
  int64_t ntiles;
  int32_t kind, type, has_seed, ipt;
};

struct BatchArgs {
  const BReq *reqs;
  const int32_t *item_req;
  int64_t nitems;
  uint64_t *status;      // 2 words per item (scan look-back)
  uint64_t *partials;    // one state per item (fold)
  uint32_t *req_ticket;  // per request, zero between launches
  uint32_t *words;       // [0] error, [1] item ticket, [2] epoch
};

// ---------------------------------------------------------------- device parts
template <class S>
__device__ __forceinline__ void b_publish(uint64_t *status, int64_t t, uint32_t epoch, uint32_t flag, S v) {
  uint64_t b = to_bits(v);
  uint64_t tag = (uint64_t)((epoch << 2) | flag) << 32;
  if constexpr (sizeof(S) == 8) st_relaxed_u64(status + 2 * t + 1, tag | (b >> 32));
  st_relaxed_u64(status + 2 * t, tag | (b & 0xffffffffull));
}
template <class S>
__device__ __forceinline__ uint32_t b_peek(const uint64_t *status, int64_t t, uint32_t epoch, S &v) {
  const SlotWords s = ld_slot(status + 2 * t);  // both words in one access
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

// CTA-wide ordered reduction (valid in thread 0).
template <class A, int NT>
__device__ __forceinline__ typename A::S b_block_reduce(typename A::S v, typename A::S *s_part) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_reduce<A>(v);
  if (lane == 0) s_part[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = lane < NT / 32 ? s_part[lane] : A::id();
    v = warp_reduce<A>(v);
  }
  __syncthreads();
  return v;
}

template <int OP, class T, int PREC, int NT>
__device__ void b_fold_tile(const BatchArgs &a, const BReq &q, int64_t item, int32_t r, unsigned char *smem) {
  using A = Acc<OP, T, PREC>;
  using S = typename A::S;
  __shared__ bool s_last;
  S *s_part = reinterpret_cast<S *>(smem);
  const int64_t tile = item - q.first_item;
  const int64_t ts = (int64_t)q.ipt * NT;
  const int64_t b = tile * ts;
  const int64_t e = b + ts < q.n ? b + ts : q.n;
  const T *src = static_cast<const T *>(q.in) + b;
  const int64_t len = e - b;
  // 16-byte vector body, scalar head and tail.
  constexpr int VEC = 16 / sizeof(T);
  S acc = A::id();
  const uintptr_t addr = reinterpret_cast<uintptr_t>(src);
  int64_t head = (int64_t)(((16u - (addr & 15u)) & 15u) / sizeof(T));
  if (head > len) head = len;
  if ((int64_t)threadIdx.x < head) acc = A::push(acc, src[threadIdx.x]);
  const int64_t nvec = (len - head) / VEC;
  const uint4 *qv = reinterpret_cast<const uint4 *>(src + head);
  for (int64_t i = threadIdx.x; i < nvec; i += NT) {
    uint4 v = ld_stream16(qv + i);
    T el[VEC];
    memcpy(el, &v, 16);
#pragma unroll
    for (int k = 0; k < VEC; ++k) acc = A::push(acc, el[k]);
  }
  const int64_t tail0 = head + nvec * VEC;
  if (tail0 + threadIdx.x < len) acc = A::push(acc, src[tail0 + threadIdx.x]);
  acc = b_block_reduce<A, NT>(acc, s_part);
  // One 8-byte slot per item whatever the state's size, so that requests of
  // different types in one batch never share partial slots.
  static_assert(sizeof(S) <= sizeof(uint64_t), "fold state larger than a partial slot");
  auto part = [&](int64_t it) { return reinterpret_cast<S *>(a.partials + it); };
  if (threadIdx.x == 0) {
    *part(item) = acc;
    __threadfence();
    const uint32_t prev = atomicAdd(a.req_ticket + r, 1u);
    s_last = prev == (uint32_t)(q.ntiles - 1);
  }
  __syncthreads();
  if (s_last) {
    __threadfence();
    S v = A::id();
    const int64_t per = (q.ntiles + NT - 1) / NT;
    const int64_t lo = threadIdx.x * per, hi = lo + per < q.ntiles ? lo + per : q.ntiles;
    for (int64_t i = lo; i < hi; ++i) v = A::comb(v, ld_state<S>(part(q.first_item + i)));
    v = b_block_reduce<A, NT>(v, s_part);
    if (threadIdx.x == 0) {
      if (q.has_seed) v = A::comb(A::lift(from_bits<T>(q.seed)), v);
      *static_cast<T *>(q.out) = A::lower(v);
      a.req_ticket[r] = 0u;  // re-arm for the next launch
    }
  }
  __syncthreads();
}

template <int OP, class T, int PREC, int IPT, int NT>
__device__ void b_scan_tile(const BatchArgs &a, const BReq &q, int64_t item, uint32_t epoch, unsigned char *smem) {
  using A = Acc<OP, T, PREC>;
  using S = typename A::S;
  __shared__ S s_warp[NT / 32];
  __shared__ S s_prefix;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int ipt = IPT;  // compile time: the staging index math is shifts and masks
  constexpr int pitch = ipt + 1;  // padded row: conflict-free thread-per-row access
  T *tile_s = reinterpret_cast<T *>(smem + 256);
  const int64_t tile = item - q.first_item;
  const int64_t ts = (int64_t)ipt * NT;
  const int64_t b = tile * ts;
  const T idT = Prim<OP, T>::id();
  const T *src = static_cast<const T *>(q.in);
  for (int k = tid; k < ts; k += NT) {
    const int64_t gi = b + k;
    tile_s[(k / ipt) * pitch + (k % ipt)] = gi < q.n ? src[gi] : idT;
  }
  __syncthreads();
  T *row = tile_s + tid * pitch;
  S agg = A::lift(row[0]);
#pragma unroll
  for (int j = 1; j < ipt; ++j) agg = A::push(agg, row[j]);
  S incl = warp_scan_incl<A>(agg);
  S up = shfl_up(incl, 1);
  const S excl_lane = lane == 0 ? A::id() : up;
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  S wpre = A::id();
  for (int w = 0; w < warp; ++w) wpre = A::comb(wpre, s_warp[w]);
  if (warp == 0) {
    S bagg = s_warp[0];
    for (int w = 1; w < NT / 32; ++w) bagg = A::comb(bagg, s_warp[w]);
    S prefix = q.has_seed ? A::lift(from_bits<T>(q.seed)) : A::id();
    if (tile > 0) {
      if (lane == 0) b_publish<S>(a.status, item, epoch, 1u, bagg);
      S acc = A::id();
      int64_t k0 = 0;
      bool gave_up = false;
      while (true) {
        const int64_t d = k0 + lane;
        const bool exists = d < tile;  // predecessors of the same request only
        const int64_t pt = item - 1 - d;
        uint32_t flag = exists ? 0u : 2u;
        S v = A::id();
        uint32_t it = 0;
        uint64_t t_wait = 0;
        while (true) {
          if (exists && flag == 0) flag = b_peek<S>(a.status, pt, epoch, v);
          if (__all_sync(0xffffffffu, flag != 0)) break;
          ++it;
          if (it == 8) t_wait = global_ns();  // first checked at it == 64
          const bool stop = gave_up || it > SPIN_LIMIT ||
                            ((it & 63u) == 0 && ((ld_relaxed_u32(a.words) & DEV_ERR_TIMEOUT) != 0u ||
                                                 global_ns() - t_wait > WAIT_LIMIT_NS));
          if (__any_sync(0xffffffffu, stop)) {
            gave_up = true;
            if (lane == 0) raise_error(a.words, DEV_ERR_TIMEOUT);
            if (flag == 0) flag = 2u;
            break;
          }
          __nanosleep(it < 8 ? 32 : 128);
        }
        const unsigned pm = __ballot_sync(0xffffffffu, flag == 2u);
        const int kp = pm ? __ffs(pm) - 1 : 32;
        if (lane > kp) v = A::id();
        S wv = warp_reduce_rev<A>(v);
        wv = shfl_idx(wv, 0);
        acc = A::comb(wv, acc);
        if (pm) break;
        k0 += 32;
      }
      prefix = acc;  // the seed already sits in the request's first tile
    }
    if (lane == 0) {
      b_publish<S>(a.status, item, epoch, 2u, A::comb(prefix, bagg));
      s_prefix = prefix;
    }
  }
  __syncthreads();
  S run = A::comb(s_prefix, A::comb(wpre, excl_lane));
#pragma unroll
  for (int j = 0; j < ipt; ++j) {
    run = A::push(run, row[j]);
    row[j] = A::lower(run);
  }
  __syncthreads();
  T *dst = static_cast<T *>(q.out);
  for (int k = tid; k < ts; k += NT) {
    const int64_t gi = b + k;
    if (gi < q.n) dst[gi] = tile_s[(k / ipt) * pitch + (k % ipt)];
  }
  __syncthreads();
}

// Scan tiles are instantiated per elements-per-thread (powers of two up to
// the 32 KiB tile limit for NT threads), picked by the tile's planned value.
template <int OP, class T, int PREC, int NT>
__device__ __forceinline__ void b_scan_tile_any(const BatchArgs &a, const BReq &q, int64_t item, uint32_t epoch,
                                                unsigned char *smem) {
  constexpr int MAXI = B_MAX_TILE_BYTES / (NT * (int)sizeof(T));
  switch (q.ipt) {
    case 1: b_scan_tile<OP, T, PREC, 1, NT>(a, q, item, epoch, smem); break;
    case 2: b_scan_tile<OP, T, PREC, 2, NT>(a, q, item, epoch, smem); break;
    case 4: b_scan_tile<OP, T, PREC, 4, NT>(a, q, item, epoch, smem); break;
    case 8: b_scan_tile<OP, T, PREC, 8, NT>(a, q, item, epoch, smem); break;
    default:
      if constexpr (MAXI >= 64) {
        if (q.ipt == 64) { b_scan_tile<OP, T, PREC, 64, NT>(a, q, item, epoch, smem); break; }
      }
      if constexpr (MAXI >= 32) {
        if (q.ipt == 32) { b_scan_tile<OP, T, PREC, 32, NT>(a, q, item, epoch, smem); break; }
      }
      if constexpr (MAXI >= 16) b_scan_tile<OP, T, PREC, 16, NT>(a, q, item, epoch, smem);
      else b_scan_tile<OP, T, PREC, 8, NT>(a, q, item, epoch, smem);
      break;
  }
}

enum { BK_FOLD = 0, BK_SCAN = 1 };

// The register budget: ~51 per thread with 256 or 512 threads (1,280 threads
// per SM), 64 with 128 threads (1,024 per SM; 48 would spill).
template <int OP, int NT>
__global__ void __launch_bounds__(NT, NT == 128 ? 8 : 1280 / NT) batch_kernel(BatchArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int64_t s_item;
  __shared__ BReq s_req;
  __shared__ uint32_t s_epoch;
  if (threadIdx.x == 0) s_epoch = (ld_relaxed_u32(a.words + 2) & ((1u << 29) - 1)) + 1;
  const uint32_t last_ticket = (uint32_t)a.nitems + gridDim.x - 1;
  while (true) {
    if (threadIdx.x == 0) {
      const uint32_t t = atomicAdd(a.words + 1, 1u);
      if (t == last_ticket) {
        // Every CTA has drawn its last ticket (and read the epoch): re-arm the
        // ticket and advance the epoch for the next launch or graph replay.
        a.words[1] = 0u;
        atomicAdd(a.words + 2, 1u);
      }
      s_item = (int64_t)t < a.nitems ? (int64_t)t : -1;
      if (s_item >= 0) s_req = a.reqs[a.item_req[s_item]];
    }
    __syncthreads();
    const int64_t item = s_item;
    if (item < 0) break;
    const BReq q = s_req;
    const int32_t r = a.item_req[item];
    const uint32_t epoch = s_epoch;
    if (q.kind == BK_FOLD) {
      switch (q.type) {
        case ACC_I32: b_fold_tile<OP, int32_t, 0, NT>(a, q, item, r, smem); break;
        case ACC_I64: b_fold_tile<OP, int64_t, 0, NT>(a, q, item, r, smem); break;
        case ACC_F32: b_fold_tile<OP, float, OP == ACC_ADD ? PREC_COMP : PREC_PLAIN, NT>(a, q, item, r, smem); break;
        default: b_fold_tile<OP, double, 0, NT>(a, q, item, r, smem); break;
      }
    } else {
      switch (q.type) {
        case ACC_I32: b_scan_tile_any<OP, int32_t, 0, NT>(a, q, item, epoch, smem); break;
        case ACC_I64: b_scan_tile_any<OP, int64_t, 0, NT>(a, q, item, epoch, smem); break;
        case ACC_F32: b_scan_tile_any<OP, float, OP == ACC_ADD ? PREC_COMP : PREC_PLAIN, NT>(a, q, item, epoch, smem); break;
        default: b_scan_tile_any<OP, double, 0, NT>(a, q, item, epoch, smem); break;
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- autotuner table
// Launch and tile shape per (kind, type, log2 size bucket): NT threads per CTA
// and IPT elements per thread (a tile is NT x IPT elements).  Filled by
// acc_batch_autotune, persisted as JSON.
constexpr int B_NT[3] = {128, 256, 512};
struct TuneKey {
  int kind, type, bucket;
  bool operator<(const TuneKey &o) const { return std::tie(kind, type, bucket) < std::tie(o.kind, o.type, o.bucket); }
};
struct TuneVal {
  int ipt, nt;
};
static std::mutex g_tune_mu;
static std::map<TuneKey, TuneVal> g_tune;

static bool valid_nt(int nt) { return nt == 128 || nt == 256 || nt == 512; }
static int type_bytes(int type) { return (type == ACC_I64 || type == ACC_F64) ? 8 : 4; }
static int max_ipt(int type, int nt) { return B_MAX_TILE_BYTES / (nt * type_bytes(type)); }
// Elements per thread as the kernel takes them: within [1, max_ipt], rounded
// down to a power of two (scan tiles are instantiated for those only).
static int norm_ipt(int ipt, int type, int nt) {
  if (ipt < 1) ipt = 1;
  if (ipt > max_ipt(type, nt)) ipt = max_ipt(type, nt);
  int p = 1;
  while (p * 2 <= ipt) p *= 2;
  return p;
}
static int bucket_of(int64_t n) {
  int b = 0;
  while (b < 62 && (int64_t(1) << (b + 1)) <= n) ++b;
  return b;
}
static int default_ipt(int kind, int type, int64_t n) {
  // Before tuning (256 threads): one wave of small tiles for small requests,
  // large tiles otherwise.
  const int cap = max_ipt(type, BT);
  int ipt = n <= (1 << 14) ? 4 : n <= (1 << 18) ? 8 : 16;
  (void)kind;
  return ipt < cap ? ipt : cap;
}
static TuneVal tuned(int kind, int type, int64_t n) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune.find(TuneKey{kind, type, bucket_of(n)});
  if (it != g_tune.end()) return it->second;
  return TuneVal{default_ipt(kind, type, n), BT};
}
// A request's elements per thread in a launch of nt threads: its tuned tile
// shape where the tuned launch shape is nt, else the same tile size in
// elements.
static int ipt_for(const acc_request &q, int nt) {
  const TuneVal v = tuned(q.kind, q.type, q.n);
  const int ipt = v.nt == nt ? v.ipt : (int)(((int64_t)v.ipt * v.nt) / nt);
  return norm_ipt(ipt, q.type, nt);
}

// ---------------------------------------------------------------- plan
struct Batch {
  int op;
  int device;
  int64_t count = 0, nitems = 0;
  BReq *d_reqs = nullptr;
  int32_t *d_item_req = nullptr;
  uint64_t *d_status = nullptr;
  uint64_t *d_partials = nullptr;
  uint32_t *d_req_ticket = nullptr;
  uint32_t *d_words = nullptr;
  int grid = 0;
  int nt = BT;  // threads per CTA
  size_t smem = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

template <int OP> static void *batch_kernel_ptr(int nt) {
  if (nt == 128) return reinterpret_cast<void *>(batch_kernel<OP, 128>);
  if (nt == 512) return reinterpret_cast<void *>(batch_kernel<OP, 512>);
  return reinterpret_cast<void *>(batch_kernel<OP, 256>);
}
static void *kernel_for(int op, int nt) {
  return op == ACC_ADD ? batch_kernel_ptr<ACC_ADD>(nt) : op == ACC_MIN ? batch_kernel_ptr<ACC_MIN>(nt)
                                                                       : batch_kernel_ptr<ACC_MAX>(nt);
}

template <int OP> static void launch_op(Batch *b, const BatchArgs &a, cudaStream_t s) {
  if (b->nt == 128) batch_kernel<OP, 128><<<b->grid, 128, b->smem, s>>>(a);
  else if (b->nt == 512) batch_kernel<OP, 512><<<b->grid, 512, b->smem, s>>>(a);
  else batch_kernel<OP, 256><<<b->grid, 256, b->smem, s>>>(a);
}
static int batch_launch_raw(Batch *b, cudaStream_t s) {
  BatchArgs a{b->d_reqs, b->d_item_req, b->nitems, b->d_status, b->d_partials, b->d_req_ticket, b->d_words};
  switch (b->op) {
    case ACC_ADD: launch_op<ACC_ADD>(b, a, s); break;
    case ACC_MIN: launch_op<ACC_MIN>(b, a, s); break;
    default: launch_op<ACC_MAX>(b, a, s); break;
  }
  return check_launch();
}

static void batch_free(Batch *b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  cudaFree(b->d_reqs);
  cudaFree(b->d_item_req);
  cudaFree(b->d_status);
  cudaFree(b->d_partials);
  cudaFree(b->d_req_ticket);
  cudaFree(b->d_words);
  delete b;
}

// nt_override > 0 fixes the launch shape (with ipt_override, the tile
// shapes: the autotuner's trial launches); otherwise the batch takes the
// tuned launch shape that most of its bytes prefer.
static int batch_make(int op, const acc_request *reqs, int64_t count, const int32_t *ipt_override, int nt_override,
                      Batch **out) {
  if (op != ACC_ADD && op != ACC_MIN && op != ACC_MAX) return ACC_ERR_UNSUPPORTED;
  if (count < 0 || (count > 0 && !reqs) || count > (1ll << 31) - 1) return ACC_ERR_INVALID;
  int nt = BT;
  if (nt_override > 0) {
    if (!valid_nt(nt_override)) return ACC_ERR_INVALID;
    nt = nt_override;
  } else {
    double weight[3] = {0.0, 0.0, 0.0};
    for (int64_t i = 0; i < count; ++i) {
      const acc_request &q = reqs[i];
      if (q.type != ACC_I32 && q.type != ACC_I64 && q.type != ACC_F32 && q.type != ACC_F64) continue;
      const int v = tuned(q.kind, q.type, q.n).nt;
      for (int c = 0; c < 3; ++c)
        if (B_NT[c] == v) weight[c] += (double)(q.n > 0 ? q.n : 0) * type_bytes(q.type);
    }
    if (weight[0] > weight[1] && weight[0] >= weight[2]) nt = B_NT[0];
    else if (weight[2] > weight[1] && weight[2] > weight[0]) nt = B_NT[2];
  }
  std::vector<BReq> h(count);
  std::vector<int32_t> item_req;
  int64_t nitems = 0;
  size_t max_tile = 0;
  for (int64_t i = 0; i < count; ++i) {
    const acc_request &q = reqs[i];
    if (q.kind != ACC_REQ_FOLD && q.kind != ACC_REQ_SCAN) return ACC_ERR_INVALID;
    if (q.type != ACC_I32 && q.type != ACC_I64 && q.type != ACC_F32 && q.type != ACC_F64) return ACC_ERR_UNSUPPORTED;
    if (q.n < 0 || (q.n > 0 && (!q.in || !q.out))) return ACC_ERR_INVALID;
    if (q.kind == ACC_REQ_FOLD && !q.out) return ACC_ERR_INVALID;  // fold z [] still writes z
    if (q.kind == ACC_REQ_FOLD && q.n == 0 && !q.has_seed) return ACC_ERR_EMPTY;
    const int ipt = ipt_override ? norm_ipt(ipt_override[i], q.type, nt) : ipt_for(q, nt);
    const int64_t ts = (int64_t)ipt * nt;
    int64_t ntl = (q.n + ts - 1) / ts;
    if (q.kind == ACC_REQ_FOLD && ntl == 0) ntl = 1;  // fold z [] = z: one (empty) tile writes the seed
    BReq &r = h[i];
    r.in = q.in; r.out = q.out; r.n = q.n; r.seed = q.seed;
    r.kind = q.kind; r.type = q.type; r.has_seed = q.has_seed; r.ipt = ipt;
    r.first_item = nitems; r.ntiles = ntl;
    for (int64_t k = 0; k < ntl; ++k) item_req.push_back((int32_t)i);
    nitems += ntl;
    const size_t tb = (size_t)(ipt + 1) * nt * type_bytes(q.type) + 256;
    if (tb > max_tile) max_tile = tb;
  }
  if (nitems >= (1ll << 31)) return ACC_ERR_TOO_LARGE;
  Batch *b = new Batch();
  b->op = op;
  b->nt = nt;
  cudaGetDevice(&b->device);
  b->count = count;
  b->nitems = nitems;
  b->smem = max_tile < 1024 ? 1024 : max_tile;
  auto fail = [&](cudaError_t e) { batch_free(b); return cuda_status(e); };
  cudaError_t e;
  if ((e = cudaMalloc(&b->d_reqs, sizeof(BReq) * (count ? count : 1))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&b->d_item_req, sizeof(int32_t) * (nitems ? nitems : 1))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&b->d_status, sizeof(uint64_t) * 2 * (nitems ? nitems : 1))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&b->d_partials, sizeof(uint64_t) * (nitems ? nitems : 1))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&b->d_req_ticket, sizeof(uint32_t) * (count ? count : 1))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&b->d_words, sizeof(uint32_t) * 64)) != cudaSuccess) return fail(e);
  if (count) cudaMemcpy(b->d_reqs, h.data(), sizeof(BReq) * count, cudaMemcpyHostToDevice);
  if (nitems) cudaMemcpy(b->d_item_req, item_req.data(), sizeof(int32_t) * nitems, cudaMemcpyHostToDevice);
  cudaMemset(b->d_status, 0, sizeof(uint64_t) * 2 * (nitems ? nitems : 1));
  cudaMemset(b->d_req_ticket, 0, sizeof(uint32_t) * (count ? count : 1));
  cudaMemset(b->d_words, 0, sizeof(uint32_t) * 64);
  void *kern = kernel_for(op, nt);
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem);
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nt, b->smem) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  int64_t grid = (int64_t)device_info().sms * per_sm;
  if (grid > nitems) grid = nitems > 0 ? nitems : 1;
  b->grid = (int)grid;
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return fail(e);
  *out = b;
  return ACC_OK;
}

// ---------------------------------------------------------------- arena
// A reusable launch area for batches assembled on the fly (the serving
// loop): device arrays sized once for up to cap_reqs requests / cap_items
// tiles, pinned host staging for the descriptors.  A launch copies the new
// descriptors with cudaMemcpyAsync and runs the kernel; it allocates nothing.
// One arena serves one stream at a time: its staging buffers are reused only
// after the previous launch from the arena has completed.
struct BatchArena {
  Batch dev;            // device arrays and launch shape (count/nitems per launch)
  int64_t cap_reqs = 0, cap_items = 0;
  BReq *h_reqs = nullptr;
  int32_t *h_item = nullptr;
};

int arena_create(int op, int64_t cap_reqs, int64_t cap_items, BatchArena **out) {
  if (op != ACC_ADD && op != ACC_MIN && op != ACC_MAX) return ACC_ERR_UNSUPPORTED;
  BatchArena *ar = new BatchArena();
  Batch *b = &ar->dev;
  b->op = op;
  cudaGetDevice(&b->device);
  ar->cap_reqs = cap_reqs;
  ar->cap_items = cap_items;
  cudaError_t e;
  if ((e = cudaMalloc(&b->d_reqs, sizeof(BReq) * cap_reqs)) != cudaSuccess ||
      (e = cudaMalloc(&b->d_item_req, sizeof(int32_t) * cap_items)) != cudaSuccess ||
      (e = cudaMalloc(&b->d_status, sizeof(uint64_t) * 2 * cap_items)) != cudaSuccess ||
      (e = cudaMalloc(&b->d_partials, sizeof(uint64_t) * cap_items)) != cudaSuccess ||
      (e = cudaMalloc(&b->d_req_ticket, sizeof(uint32_t) * cap_reqs)) != cudaSuccess ||
      (e = cudaMalloc(&b->d_words, sizeof(uint32_t) * 64)) != cudaSuccess ||
      (e = cudaMallocHost(&ar->h_reqs, sizeof(BReq) * cap_reqs)) != cudaSuccess ||
      (e = cudaMallocHost(&ar->h_item, sizeof(int32_t) * cap_items)) != cudaSuccess) {
    arena_free(ar);
    return cuda_status(e);
  }
  cudaMemset(b->d_status, 0, sizeof(uint64_t) * 2 * cap_items);
  cudaMemset(b->d_req_ticket, 0, sizeof(uint32_t) * cap_reqs);
  cudaMemset(b->d_words, 0, sizeof(uint32_t) * 64);
  b->smem = (size_t)B_MAX_TILE_BYTES + BT * 8 + 256;
  b->nt = BT;
  void *kern = kernel_for(op, BT);
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem);
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, BT, b->smem) != cudaSuccess || per_sm < 1) {
    cudaGetLastError();
    per_sm = 1;
  }
  b->grid = device_info().sms * per_sm;
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) { arena_free(ar); return cuda_status(e); }
  *out = ar;
  return ACC_OK;
}

// Tiles a request will take (0 if it does not fit the batch kernel).
int64_t arena_tiles(const acc_request &q) {
  const int ipt = ipt_for(q, BT);
  const int64_t ts = (int64_t)ipt * BT;
  const int64_t nt = (q.n + ts - 1) / ts;
  return (q.kind == ACC_REQ_FOLD && nt == 0) ? 1 : nt;
}

int arena_launch(BatchArena *ar, const acc_request *reqs, int64_t count, cudaStream_t s) {
  Batch *b = &ar->dev;
  int64_t nitems = 0;
  for (int64_t i = 0; i < count; ++i) {
    const acc_request &q = reqs[i];
    const int ipt = ipt_for(q, BT);
    const int64_t ts = (int64_t)ipt * BT;
    int64_t nt = (q.n + ts - 1) / ts;
    if (q.kind == ACC_REQ_FOLD && nt == 0) nt = 1;
    if (i >= ar->cap_reqs || nitems + nt > ar->cap_items) return ACC_ERR_TOO_LARGE;
    BReq &r = ar->h_reqs[i];
    r.in = q.in; r.out = q.out; r.n = q.n; r.seed = q.seed;
    r.kind = q.kind; r.type = q.type; r.has_seed = q.has_seed; r.ipt = ipt;
    r.first_item = nitems; r.ntiles = nt;
    for (int64_t k = 0; k < nt; ++k) ar->h_item[nitems + k] = (int32_t)i;
    nitems += nt;
  }
  if (nitems == 0) return ACC_OK;
  cudaError_t e = cudaMemcpyAsync(b->d_reqs, ar->h_reqs, sizeof(BReq) * count, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b->d_item_req, ar->h_item, sizeof(int32_t) * nitems, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_status(e);
  b->count = count;
  b->nitems = nitems;
  const int full_grid = b->grid;
  if (b->grid > nitems) b->grid = (int)nitems;
  const int st = batch_launch_raw(b, s);
  b->grid = full_grid;
  return st;
}

void arena_free(BatchArena *ar) {
  if (!ar) return;
  Batch *b = &ar->dev;
  cudaFree(b->d_reqs);
  cudaFree(b->d_item_req);
  cudaFree(b->d_status);
  cudaFree(b->d_partials);
  cudaFree(b->d_req_ticket);
  cudaFree(b->d_words);
  cudaFreeHost(ar->h_reqs);
  cudaFreeHost(ar->h_item);
  delete ar;
}

// ---------------------------------------------------------------- autotune
static int autotune_run(int kind, int type, int bucket, cudaStream_t s, void *buf, size_t buf_bytes, TuneVal *best) {
  const int64_t n = int64_t(1) << bucket;
  const int eb = type_bytes(type);
  // A batch of equal requests of this bucket's size, up to 2^24 elements in all.
  int64_t count = std::max<int64_t>(1, std::min<int64_t>(4096, (int64_t(1) << 24) / n));
  while (count > 1 && (size_t)(count * n * eb * 2 + count * 8) > buf_bytes) count /= 2;
  std::vector<acc_request> reqs(count);
  char *base = static_cast<char *>(buf);
  for (int64_t i = 0; i < count; ++i) {
    acc_request &q = reqs[i];
    q.kind = kind; q.type = type; q.n = n; q.has_seed = 0; q.seed = 0;
    q.in = base;                                  // all requests read the same input
    q.out = base + (size_t)n * eb + (kind == ACC_REQ_SCAN ? (size_t)i * n * eb : (size_t)i * eb);
  }
  float best_ms = 1e30f;
  TuneVal pick{default_ipt(kind, type, n), BT};
  // every launch shape, and for each every tile shape
  for (int nt : B_NT) {
    for (int ipt = 1; ipt <= max_ipt(type, nt); ipt *= 2) {
      std::vector<int32_t> ov(count, ipt);
      Batch *b = nullptr;
      int st = batch_make(ACC_ADD, reqs.data(), count, ov.data(), nt, &b);
      if (st) return st;
      cudaEvent_t e0, e1;
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      batch_launch_raw(b, s);
      cudaEventRecord(e0, s);
      for (int rep = 0; rep < 3; ++rep) batch_launch_raw(b, s);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      batch_free(b);
      if (ms < best_ms) { best_ms = ms; pick = TuneVal{ipt, nt}; }
    }
  }
  *best = pick;
  return check_launch();
}

}  // namespace accgb

using namespace accgb;

extern "C" int acc_batch_create(int op, const acc_request *reqs, int64_t count, acc_batch **out) {
  if (!out) return ACC_ERR_INVALID;
  Batch *b = nullptr;
  int st = batch_make(op, reqs, count, nullptr, 0, &b);
  if (st) return st;
  *out = reinterpret_cast<acc_batch *>(b);
  return ACC_OK;
}

extern "C" int acc_batch_launch(acc_batch *batch, void *stream) {
  Batch *b = reinterpret_cast<Batch *>(batch);
  if (!b) return ACC_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (b->nitems == 0) return ACC_OK;
  if (b->exec) return cuda_status(cudaGraphLaunch(b->exec, s));
  return batch_launch_raw(b, s);
}

extern "C" int acc_batch_capture(acc_batch *batch, void *stream) {
  Batch *b = reinterpret_cast<Batch *>(batch);
  if (!b) return ACC_ERR_INVALID;
  if (b->exec || b->nitems == 0) return ACC_OK;
  (void)stream;  // captured on a private stream; replays go to the launch's stream
  cudaStream_t cap = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_status(e);
  e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    batch_launch_raw(b, cap);
    e = cudaStreamEndCapture(cap, &b->graph);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
  cudaStreamDestroy(cap);
  return cuda_status(e);
}

extern "C" int acc_batch_status(acc_batch *batch, void *stream) {
  Batch *b = reinterpret_cast<Batch *>(batch);
  if (!b) return ACC_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e);
  uint32_t err = 0;
  e = cudaMemcpy(&err, b->d_words, sizeof(uint32_t), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e);
  if (!err) return ACC_OK;
  cudaMemset(b->d_words, 0, sizeof(uint32_t) * 64);
  cudaMemset(b->d_status, 0, sizeof(uint64_t) * 2 * (b->nitems ? b->nitems : 1));
  cudaMemset(b->d_req_ticket, 0, sizeof(uint32_t) * (b->count ? b->count : 1));
  return ACC_ERR_TIMEOUT;
}

extern "C" int acc_batch_destroy(acc_batch *batch) {
  Batch *b = reinterpret_cast<Batch *>(batch);
  if (b) {
    cudaDeviceSynchronize();
    batch_free(b);
  }
  return ACC_OK;
}

extern "C" int acc_batch_autotune(const char *table_path, void *stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t buf_bytes = (size_t)1 << 28;
  void *buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, buf_bytes);
  if (e != cudaSuccess) return cuda_status(e);
  cudaMemset(buf, 0, buf_bytes);
  std::map<TuneKey, TuneVal> table;
  const int kinds[2] = {ACC_REQ_FOLD, ACC_REQ_SCAN};
  const int types[4] = {ACC_I32, ACC_F32, ACC_I64, ACC_F64};
  int st = ACC_OK;
  for (int kind : kinds)
    for (int type : types)
      for (int bucket = 8; bucket <= 22 && st == ACC_OK; ++bucket) {
        TuneVal best{0, BT};
        st = autotune_run(kind, type, bucket, s, buf, buf_bytes, &best);
        if (st == ACC_OK) table[TuneKey{kind, type, bucket}] = best;
      }
  cudaFree(buf);
  if (st) return st;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (auto &kv : table) g_tune[kv.first] = kv.second;
  }
  if (table_path) {
    FILE *f = fopen(table_path, "w");
    if (!f) return ACC_ERR_INVALID;
    cudaDeviceProp p;
    cudaGetDeviceProperties(&p, 0);
    // entries: [kind, type, log2 size bucket, elements per thread, threads per CTA]
    fprintf(f, "{\"gpu\": \"%s\", \"entries\": [", p.name);
    bool first = true;
    for (auto &kv : table) {
      fprintf(f, "%s[%d, %d, %d, %d, %d]", first ? "" : ", ", kv.first.kind, kv.first.type, kv.first.bucket,
              kv.second.ipt, kv.second.nt);
      first = false;
    }
    fprintf(f, "]}\n");
    fclose(f);
  }
  return ACC_OK;
}

extern "C" int acc_batch_load_tuning(const char *table_path) {
  if (!table_path) return ACC_ERR_INVALID;
  FILE *f = fopen(table_path, "r");
  if (!f) return ACC_ERR_INVALID;
  std::string text;
  char chunk[4096];
  size_t got;
  while ((got = fread(chunk, 1, sizeof(chunk), f)) > 0) text.append(chunk, got);
  fclose(f);
  const size_t at = text.find("\"entries\"");
  if (at == std::string::npos) return ACC_ERR_INVALID;
  // entries of five numbers, or of four (tables written before the launch
  // shape was tuned: 256 threads per CTA)
  std::map<TuneKey, TuneVal> table;
  const char *p = text.c_str() + at;
  while ((p = strchr(p, '[')) != nullptr) {
    int kind, type, bucket, ipt, nt = BT;
    const int got5 = sscanf(p, "[%d, %d, %d, %d, %d]", &kind, &type, &bucket, &ipt, &nt);
    if (got5 >= 4) {
      if (got5 == 4) nt = BT;
      if (!valid_nt(nt)) return ACC_ERR_INVALID;
      table[TuneKey{kind, type, bucket}] = TuneVal{ipt, nt};
    }
    ++p;
  }
  std::lock_guard<std::mutex> lk(g_tune_mu);
  for (auto &kv : table) g_tune[kv.first] = kv.second;
  return ACC_OK;
}
