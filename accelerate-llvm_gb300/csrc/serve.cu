// serve.cu -- continuous-batching serving loop over the skeleton library.
//
// acc_serve_run plays a stream of requests (each with an arrival time) through
// one of two schedulers and returns every request's latency:
//   mode 0, continuous batching: up to `slots` CUDA streams work at once.  At
//     every turn of the loop the requests that have arrived join the ready
//     queue; each free slot takes either ALL ready small fold / scanl1
//     requests that fit (packed into one persistent batched launch from the
//     slot's preallocated batch arena) or the next other request (foldSeg,
//     permute, stencil, large fold / scan) as a single call.  Slots free up
//     as their completion events fire, so new arrivals join while earlier
//     work is still on the GPU.
//   mode 1, plain per-call: every request is launched on its own, in arrival
//     order, on one stream (the reference's execution model, one launch per
//     skeleton, PTX/Execute.hs:835-881).
// Admission by device memory, in both modes: a request without an output
// buffer (out == NULL) gets its result space from one device arena of
// `budget_bytes`, allocated before the clock starts, and is admitted only once
// that space is free (best fit; the range returns when the request
// completes); a request with its own output buffer is admitted while the
// bytes of input and output held by such requests stay within the budget.
// A request with a host buffer (host_out) has its result copied back to it
// before it counts as complete.  Latency = the host time at which the
// request's completion event is seen minus its arrival time.  Nothing is
// allocated per request: arenas, events and streams are made before the
// clock starts.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <thread>
#include <vector>

#include "common.cuh"

namespace accgb {

namespace {

constexpr int64_t SERVE_BATCH_MAX_N = 1 << 22;  // larger fold / scan requests run alone
constexpr int64_t ARENA_REQS = 1024;
constexpr int64_t ARENA_ITEMS = 1 << 17;

int64_t esize(int type) { return (type == ACC_I64 || type == ACC_F64) ? 8 : 4; }

constexpr int64_t SERVE_ALIGN = 256;

// Bytes of a request's result.
int64_t out_bytes(const acc_serve_req &q) {
  switch (q.skeleton) {
    case ACC_SK_FOLD: return esize(q.type);
    case ACC_SK_SCAN: return q.n * esize(q.type);
    case ACC_SK_FOLDSEG: return q.m * esize(q.type);
    case ACC_SK_PERMUTE: return q.m * 4;
    default: return q.n * q.m * esize(q.type);
  }
}

int64_t held_bytes(const acc_serve_req &q) {
  const int64_t e = esize(q.type);
  switch (q.skeleton) {
    case ACC_SK_FOLD: return q.n * e + e;
    case ACC_SK_SCAN: return 2 * q.n * e;
    case ACC_SK_FOLDSEG: return q.n * e + (q.m + 1) * 4 + q.m * e;
    case ACC_SK_PERMUTE: return q.n * 4 + q.m * 4;
    default: return 2 * q.n * q.m * e;
  }
}

bool batchable(const acc_serve_req &q) {
  return (q.skeleton == ACC_SK_FOLD || q.skeleton == ACC_SK_SCAN) && q.n <= SERVE_BATCH_MAX_N &&
         (q.type == ACC_I32 || q.type == ACC_I64 || q.type == ACC_F32 || q.type == ACC_F64);
}

acc_request as_batch_request(const acc_serve_req &q) {
  acc_request r{};
  r.kind = q.skeleton == ACC_SK_FOLD ? ACC_REQ_FOLD : ACC_REQ_SCAN;
  r.type = q.type;
  r.in = q.in;
  r.out = q.out;
  r.n = q.n;
  r.has_seed = q.skeleton == ACC_SK_FOLD;  // fold (+) 0
  r.seed = 0;
  return r;
}

const float kFivePointF32[9] = {0.f, 0.25f, 0.f, 0.25f, -1.f, 0.25f, 0.f, 0.25f, 0.f};
const double kFivePointF64[9] = {0., 0.25, 0., 0.25, -1., 0.25, 0., 0.25, 0.};

// One request as a single call on `s`.
int run_single(const acc_serve_req &q, cudaStream_t s) {
  void *sp = static_cast<void *>(s);
  uint64_t zero = 0;
  switch (q.skeleton) {
    case ACC_SK_FOLD: return acc_fold(ACC_ADD, q.type, ACC_PREC_DEFAULT, q.in, q.out, 1, q.n, &zero, sp);
    case ACC_SK_SCAN:
      return acc_scan(ACC_ADD, q.type, ACC_PREC_DEFAULT, ACC_L2R, ACC_SCAN_INCLUSIVE, q.in, q.out, nullptr, 1, q.n,
                      nullptr, sp);
    case ACC_SK_FOLDSEG:
      return acc_fold_seg(ACC_ADD, q.type, ACC_PREC_DEFAULT, q.in, q.aux, ACC_I32, q.out, 1, q.n, q.m, &zero, sp);
    case ACC_SK_PERMUTE: {
      cudaError_t e = cudaMemsetAsync(q.out, 0, (size_t)q.m * 4, s);
      if (e != cudaSuccess) return cuda_status(e);
      const int32_t one = 1;
      return acc_permute(ACC_ADD, ACC_I32, nullptr, &one, q.in, ACC_I32, q.out, q.n, q.m, sp);
    }
    case ACC_SK_STENCIL:
      return acc_stencil2d(q.type, 1, 1, q.type == ACC_F64 ? (const void *)kFivePointF64 : (const void *)kFivePointF32,
                           ACC_CLAMP, nullptr, q.in, q.out, q.n, q.m, sp);
    default: return ACC_ERR_INVALID;
  }
}

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  BatchArena *arena = nullptr;
  std::vector<int64_t> ids;
  bool busy = false;
};

using Clock = std::chrono::steady_clock;

}  // namespace
}  // namespace accgb

using namespace accgb;

extern "C" int acc_serve_run(const acc_serve_req *reqs, int64_t count, int64_t budget_bytes, int slots, int mode,
                             double *latency, acc_serve_stats *stats) {
  if (count < 0 || (count > 0 && (!reqs || !latency)) || slots < 1 || slots > 64 || (mode != 0 && mode != 1))
    return ACC_ERR_INVALID;
  for (int64_t i = 0; i < count; ++i) {
    const acc_serve_req &q = reqs[i];
    if (q.skeleton < ACC_SK_FOLD || q.skeleton > ACC_SK_STENCIL || q.n < 0 || q.m < 0) return ACC_ERR_INVALID;
    if (q.type < ACC_I32 || q.type > ACC_F64) return ACC_ERR_INVALID;
    // The 5-point weights (0.25, -1) are real numbers: Float32 / Float64 grids only.
    if (q.skeleton == ACC_SK_STENCIL && q.type != ACC_F32 && q.type != ACC_F64) return ACC_ERR_UNSUPPORTED;
    // Every buffer the request reads or writes must be given: a null address
    // would otherwise reach the device.
    const int64_t nin = q.skeleton == ACC_SK_STENCIL ? q.n * q.m : q.n;
    const int64_t nout = q.skeleton == ACC_SK_FOLD      ? 1
                         : q.skeleton == ACC_SK_SCAN    ? q.n
                         : q.skeleton == ACC_SK_STENCIL ? q.n * q.m
                                                        : q.m;
    (void)nout;
    if ((nin > 0 && !q.in) || (q.skeleton == ACC_SK_FOLDSEG && q.m > 0 && !q.aux)) return ACC_ERR_INVALID;
    if (i > 0 && q.arrival < reqs[i - 1].arrival) return ACC_ERR_INVALID;  // arrival order
    // A result placed in the arena takes its size rounded up to SERVE_ALIGN
    // out of an arena of the budget rounded down to SERVE_ALIGN.
    const int64_t placed_bytes = (out_bytes(q) + SERVE_ALIGN - 1) / SERVE_ALIGN * SERVE_ALIGN;
    if (q.out ? held_bytes(q) > budget_bytes : placed_bytes > budget_bytes / SERVE_ALIGN * SERVE_ALIGN)
      return ACC_ERR_TOO_LARGE;
    latency[i] = -1.0;
  }
  if (mode == 1) slots = 1;
  // The requests' inputs were produced on the caller's streams; the serving
  // streams are independent of those, so wait for the device to finish them.
  cudaError_t e0 = cudaDeviceSynchronize();
  if (e0 != cudaSuccess) return cuda_status(e0);
  // The result arena (only if some request leaves its output to the loop).
  unsigned char *arena = nullptr;
  RangeAlloc ranges;
  bool need_arena = false;
  for (int64_t i = 0; i < count; ++i) need_arena = need_arena || !reqs[i].out;
  if (need_arena) {
    const int64_t cap = budget_bytes / SERVE_ALIGN * SERVE_ALIGN;
    e0 = cudaMalloc(&arena, (size_t)cap);
    if (e0 != cudaSuccess) return cuda_status(e0);
    ranges.give(0, cap);
  }
  std::vector<int64_t> out_off(count, -1);
  int64_t used = 0, arena_used = 0, peak = 0;
  auto rounded = [](int64_t b) { return (b + SERVE_ALIGN - 1) / SERVE_ALIGN * SERVE_ALIGN; };
  // Take what request id holds while it is on the GPU; false: not now.
  auto admit = [&](int64_t id) -> bool {
    const acc_serve_req &q = reqs[id];
    if (q.out) {
      const int64_t hb = held_bytes(q);
      if (used + hb > budget_bytes) return false;
      used += hb;
    } else {
      const int64_t b = rounded(out_bytes(q));
      int64_t off = 0;
      if (b > 0 && !ranges.take(b, &off)) return false;
      out_off[id] = off;
      arena_used += b;
    }
    if (used + arena_used > peak) peak = used + arena_used;
    return true;
  };
  auto release = [&](int64_t id) {
    const acc_serve_req &q = reqs[id];
    if (q.out) {
      used -= held_bytes(q);
    } else if (out_off[id] >= 0) {
      const int64_t b = rounded(out_bytes(q));
      if (b > 0) ranges.give(out_off[id], b);
      arena_used -= b;
      out_off[id] = -1;
    }
  };
  // The request as launched: its own output, or its range of the arena.
  auto placed = [&](int64_t id) {
    acc_serve_req q = reqs[id];
    if (!q.out) q.out = arena + out_off[id];
    return q;
  };
  // Launch request id alone on stream s (its result copied back if asked).
  auto launch_one = [&](int64_t id, cudaStream_t s) -> int {
    const acc_serve_req q = placed(id);
    int r = run_single(q, s);
    if (r == ACC_OK && q.host_out) r = acc_download(q.host_out, q.out, out_bytes(q), s);
    return r;
  };
  std::vector<Slot> sl(slots);
  int st = ACC_OK;
  for (auto &s : sl) {
    cudaError_t e = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming);
    if (e != cudaSuccess) { st = cuda_status(e); break; }
    if (mode == 0 && (st = arena_create(ACC_ADD, ARENA_REQS, ARENA_ITEMS, &s.arena)) != ACC_OK) break;
  }
  // Per-call mode keeps a ring of events, one per request in flight.
  std::vector<cudaEvent_t> ring(mode == 1 ? 4096 : 0);
  for (auto &ev : ring)
    if (st == ACC_OK) {
      cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
      if (e != cudaSuccess) st = cuda_status(e);
    }
  // Warm every path once (first launches load modules and size workspaces).
  if (st == ACC_OK) {
    // Each request is admitted at most once here (its result range is taken
    // once and given back once, after the device is done with it).
    std::vector<int64_t> warm;
    for (int64_t i = 0; i < count && i < 64 && st == ACC_OK; ++i) {
      if (!admit(i)) continue;
      warm.push_back(i);
      st = run_single(placed(i), sl[0].stream);
    }
    for (int64_t i = 0; i < count && mode == 0 && st == ACC_OK; ++i) {
      if (!batchable(reqs[i])) continue;
      const bool held = i < 64 && std::find(warm.begin(), warm.end(), i) != warm.end();
      if (!held) {
        if (!admit(i)) continue;
        warm.push_back(i);
      }
      const acc_request br = as_batch_request(placed(i));
      for (auto &s : sl)
        if (st == ACC_OK) st = arena_launch(s.arena, &br, 1, s.stream);
      break;
    }
    for (auto &s : sl) cudaStreamSynchronize(s.stream);
    for (int64_t id : warm) release(id);
    peak = 0;
    if (st == ACC_OK) st = acc_sync(sl[0].stream);
  }
  int64_t served = 0, batches = 0, max_inflight = 0, inflight = 0;
  const Clock::time_point t0 = Clock::now();
  auto now_s = [&]() { return std::chrono::duration<double>(Clock::now() - t0).count(); };
  if (st == ACC_OK && mode == 0) {
    std::deque<int64_t> ready;
    std::vector<acc_request> pack;
    pack.reserve(ARENA_REQS);
    int64_t next = 0;
    while (served < count && st == ACC_OK) {
      bool progress = false;
      const double t = now_s();
      while (next < count && reqs[next].arrival <= t) ready.push_back(next++);
      for (auto &s : sl) {
        if (!s.busy) continue;
        const cudaError_t q = cudaEventQuery(s.done);
        if (q != cudaSuccess && q != cudaErrorNotReady) {
          st = cuda_status(q);  // the device failed: stop serving
          break;
        }
        if (q == cudaSuccess) {
          const double tc = now_s();
          for (int64_t id : s.ids) {
            latency[id] = tc - reqs[id].arrival;
            release(id);
          }
          served += (int64_t)s.ids.size();
          inflight -= (int64_t)s.ids.size();
          s.ids.clear();
          s.busy = false;
          progress = true;
        }
      }
      if (st != ACC_OK) break;
      for (auto &s : sl) {
        if (s.busy || ready.empty()) continue;
        const acc_serve_req &head = reqs[ready.front()];
        if (batchable(head)) {
          // Pack every ready small fold / scan that fits the memory budget
          // and the batch arena.
          pack.clear();
          int64_t items = 0;
          for (auto it = ready.begin(); it != ready.end() && (int64_t)pack.size() < ARENA_REQS;) {
            const acc_serve_req &q = reqs[*it];
            if (!batchable(q)) { ++it; continue; }
            const int64_t nt = arena_tiles(as_batch_request(q));
            if (items + nt > ARENA_ITEMS) break;
            if (!admit(*it)) { ++it; continue; }
            items += nt;
            pack.push_back(as_batch_request(placed(*it)));
            s.ids.push_back(*it);
            it = ready.erase(it);
          }
          if (pack.empty()) break;
          st = arena_launch(s.arena, pack.data(), (int64_t)pack.size(), s.stream);
          for (size_t k = 0; k < s.ids.size() && st == ACC_OK; ++k) {
            const acc_serve_req q = placed(s.ids[k]);
            if (q.host_out) st = acc_download(q.host_out, q.out, out_bytes(q), s.stream);
          }
          ++batches;
        } else {
          if (!admit(ready.front())) break;  // wait for memory to free up
          s.ids.push_back(ready.front());
          ready.pop_front();
          st = launch_one(s.ids.back(), s.stream);
        }
        if (st != ACC_OK) break;
        cudaEventRecord(s.done, s.stream);
        s.busy = true;
        inflight += (int64_t)s.ids.size();
        if (inflight > max_inflight) max_inflight = inflight;
        if (used > peak) peak = used;
        progress = true;
      }
      if (!progress) std::this_thread::yield();
    }
  } else if (st == ACC_OK) {
    // Per-call FIFO: launch each request when it arrives, one stream, one launch each.
    cudaStream_t s = sl[0].stream;
    std::deque<int64_t> pending;  // launched, not yet complete (ring slot = id % ring size)
    int64_t next = 0;
    while (served < count && st == ACC_OK) {
      bool progress = false;
      while (!pending.empty()) {
        const cudaError_t q = cudaEventQuery(ring[pending.front() % ring.size()]);
        if (q != cudaSuccess && q != cudaErrorNotReady) {
          st = cuda_status(q);  // the device failed: stop serving
          break;
        }
        if (q != cudaSuccess) break;
        const int64_t id = pending.front();
        pending.pop_front();
        latency[id] = now_s() - reqs[id].arrival;
        release(id);
        ++served;
        progress = true;
      }
      if (st != ACC_OK) break;
      const double t = now_s();
      while (next < count && reqs[next].arrival <= t && (int64_t)pending.size() < (int64_t)ring.size() &&
             admit(next)) {
        st = launch_one(next, s);
        if (st != ACC_OK) break;
        cudaEventRecord(ring[next % ring.size()], s);
        pending.push_back(next++);
        if ((int64_t)pending.size() > max_inflight) max_inflight = (int64_t)pending.size();
        progress = true;
      }
      if (!progress) std::this_thread::yield();
    }
  }
  const double wall = now_s();
  for (auto &s : sl) {
    if (s.stream) cudaStreamSynchronize(s.stream);
  }
  if (st == ACC_OK && !sl.empty()) {
    for (auto &s : sl) {
      const int e = acc_sync(s.stream);
      if (e != ACC_OK) st = e;
    }
  }
  for (auto &s : sl) {
    if (s.arena) arena_free(s.arena);
    if (s.done) cudaEventDestroy(s.done);
    if (s.stream) cudaStreamDestroy(s.stream);
  }
  for (auto &ev : ring)
    if (ev) cudaEventDestroy(ev);
  if (arena) cudaFree(arena);
  if (stats) {
    stats->wall_s = wall;
    stats->served = served;
    stats->batches = batches;
    stats->max_inflight = max_inflight;
    stats->peak_bytes = peak;
  }
  return st;
}
