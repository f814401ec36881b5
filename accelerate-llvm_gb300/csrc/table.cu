// table.cu -- host <-> device transfers and the memory table.
//
// The reference keeps device copies of host arrays in an LRU memory table
// (PTX/Array/Table.hs:35-49, Remote.malloc / withRemote in
// PTX/Array/Remote.hs:60-133), allocates them with cuMemAlloc per array and
// moves data with cuMemcpy{HtoD,DtoH}Async on the op's stream
// (useArrayAsync / pokeArrayAsync / peekArrayAsync, PTX/Array/Prim.hs:72-195).
//
// Here, for GB300:
//   * Device memory for a table is ONE arena of a fixed budget, allocated
//     when the table is made; arrays take 4 KiB-aligned ranges of it
//     (best fit, neighbours coalesced on free), so no call on the data path
//     allocates or frees device memory.
//   * Every transfer runs on one of the table's two streams (uploads,
//     downloads), ordered against the caller's stream by events, so that
//     uploads, kernels and downloads overlap on the host link (a GB300 moves
//     host->device and device->host at the same time, ~340 GB/s together).
//   * Pinned host memory goes through the copy engines.  Plain pageable
//     memory, which the GPU reads and writes through the host's page tables
//     over NVLink-C2C at the full link rate, is moved by a copy kernel: fully
//     asynchronous, no staging buffer, no pinning (a pageable cudaMemcpyAsync
//     would block the calling thread).
//   * Eviction is stream-ordered: an evicted array's range returns to the free
//     list only once its last user and its copy back (if the device wrote it)
//     have completed; the host waits only when nothing else fits.
#include <deque>
#include <map>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "runtime.h"

struct acc_table;

namespace accgb {
namespace {

constexpr int XF_THREADS = 512;
constexpr int64_t TABLE_ALIGN = 4096;        // the reference's remoteAllocationSize
constexpr int64_t TABLE_ARENA_ROUND = 2 << 20;

// Copy `bytes` between any two addresses this GPU can reach (device memory,
// pinned or pageable host memory).  Same 16-byte phase: byte head, 16-byte
// body with four loads in flight per thread, byte tail; otherwise bytes.
__global__ void __launch_bounds__(XF_THREADS)
xfer_kernel(const unsigned char *__restrict__ src, unsigned char *__restrict__ dst, int64_t bytes) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  const uintptr_t sa = reinterpret_cast<uintptr_t>(src), da = reinterpret_cast<uintptr_t>(dst);
  if (((sa ^ da) & 15u) == 0) {
    int64_t head = (int64_t)((16u - (sa & 15u)) & 15u);
    if (head > bytes) head = bytes;
    const int64_t n16 = (bytes - head) >> 4;
    const int64_t tail0 = head + (n16 << 4);
    if (tid < head) dst[tid] = src[tid];
    if (tid < bytes - tail0) dst[tail0 + tid] = src[tail0 + tid];
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src + head);
    uint4 *d4 = reinterpret_cast<uint4 *>(dst + head);
    int64_t i = tid;
    for (; i + 3 * nthr < n16; i += 4 * nthr) {
      const uint4 a = s4[i], b = s4[i + nthr], c = s4[i + 2 * nthr], d = s4[i + 3 * nthr];
      d4[i] = a;
      d4[i + nthr] = b;
      d4[i + 2 * nthr] = c;
      d4[i + 3 * nthr] = d;
    }
    for (; i < n16; i += nthr) d4[i] = s4[i];
  } else {
    for (int64_t i = tid; i < bytes; i += nthr) dst[i] = src[i];
  }
}

// Whether the current device reads pageable host memory directly
// (cudaDevAttrPageableMemoryAccess), cached per device.
bool pageable_access() {
  static std::mutex mu;
  static int known[64] = {};  // 0 unknown, 1 no, 2 yes
  const Device &d = device_info();
  std::lock_guard<std::mutex> lk(mu);
  if (!known[d.id]) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, d.id) != cudaSuccess) {
      cudaGetLastError();
      v = 0;
    }
    known[d.id] = v ? 2 : 1;
  }
  return known[d.id] == 2;
}

// Copy between `host` (host memory of any kind) and `dev` on stream s:
// the copy engines for pinned memory, the copy kernel for pageable memory
// the GPU can reach, else the driver's staged copy.
int host_copy(void *dst, const void *src, const void *host, int64_t bytes, cudaStream_t s) {
  if (bytes <= 0) return ACC_OK;
  cudaPointerAttributes at{};
  bool pageable = false;
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
    cudaGetLastError();
    pageable = true;
  } else {
    pageable = at.type == cudaMemoryTypeUnregistered;
  }
  if (pageable && pageable_access()) {
    const int64_t per_cta = (int64_t)XF_THREADS * 16 * 4;
    int64_t grid = (bytes + per_cta - 1) / per_cta;
    const int64_t cap = device_info().sms;
    if (grid > cap) grid = cap;
    if (grid < 1) grid = 1;
    xfer_kernel<<<(unsigned)grid, XF_THREADS, 0, s>>>(static_cast<const unsigned char *>(src),
                                                      static_cast<unsigned char *>(dst), bytes);
    return check_launch();
  }
  return cuda_status(cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDefault, s));
}

}  // namespace
}  // namespace accgb

using namespace accgb;

// ------------------------------------------------------------------ table
struct acc_table {
  struct Entry {
    const void *host = nullptr;
    int64_t bytes = 0, off = 0, cap = 0;
    bool dirty = false;
    int holds = 0;
    uint64_t tick = 0;
    cudaEvent_t last_use = nullptr;  // recorded by release
    cudaEvent_t xfer = nullptr;      // recorded after the latest transfer
    bool has_use = false, has_xfer = false;
  };
  struct Pending {
    int64_t off, cap;
    cudaEvent_t ev;
  };
  std::mutex mu;
  int device = -1;
  unsigned char *arena = nullptr;
  int64_t budget = 0;
  cudaStream_t up = nullptr, down = nullptr;
  cudaStream_t waiter = nullptr;  // acc_table_wait's private stream
  std::unordered_map<const void *, Entry> map;
  RangeAlloc ranges;  // the arena's free ranges
  std::deque<Pending> pending;
  uint64_t tick = 0;
  acc_table_stats st{};
  // Transfer trace (acc_table_trace): per transfer, timing events around it
  // on its stream.
  struct Trace {
    int kind;
    int64_t bytes;
    cudaEvent_t a, b;
  };
  bool tracing = false;
  std::vector<Trace> trace;
};

namespace accgb {
namespace {

// Copy on stream q as host_copy does, between timing events when the table
// traces its transfers (kind: 0 upload, 1 download, 2 copy back on eviction).
int traced_copy(acc_table *t, int kind, void *dst, const void *src, const void *host, int64_t bytes,
                cudaStream_t q) {
  cudaEvent_t a = nullptr, b = nullptr;
  if (t->tracing && cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess)
    cudaEventRecord(a, q);
  const int st = host_copy(dst, src, host, bytes, q);
  if (a && b) {
    cudaEventRecord(b, q);
    t->trace.push_back({kind, bytes, a, b});
  } else {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
  return st;
}

// Move the ranges of completed evictions back to the free list; with
// `block`, wait for the oldest one first.
int reclaim(acc_table *t, bool block) {
  while (!t->pending.empty()) {
    auto &p = t->pending.front();
    cudaError_t e = block ? cudaEventSynchronize(p.ev) : cudaEventQuery(p.ev);
    if (e == cudaErrorNotReady) { cudaGetLastError(); break; }
    if (e != cudaSuccess) return cuda_status(e);
    t->ranges.give(p.off, p.cap);
    cudaEventDestroy(p.ev);
    t->pending.pop_front();
    block = false;
  }
  return ACC_OK;
}

cudaEvent_t make_event() {
  cudaEvent_t ev = nullptr;
  if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) return nullptr;
  return ev;
}

// Record `ev` anew on stream q as a fresh event object (the old one is
// released once its waiters are done).  Re-recording one event object that
// other streams wait on serialised the table's upload and download streams
// on GB300: a step of the bench's end-to-end leg took 30 to 60 ms instead of
// 25 ms, the host link's bound being 22 ms.
int record_fresh(cudaEvent_t &ev, cudaStream_t q) {
  cudaEvent_t fresh = make_event();
  if (!fresh) return ACC_ERR_CUDA;
  const cudaError_t ce = cudaEventRecord(fresh, q);
  if (ce != cudaSuccess) {
    cudaEventDestroy(fresh);
    return cuda_status(ce);
  }
  if (ev) cudaEventDestroy(ev);
  ev = fresh;
  return ACC_OK;
}

// Evict entry e (not held): its range is reused once its last user and any
// copy back are done.  writeback: copy a device-written array back first.
int retire(acc_table *t, acc_table::Entry &e, bool writeback) {
  if (e.has_use) cudaStreamWaitEvent(t->down, e.last_use, 0);
  if (e.has_xfer) cudaStreamWaitEvent(t->down, e.xfer, 0);
  if (writeback && e.dirty && e.bytes > 0) {
    int st = traced_copy(t, 2, const_cast<void *>(e.host), t->arena + e.off, e.host, e.bytes, t->down);
    if (st) return st;
    t->st.writebacks += 1;
    t->st.downloads += 1;
    t->st.download_bytes += e.bytes;
  }
  cudaEvent_t ev = make_event();
  if (!ev) return ACC_ERR_CUDA;
  cudaError_t ce = cudaEventRecord(ev, t->down);
  if (ce != cudaSuccess) { cudaEventDestroy(ev); return cuda_status(ce); }
  if (e.cap > 0) t->pending.push_back({e.off, e.cap, ev});
  else cudaEventDestroy(ev);
  t->st.resident_bytes -= e.cap;
  t->st.arrays -= 1;
  if (e.last_use) cudaEventDestroy(e.last_use);
  if (e.xfer) cudaEventDestroy(e.xfer);
  return ACC_OK;
}

// A range of `cap` bytes: from the free list, else from completed
// evictions, else by evicting least recently used arrays that are not held
// until enough bytes are free or on their way back, waiting (on the host)
// for those ranges only then.
int arena_alloc(acc_table *t, int64_t cap, int64_t *off) {
  if (cap == 0) { *off = 0; return ACC_OK; }
  if (cap > t->budget) return ACC_ERR_NOMEM;
  int st = reclaim(t, false);
  if (st) return st;
  while (true) {
    if (t->ranges.take(cap, off)) return ACC_OK;
    int64_t avail = t->ranges.free_bytes;
    for (auto &p : t->pending) avail += p.cap;
    if (t->pending.empty() || avail < cap) {
      const void *victim = nullptr;
      uint64_t best = ~0ull;
      for (auto &kv : t->map)
        if (kv.second.holds == 0 && kv.second.tick < best) { best = kv.second.tick; victim = kv.first; }
      if (victim) {
        auto it = t->map.find(victim);
        st = retire(t, it->second, true);
        t->map.erase(it);
        t->st.evictions += 1;
        if (st) return st;
        st = reclaim(t, false);
        if (st) return st;
        continue;
      }
      if (t->pending.empty()) return ACC_ERR_NOMEM;
    }
    st = reclaim(t, true);  // waits for the oldest eviction in flight
    if (st) return st;
  }
}

int check_device(acc_table *t) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e);
  return dev == t->device ? ACC_OK : ACC_ERR_INVALID;
}

// Find or make the entry of `host` (bytes long); *fresh when it was made.
int lookup(acc_table *t, const void *host, int64_t bytes, acc_table::Entry **out, bool *fresh) {
  *fresh = false;
  auto it = t->map.find(host);
  if (it != t->map.end()) {
    if (it->second.bytes == bytes) { *out = &it->second; return ACC_OK; }
    // the same address now holds an array of another size: a new array
    if (it->second.holds > 0) return ACC_ERR_INVALID;
    int st = retire(t, it->second, false);
    t->map.erase(it);
    if (st) return st;
  }
  const int64_t cap = (bytes + TABLE_ALIGN - 1) / TABLE_ALIGN * TABLE_ALIGN;
  int64_t off = 0;
  int st = arena_alloc(t, cap, &off);
  if (st) return st;
  acc_table::Entry e;
  e.host = host;
  e.bytes = bytes;
  e.off = off;
  e.cap = cap;
  e.last_use = make_event();
  e.xfer = make_event();
  if (!e.last_use || !e.xfer) {
    if (e.last_use) cudaEventDestroy(e.last_use);
    if (e.xfer) cudaEventDestroy(e.xfer);
    t->ranges.give(off, cap);
    return ACC_ERR_CUDA;
  }
  auto ins = t->map.emplace(host, e);
  t->st.resident_bytes += cap;
  t->st.arrays += 1;
  *out = &ins.first->second;
  *fresh = true;
  return ACC_OK;
}

// Upload host -> device copy on the upload stream, after `after` (an event
// of the caller's stream, or null) and the array's last user.
int upload(acc_table *t, acc_table::Entry &e, cudaEvent_t after) {
  if (after) cudaStreamWaitEvent(t->up, after, 0);
  if (e.has_use) cudaStreamWaitEvent(t->up, e.last_use, 0);
  if (e.has_xfer) cudaStreamWaitEvent(t->up, e.xfer, 0);
  int st = traced_copy(t, 0, t->arena + e.off, e.host, e.host, e.bytes, t->up);
  if (st) return st;
  const int rs = record_fresh(e.xfer, t->up);
  if (rs) return rs;
  e.has_xfer = true;
  e.dirty = false;
  t->st.uploads += 1;
  t->st.upload_bytes += e.bytes;
  return ACC_OK;
}

// An event marking the work enqueued so far on the caller's stream.
int mark(cudaStream_t s, cudaEvent_t *ev) {
  *ev = make_event();
  if (!*ev) return ACC_ERR_CUDA;
  cudaError_t ce = cudaEventRecord(*ev, s);
  if (ce != cudaSuccess) { cudaEventDestroy(*ev); *ev = nullptr; return cuda_status(ce); }
  return ACC_OK;
}

}  // namespace
}  // namespace accgb

extern "C" int acc_upload(void *dev, const void *host, int64_t bytes, void *stream) {
  if (bytes < 0 || (bytes > 0 && (!dev || !host))) return ACC_ERR_INVALID;
  return host_copy(dev, host, host, bytes, static_cast<cudaStream_t>(stream));
}

extern "C" int acc_download(void *host, const void *dev, int64_t bytes, void *stream) {
  if (bytes < 0 || (bytes > 0 && (!dev || !host))) return ACC_ERR_INVALID;
  return host_copy(host, dev, host, bytes, static_cast<cudaStream_t>(stream));
}

extern "C" int acc_table_create(int64_t budget_bytes, acc_table **out) {
  if (!out || budget_bytes <= 0) return ACC_ERR_INVALID;
  *out = nullptr;
  auto *t = new acc_table();
  cudaError_t e = cudaGetDevice(&t->device);
  const int64_t budget = (budget_bytes + TABLE_ARENA_ROUND - 1) / TABLE_ARENA_ROUND * TABLE_ARENA_ROUND;
  if (e == cudaSuccess) e = cudaMalloc(&t->arena, (size_t)budget);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&t->up, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&t->down, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&t->waiter, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    if (t->arena) cudaFree(t->arena);
    if (t->up) cudaStreamDestroy(t->up);
    if (t->down) cudaStreamDestroy(t->down);
    delete t;
    return cuda_status(e);
  }
  t->budget = budget;
  t->st.budget = budget;
  t->ranges.give(0, budget);
  *out = t;
  return ACC_OK;
}

extern "C" int acc_table_destroy(acc_table *t) {
  if (!t) return ACC_ERR_INVALID;
  int st = ACC_OK;
  {
    std::lock_guard<std::mutex> lk(t->mu);
    for (auto &kv : t->map) {
      const int s2 = retire(t, kv.second, true);
      if (!st) st = s2;
    }
    t->map.clear();
    cudaError_t e = cudaStreamSynchronize(t->down);
    if (e == cudaSuccess) e = cudaStreamSynchronize(t->up);
    if (!st) st = cuda_status(e);
    for (auto &p : t->pending) cudaEventDestroy(p.ev);
    t->pending.clear();
    cudaFree(t->arena);
    cudaStreamSynchronize(t->waiter);
    cudaStreamDestroy(t->up);
    cudaStreamDestroy(t->down);
    cudaStreamDestroy(t->waiter);
  }
  for (auto &r : t->trace) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  delete t;
  return st;
}

extern "C" int acc_table_use(acc_table *t, const void *host, int64_t bytes, void *stream, void **dev) {
  if (!t || !host || !dev || bytes < 0) return ACC_ERR_INVALID;
  std::lock_guard<std::mutex> lk(t->mu);
  int st = check_device(t);
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  acc_table::Entry *e = nullptr;
  bool fresh = false;
  st = lookup(t, host, bytes, &e, &fresh);
  if (st) return st;
  if (fresh) {
    st = upload(t, *e, nullptr);
    if (st) {
      retire(t, *e, false);
      t->map.erase(host);
      return st;
    }
  } else {
    t->st.hits += 1;
  }
  if (e->has_xfer) cudaStreamWaitEvent(s, e->xfer, 0);
  e->holds += 1;
  e->tick = ++t->tick;
  *dev = t->arena + e->off;
  return ACC_OK;
}

extern "C" int acc_table_malloc(acc_table *t, void *host, int64_t bytes, void *stream, void **dev) {
  if (!t || !host || !dev || bytes < 0) return ACC_ERR_INVALID;
  std::lock_guard<std::mutex> lk(t->mu);
  int st = check_device(t);
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  acc_table::Entry *e = nullptr;
  bool fresh = false;
  st = lookup(t, host, bytes, &e, &fresh);
  if (st) return st;
  // A download still reading the old contents finishes before the caller's
  // work overwrites them.
  if (e->has_xfer) cudaStreamWaitEvent(s, e->xfer, 0);
  e->dirty = true;
  e->holds += 1;
  e->tick = ++t->tick;
  *dev = t->arena + e->off;
  return ACC_OK;
}

extern "C" int acc_table_poke(acc_table *t, const void *host, void *stream) {
  if (!t || !host) return ACC_ERR_INVALID;
  std::lock_guard<std::mutex> lk(t->mu);
  int st = check_device(t);
  if (st) return st;
  auto it = t->map.find(host);
  if (it == t->map.end()) return ACC_ERR_INVALID;
  // The copy waits for the array's last recorded user (release) and its
  // previous transfer, not for the rest of the caller's stream, so that it
  // overlaps the caller's kernels on other arrays.
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  st = upload(t, it->second, nullptr);
  if (st) return st;
  cudaStreamWaitEvent(s, it->second.xfer, 0);
  it->second.tick = ++t->tick;
  return ACC_OK;
}

extern "C" int acc_table_peek(acc_table *t, void *host, void *stream) {
  if (!t || !host) return ACC_ERR_INVALID;
  std::lock_guard<std::mutex> lk(t->mu);
  int st = check_device(t);
  if (st) return st;
  auto it = t->map.find(host);
  if (it == t->map.end()) return ACC_ERR_INVALID;
  acc_table::Entry &e = it->second;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaEvent_t after = nullptr;
  st = mark(s, &after);
  if (st) return st;
  cudaStreamWaitEvent(t->down, after, 0);
  cudaEventDestroy(after);
  if (e.has_xfer) cudaStreamWaitEvent(t->down, e.xfer, 0);
  st = traced_copy(t, 1, host, t->arena + e.off, host, e.bytes, t->down);
  if (st) return st;
  st = record_fresh(e.xfer, t->down);
  if (st) return st;
  e.has_xfer = true;
  e.dirty = false;
  e.tick = ++t->tick;
  t->st.downloads += 1;
  t->st.download_bytes += e.bytes;
  return ACC_OK;
}

extern "C" int acc_table_release(acc_table *t, const void *host, void *stream) {
  if (!t || !host) return ACC_ERR_INVALID;
  std::lock_guard<std::mutex> lk(t->mu);
  auto it = t->map.find(host);
  if (it == t->map.end() || it->second.holds <= 0) return ACC_ERR_INVALID;
  acc_table::Entry &e = it->second;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // Several holders on different streams: the recorded last user follows
  // every one of them.
  if (e.has_use) cudaStreamWaitEvent(s, e.last_use, 0);
  const int rs = record_fresh(e.last_use, s);
  if (rs) return rs;
  e.has_use = true;
  e.holds -= 1;
  return ACC_OK;
}

extern "C" int acc_table_wait(acc_table *t, const void *host) {
  if (!t || !host) return ACC_ERR_INVALID;
  cudaEvent_t ev = nullptr;
  {
    std::lock_guard<std::mutex> lk(t->mu);
    auto it = t->map.find(host);
    if (it == t->map.end()) return ACC_ERR_INVALID;
    if (!it->second.has_xfer) return ACC_OK;
    ev = it->second.xfer;
    // Wait on a private event that follows the array's transfers (on a
    // stream of its own, which delays no transfer), so that another thread
    // may re-record or drop the array's own event meanwhile.
    cudaEvent_t own = make_event();
    if (!own) return ACC_ERR_CUDA;
    cudaStreamWaitEvent(t->waiter, ev, 0);
    cudaError_t ce = cudaEventRecord(own, t->waiter);
    if (ce != cudaSuccess) { cudaEventDestroy(own); return cuda_status(ce); }
    ev = own;
  }
  cudaError_t e = cudaEventSynchronize(ev);
  cudaEventDestroy(ev);
  return cuda_status(e);
}

extern "C" int acc_table_join(acc_table *t, void *stream) {
  if (!t) return ACC_ERR_INVALID;
  std::lock_guard<std::mutex> lk(t->mu);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  for (cudaStream_t q : {t->up, t->down}) {
    cudaEvent_t ev = nullptr;
    int st = mark(q, &ev);
    if (st) return st;
    cudaError_t ce = cudaStreamWaitEvent(s, ev, 0);
    cudaEventDestroy(ev);
    if (ce != cudaSuccess) return cuda_status(ce);
  }
  return ACC_OK;
}

extern "C" int acc_table_free(acc_table *t, const void *host) {
  if (!t || !host) return ACC_ERR_INVALID;
  std::lock_guard<std::mutex> lk(t->mu);
  auto it = t->map.find(host);
  if (it == t->map.end() || it->second.holds > 0) return ACC_ERR_INVALID;
  const int st = retire(t, it->second, false);
  t->map.erase(it);
  return st;
}

extern "C" int acc_table_get_stats(acc_table *t, acc_table_stats *out) {
  if (!t || !out) return ACC_ERR_INVALID;
  std::lock_guard<std::mutex> lk(t->mu);
  *out = t->st;
  return ACC_OK;
}

extern "C" int acc_table_trace(acc_table *t, int enable) {
  if (!t) return ACC_ERR_INVALID;
  std::lock_guard<std::mutex> lk(t->mu);
  for (auto &r : t->trace) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  t->trace.clear();
  t->tracing = enable != 0;
  return ACC_OK;
}

extern "C" int acc_table_trace_get(acc_table *t, void *origin, acc_xfer_record *rec, int64_t cap, int64_t *count) {
  if (!t || !origin || !count || cap < 0 || (cap > 0 && !rec)) return ACC_ERR_INVALID;
  std::lock_guard<std::mutex> lk(t->mu);
  cudaEvent_t o = static_cast<cudaEvent_t>(origin);
  *count = (int64_t)t->trace.size();
  for (int64_t i = 0; i < cap && i < (int64_t)t->trace.size(); ++i) {
    const auto &r = t->trace[i];
    float a = 0.f, b = 0.f;
    cudaError_t e = cudaEventSynchronize(r.b);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&a, o, r.a);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&b, o, r.b);
    if (e != cudaSuccess) return cuda_status(e);
    rec[i].kind = r.kind;
    rec[i].bytes = r.bytes;
    rec[i].start_ms = a;
    rec[i].end_ms = b;
  }
  return ACC_OK;
}
