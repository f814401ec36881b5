// runtime.h -- host side of libaccgb: per-stream workspaces, device facts,
// TMA descriptor encoding and the (type, op) dispatch used by every entry point.
//
// The reference keeps one CUDA context per target and allocates skeleton
// temporaries per call with `allocateRemote` (PTX/Execute.hs:313,453), backed
// by an LRU memory table (PTX/Array/Table.hs:35-49).  Here each (device,
// stream) pair owns one grow-only workspace that is reused by every call on
// that stream, so a steady stream of calls performs no allocation at all.
#pragma once
#include <cstdint>
#include <cstddef>
#include <cstring>
#include <atomic>
#include <iterator>
#include <map>
#include <mutex>
#include <type_traits>
#include <cuda_runtime.h>
#include <cuda.h>

#include "../../include/acc_gb300.h"

namespace accgb {

struct Workspace {
  int device = -1;
  cudaStream_t stream = nullptr;
  // Small always-zero-between-calls area: [0] error word, [1] scan tile
  // ticket, [2] foldSeg big-segment count, [3..] per-row fold tickets.
  uint32_t *words = nullptr;
  size_t nwords = 0;
  // Look-back status slots (2 x u64 per tile), tagged with an epoch.
  uint64_t *status = nullptr;
  size_t nstatus = 0;   // in u64 words
  uint32_t epoch = 0;
  // Generic scratch (fold partials, foldSeg queues, offsets).
  void *scratch = nullptr;
  size_t nscratch = 0;
  std::mutex mu;
};

// Device-side error bits, OR-ed into the per-stream error word.
enum : uint32_t {
  DEV_ERR_TIMEOUT = 1u,  // a bounded spin-wait gave up
  DEV_ERR_INDEX   = 2u,  // permute target index out of range
};

enum { W_ERR = 0, W_TICKET = 1, W_SEGBIG = 2, W_DONE = 3, W_ROWTICKET0 = 8 };

struct Device {
  int id;
  int sms;
  int max_smem_optin;
  int cc_major, cc_minor;
};

// Current device facts (cached).
const Device &device_info();

// Workspace of (current device, stream); created on first use.
Workspace *workspace(cudaStream_t s, int *status);
int ws_words(Workspace *w, size_t n);          // ensure >= n zeroed words
int ws_status(Workspace *w, size_t u64words);  // ensure status slots
int ws_scratch(Workspace *w, size_t bytes);    // ensure scratch bytes
uint32_t ws_next_epoch(Workspace *w, cudaStream_t s);

// Map a CUDA error to a status (and remember the text for acc_strerror).
int cuda_status(cudaError_t e);
int check_launch();

// Encode a 2-D tiled tensor map (row-major, inner dim first).  Returns false
// if the driver rejects the description (alignment etc.).
bool encode_2d(CUtensorMap *map, const void *base, int elem_bytes,
               uint64_t inner, uint64_t outer, uint64_t row_pitch_bytes,
               uint32_t box_inner, uint32_t box_outer, bool swizzle128);

template <class T> constexpr bool is_fp() { return std::is_floating_point<T>::value; }

// Dispatch on the element type.
template <class F> int with_type(int type, F &&f) {
  switch (type) {
    case ACC_I32: return f(int32_t{});
    case ACC_I64: return f(int64_t{});
    case ACC_U32: return f(uint32_t{});
    case ACC_F32: return f(float{});
    case ACC_F64: return f(double{});
    default: return ACC_ERR_INVALID;
  }
}
template <int V> using IC = std::integral_constant<int, V>;
// Dispatch on the primitive; bitwise primitives exist for integral types only.
template <class T, class F> int with_op(int op, F &&f) {
  switch (op) {
    case ACC_ADD: return f(IC<ACC_ADD>{});
    case ACC_MUL: return f(IC<ACC_MUL>{});
    case ACC_MIN: return f(IC<ACC_MIN>{});
    case ACC_MAX: return f(IC<ACC_MAX>{});
    case ACC_AND: if constexpr (is_fp<T>()) return ACC_ERR_UNSUPPORTED; else return f(IC<ACC_AND>{});
    case ACC_OR:  if constexpr (is_fp<T>()) return ACC_ERR_UNSUPPORTED; else return f(IC<ACC_OR>{});
    case ACC_XOR: if constexpr (is_fp<T>()) return ACC_ERR_UNSUPPORTED; else return f(IC<ACC_XOR>{});
    default: return ACC_ERR_INVALID;
  }
}
// Accumulation policy actually used for (op, T, requested precision).
template <int OP, class T> int prec_of(int prec) {
  if constexpr (OP == ACC_ADD && std::is_same<T, float>::value) {
    if (prec == ACC_PREC_PLAIN) return 0;
    if (prec == ACC_PREC_FP64ACC) return 2;
    return 1;  // default and COMPENSATED
  }
  return 0;
}
// Dispatch on the accumulation policy (only Float32 + has more than one).
template <int OP, class T, class F> int with_prec(int prec, F &&f) {
  if constexpr (OP == ACC_ADD && std::is_same<T, float>::value) {
    switch (prec_of<OP, T>(prec)) {
      case 0: return f(IC<0>{});
      case 2: return f(IC<2>{});
      default: return f(IC<1>{});
    }
  } else {
    (void)prec;
    return f(IC<0>{});
  }
}

inline int64_t cdiv_h(int64_t a, int64_t b) { return (a + b - 1) / b; }

// A kernel's shared-memory attributes belong to the device context it runs
// in: set them once per device (bit d of `done` for device d).
template <class K>
inline void smem_attrs_once(K kern, int bytes, std::atomic<uint64_t> &done, bool max_carveout = true) {
  const int dev = device_info().id;
  const uint64_t bit = dev >= 0 && dev < 64 ? (1ull << dev) : 0ull;
  if (bit && (done.load(std::memory_order_acquire) & bit)) return;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (max_carveout) cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  done.fetch_or(bit, std::memory_order_release);
}

// Fill n elements with one value (the seed fill of empty folds and scans,
// the reference's `generate` of the seed, PTX/CodeGen/Generate.hs:40-61).
template <class T> int launch_fill(T *out, int64_t n, uint64_t bits, cudaStream_t s);

// Reusable batch launch area (batch.cu), used by the serving loop.
struct BatchArena;
int arena_create(int op, int64_t cap_reqs, int64_t cap_items, BatchArena **out);
int64_t arena_tiles(const acc_request &q);
int arena_launch(BatchArena *ar, const acc_request *reqs, int64_t count, cudaStream_t s);
void arena_free(BatchArena *ar);

// Exclusive `scanl (+) 0` of nseg segment lengths into nseg+1 offsets.
int scan_offsets(Workspace *w, int type, const void *lengths, void *offsets, int64_t nseg, cudaStream_t s);

template <class T> inline uint64_t seed_bits(const void *seed) {
  uint64_t b = 0;
  if (seed) memcpy(&b, seed, sizeof(T));
  return b;
}

inline bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Best-fit allocation of ranges of one arena (offsets and sizes in bytes,
// the caller rounds sizes to its alignment); freed ranges coalesce with free
// neighbours.  Host-side bookkeeping only: the arena itself is one device
// allocation made by its owner (a memory table, the serving loop).
struct RangeAlloc {
  std::map<int64_t, int64_t> free_off;        // offset -> size
  std::multimap<int64_t, int64_t> free_size;  // size -> offset
  int64_t free_bytes = 0;

  void give(int64_t off, int64_t size) {
    free_bytes += size;
    auto erase_size = [&](int64_t o, int64_t sz) {
      auto r = free_size.equal_range(sz);
      for (auto it = r.first; it != r.second; ++it)
        if (it->second == o) { free_size.erase(it); return; }
    };
    auto next = free_off.lower_bound(off);
    if (next != free_off.end() && next->first == off + size) {
      size += next->second;
      erase_size(next->first, next->second);
      next = free_off.erase(next);
    }
    if (next != free_off.begin()) {
      auto prev = std::prev(next);
      if (prev->first + prev->second == off) {
        off = prev->first;
        size += prev->second;
        erase_size(prev->first, prev->second);
        free_off.erase(prev);
      }
    }
    free_off[off] = size;
    free_size.emplace(size, off);
  }

  bool take(int64_t size, int64_t *off) {
    auto it = free_size.lower_bound(size);
    if (it == free_size.end()) return false;
    const int64_t sz = it->first, o = it->second;
    free_size.erase(it);
    free_off.erase(o);
    if (sz > size) {
      free_off[o + size] = sz - size;
      free_size.emplace(sz - size, o + size);
    }
    free_bytes -= size;
    *off = o;
    return true;
  }
};

}  // namespace accgb
