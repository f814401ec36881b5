// permute.cu -- permute f defaults p xs for the fixed primitives.
//
// The reference's permute_rmw issues one global atomic read-modify-write per
// source element (accelerate-llvm-ptx/src/Data/Array/Accelerate/LLVM/PTX/
// CodeGen/Permute.hs:117-213), so a skewed (Zipf) histogram serialises on the
// few hot bins in L2.  Two kernels here:
//   * permute_global -- red.global / atom.global RMW per element (any type,
//     any primitive; CAS loops for the primitives without a native atomic);
//   * permute_cluster -- for 32-bit integer targets up to 8 x 50K bins: the
//     target array is privatised in the DISTRIBUTED shared memory of a
//     thread-block cluster (each CTA of the cluster holds 1/CL of the bins,
//     filled with the identity), every element does a shared-memory atomic
//     on the CTA that owns its bin, and at the end each CTA folds its bins
//     into global memory with one atomic per touched bin.
// Each update is out[j] = f x out[j] with the new value first, the order of
// the reference's combine (Native/CodeGen/Permute.hs:112-116).  Integer
// results do not depend on the update order; Float32/Float64 + does.
#include <cooperative_groups.h>
#include <cstdlib>
#include <cstring>

#include "common.cuh"

namespace cg = cooperative_groups;

namespace accgb {

struct PermArgs {
  const void *src;
  const void *idx;
  void *out;
  int64_t n, m;
  uint64_t cval;
  int has_src;
  int idx64;
  uint32_t *err;
};

// Atomic out[j] = f(x, out[j]) on global or shared (generic address) memory.
template <int OP, class T>
__device__ __forceinline__ void atomic_combine(T *p, T x) {
  if constexpr (std::is_same<T, int32_t>::value || std::is_same<T, uint32_t>::value) {
    if constexpr (OP == ACC_ADD) atomicAdd(p, x);
    else if constexpr (OP == ACC_MIN) atomicMin(p, x);
    else if constexpr (OP == ACC_MAX) atomicMax(p, x);
    else if constexpr (OP == ACC_AND) atomicAnd(p, x);
    else if constexpr (OP == ACC_OR) atomicOr(p, x);
    else if constexpr (OP == ACC_XOR) atomicXor(p, x);
    else {
      unsigned *q = reinterpret_cast<unsigned *>(p);
      unsigned old = *q, assumed;
      do {
        assumed = old;
        T nv = Prim<OP, T>::ap(x, (T)assumed);
        old = atomicCAS(q, assumed, (unsigned)nv);
      } while (old != assumed);
    }
  } else if constexpr (std::is_same<T, int64_t>::value) {
    unsigned long long *q = reinterpret_cast<unsigned long long *>(p);
    if constexpr (OP == ACC_ADD) atomicAdd(q, (unsigned long long)x);
    else if constexpr (OP == ACC_MIN) atomicMin(reinterpret_cast<long long *>(p), (long long)x);
    else if constexpr (OP == ACC_MAX) atomicMax(reinterpret_cast<long long *>(p), (long long)x);
    else if constexpr (OP == ACC_AND) atomicAnd(q, (unsigned long long)x);
    else if constexpr (OP == ACC_OR) atomicOr(q, (unsigned long long)x);
    else if constexpr (OP == ACC_XOR) atomicXor(q, (unsigned long long)x);
    else {
      unsigned long long old = *q, assumed;
      do {
        assumed = old;
        T nv = Prim<OP, T>::ap(x, (T)assumed);
        old = atomicCAS(q, assumed, (unsigned long long)nv);
      } while (old != assumed);
    }
  } else if constexpr (std::is_same<T, float>::value) {
    if constexpr (OP == ACC_ADD) atomicAdd(p, x);
    else {
      unsigned *q = reinterpret_cast<unsigned *>(p);
      unsigned old = *q, assumed;
      do {
        assumed = old;
        float nv = Prim<OP, float>::ap(x, __uint_as_float(assumed));
        old = atomicCAS(q, assumed, __float_as_uint(nv));
      } while (old != assumed);
    }
  } else {
    if constexpr (OP == ACC_ADD) atomicAdd(p, x);
    else {
      unsigned long long *q = reinterpret_cast<unsigned long long *>(p);
      unsigned long long old = *q, assumed;
      do {
        assumed = old;
        double nv = Prim<OP, double>::ap(x, __longlong_as_double((long long)assumed));
        old = atomicCAS(q, assumed, (unsigned long long)__double_as_longlong(nv));
      } while (old != assumed);
    }
  }
}

__device__ __forceinline__ int64_t perm_idx(const PermArgs &a, int64_t i) {
  return a.idx64 ? static_cast<const int64_t *>(a.idx)[i] : (int64_t) static_cast<const int32_t *>(a.idx)[i];
}

template <int OP, class T>
__global__ void __launch_bounds__(256) permute_global(PermArgs a) {
  const T *src = static_cast<const T *>(a.src);
  T *out = static_cast<T *>(a.out);
  const T c = from_bits<T>(a.cval);
  bool bad = false;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = perm_idx(a, i);
    if (j < 0) continue;  // Nothing: the element is dropped
    if (j >= a.m) { bad = true; continue; }
    atomic_combine<OP, T>(out + j, a.has_src ? src[i] : c);
  }
  if (bad) raise_error(a.err, DEV_ERR_INDEX);
}

// Privatised permute into cluster-distributed shared memory.  CL CTAs form a
// cluster; bin j is owned by CTA (j & (CL-1)) of the cluster, at local slot
// j >> log2(CL).  An update to an owned bin is a shared-memory atomic, an
// update to a bin of the partner CTA a `red.shared::cluster` on its shared
// memory.  AGG: lanes of a warp that hit the same bin are combined first
// (match.any) so a hot bin costs one atomic per warp instead of one per lane.
__device__ __forceinline__ uint32_t mapa_shared(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
template <int OP, class T>
__device__ __forceinline__ void red_cluster(uint32_t addr, T v) {
  static_assert(sizeof(T) == 4, "32-bit bins");
  if constexpr (OP == ACC_ADD) asm volatile("red.shared::cluster.add.u32 [%0], %1;" :: "r"(addr), "r"((uint32_t)v) : "memory");
  else if constexpr (OP == ACC_AND) asm volatile("red.shared::cluster.and.b32 [%0], %1;" :: "r"(addr), "r"((uint32_t)v) : "memory");
  else if constexpr (OP == ACC_OR) asm volatile("red.shared::cluster.or.b32 [%0], %1;" :: "r"(addr), "r"((uint32_t)v) : "memory");
  else if constexpr (OP == ACC_XOR) asm volatile("red.shared::cluster.xor.b32 [%0], %1;" :: "r"(addr), "r"((uint32_t)v) : "memory");
  else if constexpr (OP == ACC_MIN) {
    if constexpr (std::is_same<T, int32_t>::value) asm volatile("red.shared::cluster.min.s32 [%0], %1;" :: "r"(addr), "r"(v) : "memory");
    else asm volatile("red.shared::cluster.min.u32 [%0], %1;" :: "r"(addr), "r"(v) : "memory");
  } else {
    if constexpr (std::is_same<T, int32_t>::value) asm volatile("red.shared::cluster.max.s32 [%0], %1;" :: "r"(addr), "r"(v) : "memory");
    else asm volatile("red.shared::cluster.max.u32 [%0], %1;" :: "r"(addr), "r"(v) : "memory");
  }
}
// Value that `cnt` equal lanes combine into (AGG): + multiplies, the
// idempotent primitives keep one, xor keeps the parity.
template <int OP, class T> __device__ __forceinline__ T agg_value(T x, int cnt) {
  if constexpr (OP == ACC_ADD) return (T)((uint32_t)x * (uint32_t)cnt);
  else if constexpr (OP == ACC_XOR) return (cnt & 1) ? x : T(0);
  else return x;
}

template <int OP, class T, int LOG_CL, bool AGG>
__global__ void __launch_bounds__(1024, 1) permute_cluster(PermArgs a, int per) {
  constexpr int CL = 1 << LOG_CL;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *bins = reinterpret_cast<T *>(smem_raw);
  const uint32_t rank = CL > 1 ? cg::this_cluster().block_rank() : 0u;
  const T idT = Prim<OP, T>::id();
  for (int b = threadIdx.x; b < per; b += blockDim.x) bins[b] = idT;
  if constexpr (CL > 1) cg::this_cluster().sync(); else __syncthreads();
  const uint32_t bins_addr = smem_addr(bins);
  uint32_t remote_base[CL];
#pragma unroll
  for (int r = 0; r < CL; ++r) remote_base[r] = CL > 1 ? mapa_shared(bins_addr, (uint32_t)r) : bins_addr;

  const T *src = static_cast<const T *>(a.src);
  const T c = from_bits<T>(a.cval);
  const uint32_t m = (uint32_t)a.m;
  bool bad = false;
  // Lanes call `one` convergently (AGG needs the whole warp); a dropped or
  // out-of-range element passes j < 0 / j >= m and does nothing.
  auto one = [&](int32_t j, T x) {
    const bool ok = j >= 0 && (uint32_t)j < m;
    bad |= (j >= 0 && !ok);
    T v = x;
    bool lead = ok;
    if constexpr (AGG) {
      // Lanes with the same target AND the same value combine into one update.
      uint32_t xb;
      memcpy(&xb, &x, 4);
      const unsigned long long key = ok ? (((unsigned long long)(uint32_t)j << 32) | xb) : ~0ull;
      const unsigned grp = __match_any_sync(0xffffffffu, key);
      lead = ok && (__ffs(grp) - 1) == (int)(threadIdx.x & 31);
      v = agg_value<OP, T>(x, __popc(grp));
    }
    if (!lead) return;
    const uint32_t owner = (uint32_t)j & (CL - 1), slot = (uint32_t)j >> LOG_CL;
    if (owner == rank) atomic_combine<OP, T>(bins + slot, v);
    else red_cluster<OP, T>(remote_base[owner] + slot * 4u, v);
  };
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  if (!a.idx64 && !a.has_src && (reinterpret_cast<uintptr_t>(a.idx) & 15u) == 0) {
    // Histogram fast path: Int32 indices, 16 per thread per round, 4 loads in flight.
    const int64_t nv = a.n / 4;
    const uint4 *iv = static_cast<const uint4 *>(a.idx);
    const int64_t rounds = (nv + 4 * nth - 1) / (4 * nth);
    for (int64_t r = 0; r < rounds; ++r) {
      uint4 q[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t v = (r * 4 + u) * nth + tid;
        q[u] = v < nv ? ld_stream16(iv + v) : make_uint4(~0u, ~0u, ~0u, ~0u);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        one((int32_t)q[u].x, c); one((int32_t)q[u].y, c); one((int32_t)q[u].z, c); one((int32_t)q[u].w, c);
      }
    }
    const int64_t tail = a.n - nv * 4;  // < 4 elements
    one(tid < tail ? static_cast<const int32_t *>(a.idx)[nv * 4 + tid] : -1, c);
  } else {
    const int64_t rounds = (a.n + nth - 1) / nth;
    for (int64_t r = 0; r < rounds; ++r) {
      const int64_t i = r * nth + tid;
      int64_t j = -1;
      T x = c;
      if (i < a.n) {
        j = perm_idx(a, i);
        if (a.has_src) x = src[i];
      }
      // 64-bit indices beyond Int32 range are out of range for a 32-bit bin array.
      if (j >= (int64_t)m) { bad = true; j = -1; }
      one((int32_t)j, x);
    }
  }
  if (bad) raise_error(a.err, DEV_ERR_INDEX);
  if constexpr (CL > 1) cg::this_cluster().sync(); else __syncthreads();

  // Fold this CTA's bins into the target; untouched bins hold the identity.
  T *out = static_cast<T *>(a.out);
  for (int b = threadIdx.x; b < per; b += blockDim.x) {
    const T v = bins[b];
    const int64_t j = ((int64_t)b << LOG_CL) | rank;
    if (v != idT && j < a.m) atomic_combine<OP, T>(out + j, v);
  }
}

// Privatised permute, split by ownership instead of remote atomics: the CL
// CTAs of a cluster all read the SAME slice of the input (co-scheduled, so
// L2 serves all but the first read of each line) and each applies only the
// updates to the bins it owns, with local shared-memory atomics.
template <int OP, class T, int LOG_CL>
__global__ void __launch_bounds__(1024, 1) permute_split(PermArgs a, int per) {
  constexpr int CL = 1 << LOG_CL;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *bins = reinterpret_cast<T *>(smem_raw);
  const uint32_t rank = CL > 1 ? cg::this_cluster().block_rank() : 0u;
  const T idT = Prim<OP, T>::id();
  for (int b = threadIdx.x; b < per; b += blockDim.x) bins[b] = idT;
  __syncthreads();
  const T *src = static_cast<const T *>(a.src);
  const T c = from_bits<T>(a.cval);
  const uint32_t m = (uint32_t)a.m;
  bool bad = false;
  auto one = [&](int32_t j, T x) {
    if (j < 0) return;
    if ((uint32_t)j >= m) { bad = true; return; }
    if (((uint32_t)j & (CL - 1)) != rank) return;
    atomic_combine<OP, T>(bins + ((uint32_t)j >> LOG_CL), x);
  };
  // Thread index within the cluster's share of the grid.
  const int64_t cluster_id = blockIdx.x >> LOG_CL;
  const int64_t nclusters = gridDim.x >> LOG_CL;
  const int64_t tid = cluster_id * blockDim.x + threadIdx.x;
  const int64_t nth = nclusters * blockDim.x;
  if (!a.idx64 && !a.has_src && (reinterpret_cast<uintptr_t>(a.idx) & 15u) == 0) {
    const int64_t nv = a.n / 4;
    const uint4 *iv = static_cast<const uint4 *>(a.idx);
    const int64_t rounds = (nv + 4 * nth - 1) / (4 * nth);
    for (int64_t r = 0; r < rounds; ++r) {
      uint4 q[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int64_t v = (r * 4 + u) * nth + tid;
        q[u] = v < nv ? __ldcg(iv + v) : make_uint4(~0u, ~0u, ~0u, ~0u);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        one((int32_t)q[u].x, c); one((int32_t)q[u].y, c); one((int32_t)q[u].z, c); one((int32_t)q[u].w, c);
      }
    }
    const int64_t tail = a.n - nv * 4;
    if (tid < tail) one(static_cast<const int32_t *>(a.idx)[nv * 4 + tid], c);
  } else {
    for (int64_t i = tid; i < a.n; i += nth) {
      const int64_t j = perm_idx(a, i);
      if (j >= (int64_t)m) { bad = true; continue; }
      one((int32_t)j, a.has_src ? src[i] : c);
    }
  }
  if (bad && rank == 0) raise_error(a.err, DEV_ERR_INDEX);
  __syncthreads();
  T *out = static_cast<T *>(a.out);
  for (int b = threadIdx.x; b < per; b += blockDim.x) {
    const T v = bins[b];
    const int64_t j = ((int64_t)b << LOG_CL) | rank;
    if (v != idT && j < a.m) atomic_combine<OP, T>(out + j, v);
  }
}

// Histogram (+ of a small positive constant) with 16-bit counters packed two
// to a word, so 2^16 bins fit in one CTA's shared memory and every update is
// local.  Word w holds bin w (low half) and bin w + half (high half), half =
// ceil(m / 2): neighbouring bins, which skewed (Zipf-like) indices make hot
// together, sit in different words and banks, so their updates do not
// serialise on one address.  A counter that wraps is repaired exactly: the
// carry that ran into the word's other counter is taken back and 65536 is
// added to the target bin in global memory.
template <bool AGG>
__global__ void __launch_bounds__(1024, 1) permute_hist16(PermArgs a) {
  extern __shared__ __align__(16) uint32_t words[];
  const uint32_t m = (uint32_t)a.m;
  const uint32_t nwords = (m + 1) / 2;
  for (uint32_t b = threadIdx.x; b < nwords; b += blockDim.x) words[b] = 0u;
  __syncthreads();
  const uint32_t c = (uint32_t)a.cval;
  uint32_t *out = static_cast<uint32_t *>(a.out);
  bool bad = false;
  auto one = [&](int32_t j) {
    const bool ok = j >= 0 && (uint32_t)j < m;
    bad |= (j >= 0 && !ok);
    uint32_t inc = c;
    bool lead = ok;
    if constexpr (AGG) {
      const unsigned grp = __match_any_sync(0xffffffffu, ok ? j : -1);
      lead = ok && (__ffs(grp) - 1) == (int)(threadIdx.x & 31);
      inc = c * (uint32_t)__popc(grp);
    }
    if (!lead) return;
    // Each bin's true count is its 16-bit counter plus 65536 for every time the
    // counter's unbounded value crossed a multiple of 65536.  Every change to
    // a counter is one atomic whose returned old word shows the crossing:
    //  * an update of bin j crosses when old16 + inc > 0xffff;
    //  * a low counter that crosses also carries +1 into the high counter
    //    (a crossing for bin j+half when the old high half was 0xffff), and
    //    the carry is then taken back with -1 (a crossing back when the high
    //    half it finds is 0).  Accounting for all three keeps every bin exact.
    const bool low = (uint32_t)j < nwords;
    const uint32_t wi = low ? (uint32_t)j : (uint32_t)j - nwords;
    const uint32_t sh = low ? 0u : 16u;
    const uint32_t old = atomicAdd(&words[wi], inc << sh);
    if (((old >> sh) & 0xffffu) + inc > 0xffffu) {
      atomicAdd(out + j, 65536u);
      if (sh == 0) {
        int d = (old >> 16) == 0xffffu ? 1 : 0;
        const uint32_t old2 = atomicSub(&words[wi], 1u << 16);
        d -= (old2 >> 16) == 0u ? 1 : 0;
        if (d != 0 && (uint32_t)j + nwords < m) atomicAdd(out + j + nwords, (uint32_t)(d * 65536));
      }
    }
  };
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  const int64_t nv = a.n / 4;
  const uint4 *iv = static_cast<const uint4 *>(a.idx);
  const int64_t rounds = (nv + 4 * nth - 1) / (4 * nth);
  for (int64_t r = 0; r < rounds; ++r) {
    uint4 q[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t v = (r * 4 + u) * nth + tid;
      q[u] = v < nv ? ld_stream16(iv + v) : make_uint4(~0u, ~0u, ~0u, ~0u);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      one((int32_t)q[u].x); one((int32_t)q[u].y); one((int32_t)q[u].z); one((int32_t)q[u].w);
    }
  }
  const int64_t tail = a.n - nv * 4;
  one(tid < tail ? static_cast<const int32_t *>(a.idx)[nv * 4 + tid] : -1);
  if (bad) raise_error(a.err, DEV_ERR_INDEX);
  __syncthreads();
  for (uint32_t b = threadIdx.x; b < nwords; b += blockDim.x) {
    const uint32_t w = words[b];
    if (w & 0xffffu) atomicAdd(out + b, w & 0xffffu);
    if ((w >> 16) && b + nwords < m) atomicAdd(out + b + nwords, w >> 16);
  }
}

// ----------------------------------------------------------------- host side
// Shared-memory privatisation pays off when there are many more source
// elements than bins.  Variant choice (tuning knob, default "auto"):
// ACC_GB300_PERMUTE = auto | cluster | hist16 | global, ACC_GB300_PERMUTE_AGG = 0 | 1.
static int env_int(const char *name, int dflt) {
  const char *v = getenv(name);
  return v ? atoi(v) : dflt;
}
static const char *env_str(const char *name) {
  const char *v = getenv(name);
  return v ? v : "auto";
}

template <class K, class... Args>
static int launch_cluster(K kern, int CL, unsigned threads, size_t smem, int64_t want_ctas, cudaStream_t s,
                          Args... args) {
  const Device &d = device_info();
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (CL > 8) cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CL;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.gridDim = dim3(CL * d.sms);
  int clusters = 0;
  if (cudaOccupancyMaxActiveClusters(&clusters, kern, &cfg) != cudaSuccess || clusters <= 0) {
    cudaGetLastError();
    clusters = d.sms / CL > 0 ? d.sms / CL : 1;
  }
  int64_t grid = (int64_t)clusters * CL;
  const int64_t want = cdiv_h(want_ctas, CL) * CL;
  if (grid > want) grid = want;
  if (grid < CL) grid = CL;
  cfg.gridDim = dim3((unsigned)grid);
  return cuda_status(cudaLaunchKernelEx(&cfg, kern, args...));
}

template <int OP, class T, int LOG_CL>
static int launch_permute_cluster(PermArgs a, bool agg, cudaStream_t s) {
  const int CL = 1 << LOG_CL;
  const int per = (int)cdiv_h(a.m, CL);
  const size_t smem = (size_t)per * sizeof(T);
  const int64_t want = cdiv_h(a.n, 1024 * 16);
  if (LOG_CL == 0 || strcmp(env_str("ACC_GB300_PERMUTE"), "split") == 0)
    return launch_cluster(permute_split<OP, T, LOG_CL>, CL, 1024, smem, want * CL, s, a, per);
  if (agg) return launch_cluster(permute_cluster<OP, T, LOG_CL, true>, CL, 1024, smem, want, s, a, per);
  return launch_cluster(permute_cluster<OP, T, LOG_CL, false>, CL, 1024, smem, want, s, a, per);
}

template <int OP, class T>
int permute_typed(Workspace *w, PermArgs a, cudaStream_t s) {
  const Device &d = device_info();
  a.err = w->words + W_ERR;
  if (a.n == 0) return ACC_OK;
  const char *variant = env_str("ACC_GB300_PERMUTE");
  const bool agg = env_int("ACC_GB300_PERMUTE_AGG", 0) != 0;
  const bool force_global = strcmp(variant, "global") == 0;
  constexpr bool int32ish = std::is_same<T, int32_t>::value || std::is_same<T, uint32_t>::value;
  if constexpr (int32ish && OP != ACC_MUL) {
    const int64_t cap_bytes = d.max_smem_optin > (200 << 10) ? (192 << 10) : (int64_t)d.max_smem_optin - (8 << 10);
    const bool many = a.m > 0 && a.n >= 4 * a.m;
    // 16-bit packed counters: + of a small positive constant, Int32 indices.
    const uint32_t c = (uint32_t)a.cval;
    const bool hist16_ok = OP == ACC_ADD && !a.has_src && !a.idx64 && c > 0 && c < 2048 &&
                           (reinterpret_cast<uintptr_t>(a.idx) & 15u) == 0 && (a.m + 1) / 2 * 4 <= cap_bytes;
    const bool want_hist16 = strcmp(variant, "hist16") == 0 ||
                             (strcmp(variant, "auto") == 0 && a.m * (int64_t)sizeof(T) > cap_bytes);
    if (!force_global && many && hist16_ok && want_hist16) {
      const size_t smem = (size_t)((a.m + 1) / 2) * 4;
      auto kern = agg ? permute_hist16<true> : permute_hist16<false>;
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      int64_t grid = cdiv_h(a.n, 1024 * 16);
      if (grid > d.sms) grid = d.sms;
      kern<<<(unsigned)grid, 1024, smem, s>>>(a);
      return check_launch();
    }
    int64_t cap = cap_bytes / (int64_t)sizeof(T);
    if (!force_global && many) {
      if (a.m <= cap) return launch_permute_cluster<OP, T, 0>(a, agg, s);
      if (a.m <= 2 * cap) return launch_permute_cluster<OP, T, 1>(a, agg, s);
      if (a.m <= 4 * cap) return launch_permute_cluster<OP, T, 2>(a, agg, s);
      if (a.m <= 8 * cap) return launch_permute_cluster<OP, T, 3>(a, agg, s);
    }
  }
  int64_t blocks = cdiv_h(a.n, 256);
  if (blocks > (int64_t)d.sms * 16) blocks = (int64_t)d.sms * 16;
  permute_global<OP, T><<<(unsigned)blocks, 256, 0, s>>>(a);
  return check_launch();
}

}  // namespace accgb

using namespace accgb;

extern "C" int acc_permute(int op, int type, const void *src, const void *cval, const void *idx,
                           int index_type, void *out, int64_t n, int64_t m, void *stream) {
  if (n < 0 || m < 0) return ACC_ERR_INVALID;
  if (index_type != ACC_I32 && index_type != ACC_I64) return ACC_ERR_INVALID;
  if (!src && !cval) return ACC_ERR_INVALID;
  if (n > 0 && (!idx || !out)) return ACC_ERR_INVALID;
  if (type < ACC_I32 || type > ACC_F64) return ACC_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st = ACC_OK;
  Workspace *w = workspace(s, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  return with_type(type, [&](auto tv) -> int {
    using T = decltype(tv);
    PermArgs a{};
    a.src = src; a.idx = idx; a.out = out; a.n = n; a.m = m;
    a.cval = src ? 0 : seed_bits<T>(cval);
    a.has_src = src != nullptr;
    a.idx64 = index_type == ACC_I64;
    return with_op<T>(op, [&](auto opc) -> int {
      constexpr int OP = decltype(opc)::value;
      return permute_typed<OP, T>(w, a, s);
    });
  });
}

extern "C" int acc_permute_clone(int op, int type, const void *defaults, const void *src, const void *cval,
                                 const void *idx, int index_type, void *out, int64_t n, int64_t m,
                                 void *stream) {
  if (m < 0 || (m > 0 && (!defaults || !out))) return ACC_ERR_INVALID;
  static const size_t esz[] = {4, 8, 4, 4, 8};
  if (type < ACC_I32 || type > ACC_F64) return ACC_ERR_INVALID;
  // acc_permute's own argument checks, made before the clone so that a
  // rejected call leaves `out` untouched.
  if (n < 0 || (index_type != ACC_I32 && index_type != ACC_I64) || (!src && !cval) || (n > 0 && !idx))
    return ACC_ERR_INVALID;
  if (op < ACC_ADD || op > ACC_XOR) return ACC_ERR_INVALID;
  if (op >= ACC_AND && (type == ACC_F32 || type == ACC_F64)) return ACC_ERR_UNSUPPORTED;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (m > 0) {
    cudaError_t e = cudaMemcpyAsync(out, defaults, (size_t)m * esz[type], cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return cuda_status(e);
  }
  return acc_permute(op, type, src, cval, idx, index_type, out, n, m, stream);
}
