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

// Privatised permute into cluster-distributed shared memory.  CL CTAs form
// a cluster; CTA rank r owns bins [r*per, (r+1)*per).
template <int OP, class T>
__global__ void __launch_bounds__(1024) permute_cluster(PermArgs a, int per) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *bins = reinterpret_cast<T *>(smem_raw);
  cg::cluster_group cluster = cg::this_cluster();
  const unsigned rank = cluster.block_rank();
  const T idT = Prim<OP, T>::id();
  for (int b = threadIdx.x; b < per; b += blockDim.x) bins[b] = idT;
  cluster.sync();

  const T *src = static_cast<const T *>(a.src);
  const T c = from_bits<T>(a.cval);
  bool bad = false;
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nth = (int64_t)gridDim.x * blockDim.x;
  auto one = [&](int64_t j, T x) {
    if (j < 0) return;
    if (j >= a.m) { bad = true; return; }
    const unsigned owner = (unsigned)(j / per);
    T *dst = owner == rank ? bins : cluster.map_shared_rank(bins, owner);
    atomic_combine<OP, T>(dst + (j - (int64_t)owner * per), x);
  };
  if (!a.idx64 && !a.has_src && (reinterpret_cast<uintptr_t>(a.idx) & 15u) == 0) {
    // Histogram fast path: four Int32 indices per 16-byte load, two loads in flight.
    const int64_t nv = a.n / 4;
    const uint4 *iv = static_cast<const uint4 *>(a.idx);
    int64_t v = tid;
    for (; v + nth < nv; v += 2 * nth) {
      uint4 q0 = ld_stream16(iv + v), q1 = ld_stream16(iv + v + nth);
      one((int32_t)q0.x, c); one((int32_t)q0.y, c); one((int32_t)q0.z, c); one((int32_t)q0.w, c);
      one((int32_t)q1.x, c); one((int32_t)q1.y, c); one((int32_t)q1.z, c); one((int32_t)q1.w, c);
    }
    for (; v < nv; v += nth) {
      uint4 q0 = ld_stream16(iv + v);
      one((int32_t)q0.x, c); one((int32_t)q0.y, c); one((int32_t)q0.z, c); one((int32_t)q0.w, c);
    }
    for (int64_t i = nv * 4 + tid; i < a.n; i += nth) one(perm_idx(a, i), c);
  } else {
    for (int64_t i = tid; i < a.n; i += nth) one(perm_idx(a, i), a.has_src ? src[i] : c);
  }
  if (bad) raise_error(a.err, DEV_ERR_INDEX);
  cluster.sync();

  // Fold this CTA's bins into the target; untouched bins hold the identity
  // and need no update.
  T *out = static_cast<T *>(a.out);
  const int64_t base = (int64_t)rank * per;
  for (int b = threadIdx.x; b < per; b += blockDim.x) {
    const T v = bins[b];
    if (v != idT && base + b < a.m) atomic_combine<OP, T>(out + base + b, v);
  }
}

// ----------------------------------------------------------------- host side
template <int OP, class T>
int permute_typed(Workspace *w, PermArgs a, cudaStream_t s) {
  const Device &d = device_info();
  a.err = w->words + W_ERR;
  if (a.n == 0) return ACC_OK;
  constexpr bool int32ish = std::is_same<T, int32_t>::value || std::is_same<T, uint32_t>::value;
  if constexpr (int32ish && OP != ACC_MUL) {
    // Bins per CTA: up to 48K Int32 (192 KiB) of the opt-in shared memory.
    const int64_t cap_bytes = (int64_t)(d.max_smem_optin > (200 << 10) ? (192 << 10) : d.max_smem_optin - (8 << 10));
    const int64_t cap = cap_bytes / (int64_t)sizeof(T);
    int CL = 1;
    while (CL <= 8 && (int64_t)CL * cap < a.m) CL *= 2;
    // Privatise only when there are many more elements than bins.
    if (CL <= 8 && a.m > 0 && a.n >= 4 * a.m) {
      const int per = (int)cdiv_h(a.m, CL);
      const size_t smem = (size_t)per * sizeof(T);
      auto kern = permute_cluster<OP, T>;
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (CL > 1) cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeClusterDimension;
      attr[0].val.clusterDim.x = CL;
      attr[0].val.clusterDim.y = 1;
      attr[0].val.clusterDim.z = 1;
      cfg.blockDim = dim3(1024);
      cfg.dynamicSmemBytes = smem;
      cfg.stream = s;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      int clusters = 0;
      cfg.gridDim = dim3(CL * d.sms);
      if (cudaOccupancyMaxActiveClusters(&clusters, kern, &cfg) != cudaSuccess || clusters <= 0) {
        cudaGetLastError();
        clusters = d.sms / CL;
      }
      int64_t want = cdiv_h(a.n, 1024 * 8);
      int64_t grid = (int64_t)clusters * CL;
      if (grid > want * CL) grid = cdiv_h(want, CL) * CL;
      if (grid < CL) grid = CL;
      cfg.gridDim = dim3((unsigned)grid);
      cudaError_t e = cudaLaunchKernelEx(&cfg, kern, a, per);
      return cuda_status(e);
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
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (m > 0) {
    cudaError_t e = cudaMemcpyAsync(out, defaults, (size_t)m * esz[type], cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return cuda_status(e);
  }
  return acc_permute(op, type, src, cval, idx, index_type, out, n, m, stream);
}
