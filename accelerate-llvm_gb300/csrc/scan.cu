// scan.cu -- the C ABI of the scans (acc_scan, acc_scan_noalloc), the fill
// kernel of empty scans and folds, and the offsets scan of foldSeg.  The
// kernels are in scan_impl.cuh.
#include "scan_impl.cuh"

namespace accgb {

template <class T>
__global__ void fill_kernel(T *out, int64_t n, uint64_t bits) {
  const T v = from_bits<T>(bits);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) out[i] = v;
}

template <class T>
int launch_fill(T *out, int64_t n, uint64_t bits, cudaStream_t s) {
  if (n <= 0) return ACC_OK;
  int64_t blocks = cdiv_h(n, 256);
  if (blocks > 4096) blocks = 4096;
  fill_kernel<T><<<(unsigned)blocks, 256, 0, s>>>(out, n, bits);
  return check_launch();
}
template int launch_fill<int32_t>(int32_t *, int64_t, uint64_t, cudaStream_t);
template int launch_fill<int64_t>(int64_t *, int64_t, uint64_t, cudaStream_t);
template int launch_fill<uint32_t>(uint32_t *, int64_t, uint64_t, cudaStream_t);
template int launch_fill<float>(float *, int64_t, uint64_t, cudaStream_t);
template int launch_fill<double>(double *, int64_t, uint64_t, cudaStream_t);

// Exclusive `scanl (+) 0` of segment lengths into offsets (nseg+1 values),
// used by acc_fold_seg_lengths.
int scan_offsets(Workspace *w, int type, const void *lengths, void *offsets, int64_t nseg, cudaStream_t s) {
  if (type == ACC_I32)
    return launch_scan_1d<ACC_ADD, int32_t, 0, false>(w, (const int32_t *)lengths, (int32_t *)offsets,
                                                       (int32_t *)offsets + nseg, nullptr, nseg, true, true, 0, s);
  if (type == ACC_I64)
    return launch_scan_1d<ACC_ADD, int64_t, 0, false>(w, (const int64_t *)lengths, (int64_t *)offsets,
                                                       (int64_t *)offsets + nseg, nullptr, nseg, true, true, 0, s);
  return ACC_ERR_INVALID;
}

}  // namespace accgb

using namespace accgb;

extern "C" int acc_scan(int op, int type, int prec, int dir, int kind, const void *in, void *out,
                        void *sums, int64_t outer, int64_t inner, const void *seed, void *stream) {
  if (outer < 0 || inner < 0) return ACC_ERR_INVALID;
  if (dir != ACC_L2R && dir != ACC_R2L) return ACC_ERR_INVALID;
  if (kind < ACC_SCAN_INCLUSIVE || kind > ACC_SCAN_PRIME) return ACC_ERR_INVALID;
  if (kind != ACC_SCAN_INCLUSIVE && !seed) return ACC_ERR_INVALID;
  if (outer == 0) return ACC_OK;
  if (!out && !(inner == 0 && kind != ACC_SCAN_SEEDED)) return ACC_ERR_INVALID;
  if (inner > 0 && !in) return ACC_ERR_INVALID;
  if (kind == ACC_SCAN_PRIME && !sums) return ACC_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st = ACC_OK;
  Workspace *w = workspace(s, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  return with_type(type, [&](auto tv) -> int {
    using T = decltype(tv);
    const uint64_t sb = seed_bits<T>(seed);
    return with_op<T>(op, [&](auto opc) -> int {
      constexpr int OP = decltype(opc)::value;
      return with_prec<OP, T>(prec, [&](auto pc) -> int {
        constexpr int P = decltype(pc)::value;
        return scan_typed<OP, T, P>(w, dir, kind, static_cast<const T *>(in), static_cast<T *>(out),
                                    static_cast<T *>(sums), outer, inner, sb, s);
      });
    });
  });
}

// --------------------------------------------------------------------------
// acc_scan_noalloc: the same scan for callers that may not allocate device
// memory.  An integration that runs under a fixed device-memory budget, a
// plugin whose host process hands out all device memory from its own pool
// allocator, or a latency-bound loop that must not stall on cudaMalloc (which
// can synchronise the device) cannot have this library call cudaMalloc behind
// its back, which the per-stream workspace of acc_scan does on first use and
// whenever an array needs more look-back slots.  This entry point keeps its
// scratch (look-back status slots, tile ticket, error word) in one
// file-scope device array instead, sized for NOALLOC_MAX_TILES tiles: 2 MiB
// plus 256 bytes, held by every GPU that loads the library until the process
// exits.  It therefore scans at most NOALLOC_MAX_ELEMS = 2^28 elements per
// row and rejects longer rows with ACC_ERR_TOO_LARGE.
namespace accgb {

constexpr int64_t NOALLOC_MAX_TILES = 1 << 17;
constexpr int64_t NOALLOC_MAX_ELEMS = 1ll << 28;
constexpr int NOALLOC_WORDS = 64;  // [0] error word, [1] tile ticket

struct NoallocScratch {
  uint64_t status[2 * NOALLOC_MAX_TILES];
  uint32_t words[NOALLOC_WORDS];
};
static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

struct NoallocDevice {
  NoallocScratch *ptr = nullptr;  // device address of g_noalloc_scratch
};

// Set-up, once per device, with that device current: the device address of
// the scratch array (the host-side symbol is only a stand-in for it).
static int noalloc_setup(NoallocDevice **out) {
  static std::mutex mu;
  static NoallocDevice devs[64];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e);
  if (dev < 0 || dev >= 64) return ACC_ERR_INVALID;
  std::lock_guard<std::mutex> lk(mu);
  NoallocDevice &d = devs[dev];
  if (!d.ptr) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_status(e);
    d.ptr = static_cast<NoallocScratch *>(p);
  }
  *out = &d;
  return ACC_OK;
}

template <int OP, class T, int PREC, bool R2L>
static int noalloc_scan_1d(NoallocDevice *nd, const T *in, T *out, T *total_out, T *seed_out, int64_t n,
                           bool has_seed, bool exclusive, uint64_t seed, cudaStream_t s) {
  constexpr int ITEMS = SCAN_ROW_BYTES / sizeof(T);
  constexpr int SUB = 2;
  CUtensorMap tin, tout;
  memset(&tin, 0, sizeof(tin));
  memset(&tout, 0, sizeof(tout));
  const int64_t full_rows = n / ITEMS;
  const bool tma = full_rows > 0 &&
                   encode_2d(&tin, in, sizeof(T), ITEMS, full_rows, SCAN_ROW_BYTES, ITEMS, SCAN_THREADS, true) &&
                   encode_2d(&tout, out, sizeof(T), ITEMS, full_rows, SCAN_ROW_BYTES, ITEMS, SCAN_THREADS, true);
  const int64_t tile_elems = (int64_t)(tma ? SUB : 1) * SCAN_THREADS * ITEMS;
  const int64_t ntiles = cdiv_h(n, tile_elems);
  if (ntiles > NOALLOC_MAX_TILES) return ACC_ERR_TOO_LARGE;
  // The array keeps the previous call's contents.  Before the launch, in
  // stream order, the ticket and the error word are set to zero and so are
  // the status slots of this call's tiles: a slot then holds a tag of this
  // call (epoch 1) only once one of its tiles has published, whatever an
  // earlier call left there.  The clearing is 16 bytes per tile of 16 to 64
  // KiB, and no epoch is kept on the host, so no host state changes between
  // calls.
  cudaError_t e = cudaMemsetAsync(nd->ptr->words, 0, sizeof(nd->ptr->words), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(nd->ptr->status, 0, (size_t)ntiles * 2 * sizeof(uint64_t), s);
  if (e != cudaSuccess) return cuda_status(e);
  ScanArgs a{};
  a.in = in; a.out = out; a.total_out = total_out; a.seed_out = seed_out;
  a.n = n;
  a.full_rows = full_rows;
  a.ntiles = ntiles;
  a.seed = seed;
  a.status = nd->ptr->status;
  a.ticket = nd->ptr->words + 1;
  a.err = nd->ptr->words + 0;
  a.epoch = 1;
  a.has_seed = has_seed;
  a.exclusive = exclusive;
  a.tma_in = a.tma_out = tma;
  if (tma) {
    const size_t smem = (size_t)SUB * SCAN_THREADS * SCAN_ROW_BYTES + 1024;
    auto kern = scan_tma_kernel<OP, T, PREC, R2L, SUB>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kern<<<(unsigned)ntiles, SCAN_THREADS, smem, s>>>(tin, tout, a);
    return check_launch();
  }
  auto kern = scan_lookback_kernel<OP, T, PREC, R2L>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SCAN_SMEM);
  kern<<<(unsigned)ntiles, SCAN_THREADS, SCAN_SMEM, s>>>(a);
  return check_launch();
}

}  // namespace accgb

extern "C" int acc_scan_noalloc(int op, int type, int prec, int dir, int kind, const void *in, void *out,
                                void *sums, int64_t outer, int64_t inner, const void *seed, void *stream) {
  if (outer < 0 || inner < 0) return ACC_ERR_INVALID;
  if (inner > NOALLOC_MAX_ELEMS) return ACC_ERR_TOO_LARGE;
  if (dir != ACC_L2R && dir != ACC_R2L) return ACC_ERR_INVALID;
  if (kind < ACC_SCAN_INCLUSIVE || kind > ACC_SCAN_PRIME) return ACC_ERR_INVALID;
  if (kind != ACC_SCAN_INCLUSIVE && !seed) return ACC_ERR_INVALID;
  if (outer == 0) return ACC_OK;
  if (!out && !(inner == 0 && kind != ACC_SCAN_SEEDED)) return ACC_ERR_INVALID;
  if (inner > 0 && !in) return ACC_ERR_INVALID;
  if (kind == ACC_SCAN_PRIME && !sums) return ACC_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  NoallocDevice *nd = nullptr;
  int st = noalloc_setup(&nd);
  if (st) return st;
  return with_type(type, [&](auto tv) -> int {
    using T = decltype(tv);
    const uint64_t sb = seed_bits<T>(seed);
    return with_op<T>(op, [&](auto opc) -> int {
      constexpr int OP = decltype(opc)::value;
      return with_prec<OP, T>(prec, [&](auto pc) -> int {
        constexpr int P = decltype(pc)::value;
        const T *tin = static_cast<const T *>(in);
        T *tout = static_cast<T *>(out);
        T *tsums = static_cast<T *>(sums);
        const bool r2l = dir == ACC_R2L;
        if (inner == 0) {
          if (kind == ACC_SCAN_SEEDED) return launch_fill<T>(tout, outer, sb, s);
          if (kind == ACC_SCAN_PRIME) return launch_fill<T>(tsums, outer, sb, s);
          return ACC_OK;
        }
        const bool exclusive = kind == ACC_SCAN_PRIME || (kind == ACC_SCAN_SEEDED && !r2l);
        if (outer > 1) {
          // Rows of a rank >= 2 array use the row kernel, which needs no scratch.
          RowScanArgs ra{};
          ra.in = tin; ra.out = tout; ra.sums = kind == ACC_SCAN_PRIME ? tsums : nullptr;
          ra.outer = outer; ra.inner = inner;
          ra.in_pitch = inner;
          ra.out_pitch = kind == ACC_SCAN_SEEDED ? inner + 1 : inner;
          ra.seed = sb; ra.has_seed = kind != ACC_SCAN_INCLUSIVE; ra.exclusive = exclusive;
          ra.seed_at_end = kind == ACC_SCAN_SEEDED && r2l;
          ra.total_at_end = kind == ACC_SCAN_SEEDED && !r2l;
          if (r2l) return launch_scan_rows<OP, T, P, true>(ra, s);
          return launch_scan_rows<OP, T, P, false>(ra, s);
        }
        T *total_out = nullptr, *seed_out = nullptr;
        if (kind == ACC_SCAN_SEEDED && !r2l) total_out = tout + inner;
        if (kind == ACC_SCAN_SEEDED && r2l) seed_out = tout + inner;
        if (kind == ACC_SCAN_PRIME) total_out = tsums;
        const bool seeded = kind != ACC_SCAN_INCLUSIVE;
        if (r2l)
          return noalloc_scan_1d<OP, T, P, true>(nd, tin, tout, total_out, seed_out, inner, seeded, exclusive, sb, s);
        return noalloc_scan_1d<OP, T, P, false>(nd, tin, tout, total_out, seed_out, inner, seeded, exclusive, sb, s);
      });
    });
  });
}

extern "C" int acc_scan_noalloc_status(void *stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e);
  NoallocDevice *nd = nullptr;
  int st = noalloc_setup(&nd);
  if (st) return st;
  uint32_t err = 0;
  e = cudaMemcpy(&err, nd->ptr->words + 0, sizeof(err), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e);
  return (err & DEV_ERR_TIMEOUT) ? ACC_ERR_TIMEOUT : ACC_OK;
}
