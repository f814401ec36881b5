// scan_zip.cu -- scans over a fused producer: scanl / scanl1 / scanr /
// scanr1 / scanl' / scanr' f z (zipWith g xs ys), and the same over
// map (\x -> g x c) xs for a constant c.
//
// The reference's scan kernels read a delayed input array: the producer of
// the scan (here \i -> g (xs!i) (ys!i)) is evaluated inside the scan's first
// pass (accelerate-llvm-ptx/src/Data/Array/Accelerate/LLVM/PTX/CodeGen/
// Scan.hs:141-439, the MIRDelayed argument of mkScanAllP1 / mkScanDim).
// Here the scan kernels of scan_impl.cuh read both arrays and zip them as the
// tile arrives, so the zipped array is never written: 12 bytes of traffic per
// Float32 element (two reads, one write) against 20 for zipWith followed by
// scan.  Each zipped element is g x y rounded to the element type, then
// scanned exactly as acc_scan scans an array.
#include "scan_impl.cuh"

using namespace accgb;

namespace {

// f in {+, min, max} and g in {+, *, min, max} over Int32, Int64, Float32 and
// Float64, as for the fused fold.
template <class F> int with_scan_op(int op, F &&f) {
  switch (op) {
    case ACC_ADD: return f(IC<ACC_ADD>{});
    case ACC_MIN: return f(IC<ACC_MIN>{});
    case ACC_MAX: return f(IC<ACC_MAX>{});
    default: return ACC_ERR_UNSUPPORTED;
  }
}
template <class F> int with_zip_type(int type, F &&f) {
  switch (type) {
    case ACC_I32: return f(int32_t{});
    case ACC_I64: return f(int64_t{});
    case ACC_F32: return f(float{});
    case ACC_F64: return f(double{});
    case ACC_U32: return ACC_ERR_UNSUPPORTED;
    default: return ACC_ERR_INVALID;
  }
}

}  // namespace

extern "C" int acc_scan_zipwith(int op, int zop, int type, int prec, int dir, int kind, const void *xs,
                                const void *ys, void *out, void *sums, int64_t outer, int64_t inner,
                                const void *seed, void *stream) {
  if (outer < 0 || inner < 0) return ACC_ERR_INVALID;
  if (op < ACC_ADD || op > ACC_XOR || zop < ACC_ADD || zop > ACC_XOR) return ACC_ERR_INVALID;
  if (dir != ACC_L2R && dir != ACC_R2L) return ACC_ERR_INVALID;
  if (kind < ACC_SCAN_INCLUSIVE || kind > ACC_SCAN_PRIME) return ACC_ERR_INVALID;
  if (kind != ACC_SCAN_INCLUSIVE && !seed) return ACC_ERR_INVALID;
  if (outer == 0) return ACC_OK;
  if (!out && !(inner == 0 && kind != ACC_SCAN_SEEDED)) return ACC_ERR_INVALID;
  if (inner > 0 && (!xs || !ys)) return ACC_ERR_INVALID;
  if (kind == ACC_SCAN_PRIME && !sums) return ACC_ERR_INVALID;
  if (zop != ACC_ADD && zop != ACC_MUL && zop != ACC_MIN && zop != ACC_MAX) return ACC_ERR_UNSUPPORTED;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st = ACC_OK;
  Workspace *w = workspace(s, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  return with_zip_type(type, [&](auto tv) -> int {
    using T = decltype(tv);
    const uint64_t sb = seed_bits<T>(seed);
    return with_scan_op(op, [&](auto opc) -> int {
      constexpr int OP = decltype(opc)::value;
      return with_prec<OP, T>(prec, [&](auto pc) -> int {
        constexpr int P = decltype(pc)::value;
        return scan_typed<OP, T, P, true>(w, dir, kind, static_cast<const T *>(xs), static_cast<T *>(out),
                                          static_cast<T *>(sums), outer, inner, sb, s, static_cast<const T *>(ys),
                                          zop);
      });
    });
  });
}

extern "C" int acc_scan_map(int op, int gop, int type, int prec, int dir, int kind, const void *xs, const void *c,
                            void *out, void *sums, int64_t outer, int64_t inner, const void *seed, void *stream) {
  if (outer < 0 || inner < 0) return ACC_ERR_INVALID;
  if (op < ACC_ADD || op > ACC_XOR || gop < ACC_ADD || gop > ACC_XOR) return ACC_ERR_INVALID;
  if (dir != ACC_L2R && dir != ACC_R2L) return ACC_ERR_INVALID;
  if (kind < ACC_SCAN_INCLUSIVE || kind > ACC_SCAN_PRIME) return ACC_ERR_INVALID;
  if (kind != ACC_SCAN_INCLUSIVE && !seed) return ACC_ERR_INVALID;
  if (!c) return ACC_ERR_INVALID;
  if (outer == 0) return ACC_OK;
  if (!out && !(inner == 0 && kind != ACC_SCAN_SEEDED)) return ACC_ERR_INVALID;
  if (inner > 0 && !xs) return ACC_ERR_INVALID;
  if (kind == ACC_SCAN_PRIME && !sums) return ACC_ERR_INVALID;
  if (gop != ACC_ADD && gop != ACC_MUL && gop != ACC_MIN && gop != ACC_MAX) return ACC_ERR_UNSUPPORTED;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st = ACC_OK;
  Workspace *w = workspace(s, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  return with_zip_type(type, [&](auto tv) -> int {
    using T = decltype(tv);
    const uint64_t sb = seed_bits<T>(seed);
    const uint64_t cb = seed_bits<T>(c);
    return with_scan_op(op, [&](auto opc) -> int {
      constexpr int OP = decltype(opc)::value;
      return with_prec<OP, T>(prec, [&](auto pc) -> int {
        constexpr int P = decltype(pc)::value;
        return scan_typed<OP, T, P, false, true>(w, dir, kind, static_cast<const T *>(xs), static_cast<T *>(out),
                                                 static_cast<T *>(sums), outer, inner, sb, s, nullptr, gop, cb);
      });
    });
  });
}
