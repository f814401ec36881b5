// scan_seg.cu -- every scan flavour (scanl1 / scanr1, scanl' / scanr',
// scanl z / scanr z) over the rows of a rank-2 array by the segmented form of
// the persistent L2-re-read scan (scan_l2_kernel with SEG, scan_impl.cuh):
// the [outer x inner] array is one contiguous sequence whose scan restarts at
// every row, so long and short rows alike stream at the 1-D
// scan's rate instead of one CTA (or warp) per row.  The reference scans the
// innermost dimension of a multidimensional array with one thread block per
// row (accelerate-llvm-ptx/src/Data/Array/Accelerate/LLVM/PTX/CodeGen/
// Scan.hs:441-611, mkScanDim); the results are those of a per-row scan.
// Kept in its own translation unit so that its instantiations compile beside
// the others.
#include "scan_impl.cuh"

namespace accgb {

int scan_rows_seg(Workspace *w, int op, int type, int prec, bool r2l, int kind, const void *in, void *out,
                  void *sums, uint64_t seed, int64_t outer, int64_t inner, cudaStream_t s, bool *launched) {
  *launched = false;
  if (op != ACC_ADD && op != ACC_MUL && op != ACC_MIN && op != ACC_MAX) return ACC_OK;
  return with_type(type, [&](auto tv) -> int {
    using T = decltype(tv);
    if (inner < (int64_t)(SCAN_ROW_BYTES / sizeof(T))) return ACC_OK;  // a line may hold one row start at most
    return with_op<T>(op, [&](auto opc) -> int {
      constexpr int OP = decltype(opc)::value;
      if constexpr (OP != ACC_ADD && OP != ACC_MUL && OP != ACC_MIN && OP != ACC_MAX) {
        return ACC_OK;
      } else {
        return with_prec<OP, T>(prec, [&](auto pc) -> int {
          constexpr int P = decltype(pc)::value;
          const T *src = static_cast<const T *>(in);
          T *dst = static_cast<T *>(out);
          const int64_t n = outer * inner;
          if (kind == ACC_SCAN_PRIME) {
            // scanl' / scanr': exclusive, every row from the seed, its total to sums
            T *rs = static_cast<T *>(sums);
            if (r2l)
              return launch_scan_l2<OP, T, P, true, 0, 2>(w, src, dst, nullptr, nullptr, n, true, true, seed, s,
                                                          launched, nullptr, 0, 0, inner, rs);
            return launch_scan_l2<OP, T, P, false, 0, 2>(w, src, dst, nullptr, nullptr, n, true, true, seed, s,
                                                         launched, nullptr, 0, 0, inner, rs);
          }
          if (kind == ACC_SCAN_SEEDED) {
            // scanl z (exclusive, the row's total last) / scanr z (inclusive
            // with the seed on the right, the seed last): rows of inner + 1
            if (r2l)
              return launch_scan_l2<OP, T, P, true, 0, 3>(w, src, dst, nullptr, nullptr, n, true, false, seed, s,
                                                          launched, nullptr, 0, 0, inner);
            return launch_scan_l2<OP, T, P, false, 0, 3>(w, src, dst, nullptr, nullptr, n, true, true, seed, s,
                                                         launched, nullptr, 0, 0, inner);
          }
          if (r2l)
            return launch_scan_l2<OP, T, P, true, 0, 1>(w, src, dst, nullptr, nullptr, n, false, false, 0, s,
                                                        launched, nullptr, 0, 0, inner);
          return launch_scan_l2<OP, T, P, false, 0, 1>(w, src, dst, nullptr, nullptr, n, false, false, 0, s,
                                                       launched, nullptr, 0, 0, inner);
        });
      }
    });
  });
}

}  // namespace accgb
