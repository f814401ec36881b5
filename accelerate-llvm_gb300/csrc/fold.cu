// fold.cu -- fold f z / fold1 f along the innermost dimension.
//
// The reference reduces a vector with a host-driven chain of launches
// (foldAllM1, then foldAllM2 re-launched until one element is left:
// accelerate-llvm-ptx/src/Data/Array/Accelerate/LLVM/PTX/Execute.hs:267-318,
// PTX/CodeGen/Fold.hs:175-285) and a rank >= 2 array with one CTA per row
// (Fold.hs:296-405).  Here every shape is one launch:
//   * fold_rows_thread  -- inner <= 16: one thread per row;
//   * fold_rows_warp    -- short rows, many of them: one warp per row;
//   * fold_split        -- long rows: a row is cut over G CTAs, each thread
//                          streams 16-byte vectors (4 in flight), the CTA
//                          partial goes to scratch, and the last CTA of the
//                          row (atomic ticket) folds the G partials in order
//                          and applies the seed.
// The seed combines on the left, z `f` (x0 `f` ...), as reduceFromTo does
// (accelerate-llvm-native/.../Native/CodeGen/Fold.hs:248-260).  Float32 (+)
// accumulates with a compensated two-sum by default.
#include "fold_impl.cuh"


using namespace accgb;

extern "C" int acc_fold(int op, int type, int prec, const void *in, void *out, int64_t outer,
                        int64_t inner, const void *seed, void *stream) {
  if (outer < 0 || inner < 0) return ACC_ERR_INVALID;
  if (outer == 0) return ACC_OK;
  if (!out) return ACC_ERR_INVALID;
  // fold1 of an empty innermost extent (PTX/Execute.hs:232 boundsCheck).
  if (inner == 0 && !seed) return ACC_ERR_EMPTY;
  if (inner > 0 && !in) return ACC_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st = ACC_OK;
  Workspace *w = workspace(s, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  return with_type(type, [&](auto tv) -> int {
    using T = decltype(tv);
    const uint64_t sb = seed_bits<T>(seed);
    if (inner == 0) return launch_fill<T>(static_cast<T *>(out), outer, sb, s);  // PTX/Execute.hs:248
    return with_op<T>(op, [&](auto opc) -> int {
      constexpr int OP = decltype(opc)::value;
      return with_prec<OP, T>(prec, [&](auto pc) -> int {
        constexpr int P = decltype(pc)::value;
        return fold_typed<OP, T, P>(w, static_cast<const T *>(in), static_cast<T *>(out), outer, inner,
                                    seed != nullptr, sb, s);
      });
    });
  });
}
