// fold.cu -- the C ABI of fold f z / fold1 f along the innermost dimension;
// the kernels and their design are in fold_impl.cuh.
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
