// fold_zip.cu -- fold over a fused producer: fold f z (zipWith g xs ys) and
// fold f z (map (\x -> g x c) xs).
//
// The reference fuses the producer of a fold into the fold's first kernel:
// its input is a delayed array, e.g. the function \i -> xs!i * ys!i of
// `dotp xs ys = fold (+) 0 (zipWith (*) xs ys)`, read inside the reduction
// (accelerate-llvm-ptx/src/Data/Array/Accelerate/LLVM/PTX/CodeGen/Fold.hs:80-97,
// mkFoldAll's MIRDelayed input).  Here the fold kernels read both arrays with
// 16-byte vector loads and apply the primitive g element by element before
// the accumulation, so the zipped array is never written: 2 x 4 bytes per
// Float32 element of traffic.  Each zipped element is g x y rounded to the
// element type, as the fused kernel computes it, and then folded exactly as
// acc_fold folds an array (Float32 (+) compensated by default).  A map with a
// constant operand (the reference's own known answer is
// `A.sum (A.map (+1) xs)`, accelerate-llvm-ptx/test/nofib/Data/Array/
// Accelerate/LLVM/PTX/NoFib/RunQ.hs:29) is applied the same way to each
// element as it is loaded: 4 bytes per Float32 element.
#include "fold_impl.cuh"

using namespace accgb;

namespace {

// The fused entry covers f in {+, min, max} and g in {+, *, min, max} over
// Int32, Int64, Float32 and Float64: the producers of dot products, sums of
// elementwise extremes and the like.
template <class F> int with_fold_op(int op, F &&f) {
  switch (op) {
    case ACC_ADD: return f(IC<ACC_ADD>{});
    case ACC_MIN: return f(IC<ACC_MIN>{});
    case ACC_MAX: return f(IC<ACC_MAX>{});
    default: return ACC_ERR_UNSUPPORTED;
  }
}
template <class F> int with_zip_op(int zop, F &&f) {
  switch (zop) {
    case ACC_ADD: return f(IC<ACC_ADD>{});
    case ACC_MUL: return f(IC<ACC_MUL>{});
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

extern "C" int acc_fold_zipwith(int op, int zop, int type, int prec, const void *xs, const void *ys, void *out,
                                int64_t outer, int64_t inner, const void *seed, void *stream) {
  if (outer < 0 || inner < 0) return ACC_ERR_INVALID;
  if (op < ACC_ADD || op > ACC_XOR || zop < ACC_ADD || zop > ACC_XOR) return ACC_ERR_INVALID;
  if (outer == 0) return ACC_OK;
  if (!out) return ACC_ERR_INVALID;
  if (inner == 0 && !seed) return ACC_ERR_EMPTY;  // fold1 of an empty row
  if (inner > 0 && (!xs || !ys)) return ACC_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st = ACC_OK;
  Workspace *w = workspace(s, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  return with_zip_type(type, [&](auto tv) -> int {
    using T = decltype(tv);
    const uint64_t sb = seed_bits<T>(seed);
    return with_fold_op(op, [&](auto opc) -> int {
      constexpr int OP = decltype(opc)::value;
      return with_zip_op(zop, [&](auto zc) -> int {
        constexpr int ZOP = decltype(zc)::value;
        if (inner == 0) return launch_fill<T>(static_cast<T *>(out), outer, sb, s);
        return with_prec<OP, T>(prec, [&](auto pc) -> int {
          constexpr int P = decltype(pc)::value;
          return fold_typed<OP, T, P, ZOP>(w, static_cast<const T *>(xs), static_cast<T *>(out), outer, inner,
                                           seed != nullptr, sb, s, static_cast<const T *>(ys));
        });
      });
    });
  });
}

extern "C" int acc_fold_map(int op, int gop, int type, int prec, const void *xs, const void *c, void *out,
                            int64_t outer, int64_t inner, const void *seed, void *stream) {
  if (outer < 0 || inner < 0) return ACC_ERR_INVALID;
  if (op < ACC_ADD || op > ACC_XOR || gop < ACC_ADD || gop > ACC_XOR) return ACC_ERR_INVALID;
  if (!c) return ACC_ERR_INVALID;
  if (outer == 0) return ACC_OK;
  if (!out) return ACC_ERR_INVALID;
  if (inner == 0 && !seed) return ACC_ERR_EMPTY;  // fold1 of an empty row
  if (inner > 0 && !xs) return ACC_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st = ACC_OK;
  Workspace *w = workspace(s, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  return with_zip_type(type, [&](auto tv) -> int {
    using T = decltype(tv);
    const uint64_t sb = seed_bits<T>(seed);
    const uint64_t cb = seed_bits<T>(c);
    return with_fold_op(op, [&](auto opc) -> int {
      constexpr int OP = decltype(opc)::value;
      return with_zip_op(gop, [&](auto gc) -> int {
        constexpr int ZOP = MAP_BASE + decltype(gc)::value;
        if (inner == 0) return launch_fill<T>(static_cast<T *>(out), outer, sb, s);
        return with_prec<OP, T>(prec, [&](auto pc) -> int {
          constexpr int P = decltype(pc)::value;
          return fold_typed<OP, T, P, ZOP>(w, static_cast<const T *>(xs), static_cast<T *>(out), outer, inner,
                                           seed != nullptr, sb, s, nullptr, cb);
        });
      });
    });
  });
}
