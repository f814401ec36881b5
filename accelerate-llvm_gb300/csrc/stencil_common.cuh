// stencil_common.cuh -- the boundary remap and the tap of the weighted-sum
// stencils, shared by the rank-1/2 kernels (stencil.cu) and the rank-3
// kernel (stencil3d.cu).
#pragma once

#include "common.cuh"

namespace accgb {

// Index i of an extent n under the boundary rule b
// (accelerate-llvm/src/Data/Array/Accelerate/LLVM/CodeGen/Stencil.hs:224-253):
// clamp i<0 -> 0, i>=n -> n-1; mirror i<0 -> -i, i>=n -> 2n-i-2; wrap i<0 ->
// n+i, i>=n -> i-n.  The constant rule reads no element (callers substitute
// the constant); it falls through to the final clamp.
__device__ __forceinline__ int64_t bound_index(int64_t i, int64_t n, int b) {
  if (i < 0) {
    if (b == ACC_CLAMP) i = 0;
    else if (b == ACC_MIRROR) i = -i;
    else if (b == ACC_WRAP) i = n + i;
  } else if (i >= n) {
    if (b == ACC_CLAMP) i = n - 1;
    else if (b == ACC_MIRROR) i = n - (i - n + 2);
    else if (b == ACC_WRAP) i = i - n;
  }
  // Radii larger than the extent: the reference's remap would step out of
  // the array again; keep the read inside it.
  return i < 0 ? 0 : (i >= n ? n - 1 : i);
}

// One tap: acc + w*x, fused (a single rounding) for floats, wrapping for ints.
template <class T> __device__ __forceinline__ T fma_tap(T w, T x, T acc) {
  if constexpr (std::is_same<T, float>::value) return __fmaf_rn(w, x, acc);
  else if constexpr (std::is_same<T, double>::value) return __fma_rn(w, x, acc);
  else { using U = typename IntBits<T>::U; return (T)((U)acc + (U)w * (U)x); }
}

}  // namespace accgb
