// stencil3d.cu -- weighted-sum stencils over rank-3 arrays [planes][rows]
// [columns] with clamp / mirror / wrap / constant boundaries.
//
// The reference's rank-3 stencil (stencil1Op / stencilCore on a DIM3 array,
// accelerate-llvm-ptx/src/Data/Array/Accelerate/LLVM/PTX/Execute.hs:652-776)
// reads a pattern that is a tuple of rank-2 patterns over the outermost index
// (StencilRtup*, accelerate-llvm/src/Data/Array/Accelerate/LLVM/CodeGen/
// Stencil.hs:126-180, which recurse on the left-most index component), so its
// taps run planes outer, then rows, then columns, each -r..r; every index
// component is remapped by the boundary (CodeGen/Stencil.hs:195-253).
//
// This is the first, direct form: one thread per output, x fastest across a
// warp (coalesced loads and stores), every tap a load through L1/L2, the
// accumulator started at the additive identity and advanced by one fused
// multiply-add per tap in tap order (bit-identical to a sequential C
// evaluation with C99 fma).  Taps whose weight is exactly zero are not part
// of the pattern and are not read.  Every tap index is remapped into the
// array before it is read, so no load leaves the input.  The 3x3x3 pattern
// has its own instantiation with the loops unrolled and the 27 weights in
// registers.
#include "stencil_common.cuh"

namespace accgb {

constexpr int S3_MAXR = 4;                        // radius limit per dimension (9-wide patterns)
constexpr int S3_MAXK = (2 * S3_MAXR + 1) * (2 * S3_MAXR + 1) * (2 * S3_MAXR + 1);
constexpr int S3_BX = 32, S3_BY = 8;              // outputs per block: 32 columns x 8 rows

// The weights travel as a kernel parameter (up to 5.8 KB), read in place
// (__grid_constant__) whatever the index.
template <class T> struct Stencil3W { T w[S3_MAXK]; };

struct Stencil3Args {
  const void *in;
  void *out;
  int64_t d, h, w;  // extent (planes, rows, columns); the input has the same extent
  int rz, ry, rx;
  int boundary;
  uint64_t cval;
};

// KR > 0: every radius is KR (taps unrolled); KR == 0: radii from the args.
template <class T, int KR>
__global__ void __launch_bounds__(S3_BX * S3_BY)
stencil3d_kernel(const __grid_constant__ Stencil3Args a, const __grid_constant__ Stencil3W<T> W) {
  const int64_t x = (int64_t)blockIdx.x * S3_BX + threadIdx.x;
  if (x >= a.w) return;
  const T *in = static_cast<const T *>(a.in);
  T *out = static_cast<T *>(a.out);
  const T cval = from_bits<T>(a.cval);
  const int b = a.boundary;
  const int rz = KR > 0 ? KR : a.rz, ry = KR > 0 ? KR : a.ry, rx = KR > 0 ? KR : a.rx;
  const int ky = 2 * ry + 1, kx = 2 * rx + 1;
  for (int64_t z = blockIdx.z; z < a.d; z += gridDim.z) {
    for (int64_t y = (int64_t)blockIdx.y * S3_BY + threadIdx.y; y < a.h; y += (int64_t)gridDim.y * S3_BY) {
      T acc = Prim<ACC_ADD, T>::id();
#pragma unroll
      for (int dz = -rz; dz <= rz; ++dz) {
        const int64_t zz = z + dz;
        const bool zin = zz >= 0 && zz < a.d;
        const int64_t zr = zin ? zz : bound_index(zz, a.d, b);
#pragma unroll
        for (int dy = -ry; dy <= ry; ++dy) {
          const int64_t yy = y + dy;
          const bool yin = yy >= 0 && yy < a.h;
          const int64_t yr = yin ? yy : bound_index(yy, a.h, b);
          const T *row = in + (zr * a.h + yr) * a.w;
#pragma unroll
          for (int dx = -rx; dx <= rx; ++dx) {
            const T wk = W.w[((dz + rz) * ky + (dy + ry)) * kx + (dx + rx)];
            if (wk == T(0)) continue;
            const int64_t xx = x + dx;
            const bool xin = xx >= 0 && xx < a.w;
            const T v = (b == ACC_CONSTANT && !(zin && yin && xin)) ? cval
                                                                      : row[xin ? xx : bound_index(xx, a.w, b)];
            acc = fma_tap(wk, v, acc);
          }
        }
      }
      out[(z * a.h + y) * a.w + x] = acc;
    }
  }
}

template <class T>
int stencil3d_typed(const Stencil3Args &a, const void *weights, cudaStream_t s) {
  Stencil3W<T> W;
  memset(&W, 0, sizeof(W));
  const int n = (2 * a.rz + 1) * (2 * a.ry + 1) * (2 * a.rx + 1);
  memcpy(W.w, weights, (size_t)n * sizeof(T));
  const int64_t gx = cdiv_h(a.w, S3_BX);
  if (gx > 0x7fffffffll) return ACC_ERR_TOO_LARGE;
  int64_t gy = cdiv_h(a.h, S3_BY);
  if (gy > 65535) gy = 65535;  // the rows loop covers the rest
  int64_t gz = a.d > 65535 ? 65535 : a.d;
  dim3 grid((unsigned)gx, (unsigned)gy, (unsigned)gz), block(S3_BX, S3_BY);
  if (a.rz == 1 && a.ry == 1 && a.rx == 1)
    stencil3d_kernel<T, 1><<<grid, block, 0, s>>>(a, W);
  else
    stencil3d_kernel<T, 0><<<grid, block, 0, s>>>(a, W);
  return check_launch();
}

}  // namespace accgb

using namespace accgb;

extern "C" int acc_stencil3d(int type, int rz, int ry, int rx, const void *weights, int boundary, const void *cval,
                             const void *in, void *out, int64_t d, int64_t h, int64_t w, void *stream) {
  if (rz < 0 || rz > S3_MAXR || ry < 0 || ry > S3_MAXR || rx < 0 || rx > S3_MAXR) return ACC_ERR_INVALID;
  if (d < 0 || h < 0 || w < 0) return ACC_ERR_INVALID;
  if (boundary < ACC_CLAMP || boundary > ACC_CONSTANT) return ACC_ERR_INVALID;
  if (boundary == ACC_CONSTANT && !cval) return ACC_ERR_INVALID;
  if (type != ACC_F32 && type != ACC_F64 && type != ACC_I32 && type != ACC_I64) return ACC_ERR_UNSUPPORTED;
  if (d == 0 || h == 0 || w == 0) return ACC_OK;
  if (!weights || !in || !out) return ACC_ERR_INVALID;
  Stencil3Args a{};
  a.in = in; a.out = out; a.d = d; a.h = h; a.w = w;
  a.rz = rz; a.ry = ry; a.rx = rx; a.boundary = boundary;
  a.cval = 0;
  if (cval) memcpy(&a.cval, cval, (type == ACC_F64 || type == ACC_I64) ? 8 : 4);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (type) {
    case ACC_F32: return stencil3d_typed<float>(a, weights, s);
    case ACC_F64: return stencil3d_typed<double>(a, weights, s);
    case ACC_I32: return stencil3d_typed<int32_t>(a, weights, s);
    default: return stencil3d_typed<int64_t>(a, weights, s);
  }
}
