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
// Two kernels: the plane-streaming form below for 3x3x3 patterns, and the
// direct form for every other pattern: one thread per output, x fastest across a
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

// The 2.5-D plane-streaming form, for cubic patterns of radius R: a CTA
// owns a 32 x (8 ROWS) tile of columns and a range of planes, and streams
// the planes of its tile's halo through shared memory in increasing order
// (plane p+1 is loaded into registers while plane p is used, then stored to
// the other buffer).  A plane contributes to the 2R+1 outputs it is a tap
// plane of; each thread keeps those outputs' accumulators for its ROWS rows
// in registers and rotates them as the planes go by, so the output of plane
// z is complete (and stored) once plane z+R has been applied.  Every plane is
// read from DRAM once per tile (plus a 2R-plane overlap between a CTA's
// plane range and its neighbours') and from shared memory 2R+1 rows per
// output row.  The planes arrive in increasing order, so each output still
// accumulates its taps planes outer, then rows, then columns, one fused
// multiply-add each, exactly as the direct kernel and the oracle do.
constexpr int S3S_TX = 32, S3S_TY = 8, S3S_ROWS = 4;
constexpr int S3S_OY = S3S_TY * S3S_ROWS;  // output rows per tile

template <class T, int R>
__global__ void __launch_bounds__(S3S_TX * S3S_TY, 3)
stencil3d_stream_kernel(const __grid_constant__ Stencil3Args a, const __grid_constant__ Stencil3W<T> W,
                        int64_t zchunk) {
  constexpr int K = 2 * R + 1;
  constexpr int PW = S3S_TX + 2 * R, PH = S3S_OY + 2 * R;  // halo plane tile
  constexpr int PN = PW * PH;
  constexpr int NT = S3S_TX * S3S_TY;
  constexpr int PER = (PN + NT - 1) / NT;  // plane cells loaded per thread
  __shared__ T plane[2][PH][PW];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * S3S_TX + tx;
  const int64_t x0 = (int64_t)blockIdx.x * S3S_TX, y0 = (int64_t)blockIdx.y * S3S_OY;
  const int64_t z0 = (int64_t)blockIdx.z * zchunk;
  int64_t z1 = z0 + zchunk;
  if (z1 > a.d) z1 = a.d;
  if (z0 >= z1) return;
  const T *in = static_cast<const T *>(a.in);
  T *out = static_cast<T *>(a.out);
  const T cval = from_bits<T>(a.cval);
  const int b = a.boundary;
  const bool inside_xy = x0 - R >= 0 && x0 + S3S_TX + R <= a.w && y0 - R >= 0 && y0 + S3S_OY + R <= a.h;
  // The weights are read where they lie (kernel parameters, compile-time
  // indices), not copied to registers.
  // The halo cells of virtual plane p (which may lie outside [0, d)).
  auto fetch = [&](int64_t p, T (&v)[PER]) {
    const bool pin = p >= 0 && p < a.d;
    const bool pconst = !pin && b == ACC_CONSTANT;
    const int64_t zr = pin ? p : bound_index(p, a.d, b);
    const T *pl = in + zr * a.h * a.w;
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int q = tid + u * NT;
      v[u] = cval;
      if (q < PN && !pconst) {
        const int sy = q / PW, sx = q % PW;
        const int64_t gy = y0 - R + sy, gx = x0 - R + sx;
        if (inside_xy) {
          v[u] = pl[gy * a.w + gx];
        } else {
          const bool yin = gy >= 0 && gy < a.h, xin = gx >= 0 && gx < a.w;
          if (b != ACC_CONSTANT || (yin && xin))
            v[u] = pl[(yin ? gy : bound_index(gy, a.h, b)) * a.w + (xin ? gx : bound_index(gx, a.w, b))];
        }
      }
    }
  };
  auto put = [&](int buf, const T (&v)[PER]) {
#pragma unroll
    for (int u = 0; u < PER; ++u) {
      const int q = tid + u * NT;
      if (q < PN) plane[buf][q / PW][q % PW] = v[u];
    }
  };

  // acc[k][r]: output plane (p - R + k) of the plane p being applied, row r
  T acc[K][S3S_ROWS];
#pragma unroll
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int r = 0; r < S3S_ROWS; ++r) acc[k][r] = Prim<ACC_ADD, T>::id();
  T v[PER];
  fetch(z0 - R, v);
  put(0, v);
  __syncthreads();
  const int64_t pend = z1 - 1 + R;
  int cur = 0;
  for (int64_t p = z0 - R; p <= pend; ++p) {
    if (p < pend) fetch(p + 1, v);  // the next plane's loads run during this plane's taps
    // plane p: weight plane (p - z) + R for output z = p - R + k is 2R - k
#pragma unroll
    for (int ir = 0; ir < S3S_ROWS + 2 * R; ++ir) {
      T xv[K];
#pragma unroll
      for (int dx = 0; dx < K; ++dx) xv[dx] = plane[cur][ty * S3S_ROWS + ir][tx + dx];
#pragma unroll
      for (int dyi = 0; dyi < K; ++dyi) {
        const int r = ir - dyi;
        if (r < 0 || r >= S3S_ROWS) continue;
#pragma unroll
        for (int k = 0; k < K; ++k) {
#pragma unroll
          for (int dx = 0; dx < K; ++dx) {
            const T wk = W.w[((2 * R - k) * K + dyi) * K + dx];
            if (wk == T(0)) continue;
            acc[k][r] = fma_tap(wk, xv[dx], acc[k][r]);
          }
        }
      }
    }
    // output plane p - R is complete
    const int64_t zo = p - R;
    if (zo >= z0) {
      const int64_t gx = x0 + tx;
#pragma unroll
      for (int r = 0; r < S3S_ROWS; ++r) {
        const int64_t gy = y0 + ty * S3S_ROWS + r;
        if (gx < a.w && gy < a.h) out[(zo * a.h + gy) * a.w + gx] = acc[0][r];
      }
    }
#pragma unroll
    for (int k = 0; k + 1 < K; ++k)
#pragma unroll
      for (int r = 0; r < S3S_ROWS; ++r) acc[k][r] = acc[k + 1][r];
#pragma unroll
    for (int r = 0; r < S3S_ROWS; ++r) acc[K - 1][r] = Prim<ACC_ADD, T>::id();
    if (p < pend) {
      put(cur ^ 1, v);  // the other buffer: last read one plane ago, before the barrier below
      __syncthreads();
      cur ^= 1;
    }
  }
}

template <class T>
int stencil3d_typed(const Stencil3Args &a, const void *weights, cudaStream_t s) {
  Stencil3W<T> W;
  memset(&W, 0, sizeof(W));
  const int n = (2 * a.rz + 1) * (2 * a.ry + 1) * (2 * a.rx + 1);
  memcpy(W.w, weights, (size_t)n * sizeof(T));
  if (a.rz == 1 && a.ry == 1 && a.rx == 1) {
    // 3x3x3: the plane-streaming kernel.  Plane ranges split so that the grid
    // has about 8 CTAs per SM.
    const int64_t sx = cdiv_h(a.w, S3S_TX), sy = cdiv_h(a.h, S3S_OY);
    if (sx <= 0x7fffffffll && sy <= 65535) {
      const int64_t want = (int64_t)device_info().sms * 8;
      int64_t nz = cdiv_h(want, sx * sy);
      if (nz > a.d) nz = a.d;
      if (nz > 65535) nz = 65535;
      if (nz < 1) nz = 1;
      const int64_t zchunk = cdiv_h(a.d, nz);
      nz = cdiv_h(a.d, zchunk);
      dim3 grid((unsigned)sx, (unsigned)sy, (unsigned)nz), block(S3S_TX, S3S_TY);
      stencil3d_stream_kernel<T, 1><<<grid, block, 0, s>>>(a, W, zchunk);
      return check_launch();
    }
  }
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
