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
#include <cmath>

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

// The 2.5-D plane-streaming form, for 3x3x3 patterns: a CTA owns a 32 x 32
// tile of columns and rows and a range of planes, and streams the planes of
// its tile's halo through a ring of S3S_STAGES shared-memory buffers in
// increasing order, S3S_STAGES - 1 planes loading (cp.async, no registers
// held) while one is used.  A plane contributes to the 3 outputs it is a tap
// plane of; each thread keeps those outputs' accumulators for its 4 rows in
// registers and rotates them as the planes go by, so the output of plane z is
// complete (and stored) once plane z+1 has been applied.  Every plane is read
// from DRAM once per tile (plus a 2-plane overlap between a CTA's plane range
// and its neighbours') and from shared memory 3 rows per output row.  The
// planes arrive in increasing order, so each output still accumulates its
// taps planes outer, then rows, then columns, one fused multiply-add each,
// exactly as the direct kernel and the oracle do.
//
// A buffer row holds columns x0-PX .. x0+32+PX-1 (PX = 16 bytes of elements,
// so each row starts on a 16-byte boundary); rows whose columns all lie in
// the array are copied in 16-byte pieces when the array's rows are 16-byte
// aligned, the rest element by element with each index remapped by the
// boundary (constant-boundary cells outside the array are written directly).
// PAT selects the taps at compile time: 0 = all 27 weights non-zero, 1 = the
// 7-point star (centre and the six face neighbours), 2 = any pattern (each tap
// tested against a mask of the non-zero weights).
// Output rows per thread: 4 (a tile of 32 x 32 outputs).  Measured on a
// GB300, 512^3 Float32: 8 rows per thread (80 registers, 3 CTAs per SM)
// 0.43 ms against 0.38 ms for 4 rows (64 registers, 4 CTAs per SM).
constexpr int S3S_TX = 32, S3S_TY = 8, S3S_ROWS = 4, S3S_STAGES = 4;
constexpr int S3S_OY = S3S_TY * S3S_ROWS;  // output rows per tile
constexpr int S3S_THREADS = S3S_TX * S3S_TY;

__device__ __forceinline__ void cp_async_16(void *dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
template <int B> __device__ __forceinline__ void cp_async_el(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_addr(dst)), "l"(src), "n"(B) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <int PAT> __device__ __forceinline__ bool s3_tap(int t, uint32_t mask) {
  if constexpr (PAT == 0) return true;
  else if constexpr (PAT == 1) return t == 4 || t == 10 || t == 12 || t == 13 || t == 14 || t == 16 || t == 22;
  else return (mask >> t) & 1u;
}

template <class T, int PAT>
__global__ void __launch_bounds__(S3S_THREADS, sizeof(T) == 4 ? 4 : 2)
stencil3d_stream_kernel(const __grid_constant__ Stencil3Args a, const __grid_constant__ Stencil3W<T> W,
                        int64_t zchunk, uint32_t mask, int vec) {
  constexpr int R = 1, K = 3;
  constexpr int PX = 16 / (int)sizeof(T);             // left/right pad: one 16-byte piece
  constexpr int PW = S3S_TX + 2 * PX, PH = S3S_OY + 2 * R;
  constexpr int CPR = PW * (int)sizeof(T) / 16;        // 16-byte pieces per buffer row
  constexpr int EPC = 16 / (int)sizeof(T);             // elements per piece
  constexpr int NPC = (PH * CPR + S3S_THREADS - 1) / S3S_THREADS;  // pieces per thread
  __shared__ __align__(16) T plane[S3S_STAGES][PH][PW];
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
  const int64_t gxs = x0 - PX;  // column of buffer column 0
  const int64_t hw = a.h * a.w;

  // This thread's pieces, the same in every plane: piece q = tid + u * threads
  // is buffer row q / CPR, columns (q % CPR) * EPC ...  Mode 0: one 16-byte
  // copy from element `off` of the plane; 1: element by element from row
  // offset `off`, each column remapped; 2: constant cells; 3: no piece.
  int64_t off[NPC];
  int mode[NPC];
#pragma unroll
  for (int u = 0; u < NPC; ++u) {
    const int q = tid + u * S3S_THREADS;
    mode[u] = 3;
    off[u] = 0;
    if (q < PH * CPR) {
      const int sy = q / CPR, c = q % CPR;
      const int64_t gy = y0 - R + sy, gx = gxs + (int64_t)c * EPC;
      const bool yin = gy >= 0 && gy < a.h;
      if (!yin && b == ACC_CONSTANT) {
        mode[u] = 2;
      } else {
        const int64_t row = (yin ? gy : bound_index(gy, a.h, b)) * a.w;
        const bool whole = vec && gx >= 0 && gx + EPC <= a.w;
        mode[u] = whole ? 0 : 1;
        off[u] = whole ? row + gx : row;
      }
    }
  }

  // Issue the copies of virtual plane p (which may lie outside [0, d)) into
  // buffer `buf`.
  auto issue = [&](int64_t p, int buf) {
    const bool pin = p >= 0 && p < a.d;
    if (!pin && b == ACC_CONSTANT) {
      for (int q = tid; q < PH * PW; q += S3S_THREADS) plane[buf][q / PW][q % PW] = cval;
      return;
    }
    const T *pl = in + (pin ? p : bound_index(p, a.d, b)) * hw;
#pragma unroll
    for (int u = 0; u < NPC; ++u) {
      const int q = tid + u * S3S_THREADS;
      T *dst = &plane[buf][0][0] + (q / CPR) * PW + (q % CPR) * EPC;
      if (mode[u] == 0) {
        cp_async_16(dst, pl + off[u]);
      } else if (mode[u] == 1) {
        const int64_t gx = gxs + (int64_t)(q % CPR) * EPC;
#pragma unroll
        for (int e = 0; e < EPC; ++e) {
          const int64_t x = gx + e;
          const bool xin = x >= 0 && x < a.w;
          if (!xin && b == ACC_CONSTANT) dst[e] = cval;
          else cp_async_el<sizeof(T)>(dst + e, pl + off[u] + (xin ? x : bound_index(x, a.w, b)));
        }
      } else if (mode[u] == 2) {
#pragma unroll
        for (int e = 0; e < EPC; ++e) dst[e] = cval;
      }
    }
  };

  // acc[s][r]: the accumulator of row r of output plane p - R + k lives in
  // slot s = (k + ROT) % K while plane p is applied; ROT advances by one per
  // plane, so the finished output's slot becomes the newest output's without
  // moving registers.
  T acc[K][S3S_ROWS];
#pragma unroll
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int r = 0; r < S3S_ROWS; ++r) acc[k][r] = Prim<ACC_ADD, T>::id();
  const int64_t ps = z0 - R, pend = z1 - 1 + R;  // planes ps .. pend
#pragma unroll
  for (int i = 0; i < S3S_STAGES - 1; ++i) {
    if (ps + i <= pend) issue(ps + i, i);
    cp_async_commit();
  }
  const int64_t gx = x0 + tx;
  const int64_t gyt = y0 + ty * S3S_ROWS;
  T wr[K * K * K];  // the weights, in registers (read once from the parameter)
#pragma unroll
  for (int t = 0; t < K * K * K; ++t) wr[t] = W.w[t];
  int buf = 0;
  auto step = [&](int64_t p, auto rot) {
    constexpr int ROT = decltype(rot)::value;
    cp_async_wait<S3S_STAGES - 2>();  // plane p's copies (this thread's) have landed
    __syncthreads();                  // ... and every thread's; the buffer of plane p-1 is free
    {
      const int64_t pn = p + S3S_STAGES - 1;
      const int nb = buf == 0 ? S3S_STAGES - 1 : buf - 1;
      if (pn <= pend) issue(pn, nb);
      cp_async_commit();
    }
    // plane p: weight plane (p - z) + R for output z = p - R + k is 2R - k
    const T *src = &plane[buf][ty * S3S_ROWS][tx + PX - R];
#pragma unroll
    for (int ir = 0; ir < S3S_ROWS + 2 * R; ++ir) {
      T xv[K];
#pragma unroll
      for (int dx = 0; dx < K; ++dx) xv[dx] = src[ir * PW + dx];
#pragma unroll
      for (int dyi = 0; dyi < K; ++dyi) {
        const int r = ir - dyi;
        if (r < 0 || r >= S3S_ROWS) continue;
#pragma unroll
        for (int k = 0; k < K; ++k) {
#pragma unroll
          for (int dx = 0; dx < K; ++dx) {
            const int t = ((2 * R - k) * K + dyi) * K + dx;
            if (!s3_tap<PAT>(t, mask)) continue;
            T &ac = acc[(k + ROT) % K][r];
            ac = fma_tap(wr[t], xv[dx], ac);
          }
        }
      }
    }
    // output plane p - R is complete
    constexpr int S0 = ROT % K;
    const int64_t zo = p - R;
    if (zo >= z0 && gx < a.w) {
      T *o = out + zo * hw + gyt * a.w + gx;
#pragma unroll
      for (int r = 0; r < S3S_ROWS; ++r)
        if (gyt + r < a.h) o[r * a.w] = acc[S0][r];
    }
#pragma unroll
    for (int r = 0; r < S3S_ROWS; ++r) acc[S0][r] = Prim<ACC_ADD, T>::id();
    buf = buf == S3S_STAGES - 1 ? 0 : buf + 1;
  };
  for (int64_t p = ps;;) {
    step(p, std::integral_constant<int, 0>());
    if (++p > pend) break;
    step(p, std::integral_constant<int, 1>());
    if (++p > pend) break;
    step(p, std::integral_constant<int, 2>());
    if (++p > pend) break;
  }
  cp_async_wait<0>();  // no copy outlives the CTA (the trailing groups are empty)
}

// Plane ranges per tile: the split whose grid fills the resident CTA slots in
// the most nearly whole waves, discounted by the 2 overlap planes each range
// reads, with ranges of at least 8 planes.
static int64_t s3_zchunk(int64_t tiles, int64_t d, int64_t resident) {
  int64_t best_n = 1;
  double best = -1.0;
  const int64_t nmax = d / 8 > 1 ? (d / 8 < 65535 ? d / 8 : 65535) : 1;
  for (int64_t nz = 1; nz <= nmax && nz <= 4096; ++nz) {
    const int64_t ch = cdiv_h(d, nz);
    const int64_t n = cdiv_h(d, ch);
    const double ctas = (double)(tiles * n);
    const double waves = ctas / (double)resident;
    const double eff = waves / std::ceil(waves) * (double)ch / (double)(ch + 2);
    if (eff > best + 1e-9) { best = eff; best_n = nz; }
  }
  return cdiv_h(d, best_n);
}

template <class T>
int stencil3d_typed(const Stencil3Args &a, const void *weights, cudaStream_t s) {
  Stencil3W<T> W;
  memset(&W, 0, sizeof(W));
  const int n = (2 * a.rz + 1) * (2 * a.ry + 1) * (2 * a.rx + 1);
  memcpy(W.w, weights, (size_t)n * sizeof(T));
  if (a.rz == 1 && a.ry == 1 && a.rx == 1) {
    // 3x3x3: the plane-streaming kernel, its tap pattern fixed at compile time
    // where it is dense or the 7-point star.
    const int64_t sx = cdiv_h(a.w, S3S_TX), sy = cdiv_h(a.h, S3S_OY);
    if (sx <= 0x7fffffffll && sy <= 65535) {
      uint32_t mask = 0;
      for (int t = 0; t < 27; ++t)
        if (!(W.w[t] == T(0))) mask |= 1u << t;
      constexpr uint32_t STAR = (1u << 4) | (1u << 10) | (1u << 12) | (1u << 13) | (1u << 14) | (1u << 16) | (1u << 22);
      const int pat = mask == (1u << 27) - 1 ? 0 : (mask == STAR ? 1 : 2);
      const void *fn = pat == 0 ? (const void *)stencil3d_stream_kernel<T, 0>
                       : pat == 1 ? (const void *)stencil3d_stream_kernel<T, 1>
                                  : (const void *)stencil3d_stream_kernel<T, 2>;
      int per_sm = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, S3S_THREADS, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
      const int64_t zchunk = s3_zchunk(sx * sy, a.d, (int64_t)device_info().sms * per_sm);
      const int64_t nz = cdiv_h(a.d, zchunk);
      const int vec = (reinterpret_cast<uintptr_t>(a.in) % 16 == 0) && ((a.w * (int64_t)sizeof(T)) % 16 == 0);
      dim3 grid((unsigned)sx, (unsigned)sy, (unsigned)nz), block(S3S_TX, S3S_TY);
      if (pat == 0) stencil3d_stream_kernel<T, 0><<<grid, block, 0, s>>>(a, W, zchunk, mask, vec);
      else if (pat == 1) stencil3d_stream_kernel<T, 1><<<grid, block, 0, s>>>(a, W, zchunk, mask, vec);
      else stencil3d_stream_kernel<T, 2><<<grid, block, 0, s>>>(a, W, zchunk, mask, vec);
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
