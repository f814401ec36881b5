// stencil.cu -- weighted-sum stencils over rank-1 / rank-2 arrays with
// clamp / mirror / wrap / constant boundaries.
//
// The reference launches `stencil_inside` over the interior (one thread per
// output, every tap a separate global load, no shared-memory reuse) and
// 2*rank `stencil_border` kernels on forked streams
// (accelerate-llvm-ptx/src/Data/Array/Accelerate/LLVM/PTX/Execute.hs:686-776,
// PTX/CodeGen/Stencil.hs:113-179).  Here one launch covers the whole array:
// each CTA pulls a (TH + 2R) x (TW + 2PX) halo tile into shared memory with
// one 2-D TMA load (the x start rounded out to a 16-byte boundary), CTAs
// whose halo leaves the array overwrite the out-of-range cells with the
// boundary rule (accelerate-llvm/src/Data/Array/Accelerate/LLVM/CodeGen/
// Stencil.hs:195-253), and each thread sweeps a column of TH/4 outputs,
// keeping one accumulator per output and visiting the taps in the
// reference's order (rows outer, -r..r; CodeGen/Stencil.hs:73-180).
//
// Arithmetic: acc starts at the additive identity (-0.0) and every tap is one
// fused multiply-add, acc = fma(w, x, acc), in tap order, so Float32 / Float64
// results are bit-identical to a sequential C evaluation with C99 fma()
// (correctly rounded).  Taps whose weight is exactly zero are not part of the
// pattern and are not read.
#include "stencil_common.cuh"

namespace accgb {

constexpr int ST_TW = 64;       // tile width (outputs)
constexpr int ST_TH = 32;       // tile height (outputs)
constexpr int ST_THREADS = 256; // 64 columns x 4 row groups of 8
constexpr int ST_ROWS = ST_TH / (ST_THREADS / ST_TW);

template <class T> struct StencilW { T w[81]; };

struct StencilArgs {
  const void *in;
  void *out;
  int64_t h, w;
  int64_t in_h, in_w;           // extent of the input (boundaries apply here)
  int64_t in_pitch, out_pitch;  // elements
  int ry, rx;
  int boundary;
  uint64_t cval;
  int accumulate;  // add onto out (second input of stencil2)
  int tma;
  uint32_t *err;
};

// RM: the largest radius this instantiation handles (ry, rx <= RM); PX: the
// halo width in x, RM rounded up to 16 bytes.
template <class T, int RM>
__global__ void __launch_bounds__(ST_THREADS)
stencil_kernel(const __grid_constant__ CUtensorMap tin, StencilArgs a, StencilW<T> W) {
  constexpr int PX = ((RM * (int)sizeof(T) + 15) / 16) * 16 / (int)sizeof(T);
  constexpr int SW = ST_TW + 2 * PX;   // smem tile width
  constexpr int SH = ST_TH + 2 * RM;   // smem tile height
  extern __shared__ unsigned char smem_raw[];
  T *tile = reinterpret_cast<T *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  __shared__ uint64_t bar;

  const int64_t tx0 = (int64_t)blockIdx.x * ST_TW, ty0 = (int64_t)blockIdx.y * ST_TH;
  const int64_t gx0 = tx0 - PX, gy0 = ty0 - RM;  // global coords of tile[0][0]
  const T *in = static_cast<const T *>(a.in);
  const bool border = gx0 < 0 || gy0 < 0 || gx0 + SW > a.in_w || gy0 + SH > a.in_h;

  if (a.tma) {
    if (threadIdx.x == 0) {
      mbar_init(&bar, 1);
      fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      mbar_expect_tx(&bar, SW * SH * sizeof(T));
      tma_load_2d(tile, &tin, (int)gx0, (int)gy0, &bar);
    }
    if (__syncthreads_or(!mbar_wait_flagged(&bar, 0, a.err))) return;  // the tile never landed
    if (border) {
      // Overwrite the cells the TMA filled with zeros (outside the array).
      for (int k = threadIdx.x; k < SW * SH; k += ST_THREADS) {
        const int sy = k / SW, sx = k % SW;
        const int64_t gy = gy0 + sy, gx = gx0 + sx;
        if (gy >= 0 && gy < a.in_h && gx >= 0 && gx < a.in_w) continue;
        T v;
        if (a.boundary == ACC_CONSTANT) v = from_bits<T>(a.cval);
        else v = in[bound_index(gy, a.in_h, a.boundary) * a.in_pitch + bound_index(gx, a.in_w, a.boundary)];
        tile[sy * SW + sx] = v;
      }
    }
  } else {
    for (int k = threadIdx.x; k < SW * SH; k += ST_THREADS) {
      const int sy = k / SW, sx = k % SW;
      const int64_t gy = gy0 + sy, gx = gx0 + sx;
      T v;
      if (gy >= 0 && gy < a.in_h && gx >= 0 && gx < a.in_w) v = in[gy * a.in_pitch + gx];
      else if (a.boundary == ACC_CONSTANT) v = from_bits<T>(a.cval);
      else v = in[bound_index(gy, a.in_h, a.boundary) * a.in_pitch + bound_index(gx, a.in_w, a.boundary)];
      tile[sy * SW + sx] = v;
    }
  }
  __syncthreads();

  const int col = threadIdx.x % ST_TW;
  const int rg = threadIdx.x / ST_TW;
  const int oy0 = rg * ST_ROWS;  // first output row of this thread (tile coords)
  T acc[ST_ROWS];
  T *out = static_cast<T *>(a.out);
  const int64_t gx = tx0 + col;
#pragma unroll
  for (int r = 0; r < ST_ROWS; ++r) {
    const int64_t gy = ty0 + oy0 + r;
    if (a.accumulate && gy < a.h && gx < a.w) acc[r] = out[gy * a.out_pitch + gx];
    else acc[r] = Prim<ACC_ADD, T>::id();
  }
  const int ry = a.ry, rx = a.rx;
  const int KW = 2 * rx + 1;
  // Input rows oy0-ry .. oy0+ST_ROWS-1+ry (tile coords, offset by RM).
#pragma unroll
  for (int ir = 0; ir < ST_ROWS + 2 * RM; ++ir) {
    const int iy = oy0 + ir - RM;       // input row relative to the tile's first output row
    const int dyl = ir - RM;            // = iy - oy0
    if (dyl < -ry || dyl > ST_ROWS - 1 + ry) continue;
    T xv[2 * RM + 1];
#pragma unroll
    for (int dx = -RM; dx <= RM; ++dx)
      xv[dx + RM] = (dx >= -rx && dx <= rx) ? tile[(iy + RM) * SW + PX + col + dx] : T(0);
#pragma unroll
    for (int r = 0; r < ST_ROWS; ++r) {
      const int dy = dyl - r;  // this input row is tap row dy of output row r
      if (dy < -ry || dy > ry) continue;
#pragma unroll
      for (int dx = -RM; dx <= RM; ++dx) {
        if (dx < -rx || dx > rx) continue;
        const T wk = W.w[(dy + ry) * KW + (dx + rx)];
        if (wk == T(0)) continue;
        acc[r] = fma_tap(wk, xv[dx + RM], acc[r]);
      }
    }
  }
#pragma unroll
  for (int r = 0; r < ST_ROWS; ++r) {
    const int64_t gy = ty0 + oy0 + r;
    if (gy < a.h && gx < a.w) out[gy * a.out_pitch + gx] = acc[r];
  }
}

// ----------------------------------------------------------------- specialised sweep
// The same computation with the radii and the tap pattern known at compile
// time: PAT 0 = every tap has a non-zero weight, PAT 1 = the cross (5-point
// style: only the corners of the 3x3 are zero), PAT 2 = any pattern (each tap
// tested against a zero mask).  Tiles are 64 x 64 outputs, 16 rows per thread.
constexpr int SF_TW = 64, SF_TH = 64, SF_ROWS = 16;

template <class T, int RY, int RX, int PAT>
__global__ void __launch_bounds__(ST_THREADS, (sizeof(T) == 4 && RY * RX <= 1) ? 4 : 2)
stencil_fast_kernel(const __grid_constant__ CUtensorMap tin, StencilArgs a, StencilW<T> W, uint32_t zmask_lo,
                    uint32_t zmask_hi) {
  constexpr int PX = ((RX * (int)sizeof(T) + 15) / 16) * 16 / (int)sizeof(T) > 0
                         ? ((RX * (int)sizeof(T) + 15) / 16) * 16 / (int)sizeof(T) : 0;
  constexpr int SW = SF_TW + 2 * PX;
  constexpr int SH = SF_TH + 2 * RY;
  constexpr int KW = 2 * RX + 1;
  constexpr int NT = (2 * RY + 1) * KW;
  extern __shared__ unsigned char smem_raw[];
  T *tile = reinterpret_cast<T *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  __shared__ uint64_t bar;

  const int64_t tx0 = (int64_t)blockIdx.x * SF_TW, ty0 = (int64_t)blockIdx.y * SF_TH;
  const int64_t gx0 = tx0 - PX, gy0 = ty0 - RY;
  const T *in = static_cast<const T *>(a.in);
  const bool border = gx0 < 0 || gy0 < 0 || gx0 + SW > a.in_w || gy0 + SH > a.in_h;

  if (a.tma) {
    if (threadIdx.x == 0) {
      mbar_init(&bar, 1);
      fence_mbar_init();
      mbar_expect_tx(&bar, SW * SH * sizeof(T));
      tma_load_2d(tile, &tin, (int)gx0, (int)gy0, &bar);
    }
    __syncthreads();
    if (__syncthreads_or(!mbar_wait_flagged(&bar, 0, a.err))) return;  // the tile never landed
    if (border) {
      for (int k = threadIdx.x; k < SW * SH; k += ST_THREADS) {
        const int sy = k / SW, sx = k % SW;
        const int64_t gy = gy0 + sy, gx = gx0 + sx;
        if (gy >= 0 && gy < a.in_h && gx >= 0 && gx < a.in_w) continue;
        tile[sy * SW + sx] = a.boundary == ACC_CONSTANT
                                 ? from_bits<T>(a.cval)
                                 : in[bound_index(gy, a.in_h, a.boundary) * a.in_pitch + bound_index(gx, a.in_w, a.boundary)];
      }
      __syncthreads();
    }
  } else {
    for (int k = threadIdx.x; k < SW * SH; k += ST_THREADS) {
      const int sy = k / SW, sx = k % SW;
      const int64_t gy = gy0 + sy, gx = gx0 + sx;
      T v;
      if (gy >= 0 && gy < a.in_h && gx >= 0 && gx < a.in_w) v = in[gy * a.in_pitch + gx];
      else if (a.boundary == ACC_CONSTANT) v = from_bits<T>(a.cval);
      else v = in[bound_index(gy, a.in_h, a.boundary) * a.in_pitch + bound_index(gx, a.in_w, a.boundary)];
      tile[sy * SW + sx] = v;
    }
    __syncthreads();
  }

  T w[NT];
#pragma unroll
  for (int k = 0; k < NT; ++k) w[k] = W.w[k];
  const int col = threadIdx.x % SF_TW;
  const int oy0 = (threadIdx.x / SF_TW) * SF_ROWS;
  T acc[SF_ROWS];
  T *out = static_cast<T *>(a.out);
  const int64_t gx = tx0 + col;
#pragma unroll
  for (int r = 0; r < SF_ROWS; ++r) {
    const int64_t gy = ty0 + oy0 + r;
    acc[r] = (a.accumulate && gy < a.h && gx < a.w) ? out[gy * a.out_pitch + gx] : Prim<ACC_ADD, T>::id();
  }
  const T *trow = tile + oy0 * SW + PX + col;  // smem row oy0 - RY + RY = oy0 (halo offset)
#pragma unroll
  for (int ir = 0; ir < SF_ROWS + 2 * RY; ++ir) {
    T xv[KW];
#pragma unroll
    for (int dx = 0; dx < KW; ++dx) xv[dx] = trow[ir * SW + dx - RX];
#pragma unroll
    for (int dyi = 0; dyi < 2 * RY + 1; ++dyi) {
      const int r = ir - dyi;  // output row for which this input row is tap row dyi - RY
      if (r < 0 || r >= SF_ROWS) continue;
#pragma unroll
      for (int dx = 0; dx < KW; ++dx) {
        const int k = dyi * KW + dx;
        if constexpr (PAT == 1) {
          if (k == 0 || k == 2 || k == 6 || k == 8) continue;  // corners of the 3x3 cross
        }
        if constexpr (PAT == 2) {
          const bool zero = k < 32 ? ((zmask_lo >> k) & 1u) : ((zmask_hi >> (k - 32)) & 1u);
          if (zero) continue;
        }
        acc[r] = fma_tap(w[k], xv[dx], acc[r]);
      }
    }
  }
#pragma unroll
  for (int r = 0; r < SF_ROWS; ++r) {
    const int64_t gy = ty0 + oy0 + r;
    if (gy < a.h && gx < a.w) out[gy * a.out_pitch + gx] = acc[r];
  }
}

// ----------------------------------------------------------------- persistent pipeline
// The specialised sweep run by persistent CTAs over a static tile schedule
// (tile = blockIdx.x + k * gridDim.x, row-major over the tile grid): the halo
// tile of tile k+2 is loading (TMA) while tile k is computed, and each output
// tile leaves through a TMA store from shared memory, clipped at the array's
// edge by the copy engine.  Used for 16-byte aligned, non-accumulating calls.
template <class T, int RY, int RX, int PAT>
__global__ void __launch_bounds__(ST_THREADS, (sizeof(T) == 4 && RY * RX <= 1) ? 3 : 1)
stencil_pipe_kernel(const __grid_constant__ CUtensorMap tin, const __grid_constant__ CUtensorMap tout,
                    StencilArgs a, StencilW<T> W, uint32_t zmask_lo, uint32_t zmask_hi, int ntx, int64_t ntiles) {
  constexpr int PX = ((RX * (int)sizeof(T) + 15) / 16) * 16 / (int)sizeof(T);
  constexpr int SW = SF_TW + 2 * PX;
  constexpr int SH = SF_TH + 2 * RY;
  constexpr int KW = 2 * RX + 1;
  constexpr int NT = (2 * RY + 1) * KW;
  constexpr int IN_BYTES = ((SW * SH * (int)sizeof(T)) + 127) / 128 * 128;
  constexpr int OUT_BYTES = SF_TW * SF_TH * (int)sizeof(T);
  extern __shared__ unsigned char smem_raw[];
  unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  auto inb = [&](int s) { return reinterpret_cast<T *>(base + s * IN_BYTES); };
  auto outb = [&](int s) { return reinterpret_cast<T *>(base + 2 * IN_BYTES + s * OUT_BYTES); };
  __shared__ uint64_t full[2];
  __shared__ int s_abort;
  const int tid = threadIdx.x;
  const T *in = static_cast<const T *>(a.in);

  auto issue = [&](int s, int64_t tile) {  // thread 0
    const int64_t ty = tile / ntx, tx = tile % ntx;
    mbar_expect_tx(&full[s], SW * SH * sizeof(T));
    tma_load_2d(inb(s), &tin, (int)(tx * SF_TW - PX), (int)(ty * SF_TH - RY), &full[s]);
  };
  if (tid == 0) {
    prefetch_tmap(&tin);
    prefetch_tmap(&tout);
    s_abort = 0;
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    fence_mbar_init();
    if ((int64_t)blockIdx.x < ntiles) issue(0, blockIdx.x);
    if ((int64_t)blockIdx.x + gridDim.x < ntiles) issue(1, (int64_t)blockIdx.x + gridDim.x);
  }
  __syncthreads();

  T w[NT];
#pragma unroll
  for (int k = 0; k < NT; ++k) w[k] = W.w[k];
  const int col = tid % SF_TW;
  const int oy0 = (tid / SF_TW) * SF_ROWS;

  for (int k = 0;; ++k) {
    const int64_t tile = (int64_t)blockIdx.x + (int64_t)k * gridDim.x;
    if (tile >= ntiles) break;
    const int s = k & 1;
    const int64_t ty = tile / ntx, tx = tile % ntx;
    const int64_t tx0 = tx * SF_TW, ty0 = ty * SF_TH;
    const int64_t gx0 = tx0 - PX, gy0 = ty0 - RY;
    // A tile that never lands sets s_abort; the CTA stops at the next
    // barrier, before it stores from or loads into its buffers (no extra
    // barrier per tile).
    if (!mbar_wait_flagged(&full[s], (uint32_t)(k >> 1) & 1u, a.err)) s_abort = 1;
    T *tile_in = inb(s);
    if (gx0 < 0 || gy0 < 0 || gx0 + SW > a.in_w || gy0 + SH > a.in_h) {
      for (int q = tid; q < SW * SH; q += ST_THREADS) {
        const int sy = q / SW, sx = q % SW;
        const int64_t gy = gy0 + sy, gx = gx0 + sx;
        if (gy >= 0 && gy < a.in_h && gx >= 0 && gx < a.in_w) continue;
        tile_in[sy * SW + sx] = a.boundary == ACC_CONSTANT
                                    ? from_bits<T>(a.cval)
                                    : in[bound_index(gy, a.in_h, a.boundary) * a.in_pitch + bound_index(gx, a.in_w, a.boundary)];
      }
      __syncthreads();
    }
    T acc[SF_ROWS];
#pragma unroll
    for (int r = 0; r < SF_ROWS; ++r) acc[r] = Prim<ACC_ADD, T>::id();
    const T *trow = tile_in + oy0 * SW + PX + col;
#pragma unroll
    for (int ir = 0; ir < SF_ROWS + 2 * RY; ++ir) {
      T xv[KW];
#pragma unroll
      for (int dx = 0; dx < KW; ++dx) xv[dx] = trow[ir * SW + dx - RX];
#pragma unroll
      for (int dyi = 0; dyi < 2 * RY + 1; ++dyi) {
        const int r = ir - dyi;
        if (r < 0 || r >= SF_ROWS) continue;
#pragma unroll
        for (int dx = 0; dx < KW; ++dx) {
          const int q = dyi * KW + dx;
          if constexpr (PAT == 1) {
            if (q == 0 || q == 2 || q == 6 || q == 8) continue;
          }
          if constexpr (PAT == 2) {
            const bool zero = q < 32 ? ((zmask_lo >> q) & 1u) : ((zmask_hi >> (q - 32)) & 1u);
            if (zero) continue;
          }
          acc[r] = fma_tap(w[q], xv[dx], acc[r]);
        }
      }
    }
    // The store issued from this output buffer two tiles ago must have read it.
    if (tid == 0 && k >= 2) asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
    __syncthreads();
    if (s_abort) {
      // bounded waits for this tile's load and the next one, issued into the
      // other stage, then stop (stores already issued complete below)
      if (tid == 0) {
        mbar_wait(&full[s], (uint32_t)(k >> 1) & 1u);
        if (tile + (int64_t)gridDim.x < ntiles) mbar_wait(&full[s ^ 1], (uint32_t)((k + 1) >> 1) & 1u);
      }
      break;
    }
    T *ob = outb(s);
#pragma unroll
    for (int r = 0; r < SF_ROWS; ++r) ob[(oy0 + r) * SF_TW + col] = acc[r];
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tma_store_2d(&tout, (int)tx0, (int)ty0, ob);
      tma_store_commit();
      const int64_t next = tile + 2 * (int64_t)gridDim.x;
      if (next < ntiles) issue(s, next);  // every thread is done with inb[s]
    }
  }
  if (tid == 0) tma_store_wait_all();
}

template <class T, int RY, int RX, int PAT>
int stencil_pipe_launch(StencilArgs a, const StencilW<T> &W, uint32_t zlo, uint32_t zhi, cudaStream_t s,
                        const CUtensorMap &tin, const CUtensorMap &tout) {
  constexpr int PX = ((RX * (int)sizeof(T) + 15) / 16) * 16 / (int)sizeof(T);
  constexpr int SW = SF_TW + 2 * PX;
  constexpr int SH = SF_TH + 2 * RY;
  constexpr int IN_BYTES = ((SW * SH * (int)sizeof(T)) + 127) / 128 * 128;
  constexpr int OUT_BYTES = SF_TW * SF_TH * (int)sizeof(T);
  const size_t smem = 2 * (size_t)IN_BYTES + 2 * (size_t)OUT_BYTES + 128;
  auto kern = stencil_pipe_kernel<T, RY, RX, PAT>;
  static int per_sm = 0;
  if (per_sm == 0) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, ST_THREADS, smem) != cudaSuccess || per_sm < 1) {
      cudaGetLastError();
      per_sm = 1;
    }
  }
  const int64_t ntx = cdiv_h(a.w, SF_TW), nty = cdiv_h(a.h, SF_TH);
  const int64_t ntiles = ntx * nty;
  if (ntx > (1 << 30) || nty > (1 << 30)) return ACC_ERR_TOO_LARGE;
  int64_t grid = (int64_t)device_info().sms * per_sm;
  if (grid > ntiles) grid = ntiles;
  kern<<<(unsigned)grid, ST_THREADS, smem, s>>>(tin, tout, a, W, zlo, zhi, (int)ntx, ntiles);
  return check_launch();
}

template <class T, int RY, int RX, int PAT>
int stencil_fast_launch(StencilArgs a, const StencilW<T> &W, uint32_t zlo, uint32_t zhi, cudaStream_t s) {
  constexpr int PX = ((RX * (int)sizeof(T) + 15) / 16) * 16 / (int)sizeof(T);
  constexpr int SW = SF_TW + 2 * PX;
  constexpr int SH = SF_TH + 2 * RY;
  const size_t smem = (size_t)SW * SH * sizeof(T) + 128;
  CUtensorMap tin;
  memset(&tin, 0, sizeof(tin));
  a.tma = encode_2d(&tin, a.in, sizeof(T), (uint64_t)a.in_w, (uint64_t)a.in_h, (uint64_t)a.in_pitch * sizeof(T),
                    SW, SH, false);
  if (a.tma && !a.accumulate) {
    CUtensorMap tout;
    memset(&tout, 0, sizeof(tout));
    if (encode_2d(&tout, a.out, sizeof(T), (uint64_t)a.w, (uint64_t)a.h, (uint64_t)a.out_pitch * sizeof(T), SF_TW,
                  SF_TH, false))
      return stencil_pipe_launch<T, RY, RX, PAT>(a, W, zlo, zhi, s, tin, tout);
  }
  auto kern = stencil_fast_kernel<T, RY, RX, PAT>;
  static std::atomic<uint64_t> attr_done{0};
  smem_attrs_once(kern, (int)smem, attr_done, false);
  const int64_t gx = cdiv_h(a.w, SF_TW), gy = cdiv_h(a.h, SF_TH);
  if (gy > 65535 || gx > (1ll << 31) - 1) return ACC_ERR_TOO_LARGE;
  kern<<<dim3((unsigned)gx, (unsigned)gy), ST_THREADS, smem, s>>>(tin, a, W, zlo, zhi);
  return check_launch();
}

// Zero-weight mask of the taps (bit k set: weight k is zero).
template <class T>
void zero_mask(const StencilW<T> &W, int n, uint32_t &lo, uint32_t &hi) {
  lo = hi = 0;
  for (int k = 0; k < n; ++k)
    if (W.w[k] == T(0)) {
      if (k < 32) lo |= 1u << k; else hi |= 1u << (k - 32);
    }
}

template <class T, int RY, int RX>
int stencil_fast_pat(StencilArgs a, const StencilW<T> &W, cudaStream_t s) {
  constexpr int NT = (2 * RY + 1) * (2 * RX + 1);
  uint32_t lo, hi;
  zero_mask(W, NT, lo, hi);
  if (lo == 0 && hi == 0) return stencil_fast_launch<T, RY, RX, 0>(a, W, 0, 0, s);
  if (RY == 1 && RX == 1 && lo == ((1u << 0) | (1u << 2) | (1u << 6) | (1u << 8)))
    return stencil_fast_launch<T, RY, RX, 1>(a, W, 0, 0, s);
  return stencil_fast_launch<T, RY, RX, 2>(a, W, lo, hi, s);
}

// ----------------------------------------------------------------- host side
template <class T, int RM>
int stencil_launch(StencilArgs a, const StencilW<T> &W, cudaStream_t s) {
  constexpr int PX = ((RM * (int)sizeof(T) + 15) / 16) * 16 / (int)sizeof(T);
  constexpr int SW = ST_TW + 2 * PX;
  constexpr int SH = ST_TH + 2 * RM;
  const size_t smem = (size_t)SW * SH * sizeof(T) + 128;
  CUtensorMap tin;
  memset(&tin, 0, sizeof(tin));
  a.tma = encode_2d(&tin, a.in, sizeof(T), (uint64_t)a.in_w, (uint64_t)a.in_h, (uint64_t)a.in_pitch * sizeof(T),
                    SW, SH, false);
  auto kern = stencil_kernel<T, RM>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int64_t gx = cdiv_h(a.w, ST_TW), gy = cdiv_h(a.h, ST_TH);
  if (gy > 65535 || gx > (1ll << 31) - 1) return ACC_ERR_TOO_LARGE;
  kern<<<dim3((unsigned)gx, (unsigned)gy), ST_THREADS, smem, s>>>(tin, a, W);
  return check_launch();
}

template <class T>
int stencil_typed(StencilArgs a, const void *weights, cudaStream_t s) {
  StencilW<T> W;
  const int nw = (2 * a.ry + 1) * (2 * a.rx + 1);
  memset(&W, 0, sizeof(W));
  memcpy(W.w, weights, (size_t)nw * sizeof(T));
  if (a.ry == 1 && a.rx == 1) return stencil_fast_pat<T, 1, 1>(a, W, s);
  if (a.ry == 0 && a.rx == 1) return stencil_fast_pat<T, 0, 1>(a, W, s);
  if (a.ry == 1 && a.rx == 0) return stencil_fast_pat<T, 1, 0>(a, W, s);
  if (a.ry == 2 && a.rx == 2) return stencil_fast_pat<T, 2, 2>(a, W, s);
  const int r = a.ry > a.rx ? a.ry : a.rx;
  if (r <= 1) return stencil_launch<T, 1>(a, W, s);
  if (r <= 2) return stencil_launch<T, 2>(a, W, s);
  return stencil_launch<T, 4>(a, W, s);
}

static int stencil_dispatch(int type, StencilArgs a, const void *weights, cudaStream_t s) {
  switch (type) {
    case ACC_F32: return stencil_typed<float>(a, weights, s);
    case ACC_F64: return stencil_typed<double>(a, weights, s);
    case ACC_I32: return stencil_typed<int32_t>(a, weights, s);
    case ACC_I64: return stencil_typed<int64_t>(a, weights, s);
    default: return ACC_ERR_UNSUPPORTED;
  }
}

static int stencil_check(int type, int ry, int rx, int boundary, const void *cval, int64_t h, int64_t w) {
  if (ry < 0 || ry > 4 || rx < 0 || rx > 4) return ACC_ERR_INVALID;
  if (h < 0 || w < 0) return ACC_ERR_INVALID;
  if (boundary < ACC_CLAMP || boundary > ACC_CONSTANT) return ACC_ERR_INVALID;
  if (boundary == ACC_CONSTANT && !cval) return ACC_ERR_INVALID;
  if (type != ACC_F32 && type != ACC_F64 && type != ACC_I32 && type != ACC_I64) return ACC_ERR_UNSUPPORTED;
  return ACC_OK;
}

}  // namespace accgb

using namespace accgb;

extern "C" int acc_stencil2d(int type, int ry, int rx, const void *weights, int boundary, const void *cval,
                             const void *in, void *out, int64_t h, int64_t w, void *stream) {
  int st = stencil_check(type, ry, rx, boundary, cval, h, w);
  if (st) return st;
  if (h == 0 || w == 0) return ACC_OK;
  if (!weights || !in || !out) return ACC_ERR_INVALID;
  StencilArgs a{};
  a.in = in; a.out = out; a.h = h; a.w = w; a.in_h = h; a.in_w = w; a.in_pitch = w; a.out_pitch = w;
  a.ry = ry; a.rx = rx; a.boundary = boundary;
  a.cval = 0;
  if (cval) memcpy(&a.cval, cval, (type == ACC_F64 || type == ACC_I64) ? 8 : 4);
  a.accumulate = 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Workspace *ws = workspace(s, &st);
  if (!ws) return st;
  a.err = ws->words + W_ERR;
  return stencil_dispatch(type, a, weights, s);
}

extern "C" int acc_stencil2d_pair(int type, int ry, int rx, const void *wa_w, const void *wb_w, int boundary_a,
                                  const void *cval_a, int boundary_b, const void *cval_b, const void *a_in,
                                  int64_t ha, int64_t wa, const void *b_in, int64_t hb, int64_t wb, void *out,
                                  void *stream) {
  int st = stencil_check(type, ry, rx, boundary_a, cval_a, ha, wa);
  if (st) return st;
  st = stencil_check(type, ry, rx, boundary_b, cval_b, hb, wb);
  if (st) return st;
  const int64_t h = ha < hb ? ha : hb, w = wa < wb ? wa : wb;
  if (h == 0 || w == 0) return ACC_OK;
  if (!wa_w || !wb_w || !a_in || !b_in || !out) return ACC_ERR_INVALID;
  const size_t esz = (type == ACC_F64 || type == ACC_I64) ? 8 : 4;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  Workspace *ws = workspace(s, &st);
  if (!ws) return st;
  // Pass 1 evaluates the taps of a; pass 2 continues the same accumulator
  // (read back from out) with the taps of b.  The accumulator is rounded to
  // the element type after every tap either way, so the two passes give the
  // bits of one fused sweep.
  StencilArgs a{};
  a.err = ws->words + W_ERR;
  a.in = a_in; a.out = out; a.h = h; a.w = w; a.in_h = ha; a.in_w = wa; a.in_pitch = wa; a.out_pitch = w;
  a.ry = ry; a.rx = rx; a.boundary = boundary_a; a.cval = 0;
  if (cval_a) memcpy(&a.cval, cval_a, esz);
  a.accumulate = 0;
  st = stencil_dispatch(type, a, wa_w, s);
  if (st) return st;
  a.in = b_in; a.in_h = hb; a.in_w = wb; a.in_pitch = wb; a.boundary = boundary_b; a.cval = 0;
  if (cval_b) memcpy(&a.cval, cval_b, esz);
  a.accumulate = 1;
  return stencil_dispatch(type, a, wb_w, s);
}
