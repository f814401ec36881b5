/*
 * acc_gb300.h -- C ABI of the GB300 (sm_103a) skeleton library `libaccgb.so`.
 *
 * These entry points replace the bodies of the `Execute PTX` skeleton
 * operations of accelerate-llvm-ptx (instance at
 * accelerate-llvm-ptx/src/Data/Array/Accelerate/LLVM/PTX/Execute.hs:83-109)
 * for the fixed associative primitives (+ * min max .&. .|. xor) over
 * Int32 / Int64 / Word32 / Float32 / Float64.  Every kernel behind them is
 * hand-written CUDA for sm_103a; there is no CPU fallback.
 *
 * Conventions (carried over from the reference runtime):
 *  - Ownership: the caller owns every input and output buffer (device
 *    pointers).  The library owns and caches its temporaries per stream, as the
 *    reference allocates its temps with `allocateRemote`
 *    (PTX/Execute.hs:313,453).
 *  - Asynchrony: work is enqueued on `stream` (a cudaStream_t, passed as
 *    void*; NULL = the legacy default stream) and the call returns at once,
 *    like the reference's `Par PTX (Future ...)` ops which record an event
 *    after the launch (PTX/Execute/Async.hs:115-126,175-187).  Device-side
 *    failures (a bounded wait that ran out, an out-of-range permutation index)
 *    are raised into a per-stream error word and reported by acc_sync().
 *  - Errors: every call returns an acc_status; nothing aborts.  A Haskell shim
 *    maps non-zero codes to `internalError`, as `evalPTX` does
 *    (PTX/State.hs:51-55).
 *  - Layout: row-major, innermost dimension contiguous (SoA components of a
 *    tuple are separate calls).  `outer` is the product of all but the
 *    innermost extent and `inner` the innermost extent; extents are int64 as
 *    the reference marshals `Int` (PTX/Execute/Marshal.hs:49).
 *  - Seeds: `seed` points to ONE host-memory element of the array's type, or
 *    is NULL for the seedless variant (fold1, scanl1, ...).  The seed is
 *    combined on the LEFT for left-to-right operations (z `f` x0 ...) and on
 *    the RIGHT for right-to-left scans (... x(n-1) `f` z), as in
 *    accelerate-llvm-native/.../Native/CodeGen/Fold.hs:256-260 and
 *    Native/CodeGen/Scan.hs:190-205.
 */
#ifndef ACC_GB300_H
#define ACC_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ACC_GB300_ABI_VERSION 1

/* Element types: the scalar types of Accelerate's `ScalarType` that the
 * skeleton layer supports (Int32, Int64, Word32, Float, Double). */
typedef enum acc_type {
  ACC_I32 = 0,
  ACC_I64 = 1,
  ACC_U32 = 2,
  ACC_F32 = 3,
  ACC_F64 = 4
} acc_type;

/* The fixed associative primitives recognised by the shim, the same set the
 * reference turns into atomic RMW operations (accelerate-llvm/src/Data/Array/
 * Accelerate/LLVM/CodeGen/Permute.hs:136-160).  Integer + and * wrap
 * (LLVM/AST/Type/Instruction.hs:429-473); float min/max are IEEE fmin/fmax,
 * integer min/max are `select` on <= / >= (CodeGen/Arithmetic.hs:456-466);
 * the bitwise primitives exist for the integral types only. */
typedef enum acc_op {
  ACC_ADD = 0,
  ACC_MUL = 1,
  ACC_MIN = 2,
  ACC_MAX = 3,
  ACC_AND = 4,
  ACC_OR  = 5,
  ACC_XOR = 6
} acc_op;

/* Float32 accumulation policy of fold / foldSeg / scan with (+).
 * COMPENSATED (the default for Float32 +) carries a two-sum error term in
 * FP32; PLAIN is an FP32 tree; FP64ACC accumulates in FP64 and rounds once.
 * Ignored for every other (op, type) pair. */
typedef enum acc_prec {
  ACC_PREC_DEFAULT     = 0,
  ACC_PREC_PLAIN       = 1,
  ACC_PREC_COMPENSATED = 2,
  ACC_PREC_FP64ACC     = 3
} acc_prec;

/* Scan direction (Accelerate `Direction`: LeftToRight / RightToLeft). */
typedef enum acc_dir { ACC_L2R = 0, ACC_R2L = 1 } acc_dir;

/* Scan flavour (accelerate-llvm/src/.../LLVM/Execute.hs:93-156,
 * `scan` True/False and `scan'`). */
typedef enum acc_scan_kind {
  ACC_SCAN_INCLUSIVE = 0, /* scanl1 / scanr1: out has n elements, seed unused           */
  ACC_SCAN_SEEDED    = 1, /* scanl z / scanr z: out has n+1 elements                    */
  ACC_SCAN_PRIME     = 2  /* scanl' z / scanr' z: out has n elements, total -> `sums`   */
} acc_scan_kind;

/* Stencil boundary conditions (accelerate-llvm/.../CodeGen/Stencil.hs:207-253).
 * The user-function boundary is out of scope. */
typedef enum acc_boundary {
  ACC_CLAMP    = 0,
  ACC_MIRROR   = 1,
  ACC_WRAP     = 2,
  ACC_CONSTANT = 3
} acc_boundary;

typedef enum acc_status {
  ACC_OK              = 0,
  ACC_ERR_INVALID     = 1, /* bad argument (null pointer, negative extent, bad enum) */
  ACC_ERR_UNSUPPORTED = 2, /* (op, type) pair outside the fixed primitives          */
  ACC_ERR_EMPTY       = 3, /* fold1 / foldSeg-without-seed over an empty extent      */
  ACC_ERR_CUDA        = 4, /* a CUDA runtime call failed                             */
  ACC_ERR_NOMEM       = 5, /* device allocation of a temporary failed                */
  ACC_ERR_TIMEOUT     = 6, /* a bounded device wait ran out (reported by acc_sync)   */
  ACC_ERR_INDEX       = 7, /* permute index >= size of the target (acc_sync)         */
  ACC_ERR_TOO_LARGE   = 8  /* an extent beyond what the entry point accepts          */
} acc_status;

/* ---------------------------------------------------------------- library */

/* ABI version (ACC_GB300_ABI_VERSION). */
int acc_version(void);

/* Human-readable text of a status code (static storage). */
const char *acc_strerror(int status);

/* Wait for all work enqueued on `stream`, then return and clear the device
 * error word of that stream (ACC_OK, ACC_ERR_TIMEOUT, ACC_ERR_INDEX) or
 * ACC_ERR_CUDA if the stream itself failed.  Plays the part of the
 * reference's `get`/`block` on a Future (PTX/Execute/Async.hs:132-165). */
int acc_sync(void *stream);

/* Drop the cached temporaries of every stream (they are re-made on demand).
 * Waits for the device first; call it only while no other host thread is
 * inside a library call, since those calls hold pointers into the cache. */
int acc_release_workspaces(void);

/* Make one of the library's bounded device waits run out, on purpose: one
 * CTA on `stream` waits on something that nothing completes --
 *   which = 0: an mbarrier phase that no copy and no thread completes (the
 *              wait every TMA-tiled kernel makes for its tile);
 *   which = 1: the decoupled look-back of tile 1 of a scan whose tile 0 never
 *              publishes (the wait of every scan and foldSeg tile on its
 *              predecessors).
 * The wait gives up after its limit (2 s of wall-clock time; the mbarrier
 * wait twice that, since a copy that may still land gets a second wait),
 * the kernel raises the stream's error word and returns; the next
 * acc_sync(stream) returns ACC_ERR_TIMEOUT and clears the word, and the
 * stream is usable as before.
 * No counterpart in the reference, whose kernels never wait on one another
 * (its scan runs as separate launches, PTX/Execute.hs:438-468).  For tests
 * and diagnostics; ACC_ERR_INVALID for another `which`. */
int acc_selftest_timeout(int which, void *stream);

/* ---------------------------------------------------------------- fold */

/* fold f z / fold1 f along the innermost dimension.
 * Replaces foldOp / fold1Op / foldCore / foldAllOp / foldDimOp
 * (PTX/Execute.hs:222-340).
 *   in  : outer*inner elements, out : outer elements.
 *   seed: NULL => fold1 (inner must be >= 1 unless outer*inner == 0,
 *         otherwise ACC_ERR_EMPTY as `boundsCheck "empty array"`,
 *         PTX/Execute.hs:232).  inner == 0 with a seed fills out with z
 *         (PTX/Execute.hs:248). */
int acc_fold(int op, int type, int prec, const void *in, void *out,
             int64_t outer, int64_t inner, const void *seed, void *stream);

/* fold f z (zipWith g xs ys) / fold1 f (zipWith g xs ys): a fold whose input
 * is the fused producer of two arrays, e.g. dotp = fold (+) 0 (zipWith (*)).
 * Replaces foldOp / foldAllOp on a delayed zipWith input
 * (PTX/CodeGen/Fold.hs:80-97, mkFoldAll's MIRDelayed argument): the zipped
 * array is never written.  xs, ys: outer*inner elements each, same layout;
 * every zipped element is g x y rounded to `type`; the fold then follows
 * acc_fold (seed on the left, `prec` for Float32 +, empty rows as acc_fold).
 * op in {ADD, MIN, MAX}, zop in {ADD, MUL, MIN, MAX}, type in {I32, I64,
 * F32, F64}; other combinations give ACC_ERR_UNSUPPORTED. */
int acc_fold_zipwith(int op, int zop, int type, int prec, const void *xs, const void *ys,
                     void *out, int64_t outer, int64_t inner, const void *seed,
                     void *stream);

/* fold f z (map (\x -> g x c) xs) / fold1 f (map ...): a fold whose input is
 * the fused producer `map` of one array with a primitive g and a constant
 * operand c (a host pointer to one element of `type`), e.g. the reference's
 * known answer `A.sum (A.map (+1) xs)` (accelerate-llvm-ptx/test/nofib/Data/
 * Array/Accelerate/LLVM/PTX/NoFib/RunQ.hs:29).  Replaces foldOp / foldAllOp
 * on a delayed map input (PTX/CodeGen/Fold.hs:80-97): the mapped array is
 * never written.  Every mapped element is g x c rounded to `type`; the fold
 * then follows acc_fold.  op in {ADD, MIN, MAX}, gop in {ADD, MUL, MIN, MAX},
 * type in {I32, I64, F32, F64}; other combinations give ACC_ERR_UNSUPPORTED. */
int acc_fold_map(int op, int gop, int type, int prec, const void *xs, const void *c, void *out,
                 int64_t outer, int64_t inner, const void *seed, void *stream);

/* ---------------------------------------------------------------- foldSeg */

/* foldSeg f z / fold1Seg f over a segment-OFFSET array (length nseg+1, the
 * `scanl (+) 0` of the lengths, as the reference receives it,
 * PTX/Execute.hs:343-374 "segments array has been 'scanl (+) 0'`ed").
 * Replaces foldSegOp.
 *   in: outer*inner elements; offsets: nseg+1 values of `offset_type`
 *   (ACC_I32 or ACC_I64), non-decreasing, 0 <= offsets[i] <= inner;
 *   out: outer*nseg elements.
 *   An empty segment gives z with a seed and is left unwritten without one
 *   (PTX/CodeGen/FoldSeg.hs:170-178). */
int acc_fold_seg(int op, int type, int prec, const void *in,
                 const void *offsets, int offset_type, void *out,
                 int64_t outer, int64_t inner, int64_t nseg,
                 const void *seed, void *stream);

/* foldSeg over segment LENGTHS: first computes the offsets with the
 * library's own single-pass scan (what the Accelerate frontend does before
 * the backend sees the array), then runs acc_fold_seg. */
int acc_fold_seg_lengths(int op, int type, int prec, const void *in,
                         const void *lengths, int length_type, void *out,
                         int64_t outer, int64_t inner, int64_t nseg,
                         const void *seed, void *stream);

/* foldSeg f z (zipWith g xs ys) / fold1Seg f (zipWith g xs ys): a segmented
 * fold whose input is the fused producer of two arrays.  Replaces foldSegOp
 * on a delayed zipWith input (PTX/CodeGen/FoldSeg.hs:56-458, the MIRDelayed
 * argument): the zipped array is never written.  xs, ys: outer*inner
 * elements each, same layout; every zipped element is g x y rounded to
 * `type`; offsets, out, seed and empty segments as for acc_fold_seg.
 * op in {ADD, MIN, MAX}, zop in {ADD, MUL, MIN, MAX}, type in {I32, I64,
 * F32, F64}; other combinations give ACC_ERR_UNSUPPORTED. */
int acc_fold_seg_zipwith(int op, int zop, int type, int prec, const void *xs,
                         const void *ys, const void *offsets, int offset_type,
                         void *out, int64_t outer, int64_t inner, int64_t nseg,
                         const void *seed, void *stream);

/* ---------------------------------------------------------------- scan */

/* scanl / scanl1 / scanr / scanr1 / scanl' / scanr' along the innermost
 * dimension.  Replaces scanOp / scan1Op / scan'Op / scanCore / scanAllOp /
 * scanDimOp (PTX/Execute.hs:377-594).
 *   in : outer*inner elements.
 *   out: outer*inner elements (INCLUSIVE, PRIME) or outer*(inner+1)
 *        (SEEDED: scanl z puts z at index 0, scanr z puts it at index n).
 *   sums: outer elements for PRIME (the per-row totals), else ignored.
 *   seed: required for SEEDED and PRIME, ignored for INCLUSIVE. */
int acc_scan(int op, int type, int prec, int dir, int kind, const void *in,
             void *out, void *sums, int64_t outer, int64_t inner,
             const void *seed, void *stream);

/* Every scan flavour of acc_scan over the fused producer zipWith g xs ys,
 * e.g. scanl1 (+) (zipWith (*) xs ys).  Replaces scanOp / scan1Op / scan'Op
 * on a delayed zipWith input (PTX/CodeGen/Scan.hs:141-439 and 746-939, the
 * MIRDelayed argument of the scan kernels): the zipped array is never
 * written.  xs, ys: outer*inner elements each, same layout; every zipped
 * element is g x y rounded to `type`; out / sums / seed / dir / kind as for
 * acc_scan.  op in {ADD, MIN, MAX}, zop in {ADD, MUL, MIN, MAX}, type in
 * {I32, I64, F32, F64}; other combinations give ACC_ERR_UNSUPPORTED. */
int acc_scan_zipwith(int op, int zop, int type, int prec, int dir, int kind,
                     const void *xs, const void *ys, void *out, void *sums,
                     int64_t outer, int64_t inner, const void *seed,
                     void *stream);

/* Every scan flavour over the fused producer map (\x -> g x c) xs, for a
 * primitive g and a constant c (a host pointer to one element of `type`):
 * e.g. scanl1 (+) (map (+1) xs).  Replaces scanOp / scan1Op / scan'Op on a
 * delayed map input (PTX/CodeGen/Scan.hs:141-439,746-939, the MIRDelayed
 * argument): the mapped array is never written.  Every mapped element is
 * g x c rounded to `type`; the scan then follows acc_scan (same `dir`,
 * `kind`, outputs and errors).  op in {ADD, MIN, MAX}, gop in {ADD, MUL,
 * MIN, MAX}, type in {I32, I64, F32, F64}; other combinations give
 * ACC_ERR_UNSUPPORTED. */
int acc_scan_map(int op, int gop, int type, int prec, int dir, int kind, const void *xs, const void *c,
                 void *out, void *sums, int64_t outer, int64_t inner, const void *seed, void *stream);

/* acc_scan without any device allocation -- no counterpart in the reference,
 * which always allocates its temporaries (PTX/Execute.hs:453).  Same
 * arguments, results and errors as acc_scan, for callers that cannot let a
 * library call cudaMalloc: an integration that runs under a fixed
 * device-memory budget, a plugin whose host process hands out all device
 * memory from its own pool allocator, or a latency-bound loop that must not
 * stall on cudaMalloc (which can synchronise the device).  The look-back
 * scratch lives in one file-scope device array of 2 MiB (plus 256 bytes)
 * that every GPU loading the library holds until the process exits, so a row
 * may have at most 2^28 elements; longer rows return ACC_ERR_TOO_LARGE before
 * anything is launched.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress): make that first call before any
 * stream capture.  Each call clears the part of the array it uses, in stream
 * order, before its kernel runs.  Every call reuses the same array, so calls
 * whose work overlaps on the GPU (other streams, other host threads) race and
 * must be serialised by the caller.  A look-back wait that runs out is not
 * reported by acc_sync (which reports only acc_scan's workspaces) but by
 * acc_scan_noalloc_status; the wait is bounded, so the call always
 * completes. */
int acc_scan_noalloc(int op, int type, int prec, int dir, int kind,
                     const void *in, void *out, void *sums, int64_t outer,
                     int64_t inner, const void *seed, void *stream);

/* Wait for the work enqueued on `stream`, then report whether the look-back
 * wait of the last acc_scan_noalloc call on this device ran out
 * (ACC_ERR_TIMEOUT; its result is then not to be trusted) or not (ACC_OK).
 * Allocates nothing: it reads the error word of the same static array.  No
 * counterpart in the reference. */
int acc_scan_noalloc_status(void *stream);

/* ---------------------------------------------------------------- permute */

/* permute f defaults p xs, for the fixed primitives.  Replaces permuteOp +
 * permute_rmw (PTX/Execute.hs:597-649; PTX/CodeGen/Permute.hs:117-213).
 *   out : m elements, ALREADY holding the defaults (the reference clones the
 *         defaults first, PTX/Execute.hs:623-625; acc_permute_clone does it).
 *   src : n source values, or NULL to combine the constant *cval (host
 *         pointer to one element) for every source index (the fused
 *         `fill n c` producer of a histogram).
 *   idx : n target indices of `index_type` (ACC_I32 / ACC_I64); a negative
 *         index is `Nothing` (the element is dropped); an index >= m is
 *         dropped and raises ACC_ERR_INDEX at the next acc_sync.
 *   Each update is out[j] = f x out[j] (new value first,
 *   Native/CodeGen/Permute.hs:112-116).  Integer results are exact under any
 *   order; Float32/Float64 (+ and *) depend on the update order. */
int acc_permute(int op, int type, const void *src, const void *cval,
                const void *idx, int index_type, void *out, int64_t n,
                int64_t m, void *stream);

/* Clone `defaults` (m elements) into `out`, then acc_permute. */
int acc_permute_clone(int op, int type, const void *defaults, const void *src,
                      const void *cval, const void *idx, int index_type,
                      void *out, int64_t n, int64_t m, void *stream);

/* ---------------------------------------------------------------- stencil */

/* stencil over a rank-2 (or rank-1 with h == 1, ry == 0) array with a
 * weighted-sum stencil function:
 *     out[y][x] = sum_{dy=-ry..ry, dx=-rx..rx} w[(dy+ry)*(2rx+1)+(dx+rx)] * in[y+dy][x+dx]
 * accumulated in that tap order (rows outer, -r..r, as the reference's
 * stencil access, accelerate-llvm/.../CodeGen/Stencil.hs:73-180), one fused
 * multiply-add per tap (acc = fma(w, x, acc), a single rounding, from
 * acc = -0.0) for the float types; taps whose weight is zero are skipped.  Out-of-range reads follow
 * `boundary` (CodeGen/Stencil.hs:207-253); `cval` (host pointer) is the
 * constant of ACC_CONSTANT.  Types ACC_F32 / ACC_F64 (float weights) and
 * ACC_I32 / ACC_I64 (integer weights, wrapping).  rx, ry in [0, 4]
 * (the reference's largest stencil pattern is 9 wide).  `weights` is a HOST
 * pointer to (2ry+1)(2rx+1) elements of `type`.
 * Replaces stencil1Op / stencilCore (PTX/Execute.hs:652-748). */
int acc_stencil2d(int type, int ry, int rx, const void *weights, int boundary,
                  const void *cval, const void *in, void *out, int64_t h,
                  int64_t w, void *stream);

/* stencil2: two inputs a (ha x wa) and b (hb x wb), out = stencil(a, wa_w)
 * followed by the taps of stencil(b, wb_w) in the same accumulator, over the
 * intersection min(ha,hb) x min(wa,wb) of the shapes (PTX/Execute.hs:682,
 * `intersect`).  Each input's boundary applies at that input's own extent, as
 * each delayed input is bounded by its own shape (CodeGen/Stencil.hs:201-210).
 * Replaces stencil2Op (PTX/Execute.hs:669-684). */
int acc_stencil2d_pair(int type, int ry, int rx, const void *wa_w,
                       const void *wb_w, int boundary_a, const void *cval_a,
                       int boundary_b, const void *cval_b, const void *a,
                       int64_t ha, int64_t wa, const void *b, int64_t hb,
                       int64_t wb, void *out, void *stream);

/* stencil over a rank-3 array in[d][h][w] with a weighted-sum stencil
 * function of (2rz+1) x (2ry+1) x (2rx+1) taps:
 *     out[z][y][x] = sum w[((dz+rz)*(2ry+1)+(dy+ry))*(2rx+1)+(dx+rx)] * in[z+dz][y+dy][x+dx]
 * in that tap order (planes outer, then rows, then columns: a rank-3
 * pattern is a tuple of rank-2 patterns over the outermost index,
 * StencilRtup*, CodeGen/Stencil.hs:126-180); arithmetic, zero-weight taps,
 * `boundary` (applied to every index component), `cval` and the types as
 * for acc_stencil2d; rz, ry, rx in [0, 4].  `weights` is a HOST pointer.
 * Replaces stencil1Op / stencilCore on DIM3 arrays (PTX/Execute.hs:652-748). */
int acc_stencil3d(int type, int rz, int ry, int rx, const void *weights,
                  int boundary, const void *cval, const void *in, void *out,
                  int64_t d, int64_t h, int64_t w, void *stream);

/* ---------------------------------------------------------------- batches */

/* Many independent fold / scanl1 requests in ONE persistent kernel launch.
 * No counterpart in the reference, which launches every skeleton separately
 * (PTX/Execute.hs:835-881): batching amortises the launch and scheduling
 * cost of many small arrays.  A request is fold z xs / fold1 xs (one output element) or
 * scanl1 xs (n outputs; with a seed, the seed is combined on the left of
 * every prefix) over one contiguous vector, element type ACC_I32 / ACC_I64 /
 * ACC_F32 / ACC_F64; every request of a batch uses the same primitive, one
 * of ACC_ADD / ACC_MIN / ACC_MAX (Float32 + is compensated). */
typedef enum acc_request_kind { ACC_REQ_FOLD = 0, ACC_REQ_SCAN = 1 } acc_request_kind;

typedef struct acc_request {
  int kind;          /* acc_request_kind                                   */
  int type;          /* acc_type                                           */
  const void *in;    /* n elements (device)                                */
  void *out;         /* fold: 1 element; scan: n elements (device)         */
  int64_t n;
  int has_seed;      /* 0: fold1 / scanl1 without seed                     */
  uint64_t seed;     /* seed bits in the element type (low bytes)          */
} acc_request;

typedef struct acc_batch acc_batch;  /* opaque plan */

/* Plan a batch: validates the requests, picks the launch shape (threads per
 * CTA) that the autotuner table prefers for most of the batch's bytes, cuts
 * each request into tiles whose shape comes from the same table
 * (acc_batch_autotune / acc_batch_load_tuning; built-in defaults otherwise:
 * 256 threads) and allocates every scratch array the launch will need.  The
 * requests' buffers must stay valid while the plan is used. */
int acc_batch_create(int op, const acc_request *reqs, int64_t count,
                     acc_batch **out);

/* Capture the batch's launch into a CUDA graph once; later acc_batch_launch
 * calls replay the graph. */
int acc_batch_capture(acc_batch *batch, void *stream);

/* Run every request of the batch: one persistent kernel (or one replay of the
 * captured graph).  Stream-ordered; allocates nothing. */
int acc_batch_launch(acc_batch *batch, void *stream);

/* Synchronise `stream` and report a device-side failure of the batch
 * (ACC_ERR_TIMEOUT if a bounded look-back wait ran out). */
int acc_batch_status(acc_batch *batch, void *stream);

/* Free the plan (waits for the device first). */
int acc_batch_destroy(acc_batch *batch);

/* Autotuner: for fold and scan, Int32 / Float32 / Int64 / Float64 and every
 * size bucket 2^8 .. 2^22, time one batched launch per candidate launch shape
 * (128, 256 or 512 threads per CTA) and tile shape (1, 2, 4, ... elements per
 * thread, tiles up to 32 KiB) and keep the fastest pair; the table is used by
 * later acc_batch_create calls and written as JSON to `table_path` (NULL:
 * not written), one entry [kind, type, bucket, elements per thread, threads
 * per CTA] per key. */
int acc_batch_autotune(const char *table_path, void *stream);

/* Load a table written by acc_batch_autotune (entries of four numbers, without
 * the threads per CTA, mean 256). */
int acc_batch_load_tuning(const char *table_path);

/* ---------------------------------------------------------------- serving */

/* A stream of mixed requests served by a continuous-batching loop (no
 * counterpart in the reference).  Request semantics, all over device-resident
 * arrays:
 *   ACC_SK_FOLD     out[0] = fold (+) 0 in[0..n)
 *   ACC_SK_SCAN     out = scanl1 (+) in[0..n)
 *   ACC_SK_FOLDSEG  out[0..m) = foldSeg (+) 0 in[0..n) with Int32 offsets aux[0..m]
 *   ACC_SK_PERMUTE  out[0..m) = histogram of the Int32 indices in[0..n) (permute (+) zeros idx 1)
 *   ACC_SK_STENCIL  out = 5-point stencil (0.25 N/S/E/W, -1 centre, clamp) of the n x m grid in
 *                   (Float32 / Float64 only; other types give ACC_ERR_UNSUPPORTED) */
typedef enum acc_skeleton {
  ACC_SK_FOLD = 0,
  ACC_SK_SCAN = 1,
  ACC_SK_FOLDSEG = 2,
  ACC_SK_PERMUTE = 3,
  ACC_SK_STENCIL = 4
} acc_skeleton;

typedef struct acc_serve_req {
  int skeleton;      /* acc_skeleton                                         */
  int type;          /* element type (permute: ACC_I32)                      */
  const void *in;
  const void *aux;   /* foldSeg offsets, else unused                          */
  void *out;         /* device buffer of the result, or NULL: the loop places
                        the result in its device arena (see acc_serve_run)    */
  int64_t n;         /* elements (stencil: grid rows)                         */
  int64_t m;         /* foldSeg segments / permute bins / stencil grid columns */
  double arrival;    /* seconds after the start of the run, non-decreasing    */
  void *host_out;    /* host buffer the result is copied back to before the
                        request counts as complete, or NULL                  */
} acc_serve_req;

typedef struct acc_serve_stats {
  double wall_s;         /* from the first arrival to the last completion seen */
  int64_t served;
  int64_t batches;       /* batched launches (mode 0)                          */
  int64_t max_inflight;  /* most requests on the GPU at once                   */
  int64_t peak_bytes;    /* most bytes held by admitted requests               */
} acc_serve_stats;

/* Serve `reqs` (sorted by arrival) and write each request's latency in
 * seconds (completion seen by the host minus arrival).  mode 0: continuous
 * batching over `slots` streams; mode 1: plain per-call launches in arrival
 * order on one stream.  Admission by device memory, in both modes: the
 * results of requests with out == NULL are placed in one device arena of
 * `budget_bytes` (allocated once, before the clock starts), and such a
 * request is admitted only once its result fits (its range returns when it
 * completes); requests with their own output buffer are admitted while the
 * bytes of input and output they hold stay within `budget_bytes`.  A result
 * with a host_out buffer (pinned or pageable) is copied back before its
 * request completes.  The call first synchronises the device (the inputs may
 * still be in flight on the caller's streams) and blocks until every request
 * is served. */
int acc_serve_run(const acc_serve_req *reqs, int64_t count, int64_t budget_bytes,
                  int slots, int mode, double *latency, acc_serve_stats *stats);

/* ------------------------------------------------- host <-> device transfer */

/* Copy `bytes` from host memory to device memory (pokeArrayAsync,
 * PTX/Array/Prim.hs:106-135) or back (peekArrayAsync, :169-195), enqueued on
 * `stream` and asynchronous to the host.  The host buffer may be pinned
 * (cudaHostAlloc / cudaHostRegister: copied by the copy engines) or plain
 * pageable memory (malloc, a GHC pinned byte array, a numpy array): on a GPU
 * that reads pageable memory through the host's page tables (GB300 with
 * NVLink-C2C) a copy kernel moves it without staging and without blocking
 * the calling thread; elsewhere the driver stages it and the call may block
 * until the copy is done.  The host buffer must stay valid until the copy
 * has completed (acc_sync on `stream`).  bytes == 0 does nothing. */
int acc_upload(void *dev, const void *host, int64_t bytes, void *stream);
int acc_download(void *host, const void *dev, int64_t bytes, void *stream);

/* A memory table: device copies of host arrays kept in one device arena of a
 * fixed byte budget, allocated once when the table is made, with
 * least-recently-used eviction.  Replaces the PTX backend's memory table
 * (PTX/Array/Table.hs:35-49; Remote.malloc / withRemote,
 * PTX/Array/Remote.hs:60-133) and the transfers the skeleton ops rely on
 * (useArrayAsync / mallocArray / pokeArrayAsync / peekArrayAsync,
 * PTX/Array/Prim.hs:72-195; the lazy copy back of copyToHostLazy,
 * PTX/Array/Data.hs:91-148).  Arrays are keyed by their host address.
 *
 * The table owns two streams, one per direction, so that uploads, the
 * caller's kernels and downloads overlap: an upload runs on the upload
 * stream and the caller's stream waits for it; a download waits for the
 * work enqueued so far on the caller's stream and runs on the download
 * stream.  Between acc_table_use/malloc and acc_table_release an array is
 * held and never evicted; release records the caller's stream as the last
 * user, and an evicted array's space is reused only after that work and any
 * copy back have completed.  An evicted array that the device has written
 * (since malloc, and not yet copied back by peek) is copied back to its host
 * array first; one that holds what its host array holds is dropped.  Calls
 * on one table may come from several host threads (one lock per table). */
typedef struct acc_table acc_table;

typedef struct acc_table_stats {
  int64_t budget;          /* bytes of the arena                                */
  int64_t resident_bytes;  /* bytes held by arrays in the table (rounded)       */
  int64_t arrays;          /* arrays in the table                               */
  int64_t uploads, upload_bytes;
  int64_t downloads, download_bytes;  /* peeks and copies back on eviction      */
  int64_t hits;            /* acc_table_use calls that found the array resident */
  int64_t evictions;
  int64_t writebacks;      /* evictions that copied the array back first        */
} acc_table_stats;

/* Make a table whose arena holds `budget_bytes` (rounded up to 2 MiB). */
int acc_table_create(int64_t budget_bytes, acc_table **out);
/* Wait for the table's work, copy back every array the device has written,
 * and free the arena and the table's streams. */
int acc_table_destroy(acc_table *t);

/* useArrayAsync: hold the device copy of the input array [host, host+bytes)
 * and put its device address in *dev.  If the array is not resident, space
 * is allocated (evicting as needed) and the array is uploaded; `stream`
 * waits for the upload.  A resident array is not copied again: its host
 * array is taken not to change while it is in the table (use poke after a
 * change).  ACC_ERR_NOMEM when the held arrays leave no room. */
int acc_table_use(acc_table *t, const void *host, int64_t bytes, void *stream, void **dev);
/* mallocArray: hold device space for the output array [host, host+bytes),
 * without any copy; the device copy counts as written from now on. */
int acc_table_malloc(acc_table *t, void *host, int64_t bytes, void *stream, void **dev);
/* pokeArrayAsync: copy the host array into its resident device copy again
 * (after the host array changed); `stream` waits for the copy, which itself
 * waits for the last recorded user of the device copy. */
int acc_table_poke(acc_table *t, const void *host, void *stream);
/* peekArrayAsync: copy the device copy back into its host array once the work
 * enqueued so far on `stream` is done.  Asynchronous: acc_table_wait (or a
 * sync of the device) before the host reads the array. */
int acc_table_peek(acc_table *t, void *host, void *stream);
/* End the hold taken by use / malloc: the work enqueued so far on `stream`
 * is the array's last user (withRemote's task). */
int acc_table_release(acc_table *t, const void *host, void *stream);
/* Block until every transfer of the array enqueued so far has completed. */
int acc_table_wait(acc_table *t, const void *host);
/* Make `stream` wait for every transfer enqueued on the table so far. */
int acc_table_join(acc_table *t, void *stream);
/* Drop the array from the table without copying it back (the host array's
 * finalizer; freeRemote).  ACC_ERR_INVALID while it is held. */
int acc_table_free(acc_table *t, const void *host);
int acc_table_get_stats(acc_table *t, acc_table_stats *out);

/* Transfer trace, as the reference times each transfer under its dump_gc
 * debug flag (PTX/Array/Remote.hs, `transfer`): acc_table_trace(t, 1)
 * clears the trace and from then on brackets every transfer with timing
 * events on its stream; acc_table_trace_get waits for the traced transfers
 * and gives, for the first `cap` of them, the kind (0 upload, 1 download,
 * 2 copy back on eviction), the bytes and the start / end in milliseconds
 * after `origin` (a cudaEvent_t created with timing, recorded before the
 * transfers); *count is the number traced. */
typedef struct acc_xfer_record {
  int kind;
  int64_t bytes;
  double start_ms, end_ms;
} acc_xfer_record;
int acc_table_trace(acc_table *t, int enable);
int acc_table_trace_get(acc_table *t, void *origin, acc_xfer_record *rec, int64_t cap, int64_t *count);

#ifdef __cplusplus
}
#endif

#endif /* ACC_GB300_H */
