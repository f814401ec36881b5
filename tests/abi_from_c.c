/*
 * abi_from_c.c -- a C99 caller of libaccgb.so, built and run by
 * tests/test_abi.py on a machine without a GPU.
 *
 * A Haskell `cbits` binding (or any other FFI) sees the library only through
 * include/acc_gb300.h.  This program is such a caller: it includes the header
 * as plain C (no C++ and no CUDA headers), links against the shared library
 * by name, and checks the calls that are answered before any device work:
 * the version and error strings, and argument validation of every skeleton
 * entry point.  Each check prints one line; the exit status is the number of
 * failed checks.
 */
#include <stdio.h>
#include <string.h>

#include "acc_gb300.h"

static int failures = 0;

static void expect(const char *what, int got, int want) {
  if (got != want) {
    printf("FAIL %s: got %d (%s), want %d\n", what, got, acc_strerror(got), want);
    ++failures;
  } else {
    printf("ok   %s\n", what);
  }
}

int main(void) {
  char buf[16];
  void *p = buf; /* a non-null host pointer; no call below dereferences it */
  const int64_t one = 1;
  acc_batch *batch = NULL;
  acc_request req;
  double latency[1];
  acc_serve_req sreq;

  memset(&req, 0, sizeof(req));
  expect("acc_version", acc_version(), ACC_GB300_ABI_VERSION);
  expect("acc_strerror(ACC_OK)", strcmp(acc_strerror(ACC_OK), "ok"), 0);

  /* fold: negative extent; fold1 of an empty row */
  expect("fold, negative outer", acc_fold(ACC_ADD, ACC_I32, ACC_PREC_DEFAULT, NULL, NULL, -1, 4, NULL, NULL),
         ACC_ERR_INVALID);
  expect("fold1, empty row", acc_fold(ACC_ADD, ACC_I32, ACC_PREC_DEFAULT, NULL, p, 2, 0, NULL, NULL),
         ACC_ERR_EMPTY);
  expect("fold zipWith, bad zip primitive",
         acc_fold_zipwith(ACC_ADD, 9, ACC_I32, ACC_PREC_DEFAULT, NULL, NULL, p, 1, 4, NULL, NULL), ACC_ERR_INVALID);

  /* scans: bad direction, scanl without a seed, scanl' without a total */
  expect("scan, bad direction", acc_scan(ACC_ADD, ACC_I32, ACC_PREC_DEFAULT, 7, ACC_SCAN_INCLUSIVE, NULL, NULL, NULL,
                                          1, 4, NULL, NULL), ACC_ERR_INVALID);
  expect("scanl without seed", acc_scan(ACC_ADD, ACC_I32, ACC_PREC_DEFAULT, ACC_L2R, ACC_SCAN_SEEDED, NULL, NULL,
                                         NULL, 1, 4, NULL, NULL), ACC_ERR_INVALID);
  expect("scan zipWith, scanl' without sums",
         acc_scan_zipwith(ACC_ADD, ACC_MUL, ACC_I32, ACC_PREC_DEFAULT, ACC_L2R, ACC_SCAN_PRIME, p, p, p, NULL, 1, 4,
                          p, NULL), ACC_ERR_INVALID);
  expect("scan noalloc, row beyond its scratch",
         acc_scan_noalloc(ACC_ADD, ACC_I64, ACC_PREC_DEFAULT, ACC_L2R, ACC_SCAN_INCLUSIVE, p, p, NULL, 1,
                          ((int64_t)1 << 28) + 1, NULL, NULL), ACC_ERR_TOO_LARGE);

  /* foldSeg: bad offset type; fused producer without its second input */
  expect("foldSeg, bad offset type", acc_fold_seg(ACC_ADD, ACC_I32, ACC_PREC_DEFAULT, NULL, NULL, 3, NULL, 1, 4, 2,
                                                  NULL, NULL), ACC_ERR_INVALID);
  expect("foldSeg zipWith, missing ys", acc_fold_seg_zipwith(ACC_ADD, ACC_MUL, ACC_I32, ACC_PREC_DEFAULT, p, NULL, p,
                                                             ACC_I32, p, 1, 4, 2, NULL, NULL), ACC_ERR_INVALID);

  /* permute: neither a source nor a constant; bad index type */
  expect("permute, no source", acc_permute(ACC_ADD, ACC_I32, NULL, NULL, NULL, ACC_I32, NULL, 4, 4, NULL),
         ACC_ERR_INVALID);
  expect("permute, bad index type", acc_permute(ACC_ADD, ACC_I32, NULL, NULL, NULL, 9, NULL, 4, 4, NULL),
         ACC_ERR_INVALID);

  /* stencils: radius above 4, Word32, constant boundary without its value */
  expect("stencil2d, radius above 4", acc_stencil2d(ACC_F32, 5, 1, NULL, ACC_CLAMP, NULL, NULL, NULL, 4, 4, NULL),
         ACC_ERR_INVALID);
  expect("stencil2d, Word32", acc_stencil2d(ACC_U32, 1, 1, NULL, ACC_CLAMP, NULL, NULL, NULL, 4, 4, NULL),
         ACC_ERR_UNSUPPORTED);
  expect("stencil3d, constant without value",
         acc_stencil3d(ACC_F32, 1, 1, 1, p, ACC_CONSTANT, NULL, p, p, 4, 4, 4, NULL), ACC_ERR_INVALID);
  expect("stencil3d, empty", acc_stencil3d(ACC_F32, 1, 1, 1, NULL, ACC_CLAMP, NULL, NULL, NULL, 0, 4, 4, NULL),
         ACC_OK);

  /* batches and serving: the host-side checks that precede any device work */
  expect("batch create, no result pointer", acc_batch_create(ACC_ADD, &req, 1, NULL), ACC_ERR_INVALID);
  req.kind = ACC_REQ_FOLD; /* fold z [] with nowhere to write z */
  req.type = ACC_I32;
  req.n = 0;
  req.has_seed = 1;
  expect("batch create, fold without output", acc_batch_create(ACC_ADD, &req, 1, &batch), ACC_ERR_INVALID);
  expect("batch launch, no batch", acc_batch_launch(NULL, NULL), ACC_ERR_INVALID);
  expect("batch destroy, no batch", acc_batch_destroy(batch), ACC_OK);
  expect("batch tuning, no path", acc_batch_load_tuning(NULL), ACC_ERR_INVALID);
  memset(&sreq, 0, sizeof(sreq));
  expect("serve, no slots", acc_serve_run(&sreq, 1, one << 20, 0, 0, latency, NULL), ACC_ERR_INVALID);
  expect("serve, bad mode", acc_serve_run(&sreq, 1, one << 20, 4, 7, latency, NULL), ACC_ERR_INVALID);
  sreq.type = ACC_F32; /* a fold with no input buffer */
  sreq.n = 16;
  sreq.in = NULL;
  expect("serve, fold without input", acc_serve_run(&sreq, 1, one << 20, 4, 0, latency, NULL), ACC_ERR_INVALID);
  sreq.in = p;
  sreq.type = 9;
  expect("serve, bad element type", acc_serve_run(&sreq, 1, one << 20, 4, 0, latency, NULL), ACC_ERR_INVALID);
  sreq.skeleton = ACC_SK_STENCIL;
  sreq.type = ACC_I32;
  expect("serve, Int32 5-point stencil", acc_serve_run(&sreq, 1, one << 20, 4, 0, latency, NULL),
         ACC_ERR_UNSUPPORTED);

  printf("%d failed\n", failures);
  return failures;
}
