// selftest.cu -- a check that the library's bounded device waits give up.
//
// Every wait of one CTA on another (the decoupled look-back of the scans and
// foldSeg) and every wait for a TMA copy (the mbarrier of every tiled kernel)
// is bounded: when it runs out, the kernel raises DEV_ERR_TIMEOUT in the
// stream's error word and returns, and acc_sync reports ACC_ERR_TIMEOUT.
// The kernels here run those same wait routines against something that
// nothing completes (an mbarrier phase without an arrival, a predecessor
// tile that never publishes), so that the give-up path runs on purpose:
// each wait ends after its limit (seconds), the kernel returns, and the
// context stays usable.
#include "scan_impl.cuh"

namespace accgb {
namespace {

// One warp waits for an mbarrier phase that no thread and no copy completes.
__global__ void selftest_mbar_kernel(uint32_t *err) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (__syncthreads_or(!mbar_wait_flagged(&bar, 0, err))) return;
  // not reached: the phase never completes
  if (threadIdx.x == 0) raise_error(err, DEV_ERR_INDEX);
}

// One warp runs the look-back of tile 1 of a two-tile scan whose tile 0
// never publishes (its slot carries no tag of this epoch).
__global__ void selftest_lookback_kernel(ScanArgs a) {
  using A = Acc<ACC_ADD, int32_t, 0>;
  const int32_t v = lookback_prefix<A, false, SCAN_LOOKBACK>(a, 1);
  // The abandoned slot counts as the identity: a result that is not the
  // identity means the wait did not end by giving up.
  if (threadIdx.x == 0 && v != A::id()) raise_error(a.err, DEV_ERR_INDEX);
}

}  // namespace
}  // namespace accgb

using namespace accgb;

extern "C" int acc_selftest_timeout(int which, void *stream) {
  if (which != 0 && which != 1) return ACC_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int st = ACC_OK;
  Workspace *w = workspace(s, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  if (which == 0) {
    selftest_mbar_kernel<<<1, 32, 0, s>>>(w->words + W_ERR);
    return check_launch();
  }
  st = ws_status(w, 2 * 2);
  if (st) return st;
  ScanArgs a{};
  a.n = 2;
  a.ntiles = 2;
  a.status = w->status;
  a.err = w->words + W_ERR;
  // A fresh epoch: no slot holds a tag of it until a tile of this launch
  // publishes, and tile 0 is never run.
  a.epoch = ws_next_epoch(w, s);
  selftest_lookback_kernel<<<1, 32, 0, s>>>(a);
  return check_launch();
}
