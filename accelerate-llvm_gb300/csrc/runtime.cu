// runtime.cu -- workspaces, device facts, tensor-map encoding, status codes.
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <utility>

#include "runtime.h"

namespace accgb {

namespace {
std::mutex g_mu;
std::map<std::pair<int, cudaStream_t>, std::unique_ptr<Workspace>> g_ws;
Device g_dev[64];
bool g_dev_ok[64] = {};

using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                   const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                   const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                   CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn g_encode = nullptr;
std::once_flag g_encode_once;
}  // namespace

const Device &device_info() {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_dev_ok[dev]) {
    Device d{};
    d.id = dev;
    cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&d.max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaDeviceGetAttribute(&d.cc_major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&d.cc_minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (d.sms <= 0) d.sms = 1;
    g_dev[dev] = d;
    g_dev_ok[dev] = true;
  }
  return g_dev[dev];
}

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return ACC_OK;
  if (e == cudaErrorMemoryAllocation) return ACC_ERR_NOMEM;
  return ACC_ERR_CUDA;
}

int check_launch() { return cuda_status(cudaGetLastError()); }

Workspace *workspace(cudaStream_t s, int *status) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) { *status = cuda_status(e); return nullptr; }
  std::lock_guard<std::mutex> lk(g_mu);
  auto key = std::make_pair(dev, s);
  auto it = g_ws.find(key);
  if (it != g_ws.end()) { *status = ACC_OK; return it->second.get(); }
  auto w = std::make_unique<Workspace>();
  w->device = dev;
  w->stream = s;
  Workspace *raw = w.get();
  g_ws.emplace(key, std::move(w));
  *status = ws_words(raw, 64);
  if (*status != ACC_OK) {
    // No control words (ticket, error word): the workspace is unusable, so it
    // is not kept for the next call on this stream either.
    g_ws.erase(key);
    return nullptr;
  }
  return raw;
}

int ws_words(Workspace *w, size_t n) {
  if (n <= w->nwords) return ACC_OK;
  size_t cap = w->nwords ? w->nwords : 64;
  while (cap < n) cap *= 2;
  uint32_t *p = nullptr;
  cudaError_t e = cudaMalloc(&p, cap * sizeof(uint32_t));
  if (e != cudaSuccess) return cuda_status(e);
  // Zero the new area, keep the error word of the old one.
  e = cudaMemsetAsync(p, 0, cap * sizeof(uint32_t), w->stream);
  if (e != cudaSuccess) { cudaFree(p); return cuda_status(e); }
  if (w->words) {
    cudaMemcpyAsync(p, w->words, sizeof(uint32_t), cudaMemcpyDeviceToDevice, w->stream);
    cudaStreamSynchronize(w->stream);
    cudaFree(w->words);
  }
  w->words = p;
  w->nwords = cap;
  return ACC_OK;
}

int ws_status(Workspace *w, size_t n) {
  if (n <= w->nstatus) return ACC_OK;
  size_t cap = w->nstatus ? w->nstatus : 4096;
  while (cap < n) cap *= 2;
  if (w->status) { cudaStreamSynchronize(w->stream); cudaFree(w->status); w->status = nullptr; w->nstatus = 0; }
  uint64_t *p = nullptr;
  cudaError_t e = cudaMalloc(&p, cap * sizeof(uint64_t));
  if (e != cudaSuccess) return cuda_status(e);
  e = cudaMemsetAsync(p, 0, cap * sizeof(uint64_t), w->stream);
  if (e != cudaSuccess) { cudaFree(p); return cuda_status(e); }
  w->status = p;
  w->nstatus = cap;
  w->epoch = 0;
  return ACC_OK;
}

int ws_scratch(Workspace *w, size_t bytes) {
  if (bytes <= w->nscratch) return ACC_OK;
  size_t cap = w->nscratch ? w->nscratch : (1u << 20);
  while (cap < bytes) cap *= 2;
  if (w->scratch) { cudaStreamSynchronize(w->stream); cudaFree(w->scratch); w->scratch = nullptr; w->nscratch = 0; }
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, cap);
  if (e != cudaSuccess) return cuda_status(e);
  w->scratch = p;
  w->nscratch = cap;
  return ACC_OK;
}

uint32_t ws_next_epoch(Workspace *w, cudaStream_t s) {
  // Epochs live in 29 bits of the status tag (the segmented scan of foldSeg
  // uses one more tag bit).  On wrap-around the slots are cleared so that no
  // stale tag can ever match.
  w->epoch += 1;
  if (w->epoch >= (1u << 29)) {
    cudaMemsetAsync(w->status, 0, w->nstatus * sizeof(uint64_t), s);
    w->epoch = 1;
  }
  return w->epoch;
}

bool encode_2d(CUtensorMap *map, const void *base, int elem_bytes, uint64_t inner,
               uint64_t outer, uint64_t row_pitch_bytes, uint32_t box_inner,
               uint32_t box_outer, bool swizzle128) {
  std::call_once(g_encode_once, [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                         cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = reinterpret_cast<EncodeTiledFn>(fn);
  });
  if (!g_encode) return false;
  if (!aligned16(base) || (row_pitch_bytes & 15u) || inner == 0 || outer == 0) return false;
  CUtensorMapDataType dt = elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_UINT32
                           : elem_bytes == 8 ? CU_TENSOR_MAP_DATA_TYPE_INT64
                                             : CU_TENSOR_MAP_DATA_TYPE_UINT8;
  cuuint64_t dims[2] = {inner, outer};
  cuuint64_t strides[1] = {row_pitch_bytes};
  cuuint32_t box[2] = {box_inner, box_outer};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(map, dt, 2, const_cast<void *>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE,
                        swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace accgb

using namespace accgb;

extern "C" int acc_version(void) { return ACC_GB300_ABI_VERSION; }

extern "C" const char *acc_strerror(int status) {
  switch (status) {
    case ACC_OK: return "ok";
    case ACC_ERR_INVALID: return "invalid argument";
    case ACC_ERR_UNSUPPORTED: return "unsupported combine function for this element type";
    case ACC_ERR_EMPTY: return "empty array";
    case ACC_ERR_CUDA: return "CUDA runtime error";
    case ACC_ERR_NOMEM: return "out of device memory";
    case ACC_ERR_TIMEOUT: return "a bounded device-side wait timed out";
    case ACC_ERR_INDEX: return "permute index out of range";
    case ACC_ERR_TOO_LARGE: return "extent larger than this entry point accepts";
    default: return "unknown status";
  }
}

extern "C" int acc_sync(void *stream) {
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_status(e);
  int st = ACC_OK;
  Workspace *w = workspace(s, &st);
  if (!w) return st;
  std::lock_guard<std::mutex> lk(w->mu);
  uint32_t err = 0;
  e = cudaMemcpy(&err, w->words + W_ERR, sizeof(uint32_t), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(e);
  if (err == 0) return ACC_OK;
  // Clear the error word and every ticket: a kernel that gave up may have
  // left its counters mid-way.
  cudaMemset(w->words, 0, w->nwords * sizeof(uint32_t));
  if (w->status) cudaMemset(w->status, 0, w->nstatus * sizeof(uint64_t));
  w->epoch = 0;
  if (err & DEV_ERR_TIMEOUT) return ACC_ERR_TIMEOUT;
  return ACC_ERR_INDEX;
}

extern "C" int acc_release_workspaces(void) {
  cudaDeviceSynchronize();
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto &kv : g_ws) {
    Workspace *w = kv.second.get();
    if (w->words) cudaFree(w->words);
    if (w->status) cudaFree(w->status);
    if (w->scratch) cudaFree(w->scratch);
  }
  g_ws.clear();
  return ACC_OK;
}
