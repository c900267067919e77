// C-ABI plumbing: status text, per-thread error messages, stream-ordered scratch.
#include <atomic>
#include <string>

#include "gbg_common.cuh"

namespace gbg {

namespace {
thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{0};
// Measurement hook: events recorded around the main kernel of a transfer call.
thread_local cudaEvent_t g_main_start = nullptr, g_main_stop = nullptr;
}

void mark_main_start(cudaStream_t st) {
  if (g_main_start) cudaEventRecord(g_main_start, st);
}

void mark_main_stop(cudaStream_t st) {
  if (g_main_stop) cudaEventRecord(g_main_stop, st);
}

gbg_status set_error(gbg_status status, const std::string &message) {
  g_last_error = message;
  return status;
}

void clear_error() { g_last_error.clear(); }

void note_launch(int n) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }

gbg_status Scratch::acquire(void *user, size_t user_bytes, size_t need, cudaStream_t s) {
  stream = s;
  if (need == 0) return GBG_OK;
  if (user) {
    if (user_bytes < need)
      return set_error(GBG_ENOMEM, "workspace too small: need " + std::to_string(need) + " bytes, got " +
                                       std::to_string(user_bytes));
    ptr = user;
    return GBG_OK;
  }
  // Keep freed blocks in the device's default pool: without a release threshold the pool
  // hands its memory back at every synchronization and the next call pays a fresh
  // allocation of the full scratch.
  static thread_local int configured_device = -1;
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev != configured_device) {
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    configured_device = dev;
  }
  cudaError_t e = cudaMallocAsync(&ptr, need, s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    ptr = nullptr;
    return set_error(GBG_ENOMEM, "cudaMallocAsync of " + std::to_string(need) + " bytes failed: " +
                                     cudaGetErrorString(e));
  }
  owned = true;
  return GBG_OK;
}

Scratch::~Scratch() {
  if (owned && ptr) cudaFreeAsync(ptr, stream);
}

}  // namespace gbg

extern "C" {

int32_t gbg_abi_version(void) { return GBG_ABI_VERSION; }

const char *gbg_status_string(gbg_status status) {
  switch (status) {
    case GBG_OK: return "ok";
    case GBG_EARG: return "invalid argument (ArgumentError)";
    case GBG_EDIM: return "dimension mismatch (DimensionMismatch)";
    case GBG_ENOMEM: return "out of device memory or workspace too small";
    case GBG_ECUDA: return "CUDA runtime error";
    case GBG_ENONFINITE: return "non-finite or out-of-range position";
    case GBG_ETIMEOUT: return "timed out";
    case GBG_EUNSUPPORTED: return "unsupported size";
    case GBG_EBUSY: return "busy: admission refused";
    case GBG_ETRAVERSAL: return "traversal order is not a permutation";
    default: return "unknown status";
  }
}

const char *gbg_last_error(void) { return gbg::g_last_error.c_str(); }

uint64_t gbg_kernel_launches(void) { return gbg::g_launches.load(std::memory_order_relaxed); }

gbg_status gbg_set_kernel_timing_events(void *start_event, void *stop_event) {
  gbg::clear_error();
  if ((start_event == nullptr) != (stop_event == nullptr))
    return gbg::set_error(GBG_EARG, "give both events or neither");
  gbg::g_main_start = static_cast<cudaEvent_t>(start_event);
  gbg::g_main_stop = static_cast<cudaEvent_t>(stop_event);
  return GBG_OK;
}

}  // extern "C"
