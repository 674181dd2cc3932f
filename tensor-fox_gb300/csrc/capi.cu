// C ABI plumbing shared by every entry point: error reporting, a launch
// counter (how many kernels this library enqueued) and version information.
#include <atomic>
#include <stdio.h>
#include <string.h>

#include "tfx_capi_internal.h"

static thread_local char g_err[512] = {0};
static std::atomic<long long> g_launches{0};

int tfx_set_error(int status, const char* msg) {
  snprintf(g_err, sizeof(g_err), "%s", msg ? msg : "");
  return status;
}

int tfx_set_cuda_error(cudaError_t e, const char* where) {
  snprintf(g_err, sizeof(g_err), "%s: %s", where ? where : "cuda", cudaGetErrorString(e));
  return TFX_STATUS_ERR_CUDA;
}

void tfx_count_launch(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

extern "C" const char* tfx_last_error(void) { return g_err; }

extern "C" long long tfx_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

extern "C" int tfx_version(void) { return 10000; }
