// Host-side staging of many small input tensors into one pinned buffer, so a
// batch crosses to the device in a single copy.  The copies are split over
// host threads by byte volume (a Grace host has tens of cores; one thread
// copies at a fraction of its memory bandwidth).
#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "tfx_capi_internal.h"

extern "C" int tfx_host_gather(const void* const* src, const long long* bytes, const long long* dst_off, int n,
                               void* dst, int threads) {
  if (n < 0 || (n > 0 && (!src || !bytes || !dst_off || !dst))) return tfx_set_error(TFX_STATUS_ERR_ARG, "host_gather");
  if (n == 0) return TFX_STATUS_OK;
  long long total = 0;
  for (int i = 0; i < n; ++i) {
    if (bytes[i] < 0 || dst_off[i] < 0 || (bytes[i] > 0 && !src[i])) return tfx_set_error(TFX_STATUS_ERR_ARG, "host_gather entry");
    total += bytes[i];
  }
  int nt = std::max(1, std::min(threads, 64));
  if (total < (8LL << 20)) nt = 1;
  // contiguous ranges of problems with about total / nt bytes each
  std::vector<int> cut(nt + 1, n);
  cut[0] = 0;
  long long acc = 0;
  int k = 1;
  for (int i = 0; i < n && k < nt; ++i) {
    acc += bytes[i];
    if (acc >= total * k / nt) cut[k++] = i + 1;
  }
  auto work = [&](int t) {
    for (int i = cut[t]; i < cut[t + 1]; ++i)
      if (bytes[i] > 0) memcpy((char*)dst + dst_off[i], src[i], (size_t)bytes[i]);
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) pool.emplace_back(work, t);
  work(0);
  for (auto& th : pool) th.join();
  return TFX_STATUS_OK;
}
