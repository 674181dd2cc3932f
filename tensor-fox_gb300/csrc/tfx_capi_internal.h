// Internal helpers of the C ABI: thread-local error message and a launch counter.
#pragma once
#include <cuda_runtime.h>
#include "../../include/tfx_gb300_types.h"

int tfx_set_error(int status, const char* msg);
int tfx_set_cuda_error(cudaError_t e, const char* where);
void tfx_count_launch(long long n);
