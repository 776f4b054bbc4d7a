// common.h — status codes, the per-thread last-error text and small helpers
// shared by the library's translation units.
#pragma once
#include <cstdarg>
#include <cstdio>
#include <string>

#include "../../include/asuna_rt.h"

namespace asuna {

// Records the failure text for asuna_last_error() and returns `code`.
int fail(int code, const char* fmt, ...);
void clearError();

}  // namespace asuna

#define ASUNA_CUDA_TRY(call)                                                                     \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess)                                                                       \
      return ::asuna::fail(e_ == cudaErrorMemoryAllocation ? ASUNA_ERR_OOM : ASUNA_ERR_CUDA,     \
                           "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)
