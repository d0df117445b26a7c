// Shared host-side plumbing of libjmmgpu.so: status codes, the per-thread
// last-error message, CUDA error checks and a device guard.
#pragma once
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/jmm_gpu.h"

namespace jmm {

// Records a formatted message as the calling thread's last error and
// returns `code`, so that call sites read `return fail(JMM_ERR_X, "...")`.
int fail(int code, const char *fmt, ...);
void clear_error();

// Status of a CUDA runtime call, with the call site in the message.
int cuda_status(cudaError_t e, const char *what, const char *file, int line);

}  // namespace jmm

#define JMM_CUDA(call)                                                          \
  do {                                                                          \
    cudaError_t jmm_e_ = (call);                                                \
    if (jmm_e_ != cudaSuccess)                                                  \
      return ::jmm::cuda_status(jmm_e_, #call, __FILE__, __LINE__);             \
  } while (0)

#define JMM_CHECK_ARG(cond, msg)                                                \
  do {                                                                          \
    if (!(cond)) return ::jmm::fail(JMM_ERR_INVALID, "%s: %s", __func__, msg);  \
  } while (0)
