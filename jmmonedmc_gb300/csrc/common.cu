// Host plumbing shared by every entry point of libjmmgpu.so.
#include <string.h>

#include "common.cuh"

namespace jmm {

static thread_local char g_last_error[1024] = "";

int fail(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

void clear_error() { g_last_error[0] = '\0'; }

int cuda_status(cudaError_t e, const char *what, const char *file, int line) {
  int code = (e == cudaErrorMemoryAllocation) ? JMM_ERR_NOMEM : JMM_ERR_CUDA;
  // a failed call leaves its (non-sticky) error as the runtime's last error:
  // clear it, so that a later launch check does not report it again
  cudaGetLastError();
  return fail(code, "%s failed at %s:%d: %s (%s)", what, file, line, cudaGetErrorName(e),
              cudaGetErrorString(e));
}

}  // namespace jmm

extern "C" const char *jmm_last_error(void) { return jmm::g_last_error; }

extern "C" int jmm_device_available(void) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return count > 0 ? 1 : 0;
}
