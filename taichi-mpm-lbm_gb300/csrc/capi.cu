// Error reporting and versioning of the C ABI.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "fsi_common.cuh"

namespace fsi {

static thread_local char g_error[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_error, sizeof(g_error), fmt, ap);
  va_end(ap);
}

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return FSI_ERR_CUDA;
  }
  return FSI_OK;
}

}  // namespace fsi

extern "C" int fsi_abi_version(void) { return FSI_ABI_VERSION; }

extern "C" size_t fsi_last_error(char* buf, size_t len) {
  size_t n = strlen(fsi::g_error);
  if (buf && len) {
    size_t m = n < len - 1 ? n : len - 1;
    memcpy(buf, fsi::g_error, m);
    buf[m] = '\0';
  }
  return n;
}
