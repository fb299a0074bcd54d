// Library-wide C ABI helpers: error reporting and version.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "common.cuh"

namespace gbdp {

static thread_local char g_last_error[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

int cuda_status(cudaError_t e, const char* where) {
  set_error("%s: CUDA error %d (%s)", where, (int)e, cudaGetErrorString(e));
  return GBDP_ERR_CUDA;
}

}  // namespace gbdp

extern "C" const char* gbdp_last_error(void) { return gbdp::g_last_error; }

extern "C" int gbdp_version(void) { return 100; }
