// Library-wide C ABI helpers: error reporting, version, and the self-test
// of the bounded device waits.
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

// ---------------------------------------------------- bounded-wait self-test --
// The tensor-core kernels wait on mbarriers through mbar_wait_bounded: after
// `limit` polls a wait gives up, raises GBDP_STATUS_TIMEOUT in the launch's
// status word and the kernel winds down instead of spinning forever.  This
// kernel runs that path where nothing can be left in flight: lane 0 first
// completes phase 0 of a barrier with a real 16-byte bulk copy (the wait is
// satisfied and the data arrives), then waits on phase 1, which nothing ever
// completes, with the caller's poll limit.
namespace {
__global__ void k_selftest_wait(int* status, int* result, long limit) {
  __shared__ __align__(16) int4 buf;
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    gbdp::mbar_init(&bar, 1);
    gbdp::fence_mbar_init();
    gbdp::mbar_expect_tx(&bar, 16);
    gbdp::bulk_g2s(&buf, result, 16, &bar);
    const bool first = gbdp::mbar_wait_bounded(&bar, 0u, status);
    const int got = first ? buf.x + 1 : -1;
    const bool second = gbdp::mbar_wait_bounded(&bar, 1u, status, limit);
    result[0] = got;
    result[1] = second ? 1 : 0;
  }
}
}  // namespace

extern "C" int gbdp_selftest_wait_timeout(int* status, int* result, long long limit,
                                          gbdp_stream stream) {
  GBDP_REQUIRE(status && result, "selftest_wait_timeout: null status/result");
  GBDP_REQUIRE(((uintptr_t)result & 15) == 0, "selftest_wait_timeout: result not 16-byte aligned");
  GBDP_REQUIRE(limit >= 1, "selftest_wait_timeout: limit must be >= 1");
  k_selftest_wait<<<1, 32, 0, (cudaStream_t)stream>>>(status, result, (long)limit);
  GBDP_CHECK_LAUNCH("selftest_wait_timeout");
  return GBDP_OK;
}
