// Fitting net of one atom type: energy per atom and dE/dD in one call
// (deepmd/pt/model/task/fitting.py:734-899 with the layer semantics of
// deepmd/dpmodel/utils/network.py: hidden layers y = tanh(x W + b) * idt
// (+ x when the width is kept), then a linear layer to one energy).
//
// The GEMMs go to cuBLAS with a caller-chosen compute type; everything
// between them (bias, tanh, time step, skip, the energy dot product and the
// backward elementwise chain) is one small fused kernel per layer:
//   forward   Z_l = H_{l-1} W_l        (GEMM)       H_l = tanh(Z_l + b_l) idt_l [+ H_{l-1}]
//   energy    e = H_L w_out + b_out + bias, and G = w_out broadcast (seed)
//   backward  GZ_l = G idt_l (1 - T_l^2);  G = GZ_l W_l^T [+ G]   (GEMM, beta 1)
//             dD = GZ_1 W_1^T
#include <cublas_v2.h>

#include <mutex>

#include "common.cuh"

namespace gbdp {
namespace {

constexpr int kMaxFitLayers = 8;

// T = tanh(T + b) in place; H = T * idt (+ Hprev)
__global__ void k_fit_act(float* __restrict__ T, float* __restrict__ H,
                          const float* __restrict__ b, const float* __restrict__ idt,
                          const float* __restrict__ Hprev, int n, int w) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)n * w) return;
  const int c = (int)(idx % w);
  const float t = tanhf(T[idx] + b[c]);
  T[idx] = t;
  if (H != T) {
    float h = idt ? t * idt[c] : t;
    if (Hprev) h += Hprev[idx];
    H[idx] = h;
  }
}

// e[r] = H[r] . w_out + b_out + bias; G[r, :] = w_out (backward seed)
__global__ void k_fit_out(float* __restrict__ e, float* __restrict__ G,
                          const float* __restrict__ H, const float* __restrict__ wout,
                          float b_out, int n, int w) {
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= n) return;
  float s = 0.f;
  for (int c = lane; c < w; c += 32) {
    const float wo = wout[c];
    s += H[(size_t)r * w + c] * wo;
    G[(size_t)r * w + c] = wo;
  }
  s = warp_sum(s);
  if (lane == 0) e[r] = s + b_out;
}

// GZ = G * idt * (1 - T^2)
__global__ void k_fit_bwd_elem(float* __restrict__ GZ, const float* __restrict__ G,
                               const float* __restrict__ T, const float* __restrict__ idt, int n,
                               int w) {
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (size_t)n * w) return;
  const int c = (int)(idx % w);
  const float t = T[idx];
  float g = G[idx];
  if (idt) g *= idt[c];
  GZ[idx] = g * (1.f - t * t);
}

std::mutex g_handle_mu;
cublasHandle_t g_handle[64] = {};

int get_handle(cublasHandle_t* h) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "fitting: cudaGetDevice");
  GBDP_REQUIRE(dev >= 0 && dev < 64, "fitting: device ordinal %d", dev);
  std::lock_guard<std::mutex> lock(g_handle_mu);
  if (!g_handle[dev]) {
    cublasStatus_t s = cublasCreate(&g_handle[dev]);
    GBDP_REQUIRE(s == CUBLAS_STATUS_SUCCESS, "fitting: cublasCreate failed (%d)", (int)s);
  }
  *h = g_handle[dev];
  return GBDP_OK;
}

size_t a256f(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kCublasWs = size_t(32) << 20;

struct FitWs {
  float* t[kMaxFitLayers];  // tanh outputs (also H when no idt/skip)
  float* h[kMaxFitLayers];  // layer outputs
  float* g;                 // running gradient
  float* gz;
  void* cublas_ws;
  size_t bytes;
};

FitWs carve_fit(void* base, int n, const int* widths, const int* has_h, int nl) {
  FitWs w{};
  char* b = static_cast<char*>(base);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char* r = b ? b + off : nullptr;
    off += a256f(bytes);
    return r;
  };
  int wmax = 0;
  for (int l = 1; l <= nl; ++l) {
    w.t[l - 1] = reinterpret_cast<float*>(take(sizeof(float) * (size_t)n * widths[l]));
    w.h[l - 1] = has_h[l - 1] ? reinterpret_cast<float*>(take(sizeof(float) * (size_t)n * widths[l]))
                             : w.t[l - 1];
    wmax = widths[l] > wmax ? widths[l] : wmax;
  }
  w.g = reinterpret_cast<float*>(take(sizeof(float) * (size_t)n * wmax));
  w.gz = reinterpret_cast<float*>(take(sizeof(float) * (size_t)n * wmax));
  w.cublas_ws = take(kCublasWs);
  w.bytes = off;
  return w;
}

cublasComputeType_t compute_type(int mode) {
  switch (mode) {
    case 1:
      return CUBLAS_COMPUTE_32F_EMULATED_16BFX9;
    case 2:
      return CUBLAS_COMPUTE_32F_FAST_TF32;
    case 3:
      return CUBLAS_COMPUTE_32F_FAST_16BF;
    default:
      return CUBLAS_COMPUTE_32F_PEDANTIC;
  }
}

// row-major C[r, c_out] = A[r, k] @ B[k, c_out] (+ beta C), i.e. column-major
// C^T = B^T A^T; trans_b: use B^T where B is stored row-major [c_out, k]
int gemm_rm(cublasHandle_t h, int mode, float* C, const float* A, const float* B, int rows,
            int k, int cols, bool trans_b, float beta) {
  const float alpha = 1.f;
  cublasStatus_t s;
  if (!trans_b)
    s = cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, cols, rows, k, &alpha, B, CUDA_R_32F, cols, A,
                     CUDA_R_32F, k, &beta, C, CUDA_R_32F, cols, compute_type(mode),
                     CUBLAS_GEMM_DEFAULT);
  else
    s = cublasGemmEx(h, CUBLAS_OP_T, CUBLAS_OP_N, cols, rows, k, &alpha, B, CUDA_R_32F, k, A,
                     CUDA_R_32F, k, &beta, C, CUDA_R_32F, cols, compute_type(mode),
                     CUBLAS_GEMM_DEFAULT);
  GBDP_REQUIRE(s == CUBLAS_STATUS_SUCCESS, "fitting: cublasGemmEx failed (%d), mode %d", (int)s,
               mode);
  return GBDP_OK;
}

}  // namespace
}  // namespace gbdp

using namespace gbdp;

static void fit_has_h(const int* widths, const float* const* idt, int nl, int* has_h) {
  for (int l = 1; l <= nl; ++l)
    has_h[l - 1] = (idt && idt[l - 1]) || widths[l] == widths[l - 1];
}

extern "C" size_t gbdp_fitting_workspace_bytes(int n, const int* widths, int n_hidden,
                                               const float* const* idt) {
  if (n_hidden < 1 || n_hidden > kMaxFitLayers || !widths) return 0;
  int has_h[kMaxFitLayers];
  fit_has_h(widths, idt, n_hidden, has_h);
  return carve_fit(nullptr, n, widths, has_h, n_hidden).bytes;
}

extern "C" int gbdp_fitting_fwd_bwd_f32(float* e, float* dD, const float* D, int n,
                                        const int* widths, int n_hidden,
                                        const float* const* w, const float* const* b,
                                        const float* const* idt, const float* w_out,
                                        float b_out, int gemm_mode, void* workspace,
                                        size_t workspace_bytes, gbdp_stream stream) {
  GBDP_REQUIRE(n_hidden >= 1 && n_hidden <= kMaxFitLayers, "fitting: %d hidden layers",
               n_hidden);
  GBDP_REQUIRE(widths && w && b && w_out, "fitting: null argument");
  GBDP_REQUIRE(gemm_mode >= 0 && gemm_mode <= 3, "fitting: gemm_mode %d", gemm_mode);
  int has_h[kMaxFitLayers];
  fit_has_h(widths, idt, n_hidden, has_h);
  FitWs ws = carve_fit(workspace, n, widths, has_h, n_hidden);
  GBDP_REQUIRE(workspace && workspace_bytes >= ws.bytes, "fitting: workspace %zu < %zu",
               workspace_bytes, ws.bytes);
  if (n == 0) return GBDP_OK;
  GBDP_REQUIRE(e && dD && D, "fitting: null input/output");
  cublasHandle_t h;
  int rc = get_handle(&h);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  cublasSetStream(h, st);
  cublasSetWorkspace(h, ws.cublas_ws, kCublasWs);
  if (gemm_mode == 1) cublasSetEmulationStrategy(h, CUBLAS_EMULATION_STRATEGY_EAGER);
  const int tb = 256;
  // ---- forward
  const float* x = D;
  for (int l = 1; l <= n_hidden; ++l) {
    const int wi = widths[l - 1], wo = widths[l];
    rc = gemm_rm(h, gemm_mode, ws.t[l - 1], x, w[l - 1], n, wi, wo, false, 0.f);
    if (rc) return rc;
    const bool skip = wi == wo;
    const size_t cnt = (size_t)n * wo;
    k_fit_act<<<(unsigned)((cnt + tb - 1) / tb), tb, 0, st>>>(
        ws.t[l - 1], ws.h[l - 1], b[l - 1], idt ? idt[l - 1] : nullptr, skip ? x : nullptr, n, wo);
    x = ws.h[l - 1];
  }
  const int wl = widths[n_hidden];
  k_fit_out<<<(unsigned)(((size_t)n * 32 + tb - 1) / tb), tb, 0, st>>>(e, ws.g, x, w_out, b_out, n,
                                                                       wl);
  // ---- backward
  for (int l = n_hidden; l >= 1; --l) {
    const int wi = widths[l - 1], wo = widths[l];
    const size_t cnt = (size_t)n * wo;
    k_fit_bwd_elem<<<(unsigned)((cnt + tb - 1) / tb), tb, 0, st>>>(
        ws.gz, ws.g, ws.t[l - 1], idt ? idt[l - 1] : nullptr, n, wo);
    if (l > 1) {
      // G_{l-1} = GZ W_l^T (+ G_l when the layer has a skip; G is wi wide then)
      const bool skip = wi == wo;
      rc = gemm_rm(h, gemm_mode, ws.g, ws.gz, w[l - 1], n, wo, wi, true, skip ? 1.f : 0.f);
    } else {
      rc = gemm_rm(h, gemm_mode, dD, ws.gz, w[0], n, wo, wi, true, 0.f);
    }
    if (rc) return rc;
  }
  GBDP_CHECK_LAUNCH("fitting_fwd_bwd");
  return GBDP_OK;
}
