// Tabulated se_e2_a embedding fused with the G^T.R contraction (sm_103a):
// the operator-contract kernels behind deepmd::tabulate_fusion_se_a.
//
// out[i, m, k] = sum_j w_j em[i, j, m] P_k(x_ij), P_k the fifth-order
// polynomial of table row locate(x_ij).  The nloc x nnei x M embedding is
// never materialised.  Reference semantics: source/lib/src/tabulate.cc:80-384
// (CPU, the oracle) and source/lib/src/gpu/tabulate.cu:196-503.
//
// Work split (one warp per centre atom):
//   forward / grad-grad: lanes over the M outputs k (coalesced row reads,
//     one broadcast em row per neighbour), neighbours sequential;
//   grad: also lanes over k; the per-neighbour sums over k are reduced six
//     neighbours at a time with a reduce-scatter across the warp.
// The padding fold (tabulate.cc:108-155): with is_sorted, the first slot
// whose x equals the last slot's x and whose em[1:4] are zero stands for all
// remaining slots (weight nnei - j) and ends the sum; slots after it get no
// gradient.
#include "common.cuh"

namespace gbdp {
namespace {

constexpr int kTabWarps = 4;

// First fold slot of atom i (nnei if none), found by the whole warp.
template <typename T>
__device__ __forceinline__ int fold_point(const T* __restrict__ em_x, const T* __restrict__ em,
                                          int i, int nnei, bool is_sorted) {
  if (!is_sorted) return nnei;
  const int lane = threadIdx.x & 31;
  const T last = em_x[(size_t)i * nnei + nnei - 1];
  for (int b = 0; b < nnei; b += 32) {
    const int j = b + lane;
    bool hit = false;
    if (j < nnei) {
      const T* e = em + ((size_t)i * nnei + j) * 4;
      hit = em_x[(size_t)i * nnei + j] == last && e[1] == T(0) && e[2] == T(0) && e[3] == T(0);
    }
    const unsigned m = __ballot_sync(kFull, hit);
    if (m) return b + __ffs(m) - 1;
  }
  return nnei;
}

template <typename T>
__device__ __forceinline__ void load_coef(T* a, const T* __restrict__ row, int k);
template <>
__device__ __forceinline__ void load_coef<float>(float* a, const float* __restrict__ row, int k) {
  const float2* p = reinterpret_cast<const float2*>(row + 6 * k);
  float2 u = __ldg(p), v = __ldg(p + 1), w = __ldg(p + 2);
  a[0] = u.x;
  a[1] = u.y;
  a[2] = v.x;
  a[3] = v.y;
  a[4] = w.x;
  a[5] = w.y;
}
template <>
__device__ __forceinline__ void load_coef<double>(double* a, const double* __restrict__ row,
                                                  int k) {
  const double2* p = reinterpret_cast<const double2*>(row + 6 * k);
  double2 u = __ldg(p), v = __ldg(p + 1), w = __ldg(p + 2);
  a[0] = u.x;
  a[1] = u.y;
  a[2] = v.x;
  a[3] = v.y;
  a[4] = w.x;
  a[5] = w.y;
}

// ------------------------------------------------------------- forward --
template <typename T, int NQ>
__global__ void __launch_bounds__(kTabWarps * 32)
    k_tab_fwd(T* __restrict__ out, const T* __restrict__ table, TableInfo<T> ti,
              const T* __restrict__ em_x, const T* __restrict__ em, int nloc, int nnei, int M,
              int k_base, bool is_sorted) {
  const int i = blockIdx.x * kTabWarps + (threadIdx.x >> 5);
  if (i >= nloc) return;
  const int lane = threadIdx.x & 31;
  const int bp = fold_point(em_x, em, i, nnei, is_sorted);
  T acc[NQ][4];
#pragma unroll
  for (int q = 0; q < NQ; ++q)
#pragma unroll
    for (int m = 0; m < 4; ++m) acc[q][m] = T(0);
  const int jend = bp < nnei ? bp + 1 : nnei;
  for (int j = 0; j < jend; ++j) {
    T x = em_x[(size_t)i * nnei + j];
    const T* e = em + ((size_t)i * nnei + j) * 4;
    const T w = (j == bp) ? T(nnei - j) : T(1);
    const T l0 = e[0], l1 = e[1], l2 = e[2], l3 = e[3];
    const int idx = locate_row(ti, x);
    const T* row = table + (size_t)idx * M * 6;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const int k = k_base + q * 32 + lane;
      if (k < M) {
        T a[6];
        load_coef<T>(a, row, k);
        const T v = poly5(a, x);
        const T wv = w * v;
        acc[q][0] += wv * l0;
        acc[q][1] += wv * l1;
        acc[q][2] += wv * l2;
        acc[q][3] += wv * l3;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    const int k = k_base + q * 32 + lane;
    if (k < M)
#pragma unroll
      for (int m = 0; m < 4; ++m) out[((size_t)i * 4 + m) * M + k] = acc[q][m];
  }
}

// ----------------------------------------------------------- grad-grad --
template <typename T, int NQ>
__global__ void __launch_bounds__(kTabWarps * 32)
    k_tab_grad_grad(T* __restrict__ dz_dy, const T* __restrict__ table, TableInfo<T> ti,
                    const T* __restrict__ em_x, const T* __restrict__ em,
                    const T* __restrict__ dz_dem_x, const T* __restrict__ dz_dem, int nloc,
                    int nnei, int M, int k_base, bool is_sorted) {
  const int i = blockIdx.x * kTabWarps + (threadIdx.x >> 5);
  if (i >= nloc) return;
  const int lane = threadIdx.x & 31;
  const int bp = fold_point(em_x, em, i, nnei, is_sorted);
  T acc[NQ][4];
#pragma unroll
  for (int q = 0; q < NQ; ++q)
#pragma unroll
    for (int m = 0; m < 4; ++m) acc[q][m] = T(0);
  const int jend = bp < nnei ? bp + 1 : nnei;
  for (int j = 0; j < jend; ++j) {
    const size_t ij = (size_t)i * nnei + j;
    T x = em_x[ij];
    const T* e = em + ij * 4;
    const T* h = dz_dem + ij * 4;
    const T dzx = dz_dem_x[ij];
    const T w = (j == bp) ? T(nnei - j) : T(1);
    const T l0 = e[0], l1 = e[1], l2 = e[2], l3 = e[3];
    const T h0 = h[0], h1 = h[1], h2 = h[2], h3 = h[3];
    const int idx = locate_row(ti, x);
    const T* row = table + (size_t)idx * M * 6;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const int k = k_base + q * 32 + lane;
      if (k < M) {
        T a[6];
        load_coef<T>(a, row, k);
        const T v = poly5(a, x);
        const T dv = dpoly5(a, x) * dzx;
        acc[q][0] += w * (v * h0 + dv * l0);
        acc[q][1] += w * (v * h1 + dv * l1);
        acc[q][2] += w * (v * h2 + dv * l2);
        acc[q][3] += w * (v * h3 + dv * l3);
      }
    }
  }
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    const int k = k_base + q * 32 + lane;
    if (k < M)
#pragma unroll
      for (int m = 0; m < 4; ++m) dz_dy[((size_t)i * 4 + m) * M + k] = acc[q][m];
  }
}

// ---------------------------------------------------------------- grad --
// Lanes over k, as the forward: every table row is read with coalesced loads.
// Neighbours are taken kGradGroup at a time; the 5 per-neighbour sums
// (4 of dy_dem and dy_dem_x) of the group are reduced across lanes with one
// 31-shuffle reduce-scatter (lane l receives the total of value l).
constexpr int kGradGroup = 6;

template <typename T>
__device__ __forceinline__ T reduce_scatter32(T (&v)[32], int lane) {
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int k = 0; k < o; ++k) {
      const T send = up ? v[k] : v[k + o];
      const T keep = up ? v[k + o] : v[k];
      v[k] = keep + __shfl_xor_sync(kFull, send, o);
    }
  }
  return v[0];
}

template <typename T, int NQ>
__global__ void __launch_bounds__(kTabWarps * 32)
    k_tab_grad(T* __restrict__ dy_dem_x, T* __restrict__ dy_dem, const T* __restrict__ table,
               TableInfo<T> ti, const T* __restrict__ em_x, const T* __restrict__ em,
               const T* __restrict__ dy, int nloc, int nnei, int M, int k_base, bool accumulate,
               bool is_sorted) {
  __shared__ T gbuf[kTabWarps][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * kTabWarps + warp;
  if (i >= nloc) return;
  T g[NQ][4];
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    const int k = k_base + q * 32 + lane;
#pragma unroll
    for (int m = 0; m < 4; ++m) g[q][m] = k < M ? dy[((size_t)i * 4 + m) * M + k] : T(0);
  }
  const int bp = fold_point(em_x, em, i, nnei, is_sorted);
  const int jend = bp < nnei ? bp + 1 : nnei;
  // slots after the fold point get no gradient (tabulate.cc:166-170, :251-256)
  if (!accumulate)
    for (int j = jend + lane; j < nnei; j += 32) {
      const size_t ij = (size_t)i * nnei + j;
      dy_dem_x[ij] = T(0);
      dy_dem[ij * 4 + 0] = dy_dem[ij * 4 + 1] = dy_dem[ij * 4 + 2] = dy_dem[ij * 4 + 3] = T(0);
    }
  for (int j0 = 0; j0 < jend; j0 += kGradGroup) {
    T part[32];
#pragma unroll
    for (int c = 0; c < 32; ++c) part[c] = T(0);
#pragma unroll
    for (int gg = 0; gg < kGradGroup; ++gg) {
      const int j = j0 + gg;
      if (j < jend) {
        const size_t ij = (size_t)i * nnei + j;
        T x = em_x[ij];
        const T* e = em + ij * 4;
        const T l0 = e[0], l1 = e[1], l2 = e[2], l3 = e[3];
        const int idx = locate_row(ti, x);
        const T* row = table + (size_t)idx * M * 6;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          const int k = k_base + q * 32 + lane;
          if (k < M) {
            T a[6];
            load_coef<T>(a, row, k);
            const T v = poly5(a, x);
            const T dv = dpoly5(a, x);
            part[gg * 5 + 0] += v * g[q][0];
            part[gg * 5 + 1] += v * g[q][1];
            part[gg * 5 + 2] += v * g[q][2];
            part[gg * 5 + 3] += v * g[q][3];
            part[gg * 5 + 4] += dv * (l0 * g[q][0] + l1 * g[q][1] + l2 * g[q][2] + l3 * g[q][3]);
          }
        }
      }
    }
    gbuf[warp][lane] = reduce_scatter32(part, lane);
    __syncwarp();
    if (lane < kGradGroup && j0 + lane < jend) {
      const int j = j0 + lane;
      const size_t ij = (size_t)i * nnei + j;
      const T w = (j == bp) ? T(nnei - j) : T(1);
      const T* gv = gbuf[warp] + lane * 5;
      if (accumulate) {
        dy_dem[ij * 4 + 0] += gv[0] * w;
        dy_dem[ij * 4 + 1] += gv[1] * w;
        dy_dem[ij * 4 + 2] += gv[2] * w;
        dy_dem[ij * 4 + 3] += gv[3] * w;
        dy_dem_x[ij] += gv[4] * w;
      } else {
        dy_dem[ij * 4 + 0] = gv[0] * w;
        dy_dem[ij * 4 + 1] = gv[1] * w;
        dy_dem[ij * 4 + 2] = gv[2] * w;
        dy_dem[ij * 4 + 3] = gv[3] * w;
        dy_dem_x[ij] = gv[4] * w;
      }
    }
    __syncwarp();
  }
}

template <typename T>
int check_common(const T* table, const T* table_info, const T* em_x, const T* em, int nloc,
                 int nnei, int M) {
  GBDP_REQUIRE(nloc >= 0 && nnei >= 0, "tabulate_fusion_se_a: negative nloc/nnei");
  GBDP_REQUIRE(M > 0 && M <= 1024, "tabulate_fusion_se_a: last_layer_size %d not in [1,1024]",
               M);
  GBDP_REQUIRE(table_info != nullptr, "tabulate_fusion_se_a: table_info (host) is null");
  GBDP_REQUIRE(nloc == 0 || nnei == 0 || (table && em_x && em),
               "tabulate_fusion_se_a: null device pointer");
  GBDP_REQUIRE(((uintptr_t)table & 15) == 0,
               "tabulate_fusion_se_a: table must be 16-byte aligned");
  GBDP_REQUIRE(table_info[3] > 0 && table_info[4] > 0,
               "tabulate_fusion_se_a: table strides must be positive");
  return GBDP_OK;
}

template <typename T, template <typename, int> class K>
struct NqDispatch;

template <typename T>
int tab_fwd(T* out, const T* table, const T* info, const T* em_x, const T* em, int nloc,
            int nnei, int M, int is_sorted, cudaStream_t st) {
  int rc = check_common(table, info, em_x, em, nloc, nnei, M);
  if (rc) return rc;
  if (nloc == 0) return GBDP_OK;
  if (nnei == 0) {
    cudaMemsetAsync(out, 0, sizeof(T) * (size_t)nloc * 4 * M, st);
    GBDP_CHECK_LAUNCH("tabulate_fusion_se_a");
    return GBDP_OK;
  }
  const TableInfo<T> ti = make_table_info(info);
  const dim3 grid((nloc + kTabWarps - 1) / kTabWarps), block(kTabWarps * 32);
  for (int kb = 0; kb < M; kb += 128) {
    const int left = (M - kb + 31) / 32;
    if (left >= 4)
      k_tab_fwd<T, 4><<<grid, block, 0, st>>>(out, table, ti, em_x, em, nloc, nnei, M, kb,
                                               is_sorted != 0);
    else if (left == 3)
      k_tab_fwd<T, 3><<<grid, block, 0, st>>>(out, table, ti, em_x, em, nloc, nnei, M, kb,
                                               is_sorted != 0);
    else if (left == 2)
      k_tab_fwd<T, 2><<<grid, block, 0, st>>>(out, table, ti, em_x, em, nloc, nnei, M, kb,
                                               is_sorted != 0);
    else
      k_tab_fwd<T, 1><<<grid, block, 0, st>>>(out, table, ti, em_x, em, nloc, nnei, M, kb,
                                               is_sorted != 0);
  }
  GBDP_CHECK_LAUNCH("tabulate_fusion_se_a");
  return GBDP_OK;
}

template <typename T>
int tab_grad_grad(T* dz_dy, const T* table, const T* info, const T* em_x, const T* em,
                  const T* dzx, const T* dzm, int nloc, int nnei, int M, int is_sorted,
                  cudaStream_t st) {
  int rc = check_common(table, info, em_x, em, nloc, nnei, M);
  if (rc) return rc;
  if (nloc == 0) return GBDP_OK;
  if (nnei == 0) {
    cudaMemsetAsync(dz_dy, 0, sizeof(T) * (size_t)nloc * 4 * M, st);
    GBDP_CHECK_LAUNCH("tabulate_fusion_se_a_grad_grad");
    return GBDP_OK;
  }
  GBDP_REQUIRE(dzx && dzm, "tabulate_fusion_se_a_grad_grad: null dz pointers");
  const TableInfo<T> ti = make_table_info(info);
  const dim3 grid((nloc + kTabWarps - 1) / kTabWarps), block(kTabWarps * 32);
  for (int kb = 0; kb < M; kb += 128) {
    const int left = (M - kb + 31) / 32;
    if (left >= 4)
      k_tab_grad_grad<T, 4><<<grid, block, 0, st>>>(dz_dy, table, ti, em_x, em, dzx, dzm, nloc,
                                                     nnei, M, kb, is_sorted != 0);
    else if (left == 3)
      k_tab_grad_grad<T, 3><<<grid, block, 0, st>>>(dz_dy, table, ti, em_x, em, dzx, dzm, nloc,
                                                     nnei, M, kb, is_sorted != 0);
    else if (left == 2)
      k_tab_grad_grad<T, 2><<<grid, block, 0, st>>>(dz_dy, table, ti, em_x, em, dzx, dzm, nloc,
                                                     nnei, M, kb, is_sorted != 0);
    else
      k_tab_grad_grad<T, 1><<<grid, block, 0, st>>>(dz_dy, table, ti, em_x, em, dzx, dzm, nloc,
                                                     nnei, M, kb, is_sorted != 0);
  }
  GBDP_CHECK_LAUNCH("tabulate_fusion_se_a_grad_grad");
  return GBDP_OK;
}

template <typename T>
int tab_grad(T* dy_dem_x, T* dy_dem, const T* table, const T* info, const T* em_x, const T* em,
             const T* dy, int nloc, int nnei, int M, int is_sorted, cudaStream_t st) {
  int rc = check_common(table, info, em_x, em, nloc, nnei, M);
  if (rc) return rc;
  if (nloc == 0 || nnei == 0) return GBDP_OK;
  GBDP_REQUIRE(dy && dy_dem_x && dy_dem, "tabulate_fusion_se_a_grad: null pointer");
  const TableInfo<T> ti = make_table_info(info);
  const dim3 grid((nloc + kTabWarps - 1) / kTabWarps), block(kTabWarps * 32);
  // k in chunks of 128 (4 lanes-wide passes); later chunks accumulate
  for (int kb = 0; kb < M; kb += 128) {
    const int left = (M - kb + 31) / 32;
    const bool acc = kb > 0;
    if (left >= 4)
      k_tab_grad<T, 4><<<grid, block, 0, st>>>(dy_dem_x, dy_dem, table, ti, em_x, em, dy, nloc,
                                                nnei, M, kb, acc, is_sorted != 0);
    else if (left == 3)
      k_tab_grad<T, 3><<<grid, block, 0, st>>>(dy_dem_x, dy_dem, table, ti, em_x, em, dy, nloc,
                                                nnei, M, kb, acc, is_sorted != 0);
    else if (left == 2)
      k_tab_grad<T, 2><<<grid, block, 0, st>>>(dy_dem_x, dy_dem, table, ti, em_x, em, dy, nloc,
                                                nnei, M, kb, acc, is_sorted != 0);
    else
      k_tab_grad<T, 1><<<grid, block, 0, st>>>(dy_dem_x, dy_dem, table, ti, em_x, em, dy, nloc,
                                                nnei, M, kb, acc, is_sorted != 0);
  }
  GBDP_CHECK_LAUNCH("tabulate_fusion_se_a_grad");
  return GBDP_OK;
}

}  // namespace
}  // namespace gbdp

using namespace gbdp;

#define GBDP_TAB_ENTRY(T, SFX)                                                                  \
  extern "C" int gbdp_tabulate_fusion_se_a_##SFX(T* out, const T* table, const T* table_info,   \
                                                 const T* em_x, const T* em, int nloc,         \
                                                 int nnei, int last_layer_size, int is_sorted, \
                                                 gbdp_stream stream) {                         \
    return tab_fwd<T>(out, table, table_info, em_x, em, nloc, nnei, last_layer_size,           \
                      is_sorted, (cudaStream_t)stream);                                        \
  }                                                                                             \
  extern "C" int gbdp_tabulate_fusion_se_a_grad_##SFX(                                          \
      T* dy_dem_x, T* dy_dem, const T* table, const T* table_info, const T* em_x, const T* em, \
      const T* dy, int nloc, int nnei, int last_layer_size, int is_sorted,                     \
      gbdp_stream stream) {                                                                     \
    return tab_grad<T>(dy_dem_x, dy_dem, table, table_info, em_x, em, dy, nloc, nnei,          \
                       last_layer_size, is_sorted, (cudaStream_t)stream);                      \
  }                                                                                             \
  extern "C" int gbdp_tabulate_fusion_se_a_grad_grad_##SFX(                                     \
      T* dz_dy, const T* table, const T* table_info, const T* em_x, const T* em,               \
      const T* dz_dy_dem_x, const T* dz_dy_dem, int nloc, int nnei, int last_layer_size,       \
      int is_sorted, gbdp_stream stream) {                                                      \
    return tab_grad_grad<T>(dz_dy, table, table_info, em_x, em, dz_dy_dem_x, dz_dy_dem, nloc,  \
                            nnei, last_layer_size, is_sorted, (cudaStream_t)stream);           \
  }

GBDP_TAB_ENTRY(float, f32)
GBDP_TAB_ENTRY(double, f64)
