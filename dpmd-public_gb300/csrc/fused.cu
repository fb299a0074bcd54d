// Fused compressed se_e2_a descriptor (sm_103a): the "chosen form" step.
//
// Tables.  The fused kernels read the compression tables in a k-planar copy
// (gbdp_table_to_planar_*): row r holds three planes, plane p the pairs
// (a_2p, a_2p+1) of every output k, each plane padded to 128 bytes.  A warp
// whose lanes walk k then loads one plane with 256 contiguous bytes (2 L1
// wavefronts) instead of the 768-byte span (6 wavefronts) of the reference's
// coefficient-minor row [M][6] (tabulate.cc:99-131 addressing).
//
// k_desc_fwd (one warp per centre atom):
//   prepass   lanes over the neighbour slots of each type section: the fold
//             point of the padding (tabulate.cc:108-115), the table row and
//             in-row offset of every slot that is evaluated, its env row
//             (times the fold weight) -> shared memory;
//   main      lanes over the M embedding outputs k (32-wide chunks): the
//             tabulated embedding G_k(x_j) times the env row, summed over j
//             (tabulate_fusion_se_a); a last chunk of at most 16 outputs runs
//             with several neighbours per warp instruction instead;
//   epilogue  X = sum / nnei and D[k, a] = sum_m X[m, k] X[m, a], a < A
//             (DescrptBlockSeA.forward, deepmd/pt/model/descriptor/
//             se_a.py:786-866), D stored with 16-byte coalesced writes.
//   Neither the nloc x nnei x M embedding nor per-section outputs reach HBM.
//
// k_desc_bwd (one warp per centre atom):
//   dX        dX = dD X[:, :A] + (dD^T X) padded to M columns, dy = dX / nnei,
//             kept in shared memory as dy4[k] = (dy_0k, dy_1k, dy_2k, dy_3k);
//   prepass   table row / offset / env row of every filled slot;
//   phase 1   16 lanes per neighbour, 2 neighbours per warp instruction;
//             lane t owns outputs k = t + 16 i and keeps their dy in
//             registers: value and slope of the row polynomial and the five
//             sums dE/d em[j, 0..3] (+ the x slope term) of the tabulation
//             gradient (tabulate.cc:158-260), reduced over the 16 lanes by 4
//             butterfly steps;
//   phase 2   lanes over filled slots: the env-matrix derivative row is
//             recomputed from the coordinates (env_mat.cc:122-226) instead of
//             being stored, and force / virial contributions
//             (prod_force.cc:22-72, prod_virial.cc:22-68) are scattered; the
//             virial of the atom is summed in FP32 over its neighbours (as
//             the reference's FPTYPE accumulation) and added to the frame's
//             FP64 accumulator (9 atomics per atom).
//   Padding slots carry no coordinate dependence and are skipped.
#include <array>
#include <atomic>
#include <map>
#include <mutex>

#include "common.cuh"

namespace gbdp {
namespace {

constexpr int kMaxTab = 16;
constexpr int kMaxTypes = 4;
constexpr int kFWarps = 4;
constexpr int kBWarps = 4;
constexpr int kAxis = 16;

template <typename T>
struct TabSet {
  const T* table[kMaxTab];
  TableInfo<T> info[kMaxTab];
  int ntypes;
  int one_side;  // 1: table per neighbour type; 0: per (neighbour, centre)
  int ps;        // plane pitch of the k-planar tables (elements)
  int sec[kMaxTab + 1];
};

template <typename T>
__device__ __forceinline__ int tab_index(const TabSet<T>& ts, int tj, int ti) {
  return ts.one_side ? tj : tj * ts.ntypes + ti;
}

// plane pitch of the k-planar layout: 2 M elements rounded up to 128 bytes
template <typename T>
__host__ __device__ constexpr int kp_pitch(int M) {
  return sizeof(T) == 4 ? (2 * M + 31) & ~31 : (2 * M + 15) & ~15;
}

template <typename T>
struct Vec;
template <>
struct Vec<float> {
  using v2 = float2;
  using v4 = float4;
};
struct alignas(32) dbl4 {
  double x, y, z, w;
};
template <>
struct Vec<double> {
  using v2 = double2;
  using v4 = dbl4;
};
template <typename T>
using V4 = typename Vec<T>::v4;

// L1 policy.  The table rows are the only data the kernels re-read across
// atoms; everything per atom (env rows, X, dE/dD) streams through once or
// twice.  Table loads carry L1::evict_last, per-atom rows L1::no_allocate
// (read once) or L1::evict_first (read twice), so that the hot band of
// table rows stays resident in L1.
__device__ __forceinline__ float2 ld_tab2(const float2* p) {
  float2 v;
  asm("ld.global.nc.L1::evict_last.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
  return v;
}
__device__ __forceinline__ double2 ld_tab2(const double2* p) {
  double2 v;
  asm("ld.global.nc.L1::evict_last.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p));
  return v;
}

// the six coefficients of output k from a k-planar row
template <typename T>
__device__ __forceinline__ void load_coef6_kp(T* a, const T* __restrict__ row, int ps, int k) {
  using P = typename Vec<T>::v2;
  const P u = ld_tab2(reinterpret_cast<const P*>(row) + k);
  const P v = ld_tab2(reinterpret_cast<const P*>(row + ps) + k);
  const P w = ld_tab2(reinterpret_cast<const P*>(row + 2 * ps) + k);
  a[0] = u.x;
  a[1] = u.y;
  a[2] = v.x;
  a[3] = v.y;
  a[4] = w.x;
  a[5] = w.y;
}

// Phase-1 sums of the FP32 backward for one neighbour per 16-lane group:
// the lane's outputs k and k + 16 share the Horner sweeps (value and slope
// of the quintic) as the two halves of packed FP32x2 FMAs (sm_100 and
// later), each half rounding as a scalar fmaf does; the sums then take
// output k and k + 16 in the scalar loop's order, so the results equal the
// scalar loop's bit for bit.  The row load for k + 16 is unconditional
// while q + 1 < NK: a plane holds kp_pitch(M) / 2 = 16 ceil(M / 16) >=
// 16 NK coefficient pairs, so k + 16 < 16 NK stays inside it (pairs past M
// are padding whose sums are not taken), and the loads issue without a
// branch.  p[0..3] += v_k dy[k][0..3], p[4] += v'_k (em . dy[k]).
template <int NK>
__device__ __forceinline__ void bwd_tab_grad_pairs(float* p, const float* __restrict__ row, int ps,
                                                   float x, const float4& e,
                                                   const float (&dr)[NK][4], int t16, int M) {
  const float2 X2 = make_float2(x, x);
#pragma unroll
  for (int q = 0; q < NK; q += 2) {
    const int k = t16 + 16 * q;
    if (k >= M) break;
    float a1[6], a2[6];
    load_coef6_kp<float>(a1, row, ps, k);
    if (q + 1 < NK) {
      load_coef6_kp<float>(a2, row, ps, k + 16);
    } else {
#pragma unroll
      for (int c = 0; c < 6; ++c) a2[c] = 0.f;
    }
    float2 A[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) A[c] = make_float2(a1[c], a2[c]);
    float2 V = A[5], DV = A[5];
    V = __ffma2_rn(V, X2, A[4]);
    DV = __ffma2_rn(DV, X2, V);
    V = __ffma2_rn(V, X2, A[3]);
    DV = __ffma2_rn(DV, X2, V);
    V = __ffma2_rn(V, X2, A[2]);
    DV = __ffma2_rn(DV, X2, V);
    V = __ffma2_rn(V, X2, A[1]);
    DV = __ffma2_rn(DV, X2, V);
    V = __ffma2_rn(V, X2, A[0]);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int qh = q + h;
      if (h == 1 && (qh >= NK || k + 16 >= M)) break;
      const float* d = dr[qh < NK ? qh : q];
      const float v = h ? V.y : V.x, dv = h ? DV.y : DV.x;
      p[0] += v * d[0];
      p[1] += v * d[1];
      p[2] += v * d[2];
      p[3] += v * d[3];
      p[4] += dv * (e.x * d[0] + e.y * d[1] + e.z * d[2] + e.w * d[3]);
    }
  }
}

// a non-binding prefetch of the 128-byte line holding p into L2
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// one row of 4 values (16-byte aligned), not allocated in L1
__device__ __forceinline__ float4 ld_stream4(const float* p) {
  float4 v;
  asm("ld.global.nc.L1::no_allocate.v4.f32 {%0, %1, %2, %3}, [%4];"
      : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
      : "l"(p));
  return v;
}
__device__ __forceinline__ dbl4 ld_stream4(const double* p) {
  dbl4 v;
  asm("ld.global.nc.L1::no_allocate.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p));
  asm("ld.global.nc.L1::no_allocate.v2.f64 {%0, %1}, [%2];" : "=d"(v.z), "=d"(v.w) : "l"(p + 2));
  return v;
}
__device__ __forceinline__ float ld_stream(const float* p) {
  float v;
  asm("ld.global.nc.L1::no_allocate.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ double ld_stream(const double* p) {
  double v;
  asm("ld.global.nc.L1::no_allocate.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}

// a row of 4 values read twice by the same warp: first out of L1
__device__ __forceinline__ float4 ld_first4(const float* p) {
  float4 v;
  asm("ld.global.nc.L1::evict_first.v4.f32 {%0, %1, %2, %3}, [%4];"
      : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
      : "l"(p));
  return v;
}
__device__ __forceinline__ dbl4 ld_first4(const double* p) {
  dbl4 v;
  asm("ld.global.nc.L1::evict_first.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p));
  asm("ld.global.nc.L1::evict_first.v2.f64 {%0, %1}, [%2];" : "=d"(v.z), "=d"(v.w) : "l"(p + 2));
  return v;
}
__device__ __forceinline__ float ld_first(const float* p) {
  float v;
  asm("ld.global.nc.L1::evict_first.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ double ld_first(const double* p) {
  double v;
  asm("ld.global.nc.L1::evict_first.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}

// one row of 4 values through the default path (16-byte aligned)
__device__ __forceinline__ float4 ld_row4(const float* p) {
  return __ldg(reinterpret_cast<const float4*>(p));
}
__device__ __forceinline__ dbl4 ld_row4(const double* p) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(p));
  const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
  return dbl4{a.x, a.y, b.x, b.y};
}

__device__ __forceinline__ void st_row4(float* p, const float4& v) {
  *reinterpret_cast<float4*>(p) = v;
}
__device__ __forceinline__ void st_row4(double* p, const dbl4& v) {
  reinterpret_cast<double2*>(p)[0] = double2{v.x, v.y};
  reinterpret_cast<double2*>(p)[1] = double2{v.z, v.w};
}

// Per-warp shared slot arrays: env row (or, after phase 1, dE/d em), in-row
// offset and table row of every evaluated slot, and the count of evaluated
// slots of each type section.
template <typename T>
struct Slots {
  V4<T>* em;
  T* xr;
  int* idx;
  int* cnt;
};

template <typename T>
__host__ __device__ constexpr size_t slots_bytes(int nnei) {
  return (((size_t)nnei * (sizeof(V4<T>) + sizeof(T) + sizeof(int)) + kMaxTypes * sizeof(int)) +
          31) &
         ~(size_t)31;
}

template <typename T>
__device__ __forceinline__ Slots<T> carve_slots(unsigned char* base, int nnei) {
  Slots<T> s;
  s.em = reinterpret_cast<V4<T>*>(base);
  s.xr = reinterpret_cast<T*>(base + (size_t)nnei * sizeof(V4<T>));
  s.idx = reinterpret_cast<int*>(base + (size_t)nnei * (sizeof(V4<T>) + sizeof(T)));
  s.cnt = s.idx + nnei;
  return s;
}

__host__ __device__ constexpr size_t max_sz(size_t a, size_t b) { return a > b ? a : b; }

template <typename T>
__host__ __device__ constexpr size_t fwd_warp_bytes(int nnei, int mp) {
  return max_sz(slots_bytes<T>(nnei), (size_t)4 * mp * sizeof(T));
}

// ---------------------------------------------------------------- forward --
// NQF: 32-wide output chunks handled lanes-over-k (the last may be partial);
// tail_w (runtime, 0..16): outputs after them, handled tw = pow2 >= tail_w
// lanes per neighbour, 32 / tw neighbours per instruction.
template <typename T, int NQF, int W>
__global__ void __launch_bounds__(W * 32)
    k_desc_fwd(T* __restrict__ X, T* __restrict__ D, void* __restrict__ D_lo,
               float* __restrict__ D_rs, const T* __restrict__ em, const int* __restrict__ atype,
               const int* __restrict__ drow, TabSet<T> ts, int nloc, int nnei, int M, int tail_w,
               int tail_lg) {
  extern __shared__ __align__(32) unsigned char smem_raw[];
  constexpr int NA = NQF + 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * W + warp;
  if (i >= nloc) return;
  const int MP = (NQF + (tail_w > 0 ? 1 : 0)) * 32;
  unsigned char* wbase = smem_raw + (size_t)warp * fwd_warp_bytes<T>(nnei, MP);
  const Slots<T> sl = carve_slots<T>(wbase, nnei);
  const int ti = atype[i];
  const int rs = 3 * ts.ps;
  T acc[NA][4];
#pragma unroll
  for (int q = 0; q < NA; ++q)
#pragma unroll
    for (int m = 0; m < 4; ++m) acc[q][m] = T(0);
  if (ti >= 0) {
    // ---- prepass: fold point, rows and weighted env rows per section
    for (int t = 0; t < ts.ntypes; ++t) {
      const int s0 = ts.sec[t], ns = ts.sec[t + 1] - s0;
      int jend = 0;
      if (ns > 0) {
        const TableInfo<T> inf = ts.info[tab_index(ts, t, ti)];
        const T* e0 = em + ((size_t)i * nnei + s0) * 4;
        const T last = e0[(ns - 1) * 4];
        // every slot up to the first chunk holding the fold point is staged;
        // the fold slot then takes the weight of the slots it stands for
        int bp = ns;
        for (int b = 0; b < ns; b += 32) {
          const int j = b + lane;
          bool hit = false;
          V4<T> e;
          if (j < ns) {
            e = ld_stream4(e0 + 4 * j);
            hit = e.x == last && e.y == T(0) && e.z == T(0) && e.w == T(0);
            T x = e.x;
            const int idx = locate_row(inf, x);
            sl.em[s0 + j] = e;
            sl.xr[s0 + j] = x;
            sl.idx[s0 + j] = idx;
          }
          const unsigned mk = __ballot_sync(kFull, hit);
          if (mk) {
            bp = b + __ffs(mk) - 1;
            if (j == bp) {
              const T w = T(ns - bp);
              e.x *= w;
              e.y *= w;
              e.z *= w;
              e.w *= w;
              sl.em[s0 + j] = e;
            }
            break;
          }
        }
        jend = bp < ns ? bp + 1 : ns;
      }
      if (lane == 0) sl.cnt[t] = jend;
    }
    __syncwarp();
    // ---- main: lanes over k
    for (int t = 0; t < ts.ntypes; ++t) {
      const int s0 = ts.sec[t], cnt = sl.cnt[t];
      const T* tab = ts.table[tab_index(ts, t, ti)];
      // the section's slots are in ascending distance, so neighbours that
      // look up the same table row are consecutive (about a third of them
      // on water, most in the outer shell where s(r) flattens): their
      // coefficients stay in registers instead of being read again
      T a[NQF > 0 ? NQF : 1][6];
      int prev = -1;
      for (int j = 0; j < cnt; ++j) {
        const V4<T> e = sl.em[s0 + j];
        const T x = sl.xr[s0 + j];
        const int idx = sl.idx[s0 + j];
        if (idx != prev) {  // uniform over the warp
          prev = idx;
          const T* row = tab + (size_t)idx * rs;
#pragma unroll
          for (int q = 0; q < NQF; ++q) {
            const int k = q * 32 + lane;
            if (k < M) load_coef6_kp<T>(a[q], row, ts.ps, k);
          }
        }
#pragma unroll
        for (int q = 0; q < NQF; ++q) {
          const int k = q * 32 + lane;
          if (k < M) {
            const T v = poly5(a[q], x);
            acc[q][0] += v * e.x;
            acc[q][1] += v * e.y;
            acc[q][2] += v * e.z;
            acc[q][3] += v * e.w;
          }
        }
      }
    }
    // ---- tail: several neighbours per instruction over the last outputs
    if (tail_w > 0) {
      const int tw = 1 << tail_lg;
      const int n = lane >> tail_lg, tt = lane & (tw - 1);
      const int npt = 32 >> tail_lg;
      const int k = NQF * 32 + tt;
      T ta[4] = {T(0), T(0), T(0), T(0)};
      for (int t = 0; t < ts.ntypes; ++t) {
        const int s0 = ts.sec[t], cnt = sl.cnt[t];
        const T* tab = ts.table[tab_index(ts, t, ti)];
        for (int j0 = 0; j0 < cnt; j0 += npt) {
          const int j = j0 + n;
          if (j < cnt && tt < tail_w) {
            const V4<T> e = sl.em[s0 + j];
            const T x = sl.xr[s0 + j];
            const T* row = tab + (size_t)sl.idx[s0 + j] * rs;
            T a[6];
            load_coef6_kp<T>(a, row, ts.ps, k);
            const T v = poly5(a, x);
            ta[0] += v * e.x;
            ta[1] += v * e.y;
            ta[2] += v * e.z;
            ta[3] += v * e.w;
          }
        }
      }
      for (int o = tw; o < 32; o <<= 1)
#pragma unroll
        for (int m = 0; m < 4; ++m) ta[m] += __shfl_xor_sync(kFull, ta[m], o);
#pragma unroll
      for (int m = 0; m < 4; ++m) acc[NQF][m] = lane < tail_w ? ta[m] : T(0);
    }
  }
  // ---- epilogue: X (coalesced over k) and D
  __syncwarp();
  T* xs = reinterpret_cast<T*>(wbase);  // [4][MP], aliases the slot arrays
  const T inv = T(1) / T(nnei);
#pragma unroll
  for (int q = 0; q < NA; ++q) {
    if (q == NQF && tail_w == 0) break;
    const int k = q * 32 + lane;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const T v = acc[q][m] * inv;
      xs[m * MP + k] = v;
      if (k < M) X[((size_t)i * 4 + m) * M + k] = v;
    }
  }
  __syncwarp();
  const size_t r = drow ? (size_t)drow[i] : (size_t)i;
  T* d = D + r * M * kAxis;
  if constexpr (sizeof(T) == 4) {
    if (D_lo) {
      // split for the tensor-core fitting: FP16 hi / lo of c D, c = 2^s from
      // |D_ka| <= |X_k| |X_a| (Cauchy-Schwarz over the 4 rows of X)
      float nk = 0.f, na = 0.f;
      for (int k = lane; k < M; k += 32) {
        float q = 0.f;
#pragma unroll
        for (int m = 0; m < 4; ++m) q += xs[m * MP + k] * xs[m * MP + k];
        nk = fmaxf(nk, q);
        if (k < kAxis) na = fmaxf(na, q);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        nk = fmaxf(nk, __shfl_xor_sync(kFull, nk, o));
        na = fmaxf(na, __shfl_xor_sync(kFull, na, o));
      }
      const float sc = f16_scale_for(sqrtf(nk * na) * 1.0001f);
      __half* dh = reinterpret_cast<__half*>(D) + r * M * kAxis;
      __half* dl = static_cast<__half*>(D_lo) + r * M * kAxis;
      for (int e = lane * 4; e < M * kAxis; e += 128) {
        const int k = e >> 4, a0 = e & 15;
        float v[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          const float xk = xs[m * MP + k];
#pragma unroll
          for (int c = 0; c < 4; ++c) v[c] += xk * xs[m * MP + a0 + c];
        }
        st_split4_f16(dh + e, dl + e, v, sc);
      }
      if (lane == 0) D_rs[r] = 1.f / sc;
      return;
    }
  }
  for (int e = lane * 4; e < M * kAxis; e += 128) {
    const int k = e >> 4, a0 = e & 15;
    T v[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const T xk = xs[m * MP + k];
#pragma unroll
      for (int c = 0; c < 4; ++c) v[c] += xk * xs[m * MP + a0 + c];
    }
    V4<T> o;
    o.x = v[0];
    o.y = v[1];
    o.z = v[2];
    o.w = v[3];
    st_row4(d + e, o);
  }
}

// --------------------------------------------------------------- backward --
template <typename T>
__device__ __forceinline__ void spline5_d(T& vv, T& dd, T xx, T rmin, T rmax) {
  if (xx < rmin) {
    dd = T(0);
    vv = T(1);
  } else if (xx < rmax) {
    T uu = (xx - rmin) / (rmax - rmin);
    T du = T(1) / (rmax - rmin);
    vv = uu * uu * uu * (T(-6) * uu * uu + T(15) * uu - T(10)) + T(1);
    dd = (T(3) * uu * uu * (T(-6) * uu * uu + T(15) * uu - T(10)) +
          uu * uu * uu * (T(-12) * uu + T(15))) *
         du;
  } else {
    dd = T(0);
    vv = T(0);
  }
}

__device__ __forceinline__ float rsqrt_t(float x) { return rsqrtf(x); }
__device__ __forceinline__ double rsqrt_t(double x) { return rsqrt(x); }

struct BwdGeom {
  const int* atom_frame;   // [nloc_total] frame of each centre
  const int* frame_aoff;   // [nframes] first local atom of each frame
  const int* frame_eoff;   // [nframes] first extended slot of each frame
};

// Number of filled slots of a section: the env kernel fills each type
// section from its start, so the filled slots are a prefix.
__device__ __forceinline__ int filled_prefix(const int* __restrict__ nl, int ns) {
  const int lane = threadIdx.x & 31;
  int n = 0;
  for (int b = 0; b < ns; b += 32) {
    const bool ok = b + lane < ns && nl[b + lane] >= 0;
    n += __popc(__ballot_sync(kFull, ok));
  }
  return n;
}

template <typename T>
__host__ __device__ constexpr size_t bwd_warp_bytes(int nnei, int m) {
  // dy4 [M] and X^T [M] while dX is formed, then the slot arrays over them
  // (dy is in registers by then): the smaller the footprint, the more L1 is
  // left for table rows (M = 100, nnei = 138: 3,328 B a warp, so that the
  // 28 resident warps fit the 100 KB shared-memory carveout and leave
  // 156 KB of L1)
  return max_sz(slots_bytes<T>(nnei), (size_t)2 * m * sizeof(V4<T>));
}

// Phase 1 runs 16 lanes per neighbour.
// NK = ceil(M / 16): outputs per lane in phase 1; NQ = ceil(M / 32); U:
// neighbours in flight per 16-lane group, 1 (28 resident warps) or 2 (more
// loads in flight per warp, 24 resident warps), chosen by the autotuner
// together with the warps per CTA (default 1).
template <typename T, int NQ, int NK, int U, int W>
__global__ void __launch_bounds__(W * 32, sizeof(T) == 4 ? (U == 1 ? 28 : 24) / W : 1)
    k_desc_bwd(T* __restrict__ force, double* __restrict__ vir_acc,
               long long* __restrict__ force_fx, const T* __restrict__ X,
               const T* __restrict__ dD, const int* __restrict__ drow, const T* __restrict__ em,
               const int* __restrict__ nlist_ext, const T* __restrict__ ext_coord,
               const int* __restrict__ ext_map, const int* __restrict__ atype,
               const T* __restrict__ inv_std, BwdGeom geo, TabSet<T> ts, T rmin, T rmax, int nloc,
               int nnei, int M, int pf_dist) {
  extern __shared__ __align__(32) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * W + warp;
  if (i >= nloc) return;
  {
    // the atom pf_dist ahead (about one wave of resident warps later):
    // its dE/dD row, X and env rows prefetched into L2, so that the warp
    // that takes it finds its first loads in L2 rather than in DRAM
    const int ip = i + pf_dist;
    if (pf_dist > 0 && ip < nloc) {
      const size_t rp = drow ? (size_t)drow[ip] : (size_t)ip;
      const char* pd = reinterpret_cast<const char*>(dD + rp * M * kAxis);
      const char* px = reinterpret_cast<const char*>(X + (size_t)ip * 4 * M);
      const char* pe = reinterpret_cast<const char*>(em + (size_t)ip * nnei * 4);
      const int ld = (int)((sizeof(T) * M * kAxis + 127) / 128),
                lx = (int)((sizeof(T) * 4 * M + 127) / 128),
                le = (int)((sizeof(T) * 4 * nnei + 127) / 128);
      for (int l = lane; l < ld + lx + le; l += 32)
        prefetch_l2(l < ld ? pd + 128 * l : l < ld + lx ? px + 128 * (l - ld) : pe + 128 * (l - ld - lx));
    }
  }
  const int ti = atype[i];
  if (ti < 0) return;
  unsigned char* wbase = smem_raw + (size_t)warp * bwd_warp_bytes<T>(nnei, M);
  V4<T>* dy4 = reinterpret_cast<V4<T>*>(wbase);
  V4<T>* xT = dy4 + M;  // X^T: xT[k] = (X_0k, X_1k, X_2k, X_3k), k < M
  T* xTs = reinterpret_cast<T*>(xT);
  // all of X's loads issued before the first is stored (no dependent chain)
  {
    T xv[4 * NQ];
#pragma unroll
    for (int q = 0; q < 4 * NQ; ++q) {
      const int u = q * 32 + lane;
      xv[q] = u < 4 * M ? ld_stream(X + (size_t)i * 4 * M + u) : T(0);
    }
#pragma unroll
    for (int q = 0; q < 4 * NQ; ++q) {
      const int u = q * 32 + lane;
      if (u < 4 * M) {
        const int m = u / M, k = u - m * M;
        xTs[4 * k + m] = xv[q];
      }
    }
  }
  __syncwarp();
  const size_t drow_i = drow ? (size_t)drow[i] : (size_t)i;
  const T* g_i = dD + drow_i * M * kAxis;
  // ---- dX = dD X[:, :A] (all k) ...
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    const int k = q * 32 + lane;
    if (k < M) {
      T g[kAxis];
#pragma unroll
      for (int a4 = 0; a4 < kAxis; a4 += 4) {
        const V4<T> v = ld_first4(g_i + k * kAxis + a4);
        g[a4] = v.x;
        g[a4 + 1] = v.y;
        g[a4 + 2] = v.z;
        g[a4 + 3] = v.w;
      }
      T dx[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
      for (int a = 0; a < kAxis; ++a) {
        const V4<T> x4 = xT[a];
        dx[0] += g[a] * x4.x;
        dx[1] += g[a] * x4.y;
        dx[2] += g[a] * x4.z;
        dx[3] += g[a] * x4.w;
      }
      V4<T> o;
      o.x = dx[0];
      o.y = dx[1];
      o.z = dx[2];
      o.w = dx[3];
      dy4[k] = o;
    }
  }
  __syncwarp();
  // ---- ... + dD^T X for the first A columns: two half-warps split kk;
  //      the loads of kDtxBatch rows are issued before they are used, so
  //      the pass waits for one memory round trip per batch, not per row
  {
    constexpr int kDtxBatch = 10;
    const int h = lane >> 4, kc = lane & 15;
    T s[4] = {T(0), T(0), T(0), T(0)};
    for (int kk0 = h; kk0 < M; kk0 += 2 * kDtxBatch) {
      T gv[kDtxBatch];
#pragma unroll
      for (int u = 0; u < kDtxBatch; ++u) {
        const int kk = kk0 + 2 * u;
        gv[u] = kk < M ? ld_first(g_i + kk * kAxis + kc) : T(0);
      }
#pragma unroll
      for (int u = 0; u < kDtxBatch; ++u) {
        const int kk = kk0 + 2 * u;
        if (kk < M) {
          const V4<T> x4 = xT[kk];
          s[0] += gv[u] * x4.x;
          s[1] += gv[u] * x4.y;
          s[2] += gv[u] * x4.z;
          s[3] += gv[u] * x4.w;
        }
      }
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) s[m] += __shfl_xor_sync(kFull, s[m], 16);
    if (h == 0) {
      V4<T> o = dy4[kc];
      o.x += s[0];
      o.y += s[1];
      o.z += s[2];
      o.w += s[3];
      dy4[kc] = o;
    }
  }
  __syncwarp();
  const T inv = T(1) / T(nnei);
  for (int k = lane; k < M; k += 32) {
    V4<T> o = dy4[k];
    o.x *= inv;
    o.y *= inv;
    o.z *= inv;
    o.w *= inv;
    dy4[k] = o;
  }
  __syncwarp();
  // phase 1 mapping: 16 lanes per neighbour; lane t16 owns outputs
  // k = t16 + 16 i and keeps their dy in registers from here on
  const int n = lane >> 4, t16 = lane & 15;
  T dr[NK][4];
#pragma unroll
  for (int q = 0; q < NK; ++q) {
    const int k = t16 + 16 * q;
    V4<T> d;
    if (k < M) {
      d = dy4[k];
    } else {
      d.x = d.y = d.z = d.w = T(0);
    }
    dr[q][0] = d.x;
    dr[q][1] = d.y;
    dr[q][2] = d.z;
    dr[q][3] = d.w;
  }
  __syncwarp();

  // ---- prepass over filled slots (the slot arrays replace dy4 and X^T)
  const Slots<T> sl = carve_slots<T>(wbase, nnei);
  const int* nl_i = nlist_ext + (size_t)i * nnei;
  for (int t = 0; t < ts.ntypes; ++t) {
    const int s0 = ts.sec[t], ns = ts.sec[t + 1] - s0;
    const int nv = filled_prefix(nl_i + s0, ns);
    const TableInfo<T> inf = ts.info[tab_index(ts, t, ti)];
    for (int j = lane; j < nv; j += 32) {
      const V4<T> e = ld_stream4(em + ((size_t)i * nnei + s0 + j) * 4);
      T x = e.x;
      const int idx = locate_row(inf, x);
      sl.em[s0 + j] = e;
      sl.xr[s0 + j] = x;
      sl.idx[s0 + j] = idx;
    }
    if (lane == 0) sl.cnt[t] = nv;
  }
  __syncwarp();

  // ---- phase 1: tabulation gradient, 16 lanes per neighbour
  const int rs = 3 * ts.ps;
  {
    // each 16-lane group carries U neighbours (j0 + n + 2 u) at once, so
    // that 3 U independent table loads are in flight per output step
    for (int t = 0; t < ts.ntypes; ++t) {
      const int s0 = ts.sec[t], nv = sl.cnt[t];
      const T* tab = ts.table[tab_index(ts, t, ti)];
      for (int j0 = 0; j0 < nv; j0 += 2 * U) {
        T p[U][5];
        V4<T> e[U];
        T x[U];
        const T* row[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          // a slot past the end re-evaluates slot j0 (always filled); its
          // sums are dropped
          const int j = j0 + n + 2 * u;
          const int js = j < nv ? j : j0;
          e[u] = sl.em[s0 + js];
          x[u] = sl.xr[s0 + js];
          row[u] = tab + (size_t)sl.idx[s0 + js] * rs;
#pragma unroll
          for (int c = 0; c < 5; ++c) p[u][c] = T(0);
        }
        if constexpr (sizeof(T) == 4 && U == 1) {
          bwd_tab_grad_pairs<NK>(p[0], row[0], ts.ps, x[0], e[0], dr, t16, M);
        } else {
#pragma unroll
          for (int q = 0; q < NK; ++q) {
            const int k = t16 + 16 * q;
            if (k >= M) break;
            T a[U][6];
#pragma unroll
            for (int u = 0; u < U; ++u) load_coef6_kp<T>(a[u], row[u], ts.ps, k);
            const T d[4] = {dr[q][0], dr[q][1], dr[q][2], dr[q][3]};
#pragma unroll
            for (int u = 0; u < U; ++u) {
              // value and slope by one Horner sweep (9 FMA)
              const T xu = x[u];
              T v = a[u][5], dv = a[u][5];
              v = v * xu + a[u][4];
              dv = dv * xu + v;
              v = v * xu + a[u][3];
              dv = dv * xu + v;
              v = v * xu + a[u][2];
              dv = dv * xu + v;
              v = v * xu + a[u][1];
              dv = dv * xu + v;
              v = v * xu + a[u][0];
              p[u][0] += v * d[0];
              p[u][1] += v * d[1];
              p[u][2] += v * d[2];
              p[u][3] += v * d[3];
              p[u][4] += dv * (e[u].x * d[0] + e[u].y * d[1] + e[u].z * d[2] + e[u].w * d[3]);
            }
          }
        }
        // dE/d em[j, :] = (p0 + p4, p1, p2, p3) summed over the 16-lane
        // group (em_x is em[:, 0]) by a reduce-scatter: the halves of the
        // group exchange half of the four sums (xor 8), then half of the
        // rest (xor 4), and the last two levels add one value each, so lane
        // t16 ends with component (t16 >> 2) & 3 (5 shuffles instead of the
        // 20 of four full butterflies over five sums)
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const bool h8 = (t16 & 8) != 0, h4 = (t16 & 4) != 0;
          const T q0 = p[u][0] + p[u][4];
          const T r0 = __shfl_xor_sync(kFull, h8 ? q0 : p[u][2], 8);
          const T r1 = __shfl_xor_sync(kFull, h8 ? p[u][1] : p[u][3], 8);
          const T a0 = (h8 ? p[u][2] : q0) + r0;
          const T a1 = (h8 ? p[u][3] : p[u][1]) + r1;
          T b = (h4 ? a1 : a0) + __shfl_xor_sync(kFull, h4 ? a0 : a1, 4);
          b += __shfl_xor_sync(kFull, b, 2);
          b += __shfl_xor_sync(kFull, b, 1);
          const int j = j0 + n + 2 * u;
          if ((t16 & 3) == 0 && j < nv) reinterpret_cast<T*>(&sl.em[s0 + j])[t16 >> 2] = b;
        }
      }
    }
  }
  __syncwarp();

  // ---- phase 2: lanes over filled slots: env-matrix derivative row
  //      d em / d x_i (env_mat.cc:157-204) / std, force and virial scatter
  const int f = geo.atom_frame[i];
  const int il = i - geo.frame_aoff[f];
  const size_t eoff = geo.frame_eoff[f];
  const int aoff = geo.frame_aoff[f];
  const T xi = ext_coord[3 * (eoff + il)], yi = ext_coord[3 * (eoff + il) + 1],
          zi = ext_coord[3 * (eoff + il) + 2];
  const T* isd = inv_std + (size_t)ti * nnei * 4;
  T ci[3] = {T(0), T(0), T(0)};
  T vir[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) vir[q] = T(0);
  for (int t = 0; t < ts.ntypes; ++t) {
    const int s0 = ts.sec[t], nv = sl.cnt[t];
    for (int jj = lane; jj < nv; jj += 32) {
      const int s = s0 + jj;
      const int je = nl_i[s];
      T rr[3];
      rr[0] = ext_coord[3 * (eoff + je)] - xi;
      rr[1] = ext_coord[3 * (eoff + je) + 1] - yi;
      rr[2] = ext_coord[3 * (eoff + je) + 2] - zi;
      const T nr2 = rr[0] * rr[0] + rr[1] * rr[1] + rr[2] * rr[2];
      const T inr = rsqrt_t(nr2);
      const T nr = nr2 * inr;
      const T inr2 = inr * inr;
      const T inr4 = inr2 * inr2;
      const T inr3 = inr4 * nr;
      T sw, dsw;
      spline5_d<T>(sw, dsw, nr, rmin, rmax);
      const T ev[4] = {inr, rr[0] * inr2, rr[1] * inr2, rr[2] * inr2};
      const V4<T> net = sl.em[s];
      const V4<T> sd = ld_row4(isd + (size_t)s * 4);
      const T gw[4] = {net.x * sd.x, net.y * sd.y, net.z * sd.z, net.w * sd.w};
      T v3[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        T acc = gw[0] * (rr[d] * inr3 * sw - ev[0] * dsw * rr[d] * inr);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          T tt = T(2) * rr[c] * rr[d] * inr4;
          if (c == d) tt -= inr2;
          acc += gw[1 + c] * (tt * sw - ev[1 + c] * dsw * rr[d] * inr);
        }
        v3[d] = acc;
      }
      const int jl = ext_map[eoff + je];
      if (force_fx)
        fx_add3(force_fx + (size_t)(aoff + jl) * 3, v3, FxScale<T>::force);
      else
        scatter3(force + (size_t)(aoff + jl) * 3, v3);
      ci[0] += v3[0];
      ci[1] += v3[1];
      ci[2] += v3[2];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) vir[a * 3 + b] += v3[a] * rr[b];
    }
  }
  ci[0] = warp_sum(ci[0]);
  ci[1] = warp_sum(ci[1]);
  ci[2] = warp_sum(ci[2]);
  if (lane == 0) {
    const T m[3] = {-ci[0], -ci[1], -ci[2]};
    if (force_fx)
      fx_add3(force_fx + (size_t)i * 3, m, FxScale<T>::force);
    else
      scatter3(force + (size_t)i * 3, m);
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    const T v = warp_sum(vir[q]);
    if (lane == 0) {
      if (force_fx)  // the accumulator holds fixed-point sums in this mode
        fx_add(reinterpret_cast<long long*>(vir_acc) + f * 9 + q, v, FxScale<T>::virial);
      else
        atomicAdd(vir_acc + f * 9 + q, (double)v);
    }
  }
}

// ------------------------------------------------------- frame energies --
// E[f] = sum of the per-row energies of frame f, in FP64.  Rows of a frame
// come in runs (rows are grouped by type, frames in order within a type),
// so each warp adds one partial per run it sees: a handful of atomics per
// warp instead of one per row.  Rows with frame -1 (padding) are skipped.
// fixed-point totals -> values (out = acc * 2^-s)
template <typename T>
__global__ void k_fx_finish(T* __restrict__ out, const long long* __restrict__ acc, size_t n,
                            int s) {
  const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[k] = (T)((double)acc[k] * pow2d(-s));
}
// the same in place: the double buffer held the int64 totals
__global__ void k_fx_finish_inplace(double* __restrict__ buf, size_t n, int s) {
  for (size_t k = threadIdx.x; k < n; k += blockDim.x) {
    const long long v = reinterpret_cast<const long long*>(buf)[k];
    buf[k] = (double)v * pow2d(-s);
  }
}

template <typename T>
__global__ void k_frame_energy(double* __restrict__ E, const T* __restrict__ ae,
                               const int* __restrict__ frame_of_row, int nrows, int det) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const int f = r < nrows ? frame_of_row[r] : -1;
  const double v = r < nrows ? (double)ae[r] : 0.;
  unsigned todo = __ballot_sync(kFull, f >= 0);
  while (todo) {
    const int leader = __ffs(todo) - 1;
    const int lf = __shfl_sync(kFull, f, leader);
    const bool mine = f == lf;
    const unsigned mk = __ballot_sync(kFull, mine);
    const double sum = warp_sum(mine ? v : 0.);
    if (lane == leader) {
      if (det)  // fixed point: the same bits whatever order the warps add in
        fx_add(reinterpret_cast<long long*>(E) + lf, sum, kFxEnergy);
      else
        atomicAdd(E + lf, sum);
    }
    todo &= ~mk;
  }
}

template <typename T>
int frame_energy(double* E, const T* ae, const int* frame_of_row, int nrows, int nframes,
                 int det, cudaStream_t st) {
  GBDP_REQUIRE(nrows >= 0 && nframes >= 1, "frame_energy: nrows %d, nframes %d", nrows, nframes);
  GBDP_REQUIRE(E != nullptr, "frame_energy: null E");
  cudaMemsetAsync(E, 0, sizeof(double) * (size_t)nframes, st);
  if (nrows == 0) return GBDP_OK;
  GBDP_REQUIRE(ae && frame_of_row, "frame_energy: null input");
  k_frame_energy<T><<<(unsigned)((nrows + 255) / 256), 256, 0, st>>>(E, ae, frame_of_row, nrows,
                                                                     det);
  if (det) k_fx_finish_inplace<<<1, 256, 0, st>>>(E, (size_t)nframes, kFxEnergy);
  GBDP_CHECK_LAUNCH("frame_energy");
  return GBDP_OK;
}

// ------------------------------------------------------ table re-layout --
// dst[r][p][2k + c] = src[r][6k + 2p + c], zero padding to the plane pitch
template <typename T>
__global__ void k_table_planar(T* __restrict__ dst, const T* __restrict__ src, int nrow, int M,
                               int ps) {
  const size_t n = (size_t)nrow * 3 * ps;
  for (size_t u = (size_t)blockIdx.x * blockDim.x + threadIdx.x; u < n;
       u += (size_t)gridDim.x * blockDim.x) {
    const size_t r = u / (3 * (size_t)ps);
    const int rem = (int)(u - r * 3 * ps);
    const int p = rem / ps, e = rem - p * ps;
    const int k = e >> 1, c = e & 1;
    dst[u] = k < M ? src[r * 6 * M + 6 * k + 2 * p + c] : T(0);
  }
}

template <typename T>
int make_tabset(TabSet<T>& ts, const T* const* tables, const T* infos, int ntypes, const int* sel,
                int one_side, int M) {
  GBDP_REQUIRE(ntypes >= 1 && ntypes <= kMaxTypes, "se_a descriptor: ntypes %d not in [1,%d]",
               ntypes, kMaxTypes);
  const int ntab = one_side ? ntypes : ntypes * ntypes;
  GBDP_REQUIRE(ntab <= kMaxTab, "se_a descriptor: too many tables");
  GBDP_REQUIRE(tables && infos && sel, "se_a descriptor: null table / info / sel array");
  ts.ntypes = ntypes;
  ts.one_side = one_side ? 1 : 0;
  ts.ps = kp_pitch<T>(M);
  ts.sec[0] = 0;
  for (int t = 0; t < ntypes; ++t) {
    GBDP_REQUIRE(sel[t] >= 0, "se_a descriptor: sel[%d] = %d", t, sel[t]);
    ts.sec[t + 1] = ts.sec[t] + sel[t];
  }
  for (int k = 0; k < ntab; ++k) {
    GBDP_REQUIRE(tables[k] != nullptr && ((uintptr_t)tables[k] & 127) == 0,
                 "se_a descriptor: table %d null or not 128-byte aligned", k);
    ts.table[k] = tables[k];
    ts.info[k] = make_table_info(infos + 6 * k);
  }
  return GBDP_OK;
}

// ------------------------------------------------------------- autotune --
// Launch shapes of the fused descriptor kernels, as a shape code: bits 0-2
// the warps per CTA (1, 2 or 4 centre atoms per CTA; per-warp shared memory,
// so only the launch shape changes: a small batch fills more SMs with
// smaller CTAs), bits 3-4 for the backward the neighbours in flight per
// 16-lane group minus one (1 or 2: more loads in flight per warp against
// fewer resident warps).  With autotuning on (gbdp_set_autotune), the first
// call for a shape key (kernel, dtype, M, nnei, floor(log2 nloc)) that is
// not under stream capture times every choice with CUDA events on the
// caller's stream (three runs each, the minimum) and keeps the fastest;
// later calls with that key use it.  The cache is the library's only mutable
// global state and sits behind a mutex.  Without a tuned entry the choice is
// 4 warps, 1 neighbour in flight.
enum { kTuneFwd = 0, kTuneBwd = 1 };
constexpr int kTuneMax = 6;
constexpr int kTuneFwdCodes[3] = {1, 2, 4};
constexpr int kTuneBwdCodes[6] = {1, 2, 4, 1 | 8, 2 | 8, 4 | 8};
inline int code_warps(int c) { return c & 7; }
inline int code_nbrs(int c) { return (c >> 3) + 1; }
struct TuneEntry {
  int code;
  int n;
  float ms[kTuneMax];
};
std::mutex g_tune_mu;
std::map<std::array<int, 5>, TuneEntry> g_tune;
std::atomic<int> g_autotune{0};

std::array<int, 5> tune_key(int kid, int tsize, int M, int nnei, int nloc) {
  int lg = 0;
  while (lg < 30 && (1 << (lg + 1)) <= nloc) ++lg;
  return {kid, tsize, M, nnei, lg};
}

int tuned_code(int kid, int tsize, int M, int nnei, int nloc, int dflt) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  const auto it = g_tune.find(tune_key(kid, tsize, M, nnei, nloc));
  return it == g_tune.end() ? dflt : it->second.code;
}

// run(c): one whole call with shape code c (0: the tuned or default
// choice), returning a status.  Tunes first when that is on and possible.
template <typename F>
int tune_run(int kid, int tsize, int M, int nnei, int nloc, cudaStream_t st, F&& run) {
  if (g_autotune.load() && nloc > 0 && nnei > 0) {
    const auto key = tune_key(kid, tsize, M, nnei, nloc);
    bool have;
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      have = g_tune.count(key) != 0;
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (!have && cudaStreamIsCapturing(st, &cs) == cudaSuccess &&
        cs == cudaStreamCaptureStatusNone) {
      const int* codes = kid == kTuneFwd ? kTuneFwdCodes : kTuneBwdCodes;
      // the FP64 backward is built for one neighbour in flight only
      const int nc = kid == kTuneFwd ? 3 : (tsize == 4 ? 6 : 3);
      cudaEvent_t e0, e1;
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      TuneEntry te{4, nc, {}};
      float best = 1e30f;
      int rc = GBDP_OK;
      for (int c = 0; c < nc && rc == GBDP_OK; ++c) {
        rc = run(codes[c]);  // warm-up
        float t = 1e30f;
        for (int rep = 0; rep < 3 && rc == GBDP_OK; ++rep) {
          cudaEventRecord(e0, st);
          rc = run(codes[c]);
          cudaEventRecord(e1, st);
          if (cudaEventSynchronize(e1) != cudaSuccess) rc = cuda_status(cudaGetLastError(), "autotune");
          float ms = 0.f;
          cudaEventElapsedTime(&ms, e0, e1);
          t = std::min(t, ms);
        }
        te.ms[c] = t;
        if (t < best) {
          best = t;
          te.code = codes[c];
        }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      if (rc != GBDP_OK) return rc;
      std::lock_guard<std::mutex> lk(g_tune_mu);
      g_tune[key] = te;
    }
  }
  return run(0);
}

inline int sum_sel(const int* sel, int ntypes) {
  int n = 0;
  if (sel)
    for (int t = 0; t < ntypes && t < kMaxTab; ++t) n += sel[t] > 0 ? sel[t] : 0;
  return n;
}

template <typename T>
int check_shapes(int M, int A, int nnei) {
  GBDP_REQUIRE(M >= kAxis && M <= 128, "se_a descriptor: neuron[-1] %d not in [%d,128]", M,
               kAxis);
  GBDP_REQUIRE(A == kAxis, "se_a descriptor: axis_neuron %d (this build supports %d)", A, kAxis);
  GBDP_REQUIRE(nnei >= 1 && nnei <= 4096, "se_a descriptor: nnei %d not in [1,4096]", nnei);
  return GBDP_OK;
}

template <typename T, int NQF, int W>
void launch_fwd(size_t warp_bytes, cudaStream_t st, T* X, T* D, void* D_lo, float* D_rs,
                const T* em, const int* atype, const int* drow, const TabSet<T>& ts, int nloc,
                int nnei, int M, int tail_w, int tail_lg) {
  auto kern = k_desc_fwd<T, NQF, W>;
  const size_t smem = (size_t)W * warp_bytes;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  // the smallest shared-memory carveout that holds the resident CTAs (36
  // warps at 56 registers in FP32): the rest of the unified L1 caches table
  // rows
  const int per_sm = (36 / W) * (int)(smem + 1024);
  cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                       per_sm >= 228 * 1024 ? 100 : (per_sm * 100 + 228 * 1024 - 1) / (228 * 1024));
  kern<<<(unsigned)((nloc + W - 1) / W), W * 32, smem, st>>>(X, D, D_lo, D_rs, em, atype, drow,
                                                             ts, nloc, nnei, M, tail_w, tail_lg);
}

template <typename T, int W>
void fwd_dispatch(int nqf, size_t warp_bytes, cudaStream_t st, T* X, T* D, void* D_lo,
                  float* D_rs, const T* em, const int* atype, const int* drow,
                  const TabSet<T>& ts, int nloc, int nnei, int M, int tail_w, int tail_lg) {
  switch (nqf) {
    case 0:
      launch_fwd<T, 0, W>(warp_bytes, st, X, D, D_lo, D_rs, em, atype, drow, ts, nloc, nnei, M,
                          tail_w, tail_lg);
      break;
    case 1:
      launch_fwd<T, 1, W>(warp_bytes, st, X, D, D_lo, D_rs, em, atype, drow, ts, nloc, nnei, M,
                          tail_w, tail_lg);
      break;
    case 2:
      launch_fwd<T, 2, W>(warp_bytes, st, X, D, D_lo, D_rs, em, atype, drow, ts, nloc, nnei, M,
                          tail_w, tail_lg);
      break;
    case 3:
      launch_fwd<T, 3, W>(warp_bytes, st, X, D, D_lo, D_rs, em, atype, drow, ts, nloc, nnei, M,
                          tail_w, tail_lg);
      break;
    default:
      launch_fwd<T, 4, W>(warp_bytes, st, X, D, D_lo, D_rs, em, atype, drow, ts, nloc, nnei, M,
                          tail_w, tail_lg);
      break;
  }
}

template <typename T>
int desc_fwd(T* X, T* D, void* D_lo, float* D_rs, const T* em, const int* atype, const int* drow,
             const T* const* tables, const T* infos, int ntypes, const int* sel, int one_side,
             int nloc, int M, int A, cudaStream_t st, int w = 0) {
  TabSet<T> ts;
  int rc = make_tabset(ts, tables, infos, ntypes, sel, one_side, M);
  if (rc) return rc;
  const int nnei = ts.sec[ntypes];
  rc = check_shapes<T>(M, A, nnei);
  if (rc) return rc;
  if (nloc == 0) return GBDP_OK;
  GBDP_REQUIRE(X && D && em && atype, "se_a descriptor fwd: null argument");
  GBDP_REQUIRE(((uintptr_t)em & 15) == 0 && ((uintptr_t)D & 15) == 0 &&
                   (!D_lo || ((uintptr_t)D_lo & 15) == 0),
               "se_a descriptor fwd: em / D must be 16-byte aligned");
  // outputs past the last full 32-chunk: at most 16 of them run as a tail
  const int mr = M & 31;
  const int nqf = (mr == 0 || mr > 16) ? (M + 31) / 32 : M / 32;
  const int tail_w = (mr == 0 || mr > 16) ? 0 : mr;
  int tail_lg = 0;
  while ((1 << tail_lg) < tail_w) ++tail_lg;
  const int mp = (nqf + (tail_w > 0 ? 1 : 0)) * 32;
  const size_t wb = fwd_warp_bytes<T>(nnei, mp);
  GBDP_REQUIRE((size_t)kFWarps * wb <= 200 * 1024,
               "se_a descriptor fwd: nnei %d needs %zu bytes of shared memory", nnei,
               (size_t)kFWarps * wb);
  if (w == 0) w = tuned_code(kTuneFwd, sizeof(T), M, nnei, nloc, kFWarps);
  if (w == 1)
    fwd_dispatch<T, 1>(nqf, wb, st, X, D, D_lo, D_rs, em, atype, drow, ts, nloc, nnei, M, tail_w,
                         tail_lg);
  else if (w == 2)
    fwd_dispatch<T, 2>(nqf, wb, st, X, D, D_lo, D_rs, em, atype, drow, ts, nloc, nnei, M, tail_w,
                         tail_lg);
  else
    fwd_dispatch<T, 4>(nqf, wb, st, X, D, D_lo, D_rs, em, atype, drow, ts, nloc, nnei, M, tail_w,
                         tail_lg);
  GBDP_CHECK_LAUNCH("se_a_descriptor_fwd");
  return GBDP_OK;
}

template <typename T, int NQ, int NK, int U, int W>
void launch_bwd(size_t warp_bytes, cudaStream_t st, T* force, double* vir_acc, long long* force_fx,
                const T* X,
                const T* dD, const int* drow, const T* em, const int* nlist_ext,
                const T* ext_coord, const int* ext_map, const int* atype, const T* inv_std,
                BwdGeom geo, const TabSet<T>& ts, T rmin, T rmax, int nloc, int nnei, int M) {
  auto kern = k_desc_bwd<T, NQ, NK, U, W>;
  const size_t smem = (size_t)W * warp_bytes;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  // the smallest shared-memory carveout that holds the resident CTAs (28
  // warps at U = 1, 24 at U = 2): the rest of the unified L1 caches table rows
  const int per_sm = ((U == 1 ? 28 : 24) / W) * (int)(smem + 1024);
  cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                       per_sm >= 228 * 1024 ? 100 : (per_sm * 100 + 228 * 1024 - 1) / (228 * 1024));
  // prefetch distance: the warps resident on the device at once (the
  // occupancy query is repeated only when the device or the shared-memory
  // size of this instantiation changes)
  thread_local int c_dev = -1, c_pf = 0;
  thread_local size_t c_smem = 0;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != c_dev || smem != c_smem) {
    int sms = 0, ctas = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ctas, kern, W * 32, smem);
    c_dev = dev;
    c_smem = smem;
    c_pf = sms * ctas * W;
  }
  const int pf_dist = c_pf;
  kern<<<(unsigned)((nloc + W - 1) / W), W * 32, smem, st>>>(
      force, vir_acc, force_fx, X, dD, drow, em, nlist_ext, ext_coord, ext_map, atype, inv_std,
      geo, ts, rmin, rmax, nloc, nnei, M, pf_dist);
}

template <typename T, int W, int U>
void bwd_dispatch(int nk, size_t wb, cudaStream_t st, T* force, double* vir_acc,
                  long long* force_fx, const T* X,
                  const T* dD, const int* drow, const T* em, const int* nlist_ext,
                  const T* ext_coord, const int* ext_map, const int* atype, const T* inv_std,
                  BwdGeom geo, const TabSet<T>& ts, T rmin, T rmax, int nloc, int nnei, int M) {
#define GBDP_BWD_CASE(NKV)                                                                    \
  case NKV:                                                                                   \
    launch_bwd<T, (NKV + 1) / 2, NKV, U, W>(wb, st, force, vir_acc, force_fx, X, dD, drow,     \
                                                em,                                         \
                                                nlist_ext, ext_coord, ext_map, atype,       \
                                                inv_std, geo, ts, rmin, rmax, nloc, nnei, M); \
    break;
  switch (nk) {
    GBDP_BWD_CASE(1)
    GBDP_BWD_CASE(2)
    GBDP_BWD_CASE(3)
    GBDP_BWD_CASE(4)
    GBDP_BWD_CASE(5)
    GBDP_BWD_CASE(6)
    GBDP_BWD_CASE(7)
    default:
      launch_bwd<T, 4, 8, U, W>(wb, st, force, vir_acc, force_fx, X, dD, drow, em, nlist_ext,
                                    ext_coord,
                                    ext_map, atype, inv_std, geo, ts, rmin, rmax, nloc, nnei, M);
      break;
  }
#undef GBDP_BWD_CASE
}

template <typename T>
int desc_bwd(T* force, double* vir_acc, const T* X, const T* dD, const int* drow, const T* em,
             const int* nlist_ext, const T* ext_coord, const int* ext_map, const int* atype,
             const T* inv_std, const int* atom_frame, const int* frame_aoff, const int* frame_eoff,
             const T* const* tables, const T* infos, int ntypes, const int* sel, int one_side,
             float rcut_smth, float rcut, int nloc, int nframes, int M, int A, cudaStream_t st,
             long long* force_fx, int w = 0) {
  TabSet<T> ts;
  int rc = make_tabset(ts, tables, infos, ntypes, sel, one_side, M);
  if (rc) return rc;
  GBDP_REQUIRE(force && vir_acc && nframes >= 1, "se_a descriptor bwd: null output / nframes");
  const int nnei = ts.sec[ntypes];
  rc = check_shapes<T>(M, A, nnei);
  if (rc) return rc;
  GBDP_REQUIRE(((uintptr_t)force_fx & 7) == 0, "se_a descriptor bwd: force_fx not 8-byte aligned");
  if (force_fx)
    cudaMemsetAsync(force_fx, 0, sizeof(long long) * 3 * (size_t)nloc, st);
  else
    cudaMemsetAsync(force, 0, sizeof(T) * 3 * (size_t)nloc, st);
  cudaMemsetAsync(vir_acc, 0, sizeof(double) * 9 * (size_t)nframes, st);
  if (nloc == 0) {
    if (force_fx) cudaMemsetAsync(force, 0, sizeof(T) * 3 * (size_t)nloc, st);
    return GBDP_OK;
  }
  GBDP_REQUIRE(X && dD && em && nlist_ext && ext_coord && ext_map && atype && inv_std &&
                   atom_frame && frame_aoff && frame_eoff,
               "se_a descriptor bwd: null argument");
  GBDP_REQUIRE(((uintptr_t)em & 15) == 0 && ((uintptr_t)dD & 15) == 0 &&
                   ((uintptr_t)inv_std & 15) == 0,
               "se_a descriptor bwd: em / dE_dD / inv_std must be 16-byte aligned");
  BwdGeom geo{atom_frame, frame_aoff, frame_eoff};
  const size_t wb = bwd_warp_bytes<T>(nnei, M);
  GBDP_REQUIRE((size_t)kBWarps * wb <= 200 * 1024,
               "se_a descriptor bwd: nnei %d needs %zu bytes of shared memory", nnei,
               (size_t)kBWarps * wb);
  const T rmin = (T)rcut_smth, rmax = (T)rcut;
  const int nk = (M + 15) / 16;
  if (w == 0) w = tuned_code(kTuneBwd, sizeof(T), M, nnei, nloc, kBWarps);
  // the FP64 backward is built for one neighbour in flight only
  const bool u2 = sizeof(T) == 4 && code_nbrs(w) == 2;
#define GBDP_BWD_ARGS                                                                         \
  nk, wb, st, force, vir_acc, force_fx, X, dD, drow, em, nlist_ext, ext_coord, ext_map, atype, \
      inv_std, geo, ts, rmin, rmax, nloc, nnei, M
  switch (code_warps(w) * (u2 ? -1 : 1)) {
    case 1:
      bwd_dispatch<T, 1, 1>(GBDP_BWD_ARGS);
      break;
    case 2:
      bwd_dispatch<T, 2, 1>(GBDP_BWD_ARGS);
      break;
    case -1:
      if constexpr (sizeof(T) == 4) bwd_dispatch<T, 1, 2>(GBDP_BWD_ARGS);
      break;
    case -2:
      if constexpr (sizeof(T) == 4) bwd_dispatch<T, 2, 2>(GBDP_BWD_ARGS);
      break;
    case -4:
      if constexpr (sizeof(T) == 4) bwd_dispatch<T, 4, 2>(GBDP_BWD_ARGS);
      break;
    default:
      bwd_dispatch<T, 4, 1>(GBDP_BWD_ARGS);
      break;
  }
#undef GBDP_BWD_ARGS
  if (force_fx) {
    const size_t nf = 3 * (size_t)nloc;
    k_fx_finish<T><<<(unsigned)((nf + 255) / 256), 256, 0, st>>>(force, force_fx, nf,
                                                                 FxScale<T>::force);
    k_fx_finish_inplace<<<1, 256, 0, st>>>(vir_acc, 9 * (size_t)nframes, FxScale<T>::virial);
  }
  GBDP_CHECK_LAUNCH("se_a_descriptor_bwd");
  return GBDP_OK;
}

template <typename T>
int table_planar(T* dst, const T* src, int nrow, int M, cudaStream_t st) {
  GBDP_REQUIRE(M >= 1 && M <= 4096 && nrow >= 0, "table_to_planar: nrow %d, M %d", nrow, M);
  if (nrow == 0) return GBDP_OK;
  GBDP_REQUIRE(dst && src, "table_to_planar: null pointer");
  GBDP_REQUIRE(((uintptr_t)dst & 127) == 0, "table_to_planar: dst not 128-byte aligned");
  const int ps = kp_pitch<T>(M);
  const size_t n = (size_t)nrow * 3 * ps;
  const unsigned blocks = (unsigned)((n + 255) / 256 < 152 * 16 ? (n + 255) / 256 : 152 * 16);
  k_table_planar<T><<<blocks, 256, 0, st>>>(dst, src, nrow, M, ps);
  GBDP_CHECK_LAUNCH("table_to_planar");
  return GBDP_OK;
}

}  // namespace
}  // namespace gbdp

using namespace gbdp;

extern "C" size_t gbdp_table_planar_row_elems(int last_layer_size, int elem_bytes) {
  if (last_layer_size < 1) return 0;
  if (elem_bytes == 4) return 3 * (size_t)kp_pitch<float>(last_layer_size);
  if (elem_bytes == 8) return 3 * (size_t)kp_pitch<double>(last_layer_size);
  return 0;
}

extern "C" int gbdp_frame_energy_f32(double* E, const float* ae, const int* frame_of_row,
                                     int nrows, int nframes, int deterministic,
                                     gbdp_stream stream) {
  return frame_energy<float>(E, ae, frame_of_row, nrows, nframes, deterministic,
                             (cudaStream_t)stream);
}

extern "C" int gbdp_frame_energy_f64(double* E, const double* ae, const int* frame_of_row,
                                     int nrows, int nframes, int deterministic,
                                     gbdp_stream stream) {
  return frame_energy<double>(E, ae, frame_of_row, nrows, nframes, deterministic,
                              (cudaStream_t)stream);
}

extern "C" int gbdp_table_to_planar_f32(float* dst, const float* src, int nrow,
                                        int last_layer_size, gbdp_stream stream) {
  return table_planar<float>(dst, src, nrow, last_layer_size, (cudaStream_t)stream);
}

extern "C" int gbdp_table_to_planar_f64(double* dst, const double* src, int nrow,
                                        int last_layer_size, gbdp_stream stream) {
  return table_planar<double>(dst, src, nrow, last_layer_size, (cudaStream_t)stream);
}

#define GBDP_FUSED_ENTRY(T, SFX)                                                                \
  extern "C" int gbdp_se_a_descriptor_fwd_##SFX(                                                \
      T* X, T* D, const T* em, const int* atype, const int* d_row, const T* const* tables,      \
      const T* table_infos, int ntypes, const int* sel, int type_one_side, int nloc,           \
      int last_layer_size, int axis_neuron, gbdp_stream stream) {                               \
    const cudaStream_t st = (cudaStream_t)stream;                                               \
    return tune_run(kTuneFwd, (int)sizeof(T), last_layer_size, sum_sel(sel, ntypes), nloc, st,  \
                    [&](int w) {                                                                \
                      return desc_fwd<T>(X, D, nullptr, nullptr, em, atype, d_row, tables,      \
                                         table_infos, ntypes, sel, type_one_side, nloc,         \
                                         last_layer_size, axis_neuron, st, w);                  \
                    });                                                                         \
  }                                                                                             \
  extern "C" int gbdp_se_a_descriptor_bwd_##SFX(                                                \
      T* force, double* virial_acc, const T* X, const T* dE_dD, const int* d_row, const T* em, \
      const int* nlist_ext, const T* ext_coord, const int* ext_map, const int* atype,          \
      const T* inv_std, const int* atom_frame, const int* frame_atom_off,                      \
      const int* frame_ext_off, const T* const* tables, const T* table_infos, int ntypes,      \
      const int* sel, int type_one_side, float rcut_smth, float rcut, int nloc, int nframes,   \
      int last_layer_size, int axis_neuron, long long* force_fx, gbdp_stream stream) {          \
    const cudaStream_t st = (cudaStream_t)stream;                                               \
    return tune_run(kTuneBwd, (int)sizeof(T), last_layer_size, sum_sel(sel, ntypes), nloc, st,  \
                    [&](int w) {                                                                \
                      return desc_bwd<T>(force, virial_acc, X, dE_dD, d_row, em, nlist_ext,     \
                                         ext_coord, ext_map, atype, inv_std, atom_frame,       \
                                         frame_atom_off, frame_ext_off, tables, table_infos,   \
                                         ntypes, sel, type_one_side, rcut_smth, rcut, nloc,    \
                                         nframes, last_layer_size, axis_neuron, st, force_fx,  \
                                         w);                                                    \
                    });                                                                         \
  }

GBDP_FUSED_ENTRY(float, f32)
GBDP_FUSED_ENTRY(double, f64)

extern "C" int gbdp_se_a_descriptor_fwd_split_f32(
    float* X, void* D_hi, void* D_lo, float* D_rscale, const float* em, const int* atype,
    const int* d_row, const float* const* tables, const float* table_infos, int ntypes,
    const int* sel, int type_one_side, int nloc, int last_layer_size, int axis_neuron,
    gbdp_stream stream) {
  GBDP_REQUIRE(D_hi && D_lo && D_rscale, "se_a_descriptor_fwd_split: null D_hi / D_lo / D_rscale");
  const cudaStream_t st = (cudaStream_t)stream;
  return tune_run(kTuneFwd, 4, last_layer_size, sum_sel(sel, ntypes), nloc, st, [&](int w) {
    return desc_fwd<float>(X, static_cast<float*>(D_hi), D_lo, D_rscale, em, atype, d_row,
                           tables, table_infos, ntypes, sel, type_one_side, nloc,
                           last_layer_size, axis_neuron, st, w);
  });
}

extern "C" void gbdp_set_autotune(int on) { g_autotune.store(on ? 1 : 0); }

extern "C" int gbdp_autotune_report(char* buf, int len) {
  std::string out;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (const auto& kv : g_tune) {
      char line[256];
      const auto& k = kv.first;
      const auto& e = kv.second;
      int w = snprintf(line, sizeof(line), "%s f%d M=%d nnei=%d nloc=2^%d warps=%d",
                       k[0] == kTuneFwd ? "se_a_descriptor_fwd" : "se_a_descriptor_bwd",
                       8 * k[1], k[2], k[3], k[4], code_warps(e.code));
      if (k[0] == kTuneBwd) w += snprintf(line + w, sizeof(line) - w, " nbrs=%d", code_nbrs(e.code));
      w += snprintf(line + w, sizeof(line) - w, " ms=");
      for (int c = 0; c < e.n; ++c)
        w += snprintf(line + w, sizeof(line) - w, c ? ",%.4f" : "%.4f", e.ms[c]);
      snprintf(line + w, sizeof(line) - w, "\n");
      out += line;
    }
  }
  if (buf && len > 0) {
    const size_t n = std::min((size_t)len - 1, out.size());
    memcpy(buf, out.data(), n);
    buf[n] = 0;
  }
  return (int)out.size();
}
