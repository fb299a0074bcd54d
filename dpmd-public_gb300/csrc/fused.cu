// Fused compressed se_e2_a descriptor (sm_103a): the "chosen form" step.
//
// k_desc_fwd (one warp per centre atom, lanes over the M embedding outputs):
//   for every neighbour-type section: tabulated embedding G_k(x_j) times the
//   env row em[j, :], summed over j (the reference's tabulate_fusion_se_a with
//   its padding fold), then X = sum_sections / nnei and the descriptor
//   D[k, a] = sum_m X[m, k] X[m, a], a < A (DescrptBlockSeA.forward,
//   deepmd/pt/model/descriptor/se_a.py:786-866).  Neither the nloc x nnei x M
//   embedding nor the per-section outputs reach HBM; X and D do.
//
// k_desc_bwd (one warp per centre atom): dX from dE/dD and X, dy = dX / nnei,
//   then lanes over the real neighbours j: the tabulation gradient
//   (tabulate.cc:158-260) gives dE/d em[j, :]; the env-matrix derivative row
//   is recomputed from the coordinates (env_mat.cc:122-226) instead of being
//   stored, and the force / virial contributions of prod_force.cc:22-72 and
//   prod_virial.cc:22-68 are scattered straight away.  Padding slots carry no
//   coordinate dependence and are skipped.
#include "common.cuh"

namespace gbdp {
namespace {

constexpr int kMaxTab = 16;
constexpr int kFWarps = 4;

template <typename T>
struct TabSet {
  const T* table[kMaxTab];
  TableInfo<T> info[kMaxTab];
  int ntypes;
  int one_side;  // 1: table per neighbour type; 0: per (neighbour, centre)
  int sec[kMaxTab + 1];
};

template <typename T>
__device__ __forceinline__ int tab_index(const TabSet<T>& ts, int tj, int ti) {
  return ts.one_side ? tj : tj * ts.ntypes + ti;
}

template <typename T>
__device__ __forceinline__ void load_coef6(T* a, const T* __restrict__ row, int k) {
  const T* p = row + 6 * k;
#pragma unroll
  for (int c = 0; c < 6; ++c) a[c] = __ldg(p + c);
}
template <>
__device__ __forceinline__ void load_coef6<float>(float* a, const float* __restrict__ row, int k) {
  const float2* p = reinterpret_cast<const float2*>(row + 6 * k);
  float2 u = __ldg(p), v = __ldg(p + 1), w = __ldg(p + 2);
  a[0] = u.x;
  a[1] = u.y;
  a[2] = v.x;
  a[3] = v.y;
  a[4] = w.x;
  a[5] = w.y;
}

__device__ __forceinline__ float tf32_head(float x) {
  return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
}
__device__ __forceinline__ double tf32_head(double x) { return x; }

// ---------------------------------------------------------------- forward --
template <typename T, int NQ, int A>
__global__ void __launch_bounds__(kFWarps * 32)
    k_desc_fwd(T* __restrict__ X, T* __restrict__ D, T* __restrict__ D_lo,
               const T* __restrict__ em, const int* __restrict__ atype,
               const int* __restrict__ drow, TabSet<T> ts, int nloc, int nnei, int M) {
  __shared__ T xs[kFWarps][4][NQ * 32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * kFWarps + warp;
  if (i >= nloc) return;
  const int ti = atype[i];
  T acc[NQ][4];
#pragma unroll
  for (int q = 0; q < NQ; ++q)
#pragma unroll
    for (int m = 0; m < 4; ++m) acc[q][m] = T(0);
  if (ti >= 0) {
    for (int t = 0; t < ts.ntypes; ++t) {
      const int s0 = ts.sec[t], ns = ts.sec[t + 1] - s0;
      if (ns == 0) continue;
      const int tb = tab_index(ts, t, ti);
      const T* tab = ts.table[tb];
      const TableInfo<T> inf = ts.info[tb];
      const T* e0 = em + ((size_t)i * nnei + s0) * 4;
      // fold point of this section (tabulate.cc:108-115)
      const T last = e0[(ns - 1) * 4];
      int bp = ns;
      for (int b = 0; b < ns; b += 32) {
        const int j = b + lane;
        bool hit = false;
        if (j < ns) {
          const T* e = e0 + j * 4;
          hit = e[0] == last && e[1] == T(0) && e[2] == T(0) && e[3] == T(0);
        }
        const unsigned mk = __ballot_sync(kFull, hit);
        if (mk) {
          bp = b + __ffs(mk) - 1;
          break;
        }
      }
      const int jend = bp < ns ? bp + 1 : ns;
      for (int j = 0; j < jend; ++j) {
        const T* e = e0 + j * 4;
        T x = e[0];
        const T l0 = e[0], l1 = e[1], l2 = e[2], l3 = e[3];
        const T w = (j == bp) ? T(ns - j) : T(1);
        const int idx = locate_row(inf, x);
        const T* row = tab + (size_t)idx * M * 6;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
          const int k = q * 32 + lane;
          if (k < M) {
            T a[6];
            load_coef6<T>(a, row, k);
            const T wv = w * poly5(a, x);
            acc[q][0] += wv * l0;
            acc[q][1] += wv * l1;
            acc[q][2] += wv * l2;
            acc[q][3] += wv * l3;
          }
        }
      }
    }
  }
  const T inv = T(1) / T(nnei);
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    const int k = q * 32 + lane;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      acc[q][m] *= inv;
      xs[warp][m][q * 32 + lane] = acc[q][m];
      if (k < M) X[((size_t)i * 4 + m) * M + k] = acc[q][m];
    }
  }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    const int k = q * 32 + lane;
    if (k >= M) continue;
    const size_t r = drow ? (size_t)drow[i] : (size_t)i;
    T* d = D + (r * M + k) * A;
    T* dl = D_lo ? D_lo + (r * M + k) * A : nullptr;
#pragma unroll
    for (int a = 0; a < A; ++a) {
      T v = acc[q][0] * xs[warp][0][a] + acc[q][1] * xs[warp][1][a] +
            acc[q][2] * xs[warp][2][a] + acc[q][3] * xs[warp][3][a];
      if (dl) {
        // TF32 head (low 13 mantissa bits cleared) and the exact remainder
        const T hi = tf32_head(v);
        d[a] = hi;
        dl[a] = v - hi;
      } else {
        d[a] = v;
      }
    }
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

// Sum of v[0..31] over the 32 lanes, scattered: lane l returns the total of
// value l.  31 shuffles for 32 sums (instead of 5 per sum): at the step with
// offset o every lane keeps the half of its values selected by lane bit o and
// adds the partner's copy of that half.
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

constexpr int kBwdGroup = 6;  // neighbours per reduce-scatter (6 x 5 sums <= 32)

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

template <typename T, int NQ, int A>
__global__ void __launch_bounds__(kFWarps * 32)
    k_desc_bwd(T* __restrict__ force, double* __restrict__ vir_acc, const T* __restrict__ X,
               const T* __restrict__ dD, const int* __restrict__ drow, const T* __restrict__ em,
               const int* __restrict__ nlist_ext, const T* __restrict__ ext_coord,
               const int* __restrict__ ext_map, const int* __restrict__ atype,
               const T* __restrict__ inv_std, BwdGeom geo, TabSet<T> ts, T rmin, T rmax, int nloc,
               int nnei, int M) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * kFWarps + warp;
  if (i >= nloc) return;
  constexpr int MP = NQ * 32;
  constexpr int GP = MP + 1;               // padded row of the transposed dE/dD
  constexpr int RW = 4 * MP + A * GP + 1;  // per-warp shared region (T elements)
  T* xs = reinterpret_cast<T*>(smem_raw) + (size_t)warp * RW;
  T* gs = xs + 4 * MP;  // dE/dD transposed, gs[a * GP + k]: conflict-free for both uses
  const int ti = atype[i];
  for (int t = lane; t < 4 * M; t += 32) {
    const int m = t / M, k = t - m * M;
    xs[m * MP + k] = X[(size_t)i * 4 * M + t];
  }
  const size_t drow_i = drow ? (size_t)drow[i] : (size_t)i;
  for (int t = lane; t < M * A; t += 32) {
    const int k = t / A, a = t - k * A;
    gs[a * GP + k] = dD[drow_i * M * A + t];
  }
  __syncwarp();
  const T inv = T(1) / T(nnei);
  // dy[m][k] = dX[m][k] / nnei, dX = sum_a G[k][a] X[m][a] + [k < A] sum_k' G[k'][k] X[m][k'],
  // kept in registers: lane owns k = q * 32 + lane
  T dyr[NQ][4];
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    const int k = q * 32 + lane;
    T dx[4] = {T(0), T(0), T(0), T(0)};
    if (k < M) {
#pragma unroll
      for (int a = 0; a < A; ++a) {
        const T g = gs[a * GP + k];
#pragma unroll
        for (int m = 0; m < 4; ++m) dx[m] += g * xs[m * MP + a];
      }
      if (k < A) {
        for (int kk = 0; kk < M; ++kk) {
          const T g = gs[k * GP + kk];
#pragma unroll
          for (int m = 0; m < 4; ++m) dx[m] += g * xs[m * MP + kk];
        }
      }
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) dyr[q][m] = dx[m] * inv;
  }
  __syncwarp();
  if (ti < 0) return;
  // the region now holds dE/d em of this atom's filled slots ([nnei][4]) and
  // the 32 scattered sums of one neighbour group
  T* nets = xs;
  T* gbuf = xs + (size_t)nnei * 4;
  const int* nl_i = nlist_ext + (size_t)i * nnei;

  // ---- phase 1: tabulation gradient, lanes over k, neighbours in groups
  for (int t = 0; t < ts.ntypes; ++t) {
    const int s0 = ts.sec[t], ns = ts.sec[t + 1] - s0;
    const int nv = filled_prefix(nl_i + s0, ns);
    const int tb = tab_index(ts, t, ti);
    const T* tab = ts.table[tb];
    const TableInfo<T> inf = ts.info[tb];
    for (int g0 = 0; g0 < nv; g0 += kBwdGroup) {
      T part[32];
#pragma unroll
      for (int c = 0; c < 32; ++c) part[c] = T(0);
#pragma unroll
      for (int gg = 0; gg < kBwdGroup; ++gg) {
        const int j = g0 + gg;
        if (j < nv) {
          const T* e = em + ((size_t)i * nnei + s0 + j) * 4;
          const T l0 = e[0], l1 = e[1], l2 = e[2], l3 = e[3];
          T x = l0;
          const int idx = locate_row(inf, x);
          const T* row = tab + (size_t)idx * M * 6;
#pragma unroll
          for (int q = 0; q < NQ; ++q) {
            const int k = q * 32 + lane;
            if (k < M) {
              T a[6];
              load_coef6<T>(a, row, k);
              // value and derivative by one Horner sweep (9 FMA)
              T v = a[5], dv = a[5];
              v = v * x + a[4];
              dv = dv * x + v;
              v = v * x + a[3];
              dv = dv * x + v;
              v = v * x + a[2];
              dv = dv * x + v;
              v = v * x + a[1];
              dv = dv * x + v;
              v = v * x + a[0];
              part[gg * 5 + 0] += v * dyr[q][0];
              part[gg * 5 + 1] += v * dyr[q][1];
              part[gg * 5 + 2] += v * dyr[q][2];
              part[gg * 5 + 3] += v * dyr[q][3];
              part[gg * 5 + 4] +=
                  dv * (l0 * dyr[q][0] + l1 * dyr[q][1] + l2 * dyr[q][2] + l3 * dyr[q][3]);
            }
          }
        }
      }
      gbuf[lane] = reduce_scatter32(part, lane);
      __syncwarp();
      if (lane < kBwdGroup && g0 + lane < nv) {
        const int s = s0 + g0 + lane;
        const T* gv = gbuf + lane * 5;
        nets[s * 4 + 0] = gv[0] + gv[4];  // em_x is em[:, 0]
        nets[s * 4 + 1] = gv[1];
        nets[s * 4 + 2] = gv[2];
        nets[s * 4 + 3] = gv[3];
      }
      __syncwarp();
    }
  }

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
  double vir[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) vir[q] = 0.;
  for (int t = 0; t < ts.ntypes; ++t) {
    const int s0 = ts.sec[t], ns = ts.sec[t + 1] - s0;
    const int nv = filled_prefix(nl_i + s0, ns);
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
      const T gw[4] = {nets[s * 4 + 0] * isd[s * 4 + 0], nets[s * 4 + 1] * isd[s * 4 + 1],
                       nets[s * 4 + 2] * isd[s * 4 + 2], nets[s * 4 + 3] * isd[s * 4 + 3]};
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
      T* fj = force + (size_t)(aoff + jl) * 3;
      atomicAdd(fj + 0, v3[0]);
      atomicAdd(fj + 1, v3[1]);
      atomicAdd(fj + 2, v3[2]);
      ci[0] += v3[0];
      ci[1] += v3[1];
      ci[2] += v3[2];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) vir[a * 3 + b] += (double)(v3[a] * rr[b]);
    }
  }
  ci[0] = warp_sum(ci[0]);
  ci[1] = warp_sum(ci[1]);
  ci[2] = warp_sum(ci[2]);
  if (lane == 0) {
    T* fi = force + (size_t)i * 3;
    atomicAdd(fi + 0, -ci[0]);
    atomicAdd(fi + 1, -ci[1]);
    atomicAdd(fi + 2, -ci[2]);
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    const double v = warp_sum(vir[q]);
    if (lane == 0) atomicAdd(vir_acc + f * 9 + q, v);
  }
}

template <typename T>
int make_tabset(TabSet<T>& ts, const T* const* tables, const T* infos, int ntypes, const int* sel,
                int one_side) {
  GBDP_REQUIRE(ntypes >= 1 && ntypes <= 4, "se_a descriptor: ntypes %d not in [1,4]", ntypes);
  const int ntab = one_side ? ntypes : ntypes * ntypes;
  GBDP_REQUIRE(ntab <= kMaxTab, "se_a descriptor: too many tables");
  ts.ntypes = ntypes;
  ts.one_side = one_side ? 1 : 0;
  ts.sec[0] = 0;
  for (int t = 0; t < ntypes; ++t) ts.sec[t + 1] = ts.sec[t] + sel[t];
  for (int k = 0; k < ntab; ++k) {
    GBDP_REQUIRE(tables[k] != nullptr && ((uintptr_t)tables[k] & 15) == 0,
                 "se_a descriptor: table %d null or not 16-byte aligned", k);
    ts.table[k] = tables[k];
    ts.info[k] = make_table_info(infos + 6 * k);
  }
  return GBDP_OK;
}

template <typename T>
int desc_fwd(T* X, T* D, T* D_lo, const T* em, const int* atype, const int* drow,
             const T* const* tables,
             const T* infos, int ntypes, const int* sel, int one_side, int nloc, int M, int A,
             cudaStream_t st) {
  TabSet<T> ts;
  int rc = make_tabset(ts, tables, infos, ntypes, sel, one_side);
  if (rc) return rc;
  GBDP_REQUIRE(M >= 1 && M <= 128, "se_a descriptor: neuron[-1] %d not in [1,128]", M);
  GBDP_REQUIRE(A == 16, "se_a descriptor: axis_neuron %d (this build supports 16)", A);
  if (nloc == 0) return GBDP_OK;
  const int nnei = ts.sec[ntypes];
  const dim3 grid((nloc + kFWarps - 1) / kFWarps), block(kFWarps * 32);
  const int nq = (M + 31) / 32;
  if (nq == 4)
    k_desc_fwd<T, 4, 16><<<grid, block, 0, st>>>(X, D, D_lo, em, atype, drow, ts, nloc, nnei, M);
  else if (nq == 3)
    k_desc_fwd<T, 3, 16><<<grid, block, 0, st>>>(X, D, D_lo, em, atype, drow, ts, nloc, nnei, M);
  else if (nq == 2)
    k_desc_fwd<T, 2, 16><<<grid, block, 0, st>>>(X, D, D_lo, em, atype, drow, ts, nloc, nnei, M);
  else
    k_desc_fwd<T, 1, 16><<<grid, block, 0, st>>>(X, D, D_lo, em, atype, drow, ts, nloc, nnei, M);
  GBDP_CHECK_LAUNCH("se_a_descriptor_fwd");
  return GBDP_OK;
}

template <typename T>
int desc_bwd(T* force, double* vir_acc, const T* X, const T* dD, const int* drow, const T* em,
             const int* nlist_ext, const T* ext_coord, const int* ext_map, const int* atype,
             const T* inv_std, const int* atom_frame, const int* frame_aoff, const int* frame_eoff,
             const T* const* tables, const T* infos, int ntypes, const int* sel, int one_side,
             float rcut_smth, float rcut, int nloc, int nframes, int M, int A, cudaStream_t st) {
  TabSet<T> ts;
  int rc = make_tabset(ts, tables, infos, ntypes, sel, one_side);
  if (rc) return rc;
  GBDP_REQUIRE(force && vir_acc && nframes >= 1, "se_a descriptor bwd: null output / nframes");
  cudaMemsetAsync(force, 0, sizeof(T) * 3 * (size_t)nloc, st);
  cudaMemsetAsync(vir_acc, 0, sizeof(double) * 9 * (size_t)nframes, st);
  GBDP_REQUIRE(M >= 1 && M <= 128, "se_a descriptor: neuron[-1] %d not in [1,128]", M);
  GBDP_REQUIRE(A == 16, "se_a descriptor: axis_neuron %d (this build supports 16)", A);
  if (nloc == 0) return GBDP_OK;
  const int nnei = ts.sec[ntypes];
  BwdGeom geo{atom_frame, frame_aoff, frame_eoff};
  const int nq = (M + 31) / 32;
  const int MP = nq * 32;
  const int RW = 4 * MP + 16 * (MP + 1) + 1;
  const size_t smem = (size_t)kFWarps * RW * sizeof(T);
  GBDP_REQUIRE(nnei * 4 + 32 <= RW, "se_a descriptor bwd: nnei %d too large for neuron[-1] %d",
               nnei, M);
  const dim3 grid((nloc + kFWarps - 1) / kFWarps), block(kFWarps * 32);
#define GBDP_LAUNCH_BWD(NQV)                                                                   \
  {                                                                                            \
    auto kern = k_desc_bwd<T, NQV, 16>;                                                        \
    if (smem > 48 * 1024)                                                                      \
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);      \
    kern<<<grid, block, smem, st>>>(force, vir_acc, X, dD, drow, em, nlist_ext, ext_coord,     \
                                    ext_map, atype, inv_std, geo, ts, (T)rcut_smth, (T)rcut,   \
                                    nloc, nnei, M);                                            \
  }
  if (nq == 4)
    GBDP_LAUNCH_BWD(4)
  else if (nq == 3)
    GBDP_LAUNCH_BWD(3)
  else if (nq == 2)
    GBDP_LAUNCH_BWD(2)
  else
    GBDP_LAUNCH_BWD(1)
#undef GBDP_LAUNCH_BWD
  GBDP_CHECK_LAUNCH("se_a_descriptor_bwd");
  return GBDP_OK;
}

}  // namespace
}  // namespace gbdp

using namespace gbdp;

#define GBDP_FUSED_ENTRY(T, SFX)                                                                \
  extern "C" int gbdp_se_a_descriptor_fwd_##SFX(                                                \
      T* X, T* D, const T* em, const int* atype, const int* d_row, const T* const* tables,      \
      const T* table_infos, int ntypes, const int* sel, int type_one_side, int nloc,           \
      int last_layer_size, int axis_neuron, gbdp_stream stream) {                               \
    return desc_fwd<T>(X, D, nullptr, em, atype, d_row, tables, table_infos, ntypes, sel,       \
                       type_one_side,                                                          \
                       nloc, last_layer_size, axis_neuron, (cudaStream_t)stream);              \
  }                                                                                             \
  extern "C" int gbdp_se_a_descriptor_bwd_##SFX(                                                \
      T* force, double* virial_acc, const T* X, const T* dE_dD, const int* d_row, const T* em, \
      const int* nlist_ext, const T* ext_coord, const int* ext_map, const int* atype,          \
      const T* inv_std, const int* atom_frame, const int* frame_atom_off,                      \
      const int* frame_ext_off, const T* const* tables, const T* table_infos, int ntypes,      \
      const int* sel, int type_one_side, float rcut_smth, float rcut, int nloc, int nframes,   \
      int last_layer_size, int axis_neuron, gbdp_stream stream) {                               \
    return desc_bwd<T>(force, virial_acc, X, dE_dD, d_row, em, nlist_ext, ext_coord, ext_map,  \
                       atype,                                                                  \
                       inv_std, atom_frame, frame_atom_off, frame_ext_off, tables, table_infos,    \
                       ntypes, sel, type_one_side, rcut_smth, rcut, nloc, nframes,             \
                       last_layer_size, axis_neuron, (cudaStream_t)stream);                    \
  }

GBDP_FUSED_ENTRY(float, f32)
GBDP_FUSED_ENTRY(double, f64)

extern "C" int gbdp_se_a_descriptor_fwd_split_f32(
    float* X, float* D_hi, float* D_lo, const float* em, const int* atype, const int* d_row,
    const float* const* tables, const float* table_infos, int ntypes, const int* sel,
    int type_one_side, int nloc, int last_layer_size, int axis_neuron, gbdp_stream stream) {
  GBDP_REQUIRE(D_lo != nullptr, "se_a_descriptor_fwd_split: null D_lo");
  return desc_fwd<float>(X, D_hi, D_lo, em, atype, d_row, tables, table_infos, ntypes, sel,
                         type_one_side, nloc, last_layer_size, axis_neuron,
                         (cudaStream_t)stream);
}
