// Periodic neighbour build + environment matrix for se_e2_a (sm_103a).
//
// Pipeline per packed batch of frames (one launch each, all stream-ordered,
// no host synchronisation, capturable in a CUDA graph):
//   k_localize   wrap local atoms into the box, write them as the first
//                extended atoms, bin them into the reference's cells;
//   k_cell_scan  one CTA per frame: cell offsets, ghost offsets, nall;
//   k_cell_bucket / k_cell_rank  atoms of each cell in ascending index order;
//   k_ghost_fill one warp per extended cell: ghost images in copy_coord order
//                and a cell-ordered packed copy of every extended atom;
//   k_nlist_env  one warp per centre atom: candidates from the stencil of
//                cells, per-type rank by (float r^2, index), env matrix row
//                and its derivative, normalised by davg/dstd.
#include <algorithm>
#include <cstring>
#include <cmath>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace gbdp {
namespace {

constexpr int kMaxTypes = 16;
constexpr int kEnvWarps = 4;  // warps (centre atoms) per CTA in k_nlist_env

struct SecInfo {
  int ntypes;
  int nnei;
  int sec[kMaxTypes + 1];
};

struct __align__(32) D4 {
  double x, y, z, w;
};

template <typename T>
struct XsOf;
template <>
struct XsOf<float> {
  using type = float4;
};
template <>
struct XsOf<double> {
  using type = D4;
};

__device__ __forceinline__ int pack_idx_type(int idx, int type) {
  return (int)(((unsigned)(type & 0xff) << 24) | (unsigned)idx);
}

__device__ __forceinline__ float4 make_xs(float x, float y, float z, int packed) {
  return make_float4(x, y, z, __int_as_float(packed));
}
__device__ __forceinline__ D4 make_xs(double x, double y, double z, int packed) {
  D4 r;
  r.x = x;
  r.y = y;
  r.z = z;
  r.w = (double)packed;
  return r;
}
__device__ __forceinline__ int xs_packed(const float4& v) { return __float_as_int(v.w); }
__device__ __forceinline__ int xs_packed(const D4& v) { return (int)v.w; }

// Exact (non-contracted) arithmetic helpers, so that the wrap into the box
// and the float r^2 sort key round exactly like the reference's CPU code.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float fmod1(float a) { return fmodf(a, 1.0f); }
__device__ __forceinline__ double fmod1(double a) { return fmod(a, 1.0); }

template <typename T>
__device__ __forceinline__ const T* box_of(const gbdp_nbr_frame& g);
template <>
__device__ __forceinline__ const float* box_of<float>(const gbdp_nbr_frame& g) {
  return g.boxf;
}
template <>
__device__ __forceinline__ const double* box_of<double>(const gbdp_nbr_frame& g) {
  return g.box;
}
template <typename T>
__device__ __forceinline__ const T* rec_of(const gbdp_nbr_frame& g);
template <>
__device__ __forceinline__ const float* rec_of<float>(const gbdp_nbr_frame& g) {
  return g.recf;
}
template <>
__device__ __forceinline__ const double* rec_of<double>(const gbdp_nbr_frame& g) {
  return g.rec;
}

__device__ __forceinline__ int floordiv(int a, int b) {
  int q = a / b;
  return (a % b != 0 && (a < 0)) ? q - 1 : q;
}

__device__ __forceinline__ int find_frame_atom(const gbdp_nbr_frame* fr, int nframes, int i) {
  int lo = 0, hi = nframes - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (fr[mid].atom_off <= i)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int find_frame_cell(const gbdp_nbr_frame* fr, int nframes, int e) {
  int lo = 0, hi = nframes - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (fr[mid].ext_cell_off <= e)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// ----------------------------------------------------------- k_localize --
// source/lib/src/coord.cc:13-28 (normalize_coord_cpu) and the cell index of
// source/lib/src/neighbor_list.cc:86-111 (build_clist).
template <typename T>
__global__ void k_localize(const gbdp_nbr_frame* __restrict__ fr, int nframes, int nloc_total,
                           const T* __restrict__ coord, const int* __restrict__ atype,
                           T* __restrict__ ext_coord, int* __restrict__ ext_type,
                           int* __restrict__ ext_map, int* __restrict__ atom_frame,
                           int* __restrict__ atom_cell, int* __restrict__ cell_count,
                           int* __restrict__ sub_count, int* __restrict__ atom_sub) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nloc_total) return;
  const int f = find_frame_atom(fr, nframes, i);
  const gbdp_nbr_frame& g = fr[f];
  const int il = i - g.atom_off;
  const T* box = box_of<T>(g);
  const T* rec = rec_of<T>(g);
  T p[3] = {coord[3 * (size_t)i], coord[3 * (size_t)i + 1], coord[3 * (size_t)i + 2]};
  T ri[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    T v = add_rn(add_rn(mul_rn(p[0], rec[d * 3 + 0]), mul_rn(p[1], rec[d * 3 + 1])),
                 mul_rn(p[2], rec[d * 3 + 2]));
    v = fmod1(v);
    if (v < T(0)) v = add_rn(v, T(1));
    ri[d] = v;
  }
  T q[3];
#pragma unroll
  for (int d = 0; d < 3; ++d)
    q[d] = add_rn(add_rn(mul_rn(ri[0], box[0 * 3 + d]), mul_rn(ri[1], box[1 * 3 + d])),
                  mul_rn(ri[2], box[2 * 3 + d]));
  const size_t e = (size_t)g.ext_off + il;
  ext_coord[3 * e + 0] = q[0];
  ext_coord[3 * e + 1] = q[1];
  ext_coord[3 * e + 2] = q[2];
  ext_type[e] = atype[i];
  ext_map[e] = il;
  // cell from the wrapped coordinate, in double (SimulationRegion<double>)
  double pd[3] = {(double)q[0], (double)q[1], (double)q[2]};
  int ci[3], sub = 0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double in = __dadd_rn(__dadd_rn(__dmul_rn(pd[0], g.rec[d * 3 + 0]),
                                    __dmul_rn(pd[1], g.rec[d * 3 + 1])),
                          __dmul_rn(pd[2], g.rec[d * 3 + 2]));
    double cs = 1. / g.ncell[d];
    int k = (int)(in / cs);
    if (in < 0.) --k;
    k = max(0, min(k, g.ncell[d] - 1));
    ci[d] = k;
    // the half of the cell along d (searched as its own cell when split)
    if ((g.subcell >> d) & 1) {
      const double u = in / cs - (double)k;
      if (u >= 0.5) sub |= 1 << d;
    }
  }
  const int c = g.cell_off + (ci[0] * g.ncell[1] + ci[1]) * g.ncell[2] + ci[2];
  atom_frame[i] = f;
  atom_cell[i] = c;
  atom_sub[i] = sub;
  atomicAdd(&cell_count[c], 1);
  atomicAdd(&sub_count[(size_t)c * 8 + sub], 1);
}

// Block-wide exclusive scan (blockDim.x multiple of 32, <= 1024).
__device__ int block_excl_scan(int v, int* warp_tot, int& total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  if (w == 0) {
    int t = lane < nw ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(kFull, t, o);
      if (lane >= o) t += y;
    }
    if (lane < nw) warp_tot[lane] = t;
  }
  __syncthreads();
  const int off = w > 0 ? warp_tot[w - 1] : 0;
  total = warp_tot[nw - 1];
  __syncthreads();
  return off + x - v;
}

__device__ __forceinline__ void ext_cell_source(const gbdp_nbr_frame& g, int e, int* ii,
                                                int* sh, int& src, bool& local) {
  const int n1 = g.ncell[1] + 2 * g.ngcell[1], n2 = g.ncell[2] + 2 * g.ngcell[2];
  int e0 = e / (n1 * n2), r = e - e0 * n1 * n2;
  int e1 = r / n2, e2 = r - e1 * n2;
  ii[0] = e0 - g.ngcell[0];
  ii[1] = e1 - g.ngcell[1];
  ii[2] = e2 - g.ngcell[2];
  local = true;
  int jj[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    // compute_pbc_shift of neighbor_list.cc:727-743 in closed form
    sh[d] = -floordiv(ii[d], g.ncell[d]);
    jj[d] = ii[d] + sh[d] * g.ncell[d];
    local = local && ii[d] >= 0 && ii[d] < g.ncell[d];
  }
  src = g.cell_off + (jj[0] * g.ncell[1] + jj[1]) * g.ncell[2] + jj[2];
}

// ---------------------------------------------------------- k_cell_scan --
__global__ void k_cell_scan(const gbdp_nbr_frame* __restrict__ fr,
                            const int* __restrict__ cell_count, int* __restrict__ cell_start,
                            int* __restrict__ ext_start, int* __restrict__ ext_cnt,
                            int* __restrict__ ghost_start, int* __restrict__ ext_nall,
                            int* __restrict__ status, const int* __restrict__ sub_count,
                            int* __restrict__ ext_sub) {
  __shared__ int warp_tot[32];
  const gbdp_nbr_frame& g = fr[blockIdx.x];
  const int ncl = g.ncell[0] * g.ncell[1] * g.ncell[2];
  int carry = 0;
  for (int base = 0; base < ncl; base += blockDim.x) {
    int c = base + threadIdx.x;
    int v = c < ncl ? cell_count[g.cell_off + c] : 0;
    int tot;
    int ex = block_excl_scan(v, warp_tot, tot);
    if (c < ncl) cell_start[g.cell_off + c] = g.atom_off + carry + ex;
    carry += tot;
  }
  const int ne = (g.ncell[0] + 2 * g.ngcell[0]) * (g.ncell[1] + 2 * g.ngcell[1]) *
                 (g.ncell[2] + 2 * g.ngcell[2]);
  int carry_all = 0, carry_ghost = 0;
  for (int base = 0; base < ne; base += blockDim.x) {
    int e = base + threadIdx.x;
    int cnt = 0, gcnt = 0, src = 0;
    if (e < ne) {
      int ii[3], sh[3];
      bool local;
      ext_cell_source(g, e, ii, sh, src, local);
      cnt = cell_count[src];
      gcnt = local ? 0 : cnt;
    }
    int tot_all, tot_ghost;
    int ex_all = block_excl_scan(cnt, warp_tot, tot_all);
    int ex_ghost = block_excl_scan(gcnt, warp_tot, tot_ghost);
    if (e < ne) {
      const int st = g.ext_off + carry_all + ex_all;
      ext_start[g.ext_cell_off + e] = st;
      ext_cnt[g.ext_cell_off + e] = cnt;
      ghost_start[g.ext_cell_off + e] = g.nloc + carry_ghost + ex_ghost;
      // xs start of each half cell (the source cell's atoms in half-cell
      // order), then the cell's end
      int* es = ext_sub + 9 * (size_t)(g.ext_cell_off + e);
      int acc = st;
#pragma unroll
      for (int h = 0; h < 8; ++h) {
        es[h] = acc;
        acc += sub_count[8 * (size_t)src + h];
      }
      es[8] = acc;
    }
    carry_all += tot_all;
    carry_ghost += tot_ghost;
  }
  if (threadIdx.x == 0) {
    const int nall = g.nloc + carry_ghost;
    ext_nall[blockIdx.x] = nall;
    if (nall > g.ext_cap) raise_status(status, GBDP_STATUS_EXT_OVERFLOW);
  }
}

// ------------------------------------------- k_cell_bucket / k_cell_rank --
__global__ void k_cell_bucket(int nloc_total, const gbdp_nbr_frame* __restrict__ fr,
                              const int* __restrict__ atom_frame,
                              const int* __restrict__ atom_cell,
                              const int* __restrict__ cell_start, int* __restrict__ cell_fill,
                              int* __restrict__ bucket) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nloc_total) return;
  const int c = atom_cell[i];
  const int slot = atomicAdd(&cell_fill[c], 1);
  bucket[cell_start[c] + slot] = i - fr[atom_frame[i]].atom_off;
}

// Ascending local index inside each cell: the order build_clist pushes them.
// The atom's position in its cell's candidate copy (xs): ordered by half
// cell, then by local index.
__global__ void k_cell_rank(int nloc_total, const gbdp_nbr_frame* __restrict__ fr,
                            const int* __restrict__ atom_frame,
                            const int* __restrict__ atom_cell,
                            const int* __restrict__ cell_start,
                            const int* __restrict__ cell_count, const int* __restrict__ bucket,
                            int* __restrict__ cell_atoms, const int* __restrict__ atom_sub,
                            int* __restrict__ atom_xpos) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nloc_total) return;
  const int c = atom_cell[i];
  const int aoff = fr[atom_frame[i]].atom_off;
  const int il = i - aoff;
  const int hs = atom_sub[i];
  const int s = cell_start[c], n = cell_count[c];
  int rank = 0, xpos = 0;
  for (int k = 0; k < n; ++k) {
    const int o = bucket[s + k];
    const int ho = atom_sub[aoff + o];
    rank += o < il;
    xpos += ho < hs || (ho == hs && o < il);
  }
  cell_atoms[s + rank] = il;
  atom_xpos[i] = xpos;
}

// --------------------------------------------------------- k_ghost_fill --
// source/lib/src/neighbor_list.cc:796-845: for each extended cell in
// lexicographic order that is not local, the atoms of its periodic source
// cell shifted by the image vector (double arithmetic, rounded to T).
template <typename T>
__global__ void k_ghost_fill(const gbdp_nbr_frame* __restrict__ fr, int nframes,
                             int next_cell_total, const int* __restrict__ cell_start,
                             const int* __restrict__ cell_count,
                             const int* __restrict__ cell_atoms,
                             const int* __restrict__ ext_start,
                             const int* __restrict__ ghost_start, T* __restrict__ ext_coord,
                             int* __restrict__ ext_type, int* __restrict__ ext_map,
                             typename XsOf<T>::type* __restrict__ xs,
                             const int* __restrict__ atom_xpos) {
  const int ew = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (ew >= next_cell_total) return;
  const int f = find_frame_cell(fr, nframes, ew);
  const gbdp_nbr_frame& g = fr[f];
  const int e = ew - g.ext_cell_off;
  int ii[3], sh[3], src;
  bool local;
  ext_cell_source(g, e, ii, sh, src, local);
  double sv[3];
#pragma unroll
  for (int d = 0; d < 3; ++d)
    sv[d] = __dadd_rn(__dadd_rn(__dmul_rn((double)sh[0], g.box[0 * 3 + d]),
                                __dmul_rn((double)sh[1], g.box[1 * 3 + d])),
                      __dmul_rn((double)sh[2], g.box[2 * 3 + d]));
  const int n = cell_count[src], s = cell_start[src];
  const int xs0 = ext_start[ew], g0 = ghost_start[ew];
  const int xs_end = g.ext_off + g.ext_cap;
  for (int k = lane; k < n; k += 32) {
    // slots past the frame's reservation are never written (k_cell_scan has
    // already raised GBDP_STATUS_EXT_OVERFLOW for that case)
    if (xs0 + k >= xs_end || (!local && g0 + k >= g.ext_cap)) break;
    const int p = cell_atoms[s + k];
    const size_t ep = (size_t)g.ext_off + p;
    T x = ext_coord[3 * ep], y = ext_coord[3 * ep + 1], z = ext_coord[3 * ep + 2];
    const int t = ext_type[ep];
    int idx = p;
    if (!local) {
      idx = g0 + k;
      x = (T)__dsub_rn((double)x, sv[0]);
      y = (T)__dsub_rn((double)y, sv[1]);
      z = (T)__dsub_rn((double)z, sv[2]);
      const size_t eg = (size_t)g.ext_off + idx;
      ext_coord[3 * eg] = x;
      ext_coord[3 * eg + 1] = y;
      ext_coord[3 * eg + 2] = z;
      ext_type[eg] = t;
      ext_map[eg] = p;
    }
    // the candidate copy is ordered by half cell (extended indices keep
    // copy_coord's order)
    const int xp = atom_xpos[(size_t)g.atom_off + p];
    if (xs0 + xp < xs_end) xs[xs0 + xp] = make_xs(x, y, z, pack_idx_type(idx, t));
  }
}

// --------------------------------------------------------- k_nlist_env --
// Candidate test and key: source/lib/src/neighbor_list.cc:893-903
// (r^2 < rc^2 in the coordinate type) and source/lib/src/fmt_nlist.cc:114-143
// (float r^2 <= float rc^2, order by (type, float r^2, index), first sel[t]
// of each type).  Env row: source/lib/src/env_mat.cc:122-226 with
// source/lib/include/switcher.h:60-83; normalisation prod_env_mat.cc:84-100.
template <typename T>
__device__ __forceinline__ void spline5(T& vv, T& dd, T xx, T rmin, T rmax) {
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

template <typename T>
__device__ __forceinline__ bool cand_test(const typename XsOf<T>::type& r, T xi, T yi, T zi,
                                          float rc2f, float& key);

template <>
__device__ __forceinline__ bool cand_test<float>(const float4& r, float xi, float yi, float zi,
                                                 float rc2f, float& key) {
  float dx = __fsub_rn(r.x, xi), dy = __fsub_rn(r.y, yi), dz = __fsub_rn(r.z, zi);
  float r2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
  key = r2;
  return r2 < rc2f;
}

template <>
__device__ __forceinline__ bool cand_test<double>(const D4& r, double xi, double yi, double zi,
                                                  float rc2f, float& key) {
  double dx = __dsub_rn(xi, r.x), dy = __dsub_rn(yi, r.y), dz = __dsub_rn(zi, r.z);
  double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  float fx = __fsub_rn((float)r.x, (float)xi), fy = __fsub_rn((float)r.y, (float)yi),
        fz = __fsub_rn((float)r.z, (float)zi);
  float r2f = __fadd_rn(__fadd_rn(__fmul_rn(fx, fx), __fmul_rn(fy, fy)), __fmul_rn(fz, fz));
  key = r2f;
  return r2 < (double)rc2f && r2f <= rc2f;
}

template <typename T>
__device__ __forceinline__ void store4(T* p, T a, T b, T c, T d);
template <>
__device__ __forceinline__ void store4<float>(float* p, float a, float b, float c, float d) {
  *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
}
template <>
__device__ __forceinline__ void store4<double>(double* p, double a, double b, double c,
                                               double d) {
  *reinterpret_cast<double2*>(p) = make_double2(a, b);
  *reinterpret_cast<double2*>(p + 2) = make_double2(c, d);
}

// a / b: the fast reciprocal-multiply division in FP32 (2 ulp), IEEE in FP64
__device__ __forceinline__ float div_t(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double div_t(double a, double b) { return a / b; }

// Env row of one slot (env_mat.cc:122-226: s(r) [1/r, x/r^2, y/r^2, z/r^2]
// and its derivative wrt r_ij), normalised by the centre type's davg/dstd
// (prod_env_mat.cc:84-100), stored at row o; xj == nullptr: the padding row
// (0 - avg) / std; centre type < 0: zeros.  1/r and x/r^2 are formed from
// 1/sqrt(r^2) and the normalisation divides with div_t (within two ulp of
// the reference's divisions in FP32); the derivative row is formed only when
// em_deriv is requested.
template <typename T>
__device__ __forceinline__ void env_row_store(const T* xj, T xi, T yi, T zi, int ti,
                                              const T* av, const T* sd, int s, T rmin, T rmax,
                                              size_t o, T* em, T* em_deriv, T* rij) {
  T e[4] = {T(0), T(0), T(0), T(0)};
  T rr[3] = {T(0), T(0), T(0)};
  T inr = T(0), inr2 = T(0), sw = T(0), dsw = T(0);
  if (xj) {
    rr[0] = xj[0] - xi;
    rr[1] = xj[1] - yi;
    rr[2] = xj[2] - zi;
    const T nr2 = rr[0] * rr[0] + rr[1] * rr[1] + rr[2] * rr[2];
    inr = T(1) / sqrt(nr2);
    const T nr = nr2 * inr;
    inr2 = inr * inr;
    spline5<T>(sw, dsw, nr, rmin, rmax);
    e[0] = inr;
    e[1] = rr[0] * inr2;
    e[2] = rr[1] * inr2;
    e[3] = rr[2] * inr2;
  }
  T out[4];
  if (ti >= 0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) out[q] = div_t(e[q] * sw - av[s * 4 + q], sd[s * 4 + q]);
  } else {
#pragma unroll
    for (int q = 0; q < 4; ++q) out[q] = T(0);
  }
  store4<T>(em + o * 4, out[0], out[1], out[2], out[3]);
  if (em_deriv) {
    T dv[12];
#pragma unroll
    for (int q = 0; q < 12; ++q) dv[q] = T(0);
    if (xj) {
      const T inr4 = inr2 * inr2;
      const T inr3 = inr2 * inr;
#pragma unroll
      for (int d = 0; d < 3; ++d) dv[d] = rr[d] * inr3 * sw - e[0] * dsw * rr[d] * inr;
#pragma unroll
      for (int a2 = 0; a2 < 3; ++a2)
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          T t = T(2) * rr[a2] * rr[d] * inr4;
          if (a2 == d) t -= inr2;
          dv[3 + a2 * 3 + d] = t * sw - e[1 + a2] * dsw * rr[d] * inr;
        }
    }
    T* dp = em_deriv + o * 12;
#pragma unroll
    for (int q = 0; q < 12; q += 4) {
      if (ti >= 0)
        store4<T>(dp + q, div_t(dv[q], sd[s * 4 + q / 3]), div_t(dv[q + 1], sd[s * 4 + (q + 1) / 3]),
                  div_t(dv[q + 2], sd[s * 4 + (q + 2) / 3]),
                  div_t(dv[q + 3], sd[s * 4 + (q + 3) / 3]));
      else
        store4<T>(dp + q, T(0), T(0), T(0), T(0));
    }
  }
  if (rij) {
    rij[o * 3] = rr[0];
    rij[o * 3 + 1] = rr[1];
    rij[o * 3 + 2] = rr[2];
  }
}

// Ascending bitonic sort of 32 E 64-bit keys held by a warp, element
// e * 32 + lane in v[e]: partners closer than 32 are in other lanes
// (shuffles), farther ones in the same lane (register swaps).
__device__ __forceinline__ uint64_t shfl_xor64(uint64_t x, int m) {
  const uint32_t lo = __shfl_xor_sync(kFull, (uint32_t)x, m);
  const uint32_t hi = __shfl_xor_sync(kFull, (uint32_t)(x >> 32), m);
  return ((uint64_t)hi << 32) | lo;
}

template <int E>
__device__ __forceinline__ void warp_bitonic(uint64_t* v, int lane) {
#pragma unroll
  for (int k = 2; k <= 32 * E; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      if (j >= 32) {
        const int je = j >> 5;
#pragma unroll
        for (int e = 0; e < E; ++e) {
          if (e & je) continue;
          const int i = e * 32 + lane;
          const bool asc = (i & k) == 0;
          const uint64_t a = v[e], b = v[e ^ je];
          if ((a > b) == asc) {
            v[e] = b;
            v[e ^ je] = a;
          }
        }
      } else {
#pragma unroll
        for (int e = 0; e < E; ++e) {
          const int i = e * 32 + lane;
          const bool asc = (i & k) == 0;
          const bool lower = (lane & j) == 0;
          const uint64_t o = shfl_xor64(v[e], j);
          const uint64_t mn = o < v[e] ? o : v[e], mx = o < v[e] ? v[e] : o;
          v[e] = (asc == lower) ? mn : mx;
        }
      }
    }
  }
}

// One type's candidates (n <= 32 E keys (r^2, index) at stage[0, n)) sorted
// by a warp and the first sel of them placed at their ranks in row[].
template <int E>
__device__ __forceinline__ void sort_type_rows(const uint64_t* stage, int n, int sel, int* row,
                                               int lane) {
  uint64_t v[E];
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int c = e * 32 + lane;
    v[e] = c < n ? stage[c] : ~0ull;
  }
  warp_bitonic<E>(v, lane);
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int pos = e * 32 + lane;
    if (pos < n && pos < sel) row[pos] = (int)(uint32_t)(v[e] & 0xffffffffu);
  }
}

// Verlet list of a skin build: per centre up to `cap` frame-local extended
// indices (every extended atom within rcut + skin at the last rebuild, in
// stencil order), their count, and the extended types.
struct VList {
  int* idx;    // [nloc_total, cap]
  int* cnt;    // [nloc_total]
  int cap;
  const int* ext_type;
};

// Modes of k_nlist_env:
//   kEnvCells  candidates from the cell stencil, formatted list + env rows
//   kEnvList   candidates from the Verlet list, formatted list + env rows
//   kEnvBuild  candidates from the cell stencil (rc2f = (rcut + skin)^2)
//              written to the Verlet list; nothing else
enum { kEnvCells = 0, kEnvList = 1, kEnvBuild = 2 };

template <typename T, int MODE>
__global__ void __launch_bounds__(kEnvWarps * 32)
    k_nlist_env(int nloc_total, const gbdp_nbr_frame* __restrict__ fr,
                const int* __restrict__ atom_frame, const int* __restrict__ atom_cell,
                const int* __restrict__ atom_sub, const int* __restrict__ ext_sub,
                const typename XsOf<T>::type* __restrict__ xs, const T* __restrict__ ext_coord,
                const int* __restrict__ ext_map, const int* __restrict__ atype,
                const T* __restrict__ avg, const T* __restrict__ stdv, SecInfo si, float rc2f,
                T rmin, T rmax, int max_cand, T* __restrict__ em, T* __restrict__ em_deriv,
                T* __restrict__ rij, int* __restrict__ nlist, int* __restrict__ nlist_ext,
                int* __restrict__ status, VList vl) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * kEnvWarps + warp;
  if (i >= nloc_total) return;
  const int nnei = si.nnei;
  uint64_t* keys = reinterpret_cast<uint64_t*>(smem) + (size_t)warp * max_cand;
  int* row = reinterpret_cast<int*>(smem + (size_t)kEnvWarps * max_cand * 8) +
             (size_t)warp * ((nnei + 3) & ~3);
  unsigned char* ctype = smem + (size_t)kEnvWarps * max_cand * 8 +
                         (size_t)kEnvWarps * ((nnei + 3) & ~3) * 4 + (size_t)warp * max_cand;

  const gbdp_nbr_frame& g = fr[atom_frame[i]];
  const int il = i - g.atom_off;
  const size_t eoff = g.ext_off;
  const T xi = ext_coord[3 * (eoff + il)], yi = ext_coord[3 * (eoff + il) + 1],
          zi = ext_coord[3 * (eoff + il) + 2];
  const int ti = atype[i];
  // (the list mode reads no cell data: its launches pass no cell arrays)
  const int c = MODE == kEnvList ? 0 : atom_cell[i] - g.cell_off;
  const int c0 = c / (g.ncell[1] * g.ncell[2]);
  const int c1 = (c / g.ncell[2]) % g.ncell[1];
  const int c2 = c % g.ncell[2];
  const int n1 = g.ncell[1] + 2 * g.ngcell[1], n2 = g.ncell[2] + 2 * g.ngcell[2];

  // ---- gather candidates from the stencil of extended cells: one lane per
  //      stencil cell fetches its (start, count) in a single round trip, a
  //      warp scan makes the cells one flat candidate range, and every pass
  //      tests 32 candidates across cell boundaries (the owning cell found by
  //      a binary search over the scan with shuffles)
  int ncand = 0;
  if (MODE == kEnvList) {
    // ---- the Verlet list's entries, 32 per pass, with the current
    //      coordinates (refreshed from the local atoms since the rebuild)
    const int* L = vl.idx + (size_t)i * vl.cap;
    const int nl_i = min(vl.cnt[i], vl.cap);
    for (int base = 0; base < nl_i; base += 32) {
      const int f = base + lane;
      bool ok = false;
      uint64_t key = 0;
      int t = 0;
      if (f < nl_i) {
        const int idx = L[f];
        const size_t ej = eoff + idx;
        t = vl.ext_type[ej];
        const auto r = make_xs(ext_coord[3 * ej], ext_coord[3 * ej + 1], ext_coord[3 * ej + 2],
                               pack_idx_type(idx, t));
        float k2;
        ok = cand_test<T>(r, xi, yi, zi, rc2f, k2) && idx != il && t >= 0 && t < si.ntypes;
        key = ((uint64_t)__float_as_uint(k2) << 32) | (uint32_t)idx;
      }
      const unsigned m = __ballot_sync(kFull, ok);
      const int pos = ncand + __popc(m & ((1u << lane) - 1u));
      if (ok && pos < max_cand) {
        keys[pos] = key;
        ctype[pos] = (unsigned char)t;
      }
      ncand += __popc(m);
    }
  }
  // the search grid: along a split dimension d the extended cells are
  // halved (fine index F = 2 cell + half) and the stencil reaches two half
  // cells either way; otherwise it is the extended cells themselves
  int fs[3], hw[3], F[3];
  {
    const int cc[3] = {c0, c1, c2};
    const int hs = MODE == kEnvList ? 0 : atom_sub[i];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const bool split = (g.subcell >> d) & 1;
      fs[d] = split ? 2 : 1;
      hw[d] = split ? 2 : g.stencil[d];
      F[d] = fs[d] * (cc[d] + g.ngcell[d]) + (split ? (hs >> d) & 1 : 0);
    }
  }
  const int sy = 2 * hw[1] + 1, sz = 2 * hw[2] + 1;
  const int nst = MODE == kEnvList ? 0 : (2 * hw[0] + 1) * sy * sz;
  // stencil offsets from the flat index by reciprocal multiplies instead of
  // integer divisions: floor((q + 1/2) / d) from FP32 is exact while
  // q + 1/2 < 2^22 (the product's relative error, 2^-23, stays below the
  // 1/(2d) gap to the nearest integer), and nst is a few hundred
  const float inv_z = 1.f / (float)sz, inv_yz = 1.f / (float)(sy * sz);
  int* vrow = MODE == kEnvBuild ? vl.idx + (size_t)i * vl.cap : nullptr;
  for (int cg = 0; cg < nst; cg += 32) {
    const int q = cg + lane;
    int st = 0, cnt = 0;
    if (q < nst) {
      const int q0 = (int)(((float)q + 0.5f) * inv_yz), rq = q - q0 * sy * sz;
      const int q1 = (int)(((float)rq + 0.5f) * inv_z), q2 = rq - q1 * sz;
      const int o[3] = {q0 - hw[0], q1 - hw[1], q2 - hw[2]};
      int E[3], h = 0;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const int fp = F[d] + o[d];  // >= 0: the ghost layers cover the stencil
        E[d] = fs[d] == 2 ? fp >> 1 : fp;
        if (fs[d] == 2) h |= (fp & 1) << d;
      }
      const int* es = ext_sub + 9 * (size_t)(g.ext_cell_off + (E[0] * n1 + E[1]) * n2 + E[2]);
      st = es[h];
      cnt = es[h + 1] - st;
    }
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += y;
    }
    const int total = __shfl_sync(kFull, incl, 31);
    const int excl = incl - cnt;
    for (int base = 0; base < total; base += 32) {
      const int f = base + lane;
      int L = 0;  // lanes whose cells end at or before f: the owner of f
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const int v = __shfl_sync(kFull, incl, L + step - 1);
        if (v <= f) L += step;
      }
      L = min(L, 31);
      const int stL = __shfl_sync(kFull, st, L), exL = __shfl_sync(kFull, excl, L);
      bool ok = false;
      uint64_t key = 0;
      int t = 0;
      if (f < total) {
        const auto r = xs[stL + (f - exL)];
        const int pk = xs_packed(r);
        const int idx = pk & 0xffffff;
        t = (int)((unsigned)pk >> 24);
        float k2;
        ok = cand_test<T>(r, xi, yi, zi, rc2f, k2) && idx != il && t != 0xff && t < si.ntypes;
        key = ((uint64_t)__float_as_uint(k2) << 32) | (uint32_t)idx;
      }
      const unsigned m = __ballot_sync(kFull, ok);
      const int pos = ncand + __popc(m & ((1u << lane) - 1u));
      if (MODE == kEnvBuild) {
        if (ok && pos < vl.cap) vrow[pos] = (int)(uint32_t)(key & 0xffffffffu);
      } else if (ok && pos < max_cand) {
        keys[pos] = key;
        ctype[pos] = (unsigned char)t;
      }
      ncand += __popc(m);
    }
  }
  if (MODE == kEnvBuild) {
    if (lane == 0) {
      vl.cnt[i] = ncand;
      if (ncand > vl.cap) raise_status(status, GBDP_STATUS_CAND_OVERFLOW);
    }
    return;
  }
  if (ncand > max_cand) {
    if (lane == 0) raise_status(status, GBDP_STATUS_CAND_OVERFLOW);
    ncand = max_cand;
  }
  for (int s = lane; s < nnei; s += 32) row[s] = -1;
  __syncwarp();
  if (ncand <= 128 && max_cand >= 256) {
    // ---- up to 128 candidates: each type's (r^2, index) keys compacted
    //      into a staging area past them (keys[128, 256)) and sorted on
    //      their own by the smallest bitonic network that holds them (32,
    //      64 or 128 keys): about half the compare-exchange steps of one
    //      128-key sort over all types on water (~30 O and ~60 H)
    uint64_t* stage = keys + 128;
    for (int t = 0; t < si.ntypes; ++t) {
      int n = 0;
      for (int c0 = 0; c0 < ncand; c0 += 32) {
        const int cc = c0 + lane;
        const bool is_t = cc < ncand && (int)ctype[cc] == t;
        const unsigned m = __ballot_sync(kFull, is_t);
        if (is_t) stage[n + __popc(m & ((1u << lane) - 1u))] = keys[cc];
        n += __popc(m);
      }
      __syncwarp();
      const int sel_t = si.sec[t + 1] - si.sec[t];
      int* rt = row + si.sec[t];
      if (n > 0 && sel_t > 0) {
        if (n <= 32)
          sort_type_rows<1>(stage, n, sel_t, rt, lane);
        else if (n <= 64)
          sort_type_rows<2>(stage, n, sel_t, rt, lane);
        else
          sort_type_rows<4>(stage, n, sel_t, rt, lane);
      }
      __syncwarp();  // the staging area is read before the next type refills it
    }
  } else if (ncand <= 128) {
    // ---- up to 128 candidates: a bitonic sort of (type, r^2, index) keys
    //      in registers; a candidate's rank in its type is its sorted
    //      position minus the number of candidates of lower types.
    uint64_t v[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int c = e * 32 + lane;
      v[e] = c < ncand ? ((uint64_t)ctype[c] << 56) | ((keys[c] >> 8) & 0x00ffffffff000000ull) |
                             (keys[c] & 0xffffffull)
                       : ~0ull;
    }
    warp_bitonic<4>(v, lane);
    int below = 0;  // candidates of types lower than the current one
    for (int t = 0; t < si.ntypes; ++t) {
      int cnt = 0;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const bool is_t = (int)(v[e] >> 56) == t;
        const int pos = e * 32 + lane - below;
        if (is_t && pos < si.sec[t + 1] - si.sec[t]) row[si.sec[t] + pos] = (int)(v[e] & 0xffffff);
        cnt += __popc(__ballot_sync(kFull, is_t));
      }
      below += cnt;
    }
  } else {
  // ---- rank inside each type: position = number of same-type candidates
  //      with a smaller (r^2, index) key.  Each lane holds up to four of its
  //      candidates in registers and every key is read once per warp (a
  //      broadcast), instead of once per candidate.
  for (int base = 0; base < ncand; base += 128) {
    uint64_t mk[4];
    int mt[4], rank[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int c = base + e * 32 + lane;
      mk[e] = c < ncand ? keys[c] : ~0ull;
      mt[e] = c < ncand ? (int)ctype[c] : -1;
      rank[e] = 0;
    }
    for (int d = 0; d < ncand; ++d) {
      const uint64_t kd = keys[d];
      const int td = ctype[d];
#pragma unroll
      for (int e = 0; e < 4; ++e) rank[e] += (td == mt[e]) & (kd < mk[e]);
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int t = mt[e];
      if (t >= 0 && rank[e] < si.sec[t + 1] - si.sec[t])
        row[si.sec[t] + rank[e]] = (int)(uint32_t)(mk[e] & 0xffffffffu);
    }
  }
  }
  __syncwarp();

  // ---- env matrix rows
  const int nem = nnei * 4;
  const T* av = avg + (size_t)max(ti, 0) * nem;
  const T* sd = stdv + (size_t)max(ti, 0) * nem;
  for (int s = lane; s < nnei; s += 32) {
    const int j = row[s];
    const size_t o = ((size_t)i * nnei + s);
    env_row_store<T>(j >= 0 ? ext_coord + 3 * (eoff + j) : nullptr, xi, yi, zi, ti, av, sd, s,
                     rmin, rmax, o, em, em_deriv, rij);
    nlist[o] = j >= 0 ? ext_map[eoff + j] : -1;
    if (nlist_ext) nlist_ext[o] = j;
  }
}

// ------------------------------------------------------ k_nlist_env_ext --
// The neighbour list of the PyTorch forward_lower path, formatted from an
// external candidate list (an MD engine's rcut + skin list, unsorted) as
// deepmd/pt/model/model/make_model.py:541-598 (_format_nlist with the forced
// sort a compressed se_e2_a asks for) and deepmd/pt/utils/nlist.py:304-337
// (nlist_distinguish_types) do: rr = |x_i - x_j| in the coordinate type,
// rr > rcut dropped, ascending rr (ties by list position), the nearest nnei
// kept, then the first sel[t] of each type in that order.  One warp per
// centre; env rows as k_nlist_env.  Indices stay in the extended space.
template <typename T>
__device__ __forceinline__ T dist_rn(T dx, T dy, T dz);
template <>
__device__ __forceinline__ float dist_rn<float>(float dx, float dy, float dz) {
  return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
}
template <>
__device__ __forceinline__ double dist_rn<double>(double dx, double dy, double dz) {
  return __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
}

template <typename T>
__global__ void __launch_bounds__(kEnvWarps * 32)
    k_nlist_env_ext(int nloc, int nall, int nnei_in, int nwork, const T* __restrict__ ext_coord,
                    const int* __restrict__ ext_type, const int* __restrict__ nlist_in,
                    const T* __restrict__ avg, const T* __restrict__ stdv, SecInfo si, T rcut,
                    T rmin, T rmax, T* __restrict__ em, T* __restrict__ em_deriv,
                    T* __restrict__ rij, int* __restrict__ nlist, int* __restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * kEnvWarps + warp;
  if (i >= nwork) return;
  const int nnei = si.nnei;
  const int cap = (nnei_in + 7) & ~7;
  // per warp: rr [cap] (T), slot row [nnei] (int), type [cap], kept [cap]
  const size_t per_warp = (size_t)cap * sizeof(T) + (size_t)((nnei + 3) & ~3) * 4 + 2 * (size_t)cap;
  unsigned char* base = smem + (size_t)warp * ((per_warp + 15) & ~(size_t)15);
  T* rr = reinterpret_cast<T*>(base);
  int* row = reinterpret_cast<int*>(base + (size_t)cap * sizeof(T));
  unsigned char* ctype = base + (size_t)cap * sizeof(T) + (size_t)((nnei + 3) & ~3) * 4;
  unsigned char* kept = ctype + cap;
  const int f = i / nloc, il = i - f * nloc;
  const T* xf = ext_coord + (size_t)f * nall * 3;
  const int* tf = ext_type + (size_t)f * nall;
  const int* nl = nlist_in + (size_t)i * nnei_in;
  const T xi = xf[3 * il], yi = xf[3 * il + 1], zi = xf[3 * il + 2];
  const int ti = tf[il];
  const T inf = T(1) / T(0);
  for (int p = lane; p < nnei_in; p += 32) {
    const int j = nl[p];
    T d = inf;
    int t = 0xff;
    if (j >= nall) {
      raise_status(status, GBDP_STATUS_BAD_INDEX);
    } else if (j >= 0) {
      d = dist_rn<T>(xi - xf[3 * j], yi - xf[3 * j + 1], zi - xf[3 * j + 2]);
      if (d > rcut) d = inf;  // dropped, as rr > rcut
      const int tj = tf[j];
      t = (tj >= 0 && tj < si.ntypes) ? tj : 0xfe;  // 0xfe: counted, never placed
    }
    rr[p] = d;
    ctype[p] = (unsigned char)t;
  }
  for (int s = lane; s < nnei; s += 32) row[s] = -1;
  __syncwarp();
  // nearest nnei over all types: rank by (rr, list position)
  for (int p = lane; p < nnei_in; p += 32) {
    const T d = rr[p];
    int rank = 0;
    if (d != inf)
      for (int q = 0; q < nnei_in; ++q) {
        const T e = rr[q];
        rank += (e < d) | ((e == d) & (q < p));
      }
    kept[p] = (d != inf && rank < nnei) ? 1 : 0;
  }
  __syncwarp();
  // section t: the first sel[t] kept neighbours of type t, in the same order
  for (int p = lane; p < nnei_in; p += 32) {
    if (!kept[p]) continue;
    const int t = ctype[p];
    if (t >= si.ntypes) continue;
    const T d = rr[p];
    int rank = 0;
    for (int q = 0; q < nnei_in; ++q) {
      const T e = rr[q];
      rank += kept[q] & (ctype[q] == t) & ((e < d) | ((e == d) & (q < p)));
    }
    if (rank < si.sec[t + 1] - si.sec[t]) row[si.sec[t] + rank] = nl[p];
  }
  __syncwarp();
  const int nem = nnei * 4;
  const T* av = avg + (size_t)max(ti, 0) * nem;
  const T* sd = stdv + (size_t)max(ti, 0) * nem;
  for (int s = lane; s < nnei; s += 32) {
    const int j = row[s];
    const size_t o = ((size_t)i * nnei + s);
    env_row_store<T>(j >= 0 ? xf + 3 * j : nullptr, xi, yi, zi, ti, av, sd, s, rmin, rmax, o, em,
                     em_deriv, rij);
    nlist[o] = j;
  }
}

// ------------------------------------------------------------ host side --
size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

struct EnvWs {
  int* status;
  int* atom_frame;
  int* atom_cell;
  int* cell_count;
  int* cell_fill;
  int* cell_start;
  int* bucket;
  int* cell_atoms;
  int* ext_start;
  int* ext_cnt;
  int* ghost_start;
  int* sub_count;  // [ncell_total][8] atoms per half cell of each local cell
  int* atom_sub;   // [nloc_total] half cell of each local atom (bit d: upper half)
  int* atom_xpos;  // [nloc_total] position of the atom in its cell's xs range
  int* ext_sub;    // [next_cell_total][9] xs start of each half cell, then the end
  void* xs;
  size_t zero_bytes;  // status .. sub_count: zeroed before every build
  size_t bytes;
};

EnvWs carve(const gbdp_nbr_plan& p, void* base, int fp64) {
  EnvWs w;
  char* b = static_cast<char*>(base);
  size_t off = 0;
  auto take = [&](size_t n) {
    char* r = b ? b + off : nullptr;
    off += align256(n);
    return r;
  };
  // status, cell_count, cell_fill and sub_count first and adjacent: one
  // zero fill
  w.status = reinterpret_cast<int*>(take(256));
  w.cell_count = reinterpret_cast<int*>(take(sizeof(int) * p.ncell_total));
  w.cell_fill = reinterpret_cast<int*>(take(sizeof(int) * p.ncell_total));
  w.sub_count = reinterpret_cast<int*>(take(sizeof(int) * 8 * (size_t)p.ncell_total));
  w.zero_bytes = off;
  w.atom_sub = reinterpret_cast<int*>(take(sizeof(int) * p.nloc_total));
  w.atom_xpos = reinterpret_cast<int*>(take(sizeof(int) * p.nloc_total));
  w.ext_sub = reinterpret_cast<int*>(take(sizeof(int) * 9 * (size_t)p.next_cell_total));
  w.atom_frame = reinterpret_cast<int*>(take(sizeof(int) * p.nloc_total));
  w.atom_cell = reinterpret_cast<int*>(take(sizeof(int) * p.nloc_total));
  w.cell_start = reinterpret_cast<int*>(take(sizeof(int) * p.ncell_total));
  w.bucket = reinterpret_cast<int*>(take(sizeof(int) * p.nloc_total));
  w.cell_atoms = reinterpret_cast<int*>(take(sizeof(int) * p.nloc_total));
  w.ext_start = reinterpret_cast<int*>(take(sizeof(int) * p.next_cell_total));
  w.ext_cnt = reinterpret_cast<int*>(take(sizeof(int) * p.next_cell_total));
  w.ghost_start = reinterpret_cast<int*>(take(sizeof(int) * p.next_cell_total));
  w.xs = take((fp64 ? 32 : 16) * (size_t)p.ext_total);
  w.bytes = off;
  return w;
}

// Shared-memory bytes of k_nlist_env: per warp the candidate keys and the
// formatted row.
inline size_t nlist_env_smem(int max_cand, int nnei) {
  return (size_t)kEnvWarps * max_cand * 9 + (size_t)kEnvWarps * ((nnei + 3) & ~3) * 4;
}

// Every argument check of the periodic env-mat pipeline that needs no
// workspace: run before any device work (the allocation-free entry point
// calls it before it copies its frame table).  Fills the section table.
template <typename T>
int env_check_args(const T* em, const T* em_deriv, const int* nlist, const T* ext_coord,
                   const int* ext_type, const int* ext_map, const int* ext_nall, const T* coord,
                   const int* atype, const T* avg, const T* stdv, const gbdp_nbr_plan* plan,
                   const int* sel, int ntypes, SecInfo* si) {
  GBDP_REQUIRE(plan, "prod_env_mat_a: null plan");
  GBDP_REQUIRE(ntypes >= 1 && ntypes <= kMaxTypes, "prod_env_mat_a: ntypes %d out of [1,%d]",
               ntypes, kMaxTypes);
  GBDP_REQUIRE(em && nlist && ext_coord && ext_type && ext_map && ext_nall && coord && atype &&
                   avg && stdv && sel,
               "prod_env_mat_a: null required pointer");
  GBDP_REQUIRE(((uintptr_t)em & 15) == 0 && (!em_deriv || ((uintptr_t)em_deriv & 15) == 0),
               "prod_env_mat_a: em / em_deriv must be 16-byte aligned");
  si->ntypes = ntypes;
  si->sec[0] = 0;
  for (int t = 0; t < ntypes; ++t) {
    GBDP_REQUIRE(sel[t] >= 0, "prod_env_mat_a: negative sel");
    si->sec[t + 1] = si->sec[t] + sel[t];
  }
  si->nnei = si->sec[ntypes];
  GBDP_REQUIRE(si->nnei > 0, "prod_env_mat_a: sum(sel) must be positive");
  GBDP_REQUIRE(nlist_env_smem(plan->max_cand, si->nnei) <= 200 * 1024,
               "prod_env_mat_a: max_cand %d needs too much shared memory", plan->max_cand);
  return GBDP_OK;
}

// The cell build and ghost images of the periodic pipeline (k_localize ..
// k_ghost_fill); clears the status word and the cell counters first.
template <typename T>
void env_ghosts(const EnvWs& w, T* ext_coord, int* ext_type, int* ext_map, int* ext_nall,
                const T* coord, const int* atype, const gbdp_nbr_plan* plan,
                const gbdp_nbr_frame* frames, cudaStream_t stream) {
  const int nl = plan->nloc_total;
  cudaMemsetAsync(w.status, 0, w.zero_bytes, stream);
  const int tb = 256;
  k_localize<T><<<(nl + tb - 1) / tb, tb, 0, stream>>>(frames, plan->nframes, nl, coord, atype,
                                                       ext_coord, ext_type, ext_map,
                                                       w.atom_frame, w.atom_cell, w.cell_count,
                                                       w.sub_count, w.atom_sub);
  k_cell_scan<<<plan->nframes, 1024, 0, stream>>>(frames, w.cell_count, w.cell_start,
                                                  w.ext_start, w.ext_cnt, w.ghost_start,
                                                  ext_nall, w.status, w.sub_count, w.ext_sub);
  k_cell_bucket<<<(nl + tb - 1) / tb, tb, 0, stream>>>(nl, frames, w.atom_frame, w.atom_cell,
                                                       w.cell_start, w.cell_fill, w.bucket);
  k_cell_rank<<<(nl + tb - 1) / tb, tb, 0, stream>>>(nl, frames, w.atom_frame, w.atom_cell,
                                                     w.cell_start, w.cell_count, w.bucket,
                                                     w.cell_atoms, w.atom_sub, w.atom_xpos);
  const int nec = plan->next_cell_total;
  k_ghost_fill<T><<<(nec * 32 + tb - 1) / tb, tb, 0, stream>>>(
      frames, plan->nframes, nec, w.cell_start, w.cell_count, w.cell_atoms, w.ext_start,
      w.ghost_start, ext_coord, ext_type, ext_map,
      static_cast<typename XsOf<T>::type*>(w.xs), w.atom_xpos);
}

// One launch of k_nlist_env in the given mode (candidates within rc).
template <typename T, int MODE>
void nlist_env_mode(const EnvWs& w, const gbdp_nbr_plan* plan, const gbdp_nbr_frame* frames,
                    const SecInfo& si, float rc, float rcut_smth, float rmax, T* em, T* em_deriv,
                    T* rij, int* nlist, int* nlist_ext, const T* ext_coord, const int* ext_map,
                    const int* atype, const T* avg, const T* stdv, const VList& vl,
                    cudaStream_t stream) {
  const int nl = plan->nloc_total;
  const int mc = plan->max_cand;
  const size_t smem = MODE == kEnvBuild ? 0 : nlist_env_smem(mc, si.nnei);
  auto kern = k_nlist_env<T, MODE>;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const bool cells = MODE != kEnvList;
  kern<<<(nl + kEnvWarps - 1) / kEnvWarps, kEnvWarps * 32, smem, stream>>>(
      nl, frames, w.atom_frame, cells ? w.atom_cell : nullptr, cells ? w.atom_sub : nullptr,
      cells ? w.ext_sub : nullptr,
      cells ? static_cast<const typename XsOf<T>::type*>(w.xs) : nullptr, ext_coord, ext_map,
      atype, avg, stdv, si, rc * rc, (T)rcut_smth, (T)rmax, mc, em, em_deriv, rij, nlist,
      nlist_ext, w.status, vl);
}

template <typename T>
int env_launch(T* em, T* em_deriv, T* rij, int* nlist, int* nlist_ext, T* ext_coord,
               int* ext_type, int* ext_map, int* ext_nall, const T* coord, const int* atype,
               const T* avg, const T* stdv, const gbdp_nbr_plan* plan,
               const gbdp_nbr_frame* frames, float rcut_smth, const int* sel, int ntypes,
               void* workspace, size_t ws_bytes, cudaStream_t stream) {
  GBDP_REQUIRE(plan && frames && workspace, "prod_env_mat_a: null plan/frames/workspace");
  SecInfo si;
  const int chk = env_check_args<T>(em, em_deriv, nlist, ext_coord, ext_type, ext_map, ext_nall,
                                    coord, atype, avg, stdv, plan, sel, ntypes, &si);
  if (chk) return chk;
  const int fp64 = sizeof(T) == 8;
  EnvWs w = carve(*plan, workspace, fp64);
  GBDP_REQUIRE(ws_bytes >= w.bytes, "prod_env_mat_a: workspace %zu < %zu bytes", ws_bytes,
               w.bytes);
  if (plan->nloc_total == 0) return GBDP_OK;
  env_ghosts<T>(w, ext_coord, ext_type, ext_map, ext_nall, coord, atype, plan, frames, stream);
  nlist_env_mode<T, kEnvCells>(w, plan, frames, si, plan->rcut, rcut_smth, plan->rcut, em,
                               em_deriv, rij, nlist, nlist_ext, ext_coord, ext_map, atype, avg,
                               stdv, VList{nullptr, nullptr, 0, nullptr}, stream);
  GBDP_CHECK_LAUNCH("prod_env_mat_a");
  return GBDP_OK;
}

// ------------------------------------------------------- Verlet (skin) list --
__device__ __forceinline__ int find_frame_ext(const gbdp_nbr_frame* fr, int nframes, int e) {
  int lo = 0, hi = nframes - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (fr[mid].ext_off <= e)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// At a rebuild: the source local atom (packed index) of every filled
// extended slot, and the shift from that atom's input coordinate to the
// slot's coordinate (the wrap into the box, plus the image vector of a
// ghost); unfilled slots get source -1.
template <typename T>
__global__ void k_ext_shift(const gbdp_nbr_frame* __restrict__ fr, int nframes, int ext_total,
                            const int* __restrict__ ext_nall, const int* __restrict__ ext_map,
                            const T* __restrict__ coord, const T* __restrict__ ext_coord,
                            T* __restrict__ shift, int* __restrict__ src) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ext_total) return;
  const int f = find_frame_ext(fr, nframes, e);
  const gbdp_nbr_frame& g = fr[f];
  const int el = e - g.ext_off;
  if (el >= ext_nall[f] || el >= g.ext_cap) {
    src[e] = -1;
    return;
  }
  const int a = g.atom_off + ext_map[e];
  src[e] = a;
#pragma unroll
  for (int d = 0; d < 3; ++d) shift[3 * (size_t)e + d] = ext_coord[3 * (size_t)e + d] - coord[3 * (size_t)a + d];
}

// Between rebuilds: every filled extended slot follows its source atom.
template <typename T>
__global__ void k_ext_refresh(int ext_total, const int* __restrict__ src,
                              const T* __restrict__ shift, const T* __restrict__ coord,
                              T* __restrict__ ext_coord) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ext_total) return;
  const int a = src[e];
  if (a < 0) return;
#pragma unroll
  for (int d = 0; d < 3; ++d)
    ext_coord[3 * (size_t)e + d] = coord[3 * (size_t)a + d] + shift[3 * (size_t)e + d];
}

template <typename T>
int env_skin_launch(T* em, T* em_deriv, T* rij, int* nlist, int* nlist_ext, T* ext_coord,
                    int* ext_type, int* ext_map, int* ext_nall, const T* coord, const int* atype,
                    const T* avg, const T* stdv, const gbdp_nbr_plan* plan,
                    const gbdp_nbr_frame* frames, float rcut, float rcut_smth, const int* sel,
                    int ntypes, int rebuild, int* vlist, int* vcnt, int vcap, T* ext_shift,
                    int* ext_src, void* workspace, size_t ws_bytes, cudaStream_t stream) {
  GBDP_REQUIRE(plan && frames && workspace, "prod_env_mat_a_skin: null plan/frames/workspace");
  SecInfo si;
  const int chk = env_check_args<T>(em, em_deriv, nlist, ext_coord, ext_type, ext_map, ext_nall,
                                    coord, atype, avg, stdv, plan, sel, ntypes, &si);
  if (chk) return chk;
  GBDP_REQUIRE(vlist && vcnt && ext_shift && ext_src && vcap >= 1,
               "prod_env_mat_a_skin: null Verlet-list buffer or capacity < 1");
  GBDP_REQUIRE(rcut > 0.f && rcut <= plan->rcut,
               "prod_env_mat_a_skin: rcut %g must be positive and at most the plan's %g", rcut,
               plan->rcut);
  const int fp64 = sizeof(T) == 8;
  EnvWs w = carve(*plan, workspace, fp64);
  GBDP_REQUIRE(ws_bytes >= w.bytes, "prod_env_mat_a_skin: workspace %zu < %zu bytes", ws_bytes,
               w.bytes);
  const int nl = plan->nloc_total;
  if (nl == 0) return GBDP_OK;
  const VList vl{vlist, vcnt, vcap, ext_type};
  const int ne = plan->ext_total;
  if (rebuild) {
    env_ghosts<T>(w, ext_coord, ext_type, ext_map, ext_nall, coord, atype, plan, frames, stream);
    k_ext_shift<T><<<(ne + 255) / 256, 256, 0, stream>>>(frames, plan->nframes, ne, ext_nall,
                                                         ext_map, coord, ext_coord, ext_shift,
                                                         ext_src);
    nlist_env_mode<T, kEnvBuild>(w, plan, frames, si, plan->rcut, rcut_smth, rcut, em, em_deriv,
                                 rij, nlist, nlist_ext, ext_coord, ext_map, atype, avg, stdv, vl,
                                 stream);
  } else {
    cudaMemsetAsync(w.status, 0, sizeof(int), stream);
    k_ext_refresh<T><<<(ne + 255) / 256, 256, 0, stream>>>(ne, ext_src, ext_shift, coord,
                                                           ext_coord);
  }
  nlist_env_mode<T, kEnvList>(w, plan, frames, si, rcut, rcut_smth, rcut, em, em_deriv, rij,
                              nlist, nlist_ext, ext_coord, ext_map, atype, avg, stdv, vl, stream);
  GBDP_CHECK_LAUNCH("prod_env_mat_a_skin");
  return GBDP_OK;
}

template <typename T>
int env_nlist_launch(T* em, T* em_deriv, T* rij, int* nlist, int* status, const T* ext_coord,
                     const int* ext_type, const int* nlist_in, const T* avg, const T* stdv,
                     int nframes, int nloc, int nall, int nnei_in, float rcut, float rcut_smth,
                     const int* sel, int ntypes, cudaStream_t stream) {
  GBDP_REQUIRE(ntypes >= 1 && ntypes <= kMaxTypes, "prod_env_mat_a_nlist: ntypes %d out of [1,%d]",
               ntypes, kMaxTypes);
  GBDP_REQUIRE(nframes >= 0 && nloc >= 0 && nall >= nloc && nnei_in >= 0 && nnei_in <= 4096,
               "prod_env_mat_a_nlist: nframes %d nloc %d nall %d nnei_in %d", nframes, nloc, nall,
               nnei_in);
  GBDP_REQUIRE(sel != nullptr, "prod_env_mat_a_nlist: null sel");
  SecInfo si;
  si.ntypes = ntypes;
  si.sec[0] = 0;
  for (int t = 0; t < ntypes; ++t) {
    GBDP_REQUIRE(sel[t] >= 0, "prod_env_mat_a_nlist: negative sel");
    si.sec[t + 1] = si.sec[t] + sel[t];
  }
  si.nnei = si.sec[ntypes];
  GBDP_REQUIRE(si.nnei > 0, "prod_env_mat_a_nlist: sum(sel) must be positive");
  const long nwork = (long)nframes * nloc;
  if (nwork == 0) return GBDP_OK;
  GBDP_REQUIRE(nwork < (1l << 31), "prod_env_mat_a_nlist: too many centres");
  GBDP_REQUIRE(em && nlist && ext_coord && ext_type && (nlist_in || nnei_in == 0) && avg && stdv,
               "prod_env_mat_a_nlist: null required pointer");
  GBDP_REQUIRE(((uintptr_t)em & 15) == 0 && (!em_deriv || ((uintptr_t)em_deriv & 15) == 0),
               "prod_env_mat_a_nlist: em / em_deriv must be 16-byte aligned");
  if (status) cudaMemsetAsync(status, 0, sizeof(int), stream);
  const int cap = (nnei_in + 7) & ~7;
  const size_t per_warp = (size_t)cap * sizeof(T) + (size_t)((si.nnei + 3) & ~3) * 4 + 2 * (size_t)cap;
  const size_t smem = (size_t)kEnvWarps * ((per_warp + 15) & ~(size_t)15);
  GBDP_REQUIRE(smem <= 200 * 1024, "prod_env_mat_a_nlist: nnei_in %d needs too much shared memory",
               nnei_in);
  auto kern = k_nlist_env_ext<T>;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  kern<<<(unsigned)((nwork + kEnvWarps - 1) / kEnvWarps), kEnvWarps * 32, smem, stream>>>(
      nloc, nall, nnei_in, (int)nwork, ext_coord, ext_type, nlist_in, avg, stdv, si, (T)rcut,
      (T)rcut_smth, (T)rcut, em, em_deriv, rij, nlist, status);
  GBDP_CHECK_LAUNCH("prod_env_mat_a_nlist");
  return GBDP_OK;
}

// reference cell geometry (mirrors the oracle's cell_geom, which follows
// source/lib/src/neighbor_list.cc:745-775 and SimulationRegion_Impl.h:364-372)
void rec_box_d(double* r, const double* b) {
  double v = b[0] * (b[4] * b[8] - b[7] * b[5]) - b[1] * (b[3] * b[8] - b[6] * b[5]) +
             b[2] * (b[3] * b[7] - b[6] * b[4]);
  double vi = 1. / std::fabs(v);
  r[0] = (b[4] * b[8] - b[7] * b[5]) * vi;
  r[4] = (b[0] * b[8] - b[6] * b[2]) * vi;
  r[8] = (b[0] * b[4] - b[3] * b[1]) * vi;
  r[1] = (-b[3] * b[8] + b[6] * b[5]) * vi;
  r[2] = (b[3] * b[7] - b[6] * b[4]) * vi;
  r[3] = (-b[1] * b[8] + b[7] * b[2]) * vi;
  r[5] = (-b[0] * b[7] + b[6] * b[1]) * vi;
  r[6] = (b[1] * b[5] - b[4] * b[2]) * vi;
  r[7] = (-b[0] * b[5] + b[3] * b[2]) * vi;
}
void rec_box_f(float* r, const float* b) {
  float v = b[0] * (b[4] * b[8] - b[7] * b[5]) - b[1] * (b[3] * b[8] - b[6] * b[5]) +
            b[2] * (b[3] * b[7] - b[6] * b[4]);
  float vi = 1.f / std::fabs(v);
  r[0] = (b[4] * b[8] - b[7] * b[5]) * vi;
  r[4] = (b[0] * b[8] - b[6] * b[2]) * vi;
  r[8] = (b[0] * b[4] - b[3] * b[1]) * vi;
  r[1] = (-b[3] * b[8] + b[6] * b[5]) * vi;
  r[2] = (b[3] * b[7] - b[6] * b[4]) * vi;
  r[3] = (-b[1] * b[8] + b[7] * b[2]) * vi;
  r[5] = (-b[0] * b[7] + b[6] * b[1]) * vi;
  r[6] = (b[1] * b[5] - b[4] * b[2]) * vi;
  r[7] = (-b[0] * b[5] + b[3] * b[2]) * vi;
}

}  // namespace
}  // namespace gbdp

using namespace gbdp;

extern "C" int gbdp_nbr_plan_make(gbdp_nbr_plan* plan, gbdp_nbr_frame* frames, int nframes,
                                  const int* nloc, const double* boxes, float rcut,
                                  int max_cand) {
  GBDP_REQUIRE(plan && frames && nloc && boxes, "nbr_plan_make: null argument");
  GBDP_REQUIRE(nframes >= 1, "nbr_plan_make: nframes must be >= 1");
  GBDP_REQUIRE(rcut > 0.f, "nbr_plan_make: rcut must be positive");
  long atom_off = 0, cell_off = 0, ecell_off = 0, ext_off = 0;
  for (int f = 0; f < nframes; ++f) {
    gbdp_nbr_frame& g = frames[f];
    std::memset(&g, 0, sizeof(g));
    const double* b = boxes + 9 * (size_t)f;
    std::copy(b, b + 9, g.box);
    for (int k = 0; k < 9; ++k) g.boxf[k] = (float)b[k];
    double vol = std::fabs(b[0] * (b[4] * b[8] - b[7] * b[5]) - b[1] * (b[3] * b[8] - b[6] * b[5]) +
                           b[2] * (b[3] * b[7] - b[6] * b[4]));
    GBDP_REQUIRE(vol > 0, "nbr_plan_make: frame %d has a zero-volume box", f);
    rec_box_d(g.rec, g.box);
    rec_box_f(g.recf, g.boxf);
    const int pa[3] = {3, 6, 0}, pb[3] = {6, 0, 3};
    long mult = 1;
    for (int d = 0; d < 3; ++d) {
      const double* u = g.box + pa[d];
      const double* v = g.box + pb[d];
      double t0 = u[1] * v[2] - u[2] * v[1], t1 = u[2] * v[0] - u[0] * v[2],
             t2 = u[0] * v[1] - u[1] * v[0];
      double face = vol * (1. / std::sqrt(t0 * t0 + t1 * t1 + t2 * t2));
      int nc = (int)(face / (double)rcut);
      if (nc == 0) nc = 1;
      double cs = face / nc;
      g.ncell[d] = nc;
      g.ngcell[d] = (int)((double)rcut / cs) + 1;
      // cells at least 0.1 % wider than rcut are searched in halves: a pair
      // within rcut is then at most two half cells apart along d (with a
      // margin far above the coordinates' rounding)
      if (g.ngcell[d] == 1 && (double)rcut <= 0.999 * cs) g.subcell |= 1 << d;
      // every extended atom within rcut of a local atom lies within ngcell
      // cells of it (cell >= rcut, or ngcell covers rcut / cell)
      g.stencil[d] = g.ngcell[d];
      // a local cell index l is imaged by every extended index in
      // [-ngcell, nc + ngcell) congruent to it: at most ceil((nc+2ng)/nc)
      mult *= (nc + 2 * g.ngcell[d] + nc - 1) / nc;
    }
    g.nloc = nloc[f];
    GBDP_REQUIRE(g.nloc >= 0, "nbr_plan_make: negative nloc");
    g.atom_off = (int)atom_off;
    g.cell_off = (int)cell_off;
    g.ext_cell_off = (int)ecell_off;
    g.ext_off = (int)ext_off;
    long cap = (long)g.nloc * mult;
    GBDP_REQUIRE(cap < (1l << 24), "nbr_plan_make: frame %d needs %ld extended slots (max 2^24)",
                 f, cap);
    g.ext_cap = (int)cap;
    atom_off += g.nloc;
    cell_off += (long)g.ncell[0] * g.ncell[1] * g.ncell[2];
    ecell_off += (long)(g.ncell[0] + 2 * g.ngcell[0]) * (g.ncell[1] + 2 * g.ngcell[1]) *
                 (g.ncell[2] + 2 * g.ngcell[2]);
    ext_off += cap;
    GBDP_REQUIRE(ext_off < (1l << 31) && ecell_off < (1l << 31),
                 "nbr_plan_make: batch too large for 32-bit offsets");
  }
  plan->nframes = nframes;
  plan->nloc_total = (int)atom_off;
  plan->ncell_total = (int)cell_off;
  plan->next_cell_total = (int)ecell_off;
  plan->ext_total = (int)ext_off;
  plan->max_cand = max_cand > 0 ? max_cand : 512;
  plan->rcut = rcut;
  plan->pad0 = 0;
  return GBDP_OK;
}

extern "C" size_t gbdp_env_workspace_bytes(const gbdp_nbr_plan* plan, int fp64) {
  if (!plan) return 0;
  return carve(*plan, nullptr, fp64).bytes;
}

extern "C" int gbdp_env_status(const void* workspace, gbdp_stream stream) {
  int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, workspace, sizeof(int), cudaMemcpyDeviceToHost,
                                  (cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_status(e, "env_status");
  return h;
}

extern "C" int gbdp_prod_env_mat_a_f32(float* em, float* em_deriv, float* rij, int* nlist,
                                       int* nlist_ext, float* ext_coord, int* ext_type,
                                       int* ext_map, int* ext_nall, const float* coord,
                                       const int* atype, const float* avg, const float* std,
                                       const gbdp_nbr_plan* plan,
                                       const gbdp_nbr_frame* frames_dev, float rcut_smth,
                                       const int* sel, int ntypes, void* workspace,
                                       size_t workspace_bytes, gbdp_stream stream) {
  return env_launch<float>(em, em_deriv, rij, nlist, nlist_ext, ext_coord, ext_type, ext_map,
                           ext_nall, coord, atype, avg, std, plan, frames_dev, rcut_smth, sel,
                           ntypes, workspace, workspace_bytes, (cudaStream_t)stream);
}

extern "C" int gbdp_prod_env_mat_a_f64(double* em, double* em_deriv, double* rij, int* nlist,
                                       int* nlist_ext, double* ext_coord, int* ext_type,
                                       int* ext_map, int* ext_nall, const double* coord,
                                       const int* atype, const double* avg, const double* std,
                                       const gbdp_nbr_plan* plan,
                                       const gbdp_nbr_frame* frames_dev, float rcut_smth,
                                       const int* sel, int ntypes, void* workspace,
                                       size_t workspace_bytes, gbdp_stream stream) {
  return env_launch<double>(em, em_deriv, rij, nlist, nlist_ext, ext_coord, ext_type, ext_map,
                            ext_nall, coord, atype, avg, std, plan, frames_dev, rcut_smth, sel,
                            ntypes, workspace, workspace_bytes, (cudaStream_t)stream);
}

#define GBDP_ENV_SKIN_ENTRY(T, SFX)                                                             \
  extern "C" int gbdp_prod_env_mat_a_skin_##SFX(                                                \
      T* em, T* em_deriv, T* rij, int* nlist, int* nlist_ext, T* ext_coord, int* ext_type,       \
      int* ext_map, int* ext_nall, const T* coord, const int* atype, const T* avg, const T* std, \
      const gbdp_nbr_plan* plan, const gbdp_nbr_frame* frames_dev, float rcut, float rcut_smth, \
      const int* sel, int ntypes, int rebuild, int* vlist, int* vcnt, int vcap, T* ext_shift,    \
      int* ext_src, void* workspace, size_t workspace_bytes, gbdp_stream stream) {              \
    return env_skin_launch<T>(em, em_deriv, rij, nlist, nlist_ext, ext_coord, ext_type, ext_map, \
                              ext_nall, coord, atype, avg, std, plan, frames_dev, rcut,          \
                              rcut_smth, sel, ntypes, rebuild, vlist, vcnt, vcap, ext_shift,     \
                              ext_src, workspace, workspace_bytes, (cudaStream_t)stream);        \
  }
GBDP_ENV_SKIN_ENTRY(float, f32)
GBDP_ENV_SKIN_ENTRY(double, f64)
#undef GBDP_ENV_SKIN_ENTRY

#define GBDP_ENV_NLIST_ENTRY(T, SFX)                                                           \
  extern "C" int gbdp_prod_env_mat_a_nlist_##SFX(                                              \
      T* em, T* em_deriv, T* rij, int* nlist, int* status, const T* ext_coord,                 \
      const int* ext_type, const int* nlist_in, const T* avg, const T* std, int nframes,       \
      int nloc, int nall, int nnei_in, float rcut, float rcut_smth, const int* sel, int ntypes, \
      gbdp_stream stream) {                                                                    \
    return env_nlist_launch<T>(em, em_deriv, rij, nlist, status, ext_coord, ext_type, nlist_in, \
                               avg, std, nframes, nloc, nall, nnei_in, rcut, rcut_smth, sel,    \
                               ntypes, (cudaStream_t)stream);                                   \
  }
GBDP_ENV_NLIST_ENTRY(float, f32)
GBDP_ENV_NLIST_ENTRY(double, f64)
#undef GBDP_ENV_NLIST_ENTRY

// ------------------------------------------------ allocation-free variant --
// Scratch for gbdp_prod_env_mat_a_noalloc_f32: a file-scope device array, so
// callers that must not allocate device memory can still run the periodic
// neighbour build.  Every GPU that loads the library holds it until exit.
// The last kNoAllocFrameBytes hold the copied frame table.
namespace {
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;  // 16 MiB
constexpr size_t kNoAllocFrameBytes = size_t(64) << 10;    // 64 KiB
// frame records the table holds: 65536 / 280 = 234
constexpr int kNoAllocMaxFrames = (int)(kNoAllocFrameBytes / sizeof(gbdp_nbr_frame));
static_assert(sizeof(gbdp_nbr_frame) == 280, "gbdp_nbr_frame layout changed: update the "
              "documented frame limit of the allocation-free entry point");
static_assert(kNoAllocMaxFrames == 234, "documented frame limit of the allocation-free entry");
constexpr int kNoAllocMaxDevices = 64;
}  // namespace

static __device__ __align__(256) unsigned char g_env_noalloc_scratch[kNoAllocScratchBytes];

namespace {
std::mutex g_noalloc_mu;
void* g_noalloc_addr[kNoAllocMaxDevices] = {};

// Device address of the scratch array for the current device.  In host code
// the array's name is only a host-side stand-in, so the address is looked up
// with the device current: again on every call made outside stream capture
// (so that a context created after cudaDeviceReset gets its own address),
// and from the per-device cache while `stream` is capturing.
int noalloc_scratch_address(cudaStream_t stream, void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "prod_env_mat_a_noalloc: cudaGetDevice");
  GBDP_REQUIRE(dev >= 0 && dev < kNoAllocMaxDevices,
               "prod_env_mat_a_noalloc: device ordinal %d above %d", dev, kNoAllocMaxDevices - 1);
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(stream, &cap);
  if (e != cudaSuccess) return cuda_status(e, "prod_env_mat_a_noalloc: cudaStreamIsCapturing");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (cap == cudaStreamCaptureStatusNone || g_noalloc_addr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_env_noalloc_scratch);
    if (e != cudaSuccess)
      return cuda_status(e, "prod_env_mat_a_noalloc: cudaGetSymbolAddress");
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return GBDP_OK;
}
}  // namespace

extern "C" int gbdp_prod_env_mat_a_noalloc_f32(
    float* em, float* em_deriv, float* rij, int* nlist, int* nlist_ext, float* ext_coord,
    int* ext_type, int* ext_map, int* ext_nall, int* status, const float* coord,
    const int* atype, const float* avg, const float* std, const gbdp_nbr_plan* plan,
    const gbdp_nbr_frame* frames_host, float rcut_smth, const int* sel, int ntypes,
    gbdp_stream stream) {
  GBDP_REQUIRE(plan && frames_host && status, "prod_env_mat_a_noalloc: null plan/frames/status");
  GBDP_REQUIRE(plan->nframes >= 1 && plan->nframes <= kNoAllocMaxFrames,
               "prod_env_mat_a_noalloc: %d frames exceed the built-in frame table (%d frames)",
               plan->nframes, kNoAllocMaxFrames);
  const size_t need = carve(*plan, nullptr, 0).bytes;
  const size_t room = kNoAllocScratchBytes - kNoAllocFrameBytes;
  GBDP_REQUIRE(need <= room,
               "prod_env_mat_a_noalloc: this batch needs %zu scratch bytes, the built-in "
               "scratch holds %zu (use gbdp_prod_env_mat_a_f32 with a workspace)",
               need, room);
  // every check of the launch before the shared frame table is overwritten
  SecInfo si;
  int rc = env_check_args<float>(em, em_deriv, nlist, ext_coord, ext_type, ext_map, ext_nall,
                                 coord, atype, avg, std, plan, sel, ntypes, &si);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  void* base = nullptr;
  rc = noalloc_scratch_address(st, &base);
  if (rc) return rc;
  const size_t fbytes = sizeof(gbdp_nbr_frame) * (size_t)plan->nframes;
  unsigned char* frames_dev = static_cast<unsigned char*>(base) + room;
  cudaError_t e = cudaMemcpyAsync(frames_dev, frames_host, fbytes, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return cuda_status(e, "prod_env_mat_a_noalloc: frame table copy");
  rc = env_launch<float>(em, em_deriv, rij, nlist, nlist_ext, ext_coord, ext_type, ext_map,
                         ext_nall, coord, atype, avg, std, plan,
                         reinterpret_cast<const gbdp_nbr_frame*>(frames_dev), rcut_smth, sel,
                         ntypes, base, room, st);
  if (rc) return rc;
  // hand the device status word to the caller's buffer (stream-ordered)
  e = cudaMemcpyAsync(status, base, sizeof(int), cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return cuda_status(e, "prod_env_mat_a_noalloc: status copy");
  return GBDP_OK;
}
