// Force and virial from dE/d(env matrix) (sm_103a), plus their backward
// kernels.  Reference semantics (the oracle restates them):
//   prod_force_a_cpu       source/lib/src/prod_force.cc:22-72
//   prod_virial_a_cpu      source/lib/src/prod_virial.cc:22-68
//   prod_force_grad_a_cpu  source/lib/src/prod_force_grad.cc:22-73
//   prod_virial_grad_a_cpu source/lib/src/prod_virial_grad.cc:20-66
//
// For a centre i and slot s (neighbour j = nlist[i, s]) the per-pair force
//   v = sum_{w<4} g[i, 4s+w] * dR[i, 4s+w, :]
// is added to F_j and subtracted from F_i; the atomic virial of j gets
// v (x) r_ij.  Two scatter modes:
//   atomics       one warp per centre, lanes over slots, atomicAdd into F_j;
//   deterministic a reverse neighbour list (CSR, each row in ascending
//                 (i, s) order) is built in the workspace and every F_j /
//                 atom_virial_j is a gather in that fixed order, so the result
//                 is bitwise reproducible run to run.
// Frame virials are reduced in double in a fixed tree.
#include <algorithm>
#include <climits>

#include "common.cuh"

namespace gbdp {
namespace {

template <typename T>
struct V4;
template <>
struct V4<float> {
  static __device__ __forceinline__ void load4(const float* p, float* o) {
    float4 v = __ldg(reinterpret_cast<const float4*>(p));
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
    o[3] = v.w;
  }
};
template <>
struct V4<double> {
  static __device__ __forceinline__ void load4(const double* p, double* o) {
    double2 a = __ldg(reinterpret_cast<const double2*>(p));
    double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
    o[0] = a.x;
    o[1] = a.y;
    o[2] = b.x;
    o[3] = b.y;
  }
};

// v = sum_w g_w dR_w for slot s of centre row (g and dR already offset to i)
template <typename T>
__device__ __forceinline__ void pair_force(const T* __restrict__ g, const T* __restrict__ dR,
                                           int s, T* v) {
  T gg[4], d[12];
  V4<T>::load4(g + 4 * s, gg);
  V4<T>::load4(dR + 12 * s, d);
  V4<T>::load4(dR + 12 * s + 4, d + 4);
  V4<T>::load4(dR + 12 * s + 8, d + 8);
  v[0] = gg[0] * d[0] + gg[1] * d[3] + gg[2] * d[6] + gg[3] * d[9];
  v[1] = gg[0] * d[1] + gg[1] * d[4] + gg[2] * d[7] + gg[3] * d[10];
  v[2] = gg[0] * d[2] + gg[1] * d[5] + gg[2] * d[8] + gg[3] * d[11];
}

// p[0..8] += t[0..8]
__device__ __forceinline__ void scatter9(double* p, const double* t) {
#pragma unroll
  for (int q = 0; q < 9; ++q) atomicAdd(p + q, t[q]);
}
__device__ __forceinline__ void scatter9(float* p, const float* t) {
  // p is 4-byte aligned; split the row at its 8- and 16-byte boundaries
  switch ((reinterpret_cast<uintptr_t>(p) >> 2) & 3) {
    case 0:
      red4(p, t[0], t[1], t[2], t[3]);
      red4(p + 4, t[4], t[5], t[6], t[7]);
      atomicAdd(p + 8, t[8]);
      break;
    case 1:
      atomicAdd(p, t[0]);
      red2(p + 1, t[1], t[2]);
      red4(p + 3, t[3], t[4], t[5], t[6]);
      red2(p + 7, t[7], t[8]);
      break;
    case 2:
      red2(p, t[0], t[1]);
      red4(p + 2, t[2], t[3], t[4], t[5]);
      red2(p + 6, t[6], t[7]);
      atomicAdd(p + 8, t[8]);
      break;
    default:
      atomicAdd(p, t[0]);
      red4(p + 1, t[1], t[2], t[3], t[4]);
      red4(p + 5, t[5], t[6], t[7], t[8]);
      break;
  }
}

// ---------------------------------------------------------- atomic mode --
// Persistent warps, each over a contiguous range of centre rows; a row is
// taken in chunks of 32 * U slots (one slot per lane and u).  The loads of
// the next chunk (net 16 B, env deriv 48 B, neighbour index, r_ij for the
// virial) are issued before the current chunk's scatter, so every warp keeps
// a chunk in flight while its reductions drain.  F_j and atom_virial_j by
// (vector) reductions, F_i by one warp reduction per row; the frame virial
// as per-lane partials in T over at most 8 rows, folded into a double on
// lane 0 and added to the frame's accumulator when the frame changes.
template <typename T, int U, bool WV>
struct ScatterChunk {
  T g[U][4], d[U][12], r[U][3];
  int j[U];
};

template <typename T, int U, bool WV>
__device__ __forceinline__ void scatter_load(ScatterChunk<T, U, WV>& c, const T* __restrict__ net,
                                             const T* __restrict__ dR, const T* __restrict__ rij,
                                             const int* __restrict__ nlist, long row, int base,
                                             int nnei, int lane) {
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const int s = base + lane + 32 * u;
    c.j[u] = -1;
    if (s < nnei) {
      const size_t rs = (size_t)row * nnei + s;
      V4<T>::load4(net + rs * 4, c.g[u]);
      V4<T>::load4(dR + rs * 12, c.d[u]);
      V4<T>::load4(dR + rs * 12 + 4, c.d[u] + 4);
      V4<T>::load4(dR + rs * 12 + 8, c.d[u] + 8);
      c.j[u] = __ldg(nlist + rs);
      if (WV) {
        c.r[u][0] = __ldg(rij + rs * 3);
        c.r[u][1] = __ldg(rij + rs * 3 + 1);
        c.r[u][2] = __ldg(rij + rs * 3 + 2);
      }
    } else {
#pragma unroll
      for (int w = 0; w < 4; ++w) c.g[u][w] = T(0);
#pragma unroll
      for (int w = 0; w < 12; ++w) c.d[u][w] = T(0);
#pragma unroll
      for (int w = 0; w < 3; ++w) c.r[u][w] = T(0);
    }
  }
}

template <typename T>
struct ScatterU {
  static constexpr int U = 2;  // two 64-slot chunks in registers per lane
};
template <>
struct ScatterU<double> {
  static constexpr int U = 1;
};

constexpr int kScatterWarps = 4;

// F4: force rows padded to 4 floats (16-byte aligned), so that each F_j is
// one red.global.add.v4.f32 instead of a v2 and a scalar reduction: the
// reductions of a warp go to 32 distinct rows, and their cost in the
// load/store unit scales with the instructions, not the bytes (measured: the
// two-instruction form spends about a quarter of the force call on them).
template <typename T, bool F4>
__device__ __forceinline__ void scatter_force(T* __restrict__ force, size_t row, const T* v) {
  if constexpr (F4) {
    red4(reinterpret_cast<float*>(force) + row * 4, v[0], v[1], v[2], 0.f);
  } else {
    scatter3(force + row * 3, v);
  }
}

template <typename T, int U, bool WV, bool F4>
__global__ void __launch_bounds__(kScatterWarps * 32) k_scatter_atomic(
    T* __restrict__ force, T* __restrict__ atom_virial, double* __restrict__ vir_acc,
    const T* __restrict__ net, const T* __restrict__ dR, const T* __restrict__ rij,
    const int* __restrict__ nlist, int nloc, int nall, int nnei, int nframes) {
  __shared__ double s_vd[kScatterWarps][9];  // lane 0's double virial sums
  const int lane = threadIdx.x & 31;
  const long nw = (long)gridDim.x * kScatterWarps;
  const long gw = (long)blockIdx.x * kScatterWarps + (threadIdx.x >> 5);
  double* vd = s_vd[threadIdx.x >> 5];
  const long rows = (long)nframes * nloc;
  const long per = (rows + nw - 1) / nw;
  const long r0 = gw * per, r1 = min(rows, r0 + per);
  if (r0 >= r1) return;  // uniform over the warp; no CTA-wide barrier below
  const int nch = (nnei + 32 * U - 1) / (32 * U);
  T vs[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) vs[q] = T(0);
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < 9; ++q) vd[q] = 0.;
  int vf = (int)(r0 / nloc);  // frame of the virial partials
  int nfold = 0;              // rows in vs since the last fold
  auto fold = [&]() {
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      const T t = warp_sum(vs[q]);
      vs[q] = T(0);
      if (lane == 0) vd[q] += (double)t;
    }
    nfold = 0;
  };
  auto flush = [&]() {
    if (lane == 0)
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        atomicAdd(vir_acc + (size_t)vf * 9 + q, vd[q]);
        vd[q] = 0.;
      }
  };
  T ci[3] = {T(0), T(0), T(0)};
  ScatterChunk<T, U, WV> cur, nxt;
  long row = r0;
  int ch = 0;
  scatter_load<T, U, WV>(cur, net, dR, rij, nlist, row, 0, nnei, lane);
  while (row < r1) {
    long nrow = row;
    int nc = ch + 1;
    if (nc == nch) {
      nc = 0;
      ++nrow;
    }
    if (nrow < r1) scatter_load<T, U, WV>(nxt, net, dR, rij, nlist, nrow, nc * 32 * U, nnei, lane);
    const int f = (int)(row / nloc);
    if (WV && f != vf) {  // uniform: close the previous frame's partials
      fold();
      flush();
      vf = f;
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      T v[3];
#pragma unroll
      for (int a = 0; a < 3; ++a)
        v[a] = cur.g[u][0] * cur.d[u][a] + cur.g[u][1] * cur.d[u][3 + a] +
               cur.g[u][2] * cur.d[u][6 + a] + cur.g[u][3] * cur.d[u][9 + a];
      ci[0] += v[0];
      ci[1] += v[1];
      ci[2] += v[2];
      const int j = cur.j[u];
      if (j < 0 || j >= nall) continue;
      if (force) scatter_force<T, F4>(force, (size_t)f * nall + j, v);
      if (WV) {
        T t[9];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b) t[a * 3 + b] = v[a] * cur.r[u][b];
        scatter9(atom_virial + ((size_t)f * nall + j) * 9, t);
#pragma unroll
        for (int q = 0; q < 9; ++q) vs[q] += t[q];
      }
    }
    if (ch == nch - 1) {  // row done: F_i -= sum over its slots
      if (force) {
        ci[0] = warp_sum(ci[0]);
        ci[1] = warp_sum(ci[1]);
        ci[2] = warp_sum(ci[2]);
        if (lane == 0) {
          const int i = (int)(row - (long)f * nloc);
          const T m[3] = {-ci[0], -ci[1], -ci[2]};
          scatter_force<T, F4>(force, (size_t)f * nall + i, m);
        }
      }
      ci[0] = ci[1] = ci[2] = T(0);
      if (WV && ++nfold == 8) fold();
    }
    cur = nxt;
    row = nrow;
    ch = nc;
  }
  if (WV) {
    fold();
    flush();
  }
}

// padded FP32 force rows [n][4] -> the output's [n][3]
__global__ void k_force4_compact(float* __restrict__ force, const float4* __restrict__ f4,
                                 size_t n) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float4 v = f4[t];
  force[3 * t] = v.x;
  force[3 * t + 1] = v.y;
  force[3 * t + 2] = v.z;
}

template <typename T>
__global__ void k_vir_finish(T* __restrict__ virial, const double* __restrict__ acc, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) virial[t] = (T)acc[t];
}

// --------------------------------------------------- deterministic mode --
__global__ void k_rev_count(const int* __restrict__ nlist, int nloc, int nall, int nnei,
                            int nframes, int* __restrict__ cnt) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)nframes * nloc * nnei) return;
  const int j = nlist[t];
  if (j < 0 || j >= nall) return;
  const int f = (int)(t / ((size_t)nloc * nnei));
  atomicAdd(&cnt[(size_t)f * nall + j], 1);
}

// three-phase exclusive scan over n ints (blocks of 1024)
__device__ int blk_scan_excl(int v, int& total) {
  __shared__ int wt[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wt[w] = x;
  __syncthreads();
  if (w == 0) {
    int t = lane < nw ? wt[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(kFull, t, o);
      if (lane >= o) t += y;
    }
    if (lane < nw) wt[lane] = t;
  }
  __syncthreads();
  const int off = w ? wt[w - 1] : 0;
  total = wt[nw - 1];
  __syncthreads();
  return off + x - v;
}

__global__ void k_scan_blocks(const int* __restrict__ in, int* __restrict__ out,
                              int* __restrict__ bsum, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  int tot;
  int ex = blk_scan_excl(t < n ? in[t] : 0, tot);
  if (t < n) out[t] = ex;
  if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}
__global__ void k_scan_sums(int* __restrict__ bsum, int nb) {
  int carry = 0;
  for (int b = 0; b < nb; b += blockDim.x) {
    const int t = b + threadIdx.x;
    int tot;
    int ex = blk_scan_excl(t < nb ? bsum[t] : 0, tot);
    if (t < nb) bsum[t] = carry + ex;
    carry += tot;
  }
}
__global__ void k_scan_add(int* __restrict__ out, const int* __restrict__ bsum, int n) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) out[t] += bsum[blockIdx.x];
}

__global__ void k_rev_fill(const int* __restrict__ nlist, int nloc, int nall, int nnei,
                           int nframes, const int* __restrict__ start, int* __restrict__ cursor,
                           int* __restrict__ pairs) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)nframes * nloc * nnei) return;
  const int j = nlist[t];
  if (j < 0 || j >= nall) return;
  const int f = (int)(t / ((size_t)nloc * nnei));
  const size_t fj = (size_t)f * nall + j;
  const int pos = atomicAdd(&cursor[fj], 1);
  pairs[start[fj] + pos] = (int)(t - (size_t)f * nloc * nnei);  // i * nnei + s
}

// Sort every row of the reverse list ascending, one warp per row.  Entries
// of a row are distinct (i * nnei + s, one per centre), so each entry's rank
// is the count of smaller ones: up to 128 entries are held in registers and
// broadcast by shuffles; longer rows rank through memory.
__global__ void __launch_bounds__(256) k_rev_sort(const int* __restrict__ pairs_in,
                                                  int* __restrict__ pairs_out,
                                                  const int* __restrict__ start,
                                                  const int* __restrict__ cnt, int nrows) {
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= nrows) return;  // uniform over the warp
  const int s = start[r], n = cnt[r];
  if (n <= 128) {
    int v[4], rank[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int a = lane + 32 * k;
      v[k] = a < n ? pairs_in[s + a] : INT_MAX;
      rank[k] = 0;
    }
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) {
      if (32 * k2 >= n) break;  // uniform
      for (int l = 0; l < 32; ++l) {
        const int b = __shfl_sync(kFull, v[k2], l);
#pragma unroll
        for (int k = 0; k < 4; ++k) rank[k] += b < v[k];
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (lane + 32 * k < n) pairs_out[s + rank[k]] = v[k];
    return;
  }
  for (int a = lane; a < n; a += 32) {
    const int v = pairs_in[s + a];
    int rank = 0;
    for (int b = 0; b < n; ++b) rank += pairs_in[s + b] < v;
    pairs_out[s + rank] = v;
  }
}

// Deterministic gather, one warp per extended atom j of a frame: lanes take
// the reverse-list entries (ascending (i, s)) in a fixed interleave, local
// atoms also subtract their own centre sum over their slots, and a fixed
// butterfly reduces the lanes, so the result is the same bits every run.
template <typename T>
__global__ void __launch_bounds__(256) k_scatter_gather(
    T* __restrict__ force, T* __restrict__ atom_virial, const T* __restrict__ net,
    const T* __restrict__ dR, const T* __restrict__ rij, const int* __restrict__ start,
    const int* __restrict__ cnt, const int* __restrict__ pairs, int nloc, int nall, int nnei,
    int nframes) {
  const long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // frame * nall + j
  const int lane = threadIdx.x & 31;
  if (r >= (long)nframes * nall) return;  // uniform over the warp
  const int f = (int)(r / nall), j = (int)(r - (long)f * nall);
  const int s0 = start[r], n = cnt[r];
  const size_t fbase = (size_t)f * nloc;
  T F[3] = {T(0), T(0), T(0)};
  T V[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) V[q] = T(0);
  for (int k = lane; k < n; k += 32) {
    const int p = pairs[s0 + k];
    const int i = p / nnei, s = p - i * nnei;
    const size_t row = fbase + i;
    T v[3];
    pair_force(net + row * nnei * 4, dR + row * nnei * 12, s, v);
    F[0] += v[0];
    F[1] += v[1];
    F[2] += v[2];
    if (atom_virial) {
      const T* rr = rij + (row * nnei + s) * 3;
      const T r0 = rr[0], r1 = rr[1], r2 = rr[2];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        V[a * 3 + 0] += v[a] * r0;
        V[a * 3 + 1] += v[a] * r1;
        V[a * 3 + 2] += v[a] * r2;
      }
    }
  }
  if (force) {
    if (j < nloc) {
      const size_t row = fbase + j;
      for (int s = lane; s < nnei; s += 32) {
        T v[3];
        pair_force(net + row * nnei * 4, dR + row * nnei * 12, s, v);
        F[0] -= v[0];
        F[1] -= v[1];
        F[2] -= v[2];
      }
    }
    F[0] = warp_sum(F[0]);
    F[1] = warp_sum(F[1]);
    F[2] = warp_sum(F[2]);
    if (lane == 0) {
      force[(size_t)r * 3 + 0] = F[0];
      force[(size_t)r * 3 + 1] = F[1];
      force[(size_t)r * 3 + 2] = F[2];
    }
  }
  if (atom_virial) {
#pragma unroll
    for (int q = 0; q < 9; ++q) V[q] = warp_sum(V[q]);
    if (lane == 0)
#pragma unroll
      for (int q = 0; q < 9; ++q) atom_virial[(size_t)r * 9 + q] = V[q];
  }
}

// Frame virial = sum_j atom_virial_j in double, fixed order: each CTA sums
// kVirChunk atoms of one frame (thread-strided, then a shared-memory tree)
// into a partial; k_vir_final adds a frame's partials in chunk order.
constexpr int kVirChunk = 2048;

template <typename T>
__global__ void __launch_bounds__(256) k_vir_partial(double* __restrict__ part,
                                                     const T* __restrict__ atom_virial,
                                                     int nall) {
  __shared__ double sh[9][256];
  const int f = blockIdx.y, c = blockIdx.x;
  const int j0 = c * kVirChunk, j1 = min(nall, j0 + kVirChunk);
  double acc[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) acc[q] = 0.;
  for (int j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    const T* av = atom_virial + ((size_t)f * nall + j) * 9;
#pragma unroll
    for (int q = 0; q < 9; ++q) acc[q] += (double)av[q];
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) sh[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
#pragma unroll
      for (int q = 0; q < 9; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 9) part[((size_t)f * gridDim.x + c) * 9 + threadIdx.x] = sh[threadIdx.x][0];
}

template <typename T>
__global__ void k_vir_final(T* __restrict__ virial, const double* __restrict__ part,
                            int nchunk) {
  const int f = blockIdx.x, q = threadIdx.x;
  if (q >= 9) return;
  double s = 0.;
  for (int c = 0; c < nchunk; ++c) s += part[((size_t)f * nchunk + c) * 9 + q];
  virial[f * 9 + q] = (T)s;
}

// ------------------------------------------------------- backward kernels --
template <typename T>
__global__ void k_force_grad(T* __restrict__ grad_net, const T* __restrict__ grad,
                             const T* __restrict__ dR, const int* __restrict__ nlist, int nloc,
                             int nnei, int nframes) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;  // row * nnei + s
  if (t >= (size_t)nframes * nloc * nnei) return;
  const size_t row = t / nnei;
  const int f = (int)(row / nloc);
  const T* gi = grad + row * 3;
  const T gi0 = gi[0], gi1 = gi[1], gi2 = gi[2];
  int j = nlist[t];
  if (j >= nloc) j = j % nloc;
  T gj0 = 0, gj1 = 0, gj2 = 0;
  if (j >= 0) {
    const T* gj = grad + ((size_t)f * nloc + j) * 3;
    gj0 = gj[0];
    gj1 = gj[1];
    gj2 = gj[2];
  }
  const T* d = dR + t * 12;
  T* o = grad_net + t * 4;
#pragma unroll
  for (int w = 0; w < 4; ++w) {
    T v = -(gi0 * d[w * 3] + gi1 * d[w * 3 + 1] + gi2 * d[w * 3 + 2]);
    if (j >= 0) v += gj0 * d[w * 3] + gj1 * d[w * 3 + 1] + gj2 * d[w * 3 + 2];
    o[w] = v;
  }
}

template <typename T>
__global__ void k_virial_grad(T* __restrict__ grad_net, const T* __restrict__ grad,
                              const T* __restrict__ dR, const T* __restrict__ rij,
                              const int* __restrict__ nlist, int nloc, int nnei, int nframes) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (size_t)nframes * nloc * nnei) return;
  const int f = (int)(t / ((size_t)nloc * nnei));
  T* o = grad_net + t * 4;
  if (nlist[t] < 0) {
    o[0] = o[1] = o[2] = o[3] = T(0);
    return;
  }
  const T* G = grad + (size_t)f * 9;
  const T* r = rij + t * 3;
  const T* d = dR + t * 12;
  // u[d0] = sum_d1 G[d0, d1] r[d1]
  T u[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) u[a] = G[a * 3] * r[0] + G[a * 3 + 1] * r[1] + G[a * 3 + 2] * r[2];
#pragma unroll
  for (int w = 0; w < 4; ++w) o[w] = u[0] * d[w * 3] + u[1] * d[w * 3 + 1] + u[2] * d[w * 3 + 2];
}

// ------------------------------------------------------------ host side --
size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

struct ProdWs {
  double* vir_acc;
  float4* force4;    // atomic mode, FP32: padded force rows [nframes * nall]
  double* vir_part;  // deterministic frame-virial partials [nframes, nchunk, 9]
  int* cnt;
  int* start;
  int* cursor;
  int* bsum;
  int* pairs_a;
  int* pairs_b;
  size_t bytes;
};

ProdWs carve_prod(void* base, int nframes, int nloc, int nall, int nnei, int det) {
  ProdWs w{};
  char* b = static_cast<char*>(base);
  size_t off = 0;
  auto take = [&](size_t n) {
    char* r = b ? b + off : nullptr;
    off += a256(n);
    return r;
  };
  w.vir_acc = reinterpret_cast<double*>(take(sizeof(double) * 9 * (size_t)nframes));
  if (!det) w.force4 = reinterpret_cast<float4*>(take(sizeof(float4) * (size_t)nframes * nall));
  if (det) {
    const size_t nchunk = (size_t)(nall + kVirChunk - 1) / kVirChunk;
    w.vir_part = reinterpret_cast<double*>(take(sizeof(double) * 9 * (size_t)nframes * nchunk));
    const size_t nrows = (size_t)nframes * nall;
    const size_t npair = (size_t)nframes * nloc * nnei;
    w.cnt = reinterpret_cast<int*>(take(sizeof(int) * nrows));
    w.start = reinterpret_cast<int*>(take(sizeof(int) * nrows));
    w.cursor = reinterpret_cast<int*>(take(sizeof(int) * nrows));
    w.bsum = reinterpret_cast<int*>(take(sizeof(int) * ((nrows + 1023) / 1024 + 1)));
    w.pairs_a = reinterpret_cast<int*>(take(sizeof(int) * npair));
    w.pairs_b = reinterpret_cast<int*>(take(sizeof(int) * npair));
  }
  w.bytes = off;
  return w;
}

int build_reverse(const ProdWs& w, const int* nlist, int nloc, int nall, int nnei, int nframes,
                  cudaStream_t st) {
  const int nrows = nframes * nall;
  const size_t npair = (size_t)nframes * nloc * nnei;
  cudaMemsetAsync(w.cnt, 0, sizeof(int) * nrows, st);
  cudaMemsetAsync(w.cursor, 0, sizeof(int) * nrows, st);
  const int tb = 256;
  const unsigned gp = (unsigned)((npair + tb - 1) / tb);
  k_rev_count<<<gp, tb, 0, st>>>(nlist, nloc, nall, nnei, nframes, w.cnt);
  const int nb = (nrows + 1023) / 1024;
  k_scan_blocks<<<nb, 1024, 0, st>>>(w.cnt, w.start, w.bsum, nrows);
  k_scan_sums<<<1, 1024, 0, st>>>(w.bsum, nb);
  k_scan_add<<<nb, 1024, 0, st>>>(w.start, w.bsum, nrows);
  k_rev_fill<<<gp, tb, 0, st>>>(nlist, nloc, nall, nnei, nframes, w.start, w.cursor, w.pairs_a);
  k_rev_sort<<<(unsigned)(((size_t)nrows * 32 + tb - 1) / tb), tb, 0, st>>>(
      w.pairs_a, w.pairs_b, w.start, w.cnt, nrows);
  GBDP_CHECK_LAUNCH("reverse neighbour list");
  return GBDP_OK;
}

// persistent grid: as many CTAs as fit on the device at once (occupancy
// queried once per kernel), never more than there are warps' worth of rows
template <typename T, bool WV>
int scatter_cap() {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, k_scatter_atomic<T, ScatterU<T>::U, WV, sizeof(T) == 4>, kScatterWarps * 32, 0);
  return std::max(1, sms * std::max(1, per_sm));
}

template <typename T, bool WV>
unsigned scatter_grid(size_t rows) {
  static const int cap = scatter_cap<T, WV>();  // initialised once, thread-safe
  const size_t need = (rows + kScatterWarps - 1) / kScatterWarps;
  return (unsigned)std::max<size_t>(1, std::min<size_t>((size_t)cap, need));
}

template <typename T>
void launch_atomic(T* force, float4* force4, T* atom_virial, double* vir_acc, const T* net,
                   const T* dR, const T* rij, const int* nlist, int nloc, int nall, int nnei,
                   int nframes, cudaStream_t st) {
  const size_t rows = (size_t)nframes * nloc;
  // FP32: forces accumulate in the padded rows of the workspace (zeroed by
  // the caller), then compacted into the output
  constexpr bool F4 = sizeof(T) == 4;
  T* fdst = F4 && force ? reinterpret_cast<T*>(force4) : force;
  if (atom_virial)
    k_scatter_atomic<T, ScatterU<T>::U, true, F4><<<scatter_grid<T, true>(rows),
                                                    kScatterWarps * 32, 0, st>>>(
        fdst, atom_virial, vir_acc, net, dR, rij, nlist, nloc, nall, nnei, nframes);
  else
    k_scatter_atomic<T, ScatterU<T>::U, false, F4><<<scatter_grid<T, false>(rows),
                                                     kScatterWarps * 32, 0, st>>>(
        fdst, nullptr, nullptr, net, dR, rij, nlist, nloc, nall, nnei, nframes);
  if constexpr (F4) {
    if (force) {
      const size_t n = (size_t)nframes * nall;
      k_force4_compact<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
          reinterpret_cast<float*>(force), force4, n);
    }
  }
}

template <typename T>
void launch_gather(T* force, T* atom_virial, const T* net, const T* dR, const T* rij,
                   const ProdWs& w, int nloc, int nall, int nnei, int nframes, cudaStream_t st) {
  const size_t rows = (size_t)nframes * nall;
  k_scatter_gather<T><<<(unsigned)((rows + 7) / 8), 256, 0, st>>>(
      force, atom_virial, net, dR, rij, w.start, w.cnt, w.pairs_b, nloc, nall, nnei, nframes);
}

template <typename T>
void launch_vir_reduce(T* virial, const T* atom_virial, const ProdWs& w, int nall, int nframes,
                       cudaStream_t st) {
  const int nchunk = (nall + kVirChunk - 1) / kVirChunk;
  if (nchunk == 0) return;  // not reached: callers with no atoms return before
  k_vir_partial<T><<<dim3(nchunk, nframes), 256, 0, st>>>(w.vir_part, atom_virial, nall);
  k_vir_final<T><<<nframes, 32, 0, st>>>(virial, w.vir_part, nchunk);
}

template <typename T>
int prod_launch(T* force, T* virial, T* atom_virial, const T* net, const T* dR, const T* rij,
                const int* nlist, int nloc, int nall, int nnei, int nframes, int det, void* ws,
                size_t ws_bytes, cudaStream_t st) {
  GBDP_REQUIRE(nloc >= 0 && nall >= nloc && nnei >= 0 && nframes >= 0,
               "prod_force/virial: bad sizes nloc=%d nall=%d nnei=%d nframes=%d", nloc, nall,
               nnei, nframes);
  ProdWs w = carve_prod(ws, nframes, nloc, nall, nnei, det);
  GBDP_REQUIRE(ws != nullptr || w.bytes == 0, "prod_force/virial: null workspace");
  GBDP_REQUIRE(ws_bytes >= w.bytes, "prod_force/virial: workspace %zu < %zu", ws_bytes, w.bytes);
  // the FP32 atomic mode writes every force word from its padded rows
  const bool f4 = !det && sizeof(T) == 4 && force;
  const bool empty = nframes == 0 || nloc == 0 || nnei == 0;
  if (force && (!f4 || empty))
    cudaMemsetAsync(force, 0, sizeof(T) * (size_t)nframes * nall * 3, st);
  if (atom_virial) cudaMemsetAsync(atom_virial, 0, sizeof(T) * (size_t)nframes * nall * 9, st);
  if (empty) {
    if (virial) cudaMemsetAsync(virial, 0, sizeof(T) * (size_t)nframes * 9, st);
    GBDP_CHECK_LAUNCH("prod_force/virial");
    return GBDP_OK;
  }
  GBDP_REQUIRE(net && dR && nlist && (!atom_virial || rij),
               "prod_force/virial: null input pointer");
  GBDP_REQUIRE(((uintptr_t)net & 15) == 0 && ((uintptr_t)dR & 15) == 0,
               "prod_force/virial: net_deriv and env_deriv must be 16-byte aligned");
  // every word of `virial` is written below (k_vir_finish, or the fixed-order
  // reduction), so it needs no zero fill; the double accumulators of the
  // atomic mode only where a virial is asked for
  if (!det) {
    if (atom_virial) cudaMemsetAsync(w.vir_acc, 0, sizeof(double) * 9 * nframes, st);
    if (f4) cudaMemsetAsync(w.force4, 0, sizeof(float4) * (size_t)nframes * nall, st);
    launch_atomic<T>(force, w.force4, atom_virial, w.vir_acc, net, dR, rij, nlist, nloc, nall,
                     nnei, nframes, st);
    if (virial) k_vir_finish<T><<<(unsigned)((9 * nframes + 255) / 256), 256, 0, st>>>(
        virial, w.vir_acc, 9 * nframes);
  } else {
    int rc = build_reverse(w, nlist, nloc, nall, nnei, nframes, st);
    if (rc) return rc;
    launch_gather<T>(force, atom_virial, net, dR, rij, w, nloc, nall, nnei, nframes, st);
    if (virial) launch_vir_reduce<T>(virial, atom_virial, w, nall, nframes, st);
  }
  GBDP_CHECK_LAUNCH("prod_force/virial");
  return GBDP_OK;
}

}  // namespace
}  // namespace gbdp

using namespace gbdp;

extern "C" size_t gbdp_prod_workspace_bytes(int nframes, int nloc, int nall, int nnei,
                                            int deterministic) {
  return carve_prod(nullptr, nframes, nloc, nall, nnei, deterministic).bytes;
}

namespace gbdp {
namespace {
// The virial op alone (no force output requested by the caller): the atomic
// path scatters into atom_virial directly; force contributions are skipped.
template <typename T>
int prod_virial_impl(T* virial, T* atom_virial, const T* net, const T* dR, const T* rij,
                     const int* nlist, int nloc, int nall, int nnei, int nframes, int det,
                     void* ws, size_t ws_bytes, cudaStream_t st) {
  GBDP_REQUIRE(nloc >= 0 && nall >= nloc && nnei >= 0 && nframes >= 0,
               "prod_virial_a: bad sizes");
  ProdWs w = carve_prod(ws, nframes, nloc, nall, nnei, det);
  GBDP_REQUIRE(ws != nullptr, "prod_virial_a: null workspace");
  GBDP_REQUIRE(ws_bytes >= w.bytes, "prod_virial_a: workspace %zu < %zu", ws_bytes, w.bytes);
  cudaMemsetAsync(atom_virial, 0, sizeof(T) * (size_t)nframes * nall * 9, st);
  if (nframes == 0 || nloc == 0 || nnei == 0) {
    cudaMemsetAsync(virial, 0, sizeof(T) * (size_t)nframes * 9, st);
    GBDP_CHECK_LAUNCH("prod_virial_a");
    return GBDP_OK;
  }
  GBDP_REQUIRE(net && dR && rij && nlist, "prod_virial_a: null input pointer");
  GBDP_REQUIRE(((uintptr_t)net & 15) == 0 && ((uintptr_t)dR & 15) == 0,
               "prod_virial_a: net_deriv and env_deriv must be 16-byte aligned");
  if (!det) {
    cudaMemsetAsync(w.vir_acc, 0, sizeof(double) * 9 * nframes, st);
    launch_atomic<T>(nullptr, nullptr, atom_virial, w.vir_acc, net, dR, rij, nlist, nloc, nall,
                     nnei, nframes, st);
    k_vir_finish<T><<<(unsigned)((9 * nframes + 255) / 256), 256, 0, st>>>(virial, w.vir_acc,
                                                                             9 * nframes);
  } else {
    int rc = build_reverse(w, nlist, nloc, nall, nnei, nframes, st);
    if (rc) return rc;
    launch_gather<T>(nullptr, atom_virial, net, dR, rij, w, nloc, nall, nnei, nframes, st);
    launch_vir_reduce<T>(virial, atom_virial, w, nall, nframes, st);
  }
  GBDP_CHECK_LAUNCH("prod_virial_a");
  return GBDP_OK;
}
}  // namespace
}  // namespace gbdp

#define GBDP_PROD_ENTRY(T, SFX)                                                                 \
  extern "C" int gbdp_prod_force_a_##SFX(T* force, const T* net_deriv, const T* env_deriv,      \
                                         const int* nlist, int nloc, int nall, int nnei,       \
                                         int nframes, int deterministic, void* workspace,      \
                                         size_t workspace_bytes, gbdp_stream stream) {         \
    GBDP_REQUIRE(force != nullptr, "prod_force_a: null force");                                \
    return prod_launch<T>(force, nullptr, nullptr, net_deriv, env_deriv, nullptr, nlist, nloc, \
                          nall, nnei, nframes, deterministic, workspace, workspace_bytes,      \
                          (cudaStream_t)stream);                                               \
  }                                                                                             \
  extern "C" int gbdp_prod_virial_a_##SFX(                                                      \
      T* virial, T* atom_virial, const T* net_deriv, const T* env_deriv, const T* rij,         \
      const int* nlist, int nloc, int nall, int nnei, int nframes, int deterministic,          \
      void* workspace, size_t workspace_bytes, gbdp_stream stream) {                           \
    GBDP_REQUIRE(virial && atom_virial, "prod_virial_a: null output");                         \
    return prod_virial_impl<T>(virial, atom_virial, net_deriv, env_deriv, rij, nlist, nloc,    \
                               nall, nnei, nframes, deterministic, workspace, workspace_bytes, \
                               (cudaStream_t)stream);                                          \
  }                                                                                             \
  extern "C" int gbdp_prod_force_virial_a_##SFX(                                                \
      T* force, T* virial, T* atom_virial, const T* net_deriv, const T* env_deriv, const T* rij, \
      const int* nlist, int nloc, int nall, int nnei, int nframes, int deterministic,          \
      void* workspace, size_t workspace_bytes, gbdp_stream stream) {                           \
    GBDP_REQUIRE(force && virial && atom_virial, "prod_force_virial_a: null output");           \
    return prod_launch<T>(force, virial, atom_virial, net_deriv, env_deriv, rij, nlist, nloc,  \
                          nall, nnei, nframes, deterministic, workspace, workspace_bytes,      \
                          (cudaStream_t)stream);                                               \
  }                                                                                             \
  extern "C" int gbdp_prod_force_grad_a_##SFX(T* grad_net, const T* grad, const T* env_deriv,   \
                                              const int* nlist, int nloc, int nnei,            \
                                              int nframes, gbdp_stream stream) {               \
    GBDP_REQUIRE(nloc >= 0 && nnei >= 0 && nframes >= 0, "prod_force_grad_a: bad sizes");     \
    const size_t n = (size_t)nframes * nloc * nnei;                                            \
    if (n == 0) return GBDP_OK;                                                                \
    GBDP_REQUIRE(grad_net && grad && env_deriv && nlist, "prod_force_grad_a: null pointer");   \
    k_force_grad<T><<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(            \
        grad_net, grad, env_deriv, nlist, nloc, nnei, nframes);                                \
    GBDP_CHECK_LAUNCH("prod_force_grad_a");                                                    \
    return GBDP_OK;                                                                            \
  }                                                                                             \
  extern "C" int gbdp_prod_virial_grad_a_##SFX(T* grad_net, const T* grad, const T* env_deriv,  \
                                               const T* rij, const int* nlist, int nloc,       \
                                               int nnei, int nframes, gbdp_stream stream) {    \
    GBDP_REQUIRE(nloc >= 0 && nnei >= 0 && nframes >= 0, "prod_virial_grad_a: bad sizes");    \
    const size_t n = (size_t)nframes * nloc * nnei;                                            \
    if (n == 0) return GBDP_OK;                                                                \
    GBDP_REQUIRE(grad_net && grad && env_deriv && rij && nlist,                                \
                 "prod_virial_grad_a: null pointer");                                          \
    k_virial_grad<T><<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(           \
        grad_net, grad, env_deriv, rij, nlist, nloc, nnei, nframes);                           \
    GBDP_CHECK_LAUNCH("prod_virial_grad_a");                                                   \
    return GBDP_OK;                                                                            \
  }

GBDP_PROD_ENTRY(float, f32)
GBDP_PROD_ENTRY(double, f64)
