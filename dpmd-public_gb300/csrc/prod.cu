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

// ---------------------------------------------------------- atomic mode --
template <typename T>
__global__ void k_force_atomic(T* __restrict__ force, T* __restrict__ atom_virial,
                               double* __restrict__ vir_acc, const T* __restrict__ net,
                               const T* __restrict__ dR, const T* __restrict__ rij,
                               const int* __restrict__ nlist, int nloc, int nall, int nnei,
                               int nframes) {
  const int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // frame * nloc + i
  const int lane = threadIdx.x & 31;
  if (row >= nframes * nloc) return;
  const int f = row / nloc, i = row - f * nloc;
  const T* g = net + (size_t)row * nnei * 4;
  const T* d = dR + (size_t)row * nnei * 12;
  T ci[3] = {T(0), T(0), T(0)};
  double vs[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) vs[q] = 0.;
  for (int s = lane; s < nnei; s += 32) {
    T v[3];
    pair_force(g, d, s, v);
    ci[0] += v[0];
    ci[1] += v[1];
    ci[2] += v[2];
    const int j = nlist[(size_t)row * nnei + s];
    if (j < 0 || j >= nall) continue;
    if (force) {
      T* fj = force + ((size_t)f * nall + j) * 3;
      atomicAdd(fj + 0, v[0]);
      atomicAdd(fj + 1, v[1]);
      atomicAdd(fj + 2, v[2]);
    }
    if (atom_virial) {
      const T* r = rij + ((size_t)row * nnei + s) * 3;
      const T r0 = r[0], r1 = r[1], r2 = r[2];
      T* av = atom_virial + ((size_t)f * nall + j) * 9;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const T t0 = v[a] * r0, t1 = v[a] * r1, t2 = v[a] * r2;
        atomicAdd(av + a * 3 + 0, t0);
        atomicAdd(av + a * 3 + 1, t1);
        atomicAdd(av + a * 3 + 2, t2);
        vs[a * 3 + 0] += (double)t0;
        vs[a * 3 + 1] += (double)t1;
        vs[a * 3 + 2] += (double)t2;
      }
    }
  }
  ci[0] = warp_sum(ci[0]);
  ci[1] = warp_sum(ci[1]);
  ci[2] = warp_sum(ci[2]);
  if (lane == 0 && force) {
    T* fi = force + ((size_t)f * nall + i) * 3;
    atomicAdd(fi + 0, -ci[0]);
    atomicAdd(fi + 1, -ci[1]);
    atomicAdd(fi + 2, -ci[2]);
  }
  if (atom_virial) {
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      double t = warp_sum(vs[q]);
      if (lane == 0) atomicAdd(vir_acc + f * 9 + q, t);
    }
  }
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

// sort every row of the reverse list ascending (rows are short)
__global__ void k_rev_sort(const int* __restrict__ pairs_in, int* __restrict__ pairs_out,
                           const int* __restrict__ start, const int* __restrict__ cnt,
                           int nrows) {
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= nrows) return;
  const int s = start[r], n = cnt[r];
  for (int a = lane; a < n; a += 32) {
    const int v = pairs_in[s + a];
    int rank = 0;
    for (int b = 0; b < n; ++b) rank += pairs_in[s + b] < v;
    pairs_out[s + rank] = v;
  }
}

template <typename T>
__global__ void k_force_gather(T* __restrict__ force, T* __restrict__ atom_virial,
                               const T* __restrict__ net, const T* __restrict__ dR,
                               const T* __restrict__ rij, const int* __restrict__ start,
                               const int* __restrict__ cnt, const int* __restrict__ pairs,
                               int nloc, int nall, int nnei, int nframes) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;  // frame * nall + j
  if (r >= nframes * nall) return;
  const int f = r / nall, j = r - f * nall;
  const int s0 = start[r], n = cnt[r];
  T F[3] = {T(0), T(0), T(0)};
  T V[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) V[q] = T(0);
  const size_t fbase = (size_t)f * nloc;
  for (int k = 0; k < n; ++k) {
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
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) V[a * 3 + b] += v[a] * rr[b];
    }
  }
  if (j < nloc) {
    const size_t row = fbase + j;
    T c[3] = {T(0), T(0), T(0)};
    for (int s = 0; s < nnei; ++s) {
      T v[3];
      pair_force(net + row * nnei * 4, dR + row * nnei * 12, s, v);
      c[0] += v[0];
      c[1] += v[1];
      c[2] += v[2];
    }
    F[0] -= c[0];
    F[1] -= c[1];
    F[2] -= c[2];
  }
  if (force) {
    force[(size_t)r * 3 + 0] = F[0];
    force[(size_t)r * 3 + 1] = F[1];
    force[(size_t)r * 3 + 2] = F[2];
  }
  if (atom_virial)
#pragma unroll
    for (int q = 0; q < 9; ++q) atom_virial[(size_t)r * 9 + q] = V[q];
}

// frame virial = sum_j atom_virial_j, double, fixed tree (one CTA per frame)
template <typename T>
__global__ void k_vir_reduce(T* __restrict__ virial, const T* __restrict__ atom_virial,
                             int nall) {
  __shared__ double sh[9][256];
  const int f = blockIdx.x;
  double acc[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) acc[q] = 0.;
  for (int j = threadIdx.x; j < nall; j += blockDim.x)
#pragma unroll
    for (int q = 0; q < 9; ++q) acc[q] += (double)atom_virial[((size_t)f * nall + j) * 9 + q];
#pragma unroll
  for (int q = 0; q < 9; ++q) sh[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
#pragma unroll
      for (int q = 0; q < 9; ++q) sh[q][threadIdx.x] += sh[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 9) virial[f * 9 + threadIdx.x] = (T)sh[threadIdx.x][0];
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
  if (det) {
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
  k_rev_sort<<<(nrows * 32 + tb - 1) / tb, tb, 0, st>>>(w.pairs_a, w.pairs_b, w.start, w.cnt,
                                                        nrows);
  GBDP_CHECK_LAUNCH("reverse neighbour list");
  return GBDP_OK;
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
  if (force) cudaMemsetAsync(force, 0, sizeof(T) * (size_t)nframes * nall * 3, st);
  if (atom_virial) cudaMemsetAsync(atom_virial, 0, sizeof(T) * (size_t)nframes * nall * 9, st);
  if (virial) cudaMemsetAsync(virial, 0, sizeof(T) * (size_t)nframes * 9, st);
  if (nframes == 0 || nloc == 0 || nnei == 0) {
    GBDP_CHECK_LAUNCH("prod_force/virial");
    return GBDP_OK;
  }
  GBDP_REQUIRE(net && dR && nlist && (!atom_virial || rij),
               "prod_force/virial: null input pointer");
  GBDP_REQUIRE(((uintptr_t)net & 15) == 0 && ((uintptr_t)dR & 15) == 0,
               "prod_force/virial: net_deriv and env_deriv must be 16-byte aligned");
  const int tb = 256;
  if (!det) {
    cudaMemsetAsync(w.vir_acc, 0, sizeof(double) * 9 * nframes, st);
    const long warps = (long)nframes * nloc;
    k_force_atomic<T><<<(unsigned)((warps * 32 + tb - 1) / tb), tb, 0, st>>>(
        force, atom_virial, w.vir_acc, net, dR, rij, nlist, nloc, nall, nnei, nframes);
    if (virial) k_vir_finish<T><<<1, 256, 0, st>>>(virial, w.vir_acc, 9 * nframes);
  } else {
    int rc = build_reverse(w, nlist, nloc, nall, nnei, nframes, st);
    if (rc) return rc;
    const int nrows = nframes * nall;
    k_force_gather<T><<<(nrows + tb - 1) / tb, tb, 0, st>>>(force, atom_virial, net, dR, rij,
                                                           w.start, w.cnt, w.pairs_b, nloc,
                                                           nall, nnei, nframes);
    if (virial) k_vir_reduce<T><<<nframes, 256, 0, st>>>(virial, atom_virial, nall);
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
  cudaMemsetAsync(virial, 0, sizeof(T) * (size_t)nframes * 9, st);
  if (nframes == 0 || nloc == 0 || nnei == 0) {
    GBDP_CHECK_LAUNCH("prod_virial_a");
    return GBDP_OK;
  }
  GBDP_REQUIRE(net && dR && rij && nlist, "prod_virial_a: null input pointer");
  const int tb = 256;
  if (!det) {
    cudaMemsetAsync(w.vir_acc, 0, sizeof(double) * 9 * nframes, st);
    const long warps = (long)nframes * nloc;
    k_force_atomic<T><<<(unsigned)((warps * 32 + tb - 1) / tb), tb, 0, st>>>(
        nullptr, atom_virial, w.vir_acc, net, dR, rij, nlist, nloc, nall, nnei, nframes);
    k_vir_finish<T><<<1, 256, 0, st>>>(virial, w.vir_acc, 9 * nframes);
  } else {
    int rc = build_reverse(w, nlist, nloc, nall, nnei, nframes, st);
    if (rc) return rc;
    const int nrows = nframes * nall;
    k_force_gather<T><<<(nrows + tb - 1) / tb, tb, 0, st>>>(nullptr, atom_virial, net, dR, rij,
                                                           w.start, w.cnt, w.pairs_b, nloc,
                                                           nall, nnei, nframes);
    k_vir_reduce<T><<<nframes, 256, 0, st>>>(virial, atom_virial, nall);
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
