// Embedding net of the uncompressed se_e2_a descriptor on the 5th-generation
// tensor cores (sm_103a), fused with the G^T R contraction so that the
// nloc x nnei x M embedding never reaches HBM.
//
// Reference semantics: DescrptBlockSeA.forward
// (deepmd/pt/model/descriptor/se_a.py:750-866) with EmbeddingNet /
// MLPLayer (deepmd/pt/model/network/mlp.py:188-219): per neighbour-type
// section t (and centre type when !type_one_side), s = em[..., 0],
// G = net(s) with 1 -> N1 -> N2 -> N3 tanh layers (identity or [x, x]
// skips), X = sum_j em[j, :]^T G[j, :] / nnei; D = X^T X[:, :A].
//
// Precision: layers 2 and 3 are BF16 tcgen05.mma (kind::f16, FP32
// accumulation in tensor memory); layer 1, the activations (tanh.approx),
// the skips, G^T R and D are FP32.
//
// Work unit: two atoms of one centre type.  For each neighbour type the two
// atoms' section rows are concatenated and cut into 128-row tiles; a tile's
// rows are one thread's each (thread r <-> TMEM lane r); one warpgroup per
// CTA, two CTAs per SM.
//   layer 1 (SIMT)  -> A (bf16, 128 x 64, SW128 K-major, shared)
//   MMA  D2 = A W2   (N 64, TMEM columns 0-63)
//   epilogue 2       -> A (bf16), the layer-2 output in FP32 registers
//   MMA  D3 = A W3   (N 128, TMEM columns 128-255)
//   epilogue 3       -> G (FP32, shared), every column of the thread's row
//   G^T R            -> X of the two atoms (FP32, shared)
#include <cuda_bf16.h>

#include <algorithm>

#include "common.cuh"

namespace gbdp {
namespace {

// ----------------------------------------------------- per-net parameters --
// One block of kNetBytes per embedding net (built on the host): the weight
// images in the exact shared-memory layout the MMAs read (bf16, K-major,
// 128-byte swizzle: 16-byte piece p of row n at piece p ^ (n & 7), rows of
// 128 B, K beyond 64 in further [rows x 128 B] chunks), then FP32 params.
constexpr int kNetB2 = 0;       // W2^T  [64 n][64 k]       8 KiB
constexpr int kNetB3 = 8192;    // W3^T  [128 n][64 k]     16 KiB
constexpr int kNetPar = 24576;  // w1[64] b1[64] b2[64] b3[128] (FP32)
constexpr int kNetB3T = 26624;  // W3    [64 n][128 k]     16 KiB (backward)
constexpr int kNetB2T = 43008;  // W2    [64 n][64 k]       8 KiB (backward)
constexpr int kNetBytes = 51200;
constexpr int kNetFwdBytes = kNetPar + 320 * 4;  // what the forward stages
constexpr int kParW1 = 0, kParB1 = 64, kParB2 = 128, kParB3 = 192;

constexpr int kRows = 128;
// FP32 rows of G / dG in shared memory: an odd stride, so that a warp's
// 32 rows writing one column hit 32 banks
template <int N3>
__host__ __device__ constexpr int gstride() { return N3 % 2 ? N3 : N3 + 1; }
constexpr int kSlot = 26624;   // one staged net, forward part (1024-aligned)
constexpr int kMaxTypes = 8;

struct EmbArgs {
  float* X;           // [nloc, 4, N3]
  void* D;            // [rows, N3 * A]: FP32, or FP16 hi with D_lo
  void* D_lo;         // optional FP16 lo part (split for the tensor-core fitting)
  float* D_rs;        // with D_lo: [rows] inverse scale of each D row
  const int* drow;    // D row of each atom (null: the atom index)
  const float* em;    // [nloc, nnei, 4]
  const int* units;   // [nunits, 2] atom pairs of one centre type (-1: none)
  const int* atype;   // [nloc]
  const unsigned char* nets;
  int* status;
  int nunits, ntypes, type_one_side, nloc, nnei, A;
  int sec[kMaxTypes + 1];
};

// ------------------------------------------------------------------ PTX --
__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address
  d |= (uint64_t)1 << 16;                    // leading byte offset (unused with swizzle)
  d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                    // descriptor version (sm_100 family)
  d |= (uint64_t)2 << 61;                    // 128-byte swizzle
  return d;
}

// kind::f16 with BF16 A and B, FP32 D, both K-major, M = 128
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((128u >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

// the same load without the wait: several may be in flight before one
// tcgen05.wait::ld (tmem_wait) makes all their registers valid
__device__ __forceinline__ void tmem_ld16_nw(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t*>(&h);
}

// one row's 16-byte piece u (columns 8u..8u+7) of a [128 x 64] bf16 SW128 tile
__device__ __forceinline__ void st_piece(unsigned char* tile, int r, int u, const float* v8) {
  uint4 w;
  w.x = pack_bf16(v8[0], v8[1]);
  w.y = pack_bf16(v8[2], v8[3]);
  w.z = pack_bf16(v8[4], v8[5]);
  w.w = pack_bf16(v8[6], v8[7]);
  *reinterpret_cast<uint4*>(tile + r * 128 + ((u ^ (r & 7)) << 4)) = w;
}

// Half G0 (pieces 4 G0 .. 4 G0 + 3, columns 32 G0 .. 32 G0 + 31) of a tile
// row from the NV activations h (zero beyond NV); G0 is
// compile-time so that h is indexed statically.
template <int NV, int G0>
__device__ __forceinline__ void st_half(unsigned char* tile, int r, const float* h) {
#pragma unroll
  for (int uu = 0; uu < 4; ++uu) {
    const int u8 = G0 * 4 + uu;
    float v8[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int j = u8 * 8 + c;
      v8[c] = j < NV ? h[j < NV ? j : 0] : 0.f;
    }
    st_piece(tile, r, u8, v8);
  }
}

// skip of a layer from width NI to NO: identity, [x, x] or none
template <int NI, int NO>
struct Skip {
  static constexpr int kind = NI == NO ? 1 : (NO == 2 * NI ? 2 : 0);
  __device__ static __forceinline__ float at(const float* x, int j) {
    if (kind == 1) return x[j];
    if (kind == 2) return x[j < NI ? j : j - NI];
    return 0.f;
  }
};

// Epilogue 3 for one half of the D3 columns (G0 compile-time, so
// that the skip reads h2 with static register indices): G row -> grow.
template <int N2, int N3, int G0>
__device__ __forceinline__ void epi3(uint32_t trow, const float* par, const float* h2, bool live,
                                     float* grow) {
  constexpr int NC = N3 > G0 * 64 ? ((N3 - G0 * 64 + 15) / 16 < 4 ? (N3 - G0 * 64 + 15) / 16 : 4)
                                  : 0;  // 16-column chunks of this half
  if constexpr (NC > 0) {
  uint32_t v[4][16];
#pragma unroll
  for (int c16 = 0; c16 < NC; ++c16) tmem_ld16_nw(trow + 128 + G0 * 64 + c16 * 16, v[c16]);
  tmem_wait();
#pragma unroll
  for (int c16 = 0; c16 < NC; ++c16) {
    const int m0 = G0 * 64 + c16 * 16;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const int m = m0 + k;
      if (m < N3) {
        float gv = 0.f;
        if (live)
          gv = tanh_fast(__uint_as_float(v[c16][k]) + par[kParB3 + m]) + Skip<N2, N3>::at(h2, m);
        grow[m] = gv;
      }
    }
  }
  }
}

// ---------------------------------------------------------------- kernel --
template <int N1, int N2, int N3>
__global__ void __launch_bounds__(128, 2) k_emb_fwd(const __grid_constant__ EmbArgs p) {
  static_assert(N1 <= 32 && N2 <= 64 && N3 <= 128 && N3 >= 1, "embedding widths");
  constexpr int kGStride = gstride<N3>();
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* slot = sm;                   // the staged net (one at a time)
  unsigned char* atile = sm + kSlot;          // A operand, 16 KiB
  float* gsm = reinterpret_cast<float*>(atile + 16384);   // [128][kGStride]
  float* rsm = gsm + kRows * kGStride;                    // [128][4]
  float* xacc = rsm + kRows * 4;                          // [2][4][128]
  uint64_t* bar = reinterpret_cast<uint64_t*>(xacc + 2 * 4 * 128);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
  int* cached = reinterpret_cast<int*>(tslot + 1);        // net index held by each slot
  __shared__ float dred[8];                               // D-row bound: [warp][k, a] maxima

  const int tid = threadIdx.x, warp = tid >> 5;
  const int r = tid;                       // this thread's tile row = TMEM lane

  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
    cached[0] = -1;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(
                     smem_addr(tslot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  for (int k = tid; k < 2 * 4 * 128; k += 128) xacc[k] = 0.f;
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
  unsigned phase = 0;
  bool alive = true;

  const int per = (p.nunits + gridDim.x - 1) / gridDim.x;
  const int u0 = blockIdx.x * per, u1 = min(p.nunits, u0 + per);
  const float inv_nnei = 1.f / (float)p.nnei;

  for (int u = u0; u < u1 && alive; ++u) {
    const int at0 = p.units[2 * u], at1 = p.units[2 * u + 1];
    const int na = at1 >= 0 ? 2 : 1;
    const int ti = p.atype[at0];
    for (int tj = 0; tj < p.ntypes && alive; ++tj) {
      const int sel = p.sec[tj + 1] - p.sec[tj];
      if (sel == 0) continue;
      const int net = p.type_one_side ? tj : tj * p.ntypes + ti;
      if (cached[0] != net) {  // uniform: stage this net's weights and params
        __syncthreads();
        const uint4* src = reinterpret_cast<const uint4*>(p.nets + (size_t)net * kNetBytes);
        uint4* dst = reinterpret_cast<uint4*>(slot);
        for (int k = tid; k < kNetFwdBytes / 16; k += 128) dst[k] = __ldg(src + k);
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) cached[0] = net;
        __syncthreads();
      }
      const float* par = reinterpret_cast<const float*>(slot + kNetPar);
      const uint32_t b2 = smem_addr(slot + kNetB2), b3 = smem_addr(slot + kNetB3);
      const uint32_t aaddr = smem_addr(atile);
      const int nr_all = na * sel;
      for (int t0 = 0; t0 < nr_all && alive; t0 += kRows) {
        const int nrow = min(kRows, nr_all - t0);
        const bool live = r < nrow;
        const int gi = t0 + r;
        const int a = live ? gi / sel : 0;
        float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
        if (live) {
          const int atom = a ? at1 : at0;
          const int slot_j = p.sec[tj] + gi - a * sel;
          e = __ldg(reinterpret_cast<const float4*>(p.em + ((size_t)atom * p.nnei + slot_j) * 4));
        }
        reinterpret_cast<float4*>(rsm)[r] = e;
        // ---- layer 1 (FP32): h1 = tanh(s w1 + b1), all N1 columns per thread
        float h1[N1];
#pragma unroll
        for (int j = 0; j < N1; ++j) h1[j] = tanh_fast(fmaf(e.x, par[kParW1 + j], par[kParB1 + j]));
        // A = h1 (bf16), the row's eight 16-byte pieces
        st_half<N1, 0>(atile, r, h1);
        st_half<N1, 1>(atile, r, h1);
        fence_proxy_async_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
          tc_fence_after();
#pragma unroll
          for (int kk = 0; kk < 4; ++kk)
            umma_bf16(tmem, sdesc_sw128(aaddr + kk * 32), sdesc_sw128(b2 + kk * 32),
                      idesc_bf16(64), kk > 0);
          umma_commit(bar);
        }
        alive = __syncthreads_and(mbar_wait_bounded(bar, phase, p.status));
        phase ^= 1u;
        if (!alive) break;
        tc_fence_after();
        // ---- epilogue 2: h2 = tanh(D2 + b2) + skip(h1), all N2 columns
        float h2[N2];
        {
          constexpr int NC = (N2 + 15) / 16;
          uint32_t v[NC][16];
#pragma unroll
          for (int c16 = 0; c16 < NC; ++c16) tmem_ld16_nw(trow + c16 * 16, v[c16]);
          tmem_wait();
#pragma unroll
          for (int c16 = 0; c16 < NC; ++c16)
#pragma unroll
            for (int k = 0; k < 16; ++k) {
              const int j = c16 * 16 + k;
              if (j < N2)
                h2[j] = tanh_fast(__uint_as_float(v[c16][k]) + par[kParB2 + j]) +
                        Skip<N1, N2>::at(h1, j);
            }
        }
        tc_fence_before();
        __syncthreads();  // every lane has read D2 and MMA 2 is done with A
        st_half<N2, 0>(atile, r, h2);
        st_half<N2, 1>(atile, r, h2);
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
          tc_fence_after();
#pragma unroll
          for (int kk = 0; kk < 4; ++kk)
            umma_bf16(tmem + 128, sdesc_sw128(aaddr + kk * 32), sdesc_sw128(b3 + kk * 32),
                      idesc_bf16(128), kk > 0);
          umma_commit(bar);
        }
        alive = __syncthreads_and(mbar_wait_bounded(bar, phase, p.status));
        phase ^= 1u;
        if (!alive) break;
        tc_fence_after();
        // ---- epilogue 3: G = tanh(D3 + b3) + skip(h2), both column halves
        epi3<N2, N3, 0>(trow, par, h2, live, gsm + r * kGStride);
        epi3<N2, N3, 1>(trow, par, h2, live, gsm + r * kGStride);
        tc_fence_before();
        __syncthreads();
        // ---- G^T R: thread m, for each atom over that atom's tile rows
        for (int ah = 0; ah < na; ++ah) {
          const int m = tid;
          if (m < N3) {
            const int lo = max(0, ah * sel - t0), hi = min(nrow, (ah + 1) * sel - t0);
            float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
            for (int rr = lo; rr < hi; ++rr) {
              const float4 R = reinterpret_cast<const float4*>(rsm)[rr];
              const float gv = gsm[rr * kGStride + m];
              acc[0] = fmaf(R.x, gv, acc[0]);
              acc[1] = fmaf(R.y, gv, acc[1]);
              acc[2] = fmaf(R.z, gv, acc[2]);
              acc[3] = fmaf(R.w, gv, acc[3]);
            }
#pragma unroll
            for (int c = 0; c < 4; ++c) xacc[(ah * 4 + c) * 128 + m] += acc[c];
          }
        }
        __syncthreads();
      }
    }
    if (!alive) break;
    // ---- X and D of the unit's atoms
    for (int ah = 0; ah < na; ++ah) {
      const int m = tid;
      const int atom = ah ? at1 : at0;
      const size_t row = p.drow ? (size_t)p.drow[atom] : (size_t)atom;
      float xm[4] = {0.f, 0.f, 0.f, 0.f};
      if (m < N3) {
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          xm[c] = xacc[(ah * 4 + c) * 128 + m] * inv_nnei;
          p.X[((size_t)atom * 4 + c) * N3 + m] = xm[c];
        }
      }
      if (p.D_lo) {
        // split for the tensor-core fitting: FP16 hi / lo of c D, c = 2^s
        // from |D_ka| <= |X_k| |X_a| (Cauchy-Schwarz over the 4 rows of X)
        const float q = xm[0] * xm[0] + xm[1] * xm[1] + xm[2] * xm[2] + xm[3] * xm[3];
        float qk = q, qa = m < p.A ? q : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          qk = fmaxf(qk, __shfl_xor_sync(kFull, qk, o));
          qa = fmaxf(qa, __shfl_xor_sync(kFull, qa, o));
        }
        if ((tid & 31) == 0) {
          dred[warp * 2] = qk;
          dred[warp * 2 + 1] = qa;
        }
        __syncthreads();
        qk = fmaxf(fmaxf(dred[0], dred[2]), fmaxf(dred[4], dred[6]));
        qa = fmaxf(fmaxf(dred[1], dred[3]), fmaxf(dred[5], dred[7]));
        __syncthreads();  // dred is reused by the next atom
        const float sc = f16_scale_for(sqrtf(qk * qa) * 1.0001f);
        if (m < N3) {
          __half* dh = static_cast<__half*>(p.D) + row * (size_t)N3 * p.A + (size_t)m * p.A;
          __half* dl = static_cast<__half*>(p.D_lo) + row * (size_t)N3 * p.A + (size_t)m * p.A;
          for (int a2 = 0; a2 < p.A; a2 += 4) {
            float v[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              v[j] = 0.f;
#pragma unroll
              for (int c = 0; c < 4; ++c)
                v[j] = fmaf(xm[c], xacc[(ah * 4 + c) * 128 + a2 + j] * inv_nnei, v[j]);
            }
            st_split4_f16(dh + a2, dl + a2, v, sc);
          }
        }
        if (tid == 0) p.D_rs[row] = 1.f / sc;
      } else if (m < N3) {
        float* d = static_cast<float*>(p.D) + row * (size_t)N3 * p.A + (size_t)m * p.A;
        for (int a2 = 0; a2 < p.A; ++a2) {
          float v = 0.f;
#pragma unroll
          for (int c = 0; c < 4; ++c) v = fmaf(xm[c], xacc[(ah * 4 + c) * 128 + a2] * inv_nnei, v);
          d[a2] = v;
        }
      }
    }
    __syncthreads();
    for (int k = tid; k < 2 * 4 * 128; k += 128) xacc[k] = 0.f;
    __syncthreads();
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem) : "memory");
}

// ------------------------------------------------------------- backward --
// dX (gradient wrt the un-normalised sums X * nnei) of every atom from dE/dD:
// D[m][a] = sum_c X[c][m] X[c][a] (a < A), so
//   dX[c][m] = sum_a dD[m][a] X[c][a] + [m < A] sum_m' dD[m'][m] X[c][m'].
// One CTA per atom: threads over m for the first term, threads over (c, a)
// for the second (4 A sums of N3 terms), combined through shared memory.
__global__ void k_emb_dx(float* __restrict__ dxs, const float* __restrict__ dD,
                         const float* __restrict__ X, const int* __restrict__ drow, int N3, int A,
                         float inv_nnei) {
  extern __shared__ float sh[];
  float* xs = sh;                // [4][N3]
  const int As = A + 1;          // odd row stride: threads over m hit distinct banks
  float* dds = sh + 4 * N3;      // [N3][As]
  float* t2 = dds + N3 * As;     // [4][A] second term
  const int atom = blockIdx.x;
  const size_t row = drow ? (size_t)drow[atom] : (size_t)atom;
  for (int k = threadIdx.x; k < 4 * N3; k += blockDim.x) xs[k] = X[(size_t)atom * 4 * N3 + k];
  {  // warps over rows m, lanes over columns a: no division by A
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const float* src = dD + row * N3 * A;
    for (int m = w; m < N3; m += nw)
      for (int a = lane; a < A; a += 32) dds[m * As + a] = src[m * A + a];
  }
  __syncthreads();
  for (int k = threadIdx.x; k < 4 * A; k += blockDim.x) {
    const int c = k / A, a = k - c * A;
    float o = 0.f;
    for (int m2 = 0; m2 < N3; ++m2) o = fmaf(dds[m2 * As + a], xs[c * N3 + m2], o);
    t2[k] = o;
  }
  __syncthreads();
  for (int m = threadIdx.x; m < N3; m += blockDim.x) {
    float o[4] = {0.f, 0.f, 0.f, 0.f};
    for (int a = 0; a < A; ++a) {
      const float w = dds[m * As + a];
#pragma unroll
      for (int c = 0; c < 4; ++c) o[c] = fmaf(w, xs[c * N3 + a], o[c]);
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      if (m < A) o[c] += t2[c * A + m];
      dxs[((size_t)atom * 4 + c) * N3 + m] = o[c] * inv_nnei;
    }
  }
}

struct EmbBwdArgs {
  float* net;          // [nloc, nnei, 4] dE/d(env matrix)
  const float* dxs;    // [nloc, 4, N3] from k_emb_dx
  const float* em;     // [nloc, nnei, 4]
  const int* units;
  const int* atype;
  const unsigned char* nets;
  int* status;
  int nunits, ntypes, type_one_side, nloc, nnei;
  int sec[kMaxTypes + 1];
};

constexpr int kBwdSlot = kNetBytes;  // the whole net block (forward and transposed images)

// Backward epilogue 3 over one half of the D3 columns (G0 compile-time, so
// that every register array is indexed statically): G (recomputed) and the
// incoming dG = R . dX give dR, the skip gradient of dG into sk (the layer
// 2 -> 3 skip: identity or [x, x]) and dZ3 = dG (1 - t3^2) -> the K = 128 A
// operand (bf16, chunk G0).
template <int N1, int N2, int N3, int G0>
__device__ __forceinline__ void bepi3(uint32_t trow, const float* par, const float* t2,
                                      const float* h1, bool live, float4 R, const float* dx,
                                      float* sk, unsigned char* atile, int r, float* dr) {
  unsigned char* chunk = atile + G0 * 16384;
#pragma unroll
  for (int c16 = 0; c16 < 4; ++c16) {
    const int m0 = G0 * 64 + c16 * 16;
    float dz[16];
    if (m0 >= N3) {
#pragma unroll
      for (int k = 0; k < 16; ++k) dz[k] = 0.f;
    } else {
      float v[16];
      tmem_ld16(trow + 128 + m0, v);
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        const int m = m0 + k;
        float z = 0.f;
        if (m < N3 && live) {
          const float t3 = tanh_fast(v[k] + par[kParB3 + m]);
          float gv = t3;
          if (Skip<N2, N3>::kind != 0) {  // h2 at the skip index, from t2 and h1
            const int j = m < N2 ? m : m - N2;
            gv += t2[j] + Skip<N1, N2>::at(h1, j);
          }
          const float d0 = dx[m], d1 = dx[128 + m], d2 = dx[256 + m], d3 = dx[384 + m];
          const float dg = R.x * d0 + R.y * d1 + R.z * d2 + R.w * d3;
          dr[0] = fmaf(gv, d0, dr[0]);
          dr[1] = fmaf(gv, d1, dr[1]);
          dr[2] = fmaf(gv, d2, dr[2]);
          dr[3] = fmaf(gv, d3, dr[3]);
          if (Skip<N2, N3>::kind == 1) sk[m] += dg;
          if (Skip<N2, N3>::kind == 2) sk[m < N2 ? m : m - N2] += dg;
          z = dg * (1.f - t3 * t3);
        }
        dz[k] = z;
      }
    }
    st_piece(chunk, r, c16 * 2, dz);
    st_piece(chunk, r, c16 * 2 + 1, dz + 8);
  }
}

template <int N1, int N2, int N3>
__global__ void __launch_bounds__(128, 2) k_emb_bwd(const __grid_constant__ EmbBwdArgs p) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* slot = sm;                      // one staged net (all images)
  unsigned char* atile = sm + kBwdSlot;          // A operand, 2 chunks of 16 KiB
  float* dxsm = reinterpret_cast<float*>(atile + 32768);  // [2 atoms][4][128]
  uint64_t* bar = reinterpret_cast<uint64_t*>(dxsm + 2 * 4 * 128);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 1);
  int* cached = reinterpret_cast<int*>(tslot + 1);

  const int tid = threadIdx.x, warp = tid >> 5;
  const int r = tid;  // this thread's tile row = TMEM lane

  if (tid == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
    cached[0] = -1;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(
                     smem_addr(tslot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
  unsigned phase = 0;
  bool alive = true;

  const int per = (p.nunits + gridDim.x - 1) / gridDim.x;
  const int u0 = blockIdx.x * per, u1 = min(p.nunits, u0 + per);
  const uint32_t aaddr = smem_addr(atile);

  for (int tj = 0; tj < p.ntypes && alive; ++tj) {
    const int sel = p.sec[tj + 1] - p.sec[tj];
    if (sel == 0) continue;
    for (int u = u0; u < u1 && alive; ++u) {
      const int at0 = p.units[2 * u], at1 = p.units[2 * u + 1];
      const int na = at1 >= 0 ? 2 : 1;
      const int ti = p.atype[at0];
      const int net = p.type_one_side ? tj : tj * p.ntypes + ti;
      __syncthreads();  // the previous unit is done with the shared buffers
      if (cached[0] != net) {
        const uint4* src = reinterpret_cast<const uint4*>(p.nets + (size_t)net * kNetBytes);
        uint4* dst = reinterpret_cast<uint4*>(slot);
        for (int k = tid; k < kNetBytes / 16; k += 128) dst[k] = __ldg(src + k);
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) cached[0] = net;
      }
      for (int k = tid; k < 2 * 4 * 128; k += 128) {
        const int ah = k >> 9, c = (k >> 7) & 3, m = k & 127;
        float v = 0.f;
        if (ah < na && m < N3) v = p.dxs[((size_t)(ah ? at1 : at0) * 4 + c) * N3 + m];
        dxsm[k] = v;
      }
      __syncthreads();
      const float* par = reinterpret_cast<const float*>(slot + kNetPar);
      const uint32_t b2 = smem_addr(slot + kNetB2), b3 = smem_addr(slot + kNetB3);
      const uint32_t b3t = smem_addr(slot + kNetB3T), b2t = smem_addr(slot + kNetB2T);
      const int nr_all = na * sel;
      for (int t0 = 0; t0 < nr_all && alive; t0 += kRows) {
        const int nrow = min(kRows, nr_all - t0);
        const bool live = r < nrow;
        const int gi = t0 + r;
        const int a = live ? gi / sel : 0;
        const int atom = a ? at1 : at0;
        const int slot_j = p.sec[tj] + gi - a * sel;
        float4 e = make_float4(0.f, 0.f, 0.f, 0.f);
        if (live)
          e = __ldg(reinterpret_cast<const float4*>(p.em + ((size_t)atom * p.nnei + slot_j) * 4));
        // ---- forward recompute: layer 1, MMA 2, epilogue 2, MMA 3
        float h1[N1];
#pragma unroll
        for (int j = 0; j < N1; ++j) h1[j] = tanh_fast(fmaf(e.x, par[kParW1 + j], par[kParB1 + j]));
        st_half<N1, 0>(atile, r, h1);
        st_half<N1, 1>(atile, r, h1);
        fence_proxy_async_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
          tc_fence_after();
#pragma unroll
          for (int kk = 0; kk < 4; ++kk)
            umma_bf16(tmem, sdesc_sw128(aaddr + kk * 32), sdesc_sw128(b2 + kk * 32),
                      idesc_bf16(64), kk > 0);
          umma_commit(bar);
        }
        alive = __syncthreads_and(mbar_wait_bounded(bar, phase, p.status));
        phase ^= 1u;
        if (!alive) break;
        tc_fence_after();
        float t2[N2];
#pragma unroll
        for (int c16 = 0; c16 < (N2 + 15) / 16; ++c16) {
          float v[16];
          tmem_ld16(trow + c16 * 16, v);
#pragma unroll
          for (int k = 0; k < 16; ++k) {
            const int j = c16 * 16 + k;
            if (j < N2) t2[j] = tanh_fast(v[k] + par[kParB2 + j]);
          }
        }
        tc_fence_before();
        __syncthreads();
        {
          float h2[N2];
#pragma unroll
          for (int j = 0; j < N2; ++j) h2[j] = t2[j] + Skip<N1, N2>::at(h1, j);
          st_half<N2, 0>(atile, r, h2);
          st_half<N2, 1>(atile, r, h2);
        }
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
          tc_fence_after();
#pragma unroll
          for (int kk = 0; kk < 4; ++kk)
            umma_bf16(tmem + 128, sdesc_sw128(aaddr + kk * 32), sdesc_sw128(b3 + kk * 32),
                      idesc_bf16(128), kk > 0);
          umma_commit(bar);
        }
        alive = __syncthreads_and(mbar_wait_bounded(bar, phase, p.status));
        phase ^= 1u;
        if (!alive) break;
        tc_fence_after();
        // ---- backward epilogue 3: dG, dR, the skip gradient, dZ3 -> A (K = 128)
        float dr[4] = {0.f, 0.f, 0.f, 0.f};
        float sk[N2];
#pragma unroll
        for (int j = 0; j < N2; ++j) sk[j] = 0.f;
        const float* dx = dxsm + a * 512;
        bepi3<N1, N2, N3, 0>(trow, par, t2, h1, live, e, dx, sk, atile, r, dr);
        bepi3<N1, N2, N3, 1>(trow, par, t2, h1, live, e, dx, sk, atile, r, dr);
        fence_proxy_async_smem();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {  // dH2 (partial) = dZ3 W3: K = 128 in two 64-column chunks
          tc_fence_after();
#pragma unroll
          for (int kk = 0; kk < 8; ++kk) {
            const uint32_t ca = aaddr + (kk >> 2) * 16384 + (kk & 3) * 32;
            const uint32_t cb = b3t + (kk >> 2) * 8192 + (kk & 3) * 32;
            umma_bf16(tmem, sdesc_sw128(ca), sdesc_sw128(cb), idesc_bf16(64), kk > 0);
          }
          umma_commit(bar);
        }
        alive = __syncthreads_and(mbar_wait_bounded(bar, phase, p.status));
        phase ^= 1u;
        if (!alive) break;
        tc_fence_after();
        // ---- epilogue 4: dH2 = dZ3 W3 + skip(dG), dZ2 = dH2 (1 - t2^2)
        float sb1[N1];  // t2 becomes dZ2 in place
        {
          float dh2[N2];
#pragma unroll
          for (int c16 = 0; c16 < (N2 + 15) / 16; ++c16) {
            float v[16];
            tmem_ld16(trow + c16 * 16, v);
#pragma unroll
            for (int k = 0; k < 16; ++k) {
              const int j = c16 * 16 + k;
              if (j < N2) {
                dh2[j] = v[k] + sk[j];
                t2[j] = dh2[j] * (1.f - t2[j] * t2[j]);
              }
            }
          }
#pragma unroll
          for (int j = 0; j < N1; ++j) {
            float sk = 0.f;
            if (Skip<N1, N2>::kind == 1) sk = dh2[j];
            if (Skip<N1, N2>::kind == 2) sk = dh2[j] + dh2[j + N1];
            sb1[j] = sk;
          }
        }
        tc_fence_before();
        __syncthreads();  // MMA 4 done with A; every lane has read D4
        st_half<N2, 0>(atile, r, t2);
        st_half<N2, 1>(atile, r, t2);
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {  // dH1 (partial) = dZ2 W2
          tc_fence_after();
#pragma unroll
          for (int kk = 0; kk < 4; ++kk)
            umma_bf16(tmem + 64, sdesc_sw128(aaddr + kk * 32), sdesc_sw128(b2t + kk * 32),
                      idesc_bf16(64), kk > 0);
          umma_commit(bar);
        }
        alive = __syncthreads_and(mbar_wait_bounded(bar, phase, p.status));
        phase ^= 1u;
        if (!alive) break;
        tc_fence_after();
        // ---- epilogue 5: dZ1, ds, and the env-matrix gradient of the row
        float ds = 0.f;
#pragma unroll
        for (int c16 = 0; c16 < (N1 + 15) / 16; ++c16) {
          float v[16];
          tmem_ld16(trow + 64 + c16 * 16, v);
#pragma unroll
          for (int k = 0; k < 16; ++k) {
            const int j = c16 * 16 + k;
            if (j < N1) {
              const float dz1 = (v[k] + sb1[j]) * (1.f - h1[j] * h1[j]);
              ds = fmaf(dz1, par[kParW1 + j], ds);
            }
          }
        }
        if (live)
          *reinterpret_cast<float4*>(p.net + ((size_t)atom * p.nnei + slot_j) * 4) =
              make_float4(ds + dr[0], dr[1], dr[2], dr[3]);
        tc_fence_before();
        __syncthreads();  // every lane has read D5 before the next tile
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem) : "memory");
}

// about 88 KiB: two CTAs per SM (2 x 256 TMEM columns)
template <int N3>
constexpr size_t bwd_smem() {
  return 1024 + kBwdSlot + 32768 + 2 * 4 * 128 * 4 + 64;
}

template <int N1, int N2, int N3>
int emb_bwd_launch(const EmbBwdArgs& a, cudaStream_t st) {
  auto kern = k_emb_bwd<N1, N2, N3>;
  constexpr size_t smem = bwd_smem<N3>();
  static const cudaError_t attr = [&] {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared);
    return e;
  }();
  if (attr != cudaSuccess) return cuda_status(attr, "embed_bwd_tc attribute");
  // two CTAs per SM: registers by __launch_bounds__(128, 2), shared memory
  // below half an SM's
  static_assert(2 * (smem + 1024) <= 228 * 1024, "two CTAs per SM");
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = std::max(1, std::min(2 * sms, a.nunits));
  kern<<<grid, 128, smem, st>>>(a);
  GBDP_CHECK_LAUNCH("embed_bwd_tc");
  return GBDP_OK;
}

// about 100 KiB for N3 = 100: two CTAs per SM (2 x 256 TMEM columns)
template <int N3>
constexpr size_t fwd_smem() {
  return 1024 + kSlot + 16384 + (size_t)kRows * gstride<N3>() * 4 + kRows * 4 * 4 +
         2 * 4 * 128 * 4 + 64;
}

template <int N1, int N2, int N3>
int emb_fwd_launch(const EmbArgs& a, cudaStream_t st) {
  auto kern = k_emb_fwd<N1, N2, N3>;
  constexpr size_t smem = fwd_smem<N3>();
  // the largest shared-memory carveout, so that two CTAs fit an SM
  static const cudaError_t attr = [&] {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                               (int)cudaSharedmemCarveoutMaxShared);
    return e;
  }();
  if (attr != cudaSuccess) return cuda_status(attr, "embed_fwd_tc attribute");
  // two CTAs per SM: registers by __launch_bounds__(128, 2), shared memory
  // below half an SM's
  static_assert(2 * (smem + 1024) <= 228 * 1024, "two CTAs per SM");
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int grid = std::max(1, std::min(2 * sms, a.nunits));
  kern<<<grid, 128, smem, st>>>(a);
  GBDP_CHECK_LAUNCH("embed_fwd_tc");
  return GBDP_OK;
}

}  // namespace
}  // namespace gbdp

using namespace gbdp;

extern "C" size_t gbdp_embed_tc_net_bytes(void) { return (size_t)kNetBytes; }

extern "C" int gbdp_embed_fwd_tc_bf16(float* X, void* D, void* D_lo, float* D_rscale,
                                      const int* drow, const float* em, const int* atype,
                                      const int* units, int nunits, const void* nets, int ntypes,
                                      const int* sel, int type_one_side, int nloc, int nnei,
                                      int n1, int n2, int n3, int axis, int* status,
                                      gbdp_stream stream) {
  GBDP_REQUIRE(ntypes >= 1 && ntypes <= kMaxTypes, "embed_fwd_tc: ntypes %d not in [1, %d]",
               ntypes, kMaxTypes);
  GBDP_REQUIRE(nloc >= 0 && nunits >= 0 && nnei > 0, "embed_fwd_tc: bad sizes");
  GBDP_REQUIRE(axis >= 1 && axis <= n3, "embed_fwd_tc: axis_neuron %d not in [1, %d]", axis, n3);
  GBDP_REQUIRE(X && D && em && atype && units && nets && status,
               "embed_fwd_tc: null pointer");
  GBDP_REQUIRE(((uintptr_t)em & 15) == 0 && ((uintptr_t)nets & 15) == 0,
               "embed_fwd_tc: em and nets must be 16-byte aligned");
  GBDP_REQUIRE(!D_lo || (D_rscale && axis % 4 == 0 && ((uintptr_t)D & 7) == 0 &&
                          ((uintptr_t)D_lo & 7) == 0),
               "embed_fwd_tc: the split D needs D_rscale, axis_neuron %% 4 == 0 and 8-byte "
               "aligned parts");
  EmbArgs a{};
  a.X = X;
  a.D = D;
  a.D_lo = D_lo;
  a.D_rs = D_rscale;
  a.drow = drow;
  a.em = em;
  a.units = units;
  a.atype = atype;
  a.nets = static_cast<const unsigned char*>(nets);
  a.status = status;
  a.nunits = nunits;
  a.ntypes = ntypes;
  a.type_one_side = type_one_side;
  a.nloc = nloc;
  a.nnei = nnei;
  a.A = axis;
  a.sec[0] = 0;
  for (int t = 0; t < ntypes; ++t) {
    GBDP_REQUIRE(sel[t] >= 0, "embed_fwd_tc: negative sel");
    a.sec[t + 1] = a.sec[t] + sel[t];
  }
  GBDP_REQUIRE(a.sec[ntypes] == nnei, "embed_fwd_tc: sum(sel) %d != nnei %d", a.sec[ntypes], nnei);
  if (nunits == 0) return GBDP_OK;
  const cudaStream_t st = (cudaStream_t)stream;
  if (n1 == 25 && n2 == 50 && n3 == 100) return emb_fwd_launch<25, 50, 100>(a, st);
  if (n1 == 3 && n2 == 6 && n3 == 12) return emb_fwd_launch<3, 6, 12>(a, st);
  set_error("embed_fwd_tc: embedding widths %d-%d-%d not built (25-50-100, 3-6-12)", n1, n2, n3);
  return GBDP_ERR_INVALID;
}

extern "C" int gbdp_embed_bwd_tc_bf16(float* net_deriv, float* dx_work, const float* dD,
                                      const float* X, const int* drow, const float* em,
                                      const int* atype, const int* units, int nunits,
                                      const void* nets, int ntypes, const int* sel,
                                      int type_one_side, int nloc, int nnei, int n1, int n2,
                                      int n3, int axis, int* status, gbdp_stream stream) {
  GBDP_REQUIRE(ntypes >= 1 && ntypes <= kMaxTypes, "embed_bwd_tc: ntypes %d not in [1, %d]",
               ntypes, kMaxTypes);
  GBDP_REQUIRE(nloc >= 0 && nunits >= 0 && nnei > 0, "embed_bwd_tc: bad sizes");
  GBDP_REQUIRE(axis >= 1 && axis <= n3, "embed_bwd_tc: axis_neuron %d not in [1, %d]", axis, n3);
  GBDP_REQUIRE(net_deriv && dx_work && dD && X && em && atype && units && nets && status,
               "embed_bwd_tc: null pointer");
  GBDP_REQUIRE(((uintptr_t)em & 15) == 0 && ((uintptr_t)net_deriv & 15) == 0 &&
                   ((uintptr_t)nets & 15) == 0,
               "embed_bwd_tc: em, net_deriv and nets must be 16-byte aligned");
  EmbBwdArgs a{};
  a.net = net_deriv;
  a.dxs = dx_work;
  a.em = em;
  a.units = units;
  a.atype = atype;
  a.nets = static_cast<const unsigned char*>(nets);
  a.status = status;
  a.nunits = nunits;
  a.ntypes = ntypes;
  a.type_one_side = type_one_side;
  a.nloc = nloc;
  a.nnei = nnei;
  a.sec[0] = 0;
  for (int t = 0; t < ntypes; ++t) {
    GBDP_REQUIRE(sel[t] >= 0, "embed_bwd_tc: negative sel");
    a.sec[t + 1] = a.sec[t] + sel[t];
  }
  GBDP_REQUIRE(a.sec[ntypes] == nnei, "embed_bwd_tc: sum(sel) %d != nnei %d", a.sec[ntypes], nnei);
  if (nloc == 0 || nunits == 0) return GBDP_OK;
  const cudaStream_t st = (cudaStream_t)stream;
  const bool w25 = n1 == 25 && n2 == 50 && n3 == 100, w3 = n1 == 3 && n2 == 6 && n3 == 12;
  if (!w25 && !w3) {
    set_error("embed_bwd_tc: embedding widths %d-%d-%d not built (25-50-100, 3-6-12)", n1, n2, n3);
    return GBDP_ERR_INVALID;
  }
  const size_t shm = sizeof(float) * (size_t)(4 * n3 + n3 * (axis + 1) + 4 * axis);
  GBDP_REQUIRE(shm <= 48 * 1024, "embed_bwd_tc: N3 * axis too large");
  k_emb_dx<<<nloc, 128, shm, st>>>(dx_work, dD, X, drow, n3, axis, 1.f / (float)nnei);
  GBDP_CHECK_LAUNCH("embed_dx");
  return w25 ? emb_bwd_launch<25, 50, 100>(a, st) : emb_bwd_launch<3, 6, 12>(a, st);
}
