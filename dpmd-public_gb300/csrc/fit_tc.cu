// Fitting nets on the 5th-generation tensor cores (sm_103a): tcgen05.mma
// kind::f16 with operands staged in shared memory by TMA and accumulators
// in tensor memory.  FP32-level accuracy from a split: every FP32 operand x
// is taken under a power-of-two scale 2^s as x 2^s = x_hi + x_lo, x_hi =
// fp16(x 2^s) and x_lo = fp16(x 2^s - x_hi), both with 11 significant bits
// (|x 2^s - x_hi - x_lo| <= 2^-22 |x 2^s|), and each product is
// A_hi B_hi + A_lo B_hi + A_hi B_lo (the A_lo B_lo term is below FP32
// rounding).  FP16 holds as many significant bits as TF32 at twice its MMA
// rate and half its bytes; its narrow exponent range is what the scales are
// for.  They are exact powers of two that factor out of every dot product,
// chosen so that a bound on each block's magnitudes maps below 2^15:
//   D rows        per row, from |D_ka| <= |X_k| |X_a| (written by the
//                 descriptor kernel with D, as the row's inverse scale)
//   weights       per output column of each GEMM (host, once per model)
//   H1, H2, GZ*   per layer and type, from bounds the host derives from the
//                 parameters (|tanh| <= 1, 0 <= 1 - T^2 <= 1, row sums of
//                 |W|); a layer's bound may be loose by a large factor
//                 before any precision is lost.
// The epilogue multiplies each accumulator by its column's (and for F1 its
// row's) inverse scale.  The tensor core's FP32 accumulator does not round
// to nearest on every addition, so long accumulation chains are kept
// short: the A_hi B_hi products of k-block kb go to main accumulator
// kb % 3, the two small cross terms to a fourth accumulator, and the
// epilogue adds the four in IEEE FP32.
//
// One kernel computes a 128-row tile of C = A B for one layer (tile widths
// per layer in the TcCfg configurations below); its fused
// epilogue applies the layer's activation (forward) or gradient chain
// (backward) and writes the next GEMM's A operand already split, so the
// whole per-type fitting net (deepmd/pt/model/task/fitting.py:734-899,
// layer semantics deepmd/dpmodel/utils/network.py) is six launches:
//   F1  T1 = tanh(D W1 + b1)                    -> H1 = T1 (split)
//   F2  T2 = tanh(H1 W2 + b2), H2 = T2 idt2 + T1 (split)
//   F3  T3 = tanh(H2 W3 + b3), H3 = T3 idt3 + H2, e += H3 w_out,
//       GZ3 = w_out idt3 (1 - T3^2) (split); H2 recomputed from T1, T2
//   B3  G2 = GZ3 W3^T + w_out, GZ2 = G2 idt2 (1 - T2^2) (split)
//   B2  G1 = GZ2 W2^T + G2,    GZ1 = G1 (1 - T1^2) (split)
//   B1  dE/dD = GZ1 W1^T
// Rows of all activations are grouped by atom type, each type's block padded
// to a multiple of 128, so a tile never mixes types.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <atomic>
#include <cstring>
#include <mutex>

#include "common.cuh"

namespace gbdp {
namespace {

constexpr int TBM = 128, TBK = 64;     // a k-block: 64 FP16 = one 128-byte swizzle row
constexpr int A_TILE = TBM * TBK * 2;  // 16 KiB

// Tile configurations of the per-tile kernel k_fit_tc:
//   CfgLongK   F1 (K 1600): 128 x 128 tiles (two N tiles, the second
//              holding columns 128-239 and 16 zero-filled ones that the
//              epilogue skips), 3 stages, 3 main accumulators, one CTA per
//              SM (196 KB shared, 512 TMEM columns): A is read twice per row
//              block instead of three times with 80-wide tiles, and each
//              stage carries 1.6x the MMA work for 1.23x the bytes
//              (the fitting 4.56 -> 4.19 ms on the 512-frame ragged batch,
//              same bits).  The 3 accumulators keep the long chain
//              FP32-accurate: one main accumulator measured
//              2.3x the energy error and 7x the frame-virial error, its
//              truncation errors adding up coherently over a frame.
//   CfgShortK  K 240 layers: 128 x 80 tiles, 2 stages, 1 main accumulator, two CTAs per SM
//              (105 KB shared, 256 TMEM columns each): with about two tiles
//              per SM, a second CTA's epilogue overlapping the first's main
//              loop measured faster than the persistent kernel (about 21 us
//              against 25-27 us a layer).
// B1 runs on the persistent kernel k_fit_pers (with 128 x 80 tiles on the
// 12,288-row step: 64 us per tile-CTA -> 49 us persistent).
template <int TBN_, int STAGES_, int NACC_>
struct TcCfg {
  static constexpr int TBN = TBN_, STAGES = STAGES_, NACC = NACC_;
  static constexpr int B_TILE = TBN * TBK * 2;
  static constexpr int STAGE = 2 * A_TILE + 2 * B_TILE;
  static constexpr uint32_t ACC_COLS = TBN <= 128 ? 128 : 256;  // TMEM columns per accumulator
  static constexpr int TMEM_COLS = (NACC + 1) * (int)ACC_COLS;   // NACC main + 1 cross-term
  static constexpr int COLP = ((5 * TBN * 4) + 127) & ~127;       // per-column epilogue parameters
  static constexpr int SMEM = STAGES * STAGE + 1024 + 256 + COLP;  // + alignment slack + barriers
  static_assert(TBN % 16 == 0 && TBN <= 256, "tcgen05 M=128 needs N % 16 == 0, N <= 256");
  // CTAs that fit an SM by shared memory must also fit its 512 TMEM columns
  static_assert((228 * 1024 / SMEM) * TMEM_COLS <= 512, "TMEM over-subscribed");
  static_assert(SMEM <= 227 * 1024, "shared memory per CTA");
};
using CfgLongK = TcCfg<128, 3, 3>;
using CfgShortK = TcCfg<80, 2, 1>;
constexpr int FIT_W = 240;                           // hidden width this kernel serves
constexpr int FIT_D = 1600;                          // descriptor width this kernel serves

struct TcMaps {
  CUtensorMap a_hi, a_lo;   // FP16 [rows, K], boxes of 64 columns x 128 rows
  CUtensorMap b_hi[2], b_lo[2];
  CUtensorMap in[2];   // FP32 per-row epilogue inputs, boxes of 16 columns x 32 rows
  CUtensorMap out[3];  // epilogue outputs: o0 (FP32), hi, lo (FP16), same boxes
};

// Epilogue staging per warp (in the pipeline buffers, free once the last
// MMA has completed): two input chunks and two output chunks in flight.
// An FP32 chunk is 32 rows x 16 floats (2 KiB, rows of 64 B, 64-byte TMA
// swizzle); an FP16 chunk 32 rows x 16 halves (1 KiB, rows of 32 B, 32-byte
// swizzle).
constexpr int EPI_CHUNK = 32 * 16;                   // elements per array chunk
constexpr int EPI_IN_BYTES = 2 * 2 * EPI_CHUNK * 4;  // 8 KiB
constexpr int EPI_OUT_BUF = EPI_CHUNK * 4 + 2 * EPI_CHUNK * 2;  // o0 + hi + lo: 4 KiB
constexpr int EPI_WARP_BYTES = EPI_IN_BYTES + 2 * EPI_OUT_BUF;  // 16 KiB

enum { EPI_F1 = 0, EPI_F2, EPI_F3, EPI_B3, EPI_B2, EPI_B1 };

// Per-row inputs and outputs of each epilogue kind (maps.in / maps.out):
//   F1  out T1, H1 hi/lo        F2  in T1; out T2, H2 hi/lo
//   F3  in T1, T2; out GZ3 hi/lo (+ energy partials)
//   B3  in T2; out G2, GZ2 hi/lo      B2  in T1, G2; out GZ1 hi/lo
//   B1  out dE/dD
struct TcEpi {
  int kind;
  int ntypes;
  int row_off[3];   // padded row block of each type; row_off[ntypes] = total rows
  int ntile_n;      // tiles along N (F3: partial energies per row)
  int nin;          // per-row input arrays (maps.in[0..nin))
  int out_mask;     // bit a: maps.out[a] is written
  const float* bias[2];
  const float* idt[2];
  const float* idt2[2];   // F3: idt of layer 2 (H2 = T2 idt2 + T1)
  const float* wout[2];
  const float* cscale[2]; // [N] inverse scale of each output column
  const float* rscale;    // F1: [rows] inverse scale of each D row
  float oscale[2];        // 2^s of the split output (hi / lo)
  float* epart;           // [rows, ntile_n] partial energies (F3)
  int ncols;              // the layer's output columns (N): a tile's columns past it are skipped
  int* status;
};

// ---------------------------------------------------------------- PTX --
__device__ __forceinline__ void tma_2d(void* dst, const CUtensorMap* map, int x, int y,
                                       uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 B apart (the layout a TMA SWIZZLE_128B box of 128-byte rows produces)
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address
  d |= (uint64_t)1 << 16;                    // leading byte offset (unused here), 16 B
  d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset
  d |= (uint64_t)1 << 46;                    // descriptor version (sm_100 family)
  d |= (uint64_t)2 << 61;                    // swizzle: 128 B
  return d;
}

// bulk tensor store of one box from shared memory (bulk-group completion)
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y,
                                             const void* src) {
  asm volatile(
      "cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
          reinterpret_cast<uint64_t>(map)),
      "r"(x), "r"(y), "r"(smem_addr(src))
      : "memory");
}
__device__ __forceinline__ void bulk_commit() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// at most one group still reading its shared-memory source
__device__ __forceinline__ void bulk_wait_read1() {
  asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void umma_f16(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc,
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

// 16 scaled values split into FP16 hi / lo parts, two halves per word
// (element 2j in the low half of word j)
__device__ __forceinline__ void pack_split16(const float* x, uint32_t* hw, uint32_t* lw) {
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    __half h0, l0, h1, l1;
    split_f16(x[2 * j], h0, l0);
    split_f16(x[2 * j + 1], h1, l1);
    hw[j] = (uint32_t)__half_as_ushort(h0) | ((uint32_t)__half_as_ushort(h1) << 16);
    lw[j] = (uint32_t)__half_as_ushort(l0) | ((uint32_t)__half_as_ushort(l1) << 16);
  }
}

// Two 16-column TMEM loads (this warp's lanes) with a single wait
__device__ __forceinline__ void tmem_ld16x2(uint32_t ta, uint32_t tb, float* v, float* w) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15}, [%32];\n"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16, %17, %18, %19, %20, %21, %22, %23, %24, "
      "%25, %26, %27, %28, %29, %30, %31}, [%33];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(ta), "r"(tb)
      : "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    v[k] = __uint_as_float(r[k]);
    w[k] = __uint_as_float(r[16 + k]);
  }
}

// 16 per-column parameters from shared or global memory (16-byte aligned)
__device__ __forceinline__ void colp_ld16(const float* p, float* v) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float4 u = reinterpret_cast<const float4*>(p)[q];
    v[q * 4] = u.x;
    v[q * 4 + 1] = u.y;
    v[q * 4 + 2] = u.z;
    v[q * 4 + 3] = u.w;
  }
}

// The epilogue's per-column parameters of one tile (each pointer at the
// tile's first column): inverse column scale, bias, time step, the layer-2
// time step (F3), output weights; unused ones may be null
struct ColP {
  const float *cs, *bias, *idt, *idt2, *wout;
};

// One thread's row (16 halves as 8 words) of a [32 rows][32 B] staging
// chunk in the TMA 32-byte swizzle: logical 16-byte piece q of row r sits at
// piece q ^ ((r >> 2) & 1) (address bit 4 XOR bit 7; chunks 256-byte
// aligned).
__device__ __forceinline__ void row_st16h(__half* chunk, int lane, const uint32_t* w) {
  const int sw = (lane >> 2) & 1;
#pragma unroll
  for (int q = 0; q < 2; ++q)
    *reinterpret_cast<uint4*>(chunk + lane * 16 + ((q ^ sw) << 3)) =
        make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
}

// One thread's row (16 floats) of a [32 rows][64 B] staging chunk in the
// TMA 64-byte swizzle: logical 16-byte piece q of row r sits at piece
// q ^ ((r >> 1) & 3) (address bits 4-5 XOR bits 7-8; chunks 512-byte
// aligned), so the 8 rows of a warp phase use 8 distinct bank groups.
__device__ __forceinline__ void row_st16(float* chunk, int lane, const float* v) {
  const int sw = (lane >> 1) & 3;
#pragma unroll
  for (int q = 0; q < 4; ++q)
    *reinterpret_cast<float4*>(chunk + lane * 16 + ((q ^ sw) << 2)) =
        make_float4(v[q * 4], v[q * 4 + 1], v[q * 4 + 2], v[q * 4 + 3]);
}
__device__ __forceinline__ void row_ld16(const float* chunk, int lane, float* v) {
  const int sw = (lane >> 1) & 3;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float4 u = *reinterpret_cast<const float4*>(chunk + lane * 16 + ((q ^ sw) << 2));
    v[q * 4] = u.x;
    v[q * 4 + 1] = u.y;
    v[q * 4 + 2] = u.z;
    v[q * 4 + 3] = u.w;
  }
}

// programmatic dependent launch: wait for the grid this one depends on (all
// its writes visible); let the dependent grid be scheduled
__device__ __forceinline__ void griddep_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}
__device__ __forceinline__ void griddep_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Per-warp epilogue progress, carried across the tiles a CTA processes:
// chunks done (input and output staging buffers alternate by chunk) and
// input loads issued / received.
struct EpiState {
  int gci, in_issued, in_done;
};

// The epilogue of one warp's 32 rows of a tile: TBN / 16 chunks of 16
// columns.  Accumulators at tacc (this warp's TMEM lanes, the tile's first
// column): nmain main accumulators acc_stride columns apart and the cross
// terms at cross_off.  Per-row inputs arrive by TMA into the warp's staging
// (wsm, barriers ib[2]), outputs leave by TMA bulk stores.  Returns false
// after a timeout.
template <int TBN>
__device__ __forceinline__ bool epi_tile(const TcMaps& maps, const TcEpi& ep, int t, int yrow,
                                         int n0, int lane, unsigned char* wsm, uint64_t* ib,
                                         uint32_t tacc, int nmain, uint32_t acc_stride,
                                         uint32_t cross_off, const ColP& cp, EpiState& es,
                                         float& esum) {
  float* inb = reinterpret_cast<float*>(wsm);  // [2 buf][2 arr][chunk]
  unsigned char* outb = wsm + EPI_IN_BYTES;    // [2 buf][o0 | hi | lo]
  const int nin = ep.nin;
  constexpr int NCH = TBN / 16;
  // a layer's last tile may be partial (columns past ep.ncols skipped); the
  // chunk counter advances by the chunks done, so that the staging buffers'
  // barrier phases stay in step across the tiles of a persistent CTA
  const int nch = min(NCH, (ep.ncols - n0 + 15) / 16);
  // F1: the inverse scale of this thread's D row; the split output's scale
  const float rsc = ep.kind == EPI_F1 ? __ldg(ep.rscale + yrow + lane) : 1.f;
  const float osc = ep.oscale[t];
  if (nin > 0) {
    // the first chunk's inputs; their buffer was last read two chunks ago
    const int b0 = es.gci & 1;
    fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0) {
      mbar_expect_tx(&ib[b0], nin * EPI_CHUNK * 4);
      for (int a = 0; a < nin; ++a)
        tma_2d(inb + (b0 * 2 + a) * EPI_CHUNK, &maps.in[a], n0, yrow, &ib[b0]);
    }
    ++es.in_issued;
  }
#pragma unroll 1
  for (int ci = 0; ci < nch; ++ci) {
    const int c0 = ci * 16, g = es.gci + ci, buf = g & 1;
    if (ci + 1 < nch && nin > 0) {
      // the other input buffer was last read by the previous chunk
      fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) {
        mbar_expect_tx(&ib[buf ^ 1], nin * EPI_CHUNK * 4);
        for (int a = 0; a < nin; ++a)
          tma_2d(inb + ((buf ^ 1) * 2 + a) * EPI_CHUNK, &maps.in[a], n0 + c0 + 16, yrow,
                 &ib[buf ^ 1]);
      }
      ++es.in_issued;
    }
    float v[16], w[16];
    const uint32_t ta = tacc + (uint32_t)c0;
    if (nmain == 1) {
      tmem_ld16x2(ta, ta + cross_off, v, w);
    } else {
      tmem_ld16(ta, v);
      for (int a = 1; a < nmain; ++a) {
        tmem_ld16(ta + (uint32_t)a * acc_stride, w);
#pragma unroll
        for (int k = 0; k < 16; ++k) v[k] += w[k];
      }
      tmem_ld16(ta + cross_off, w);
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] += w[k];
    const int c = n0 + c0;
    // undo the operand scales (powers of two: exact)
    colp_ld16(cp.cs + c0, w);
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = v[k] * w[k] * rsc;
    float x0[16], x1[16];
    if (nin > 0) {
      if (!__all_sync(kFull, mbar_wait_bounded(&ib[buf], (unsigned)(g >> 1) & 1u, ep.status)))
        return false;
      ++es.in_done;
      row_ld16(inb + (buf * 2) * EPI_CHUNK, lane, x0);
      if (nin > 1) row_ld16(inb + (buf * 2 + 1) * EPI_CHUNK, lane, x1);
    }
    float o0[16], sv[16];  // sv: the next operand, scaled, to be split
    if (ep.kind == EPI_B1) {
#pragma unroll
      for (int k = 0; k < 16; ++k) o0[k] = v[k];
    } else if (ep.kind == EPI_F1 || ep.kind == EPI_F2 || ep.kind == EPI_F3) {
      float bb[16], id[16], wo[16], i2[16];
      colp_ld16(cp.bias + c0, bb);
      if (ep.kind != EPI_F1) colp_ld16(cp.idt + c0, id);
      if (ep.kind == EPI_F3) {
        colp_ld16(cp.wout + c0, wo);
        colp_ld16(cp.idt2 + c0, i2);
      }
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        const float tt = tanhf(v[k] + bb[k]);
        float h = tt;                                      // F1: H1 = T1
        if (ep.kind == EPI_F2) h = tt * id[k] + x0[k];     // H2 = T2 idt2 + T1
        if (ep.kind == EPI_F3) {
          h = tt * id[k] + (x1[k] * i2[k] + x0[k]);        // H3 = T3 idt3 + H2
          esum += h * wo[k];
          sv[k] = wo[k] * id[k] * (1.f - tt * tt) * osc;  // GZ3
        } else {
          sv[k] = h * osc;
        }
        o0[k] = tt;
      }
    } else {  // B3: x0 = T2; B2: x0 = T1, x1 = G2
      float id[16], wo[16];
      if (ep.kind == EPI_B3) {
        colp_ld16(cp.idt + c0, id);
        colp_ld16(cp.wout + c0, wo);
      }
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        const float g = v[k] + (ep.kind == EPI_B3 ? wo[k] : x1[k]);
        o0[k] = g;
        const float tt = x0[k];
        sv[k] = (ep.kind == EPI_B3 ? g * id[k] : g) * (1.f - tt * tt) * osc;
      }
    }
    uint32_t hw[8], lw[8];
    if (ep.out_mask & 6) pack_split16(sv, hw, lw);
    // the output buffer was last used by the stores of chunk g - 2
    if (lane == 0 && g >= 2) bulk_wait_read1();
    __syncwarp();
    unsigned char* ob = outb + buf * EPI_OUT_BUF;
    float* o0b = reinterpret_cast<float*>(ob);
    __half* hib = reinterpret_cast<__half*>(ob + EPI_CHUNK * 4);
    __half* lob = hib + EPI_CHUNK;
    if (ep.out_mask & 1) row_st16(o0b, lane, o0);
    if (ep.out_mask & 2) row_st16h(hib, lane, hw);
    if (ep.out_mask & 4) row_st16h(lob, lane, lw);
    fence_proxy_async_smem();
    __syncwarp();
    if (lane == 0) {
      if (ep.out_mask & 1) tma_store_2d(&maps.out[0], c, yrow, o0b);
      if (ep.out_mask & 2) tma_store_2d(&maps.out[1], c, yrow, hib);
      if (ep.out_mask & 4) tma_store_2d(&maps.out[2], c, yrow, lob);
      bulk_commit();
    }
  }
  es.gci += nch;
  return true;
}

// Lane 0, at the end of a warp's epilogue work: its bulk stores complete and
// no input chunk still in flight (after a timeout) lands once the CTA exits.
__device__ __forceinline__ void epi_drain(uint64_t* ib, const EpiState& es, int* status) {
  bulk_wait_all();
  for (int ch = es.in_done; ch < es.in_issued; ++ch)
    mbar_wait_bounded(&ib[ch & 1], (unsigned)(ch >> 1) & 1u, status);
}

// ------------------------------------------------------------- kernel --
template <class C>
__global__ void __launch_bounds__(128, 1)
    k_fit_tc(const __grid_constant__ TcMaps maps, const __grid_constant__ TcEpi ep, int K) {
  constexpr int TSTAGES = C::STAGES, NACC = C::NACC, TBN = C::TBN, STAGE = C::STAGE,
                B_TILE = C::B_TILE, TMEM_COLS = C::TMEM_COLS;
  constexpr uint32_t ACC_COLS = C::ACC_COLS;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + TSTAGES * STAGE);
  uint64_t* empty = full + TSTAGES;
  uint64_t* tfull = empty + TSTAGES;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tfull + 1);
  uint64_t* inbar = tfull + 2;  // [4 warps][2 buffers]: epilogue input chunks
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // N tiles of one row block are adjacent in launch order: A is read from
  // DRAM once and re-read from L2
  const int row0 = blockIdx.y * TBM, n0 = blockIdx.x * TBN;
  int t = 0;
  while (t + 1 < ep.ntypes && row0 >= ep.row_off[t + 1]) ++t;
  const int nkb = (K + TBK - 1) / TBK;
  // the tile's per-column epilogue parameters, staged once (weights: no
  // dependence on the previous layer) so that the epilogue reads them as
  // shared-memory broadcasts
  float* colp = reinterpret_cast<float*>(smem + TSTAGES * STAGE + 256);
  {
    for (int u = threadIdx.x; u < 5 * TBN; u += blockDim.x) {
      const int a = u / TBN, c = u - a * TBN;
      const float* src = a == 0   ? ep.cscale[t]
                         : a == 1 ? ep.bias[t]
                         : a == 2 ? ep.idt[t]
                         : a == 3 ? ep.idt2[t]
                                  : ep.wout[t];
      colp[u] = src && n0 + c < ep.ncols ? __ldg(src + n0 + c) : 0.f;
    }
  }

  if (threadIdx.x == 0) {
    for (int s = 0; s < TSTAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(tfull, 1);
    for (int b = 0; b < 8; ++b) mbar_init(&inbar[b], 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  int issued = 0;
  if (warp == 0 && lane == 0) {
    // ---- TMA producer.  The weights (B) do not depend on the previous
    //      layer: the first stages' B tiles are requested before waiting for
    //      that layer (programmatic dependent launch), the A tiles after.
    const int pre = nkb < TSTAGES ? nkb : TSTAGES;
    for (int kb = 0; kb < pre; ++kb) {
      unsigned char* st = smem + kb * STAGE;
      mbar_expect_tx(&full[kb], STAGE);
      tma_2d(st + 2 * A_TILE, &maps.b_hi[t], kb * TBK, n0, &full[kb]);
      tma_2d(st + 2 * A_TILE + B_TILE, &maps.b_lo[t], kb * TBK, n0, &full[kb]);
    }
    issued = pre;
    griddep_wait();
    for (int kb = 0; kb < nkb; ++kb) {
      const int s = kb % TSTAGES;
      const unsigned ph = (kb / TSTAGES) & 1u;
      unsigned char* st = smem + s * STAGE;
      if (kb >= TSTAGES) {
        if (!mbar_wait_bounded(&empty[s], ph ^ 1u, ep.status)) break;
        mbar_expect_tx(&full[s], STAGE);
        tma_2d(st + 2 * A_TILE, &maps.b_hi[t], kb * TBK, n0, &full[s]);
        tma_2d(st + 2 * A_TILE + B_TILE, &maps.b_lo[t], kb * TBK, n0, &full[s]);
      }
      tma_2d(st, &maps.a_hi, kb * TBK, row0, &full[s]);
      tma_2d(st + A_TILE, &maps.a_lo, kb * TBK, row0, &full[s]);
      issued = kb + 1 > issued ? kb + 1 : issued;
    }
  } else if (warp == 1 && lane == 0) {
    // ---- MMA issuer: D(f32) += A(f16, K-major) B(f16, K-major), M 128, N 80
    const uint32_t idesc = (1u << 4) | ((uint32_t)(TBN >> 3) << 17) | ((uint32_t)(TBM >> 4) << 24);
    const uint32_t dsmall = tmem + (uint32_t)NACC * ACC_COLS;
    for (int kb = 0; kb < nkb; ++kb) {
      const int s = kb % TSTAGES;
      const unsigned ph = (kb / TSTAGES) & 1u;
      if (!mbar_wait_bounded(&full[s], ph, ep.status)) break;
      tc_fence_after();
      const uint32_t ah = smem_addr(smem + s * STAGE), al = ah + A_TILE, bh = ah + 2 * A_TILE,
                     bl = bh + B_TILE;
      const uint32_t dmain = tmem + (uint32_t)(kb % NACC) * ACC_COLS;
#pragma unroll
      for (int kk = 0; kk < TBK / 16; ++kk) {
        const uint32_t off = kk * 32;  // 16 halves along K within the 128-byte row
        const uint64_t dah = sdesc_sw128(ah + off), dal = sdesc_sw128(al + off),
                       dbh = sdesc_sw128(bh + off), dbl = sdesc_sw128(bl + off);
        umma_f16(dmain, dah, dbh, idesc, (kb >= NACC || kk > 0) ? 1u : 0u);
        umma_f16(dsmall, dal, dbh, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
        umma_f16(dsmall, dah, dbl, idesc, 1u);
      }
      umma_commit(&empty[s]);
    }
    umma_commit(tfull);
  }
  __syncwarp();

  // ---- epilogue: warp w owns rows 32w..32w+31 of the tile (TMEM lanes);
  //      per-row inputs arrive by TMA, outputs leave by TMA bulk stores
  // lanes poll on their own: agree on the outcome before any warp-wide op
  const bool got = __all_sync(kFull, mbar_wait_bounded(tfull, 0, ep.status));
  tc_fence_after();
  // the next layer may start filling SMs as this grid's CTAs leave; this
  // thread's own reads of the previous layer's outputs come after its wait
  griddep_launch_dependents();
  griddep_wait();
  float esum = 0.f;
  if (got) {
    static_assert(4 * EPI_WARP_BYTES <= TSTAGES * STAGE, "epilogue staging exceeds the stage buffers");
    uint64_t* ib = inbar + warp * 2;
    const int yrow = row0 + warp * 32;
    EpiState es{0, 0, 0};
    const int nmain = NACC < nkb ? NACC : nkb;
    const ColP cp{colp, colp + TBN, colp + 2 * TBN, colp + 3 * TBN, colp + 4 * TBN};
    epi_tile<TBN>(maps, ep, t, yrow, n0, lane, smem + warp * EPI_WARP_BYTES, ib,
                  tmem + ((uint32_t)(warp * 32) << 16), nmain, ACC_COLS,
                  (uint32_t)NACC * ACC_COLS, cp, es, esum);
    if (lane == 0) epi_drain(ib, es, ep.status);
    if (ep.kind == EPI_F3) ep.epart[(size_t)(yrow + lane) * ep.ntile_n + blockIdx.x] = esum;
  }
  // ---- drain: no bulk copy of this CTA may land after it exits
  if (warp == 0 && lane == 0) {
    for (int kb = (issued > TSTAGES ? issued - TSTAGES : 0); kb < issued; ++kb)
      mbar_wait_bounded(&full[kb % TSTAGES], (kb / TSTAGES) & 1u, ep.status);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS)
                 : "memory");
}

// Persistent form of k_fit_tc for a layer with one main accumulator, used for
// B1 (13 N tiles of 128 per row block: about 8 tiles per SM on the
// 12,288-row step) and for the K-240 layers once they have many tiles per
// SM (on the 12,288-row step they have about two and run faster as two
// per-tile CTAs per SM): one CTA per SM walks the layer's tiles, the N tiles
// of a row block consecutively so that they run at the same time on
// neighbouring SMs and share A through L2.  Warp 0 issues the TMA loads,
// warp 1 the MMAs, warps 2-5 run the epilogue (warp w reads TMEM lanes
// 32 (w % 4) ..).  Two tensor-memory buffers of (main, cross) accumulators
// let the MMAs of the next tile run while the epilogue drains the last one.
// 128-wide tiles (the last one of a layer partial: 240 = 128 + 112, 1600 =
// 12 x 128 + 64, its padding columns skipped by the epilogue), two stages.
constexpr int PERS_TBN = 128, PERS_STAGES = 2;
constexpr int PERS_STAGE = 2 * A_TILE + 2 * PERS_TBN * TBK * 2;  // 64 KiB
constexpr int PERS_SMEM = PERS_STAGES * PERS_STAGE + 4 * EPI_WARP_BYTES + 1024 + 256;
static_assert(PERS_SMEM <= 227 * 1024, "persistent fitting kernel shared memory");

__global__ void __launch_bounds__(192, 1)
    k_fit_pers(const __grid_constant__ TcMaps maps, const __grid_constant__ TcEpi ep, int K,
               int ntn, int ntiles) {
  constexpr int S = PERS_STAGES, STAGE = PERS_STAGE, B_TILE = PERS_TBN * TBK * 2;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* epi = smem + S * STAGE;  // [4 warps][EPI_WARP_BYTES]
  uint64_t* full = reinterpret_cast<uint64_t*>(epi + 4 * EPI_WARP_BYTES);
  uint64_t* empty = full + S;
  uint64_t* tfull = empty + S;    // [2] accumulator buffer ready
  uint64_t* tempty = tfull + 2;   // [2] accumulator buffer read (4 epilogue warps)
  uint64_t* inbar = tempty + 2;   // [4 warps][2]: epilogue input chunks
  uint64_t* mdone = inbar + 8;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mdone + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nkb = (K + TBK - 1) / TBK;
  auto tile_at = [&](int tile, int& row0, int& n0, int& nt, int& t) {
    const int rb = tile / ntn;
    nt = tile - rb * ntn;
    row0 = rb * TBM;
    n0 = nt * PERS_TBN;
    t = 0;
    while (t + 1 < ep.ntypes && row0 >= ep.row_off[t + 1]) ++t;
  };

  if (threadIdx.x == 0) {
    for (int i = 0; i < S; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    for (int j = 0; j < 2; ++j) {
      mbar_init(&tfull[j], 1);
      mbar_init(&tempty[j], 4);
    }
    for (int b = 0; b < 8; ++b) mbar_init(&inbar[b], 1);
    mbar_init(mdone, 1);
    fence_mbar_init();
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
                     smem_addr(tmem_slot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // ---- TMA producer.  The first tile's first B tiles (weights: no
      //      dependence on the previous layer) are requested before waiting
      //      for that layer, its A tiles after.
      int issued = 0, pre = 0;
      bool ok = true;
      if ((int)blockIdx.x < ntiles) {
        int row0, n0, nt, t;
        tile_at(blockIdx.x, row0, n0, nt, t);
        pre = nkb < S ? nkb : S;
        for (int kb = 0; kb < pre; ++kb) {
          unsigned char* st = smem + kb * STAGE;
          mbar_expect_tx(&full[kb], STAGE);
          tma_2d(st + 2 * A_TILE, &maps.b_hi[t], kb * TBK, n0, &full[kb]);
          tma_2d(st + 2 * A_TILE + B_TILE, &maps.b_lo[t], kb * TBK, n0, &full[kb]);
        }
        griddep_wait();
        for (int kb = 0; kb < pre; ++kb) {
          unsigned char* st = smem + kb * STAGE;
          tma_2d(st, &maps.a_hi, kb * TBK, row0, &full[kb]);
          tma_2d(st + A_TILE, &maps.a_lo, kb * TBK, row0, &full[kb]);
        }
        issued = pre;
      } else {
        griddep_wait();
      }
      int it = 0;
      for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++it) {
        int row0, n0, nt, t;
        tile_at(tile, row0, n0, nt, t);
        for (int kb = (it == 0 ? pre : 0); kb < nkb; ++kb) {
          const int st_i = issued % S;
          if (issued >= S &&
              !mbar_wait_bounded(&empty[st_i], ((issued / S) & 1u) ^ 1u, ep.status)) {
            ok = false;
            break;
          }
          unsigned char* st = smem + st_i * STAGE;
          mbar_expect_tx(&full[st_i], STAGE);
          tma_2d(st + 2 * A_TILE, &maps.b_hi[t], kb * TBK, n0, &full[st_i]);
          tma_2d(st + 2 * A_TILE + B_TILE, &maps.b_lo[t], kb * TBK, n0, &full[st_i]);
          tma_2d(st, &maps.a_hi, kb * TBK, row0, &full[st_i]);
          tma_2d(st + A_TILE, &maps.a_lo, kb * TBK, row0, &full[st_i]);
          ++issued;
        }
      }
      // no bulk copy of this CTA may land after it exits
      for (int k = (issued > S ? issued - S : 0); k < issued; ++k)
        mbar_wait_bounded(&full[k % S], (k / S) & 1u, ep.status);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer: D(f32) += A(f16, K-major) B(f16, K-major), M 128, N 80
      const uint32_t idesc =
          (1u << 4) | ((uint32_t)(PERS_TBN >> 3) << 17) | ((uint32_t)(TBM >> 4) << 24);
      int cons = 0, use[2] = {0, 0}, seen[2] = {0, 0};
      bool ok = true;
      int it = 0;
      for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++it) {
        const int j = it & 1;
        while (ok && seen[j] < use[j]) {
          ok = mbar_wait_bounded(&tempty[j], seen[j] & 1u, ep.status);
          ++seen[j];
        }
        if (!ok) break;
        tc_fence_after();
        const uint32_t dm = tmem + (uint32_t)(j * 256), dc = dm + 128u;
        for (int kb = 0; kb < nkb; ++kb) {
          const int st_i = cons % S;
          if (!mbar_wait_bounded(&full[st_i], (cons / S) & 1u, ep.status)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t ah = smem_addr(smem + st_i * STAGE), al = ah + A_TILE,
                         bh = ah + 2 * A_TILE, bl = bh + B_TILE;
#pragma unroll
          for (int kk = 0; kk < TBK / 16; ++kk) {
            const uint32_t off = kk * 32;
            const uint64_t dah = sdesc_sw128(ah + off), dal = sdesc_sw128(al + off),
                           dbh = sdesc_sw128(bh + off), dbl = sdesc_sw128(bl + off);
            const uint32_t acc = (kb > 0 || kk > 0) ? 1u : 0u;
            umma_f16(dm, dah, dbh, idesc, acc);
            umma_f16(dc, dal, dbh, idesc, acc);
            umma_f16(dc, dah, dbl, idesc, 1u);
          }
          umma_commit(&empty[st_i]);
          ++cons;
        }
        if (ok) {
          umma_commit(&tfull[j]);
          ++use[j];
        }
      }
      // every MMA issued complete before TMEM is released
      umma_commit(mdone);
      mbar_wait_bounded(mdone, 0, ep.status);
    }
  } else {
    // ---- epilogue warps: this warp's rows of each tile
    griddep_wait();  // the previous layer's outputs visible to this thread
    const int ew = warp - 2, q = warp & 3;
    unsigned char* wsm = epi + ew * EPI_WARP_BYTES;
    uint64_t* ib = inbar + ew * 2;
    EpiState es{0, 0, 0};
    int seen[2] = {0, 0};
    int it = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
      const int j = it & 1;
      if (!__all_sync(kFull, mbar_wait_bounded(&tfull[j], seen[j] & 1u, ep.status))) break;
      ++seen[j];
      tc_fence_after();
      // the next layer may start filling SMs once this CTA's last tile drains
      if (tile + (int)gridDim.x >= ntiles) griddep_launch_dependents();
      int row0, n0, nt, t;
      tile_at(tile, row0, n0, nt, t);
      const int yrow = row0 + q * 32;
      float esum = 0.f;
      // the tile's per-column parameters, read from global memory (the
      // kinds that read one have it set; every pointer is 16-byte aligned
      // and n0 a multiple of 16 columns)
      auto col = [n0](const float* p) { return p ? p + n0 : nullptr; };
      const ColP cp{ep.cscale[t] + n0, col(ep.bias[t]), col(ep.idt[t]), col(ep.idt2[t]),
                    col(ep.wout[t])};
      const bool ok = epi_tile<PERS_TBN>(maps, ep, t, yrow, n0, lane, wsm, ib,
                                         tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(j * 256),
                                         1, 0u, 128u, cp, es, esum);
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&tempty[j]);
      if (ep.kind == EPI_F3) ep.epart[(size_t)(yrow + lane) * ep.ntile_n + nt] = esum;
      if (!ok) break;
    }
    if (lane == 0) epi_drain(ib, es, ep.status);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
}

// per-row energy: e = sum of the F3 partials + b_out; padding rows get 0
struct TcRows {
  int row_off[3];
  int nrows[2];
  float b_out[2];
  int ntypes;
};

__global__ void k_fit_tc_energy(float* __restrict__ e, const float* __restrict__ epart,
                                int ntile_n, TcRows rw) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rw.row_off[rw.ntypes]) return;
  int t = 0;
  while (t + 1 < rw.ntypes && r >= rw.row_off[t + 1]) ++t;
  float s = 0.f;
  if (r - rw.row_off[t] < rw.nrows[t]) {
    for (int k = 0; k < ntile_n; ++k) s += epart[(size_t)r * ntile_n + k];
    s += rw.b_out[t];
  }
  e[r] = s;
}

// ------------------------------------------------------------ host side --
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::mutex g_encode_mu;

int get_encode() {
  std::lock_guard<std::mutex> lock(g_encode_mu);
  if (g_encode) return GBDP_OK;
  cudaDriverEntryPointQueryResult q;
  void* fn = nullptr;
  cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                   cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) {
    set_error("fit_tc: cuTensorMapEncodeTiled is unavailable");
    return GBDP_ERR_CUDA;
  }
  g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  return GBDP_OK;
}

// [rows, cols] row-major FP32 (esz 4) or FP16 (esz 2) in boxes of box_x
// columns x box_y rows
int make_map_box(CUtensorMap* m, const void* base, int esz, long rows, long cols, int box_x,
                 int box_y, CUtensorMapSwizzle swz) {
  GBDP_REQUIRE(base != nullptr && ((uintptr_t)base & 15) == 0,
               "fit_tc: operand null or not 16-byte aligned");
  GBDP_REQUIRE((cols * esz) % 16 == 0, "fit_tc: row pitch not a multiple of 16 bytes");
  cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)cols * esz};
  cuuint32_t box[2] = {(cuuint32_t)box_x, (cuuint32_t)box_y};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = g_encode(m, esz == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16,
                        2, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  GBDP_REQUIRE(r == CUDA_SUCCESS, "fit_tc: cuTensorMapEncodeTiled failed (%d)", (int)r);
  return GBDP_OK;
}

// MMA operand (FP16): boxes of 64 columns (128 B) x box_rows rows, 128 B swizzle
int make_map(CUtensorMap* m, const void* base, long rows, long cols, int box_rows) {
  return make_map_box(m, base, 2, rows, cols, TBK, box_rows, CU_TENSOR_MAP_SWIZZLE_128B);
}

// epilogue row array: boxes of 16 columns x 32 rows (one warp's chunk);
// FP32 with the 64-byte swizzle of row_st16 / row_ld16, FP16 with the
// 32-byte swizzle of row_st16h
int make_epi_map(CUtensorMap* m, const void* base, int esz, long rows, long cols) {
  return make_map_box(m, base, esz, rows, cols, 16, 32,
                      esz == 4 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B);
}

size_t a256t(size_t x) { return (x + 255) & ~(size_t)255; }

// FP32 activations (t1, t2, g2), FP16 split operands (*h, *l)
struct TcWs {
  float *t1, *t2, *g2, *epart;
  __half *h1h, *h1l, *h2h, *h2l, *gz3h, *gz3l, *gz2h, *gz2l, *gz1h, *gz1l;
  size_t bytes;
};

TcWs carve_tc(void* base, long rows) {
  TcWs w{};
  char* b = static_cast<char*>(base);
  size_t off = 0;
  auto take = [&](size_t n) {
    void* r = b ? static_cast<void*>(b + off) : nullptr;
    off += a256t(n);
    return r;
  };
  const size_t act = (size_t)rows * FIT_W;
  auto f32 = [&]() { return static_cast<float*>(take(sizeof(float) * act)); };
  auto f16 = [&]() { return static_cast<__half*>(take(sizeof(__half) * act)); };
  w.t1 = f32();
  w.t2 = f32();
  w.g2 = f32();
  w.h1h = f16();
  w.h1l = f16();
  w.h2h = f16();
  w.h2l = f16();
  w.gz3h = f16();
  w.gz3l = f16();
  w.gz2h = f16();
  w.gz2l = f16();
  w.gz1h = f16();
  w.gz1l = f16();
  w.epart = static_cast<float*>(take(sizeof(float) * (size_t)rows * (FIT_W / 80)));
  w.bytes = off;
  return w;
}

}  // namespace
}  // namespace gbdp

using namespace gbdp;

namespace {
// tiles per SM from which the K-240 layers run on the persistent kernel
// (measured on the ragged water batches: per-tile and persistent within 1 %
// from 4 to 60 tiles per SM; the layers are bound by their activation
// traffic, not by launches)
std::atomic<int> g_short_pers_min_tiles{32};
}  // namespace

extern "C" void gbdp_fitting_tc_set_persistent_min_tiles(int tiles_per_sm) {
  g_short_pers_min_tiles.store(tiles_per_sm < 1 ? 1 : tiles_per_sm);
}

extern "C" size_t gbdp_fitting_tc_workspace_bytes(int rows) {
  return carve_tc(nullptr, rows).bytes + 256;
}

extern "C" int gbdp_fitting_tc_f32(float* e, float* dE_dD, const void* D_hi, const void* D_lo,
                                   const float* D_rscale, int ntypes, const int* nrows,
                                   const int* row_off, const gbdp_fit_tc_net* nets,
                                   void* workspace, size_t workspace_bytes, gbdp_stream stream) {
  GBDP_REQUIRE(ntypes >= 1 && ntypes <= 2, "fit_tc: ntypes %d (1 or 2 supported)", ntypes);
  GBDP_REQUIRE(e && dE_dD && D_hi && D_lo && D_rscale && nrows && row_off && nets && workspace,
               "fit_tc: null argument");
  const long rows = row_off[ntypes];
  for (int t = 0; t < ntypes; ++t) {
    GBDP_REQUIRE(row_off[t] % TBM == 0 && row_off[t + 1] >= row_off[t] + nrows[t],
                 "fit_tc: type %d row block not 128-aligned or too small", t);
    const gbdp_fit_tc_net& n = nets[t];
    for (int l = 0; l < 3; ++l) {
      GBDP_REQUIRE(n.wt_hi[l] && n.wt_lo[l] && n.w_hi[l] && n.w_lo[l] && n.b[l],
                   "fit_tc: type %d layer %d weights missing", t, l);
      GBDP_REQUIRE(n.cs_fwd[l] && n.cs_bwd[l] && ((uintptr_t)n.cs_fwd[l] & 15) == 0 &&
                       ((uintptr_t)n.cs_bwd[l] & 15) == 0,
                   "fit_tc: type %d layer %d column scales missing or not 16-byte aligned", t, l);
    }
    GBDP_REQUIRE(n.idt[1] && n.idt[2] && n.w_out, "fit_tc: type %d idt / output layer missing",
                 t);
    for (int a = 0; a < 5; ++a)
      GBDP_REQUIRE(n.act_scale[a] > 0.f, "fit_tc: type %d act_scale[%d] not positive", t, a);
  }
  GBDP_REQUIRE(rows % TBM == 0, "fit_tc: total rows %ld not a multiple of 128", rows);
  TcWs ws = carve_tc(workspace, rows);
  GBDP_REQUIRE(workspace_bytes >= gbdp_fitting_tc_workspace_bytes((int)rows),
               "fit_tc: workspace %zu < %zu", workspace_bytes,
               gbdp_fitting_tc_workspace_bytes((int)rows));
  if (rows == 0) return GBDP_OK;
  int rc = get_encode();
  if (rc) return rc;
  int* status = reinterpret_cast<int*>(static_cast<char*>(workspace) + ws.bytes);
  cudaStream_t st = (cudaStream_t)stream;
  cudaMemsetAsync(status, 0, sizeof(int) * 4, st);
  cudaFuncSetAttribute(k_fit_tc<CfgLongK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       CfgLongK::SMEM);
  cudaFuncSetAttribute(k_fit_tc<CfgShortK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       CfgShortK::SMEM);
  cudaFuncSetAttribute(k_fit_pers, cudaFuncAttributeMaxDynamicSharedMemorySize, PERS_SMEM);
  // SM count of the device (initialised once, thread-safe)
  static const int nsm = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
  }();
  GBDP_REQUIRE(rows / TBM <= 65535, "fit_tc: %ld rows exceed the grid limit", rows);
  TcEpi base{};
  base.ntypes = ntypes;
  for (int t = 0; t <= ntypes; ++t) base.row_off[t] = row_off[t];
  base.status = status;
  // (base.ntile_n, F3's N tiles, is set below with the K-240 layers' kernel)
  for (int t = 0; t < ntypes; ++t) {
    base.wout[t] = nets[t].w_out;
    base.idt2[t] = nets[t].idt[1];
    const float* cols[4] = {nets[t].w_out, nets[t].b[0], nets[t].b[1], nets[t].b[2]};
    for (const float* p : cols)
      GBDP_REQUIRE(((uintptr_t)p & 15) == 0, "fit_tc: bias / w_out not 16-byte aligned");
    GBDP_REQUIRE(((uintptr_t)nets[t].idt[1] & 15) == 0 && ((uintptr_t)nets[t].idt[2] & 15) == 0,
                 "fit_tc: idt not 16-byte aligned");
  }
  enum { LONGK = 0, SHORTK, PERSIST };
  // the K-240 layers go to the persistent kernel from this many tiles per SM
  const long short_tiles = (rows / TBM) * (FIT_W / CfgShortK::TBN);
  const int short_cfg =
      short_tiles >= (long)g_short_pers_min_tiles.load() * nsm ? PERSIST : SHORTK;
  // F3's partial energies: one per N tile of the kernel that runs it
  base.ntile_n = short_cfg == PERSIST ? (FIT_W + PERS_TBN - 1) / PERS_TBN : FIT_W / CfgShortK::TBN;
  // act: index into act_scale of the split output (-1: none)
  struct Step {
    int kind;
    const void *a_hi, *a_lo;
    int K, N, layer;
    bool fwd;
    const float* in[2];
    void* out[3];
    int act;
    int cfg;
  };
  static_assert(FIT_W % CfgShortK::TBN == 0 && PERS_TBN % 16 == 0 && CfgLongK::TBN % 16 == 0 &&
                    FIT_W / CfgShortK::TBN <= 3 && (FIT_W + PERS_TBN - 1) / PERS_TBN <= 3,
                "tile widths must divide the layer widths (F1's last tile may be partial)");
  const Step steps[6] = {
      {EPI_F1, D_hi, D_lo, FIT_D, FIT_W, 0, true, {nullptr, nullptr}, {ws.t1, ws.h1h, ws.h1l}, 0,
       LONGK},
      {EPI_F2, ws.h1h, ws.h1l, FIT_W, FIT_W, 1, true, {ws.t1, nullptr}, {ws.t2, ws.h2h, ws.h2l},
       1, short_cfg},
      {EPI_F3, ws.h2h, ws.h2l, FIT_W, FIT_W, 2, true, {ws.t1, ws.t2},
       {nullptr, ws.gz3h, ws.gz3l}, 2, short_cfg},
      {EPI_B3, ws.gz3h, ws.gz3l, FIT_W, FIT_W, 2, false, {ws.t2, nullptr},
       {ws.g2, ws.gz2h, ws.gz2l}, 3, short_cfg},
      {EPI_B2, ws.gz2h, ws.gz2l, FIT_W, FIT_W, 1, false, {ws.t1, ws.g2},
       {nullptr, ws.gz1h, ws.gz1l}, 4, short_cfg},
      {EPI_B1, ws.gz1h, ws.gz1l, FIT_W, FIT_D, 0, false, {nullptr, nullptr},
       {dE_dD, nullptr, nullptr}, -1, PERSIST}};
  for (const Step& sp : steps) {
    TcMaps maps;
    memset(&maps, 0, sizeof(maps));
    rc = make_map(&maps.a_hi, sp.a_hi, rows, sp.K, TBM);
    if (!rc) rc = make_map(&maps.a_lo, sp.a_lo, rows, sp.K, TBM);
    for (int t = 0; t < 2 && !rc; ++t) {
      const gbdp_fit_tc_net& n = nets[t < ntypes ? t : 0];
      // forward B = W_l^T [out, in]; backward B = W_l [in, out]: both K-major
      const void* bh = sp.fwd ? n.wt_hi[sp.layer] : n.w_hi[sp.layer];
      const void* bl = sp.fwd ? n.wt_lo[sp.layer] : n.w_lo[sp.layer];
      const int tbn = sp.cfg == LONGK ? CfgLongK::TBN : sp.cfg == SHORTK ? CfgShortK::TBN : PERS_TBN;
      rc = make_map(&maps.b_hi[t], bh, sp.N, sp.K, tbn);
      if (!rc) rc = make_map(&maps.b_lo[t], bl, sp.N, sp.K, tbn);
    }
    TcEpi ep = base;
    ep.kind = sp.kind;
    ep.ncols = sp.N;
    ep.nin = 0;
    ep.out_mask = 0;
    // per-row inputs and outputs are [rows, N] arrays, N = this layer's width
    for (int a = 0; a < 2 && !rc; ++a)
      if (sp.in[a]) {
        rc = make_epi_map(&maps.in[a], sp.in[a], 4, rows, sp.N);
        ep.nin = a + 1;
      }
    for (int a = 0; a < 3 && !rc; ++a)
      if (sp.out[a]) {
        rc = make_epi_map(&maps.out[a], sp.out[a], a == 0 ? 4 : 2, rows, sp.N);
        ep.out_mask |= 1 << a;
      }
    if (rc) return rc;
    for (int t = 0; t < ntypes; ++t) {
      ep.bias[t] = nets[t].b[sp.layer];
      ep.idt[t] = nets[t].idt[sp.layer];
      ep.cscale[t] = sp.fwd ? nets[t].cs_fwd[sp.layer] : nets[t].cs_bwd[sp.layer];
      ep.oscale[t] = sp.act >= 0 ? nets[t].act_scale[sp.act] : 1.f;
    }
    if (sp.kind == EPI_B3)
      for (int t = 0; t < ntypes; ++t) ep.idt[t] = nets[t].idt[1];
    if (sp.kind == EPI_F1) ep.rscale = D_rscale;
    if (sp.kind == EPI_F3) ep.epart = ws.epart;
    // launched with programmatic stream serialization: each layer's CTAs
    // start (barriers, TMEM, weight tiles) while the previous layer drains
    cudaLaunchConfig_t lc = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    lc.blockDim = dim3(128);
    lc.stream = st;
    cudaError_t le;
    if (sp.cfg == LONGK) {
      lc.gridDim = dim3((sp.N + CfgLongK::TBN - 1) / CfgLongK::TBN, (unsigned)(rows / TBM));
      lc.dynamicSmemBytes = CfgLongK::SMEM;
      le = cudaLaunchKernelEx(&lc, k_fit_tc<CfgLongK>, maps, ep, sp.K);
    } else if (sp.cfg == SHORTK) {
      lc.gridDim = dim3(sp.N / CfgShortK::TBN, (unsigned)(rows / TBM));
      lc.dynamicSmemBytes = CfgShortK::SMEM;
      le = cudaLaunchKernelEx(&lc, k_fit_tc<CfgShortK>, maps, ep, sp.K);
    } else {
      // one CTA per SM walking the layer's tiles
      const int ntn = (sp.N + PERS_TBN - 1) / PERS_TBN, ntiles = ntn * (int)(rows / TBM);
      lc.gridDim = dim3((unsigned)(ntiles < nsm ? ntiles : nsm));
      lc.blockDim = dim3(192);
      lc.dynamicSmemBytes = PERS_SMEM;
      le = cudaLaunchKernelEx(&lc, k_fit_pers, maps, ep, sp.K, ntn, ntiles);
    }
    if (le != cudaSuccess) return cuda_status(le, "fit_tc gemm launch");
    GBDP_CHECK_LAUNCH("fit_tc gemm");
  }
  TcRows rw{};
  rw.ntypes = ntypes;
  for (int t = 0; t <= ntypes; ++t) rw.row_off[t] = row_off[t];
  for (int t = 0; t < ntypes; ++t) {
    rw.nrows[t] = nrows[t];
    rw.b_out[t] = nets[t].b_out;
  }
  k_fit_tc_energy<<<(unsigned)((rows + 255) / 256), 256, 0, st>>>(e, ws.epart, base.ntile_n, rw);
  GBDP_CHECK_LAUNCH("fit_tc energy");
  return GBDP_OK;
}

extern "C" int gbdp_fitting_tc_status(const void* workspace, int rows, gbdp_stream stream) {
  TcWs ws = carve_tc(nullptr, rows);
  int h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, static_cast<const char*>(workspace) + ws.bytes, sizeof(int),
                                  cudaMemcpyDeviceToHost, (cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_status(e, "fit_tc status");
  return h;
}
