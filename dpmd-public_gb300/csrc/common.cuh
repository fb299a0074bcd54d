// Shared device/host helpers for the GB300 (sm_103a) se_e2_a kernels.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>

#include "../../include/gbdp.h"

namespace gbdp {

constexpr int kWarp = 32;
constexpr unsigned kFull = 0xffffffffu;

// ------------------------------------------------------------ error state --
// The last error message is thread-local; entry points return a status code
// and never throw across the C ABI.
void set_error(const char* fmt, ...);
int cuda_status(cudaError_t e, const char* where);

#define GBDP_CHECK_LAUNCH(where)                                        \
  do {                                                                  \
    cudaError_t _e = cudaGetLastError();                                \
    if (_e != cudaSuccess) return ::gbdp::cuda_status(_e, where);       \
  } while (0)

#define GBDP_REQUIRE(cond, ...)                \
  do {                                         \
    if (!(cond)) {                             \
      ::gbdp::set_error(__VA_ARGS__);          \
      return GBDP_ERR_INVALID;                 \
    }                                          \
  } while (0)

// ------------------------------------------------------------ warp helpers --
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// ------------------------------------------------------ vector reductions --
// red.global.add over 2 or 4 consecutive floats (sm_90 and later) where the
// address is 8- / 16-byte aligned; scalar atomics for the rest and for double
__device__ __forceinline__ void red2(float* p, float a, float b) {
  asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(a), "f"(b) : "memory");
}
__device__ __forceinline__ void red4(float* p, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(p), "f"(a), "f"(b), "f"(c),
               "f"(d)
               : "memory");
}

// p[0..2] += v[0..2]
__device__ __forceinline__ void scatter3(double* p, const double* v) {
  atomicAdd(p, v[0]);
  atomicAdd(p + 1, v[1]);
  atomicAdd(p + 2, v[2]);
}
__device__ __forceinline__ void scatter3(float* p, const float* v) {
  if ((reinterpret_cast<uintptr_t>(p) & 7) == 0) {
    red2(p, v[0], v[1]);
    atomicAdd(p + 2, v[2]);
  } else {
    atomicAdd(p, v[0]);
    red2(p + 1, v[1], v[2]);
  }
}

// ------------------------------------------------------ fixed-point sums --
// Deterministic accumulation: a value v is added as the 64-bit integer
// round(v * 2^s).  Integer addition is associative, so a total has the
// same bits whatever order the additions arrive in; it is read back as
// total * 2^-s.  Scaling by a power of two is exact, so the only rounding is
// that of each term to the grid 2^-s.
template <typename T>
struct FxScale;
template <>
struct FxScale<float> {
  static constexpr int force = 32;  // 2.3e-10 grid, |F| < 2^31
  static constexpr int virial = 32;
};
template <>
struct FxScale<double> {
  static constexpr int force = 40;  // 9.1e-13 grid, |F| < 2^23
  static constexpr int virial = 36;
};
constexpr int kFxEnergy = 30;  // 9.3e-10 grid, |E| per frame < 2^33

// 2^s from its bit pattern (|s| well inside the exponent range)
__host__ __device__ inline float pow2f(int s) {
  union {
    unsigned u;
    float f;
  } x{(unsigned)(127 + s) << 23};
  return x.f;
}
__host__ __device__ inline double pow2d(int s) {
  union {
    unsigned long long u;
    double d;
  } x{(unsigned long long)(1023 + s) << 52};
  return x.d;
}
__device__ __forceinline__ long long fx_of(float v, int s) { return __float2ll_rn(v * pow2f(s)); }
__device__ __forceinline__ long long fx_of(double v, int s) { return __double2ll_rn(v * pow2d(s)); }
template <typename T>
__device__ __forceinline__ void fx_add(long long* p, T v, int s) {
  atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long)fx_of(v, s));
}
template <typename T>
__device__ __forceinline__ void fx_add3(long long* p, const T* v, int s) {
  fx_add(p, v[0], s);
  fx_add(p + 1, v[1], s);
  fx_add(p + 2, v[2], s);
}

// Device-side error word: kernels record the first problem they hit and
// return; the host reads the word after the stream is synchronised.
__device__ __forceinline__ void raise_status(int* status, int code) {
  if (status) atomicCAS(status, 0, code);
}

// ------------------------------------------------------- table addressing --
// locate_xx of the reference (source/lib/src/tabulate.cc:19-42): the row of a
// normalised s value and its offset inside that row, two uniform strides,
// clamped outside [lower, max).
template <typename T>
struct TableInfo {
  T lower, upper, max, stride0, stride1;
  int first_stride;  // int((upper - lower) / stride0)
  int last_row;      // first_stride + int((max - upper) / stride1) - 1
};

__device__ __forceinline__ float fmul_x(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double fmul_x(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float fadd_x(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double fadd_x(double a, double b) { return __dadd_rn(a, b); }

// The row offset is formed as in the reference (multiply, round, add, round;
// no fused multiply-add) so that every x lands in the same row.
template <typename T>
__device__ __forceinline__ int locate_row(const TableInfo<T>& ti, T& xx) {
  int idx;
  if (xx < ti.lower) {
    idx = 0;
    xx = T(0);
  } else if (xx < ti.upper) {
    idx = (int)((xx - ti.lower) / ti.stride0);
    xx -= fadd_x(fmul_x((T)idx, ti.stride0), ti.lower);
  } else if (xx < ti.max) {
    idx = ti.first_stride + (int)((xx - ti.upper) / ti.stride1);
    xx -= fadd_x(fmul_x((T)(idx - ti.first_stride), ti.stride1), ti.upper);
  } else {
    idx = ti.last_row;
    xx = T(0);
  }
  return idx;
}

template <typename T>
TableInfo<T> make_table_info(const T* info) {
  TableInfo<T> ti;
  ti.lower = info[0];
  ti.upper = info[1];
  ti.max = info[2];
  ti.stride0 = info[3];
  ti.stride1 = info[4];
  ti.first_stride = int((ti.upper - ti.lower) / ti.stride0);
  ti.last_row = ti.first_stride + int((ti.max - ti.upper) / ti.stride1) - 1;
  return ti;
}

// Horner forms of the fifth-order row polynomial and its derivative, in the
// reference's evaluation order (tabulate.cc:119-128, :214-219).
template <typename T>
__device__ __forceinline__ T poly5(const T* a, T x) {
  return a[0] + (a[1] + (a[2] + (a[3] + (a[4] + a[5] * x) * x) * x) * x) * x;
}
template <typename T>
__device__ __forceinline__ T dpoly5(const T* a, T x) {
  return a[1] + (T(2) * a[2] + (T(3) * a[3] + (T(4) * a[4] + T(5) * a[5] * x) * x) * x) * x;
}

// --------------------------------------------------- bulk async copy (TMA) --
// cp.async.bulk global -> shared completing on an mbarrier.  Both addresses
// must be 16-byte aligned and the size a multiple of 16.
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, "
      "1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

// Bounded wait: gives up after `limit` polls and reports it through `status`.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned phase, int* status,
                                                  long limit = (1l << 26)) {
  for (long it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, phase)) return true;
  raise_status(status, GBDP_STATUS_TIMEOUT);
  return false;
}

// ------------------------------------------------ FP16 hi/lo operand split --
// The tensor-core fitting takes each FP32 operand x as two FP16 parts under
// a power-of-two scale 2^s: hi = fp16(x 2^s), lo = fp16(x 2^s - hi).  Both
// parts carry 11 significant bits (as TF32 does), so hi + lo holds x to
// about 2^-22 relative, and the scale, exact in both directions, factors
// out of every dot product.  It brings a bound on the magnitudes of the
// block it applies to below 2^15: no part can overflow FP16 (65504), and the
// lo parts stay normal (>= 2^-14) for every x 2^s >= 2^-3.

// 2^s with bound * 2^s < 2^15 (1 for a zero or non-finite bound)
__device__ __forceinline__ float f16_scale_for(float bound) {
  if (!(bound > 0.f) || bound > 3.0e38f) return 1.f;
  int e;
  frexpf(bound, &e);  // bound < 2^e
  e = e < -100 ? -100 : e;
  return ldexpf(1.f, 15 - e);
}

__device__ __forceinline__ void split_f16(float x, __half& hi, __half& lo) {
  hi = __float2half_rn(x);
  lo = __float2half_rn(x - __half2float(hi));
}

// four consecutive values of a scaled row, split: 8-byte stores of 4 halves
__device__ __forceinline__ void st_split4_f16(__half* hi, __half* lo, const float* v, float sc) {
  __align__(8) __half h[4], l[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) split_f16(v[c] * sc, h[c], l[c]);
  *reinterpret_cast<uint2*>(hi) = *reinterpret_cast<const uint2*>(h);
  *reinterpret_cast<uint2*>(lo) = *reinterpret_cast<const uint2*>(l);
}

}  // namespace gbdp
