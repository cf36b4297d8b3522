// jfem_df.cuh — double-float ("float-float") arithmetic on the FP32 pipe.
//
// GB300 executes FP64 at about 1/64 of its FP32 rate, so the PCG vector updates
// and dot products of the mixed-precision solver, a handful of FP64 operations
// per DOF, are FP64-pipe-bound when written in double.  They run instead on
// unevaluated pairs (hi, lo) of floats with |lo| ≤ ulp(hi)/2: a 48-bit
// significand (relative rounding ≈ 2⁻⁴⁸ ≈ 3.6e-15) in the FP32 exponent range,
// stored in HBM as float2 (8 bytes, as a double).
//
// Building blocks (published algorithms, written here with the round-to-nearest
// intrinsics so the compiler neither contracts nor reorders them):
//   TwoSum (Knuth), Fast2Sum (Dekker), TwoProd by FMA;
//   double-word + double-word, × float and × double-word as in Joldes, Muller &
//   Popescu, "Tight and rigorous error bounds for basic building blocks of
//   double-word arithmetic", ACM TOMS 44(2), 2017: AccurateDWPlusDW (rel. error
//   ≤ 3u²), DWTimesFP3 (≤ 2u²), DWTimesDW2 (≤ 5u²), u = 2⁻²⁴.
// Conversions to and from double use the FP64 pipe and are kept off the
// per-iteration path.
#pragma once

#include <cuda_runtime.h>

namespace jfem {

__device__ __forceinline__ float2 df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return make_float2(s, e);
}

// requires |a| ≥ |b| (or a = 0)
__device__ __forceinline__ float2 df_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return make_float2(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ float2 df_two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return make_float2(p, __fmaf_rn(a, b, -p));
}

__device__ __forceinline__ float2 df_add(float2 x, float2 y) {
  const float2 s = df_two_sum(x.x, y.x);
  const float2 t = df_two_sum(x.y, y.y);
  const float2 v = df_fast_two_sum(s.x, __fadd_rn(s.y, t.x));
  return df_fast_two_sum(v.x, __fadd_rn(t.y, v.y));
}

// Dekker's double-word sum (SloppyDWPlusDW): TwoSum of the high parts, the low
// parts added in FP32, one Fast2Sum.  Its error is bounded in absolute terms,
// ≈ 2u²(|x| + |y|), not relative to the result (no bound under cancellation):
// for sums judged against the size of their terms, e.g. matrix entries
// compared relative to max |K|, the dot products of the solvers, whose
// per-thread sums of a few terms then meet FP64 block sums (error ≈ 2u² of the
// summed magnitudes per term, FP64-class), and the updates of the correction
// δx and of the search direction p (errors ≈ 2u² of |δx| or |p|, where FP32
// operators already perturb far more; the residual update r −= αq, which
// cancels, keeps df_add).  11 operations against 20 for df_add.
__device__ __forceinline__ float2 df_add_abs(float2 x, float2 y) {
  const float2 s = df_two_sum(x.x, y.x);
  return df_fast_two_sum(s.x, __fadd_rn(s.y, __fadd_rn(x.y, y.y)));
}

// x·y for a dot-product sum: hi·y exactly (TwoProd) plus lo·y in FP32, left
// unnormalised (the next df_add_abs renormalises); 3 operations.
__device__ __forceinline__ float2 df_dot_term(float2 x, float y) {
  const float2 p = df_two_prod(x.x, y);
  return make_float2(p.x, __fmaf_rn(x.y, y, p.y));
}

__device__ __forceinline__ float2 df_mul_f(float2 x, float y) {
  const float2 p = df_two_prod(x.x, y);
  return df_fast_two_sum(p.x, __fmaf_rn(x.y, y, p.y));
}

__device__ __forceinline__ float2 df_mul(float2 x, float2 y) {
  const float2 p = df_two_prod(x.x, y.x);
  const float t = __fmaf_rn(x.y, y.x, __fmul_rn(x.x, y.y));
  return df_fast_two_sum(p.x, __fadd_rn(p.y, t));
}

__device__ __forceinline__ float2 df_neg(float2 x) { return make_float2(-x.x, -x.y); }

// FP64 pipe (off the hot loop)
__host__ __device__ __forceinline__ float2 df_from_double(double d) {
  const float hi = (float)d;
  return make_float2(hi, (float)(d - (double)hi));
}
__host__ __device__ __forceinline__ double df_to_double(float2 a) { return (double)a.x + (double)a.y; }

// Block-wide deterministic sum of double-float values, returned as a double to
// every thread: warps combine by shuffles in double-float, the (≤ 32) warp sums
// are converted once and added in FP64 in warp order.  blockDim.x multiple of 32.
__device__ __forceinline__ double block_sum_df(float2 v, double* sh /* ≥ 32 entries */) {
  for (int o = 16; o > 0; o >>= 1) {
    const float2 w = make_float2(__shfl_down_sync(0xffffffffu, v.x, o), __shfl_down_sync(0xffffffffu, v.y, o));
    v = df_add(v, w);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = df_to_double(v);
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sh[k];
    sh[0] = s;
  }
  __syncthreads();
  const double r = sh[0];
  __syncthreads();
  return r;
}

// Two block sums in one pass (same order per value as block_sum_df; ≤ 16 warps).
__device__ __forceinline__ double2 block_sum2_df(float2 u, float2 v, double* sh /* ≥ 32 entries */) {
  for (int o = 16; o > 0; o >>= 1) {
    const float2 wu = make_float2(__shfl_down_sync(0xffffffffu, u.x, o), __shfl_down_sync(0xffffffffu, u.y, o));
    const float2 wv = make_float2(__shfl_down_sync(0xffffffffu, v.x, o), __shfl_down_sync(0xffffffffu, v.y, o));
    u = df_add(u, wu);
    v = df_add(v, wv);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) {
    sh[w] = df_to_double(u);
    sh[16 + w] = df_to_double(v);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0, t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      s += sh[k];
      t += sh[16 + k];
    }
    sh[0] = s;
    sh[16] = t;
  }
  __syncthreads();
  const double2 r = make_double2(sh[0], sh[16]);
  __syncthreads();
  return r;
}

// "Last block" detection for a fixed-order grid reduction without a second
// launch: each block publishes its partial, fences, and counts itself in; the
// block that arrives last (every partial is then visible) reduces all partials
// in index order and resets the counter.  Nothing waits on another block.
// Call with the block's partial already written by thread 0.
__device__ __forceinline__ bool arrive_last(unsigned* counter) {
  __shared__ int last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = (atomicAdd(counter, 1u) == gridDim.x - 1) ? 1 : 0;
  }
  __syncthreads();
  if (last) __threadfence();
  return last != 0;
}

// Fixed-order sum of n partials read past L1 (they were written by other
// blocks of the same launch).
__device__ __forceinline__ double reduce_partials_cg(const double* part, int n, double* sh) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += __ldcg(part + i);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sh[k];
    sh[0] = t;
  }
  __syncthreads();
  const double r = sh[0];
  __syncthreads();
  return r;
}

// Two fixed-order sums of n partials each in one pass (same order per value as
// reduce_partials_cg; ≤ 16 warps).
__device__ __forceinline__ double2 reduce_partials2_cg(const double* a, const double* b, int n, double* sh) {
  double s = 0.0, t = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    s += __ldcg(a + i);
    t += __ldcg(b + i);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_down_sync(0xffffffffu, s, o);
    t += __shfl_down_sync(0xffffffffu, t, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) {
    sh[w] = s;
    sh[16 + w] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double u = 0.0, v = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      u += sh[k];
      v += sh[16 + k];
    }
    sh[0] = u;
    sh[16] = v;
  }
  __syncthreads();
  const double2 r = make_double2(sh[0], sh[16]);
  __syncthreads();
  return r;
}

}  // namespace jfem
