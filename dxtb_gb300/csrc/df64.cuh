// Double-float ("df64") arithmetic: a value is an unevaluated sum hi + lo
// of two FP32 numbers with |lo| <= ulp(hi) / 2, about 48 significant bits.
//
// This GPU retires 128 FP32 FMAs per clock per SM but only 2 FP64 FMAs, so
// an FP64-bound inner loop runs several times faster when its arithmetic is
// carried out in pairs of FP32 numbers.  The operations below are the
// classical error-free transformations (Knuth's two-sum, the FMA-based
// exact product; Dekker 1971, Shewchuk 1997) composed into accurate
// additions and products; relative error per operation ~2^-47.  They rely
// on IEEE FP32 rounding with no reassociation (no fast-math).
#pragma once

#include <cuda_runtime.h>

namespace gbxtb {

struct __align__(8) df64 {
  float hi, lo;
  df64() = default;
  __host__ __device__ constexpr df64(float h, float l = 0.f) : hi(h), lo(l) {}
};

// s + e = a + b exactly (Knuth)
__device__ __forceinline__ df64 df_two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return df64(s, (a - (s - bb)) + (b - bb));
}

// p + e = a * b exactly
__device__ __forceinline__ df64 df_two_prod(float a, float b) {
  const float p = a * b;
  return df64(p, fmaf(a, b, -p));
}

__device__ __forceinline__ df64 df_from_double(double x) {
  const float h = __double2float_rn(x);
  return df64(h, __double2float_rn(x - (double)h));
}

__device__ __forceinline__ double df_to_double(df64 a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ df64 df_neg(df64 a) { return df64(-a.hi, -a.lo); }

// a + b, accurate also under cancellation
__device__ __forceinline__ df64 df_add(df64 a, df64 b) {
  const df64 s = df_two_sum(a.hi, b.hi);
  const df64 t = df_two_sum(a.lo, b.lo);
  const df64 u = df_two_sum(s.hi, s.lo + t.hi);
  return df_two_sum(u.hi, u.lo + t.lo);
}

__device__ __forceinline__ df64 df_mul(df64 a, df64 b) {
  const df64 p = df_two_prod(a.hi, b.hi);
  return df_two_sum(p.hi, fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, p.lo)));
}

// a - v_i w_j - w_i v_j (the rank-2 update of one matrix element): both
// leading products exact, the cross terms in FP32
__device__ __forceinline__ df64 df_rank2(df64 a, df64 vi, df64 wj, df64 wi, df64 vj) {
  const df64 p1 = df_two_prod(vi.hi, wj.hi);
  const df64 p2 = df_two_prod(wi.hi, vj.hi);
  const float c = fmaf(vi.hi, wj.lo, fmaf(vi.lo, wj.hi, fmaf(wi.hi, vj.lo, wi.lo * vj.hi)));
  const df64 s1 = df_two_sum(a.hi, -p1.hi);
  const df64 s2 = df_two_sum(s1.hi, -p2.hi);
  const float lo = (a.lo + (s1.lo + s2.lo)) - ((p1.lo + p2.lo) + c);
  return df_two_sum(s2.hi, lo);
}

// Running dot product: hi carries the sum, lo the rounding errors and the
// low-order product terms, renormalised once at the end (df_dot_final).
struct DfAcc {
  float hi = 0.f, lo = 0.f;
};

__device__ __forceinline__ void df_dot_add(DfAcc &acc, df64 a, df64 b) {
  const df64 p = df_two_prod(a.hi, b.hi);
  const float c = fmaf(a.hi, b.lo, a.lo * b.hi);
  const df64 s = df_two_sum(acc.hi, p.hi);
  acc.hi = s.hi;
  acc.lo += s.lo + (p.lo + c);
}

__device__ __forceinline__ df64 df_dot_final(const DfAcc &acc) { return df_two_sum(acc.hi, acc.lo); }

__device__ __forceinline__ df64 df_shfl_xor(df64 a, int off) {
  return df64(__shfl_xor_sync(0xffffffffu, a.hi, off), __shfl_xor_sync(0xffffffffu, a.lo, off));
}

__device__ __forceinline__ df64 df_shfl(df64 a, int src) {
  return df64(__shfl_sync(0xffffffffu, a.hi, src), __shfl_sync(0xffffffffu, a.lo, src));
}

}  // namespace gbxtb
