// common.cuh -- device helpers shared by the SCF kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

template <typename T> struct Cplx;
template <> struct Cplx<float> { using type = float2; };
template <> struct Cplx<double> { using type = double2; };
template <typename T> using cplx = typename Cplx<T>::type;

template <typename T> __host__ __device__ __forceinline__ cplx<T> mk(T x, T y) {
  cplx<T> r; r.x = x; r.y = y; return r;
}
template <typename T> __device__ __forceinline__ cplx<T> cadd(cplx<T> a, cplx<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ cplx<T> csub(cplx<T> a, cplx<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <typename T> __device__ __forceinline__ cplx<T> cmul(cplx<T> a, cplx<T> b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename T> __device__ __forceinline__ cplx<T> cmulc(cplx<T> a, cplx<T> b) {
  return mk<T>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename T> __device__ __forceinline__ cplx<T> cscale(cplx<T> a, T s) { return mk<T>(a.x * s, a.y * s); }
// multiply by -i*sg  (sg = +1 forward, -1 inverse)
template <typename T> __device__ __forceinline__ cplx<T> mul_mi(cplx<T> a, int sg) {
  return sg > 0 ? mk<T>(a.y, -a.x) : mk<T>(-a.y, a.x);
}

// ---- deterministic block reductions -----------------------------------
// Sum K doubles across a block of `blockDim.x` threads (multiple of 32).
// Result valid in threads 0..K-1 (value for index = threadIdx.x).
template <int K>
__device__ __forceinline__ double block_reduce_k(double (&v)[K], double* sm /* >= K*32 */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double x = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sm[k * 32 + warp] = x;
  }
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < K) {
    for (int w = 0; w < nw; ++w) r += sm[threadIdx.x * 32 + w];
  }
  __syncthreads();
  return r;
}

__device__ __forceinline__ double block_reduce_1(double v, double* sm) {
  double a[1] = {v};
  return block_reduce_k<1>(a, sm);
}

// e^a for the Boltzmann factor exp(-ds w / 2).  Its argument is small (|a| is
// ds/2 times the field), so the Taylor series sum_k a^k / k! to k = 12 has a
// truncation error below 1e-20 for |a| <= 1/8 (the result is within FP64
// rounding, ~2e-16 relative) and costs 12 FP64 FMAs; larger arguments fall
// back to exp().
__device__ __forceinline__ double exp_boltzmann(double a) {
  if (fabs(a) > 0.125) return exp(a);
  double p = 1.0 / 479001600.0;                 // 1/12!
  p = fma(p, a, 1.0 / 39916800.0);              // 1/11!
  p = fma(p, a, 1.0 / 3628800.0);               // 1/10!
  p = fma(p, a, 1.0 / 362880.0);                // 1/9!
  p = fma(p, a, 1.0 / 40320.0);                 // 1/8!
  p = fma(p, a, 1.0 / 5040.0);                  // 1/7!
  p = fma(p, a, 1.0 / 720.0);                   // 1/6!
  p = fma(p, a, 1.0 / 120.0);                   // 1/5!
  p = fma(p, a, 1.0 / 24.0);                    // 1/4!
  p = fma(p, a, 1.0 / 6.0);                     // 1/3!
  p = fma(p, a, 0.5);                           // 1/2!
  p = fma(p, a, 1.0);
  return fma(p, a, 1.0);
}

// e^a as an unevaluated pair of floats hi + lo (|lo| <= ulp(hi)/2), for the
// split path's Boltzmann factors, which are stored as exactly such a pair.
// a = ah + al in floats; e^ah by the Taylor series to k = 9 (truncation below
// 3e-16 for |a| <= 1/8) in float-float Horner form (products split by FMA,
// sums by Knuth's TwoSum, every operation explicitly rounded so the compiler
// cannot contract them), times (1 + al).  Relative error about 2^-47 (an FP32
// emulation over |a| <= 1/8 gives 6e-15), on the FP32 pipe: the FP64 series
// keeps GB300's narrow FP64 pipe busy.  Larger |a| falls back to FP64 exp().
__device__ __forceinline__ void exp_ff(double a, float& hi, float& lo) {
  if (fabs(a) > 0.125) {
    const double e = exp(a);
    hi = (float)e;
    lo = (float)(e - (double)hi);
    return;
  }
  constexpr double c[10] = {1.0, 1.0, 1.0 / 2, 1.0 / 6, 1.0 / 24, 1.0 / 120, 1.0 / 720, 1.0 / 5040,
                            1.0 / 40320, 1.0 / 362880};
  const float ah = (float)a;
  const float al = (float)(a - (double)ah);
  float ph = (float)c[9], pl = (float)(c[9] - (double)(float)c[9]);
#pragma unroll
  for (int k = 8; k >= 0; --k) {
    const float t = __fmul_rn(ph, ah);
    float e = __fmaf_rn(ph, ah, -t);
    e = __fmaf_rn(pl, ah, e);
    const float ch = (float)c[k], cl = (float)(c[k] - (double)(float)c[k]);
    const float s = __fadd_rn(t, ch);
    const float bb = __fsub_rn(s, t);
    float err = __fadd_rn(__fsub_rn(t, __fsub_rn(s, bb)), __fsub_rn(ch, bb));
    err = __fadd_rn(err, __fadd_rn(e, cl));
    ph = __fadd_rn(s, err);
    pl = __fsub_rn(err, __fsub_rn(ph, s));
  }
  const float e = __fmaf_rn(ph, al, pl);
  hi = __fadd_rn(ph, e);
  lo = __fsub_rn(e, __fsub_rn(hi, ph));
}
