// fft_reg.cuh -- register-resident line FFTs for power-of-two lines (sm_103a).
//
// A line of N = R1 * TPL complex points is held by TPL consecutive lanes of
// one warp, R1 points per lane, so a whole 1D transform costs one in-warp
// shared-memory exchange and no block barrier.  Two register distributions
// are used:
//   D_in : lane t holds x[t + TPL*m],               m  = 0..R1-1
//   D_out: lane u holds X[(u + TPL*g) + R1*k2],      g  = 0..G-1, k2 = 0..TPL-1
// (G = R1/TPL).  forward() maps D_in -> D_out and inverse() maps D_out ->
// D_in, so a forward/pointwise/inverse sequence never reorders data: the
// index of every element is known from (lane, register) and the k-space
// factor is applied in place.
//
// Decomposition (n = n1 + TPL*n2, k = k1 + R1*k2):
//   X[k1 + R1 k2] = sum_{n1} W_TPL^{n1 k2} [ W_N^{n1 k1} sum_{n2} x[n1 + TPL n2] W_R1^{n2 k1} ]
#pragma once
#include "fft.cuh"

#define K_C8 0.92387953251128675613   /* cos(pi/8) */
#define K_S8 0.38268343236508977173   /* sin(pi/8) */

// v * W16^m, W16 = exp(-i sg 2 pi / 16); m is a compile-time constant after unrolling
template <typename T>
__device__ __forceinline__ cplx<T> tw16(cplx<T> v, int m, int sg) {
  const T c8 = (T)K_C8, s8 = (T)K_S8, h = (T)K_SQRT1_2;
  T c, s;  // W = c - i sg s
  switch (m & 15) {
    case 0: return v;
    case 1: c = c8; s = s8; break;
    case 2: c = h; s = h; break;
    case 3: c = s8; s = c8; break;
    case 4: return mul_mi<T>(v, sg);
    case 6: c = -h; s = h; break;
    case 9: c = -c8; s = -s8; break;
    default: return v;  // n1*k2 of the 4x4 split is one of the cases above
  }
  // (vx + i vy)(c - i sg s)
  return mk<T>(v.x * c + sg * v.y * s, v.y * c - sg * v.x * s);
}

template <typename T>
__device__ __forceinline__ void dft16(cplx<T>* v, int sg) {
  cplx<T> a[4][4];  // a[n1][k2]
#pragma unroll
  for (int n1 = 0; n1 < 4; ++n1) {
    cplx<T> t[4] = {v[n1], v[n1 + 4], v[n1 + 8], v[n1 + 12]};
    dft4<T>(t, sg);
#pragma unroll
    for (int k2 = 0; k2 < 4; ++k2) a[n1][k2] = tw16<T>(t[k2], n1 * k2, sg);
  }
#pragma unroll
  for (int k2 = 0; k2 < 4; ++k2) {
    cplx<T> t[4] = {a[0][k2], a[1][k2], a[2][k2], a[3][k2]};
    dft4<T>(t, sg);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) v[k2 + 4 * k1] = t[k1];
  }
}


// v * W_R^m, W_R = exp(-i sg 2 pi / R), for the composite DFTs of 12 and 20
// points (m compile-time after unrolling; cos and sin of 2 pi m / R from
// their closed forms)
template <typename T, int R>
__device__ __forceinline__ cplx<T> twr(cplx<T> v, int m, int sg) {
  constexpr double h = K_SQRT3_2;
  constexpr double c12[10] = {1.0, h, 0.5, 0.0, -0.5, -h, -1.0, -h, -0.5, 0.0};
  constexpr double s12[10] = {0.0, 0.5, h, 1.0, h, 0.5, 0.0, -0.5, -h, -1.0};
  // angles of 18 degrees: cos 18 = sin 72, cos 36 = -cos 144, ...
  constexpr double c20[13] = {1.0, K_S5_1, -K_C5_2, K_S5_2, K_C5_1, 0.0, -K_C5_1,
                              -K_S5_2, K_C5_2, -K_S5_1, -1.0, -K_S5_1, K_C5_2};
  constexpr double s20[13] = {0.0, K_C5_1, K_S5_2, -K_C5_2, K_S5_1, 1.0, K_S5_1,
                              -K_C5_2, K_S5_2, K_C5_1, 0.0, -K_C5_1, -K_S5_2};
  if (m == 0) return v;
  const T c = (T)(R == 12 ? c12[m] : c20[m]);
  const T s = (T)(R == 12 ? s12[m] : s20[m]);
  return mk<T>(v.x * c + sg * v.y * s, v.y * c - sg * v.x * s);
}

template <typename T, int R>
__device__ __forceinline__ void dft_c(cplx<T>* v, int sg);

// R = P Q points, natural order in and out (Cooley-Tukey: n = n1 + P n2,
// k = k2 + Q k1): Q-point DFTs over n2, twiddles W_R^(n1 k2), P-point DFTs
// over n1
template <typename T, int P, int Q>
__device__ __forceinline__ void dft_pq(cplx<T>* v, int sg) {
  cplx<T> a[P][Q];
#pragma unroll
  for (int n1 = 0; n1 < P; ++n1) {
    cplx<T> t[Q];
#pragma unroll
    for (int n2 = 0; n2 < Q; ++n2) t[n2] = v[n1 + P * n2];
    dft_c<T, Q>(t, sg);
#pragma unroll
    for (int k2 = 0; k2 < Q; ++k2) a[n1][k2] = twr<T, P * Q>(t[k2], n1 * k2, sg);
  }
#pragma unroll
  for (int k2 = 0; k2 < Q; ++k2) {
    cplx<T> t[P];
#pragma unroll
    for (int n1 = 0; n1 < P; ++n1) t[n1] = a[n1][k2];
    dft_c<T, P>(t, sg);
#pragma unroll
    for (int k1 = 0; k1 < P; ++k1) v[k2 + Q * k1] = t[k1];
  }
}

template <typename T, int R>
__device__ __forceinline__ void dft_c(cplx<T>* v, int sg) {
  if constexpr (R == 4) dft4<T>(v, sg);
  else if constexpr (R == 8) dft8<T>(v, sg);
  else if constexpr (R == 16) dft16<T>(v, sg);
  else if constexpr (R == 2) dft2<T>(v);
  else if constexpr (R == 3) dft3<T>(v, sg);
  else if constexpr (R == 5) dft5<T>(v, sg);
  else if constexpr (R == 12) dft_pq<T, 4, 3>(v, sg);
  else if constexpr (R == 20) dft_pq<T, 4, 5>(v, sg);
  else static_assert(R == 4, "no register DFT of this size");
}

template <typename T, int R1_, int TPL_>
struct RegFFT {
  static constexpr int R1 = R1_;
  static constexpr int TPL = TPL_;
  static constexpr int N = R1 * TPL;
  static constexpr int G = R1 / TPL;
  static constexpr int PITCH = TPL + 1;
  // scratch per line (complex elements): rows k1 of pitch TPL+1, padded so
  // consecutive lines start half a bank cycle apart
  static constexpr int LS = ((R1 * PITCH + 15) / 16) * 16 + 8;
  static_assert(R1 % TPL == 0, "R1 must be a multiple of TPL");

  // forward: v in D_in (lane t), out in D_out (lane t plays u)
  __device__ __forceinline__ static void forward(cplx<T> (&v)[R1], cplx<T>* sc,
                                                 const cplx<T>* tw, int t) {
    dft_c<T, R1>(v, +1);
#pragma unroll
    for (int k1 = 1; k1 < R1; ++k1)
      if (t) v[k1] = cmul<T>(v[k1], tw[t * k1]);
    __syncwarp();
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1) sc[k1 * PITCH + t] = v[k1];
    __syncwarp();
#pragma unroll
    for (int g = 0; g < G; ++g) {
#pragma unroll
      for (int n1 = 0; n1 < TPL; ++n1) v[g * TPL + n1] = sc[(t + TPL * g) * PITCH + n1];
      dft_c<T, TPL>(&v[g * TPL], +1);
    }
  }

  // inverse: v in D_out, out in D_in (unnormalised)
  __device__ __forceinline__ static void inverse(cplx<T> (&v)[R1], cplx<T>* sc,
                                                 const cplx<T>* tw, int t) {
#pragma unroll
    for (int g = 0; g < G; ++g) {
      dft_c<T, TPL>(&v[g * TPL], -1);
      const int k1 = t + TPL * g;
#pragma unroll
      for (int n1 = 1; n1 < TPL; ++n1)
        if (k1) v[g * TPL + n1] = cmulc<T>(v[g * TPL + n1], tw[n1 * k1]);
    }
    __syncwarp();
#pragma unroll
    for (int g = 0; g < G; ++g)
#pragma unroll
      for (int n1 = 0; n1 < TPL; ++n1) sc[(t + TPL * g) * PITCH + n1] = v[g * TPL + n1];
    __syncwarp();
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1) v[k1] = sc[k1 * PITCH + t];
    dft_c<T, R1>(v, -1);
  }

  // element index of register r in each distribution
  __device__ __forceinline__ static int in_index(int t, int r) { return t + TPL * r; }
  __device__ __forceinline__ static int out_index(int t, int r) {
    return (t + TPL * (r / TPL)) + R1 * (r % TPL);
  }
};
