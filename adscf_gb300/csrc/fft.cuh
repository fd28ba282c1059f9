// fft.cuh -- batched shared-memory Stockham FFT lines for the bulk propagator.
//
// A CTA holds LPC lines of length N in shared memory; TPL threads work on
// one line.  Each stage is a radix-R (R in {2,3,4,5,8}) butterfly of the
// Stockham autosort form: input and output stay in natural order, so the
// k-space factor exp(-k^2 ds) can be applied from plain indices.  Twiddles
// W_N^m come from a host-made FP64 table rounded to T.
#pragma once
#include "common.cuh"

#define ADSCF_MAX_STAGES 8

struct Plan1D {
  int n;                      // line length
  int nst;                    // number of stages (0 for n == 1)
  int tpl;                    // threads per line
  int lpc;                    // lines per CTA (256 / tpl)
  int ld;                     // shared-memory line pitch (elements)
  int tw_off;                 // offset of W_n^m (m < n) in the twiddle table
  int rad[ADSCF_MAX_STAGES];  // radices, first stage first
};

// fixed constants of the small DFTs (values of cos/sin at rational
// multiples of pi, written out from their closed forms)
#define K_SQRT1_2 0.70710678118654752440
#define K_SQRT3_2 0.86602540378443864676
#define K_C5_1 0.30901699437494742410   /* cos(2 pi/5) = (sqrt5-1)/4 */
#define K_C5_2 -0.80901699437494742410  /* cos(4 pi/5) = -(sqrt5+1)/4 */
#define K_S5_1 0.95105651629515357212   /* sin(2 pi/5) */
#define K_S5_2 0.58778525229247312917   /* sin(4 pi/5) */

// in-register DFT of size R; sg = +1 forward (exp(-2 pi i nk/R)), -1 inverse
template <typename T>
__device__ __forceinline__ void dft2(cplx<T>* v) {
  cplx<T> a = v[0], b = v[1];
  v[0] = cadd<T>(a, b); v[1] = csub<T>(a, b);
}

template <typename T>
__device__ __forceinline__ void dft4(cplx<T>* v, int sg) {
  cplx<T> t0 = cadd<T>(v[0], v[2]), t1 = csub<T>(v[0], v[2]);
  cplx<T> t2 = cadd<T>(v[1], v[3]), t3 = mul_mi<T>(csub<T>(v[1], v[3]), sg);
  v[0] = cadd<T>(t0, t2); v[2] = csub<T>(t0, t2);
  v[1] = cadd<T>(t1, t3); v[3] = csub<T>(t1, t3);
}

template <typename T>
__device__ __forceinline__ void dft8(cplx<T>* v, int sg) {
  cplx<T> e[4] = {v[0], v[2], v[4], v[6]};
  cplx<T> o[4] = {v[1], v[3], v[5], v[7]};
  dft4<T>(e, sg); dft4<T>(o, sg);
  const T h = (T)K_SQRT1_2;
  // o[k] *= W8^k  (W8 = exp(-i sg pi/4))
  cplx<T> o1 = o[1], o3 = o[3];
  o[1] = mk<T>(h * (o1.x + sg * o1.y), h * (o1.y - sg * o1.x));
  o[2] = mul_mi<T>(o[2], sg);
  o[3] = mk<T>(h * (-o3.x + sg * o3.y), h * (-o3.y - sg * o3.x));
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = cadd<T>(e[k], o[k]);
    v[k + 4] = csub<T>(e[k], o[k]);
  }
}

template <typename T>
__device__ __forceinline__ void dft3(cplx<T>* v, int sg) {
  const T c = (T)K_SQRT3_2;
  cplx<T> t1 = cadd<T>(v[1], v[2]), t2 = csub<T>(v[1], v[2]);
  cplx<T> m = mk<T>(v[0].x - (T)0.5 * t1.x, v[0].y - (T)0.5 * t1.y);
  cplx<T> r = mul_mi<T>(cscale<T>(t2, c), sg);
  v[0] = cadd<T>(v[0], t1);
  v[1] = cadd<T>(m, r);
  v[2] = csub<T>(m, r);
}

template <typename T>
__device__ __forceinline__ void dft5(cplx<T>* v, int sg) {
  const T c1 = (T)K_C5_1, c2 = (T)K_C5_2, s1 = (T)K_S5_1, s2 = (T)K_S5_2;
  cplx<T> b1 = cadd<T>(v[1], v[4]), b2 = cadd<T>(v[2], v[3]);
  cplx<T> d1 = csub<T>(v[1], v[4]), d2 = csub<T>(v[2], v[3]);
  cplx<T> a0 = v[0];
  cplx<T> m1 = mk<T>(a0.x + c1 * b1.x + c2 * b2.x, a0.y + c1 * b1.y + c2 * b2.y);
  cplx<T> m2 = mk<T>(a0.x + c2 * b1.x + c1 * b2.x, a0.y + c2 * b1.y + c1 * b2.y);
  cplx<T> n1 = mul_mi<T>(mk<T>(s1 * d1.x + s2 * d2.x, s1 * d1.y + s2 * d2.y), sg);
  cplx<T> n2 = mul_mi<T>(mk<T>(s2 * d1.x - s1 * d2.x, s2 * d1.y - s1 * d2.y), sg);
  v[0] = cadd<T>(a0, cadd<T>(b1, b2));
  v[1] = cadd<T>(m1, n1);
  v[4] = csub<T>(m1, n1);
  v[2] = cadd<T>(m2, n2);
  v[3] = csub<T>(m2, n2);
}

template <typename T>
__device__ __forceinline__ void dft_r(cplx<T>* v, int R, int sg) {
  switch (R) {
    case 2: dft2<T>(v); break;
    case 3: dft3<T>(v, sg); break;
    case 4: dft4<T>(v, sg); break;
    case 5: dft5<T>(v, sg); break;
    default: dft8<T>(v, sg); break;
  }
}

// Transform the line group of this CTA.  `a` holds the input (lines of
// pitch P.ld), `b` is scratch of the same size, `tw` the forward twiddle
// table W_N^m in shared memory.  All threads of the CTA must call this.
// Returns the buffer holding the result (a or b).
template <typename T>
__device__ cplx<T>* fft_lines(cplx<T>* a, cplx<T>* b, const cplx<T>* tw,
                              const Plan1D& P, int line, int lt, bool active,
                              int sg) {
  const int N = P.n;
  cplx<T>* src = a;
  cplx<T>* dst = b;
  int Ns = 1;
  for (int st = 0; st < P.nst; ++st) {
    const int R = P.rad[st];
    const int nb = N / R;
    const int stride = N / (Ns * R);
    if (active) {
      cplx<T>* s = src + line * P.ld;
      cplx<T>* d = dst + line * P.ld;
      for (int j = lt; j < nb; j += P.tpl) {
        const int k = j % Ns;
        cplx<T> v[8];
#pragma unroll
        for (int r = 0; r < 8; ++r)
          if (r < R) v[r] = s[j + r * nb];
#pragma unroll
        for (int r = 1; r < 8; ++r) {
          if (r < R && k != 0) {
            cplx<T> w = tw[r * k * stride];
            v[r] = sg > 0 ? cmul<T>(v[r], w) : cmulc<T>(v[r], w);
          }
        }
        dft_r<T>(v, R, sg);
        const int base = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int r = 0; r < 8; ++r)
          if (r < R) d[base + r * Ns] = v[r];
      }
    }
    __syncthreads();
    cplx<T>* t = src; src = dst; dst = t;
    Ns *= R;
  }
  return src;
}
