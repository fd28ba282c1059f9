// bulk_kernels.cuh -- pseudo-spectral diblock propagator on sm_103a.
//
// Reference: Propagate_Step (Bulk_3D_FFT/General_Routines/mod_propagate.f90:
// 40-68), Real2Fourier/Fourier2Real (Bulk_3D_FFT/Geometry_Modules/Bulk/
// mod_fourier.f90:75-105), Calculate_Laplace (:165-198) and the chain loops
// and contour integral of Propagate_Diblock (Bulk_3D_FFT/Polymer_Modules/
// mod_diblock.f90:116-154).
//
// Design.  The forward propagator q and the backward propagator q-dagger
// are real, and the diffusion factor exp(-k^2 ds) is real and even in k, so
// one complex 3D FFT of z = E_f q + i E_b q-dagger advances both chains by
// one contour step: IFFT(G FFT(z)) = IFFT(G FFT(E_f q)) + i IFFT(G FFT(E_b
// q-dagger)) exactly.  A "double step" t therefore produces contour node t of
// both chains, stored as one complex slice (q_t, q-dagger_t).  The 3D FFT
// is three line passes over an L2-resident spectrum buffer:
//   X(t)  : inverse x-FFT -> q_t = E(t) * z -> store slice t ->
//           z = E(t+1) * q_t -> forward x-FFT            (fused real space)
//   Yf(t) : forward y-FFT
//   Z(t)  : forward z-FFT -> * exp(-ds k^2)/N -> inverse z-FFT
//   Yi(t) : inverse y-FFT
// so the real-space Boltzmann factors, the slice store and the k-space
// factor never take an extra pass over memory.
#pragma once
#include "adscf.h"
#include "fft.cuh"

#define BULK_THREADS 256

template <typename T>
struct BulkDev {
  int gx, gy, gz;
  int npts;
  int ns, na, nb;            // contour steps, A-block steps (fwd), B-block steps (bwd)
  // linear block sequence (nblk > 0; 0 = the diblock of na / nb): block k
  // ends at contour node bend[k] and has monomer type bit k of btype; node
  // weights per type in wtab [ns+1] (trapezoid per block, summed by type)
  int nblk;
  int bend[ADSCF_MAX_BLOCKS];
  unsigned btype;
  const float2* wtab;
  Plan1D px, py, pz;
  // exp(-ds k^2) tables in `fk`: g_xy[gy*gx] (hi then lo), g_z[gz]/N (hi then
  // lo); lo parts are the FP32 rounding residues (zero in FP64)
  int gxy_off, gz_off;
  int tw64_off, g64_off;     // FP64 twiddles / factors of the (0,0) z pencil
  cplx<T>* spec;             // [npts] complex spectrum / work buffer
  cplx<T>* slices;           // [(ns+1)][npts] (q_t, qdag_t)
  T* E;                      // [npts] interleaved exp(-ds w/2) (see EPt)
  double* dist;              // [2][npts] contour integrals (block A, block B)
  double* qpart;             // [gridDim] partial sums of q_N
  double ds;                 // contour step
  int wait_polls;            // polls of one pipeline mbarrier wait of the TMA passes
};

// X-pass modes (XM_FROM: start a chain segment at node t from a stored
// state (q_t, qdag_t) in aux.in, as XM_INIT does from (1, 1) at node 0)
// (XM_C2S / XM_S2C: complex data in aux.in / aux.out, forward x FFT into
// the spectrum / inverse x FFT out of it, nothing else)
enum { XM_INIT = 0, XM_STEP = 1, XM_R2S = 2, XM_S2R = 3, XM_FROM = 4, XM_C2S = 5, XM_S2C = 6 };

struct XAux {
  const void* in;   // XM_R2S: real input [npts] (T); XM_FROM: state [npts] (cplx<T>)
  void* out;        // XM_S2R: real output [npts] (T)
  const void* e;    // XM_R2S / XM_S2R: real factor [npts] (T) or null
};

// z * (hi + lo) with one rounding: the FP32 residue of E keeps the Boltzmann
// factor exact to ~1e-14 so its rounding cannot bias every step the same way
__device__ __forceinline__ float emul(float z, float hi, float lo) { return fmaf(z, hi, z * lo); }
__device__ __forceinline__ double emul(double z, double hi, double) { return z * hi; }

// Boltzmann factors of one point, stored interleaved so one 16-byte (FP32)
// or 16-byte (FP64) load brings both species: FP32 keeps (A, B, A residue,
// B residue) as float4, FP64 keeps (A, B) as double2.  No kernel that reads
// them writes them, so they are read through the non-coherent path: the
// compiler may then issue these loads ahead of the slice stores that follow
// them (which it cannot prove do not alias).
template <typename T>
struct EPt { T a, b, al, bl; };
__device__ __forceinline__ EPt<float> load_ept(const float* E, size_t g) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(E) + g);
  return {v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ EPt<double> load_ept(const double* E, size_t g) {
  const double2 v = __ldg(reinterpret_cast<const double2*>(E) + g);
  return {v.x, v.y, 0.0, 0.0};
}
// the Boltzmann factor e^a of species c at point p: float-float on the split
// path (exp_ff), the FP64 series on the FP64 path
__device__ __forceinline__ void store_boltzmann(float* E, size_t p, int c, double a) {
  float h, l;
  exp_ff(a, h, l);
  E[4 * p + c] = h;
  E[4 * p + 2 + c] = l;
}
__device__ __forceinline__ void store_boltzmann(double* E, size_t p, int c, double a) {
  E[2 * p + c] = exp_boltzmann(a);
}

template <typename T>
__device__ __forceinline__ int seq_type(const BulkDev<T>& I, int t) {
  int k = 0;
  while (k < I.nblk - 1 && t > I.bend[k]) ++k;
  return (int)((I.btype >> k) & 1u);
}
// monomer type (0 A, 1 B) of step t (node t-1 -> t) of the forward chain,
// and of step t of the backward chain (forward step Ns + 1 - t)
template <typename T>
__device__ __forceinline__ int chain_type_fwd(const BulkDev<T>& I, int t) {
  return I.nblk ? seq_type(I, t) : (t <= I.na ? 0 : 1);
}
template <typename T>
__device__ __forceinline__ int chain_type_bwd(const BulkDev<T>& I, int t) {
  return I.nblk ? seq_type(I, I.ns + 1 - t) : (t <= I.nb ? 1 : 0);
}

// ---------------------------------------------------------------------------
// The (kx, ky) = (0, 0) z pencil carries the mean of both propagators; FP32
// rounding of it would be coherent over the whole box and accumulate over the
// contour.  Its forward z-FFT, factor exp(-ds kz^2)/N and inverse z-FFT are a
// circular convolution with the real kernel c(d) = sum_kz G(kz) cos(2 pi kz
// d / gz) (FP64 table), evaluated here in float-float arithmetic: exact
// products (TwoProd) and compensated sums (TwoSum), ~48-bit accurate on FP32
// units.  All threads of the block call dc_pencil_load / _apply / _store.
// ---------------------------------------------------------------------------
struct DcPencil {
  float2* in;    // [n] pencil before the pass (as loaded)
  float2* out;   // [n] convolved pencil
  float2* c;     // [n] kernel, (hi, lo) FP32 split of c(d)
};

template <typename T>
__device__ __forceinline__ void dc_pencil_load(const cplx<T>* spec, size_t es, int n,
                                               const double* c64, DcPencil D) {
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    const cplx<T> v = spec[(size_t)j * es];
    D.in[j] = make_float2((float)v.x, (float)v.y);
    const double c = c64[j];
    const float h = (float)c;
    D.c[j] = make_float2(h, (float)(c - (double)h));
  }
}

__device__ __forceinline__ void ff_fma(float& sh, float& sl, float ch, float cl, float x) {
  const float p = ch * x;
  const float e = fmaf(ch, x, -p) + cl * x;   // exact product plus the lo term
  const float s = sh + p;
  const float bb = s - sh;
  const float t = (sh - (s - bb)) + (p - bb) + sl + e;
  sh = s + t;
  sl = t - (sh - s);
}

// (ah, al) += (bh, bl) in float-float (TwoSum of the high parts)
__device__ __forceinline__ void ff_add(float& ah, float& al, float bh, float bl) {
  const float s = ah + bh;
  const float bb = s - ah;
  const float t = (ah - (s - bb)) + (bh - bb) + al + bl;
  ah = s + t;
  al = t - (ah - s);
}

// out[z] = sum_d c[d] in[z - d mod n] in float-float.  The pencil is one
// CTA's extra work in its pass, so its serial chain sets that CTA's finish:
// eight interleaved partial sums per output (chain u = d mod 8, each in
// increasing d) shorten the dependent chain eightfold, and are combined
// pairwise: ((0+1) + (2+3)) + ((4+5) + (6+7)).  In the fused plan the z
// pass's light CTAs evaluate the same sums with one lane per chain
// (dc_point) and get the same bits.
constexpr int kDcChains = 8;
__device__ __forceinline__ void dc_pencil_apply(int n, DcPencil D) {
  for (int z = threadIdx.x; z < n; z += blockDim.x) {
    float rh[kDcChains], rl[kDcChains], ih[kDcChains], il[kDcChains];
#pragma unroll
    for (int u = 0; u < kDcChains; ++u) rh[u] = rl[u] = ih[u] = il[u] = 0.f;
    for (int d0 = 0; d0 < n; d0 += kDcChains) {
#pragma unroll
      for (int u = 0; u < kDcChains; ++u) {
        const int d = d0 + u;
        if (d < n) {
          int zz = z - d;
          if (zz < 0) zz += n;
          const float2 p = D.in[zz];
          const float2 c = D.c[d];
          ff_fma(rh[u], rl[u], c.x, c.y, p.x);
          ff_fma(ih[u], il[u], c.x, c.y, p.y);
        }
      }
    }
#pragma unroll
    for (int st = 1; st < kDcChains; st *= 2)
#pragma unroll
      for (int u = 0; u < kDcChains; u += 2 * st) {
        ff_add(rh[u], rl[u], rh[u + st], rl[u + st]);
        ff_add(ih[u], il[u], ih[u + st], il[u + st]);
      }
    D.out[z] = make_float2(rh[0] + rl[0], ih[0] + il[0]);
  }
}

template <typename T>
__device__ __forceinline__ void dc_pencil_store(cplx<T>* spec, size_t es, int n, DcPencil D) {
  for (int j = threadIdx.x; j < n; j += blockDim.x)
    spec[(size_t)j * es] = mk<T>((T)D.out[j].x, (T)D.out[j].y);
}

// shared-memory carve-up for one pass: twiddles (N) + two line buffers
template <typename T>
__device__ __forceinline__ void carve(unsigned char* raw, const Plan1D& P, cplx<T>*& tw,
                                      cplx<T>*& b0, cplx<T>*& b1) {
  tw = reinterpret_cast<cplx<T>*>(raw);
  int twn = (P.n + 1) & ~1;
  b0 = tw + twn;
  b1 = b0 + P.lpc * P.ld;
}

template <typename T>
__device__ __forceinline__ void load_twiddles(cplx<T>* tw, const cplx<T>* gtw, const Plan1D& P) {
  for (int i = threadIdx.x; i < P.n; i += blockDim.x) tw[i] = gtw[P.tw_off + i];
}

// ---------------------------------------------------------------------------
// X pass: lines along x (contiguous rows).  work.y = row tile.
// ---------------------------------------------------------------------------
// One tile (LPC x-rows of instance w.x, tile w.y) of the X pass; every
// thread of the block calls it (shared memory `smraw` per plan_smem).
template <typename T>
__device__ __forceinline__ void xpass_tile(const BulkDev<T>* __restrict__ insts, const int2 w,
                                           const cplx<T>* __restrict__ gtw, int t, int mode, XAux aux,
                                           unsigned char* smraw) {
  const BulkDev<T> I = insts[w.x];
  if (mode == XM_STEP && t > I.ns) return;
  const Plan1D P = I.px;
  cplx<T> *tw, *b0, *b1;
  carve<T>(smraw, P, tw, b0, b1);
  load_twiddles<T>(tw, gtw, P);
  const int N = P.n, LPC = P.lpc;
  const int nrows = I.gy * I.gz;
  const int row0 = w.y * LPC;
  const int nl = min(LPC, nrows - row0);
  const size_t base = (size_t)row0 * N;
  const int tot = nl * N;
  const int line = threadIdx.x / P.tpl, lt = threadIdx.x % P.tpl;
  const bool active = line < nl;

  if (mode == XM_INIT) {
    // slice 0 = (1, 1); z = (E_f(1), E_b(1)) -> forward
    const bool fA = chain_type_fwd(I, 1) == 0, bA = chain_type_bwd(I, 1) == 0;
    cplx<T>* s0 = I.slices;
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
      const size_t g = base + e;
      s0[g] = mk<T>((T)1, (T)1);
      const EPt<T> ev = load_ept(I.E, g);
      b0[(e / N) * P.ld + (e % N)] = mk<T>(fA ? ev.a : ev.b, bA ? ev.a : ev.b);
    }
    __syncthreads();
    cplx<T>* r = fft_lines<T>(b0, b1, tw, P, line, lt, active, +1);
    for (int e = threadIdx.x; e < tot; e += blockDim.x)
      I.spec[base + e] = r[(e / N) * P.ld + (e % N)];
    return;
  }
  if (mode == XM_FROM) {
    // slice t = the stored state; z = (E_f(t+1) q_t, E_b(t+1) qdag_t) -> forward
    const bool fA = chain_type_fwd(I, t + 1) == 0, bA = chain_type_bwd(I, t + 1) == 0;
    const cplx<T>* st = static_cast<const cplx<T>*>(aux.in);
    cplx<T>* sl = I.slices + (size_t)t * I.npts;
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
      const size_t g = base + e;
      const cplx<T> q = st[g];
      sl[g] = q;
      const EPt<T> ev = load_ept(I.E, g);
      b0[(e / N) * P.ld + (e % N)] = mk<T>(q.x * (fA ? ev.a : ev.b), q.y * (bA ? ev.a : ev.b));
    }
    __syncthreads();
    cplx<T>* r = fft_lines<T>(b0, b1, tw, P, line, lt, active, +1);
    for (int e = threadIdx.x; e < tot; e += blockDim.x)
      I.spec[base + e] = r[(e / N) * P.ld + (e % N)];
    return;
  }
  if (mode == XM_C2S) {
    const cplx<T>* in = static_cast<const cplx<T>*>(aux.in);
    for (int e = threadIdx.x; e < tot; e += blockDim.x) b0[(e / N) * P.ld + (e % N)] = in[base + e];
    __syncthreads();
    cplx<T>* r = fft_lines<T>(b0, b1, tw, P, line, lt, active, +1);
    for (int e = threadIdx.x; e < tot; e += blockDim.x)
      I.spec[base + e] = r[(e / N) * P.ld + (e % N)];
    return;
  }
  if (mode == XM_R2S) {
    const T* in = static_cast<const T*>(aux.in);
    const T* ee = static_cast<const T*>(aux.e);
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
      const size_t g = base + e;
      T v = in[g];
      if (ee) v *= ee[g];
      b0[(e / N) * P.ld + (e % N)] = mk<T>(v, (T)0);
    }
    __syncthreads();
    cplx<T>* r = fft_lines<T>(b0, b1, tw, P, line, lt, active, +1);
    for (int e = threadIdx.x; e < tot; e += blockDim.x)
      I.spec[base + e] = r[(e / N) * P.ld + (e % N)];
    return;
  }
  // XM_STEP / XM_S2R: inverse x-FFT of the spectrum rows first
  for (int e = threadIdx.x; e < tot; e += blockDim.x)
    b0[(e / N) * P.ld + (e % N)] = I.spec[base + e];
  __syncthreads();
  cplx<T>* r = fft_lines<T>(b0, b1, tw, P, line, lt, active, -1);
  cplx<T>* o = (r == b0) ? b1 : b0;
  if (mode == XM_S2R) {
    T* out = static_cast<T*>(aux.out);
    const T* ee = static_cast<const T*>(aux.e);
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
      const size_t g = base + e;
      T v = r[(e / N) * P.ld + (e % N)].x;
      if (ee) v *= ee[g];
      out[g] = v;
    }
    return;
  }
  if (mode == XM_S2C) {
    cplx<T>* out = static_cast<cplx<T>*>(aux.out);
    for (int e = threadIdx.x; e < tot; e += blockDim.x) out[base + e] = r[(e / N) * P.ld + (e % N)];
    return;
  }
  // contour node t of both chains (A or B factor per chain and step)
  const bool fA = chain_type_fwd(I, t) == 0, bA = chain_type_bwd(I, t) == 0;
  const bool more = t < I.ns;
  const bool fA2 = chain_type_fwd(I, t + 1) == 0, bA2 = chain_type_bwd(I, t + 1) == 0;
  cplx<T>* sl = I.slices + (size_t)t * I.npts;
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    const size_t g = base + e;
    const int si = (e / N) * P.ld + (e % N);
    const cplx<T> z = r[si];
    const EPt<T> ev = load_ept(I.E, g);
    const cplx<T> q = mk<T>(emul(z.x, fA ? ev.a : ev.b, fA ? ev.al : ev.bl),
                            emul(z.y, bA ? ev.a : ev.b, bA ? ev.al : ev.bl));
    sl[g] = q;
    if (more)
      o[si] = mk<T>(emul(q.x, fA2 ? ev.a : ev.b, fA2 ? ev.al : ev.bl),
                    emul(q.y, bA2 ? ev.a : ev.b, bA2 ? ev.al : ev.bl));
  }
  if (!more) return;
  __syncthreads();
  cplx<T>* r2 = fft_lines<T>(o, r, tw, P, line, lt, active, +1);
  for (int e = threadIdx.x; e < tot; e += blockDim.x)
    I.spec[base + e] = r2[(e / N) * P.ld + (e % N)];
}

template <typename T>
__global__ void __launch_bounds__(BULK_THREADS)
k_bulk_xpass(const BulkDev<T>* __restrict__ insts, const int2* __restrict__ work,
             const cplx<T>* __restrict__ gtw, int t, int mode, XAux aux) {
  extern __shared__ __align__(16) unsigned char smraw[];
  xpass_tile<T>(insts, work[blockIdx.x], gtw, t, mode, aux, smraw);
}

// ---------------------------------------------------------------------------
// Y / Z passes: lines along a strided axis.  Lines are flattened as
// L = o*gx + x (o = z for Y passes, y for Z passes); a tile is LPC
// consecutive lines, so consecutive threads read consecutive x.
//   kind 0: forward y, 1: inverse y, 2: z (forward, exp(-ds k^2)/N, inverse),
//   3: forward z only, 4: inverse z only
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void strided_tile(const BulkDev<T>* __restrict__ insts, const int2 w,
                                             const cplx<T>* __restrict__ gtw, const T* __restrict__ fk,
                                             const double2* __restrict__ gtw64,
                                             const double* __restrict__ g64, int t, int kind,
                                             unsigned char* smraw) {
  const BulkDev<T> I = insts[w.x];
  if (t > I.ns) return;
  const bool zdir = kind >= 2;
  const Plan1D P = zdir ? I.pz : I.py;
  cplx<T> *tw, *b0, *b1;
  carve<T>(smraw, P, tw, b0, b1);
  load_twiddles<T>(tw, gtw, P);
  const int N = P.n, LPC = P.lpc;
  const int nlines = I.gx * (zdir ? I.gy : I.gz);
  const int L0 = w.y * LPC;
  const int nl = min(LPC, nlines - L0);
  const size_t es = zdir ? (size_t)I.gx * I.gy : (size_t)I.gx;
  const size_t ostride = zdir ? (size_t)I.gx : (size_t)I.gx * I.gy;
  const int tot = nl * N;
  const int line = threadIdx.x / P.tpl, lt = threadIdx.x % P.tpl;
  const bool active = line < nl;
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    const int j = e / nl, l = e % nl;
    const int L = L0 + l;
    const size_t b = (size_t)(L / I.gx) * ostride + (L % I.gx);
    b0[l * P.ld + j] = I.spec[b + (size_t)j * es];
  }
  __syncthreads();
  cplx<T>* r;
  if (kind == 2) {
    // the (kx, ky) = (0, 0) pencil in float-float (see DcPencil)
    constexpr bool dc64 = sizeof(T) == 4;
    const bool dcline = dc64 && L0 == 0;
    unsigned char* tail = reinterpret_cast<unsigned char*>(b1 + P.lpc * P.ld);
    tail = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tail) + 15) & ~uintptr_t(15));
    float2* dcf = reinterpret_cast<float2*>(tail);
    const DcPencil dcp{dcf, dcf + N, dcf + 2 * N};
    if (dcline) {
      for (int i = threadIdx.x; i < N; i += blockDim.x) {
        dcf[i] = make_float2((float)b0[i].x, (float)b0[i].y);   // line 0 = (x, y) = (0, 0)
        const double c = g64[I.g64_off + i];
        const float h = (float)c;
        dcp.c[i] = make_float2(h, (float)(c - (double)h));
      }
      __syncthreads();
      dc_pencil_apply(N, dcp);
    }
    r = fft_lines<T>(b0, b1, tw, P, line, lt, active, +1);
    // exp(-ds (kx^2 + ky^2 + kz^2)) / N from the separable tables, applied with
    // one rounding (compensated product of the hi/lo parts)
    const T* gxy = fk + I.gxy_off;
    const T* gzt = fk + I.gz_off;
    const int nxy = I.gx * I.gy;
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
      const int l = e / N, j = e % N;
      const int L = L0 + l;
      cplx<T>& v = r[l * P.ld + j];
      if constexpr (sizeof(T) == 4) {
        const float ah = gxy[L], al = gxy[nxy + L], bh = gzt[j], bl = gzt[N + j];
        const float gh = ah * bh;
        const float gl = fmaf(ah, bh, -gh) + fmaf(ah, bl, al * bh);
        v = mk<T>(fmaf(v.x, gh, v.x * gl), fmaf(v.y, gh, v.y * gl));
      } else {
        const T f = gxy[L] * gzt[j];
        v = mk<T>(v.x * f, v.y * f);
      }
    }
    __syncthreads();
    cplx<T>* o = (r == b0) ? b1 : b0;
    r = fft_lines<T>(r, o, tw, P, line, lt, active, -1);
    if (dcline) {
      for (int j = threadIdx.x; j < N; j += blockDim.x)
        r[j] = mk<T>((T)dcp.out[j].x, (T)dcp.out[j].y);
      __syncthreads();
    }
  } else {
    const int sg = (kind == 0 || kind == 3) ? +1 : -1;
    r = fft_lines<T>(b0, b1, tw, P, line, lt, active, sg);
  }
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    const int j = e / nl, l = e % nl;
    const int L = L0 + l;
    const size_t b = (size_t)(L / I.gx) * ostride + (L % I.gx);
    I.spec[b + (size_t)j * es] = r[l * P.ld + j];
  }
}

template <typename T>
__global__ void __launch_bounds__(BULK_THREADS)
k_bulk_strided(const BulkDev<T>* __restrict__ insts, const int2* __restrict__ work,
               const cplx<T>* __restrict__ gtw, const T* __restrict__ fk,
               const double2* __restrict__ gtw64, const double* __restrict__ g64,
               int t, int kind) {
  extern __shared__ __align__(16) unsigned char smraw[];
  strided_tile<T>(insts, work[blockIdx.x], gtw, fk, gtw64, g64, t, kind, smraw);
}

// ---------------------------------------------------------------------------
// Contour integral (mod_diblock.f90:143-154) and sum of q_N (:141).
// Nodes s and N-s are read together: slice s = (q_s, qdag_s) and slice N-s
// = (q_{N-s}, qdag_{N-s}) give the products q_s qdag_{N-s} (node s) and
// q_{N-s} qdag_s (node N-s).  Trapezoid weights per block: 1/2 at the block
// ends, 1 inside (times ds, applied at the end).
//   FP32 slices: each product is split exactly (TwoProd via FMA) and summed
//   with a compensated (Kahan/TwoSum) float pair, ~48 bits over the whole
//   contour, converted to FP64 once per point (conversions run on GB300's
//   narrow FP64 pipe).
//   FP64 slices: plain FP64 accumulation, as the reference.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float wA_of(int s, int na) {
  return (s == 0 ? 0.5f : 0.f) + (s == na ? 0.5f : 0.f) + ((s > 0 && s < na) ? 1.f : 0.f);
}
__device__ __forceinline__ float wB_of(int s, int na, int n) {
  return (s == na ? 0.5f : 0.f) + (s == n ? 0.5f : 0.f) + ((s > na && s < n) ? 1.f : 0.f);
}
// contour weights of node s for types A and B
template <typename T>
__device__ __forceinline__ float2 node_weights(const BulkDev<T>& I, int s) {
  if (I.nblk) return I.wtab[s];
  return make_float2(wA_of(s, I.na), wB_of(s, I.na, I.ns));
}

struct FF {  // compensated float accumulator
  float hi, lo;
};
__device__ __forceinline__ void ff_add_prod(FF& a, float x, float y, float wgt) {
  const float p = x * y;
  const float e = fmaf(x, y, -p);          // exact: x*y = p + e
  const float pw = p * wgt, ew = e * wgt;  // wgt in {1/2, 1}: exact
  const float s = a.hi + pw;
  const float bp = s - a.hi;
  const float err = (a.hi - (s - bp)) + (pw - bp);
  a.lo += err + ew;
  a.hi = s;
}

template <typename T>
__global__ void __launch_bounds__(BULK_THREADS)
k_bulk_contour(const BulkDev<T>* __restrict__ insts) {
  __shared__ double red[32];
  const BulkDev<T> I = insts[blockIdx.y];
  const double ds = I.ds;
  const int N = I.ns;
  const cplx<T>* sl = I.slices;
  const size_t np = I.npts;
  double qsum = 0.0;
  if constexpr (sizeof(T) == 4) {
    if ((np & 1) == 0) {
      // two adjacent points per thread: 16-byte loads of both slices, twice
      // the bytes in flight per load instruction (slice bases are 16-byte
      // aligned when npts is even)
      const size_t np2 = np / 2;
      for (size_t p2 = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p2 < np2;
           p2 += (size_t)gridDim.x * blockDim.x) {
        FF fa0 = {0.f, 0.f}, fb0 = {0.f, 0.f}, fa1 = {0.f, 0.f}, fb1 = {0.f, 0.f};
#pragma unroll 4
        for (int s = 0; 2 * s <= N; ++s) {
          const int u = N - s;
          const float4 a = reinterpret_cast<const float4*>(sl + (size_t)s * np)[p2];
          const float4 b = reinterpret_cast<const float4*>(sl + (size_t)u * np)[p2];
          if (s == 0) qsum += (double)b.x + (double)b.z;
          float2 wn = node_weights(I, s);          // node s: q_s * qdag_{N-s}
          if (wn.x != 0.f) { ff_add_prod(fa0, a.x, b.y, wn.x); ff_add_prod(fa1, a.z, b.w, wn.x); }
          if (wn.y != 0.f) { ff_add_prod(fb0, a.x, b.y, wn.y); ff_add_prod(fb1, a.z, b.w, wn.y); }
          if (u != s) {                             // node N-s: q_{N-s} * qdag_s
            wn = node_weights(I, u);
            if (wn.x != 0.f) { ff_add_prod(fa0, b.x, a.y, wn.x); ff_add_prod(fa1, b.z, a.w, wn.x); }
            if (wn.y != 0.f) { ff_add_prod(fb0, b.x, a.y, wn.y); ff_add_prod(fb1, b.z, a.w, wn.y); }
          }
        }
        reinterpret_cast<double2*>(I.dist)[p2] =
            make_double2(ds * ((double)fa0.hi + (double)fa0.lo), ds * ((double)fa1.hi + (double)fa1.lo));
        reinterpret_cast<double2*>(I.dist + np)[p2] =
            make_double2(ds * ((double)fb0.hi + (double)fb0.lo), ds * ((double)fb1.hi + (double)fb1.lo));
      }
      const double tot = block_reduce_1(qsum, red);
      if (threadIdx.x == 0) I.qpart[blockIdx.x] = tot;
      return;
    }
  }
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < I.npts; p += gridDim.x * blockDim.x) {
    double accA = 0.0, accB = 0.0;
    if constexpr (sizeof(T) == 4) {
      FF fa = {0.f, 0.f}, fb = {0.f, 0.f};
#pragma unroll 4
      for (int s = 0; 2 * s <= N; ++s) {
        const int u = N - s;
        const cplx<T> a = sl[(size_t)s * np + p];
        const cplx<T> b = sl[(size_t)u * np + p];
        if (s == 0) qsum += (double)b.x;
        // node s: q_s * qdag_{N-s}
        const float x1 = (float)a.x, y1 = (float)b.y;
        float2 wn = node_weights(I, s);
        if (wn.x != 0.f) ff_add_prod(fa, x1, y1, wn.x);
        if (wn.y != 0.f) ff_add_prod(fb, x1, y1, wn.y);
        if (u != s) {  // node N-s: q_{N-s} * qdag_s
          const float x2 = (float)b.x, y2 = (float)a.y;
          wn = node_weights(I, u);
          if (wn.x != 0.f) ff_add_prod(fa, x2, y2, wn.x);
          if (wn.y != 0.f) ff_add_prod(fb, x2, y2, wn.y);
        }
      }
      accA += (double)fa.hi + (double)fa.lo;
      accB += (double)fb.hi + (double)fb.lo;
    } else {
#pragma unroll 4
      for (int s = 0; 2 * s <= N; ++s) {
        const int u = N - s;
        const cplx<T> a = sl[(size_t)s * np + p];
        const cplx<T> b = sl[(size_t)u * np + p];
        if (s == 0) qsum += (double)b.x;
        double pr = (double)a.x * (double)b.y;
        float2 wn = node_weights(I, s);
        accA += (double)wn.x * pr;
        accB += (double)wn.y * pr;
        if (u != s) {
          pr = (double)b.x * (double)a.y;
          wn = node_weights(I, u);
          accA += (double)wn.x * pr;
          accB += (double)wn.y * pr;
        }
      }
    }
    I.dist[p] = ds * accA;
    I.dist[np + p] = ds * accB;
  }
  const double tot = block_reduce_1(qsum, red);
  if (threadIdx.x == 0) I.qpart[blockIdx.x] = tot;
}

// E = exp(-0.5 ds w) for both species (Calculate_Expfield, mod_propagate.f90:28)
// w [2][npts] -> interleaved factors (see EPt)
template <typename T>
__global__ void k_expfield(const double* __restrict__ w, T* __restrict__ E, size_t npts, double ds) {
  for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < npts; p += (size_t)gridDim.x * blockDim.x) {
    store_boltzmann(E, p, 0, -0.5 * ds * w[p]);
    store_boltzmann(E, p, 1, -0.5 * ds * w[npts + p]);
  }
}

template <typename TO, typename TI>
__global__ void k_convert(const TI* __restrict__ in, TO* __restrict__ out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (TO)in[i];
}

// spectrum (full complex, T) -> FP64 copy scaled by s
template <typename T>
__global__ void k_spec_to_f64(const cplx<T>* __restrict__ in, double2* __restrict__ out, size_t n, double s) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    cplx<T> v = in[i];
    out[i] = make_double2((double)v.x * s, (double)v.y * s);
  }
}
template <typename T>
__global__ void k_f64_to_spec(const double2* __restrict__ in, cplx<T>* __restrict__ out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double2 v = in[i];
    out[i] = mk<T>((T)v.x, (T)v.y);
  }
}
