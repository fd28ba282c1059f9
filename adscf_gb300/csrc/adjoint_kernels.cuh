// adjoint_kernels.cuh -- reverse-mode adjoint of the discrete bulk diblock
// free energy (FP64), giving dF/dL_x, dF/dL_y, dF/dL_z and dF/dchi at fixed
// fields.
//
// Forward quantities (Propagate_Diblock, Bulk_3D_FFT/Polymer_Modules/
// mod_diblock.f90:100-173, and Calculate_Energy, Bulk_3D_FFT/Main_Diblock_Melt/
// main_diblock.f90:295-307, canonical ensemble):
//   q_t = E(t) P E(t) q_{t-1},  P = IFFT diag(G) FFT,  G(k) = exp(-ds |k|^2)
//   S = sum_r q_Ns(r),   dist_i(r) = sum_s c_{i,s} q_s(r) qdag_{Ns-s}(r)
//   phi_i = rho M dist_i / S          (M grid points; rho V / Q = rho M / S)
//   F = log(rho M / S) - 1 + [ -sum phi.w + E_int(phi) ] / (rho M)
// At fixed w the box lengths enter only through G.  With R_i = w_new_i - w_i
// (w_new = the mean field of phi), the cotangents are
//   dF/dS = aS = -(1 + sum_r,i R_i phi_i / (rho M)) / S,   dF/d dist_i = R_i / S
// and the adjoint chains lambda_t = dF/dq_t, mu_t = dF/dqdag_t obey the same
// recursion backwards, seeded from the stored slices:
//   lambda_t = E(t+1) P E(t+1) lambda_{t+1} + sum_i (R_i/S) c_{i,t} qdag_{Ns-t} [+ aS at t = Ns]
//   mu_t     = E(t+1) P E(t+1) mu_{t+1}     + sum_i (R_i/S) c_{i,Ns-t} q_{Ns-t}
// The gradient of step t is <E(t) lambda_t, dP E(t) q_{t-1}> (+ the same for
// the backward chain) = (1/M) sum_k dG(k) Re(conj(Xf(k)) Ya(k)), with Xf =
// FFT(E(t) z_{t-1}), Ya = FFT(E(t) zbar_t) of the packed complex pairs
// z = q + i qdag and zbar = lambda + i mu: for real fields and a real, even
// dG the cross terms of the packed product cancel.  dG/dL_c = 2 ds k_c^2 G /
// L_c.  dF/dchi at fixed w = sum_r v_A phi_A v_B phi_B / (rho M).
//
// Each adjoint double step is four launches, like the forward one:
//   k_adj_x(t) : inverse x of the adjoint spectrum -> E(t+1) -> + seeds ->
//                E(t) -> forward x (adjoint);  slice t-1 -> E(t) -> forward x
//   Yf         : forward y of both spectra (k_bulk_strided, two instances)
//   k_adj_z(t) : forward z of both, stress accumulation, G/M, inverse z
//   Yi         : inverse y of the adjoint spectrum
// The slices (q_t, qdag_t) of the forward pass are read, not recomputed.
#pragma once
#include "bulk_kernels.cuh"

struct AdjDev {
  BulkDev<double> I;        // FP64 instance: plans, tables, slices, E, dist, qpart
  double2* sa;              // adjoint spectrum (the instance's work buffer)
  double2* sf;              // forward-chain spectrum of the current step
  double* b;                // [2][npts] dF/d dist_i = R_i / S
  const double* w;          // [2][npts] fields
  double* part;             // [nclos][4] closure partials
  double* gpart;            // [nz tiles][3] stress partials (accumulated over t)
  double* sc;               // scalars: S, F, aS, dF/dchi, dF/dLx, dF/dLy, dF/dLz
  int nqpart, nclos, nztiles;
  double rho, kappa, chi, v0, v1, ds;
  double lx, ly, lz;
  // where the reverse sweep finds the stored nodes: node t of the forward
  // chains at slA + (t - tA0) npts (z_{t-1}) and slB + (t - tB0) npts (the
  // mirror node Ns - t); both are I.slices with offset 0 when every node is
  // stored, two recomputed segments under checkpointing
  const double2* slA;
  const double2* slB;
  int tA0, tB0;
};

enum { ADJ_S = 0, ADJ_F = 1, ADJ_AS = 2, ADJ_DCHI = 3, ADJ_DLX = 4, ADJ_DLY = 5, ADJ_DLZ = 6, ADJ_NSC = 8 };

__device__ __forceinline__ double adj_k2(int i, int n, double len) {
  const double m = (i > n / 2) ? double(i - n) : double(i);
  const double k = 2.0 * 3.14159265358979323846 * m / len;
  return k * k;
}

// densities, mean-field residual and the cotangents of the contour integrals
__device__ __forceinline__ void adj_closure_body(const AdjDev& A, int bid, int nb) {
  __shared__ double red[4 * 32];
  __shared__ double sS;
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < A.nqpart; ++i) s += A.I.qpart[i];
    sS = s;
  }
  __syncthreads();
  const double S = sS;
  const size_t np = (size_t)A.I.npts;
  const double scale = A.rho * (double)np / S;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (size_t p = (size_t)bid * blockDim.x + threadIdx.x; p < np; p += (size_t)nb * blockDim.x) {
    const double pa = scale * A.I.dist[p], pb = scale * A.I.dist[np + p];
    const double va = A.v0 * pa, vb = A.v1 * pb;
    const double tot = va + vb - 1.0;
    const double wa = A.w[p], wb = A.w[np + p];
    const double ra = A.v0 * (A.kappa * tot + A.chi * vb) - wa;
    const double rb = A.v1 * (A.kappa * tot + A.chi * va) - wb;
    A.b[p] = ra / S;
    A.b[np + p] = rb / S;
    acc[0] += ra * pa + rb * pb;
    acc[1] += pa * wa + pb * wb;
    acc[2] += 0.5 * A.kappa * tot * tot + A.chi * va * vb;
    acc[3] += va * vb;
  }
  const double r = block_reduce_k<4>(acc, red);
  if (threadIdx.x < 4) A.part[bid * 4 + threadIdx.x] = r;
}

static __global__ void __launch_bounds__(BULK_THREADS) k_adj_closure(AdjDev A) {
  adj_closure_body(A, blockIdx.x, gridDim.x);
}

// batch: instance blockIdx.y, A.nclos blocks each
static __global__ void __launch_bounds__(BULK_THREADS) k_adj_closure_b(const AdjDev* __restrict__ As) {
  const AdjDev& A = As[blockIdx.y];
  if ((int)blockIdx.x >= A.nclos) return;
  adj_closure_body(A, blockIdx.x, A.nclos);
}

__device__ __forceinline__ void adj_scalars_body(const AdjDev& A) {
  if (threadIdx.x != 0) return;
  double S = 0.0, p[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = 0; i < A.nqpart; ++i) S += A.I.qpart[i];
  for (int b = 0; b < A.nclos; ++b)
    for (int k = 0; k < 4; ++k) p[k] += A.part[b * 4 + k];
  const double rm = A.rho * (double)A.I.npts;
  A.sc[ADJ_S] = S;
  A.sc[ADJ_F] = log(rm / S) - 1.0 + (p[2] - p[1]) / rm;
  A.sc[ADJ_AS] = -(1.0 + p[0] / rm) / S;
  A.sc[ADJ_DCHI] = p[3] / rm;
}

static __global__ void k_adj_scalars(AdjDev A) { adj_scalars_body(A); }
static __global__ void k_adj_scalars_b(const AdjDev* __restrict__ As) { adj_scalars_body(As[blockIdx.x]); }

// adjoint x pass of step t (see the file comment) on row tile `tile`
__device__ __forceinline__ void adj_x_body(const AdjDev& A, int tile, const double2* __restrict__ gtw, int t) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const BulkDev<double>& I = A.I;
  const Plan1D P = I.px;
  double2 *tw, *b0, *b1;
  carve<double>(smraw, P, tw, b0, b1);
  load_twiddles<double>(tw, gtw, P);
  const int N = P.n, LPC = P.lpc;
  const int nrows = I.gy * I.gz;
  const int row0 = tile * LPC;
  const int nl = min(LPC, nrows - row0);
  const size_t base = (size_t)row0 * N;
  const int tot = nl * N;
  const int line = threadIdx.x / P.tpl, lt = threadIdx.x % P.tpl;
  const bool active = line < nl;
  const size_t np = (size_t)I.npts;
  const bool fA = chain_type_fwd(I, t) == 0, bA = chain_type_bwd(I, t) == 0;

  // forward-chain spectrum: E(t) (q_{t-1}, qdag_{t-1}) -> forward x
  const double2* slp = A.slA + (size_t)(t - 1 - A.tA0) * np;
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    const size_t g = base + e;
    const double2 v = slp[g];
    const EPt<double> ev = load_ept(I.E, g);
    b0[(e / N) * P.ld + (e % N)] = make_double2(v.x * (fA ? ev.a : ev.b), v.y * (bA ? ev.a : ev.b));
  }
  __syncthreads();
  double2* r = fft_lines<double>(b0, b1, tw, P, line, lt, active, +1);
  for (int e = threadIdx.x; e < tot; e += blockDim.x) A.sf[base + e] = r[(e / N) * P.ld + (e % N)];
  __syncthreads();

  // adjoint state at node t
  const bool first = t == I.ns;
  double2* o;
  if (!first) {
    for (int e = threadIdx.x; e < tot; e += blockDim.x) b0[(e / N) * P.ld + (e % N)] = A.sa[base + e];
    __syncthreads();
    r = fft_lines<double>(b0, b1, tw, P, line, lt, active, -1);
    o = (r == b0) ? b1 : b0;
  } else {
    r = b0;
    o = b1;
  }
  const bool fA1 = chain_type_fwd(I, t + 1) == 0, bA1 = chain_type_bwd(I, t + 1) == 0;
  const int u = I.ns - t;
  const double ds = A.ds;
  const float2 wnt = node_weights(I, t), wnu = node_weights(I, u);
  const double cat = ds * (double)wnt.x, cbt = ds * (double)wnt.y;
  const double cau = ds * (double)wnu.x, cbu = ds * (double)wnu.y;
  const double aS = first ? A.sc[ADJ_AS] : 0.0;
  const double2* slu = A.slB + (size_t)(u - A.tB0) * np;
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    const size_t g = base + e;
    const int si = (e / N) * P.ld + (e % N);
    const EPt<double> ev = load_ept(I.E, g);
    double lam = 0.0, mu = 0.0;
    if (!first) {
      const double2 z = r[si];
      lam = z.x * (fA1 ? ev.a : ev.b);
      mu = z.y * (bA1 ? ev.a : ev.b);
    }
    const double2 s2 = slu[g];   // (q_{Ns-t}, qdag_{Ns-t})
    const double ba = A.b[g], bb = A.b[np + g];
    lam += (cat * ba + cbt * bb) * s2.y + aS;
    mu += (cau * ba + cbu * bb) * s2.x;
    o[si] = make_double2(lam * (fA ? ev.a : ev.b), mu * (bA ? ev.a : ev.b));
  }
  __syncthreads();
  double2* r2 = fft_lines<double>(o, r, tw, P, line, lt, active, +1);
  for (int e = threadIdx.x; e < tot; e += blockDim.x) A.sa[base + e] = r2[(e / N) * P.ld + (e % N)];
}

static __global__ void __launch_bounds__(BULK_THREADS)
k_adj_x(AdjDev A, const int2* __restrict__ work, const double2* __restrict__ gtw, int t) {
  adj_x_body(A, work[blockIdx.x].y, gtw, t);
}

// batch: work = (instance, row tile); every listed instance has t <= its Ns
static __global__ void __launch_bounds__(BULK_THREADS)
k_adj_x_b(const AdjDev* __restrict__ As, const int2* __restrict__ work, const double2* __restrict__ gtw, int t) {
  const int2 w = work[blockIdx.x];
  if (t > As[w.x].I.ns) return;
  adj_x_body(As[w.x], w.y, gtw, t);
}

// adjoint z pass of step t: forward z of both spectra, stress partials,
// factor G/M on the adjoint spectrum, inverse z.  Three line buffers.
__device__ __forceinline__ void adj_z_body(const AdjDev& A, int tile, const double2* __restrict__ gtw,
                                           const double* __restrict__ fk) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ double red[3 * 32];
  const BulkDev<double>& I = A.I;
  const Plan1D P = I.pz;
  double2 *tw, *b0, *b1;
  carve<double>(smraw, P, tw, b0, b1);
  double2* fb = b1 + P.lpc * P.ld;
  load_twiddles<double>(tw, gtw, P);
  const int N = P.n, LPC = P.lpc;
  const int gx = I.gx, gy = I.gy;
  const int nlines = gx * gy;
  const int L0 = tile * LPC;
  const int nl = min(LPC, nlines - L0);
  const size_t es = (size_t)gx * gy;
  const int tot = nl * N;
  const int line = threadIdx.x / P.tpl, lt = threadIdx.x % P.tpl;
  const bool active = line < nl;
  // forward-chain pencils
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    const int j = e / nl, l = e % nl;
    const int L = L0 + l;
    b0[l * P.ld + j] = A.sf[(size_t)(L / gx) * gx + (L % gx) + (size_t)j * es];
  }
  __syncthreads();
  double2* r = fft_lines<double>(b0, b1, tw, P, line, lt, active, +1);
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    const int l = e / N, j = e % N;
    fb[l * P.ld + j] = r[l * P.ld + j];
  }
  __syncthreads();
  // adjoint pencils
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    const int j = e / nl, l = e % nl;
    const int L = L0 + l;
    b0[l * P.ld + j] = A.sa[(size_t)(L / gx) * gx + (L % gx) + (size_t)j * es];
  }
  __syncthreads();
  r = fft_lines<double>(b0, b1, tw, P, line, lt, active, +1);
  const double* gxy = fk + I.gxy_off;
  const double* gzt = fk + I.gz_off;
  double acc[3] = {0.0, 0.0, 0.0};
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    const int l = e / N, j = e % N;
    const int L = L0 + l;
    const double g = gxy[L] * gzt[j];                 // G(k) / M
    double2& a = r[l * P.ld + j];
    const double2 f = fb[l * P.ld + j];
    const double re = g * (f.x * a.x + f.y * a.y);
    acc[0] += re * adj_k2(L % gx, gx, A.lx);
    acc[1] += re * adj_k2(L / gx, gy, A.ly);
    acc[2] += re * adj_k2(j, I.gz, A.lz);
    a = make_double2(a.x * g, a.y * g);
  }
  const double s = block_reduce_k<3>(acc, red);
  if (threadIdx.x < 3) A.gpart[tile * 3 + threadIdx.x] += s;   // one tile per block: deterministic
  double2* o = (r == b0) ? b1 : b0;
  r = fft_lines<double>(r, o, tw, P, line, lt, active, -1);
  for (int e = threadIdx.x; e < tot; e += blockDim.x) {
    const int j = e / nl, l = e % nl;
    const int L = L0 + l;
    A.sa[(size_t)(L / gx) * gx + (L % gx) + (size_t)j * es] = r[l * P.ld + j];
  }
}

static __global__ void __launch_bounds__(BULK_THREADS)
k_adj_z(AdjDev A, const int2* __restrict__ work, const double2* __restrict__ gtw,
        const double* __restrict__ fk) {
  adj_z_body(A, work[blockIdx.x].y, gtw, fk);
}

static __global__ void __launch_bounds__(BULK_THREADS)
k_adj_z_b(const AdjDev* __restrict__ As, const int2* __restrict__ work, const double2* __restrict__ gtw,
          const double* __restrict__ fk, int t) {
  const int2 w = work[blockIdx.x];
  if (t > As[w.x].I.ns) return;
  adj_z_body(As[w.x], w.y, gtw, fk);
}

__device__ __forceinline__ void adj_grad_body(const AdjDev& A) {
  if (threadIdx.x != 0) return;
  double g[3] = {0.0, 0.0, 0.0};
  for (int b = 0; b < A.nztiles; ++b)
    for (int c = 0; c < 3; ++c) g[c] += A.gpart[b * 3 + c];
  A.sc[ADJ_DLX] = 2.0 * A.ds * g[0] / A.lx;
  A.sc[ADJ_DLY] = 2.0 * A.ds * g[1] / A.ly;
  A.sc[ADJ_DLZ] = 2.0 * A.ds * g[2] / A.lz;
}

static __global__ void k_adj_grad(AdjDev A) { adj_grad_body(A); }
static __global__ void k_adj_grad_b(const AdjDev* __restrict__ As) { adj_grad_body(As[blockIdx.x]); }

// Contour integral over one segment of nodes s in [s_lo, s_hi] from two
// recomputed node ranges: q_s at A + (s - a0) npts, qdag_{Ns-s} at
// B + (Ns - s - b0) npts (trapezoid weights of mod_diblock.f90:143-154).
// dist accumulates (+=) over the segments in a fixed order; the segment that
// holds s = 0 also writes the partial sums of q_Ns (= B node Ns).
static __global__ void __launch_bounds__(BULK_THREADS)
k_contour_segment(BulkDev<double> I, const double2* __restrict__ A, int a0, const double2* __restrict__ B,
                  int b0, int s_lo, int s_hi) {
  __shared__ double red[32];
  const size_t np = (size_t)I.npts;
  const int N = I.ns;
  double qs = 0.0;
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < np; p += (size_t)gridDim.x * blockDim.x) {
    double accA = 0.0, accB = 0.0;
    for (int s = s_lo; s <= s_hi; ++s) {
      const double pr = A[(size_t)(s - a0) * np + p].x * B[(size_t)(N - s - b0) * np + p].y;
      const float2 wn = node_weights(I, s);
      accA += (double)wn.x * pr;
      accB += (double)wn.y * pr;
    }
    I.dist[p] += I.ds * accA;
    I.dist[np + p] += I.ds * accB;
    if (s_lo == 0) qs += B[(size_t)(N - b0) * np + p].x;
  }
  const double tot = block_reduce_1(qs, red);
  if (s_lo == 0 && threadIdx.x == 0) I.qpart[blockIdx.x] = tot;
}

// (1, 1) at every point: node 0 of both chains
static __global__ void k_fill_ones(double2* __restrict__ z, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    z[i] = make_double2(1.0, 1.0);
}
