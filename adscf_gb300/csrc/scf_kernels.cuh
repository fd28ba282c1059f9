// scf_kernels.cuh -- closure, mean fields, residual and mixing on the device.
//
// Reference: ensemble closure of Propagate_Diblock (Bulk_3D_FFT/
// Polymer_Modules/mod_diblock.f90:156-167), Check_Accuracy
// (main_diblock.f90:380-390), Calculate_Mean_Fields (Bulk_3D_FFT/
// Interaction_Modules/mod_FloryHuggins.f90:104-129) and its film form with
// a wall potential (Film_CK_AD/Film_1D/Interaction_Modules/
// mod_FloryHuggins.f90:140-167), Interaction_Energy (:74-96), Calculate_Energy
// (main_diblock.f90:295-307) and Mixing_Simple / Mixing_Lambda /
// Mixing_Anderson with ludcmp/lubksb (Bulk_3D_FFT/General_Routines/
// mod_iterate.f90:27-150,232-337).
//
// One closure kernel per iteration does, per point: density = scale*dist,
// the accuracy term, the new mean field, the residual r_k = w_new - x_k
// (written straight into the mixing history), the energy integrands and the
// Anderson Gram row <r_k, r_j> over the history -- so the whole SCF
// bookkeeping is one read of dist, phi_old, x_k and the history.  All
// reductions are per-block partials summed in a fixed order (bitwise
// reproducible).  A one-CTA kernel then forms the m x m system, solves it in
// FP64 exactly as ludcmp/lubksb, and writes mixing coefficients; one mixing
// kernel writes x_{k+1} and, for the pseudo-spectral path, E = exp(-ds x/2).
#pragma once
#include "common.cuh"

#define SCF_THREADS 256
#define SCF_MAX_HIST 16
#define SCF_MAX_SLOTS (SCF_MAX_HIST + 1)
#define NP_FIXED 7
#define NPART (NP_FIXED + SCF_MAX_SLOTS)
// the solve's block: one warp per partial-sum entry at a time (8 warps)
#define SOLVE_THREADS 256

enum { P_ACC = 0, P_PHIW = 1, P_EINT = 2, P_RHO = 3, P_EEXT = 4, P_LNUM = 5, P_LDEN = 6 };

// result scalars on the device (mirrors adscf_iter_result + internals)
enum {
  R_ACC = 0, R_F, R_Q, R_LOGQ, R_MU, R_RHO, R_LAMBDA, R_ITER, R_ENERGY, R_PHIW,
  R_EINT, R_EEXT, R_STATUS, R_COUNT
};

struct ScfDev {
  int npts;          // points per species
  int ntypes;        // 2 (diblock) or 1 (homopolymer)
  int plane;         // points per z plane (gx*gy)
  int nplanes;       // gz (bulk) or gz+1 (films)
  int wall_mask;     // films: mix only interior planes 1..nplanes-2
  double dvol;       // bulk volume element (used when wz == null)
  const double* wz;  // per-plane integration weights (dx dy w_z), or null
  const double* ext; // [ntypes][nplanes] wall potential, or null
  double kappa, chi, v0, v1, ww;
  int homopolymer;   // brush model: w = ww phi + U
  int ensemble;      // 1 canonical, 2 grand canonical
  double rho, mu, volume, chain_len;   // chain_len = ds * segments (GC rho)
  const double* dist;        // [ntypes][npts] contour integrals
  double* dens;              // [ntypes][npts] phi (old in, new out)
  const double* target;      // [ntypes][npts] density of the conjugate-field solve (CL_CONJ)
  double* hx;                // [slots][ntypes*npts] field history
  double* hr;                // [slots][ntypes*npts] residual history
  double* hy;                // [slots][ntypes*npts] x_j + lambda r_j (Anderson), or null
  int slots;                 // m+1
  int mixing_type, warm;     // warm: Anderson for iter > warm
  double lambda, lam_warm;
  const double* qpart; int nqpart; double qscale;
  double* part;              // [gridDim.x][NPART]
  int npart_blocks;
  double* gram;              // [slots][slots]
  double* coef;              // [2][slots]
  int* iter;                 // 1-based iteration counter
  double* res;               // [R_COUNT]
  void* mixE;                // batched mixing: this instance's Boltzmann factors (T*)
  double mixds;              //   and contour step
};

// Q = qscale * (sum of the contour kernel's per-block partials) in one fixed
// order: lane-strided partial sums s_l (blocks b = l mod 32, increasing b),
// then a butterfly over the 32 lanes.  Floating-point addition commutes
// exactly, so every lane of the butterfly ends with the same bits, and
// q_total_serial replays the same additions in one thread: every caller sees
// the same Q.  All 32 lanes of a warp must call q_total.
__device__ __forceinline__ double warp_sum_fixed(const double* v, int n, size_t stride) {
  const int lane = threadIdx.x & 31;
  double s = 0.0;
  for (int b = lane; b < n; b += 32) s += v[(size_t)b * stride];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}
__device__ __forceinline__ double q_total(const ScfDev& S) {
  return warp_sum_fixed(S.qpart, S.nqpart, 1) * S.qscale;
}
__device__ __forceinline__ double q_total_serial(const ScfDev& S) {
  double s[32];
  for (int l = 0; l < 32; ++l) {
    s[l] = 0.0;
    for (int b = l; b < S.nqpart; b += 32) s[l] += S.qpart[b];
  }
  for (int o = 16; o > 0; o >>= 1) {
    double t[32];
    for (int l = 0; l < 32; ++l) t[l] = s[l] + s[l ^ o];
    for (int l = 0; l < 32; ++l) s[l] = t[l];
  }
  return s[0] * S.qscale;
}

__device__ __forceinline__ double density_scale(const ScfDev& S, double Q) {
  return S.ensemble == 1 ? S.rho * S.volume / Q : exp(S.mu);
}

// flags for k_closure
// CL_CONJ: the inverse problem of Get_Conjugate_Fields (main_multiblock.f90:
// 566-640): residual phi[w] - target instead of the mean-field residual, and
// the accuracy max |residual| (Check_Accuracy of that driver, :773-783)
enum { CL_MEANFIELD = 1, CL_MIXDOTS = 2, CL_KEEP_OLD = 4, CL_CONJ = 8 };

// Non-template kernels are defined once, in scf.cu.  The `_b` forms run a
// batch of independent instances: instance blockIdx.y (closure, mix) or
// blockIdx.x (solve) of the ScfDev array, with per-instance partials.
// closure launches (the kernels are specialised by history length)
// Threads of a closure block: an instance of at most 256 points (a one-line
// film or brush, one closure block) takes 64, so a batch of such films runs
// four times as many closure blocks per SM; alone and in a batch a film sums
// its points in the same order.
inline int closure_threads(long long npts) { return npts <= 256 ? 64 : SCF_THREADS; }
void launch_closure(const ScfDev& S, int flags, int grid, cudaStream_t st);
void launch_closure_b(const ScfDev* Ss, int max_slots, int flags, dim3 grid, cudaStream_t st,
                      int threads = SCF_THREADS);
__global__ void k_mixdots(ScfDev S);
__global__ void k_solve(ScfDev S, int have_closure, int do_mix);
__global__ void k_solve_b(const ScfDev* __restrict__ Ss, int have_closure, int do_mix);
__global__ void k_meanfield_only(ScfDev S, const double* __restrict__ dens, double* __restrict__ field);

#ifdef ADSCF_SCF_IMPL
// Per point: phi_new = scale*dist; accuracy; mean field; residual into the
// history slot of iteration k; energy and mixing partial sums.  Block `bid`
// of `nb` blocks working on this instance.
template <int NS>
__device__ __forceinline__ void closure_body(const ScfDev& S, int flags, int bid, int nb) {
  constexpr int NA = NP_FIXED + NS;   // partial sums held per thread
  __shared__ double red[NA * 32];
  const double Q = q_total(S);
  const double scale = density_scale(S, Q);
  const int k = *S.iter;
  const int cur = k % S.slots;
  const int prv = (k - 1 + S.slots) % S.slots;
  const size_t nv = (size_t)S.ntypes * S.npts;
  const double* xk = S.hx + (size_t)cur * nv;
  double* rk = S.hr + (size_t)cur * nv;
  const bool anderson = (flags & CL_MIXDOTS) && S.mixing_type == 3;
  const bool lam = (flags & CL_MIXDOTS) && S.mixing_type == 2 && k > 1;
  double acc[NA];
#pragma unroll
  for (int i = 0; i < NA; ++i) acc[i] = 0.0;
  for (int p = bid * blockDim.x + threadIdx.x; p < S.npts; p += nb * blockDim.x) {
    const int z = p / S.plane;
    const double wgt = S.wz ? S.wz[z] : S.dvol;
    const bool interior = !S.wall_mask || (z > 0 && z < S.nplanes - 1);
    double phi[2], wn[2];
    for (int c = 0; c < S.ntypes; ++c) {
      phi[c] = scale * S.dist[(size_t)c * S.npts + p];
      const double old = S.dens[(size_t)c * S.npts + p];
      if (!(flags & CL_CONJ)) acc[P_ACC] += (old - phi[c]) * (old - phi[c]);
      if (!(flags & CL_KEEP_OLD)) S.dens[(size_t)c * S.npts + p] = phi[c];
    }
    if (S.ntypes == 2) acc[P_RHO] += wgt * (phi[0] + phi[1]);
    else acc[P_RHO] += wgt * phi[0];
    if (flags & CL_CONJ) {
      for (int c = 0; c < S.ntypes; ++c) {
        const size_t i = (size_t)c * S.npts + p;
        const double x = xk[i];
        const double r = phi[c] - S.target[i];
        rk[i] = r;
        acc[P_ACC] = fmax(acc[P_ACC], fabs(r));
        if (anderson && S.hy) S.hy[(size_t)cur * nv + i] = x + S.lambda * r;
        if (anderson) {
#pragma unroll
          for (int j = 0; j < NS; ++j) {
            if (j < S.slots) {
              const double rj = (j == cur) ? r : S.hr[(size_t)j * nv + i];
              acc[NP_FIXED + j] += r * rj;
            }
          }
        }
      }
      continue;
    }
    if (!(flags & CL_MEANFIELD)) continue;
    if (S.homopolymer) {
      const double u = S.ext ? S.ext[z] : 0.0;
      wn[0] = S.ww * phi[0] + u;
      acc[P_EINT] += wgt * 0.5 * S.ww * phi[0] * phi[0];
      acc[P_EEXT] += wgt * u * phi[0];
    } else {
      const double f0 = phi[0] * S.v0, f1 = phi[1] * S.v1;
      const double tot = f0 + f1;
      const double u0 = S.ext ? S.ext[z] : 0.0;
      const double u1 = S.ext ? S.ext[S.nplanes + z] : 0.0;
      wn[0] = (S.kappa * (tot - 1.0) + S.chi * f1 + u0) * S.v0;
      wn[1] = (S.kappa * (tot - 1.0) + S.chi * f0 + u1) * S.v1;
      acc[P_EINT] += wgt * (0.5 * S.kappa * (tot - 1.0) * (tot - 1.0) + S.chi * f0 * f1);
      acc[P_EEXT] += wgt * (u0 * f0 + u1 * f1);
    }
    for (int c = 0; c < S.ntypes; ++c) {
      const size_t i = (size_t)c * S.npts + p;
      const double x = xk[i];
      acc[P_PHIW] += wgt * phi[c] * x;
      const double r = interior ? wn[c] - x : 0.0;
      rk[i] = r;
      if (anderson && S.hy) S.hy[(size_t)cur * nv + i] = x + S.lambda * r;
      if (!interior) continue;
      if (lam) {
        const double dx = x - S.hx[(size_t)prv * nv + i];
        const double dr = r - S.hr[(size_t)prv * nv + i];
        acc[P_LNUM] += dx * dx;
        acc[P_LDEN] += dr * dr;
      }
      if (anderson) {
#pragma unroll
        for (int j = 0; j < NS; ++j) {
          if (j < S.slots) {
            const double rj = (j == cur) ? r : S.hr[(size_t)j * nv + i];
            acc[NP_FIXED + j] += r * rj;
          }
        }
      }
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const bool amax = flags & CL_CONJ;   // P_ACC holds a maximum
#pragma unroll
  for (int i = 0; i < NA; ++i) {
    double x = acc[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double y = __shfl_down_sync(0xffffffffu, x, o);
      x = (amax && i == P_ACC) ? fmax(x, y) : x + y;
    }
    if (lane == 0) red[i * 32 + warp] = x;
  }
  __syncthreads();
  if (threadIdx.x < NPART) {   // entries past NA (slots this closure does not hold) are 0
    double r = 0.0;
    if (threadIdx.x < NA)
      for (int w = 0; w < nw; ++w)
        r = (amax && threadIdx.x == P_ACC) ? fmax(r, red[threadIdx.x * 32 + w]) : r + red[threadIdx.x * 32 + w];
    S.part[(size_t)bid * NPART + threadIdx.x] = r;
  }
}

// one kernel per slot capacity (3: lambda/simple or m <= 2, 11: m <= 10,
// SCF_MAX_SLOTS), so the partial sums held per thread fit the history
// Up to 11 slots the closure is held to 64 registers, so the 4 x 152 blocks
// of a bulk context run as one wave (at 80 registers, three blocks per SM
// left a second wave of a third of the blocks).
template <int NS>
__global__ void __launch_bounds__(SCF_THREADS, NS <= 11 ? 4 : 3)
k_closure(ScfDev S, int flags) { closure_body<NS>(S, flags, blockIdx.x, gridDim.x); }

// held to the register budget of k_closure (the instance's ScfDev is read in
// place from global memory rather than copied into registers)
template <int NS>
__global__ void __launch_bounds__(SCF_THREADS, NS <= 11 ? 4 : 3)
k_closure_b(const ScfDev* __restrict__ Ss, int flags) {
  const ScfDev& S = Ss[blockIdx.y];
  if ((int)blockIdx.x >= S.npart_blocks) return;
  closure_body<NS>(S, flags, blockIdx.x, S.npart_blocks);
}

void launch_closure(const ScfDev& S, int flags, int grid, cudaStream_t st) {
  const int nt = closure_threads(S.npts);
  if (S.slots <= 3) k_closure<3><<<grid, nt, 0, st>>>(S, flags);
  else if (S.slots <= 11) k_closure<11><<<grid, nt, 0, st>>>(S, flags);
  else k_closure<SCF_MAX_SLOTS><<<grid, nt, 0, st>>>(S, flags);
}
void launch_closure_b(const ScfDev* Ss, int max_slots, int flags, dim3 grid, cudaStream_t st, int threads) {
  if (max_slots <= 3) k_closure_b<3><<<grid, threads, 0, st>>>(Ss, flags);
  else if (max_slots <= 11) k_closure_b<11><<<grid, threads, 0, st>>>(Ss, flags);
  else k_closure_b<SCF_MAX_SLOTS><<<grid, threads, 0, st>>>(Ss, flags);
}

// Mixing dots only (for adscf_mix): x_k, r_k already in the history slot.
__global__ void __launch_bounds__(SCF_THREADS)
k_mixdots(ScfDev S) {
  __shared__ double red[NPART * 32];
  const int k = *S.iter;
  const int cur = k % S.slots;
  const int prv = (k - 1 + S.slots) % S.slots;
  const size_t nv = (size_t)S.ntypes * S.npts;
  double acc[NPART];
#pragma unroll
  for (int i = 0; i < NPART; ++i) acc[i] = 0.0;
  const bool lam = S.mixing_type == 2 && k > 1;
  const bool anderson = S.mixing_type == 3;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nv; i += (size_t)gridDim.x * blockDim.x) {
    const double r = S.hr[(size_t)cur * nv + i];
    if (lam) {
      const double dx = S.hx[(size_t)cur * nv + i] - S.hx[(size_t)prv * nv + i];
      const double dr = r - S.hr[(size_t)prv * nv + i];
      acc[P_LNUM] += dx * dx;
      acc[P_LDEN] += dr * dr;
    }
    if (anderson) {
#pragma unroll
      for (int j = 0; j < SCF_MAX_SLOTS; ++j)
        if (j < S.slots) acc[NP_FIXED + j] += r * S.hr[(size_t)j * nv + i];
      if (S.hy) S.hy[(size_t)cur * nv + i] = S.hx[(size_t)cur * nv + i] + S.lambda * r;
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int i = 0; i < NPART; ++i) {
    double x = acc[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[i * 32 + warp] = x;
  }
  __syncthreads();
  if (threadIdx.x < NPART) {
    double r = 0.0;
    for (int w = 0; w < nw; ++w) r += red[threadIdx.x * 32 + w];
    S.part[(size_t)blockIdx.x * NPART + threadIdx.x] = r;
  }
}

// ludcmp + lubksb (mod_iterate.f90:232-337), row-major a[n][n], in place.
__device__ void lu_solve_nr(double* a, double* b, int n) {
  int indx[SCF_MAX_HIST];
  double vv[SCF_MAX_HIST];
  const double tiny = 1.0e-20;
  for (int i = 0; i < n; ++i) {
    double aamax = 0.0;
    for (int j = 0; j < n; ++j) aamax = fmax(aamax, fabs(a[i * n + j]));
    vv[i] = 1.0 / aamax;  // the reference only prints on a singular row
  }
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < j; ++i) {
      double s = a[i * n + j];
      for (int k = 0; k < i; ++k) s -= a[i * n + k] * a[k * n + j];
      a[i * n + j] = s;
    }
    double aamax = 0.0;
    int imax = j;
    for (int i = j; i < n; ++i) {
      double s = a[i * n + j];
      for (int k = 0; k < j; ++k) s -= a[i * n + k] * a[k * n + j];
      a[i * n + j] = s;
      const double dum = vv[i] * fabs(s);
      if (dum >= aamax) { imax = i; aamax = dum; }
    }
    if (j != imax) {
      for (int k = 0; k < n; ++k) {
        const double d = a[imax * n + k];
        a[imax * n + k] = a[j * n + k];
        a[j * n + k] = d;
      }
      vv[imax] = vv[j];
    }
    indx[j] = imax;
    if (a[j * n + j] == 0.0) a[j * n + j] = tiny;
    if (j != n - 1) {
      const double dum = 1.0 / a[j * n + j];
      for (int i = j + 1; i < n; ++i) a[i * n + j] *= dum;
    }
  }
  int ii = -1;
  for (int i = 0; i < n; ++i) {
    const int ll = indx[i];
    double s = b[ll];
    b[ll] = b[i];
    if (ii >= 0) {
      for (int j = ii; j < i; ++j) s -= a[i * n + j] * b[j];
    } else if (s != 0.0) {
      ii = i;
    }
    b[i] = s;
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = b[i];
    for (int j = i + 1; j < n; ++j) s -= a[i * n + j] * b[j];
    b[i] = s / a[i * n + i];
  }
}

// One CTA: reduce partials, closure scalars, energy, mixing coefficients,
// advance the iteration counter.  `have_closure` = partials include the
// density/energy terms (k_closure) rather than only mixing dots.
__device__ __forceinline__ void solve_body(const ScfDev& S, int have_closure, int do_mix) {
  __shared__ double tot[NPART];
  __shared__ double qsh;
  {  // each entry summed by one warp in a fixed order (whatever the block size)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = warp; i < NPART; i += nw) {
      double r;
      if (have_closure == 2 && i == P_ACC) {   // conjugate-field solve: max over blocks
        r = 0.0;
        for (int b = lane; b < S.npart_blocks; b += 32) r = fmax(r, S.part[(size_t)b * NPART + i]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r = fmax(r, __shfl_xor_sync(0xffffffffu, r, o));
      } else {
        r = warp_sum_fixed(S.part + i, S.npart_blocks, NPART);
      }
      if (lane == 0) tot[i] = r;
    }
    if (have_closure && warp == 0) {
      const double q = q_total(S);
      if (lane == 0) qsh = q;
    }
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  const int k = *S.iter;
  const int cur = k % S.slots;
  double* res = S.res;
  if (have_closure) {
    const double Q = qsh;
    double mu, rho, energy;
    if (S.ensemble == 1) {
      rho = S.rho;
      mu = log(S.rho * S.volume / Q);
      energy = S.rho * S.volume * (mu - 1.0);
    } else {
      mu = S.mu;
      rho = tot[P_RHO] / S.volume / S.chain_len;
      energy = -rho * S.volume;
    }
    res[R_ACC] = tot[P_ACC];
    res[R_Q] = Q;
    res[R_LOGQ] = log(Q);
    res[R_MU] = mu;
    res[R_RHO] = rho;
    res[R_ENERGY] = energy;
    res[R_PHIW] = tot[P_PHIW];
    res[R_EINT] = tot[P_EINT];
    res[R_EEXT] = tot[P_EEXT];
    const double F = energy - tot[P_PHIW] + tot[P_EINT] + tot[P_EEXT];
    res[R_F] = F / (rho * S.volume);
    res[R_STATUS] = (isfinite(Q) && Q > 0.0 && isfinite(tot[P_ACC])) ? 0.0 : 4.0;
  }
  res[R_ITER] = (double)k;
  if (!do_mix) return;
  // Gram row of iteration k
  if (S.mixing_type == 3) {
    for (int j = 0; j < S.slots; ++j) {
      S.gram[cur * S.slots + j] = tot[NP_FIXED + j];
      S.gram[j * S.slots + cur] = tot[NP_FIXED + j];
    }
  }
  double* a = S.coef;
  double* b = S.coef + S.slots;
  for (int j = 0; j < S.slots; ++j) { a[j] = 0.0; b[j] = 0.0; }
  double lamused;
  if (S.mixing_type == 1) {
    lamused = S.lambda;
    a[cur] = 1.0; b[cur] = lamused;
  } else if (S.mixing_type == 2) {
    const double lammin = 1.0e-5;
    if (k == 1) {
      lamused = lammin;
    } else if (tot[P_LDEN] > 1.0e-50) {
      lamused = sqrt(tot[P_LNUM] / tot[P_LDEN]);
      if (lamused < lammin) lamused = lammin;
      else if (lamused > S.lambda) lamused = S.lambda;
    } else {
      lamused = lammin;
    }
    a[cur] = 1.0; b[cur] = lamused;
  } else {
    const int m = S.slots - 1;
    if (k > S.warm) {
      double U[SCF_MAX_HIST * SCF_MAX_HIST], v[SCF_MAX_HIST];
      const double g00 = S.gram[cur * S.slots + cur];
      for (int i = 0; i < m; ++i) {
        const int si = ((k - 1 - i) % S.slots + S.slots) % S.slots;
        const double g0i = S.gram[cur * S.slots + si];
        v[i] = g00 - g0i;
        for (int j = 0; j < m; ++j) {
          const int sj = ((k - 1 - j) % S.slots + S.slots) % S.slots;
          U[i * m + j] = g00 - g0i - S.gram[cur * S.slots + sj] + S.gram[si * S.slots + sj];
        }
      }
      lu_solve_nr(U, v, m);
      double csum = 0.0;
      for (int i = 0; i < m; ++i) {
        const int si = ((k - 1 - i) % S.slots + S.slots) % S.slots;
        a[si] = v[i];
        b[si] = S.lambda * v[i];
        csum += v[i];
      }
      lamused = S.lambda;
      a[cur] = 1.0 - csum;
      b[cur] = S.lambda * (1.0 - csum);
    } else {
      lamused = S.lam_warm;
      a[cur] = 1.0; b[cur] = lamused;
    }
  }
  res[R_LAMBDA] = lamused;
  *S.iter = k + 1;
}

__global__ void k_solve(ScfDev S, int have_closure, int do_mix) { solve_body(S, have_closure, do_mix); }

__global__ void k_solve_b(const ScfDev* __restrict__ Ss, int have_closure, int do_mix) {
  const ScfDev S = Ss[blockIdx.x];
  solve_body(S, have_closure, do_mix);
}

#endif  // ADSCF_SCF_IMPL

// x_{k+1} = sum_j a_j x_j + b_j r_j into the next history slot; optional
// E = exp(-ds x/2) for the pseudo-spectral propagator.  After the Anderson
// warm-up every b_j is lambda a_j, so with the history y_j = x_j + lambda r_j
// (written by the closure) the step is sum_j a_j y_j: half the history reads
// and FP64 multiply-adds.
template <typename T>
__device__ __forceinline__ void mix_body(const ScfDev& S, T* E, double ds, int bid, int nb) {
  __shared__ double ca[SCF_MAX_SLOTS], cb[SCF_MAX_SLOTS];
  __shared__ int nzj[SCF_MAX_SLOTS], nnz;
  const int kn = *S.iter;               // already advanced to k+1
  const int nxt = kn % S.slots;
  const int cur = (kn - 1) % S.slots;
  if (threadIdx.x < S.slots) {
    ca[threadIdx.x] = S.coef[threadIdx.x];
    cb[threadIdx.x] = S.coef[S.slots + threadIdx.x];
  }
  __syncthreads();
  // the slots with a nonzero a_j, in increasing j: the sum below skips the
  // others without a per-point FP64 comparison (GB300's FP64 pipe bounds
  // this kernel)
  if (threadIdx.x == 0) {
    int k = 0;
    for (int j = 0; j < S.slots; ++j)
      if (ca[j] != 0.0) nzj[k++] = j;
    nnz = k;
  }
  __syncthreads();
  const size_t nv = (size_t)S.ntypes * S.npts;
  const bool use_y = S.hy && S.mixing_type == 3 && kn - 1 > S.warm;
  for (size_t i = bid * (size_t)blockDim.x + threadIdx.x; i < nv; i += (size_t)nb * blockDim.x) {
    double x;
    const int z = (int)((i % S.npts) / S.plane);
    const bool interior = !S.wall_mask || (z > 0 && z < S.nplanes - 1);
    if (!interior) {
      x = S.hx[(size_t)cur * nv + i];
    } else if (use_y) {
      x = 0.0;
      for (int k = 0; k < nnz; ++k) {
        const int j = nzj[k];
        x += ca[j] * S.hy[(size_t)j * nv + i];
      }
    } else {
      x = 0.0;
      for (int j = 0; j < S.slots; ++j) {
        if (ca[j] != 0.0) x += ca[j] * S.hx[(size_t)j * nv + i];
        if (cb[j] != 0.0) x += cb[j] * S.hr[(size_t)j * nv + i];
      }
    }
    S.hx[(size_t)nxt * nv + i] = x;
    if (E) {  // interleaved Boltzmann factors of the next propagation (two species)
      const int c = i >= (size_t)S.npts;
      store_boltzmann(E, i - (size_t)c * S.npts, c, -0.5 * ds * x);
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(SCF_THREADS)
k_mix(ScfDev S, T* E, double ds) { mix_body<T>(S, E, ds, blockIdx.x, gridDim.x); }

// batch: instance blockIdx.y, its Boltzmann factors and ds from the ScfDev
template <typename T>
__global__ void __launch_bounds__(SCF_THREADS)
k_mix_b(const ScfDev* __restrict__ Ss, int nblocks) {
  const ScfDev S = Ss[blockIdx.y];
  mix_body<T>(S, static_cast<T*>(S.mixE), S.mixds, blockIdx.x, nblocks);
}

#ifdef ADSCF_SCF_IMPL
// Calculate_Mean_Fields alone (adscf_mean_fields), density -> field
__global__ void k_meanfield_only(ScfDev S, const double* __restrict__ dens, double* __restrict__ field) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < S.npts; p += gridDim.x * blockDim.x) {
    const int z = p / S.plane;
    if (S.homopolymer) {
      field[p] = S.ww * dens[p] + (S.ext ? S.ext[z] : 0.0);
      continue;
    }
    const double f0 = dens[p] * S.v0, f1 = dens[S.npts + p] * S.v1;
    const double tot = f0 + f1;
    const double u0 = S.ext ? S.ext[z] : 0.0;
    const double u1 = S.ext ? S.ext[S.nplanes + z] : 0.0;
    field[p] = (S.kappa * (tot - 1.0) + S.chi * f1 + u0) * S.v0;
    field[S.npts + p] = (S.kappa * (tot - 1.0) + S.chi * f0 + u1) * S.v1;
  }
}
#endif  // ADSCF_SCF_IMPL
