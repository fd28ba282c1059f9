// film_kernels.cuh -- Crank-Nicolson / Douglas-ADI propagators for films and
// brushes on sm_103a.
//
// Reference: Propagate_Step of Film_CK_AD/Film_1D/Geometry_Modules/
// mod_realspace.f90:24-79 (1D CN, Dirichlet walls), of Brush_CK_AD/
// Geometry_Modules/mod_realspace.f90:26-79 (same with a per-call ds), of
// Film_CK_AD/Film_3D/Geometry_Modules/mod_realspace.f90:22-140 (Douglas ADI,
// periodic x/y with Sherman-Morrison cyclic solves :149-176, Dirichlet z with
// tridiag :184-215), the chain loops of Propagate_Diblock (Film_1D/
// Polymer_Modules/mod_diblock.f90:127-150) and Propagate_Homopolymer
// (Brush_CK_AD/Polymer_Modules/mod_homopolymer.f90:204-239).
//
// Layout: films are [z][y][x] with z = 0..gz (both walls); a "line" is one
// (x, y) column.  All arrays indexed [z][line] so consecutive threads
// (consecutive lines) touch consecutive addresses.
#pragma once
#include "common.cuh"
#include "scf_kernels.cuh"

#define FILM_THREADS 128

// where a chain finds its field: a direct pointer, or the current slot of
// the device SCF history (located through the device iteration counter)
struct FieldRef {
  const double* direct;
  const double* hx;
  const int* iter;
  int slots;
  size_t nv;
  __device__ __forceinline__ const double* get() const {
    if (direct) return direct;
    return hx + (size_t)((*iter) % slots) * nv;
  }
};

template <typename T>
struct FilmDev {
  int gx, gy, gz;        // gz = intervals, planes 0..gz
  int nlines, npts;      // gx*gy, nlines*(gz+1)
  int ns, na;            // contour steps; A-block steps of the forward chain
  int ntypes;            // 2 diblock, 1 homopolymer
  int brush;             // q-dagger starts from the grafting distribution
  int single;            // one step of one propagator already in slice 0 (field type 0)
  int span;              // integrator span: 0 full (Film_3D), 1 interior
  const double* alpha;   // [gz+1] 1/(h1 (h1+h2))  (a_z = -ds alpha)
  const double* beta;    // [gz+1] b_z / ds
  const double* gamma;   // [gz+1] 1/(h2 (h1+h2))  (c_z = -ds gamma)
  const double* dss;     // [ns+1] contour steps, dss[0] = 0
  const double* wA;      // [ns+1] contour weights of block A (or homopolymer)
  const double* wB;      // [ns+1] contour weights of block B
  const double* wz;      // [gz+1] integration weights dx dy w_z
  const double* graft;   // [gz+1] grafting distribution (brush), or null
  T* q;                  // [(ns+1)][npts]
  T* qd;                 // [(ns+1)][npts]
  T* gam;                // [2][gz+1][nlines] Thomas scratch (one per chain)
  double* dist;          // [ntypes][npts]
  double* qpart;         // [nblocks] partial sums of Q
  int* err;              // pivot / non-finite flags
  // ADI (Film_3D) only
  double dx, dy;
  T* w1;                 // [2][npts] intermediate q*, q** of the ADI sweeps
};

// chain type of step s: forward A then B, backward B then A
__device__ __forceinline__ int film_type(int dir, int s, int ns, int na) {
  return dir == 0 ? (s <= na ? 0 : 1) : (s <= ns - na ? 1 : 0);
}
__device__ __forceinline__ double film_ds(const double* dss, int dir, int s, int ns) {
  return dir == 0 ? dss[s] : dss[ns + 1 - s];
}

// ---------------------------------------------------------------------------
// 1D CN chains: one thread per (line, chain) walks all contour steps; the
// NR Thomas sweep (Film_3D/.../mod_realspace.f90:184-215) in precision T.
// Row j of step s: a_j = -ds alpha_j, c_j = -ds gamma_j, b_j = ds beta_j,
//   (1 + b_j + ds w_j / 2) q'_j + a_j q'_{j-1} + c_j q'_{j+1}
//     = -a_j q_{j-1} + (1 - b_j - ds w_j / 2) q_j - c_j q_{j+1},
// rows 0 and gz are identity with zero right-hand side (Dirichlet walls).
// blockIdx.y = chain (0 forward, 1 backward).
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void film1d_chain(const FilmDev<T>& F, const double* field, int line, int dir) {
  const int L = F.nlines, gz = F.gz;
  T* chain = dir == 0 ? F.q : F.qd;
  T* gam = F.gam + (size_t)dir * (gz + 1) * L;
  // node 0: q_0 = 1; the brush's q-dagger_0 is the grafting distribution
  if (!F.single)
    for (int j = 0; j <= gz; ++j)
      chain[(size_t)j * L + line] = (dir == 1 && F.brush) ? (T)F.graft[j] : (T)1;
  for (int s = 1; s <= F.ns; ++s) {
    const double ds = film_ds(F.dss, dir, s, F.ns);
    const int ty = (F.brush || F.single) ? 0 : film_type(dir, s, F.ns, F.na);
    const double* w = field + (size_t)ty * F.npts;
    const T* qp = chain + (size_t)(s - 1) * F.npts;
    T* qn = chain + (size_t)s * F.npts;
    // forward elimination
    T bet = (T)1;            // row 0: identity
    T uprev = (T)0;          // u_0 = 0 (zero right-hand side)
    qn[line] = (T)0;
    T cprev = (T)0;          // c_0 = 0
    T q_jm1 = qp[line], q_j = qp[(size_t)L + line];
    for (int j = 1; j <= gz; ++j) {
      T a, c, diag, rhs;
      if (j < gz) {
        const T q_jp1 = qp[(size_t)(j + 1) * L + line];
        a = (T)(-ds * F.alpha[j]);
        c = (T)(-ds * F.gamma[j]);
        const T b = (T)(ds * F.beta[j]);
        const T hw = (T)(0.5 * ds * w[(size_t)j * L + line]);
        diag = (T)1 + b + hw;
        rhs = -a * q_jm1 + ((T)1 - b - hw) * q_j - c * q_jp1;
        q_jm1 = q_j;
        q_j = q_jp1;
      } else {
        a = (T)0; c = (T)0; diag = (T)1; rhs = (T)0;
      }
      const T g = cprev / bet;
      bet = diag - a * g;
      if (bet == (T)0) atomicOr(F.err, 1);
      uprev = (rhs - a * uprev) / bet;
      gam[(size_t)j * L + line] = g;
      qn[(size_t)j * L + line] = uprev;
      cprev = c;
    }
    // back substitution u_j -= gam_{j+1} u_{j+1}
    T unext = uprev;
    for (int j = gz - 1; j >= 0; --j) {
      const T u = qn[(size_t)j * L + line] - gam[(size_t)(j + 1) * L + line] * unext;
      qn[(size_t)j * L + line] = u;
      unext = u;
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(FILM_THREADS)
k_film1d_chains(FilmDev<T> F, FieldRef fr) {
  const int line = blockIdx.x * blockDim.x + threadIdx.x;
  if (line >= F.nlines) return;
  film1d_chain<T>(F, fr.get(), line, blockIdx.y);
}

// ---------------------------------------------------------------------------
// Douglas ADI (Film_3D/.../mod_realspace.f90:22-140), one contour step, both
// chains (blockIdx.y).  Sweep kernels work in precision T on slices T.
// ---------------------------------------------------------------------------
// NR Thomas on a register-free line held in shared/global memory is done
// inline below.  Cyclic solve (Sherman-Morrison, :149-176) for constant
// coefficients a, b, c on a periodic line of n points: corners m(0,n-1) = a,
// m(n-1,0) = c.  rhs/out are strided views.
template <typename T>
__device__ __forceinline__ void cyclic_solve(const T a, const T b, const T c, int n,
                                             const T* rhs, size_t rs, T* out, size_t os,
                                             T* gam, T* z, size_t gs, int* err) {
  if (n < 3) {  // Film_3D/.../mod_realspace.f90:157-158
    const T v = rhs[0] / (b + a + c);
    for (int i = 0; i < n; ++i) out[i * os] = v;
    return;
  }
  const T gmm = -b;
  // B = A with bb(0) = b - gamma, bb(n-1) = b - a c / gamma; solve B y = r and
  // B z = u (u_0 = gamma, u_{n-1} = c) in one sweep (same pivots)
  T bet = b - gmm;
  T y = rhs[0] / bet;
  T zz = gmm / bet;
  out[0] = y;
  z[0] = zz;
  for (int j = 1; j < n; ++j) {
    const T g = c / bet;
    const T bj = (j == n - 1) ? b - a * c / gmm : b;
    bet = bj - a * g;
    if (bet == (T)0) atomicOr(err, 1);
    y = (rhs[j * rs] - a * y) / bet;
    const T uj = (j == n - 1) ? c : (T)0;
    zz = (uj - a * zz) / bet;
    gam[j * gs] = g;
    out[j * os] = y;
    z[j * gs] = zz;
  }
  for (int j = n - 2; j >= 0; --j) {
    out[j * os] = out[j * os] - gam[(j + 1) * gs] * out[(j + 1) * os];
    z[j * gs] = z[j * gs] - gam[(j + 1) * gs] * z[(j + 1) * gs];
  }
  const T fact = (out[0] + a * out[(n - 1) * os] / gmm) / ((T)1 + z[0] + a * z[(n - 1) * gs] / gmm);
  for (int j = 0; j < n; ++j) out[j * os] = out[j * os] - fact * z[j * gs];
}

// x sweep: (1 - ds Dxx/2) q* = [1 + ds Dxx/2 + ds Dyy + ds Dzz - ds w] q  (:90-102)
// one thread per (y, z interior); q* written to w1.
template <typename T>
__global__ void __launch_bounds__(FILM_THREADS)
k_adi_x(FilmDev<T> F, FieldRef fr, int s) {
  const int gx = F.gx, gy = F.gy, gz = F.gz, L = F.nlines;
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  const int dir = blockIdx.y;
  if (id >= gy * (gz - 1)) return;
  const int y = id % gy, z = 1 + id / gy;
  const double ds = film_ds(F.dss, dir, s, F.ns);
  const int ty = (F.brush || F.single) ? 0 : film_type(dir, s, F.ns, F.na);
  const double* w = fr.get() + (size_t)ty * F.npts;
  const T* p0 = (dir == 0 ? F.q : F.qd) + (size_t)(s - 1) * F.npts;
  T* out = F.w1 + (size_t)dir * F.npts;
  const T ax = (T)(-ds / F.dx / F.dx / 2.0), bx = (T)(ds / F.dx / F.dx), cx = ax;
  const T ay = (T)(-ds / F.dy / F.dy / 2.0), by = (T)(ds / F.dy / F.dy), cy = ay;
  const T az = (T)(-ds * F.alpha[z]), bz = (T)(ds * F.beta[z]), cz = (T)(-ds * F.gamma[z]);
  const int ym = (y + gy - 1) % gy, yp = (y + 1) % gy;
  const size_t row = (size_t)z * L + (size_t)y * gx;
  // right-hand side into the output row (then solved in place)
  for (int x = 0; x < gx; ++x) {
    const int xm = (x + gx - 1) % gx, xp = (x + 1) % gx;
    const T c0 = p0[row + x];
    const T r = -ax * p0[row + xm] - (T)2 * ay * p0[(size_t)z * L + (size_t)ym * gx + x] -
                (T)2 * az * p0[(size_t)(z - 1) * L + (size_t)y * gx + x] - cx * p0[row + xp] -
                (T)2 * cy * p0[(size_t)z * L + (size_t)yp * gx + x] -
                (T)2 * cz * p0[(size_t)(z + 1) * L + (size_t)y * gx + x] +
                ((T)1 - bx - by * (T)2 - bz * (T)2 - (T)(ds * w[row + x])) * c0;
    out[row + x] = r;
  }
  // scratch for this line: gam and z vectors in the gam buffer, [x][line id]
  T* gbase = F.gam + (size_t)dir * 2 * (size_t)gx * (gy * (gz - 1)) ;
  cyclic_solve<T>(ax, (T)1 + bx, cx, gx, out + row, 1, out + row, 1, gbase + id,
                  gbase + (size_t)gx * (gy * (gz - 1)) + id, (size_t)(gy * (gz - 1)), F.err);
}

// y sweep: (1 - ds Dyy/2) q** = q* - ds Dyy q / 2  (:108-119); one thread
// per (x, z interior); q** written to w1 in place.
template <typename T>
__global__ void __launch_bounds__(FILM_THREADS)
k_adi_y(FilmDev<T> F, int s) {
  const int gx = F.gx, gy = F.gy, gz = F.gz, L = F.nlines;
  const int id = blockIdx.x * blockDim.x + threadIdx.x;
  const int dir = blockIdx.y;
  if (id >= gx * (gz - 1)) return;
  const int x = id % gx, z = 1 + id / gx;
  const double ds = film_ds(F.dss, dir, s, F.ns);
  const T* p0 = (dir == 0 ? F.q : F.qd) + (size_t)(s - 1) * F.npts;
  T* w1 = F.w1 + (size_t)dir * F.npts;
  const T ay = (T)(-ds / F.dy / F.dy / 2.0), by = (T)(ds / F.dy / F.dy), cy = ay;
  const size_t col = (size_t)z * L + x;
  for (int y = 0; y < gy; ++y) {
    const int ym = (y + gy - 1) % gy, yp = (y + 1) % gy;
    const size_t i = col + (size_t)y * gx;
    w1[i] = ay * p0[col + (size_t)ym * gx] + w1[i] + by * p0[i] + cy * p0[col + (size_t)yp * gx];
  }
  T* gbase = F.gam + (size_t)dir * 2 * (size_t)gy * (gx * (gz - 1));
  cyclic_solve<T>(ay, (T)1 + by, cy, gy, w1 + col, gx, w1 + col, gx, gbase + id,
                  gbase + (size_t)gy * (gx * (gz - 1)) + id, (size_t)(gx * (gz - 1)), F.err);
}

// z sweep: (1 - ds Dzz/2 + ds w/2) q' = q** - ds Dzz q / 2 + ds w q / 2
// (:125-139), Dirichlet rows 0 and gz; one thread per (x, y); writes slice s.
template <typename T>
__global__ void __launch_bounds__(FILM_THREADS)
k_adi_z(FilmDev<T> F, FieldRef fr, int s) {
  const int gz = F.gz, L = F.nlines;
  const int line = blockIdx.x * blockDim.x + threadIdx.x;
  const int dir = blockIdx.y;
  if (line >= L) return;
  const double ds = film_ds(F.dss, dir, s, F.ns);
  const int ty = (F.brush || F.single) ? 0 : film_type(dir, s, F.ns, F.na);
  const double* w = fr.get() + (size_t)ty * F.npts;
  const T* p0 = (dir == 0 ? F.q : F.qd) + (size_t)(s - 1) * F.npts;
  const T* w1 = F.w1 + (size_t)dir * F.npts;
  T* qn = (dir == 0 ? F.q : F.qd) + (size_t)s * F.npts;
  T* gam = F.gam + (size_t)dir * (gz + 1) * L;
  T bet = (T)1, uprev = (T)0, cprev = (T)0;
  qn[line] = (T)0;
  for (int j = 1; j <= gz; ++j) {
    T a, c, diag, rhs;
    const size_t i = (size_t)j * L + line;
    if (j < gz) {
      a = (T)(-ds * F.alpha[j]);
      c = (T)(-ds * F.gamma[j]);
      const T bz = (T)(ds * F.beta[j]);
      const T hw = (T)(0.5 * ds * w[i]);
      diag = (T)1 + bz + hw;
      rhs = a * p0[i - L] + w1[i] + (bz + hw) * p0[i] + c * p0[i + L];
    } else {
      a = (T)0; c = (T)0; diag = (T)1; rhs = (T)0;
    }
    const T g = cprev / bet;
    bet = diag - a * g;
    if (bet == (T)0) atomicOr(F.err, 1);
    uprev = (rhs - a * uprev) / bet;
    gam[i] = g;
    qn[i] = uprev;
    cprev = c;
  }
  T unext = uprev;
  for (int j = gz - 1; j >= 0; --j) {
    const size_t i = (size_t)j * L + line;
    const T u = qn[i] - gam[i + L] * unext;
    qn[i] = u;
    unext = u;
  }
}

// node 0 of both chains = 1 (ADI films)
template <typename T>
__global__ void k_film_fill(T* __restrict__ q, T* __restrict__ qd, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    q[i] = (T)1;
    qd[i] = (T)1;
  }
}

// ---------------------------------------------------------------------------
// Contour integrals phi_c = sum_s W_c[s] q_s qdag_{N-s} (FP64 accumulation of
// exact products) and Q = integrator(q_N) (diblock, Film_1D/.../
// mod_diblock.f90:154) or integrator(qdag_0 q_N) (brush, mod_homopolymer.f90:
// 226), with the per-plane weights wz.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void film_contour_body(const FilmDev<T>& F, int bid, int nb) {
  __shared__ double red[32];
  const int N = F.ns;
  const size_t np = F.npts;
  double qs = 0.0;
  for (int p = bid * blockDim.x + threadIdx.x; p < F.npts; p += nb * blockDim.x) {
    double a0 = 0.0, a1 = 0.0;
    for (int s = 0; s <= N; ++s) {
      const double pr = (double)F.q[(size_t)s * np + p] * (double)F.qd[(size_t)(N - s) * np + p];
      a0 += F.wA[s] * pr;
      if (F.ntypes == 2) a1 += F.wB[s] * pr;
    }
    F.dist[p] = a0;
    if (F.ntypes == 2) F.dist[np + p] = a1;
    const int z = p / F.nlines;
    double qn = (double)F.q[(size_t)N * np + p];
    if (F.brush) qn *= (double)F.qd[p];
    qs += F.wz[z] * qn;
  }
  const double tot = block_reduce_1(qs, red);
  if (threadIdx.x == 0) F.qpart[bid] = tot;
}

template <typename T>
__global__ void __launch_bounds__(256)
k_film_contour(FilmDev<T> F) { film_contour_body<T>(F, blockIdx.x, gridDim.x); }

// ---------------------------------------------------------------------------
// Film batches: many independent one-line films (Film_1D or brush), each
// with its own mesh, contour schedule and SCF state.  `films` lists the batch
// instances that sweep in precision T (a graded mesh keeps FP64), ordered by
// contour length so a warp's threads walk similar step counts.  The field of
// instance f is the current slot of its SCF history.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(FILM_THREADS)
k_film1d_chains_b(const FilmDev<T>* __restrict__ Fs, const ScfDev* __restrict__ Ss,
                  const int* __restrict__ films, int nf) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nf) return;
  const int f = films[k];
  // by value: the sweep's stores could alias a struct read through a pointer,
  // which would force a reload of every field pointer per point
  const FilmDev<T> F = Fs[f];
  const double* field = Ss[f].hx + (size_t)((*Ss[f].iter) % Ss[f].slots) * ((size_t)Ss[f].ntypes * Ss[f].npts);
  film1d_chain<T>(F, field, 0, blockIdx.y);
}

// One-line films of a batch with the line held in shared memory.  One thread
// per (film, chain), blockIdx.y = chain; blockDim.x = W lanes.  The Thomas
// sweep of film1d_chain runs on the same arithmetic in the same order, but q
// is updated in place in shared memory (u_j replaces q_j once q_j and
// q_{j+1} have been read) with the elimination factors beside it, both
// interleaved [j][lane] so that a warp's accesses fall in distinct banks.
// Only the finished slice goes to global memory (for the contour integral);
// the sweep itself never waits on a global load of its own stores.
// Shared memory: 2 zcap W elements, zcap >= gz + 1 of every listed film.
template <typename T>
__global__ void __launch_bounds__(32)
k_film1d_chains_sm(const FilmDev<T>* __restrict__ Fs, const ScfDev* __restrict__ Ss,
                   const int* __restrict__ films, int nf, int zcap) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int W = blockDim.x, lane = threadIdx.x;
  const int k = blockIdx.x * W + lane;
  if (k >= nf) return;
  const int f = films[k];
  const FilmDev<T> F = Fs[f];
  const double* field = Ss[f].hx + (size_t)((*Ss[f].iter) % Ss[f].slots) * ((size_t)Ss[f].ntypes * Ss[f].npts);
  T* qv = reinterpret_cast<T*>(smraw) + lane;
  T* gv = qv + (size_t)zcap * W;
  const int dir = blockIdx.y, gz = F.gz;
  T* chain = dir == 0 ? F.q : F.qd;
  for (int j = 0; j <= gz; ++j) {
    const T v = (dir == 1 && F.brush) ? (T)F.graft[j] : (T)1;
    qv[j * W] = v;
    chain[j] = v;
  }
  for (int s = 1; s <= F.ns; ++s) {
    const double ds = film_ds(F.dss, dir, s, F.ns);
    const int ty = F.brush ? 0 : film_type(dir, s, F.ns, F.na);
    const double* w = field + (size_t)ty * F.npts;
    T* qn = chain + (size_t)s * F.npts;
    T bet = (T)1, uprev = (T)0, cprev = (T)0;
    T q_jm1 = qv[0], q_j = qv[W];
    qv[0] = (T)0;
#pragma unroll 4
    for (int j = 1; j < gz; ++j) {
      const T q_jp1 = qv[(j + 1) * W];
      const T a = (T)(-ds * F.alpha[j]);
      const T c = (T)(-ds * F.gamma[j]);
      const T b = (T)(ds * F.beta[j]);
      const T hw = (T)(0.5 * ds * w[j]);
      const T diag = (T)1 + b + hw;
      const T rhs = -a * q_jm1 + ((T)1 - b - hw) * q_j - c * q_jp1;
      q_jm1 = q_j;
      q_j = q_jp1;
      const T g = cprev / bet;
      bet = diag - a * g;
      if (bet == (T)0) atomicOr(F.err, 1);
      uprev = (rhs - a * uprev) / bet;
      gv[j * W] = g;
      qv[j * W] = uprev;
      cprev = c;
    }
    {  // row gz: identity, zero right-hand side
      const T g = cprev / bet;
      bet = (T)1;
      uprev = ((T)0 - (T)0 * uprev) / bet;
      gv[gz * W] = g;
    }
    T unext = uprev;
    qv[gz * W] = unext;
    qn[gz] = unext;
    for (int j = gz - 1; j >= 0; --j) {
      const T u = qv[j * W] - gv[(j + 1) * W] * unext;
      qv[j * W] = u;
      qn[j] = u;
      unext = u;
    }
  }
}

// one block per film of the list
template <typename T>
__global__ void __launch_bounds__(256)
k_film_contour_b(const FilmDev<T>* __restrict__ Fs, const int* __restrict__ films) {
  const FilmDev<T> F = Fs[films[blockIdx.x]];
  film_contour_body<T>(F, 0, 1);
}

// ---------------------------------------------------------------------------
// Free energy of a film or brush at fixed fields and its gradient with
// respect to the wall potential U_c(z), chi (diblock) or ww (brush).  At fixed
// w the densities do not depend on U, so dF/dU_c(z) = w_z sum_xy v_c phi_c /
// (rho V); the energy terms follow Calculate_Energy with the external term
// (Film_CK_AD/Film_1D/Main_Diblock_Melt/main_diblock_melt.f90).  One block
// per plane sums its lines; a one-thread kernel combines the planes.
// ---------------------------------------------------------------------------
enum { FE_S0 = 0, FE_S1, FE_PHIW, FE_EINT, FE_EEXT, FE_X01, FE_RHO, FE_N };

static __global__ void __launch_bounds__(256) k_film_fe(ScfDev S, const double* __restrict__ w,
                                                 double* __restrict__ part) {
  __shared__ double red[FE_N * 32];
  const double Q = q_total(S);
  const double scale = density_scale(S, Q);
  const int z = blockIdx.x;
  double acc[FE_N];
#pragma unroll
  for (int k = 0; k < FE_N; ++k) acc[k] = 0.0;
  for (int l = threadIdx.x; l < S.plane; l += blockDim.x) {
    const int p = z * S.plane + l;
    const double phi0 = scale * S.dist[p];
    if (S.homopolymer) {
      const double u = S.ext ? S.ext[z] : 0.0;
      acc[FE_S0] += phi0;
      acc[FE_PHIW] += phi0 * w[p];
      acc[FE_EINT] += 0.5 * S.ww * phi0 * phi0;
      acc[FE_EEXT] += u * phi0;
      acc[FE_X01] += 0.5 * phi0 * phi0;
      acc[FE_RHO] += phi0;
    } else {
      const double phi1 = scale * S.dist[S.npts + p];
      const double f0 = S.v0 * phi0, f1 = S.v1 * phi1, tot = f0 + f1;
      const double u0 = S.ext ? S.ext[z] : 0.0, u1 = S.ext ? S.ext[S.nplanes + z] : 0.0;
      acc[FE_S0] += f0;
      acc[FE_S1] += f1;
      acc[FE_PHIW] += phi0 * w[p] + phi1 * w[S.npts + p];
      acc[FE_EINT] += 0.5 * S.kappa * (tot - 1.0) * (tot - 1.0) + S.chi * f0 * f1;
      acc[FE_EEXT] += u0 * f0 + u1 * f1;
      acc[FE_X01] += f0 * f1;
      acc[FE_RHO] += phi0 + phi1;
    }
  }
  const double r = block_reduce_k<FE_N>(acc, red);
  if (threadIdx.x < FE_N) part[z * FE_N + threadIdx.x] = r;
}

// out: [0] F, [1] dF/dchi (brush: dF/dww), [2 + c*nplanes + z] dF/dU_c(z)
static __global__ void k_film_fe_sc(ScfDev S, const double* __restrict__ part, double* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double Q = q_total(S);
  double t[FE_N] = {0, 0, 0, 0, 0, 0, 0};
  for (int z = 0; z < S.nplanes; ++z)
    for (int k = 0; k < FE_N; ++k) t[k] += S.wz[z] * part[z * FE_N + k];
  double rho, energy;
  if (S.ensemble == 1) {
    rho = S.rho;
    energy = S.rho * S.volume * (log(S.rho * S.volume / Q) - 1.0);
  } else {
    rho = t[FE_RHO] / S.volume / S.chain_len;
    energy = -rho * S.volume;
  }
  const double rv = rho * S.volume;
  out[0] = (energy - t[FE_PHIW] + t[FE_EINT] + t[FE_EEXT]) / rv;
  out[1] = t[FE_X01] / rv;
  for (int z = 0; z < S.nplanes; ++z) {
    out[2 + z] = S.wz[z] * part[z * FE_N + FE_S0] / rv;
    if (S.ntypes == 2) out[2 + S.nplanes + z] = S.wz[z] * part[z * FE_N + FE_S1] / rv;
  }
}
