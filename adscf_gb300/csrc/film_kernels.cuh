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
  // FP32 line sweeps (1D chains): FP32 copies of the mesh factors and, for
  // single contexts, of the field ([ntypes][npts], filled per propagation)
  const float* alf;
  const float* bef;
  const float* gaf;
  float* wf;
  // FP32 ADI sweeps: per contour-schedule entry k (ds = dss[k]) the FP32
  // coefficients ax, bx, ay, by, ds, ds/2, formed in FP64 on the host
  const float* adicf;
};

// ---------------------------------------------------------------------------
// Coefficients of CN row j at step size ds: a = -ds alpha_j, c = -ds gamma_j,
// b = ds beta_j and hw = ds w_j / 2.  FP64 sweeps form each product in FP64
// and round once.  FP32 sweeps multiply FP32 copies of the mesh factors and
// of the field by the FP32 step: at most one more rounding per factor, on a
// sweep that rounds every operation at that level.  Two FP64 products and a
// conversion per factor per row would make the FP32 sweeps wait on GB300's
// narrow FP64 pipe.
// ---------------------------------------------------------------------------
// Right-hand side of CN row j.  FP64 sweeps use the reference's form,
// -a q_{j-1} + (1 - b - hw) q_j - c q_{j+1}.  FP32 sweeps solve for the
// increment u = q' - q of the step instead: the same matrix with right-hand
// side -2 [a (q_{j-1} - q_j) + c (q_{j+1} - q_j) + hw q_j] (b = -(a + c)
// exactly in the mesh formulas), and rows 0 and gz give u = -q.  The
// differences keep a constant profile invariant under the rounded
// coefficients, and the solve's rounding is relative to the O(ds) increment
// rather than to the O(ds/dz^2) matrix entries, which would otherwise bias
// the decay of smooth modes coherently over the contour.
// Explicitly rounded arithmetic of the 1D line sweeps.  The single-context
// and the batched kernels inline the same sweep into different code; with
// every operation rounded explicitly no contraction choice of the compiler
// can make the two differ, and a batched film follows its single context
// bit for bit in either precision.
__device__ __forceinline__ float r_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double r_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float r_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double r_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float r_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double r_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float r_div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double r_div(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float r_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double r_fma(double a, double b, double c) { return __fma_rn(a, b, c); }

template <typename T>
__device__ __forceinline__ T cn_rhs(T a, T b, T c, T hw, T qm, T q0, T qp) {
  if constexpr (sizeof(T) == 4) {
    T t = r_mul(hw, q0);
    t = r_fma(c, r_sub(qp, q0), t);
    t = r_fma(a, r_sub(qm, q0), t);
    return r_mul((T)-2, t);
  } else {
    T t = r_mul(-a, qm);
    t = r_fma(r_sub(r_sub((T)1, b), hw), q0, t);
    return r_fma(-c, qp, t);
  }
}

struct CnStep {
  double ds;
  float dsf, hdsf;       // (float)ds, (float)(ds / 2)
};
__device__ __forceinline__ CnStep cn_step(double ds) {
  return CnStep{ds, (float)ds, (float)(0.5 * ds)};
}
template <typename T>
__device__ __forceinline__ void cn_row(const FilmDev<T>& F, const CnStep& st, int j, double w64, float w32,
                                       T& a, T& c, T& b, T& hw) {
  if constexpr (sizeof(T) == 4) {
    // b_j = ds (alpha_j + gamma_j) exactly in the mesh formulas: b = -(a + c)
    // keeps the rounded row conservative and spares a load and a product
    a = r_mul(-st.dsf, F.alf[j]);
    c = r_mul(-st.dsf, F.gaf[j]);
    b = -r_add(a, c);
    hw = r_mul(st.hdsf, w32);
  } else {
    a = (T)(-st.ds * F.alpha[j]);
    c = (T)(-st.ds * F.gamma[j]);
    b = (T)(st.ds * F.beta[j]);
    hw = (T)(0.5 * st.ds * w64);
  }
}

// the hardware reciprocal (MUFU, within one ulp): one instruction on the
// sweep's critical path instead of a correctly rounded sequence
__device__ __forceinline__ float rcp_hw(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// One row of the Thomas elimination: returns gam_j and advances the pivot
// state, the eliminated right-hand side and c_{j-1}.  FP64 divides by the
// pivot (bet = pivot); FP32 keeps its reciprocal (bet = 1 / pivot) and
// multiplies: one reciprocal instead of two divisions per row (the FP32
// sweeps are bound by instruction issue; the increment form keeps the
// reciprocal's ulp relative to the small increment).  Row 0 starts from
// bet = 1 in both forms.
template <typename T>
__device__ __forceinline__ T thomas_row(T& bet, T& cprev, T& uprev, T a, T c, T diag, T rhs, int* err) {
  if constexpr (sizeof(T) == 4) {
    const T g = r_mul(cprev, bet);
    const T piv = r_fma(-a, g, diag);
    if (piv == (T)0) atomicOr(err, 1);
    bet = rcp_hw(piv);
    uprev = r_mul(r_fma(-a, uprev, rhs), bet);
    cprev = c;
    return g;
  } else {
    const T g = r_div(cprev, bet);
    bet = r_fma(-a, g, diag);
    if (bet == (T)0) atomicOr(err, 1);
    uprev = r_div(r_fma(-a, uprev, rhs), bet);
    cprev = c;
    return g;
  }
}

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
    const CnStep st = cn_step(film_ds(F.dss, dir, s, F.ns));
    const int ty = (F.brush || F.single) ? 0 : film_type(dir, s, F.ns, F.na);
    const double* w = field + (size_t)ty * F.npts;
    const float* wl = sizeof(T) == 4 ? F.wf + (size_t)ty * F.npts : nullptr;
    const T* qp = chain + (size_t)(s - 1) * F.npts;
    T* qn = chain + (size_t)s * F.npts;
    // forward elimination (increment form for FP32 sweeps, see cn_rhs)
    constexpr bool inc = sizeof(T) == 4;
    T bet = (T)1;            // row 0: identity
    T q_jm1 = qp[line], q_j = qp[(size_t)L + line];
    T uprev = inc ? -q_jm1 : (T)0;   // zero right-hand side (increment: -q_0)
    qn[line] = uprev;
    T cprev = (T)0;          // c_0 = 0
    for (int j = 1; j <= gz; ++j) {
      T a, c, diag, rhs;
      if (j < gz) {
        const T q_jp1 = qp[(size_t)(j + 1) * L + line];
        const size_t i = (size_t)j * L + line;
        T b, hw;
        cn_row<T>(F, st, j, sizeof(T) == 4 ? 0.0 : w[i], sizeof(T) == 4 ? wl[i] : 0.f, a, c, b, hw);
        diag = r_add(r_add((T)1, b), hw);
        rhs = cn_rhs<T>(a, b, c, hw, q_jm1, q_j, q_jp1);
        q_jm1 = q_j;
        q_j = q_jp1;
      } else {
        a = (T)0; c = (T)0; diag = (T)1; rhs = inc ? -q_j : (T)0;
      }
      gam[(size_t)j * L + line] = thomas_row<T>(bet, cprev, uprev, a, c, diag, rhs, F.err);
      qn[(size_t)j * L + line] = uprev;
    }
    // back substitution u_j -= gam_{j+1} u_{j+1} (increment: q' = q + u)
    T unext = uprev;
    if (inc) qn[(size_t)gz * L + line] = r_add(q_j, unext);
    for (int j = gz - 1; j >= 0; --j) {
      const size_t i = (size_t)j * L + line;
      const T u = r_fma(-gam[i + L], unext, qn[i]);
      qn[i] = inc ? r_add(qp[i], u) : u;
      unext = u;
    }
  }
}

// FP32 copy of the current field for the FP32 line sweeps of a single context
static __global__ void k_film_wconv(FieldRef fr, float* __restrict__ wf, size_t n) {
  const double* w = fr.get();
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    wf[i] = (float)w[i];
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

// The three sweeps keep each thread's line in shared memory, interleaved
// [point][lane] (blockDim.x = W lanes, conflict-free): the right-hand side
// is formed there, solved in place, and written out once, so the serial
// recurrences wait on shared-memory latency instead of on global loads of
// their own stores.  The slices and q* that a sweep only reads go through
// the non-coherent path (__ldg), and the write-back loops load nothing they
// store: otherwise the compiler keeps every load behind the previous
// point's store (it cannot prove them disjoint) and a line's write-back
// waits on one memory latency per point.  Shared memory per block: adi_smem(n, W, sizeof(T)).
__host__ __device__ __forceinline__ size_t adi_smem(int n, int W, size_t es) { return 3 * (size_t)n * W * es; }
// the y sweep also keeps q* of its line (write-back without reloads)
__host__ __device__ __forceinline__ size_t adi_smem_y(int n, int W, size_t es) { return 4 * (size_t)n * W * es; }

// FP32 sweeps read the FP32 field copy; FP64 sweeps the field
template <typename T>
__device__ __forceinline__ T adi_dsw(const FilmDev<T>& F, const CnStep& st, const double* w, int ty, size_t i) {
  if constexpr (sizeof(T) == 4) return st.dsf * F.wf[(size_t)ty * F.npts + i];
  else return (T)(st.ds * w[i]);
}

// x sweep: (1 - ds Dxx/2) q* = [1 + ds Dxx/2 + ds Dyy + ds Dzz - ds w] q  (:90-102)
// one thread per (y, z interior); q* written to w1.
template <typename T>
__global__ void __launch_bounds__(FILM_THREADS)
k_adi_x(FilmDev<T> F, FieldRef fr, int s) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int gx = F.gx, gy = F.gy, gz = F.gz, L = F.nlines, W = blockDim.x;
  const int id = blockIdx.x * W + threadIdx.x;
  const int dir = blockIdx.y;
  if (id >= gy * (gz - 1)) return;
  T* r = reinterpret_cast<T*>(smraw) + threadIdx.x;
  T* gs = r + (size_t)gx * W;
  T* zs = gs + (size_t)gx * W;
  const int y = id % gy, z = 1 + id / gy;
  const double ds = film_ds(F.dss, dir, s, F.ns);
  const CnStep st = cn_step(ds);
  const int ty = (F.brush || F.single) ? 0 : film_type(dir, s, F.ns, F.na);
  const double* w = sizeof(T) == 4 ? nullptr : fr.get() + (size_t)ty * F.npts;
  const T* p0 = (dir == 0 ? F.q : F.qd) + (size_t)(s - 1) * F.npts;
  T* out = F.w1 + (size_t)dir * F.npts;
  const T ax = (T)(-ds / F.dx / F.dx / 2.0), bx = (T)(ds / F.dx / F.dx), cx = ax;
  const T ay = (T)(-ds / F.dy / F.dy / 2.0), by = (T)(ds / F.dy / F.dy), cy = ay;
  const T az = (T)(-ds * F.alpha[z]), bz = (T)(ds * F.beta[z]), cz = (T)(-ds * F.gamma[z]);
  const int ym = (y + gy - 1) % gy, yp = (y + 1) % gy;
  const size_t row = (size_t)z * L + (size_t)y * gx;
  for (int x = 0; x < gx; ++x) {
    const int xm = (x + gx - 1) % gx, xp = (x + 1) % gx;
    const T c0 = __ldg(p0 + row + x);
    const T qxm = __ldg(p0 + row + xm), qxp = __ldg(p0 + row + xp);
    const T qym = __ldg(p0 + (size_t)z * L + (size_t)ym * gx + x);
    const T qyp = __ldg(p0 + (size_t)z * L + (size_t)yp * gx + x);
    const T qzm = __ldg(p0 + (size_t)(z - 1) * L + (size_t)y * gx + x);
    const T qzp = __ldg(p0 + (size_t)(z + 1) * L + (size_t)y * gx + x);
    const T dsw = adi_dsw<T>(F, st, w, ty, row + x);
    if constexpr (sizeof(T) == 4)   // increment q* - q (b = -(a + c) on every axis; see cn_rhs)
      r[x * W] = (T)-2 * (ax * (qxm - c0) + cx * (qxp - c0) + ay * (qym - c0) + cy * (qyp - c0) +
                          az * (qzm - c0) + cz * (qzp - c0)) - dsw * c0;
    else
      r[x * W] = -ax * qxm - (T)2 * ay * qym - (T)2 * az * qzm - cx * qxp - (T)2 * cy * qyp - (T)2 * cz * qzp +
                 ((T)1 - bx - by * (T)2 - bz * (T)2 - dsw) * c0;
  }
  cyclic_solve<T>(ax, (T)1 + bx, cx, gx, r, W, r, W, gs, zs, W, F.err);
  for (int x = 0; x < gx; ++x) out[row + x] = sizeof(T) == 4 ? __ldg(p0 + row + x) + r[x * W] : r[x * W];
}

// y sweep: (1 - ds Dyy/2) q** = q* - ds Dyy q / 2  (:108-119); one thread
// per (x, z interior); q** written to w1 in place.
template <typename T>
__global__ void __launch_bounds__(FILM_THREADS)
k_adi_y(FilmDev<T> F, int s) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int gx = F.gx, gy = F.gy, gz = F.gz, L = F.nlines, W = blockDim.x;
  const int id = blockIdx.x * W + threadIdx.x;
  const int dir = blockIdx.y;
  if (id >= gx * (gz - 1)) return;
  T* r = reinterpret_cast<T*>(smraw) + threadIdx.x;
  T* gs = r + (size_t)gy * W;
  T* zs = gs + (size_t)gy * W;
  T* ws = zs + (size_t)gy * W;      // q* of the line, for the write-back
  const int x = id % gx, z = 1 + id / gx;
  const double ds = film_ds(F.dss, dir, s, F.ns);
  const T* p0 = (dir == 0 ? F.q : F.qd) + (size_t)(s - 1) * F.npts;
  T* w1 = F.w1 + (size_t)dir * F.npts;
  const T ay = (T)(-ds / F.dy / F.dy / 2.0), by = (T)(ds / F.dy / F.dy), cy = ay;
  const size_t col = (size_t)z * L + x;
  for (int y = 0; y < gy; ++y) {
    const int ym = (y + gy - 1) % gy, yp = (y + 1) % gy;
    const size_t i = col + (size_t)y * gx, im = col + (size_t)ym * gx, ip = col + (size_t)yp * gx;
    if constexpr (sizeof(T) == 4) {   // increment q** - q* from e = q - q*
      const T w1i = w1[i];
      ws[y * W] = w1i;
      const T e0 = __ldg(p0 + i) - w1i;
      r[y * W] = ay * ((__ldg(p0 + im) - w1[im]) - e0) + cy * ((__ldg(p0 + ip) - w1[ip]) - e0);
    } else {
      r[y * W] = ay * __ldg(p0 + im) + w1[i] + by * __ldg(p0 + i) + cy * __ldg(p0 + ip);
    }
  }
  cyclic_solve<T>(ay, (T)1 + by, cy, gy, r, W, r, W, gs, zs, W, F.err);
  for (int y = 0; y < gy; ++y) {
    const size_t i = col + (size_t)y * gx;
    w1[i] = sizeof(T) == 4 ? ws[y * W] + r[y * W] : r[y * W];
  }
}

// z sweep: (1 - ds Dzz/2 + ds w/2) q' = q** - ds Dzz q / 2 + ds w q / 2
// (:125-139), Dirichlet rows 0 and gz; one thread per (x, y); writes slice s.
template <typename T>
__global__ void __launch_bounds__(FILM_THREADS)
k_adi_z(FilmDev<T> F, FieldRef fr, int s) {
  extern __shared__ __align__(16) unsigned char smraw[];
  const int gz = F.gz, L = F.nlines, W = blockDim.x;
  const int line = blockIdx.x * W + threadIdx.x;
  const int dir = blockIdx.y;
  if (line >= L) return;
  T* us = reinterpret_cast<T*>(smraw) + threadIdx.x;
  T* gs = us + (size_t)(gz + 1) * W;
  const CnStep st = cn_step(film_ds(F.dss, dir, s, F.ns));
  const int ty = (F.brush || F.single) ? 0 : film_type(dir, s, F.ns, F.na);
  const double* w = sizeof(T) == 4 ? nullptr : fr.get() + (size_t)ty * F.npts;
  const float* wl = sizeof(T) == 4 ? F.wf + (size_t)ty * F.npts : nullptr;
  const T* p0 = (dir == 0 ? F.q : F.qd) + (size_t)(s - 1) * F.npts;
  const T* w1 = F.w1 + (size_t)dir * F.npts;
  T* qn = (dir == 0 ? F.q : F.qd) + (size_t)s * F.npts;
  // FP32: increment q' - q** from f = q - q** (q** = 0 on the walls)
  constexpr bool inc = sizeof(T) == 4;
  T bet = (T)1, uprev = (T)0, cprev = (T)0;
  T f_jm1 = __ldg(p0 + line), f_j = inc && gz > 1 ? __ldg(p0 + (size_t)L + line) - __ldg(w1 + (size_t)L + line) : (T)0;
  us[0] = (T)0;
  for (int j = 1; j <= gz; ++j) {
    T a, c, diag, rhs;
    const size_t i = (size_t)j * L + line;
    if (j < gz) {
      T bz, hw;
      cn_row<T>(F, st, j, sizeof(T) == 4 ? 0.0 : w[i], sizeof(T) == 4 ? wl[i] : 0.f, a, c, bz, hw);
      diag = (T)1 + bz + hw;
      if constexpr (inc) {
        const T f_jp1 = j + 1 < gz ? __ldg(p0 + i + L) - __ldg(w1 + i + L) : __ldg(p0 + i + L);
        rhs = a * (f_jm1 - f_j) + c * (f_jp1 - f_j) + hw * f_j;
        f_jm1 = f_j;
        f_j = f_jp1;
      } else {
        rhs = a * __ldg(p0 + i - L) + __ldg(w1 + i) + (bz + hw) * __ldg(p0 + i) + c * __ldg(p0 + i + L);
      }
    } else {
      a = (T)0; c = (T)0; diag = (T)1; rhs = (T)0;
    }
    gs[j * W] = thomas_row<T>(bet, cprev, uprev, a, c, diag, rhs, F.err);
    us[j * W] = uprev;
  }
  T unext = uprev;
  qn[(size_t)gz * L + line] = unext;
  for (int j = gz - 1; j >= 0; --j) {
    const size_t i = (size_t)j * L + line;
    const T u = us[j * W] - gs[(j + 1) * W] * unext;
    qn[i] = inc && j > 0 ? __ldg(w1 + i) + u : u;
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
// FP32 slices: each product q_s qdag_{N-s} is exact as a float pair (TwoProd),
// the weight is split into a float pair staged in shared memory, and the sum
// over s is compensated (float-float, ~48 bits): FP32 units instead of
// GB300's narrow FP64 pipe, which two FP64 multiply-adds per node and point
// would wait on.  FP64 slices keep plain FP64 accumulation.
constexpr int kFilmContourChunk = 256;   // contour nodes per staged weight chunk

__device__ __forceinline__ void ffw_add(float& sh, float& sl, float x, float y, float2 w) {
  const float p = x * y;
  const float e = fmaf(x, y, -p);                // x y = p + e exactly
  const float t = p * w.x;
  const float te = fmaf(p, w.x, -t);             // p wh = t + te exactly
  const float lo = fmaf(e, w.x, fmaf(p, w.y, te));
  const float s = sh + t;                        // TwoSum(sh, t)
  const float bp = s - sh;
  const float err = (sh - (s - bp)) + (t - bp);
  sl += err + lo;
  sh = s;
}

template <typename T>
__device__ __forceinline__ void film_contour_body(const FilmDev<T>& F, int bid, int nb) {
  __shared__ double red[32];
  const int N = F.ns;
  const size_t np = F.npts;
  double qs = 0.0;
  if constexpr (sizeof(T) == 4) {
    __shared__ float2 wsh[2][kFilmContourChunk];
    for (int pb = bid * blockDim.x; pb < F.npts; pb += nb * blockDim.x) {   // uniform per block
      const int p = pb + threadIdx.x;
      const bool ok = p < F.npts;
      float ah = 0.f, al = 0.f, bh = 0.f, bl = 0.f;
      for (int s0 = 0; s0 <= N; s0 += kFilmContourChunk) {
        const int cn = min(kFilmContourChunk, N + 1 - s0);
        __syncthreads();
        for (int k = threadIdx.x; k < cn; k += blockDim.x) {
          const double wa = F.wA[s0 + k];
          const float wah = (float)wa;
          wsh[0][k] = make_float2(wah, (float)(wa - (double)wah));
          const double wb = F.ntypes == 2 ? F.wB[s0 + k] : 0.0;
          const float wbh = (float)wb;
          wsh[1][k] = make_float2(wbh, (float)(wb - (double)wbh));
        }
        __syncthreads();
        if (ok) {
#pragma unroll 8
          for (int k = 0; k < cn; ++k) {
            const int s = s0 + k;
            const float x = F.q[(size_t)s * np + p], y = F.qd[(size_t)(N - s) * np + p];
            ffw_add(ah, al, x, y, wsh[0][k]);
            if (F.ntypes == 2) ffw_add(bh, bl, x, y, wsh[1][k]);
          }
        }
      }
      if (ok) {
        F.dist[p] = (double)ah + (double)al;
        if (F.ntypes == 2) F.dist[np + p] = (double)bh + (double)bl;
        const int z = p / F.nlines;
        double qn = (double)F.q[(size_t)N * np + p];
        if (F.brush) qn *= (double)F.qd[p];
        qs += F.wz[z] * qn;
      }
    }
  } else {
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
// per (film, chain), blockIdx.y = chain; W = per_warp lanes in each warp of
// the block.  The Thomas
// sweep of film1d_chain runs on the same arithmetic in the same order, on
// q, the elimination factors and the eliminated right-hand side in shared
// memory, interleaved [j][lane] so that a warp's accesses fall in distinct
// banks; the back substitution writes the new q over the old one.
// Only the finished slice goes to global memory (for the contour integral);
// the sweep itself never waits on a global load of its own stores.  FP32
// sweeps also keep the film's field in FP32 there.
// Shared memory: 3 zcap W elements of T (q, gam, the eliminated right-hand
// side) + 2 zcap W floats for FP32 sweeps, zcap >= gz + 1 of every film.
template <typename T>
__global__ void __launch_bounds__(256)
k_film1d_chains_sm(const FilmDev<T>* __restrict__ Fs, const ScfDev* __restrict__ Ss,
                   const int* __restrict__ films, int nf, int zcap, int per_warp) {
  extern __shared__ __align__(16) unsigned char smraw[];
  constexpr bool inc = sizeof(T) == 4;
  // the first per_warp lanes of each warp work (a warp's instruction stream
  // is serial, so few lanes per warp means more streams per SM)
  if ((threadIdx.x & 31) >= per_warp) return;
  const int W = (blockDim.x >> 5) * per_warp;
  const int lane = (threadIdx.x >> 5) * per_warp + (threadIdx.x & 31);
  const int k = blockIdx.x * W + lane;
  if (k >= nf) return;
  const int f = films[k];
  const FilmDev<T> F = Fs[f];
  const double* field = Ss[f].hx + (size_t)((*Ss[f].iter) % Ss[f].slots) * ((size_t)Ss[f].ntypes * Ss[f].npts);
  T* qv = reinterpret_cast<T*>(smraw) + lane;
  T* gv = qv + (size_t)zcap * W;
  T* dv = gv + (size_t)zcap * W;
  float* wv = reinterpret_cast<float*>(reinterpret_cast<T*>(smraw) + 3 * (size_t)zcap * W) + lane;
  const int dir = blockIdx.y, gz = F.gz;
  T* chain = dir == 0 ? F.q : F.qd;
  for (int j = 0; j <= gz; ++j) {
    const T v = (dir == 1 && F.brush) ? (T)F.graft[j] : (T)1;
    qv[j * W] = v;
    chain[j] = v;
  }
  if constexpr (sizeof(T) == 4) {   // the field in FP32, once per propagation
    for (int ty = 0; ty < F.ntypes; ++ty)
      for (int j = 0; j <= gz; ++j) wv[((size_t)ty * zcap + j) * W] = (float)field[(size_t)ty * F.npts + j];
  }
  for (int s = 1; s <= F.ns; ++s) {
    const CnStep st = cn_step(film_ds(F.dss, dir, s, F.ns));
    const int ty = F.brush ? 0 : film_type(dir, s, F.ns, F.na);
    const double* w = field + (size_t)ty * F.npts;
    const float* wl = wv + (size_t)ty * zcap * W;
    T* qn = chain + (size_t)s * F.npts;
    T bet = (T)1, cprev = (T)0;
    T q_jm1 = qv[0], q_j = qv[W];
    T uprev = inc ? -q_jm1 : (T)0;
    dv[0] = uprev;
#pragma unroll 4
    for (int j = 1; j < gz; ++j) {
      const T q_jp1 = qv[(j + 1) * W];
      T a, c, b, hw;
      cn_row<T>(F, st, j, sizeof(T) == 4 ? 0.0 : w[j], sizeof(T) == 4 ? wl[j * W] : 0.f, a, c, b, hw);
      const T diag = r_add(r_add((T)1, b), hw);
      const T rhs = cn_rhs<T>(a, b, c, hw, q_jm1, q_j, q_jp1);
      q_jm1 = q_j;
      q_j = q_jp1;
      gv[j * W] = thomas_row<T>(bet, cprev, uprev, a, c, diag, rhs, F.err);
      dv[j * W] = uprev;
    }
    // row gz: identity (zero right-hand side; increment: -q_gz)
    gv[gz * W] = thomas_row<T>(bet, cprev, uprev, (T)0, (T)0, (T)1, inc ? -q_j : (T)0, F.err);
    T unext = uprev;
    {
      const T v = inc ? r_add(q_j, unext) : unext;
      qv[gz * W] = v;
      qn[gz] = v;
    }
#pragma unroll 4
    for (int j = gz - 1; j >= 0; --j) {
      const T u = r_fma(-gv[(j + 1) * W], unext, dv[j * W]);
      const T v = inc ? r_add(qv[j * W], u) : u;
      qv[j * W] = v;
      qn[j] = v;
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
  const double Q = q_total_serial(S);
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
