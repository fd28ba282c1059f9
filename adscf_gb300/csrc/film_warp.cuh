// film_warp.cuh -- warp-cooperative tridiagonal line solves for the FP32
// (split precision) Crank-Nicolson sweeps of films and brushes.
//
// The reference solves every line with a serial Thomas recurrence (tridiag,
// Film_CK_AD/Film_3D/Geometry_Modules/mod_realspace.f90:184-215; the 1D CN
// step of Film_1D/.../mod_realspace.f90:24-79).  One thread per line leaves
// a GB300 with a few warps per SM, each waiting on a chain of dependent
// operations as long as the line.  Here G lanes of a warp share one line:
//
//  - lane l owns the contiguous rows [s_l, e_l] of the line (a chunk of at
//    most M rows, held in registers across all contour steps); the last row
//    e_l of each chunk is a separator;
//  - each lane eliminates its interior rows [s_l, e_l - 1] once with three
//    right-hand sides, so that every interior unknown is
//    u_i = x_i + y_i u(e_{l-1}) + z_i u(e_l)   (left and own separator);
//  - substituting these into the separator rows gives one tridiagonal
//    equation per lane in the separators alone,
//    A_l u(e_{l-1}) + B_l u(e_l) + C_l u(e_{l+1}) = R_l,
//    solved by parallel cyclic reduction across the G lanes (log2 G steps of
//    shuffles); a periodic line closes the reduced system cyclically;
//  - the interior unknowns then follow from their lane's two separators.
//
// The matrix is that of the reference; only the elimination order differs,
// so the result equals the serial solve up to FP32 rounding (the systems are
// diagonally dominant: 1 + hw > 0 beyond the off-diagonals).  Pivots are FP32
// reciprocals (rcp.approx, as the serial FP32 sweeps); a zero pivot sets the
// error flag like the serial solve.  The sweeps solve for the increment
// u = q' - q of the step (see cn_rhs), so Dirichlet rows give u = -q.
#pragma once
#include "film_kernels.cuh"

namespace fw {

// One line system on the G-lane group of the calling lane.  Lane l of the
// group owns K consecutive rows (rows past the line's end are identity rows
// that couple to nothing); row K-1 of each lane is its separator.  The rows
// are given as arrays of the sub-diagonal a, the diagonal d, the
// super-diagonal c and the right-hand side r; the solution u is returned in
// place of r.  `periodic`: row 0 of lane 0 couples to the last lane's
// separator through a, and that separator to row 0 through c (all G lanes
// own rows).  K is a compile-time constant so that every row stays in
// registers.  All G lanes of the group must call it together.
template <int G, int K>
__device__ __forceinline__ void solve(const float (&a)[K], const float (&d)[K], const float (&c)[K],
                                      float (&r)[K], bool periodic, int* err) {
  static_assert(K >= 2, "a lane needs an interior row and a separator");
  const int lane = threadIdx.x & 31;
  const int gl = lane & (G - 1);          // lane within the group
  const int base = lane - gl;
  const unsigned mask = 0xffffffffu;
  float x[K - 1], y[K - 1], z[K - 1], g[K - 1];
  // local elimination of the interior rows 0..K-2 with three right-hand
  // sides: r, -a_0 at the first row, -c_{K-2} at the last row
  float bet = 1.f;
#pragma unroll
  for (int i = 0; i < K - 1; ++i) {
    const int im = i > 0 ? i - 1 : 0;
    const float gi = i == 0 ? 0.f : __fmul_rn(c[im], bet);
    const float piv = i == 0 ? d[0] : __fmaf_rn(-a[i], gi, d[i]);
    if (piv == 0.f) atomicOr(err, 1);
    bet = rcp_hw(piv);
    g[i] = gi;
    x[i] = __fmul_rn(i == 0 ? r[0] : __fmaf_rn(-a[i], x[im], r[i]), bet);
    y[i] = __fmul_rn(i == 0 ? -a[0] : __fmul_rn(-a[i], y[im]), bet);
    const float zr = i == K - 2 ? -c[i] : 0.f;
    z[i] = __fmul_rn(i == 0 ? zr : __fmaf_rn(-a[i], z[im], zr), bet);
  }
#pragma unroll
  for (int i = K - 3; i >= 0; --i) {
    x[i] = __fmaf_rn(-g[i + 1], x[i + 1], x[i]);
    y[i] = __fmaf_rn(-g[i + 1], y[i + 1], y[i]);
    z[i] = __fmaf_rn(-g[i + 1], z[i + 1], z[i]);
  }
  // the separator row in its neighbours' terms: the last interior row of this
  // lane and the first interior row of the next lane
  constexpr int S = K - 1, Li = K - 2;
  const int nx = base + ((gl + 1) & (G - 1));
  float xn = __shfl_sync(mask, x[0], nx), yn = __shfl_sync(mask, y[0], nx), zn = __shfl_sync(mask, z[0], nx);
  if (!periodic && gl == G - 1) { xn = 0.f; yn = 0.f; zn = 0.f; }
  float A = __fmul_rn(a[S], y[Li]);
  float B = __fmaf_rn(c[S], yn, __fmaf_rn(a[S], z[Li], d[S]));
  float C = __fmul_rn(c[S], zn);
  float R = __fmaf_rn(-c[S], xn, __fmaf_rn(-a[S], x[Li], r[S]));
  // parallel cyclic reduction over the group (identity beyond its ends
  // unless periodic)
#pragma unroll
  for (int st = 1; st < G; st *= 2) {
    const int su = base + ((gl - st) & (G - 1)), sd = base + ((gl + st) & (G - 1));
    float Au = __shfl_sync(mask, A, su), Bu = __shfl_sync(mask, B, su);
    float Cu = __shfl_sync(mask, C, su), Ru = __shfl_sync(mask, R, su);
    float Ad = __shfl_sync(mask, A, sd), Bd = __shfl_sync(mask, B, sd);
    float Cd = __shfl_sync(mask, C, sd), Rd = __shfl_sync(mask, R, sd);
    if (!periodic && gl - st < 0) { Au = 0.f; Bu = 1.f; Cu = 0.f; Ru = 0.f; }
    if (!periodic && gl + st >= G) { Ad = 0.f; Bd = 1.f; Cd = 0.f; Rd = 0.f; }
    if (Bu == 0.f || Bd == 0.f) atomicOr(err, 1);
    const float kl = __fmul_rn(A, rcp_hw(Bu));
    const float kr = __fmul_rn(C, rcp_hw(Bd));
    const float nB = __fmaf_rn(-kr, Ad, __fmaf_rn(-kl, Cu, B));
    const float nR = __fmaf_rn(-kr, Rd, __fmaf_rn(-kl, Ru, R));
    A = __fmul_rn(-kl, Au);
    C = __fmul_rn(-kr, Cd);
    B = nB;
    R = nR;
  }
  // after log2 G steps the reduced equation couples only to the lane itself:
  // periodic lines reach it through both neighbours, open lines never
  const float den = periodic ? __fadd_rn(__fadd_rn(A, C), B) : B;
  if (den == 0.f) atomicOr(err, 1);
  const float v = __fmul_rn(R, rcp_hw(den));          // u at this lane's separator
  float vl = __shfl_sync(mask, v, base + ((gl - 1) & (G - 1)));
  if (!periodic && gl == 0) vl = 0.f;
#pragma unroll
  for (int i = 0; i < K - 1; ++i) r[i] = __fmaf_rn(z[i], v, __fmaf_rn(y[i], vl, x[i]));
  r[S] = v;
}

}  // namespace fw

// ---------------------------------------------------------------------------
// 1D CN chain (Film_1D / brush, FP32 increment form) with one warp per
// (line, chain): lane l owns rows [l K, l K + K - 1] of the line's gz + 1
// rows (K = film_warp_rows; rows past the wall are identity padding), keeps
// their q in registers for the whole contour, exchanges edge values by
// shuffles, and solves each step with fw::solve.  Per-warp shared
// memory `sm` holds, by row: the FP32 mesh factors alpha, gamma, the FP32
// field of types 0 and 1, and a staging row through which each finished
// slice goes to global memory (coalesced for one-line films).  `chain`:
// slices [(ns+1)][npts] of the chain, rows of this line at stride `stride`.
// ---------------------------------------------------------------------------
constexpr int kFilmWarpM = 8;                 // rows per lane at most: lines up to 32 * 8 planes
constexpr int kFilmWarpRows = 32 * kFilmWarpM;
struct FilmWarpSm {
  float al[kFilmWarpRows], ga[kFilmWarpRows], w0[kFilmWarpRows], w1[kFilmWarpRows], stage[kFilmWarpRows];
};

template <int K>
__device__ __forceinline__ void film1d_chain_warp(const FilmDev<float>& F, int dir, float* chain,
                                                  size_t stride, FilmWarpSm& sm) {
  const int lane = threadIdx.x & 31;
  const int n = F.gz + 1;
  const int s0 = lane * K;                    // this lane's rows s0 .. s0 + K - 1
  float q[K];
#pragma unroll
  for (int i = 0; i < K; ++i) {
    const int j = s0 + i;
    float v = 0.f;
    if (j < n) v = F.single ? chain[(size_t)j * stride] : (dir == 1 && F.brush) ? (float)F.graft[j] : 1.f;
    q[i] = v;
  }
  if (!F.single) {
#pragma unroll
    for (int i = 0; i < K; ++i)
      if (s0 + i < n) sm.stage[s0 + i] = q[i];
    __syncwarp();
    for (int j = lane; j < n; j += 32) chain[(size_t)j * stride] = sm.stage[j];
    __syncwarp();
  }
  for (int s = 1; s <= F.ns; ++s) {
    const CnStep st = cn_step(film_ds(F.dss, dir, s, F.ns));
    const int ty = (F.brush || F.single) ? 0 : film_type(dir, s, F.ns, F.na);
    const float* wl = ty == 0 ? sm.w0 : sm.w1;
    // edge values of the neighbouring lanes' rows
    const float qprev = __shfl_up_sync(0xffffffffu, q[K - 1], 1);
    const float qnext = __shfl_down_sync(0xffffffffu, q[0], 1);
    float a[K], d[K], c[K], r[K];
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const int j = s0 + i;
      a[i] = 0.f; d[i] = 1.f; c[i] = 0.f; r[i] = 0.f;
      if (j < n) {
        if (j == 0 || j == n - 1) {
          r[i] = -q[i];                        // Dirichlet wall: q' = 0
        } else {
          const float qm = i == 0 ? qprev : q[i > 0 ? i - 1 : 0];
          const float qp = i == K - 1 ? qnext : q[i + 1 < K ? i + 1 : i];
          const float ai = __fmul_rn(-st.dsf, sm.al[j]);
          const float ci = __fmul_rn(-st.dsf, sm.ga[j]);
          const float bi = -__fadd_rn(ai, ci);
          const float hw = __fmul_rn(st.hdsf, wl[j]);
          a[i] = ai;
          c[i] = ci;
          d[i] = __fadd_rn(__fadd_rn(1.f, bi), hw);
          r[i] = cn_rhs<float>(ai, bi, ci, hw, qm, q[i], qp);
        }
      }
    }
    fw::solve<32, K>(a, d, c, r, false, F.err);
    float* qn = chain + (size_t)s * F.npts;
#pragma unroll
    for (int i = 0; i < K; ++i) {
      q[i] = __fadd_rn(q[i], r[i]);
      if (s0 + i < n) sm.stage[s0 + i] = q[i];
    }
    __syncwarp();
    for (int j = lane; j < n; j += 32) qn[(size_t)j * stride] = sm.stage[j];
    __syncwarp();
  }
}

// rows per lane of an n-row line: the smallest K >= 2 with 32 K >= n
__host__ __device__ __forceinline__ int film_warp_rows(int n) { return n <= 64 ? 2 : (n + 31) / 32; }

__device__ __forceinline__ void film1d_chain_warp_any(const FilmDev<float>& F, int dir, float* chain,
                                                      size_t stride, FilmWarpSm& sm) {
  switch (film_warp_rows(F.gz + 1)) {
    case 2: film1d_chain_warp<2>(F, dir, chain, stride, sm); break;
    case 3: film1d_chain_warp<3>(F, dir, chain, stride, sm); break;
    case 4: film1d_chain_warp<4>(F, dir, chain, stride, sm); break;
    case 5: film1d_chain_warp<5>(F, dir, chain, stride, sm); break;
    case 6: film1d_chain_warp<6>(F, dir, chain, stride, sm); break;
    case 7: film1d_chain_warp<7>(F, dir, chain, stride, sm); break;
    default: film1d_chain_warp<8>(F, dir, chain, stride, sm); break;
  }
}

// mesh factors and FP32 field of one line into the warp's shared memory
__device__ __forceinline__ void film_warp_tables(const FilmDev<float>& F, const float* w0, const float* w1,
                                                 size_t wstride, FilmWarpSm& sm) {
  const int lane = threadIdx.x & 31;
  for (int j = lane; j <= F.gz; j += 32) {
    sm.al[j] = F.alf[j];
    sm.ga[j] = F.gaf[j];
    sm.w0[j] = w0[(size_t)j * wstride];
    sm.w1[j] = w1 ? w1[(size_t)j * wstride] : 0.f;
  }
  __syncwarp();
}

// Single context (Film_1D / brush lines of one film): one warp per (line,
// chain); blockIdx.y = chain.
static __global__ void __launch_bounds__(128)
k_film1d_warp(FilmDev<float> F) {
  __shared__ FilmWarpSm sm_all[4];
  const int wib = threadIdx.x >> 5;
  const int line = blockIdx.x * 4 + wib;
  if (line >= F.nlines) return;
  const int dir = blockIdx.y;
  const size_t L = F.nlines;
  FilmWarpSm& sm = sm_all[wib];
  film_warp_tables(F, F.wf + line, F.ntypes == 2 ? F.wf + F.npts + line : nullptr, L, sm);
  film1d_chain_warp_any(F, dir, (dir == 0 ? F.q : F.qd) + line, L, sm);
}

// Batch: one warp per (film, chain) of `items` ((film << 1) | chain, longest
// contours first), the field from the film's current SCF history slot.
static __global__ void __launch_bounds__(128)
k_film1d_warp_b(const FilmDev<float>* __restrict__ Fs, const ScfDev* __restrict__ Ss,
                const int* __restrict__ items, int nitems) {
  __shared__ FilmWarpSm sm_all[4];
  const int wib = threadIdx.x >> 5;
  const int it = blockIdx.x * 4 + wib;
  if (it >= nitems) return;
  const int f = items[it] >> 1, dir = items[it] & 1;
  const FilmDev<float> F = Fs[f];
  const ScfDev& S = Ss[f];
  const double* field = S.hx + (size_t)((*S.iter) % S.slots) * ((size_t)S.ntypes * S.npts);
  FilmWarpSm& sm = sm_all[wib];
  const int lane = threadIdx.x & 31;
  for (int j = lane; j <= F.gz; j += 32) {
    sm.al[j] = F.alf[j];
    sm.ga[j] = F.gaf[j];
    sm.w0[j] = (float)field[j];
    sm.w1[j] = F.ntypes == 2 ? (float)field[F.npts + j] : 0.f;
  }
  __syncwarp();
  film1d_chain_warp_any(F, dir, dir == 0 ? F.q : F.qd, 1, sm);
}

// ---------------------------------------------------------------------------
// Douglas ADI sweeps (Film_CK_AD/Film_3D/Geometry_Modules/mod_realspace.f90:
// 22-140) in FP32 increment form with the warp solver: G lanes per line, K
// consecutive points per lane (G K = gx or gy for the periodic x and y lines;
// G K >= gz + 1 for the Dirichlet z lines, padded with identity rows), 32 / G
// lines per warp.  Same right-hand sides as k_adi_x / k_adi_y / k_adi_z; the
// x and y systems are the reference's periodic ones (cyclicTriDiag, :149-176)
// solved with the reduced system closed cyclically.  blockIdx.y = chain.
// ---------------------------------------------------------------------------
// Shape of a warp-solver sweep: G lanes per line, K points per lane (g = 0:
// the one-thread-per-line kernels); staged: the tile goes through shared
// memory (k_adi_yz_s, y and z sweeps).
struct AdiShape {
  int g, k, staged;
};

// Per-chain FP32 coefficients of a step, read from the context's table
// (formed in FP64 on the host, rounded as k_adi_x / k_adi_y form them per
// thread): forming them on the device would keep GB300's narrow FP64 pipe
// and a block barrier on every sweep's critical path.
struct AdiCoef {
  float ax, bx, ay, by, dsf, hdsf;
};
__device__ __forceinline__ AdiCoef adi_coef(const FilmDev<float>& F, int dir, int s) {
  const float* c = F.adicf + 6 * (dir == 0 ? s : F.ns + 1 - s);
  return AdiCoef{__ldg(c), __ldg(c + 1), __ldg(c + 2), __ldg(c + 3), __ldg(c + 4), __ldg(c + 5)};
}

template <int G, int K>
__global__ void __launch_bounds__(128)
k_adi_x_w(FilmDev<float> F, int s) {
  constexpr int LPW = 32 / G;
  const int gx = F.gx, gy = F.gy, gz = F.gz, L = F.nlines;
  const int lane = threadIdx.x & 31, gl = lane & (G - 1);
  const int id = (blockIdx.x * 4 + (threadIdx.x >> 5)) * LPW + lane / G;   // line (y, z interior)
  const int dir = blockIdx.y;
  const bool live = id < gy * (gz - 1);
  const int y = live ? id % gy : 0, z = live ? 1 + id / gy : 1;
  const AdiCoef cf = adi_coef(F, dir, s);
  const int ty = (F.brush || F.single) ? 0 : film_type(dir, s, F.ns, F.na);
  const float* p0 = (dir == 0 ? F.q : F.qd) + (size_t)(s - 1) * F.npts;
  float* out = F.w1 + (size_t)dir * F.npts;
  const float* wf = F.wf + (size_t)ty * F.npts;
  const float ax = cf.ax, bx = cf.bx, cx = ax;
  const float ay = cf.ay, cy = ay;
  // z couplings as the z sweep forms them (cn_row, FP32 mesh factors)
  const float az = __fmul_rn(-cf.dsf, F.alf[z]), cz = __fmul_rn(-cf.dsf, F.gaf[z]);
  const int ym = (y + gy - 1) % gy, yp = (y + 1) % gy;
  const size_t row = (size_t)z * L + (size_t)y * gx, rym = (size_t)z * L + (size_t)ym * gx,
               ryp = (size_t)z * L + (size_t)yp * gx, rzm = row - L, rzp = row + L;
  const int x0 = gl * K;
  float c0[K];
#pragma unroll
  for (int i = 0; i < K; ++i) c0[i] = live ? __ldg(p0 + row + x0 + i) : 0.f;
  const int base = lane - gl;
  const float left = __shfl_sync(0xffffffffu, c0[K - 1], base + ((gl - 1) & (G - 1)));
  const float right = __shfl_sync(0xffffffffu, c0[0], base + ((gl + 1) & (G - 1)));
  float a[K], d[K], c[K], r[K];
#pragma unroll
  for (int i = 0; i < K; ++i) {
    const int x = x0 + i;
    const float qxm = i == 0 ? left : c0[i > 0 ? i - 1 : 0];
    const float qxp = i == K - 1 ? right : c0[i + 1 < K ? i + 1 : i];
    float qym = 0.f, qyp = 0.f, qzm = 0.f, qzp = 0.f, dsw = 0.f;
    if (live) {
      qym = __ldg(p0 + rym + x); qyp = __ldg(p0 + ryp + x);
      qzm = __ldg(p0 + rzm + x); qzp = __ldg(p0 + rzp + x);
      dsw = cf.dsf * wf[row + x];
    }
    const float q0 = c0[i];
    r[i] = -2.f * (ax * (qxm - q0) + cx * (qxp - q0) + ay * (qym - q0) + cy * (qyp - q0) +
                   az * (qzm - q0) + cz * (qzp - q0)) - dsw * q0;
    a[i] = ax; c[i] = cx; d[i] = 1.f + bx;
  }
  fw::solve<G, K>(a, d, c, r, true, F.err);
  if (live) {
#pragma unroll
    for (int i = 0; i < K; ++i) out[row + x0 + i] = c0[i] + r[i];
  }
}

template <int G, int K>
__global__ void __launch_bounds__(128)
k_adi_y_w(FilmDev<float> F, int s) {
  constexpr int LPW = 32 / G;
  const int gx = F.gx, gy = F.gy, gz = F.gz, L = F.nlines;
  const int lane = threadIdx.x & 31, gl = lane & (G - 1);
  const int id = (blockIdx.x * 4 + (threadIdx.x >> 5)) * LPW + lane / G;   // line (x, z interior)
  const int dir = blockIdx.y;
  const bool live = id < gx * (gz - 1);
  const int x = live ? id % gx : 0, z = live ? 1 + id / gx : 1;
  const AdiCoef cf = adi_coef(F, dir, s);
  const float* p0 = (dir == 0 ? F.q : F.qd) + (size_t)(s - 1) * F.npts;
  float* w1 = F.w1 + (size_t)dir * F.npts;
  const float ay = cf.ay, by = cf.by, cy = ay;
  const size_t col = (size_t)z * L + x;
  const int y0 = gl * K;
  // e = q - q* at the lane's points; q* kept for the write-back
  float e[K], ws[K];
#pragma unroll
  for (int i = 0; i < K; ++i) {
    const size_t idx = col + (size_t)(y0 + i) * gx;
    ws[i] = live ? w1[idx] : 0.f;
    e[i] = live ? __ldg(p0 + idx) - ws[i] : 0.f;
  }
  const int base = lane - gl;
  const float left = __shfl_sync(0xffffffffu, e[K - 1], base + ((gl - 1) & (G - 1)));
  const float right = __shfl_sync(0xffffffffu, e[0], base + ((gl + 1) & (G - 1)));
  float a[K], d[K], c[K], r[K];
#pragma unroll
  for (int i = 0; i < K; ++i) {
    const float em = i == 0 ? left : e[i > 0 ? i - 1 : 0];
    const float ep = i == K - 1 ? right : e[i + 1 < K ? i + 1 : i];
    r[i] = ay * (em - e[i]) + cy * (ep - e[i]);
    a[i] = ay; c[i] = cy; d[i] = 1.f + by;
  }
  fw::solve<G, K>(a, d, c, r, true, F.err);
  if (live) {
#pragma unroll
    for (int i = 0; i < K; ++i) w1[col + (size_t)(y0 + i) * gx] = ws[i] + r[i];
  }
}

// x and y sweeps of one interior plane in one block (gx = gy = N = G K, all N
// lines of a sweep at once: N G threads).  The plane of the previous slice
// and the x sweep's result stay in shared memory ([y][x]), so the y sweep
// reads no global memory and the plane leaves once, row by row.  Right-hand
// sides, matrices and solver are those of k_adi_x_w and k_adi_y_w with the
// same shape, operation for operation; the neighbouring planes z - 1 and
// z + 1 (the x sweep's z couplings) are read from global memory as there.
// grid (gz - 1 planes, chains).
template <int G, int K>
__global__ void __launch_bounds__(G * K * G, 1)
k_adi_xy_p(FilmDev<float> F, int s) {
  constexpr int N = G * K;                 // points of an x or a y line
  constexpr int LPW = 32 / G;              // lines per warp
  static_assert(N * G <= 1024 && N % LPW == 0, "one block holds every line of the plane");
  __shared__ float P[N * N];               // previous slice, plane z
  __shared__ float Wp[N * N];              // x sweep's result, then the y sweep's
  const int L = F.nlines;                  // = N * N
  const int z = 1 + blockIdx.x, dir = blockIdx.y;
  const int lane = threadIdx.x & 31, gl = lane & (G - 1);
  const int line = (threadIdx.x >> 5) * LPW + lane / G;   // y for the x sweep, x for the y sweep
  const AdiCoef cf = adi_coef(F, dir, s);
  const int ty = (F.brush || F.single) ? 0 : film_type(dir, s, F.ns, F.na);
  const float* p0 = (dir == 0 ? F.q : F.qd) + (size_t)(s - 1) * F.npts;
  float* out = F.w1 + (size_t)dir * F.npts;
  const float* wf = F.wf + (size_t)ty * F.npts;
  const size_t pz = (size_t)z * L;
  for (int i = threadIdx.x; i < N * N; i += blockDim.x) P[i] = __ldg(p0 + pz + i);
  __syncthreads();
  const int base = lane - gl;
  {  // x sweep: line y, lane points x0 .. x0 + K - 1
    const int y = line, x0 = gl * K;
    const float ax = cf.ax, bx = cf.bx, cx = ax;
    const float ay = cf.ay, cy = ay;
    const float az = __fmul_rn(-cf.dsf, F.alf[z]), cz = __fmul_rn(-cf.dsf, F.gaf[z]);
    const int ym = (y + N - 1) % N, yp = (y + 1) % N;
    const size_t row = pz + (size_t)y * N, rzm = row - L, rzp = row + L;
    float c0[K];
#pragma unroll
    for (int i = 0; i < K; ++i) c0[i] = P[y * N + x0 + i];
    const float left = __shfl_sync(0xffffffffu, c0[K - 1], base + ((gl - 1) & (G - 1)));
    const float right = __shfl_sync(0xffffffffu, c0[0], base + ((gl + 1) & (G - 1)));
    float a[K], d[K], c[K], r[K];
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const int x = x0 + i;
      const float qxm = i == 0 ? left : c0[i > 0 ? i - 1 : 0];
      const float qxp = i == K - 1 ? right : c0[i + 1 < K ? i + 1 : i];
      const float qym = P[ym * N + x], qyp = P[yp * N + x];
      const float qzm = __ldg(p0 + rzm + x), qzp = __ldg(p0 + rzp + x);
      const float dsw = cf.dsf * wf[row + x];
      const float q0 = c0[i];
      r[i] = -2.f * (ax * (qxm - q0) + cx * (qxp - q0) + ay * (qym - q0) + cy * (qyp - q0) +
                     az * (qzm - q0) + cz * (qzp - q0)) - dsw * q0;
      a[i] = ax; c[i] = cx; d[i] = 1.f + bx;
    }
    fw::solve<G, K>(a, d, c, r, true, F.err);
#pragma unroll
    for (int i = 0; i < K; ++i) Wp[y * N + x0 + i] = c0[i] + r[i];
  }
  __syncthreads();
  {  // y sweep: line x, lane points y0 .. y0 + K - 1; each lane rewrites only its own points
    const int x = line, y0 = gl * K;
    const float ay = cf.ay, by = cf.by, cy = ay;
    float e[K], ws[K];
#pragma unroll
    for (int i = 0; i < K; ++i) {
      ws[i] = Wp[(y0 + i) * N + x];
      e[i] = P[(y0 + i) * N + x] - ws[i];
    }
    const float left = __shfl_sync(0xffffffffu, e[K - 1], base + ((gl - 1) & (G - 1)));
    const float right = __shfl_sync(0xffffffffu, e[0], base + ((gl + 1) & (G - 1)));
    float a[K], d[K], c[K], r[K];
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const float em = i == 0 ? left : e[i > 0 ? i - 1 : 0];
      const float ep = i == K - 1 ? right : e[i + 1 < K ? i + 1 : i];
      r[i] = ay * (em - e[i]) + cy * (ep - e[i]);
      a[i] = ay; c[i] = cy; d[i] = 1.f + by;
    }
    fw::solve<G, K>(a, d, c, r, true, F.err);
#pragma unroll
    for (int i = 0; i < K; ++i) Wp[(y0 + i) * N + x] = ws[i] + r[i];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < N * N; i += blockDim.x) out[pz + i] = Wp[i];
}

template <int G, int K>
__global__ void __launch_bounds__(128)
k_adi_z_w(FilmDev<float> F, int s) {
  constexpr int LPW = 32 / G;
  const int gz = F.gz, L = F.nlines, n = gz + 1;
  const int lane = threadIdx.x & 31, gl = lane & (G - 1);
  const int line0 = (blockIdx.x * 4 + (threadIdx.x >> 5)) * LPW + lane / G;
  const int dir = blockIdx.y;
  const bool live = line0 < L;
  const int line = live ? line0 : 0;
  const AdiCoef cf = adi_coef(F, dir, s);
  const CnStep st{0.0, cf.dsf, cf.hdsf};
  const int ty = (F.brush || F.single) ? 0 : film_type(dir, s, F.ns, F.na);
  const float* wl = F.wf + (size_t)ty * F.npts;
  const float* p0 = (dir == 0 ? F.q : F.qd) + (size_t)(s - 1) * F.npts;
  const float* w1 = F.w1 + (size_t)dir * F.npts;
  float* qn = (dir == 0 ? F.q : F.qd) + (size_t)s * F.npts;
  const int j0 = gl * K;
  // f = q - q** (q** = 0 on the walls); q** kept for the write-back
  float f[K], wq[K];
#pragma unroll
  for (int i = 0; i < K; ++i) {
    const int j = j0 + i;
    const size_t idx = (size_t)j * L + line;
    const bool in = live && j < n;
    const bool wall = j == 0 || j == n - 1;
    wq[i] = in && !wall ? __ldg(w1 + idx) : 0.f;
    f[i] = in ? __ldg(p0 + idx) - wq[i] : 0.f;
  }
  const int base = lane - gl;
  const float fprev = __shfl_sync(0xffffffffu, f[K - 1], base + ((gl - 1) & (G - 1)));
  const float fnext = __shfl_sync(0xffffffffu, f[0], base + ((gl + 1) & (G - 1)));
  float a[K], d[K], c[K], r[K];
#pragma unroll
  for (int i = 0; i < K; ++i) {
    const int j = j0 + i;
    a[i] = 0.f; d[i] = 1.f; c[i] = 0.f; r[i] = 0.f;
    if (j > 0 && j < n - 1) {
      const float fm = i == 0 ? fprev : f[i > 0 ? i - 1 : 0];
      const float fp = i == K - 1 ? fnext : f[i + 1 < K ? i + 1 : i];
      float ai, ci, bi, hw;
      cn_row<float>(F, st, j, 0.0, live ? wl[(size_t)j * L + line] : 0.f, ai, ci, bi, hw);
      a[i] = ai; c[i] = ci;
      d[i] = 1.f + bi + hw;
      r[i] = ai * (fm - f[i]) + ci * (fp - f[i]) + hw * f[i];
    }
  }
  fw::solve<G, K>(a, d, c, r, false, F.err);
  if (live) {
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const int j = j0 + i;
      if (j < n) qn[(size_t)j * L + line] = (j > 0 && j < n - 1) ? wq[i] + r[i] : r[i];
    }
  }
}

// ---------------------------------------------------------------------------
// Shared-memory staged y and z sweeps.  The y lines (stride gx) and z lines
// (stride gx gy) run across x, so a warp that holds one line reads a
// different 32-byte sector per lane.  Here a block takes a tile of 32
// neighbouring lines (32 consecutive x of one plane for y, 32 consecutive
// (y, x) lines for z), reads every row of the tile with 32 consecutive
// floats per warp load, keeps the tile in shared memory (rows padded to 33
// floats), solves its lines there with the warp solver (G lanes, K rows per
// lane, 128 / G lines per round of the block's four warps) and writes the
// tile back the same way.  Right-hand sides, matrices and the solver are
// those of k_adi_y_w / k_adi_z_w; neighbour values come from shared memory
// instead of shuffles.  Shared memory: (Z ? 3 : 2) n 33 floats.
// ---------------------------------------------------------------------------
constexpr int kAdiTile = 32;
constexpr int kAdiPad = 33;

__host__ __device__ constexpr size_t adi_staged_smem(int n, bool z) {
  return (size_t)(z ? 3 : 2) * n * kAdiPad * sizeof(float);
}

template <int G, int K, bool Z>
__global__ void __launch_bounds__(128)
k_adi_yz_s(FilmDev<float> F, int s) {
  static_assert(G >= 4, "four warps cover 32 lines per round at G >= 4");
  extern __shared__ __align__(16) float smf[];
  constexpr int LPW = 32 / G;
  const int gx = F.gx, L = F.nlines;
  const int n = Z ? F.gz + 1 : F.gy;
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5, gl = lane & (G - 1);
  size_t base, rstride;
  int cnt;
  if (Z) {
    const int l0 = blockIdx.x * kAdiTile;
    base = (size_t)l0;
    rstride = (size_t)L;
    cnt = min(kAdiTile, L - l0);
  } else {
    const int tx = (gx + kAdiTile - 1) / kAdiTile;
    const int z = 1 + blockIdx.x / tx, x0 = (blockIdx.x % tx) * kAdiTile;
    base = (size_t)z * L + x0;
    rstride = (size_t)gx;
    cnt = min(kAdiTile, gx - x0);
  }
  const int dir = blockIdx.y;
  const AdiCoef cf = adi_coef(F, dir, s);
  const float* p0 = (dir == 0 ? F.q : F.qd) + (size_t)(s - 1) * F.npts;
  float* w1 = F.w1 + (size_t)dir * F.npts;
  const int ty = (F.brush || F.single) ? 0 : film_type(dir, s, F.ns, F.na);
  const float* wl = F.wf + (size_t)ty * F.npts;
  float* sf = smf;                       // q - q** (z) or q - q* (y); then the result
  float* sw = smf + n * kAdiPad;         // q** (z, 0 on the walls) or q*
  float* sl = smf + 2 * n * kAdiPad;     // z: field of the step's type
  for (int j = wp; j < n; j += 4) {
    float f = 0.f, wq = 0.f, wv = 0.f;
    if (lane < cnt) {
      const size_t idx = base + (size_t)j * rstride + lane;
      if (Z) {
        wq = (j == 0 || j == n - 1) ? 0.f : __ldg(w1 + idx);
        wv = __ldg(wl + idx);
      } else {
        wq = w1[idx];
      }
      f = __ldg(p0 + idx) - wq;
    }
    sf[j * kAdiPad + lane] = f;
    sw[j * kAdiPad + lane] = wq;
    if (Z) sl[j * kAdiPad + lane] = wv;
  }
  __syncthreads();
  const CnStep st{0.0, cf.dsf, cf.hdsf};
  const float ay = cf.ay, by = cf.by, cy = ay;
#pragma unroll 1
  for (int r0 = 0; r0 < kAdiTile; r0 += 4 * LPW) {
    const int tl = r0 + wp * LPW + lane / G;   // line of the tile
    const int j0 = gl * K;
    float a[K], d[K], c[K], r[K], wq[K];
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const int j = j0 + i;
      a[i] = 0.f; d[i] = 1.f; c[i] = 0.f; r[i] = 0.f; wq[i] = 0.f;
      if (j < n) {
        const float f = sf[j * kAdiPad + tl];
        wq[i] = sw[j * kAdiPad + tl];
        if (Z) {
          if (j > 0 && j < n - 1) {
            const float fm = sf[(j - 1) * kAdiPad + tl], fp = sf[(j + 1) * kAdiPad + tl];
            float ai, ci, bi, hw;
            cn_row<float>(F, st, j, 0.0, sl[j * kAdiPad + tl], ai, ci, bi, hw);
            a[i] = ai; c[i] = ci;
            d[i] = 1.f + bi + hw;
            r[i] = ai * (fm - f) + ci * (fp - f) + hw * f;
          }
        } else {
          const float em = sf[(j == 0 ? n - 1 : j - 1) * kAdiPad + tl];
          const float ep = sf[(j == n - 1 ? 0 : j + 1) * kAdiPad + tl];
          r[i] = ay * (em - f) + cy * (ep - f);
          a[i] = ay; c[i] = cy; d[i] = 1.f + by;
        }
      }
    }
    fw::solve<G, K>(a, d, c, r, !Z, F.err);
    __syncwarp();   // every lane of the line has read its rows
#pragma unroll
    for (int i = 0; i < K; ++i) {
      const int j = j0 + i;
      if (j < n) sf[j * kAdiPad + tl] = (!Z || (j > 0 && j < n - 1)) ? wq[i] + r[i] : r[i];
    }
  }
  __syncthreads();
  float* out = Z ? (dir == 0 ? F.q : F.qd) + (size_t)s * F.npts : w1;
  if (lane < cnt)
    for (int j = wp; j < n; j += 4) out[base + (size_t)j * rstride + lane] = sf[j * kAdiPad + lane];
}
