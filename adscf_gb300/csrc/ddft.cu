// ddft.cu -- the dynamic density functional theory step of the multiblock
// driver (Bulk_3D_FFT/Main_Multiblock/main_multiblock.f90) on the device:
//   * Read_Mobilities (:441-506): mobility_qq(k) = min(|k|^2 Lambda(|k|),
//     wcutoff) per type pair, Lambda interpolated from the tabulated q grid;
//   * Get_Conjugate_Fields (:566-640): the field whose densities equal a
//     given density, by the SCF machinery with the residual phi[w] - target
//     and the accuracy max |residual| (:773-783);
//   * DDFT_Timestep_Euler (:794-880): mu = w_mean(rho) - w_conj(rho),
//     d rho / dt = -IFFT(M(k) FFT(mu)), a forward Euler step, the optional
//     floor at 1e-4, and the conjugate fields of the new density.
// The k-space product runs on the generic FFT passes: both types' mu are
// packed as one complex field z = mu_A + i mu_B, so one 3D FFT pair serves
// both, and the type mixing by the real, even M(k) is unpacked in place by
// pairing k with -k.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"
#include "bulk_host.h"

namespace {

// one thread per pair {k, -k}: Z'(k) = -s [ (Maa+Mbb)/2 Z(k) + ((Maa-Mbb)/2 + i Mab) conj(Z(-k)) ]
// (mu_A(k) = (Z(k) + conj Z(-k)) / 2 and mu_B(k) = (Z(k) - conj Z(-k)) / 2i
// for the real fields mu_A, mu_B; s = 1/N is the forward normalisation of
// Real2Fourier, mod_fourier.f90:102)
template <typename T>
__global__ void k_ddft_kspace(cplx<T>* __restrict__ z, const double* __restrict__ mob, int gx, int gy, int gz,
                              double s) {
  const size_t n = (size_t)gx * gy * gz;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % gx), y = (int)((i / gx) % gy), zz = (int)(i / ((size_t)gx * gy));
    const size_t j = ((size_t)((gz - zz) % gz) * gy + (gy - y) % gy) * gx + (gx - x) % gx;
    if (j < i) continue;   // the partner's thread handles the pair
    const double maa = mob[i], mab = mob[n + i], mbb = mob[2 * n + i];
    const double p = 0.5 * (maa + mbb), qr = 0.5 * (maa - mbb), qi = mab;
    const double ar = (double)z[i].x, ai = (double)z[i].y;
    const double br = (double)z[j].x, bi = (double)z[j].y;
    // Z'(k) from Z(k) and conj Z(-k) = (br, -bi)
    const double kr = -s * (p * ar + qr * br + qi * bi);
    const double ki = -s * (p * ai - qr * bi + qi * br);
    if (j == i) {
      z[i] = mk<T>((T)kr, (T)ki);
    } else {  // Z'(-k) from Z(-k) and conj Z(k) = (ar, -ai)
      const double jr = -s * (p * br + qr * ar + qi * ai);
      const double ji = -s * (p * bi - qr * ai + qi * ar);
      z[i] = mk<T>((T)kr, (T)ki);
      z[j] = mk<T>((T)jr, (T)ji);
    }
  }
}

template <typename T>
__global__ void k_ddft_pack(const double* __restrict__ mu, cplx<T>* __restrict__ z, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    z[i] = mk<T>((T)mu[i], (T)mu[n + i]);
}

template <typename T>
__global__ void k_ddft_unpack(const cplx<T>* __restrict__ z, double* __restrict__ out, size_t n) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    out[i] = (double)z[i].x;
    out[n + i] = (double)z[i].y;
  }
}

// mu_c = w_mean(rho)_c - w_c: Calculate_Mean_Fields (mod_FloryHuggins.f90:
// 104-129) of the density, minus the conjugate field
__global__ void k_ddft_mu(ScfDev S, const double* __restrict__ rho, const double* __restrict__ w,
                          double* __restrict__ mu) {
  const size_t n = (size_t)S.npts;
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (size_t)gridDim.x * blockDim.x) {
    const double f0 = rho[p] * S.v0, f1 = rho[n + p] * S.v1, tot = f0 + f1;
    mu[p] = (S.kappa * (tot - 1.0) + S.chi * f1) * S.v0 - w[p];
    mu[n + p] = (S.kappa * (tot - 1.0) + S.chi * f0) * S.v1 - w[n + p];
  }
}

// density = density + dt * ddensity, floored at dsmall when asked
// (main_multiblock.f90:866-872: max(density, dsmall) once the minimum is at
// or below dsmall, which is the same as always taking the maximum)
__global__ void k_ddft_euler(double* __restrict__ rho, const double* __restrict__ drho, size_t n, double dt,
                             int floor_on, double dsmall) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double v = rho[i] + dt * drho[i];
    if (floor_on) v = fmax(v, dsmall);
    rho[i] = v;
  }
}

template <typename T>
const BulkDev<T>& host_inst(const adscf_ctx* ctx) {
  if constexpr (sizeof(T) == 4) return ctx->hb32;
  else return ctx->hb64;
}

int gb(size_t n) { return (int)std::min<size_t>(std::max<size_t>(1, (n + 255) / 256), 152 * 8); }

int need_bulk(adscf_ctx* ctx) {
  if (ctx->geometry != ADSCF_BULK || ctx->ntypes != 2)
    return set_err(ctx, ADSCF_E_STATE, "DDFT: bulk contexts with two monomer types");
  return ADSCF_OK;
}

int ddft_alloc(adscf_ctx* ctx) {
  if (ctx->d_ddft) return ADSCF_OK;
  const size_t n = (size_t)ctx->npts;
  // rho [2n], drho [2n], mu [2n], z [n] complex (FP64 size covers FP32)
  if (cudaMalloc(&ctx->d_ddft, (6 * n + 2 * n) * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(ctx, ADSCF_E_OOM, "DDFT buffers");
  }
  return ADSCF_OK;
}

// generic passes of this file's FFT: work lists (instance 0) and limits
struct Passes {
  int2 *wx = nullptr, *wy = nullptr, *wz = nullptr;
  int nx = 0, ny = 0, nz = 0;
};

int mk_tiles(adscf_ctx* ctx, int nlines, int lpc, int2*& d, int& n) {
  std::vector<int2> w;
  for (int i = 0; i * lpc < nlines; ++i) w.push_back(make_int2(0, i));
  n = (int)w.size();
  CK(cudaMalloc(&d, w.size() * sizeof(int2)));
  CK(cudaMemcpy(d, w.data(), w.size() * sizeof(int2), cudaMemcpyHostToDevice));
  return ADSCF_OK;
}

// d_out = -IFFT(M(k) FFT(mu)) / N for the packed pair of types
template <typename T>
int rhs_t(adscf_ctx* ctx, const double* d_mu, double* d_out) {
  const BulkDev<T>& I = host_inst<T>(ctx);
  const size_t n = (size_t)ctx->npts;
  cudaStream_t st = ctx->stream;
  static_assert(sizeof(cplx<T>) <= 2 * sizeof(double), "complex staging");
  cplx<T>* z = reinterpret_cast<cplx<T>*>(ctx->d_ddft + 6 * n);
  int optin = 0;
  CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->dev));
  // the limit is per kernel and per translation unit: this file's instances
  CK(cudaFuncSetAttribute(k_bulk_xpass<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
  CK(cudaFuncSetAttribute(k_bulk_strided<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
  Passes P;
  int rc;
  if ((rc = mk_tiles(ctx, ctx->gy * ctx->gz, I.px.lpc, P.wx, P.nx)) ||
      (rc = mk_tiles(ctx, ctx->gx * ctx->gz, I.py.lpc, P.wy, P.ny)) ||
      (rc = mk_tiles(ctx, ctx->gx * ctx->gy, I.pz.lpc, P.wz, P.nz))) {
    cudaFree(P.wx); cudaFree(P.wy); cudaFree(P.wz);
    return rc;
  }
  const size_t smx = bulkhost::plan_smem<T>(I.px), smy = bulkhost::plan_smem<T>(I.py),
               smz = bulkhost::plan_smem<T>(I.pz);
  const BulkDev<T>* d = static_cast<const BulkDev<T>*>(ctx->d_inst);
  const cplx<T>* tw = static_cast<const cplx<T>*>(ctx->d_tw);
  const T* fk = static_cast<const T*>(ctx->d_fk);
  const double2* tw64 = static_cast<const double2*>(ctx->d_tw64);
  k_ddft_pack<T><<<gb(n), 256, 0, st>>>(d_mu, z, n);
  const XAux in{z, nullptr, nullptr}, out{nullptr, z, nullptr};
  k_bulk_xpass<T><<<P.nx, BULK_THREADS, smx, st>>>(d, P.wx, tw, 0, XM_C2S, in);
  k_bulk_strided<T><<<P.ny, BULK_THREADS, smy, st>>>(d, P.wy, tw, fk, tw64, ctx->d_g64, 0, 0);
  k_bulk_strided<T><<<P.nz, BULK_THREADS, smz, st>>>(d, P.wz, tw, fk, tw64, ctx->d_g64, 0, 3);
  k_ddft_kspace<T><<<gb(n), 256, 0, st>>>(I.spec, ctx->d_mob, ctx->gx, ctx->gy, ctx->gz, 1.0 / (double)n);
  k_bulk_strided<T><<<P.nz, BULK_THREADS, smz, st>>>(d, P.wz, tw, fk, tw64, ctx->d_g64, 0, 4);
  k_bulk_strided<T><<<P.ny, BULK_THREADS, smy, st>>>(d, P.wy, tw, fk, tw64, ctx->d_g64, 0, 1);
  k_bulk_xpass<T><<<P.nx, BULK_THREADS, smx, st>>>(d, P.wx, tw, 0, XM_S2C, out);
  k_ddft_unpack<T><<<gb(n), 256, 0, st>>>(z, d_out, n);
  cudaError_t e = cudaGetLastError();
  cudaStreamSynchronize(st);
  cudaFree(P.wx); cudaFree(P.wy); cudaFree(P.wz);
  if (e != cudaSuccess) return set_err(ctx, ADSCF_E_CUDA, cudaGetErrorString(e));
  return ADSCF_OK;
}

int rhs(adscf_ctx* ctx, const double* d_mu, double* d_out) {
  if (!ctx->d_mob) return set_err(ctx, ADSCF_E_STATE, "DDFT: no mobilities (adscf_ddft_set_mobility)");
  return ctx->prec == ADSCF_SPLIT ? rhs_t<float>(ctx, d_mu, d_out) : rhs_t<double>(ctx, d_mu, d_out);
}

int current_iter(adscf_ctx* ctx, int* k) {
  CK(cudaMemcpyAsync(k, ctx->d_iter, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return ADSCF_OK;
}

// Get_Conjugate_Fields from the context's current field; leaves the
// conjugate field as the current field and phi[field] in ctx->d_dens.
int conj_solve(adscf_ctx* ctx, const double* d_target, double tol, int itermax, int* status, int* iters) {
  const size_t nv = (size_t)ctx->ntypes * ctx->npts;
  cudaStream_t st = ctx->stream;
  int k = 1, rc;
  if ((rc = current_iter(ctx, &k))) return rc;
  // the reference restarts iter_status at 1 on every call (warm-up first)
  const int slots = ctx->hist_slots;
  double* x1 = ctx->d_hx + (size_t)(1 % slots) * nv;
  if (k % slots != 1 % slots)
    CK(cudaMemcpyAsync(x1, ctx->d_hx + (size_t)(k % slots) * nv, nv * sizeof(double), cudaMemcpyDeviceToDevice, st));
  const int one = 1;
  CK(cudaMemcpyAsync(ctx->d_iter, &one, sizeof(int), cudaMemcpyHostToDevice, st));
  if ((rc = bulk_enqueue_expfield(ctx, x1))) return rc;
  ScfDev S2 = ctx->S;
  S2.target = d_target;
  double acc = NAN;
  int it = 0;
  bool done = false;
  for (it = 1; it <= itermax; ++it) {
    if ((rc = bulk_enqueue_propagate(ctx))) return rc;
    launch_closure(S2, CL_CONJ | CL_MIXDOTS, ctx->closure_blocks, st);
    k_solve<<<1, SOLVE_THREADS, 0, st>>>(S2, 2, 1);
    CK(cudaGetLastError());
    double r[R_COUNT];
    CK(cudaMemcpyAsync(r, ctx->d_res, sizeof(r), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    acc = r[R_ACC];
    if (!(acc > tol * 0.5)) {   // main_multiblock.f90:603: converged (NaN continues)
      // keep x_k: undo the counter advance of the solve
      CK(cudaMemcpyAsync(ctx->d_iter, &it, sizeof(int), cudaMemcpyHostToDevice, st));
      done = true;
      break;
    }
    if ((rc = bulk_mix_e(ctx))) return rc;
  }
  if (iters) *iters = done ? it : itermax;
  ++ctx->prop_gen;
  if (done) {
    *status = 0;
  } else if (acc < tol) {
    *status = 1;   // "iteration slow"
  } else {
    *status = 2;
    if (!(acc < 0.1))   // the reference stops here (:624-626)
      return set_err(ctx, ADSCF_E_NONFINITE, "conjugate fields not found (accuracy " + std::to_string(acc) + ")");
  }
  CK(cudaStreamSynchronize(st));
  return ADSCF_OK;
}

}  // namespace

extern "C" {

int adscf_ddft_set_mobility(adscf_ctx* ctx, int nq, double dq, const double* table, double wcutoff) {
  if (!ctx || nq < 1 || !(dq > 0) || !table) return ADSCF_E_ARG;
  int rc;
  if ((rc = need_bulk(ctx))) return rc;
  const int gx = ctx->gx, gy = ctx->gy, gz = ctx->gz;
  const size_t n = (size_t)ctx->npts;
  std::vector<double> m(3 * n);
  for (int z = 0; z < gz; ++z)
    for (int y = 0; y < gy; ++y)
      for (int x = 0; x < gx; ++x) {
        // -laplace of Calculate_Laplace (mod_fourier.f90:165-198): |k|^2 with
        // the wrapped wave numbers
        const double kx = bulkhost::wavenum(x, gx, ctx->p.sizex), ky = bulkhost::wavenum(y, gy, ctx->p.sizey),
                     kz = bulkhost::wavenum(z, gz, ctx->p.sizez);
        const double qq = kx * kx + ky * ky + kz * kz, q = std::sqrt(qq);
        const int iq = (int)(q / dq);
        double v[3];
        for (int c = 0; c < 3; ++c) {
          // main_multiblock.f90:490-500, table rows 1-based: row iq is q = iq dq
          if (iq == 0) v[c] = table[c] * q / dq;
          else if (iq >= nq) v[c] = table[(size_t)(nq - 1) * 3 + c];
          else v[c] = (table[(size_t)(iq - 1) * 3 + c] * (q - iq * dq) + table[(size_t)iq * 3 + c] * ((iq + 1) * dq - q)) / dq;
          v[c] = std::min(qq * v[c], wcutoff);
        }
        const size_t i = ((size_t)z * gy + y) * gx + x;
        m[i] = v[0];
        m[n + i] = v[1];
        m[2 * n + i] = v[2];
      }
  if (!ctx->d_mob && cudaMalloc(&ctx->d_mob, 3 * n * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return set_err(ctx, ADSCF_E_OOM, "mobility table");
  }
  CK(cudaMemcpy(ctx->d_mob, m.data(), 3 * n * sizeof(double), cudaMemcpyHostToDevice));
  return ADSCF_OK;
}

int adscf_ddft_rhs(adscf_ctx* ctx, const double* mu, double* ddensity) {
  if (!ctx || !mu || !ddensity) return ADSCF_E_ARG;
  int rc;
  if ((rc = need_bulk(ctx)) || (rc = ddft_alloc(ctx))) return rc;
  const size_t n = (size_t)ctx->npts;
  double* d_mu = ctx->d_ddft + 4 * n;
  double* d_out = ctx->d_ddft + 2 * n;
  CK(cudaMemcpy(d_mu, mu, 2 * n * sizeof(double), cudaMemcpyHostToDevice));
  if ((rc = rhs(ctx, d_mu, d_out))) return rc;
  ++ctx->prop_gen;
  CK(cudaMemcpy(ddensity, d_out, 2 * n * sizeof(double), cudaMemcpyDeviceToHost));
  return ADSCF_OK;
}

int adscf_conjugate_fields(adscf_ctx* ctx, const double* density, double accuracy, int itermax, int* status,
                           int* iterations) {
  ADSCF_RANGE("adscf_conjugate_fields");
  if (!ctx || !density || !status || itermax < 1) return ADSCF_E_ARG;
  int rc;
  if ((rc = need_bulk(ctx)) || (rc = ddft_alloc(ctx))) return rc;
  const size_t n = (size_t)ctx->npts;
  double* d_rho = ctx->d_ddft;
  CK(cudaMemcpy(d_rho, density, 2 * n * sizeof(double), cudaMemcpyHostToDevice));
  return conj_solve(ctx, d_rho, accuracy, itermax, status, iterations);
}

int adscf_ddft_step(adscf_ctx* ctx, double* density, double timestep, int floor_density, double accuracy,
                    int itermax, int* status) {
  ADSCF_RANGE("adscf_ddft_step");
  if (!ctx || !density || !status || itermax < 1) return ADSCF_E_ARG;
  int rc;
  if ((rc = need_bulk(ctx)) || (rc = ddft_alloc(ctx))) return rc;
  if (!ctx->d_mob) return set_err(ctx, ADSCF_E_STATE, "DDFT: no mobilities (adscf_ddft_set_mobility)");
  const size_t n = (size_t)ctx->npts;
  double* d_rho = ctx->d_ddft;
  double* d_drho = ctx->d_ddft + 2 * n;
  double* d_mu = ctx->d_ddft + 4 * n;
  cudaStream_t st = ctx->stream;
  CK(cudaMemcpy(d_rho, density, 2 * n * sizeof(double), cudaMemcpyHostToDevice));
  int gcf = 0;
  // local potential of the density (main_multiblock.f90:824-826)
  if ((rc = conj_solve(ctx, d_rho, accuracy, itermax, &gcf, nullptr))) return rc;
  int k = 1;
  if ((rc = current_iter(ctx, &k))) return rc;
  const double* w = ctx->d_hx + (size_t)(k % ctx->hist_slots) * 2 * n;
  k_ddft_mu<<<gb(n), 256, 0, st>>>(ctx->S, d_rho, w, d_mu);
  CK(cudaGetLastError());
  // d rho / dt in Fourier space and back (:836-861), Euler step (:866-872)
  if ((rc = rhs(ctx, d_mu, d_drho))) return rc;
  k_ddft_euler<<<gb(2 * n), 256, 0, st>>>(d_rho, d_drho, 2 * n, timestep, floor_density, 1.0e-4);
  CK(cudaGetLastError());
  // the field of the new density (:873-877)
  if ((rc = conj_solve(ctx, d_rho, accuracy, itermax, &gcf, nullptr))) return rc;
  if (floor_density && gcf >= 1) {   // the densities of the field found
    if ((rc = current_iter(ctx, &k))) return rc;
    const double* wn = ctx->d_hx + (size_t)(k % ctx->hist_slots) * 2 * n;
    if ((rc = adscf_propagate_diblock_dev(ctx, wn, d_rho, nullptr))) return rc;
  }
  *status = gcf;
  CK(cudaMemcpy(density, d_rho, 2 * n * sizeof(double), cudaMemcpyDeviceToHost));
  return ADSCF_OK;
}

}  // extern "C"
