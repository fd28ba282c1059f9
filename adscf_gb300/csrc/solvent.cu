// solvent.cu -- Update_Solvent (Bulk_3D_FFT/Polymer_Modules/mod_solvent.f90:
// 85-110): the Boltzmann distribution of a monomeric solvent in its field,
// its single-particle partition function and density in either ensemble.
#include <cmath>

#include "internal.h"

namespace {

constexpr int kSolventThreads = 256;

// distribution = exp(-field) in place of the field copy; one partial sum per
// block (fixed order within the block)
__global__ void __launch_bounds__(kSolventThreads)
k_solvent_dist(double* __restrict__ w, size_t n, double* __restrict__ part) {
  __shared__ double red[kSolventThreads / 32];
  double acc = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double d = exp(-w[i]);
    w[i] = d;
    acc += d;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < kSolventThreads / 32; ++k) s += red[k];
    part[blockIdx.x] = s;
  }
}

// density = scale * distribution; grand canonical runs also sum the density
__global__ void __launch_bounds__(kSolventThreads)
k_solvent_density(const double* __restrict__ dist, double* __restrict__ dens, size_t n, double scale,
                  double* __restrict__ part) {
  __shared__ double red[kSolventThreads / 32];
  double acc = 0.0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double d = scale * dist[i];
    dens[i] = d;
    acc += d;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < kSolventThreads / 32; ++k) s += red[k];
    part[blockIdx.x] = s;
  }
}

// sum of the blocks' partials on the host, in block order
int sum_parts(adscf_ctx* ctx, int nb, double* out) {
  std::vector<double> h(nb);
  CK(cudaMemcpyAsync(h.data(), ctx->d_part, nb * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  double s = 0.0;
  for (double v : h) s += v;
  *out = s;
  return ADSCF_OK;
}

}  // namespace

extern "C" int adscf_update_solvent(adscf_ctx* ctx, const double* field, int ensemble, double* rho, double* mu,
                                    double* Qsum, double* energy, double* density, double* distribution) {
  ADSCF_RANGE("adscf_update_solvent");
  if (!ctx || !field || !rho || !mu || !density) return ADSCF_E_ARG;
  if (ensemble != 1 && ensemble != 2) return set_err(ctx, ADSCF_E_ARG, "Invalid ensemble; Cannot calculate Density");
  if (ctx->geometry != ADSCF_BULK) return set_err(ctx, ADSCF_E_STATE, "the solvent is a bulk routine");
  const size_t n = (size_t)ctx->npts;
  double* d_dist = ctx->d_tmp;        // field, then distribution
  double* d_dens = ctx->d_tmp + n;
  int rc = h2d(ctx, d_dist, field, n);
  if (rc) return rc;
  const int nb = grid_blocks(n, kSolventThreads, 152 * 4);   // d_part holds >= 152 * 4 values
  k_solvent_dist<<<nb, kSolventThreads, 0, ctx->stream>>>(d_dist, n, ctx->d_part);
  CK(cudaGetLastError());
  double sum = 0.0;
  if ((rc = sum_parts(ctx, nb, &sum))) return rc;
  const double Q = ctx->dvol * sum;
  const double V = ctx->volume;
  if (!(Q > 0.0) || !std::isfinite(Q)) return set_err(ctx, ADSCF_E_NONFINITE, "solvent partition function");
  const double scale = ensemble == 1 ? *rho * V / Q : std::exp(*mu);
  k_solvent_density<<<nb, kSolventThreads, 0, ctx->stream>>>(d_dist, d_dens, n, scale, ctx->d_part);
  CK(cudaGetLastError());
  double dsum = 0.0;
  if ((rc = sum_parts(ctx, nb, &dsum))) return rc;
  if (ensemble == 1) {
    *mu = std::log(*rho * V / Q);
    if (energy) *energy = *rho * V * (*mu - 1.0);
  } else {
    *rho = dsum * ctx->dvol / V;
    if (energy) *energy = -*rho * V;
  }
  if (Qsum) *Qsum = Q;
  if (distribution && (rc = d2h(ctx, distribution, d_dist, n))) return rc;
  return d2h(ctx, density, d_dens, n);
}
