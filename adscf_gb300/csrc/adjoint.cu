// adjoint.cu -- forward/backward pair of the bulk diblock free energy (FP64).
//
// adscf_forward evaluates the free energy per chain at given fields the way
// the SCF loop reports it (Calculate_Energy, Bulk_3D_FFT/Main_Diblock_Melt/
// main_diblock.f90:295-307, densities of Propagate_Diblock, Bulk_3D_FFT/
// Polymer_Modules/mod_diblock.f90:100-173) and keeps every propagator slice;
// adscf_backward runs the reverse-mode adjoint of the discrete chain
// (adjoint_kernels.cuh) and returns dF/dL_x, dF/dL_y, dF/dL_z and dF/dchi at
// the same fields.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"
#include "adjoint_kernels.cuh"

struct AdjState {
  AdjDev A{};
  BulkDev<double>* d_inst2 = nullptr;   // [0] adjoint spectrum, [1] forward-chain spectrum
  int2* wx = nullptr; int nwx = 0;
  int2* wy2 = nullptr; int nwy2 = 0;    // both instances (forward y)
  int2* wy1 = nullptr; int nwy1 = 0;    // adjoint instance (inverse y)
  int2* wz = nullptr; int nwz = 0;
  size_t smx = 0, smy = 0, smz = 0;
  double* d_w = nullptr;
  long long gen = -1;                   // propagation generation of the last forward
};

namespace {

size_t plan_bytes(const Plan1D& P, int nbuf) {
  const size_t twn = (P.n + 1) & ~1;
  return (twn + (size_t)nbuf * P.lpc * P.ld) * sizeof(double2);
}

int mk_work(adscf_ctx* ctx, const std::vector<int2>& w, int2*& d, int& n) {
  n = (int)w.size();
  CK(cudaMalloc(&d, w.size() * sizeof(int2)));
  CK(cudaMemcpy(d, w.data(), w.size() * sizeof(int2), cudaMemcpyHostToDevice));
  return ADSCF_OK;
}

std::vector<int2> tiles(int inst, int nlines, int lpc) {
  std::vector<int2> w;
  for (int i = 0; i * lpc < nlines; ++i) w.push_back(make_int2(inst, i));
  return w;
}

int adj_setup(adscf_ctx* ctx) {
  if (ctx->adj) return ADSCF_OK;
  AdjState* s = new (std::nothrow) AdjState();
  if (!s) return set_err(ctx, ADSCF_E_OOM, "adjoint state");
  ctx->adj = s;
  const BulkDev<double>& I = ctx->hb64;
  const size_t np = (size_t)ctx->npts;
  AdjDev& A = s->A;
  A.I = I;
  A.sa = I.spec;
  if (cudaMalloc(&A.sf, np * sizeof(double2)) || cudaMalloc(&A.b, 2 * np * sizeof(double)) ||
      cudaMalloc(&s->d_w, 2 * np * sizeof(double))) {
    cudaGetLastError();
    return set_err(ctx, ADSCF_E_OOM, "adjoint buffers");
  }
  A.w = s->d_w;
  A.nqpart = ctx->contour_blocks;
  A.nclos = std::min<int>((int)((np + BULK_THREADS - 1) / BULK_THREADS), 152 * 4);
  CK(cudaMalloc(&A.part, (size_t)A.nclos * 4 * sizeof(double)));
  CK(cudaMalloc(&A.sc, ADJ_NSC * sizeof(double)));
  A.rho = ctx->p.rho; A.kappa = ctx->p.kappa; A.chi = ctx->p.chi;
  A.v0 = ctx->p.monomer_volume[0] != 0 ? ctx->p.monomer_volume[0] : 1.0;
  A.v1 = ctx->p.monomer_volume[1] != 0 ? ctx->p.monomer_volume[1] : 1.0;
  A.ds = ctx->p.ds;
  A.lx = ctx->p.sizex; A.ly = ctx->p.sizey; A.lz = ctx->p.sizez;
  int rc;
  if ((rc = mk_work(ctx, tiles(0, ctx->gy * ctx->gz, I.px.lpc), s->wx, s->nwx))) return rc;
  std::vector<int2> y2 = tiles(0, ctx->gx * ctx->gz, I.py.lpc);
  const std::vector<int2> y1 = y2;
  for (const int2& v : y1) y2.push_back(make_int2(1, v.y));
  if ((rc = mk_work(ctx, y2, s->wy2, s->nwy2))) return rc;
  if ((rc = mk_work(ctx, y1, s->wy1, s->nwy1))) return rc;
  if ((rc = mk_work(ctx, tiles(0, ctx->gx * ctx->gy, I.pz.lpc), s->wz, s->nwz))) return rc;
  A.nztiles = s->nwz;
  CK(cudaMalloc(&A.gpart, (size_t)s->nwz * 3 * sizeof(double)));
  s->smx = plan_bytes(I.px, 2);
  s->smy = plan_bytes(I.py, 2);
  s->smz = plan_bytes(I.pz, 3);
  int optin = 0;
  CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->dev));
  if (s->smx > (size_t)optin || s->smy > (size_t)optin || s->smz + 3 * 32 * sizeof(double) > (size_t)optin)
    return set_err(ctx, ADSCF_E_ARG, "grid line too long for the adjoint passes");
  CK(cudaFuncSetAttribute(k_adj_x, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->smx));
  CK(cudaFuncSetAttribute(k_adj_z, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->smz));
  // this translation unit's instance of the generic strided pass is a kernel
  // of its own (one device module per .cu file): it needs its own limit
  CK(cudaFuncSetAttribute(k_bulk_strided<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
  BulkDev<double> two[2] = {I, I};
  two[1].spec = A.sf;
  CK(cudaMalloc(&s->d_inst2, sizeof(two)));
  CK(cudaMemcpy(s->d_inst2, two, sizeof(two), cudaMemcpyHostToDevice));
  return ADSCF_OK;
}

int check_ctx(adscf_ctx* ctx) {
  if (ctx->geometry != ADSCF_BULK) return set_err(ctx, ADSCF_E_STATE, "the adjoint covers bulk contexts");
  if (ctx->prec != ADSCF_FP64) return set_err(ctx, ADSCF_E_STATE, "the adjoint needs an FP64 context");
  if (ctx->p.ensemble != 1) return set_err(ctx, ADSCF_E_STATE, "the adjoint covers the canonical ensemble");
  return ADSCF_OK;
}

int read_scalars(adscf_ctx* ctx, double* sc) {
  CK(cudaMemcpyAsync(sc, ctx->adj->A.sc, ADJ_NSC * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return ADSCF_OK;
}

}  // namespace

void adj_set_box(adscf_ctx* ctx) {
  if (!ctx->adj) return;
  ctx->adj->A.lx = ctx->p.sizex;
  ctx->adj->A.ly = ctx->p.sizey;
  ctx->adj->A.lz = ctx->p.sizez;
  ctx->adj->gen = -1;          // a forward at the old box no longer matches
}

void adj_destroy(adscf_ctx* ctx) {
  AdjState* s = ctx->adj;
  if (!s) return;
  cudaFree(s->A.sf); cudaFree(s->A.b); cudaFree(s->d_w); cudaFree(s->A.part);
  cudaFree(s->A.sc); cudaFree(s->A.gpart); cudaFree(s->d_inst2);
  cudaFree(s->wx); cudaFree(s->wy2); cudaFree(s->wy1); cudaFree(s->wz);
  delete s;
  ctx->adj = nullptr;
}

namespace {
// the forward pass from the fields already in the adjoint buffer
int forward_core(adscf_ctx* ctx, double* free_energy, double* sc_out) {
  int rc;
  AdjState* s = ctx->adj;
  if ((rc = bulk_enqueue_expfield(ctx, s->d_w))) return rc;
  if ((rc = bulk_enqueue_propagate(ctx))) return rc;
  k_adj_closure<<<s->A.nclos, BULK_THREADS, 0, ctx->stream>>>(s->A);
  k_adj_scalars<<<1, 32, 0, ctx->stream>>>(s->A);
  CK(cudaGetLastError());
  double sc[ADJ_NSC];
  if ((rc = read_scalars(ctx, sc))) return rc;
  if (!(sc[ADJ_S] > 0.0) || !std::isfinite(sc[ADJ_F]))
    return set_err(ctx, ADSCF_E_NONFINITE, "non-finite or non-positive Q in the forward pass");
  s->gen = ++ctx->prop_gen;
  if (free_energy) *free_energy = sc[ADJ_F];
  if (sc_out) std::memcpy(sc_out, sc, sizeof(sc));
  return ADSCF_OK;
}
}  // namespace

extern "C" {

int adscf_forward(adscf_ctx* ctx, const double* field, double* free_energy) {
  if (!ctx || !field) return ADSCF_E_ARG;
  int rc;
  if (ctx->geometry != ADSCF_BULK) {   // films and brushes: F and its wall-potential gradient
    double* d = film_fe_field(ctx);
    if (!d) return set_err(ctx, ADSCF_E_OOM, "film forward buffer");
    const size_t nvf = (size_t)ctx->ntypes * ctx->npts;
    CK(cudaMemcpyAsync(d, field, nvf * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    return film_forward(ctx, free_energy);
  }
  if ((rc = check_ctx(ctx)) || (rc = adj_setup(ctx))) return rc;
  const size_t nv = 2 * (size_t)ctx->npts;
  std::vector<double> tmp(field, field + nv);
  CK(cudaMemcpyAsync(ctx->adj->d_w, tmp.data(), nv * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  return forward_core(ctx, free_energy, nullptr);
}

int adscf_forward_dev(adscf_ctx* ctx, const double* d_field, double* free_energy) {
  if (!ctx || !d_field) return ADSCF_E_ARG;
  int rc;
  if ((rc = check_ctx(ctx)) || (rc = adj_setup(ctx))) return rc;
  const size_t nv = 2 * (size_t)ctx->npts;
  CK(cudaMemcpyAsync(ctx->adj->d_w, d_field, nv * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  return forward_core(ctx, free_energy, nullptr);
}

// FP64 free energy at the context's current (device-resident) SCF field.  A
// split context evaluates it on an FP64 sibling context created on first use.
int adscf_free_energy_fp64(adscf_ctx* ctx, adscf_iter_result* out) {
  if (!ctx || !out) return ADSCF_E_ARG;
  if (ctx->geometry != ADSCF_BULK || ctx->p.ensemble != 1)
    return set_err(ctx, ADSCF_E_STATE, "FP64 free energy: bulk contexts, canonical ensemble");
  adscf_ctx* c64 = ctx;
  int rc;
  if (ctx->prec != ADSCF_FP64) {
    if (!ctx->sib64) {
      adscf_params q = ctx->p;
      q.precision = ADSCF_FP64;
      if ((rc = adscf_ctx_create(&q, &ctx->sib64))) return set_err(ctx, rc, "FP64 sibling context");
    }
    c64 = ctx->sib64;
    if ((rc = adscf_set_stream(c64, ctx->stream))) return set_err(ctx, rc, c64->err);
  }
  int k = 0;
  CK(cudaMemcpyAsync(&k, ctx->d_iter, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const double* field = ctx->d_hx + (size_t)(k % ctx->hist_slots) * 2 * (size_t)ctx->npts;
  if ((rc = check_ctx(c64)) || (rc = adj_setup(c64))) return set_err(ctx, rc, c64->err);
  const size_t nv = 2 * (size_t)ctx->npts;
  CK(cudaMemcpyAsync(c64->adj->d_w, field, nv * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  double sc[ADJ_NSC];
  double F = 0.0;
  if ((rc = forward_core(c64, &F, sc))) return set_err(ctx, rc, c64->err);
  *out = adscf_iter_result{};
  out->free_energy = F;
  out->Qsum = c64->dvol * sc[ADJ_S];
  out->logQ = std::log(out->Qsum);
  out->rho = ctx->p.rho;
  out->mu = std::log(ctx->p.rho * ctx->volume / out->Qsum);
  out->iter = k;
  return ADSCF_OK;
}

int adscf_backward_surface(adscf_ctx* ctx, double* dF_dchi, double* dF_dU) {
  if (!ctx) return ADSCF_E_ARG;
  if (ctx->geometry == ADSCF_BULK) return set_err(ctx, ADSCF_E_STATE, "wall-potential gradients are for films and brushes");
  return film_backward(ctx, dF_dchi, dF_dU);
}

int adscf_backward(adscf_ctx* ctx, double* grad) {
  if (!ctx || !grad) return ADSCF_E_ARG;
  if (ctx->geometry != ADSCF_BULK)
    return set_err(ctx, ADSCF_E_STATE, "films and brushes: use adscf_backward_surface");
  int rc;
  if ((rc = check_ctx(ctx))) return rc;
  AdjState* s = ctx->adj;
  if (!s || s->gen != ctx->prop_gen)
    return set_err(ctx, ADSCF_E_STATE, "adscf_backward needs the state of an immediately preceding adscf_forward");
  const AdjDev& A = s->A;
  cudaStream_t st = ctx->stream;
  const double2* tw = static_cast<const double2*>(ctx->d_tw);
  const double* fk = static_cast<const double*>(ctx->d_fk);
  const double2* tw64 = static_cast<const double2*>(ctx->d_tw64);
  CK(cudaMemsetAsync(A.gpart, 0, (size_t)s->nwz * 3 * sizeof(double), st));
  for (int t = ctx->ns; t >= 1; --t) {
    k_adj_x<<<s->nwx, BULK_THREADS, s->smx, st>>>(A, s->wx, tw, t);
    k_bulk_strided<double><<<s->nwy2, BULK_THREADS, s->smy, st>>>(s->d_inst2, s->wy2, tw, fk, tw64,
                                                                   ctx->d_g64, t, 0);
    k_adj_z<<<s->nwz, BULK_THREADS, s->smz, st>>>(A, s->wz, tw, fk);
    if (t > 1)
      k_bulk_strided<double><<<s->nwy1, BULK_THREADS, s->smy, st>>>(s->d_inst2, s->wy1, tw, fk, tw64,
                                                                     ctx->d_g64, t, 1);
  }
  k_adj_grad<<<1, 32, 0, st>>>(A);
  CK(cudaGetLastError());
  double sc[ADJ_NSC];
  if ((rc = read_scalars(ctx, sc))) return rc;
  grad[0] = sc[ADJ_DLX];
  grad[1] = sc[ADJ_DLY];
  grad[2] = sc[ADJ_DLZ];
  grad[3] = sc[ADJ_DCHI];
  for (int i = 0; i < 4; ++i)
    if (!std::isfinite(grad[i])) return set_err(ctx, ADSCF_E_NONFINITE, "non-finite adjoint gradient");
  return ADSCF_OK;
}

}  // extern "C"
