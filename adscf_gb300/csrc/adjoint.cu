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
  // checkpointing (K > 0): node states every K steps and two recomputed
  // segments replace the full slice storage
  int K = 0, nseg = 0;
  double2* ck = nullptr;                // [nseg+1][npts] states at nodes 0, K, 2K, ..., Ns
  double2* bufA = nullptr;              // [K+1][npts]
  double2* bufB = nullptr;              // [2K+1][npts]
  double2* seg_spec = nullptr;          // spectrum of the segment runs
  BulkDev<double>* d_seg = nullptr;
  size_t smz2 = 0;                      // generic z pass (two line buffers)
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
  A.slA = A.slB = I.slices;
  A.tA0 = A.tB0 = 0;
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
  s->smz2 = plan_bytes(I.pz, 2);
  int optin = 0;
  CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->dev));
  if (s->smx > (size_t)optin || s->smy > (size_t)optin || s->smz + 3 * 32 * sizeof(double) > (size_t)optin)
    return set_err(ctx, ADSCF_E_ARG, "grid line too long for the adjoint passes");
  CK(cudaFuncSetAttribute(k_adj_x, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->smx));
  CK(cudaFuncSetAttribute(k_adj_z, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->smz));
  // this translation unit's instance of the generic strided pass is a kernel
  // of its own (one device module per .cu file): it needs its own limit
  CK(cudaFuncSetAttribute(k_bulk_strided<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
  CK(cudaFuncSetAttribute(k_bulk_xpass<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
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
  cudaFree(s->ck); cudaFree(s->bufA); cudaFree(s->bufB); cudaFree(s->seg_spec); cudaFree(s->d_seg);
  cudaFree(s->A.sf); cudaFree(s->A.b); cudaFree(s->d_w); cudaFree(s->A.part);
  cudaFree(s->A.sc); cudaFree(s->A.gpart); cudaFree(s->d_inst2);
  cudaFree(s->wx); cudaFree(s->wy2); cudaFree(s->wy1); cudaFree(s->wz);
  delete s;
  ctx->adj = nullptr;
}

namespace {

int ckpt_alloc(adscf_ctx* ctx, AdjState* s) {
  const int K = ctx->adj_ckpt < 0 ? (int)std::ceil(std::sqrt((double)ctx->ns)) : ctx->adj_ckpt;
  if (K == s->K && s->ck) return ADSCF_OK;
  cudaFree(s->ck); cudaFree(s->bufA); cudaFree(s->bufB); cudaFree(s->seg_spec);
  s->ck = s->bufA = s->bufB = s->seg_spec = nullptr;
  s->K = std::max(1, std::min(K, ctx->ns));
  s->nseg = (ctx->ns + s->K - 1) / s->K;
  const size_t sl = (size_t)ctx->npts * sizeof(double2);
  // nodes kK (k = 0..nseg), then the mirror nodes Ns - (k+1)K + 1 (k = 0..nseg-2)
  if (cudaMalloc(&s->ck, (size_t)(2 * s->nseg) * sl) || cudaMalloc(&s->bufA, (size_t)(s->K + 1) * sl) ||
      cudaMalloc(&s->bufB, (size_t)(s->K + 1) * sl) || cudaMalloc(&s->seg_spec, sl)) {
    cudaGetLastError();
    return set_err(ctx, ADSCF_E_OOM, "adjoint checkpoint buffers");
  }
  if (!s->d_seg) CK(cudaMalloc(&s->d_seg, sizeof(BulkDev<double>)));
  return ADSCF_OK;
}

// Recompute nodes t0..t1 of both chains from the stored state of node t0
// into buf (node t at buf + (t - t0) npts), on the generic passes and a
// spectrum of its own.
int run_segment(adscf_ctx* ctx, AdjState* s, const double2* state, int t0, int t1, double2* buf) {
  BulkDev<double> I = ctx->hb64;
  I.spec = s->seg_spec;
  I.slices = buf - (ptrdiff_t)t0 * ctx->npts;   // the kernels index slices by node
  cudaStream_t st = ctx->stream;
  CK(cudaMemcpyAsync(s->d_seg, &I, sizeof(I), cudaMemcpyHostToDevice, st));
  const double2* tw = static_cast<const double2*>(ctx->d_tw);
  const double* fk = static_cast<const double*>(ctx->d_fk);
  const double2* tw64 = static_cast<const double2*>(ctx->d_tw64);
  const XAux from{state, nullptr, nullptr}, none{nullptr, nullptr, nullptr};
  k_bulk_xpass<double><<<s->nwx, BULK_THREADS, s->smx, st>>>(s->d_seg, s->wx, tw, t0, XM_FROM, from);
  for (int t = t0 + 1; t <= t1; ++t) {
    k_bulk_strided<double><<<s->nwy1, BULK_THREADS, s->smy, st>>>(s->d_seg, s->wy1, tw, fk, tw64, ctx->d_g64, t, 0);
    k_bulk_strided<double><<<s->nwz, BULK_THREADS, s->smz2, st>>>(s->d_seg, s->wz, tw, fk, tw64, ctx->d_g64, t, 2);
    k_bulk_strided<double><<<s->nwy1, BULK_THREADS, s->smy, st>>>(s->d_seg, s->wy1, tw, fk, tw64, ctx->d_g64, t, 1);
    k_bulk_xpass<double><<<s->nwx, BULK_THREADS, s->smx, st>>>(s->d_seg, s->wx, tw, t, XM_STEP, none);
  }
  CK(cudaGetLastError());
  return ADSCF_OK;
}

// Checkpointed forward.  A first pass over the contour keeps the states of
// nodes kK and of the mirror nodes Ns - (k+1)K + 1.  The contour integral
// then takes the segments s in [kK, (k+1)K - 1] (the last one up to Ns) one
// at a time: q_s is recomputed from node kK and q-dagger_{Ns-s} from the
// mirror node (from node 0 for the last segment), K + 1 nodes each.
int propagate_ckpt(adscf_ctx* ctx, AdjState* s) {
  int rc;
  if ((rc = ckpt_alloc(ctx, s))) return rc;
  const size_t np = (size_t)ctx->npts;
  const int K = s->K, Ns = ctx->ns, ns = s->nseg;
  double2* mirror = s->ck + (size_t)(ns + 1) * np;
  cudaStream_t st = ctx->stream;
  k_fill_ones<<<(int)std::min<size_t>((np + 255) / 256, 152 * 8), 256, 0, st>>>(s->ck, np);
  for (int k = 0; k < ns; ++k) {
    const int t0 = k * K, t1 = std::min(t0 + K, Ns);
    if ((rc = run_segment(ctx, s, s->ck + (size_t)k * np, t0, t1, s->bufA))) return rc;
    CK(cudaMemcpyAsync(s->ck + (size_t)(k + 1) * np, s->bufA + (size_t)(t1 - t0) * np, np * sizeof(double2),
                       cudaMemcpyDeviceToDevice, st));
    for (int j = 0; j + 1 < ns; ++j) {
      const int m = Ns - (j + 1) * K + 1;
      if (m > t0 && m <= t1)
        CK(cudaMemcpyAsync(mirror + (size_t)j * np, s->bufA + (size_t)(m - t0) * np, np * sizeof(double2),
                           cudaMemcpyDeviceToDevice, st));
    }
  }
  CK(cudaMemsetAsync(ctx->d_dist, 0, 2 * np * sizeof(double), st));
  for (int k = 0; k < ns; ++k) {
    const bool last = k == ns - 1;
    const int s_lo = k * K, s_hi = last ? Ns : (k + 1) * K - 1;
    if ((rc = run_segment(ctx, s, s->ck + (size_t)k * np, s_lo, std::min(s_lo + K, Ns), s->bufA))) return rc;
    const int u_lo = Ns - s_hi, u_hi = Ns - s_lo;
    if ((rc = run_segment(ctx, s, last ? s->ck : mirror + (size_t)k * np, u_lo, u_hi, s->bufB))) return rc;
    k_contour_segment<<<ctx->contour_blocks, BULK_THREADS, 0, st>>>(ctx->hb64, s->bufA, s_lo, s->bufB, u_lo,
                                                                     s_lo, s_hi);
  }
  CK(cudaGetLastError());
  return ADSCF_OK;
}

// the forward pass from the fields already in the adjoint buffer
int forward_core(adscf_ctx* ctx, double* free_energy, double* sc_out) {
  int rc;
  AdjState* s = ctx->adj;
  if ((rc = bulk_enqueue_expfield(ctx, s->d_w))) return rc;
  if (ctx->adj_ckpt) {
    if ((rc = propagate_ckpt(ctx, s))) return rc;
  } else {
    if ((rc = bulk_enqueue_propagate(ctx))) return rc;
  }
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
  ADSCF_RANGE("adscf_forward");
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
  ADSCF_RANGE("adscf_forward_dev");
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
  ADSCF_RANGE("adscf_free_energy_fp64");
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

int adscf_set_adjoint_checkpoint(adscf_ctx* ctx, int every) {
  if (!ctx) return ADSCF_E_ARG;
  int rc;
  if ((rc = check_ctx(ctx)) || (rc = adj_setup(ctx))) return rc;
  // checkpointed passes never read the context's slices: release them
  if ((rc = bulk_hold_slices(ctx, every == 0))) return rc;
  AdjState* s = ctx->adj;
  s->A.I.slices = ctx->hb64.slices;
  s->A.slA = s->A.slB = ctx->hb64.slices;
  BulkDev<double> two[2] = {s->A.I, s->A.I};
  two[1].spec = s->A.sf;
  CK(cudaMemcpy(s->d_inst2, two, sizeof(two), cudaMemcpyHostToDevice));
  ctx->adj_ckpt = every;
  ++ctx->prop_gen;   // a forward made under the other mode no longer matches
  return ADSCF_OK;
}

int adscf_backward_surface(adscf_ctx* ctx, double* dF_dchi, double* dF_dU) {
  ADSCF_RANGE("adscf_backward_surface");
  if (!ctx) return ADSCF_E_ARG;
  if (ctx->geometry == ADSCF_BULK) return set_err(ctx, ADSCF_E_STATE, "wall-potential gradients are for films and brushes");
  return film_backward(ctx, dF_dchi, dF_dU);
}

int adscf_backward(adscf_ctx* ctx, double* grad) {
  ADSCF_RANGE("adscf_backward");
  if (!ctx || !grad) return ADSCF_E_ARG;
  if (ctx->geometry != ADSCF_BULK)
    return set_err(ctx, ADSCF_E_STATE, "films and brushes: use adscf_backward_surface");
  int rc;
  if ((rc = check_ctx(ctx))) return rc;
  AdjState* s = ctx->adj;
  if (!s || s->gen != ctx->prop_gen)
    return set_err(ctx, ADSCF_E_STATE, "adscf_backward needs the state of an immediately preceding adscf_forward");
  AdjDev A = s->A;
  cudaStream_t st = ctx->stream;
  const double2* tw = static_cast<const double2*>(ctx->d_tw);
  const double* fk = static_cast<const double*>(ctx->d_fk);
  const double2* tw64 = static_cast<const double2*>(ctx->d_tw64);
  CK(cudaMemsetAsync(A.gpart, 0, (size_t)s->nwz * 3 * sizeof(double), st));
  const int K = ctx->adj_ckpt ? s->K : 0;   // the mode of the forward (a mode change voids it)
  const size_t np = (size_t)ctx->npts;
  int ka_cur = -1, kb_cur = -1;
  for (int t = ctx->ns; t >= 1; --t) {
    if (K) {   // checkpointed: the segments holding node t-1 and node Ns-t
      const int ka = (t - 1) / K, kb = (ctx->ns - t) / K;
      if (ka != ka_cur) {
        if ((rc = run_segment(ctx, s, s->ck + (size_t)ka * np, ka * K, std::min(ka * K + K, ctx->ns), s->bufA)))
          return rc;
        ka_cur = ka;
      }
      if (kb != kb_cur) {
        if ((rc = run_segment(ctx, s, s->ck + (size_t)kb * np, kb * K, std::min(kb * K + K, ctx->ns), s->bufB)))
          return rc;
        kb_cur = kb;
      }
      A.slA = s->bufA; A.tA0 = ka * K;
      A.slB = s->bufB; A.tB0 = kb * K;
    }
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
