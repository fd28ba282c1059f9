// capi.cu -- the C ABI (include/adscf.h): context, host copies, SCF driver.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "internal.h"

int set_err(adscf_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

namespace {

// nint: round half away from zero (Fortran NINT)
int nint(double x) { return x >= 0 ? (int)std::floor(x + 0.5) : -(int)std::floor(-x + 0.5); }

}  // namespace

int grid_blocks(size_t n, int per, int cap) {
  size_t b = (n + per - 1) / per;
  if (b < 1) b = 1;
  return (int)std::min<size_t>(b, (size_t)cap);
}

int ensure_pinned(adscf_ctx* ctx, size_t bytes) {
  if (bytes <= ctx->pinned_bytes) return ADSCF_OK;
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  ctx->h_pinned = nullptr;
  ctx->pinned_bytes = 0;
  CK(cudaMallocHost(&ctx->h_pinned, bytes));
  ctx->pinned_bytes = bytes;
  return ADSCF_OK;
}

// page-locked (cudaHostAlloc / cudaHostRegister) host memory: DMA copies go
// to and from it directly, without the staging memcpy
bool host_pinned(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// host -> device through pinned staging (one cudaMemcpyAsync per copy)
int h2d(adscf_ctx* ctx, double* d, const double* h, size_t n) {
  int rc = ensure_pinned(ctx, n * sizeof(double));
  if (rc) return rc;
  std::memcpy(ctx->h_pinned, h, n * sizeof(double));
  CK(cudaMemcpyAsync(d, ctx->h_pinned, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return ADSCF_OK;
}
int d2h(adscf_ctx* ctx, double* h, const double* d, size_t n) {
  int rc = ensure_pinned(ctx, n * sizeof(double));
  if (rc) return rc;
  CK(cudaMemcpyAsync(ctx->h_pinned, d, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  std::memcpy(h, ctx->h_pinned, n * sizeof(double));
  return ADSCF_OK;
}

namespace {

size_t nvar(const adscf_ctx* c) { return (size_t)c->ntypes * c->npts; }
double* hx_slot(adscf_ctx* c, int s) { return c->d_hx + (size_t)s * nvar(c); }
double* hr_slot(adscf_ctx* c, int s) { return c->d_hr + (size_t)s * nvar(c); }

int read_result(adscf_ctx* ctx, adscf_iter_result* out, adscf_chain_result* ch) {
  double r[R_COUNT];
  CK(cudaMemcpyAsync(r, ctx->d_res, sizeof(r), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (out) {
    out->accuracy = r[R_ACC];
    out->free_energy = r[R_F];
    out->Qsum = r[R_Q];
    out->logQ = r[R_LOGQ];
    out->mu = r[R_MU];
    out->rho = r[R_RHO];
    out->lambda = r[R_LAMBDA];
    out->iter = (int)r[R_ITER];
    out->status = (int)r[R_STATUS];
  }
  if (ch) {
    ch->Qsum = r[R_Q];
    ch->logQ = r[R_LOGQ];
    ch->mu = r[R_MU];
    ch->rho = r[R_RHO];
    ch->energy = r[R_ENERGY];
  }
  if (ctx->d_flags) {  // a bounded device wait expired (TMA passes)
    int f = 0;
    CK(cudaMemcpyAsync(&f, ctx->d_flags, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (f) {
      CK(cudaMemsetAsync(ctx->d_flags, 0, sizeof(int), ctx->stream));
      return set_err(ctx, ADSCF_E_TIMEOUT, "a bounded wait for a TMA tile expired");
    }
  }
  if (r[R_STATUS] != 0.0) return set_err(ctx, ADSCF_E_NONFINITE, "non-finite or non-positive Q / accuracy");
  return ADSCF_OK;
}

// propagate from the current device field/E into dist + qpart
int enqueue_propagate(adscf_ctx* ctx, const double* d_w) {
  if (ctx->geometry == ADSCF_BULK) return bulk_enqueue_propagate(ctx);
  return film_enqueue_propagate(ctx, d_w);
}

// whole iteration: propagate(x_k) -> closure -> solve -> mix (x_{k+1}, E)
int enqueue_iteration(adscf_ctx* ctx) {
  int rc;
  // films read the field from the current history slot: the closure kernel
  // and the film sweep both locate it through the device counter
  if ((rc = enqueue_propagate(ctx, nullptr))) return rc;
  launch_closure(ctx->S, CL_MEANFIELD | CL_MIXDOTS, ctx->closure_blocks, ctx->stream);
  CK(cudaEventRecordWithFlags(ctx->ev_dens, ctx->stream, cudaEventRecordExternal));   // densities written
  k_solve<<<1, SOLVE_THREADS, 0, ctx->stream>>>(ctx->S, 1, 1);
  CK(cudaGetLastError());
  if (ctx->geometry == ADSCF_BULK) return bulk_mix_e(ctx);
  k_mix<float><<<ctx->mix_blocks, SCF_THREADS, 0, ctx->stream>>>(ctx->S, nullptr, 0.0);
  CK(cudaGetLastError());
  return ADSCF_OK;
}

int build_iteration_graph(adscf_ctx* ctx) {
  if (ctx->g_iter) return ADSCF_OK;
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_iteration(ctx);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (rc) return rc;
  if (e != cudaSuccess) return set_err(ctx, ADSCF_E_CUDA, std::string("capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&ctx->g_iter, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return set_err(ctx, ADSCF_E_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
  return ADSCF_OK;
}

int build_prop_graph(adscf_ctx* ctx) {
  if (ctx->g_prop) return ADSCF_OK;
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_propagate(ctx, ctx->d_tmp);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (rc) return rc;
  if (e != cudaSuccess) return set_err(ctx, ADSCF_E_CUDA, std::string("capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&ctx->g_prop, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return set_err(ctx, ADSCF_E_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
  return ADSCF_OK;
}

int validate(const adscf_params* p, std::string& why) {
  if (!p) { why = "null params"; return ADSCF_E_ARG; }
  if (p->geometry < ADSCF_BULK || p->geometry > ADSCF_BRUSH) { why = "geometry"; return ADSCF_E_ARG; }
  if (p->gx < 1 || p->gy < 1 || p->gz < 1) { why = "grid"; return ADSCF_E_ARG; }
  if ((long long)p->gx * p->gy * (p->gz + 1) > (1LL << 30)) { why = "grid too large"; return ADSCF_E_ARG; }
  if (p->precision != ADSCF_FP64 && p->precision != ADSCF_SPLIT) { why = "precision"; return ADSCF_E_ARG; }
  if (p->mixing_type < 1 || p->mixing_type > 3) { why = "mixing_type"; return ADSCF_E_ARG; }
  if (p->mixing_type == 3 && (p->mixing_dim < 1 || p->mixing_dim > SCF_MAX_HIST)) {
    why = "mixing_dim must be 1..16"; return ADSCF_E_ARG;
  }
  if (p->ensemble != 1 && p->ensemble != 2) { why = "ensemble"; return ADSCF_E_ARG; }
  if (!(p->sizex > 0 && p->sizey > 0 && p->sizez > 0)) { why = "box size"; return ADSCF_E_ARG; }
  if (p->geometry != ADSCF_BULK && !p->dz) { why = "films need dz"; return ADSCF_E_ARG; }
  if (p->geometry != ADSCF_BULK && p->gz < 2) { why = "films need an interior plane (gz >= 2)"; return ADSCF_E_ARG; }
  if (!p->dss && !(p->ds > 0)) { why = "ds"; return ADSCF_E_ARG; }
  if (p->nblocks) {
    if (p->geometry != ADSCF_BULK) { why = "block sequences are for bulk contexts"; return ADSCF_E_ARG; }
    if (p->dss) { why = "block sequences take the uniform step ds"; return ADSCF_E_ARG; }
    if (p->nblocks < 1 || p->nblocks > ADSCF_MAX_BLOCKS || !p->blocks || !p->block_types) {
      why = "nblocks must be 1..16 with blocks and block_types"; return ADSCF_E_ARG;
    }
    for (int k = 0; k < p->nblocks; ++k)
      if (!(p->blocks[k] >= 0) || (p->block_types[k] != 0 && p->block_types[k] != 1)) {
        why = "block lengths >= 0, block types 0 (A) or 1 (B)"; return ADSCF_E_ARG;
      }
  }
  return ADSCF_OK;
}

}  // namespace

extern "C" {

int adscf_abi_version(void) { return ADSCF_ABI_VERSION; }

const char* adscf_status_string(int s) {
  switch (s) {
    case ADSCF_OK: return "ok";
    case ADSCF_E_ARG: return "invalid argument";
    case ADSCF_E_CUDA: return "CUDA error";
    case ADSCF_E_PIVOT: return "zero tridiagonal pivot";
    case ADSCF_E_NONFINITE: return "non-finite result";
    case ADSCF_E_TIMEOUT: return "device wait timed out";
    case ADSCF_E_OOM: return "device out of memory";
    case ADSCF_E_STATE: return "invalid state";
    case ADSCF_E_TOO_LARGE: return "problem larger than the fixed scratch of the allocation-free entry point";
    default: return "unknown status";
  }
}

const char* adscf_last_error(const adscf_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

long long adscf_field_points(const adscf_ctx* ctx) { return ctx ? (long long)ctx->npts : -1; }

int adscf_contour_info(const adscf_ctx* ctx, int* ns, int* n_a) {
  if (!ctx) return ADSCF_E_ARG;
  if (ns) *ns = ctx->ns;
  if (n_a) *n_a = ctx->na;
  return ADSCF_OK;
}

int adscf_ctx_create(const adscf_params* p, adscf_ctx** out) {
  ADSCF_RANGE("adscf_ctx_create");
  if (!out) return ADSCF_E_ARG;
  *out = nullptr;
  std::string why;
  int rc = validate(p, why);
  if (rc) return rc;
  adscf_ctx* ctx = new (std::nothrow) adscf_ctx();
  if (!ctx) return ADSCF_E_OOM;
  ctx->p = *p;
  ctx->p.dss = nullptr; ctx->p.dz = nullptr; ctx->p.ext_potential = nullptr; ctx->p.graft = nullptr;
  ctx->p.blocks = nullptr; ctx->p.block_types = nullptr;
  if (p->nblocks) {   // own copies, so that ctx->p can create sibling contexts
    ctx->blk_len.assign(p->blocks, p->blocks + p->nblocks);
    ctx->blk_type.assign(p->block_types, p->block_types + p->nblocks);
    ctx->p.blocks = ctx->blk_len.data();
    ctx->p.block_types = ctx->blk_type.data();
  }
  ctx->geometry = p->geometry;
  ctx->prec = p->precision;
  // kernel-variant switches for A/B checks (results are identical in exact
  // arithmetic): the generic mixed-radix FFT, and the non-persistent passes
  ctx->use_generic = std::getenv("ADSCF_GENERIC_FFT") != nullptr;
  ctx->no_persistent = std::getenv("ADSCF_NO_PERSISTENT") != nullptr;
  ctx->no_tma = std::getenv("ADSCF_NO_TMA") != nullptr;
  {
    const char* at = std::getenv("ADSCF_AUTOTUNE");
    ctx->autotune = !(at && at[0] == '0');
  }
  ctx->gx = p->gx; ctx->gy = p->gy; ctx->gz = p->gz;
  ctx->nplanes = p->geometry == ADSCF_BULK ? p->gz : p->gz + 1;
  ctx->npts = p->gx * p->gy * ctx->nplanes;
  ctx->ntypes = p->geometry == ADSCF_BRUSH ? 1 : 2;
  // contour discretisation (Initialize_Diblock, mod_diblock.f90:74-75)
  if (p->nblocks) {
    // Initialize_Multiblock (mod_multiblock.f90:80-81): nint(length / ds) per block
    ctx->nblk = p->nblocks;
    int s0 = 0;
    for (int k = 0; k < p->nblocks; ++k) {
      s0 += nint(p->blocks[k] / p->ds);
      ctx->bend[k] = s0;
      if (p->block_types[k]) ctx->btype |= 1u << k;
    }
    ctx->ns = s0;
    ctx->na = (ctx->btype & 1u) ? 0 : ctx->bend[0];   // first block's A steps (diagnostics)
  } else if (p->dss) {
    ctx->ns = p->ns;
    ctx->na = p->geometry == ADSCF_BRUSH ? p->ns : p->n_a;
  } else {
    const int sa = nint(p->block_length[0] / p->ds);
    const int sb = p->geometry == ADSCF_BRUSH ? 0 : nint(p->block_length[1] / p->ds);
    ctx->ns = sa + sb;
    ctx->na = sa;
  }
  ctx->nb = ctx->ns - ctx->na;
  if (ctx->ns < 1 || ctx->na < 0 || ctx->nb < 0) { delete ctx; return ADSCF_E_ARG; }
  ctx->volume = p->sizex * p->sizey * p->sizez;
  ctx->dvol = ctx->volume / ((double)p->gx * p->gy * p->gz);

  auto fail = [&](int code) { adscf_ctx_destroy(ctx); return code; };
  if (cudaGetDevice(&ctx->dev) != cudaSuccess) { delete ctx; return ADSCF_E_CUDA; }
  if (cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete ctx;
    return ADSCF_E_CUDA;
  }
  ctx->stream = ctx->own_stream;
  if (cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_dens, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_copy, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    return fail(ADSCF_E_CUDA);
  }
  const size_t nv = nvar(ctx);
  ctx->hist_slots = p->mixing_type == 3 ? p->mixing_dim + 1 : 2;
  if (cudaMalloc(&ctx->d_dist, nv * sizeof(double)) ||
      cudaMalloc(&ctx->d_dens, nv * sizeof(double)) ||
      cudaMalloc(&ctx->d_tmp, std::max<size_t>(2 * nv, 2 * (size_t)ctx->npts) * sizeof(double)) ||
      cudaMalloc(&ctx->d_hx, ctx->hist_slots * nv * sizeof(double)) ||
      cudaMalloc(&ctx->d_hr, ctx->hist_slots * nv * sizeof(double)) ||
      (p->mixing_type == 3 && cudaMalloc(&ctx->d_hy, ctx->hist_slots * nv * sizeof(double))) ||
      cudaMalloc(&ctx->d_gram, SCF_MAX_SLOTS * SCF_MAX_SLOTS * sizeof(double)) ||
      cudaMalloc(&ctx->d_coef, 2 * SCF_MAX_SLOTS * sizeof(double)) ||
      cudaMalloc(&ctx->d_res, R_COUNT * sizeof(double)) ||
      cudaMalloc(&ctx->d_iter, sizeof(int))) {
    cudaGetLastError();
    ctx->err = "device allocation failed";
    return fail(ADSCF_E_OOM);
  }
  cudaMemsetAsync(ctx->d_dens, 0, nv * sizeof(double), ctx->stream);
  cudaMemsetAsync(ctx->d_hx, 0, ctx->hist_slots * nv * sizeof(double), ctx->stream);
  cudaMemsetAsync(ctx->d_hr, 0, ctx->hist_slots * nv * sizeof(double), ctx->stream);
  cudaMemsetAsync(ctx->d_gram, 0, SCF_MAX_SLOTS * SCF_MAX_SLOTS * sizeof(double), ctx->stream);
  cudaMemsetAsync(ctx->d_res, 0, R_COUNT * sizeof(double), ctx->stream);
  const int one = 1;
  cudaMemcpyAsync(ctx->d_iter, &one, sizeof(int), cudaMemcpyHostToDevice, ctx->stream);
  ctx->closure_blocks = grid_blocks(ctx->npts, SCF_THREADS, 152 * 4);
  ctx->mix_blocks = grid_blocks(nv, SCF_THREADS, 152 * 8);
  if (cudaMalloc(&ctx->d_part, (size_t)std::max(ctx->closure_blocks, 152 * 4) * NPART * sizeof(double))) {
    cudaGetLastError();
    return fail(ADSCF_E_OOM);
  }

  if (ctx->geometry == ADSCF_BULK) {
    rc = bulk_create(ctx);
  } else {
    // per-plane integration weights and wall potential (films / brush)
    rc = film_create(ctx, p);
  }
  if (rc) return fail(rc);

  ScfDev& S = ctx->S;
  S.npts = ctx->npts;
  S.ntypes = ctx->ntypes;
  S.plane = ctx->gx * ctx->gy;
  S.nplanes = ctx->nplanes;
  S.wall_mask = ctx->geometry != ADSCF_BULK;
  S.dvol = ctx->dvol;
  S.wz = ctx->d_wz;
  S.ext = ctx->d_ext;
  S.kappa = p->kappa; S.chi = p->chi;
  S.v0 = p->monomer_volume[0] != 0 ? p->monomer_volume[0] : 1.0;
  S.v1 = p->monomer_volume[1] != 0 ? p->monomer_volume[1] : 1.0;
  S.ww = p->ww;
  S.homopolymer = ctx->geometry == ADSCF_BRUSH;
  S.ensemble = p->ensemble;
  S.rho = p->rho; S.mu = p->mu; S.volume = ctx->volume;
  if (ctx->geometry == ADSCF_BULK) S.chain_len = p->ds * ctx->ns;
  S.dist = ctx->d_dist;
  S.dens = ctx->d_dens;
  S.hx = ctx->d_hx; S.hr = ctx->d_hr; S.hy = ctx->d_hy;
  S.slots = ctx->hist_slots;
  S.mixing_type = p->mixing_type;
  S.warm = p->warm_iters > p->mixing_dim ? p->warm_iters : p->mixing_dim;
  S.lambda = p->lambda;
  S.lam_warm = p->lam_warm > 0 ? p->lam_warm : 1.0e-3;
  S.qpart = ctx->d_qpart;
  S.nqpart = ctx->contour_blocks;
  S.qscale = ctx->geometry == ADSCF_BULK ? ctx->dvol : 1.0;
  S.part = ctx->d_part;
  S.npart_blocks = ctx->closure_blocks;
  S.gram = ctx->d_gram;
  S.coef = ctx->d_coef;
  S.iter = ctx->d_iter;
  S.res = ctx->d_res;
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return fail(ADSCF_E_CUDA);
  *out = ctx;
  return ADSCF_OK;
}

int adscf_ctx_destroy(adscf_ctx* ctx) {
  if (!ctx) return ADSCF_OK;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->g_iter) cudaGraphExecDestroy(ctx->g_iter);
  if (ctx->g_prop) cudaGraphExecDestroy(ctx->g_prop);
  adj_destroy(ctx);
  if (ctx->sib64) adscf_ctx_destroy(ctx->sib64);
  if (ctx->geometry == ADSCF_BULK) bulk_destroy(ctx);
  else film_destroy(ctx);
  cudaFree(ctx->d_dist); cudaFree(ctx->d_dens); cudaFree(ctx->d_tmp);
  cudaFree(ctx->d_hx); cudaFree(ctx->d_hr); cudaFree(ctx->d_hy); cudaFree(ctx->d_gram);
  cudaFree(ctx->d_coef); cudaFree(ctx->d_res); cudaFree(ctx->d_iter);
  cudaFree(ctx->d_part); cudaFree(ctx->d_wz); cudaFree(ctx->d_ext);
  cudaFree(ctx->d_mob); cudaFree(ctx->d_ddft);
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  if (ctx->ev_dens) cudaEventDestroy(ctx->ev_dens);
  if (ctx->ev_copy) cudaEventDestroy(ctx->ev_copy);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
  return ADSCF_OK;
}

// ---- propagator ----------------------------------------------------------
int adscf_propagate_diblock_dev(adscf_ctx* ctx, const double* d_field, double* d_density,
                                adscf_chain_result* out) {
  ADSCF_RANGE("adscf_propagate_diblock_dev");
  if (!ctx || !d_field || !d_density) return ADSCF_E_ARG;
  ++ctx->prop_gen;
  if (ctx->geometry == ADSCF_BRUSH) return set_err(ctx, ADSCF_E_STATE, "brush context: use adscf_propagate_homopolymer");
  int rc;
  if (ctx->geometry == ADSCF_BULK) {
    if ((rc = bulk_enqueue_expfield(ctx, d_field))) return rc;
    if ((rc = bulk_enqueue_propagate(ctx))) return rc;
  } else {
    if ((rc = film_enqueue_propagate(ctx, d_field))) return rc;
    if ((rc = film_check_pivot(ctx))) return rc;
  }
  ScfDev S2 = ctx->S;
  S2.dens = d_density;
  // the closure's accuracy term compares with what the output holds: start
  // from zero, so the status reflects this call's Q and densities only
  CK(cudaMemsetAsync(d_density, 0, nvar(ctx) * sizeof(double), ctx->stream));
  launch_closure(S2, 0, ctx->closure_blocks, ctx->stream);
  k_solve<<<1, SOLVE_THREADS, 0, ctx->stream>>>(S2, 1, 0);
  CK(cudaGetLastError());
  return read_result(ctx, nullptr, out);
}

int adscf_propagate_diblock(adscf_ctx* ctx, const double* field, double* density,
                            adscf_chain_result* out) {
  ADSCF_RANGE("adscf_propagate_diblock");
  if (!ctx || !field || !density) return ADSCF_E_ARG;
  const size_t nv = nvar(ctx);
  double* d_w = ctx->d_tmp;
  double* d_out = ctx->d_tmp + nv;
  int rc = h2d(ctx, d_w, field, nv);
  if (rc) return rc;
  rc = adscf_propagate_diblock_dev(ctx, d_w, d_out, out);
  if (rc) return rc;
  return d2h(ctx, density, d_out, nv);
}

int adscf_propagate_homopolymer(adscf_ctx* ctx, const double* field, double* density,
                                adscf_chain_result* out) {
  ADSCF_RANGE("adscf_propagate_homopolymer");
  if (!ctx || !field || !density) return ADSCF_E_ARG;
  ++ctx->prop_gen;
  if (ctx->geometry != ADSCF_BRUSH) return set_err(ctx, ADSCF_E_STATE, "not a brush context");
  const size_t nv = nvar(ctx);
  double* d_w = ctx->d_tmp;
  double* d_out = ctx->d_tmp + nv;
  int rc = h2d(ctx, d_w, field, nv);
  if (rc) return rc;
  if ((rc = film_enqueue_propagate(ctx, d_w))) return rc;
  if ((rc = film_check_pivot(ctx))) return rc;
  ScfDev S2 = ctx->S;
  S2.dens = d_out;
  CK(cudaMemsetAsync(d_out, 0, nv * sizeof(double), ctx->stream));   // see adscf_propagate_diblock_dev
  launch_closure(S2, 0, ctx->closure_blocks, ctx->stream);
  k_solve<<<1, SOLVE_THREADS, 0, ctx->stream>>>(S2, 1, 0);
  CK(cudaGetLastError());
  if ((rc = read_result(ctx, nullptr, out))) return rc;
  return d2h(ctx, density, d_out, nv);
}

int adscf_propagate_step(adscf_ctx* ctx, double* prop, const double* aux, double ds) {
  ADSCF_RANGE("adscf_propagate_step");
  if (!ctx || !prop || !aux) return ADSCF_E_ARG;
  ++ctx->prop_gen;
  const size_t n = ctx->npts;
  double* d_p = ctx->d_tmp;
  double* d_a = ctx->d_tmp + n;
  int rc;
  if ((rc = h2d(ctx, d_p, prop, n))) return rc;
  if ((rc = h2d(ctx, d_a, aux, n))) return rc;
  if (ctx->geometry == ADSCF_BULK) rc = bulk_step_single(ctx, d_p, d_a);
  else if (!(rc = film_step_single(ctx, d_p, d_a, ds > 0 ? ds : ctx->p.ds))) rc = film_check_pivot(ctx);
  if (rc) return rc;
  return d2h(ctx, prop, d_p, n);
}

int adscf_real2fourier(adscf_ctx* ctx, const double* prop, double* spectrum) {
  ADSCF_RANGE("adscf_real2fourier");
  if (!ctx || !prop || !spectrum) return ADSCF_E_ARG;
  ++ctx->prop_gen;
  if (ctx->geometry != ADSCF_BULK) return set_err(ctx, ADSCF_E_STATE, "bulk only");
  // the spectrum staging uses d_tmp (2*npts doubles); stage the input in d_dist
  int rc = h2d(ctx, ctx->d_dist, prop, ctx->npts);
  if (rc) return rc;
  return bulk_r2c(ctx, ctx->d_dist, spectrum);
}

int adscf_fourier2real(adscf_ctx* ctx, const double* spectrum, double* prop) {
  ADSCF_RANGE("adscf_fourier2real");
  if (!ctx || !prop || !spectrum) return ADSCF_E_ARG;
  ++ctx->prop_gen;
  if (ctx->geometry != ADSCF_BULK) return set_err(ctx, ADSCF_E_STATE, "bulk only");
  int rc = bulk_c2r(ctx, spectrum, ctx->d_dist);
  if (rc) return rc;
  return d2h(ctx, prop, ctx->d_dist, ctx->npts);
}

// ---- interactions -------------------------------------------------------
int adscf_mean_fields(adscf_ctx* ctx, const double* density, double* field) {
  ADSCF_RANGE("adscf_mean_fields");
  if (!ctx || !density || !field) return ADSCF_E_ARG;
  const size_t nv = nvar(ctx);
  int rc = h2d(ctx, ctx->d_tmp, density, nv);
  if (rc) return rc;
  k_meanfield_only<<<grid_blocks(ctx->npts, 256, 152 * 8), 256, 0, ctx->stream>>>(ctx->S, ctx->d_tmp, ctx->d_tmp + nv);
  CK(cudaGetLastError());
  return d2h(ctx, field, ctx->d_tmp + nv, nv);
}

int adscf_interaction_energy(adscf_ctx* ctx, const double* density, double* energy) {
  if (!ctx || !density || !energy) return ADSCF_E_ARG;
  // closure with dist := density and scale 1: use a zero field slot so only
  // the interaction partials matter
  const size_t nv = nvar(ctx);
  int rc = h2d(ctx, ctx->d_tmp, density, nv);
  if (rc) return rc;
  ScfDev S2 = ctx->S;
  S2.dist = ctx->d_tmp;
  S2.dens = ctx->d_tmp + nv;
  S2.ensemble = 2;
  S2.mu = 0.0;  // scale = exp(0) = 1
  S2.hx = ctx->d_tmp + nv;  // x_k irrelevant for the interaction sum
  S2.hr = ctx->d_tmp + nv;
  S2.slots = 1;
  S2.mixing_type = 1;
  // the closure reads *iter to locate slots; slot 0 of S2 is d_tmp+nv
  launch_closure(S2, CL_MEANFIELD | CL_KEEP_OLD, ctx->closure_blocks, ctx->stream);
  k_solve<<<1, SOLVE_THREADS, 0, ctx->stream>>>(S2, 1, 0);
  CK(cudaGetLastError());
  double r[R_COUNT];
  CK(cudaMemcpyAsync(r, ctx->d_res, sizeof(r), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  *energy = r[R_EINT];
  return ADSCF_OK;
}

int adscf_integrator(adscf_ctx* ctx, const double* integrand, double* integral) {
  if (!ctx || !integrand || !integral) return ADSCF_E_ARG;
  std::vector<double> wz(ctx->nplanes, ctx->dvol);
  if (ctx->d_wz) CK(cudaMemcpy(wz.data(), ctx->d_wz, ctx->nplanes * sizeof(double), cudaMemcpyDeviceToHost));
  const int plane = ctx->gx * ctx->gy;
  double s = 0.0;
  for (int z = 0; z < ctx->nplanes; ++z) {
    double t = 0.0;
    for (int i = 0; i < plane; ++i) t += integrand[(size_t)z * plane + i];
    s += wz[z] * t;
  }
  *integral = s;
  return ADSCF_OK;
}

// ---- mixing ---------------------------------------------------------------
int adscf_mix_dev(adscf_ctx* ctx, double* d_field, const double* d_dfield, int iter) {
  ADSCF_RANGE("adscf_mix_dev");
  if (!ctx || !d_field || !d_dfield || iter < 1) return ADSCF_E_ARG;
  const size_t nv = nvar(ctx);
  const int cur = iter % ctx->hist_slots;
  CK(cudaMemcpyAsync(hx_slot(ctx, cur), d_field, nv * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  CK(cudaMemcpyAsync(hr_slot(ctx, cur), d_dfield, nv * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  CK(cudaMemcpyAsync(ctx->d_iter, &iter, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  ScfDev S2 = ctx->S;
  S2.wall_mask = 0;  // the caller packs what is mixed (Mix_Fields)
  k_mixdots<<<ctx->closure_blocks, SCF_THREADS, 0, ctx->stream>>>(S2);
  k_solve<<<1, SOLVE_THREADS, 0, ctx->stream>>>(S2, 0, 1);
  k_mix<float><<<ctx->mix_blocks, SCF_THREADS, 0, ctx->stream>>>(S2, nullptr, 0.0);
  CK(cudaGetLastError());
  const int nxt = (iter + 1) % ctx->hist_slots;
  CK(cudaMemcpyAsync(d_field, hx_slot(ctx, nxt), nv * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return ADSCF_OK;
}

int adscf_mix(adscf_ctx* ctx, double* field, const double* dfield, int iter) {
  ADSCF_RANGE("adscf_mix");
  if (!ctx || !field || !dfield) return ADSCF_E_ARG;
  const size_t nv = nvar(ctx);
  int rc;
  if ((rc = h2d(ctx, ctx->d_tmp, field, nv))) return rc;
  if ((rc = h2d(ctx, ctx->d_tmp + nv, dfield, nv))) return rc;
  if ((rc = adscf_mix_dev(ctx, ctx->d_tmp, ctx->d_tmp + nv, iter))) return rc;
  return d2h(ctx, field, ctx->d_tmp, nv);
}

int adscf_mix_reset(adscf_ctx* ctx) {
  if (!ctx) return ADSCF_E_ARG;
  const size_t nv = nvar(ctx);
  CK(cudaMemsetAsync(ctx->d_hx, 0, ctx->hist_slots * nv * sizeof(double), ctx->stream));
  CK(cudaMemsetAsync(ctx->d_hr, 0, ctx->hist_slots * nv * sizeof(double), ctx->stream));
  CK(cudaMemsetAsync(ctx->d_gram, 0, SCF_MAX_SLOTS * SCF_MAX_SLOTS * sizeof(double), ctx->stream));
  const int one = 1;
  CK(cudaMemcpyAsync(ctx->d_iter, &one, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return ADSCF_OK;
}

// ---- device SCF loop --------------------------------------------------------
int adscf_set_field(adscf_ctx* ctx, const double* field) {
  if (!ctx || !field) return ADSCF_E_ARG;
  int rc = adscf_mix_reset(ctx);
  if (rc) return rc;
  double* x1 = hx_slot(ctx, 1 % ctx->hist_slots);
  if ((rc = h2d(ctx, x1, field, nvar(ctx)))) return rc;
  if (ctx->geometry == ADSCF_BULK) {
    if ((rc = bulk_enqueue_expfield(ctx, x1))) return rc;
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return ADSCF_OK;
}

int adscf_set_density(adscf_ctx* ctx, const double* density) {
  if (!ctx || !density) return ADSCF_E_ARG;
  return h2d(ctx, ctx->d_dens, density, nvar(ctx));
}

int adscf_get_field(adscf_ctx* ctx, double* field) {
  if (!ctx || !field) return ADSCF_E_ARG;
  int k = 1;
  CK(cudaMemcpyAsync(&k, ctx->d_iter, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  return d2h(ctx, field, hx_slot(ctx, k % ctx->hist_slots), nvar(ctx));
}

int adscf_get_density(adscf_ctx* ctx, double* density) {
  if (!ctx || !density) return ADSCF_E_ARG;
  return d2h(ctx, density, ctx->d_dens, nvar(ctx));
}

int adscf_scf_run(adscf_ctx* ctx, int n_iter, double tol, adscf_iter_result* out) {
  ADSCF_RANGE("adscf_scf_run");
  if (!ctx || n_iter < 0) return ADSCF_E_ARG;
  ++ctx->prop_gen;
  int rc = build_iteration_graph(ctx);
  if (rc) return rc;
  for (int i = 0; i < n_iter; ++i) {
    CK(cudaGraphLaunch(ctx->g_iter, ctx->stream));
    if (tol >= 0.0) {
      adscf_iter_result r{};
      if ((rc = read_result(ctx, &r, nullptr))) return rc;
      if (out) *out = r;
      if (!(r.accuracy > tol)) return ADSCF_OK;  // NaN-safe as the reference
    }
  }
  adscf_iter_result r{};
  rc = read_result(ctx, &r, nullptr);  // synchronises the stream
  if (out) *out = r;
  if (!rc && ctx->film) rc = film_check_pivot(ctx);
  return rc;
}

int adscf_scf_iteration(adscf_ctx* ctx, double* field, double* density, adscf_iter_result* out) {
  ADSCF_RANGE("adscf_scf_iteration");
  if (!ctx || !field || !density) return ADSCF_E_ARG;
  ++ctx->prop_gen;
  int rc = build_iteration_graph(ctx);
  if (rc) return rc;
  int k = 1;
  CK(cudaMemcpyAsync(&k, ctx->d_iter, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  const size_t nv = nvar(ctx);
  double* xk = hx_slot(ctx, k % ctx->hist_slots);
  // page-locked caller buffers are copied directly; others through staging
  const bool pin = host_pinned(field) && host_pinned(density);
  if (!pin) {
    if ((rc = ensure_pinned(ctx, 2 * nv * sizeof(double)))) return rc;
    std::memcpy(ctx->h_pinned, field, nv * sizeof(double));
  }
  double* hf = pin ? field : ctx->h_pinned;
  double* hd = pin ? density : ctx->h_pinned + nv;
  CK(cudaMemcpyAsync(xk, hf, nv * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  if (ctx->geometry == ADSCF_BULK && (rc = bulk_enqueue_expfield(ctx, xk))) return rc;
  CK(cudaGraphLaunch(ctx->g_iter, ctx->stream));
  // densities to the host as soon as the closure has written them (the
  // graph's event), beside the solve and the mix; the field after the mix
  CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_dens, 0));
  CK(cudaMemcpyAsync(hd, ctx->d_dens, nv * sizeof(double), cudaMemcpyDeviceToHost, ctx->copy_stream));
  CK(cudaEventRecord(ctx->ev_copy, ctx->copy_stream));
  double* xn = hx_slot(ctx, (k + 1) % ctx->hist_slots);
  CK(cudaMemcpyAsync(hf, xn, nv * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_copy, 0));
  adscf_iter_result r{};
  rc = read_result(ctx, &r, nullptr);  // synchronises the stream
  if (!pin) {
    std::memcpy(field, ctx->h_pinned, nv * sizeof(double));
    std::memcpy(density, ctx->h_pinned + nv, nv * sizeof(double));
  }
  if (out) *out = r;
  return rc;
}

int adscf_set_stream(adscf_ctx* ctx, void* stream) {
  if (!ctx) return ADSCF_E_ARG;
  CK(cudaStreamSynchronize(ctx->stream));
  ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
  return ADSCF_OK;
}

int adscf_set_wait_limit(adscf_ctx* ctx, int polls) {
  if (!ctx) return ADSCF_E_ARG;
  if (ctx->geometry != ADSCF_BULK) return set_err(ctx, ADSCF_E_STATE, "bulk contexts only");
  return bulk_set_wait_polls(ctx, polls < 0 ? (1 << 22) : polls);
}

int adscf_set_box(adscf_ctx* ctx, double sizex, double sizey, double sizez) {
  ADSCF_RANGE("adscf_set_box");
  if (!ctx || !(sizex > 0 && sizey > 0 && sizez > 0)) return ADSCF_E_ARG;
  if (ctx->geometry != ADSCF_BULK) return set_err(ctx, ADSCF_E_STATE, "box updates are for bulk contexts");
  ++ctx->prop_gen;
  ctx->p.sizex = sizex; ctx->p.sizey = sizey; ctx->p.sizez = sizez;
  ctx->volume = sizex * sizey * sizez;
  ctx->dvol = ctx->volume / ((double)ctx->gx * ctx->gy * ctx->gz);
  ctx->S.volume = ctx->volume;
  ctx->S.dvol = ctx->dvol;
  ctx->S.qscale = ctx->dvol;
  int rc = bulk_set_box(ctx);
  if (rc) return rc;
  adj_set_box(ctx);
  // graphs hold the closure parameters by value: capture again on next use
  if (ctx->g_iter) { cudaGraphExecDestroy(ctx->g_iter); ctx->g_iter = nullptr; }
  if (ctx->g_prop) { cudaGraphExecDestroy(ctx->g_prop); ctx->g_prop = nullptr; }
  if (ctx->sib64) { adscf_ctx_destroy(ctx->sib64); ctx->sib64 = nullptr; }
  return ADSCF_OK;
}

int adscf_tuning(const adscf_ctx* ctx, char* buf, int len) {
  if (!ctx || !buf || len < 1) return ADSCF_E_ARG;
  char plan[96];
  std::snprintf(plan, sizeof(plan), "plan y=%d z=%d x=%d; ", ctx->plan_y, ctx->plan_z, ctx->plan_x);
  const std::string s = std::string(plan) + (ctx->tune_report.empty() ? "not tuned" : ctx->tune_report);
  std::snprintf(buf, (size_t)len, "%s", s.c_str());
  return ADSCF_OK;
}

int adscf_set_adi_plan(adscf_ctx* ctx, int x_lanes, int y_lanes, int z_lanes, int staged) {
  if (!ctx) return ADSCF_E_ARG;
  const int lanes[3] = {x_lanes, y_lanes, z_lanes};
  const int rc = ctx->film ? film_set_adi_plan(ctx, lanes, staged) : ADSCF_E_STATE;
  if (rc == ADSCF_E_STATE) return set_err(ctx, rc, "ADI plans are for Film_3D contexts with FP32 sweeps");
  if (rc) return set_err(ctx, rc, "no warp-solver shape with that many lanes for these lines");
  if (ctx->g_iter) { cudaGraphExecDestroy(ctx->g_iter); ctx->g_iter = nullptr; }
  if (ctx->g_prop) { cudaGraphExecDestroy(ctx->g_prop); ctx->g_prop = nullptr; }
  return ADSCF_OK;
}

int adscf_set_pass_plan(adscf_ctx* ctx, int y, int z, int x) {
  if (!ctx) return ADSCF_E_ARG;
  if (ctx->geometry != ADSCF_BULK) return set_err(ctx, ADSCF_E_STATE, "pass plans are for bulk contexts");
  auto ok_yz = [&](int k) {
    return k == ADSCF_PASS_PLAIN || (k == ADSCF_PASS_PERSISTENT && ctx->pgrid_y) || (k == ADSCF_PASS_TMA && ctx->tma);
  };
  const bool ok_x = x == ADSCF_PASS_PLAIN || (x == ADSCF_PASS_PERSISTENT && ctx->pgrid_x) ||
                    (x == ADSCF_PASS_FUSED && ctx->tma && ctx->xy_grid);
  if (!ok_yz(y) || !ok_yz(z) || !ok_x) return set_err(ctx, ADSCF_E_ARG, "pass kernel not available for this shape");
  ctx->plan_y = y; ctx->plan_z = z; ctx->plan_x = x;
  if (ctx->g_iter) { cudaGraphExecDestroy(ctx->g_iter); ctx->g_iter = nullptr; }
  if (ctx->g_prop) { cudaGraphExecDestroy(ctx->g_prop); ctx->g_prop = nullptr; }
  return ADSCF_OK;
}

int adscf_stage_launches(const adscf_ctx* ctx, int stage) {
  if (!ctx) return -1;
  int prop, contour = 1, update = 3;
  if (ctx->geometry == ADSCF_BULK) prop = 1 + (ctx->plan_x == PK_FUSED ? 2 : 4) * ctx->ns;
  else prop = ctx->film_launches;
  if (ctx->geometry != ADSCF_BULK) contour = ctx->film_contour_launches;
  switch (stage) {
    case ADSCF_STAGE_ITERATION: return prop + contour + update;
    case ADSCF_STAGE_PROPAGATE: return prop;
    case ADSCF_STAGE_CONTOUR: return contour;
    case ADSCF_STAGE_UPDATE: return update;
    default: return -1;
  }
}

int adscf_enqueue(adscf_ctx* ctx, int stage, int repeats) {
  ADSCF_RANGE("adscf_enqueue");
  if (!ctx || repeats < 0) return ADSCF_E_ARG;
  ++ctx->prop_gen;
  int rc;
  if (stage == ADSCF_STAGE_ITERATION) {
    if ((rc = build_iteration_graph(ctx))) return rc;
    for (int i = 0; i < repeats; ++i) CK(cudaGraphLaunch(ctx->g_iter, ctx->stream));
    return ADSCF_OK;
  }
  for (int i = 0; i < repeats; ++i) {
    if (stage == ADSCF_STAGE_PROPAGATE) {
      if (ctx->geometry == ADSCF_BULK) rc = bulk_enqueue_chains(ctx);
      else rc = film_enqueue_chains(ctx, nullptr);
    } else if (stage == ADSCF_STAGE_CONTOUR) {
      if (ctx->geometry == ADSCF_BULK) rc = bulk_enqueue_contour(ctx);
      else rc = film_enqueue_contour(ctx);
    } else if (stage == ADSCF_STAGE_UPDATE) {
      launch_closure(ctx->S, CL_MEANFIELD | CL_MIXDOTS, ctx->closure_blocks, ctx->stream);
      k_solve<<<1, SOLVE_THREADS, 0, ctx->stream>>>(ctx->S, 1, 1);
      CK(cudaGetLastError());
      rc = ctx->geometry == ADSCF_BULK ? bulk_mix_e(ctx)
           : (k_mix<float><<<ctx->mix_blocks, SCF_THREADS, 0, ctx->stream>>>(ctx->S, nullptr, 0.0),
              cudaGetLastError() == cudaSuccess ? ADSCF_OK : ADSCF_E_CUDA);
    } else {
      return set_err(ctx, ADSCF_E_ARG, "unknown stage");
    }
    if (rc) return rc;
  }
  return ADSCF_OK;
}

}  // extern "C"
