// film.cu -- film (Film_1D, Film_3D) and brush contexts: meshes, contour
// schedules, weights and launch sequences.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "film_host.h"
#include "film_kernels.cuh"
#include "film_warp.cuh"
#include "internal.h"

struct FilmState {
  bool t64 = true;              // FP64 sweeps (FP64 context, or split with a graded mesh)
  FilmDev<double> f64{};
  FilmDev<float> f32{};
  double* d_alpha = nullptr;
  double* d_beta = nullptr;
  double* d_gamma = nullptr;
  double* d_dss = nullptr;
  double* d_wA = nullptr;
  double* d_wB = nullptr;
  double* d_graft = nullptr;
  float* d_adicf = nullptr;     // FP32 ADI coefficients per schedule entry [ns+3][6]
  float* d_alf = nullptr;       // FP32 mesh factors and field of FP32 line sweeps
  float* d_wf = nullptr;
  void* d_q = nullptr;
  void* d_qd = nullptr;
  void* d_gam = nullptr;
  void* d_w1 = nullptr;
  int* d_err = nullptr;
  double max_ratio = 1.0;       // largest neighbour spacing ratio of the mesh
  int optin = 0;                // opt-in shared memory per block
  // free energy at fixed fields and its wall-potential gradient
  double* d_fe_w = nullptr;     // [ntypes][npts] field copy
  double* d_fe_part = nullptr;  // [nplanes][FE_N]
  double* d_fe_out = nullptr;   // [2 + ntypes*nplanes]
  long long fe_gen = -1;
  // FP32 ADI sweeps x, y, z: warp-solver shape of each (g = 0: one thread
  // per line), from the autotuner or the defaults
  AdiShape adi[3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  bool adi_fuse = false;        // x and y sweeps as one plane kernel (shape adi[0])
  bool adi_set = false;
};

// warp-cooperative FP32 ADI sweeps (film_adi.cu); dim 0: x, 1: y, 2: z
std::vector<AdiShape> adi_shapes(int dim, const FilmDev<float>& D);
AdiShape adi_default_shape(int dim, const FilmDev<float>& D);
void adi_warp_sweep(int dim, AdiShape sh, const FilmDev<float>& D, int step, int chains, cudaStream_t s);
bool adi_fused_ok(AdiShape x, AdiShape y, const FilmDev<float>& D);
void adi_fused_sweep(AdiShape sh, const FilmDev<float>& D, int step, int chains, cudaStream_t s);

namespace {

int nint_f(double x) { return x >= 0 ? (int)std::floor(x + 0.5) : -(int)std::floor(-x + 0.5); }

// FP32 ADI coefficients of step sizes ds[0..n): ax, bx, ay, by, ds, ds/2 per
// step, in the FP64 expressions of the per-thread sweeps
void adi_coef_rows(const double* ds, int n, double dx, double dy, float* out) {
  for (int k = 0; k < n; ++k) {
    const double h = ds[k];
    float* c = out + 6 * k;
    c[0] = (float)(-h / dx / dx / 2.0);
    c[1] = (float)(h / dx / dx);
    c[2] = (float)(-h / dy / dy / 2.0);
    c[3] = (float)(h / dy / dy);
    c[4] = (float)h;
    c[5] = (float)(0.5 * h);
  }
}

template <typename T>
FilmDev<T>& fdev(FilmState* F);
template <>
FilmDev<double>& fdev<double>(FilmState* F) { return F->f64; }
template <>
FilmDev<float>& fdev<float>(FilmState* F) { return F->f32; }

FieldRef make_ref(adscf_ctx* ctx, const double* d_w) {
  FieldRef r;
  r.direct = d_w;
  r.hx = ctx->d_hx;
  r.iter = ctx->d_iter;
  r.slots = ctx->hist_slots;
  r.nv = (size_t)ctx->ntypes * ctx->npts;
  return r;
}

// grids, lanes per block and shared memory of the three ADI sweeps: lines of
// gx, gy and gz + 1 points per lane.  Each lane runs a serial recurrence, so
// FILM_THREADS lanes are halved until the blocks cover every SM twice (152
// SMs) and a block's lines fit in shared memory.
struct AdiLaunch {
  dim3 gx, gy, gz;
  int wx, wy, wz;
  size_t sx, sy, sz;
  AdiShape sh[3];   // FP32 warp-solver shapes (g = 0: the kernels above)
  bool fuse = false;  // FP32: x and y sweeps in one plane kernel of shape sh[0]
};
template <typename T>
AdiLaunch adi_launch(const FilmState* F, const FilmDev<T>& D, int chains) {
  AdiLaunch A;
  auto lanes = [&](int n, size_t per, int nl) {
    int W = FILM_THREADS;
    while (W > 1 && (per * n * W * sizeof(T) > (size_t)F->optin || (size_t)((nl + W - 1) / W) * chains < 2 * 152))
      W >>= 1;
    return W;
  };
  A.wx = lanes(D.gx, 3, D.gy * (D.gz - 1));
  A.wy = lanes(D.gy, 4, D.gx * (D.gz - 1));
  A.wz = lanes(D.gz + 1, 2, D.nlines);
  A.sx = adi_smem(D.gx, A.wx, sizeof(T));
  A.sy = adi_smem_y(D.gy, A.wy, sizeof(T));
  A.sz = 2 * (size_t)(D.gz + 1) * A.wz * sizeof(T);
  A.gx = dim3((D.gy * (D.gz - 1) + A.wx - 1) / A.wx, chains);
  A.gy = dim3((D.gx * (D.gz - 1) + A.wy - 1) / A.wy, chains);
  A.gz = dim3((D.nlines + A.wz - 1) / A.wz, chains);
  for (int d = 0; d < 3; ++d) A.sh[d] = sizeof(T) == 4 ? F->adi[d] : AdiShape{0, 0, 0};
  A.fuse = sizeof(T) == 4 && F->adi_fuse;
  return A;
}

// One sweep of a Douglas ADI step: the FP32 warp solver with the sweep's
// shape, or the one-thread-per-line kernel.
template <typename T>
void adi_sweep(int dim, const AdiLaunch& A, const FilmDev<T>& D, const FieldRef& fr, int st, int chains,
               cudaStream_t s) {
  if constexpr (sizeof(T) == 4) {
    if (A.sh[dim].g) {
      adi_warp_sweep(dim, A.sh[dim], D, st, chains, s);
      return;
    }
  }
  if (dim == 0) k_adi_x<T><<<A.gx, A.wx, A.sx, s>>>(D, fr, st);
  else if (dim == 1) k_adi_y<T><<<A.gy, A.wy, A.sy, s>>>(D, st);
  else k_adi_z<T><<<A.gz, A.wz, A.sz, s>>>(D, fr, st);
}

// One Douglas ADI step (three sweeps) of `chains` chains.
template <typename T>
void adi_step(const AdiLaunch& A, const FilmDev<T>& D, const FieldRef& fr, int st, int chains, cudaStream_t s) {
  if constexpr (sizeof(T) == 4) {
    if (A.fuse) {
      adi_fused_sweep(A.sh[0], D, st, chains, s);
      adi_sweep<T>(2, A, D, fr, st, chains, s);
      return;
    }
  }
  for (int d = 0; d < 3; ++d) adi_sweep<T>(d, A, D, fr, st, chains, s);
}

// Autotuner of the FP32 ADI sweeps, run once at context creation (outside
// any stream capture): every warp-solver shape of each sweep and the
// one-thread-per-line kernel are timed on this context's buffers (node 0
// filled, a zero field) at step 1 with both chains: a CUDA graph of sixteen
// back-to-back sweeps, launched once to warm up and then timed five times
// with CUDA events on the context stream (the minimum counts); each sweep
// keeps its fastest.  The x sweep runs first and
// the z sweep last, so every candidate reads finite values written by the
// sweep before it.  Shapes are cached per (device, grid).  Shapes differ in
// the order of the FP32 line-solve arithmetic (results agree to rounding);
// ADSCF_AUTOTUNE=0 keeps the default shapes.
struct AdiTuneKey {
  int dev, gx, gy, gz;
  bool operator<(const AdiTuneKey& o) const {
    return std::tie(dev, gx, gy, gz) < std::tie(o.dev, o.gx, o.gy, o.gz);
  }
};
struct AdiTuneVal {
  AdiShape sh[3];
  bool fuse = false;
  std::string report;
};
std::mutex g_adi_mu;
std::map<AdiTuneKey, AdiTuneVal> g_adi_tune;

void adi_defaults(FilmState* F, const FilmDev<float>& D) {
  for (int d = 0; d < 3; ++d) F->adi[d] = adi_default_shape(d, D);
  F->adi_fuse = false;
  F->adi_set = true;
}

int adi_tune(adscf_ctx* ctx, FilmState* F, const FilmDev<float>& D, const FieldRef& fr) {
  const AdiTuneKey key{ctx->dev, D.gx, D.gy, D.gz};
  {
    std::lock_guard<std::mutex> lk(g_adi_mu);
    auto it = g_adi_tune.find(key);
    if (it != g_adi_tune.end()) {
      for (int d = 0; d < 3; ++d) F->adi[d] = it->second.sh[d];
      F->adi_fuse = it->second.fuse;
      F->adi_set = true;
      ctx->film_launches = 1 + (F->adi_fuse ? 2 : 3) * ctx->ns;
      ctx->tune_report = it->second.report + " (cached)";
      return ADSCF_OK;
    }
  }
  cudaStream_t s = ctx->stream;
  AdiLaunch A = adi_launch<float>(F, D, 2);
  EventPair ev;
  CK(ev.create());
  cudaEvent_t e0 = ev.a, e1 = ev.b;
  std::string rep = "adi";
  static const char* nm[3] = {"x", "y", "z"};
  AdiTuneVal val;
  // each candidate as a graph of sixteen back-to-back sweeps, as the
  // iteration graph runs them (stream launches of ~5 us kernels would time
  // the host's launch rate); the best of five timed launches, in us per sweep
  constexpr int kReps = 16;
  auto time_graph = [&](auto&& sweep, float* us) -> int {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int r = 0; r < kReps; ++r) sweep();
    CK(cudaStreamEndCapture(s, &g));
    const cudaError_t ie = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    CK(ie);
    for (int round = 0; round < 5; ++round) {
      cudaGraphLaunch(ge, s);
      cudaEventRecord(e0, s);
      cudaGraphLaunch(ge, s);
      cudaEventRecord(e1, s);
      const cudaError_t se = cudaEventSynchronize(e1);
      if (se != cudaSuccess) {
        cudaGraphExecDestroy(ge);
        CK(se);
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      *us = std::min(*us, 1000.f * ms / kReps);
    }
    cudaGraphExecDestroy(ge);
    return ADSCF_OK;
  };
  float best_us[3] = {0.f, 0.f, 0.f};
  for (int d = 0; d < 3; ++d) {
    std::vector<AdiShape> cand = adi_shapes(d, D);
    cand.push_back({0, 0, 0});
    std::vector<float> us(cand.size(), 1e30f);
    for (size_t c = 0; c < cand.size(); ++c) {
      A.sh[d] = cand[c];
      const int rc = time_graph([&] { adi_sweep<float>(d, A, D, fr, 1, 2, s); }, &us[c]);
      if (rc) return rc;
    }
    size_t best = 0;
    for (size_t c = 1; c < cand.size(); ++c)
      if (us[c] < us[best]) best = c;
    val.sh[d] = cand[best];
    best_us[d] = us[best];
    A.sh[d] = cand[best];   // the next sweep's candidates read this one's output
    char line[96];
    std::snprintf(line, sizeof(line), " %s=%dx%d%s", nm[d], cand[best].g, cand[best].k, cand[best].staged ? "s" : "");
    rep += line;
    for (size_t c = 0; c < cand.size(); ++c) {
      std::snprintf(line, sizeof(line), " [%s %dx%d%s %.2f us]", nm[d], cand[c].g, cand[c].k,
                    cand[c].staged ? "s" : "", us[c]);
      rep += line;
    }
    rep += ";";
    // after the y sweep: the x + y plane kernel with the x sweep's shape,
    // where both sweeps chose it, against the two sweeps' times
    if (d == 1 && adi_fused_ok(val.sh[0], val.sh[1], D)) {
      float fus = 1e30f;
      const int rc = time_graph([&] { adi_fused_sweep(val.sh[0], D, 1, 2, s); }, &fus);
      if (rc) return rc;
      val.fuse = fus < best_us[0] + best_us[1];
      std::snprintf(line, sizeof(line), " xy=%s [xy %dx%d %.2f us against %.2f us];", val.fuse ? "fused" : "apart",
                    val.sh[0].g, val.sh[0].k, fus, best_us[0] + best_us[1]);
      rep += line;
    }
  }
  CK(cudaGetLastError());
  for (int d = 0; d < 3; ++d) F->adi[d] = val.sh[d];
  F->adi_fuse = val.fuse;
  F->adi_set = true;
  ctx->film_launches = 1 + (F->adi_fuse ? 2 : 3) * ctx->ns;
  val.report = rep;
  ctx->tune_report = rep;
  std::lock_guard<std::mutex> lk(g_adi_mu);
  g_adi_tune[key] = val;
  return ADSCF_OK;
}

// 1D chains of every line: FP32 sweeps on lines of up to 32 * kFilmWarpM
// planes with one warp per (line, chain) (film_warp.cuh); FP64 sweeps (the
// reference's serial Thomas) and longer lines with one thread per (line,
// chain).
template <typename T>
void launch_chains_1d(const FilmDev<T>& D, const FieldRef& fr, int chains, cudaStream_t s) {
  if constexpr (sizeof(T) == 4) {
    if (D.gz + 1 <= 32 * kFilmWarpM) {
      k_film1d_warp<<<dim3((D.nlines + 3) / 4, chains), 128, 0, s>>>(D);
      return;
    }
  }
  const dim3 g((D.nlines + FILM_THREADS - 1) / FILM_THREADS, chains);
  k_film1d_chains<T><<<g, FILM_THREADS, 0, s>>>(D, fr);
}

template <typename T>
int chains_t(adscf_ctx* ctx, const double* d_w) {
  FilmState* F = ctx->film;
  FilmDev<T> D = fdev<T>(F);
  const FieldRef fr = make_ref(ctx, d_w);
  cudaStream_t s = ctx->stream;
  if (ctx->geometry == ADSCF_FILM_3D) {
    // node 0 of both chains = 1, then ns Douglas ADI steps (three sweeps each)
    k_film_fill<T><<<std::max(1, (D.npts + 255) / 256), 256, 0, s>>>(D.q, D.qd, D.npts);
    if (sizeof(T) == 4) {
      const size_t n = (size_t)ctx->ntypes * D.npts;
      k_film_wconv<<<(int)std::min<size_t>((n + 255) / 256, 152 * 4), 256, 0, s>>>(fr, D.wf, n);
    }
    if constexpr (sizeof(T) == 4) {
      if (!F->adi_set) adi_defaults(F, D);
    }
    const AdiLaunch A = adi_launch<T>(F, D, 2);
    for (int st = 1; st <= D.ns; ++st) adi_step<T>(A, D, fr, st, 2, s);
  } else {
    if (sizeof(T) == 4) {
      const size_t n = (size_t)ctx->ntypes * D.npts;
      k_film_wconv<<<(int)std::min<size_t>((n + 255) / 256, 152 * 4), 256, 0, s>>>(fr, D.wf, n);
    }
    launch_chains_1d<T>(D, fr, 2, s);
  }
  CK(cudaGetLastError());
  return ADSCF_OK;
}

template <typename T>
int contour_t(adscf_ctx* ctx) {
  FilmDev<T> D = fdev<T>(ctx->film);
  k_film_contour<T><<<ctx->contour_blocks, 256, 0, ctx->stream>>>(D);
  CK(cudaGetLastError());
  return ADSCF_OK;
}

// one step of one propagator: slice 0 <- prop, step with field w and ds,
// prop <- slice 1
template <typename T>
int step_single_t(adscf_ctx* ctx, double* d_prop, const double* d_w, double ds) {
  FilmState* F = ctx->film;
  FilmDev<T> D = fdev<T>(F);
  cudaStream_t s = ctx->stream;
  double h_dss[2] = {0.0, ds};
  // a one-step schedule in the 2 spare entries past the contour schedule
  CK(cudaMemcpyAsync(F->d_dss + D.ns + 1, h_dss, sizeof(h_dss), cudaMemcpyHostToDevice, s));
  if (F->d_adicf) {   // and its ADI coefficients
    float h_cf[12];
    adi_coef_rows(h_dss, 2, D.dx, D.dy, h_cf);
    CK(cudaMemcpyAsync(F->d_adicf + 6 * (D.ns + 1), h_cf, sizeof(h_cf), cudaMemcpyHostToDevice, s));
    D.adicf = F->d_adicf + 6 * (D.ns + 1);
  }
  D.dss = F->d_dss + D.ns + 1;
  D.ns = 1;
  D.na = 1;
  D.single = 1;
  D.brush = 0;
  const size_t n = (size_t)ctx->npts;
  k_convert<T, double><<<std::max<size_t>(1, (n + 255) / 256), 256, 0, s>>>(d_prop, D.q, n);
  FieldRef fr{};
  fr.direct = d_w;
  if (ctx->geometry == ADSCF_FILM_3D) {
    if (sizeof(T) == 4)   // one field (type 0) of npts values
      k_film_wconv<<<(int)std::min<size_t>((n + 255) / 256, 152 * 4), 256, 0, s>>>(fr, D.wf, n);
    if constexpr (sizeof(T) == 4) {
      if (!F->adi_set) adi_defaults(F, fdev<float>(F));
    }
    const AdiLaunch A = adi_launch<T>(F, D, 1);
    adi_step<T>(A, D, fr, 1, 1, s);
  } else {
    if (sizeof(T) == 4)   // one field (type 0) of npts values
      k_film_wconv<<<(int)std::min<size_t>((n + 255) / 256, 152 * 4), 256, 0, s>>>(fr, D.wf, n);
    launch_chains_1d<T>(D, fr, 1, s);
  }
  k_convert<double, T><<<std::max<size_t>(1, (n + 255) / 256), 256, 0, s>>>(D.q + n, d_prop, n);
  CK(cudaGetLastError());
  return ADSCF_OK;
}

template <typename T>
int alloc_t(adscf_ctx* ctx, FilmState* F, size_t gam_elems) {
  const size_t n = (size_t)ctx->npts;
  const size_t sl = (size_t)(ctx->ns + 1) * n;
  if (cudaMalloc(&F->d_q, sl * sizeof(T)) || cudaMalloc(&F->d_qd, sl * sizeof(T)) ||
      cudaMalloc(&F->d_gam, gam_elems * sizeof(T)) ||
      (ctx->geometry == ADSCF_FILM_3D && cudaMalloc(&F->d_w1, 2 * n * sizeof(T)))) {
    cudaGetLastError();
    return set_err(ctx, ADSCF_E_OOM, "device allocation of film propagators failed");
  }
  return ADSCF_OK;
}

template <typename T>
void fill_dev(adscf_ctx* ctx, FilmState* F, const adscf_params* p) {
  FilmDev<T>& D = fdev<T>(F);
  D.gx = ctx->gx; D.gy = ctx->gy; D.gz = ctx->gz;
  D.nlines = ctx->gx * ctx->gy;
  D.npts = ctx->npts;
  D.ns = ctx->ns; D.na = ctx->na;
  D.ntypes = ctx->ntypes;
  D.brush = ctx->geometry == ADSCF_BRUSH;
  D.single = 0;
  D.span = p->int_span;
  D.alpha = F->d_alpha; D.beta = F->d_beta; D.gamma = F->d_gamma;
  D.dss = F->d_dss; D.wA = F->d_wA; D.wB = F->d_wB;
  D.adicf = F->d_adicf;
  D.wz = ctx->d_wz;
  D.graft = F->d_graft;
  D.q = static_cast<T*>(F->d_q);
  D.qd = static_cast<T*>(F->d_qd);
  D.gam = static_cast<T*>(F->d_gam);
  D.dist = ctx->d_dist;
  D.qpart = ctx->d_qpart;
  D.err = F->d_err;
  D.dx = p->sizex / p->gx;
  D.dy = p->sizey / p->gy;
  D.w1 = static_cast<T*>(F->d_w1);
  const size_t n1 = (size_t)ctx->gz + 1;
  D.alf = F->d_alf;
  D.bef = F->d_alf ? F->d_alf + n1 : nullptr;
  D.gaf = F->d_alf ? F->d_alf + 2 * n1 : nullptr;
  D.wf = F->d_wf;
}

}  // namespace

int film_create(adscf_ctx* ctx, const adscf_params* p) {
  FilmState* F = new (std::nothrow) FilmState();
  if (!F) return ADSCF_E_OOM;
  ctx->film = F;
  const int gz = ctx->gz;
  if (ctx->geometry == ADSCF_FILM_3D && (ctx->gx < 1 || ctx->gy < 1))
    return set_err(ctx, ADSCF_E_ARG, "grid");
  FilmTables tb;
  std::string why;
  if (film_tables(*p, ctx->ns, ctx->na, tb, why)) return set_err(ctx, ADSCF_E_ARG, why);
  F->max_ratio = tb.max_ratio;
  ctx->S.chain_len = tb.chain_len;
  const std::vector<double>& al = tb.al;
  const std::vector<double>& be = tb.be;
  const std::vector<double>& ga = tb.ga;
  const std::vector<double>& wz = tb.wz;
  const std::vector<double>& dss = tb.dss;
  const std::vector<double>& wA = tb.wA;
  const std::vector<double>& wB = tb.wB;
  F->t64 = film_sweep_fp64(ctx->prec, F->max_ratio);
  const size_t L = (size_t)ctx->gx * ctx->gy;
  size_t gam_elems = 2 * (size_t)(gz + 1) * L;
  if (ctx->geometry == ADSCF_FILM_3D) {
    const size_t lx = (size_t)ctx->gy * (gz - 1), ly = (size_t)ctx->gx * (gz - 1);
    gam_elems = std::max(gam_elems, std::max(2 * 2 * (size_t)ctx->gx * lx, 2 * 2 * (size_t)ctx->gy * ly));
  }
  CK(cudaMalloc(&F->d_alpha, (gz + 1) * sizeof(double)));
  CK(cudaMalloc(&F->d_beta, (gz + 1) * sizeof(double)));
  CK(cudaMalloc(&F->d_gamma, (gz + 1) * sizeof(double)));
  CK(cudaMalloc(&F->d_dss, (ctx->ns + 3) * sizeof(double)));
  CK(cudaMalloc(&F->d_wA, (ctx->ns + 1) * sizeof(double)));
  CK(cudaMalloc(&F->d_wB, (ctx->ns + 1) * sizeof(double)));
  CK(cudaMalloc(&F->d_err, sizeof(int)));
  CK(cudaMalloc(&ctx->d_wz, (gz + 1) * sizeof(double)));
  CK(cudaMemcpy(F->d_alpha, al.data(), (gz + 1) * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(F->d_beta, be.data(), (gz + 1) * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(F->d_gamma, ga.data(), (gz + 1) * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(F->d_dss, dss.data(), (ctx->ns + 1) * sizeof(double), cudaMemcpyHostToDevice));
  if (ctx->geometry == ADSCF_FILM_3D) {
    std::vector<float> cf(6 * ((size_t)ctx->ns + 3), 0.f);
    adi_coef_rows(dss.data(), ctx->ns + 1, p->sizex / p->gx, p->sizey / p->gy, cf.data());
    CK(cudaMalloc(&F->d_adicf, cf.size() * sizeof(float)));
    CK(cudaMemcpy(F->d_adicf, cf.data(), cf.size() * sizeof(float), cudaMemcpyHostToDevice));
  }
  CK(cudaMemcpy(F->d_wA, wA.data(), (ctx->ns + 1) * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(F->d_wB, wB.data(), (ctx->ns + 1) * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_wz, wz.data(), (gz + 1) * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemset(F->d_err, 0, sizeof(int)));
  if (p->ext_potential) {
    CK(cudaMalloc(&ctx->d_ext, (size_t)ctx->ntypes * (gz + 1) * sizeof(double)));
    CK(cudaMemcpy(ctx->d_ext, p->ext_potential, (size_t)ctx->ntypes * (gz + 1) * sizeof(double),
                  cudaMemcpyHostToDevice));
  }
  if (ctx->geometry == ADSCF_BRUSH) {
    if (!p->graft) return set_err(ctx, ADSCF_E_ARG, "brush needs the grafting distribution");
    CK(cudaMalloc(&F->d_graft, (gz + 1) * sizeof(double)));
    CK(cudaMemcpy(F->d_graft, p->graft, (gz + 1) * sizeof(double), cudaMemcpyHostToDevice));
  }
  CK(cudaDeviceGetAttribute(&F->optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->dev));
  if (ctx->geometry == ADSCF_FILM_3D) {
    const size_t es = F->t64 ? sizeof(double) : sizeof(float);
    const int nmax = std::max(ctx->gx, std::max(ctx->gy, gz + 1));
    if (adi_smem_y(nmax, 1, es) > (size_t)F->optin) return set_err(ctx, ADSCF_E_ARG, "ADI line too long for shared memory");
    // shared memory is a per-function limit set in the launching file
    CK(cudaFuncSetAttribute(k_adi_x<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, F->optin));
    CK(cudaFuncSetAttribute(k_adi_y<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, F->optin));
    CK(cudaFuncSetAttribute(k_adi_z<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, F->optin));
    CK(cudaFuncSetAttribute(k_adi_x<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, F->optin));
    CK(cudaFuncSetAttribute(k_adi_y<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, F->optin));
    CK(cudaFuncSetAttribute(k_adi_z<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, F->optin));
  }
  if (!F->t64) {
    std::vector<float> f3(3 * (size_t)(gz + 1));
    for (int j = 0; j <= gz; ++j) {
      f3[j] = (float)al[j];
      f3[gz + 1 + j] = (float)be[j];
      f3[2 * (gz + 1) + j] = (float)ga[j];
    }
    CK(cudaMalloc(&F->d_alf, f3.size() * sizeof(float)));
    CK(cudaMemcpy(F->d_alf, f3.data(), f3.size() * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMalloc(&F->d_wf, (size_t)ctx->ntypes * ctx->npts * sizeof(float)));
  }
  ctx->contour_blocks = (int)std::min<size_t>(((size_t)ctx->npts + 255) / 256, 152 * 4);
  CK(cudaMalloc(&ctx->d_qpart, ctx->contour_blocks * sizeof(double)));
  int rc = F->t64 ? alloc_t<double>(ctx, F, gam_elems) : alloc_t<float>(ctx, F, gam_elems);
  if (rc) return rc;
  if (F->t64) fill_dev<double>(ctx, F, p);
  else fill_dev<float>(ctx, F, p);
  ctx->film_launches = ctx->geometry == ADSCF_FILM_3D ? 1 + 3 * ctx->ns : 1;
  ctx->film_contour_launches = 1;
  if (ctx->geometry == ADSCF_FILM_3D && !F->t64) {   // FP32 ADI sweeps: pick their shapes
    FilmDev<float>& D = F->f32;
    if (!ctx->autotune) {
      adi_defaults(F, D);
      return ADSCF_OK;
    }
    const size_t n = (size_t)ctx->ntypes * D.npts;
    CK(cudaMemsetAsync(ctx->d_tmp, 0, n * sizeof(double), ctx->stream));
    const FieldRef fr = make_ref(ctx, ctx->d_tmp);
    k_film_fill<float><<<std::max(1, (D.npts + 255) / 256), 256, 0, ctx->stream>>>(D.q, D.qd, D.npts);
    k_film_wconv<<<(int)std::min<size_t>((n + 255) / 256, 152 * 4), 256, 0, ctx->stream>>>(fr, D.wf, n);
    CK(cudaGetLastError());
    return adi_tune(ctx, F, D, fr);
  }
  return ADSCF_OK;
}

// Pin the FP32 ADI sweep shapes by lanes per line (0: one thread per line),
// staging through shared memory (mask: 2 y, 4 z) and the fused x + y plane
// kernel (mask 8; the x and y shapes must allow it).
int film_set_adi_plan(adscf_ctx* ctx, const int lanes[3], int staged) {
  FilmState* F = ctx->film;
  if (ctx->geometry != ADSCF_FILM_3D || F->t64) return ADSCF_E_STATE;
  const bool fuse = (staged & 8) != 0;
  staged &= 7;
  AdiShape sh[3];
  for (int d = 0; d < 3; ++d) {
    sh[d] = {0, 0, 0};
    const int st = (staged >> d) & 1;
    if (lanes[d] == 0 && !st) continue;
    bool found = false;
    for (const AdiShape& a : adi_shapes(d, F->f32))
      if (a.g == lanes[d] && a.staged == st) { sh[d] = a; found = true; }
    if (!found) return ADSCF_E_ARG;
  }
  if (fuse && !adi_fused_ok(sh[0], sh[1], F->f32)) return ADSCF_E_ARG;
  for (int d = 0; d < 3; ++d) F->adi[d] = sh[d];
  F->adi_fuse = fuse;
  F->adi_set = true;
  ctx->film_launches = 1 + (fuse ? 2 : 3) * ctx->ns;
  return ADSCF_OK;
}

// F at the fields in d_fe_w (copied there by the caller) and its gradient
int film_forward(adscf_ctx* ctx, double* out_F) {
  FilmState* F = ctx->film;
  const size_t nv = (size_t)ctx->ntypes * ctx->npts;
  if (!F->d_fe_part) {
    CK(cudaMalloc(&F->d_fe_part, (size_t)ctx->nplanes * FE_N * sizeof(double)));
    CK(cudaMalloc(&F->d_fe_out, (2 + (size_t)ctx->ntypes * ctx->nplanes) * sizeof(double)));
  }
  int rc = film_enqueue_propagate(ctx, F->d_fe_w);
  if (rc) return rc;
  if ((rc = film_check_pivot(ctx))) return rc;
  k_film_fe<<<ctx->nplanes, 256, 0, ctx->stream>>>(ctx->S, F->d_fe_w, F->d_fe_part);
  k_film_fe_sc<<<1, 32, 0, ctx->stream>>>(ctx->S, F->d_fe_part, F->d_fe_out);
  CK(cudaGetLastError());
  double f = 0.0;
  CK(cudaMemcpyAsync(&f, F->d_fe_out, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (!std::isfinite(f)) return set_err(ctx, ADSCF_E_NONFINITE, "non-finite free energy");
  F->fe_gen = ++ctx->prop_gen;
  if (out_F) *out_F = f;
  return ADSCF_OK;
}

double* film_fe_field(adscf_ctx* ctx) {
  FilmState* F = ctx->film;
  if (!F->d_fe_w && cudaMalloc(&F->d_fe_w, (size_t)ctx->ntypes * ctx->npts * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return F->d_fe_w;
}

int film_backward(adscf_ctx* ctx, double* dF_dchi, double* dF_dU) {
  FilmState* F = ctx->film;
  if (F->fe_gen != ctx->prop_gen || !F->d_fe_out)
    return set_err(ctx, ADSCF_E_STATE, "the film gradient needs the state of an immediately preceding adscf_forward");
  const size_t n = 2 + (size_t)ctx->ntypes * ctx->nplanes;
  std::vector<double> h(n);
  CK(cudaMemcpyAsync(h.data(), F->d_fe_out, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (dF_dchi) *dF_dchi = h[1];
  if (dF_dU) std::memcpy(dF_dU, h.data() + 2, (n - 2) * sizeof(double));
  return ADSCF_OK;
}

void film_destroy(adscf_ctx* ctx) {
  FilmState* F = ctx->film;
  if (!F) return;
  cudaFree(F->d_fe_w); cudaFree(F->d_fe_part); cudaFree(F->d_fe_out);
  cudaFree(F->d_alpha); cudaFree(F->d_beta); cudaFree(F->d_gamma);
  cudaFree(F->d_dss); cudaFree(F->d_adicf); cudaFree(F->d_wA); cudaFree(F->d_wB); cudaFree(F->d_graft);
  cudaFree(F->d_alf); cudaFree(F->d_wf);
  cudaFree(F->d_q); cudaFree(F->d_qd); cudaFree(F->d_gam); cudaFree(F->d_w1);
  cudaFree(F->d_err); cudaFree(ctx->d_qpart);
  delete F;
  ctx->film = nullptr;
}

int film_enqueue_chains(adscf_ctx* ctx, const double* d_w) {
  return ctx->film->t64 ? chains_t<double>(ctx, d_w) : chains_t<float>(ctx, d_w);
}
int film_enqueue_contour(adscf_ctx* ctx) {
  return ctx->film->t64 ? contour_t<double>(ctx) : contour_t<float>(ctx);
}
int film_enqueue_propagate(adscf_ctx* ctx, const double* d_w) {
  int rc = film_enqueue_chains(ctx, d_w);
  return rc ? rc : film_enqueue_contour(ctx);
}
int film_step_single(adscf_ctx* ctx, double* d_prop, const double* d_w, double ds) {
  return ctx->film->t64 ? step_single_t<double>(ctx, d_prop, d_w, ds)
                        : step_single_t<float>(ctx, d_prop, d_w, ds);
}
// pivot flag set by any sweep since the last check (cleared on read)
int film_check_pivot(adscf_ctx* ctx) {
  if (!ctx->film) return ADSCF_OK;
  int e = 0;
  CK(cudaMemcpyAsync(&e, ctx->film->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (e) {
    CK(cudaMemsetAsync(ctx->film->d_err, 0, sizeof(int), ctx->stream));
    return set_err(ctx, ADSCF_E_PIVOT, "zero pivot in a tridiagonal sweep (TriDiag Error)");
  }
  return ADSCF_OK;
}
