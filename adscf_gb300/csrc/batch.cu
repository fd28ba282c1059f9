// batch.cu -- many independent bulk diblock SCF instances as one device job.
//
// Each instance is the bulk SCF loop of Bulk_3D_FFT/Main_Diblock_Melt/
// main_diblock.f90:410-429 with its own grid, box, contour step, block
// lengths, chi and kappa (a phase-diagram or box-size scan); the reference
// runs such scans as separate program invocations.  All instances advance
// together: one launch per pass and contour step covers every instance still
// on its contour (work lists sorted by Ns, so the active tiles of step t are
// a prefix), one contour launch, and batched closure / Anderson solve / mix
// launches with each instance's mixing history on the device.  One batch
// iteration is one CUDA graph.  The line passes are the generic mixed-radix
// kernels of bulk_kernels.cuh (any grid of 2, 3 and 5 factors).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "internal.h"
#include "bulk_host.h"

struct adscf_batch {
  int n = 0, prec = ADSCF_SPLIT;
  std::string err;
  int dev = 0;
  cudaStream_t stream = nullptr, own_stream = nullptr;
  std::vector<adscf_params> p;
  std::vector<int> ns, npts, slots;
  std::vector<size_t> foff;             // packed [2][npts_i] offsets (doubles), n+1 entries
  void* pool = nullptr;                 // every per-instance buffer
  void* d_inst = nullptr;               // BulkDev<T>[n]
  ScfDev* d_S = nullptr;                // ScfDev[n]
  std::vector<ScfDev> hS;
  std::vector<void*> E;                 // per-instance Boltzmann factors
  double* d_resall = nullptr;           // [n][R_COUNT]
  int* d_iterall = nullptr;             // [n]
  void* d_tw = nullptr;
  void* d_fk = nullptr;
  double* d_g64 = nullptr;
  int2 *d_wx = nullptr, *d_wy = nullptr, *d_wz = nullptr;
  std::vector<int> pre_x, pre_y, pre_z;  // tiles active at contour step t (t = 0..maxns)
  size_t smx = 0, smy = 0, smz = 0;
  int maxns = 0, cont_blocks = 64, clos_grid = 0, mix_grid = 0;
  cudaGraphExec_t g_iter = nullptr;
  double* h_pinned = nullptr;
  size_t pinned_bytes = 0;
};

namespace {

int berr(adscf_batch* b, int code, const std::string& m) {
  if (b) b->err = m;
  return code;
}
#define BK(call)                                                                             \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) return berr(b, ADSCF_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

int nint_b(double x) { return x >= 0 ? (int)std::floor(x + 0.5) : -(int)std::floor(-x + 0.5); }

struct Carve {
  size_t off = 0;
  size_t take(size_t bytes) {
    const size_t o = off;
    off += (bytes + 255) & ~size_t(255);
    return o;
  }
};

int check_params(const adscf_params& q, int prec, std::string& why) {
  if (q.geometry != ADSCF_BULK) { why = "batch instances are bulk"; return ADSCF_E_ARG; }
  if (q.precision != prec) { why = "one precision for the whole batch"; return ADSCF_E_ARG; }
  if (q.gx < 1 || q.gy < 1 || q.gz < 1) { why = "grid"; return ADSCF_E_ARG; }
  if (!(q.sizex > 0 && q.sizey > 0 && q.sizez > 0)) { why = "box size"; return ADSCF_E_ARG; }
  if (!(q.ds > 0) || q.dss) { why = "bulk instances take ds"; return ADSCF_E_ARG; }
  if (q.mixing_type < 1 || q.mixing_type > 3) { why = "mixing_type"; return ADSCF_E_ARG; }
  if (q.mixing_type == 3 && (q.mixing_dim < 1 || q.mixing_dim > SCF_MAX_HIST)) { why = "mixing_dim"; return ADSCF_E_ARG; }
  if (q.ensemble != 1 && q.ensemble != 2) { why = "ensemble"; return ADSCF_E_ARG; }
  return ADSCF_OK;
}

template <typename T>
int build(adscf_batch* b) {
  const int n = b->n;
  std::vector<BulkDev<T>> I(n);
  std::vector<cplx<T>> tw;
  std::vector<std::pair<int, int>> seen;
  std::vector<T> fk;
  std::vector<double> g64;
  b->ns.resize(n); b->npts.resize(n); b->slots.resize(n); b->foff.assign(n + 1, 0);
  b->hS.resize(n); b->E.resize(n);
  for (int i = 0; i < n; ++i) {
    const adscf_params& q = b->p[i];
    BulkDev<T>& d = I[i];
    d.gx = q.gx; d.gy = q.gy; d.gz = q.gz;
    d.npts = q.gx * q.gy * q.gz;
    const int sa = nint_b(q.block_length[0] / q.ds), sb = nint_b(q.block_length[1] / q.ds);
    d.ns = sa + sb; d.na = sa; d.nb = sb;
    d.ds = q.ds;
    if (d.ns < 1 || sa < 0 || sb < 0) return berr(b, ADSCF_E_ARG, "instance " + std::to_string(i) + ": contour");
    if (!bulkhost::make_plan(q.gx, d.px) || !bulkhost::make_plan(q.gy, d.py) || !bulkhost::make_plan(q.gz, d.pz))
      return berr(b, ADSCF_E_ARG, "instance " + std::to_string(i) + ": grid sizes must be products of 2, 3 and 5");
    d.px.tw_off = bulkhost::twiddle_offset<T>(q.gx, tw, seen);
    d.py.tw_off = bulkhost::twiddle_offset<T>(q.gy, tw, seen);
    d.pz.tw_off = bulkhost::twiddle_offset<T>(q.gz, tw, seen);
    bulkhost::append_tables<T>(q.gx, q.gy, q.gz, q.sizex, q.sizey, q.sizez, q.ds, fk, g64,
                               d.gxy_off, d.gz_off, d.g64_off);
    d.tw64_off = 0;
    b->ns[i] = d.ns;
    b->npts[i] = d.npts;
    b->slots[i] = q.mixing_type == 3 ? q.mixing_dim + 1 : 2;
    b->foff[i + 1] = b->foff[i] + 2 * (size_t)d.npts;
    b->maxns = std::max(b->maxns, d.ns);
  }
  // pool: one allocation, 256-byte aligned regions
  Carve c;
  struct Off { size_t spec, slices, E, dist, dens, hx, hr, qpart, part, gram, coef; };
  std::vector<Off> o(n);
  int clos_max = 1;
  std::vector<int> clos(n);
  for (int i = 0; i < n; ++i) {
    const size_t np = b->npts[i];
    clos[i] = (int)std::min<size_t>((np + SCF_THREADS - 1) / SCF_THREADS, 128);
    clos_max = std::max(clos_max, clos[i]);
    o[i].spec = c.take(np * sizeof(cplx<T>));
    o[i].slices = c.take((size_t)(b->ns[i] + 1) * np * sizeof(cplx<T>));
    o[i].E = c.take((sizeof(T) == 4 ? 4 : 2) * np * sizeof(T));
    o[i].dist = c.take(2 * np * sizeof(double));
    o[i].dens = c.take(2 * np * sizeof(double));
    o[i].hx = c.take((size_t)b->slots[i] * 2 * np * sizeof(double));
    o[i].hr = c.take((size_t)b->slots[i] * 2 * np * sizeof(double));
    o[i].qpart = c.take((size_t)b->cont_blocks * sizeof(double));
    o[i].part = c.take((size_t)clos[i] * NPART * sizeof(double));
    o[i].gram = c.take(SCF_MAX_SLOTS * SCF_MAX_SLOTS * sizeof(double));
    o[i].coef = c.take(2 * SCF_MAX_SLOTS * sizeof(double));
  }
  const size_t o_res = c.take((size_t)n * R_COUNT * sizeof(double));
  const size_t o_iter = c.take((size_t)n * sizeof(int));
  if (cudaMalloc(&b->pool, c.off) != cudaSuccess) {
    cudaGetLastError();
    return berr(b, ADSCF_E_OOM, "batch pool of " + std::to_string(c.off >> 20) + " MiB");
  }
  unsigned char* base = static_cast<unsigned char*>(b->pool);
  BK(cudaMemsetAsync(b->pool, 0, c.off, b->stream));
  b->d_resall = reinterpret_cast<double*>(base + o_res);
  b->d_iterall = reinterpret_cast<int*>(base + o_iter);
  b->clos_grid = clos_max;
  b->mix_grid = clos_max;
  for (int i = 0; i < n; ++i) {
    const adscf_params& q = b->p[i];
    BulkDev<T>& d = I[i];
    d.spec = reinterpret_cast<cplx<T>*>(base + o[i].spec);
    d.slices = reinterpret_cast<cplx<T>*>(base + o[i].slices);
    d.E = reinterpret_cast<T*>(base + o[i].E);
    d.dist = reinterpret_cast<double*>(base + o[i].dist);
    d.qpart = reinterpret_cast<double*>(base + o[i].qpart);
    b->E[i] = d.E;
    ScfDev& S = b->hS[i];
    S = ScfDev{};
    const double volume = q.sizex * q.sizey * q.sizez;
    S.npts = d.npts; S.ntypes = 2; S.plane = q.gx * q.gy; S.nplanes = q.gz; S.wall_mask = 0;
    S.dvol = volume / (double)d.npts;
    S.kappa = q.kappa; S.chi = q.chi;
    S.v0 = q.monomer_volume[0] != 0 ? q.monomer_volume[0] : 1.0;
    S.v1 = q.monomer_volume[1] != 0 ? q.monomer_volume[1] : 1.0;
    S.ww = q.ww; S.homopolymer = 0;
    S.ensemble = q.ensemble; S.rho = q.rho; S.mu = q.mu; S.volume = volume;
    S.chain_len = q.ds * d.ns;
    S.dist = d.dist;
    S.dens = reinterpret_cast<double*>(base + o[i].dens);
    S.hx = reinterpret_cast<double*>(base + o[i].hx);
    S.hr = reinterpret_cast<double*>(base + o[i].hr);
    S.slots = b->slots[i];
    S.mixing_type = q.mixing_type;
    S.warm = q.warm_iters > q.mixing_dim ? q.warm_iters : q.mixing_dim;
    S.lambda = q.lambda;
    S.lam_warm = q.lam_warm > 0 ? q.lam_warm : 1.0e-3;
    S.qpart = d.qpart; S.nqpart = b->cont_blocks; S.qscale = S.dvol;
    S.part = reinterpret_cast<double*>(base + o[i].part);
    S.npart_blocks = clos[i];
    S.gram = reinterpret_cast<double*>(base + o[i].gram);
    S.coef = reinterpret_cast<double*>(base + o[i].coef);
    S.iter = b->d_iterall + i;
    S.res = b->d_resall + (size_t)i * R_COUNT;
    S.mixE = d.E;
    S.mixds = q.ds;
  }
  BK(cudaMalloc(&b->d_inst, n * sizeof(BulkDev<T>)));
  BK(cudaMemcpyAsync(b->d_inst, I.data(), n * sizeof(BulkDev<T>), cudaMemcpyHostToDevice, b->stream));
  BK(cudaMalloc(&b->d_S, n * sizeof(ScfDev)));
  BK(cudaMemcpyAsync(b->d_S, b->hS.data(), n * sizeof(ScfDev), cudaMemcpyHostToDevice, b->stream));
  BK(cudaMalloc(&b->d_tw, tw.size() * sizeof(cplx<T>)));
  BK(cudaMemcpyAsync(b->d_tw, tw.data(), tw.size() * sizeof(cplx<T>), cudaMemcpyHostToDevice, b->stream));
  BK(cudaMalloc(&b->d_fk, fk.size() * sizeof(T)));
  BK(cudaMemcpyAsync(b->d_fk, fk.data(), fk.size() * sizeof(T), cudaMemcpyHostToDevice, b->stream));
  BK(cudaMalloc(&b->d_g64, g64.size() * sizeof(double)));
  BK(cudaMemcpyAsync(b->d_g64, g64.data(), g64.size() * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  std::vector<int> ones(n, 1);
  BK(cudaMemcpyAsync(b->d_iterall, ones.data(), n * sizeof(int), cudaMemcpyHostToDevice, b->stream));

  // work lists, instances by descending Ns: the tiles of the instances still
  // on their contour at step t are a prefix
  std::vector<int> ord(n);
  for (int i = 0; i < n; ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int c2) { return b->ns[a] > b->ns[c2]; });
  std::vector<int2> wx, wy, wz;
  std::vector<int> tx(n), ty(n), tz(n);
  for (int i : ord) {
    const BulkDev<T>& d = I[i];
    tx[i] = (d.gy * d.gz + d.px.lpc - 1) / d.px.lpc;
    ty[i] = (d.gx * d.gz + d.py.lpc - 1) / d.py.lpc;
    tz[i] = (d.gx * d.gy + d.pz.lpc - 1) / d.pz.lpc;
    for (int k = 0; k < tx[i]; ++k) wx.push_back(make_int2(i, k));
    for (int k = 0; k < ty[i]; ++k) wy.push_back(make_int2(i, k));
    for (int k = 0; k < tz[i]; ++k) wz.push_back(make_int2(i, k));
    b->smx = std::max(b->smx, bulkhost::plan_smem<T>(d.px));
    b->smy = std::max(b->smy, bulkhost::plan_smem<T>(d.py));
    b->smz = std::max(b->smz, bulkhost::plan_smem_z<T>(d.pz));
  }
  b->pre_x.assign(b->maxns + 1, 0); b->pre_y.assign(b->maxns + 1, 0); b->pre_z.assign(b->maxns + 1, 0);
  for (int t = 0; t <= b->maxns; ++t)
    for (int i : ord)
      if (b->ns[i] >= t) { b->pre_x[t] += tx[i]; b->pre_y[t] += ty[i]; b->pre_z[t] += tz[i]; }
  BK(cudaMalloc(&b->d_wx, wx.size() * sizeof(int2)));
  BK(cudaMalloc(&b->d_wy, wy.size() * sizeof(int2)));
  BK(cudaMalloc(&b->d_wz, wz.size() * sizeof(int2)));
  BK(cudaMemcpyAsync(b->d_wx, wx.data(), wx.size() * sizeof(int2), cudaMemcpyHostToDevice, b->stream));
  BK(cudaMemcpyAsync(b->d_wy, wy.data(), wy.size() * sizeof(int2), cudaMemcpyHostToDevice, b->stream));
  BK(cudaMemcpyAsync(b->d_wz, wz.data(), wz.size() * sizeof(int2), cudaMemcpyHostToDevice, b->stream));
  int optin = 0;
  BK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->dev));
  if (std::max(b->smx, std::max(b->smy, b->smz)) > (size_t)optin)
    return berr(b, ADSCF_E_ARG, "grid line too long for shared memory");
  // this translation unit's instances of the generic passes (own device module)
  BK(cudaFuncSetAttribute(k_bulk_xpass<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
  BK(cudaFuncSetAttribute(k_bulk_strided<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
  BK(cudaStreamSynchronize(b->stream));
  return ADSCF_OK;
}

template <typename T>
int enqueue_iteration(adscf_batch* b) {
  const BulkDev<T>* d = static_cast<const BulkDev<T>*>(b->d_inst);
  const cplx<T>* tw = static_cast<const cplx<T>*>(b->d_tw);
  const T* fk = static_cast<const T*>(b->d_fk);
  cudaStream_t s = b->stream;
  const XAux none{nullptr, nullptr, nullptr};
  k_bulk_xpass<T><<<b->pre_x[0], BULK_THREADS, b->smx, s>>>(d, b->d_wx, tw, 0, XM_INIT, none);
  for (int t = 1; t <= b->maxns; ++t) {
    k_bulk_strided<T><<<b->pre_y[t], BULK_THREADS, b->smy, s>>>(d, b->d_wy, tw, fk, nullptr, b->d_g64, t, 0);
    k_bulk_strided<T><<<b->pre_z[t], BULK_THREADS, b->smz, s>>>(d, b->d_wz, tw, fk, nullptr, b->d_g64, t, 2);
    k_bulk_strided<T><<<b->pre_y[t], BULK_THREADS, b->smy, s>>>(d, b->d_wy, tw, fk, nullptr, b->d_g64, t, 1);
    k_bulk_xpass<T><<<b->pre_x[t], BULK_THREADS, b->smx, s>>>(d, b->d_wx, tw, t, XM_STEP, none);
  }
  k_bulk_contour<T><<<dim3(b->cont_blocks, b->n), BULK_THREADS, 0, s>>>(d);
  k_closure_b<<<dim3(b->clos_grid, b->n), SCF_THREADS, 0, s>>>(b->d_S, CL_MEANFIELD | CL_MIXDOTS);
  k_solve_b<<<b->n, 64, 0, s>>>(b->d_S, 1, 1);
  k_mix_b<T><<<dim3(b->mix_grid, b->n), SCF_THREADS, 0, s>>>(b->d_S, b->mix_grid);
  BK(cudaGetLastError());
  return ADSCF_OK;
}

int enqueue(adscf_batch* b) {
  return b->prec == ADSCF_SPLIT ? enqueue_iteration<float>(b) : enqueue_iteration<double>(b);
}

int build_graph(adscf_batch* b) {
  if (b->g_iter) return ADSCF_OK;
  cudaGraph_t g;
  BK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  const int rc = enqueue(b);
  cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (rc) return rc;
  if (e != cudaSuccess) return berr(b, ADSCF_E_CUDA, std::string("capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&b->g_iter, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return berr(b, ADSCF_E_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
  return ADSCF_OK;
}

int pinned(adscf_batch* b, size_t bytes) {
  if (bytes <= b->pinned_bytes) return ADSCF_OK;
  if (b->h_pinned) cudaFreeHost(b->h_pinned);
  b->h_pinned = nullptr;
  b->pinned_bytes = 0;
  BK(cudaMallocHost(&b->h_pinned, bytes));
  b->pinned_bytes = bytes;
  return ADSCF_OK;
}

int read_iters(adscf_batch* b, std::vector<int>& it) {
  it.resize(b->n);
  BK(cudaMemcpyAsync(it.data(), b->d_iterall, b->n * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  BK(cudaStreamSynchronize(b->stream));
  return ADSCF_OK;
}

int read_results(adscf_batch* b, adscf_iter_result* out, double* max_acc) {
  std::vector<double> r((size_t)b->n * R_COUNT);
  BK(cudaMemcpyAsync(r.data(), b->d_resall, r.size() * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  BK(cudaStreamSynchronize(b->stream));
  double mx = 0.0;
  int bad = -1;
  for (int i = 0; i < b->n; ++i) {
    const double* q = r.data() + (size_t)i * R_COUNT;
    if (out) {
      out[i].accuracy = q[R_ACC]; out[i].free_energy = q[R_F]; out[i].Qsum = q[R_Q];
      out[i].logQ = q[R_LOGQ]; out[i].mu = q[R_MU]; out[i].rho = q[R_RHO];
      out[i].lambda = q[R_LAMBDA]; out[i].iter = (int)q[R_ITER]; out[i].status = (int)q[R_STATUS];
    }
    if (q[R_STATUS] != 0.0 && bad < 0) bad = i;
    if (!(q[R_ACC] <= mx)) mx = q[R_ACC];   // NaN propagates
  }
  if (max_acc) *max_acc = mx;
  if (bad >= 0) return berr(b, ADSCF_E_NONFINITE, "instance " + std::to_string(bad) + ": non-finite or non-positive Q");
  return ADSCF_OK;
}

template <typename T>
int set_fields_t(adscf_batch* b, const double* fields) {
  const size_t tot = b->foff[b->n];
  int rc = pinned(b, tot * sizeof(double));
  if (rc) return rc;
  std::memcpy(b->h_pinned, fields, tot * sizeof(double));
  for (int i = 0; i < b->n; ++i) {
    const ScfDev& S = b->hS[i];
    const size_t nv = 2 * (size_t)S.npts;
    BK(cudaMemsetAsync(S.hx, 0, (size_t)S.slots * nv * sizeof(double), b->stream));
    BK(cudaMemsetAsync(S.hr, 0, (size_t)S.slots * nv * sizeof(double), b->stream));
    BK(cudaMemsetAsync(S.gram, 0, SCF_MAX_SLOTS * SCF_MAX_SLOTS * sizeof(double), b->stream));
    double* x1 = S.hx + (size_t)(1 % S.slots) * nv;
    BK(cudaMemcpyAsync(x1, b->h_pinned + b->foff[i], nv * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    const int gb = (int)std::min<size_t>((nv + 255) / 256, 152 * 8);
    k_expfield<T><<<gb, 256, 0, b->stream>>>(x1, static_cast<T*>(b->E[i]), (size_t)S.npts, b->p[i].ds);
  }
  std::vector<int> ones(b->n, 1);
  BK(cudaMemcpyAsync(b->d_iterall, ones.data(), b->n * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  BK(cudaGetLastError());
  BK(cudaStreamSynchronize(b->stream));
  return ADSCF_OK;
}

// current fields (the history slot of each instance's iteration counter) or densities
int get_t(adscf_batch* b, double* out, bool fields) {
  std::vector<int> it;
  int rc = read_iters(b, it);
  if (rc) return rc;
  const size_t tot = b->foff[b->n];
  if ((rc = pinned(b, tot * sizeof(double)))) return rc;
  for (int i = 0; i < b->n; ++i) {
    const ScfDev& S = b->hS[i];
    const size_t nv = 2 * (size_t)S.npts;
    const double* src = fields ? S.hx + (size_t)(it[i] % S.slots) * nv : S.dens;
    BK(cudaMemcpyAsync(b->h_pinned + b->foff[i], src, nv * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  }
  BK(cudaStreamSynchronize(b->stream));
  std::memcpy(out, b->h_pinned, tot * sizeof(double));
  return ADSCF_OK;
}

}  // namespace

extern "C" {

int adscf_batch_create(const adscf_params* params, int n, adscf_batch** out) {
  if (!out) return ADSCF_E_ARG;
  *out = nullptr;
  if (!params || n < 1) return ADSCF_E_ARG;
  adscf_batch* b = new (std::nothrow) adscf_batch();
  if (!b) return ADSCF_E_OOM;
  b->n = n;
  b->prec = params[0].precision;
  if (b->prec != ADSCF_FP64 && b->prec != ADSCF_SPLIT) { delete b; return ADSCF_E_ARG; }
  b->p.assign(params, params + n);
  for (int i = 0; i < n; ++i) {
    std::string why;
    if (check_params(b->p[i], b->prec, why)) { delete b; return ADSCF_E_ARG; }
    b->p[i].dss = nullptr; b->p[i].dz = nullptr; b->p[i].ext_potential = nullptr; b->p[i].graft = nullptr;
  }
  if (cudaGetDevice(&b->dev) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete b;
    return ADSCF_E_CUDA;
  }
  b->stream = b->own_stream;
  const int rc = b->prec == ADSCF_SPLIT ? build<float>(b) : build<double>(b);
  if (rc) {
    adscf_batch_destroy(b);
    return rc;
  }
  *out = b;
  return ADSCF_OK;
}

int adscf_batch_destroy(adscf_batch* b) {
  if (!b) return ADSCF_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->g_iter) cudaGraphExecDestroy(b->g_iter);
  cudaFree(b->pool); cudaFree(b->d_inst); cudaFree(b->d_S);
  cudaFree(b->d_tw); cudaFree(b->d_fk); cudaFree(b->d_g64);
  cudaFree(b->d_wx); cudaFree(b->d_wy); cudaFree(b->d_wz);
  if (b->h_pinned) cudaFreeHost(b->h_pinned);
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  delete b;
  return ADSCF_OK;
}

const char* adscf_batch_last_error(const adscf_batch* b) { return b ? b->err.c_str() : "null batch"; }

long long adscf_batch_offset(const adscf_batch* b, int i) {
  if (!b || i < 0 || i > b->n) return -1;
  return (long long)b->foff[i];
}

int adscf_batch_set_fields(adscf_batch* b, const double* fields) {
  if (!b || !fields) return ADSCF_E_ARG;
  return b->prec == ADSCF_SPLIT ? set_fields_t<float>(b, fields) : set_fields_t<double>(b, fields);
}

int adscf_batch_get_fields(adscf_batch* b, double* fields) {
  if (!b || !fields) return ADSCF_E_ARG;
  return get_t(b, fields, true);
}

int adscf_batch_get_densities(adscf_batch* b, double* densities) {
  if (!b || !densities) return ADSCF_E_ARG;
  return get_t(b, densities, false);
}

int adscf_batch_scf_run(adscf_batch* b, int n_iter, double tol, adscf_iter_result* out) {
  if (!b || n_iter < 0) return ADSCF_E_ARG;
  int rc = build_graph(b);
  if (rc) return rc;
  for (int i = 0; i < n_iter; ++i) {
    BK(cudaGraphLaunch(b->g_iter, b->stream));
    if (tol >= 0.0) {
      double mx = 0.0;
      if ((rc = read_results(b, out, &mx))) return rc;
      if (!(mx > tol)) return ADSCF_OK;
    }
  }
  return read_results(b, out, nullptr);
}

int adscf_batch_set_stream(adscf_batch* b, void* cuda_stream) {
  if (!b) return ADSCF_E_ARG;
  BK(cudaStreamSynchronize(b->stream));
  b->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : b->own_stream;
  return ADSCF_OK;
}

int adscf_batch_enqueue(adscf_batch* b, int repeats) {
  if (!b || repeats < 0) return ADSCF_E_ARG;
  int rc = build_graph(b);
  if (rc) return rc;
  for (int i = 0; i < repeats; ++i) BK(cudaGraphLaunch(b->g_iter, b->stream));
  return ADSCF_OK;
}

int adscf_batch_results(adscf_batch* b, adscf_iter_result* out) {
  if (!b || !out) return ADSCF_E_ARG;
  return read_results(b, out, nullptr);
}

int adscf_batch_launches(const adscf_batch* b) { return b ? 1 + 4 * b->maxns + 4 : -1; }

}  // extern "C"
