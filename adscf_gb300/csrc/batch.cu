// batch.cu -- many independent SCF instances (bulk, or one-line films and
// brushes) as one device job.
//
// Each instance is the bulk SCF loop of Bulk_3D_FFT/Main_Diblock_Melt/
// main_diblock.f90:410-429 with its own grid, box, contour step, block
// lengths, chi and kappa (a phase-diagram or box-size scan); the reference
// runs such scans as separate program invocations.  All instances advance
// together: one launch per pass and contour step covers every instance still
// on its contour (work lists sorted by Ns, so the active tiles of step t are
// a prefix), one contour launch, and batched closure / Anderson solve / mix
// launches with each instance's mixing history on the device.  One batch
// iteration is one CUDA graph.  Instances are grouped by pass kernel: cubic
// grids of 32..256 points run the register-FFT passes of bulk_reg.cuh, every
// other grid of 2, 3 and 5 factors the generic mixed-radix passes of
// bulk_kernels.cuh; each group has its own Ns-sorted work lists and launches.
//
// Film batches (Film_CK_AD/Film_1D, Brush_CK_AD: one z line per film with its
// own graded mesh, adaptive contour and wall potential) sweep every film's
// two chains in one launch (one thread per film and chain, CN with the NR
// Thomas solve), take one contour launch and the same batched closure,
// solve and mix.  A film whose mesh is graded past a spacing ratio of 1.5
// keeps its sweep in FP64 on the split path (a second list and launch).
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

#include "internal.h"
#include "bulk_host.h"
#include "bulk_reg.cuh"
#include "film_host.h"
#include "film_kernels.cuh"
#include "film_warp.cuh"
#include "adjoint_kernels.cuh"

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
  // bulk instances grouped by pass kernel: register FFT of one line length
  // on all three axes (32..256), or the generic mixed-radix kernels (n = 0)
  struct PassClass {
    int n = 0;
    int2 *wx = nullptr, *wy = nullptr, *wz = nullptr;
    std::vector<int> px, py, pz;        // tiles active at contour step t (t = 0..maxns)
    size_t smx = 0, smy = 0, smz = 0;
  };
  std::vector<PassClass> cls;
  int maxns = 0, cont_blocks = 64, clos_grid = 0, mix_grid = 0;
  // persistent sweep: one launch, a CTA range per kernel class, work items
  // of every pass of every instance of the class in dependency order;
  // control words [class counters][error flag][items done per instance]
  struct SweepClass {
    int n = 0;                          // kernel class (line length; 0: generic)
    int off = 0, count = 0;             // its items in d_items
  };
  std::vector<SweepClass> sw;
  int4* d_items = nullptr;
  int* d_ctl = nullptr;
  void* d_ranges = nullptr;             // SweepRange per class
  int sweep_grid = 0;
  int sweep_help = 0;                   // class with the most point-steps (finished CTAs help it)
  size_t sweep_smem = 0;
  bool sweep = true;                    // persistent sweeps (ADSCF_BATCH_SWEEP=0: one launch per pass)
  int sweep_tiles = 8;                  // tiles per sweep item (ADSCF_SWEEP_TILES)
  cudaGraphExec_t g_iter = nullptr;
  double* h_pinned = nullptr;
  size_t pinned_bytes = 0;
  // film batches (Film_1D / brush, one line per film)
  bool film = false;
  int ntypes = 2;
  void* d_f32 = nullptr;                // FilmDev<float>[n]
  void* d_f64 = nullptr;                // FilmDev<double>[n]
  int* d_list32 = nullptr;              // films sweeping in FP32 / FP64, by contour length
  int* d_items32 = nullptr;             // (film << 1) | chain of the FP32 films, same order
  int* d_list64 = nullptr;
  int n32 = 0, n64 = 0;
  // shared-memory line sweeps: rows per line (max gz + 1 of the list) and
  // lanes per block (0: the list sweeps on global memory)
  int zcap32 = 0, zcap64 = 0, lanes32 = 0, lanes64 = 0;
  int film_per_warp = 2, film_warps = 2;
  int max_slots = 2;                    // longest mixing history of the instances
  int film_cl_threads = SCF_THREADS;    // closure and solve block of a film batch
  float* d_tabf = nullptr;              // FP32 mesh factors of the FP32 sweeps
  int* d_err = nullptr;                 // zero-pivot flag of the sweeps
  // FP64 bulk batches: host copies of the instances and the adjoint state
  std::vector<BulkDev<double>> hI64;
  struct BatchAdj* adj = nullptr;
  long long prop_gen = 0;
};

// forward/backward of every instance of an FP64 bulk batch (adjoint_kernels.cuh)
struct BatchAdj {
  AdjDev* d_adj = nullptr;              // [n]
  BulkDev<double>* d_inst2 = nullptr;   // [2n]: (adjoint spectrum, forward-chain spectrum) per instance
  void* pool = nullptr;
  double* d_w = nullptr;                // packed fields
  double* d_sc = nullptr;               // [n][ADJ_NSC]
  int2 *wx = nullptr, *wy2 = nullptr, *wy1 = nullptr, *wz = nullptr;
  std::vector<int> px, py2, py1, pz;    // tiles active at reverse step T
  std::vector<size_t> gpart_off;
  size_t gpart_bytes = 0;
  size_t smx = 0, smy = 0, smz = 0;
  int nclos_max = 1;
  long long gen = -1;
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

int reg_tpl(int n) {
  switch (n) {
    case 24: return regk::Cfg<24>::TPL;
    case 32: return regk::Cfg<32>::TPL;
    case 40: return regk::Cfg<40>::TPL;
    case 48: return regk::Cfg<48>::TPL;
    case 64: return regk::Cfg<64>::TPL;
    case 128: return regk::Cfg<128>::TPL;
    default: return regk::Cfg<256>::TPL;
  }
}
template <typename T>
size_t reg_smem(int n) {
  switch (n) {
    case 24: return regk::Layout<T, 24>::bytes;
    case 32: return regk::Layout<T, 32>::bytes;
    case 40: return regk::Layout<T, 40>::bytes;
    case 48: return regk::Layout<T, 48>::bytes;
    case 64: return regk::Layout<T, 64>::bytes;
    case 128: return regk::Layout<T, 128>::bytes;
    default: return regk::Layout<T, 256>::bytes;
  }
}
// cubic grids whose lines run on the register FFT kernels in batches
__host__ __device__ inline bool batch_reg_size(int g) {
  return g == 24 || g == 32 || g == 40 || g == 48 || g == 64 || g == 128 || g == 256;
}

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

// ---------------------------------------------------------------------------
// Persistent sweep of a bulk batch: every line pass of every contour step of
// every instance in one launch.  Instances fall into kernel classes (register
// FFT of one cubic size, or the generic mixed-radix passes); each class gets
// a range of the CTAs in proportion to its point-steps and runs its own
// instantiation of the tile functions, so the classes share the GPU without
// sharing registers; a CTA whose class has run out of items then takes items
// of the class with the most work, which finishes last.  The host lists each class's work items in dependency
// order -- X of node 0, then per step t the Yf, Z, Yi and X passes -- with the
// instances interleaved within each pass; an item is a few tiles of one pass
// of one instance and carries the number of items of that instance listed
// before it.  The CTAs of a class take its items in list order from the
// class's atomic counter, wait (bounded) until their instance has completed
// that many items, run the pass's tile function, and count the item done
// with release semantics.  Every item an item waits for was taken earlier by
// a running CTA that waits only on earlier items, so the sweep cannot
// deadlock, however many of its CTAs are resident; a wait that runs out sets
// the error flag and ends its CTA, and the CTAs waiting on it run out in
// turn.  The tile functions are those of the per-pass kernels, so results are
// bit for bit those of the launch-per-pass schedule.
// item: x instance, y first tile | ntiles << 20, z t << 3 | pass, w items before
// ---------------------------------------------------------------------------
enum { SW_XINIT = 0, SW_YF = 1, SW_Z = 2, SW_YI = 3, SW_X = 4 };
constexpr int kSweepPolls = 1 << 22;

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// one tile of a pass of kernel class N (0: generic mixed-radix passes)
template <typename T, int N>
__device__ __forceinline__ void sweep_tile(const BulkDev<T>* insts, int2 w, int pass, int t, const cplx<T>* tw,
                                           const T* fk, const double* g64, unsigned char* sm) {
  const XAux none{nullptr, nullptr, nullptr};
  if constexpr (N == 0) {
    if (pass == SW_XINIT) xpass_tile<T>(insts, w, tw, 0, XM_INIT, none, sm);
    else if (pass == SW_X) xpass_tile<T>(insts, w, tw, t, XM_STEP, none, sm);
    else strided_tile<T>(insts, w, tw, fk, nullptr, g64, t, pass == SW_YF ? 0 : pass == SW_Z ? 2 : 1, sm);
  } else {
    switch (pass) {
      case SW_XINIT: rx_tile<T, N>(insts, w, tw, 0, XM_INIT, none, sm); break;
      case SW_YF: rs_tile<T, N, 0>(insts, w, tw, fk, nullptr, g64, t, sm); break;
      case SW_Z: rs_tile<T, N, 2>(insts, w, tw, fk, nullptr, g64, t, sm); break;
      case SW_YI: rs_tile<T, N, 1>(insts, w, tw, fk, nullptr, g64, t, sm); break;
      default: rx_tile<T, N>(insts, w, tw, t, XM_STEP, none, sm); break;
    }
  }
}

// One class's share of the sweep: CTAs take that class's items until its
// list is exhausted.  next: the class's item counter, err: the batch's error
// flag, done: items completed per instance; s_q: two shared slots for the
// current and the reserved next item.  Per item, thread 0 waits for the
// item's dependencies and reserves the next item (so the atomic's latency
// overlaps the tiles); thread 32 releases the previous item after the loop's
// barrier, while thread 0 waits.  An item reserved early waits only on items
// taken before it, and a release never waits, so neither can deadlock.
template <typename T, int N>
__device__ __forceinline__ bool sweep_class(const BulkDev<T>* __restrict__ insts, const int4* __restrict__ items,
                                            int nitems, int* next, int* err, int* done_all, int* s_q,
                                            const cplx<T>* __restrict__ tw, const T* __restrict__ fk,
                                            const double* __restrict__ g64, unsigned char* smraw) {
  int pend = -1;                         // instance of the finished, unreleased item
  __syncthreads();                       // every thread has read s_q of the class before
  if (threadIdx.x == 0) s_q[0] = atomicAdd(next, 1);
  for (int par = 0;; par ^= 1) {
    __syncthreads();                     // the previous item's stores are issued; s_q[par] is set
    if (threadIdx.x == 32 && pend >= 0) {
      __threadfence();
      atomicAdd(done_all + pend, 1);
    }
    const int k = s_q[par];
    if (k >= nitems) break;
    const int4 it = items[k];
    const int* done = done_all + it.x;
    bool ok = true;
    if (threadIdx.x == 0) {
      for (int i = 0; ld_acquire_gpu(done) < it.w; ++i) {
        if (i >= kSweepPolls) { ok = false; break; }
        __nanosleep(64);
      }
      if (!ok) atomicOr(err, 1);
      __threadfence();                   // the CTA's loads of the item follow the producers' stores
      s_q[par ^ 1] = ok ? atomicAdd(next, 1) : nitems;
    }
    if (__syncthreads_or(!ok)) return false;
    const int pass = it.z & 7, t = it.z >> 3;
    const int tile0 = it.y & 0xfffff, nt = it.y >> 20;
    for (int j = 0; j < nt; ++j) {
      if (j) __syncthreads();            // the tile function reuses shared memory
      sweep_tile<T, N>(insts, make_int2(it.x, tile0 + j), pass, t, tw, fk, g64, smraw);
    }
    pend = it.x;
  }
  return true;
}

// Kernel class of a CTA range of the sweep: line length n (0: generic), its
// items [off, off + count) and CTAs [cta0, cta0 + ncta).
struct SweepRange {
  int n, off, count, cta0, ncta;
};
constexpr int kMaxSweepClasses = 8;

// run class c of the sweep until its items run out (false: a bounded wait
// ran out)
template <typename T>
__device__ __forceinline__ bool sweep_dispatch(const SweepRange R, int c, const BulkDev<T>* __restrict__ insts,
                                               const int4* __restrict__ items, int* ctl, int* err, int* done,
                                               int* s_q, const cplx<T>* __restrict__ tw, const T* __restrict__ fk,
                                               const double* __restrict__ g64, unsigned char* smraw) {
  const int4* it = items + R.off;
  switch (R.n) {
    case 24: return sweep_class<T, 24>(insts, it, R.count, ctl + c, err, done, s_q, tw, fk, g64, smraw);
    case 32: return sweep_class<T, 32>(insts, it, R.count, ctl + c, err, done, s_q, tw, fk, g64, smraw);
    case 40: return sweep_class<T, 40>(insts, it, R.count, ctl + c, err, done, s_q, tw, fk, g64, smraw);
    case 48: return sweep_class<T, 48>(insts, it, R.count, ctl + c, err, done, s_q, tw, fk, g64, smraw);
    case 64: return sweep_class<T, 64>(insts, it, R.count, ctl + c, err, done, s_q, tw, fk, g64, smraw);
    case 128: return sweep_class<T, 128>(insts, it, R.count, ctl + c, err, done, s_q, tw, fk, g64, smraw);
    case 256: return sweep_class<T, 256>(insts, it, R.count, ctl + c, err, done, s_q, tw, fk, g64, smraw);
    default: return sweep_class<T, 0>(insts, it, R.count, ctl + c, err, done, s_q, tw, fk, g64, smraw);
  }
}

// One launch for every class: the CTAs of range c work on class c only, so
// each class keeps its share of the GPU whatever the others do; each range
// runs the class's own instantiation of the loop (inlined).  ctl: [class
// counters][error flag][items done per instance].
template <typename T>
__global__ void __launch_bounds__(BULK_THREADS, 2)
k_batch_sweep(const BulkDev<T>* __restrict__ insts, const int4* __restrict__ items,
              const SweepRange* __restrict__ ranges, int ncls, int help, int* __restrict__ ctl,
              const cplx<T>* __restrict__ tw, const T* __restrict__ fk, const double* __restrict__ g64) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ int s_q[2];
  int c = 0;
  while (c + 1 < ncls && (int)blockIdx.x >= ranges[c + 1].cta0) ++c;
  int* err = ctl + ncls;
  int* done = err + 1;
  // the CTA's own class, then (once its class has run out of items) the class
  // with the most work, which finishes last
  if (!sweep_dispatch<T>(ranges[c], c, insts, items, ctl, err, done, s_q, tw, fk, g64, smraw)) return;
  if (c != help) sweep_dispatch<T>(ranges[help], help, insts, items, ctl, err, done, s_q, tw, fk, g64, smraw);
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
    if (q.nblocks) return berr(b, ADSCF_E_ARG, "instance " + std::to_string(i) + ": batches take diblock chains");
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
    b->max_slots = std::max(b->max_slots, b->slots[i]);
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
  if constexpr (sizeof(T) == 8) b->hI64.assign(I.begin(), I.end());
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

  // work lists per kernel class, instances by descending Ns: the tiles of the
  // instances still on their contour at step t are a prefix
  std::vector<int> ord(n);
  for (int i = 0; i < n; ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int c2) { return b->ns[a] > b->ns[c2]; });
  auto class_of = [&](int i) {
    const BulkDev<T>& d = I[i];
    const int g = d.gx;
    return (d.gy == g && d.gz == g && batch_reg_size(g)) ? g : 0;
  };
  for (int cn : {24, 32, 40, 48, 64, 128, 256, 0}) {
    adscf_batch::PassClass C;
    C.n = cn;
    std::vector<int2> wx, wy, wz;
    std::vector<int> tx(n, 0), ty(n, 0), tz(n, 0);
    for (int i : ord) {
      if (class_of(i) != cn) continue;
      const BulkDev<T>& d = I[i];
      const int lx = cn ? BULK_THREADS / reg_tpl(cn) : d.px.lpc;
      const int ly = cn ? BULK_THREADS / reg_tpl(cn) : d.py.lpc;
      const int lz = cn ? BULK_THREADS / reg_tpl(cn) : d.pz.lpc;
      tx[i] = (d.gy * d.gz + lx - 1) / lx;
      ty[i] = (d.gx * d.gz + ly - 1) / ly;
      tz[i] = (d.gx * d.gy + lz - 1) / lz;
      for (int k = 0; k < tx[i]; ++k) wx.push_back(make_int2(i, k));
      for (int k = 0; k < ty[i]; ++k) wy.push_back(make_int2(i, k));
      for (int k = 0; k < tz[i]; ++k) wz.push_back(make_int2(i, k));
      if (cn) {
        C.smx = C.smy = C.smz = reg_smem<T>(cn);
      } else {
        C.smx = std::max(C.smx, bulkhost::plan_smem<T>(d.px));
        C.smy = std::max(C.smy, bulkhost::plan_smem<T>(d.py));
        C.smz = std::max(C.smz, bulkhost::plan_smem_z<T>(d.pz));
      }
    }
    if (wx.empty()) continue;
    C.px.assign(b->maxns + 1, 0); C.py.assign(b->maxns + 1, 0); C.pz.assign(b->maxns + 1, 0);
    for (int t = 0; t <= b->maxns; ++t)
      for (int i = 0; i < n; ++i)
        if (class_of(i) == cn && b->ns[i] >= t) { C.px[t] += tx[i]; C.py[t] += ty[i]; C.pz[t] += tz[i]; }
    BK(cudaMalloc(&C.wx, wx.size() * sizeof(int2)));
    BK(cudaMalloc(&C.wy, wy.size() * sizeof(int2)));
    BK(cudaMalloc(&C.wz, wz.size() * sizeof(int2)));
    b->cls.push_back(C);   // owns the device lists from here (freed on destroy)
    BK(cudaMemcpyAsync(C.wx, wx.data(), wx.size() * sizeof(int2), cudaMemcpyHostToDevice, b->stream));
    BK(cudaMemcpyAsync(C.wy, wy.data(), wy.size() * sizeof(int2), cudaMemcpyHostToDevice, b->stream));
    BK(cudaMemcpyAsync(C.wz, wz.data(), wz.size() * sizeof(int2), cudaMemcpyHostToDevice, b->stream));
  }
  // items of the persistent sweeps (k_batch_sweep), class by class: per step
  // and pass, the class's instances still on their contour in the same order
  // as the work lists
  {
    if (const char* e = std::getenv("ADSCF_SWEEP_TILES")) b->sweep_tiles = std::max(1, std::min(64, std::atoi(e)));
    if (const char* e = std::getenv("ADSCF_BATCH_SWEEP")) b->sweep = std::atoi(e) != 0;
    std::vector<int> tx(n), ty(n), tz(n), before(n, 0);
    for (int i = 0; i < n; ++i) {
      const BulkDev<T>& d = I[i];
      const int cn = class_of(i);
      const int lx = cn ? BULK_THREADS / reg_tpl(cn) : d.px.lpc;
      const int ly = cn ? BULK_THREADS / reg_tpl(cn) : d.py.lpc;
      const int lz = cn ? BULK_THREADS / reg_tpl(cn) : d.pz.lpc;
      tx[i] = (d.gy * d.gz + lx - 1) / lx;
      ty[i] = (d.gx * d.gz + ly - 1) / ly;
      tz[i] = (d.gx * d.gy + lz - 1) / lz;
    }
    std::vector<int4> items;
    auto add = [&](int i, int ntiles, int pass, int t) {
      int k = 0;
      for (int t0 = 0; t0 < ntiles; t0 += b->sweep_tiles, ++k) {
        const int nt = std::min(b->sweep_tiles, ntiles - t0);
        items.push_back(make_int4(i, t0 | (nt << 20), (t << 3) | pass, before[i]));
      }
      before[i] += k;
    };
    for (const auto& C : b->cls) {
      adscf_batch::SweepClass W;
      W.n = C.n;
      W.off = (int)items.size();
      for (int i : ord)
        if (class_of(i) == C.n) add(i, tx[i], SW_XINIT, 0);
      for (int t = 1; t <= b->maxns; ++t)
        for (int pass : {SW_YF, SW_Z, SW_YI, SW_X})
          for (int i : ord)
            if (class_of(i) == C.n && b->ns[i] >= t)
              add(i, pass == SW_X ? tx[i] : pass == SW_Z ? tz[i] : ty[i], pass, t);
      W.count = (int)items.size() - W.off;
      b->sw.push_back(W);
    }
    BK(cudaMalloc(&b->d_items, items.size() * sizeof(int4)));
    BK(cudaMemcpyAsync(b->d_items, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice, b->stream));
    const size_t nctl = b->sw.size() + 1 + (size_t)n;
    BK(cudaMalloc(&b->d_ctl, nctl * sizeof(int)));
    BK(cudaMemsetAsync(b->d_ctl, 0, nctl * sizeof(int), b->stream));
  }
  size_t smmax = 0;
  for (const auto& C : b->cls) smmax = std::max(smmax, std::max(C.smx, std::max(C.smy, C.smz)));
  int optin = 0;
  BK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->dev));
  if (smmax > (size_t)optin) return berr(b, ADSCF_E_ARG, "grid line too long for shared memory");
  // this translation unit's instances of the pass kernels (own device module)
  BK(cudaFuncSetAttribute(k_bulk_xpass<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
  BK(cudaFuncSetAttribute(k_bulk_strided<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
#define ADSCF_BATTR(NN)                                                                                   \
  BK(cudaFuncSetAttribute(k_rx<T, NN>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));              \
  BK(cudaFuncSetAttribute(k_rs<T, NN, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));           \
  BK(cudaFuncSetAttribute(k_rs<T, NN, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));           \
  BK(cudaFuncSetAttribute(k_rs<T, NN, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
  ADSCF_BATTR(24) ADSCF_BATTR(32) ADSCF_BATTR(40) ADSCF_BATTR(48) ADSCF_BATTR(64) ADSCF_BATTR(128)
  ADSCF_BATTR(256)
#undef ADSCF_BATTR
  {  // persistent sweep: each class's share of the resident CTAs in proportion
     // to its point-steps (at least one CTA); the kernel's static shared
     // memory counts against the opt-in limit
    const int ncls = (int)b->sw.size();
    if (ncls > kMaxSweepClasses) b->sweep = false;
    int nsm = 0, occ = 0;
    BK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, b->dev));
    // two resident CTAs per SM (128 registers): at three, the register-FFT
    // classes spill and the C5 sweep ran 4% slower
    const auto kern = k_batch_sweep<T>;
    cudaFuncAttributes fa{};
    BK(cudaFuncGetAttributes(&fa, kern));
    b->sweep_smem = std::max<size_t>(smmax, 16);
    if (b->sweep_smem + fa.sharedSizeBytes <= (size_t)optin) {
      BK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->sweep_smem));
      BK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, BULK_THREADS, b->sweep_smem));
    }
    if (occ < 1) b->sweep = false;
    const int slots = std::max(1, occ) * nsm;
    double total = 0.0;
    std::vector<double> work(ncls, 0.0);
    for (int c = 0; c < ncls; ++c) {
      for (int i = 0; i < n; ++i)
        if (class_of(i) == b->sw[c].n) work[c] += (double)I[i].npts * b->ns[i];
      total += work[c];
    }
    std::vector<SweepRange> rg(std::max(ncls, 1));
    int cta = 0;
    for (int c = 0; c < ncls; ++c) {
      const int share = std::max(1, (int)(slots * (total > 0 ? work[c] / total : 1.0 / ncls)));
      rg[c] = SweepRange{b->sw[c].n, b->sw[c].off, b->sw[c].count, cta, share};
      cta += share;
    }
    b->sweep_grid = cta;
    for (int c = 1; c < ncls; ++c)
      if (work[c] > work[b->sweep_help]) b->sweep_help = c;
    BK(cudaMalloc(&b->d_ranges, rg.size() * sizeof(SweepRange)));
    BK(cudaMemcpyAsync(b->d_ranges, rg.data(), rg.size() * sizeof(SweepRange), cudaMemcpyHostToDevice, b->stream));
  }
  BK(cudaStreamSynchronize(b->stream));
  return ADSCF_OK;
}

int check_film(const adscf_params& q, int prec, int geom, std::string& why) {
  if (q.geometry != geom) { why = "one geometry for the whole batch"; return ADSCF_E_ARG; }
  if (q.precision != prec) { why = "one precision for the whole batch"; return ADSCF_E_ARG; }
  if (q.gx != 1 || q.gy != 1) { why = "batched films are one line (gx = gy = 1)"; return ADSCF_E_ARG; }
  if (q.gz < 2 || !q.dz) { why = "films need gz >= 2 and dz"; return ADSCF_E_ARG; }
  if (!(q.sizex > 0 && q.sizey > 0 && q.sizez > 0)) { why = "box size"; return ADSCF_E_ARG; }
  if (!q.dss && !(q.ds > 0)) { why = "ds or dss"; return ADSCF_E_ARG; }
  if (q.mixing_type < 1 || q.mixing_type > 3) { why = "mixing_type"; return ADSCF_E_ARG; }
  if (q.mixing_type == 3 && (q.mixing_dim < 1 || q.mixing_dim > SCF_MAX_HIST)) { why = "mixing_dim"; return ADSCF_E_ARG; }
  if (q.ensemble != 1 && q.ensemble != 2) { why = "ensemble"; return ADSCF_E_ARG; }
  if (geom == ADSCF_BRUSH && !q.graft) { why = "brush needs the grafting distribution"; return ADSCF_E_ARG; }
  return ADSCF_OK;
}

// Film batch: one line per film; tables (coefficients, weights, schedules,
// wall potentials) in one FP64 array, propagators and SCF state in the pool.
// shared memory of k_film1d_chains_sm: q, gam and the eliminated right-hand
// side, and the FP32 field of both types for FP32 sweeps
size_t film_sweep_smem(int zcap, int W, size_t es) {
  return 3 * (size_t)zcap * W * es + (es == 4 ? 2 * (size_t)zcap * W * sizeof(float) : 0);
}

int build_film(adscf_batch* b) {
  const int n = b->n;
  const int geom = b->p[0].geometry;
  const bool brush = geom == ADSCF_BRUSH;
  b->film = true;
  b->ntypes = brush ? 1 : 2;
  const int nt = b->ntypes;
  std::vector<FilmTables> tb(n);
  std::vector<int> na(n), t64(n);
  b->ns.resize(n); b->npts.resize(n); b->slots.resize(n); b->foff.assign(n + 1, 0);
  b->hS.resize(n);
  for (int i = 0; i < n; ++i) {
    const adscf_params& q = b->p[i];
    std::string why;
    if (check_film(q, b->prec, geom, why)) return berr(b, ADSCF_E_ARG, "instance " + std::to_string(i) + ": " + why);
    int ns, a;
    if (q.dss) {
      ns = q.ns;
      a = brush ? q.ns : q.n_a;
    } else {
      a = nint_b(q.block_length[0] / q.ds);
      ns = a + (brush ? 0 : nint_b(q.block_length[1] / q.ds));
    }
    if (ns < 1 || a < 0 || a > ns) return berr(b, ADSCF_E_ARG, "instance " + std::to_string(i) + ": contour");
    if (film_tables(q, ns, a, tb[i], why)) return berr(b, ADSCF_E_ARG, "instance " + std::to_string(i) + ": " + why);
    b->ns[i] = ns;
    na[i] = a;
    b->npts[i] = q.gz + 1;
    b->slots[i] = q.mixing_type == 3 ? q.mixing_dim + 1 : 2;
    b->max_slots = std::max(b->max_slots, b->slots[i]);
    b->foff[i + 1] = b->foff[i] + (size_t)nt * b->npts[i];
    b->maxns = std::max(b->maxns, ns);
    t64[i] = film_sweep_fp64(b->prec, tb[i].max_ratio) ? 1 : 0;
  }
  // FP64 tables: al, be, ga, wz [npts]; dss, wA, wB [ns+1]; ext [nt][npts]; graft [npts]
  std::vector<double> tab;
  struct TOff { size_t al, be, ga, wz, dss, wA, wB, ext, graft; };
  std::vector<TOff> to(n);
  auto put = [&](const double* v, size_t cnt) {
    const size_t o = tab.size();
    tab.insert(tab.end(), v, v + cnt);
    tab.resize((tab.size() + 3) & ~size_t(3));   // 32-byte granules
    return o;
  };
  for (int i = 0; i < n; ++i) {
    const size_t np = b->npts[i], ns1 = b->ns[i] + 1;
    to[i].al = put(tb[i].al.data(), np); to[i].be = put(tb[i].be.data(), np);
    to[i].ga = put(tb[i].ga.data(), np); to[i].wz = put(tb[i].wz.data(), np);
    to[i].dss = put(tb[i].dss.data(), ns1); to[i].wA = put(tb[i].wA.data(), ns1);
    to[i].wB = put(tb[i].wB.data(), ns1);
    to[i].ext = b->p[i].ext_potential ? put(b->p[i].ext_potential, (size_t)nt * np) : SIZE_MAX;
    to[i].graft = brush ? put(b->p[i].graft, np) : SIZE_MAX;
  }
  BK(cudaMalloc(&b->d_fk, tab.size() * sizeof(double)));
  BK(cudaMemcpyAsync(b->d_fk, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  const double* dtab = static_cast<const double*>(b->d_fk);
  // FP32 mesh factors of the FP32 sweeps: al, be, ga [npts] per film
  std::vector<float> tabf;
  std::vector<size_t> tof(n, SIZE_MAX);
  for (int i = 0; i < n; ++i) {
    if (t64[i]) continue;
    tof[i] = tabf.size();
    for (const std::vector<double>* v : {&tb[i].al, &tb[i].be, &tb[i].ga})
      for (size_t j = 0; j < b->npts[i]; ++j) tabf.push_back((float)(*v)[j]);
  }
  BK(cudaMalloc(&b->d_tabf, std::max<size_t>(1, tabf.size()) * sizeof(float)));
  if (!tabf.empty())
    BK(cudaMemcpyAsync(b->d_tabf, tabf.data(), tabf.size() * sizeof(float), cudaMemcpyHostToDevice, b->stream));
  // pool
  Carve c;
  struct Off { size_t q, qd, gam, dist, dens, hx, hr, qpart, part, gram, coef; };
  std::vector<Off> o(n);
  for (int i = 0; i < n; ++i) {
    const size_t np = b->npts[i], es = t64[i] ? 8 : 4;
    o[i].q = c.take((size_t)(b->ns[i] + 1) * np * es);
    o[i].qd = c.take((size_t)(b->ns[i] + 1) * np * es);
    o[i].gam = c.take(2 * np * es);
    o[i].dist = c.take((size_t)nt * np * sizeof(double));
    o[i].dens = c.take((size_t)nt * np * sizeof(double));
    o[i].hx = c.take((size_t)b->slots[i] * nt * np * sizeof(double));
    o[i].hr = c.take((size_t)b->slots[i] * nt * np * sizeof(double));
    o[i].qpart = c.take(sizeof(double));
    o[i].part = c.take(NPART * sizeof(double));
    o[i].gram = c.take(SCF_MAX_SLOTS * SCF_MAX_SLOTS * sizeof(double));
    o[i].coef = c.take(2 * SCF_MAX_SLOTS * sizeof(double));
  }
  const size_t o_res = c.take((size_t)n * R_COUNT * sizeof(double));
  const size_t o_iter = c.take((size_t)n * sizeof(int));
  const size_t o_err = c.take(sizeof(int));
  if (cudaMalloc(&b->pool, c.off) != cudaSuccess) {
    cudaGetLastError();
    return berr(b, ADSCF_E_OOM, "batch pool of " + std::to_string(c.off >> 20) + " MiB");
  }
  unsigned char* base = static_cast<unsigned char*>(b->pool);
  BK(cudaMemsetAsync(b->pool, 0, c.off, b->stream));
  b->d_resall = reinterpret_cast<double*>(base + o_res);
  b->d_iterall = reinterpret_cast<int*>(base + o_iter);
  b->d_err = reinterpret_cast<int*>(base + o_err);
  std::vector<FilmDev<float>> f32(n);
  std::vector<FilmDev<double>> f64(n);
  std::vector<int> l32, l64;
  for (int i = 0; i < n; ++i) {
    const adscf_params& q = b->p[i];
    const size_t np = b->npts[i];
    auto fill = [&](auto& D) {
      using T = std::remove_reference_t<decltype(*D.q)>;
      D.gx = 1; D.gy = 1; D.gz = q.gz;
      D.nlines = 1; D.npts = (int)np;
      D.ns = b->ns[i]; D.na = na[i];
      D.ntypes = nt; D.brush = brush; D.single = 0; D.span = q.int_span;
      D.alpha = dtab + to[i].al; D.beta = dtab + to[i].be; D.gamma = dtab + to[i].ga;
      D.dss = dtab + to[i].dss; D.wA = dtab + to[i].wA; D.wB = dtab + to[i].wB;
      D.wz = dtab + to[i].wz;
      D.graft = brush ? dtab + to[i].graft : nullptr;
      D.q = reinterpret_cast<T*>(base + o[i].q);
      D.qd = reinterpret_cast<T*>(base + o[i].qd);
      D.gam = reinterpret_cast<T*>(base + o[i].gam);
      D.dist = reinterpret_cast<double*>(base + o[i].dist);
      D.qpart = reinterpret_cast<double*>(base + o[i].qpart);
      D.err = b->d_err;
      D.dx = q.sizex; D.dy = q.sizey;
      D.w1 = nullptr;
      D.alf = tof[i] == SIZE_MAX ? nullptr : b->d_tabf + tof[i];
      D.bef = tof[i] == SIZE_MAX ? nullptr : b->d_tabf + tof[i] + np;
      D.gaf = tof[i] == SIZE_MAX ? nullptr : b->d_tabf + tof[i] + 2 * np;
      D.wf = nullptr;   // the batch sweep keeps the FP32 field in shared memory
    };
    if (t64[i]) { fill(f64[i]); l64.push_back(i); }
    else { fill(f32[i]); l32.push_back(i); }
    ScfDev& S = b->hS[i];
    S = ScfDev{};
    const double volume = q.sizex * q.sizey * q.sizez;
    S.npts = (int)np; S.ntypes = nt; S.plane = 1; S.nplanes = q.gz + 1; S.wall_mask = 1;
    S.dvol = volume / (double)q.gz;
    S.wz = dtab + to[i].wz;
    S.ext = b->p[i].ext_potential ? dtab + to[i].ext : nullptr;
    S.kappa = q.kappa; S.chi = q.chi;
    S.v0 = q.monomer_volume[0] != 0 ? q.monomer_volume[0] : 1.0;
    S.v1 = q.monomer_volume[1] != 0 ? q.monomer_volume[1] : 1.0;
    S.ww = q.ww; S.homopolymer = brush;
    S.ensemble = q.ensemble; S.rho = q.rho; S.mu = q.mu; S.volume = volume;
    S.chain_len = tb[i].chain_len;
    S.dist = reinterpret_cast<double*>(base + o[i].dist);
    S.dens = reinterpret_cast<double*>(base + o[i].dens);
    S.hx = reinterpret_cast<double*>(base + o[i].hx);
    S.hr = reinterpret_cast<double*>(base + o[i].hr);
    S.slots = b->slots[i];
    S.mixing_type = q.mixing_type;
    S.warm = q.warm_iters > q.mixing_dim ? q.warm_iters : q.mixing_dim;
    S.lambda = q.lambda;
    S.lam_warm = q.lam_warm > 0 ? q.lam_warm : 1.0e-3;
    S.qpart = reinterpret_cast<double*>(base + o[i].qpart); S.nqpart = 1; S.qscale = 1.0;
    S.part = reinterpret_cast<double*>(base + o[i].part); S.npart_blocks = 1;
    S.gram = reinterpret_cast<double*>(base + o[i].gram);
    S.coef = reinterpret_cast<double*>(base + o[i].coef);
    S.iter = b->d_iterall + i;
    S.res = b->d_resall + (size_t)i * R_COUNT;
    S.mixE = nullptr;
    S.mixds = 0.0;
  }
  // longest contours first: a warp's threads then walk similar step counts
  auto by_work = [&](int a, int c2) {
    return (long long)b->ns[a] * b->npts[a] > (long long)b->ns[c2] * b->npts[c2];
  };
  std::stable_sort(l32.begin(), l32.end(), by_work);
  std::stable_sort(l64.begin(), l64.end(), by_work);
  long long max_npts = 0;
  for (int i = 0; i < n; ++i) max_npts = std::max<long long>(max_npts, b->npts[i]);
  b->film_cl_threads = closure_threads(max_npts);
  b->n32 = (int)l32.size();
  b->n64 = (int)l64.size();
  // layout of the shared-memory sweeps: one thread per (film, chain) runs a
  // serial recurrence, so the first `per_warp` lanes of each warp work and
  // a block holds `warps` warps: W = warps * per_warp lines share the
  // block's shared memory.  ADSCF_FILM_LANES / ADSCF_FILM_WARPS override.
  {
    int optin = 0;
    BK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->dev));
    b->film_per_warp = 2;
    b->film_warps = 2;
    if (const char* e = std::getenv("ADSCF_FILM_LANES")) b->film_per_warp = std::max(1, std::min(32, std::atoi(e)));
    if (const char* e = std::getenv("ADSCF_FILM_WARPS")) b->film_warps = std::max(1, std::min(8, std::atoi(e)));
    auto lanes = [&](const std::vector<int>& l, size_t es, int& zcap, int& W) {
      zcap = 0;
      for (int i : l) zcap = std::max(zcap, b->npts[i]);
      W = b->film_warps * b->film_per_warp;
      // fewer warps while a block's lines do not fit (W = 0: global sweep)
      int warps = b->film_warps;
      while (warps > 0 && film_sweep_smem(zcap, warps * b->film_per_warp, es) > (size_t)optin) --warps;
      W = warps * b->film_per_warp;
      if (warps == 0) W = 0;
    };
    lanes(l32, sizeof(float), b->zcap32, b->lanes32);
    lanes(l64, sizeof(double), b->zcap64, b->lanes64);
    BK(cudaFuncSetAttribute(k_film1d_chains_sm<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    BK(cudaFuncSetAttribute(k_film1d_chains_sm<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
  }
  BK(cudaMalloc(&b->d_f32, n * sizeof(FilmDev<float>)));
  BK(cudaMalloc(&b->d_f64, n * sizeof(FilmDev<double>)));
  BK(cudaMemcpyAsync(b->d_f32, f32.data(), n * sizeof(FilmDev<float>), cudaMemcpyHostToDevice, b->stream));
  BK(cudaMemcpyAsync(b->d_f64, f64.data(), n * sizeof(FilmDev<double>), cudaMemcpyHostToDevice, b->stream));
  BK(cudaMalloc(&b->d_list32, std::max<size_t>(1, l32.size()) * sizeof(int)));
  BK(cudaMalloc(&b->d_list64, std::max<size_t>(1, l64.size()) * sizeof(int)));
  if (!l32.empty())
    BK(cudaMemcpyAsync(b->d_list32, l32.data(), l32.size() * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  {  // (film, chain) items of the warp sweep, in the order of l32
    std::vector<int> items;
    for (int f : l32) { items.push_back(f << 1); items.push_back((f << 1) | 1); }
    BK(cudaMalloc(&b->d_items32, std::max<size_t>(1, items.size()) * sizeof(int)));
    if (!items.empty())
      BK(cudaMemcpyAsync(b->d_items32, items.data(), items.size() * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  }
  if (!l64.empty())
    BK(cudaMemcpyAsync(b->d_list64, l64.data(), l64.size() * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  BK(cudaMalloc(&b->d_S, n * sizeof(ScfDev)));
  BK(cudaMemcpyAsync(b->d_S, b->hS.data(), n * sizeof(ScfDev), cudaMemcpyHostToDevice, b->stream));
  std::vector<int> ones(n, 1);
  BK(cudaMemcpyAsync(b->d_iterall, ones.data(), n * sizeof(int), cudaMemcpyHostToDevice, b->stream));
  b->clos_grid = 1;
  b->mix_grid = 1;
  BK(cudaStreamSynchronize(b->stream));
  return ADSCF_OK;
}

int enqueue_film(adscf_batch* b) {
  cudaStream_t s = b->stream;
  const FilmDev<float>* f32 = static_cast<const FilmDev<float>*>(b->d_f32);
  const FilmDev<double>* f64 = static_cast<const FilmDev<double>*>(b->d_f64);
  const int pw = b->film_per_warp;
  if (b->n32 && b->zcap32 <= 32 * kFilmWarpM) {
    // one warp per (film, chain), longest contours first
    k_film1d_warp_b<<<(2 * b->n32 + 3) / 4, 128, 0, s>>>(f32, b->d_S, b->d_items32, 2 * b->n32);
  } else if (b->n32 && b->lanes32) {
    const int W = b->lanes32;
    k_film1d_chains_sm<float><<<dim3((b->n32 + W - 1) / W, 2), 32 * (W / pw),
                                film_sweep_smem(b->zcap32, W, sizeof(float)), s>>>(
        f32, b->d_S, b->d_list32, b->n32, b->zcap32, pw);
  } else if (b->n32) {
    k_film1d_chains_b<float><<<dim3((b->n32 + FILM_THREADS - 1) / FILM_THREADS, 2), FILM_THREADS, 0, s>>>(
        f32, b->d_S, b->d_list32, b->n32);
  }
  if (b->n64 && b->lanes64) {
    const int W = b->lanes64;
    k_film1d_chains_sm<double><<<dim3((b->n64 + W - 1) / W, 2), 32 * (W / pw),
                                 film_sweep_smem(b->zcap64, W, sizeof(double)), s>>>(
        f64, b->d_S, b->d_list64, b->n64, b->zcap64, pw);
  } else if (b->n64) {
    k_film1d_chains_b<double><<<dim3((b->n64 + FILM_THREADS - 1) / FILM_THREADS, 2), FILM_THREADS, 0, s>>>(
        f64, b->d_S, b->d_list64, b->n64);
  }
  // one-line films: blocks of 128 points, twice as many resident films as
  // with 256 (a longer line takes its points in passes)
  if (b->n32) k_film_contour_b<float><<<b->n32, 128, 0, s>>>(f32, b->d_list32);
  if (b->n64) k_film_contour_b<double><<<b->n64, 256, 0, s>>>(f64, b->d_list64);
  launch_closure_b(b->d_S, b->max_slots, CL_MEANFIELD | CL_MIXDOTS, dim3(1, b->n), s, b->film_cl_threads);
  // each partial is summed by one warp whatever the block size
  k_solve_b<<<b->n, b->film_cl_threads, 0, s>>>(b->d_S, 1, 1);
  k_mix_b<float><<<dim3(1, b->n), SCF_THREADS, 0, s>>>(b->d_S, 1);
  BK(cudaGetLastError());
  return ADSCF_OK;
}

template <typename T>
int enqueue_propagation(adscf_batch* b) {
  const BulkDev<T>* d = static_cast<const BulkDev<T>*>(b->d_inst);
  const cplx<T>* tw = static_cast<const cplx<T>*>(b->d_tw);
  const T* fk = static_cast<const T*>(b->d_fk);
  cudaStream_t s = b->stream;
  const XAux none{nullptr, nullptr, nullptr};
  const double* g64 = b->d_g64;
  // one launch per kernel class and pass; a class with no instance left on
  // its contour at step t launches nothing
  auto xpass = [&](const adscf_batch::PassClass& C, int grid, int t, int mode) {
    if (grid <= 0) return;
    switch (C.n) {
      case 24: k_rx<T, 24><<<grid, BULK_THREADS, C.smx, s>>>(d, C.wx, tw, t, mode, none); break;
      case 40: k_rx<T, 40><<<grid, BULK_THREADS, C.smx, s>>>(d, C.wx, tw, t, mode, none); break;
      case 48: k_rx<T, 48><<<grid, BULK_THREADS, C.smx, s>>>(d, C.wx, tw, t, mode, none); break;
      case 32: k_rx<T, 32><<<grid, BULK_THREADS, C.smx, s>>>(d, C.wx, tw, t, mode, none); break;
      case 64: k_rx<T, 64><<<grid, BULK_THREADS, C.smx, s>>>(d, C.wx, tw, t, mode, none); break;
      case 128: k_rx<T, 128><<<grid, BULK_THREADS, C.smx, s>>>(d, C.wx, tw, t, mode, none); break;
      case 256: k_rx<T, 256><<<grid, BULK_THREADS, C.smx, s>>>(d, C.wx, tw, t, mode, none); break;
      default: k_bulk_xpass<T><<<grid, BULK_THREADS, C.smx, s>>>(d, C.wx, tw, t, mode, none);
    }
  };
  if (b->sweep) {
    const int ncls = (int)b->sw.size();
    BK(cudaMemsetAsync(b->d_ctl, 0, (ncls + 1 + (size_t)b->n) * sizeof(int), s));
    k_batch_sweep<T><<<b->sweep_grid, BULK_THREADS, b->sweep_smem, s>>>(
        d, b->d_items, static_cast<const SweepRange*>(b->d_ranges), ncls, b->sweep_help, b->d_ctl, tw, fk, g64);
    k_bulk_contour<T><<<dim3(b->cont_blocks, b->n), BULK_THREADS, 0, s>>>(d);
    BK(cudaGetLastError());
    return ADSCF_OK;
  }
  auto spass = [&](const adscf_batch::PassClass& C, int t, int kind) {
    const bool z = kind == 2;
    const int grid = z ? C.pz[t] : C.py[t];
    const int2* w = z ? C.wz : C.wy;
    const size_t sm = z ? C.smz : C.smy;
    if (grid <= 0) return;
#define ADSCF_BS(NN)                                                                              \
  if (kind == 0) k_rs<T, NN, 0><<<grid, BULK_THREADS, sm, s>>>(d, w, tw, fk, nullptr, g64, t);     \
  else if (kind == 1) k_rs<T, NN, 1><<<grid, BULK_THREADS, sm, s>>>(d, w, tw, fk, nullptr, g64, t); \
  else k_rs<T, NN, 2><<<grid, BULK_THREADS, sm, s>>>(d, w, tw, fk, nullptr, g64, t);
    switch (C.n) {
      case 24: ADSCF_BS(24) break;
      case 40: ADSCF_BS(40) break;
      case 48: ADSCF_BS(48) break;
      case 32: ADSCF_BS(32) break;
      case 64: ADSCF_BS(64) break;
      case 128: ADSCF_BS(128) break;
      case 256: ADSCF_BS(256) break;
      default: k_bulk_strided<T><<<grid, BULK_THREADS, sm, s>>>(d, w, tw, fk, nullptr, g64, t, kind);
    }
#undef ADSCF_BS
  };
  for (const auto& C : b->cls) xpass(C, C.px[0], 0, XM_INIT);
  for (int t = 1; t <= b->maxns; ++t) {
    for (const auto& C : b->cls) spass(C, t, 0);
    for (const auto& C : b->cls) spass(C, t, 2);
    for (const auto& C : b->cls) spass(C, t, 1);
    for (const auto& C : b->cls) xpass(C, C.px[t], t, XM_STEP);
  }
  k_bulk_contour<T><<<dim3(b->cont_blocks, b->n), BULK_THREADS, 0, s>>>(d);
  BK(cudaGetLastError());
  return ADSCF_OK;
}

template <typename T>
int enqueue_iteration(adscf_batch* b) {
  int rc = enqueue_propagation<T>(b);
  if (rc) return rc;
  cudaStream_t s = b->stream;
  launch_closure_b(b->d_S, b->max_slots, CL_MEANFIELD | CL_MIXDOTS, dim3(b->clos_grid, b->n), s);
  k_solve_b<<<b->n, SOLVE_THREADS, 0, s>>>(b->d_S, 1, 1);
  k_mix_b<T><<<dim3(b->mix_grid, b->n), SCF_THREADS, 0, s>>>(b->d_S, b->mix_grid);
  BK(cudaGetLastError());
  return ADSCF_OK;
}

int enqueue(adscf_batch* b) {
  if (b->film) return enqueue_film(b);
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
  if (b->d_ctl) {   // a bounded wait of a persistent sweep expired
    int f = 0;
    int* err = b->d_ctl + b->sw.size();
    BK(cudaMemcpyAsync(&f, err, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    if (f) {
      BK(cudaMemsetAsync(err, 0, sizeof(int), b->stream));
      return berr(b, ADSCF_E_TIMEOUT, "a bounded wait of the persistent sweep expired");
    }
  }
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

// zero-pivot flag of the film sweeps since the last check (cleared on read)
int check_pivot(adscf_batch* b) {
  if (!b->d_err) return ADSCF_OK;
  int e = 0;
  BK(cudaMemcpyAsync(&e, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  BK(cudaStreamSynchronize(b->stream));
  if (e) {
    BK(cudaMemsetAsync(b->d_err, 0, sizeof(int), b->stream));
    return berr(b, ADSCF_E_PIVOT, "zero pivot in a tridiagonal sweep (TriDiag Error)");
  }
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
    const size_t nv = (size_t)S.ntypes * S.npts;
    BK(cudaMemsetAsync(S.hx, 0, (size_t)S.slots * nv * sizeof(double), b->stream));
    BK(cudaMemsetAsync(S.hr, 0, (size_t)S.slots * nv * sizeof(double), b->stream));
    BK(cudaMemsetAsync(S.gram, 0, SCF_MAX_SLOTS * SCF_MAX_SLOTS * sizeof(double), b->stream));
    double* x1 = S.hx + (size_t)(1 % S.slots) * nv;
    BK(cudaMemcpyAsync(x1, b->h_pinned + b->foff[i], nv * sizeof(double), cudaMemcpyHostToDevice, b->stream));
    if (b->film) continue;
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
    const size_t nv = (size_t)S.ntypes * S.npts;
    const double* src = fields ? S.hx + (size_t)(it[i] % S.slots) * nv : S.dens;
    BK(cudaMemcpyAsync(b->h_pinned + b->foff[i], src, nv * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  }
  BK(cudaStreamSynchronize(b->stream));
  std::memcpy(out, b->h_pinned, tot * sizeof(double));
  return ADSCF_OK;
}

size_t plan_bytes_d(const Plan1D& P, int nbuf) {
  const size_t twn = (P.n + 1) & ~1;
  return (twn + (size_t)nbuf * P.lpc * P.ld) * sizeof(double2);
}

int batch_adj_setup(adscf_batch* b) {
  if (b->adj) return ADSCF_OK;
  BatchAdj* a = new (std::nothrow) BatchAdj();
  if (!a) return berr(b, ADSCF_E_OOM, "batch adjoint state");
  b->adj = a;
  const int n = b->n;
  // pool: per instance forward-chain spectrum, seeds, closure and stress partials
  Carve c;
  struct Off { size_t sf, bb, part, gpart; };
  std::vector<Off> o(n);
  std::vector<int> nclos(n), nzt(n);
  for (int i = 0; i < n; ++i) {
    const BulkDev<double>& I = b->hI64[i];
    const size_t np = I.npts;
    nclos[i] = (int)std::min<size_t>((np + BULK_THREADS - 1) / BULK_THREADS, 128);
    nzt[i] = (I.gx * I.gy + I.pz.lpc - 1) / I.pz.lpc;
    a->nclos_max = std::max(a->nclos_max, nclos[i]);
    o[i].sf = c.take(np * sizeof(double2));
    o[i].bb = c.take(2 * np * sizeof(double));
    o[i].part = c.take((size_t)nclos[i] * 4 * sizeof(double));
    o[i].gpart = c.take((size_t)nzt[i] * 3 * sizeof(double));
  }
  const size_t o_sc = c.take((size_t)n * ADJ_NSC * sizeof(double));
  const size_t o_w = c.take(b->foff[n] * sizeof(double));
  if (cudaMalloc(&a->pool, c.off) != cudaSuccess) {
    cudaGetLastError();
    return berr(b, ADSCF_E_OOM, "batch adjoint pool");
  }
  unsigned char* base = static_cast<unsigned char*>(a->pool);
  a->d_sc = reinterpret_cast<double*>(base + o_sc);
  a->d_w = reinterpret_cast<double*>(base + o_w);
  std::vector<AdjDev> h(n);
  std::vector<BulkDev<double>> two(2 * n);
  for (int i = 0; i < n; ++i) {
    const adscf_params& q = b->p[i];
    AdjDev& A = h[i];
    A.I = b->hI64[i];
    A.sa = A.I.spec;
    A.slA = A.slB = A.I.slices;
    A.tA0 = A.tB0 = 0;
    A.sf = reinterpret_cast<double2*>(base + o[i].sf);
    A.b = reinterpret_cast<double*>(base + o[i].bb);
    A.w = a->d_w + b->foff[i];
    A.part = reinterpret_cast<double*>(base + o[i].part);
    A.gpart = reinterpret_cast<double*>(base + o[i].gpart);
    A.sc = a->d_sc + (size_t)i * ADJ_NSC;
    A.nqpart = b->cont_blocks;
    A.nclos = nclos[i];
    A.nztiles = nzt[i];
    A.rho = q.rho; A.kappa = q.kappa; A.chi = q.chi;
    A.v0 = q.monomer_volume[0] != 0 ? q.monomer_volume[0] : 1.0;
    A.v1 = q.monomer_volume[1] != 0 ? q.monomer_volume[1] : 1.0;
    A.ds = q.ds;
    A.lx = q.sizex; A.ly = q.sizey; A.lz = q.sizez;
    two[2 * i] = A.I;
    two[2 * i + 1] = A.I;
    two[2 * i + 1].spec = A.sf;
    a->smx = std::max(a->smx, plan_bytes_d(A.I.px, 2));
    a->smy = std::max(a->smy, plan_bytes_d(A.I.py, 2));
    a->smz = std::max(a->smz, plan_bytes_d(A.I.pz, 3));
  }
  BK(cudaMalloc(&a->d_adj, n * sizeof(AdjDev)));
  BK(cudaMemcpyAsync(a->d_adj, h.data(), n * sizeof(AdjDev), cudaMemcpyHostToDevice, b->stream));
  BK(cudaMalloc(&a->d_inst2, 2 * n * sizeof(BulkDev<double>)));
  BK(cudaMemcpyAsync(a->d_inst2, two.data(), 2 * n * sizeof(BulkDev<double>), cudaMemcpyHostToDevice, b->stream));
  a->gpart_off.resize(n);
  for (int i = 0; i < n; ++i) a->gpart_off[i] = o[i].gpart;
  // generic-plan work lists by descending Ns: the instances still on their
  // reverse sweep at step T are a prefix
  std::vector<int> ord(n);
  for (int i = 0; i < n; ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return b->ns[x] > b->ns[y]; });
  std::vector<int2> wx, wy2, wy1, wz;
  std::vector<int> tx(n), ty(n), tz(n);
  for (int i : ord) {
    const BulkDev<double>& I = b->hI64[i];
    tx[i] = (I.gy * I.gz + I.px.lpc - 1) / I.px.lpc;
    ty[i] = (I.gx * I.gz + I.py.lpc - 1) / I.py.lpc;
    tz[i] = nzt[i];
    for (int k = 0; k < tx[i]; ++k) wx.push_back(make_int2(i, k));
    for (int k = 0; k < ty[i]; ++k) { wy2.push_back(make_int2(2 * i, k)); wy2.push_back(make_int2(2 * i + 1, k)); }
    for (int k = 0; k < ty[i]; ++k) wy1.push_back(make_int2(2 * i, k));
    for (int k = 0; k < tz[i]; ++k) wz.push_back(make_int2(i, k));
  }
  a->px.assign(b->maxns + 1, 0); a->py2.assign(b->maxns + 1, 0);
  a->py1.assign(b->maxns + 1, 0); a->pz.assign(b->maxns + 1, 0);
  for (int T = 1; T <= b->maxns; ++T)
    for (int i = 0; i < n; ++i)
      if (b->ns[i] >= T) { a->px[T] += tx[i]; a->py2[T] += 2 * ty[i]; a->py1[T] += ty[i]; a->pz[T] += tz[i]; }
  auto up = [&](const std::vector<int2>& v, int2*& d) -> int {
    BK(cudaMalloc(&d, v.size() * sizeof(int2)));
    BK(cudaMemcpyAsync(d, v.data(), v.size() * sizeof(int2), cudaMemcpyHostToDevice, b->stream));
    return ADSCF_OK;
  };
  int rc;
  if ((rc = up(wx, a->wx)) || (rc = up(wy2, a->wy2)) || (rc = up(wy1, a->wy1)) || (rc = up(wz, a->wz))) return rc;
  a->gpart_bytes = c.off;   // the whole pool is cleared before a backward pass
  int optin = 0;
  BK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->dev));
  if (a->smx > (size_t)optin || a->smy > (size_t)optin || a->smz + 3 * 32 * sizeof(double) > (size_t)optin)
    return berr(b, ADSCF_E_ARG, "grid line too long for the adjoint passes");
  BK(cudaFuncSetAttribute(k_adj_x_b, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)a->smx));
  BK(cudaFuncSetAttribute(k_adj_z_b, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)a->smz));
  BK(cudaStreamSynchronize(b->stream));
  return ADSCF_OK;
}

void batch_adj_destroy(adscf_batch* b) {
  BatchAdj* a = b->adj;
  if (!a) return;
  cudaFree(a->d_adj); cudaFree(a->d_inst2); cudaFree(a->pool);
  cudaFree(a->wx); cudaFree(a->wy2); cudaFree(a->wy1); cudaFree(a->wz);
  delete a;
  b->adj = nullptr;
}

int batch_adj_check(adscf_batch* b) {
  if (b->film || b->prec != ADSCF_FP64) return berr(b, ADSCF_E_STATE, "the batch adjoint needs an FP64 bulk batch");
  for (const adscf_params& q : b->p)
    if (q.ensemble != 1) return berr(b, ADSCF_E_STATE, "the batch adjoint covers the canonical ensemble");
  return ADSCF_OK;
}

}  // namespace

extern "C" {

int adscf_batch_forward(adscf_batch* b, const double* fields, double* free_energy) {
  ADSCF_RANGE("adscf_batch_forward");
  if (!b || !fields || !free_energy) return ADSCF_E_ARG;
  int rc;
  if ((rc = batch_adj_check(b)) || (rc = batch_adj_setup(b))) return rc;
  BatchAdj* a = b->adj;
  const int n = b->n;
  BK(cudaMemcpyAsync(a->d_w, fields, b->foff[n] * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  for (int i = 0; i < n; ++i) {
    const size_t np = b->npts[i];
    const int gb = (int)std::min<size_t>((2 * np + 255) / 256, 152 * 8);
    k_expfield<double><<<gb, 256, 0, b->stream>>>(a->d_w + b->foff[i], static_cast<double*>(b->E[i]), np, b->p[i].ds);
  }
  if ((rc = enqueue_propagation<double>(b))) return rc;
  k_adj_closure_b<<<dim3(a->nclos_max, n), BULK_THREADS, 0, b->stream>>>(a->d_adj);
  k_adj_scalars_b<<<n, 32, 0, b->stream>>>(a->d_adj);
  BK(cudaGetLastError());
  std::vector<double> sc((size_t)n * ADJ_NSC);
  BK(cudaMemcpyAsync(sc.data(), a->d_sc, sc.size() * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  BK(cudaStreamSynchronize(b->stream));
  for (int i = 0; i < n; ++i) {
    const double* q = sc.data() + (size_t)i * ADJ_NSC;
    if (!(q[ADJ_S] > 0.0) || !std::isfinite(q[ADJ_F]))
      return berr(b, ADSCF_E_NONFINITE, "instance " + std::to_string(i) + ": non-finite or non-positive Q");
    free_energy[i] = q[ADJ_F];
  }
  a->gen = ++b->prop_gen;
  return ADSCF_OK;
}

int adscf_batch_backward(adscf_batch* b, double* grad) {
  ADSCF_RANGE("adscf_batch_backward");
  if (!b || !grad) return ADSCF_E_ARG;
  int rc;
  if ((rc = batch_adj_check(b))) return rc;
  BatchAdj* a = b->adj;
  if (!a || a->gen != b->prop_gen)
    return berr(b, ADSCF_E_STATE, "adscf_batch_backward needs an immediately preceding adscf_batch_forward");
  cudaStream_t s = b->stream;
  const double2* tw = static_cast<const double2*>(b->d_tw);
  const double* fk = static_cast<const double*>(b->d_fk);
  for (int i = 0; i < b->n; ++i) {
    const int nzt = (b->hI64[i].gx * b->hI64[i].gy + b->hI64[i].pz.lpc - 1) / b->hI64[i].pz.lpc;
    BK(cudaMemsetAsync(static_cast<unsigned char*>(a->pool) + a->gpart_off[i], 0, (size_t)nzt * 3 * sizeof(double), s));
  }
  for (int T = b->maxns; T >= 1; --T) {
    if (a->px[T] <= 0) continue;
    k_adj_x_b<<<a->px[T], BULK_THREADS, a->smx, s>>>(a->d_adj, a->wx, tw, T);
    k_bulk_strided<double><<<a->py2[T], BULK_THREADS, a->smy, s>>>(a->d_inst2, a->wy2, tw, fk, nullptr, b->d_g64, T, 0);
    k_adj_z_b<<<a->pz[T], BULK_THREADS, a->smz, s>>>(a->d_adj, a->wz, tw, fk, T);
    if (T > 1)
      k_bulk_strided<double><<<a->py1[T], BULK_THREADS, a->smy, s>>>(a->d_inst2, a->wy1, tw, fk, nullptr, b->d_g64, T, 1);
  }
  k_adj_grad_b<<<b->n, 32, 0, s>>>(a->d_adj);
  BK(cudaGetLastError());
  std::vector<double> sc((size_t)b->n * ADJ_NSC);
  BK(cudaMemcpyAsync(sc.data(), a->d_sc, sc.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  BK(cudaStreamSynchronize(s));
  for (int i = 0; i < b->n; ++i) {
    const double* q = sc.data() + (size_t)i * ADJ_NSC;
    grad[4 * i + 0] = q[ADJ_DLX];
    grad[4 * i + 1] = q[ADJ_DLY];
    grad[4 * i + 2] = q[ADJ_DLZ];
    grad[4 * i + 3] = q[ADJ_DCHI];
  }
  return ADSCF_OK;
}

int adscf_batch_create(const adscf_params* params, int n, adscf_batch** out) {
  ADSCF_RANGE("adscf_batch_create");
  if (!out) return ADSCF_E_ARG;
  *out = nullptr;
  if (!params || n < 1) return ADSCF_E_ARG;
  adscf_batch* b = new (std::nothrow) adscf_batch();
  if (!b) return ADSCF_E_OOM;
  b->n = n;
  b->prec = params[0].precision;
  if (b->prec != ADSCF_FP64 && b->prec != ADSCF_SPLIT) { delete b; return ADSCF_E_ARG; }
  b->p.assign(params, params + n);
  const bool film = params[0].geometry == ADSCF_FILM_1D || params[0].geometry == ADSCF_BRUSH;
  for (int i = 0; i < n && !film; ++i) {
    std::string why;
    if (check_params(b->p[i], b->prec, why)) { delete b; return ADSCF_E_ARG; }
  }
  if (cudaGetDevice(&b->dev) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete b;
    return ADSCF_E_CUDA;
  }
  b->stream = b->own_stream;
  const int rc = film ? build_film(b) : b->prec == ADSCF_SPLIT ? build<float>(b) : build<double>(b);
  // the caller's arrays were read during the build only
  for (adscf_params& q : b->p) { q.dss = nullptr; q.dz = nullptr; q.ext_potential = nullptr; q.graft = nullptr; }
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
  batch_adj_destroy(b);
  if (b->g_iter) cudaGraphExecDestroy(b->g_iter);
  cudaFree(b->pool); cudaFree(b->d_inst); cudaFree(b->d_S);
  cudaFree(b->d_tw); cudaFree(b->d_fk); cudaFree(b->d_g64);
  for (auto& C : b->cls) { cudaFree(C.wx); cudaFree(C.wy); cudaFree(C.wz); }
  cudaFree(b->d_f32); cudaFree(b->d_f64); cudaFree(b->d_list32); cudaFree(b->d_list64); cudaFree(b->d_items32);
  cudaFree(b->d_items); cudaFree(b->d_ctl); cudaFree(b->d_ranges);
  cudaFree(b->d_tabf);
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
  ADSCF_RANGE("adscf_batch_scf_run");
  if (!b || n_iter < 0) return ADSCF_E_ARG;
  ++b->prop_gen;
  int rc = build_graph(b);
  if (rc) return rc;
  for (int i = 0; i < n_iter; ++i) {
    BK(cudaGraphLaunch(b->g_iter, b->stream));
    if (tol >= 0.0) {
      double mx = 0.0;
      if ((rc = read_results(b, out, &mx))) return rc;
      if (!(mx > tol)) return check_pivot(b);
    }
  }
  rc = read_results(b, out, nullptr);
  return rc ? rc : check_pivot(b);
}

int adscf_batch_set_stream(adscf_batch* b, void* cuda_stream) {
  if (!b) return ADSCF_E_ARG;
  BK(cudaStreamSynchronize(b->stream));
  b->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : b->own_stream;
  return ADSCF_OK;
}

int adscf_batch_enqueue(adscf_batch* b, int repeats) {
  ADSCF_RANGE("adscf_batch_enqueue");
  if (!b || repeats < 0) return ADSCF_E_ARG;
  ++b->prop_gen;
  int rc = build_graph(b);
  if (rc) return rc;
  for (int i = 0; i < repeats; ++i) BK(cudaGraphLaunch(b->g_iter, b->stream));
  return ADSCF_OK;
}

int adscf_batch_results(adscf_batch* b, adscf_iter_result* out) {
  if (!b || !out) return ADSCF_E_ARG;
  return read_results(b, out, nullptr);
}

int adscf_batch_launches(const adscf_batch* b) {
  if (!b) return -1;
  if (b->film) return 2 * ((b->n32 > 0) + (b->n64 > 0)) + 3;
  if (b->sweep) return 5;   // sweep, contour, closure, solve, mix (and a memset of the counters)
  int k = 4;   // contour, closure, solve, mix
  for (const auto& C : b->cls) {
    k += C.px[0] > 0;
    for (int t = 1; t <= b->maxns; ++t) k += 2 * (C.py[t] > 0) + (C.pz[t] > 0) + (C.px[t] > 0);
  }
  return k;
}

}  // extern "C"
