// internal.h -- host-side context of the SCF library (not part of the ABI).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <string>
#include <vector>

#include "../../include/adscf.h"
#include "bulk_kernels.cuh"
#include "scf_kernels.cuh"

struct FilmState;  // film / brush device state (film.cu)
// pass kernels of a bulk double step
enum { PK_PLAIN = 0, PK_PERSISTENT = 1, PK_TMA = 2, PK_FUSED = 3 };
struct AdjState;   // adjoint buffers and work lists (adjoint.cu)

struct adscf_ctx {
  adscf_params p{};
  std::string err;
  int geometry = 0;
  int prec = 0;                 // ADSCF_FP64 / ADSCF_SPLIT
  int gx = 0, gy = 0, gz = 0;   // bulk grid; films: gz intervals
  int nplanes = 0;              // bulk gz, films gz+1
  int npts = 0;                 // points per species
  int ntypes = 2;
  int ns = 0, na = 0, nb = 0;   // contour steps
  int nblk = 0;                 // bulk block sequence (0: the diblock of na / nb)
  int bend[ADSCF_MAX_BLOCKS] = {};
  unsigned btype = 0;
  float2* d_wtab = nullptr;     // [ns+1] node weights (A, B) of a block sequence
  double* d_mob = nullptr;      // DDFT: [3][npts] mobility_qq (AA, AB, BB) per wave vector
  double* d_ddft = nullptr;     // DDFT: density, its rate, mu [2][npts] each, complex staging
  std::vector<double> blk_len;  // the block sequence's lengths and types
  std::vector<int> blk_type;
  double volume = 0, dvol = 0;
  cudaStream_t stream = nullptr;      // stream all work goes to
  cudaStream_t own_stream = nullptr;  // the context's own stream
  // adscf_scf_iteration: the iteration graph records ev_dens once the
  // closure has written the densities, so their copy to the host runs on
  // copy_stream while the solve and the mix finish
  cudaEvent_t ev_dens = nullptr, ev_copy = nullptr;
  cudaStream_t copy_stream = nullptr;
  int dev = 0;
  int film_launches = 0, film_contour_launches = 0;

  // ---- bulk propagator (one of the two precisions is populated)
  void* d_inst = nullptr;       // BulkDev<T> on device
  BulkDev<float> hb32{};
  BulkDev<double> hb64{};
  void* d_tw = nullptr;         // twiddles (cplx<T>)
  void* d_fk = nullptr;         // diffusion factors (T)
  void* d_tw64 = nullptr;       // FP64 twiddles of the (0,0) z pencil
  double* d_g64 = nullptr;      // FP64 diffusion factors of that pencil
  int2* d_work_x = nullptr; int n_work_x = 0;
  int2* d_work_y = nullptr; int n_work_y = 0;
  int2* d_work_z = nullptr; int n_work_z = 0;
  size_t smem_x = 0, smem_y = 0, smem_z = 0;
  int regx = 0, regy = 0, regz = 0;   // register-FFT line length per pass (0: generic)
  int use_generic = 0;                // force the generic mixed-radix kernels
  int no_persistent = 0;              // disable the persistent pipelined passes
  int pgrid_x = 0, pgrid_y = 0, pgrid_z = 0;  // persistent grid sizes (0: not used)
  // TMA-fed strided passes (FP32, one line length on all axes)
  int tma = 0, no_tma = 0;
  CUtensorMap tmap_y{}, tmap_z{};
  int tma_tiles_y = 0, tma_tiles_z = 0, tma_grid = 0;
  size_t tma_smem = 0;
  size_t xy_smem = 0;                 // fused XY plane pass (FP32, gx = gy = 64/128)
  int xy_grid = 0;
  int* d_flags = nullptr;             // device error flags (bounded-wait expiry)
  float2* d_dcin = nullptr;           // fused XY plan: [2][gz] (0,0) pencils entering the z pass, [gz] convolved
  // kernel per pass of a double step (PK_*), chosen by the autotuner
  int plan_y = PK_PLAIN, plan_z = PK_PLAIN, plan_x = PK_PLAIN;
  int autotune = 1;
  std::string tune_report;
  int contour_blocks = 0;

  // ---- SCF state (FP64)
  ScfDev S{};
  double* d_dist = nullptr;     // [ntypes][npts]
  double* d_dens = nullptr;
  double* d_hx = nullptr;
  double* d_hr = nullptr;
  double* d_hy = nullptr;       // Anderson: x_j + lambda r_j per slot
  double* d_qpart = nullptr;
  double* d_part = nullptr;
  double* d_gram = nullptr;
  double* d_coef = nullptr;
  double* d_res = nullptr;
  int* d_iter = nullptr;
  double* d_wz = nullptr;
  double* d_ext = nullptr;
  double* d_tmp = nullptr;      // [ntypes][npts] FP64 staging
  double* h_pinned = nullptr;   // pinned staging for host copies
  size_t pinned_bytes = 0;
  int closure_blocks = 0;
  int mix_blocks = 0;
  int hist_slots = 2;

  // graph of one whole SCF iteration (bulk) and of one propagation
  cudaGraphExec_t g_iter = nullptr;
  cudaGraphExec_t g_prop = nullptr;

  FilmState* film = nullptr;

  // adjoint (adjoint.cu): state of the last adscf_forward, and a counter that
  // every propagating entry point advances so a stale forward is detected
  AdjState* adj = nullptr;
  long long prop_gen = 0;
  adscf_ctx* sib64 = nullptr;   // FP64 sibling of a split context (adscf_free_energy_fp64)
  int adj_ckpt = 0;             // adjoint checkpoint interval (0: every slice stored, < 0: ceil(sqrt(Ns)))
  bool slices_full = true;      // all Ns + 1 propagator slices held (bulk_hold_slices)
};

// NVTX range over an entry point (header-only NVTX v3: without a profiler
// attached each push / pop is a cheap no-op)
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
#define ADSCF_RANGE(name) NvtxRange adscf_nvtx_range_(name)

// errors
int set_err(adscf_ctx* c, int code, const std::string& msg);
// two timing events destroyed with their scope (the tuners return early on
// a CUDA error)
struct EventPair {
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t create() {
    cudaError_t e = cudaEventCreate(&a);
    return e != cudaSuccess ? e : cudaEventCreate(&b);
  }
  ~EventPair() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};
// host helpers (capi.cu): blocks for n items, capped; host <-> device copies of
// n doubles through the context's page-locked staging buffer (synchronous)
int grid_blocks(size_t n, int per, int cap);
int ensure_pinned(adscf_ctx* ctx, size_t bytes);
bool host_pinned(const void* p);
int h2d(adscf_ctx* ctx, double* d, const double* h, size_t n);
int d2h(adscf_ctx* ctx, double* h, const double* d, size_t n);
#define CK(call)                                                              \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess)                                                    \
      return set_err(ctx, ADSCF_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// bulk (bulk.cu)
int bulk_create(adscf_ctx* ctx);
void bulk_destroy(adscf_ctx* ctx);
int bulk_enqueue_propagate(adscf_ctx* ctx);     // from E to dist + qpart
int bulk_enqueue_chains(adscf_ctx* ctx);        // both chains, all steps
int bulk_enqueue_contour(adscf_ctx* ctx);       // contour integral + Q
int bulk_enqueue_expfield(adscf_ctx* ctx, const double* d_w);
int bulk_step_single(adscf_ctx* ctx, double* d_prop, const double* d_e);
int bulk_r2c(adscf_ctx* ctx, const double* d_prop, double* h_half);
int bulk_c2r(adscf_ctx* ctx, const double* h_half, double* d_prop);
int bulk_mix_e(adscf_ctx* ctx);                 // k_mix with E update
int bulk_set_box(adscf_ctx* ctx);               // k-space tables for new side lengths
int bulk_hold_slices(adscf_ctx* ctx, bool full);
int bulk_set_wait_polls(adscf_ctx* ctx, int polls);  // pipeline wait bound of the TMA passes   // all Ns + 1 slices, or two of scratch (FP64)
void adj_set_box(adscf_ctx* ctx);               // adjoint's copy of the side lengths
// adjoint (adjoint.cu)
void adj_destroy(adscf_ctx* ctx);
// films (film.cu)
int film_create(adscf_ctx* ctx, const adscf_params* p);
int film_check_pivot(adscf_ctx* ctx);
void film_destroy(adscf_ctx* ctx);
int film_enqueue_propagate(adscf_ctx* ctx, const double* d_w);
int film_enqueue_chains(adscf_ctx* ctx, const double* d_w);
int film_enqueue_contour(adscf_ctx* ctx);
int film_step_single(adscf_ctx* ctx, double* d_prop, const double* d_w, double ds);
int film_set_adi_plan(adscf_ctx* ctx, const int lanes[3], int staged);   // FP32 ADI lanes per line (x, y, z)
double* film_fe_field(adscf_ctx* ctx);                           // device buffer for the fields of film_forward
int film_forward(adscf_ctx* ctx, double* out_F);                // F at fixed fields (films, brush)
int film_backward(adscf_ctx* ctx, double* dF_dchi, double* dF_dU);
