// bulk.cu -- plans, tables and launch sequences of the bulk propagator.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "internal.h"
#include "bulk_reg.cuh"
#include "bulk_tma.cuh"
#include "bulk_host.h"

namespace {

using bulkhost::make_plan;
using bulkhost::plan_smem;

template <typename T>
BulkDev<T>& hb(adscf_ctx* c);
template <>
BulkDev<float>& hb<float>(adscf_ctx* c) { return c->hb32; }
template <>
BulkDev<double>& hb<double>(adscf_ctx* c) { return c->hb64; }

bool is_pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }
int reg_size(int n) { return (n == 32 || n == 64 || n == 128 || n == 256) ? n : 0; }

template <typename T>
size_t reg_smem(int n) {
  switch (n) {
    case 32: return regk::Layout<T, 32>::bytes;
    case 64: return regk::Layout<T, 64>::bytes;
    case 128: return regk::Layout<T, 128>::bytes;
    case 256: return regk::Layout<T, 256>::bytes;
  }
  return 0;
}
int reg_lpc(int n) {
  switch (n) {
    case 32: return BULK_THREADS / regk::Cfg<32>::TPL;
    case 64: return BULK_THREADS / regk::Cfg<64>::TPL;
    case 128: return BULK_THREADS / regk::Cfg<128>::TPL;
    case 256: return BULK_THREADS / regk::Cfg<256>::TPL;
  }
  return 0;
}

template <typename T>
int set_reg_attrs(adscf_ctx* ctx) {
#define ADSCF_ATTR1(NN, KK)                                                                   \
  CK(cudaFuncSetAttribute(k_rs<T, NN, KK>, cudaFuncAttributeMaxDynamicSharedMemorySize,      \
                          (int)regk::Layout<T, NN>::bytes));
#define ADSCF_ATTR(NN)                                                                        \
  CK(cudaFuncSetAttribute(k_rx<T, NN>, cudaFuncAttributeMaxDynamicSharedMemorySize,          \
                          (int)regk::Layout<T, NN>::bytes));                                  \
  ADSCF_ATTR1(NN, 0) ADSCF_ATTR1(NN, 1) ADSCF_ATTR1(NN, 2) ADSCF_ATTR1(NN, 3) ADSCF_ATTR1(NN, 4)
  ADSCF_ATTR(32) ADSCF_ATTR(64) ADSCF_ATTR(128) ADSCF_ATTR(256)
#undef ADSCF_ATTR
#undef ADSCF_ATTR1
  return ADSCF_OK;
}

// X pass launch: register kernel for 32..256-point rows, generic otherwise
template <typename T>
void launch_x(adscf_ctx* ctx, int t, int mode, XAux aux) {
  const BulkDev<T>* d = static_cast<const BulkDev<T>*>(ctx->d_inst);
  const cplx<T>* tw = static_cast<const cplx<T>*>(ctx->d_tw);
  cudaStream_t s = ctx->stream;
  const dim3 g(ctx->n_work_x), b(BULK_THREADS);
  switch (ctx->regx) {
    case 32: k_rx<T, 32><<<g, b, ctx->smem_x, s>>>(d, ctx->d_work_x, tw, t, mode, aux); break;
    case 64: k_rx<T, 64><<<g, b, ctx->smem_x, s>>>(d, ctx->d_work_x, tw, t, mode, aux); break;
    case 128: k_rx<T, 128><<<g, b, ctx->smem_x, s>>>(d, ctx->d_work_x, tw, t, mode, aux); break;
    case 256: k_rx<T, 256><<<g, b, ctx->smem_x, s>>>(d, ctx->d_work_x, tw, t, mode, aux); break;
    default: k_bulk_xpass<T><<<g, b, ctx->smem_x, s>>>(d, ctx->d_work_x, tw, t, mode, aux);
  }
}

// Y (kind 0/1) and Z (kind 2/3/4) pass launch
template <typename T>
void launch_s(adscf_ctx* ctx, int t, int kind) {
  const BulkDev<T>* d = static_cast<const BulkDev<T>*>(ctx->d_inst);
  const cplx<T>* tw = static_cast<const cplx<T>*>(ctx->d_tw);
  const T* fk = static_cast<const T*>(ctx->d_fk);
  const double2* tw64 = static_cast<const double2*>(ctx->d_tw64);
  const double* g64 = ctx->d_g64;
  cudaStream_t s = ctx->stream;
  const bool z = kind >= 2;
  const int n = z ? ctx->regz : ctx->regy;
  const int2* work = z ? ctx->d_work_z : ctx->d_work_y;
  const dim3 g(z ? ctx->n_work_z : ctx->n_work_y), b(BULK_THREADS);
  const size_t sm = z ? ctx->smem_z : ctx->smem_y;
#define ADSCF_KS(NN)                                                                          \
  switch (kind) {                                                                             \
    case 0: k_rs<T, NN, 0><<<g, b, sm, s>>>(d, work, tw, fk, tw64, g64, t); break;           \
    case 1: k_rs<T, NN, 1><<<g, b, sm, s>>>(d, work, tw, fk, tw64, g64, t); break;           \
    case 2: k_rs<T, NN, 2><<<g, b, sm, s>>>(d, work, tw, fk, tw64, g64, t); break;           \
    case 3: k_rs<T, NN, 3><<<g, b, sm, s>>>(d, work, tw, fk, tw64, g64, t); break;           \
    default: k_rs<T, NN, 4><<<g, b, sm, s>>>(d, work, tw, fk, tw64, g64, t); break;          \
  }
  switch (n) {
    case 32: ADSCF_KS(32) break;
    case 64: ADSCF_KS(64) break;
    case 128: ADSCF_KS(128) break;
    case 256: ADSCF_KS(256) break;
    default: k_bulk_strided<T><<<g, b, sm, s>>>(d, work, tw, fk, tw64, g64, t, kind);
  }
#undef ADSCF_KS
}

// persistent pipelined passes: grid = resident CTAs (occupancy x SMs)
template <typename T, int NN>
int setup_persistent(adscf_ctx* ctx) {
  const int sm = (int)regk::Layout<T, NN>::bytes;
  int nsm = 0, o0 = 0, o1 = 0, o2 = 0, ox = 0;
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->dev));
  CK(cudaFuncSetAttribute(k_rs_p<T, NN, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
  CK(cudaFuncSetAttribute(k_rs_p<T, NN, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
  CK(cudaFuncSetAttribute(k_rs_p<T, NN, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
  CK(cudaFuncSetAttribute(k_rx_p<T, NN>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o0, k_rs_p<T, NN, 0>, BULK_THREADS, sm));
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o1, k_rs_p<T, NN, 1>, BULK_THREADS, sm));
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o2, k_rs_p<T, NN, 2>, BULK_THREADS, sm));
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ox, k_rx_p<T, NN>, BULK_THREADS, sm));
  ctx->pgrid_y = std::min(ctx->n_work_y, nsm * std::max(1, std::min(o0, o1)));
  ctx->pgrid_z = std::min(ctx->n_work_z, nsm * std::max(1, o2));
  ctx->pgrid_x = std::min(ctx->n_work_x, nsm * std::max(1, ox));
  return ADSCF_OK;
}

// tensor maps of the spectrum for the TMA-fed Y and Z passes (FP32, 8-byte
// complex elements, 128-byte swizzle, boxes of 16 x-lines)
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int encode_map(adscf_ctx* ctx, CUtensorMap* m, void* base, const cuuint32_t box[3]) {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !p) {
      cudaGetLastError();
      return set_err(ctx, ADSCF_E_CUDA, "cuTensorMapEncodeTiled not available");
    }
    fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  const cuuint64_t dims[3] = {(cuuint64_t)ctx->gx, (cuuint64_t)ctx->gy, (cuuint64_t)ctx->gz};
  const cuuint64_t strides[2] = {(cuuint64_t)ctx->gx * 8, (cuuint64_t)ctx->gx * ctx->gy * 8};
  const cuuint32_t es[3] = {1, 1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, base, dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_err(ctx, ADSCF_E_CUDA, "cuTensorMapEncodeTiled failed");
  return ADSCF_OK;
}

template <int NN>
int setup_tma(adscf_ctx* ctx, void* spec) {
  using LY = tmak::TmaLayout<NN>;
  const cuuint32_t by[3] = {(cuuint32_t)tmak::kBoxCols, (cuuint32_t)NN, 1};
  const cuuint32_t bz[3] = {(cuuint32_t)tmak::kBoxCols, 1, (cuuint32_t)NN};
  int rc;
  if ((rc = encode_map(ctx, &ctx->tmap_y, spec, by))) return rc;
  if ((rc = encode_map(ctx, &ctx->tmap_z, spec, bz))) return rc;
  ctx->tma_smem = LY::bytes;
  CK(cudaFuncSetAttribute(k_rs_tma<NN, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LY::bytes));
  CK(cudaFuncSetAttribute(k_rs_tma<NN, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LY::bytes));
  CK(cudaFuncSetAttribute(k_rs_tma<NN, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LY::bytes));
  int nsm = 0, occ = 0;
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->dev));
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_rs_tma<NN, 2>, BULK_THREADS, LY::bytes));
  using LXY = tmak::XYLayout<NN>;
  CK(cudaFuncSetAttribute(k_xy_tma<NN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LXY::bytes));
  int occ_xy = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_xy, k_xy_tma<NN>, LXY::THREADS, LXY::bytes));
  ctx->xy_smem = LXY::bytes;
  ctx->tma_tiles_y = ctx->gx * ctx->gz / LY::LPC;
  ctx->tma_tiles_z = ctx->gx * ctx->gy / LY::LPC;
  ctx->tma_grid = nsm * std::max(1, occ);
  ctx->xy_grid = std::min(ctx->gz, nsm * std::max(1, occ_xy));
  if (!ctx->d_flags) {
    CK(cudaMalloc(&ctx->d_flags, sizeof(int)));
    CK(cudaMemset(ctx->d_flags, 0, sizeof(int)));
  }
  if (!ctx->d_dcin) {   // [2][NN] pencils kept by the plane pass | [NN] convolved by the z pass
    CK(cudaMalloc(&ctx->d_dcin, 3 * (size_t)NN * sizeof(float2)));
    CK(cudaMemset(ctx->d_dcin, 0, 3 * (size_t)NN * sizeof(float2)));
  }
  ctx->tma = NN;
  return ADSCF_OK;
}

template <typename T>
int tune_t(adscf_ctx* ctx);

template <typename T>
int create_t(adscf_ctx* ctx) {
  BulkDev<T> I{};
  I.gx = ctx->gx; I.gy = ctx->gy; I.gz = ctx->gz;
  I.npts = ctx->npts;
  I.ns = ctx->ns; I.na = ctx->na; I.nb = ctx->nb;
  I.nblk = ctx->nblk;
  for (int k = 0; k < ADSCF_MAX_BLOCKS; ++k) I.bend[k] = ctx->bend[k];
  I.btype = ctx->btype;
  I.wtab = nullptr;
  if (ctx->nblk) {
    // Propagate_Multiblock (mod_multiblock.f90:148-160): per block, 1/2 at
    // its end nodes and 1 inside, summed by monomer type
    std::vector<float2> wt(ctx->ns + 1, make_float2(0.f, 0.f));
    int s0 = 0;
    for (int k = 0; k < ctx->nblk; ++k) {
      const int s1 = ctx->bend[k];
      float* acc = (ctx->btype >> k) & 1u ? &wt[0].y : &wt[0].x;
      for (int s = s0; s <= s1; ++s) {
        const float w = (s == s0 ? 0.5f : 0.f) + (s == s1 ? 0.5f : 0.f) + ((s > s0 && s < s1) ? 1.f : 0.f);
        acc[2 * s] += w;
      }
      s0 = s1;
    }
    CK(cudaMalloc(&ctx->d_wtab, wt.size() * sizeof(float2)));
    CK(cudaMemcpy(ctx->d_wtab, wt.data(), wt.size() * sizeof(float2), cudaMemcpyHostToDevice));
    I.wtab = ctx->d_wtab;
  }
  I.ds = ctx->p.ds;
  if (!make_plan(ctx->gx, I.px) || !make_plan(ctx->gy, I.py) || !make_plan(ctx->gz, I.pz))
    return set_err(ctx, ADSCF_E_ARG, "grid sizes must be products of 2, 3 and 5");
  // twiddle tables W_n^m = exp(-2 pi i m / n), computed in FP64
  std::vector<cplx<T>> tw;
  std::vector<std::pair<int, int>> seen;
  I.px.tw_off = bulkhost::twiddle_offset<T>(ctx->gx, tw, seen);
  I.py.tw_off = bulkhost::twiddle_offset<T>(ctx->gy, tw, seen);
  I.pz.tw_off = bulkhost::twiddle_offset<T>(ctx->gz, tw, seen);
  // diffusion factors exp(-ds k^2) (mod_fourier.f90:188) and the (0,0)
  // pencil's circulant kernel
  std::vector<T> fk;
  std::vector<double> g64;
  bulkhost::append_tables<T>(ctx->gx, ctx->gy, ctx->gz, ctx->p.sizex, ctx->p.sizey, ctx->p.sizez,
                             ctx->p.ds, fk, g64, I.gxy_off, I.gz_off, I.g64_off);
  std::vector<double2> tw64(ctx->gz);
  for (int z = 0; z < ctx->gz; ++z) {
    const double a = -2.0 * M_PI * (double)z / (double)ctx->gz;
    tw64[z] = make_double2(std::cos(a), std::sin(a));
  }
  I.tw64_off = 0;
  CK(cudaMalloc(&ctx->d_tw64, tw64.size() * sizeof(double2)));
  CK(cudaMemcpy(ctx->d_tw64, tw64.data(), tw64.size() * sizeof(double2), cudaMemcpyHostToDevice));
  CK(cudaMalloc(&ctx->d_g64, g64.size() * sizeof(double)));
  CK(cudaMemcpy(ctx->d_g64, g64.data(), g64.size() * sizeof(double), cudaMemcpyHostToDevice));

  CK(cudaMalloc(&ctx->d_tw, tw.size() * sizeof(cplx<T>)));
  CK(cudaMemcpy(ctx->d_tw, tw.data(), tw.size() * sizeof(cplx<T>), cudaMemcpyHostToDevice));
  CK(cudaMalloc(&ctx->d_fk, fk.size() * sizeof(T)));
  CK(cudaMemcpy(ctx->d_fk, fk.data(), fk.size() * sizeof(T), cudaMemcpyHostToDevice));

  const size_t np = (size_t)ctx->npts;
  cplx<T>* spec = nullptr;
  cplx<T>* slices = nullptr;
  T* E = nullptr;
  const size_t ne = sizeof(T) == 4 ? 4 * np : 2 * np;   // FP32 keeps the residue
  if (cudaMalloc(&spec, np * sizeof(cplx<T>)) != cudaSuccess ||
      cudaMalloc(&slices, (size_t)(ctx->ns + 1) * np * sizeof(cplx<T>)) != cudaSuccess ||
      cudaMalloc(&E, ne * sizeof(T)) != cudaSuccess) {
    cudaFree(spec); cudaFree(slices); cudaFree(E);
    cudaGetLastError();
    return set_err(ctx, ADSCF_E_OOM, "device allocation of propagator slices failed");
  }
  I.spec = spec; I.slices = slices; I.E = E;
  I.dist = ctx->d_dist;
  {  // one resident wave of the contour kernel (a streaming grid-stride loop)
    int per_sm = 0, nsm = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bulk_contour<T>, BULK_THREADS, 0));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, ctx->dev));
    ctx->contour_blocks = (int)std::min<size_t>((np + BULK_THREADS - 1) / BULK_THREADS,
                                                (size_t)std::max(1, per_sm) * std::max(1, nsm));
  }
  CK(cudaMalloc(&ctx->d_qpart, ctx->contour_blocks * sizeof(double)));
  I.qpart = ctx->d_qpart;

  // work lists (single instance)
  auto mkwork = [&](int ntiles, int2*& d, int& n) -> int {
    std::vector<int2> w(ntiles);
    for (int i = 0; i < ntiles; ++i) w[i] = make_int2(0, i);
    n = ntiles;
    CK(cudaMalloc(&d, ntiles * sizeof(int2)));
    CK(cudaMemcpy(d, w.data(), ntiles * sizeof(int2), cudaMemcpyHostToDevice));
    return ADSCF_OK;
  };
  int rc;
  // per-axis kernel choice: register FFT for 32..256-point lines (the strided
  // passes also need a power-of-two gx for their line indexing)
  ctx->regx = ctx->use_generic ? 0 : reg_size(ctx->gx);
  ctx->regy = (ctx->use_generic || !is_pow2(ctx->gx)) ? 0 : reg_size(ctx->gy);
  ctx->regz = (ctx->use_generic || !is_pow2(ctx->gx)) ? 0 : reg_size(ctx->gz);
  const int lx = ctx->regx ? reg_lpc(ctx->regx) : I.px.lpc;
  const int ly = ctx->regy ? reg_lpc(ctx->regy) : I.py.lpc;
  const int lz = ctx->regz ? reg_lpc(ctx->regz) : I.pz.lpc;
  if ((rc = mkwork((ctx->gy * ctx->gz + lx - 1) / lx, ctx->d_work_x, ctx->n_work_x))) return rc;
  if ((rc = mkwork((ctx->gx * ctx->gz + ly - 1) / ly, ctx->d_work_y, ctx->n_work_y))) return rc;
  if ((rc = mkwork((ctx->gx * ctx->gy + lz - 1) / lz, ctx->d_work_z, ctx->n_work_z))) return rc;
  ctx->smem_x = ctx->regx ? reg_smem<T>(ctx->regx) : plan_smem<T>(I.px);
  ctx->smem_y = ctx->regy ? reg_smem<T>(ctx->regy) : plan_smem<T>(I.py);
  ctx->smem_z = ctx->regz ? reg_smem<T>(ctx->regz)
                          : plan_smem<T>(I.pz) + 16 + (((I.pz.n + 1) & ~1) + 2 * (size_t)I.pz.ld) * sizeof(double2);
  size_t mx = std::max(ctx->smem_x, std::max(ctx->smem_y, ctx->smem_z));
  if (mx > 227 * 1024) return set_err(ctx, ADSCF_E_ARG, "grid line too long for shared memory");
  // the limit is a per-function setting shared by every context: raise it to
  // the device maximum so a later, smaller context cannot lower it below what
  // an earlier one launches with
  int optin = 0;
  CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->dev));
  if (mx > (size_t)optin) return set_err(ctx, ADSCF_E_ARG, "grid line too long for shared memory");
  CK(cudaFuncSetAttribute(k_bulk_xpass<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
  CK(cudaFuncSetAttribute(k_bulk_strided<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
  if ((rc = set_reg_attrs<T>(ctx))) return rc;
  // the persistent passes need one register length on all three axes
  if (ctx->regx && ctx->regx == ctx->regy && ctx->regx == ctx->regz && !ctx->no_persistent) {
    switch (ctx->regx) {
      case 32: rc = setup_persistent<T, 32>(ctx); break;
      case 64: rc = setup_persistent<T, 64>(ctx); break;
      case 128: rc = setup_persistent<T, 128>(ctx); break;
      case 256: rc = setup_persistent<T, 256>(ctx); break;
    }
    if (rc) return rc;
  }
  // TMA-fed Y and Z passes: FP32, 64- or 128-point lines on all three axes
  if (sizeof(T) == 4 && ctx->pgrid_x && !ctx->no_tma && (ctx->regx == 64 || ctx->regx == 128)) {
    rc = ctx->regx == 64 ? setup_tma<64>(ctx, I.spec) : setup_tma<128>(ctx, I.spec);
    if (rc) return rc;
  }

  I.wait_polls = tmak::kWaitPolls;
  CK(cudaMalloc(&ctx->d_inst, sizeof(BulkDev<T>)));
  CK(cudaMemcpy(ctx->d_inst, &I, sizeof(I), cudaMemcpyHostToDevice));
  hb<T>(ctx) = I;
  // default plan: the most specialised kernel available for each pass (the
  // fused plane pass where the TMA passes run: the tuner's choice at 64^3 and
  // 128^3 on GB300)
  ctx->plan_y = ctx->plan_z = ctx->tma ? PK_TMA : ctx->pgrid_y ? PK_PERSISTENT : PK_PLAIN;
  ctx->plan_x = ctx->tma && ctx->xy_grid ? PK_FUSED : ctx->pgrid_x ? PK_PERSISTENT : PK_PLAIN;
  if (ctx->autotune) return tune_t<T>(ctx);
  return ADSCF_OK;
}

// One double step t: Yf, Z, Yi, X with the kernel the pass plan names for
// each pass (PK_PLAIN: one CTA per tile; PK_PERSISTENT: resident grid with
// register prefetch; PK_TMA: TMA-fed tiles, FP32 64/128).  Every choice does
// the same arithmetic on the same natural-order spectrum.
template <typename T>
int expfield_t(adscf_ctx* ctx, const double* d_w);

// Launch with programmatic stream serialisation: the kernel may start while
// the previous kernel on the stream finishes; the TMA passes wait for it
// (griddepcontrol.wait) before they touch its output.
template <typename... KArgs, typename... Args>
void launch_pdl(void (*kern)(KArgs...), int grid, int block, size_t smem, cudaStream_t s,
                Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

// fused XY plane pass of step t (t = 0: the initial plane)
template <int NN>
void xy_pass(adscf_ctx* ctx, int t) {
  const BulkDev<float>* df = static_cast<const BulkDev<float>*>(ctx->d_inst);
  const float2* twf = static_cast<const float2*>(ctx->d_tw);
  launch_pdl(k_xy_tma<NN>, ctx->xy_grid, tmak::XYLayout<NN>::THREADS, ctx->xy_smem, ctx->stream,
             df, ctx->tmap_y, twf,
             ctx->plan_z == PK_TMA ? (const float2*)(ctx->d_dcin + 2 * NN) : nullptr,
             ctx->d_dcin, t, ctx->d_flags);
}

template <typename T, int NN>
void step_nn(adscf_ctx* ctx, int t) {
  const BulkDev<T>* d = static_cast<const BulkDev<T>*>(ctx->d_inst);
  const cplx<T>* tw = static_cast<const cplx<T>*>(ctx->d_tw);
  const T* fk = static_cast<const T*>(ctx->d_fk);
  const double2* tw64 = static_cast<const double2*>(ctx->d_tw64);
  const double* g64 = ctx->d_g64;
  cudaStream_t s = ctx->stream;
  const size_t sm = ctx->smem_x;
  // dc = 0: the TMA z pass leaves the (0, 0) pencil to the fused XY pass
  auto spass = [&](int kind, int dc = 1) {
    const int pk = kind == 2 ? ctx->plan_z : ctx->plan_y;
    if constexpr (sizeof(T) == 4 && (NN == 64 || NN == 128)) {
      if (pk == PK_TMA) {
        const BulkDev<float>* df = reinterpret_cast<const BulkDev<float>*>(d);
        const float2* twf = reinterpret_cast<const float2*>(tw);
        const float* fkf = reinterpret_cast<const float*>(fk);
        const bool z = kind == 2;
        const int tiles = z ? ctx->tma_tiles_z : ctx->tma_tiles_y;
        const int grid = std::min(ctx->tma_grid, tiles);
        const CUtensorMap& map = z ? ctx->tmap_z : ctx->tmap_y;
        if (kind == 0) launch_pdl(k_rs_tma<NN, 0>, grid, BULK_THREADS, ctx->tma_smem, s, df, map, tiles, twf, fkf, g64, t, dc,
                   (const float2*)ctx->d_dcin, ctx->d_dcin + 2 * NN, ctx->d_flags);
        else if (kind == 1) launch_pdl(k_rs_tma<NN, 1>, grid, BULK_THREADS, ctx->tma_smem, s, df, map, tiles, twf, fkf, g64, t, dc,
                   (const float2*)ctx->d_dcin, ctx->d_dcin + 2 * NN, ctx->d_flags);
        else launch_pdl(k_rs_tma<NN, 2>, grid, BULK_THREADS, ctx->tma_smem, s, df, map, tiles, twf, fkf, g64, t, dc,
                   (const float2*)ctx->d_dcin, ctx->d_dcin + 2 * NN, ctx->d_flags);
        return;
      }
    }
    if (pk == PK_PERSISTENT) {
      if (kind == 0) k_rs_p<T, NN, 0><<<ctx->pgrid_y, BULK_THREADS, sm, s>>>(d, ctx->n_work_y, tw, fk, tw64, g64, t);
      else if (kind == 1) k_rs_p<T, NN, 1><<<ctx->pgrid_y, BULK_THREADS, sm, s>>>(d, ctx->n_work_y, tw, fk, tw64, g64, t);
      else k_rs_p<T, NN, 2><<<ctx->pgrid_z, BULK_THREADS, sm, s>>>(d, ctx->n_work_z, tw, fk, tw64, g64, t);
      return;
    }
    launch_s<T>(ctx, t, kind);
  };
  if constexpr (sizeof(T) == 4 && (NN == 64 || NN == 128)) {
    if (ctx->plan_x == PK_FUSED) {   // Z, then Yi + X + Yf of the next step in one plane pass
      spass(2, 0);
      xy_pass<NN>(ctx, t);
      return;
    }
  }
  spass(0);
  spass(2);
  spass(1);
  if (ctx->plan_x == PK_PERSISTENT) {
    k_rx_p<T, NN><<<ctx->pgrid_x, BULK_THREADS, sm, s>>>(d, ctx->n_work_x, tw, t);
  } else {
    const XAux none{nullptr, nullptr, nullptr};
    launch_x<T>(ctx, t, XM_STEP, none);
  }
}

template <typename T>
void step_t(adscf_ctx* ctx, int t) {
  // persistent and TMA passes need one register line length on all axes
  const int nn = (ctx->regx && ctx->regx == ctx->regy && ctx->regx == ctx->regz) ? ctx->regx : 0;
  switch (nn) {
    case 32: step_nn<T, 32>(ctx, t); break;
    case 64: step_nn<T, 64>(ctx, t); break;
    case 128: step_nn<T, 128>(ctx, t); break;
    case 256: step_nn<T, 256>(ctx, t); break;
    default: {
      const XAux none{nullptr, nullptr, nullptr};
      launch_s<T>(ctx, t, 0);
      launch_s<T>(ctx, t, 2);
      launch_s<T>(ctx, t, 1);
      launch_x<T>(ctx, t, XM_STEP, none);
    }
  }
}

template <typename T>
int chains_t(adscf_ctx* ctx) {
  const XAux none{nullptr, nullptr, nullptr};
  if (sizeof(T) == 4 && ctx->plan_x == PK_FUSED) {
    // the initial plane pass also does Yf of step 1
    if (ctx->tma == 64) xy_pass<64>(ctx, 0);
    else xy_pass<128>(ctx, 0);
  } else {
    launch_x<T>(ctx, 0, XM_INIT, none);
  }
  for (int t = 1; t <= ctx->ns; ++t) step_t<T>(ctx, t);
  CK(cudaGetLastError());
  return ADSCF_OK;
}

// ---------------------------------------------------------------------------
// Autotuner: time every available pass plan on this context's buffers and
// keep the fastest.  Candidates per pass: Y and Z {plain, persistent, TMA},
// X {plain, persistent}, as the shape and precision allow.  Each candidate
// runs a few double steps (after two warm-up steps) on unit Boltzmann
// factors, twice, timed with CUDA events on the context stream; the minimum
// per-step time decides.  Plans are cached per (device, grid, precision), so
// contexts of a shape already seen reuse the choice.
// ---------------------------------------------------------------------------
struct TuneKey {
  int dev, gx, gy, gz, prec, avail;   // avail: bit set of the kernels this context can run
  bool operator<(const TuneKey& o) const {
    return std::tie(dev, gx, gy, gz, prec, avail) < std::tie(o.dev, o.gx, o.gy, o.gz, o.prec, o.avail);
  }
};
struct TuneVal {
  int y, z, x;
  std::string report;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneVal> g_tune;

const char* pk_name(int k) {
  return k == PK_FUSED ? "fused-xy" : k == PK_TMA ? "tma" : k == PK_PERSISTENT ? "persistent" : "plain";
}

template <typename T>
int tune_t(adscf_ctx* ctx) {
  const int avail = (ctx->tma ? 1 : 0) | (ctx->pgrid_y ? 2 : 0) | (ctx->pgrid_x ? 4 : 0) |
                    (ctx->use_generic ? 8 : 0);
  const TuneKey key{ctx->dev, ctx->gx, ctx->gy, ctx->gz, ctx->prec, avail};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      ctx->plan_y = it->second.y; ctx->plan_z = it->second.z; ctx->plan_x = it->second.x;
      ctx->tune_report = it->second.report + " (cached)";
      return ADSCF_OK;
    }
  }
  std::vector<int> ys = {PK_PLAIN}, xs = {PK_PLAIN};
  if (ctx->pgrid_y) ys.push_back(PK_PERSISTENT);
  if (ctx->tma) ys.push_back(PK_TMA);
  if (ctx->pgrid_x) xs.push_back(PK_PERSISTENT);
  if (ctx->tma && ctx->xy_grid) xs.push_back(PK_FUSED);
  const std::vector<int>& zs = ys;
  if (ys.size() * xs.size() == 1) return ADSCF_OK;
  // unit Boltzmann factors from a zero field; the slice buffer takes the steps
  CK(cudaMemsetAsync(ctx->d_tmp, 0, 2 * (size_t)ctx->npts * sizeof(double), ctx->stream));
  int rc = expfield_t<T>(ctx, ctx->d_tmp);
  if (rc) return rc;
  const XAux none{nullptr, nullptr, nullptr};
  launch_x<T>(ctx, 0, XM_INIT, none);
  const int steps = std::min(ctx->ns, 6);
  EventPair ev;
  CK(ev.create());
  cudaEvent_t e0 = ev.a, e1 = ev.b;
  struct Cand { int y, z, x; float us; };
  std::vector<Cand> cands;
  for (int x : xs)
    for (int z : zs)
      for (int y : ys) {
        if (x == PK_FUSED && y != ys[0]) continue;   // the fused pass has no separate Y
        cands.push_back({x == PK_FUSED ? ys.back() : y, z, x, 1e30f});
      }
  for (int round = 0; round < 2; ++round) {
    for (Cand& c : cands) {
      ctx->plan_y = c.y; ctx->plan_z = c.z; ctx->plan_x = c.x;
      step_t<T>(ctx, 1);
      step_t<T>(ctx, 2 <= ctx->ns ? 2 : 1);
      cudaEventRecord(e0, ctx->stream);
      for (int t = 1; t <= steps; ++t) step_t<T>(ctx, t);
      cudaEventRecord(e1, ctx->stream);
      CK(cudaEventSynchronize(e1));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      c.us = std::min(c.us, 1000.f * ms / steps);
    }
  }
  CK(cudaGetLastError());
  const Cand* best = &cands[0];
  for (const Cand& c : cands)
    if (c.us < best->us) best = &c;
  ctx->plan_y = best->y; ctx->plan_z = best->z; ctx->plan_x = best->x;
  char line[160];
  std::snprintf(line, sizeof(line), "y=%s z=%s x=%s %.2f us/double step;", pk_name(best->y),
                pk_name(best->z), pk_name(best->x), best->us);
  std::string rep = line;
  for (const Cand& c : cands) {
    std::snprintf(line, sizeof(line), " %s/%s/%s %.2f", pk_name(c.y), pk_name(c.z), pk_name(c.x), c.us);
    rep += line;
  }
  ctx->tune_report = rep;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = TuneVal{best->y, best->z, best->x, rep};
  return ADSCF_OK;
}

template <typename T>
int contour_t(adscf_ctx* ctx) {
  const BulkDev<T>* d = static_cast<const BulkDev<T>*>(ctx->d_inst);
  k_bulk_contour<T><<<dim3(ctx->contour_blocks, 1), BULK_THREADS, 0, ctx->stream>>>(d);
  CK(cudaGetLastError());
  return ADSCF_OK;
}

template <typename T>
int propagate_t(adscf_ctx* ctx) {
  int rc = chains_t<T>(ctx);
  return rc ? rc : contour_t<T>(ctx);
}

template <typename T>
int expfield_t(adscf_ctx* ctx, const double* d_w) {
  T* E = hb<T>(ctx).E;
  const size_t n = 2 * (size_t)ctx->npts;
  k_expfield<T><<<std::min<size_t>((n + 255) / 256, 152 * 8), 256, 0, ctx->stream>>>(d_w, E, (size_t)ctx->npts, ctx->p.ds);
  CK(cudaGetLastError());
  return ADSCF_OK;
}

// one Propagate_Step on a single real field: prop <- E IFFT(G FFT(E prop))
template <typename T>
int step_single_t(adscf_ctx* ctx, double* d_prop, const double* d_e) {
  BulkDev<T>& I = hb<T>(ctx);
  const BulkDev<T>* d = static_cast<const BulkDev<T>*>(ctx->d_inst);
  const cplx<T>* tw = static_cast<const cplx<T>*>(ctx->d_tw);
  const T* fk = static_cast<const T*>(ctx->d_fk);
  const double2* tw64 = static_cast<const double2*>(ctx->d_tw64);
  const double* g64 = ctx->d_g64;
  cudaStream_t s = ctx->stream;
  const size_t n = (size_t)ctx->npts;
  // T staging inside the slice buffer: [prop | E]
  T* tp = reinterpret_cast<T*>(I.slices);
  T* te = tp + n;
  const int gb = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
  k_convert<T, double><<<gb, 256, 0, s>>>(d_prop, tp, n);
  k_convert<T, double><<<gb, 256, 0, s>>>(d_e, te, n);
  XAux a{tp, nullptr, te};
  launch_x<T>(ctx, 0, XM_R2S, a);
  launch_s<T>(ctx, 0, 0);
  launch_s<T>(ctx, 0, 2);
  launch_s<T>(ctx, 0, 1);
  XAux b{nullptr, tp, te};
  launch_x<T>(ctx, 0, XM_S2R, b);
  k_convert<double, T><<<gb, 256, 0, s>>>(tp, d_prop, n);
  CK(cudaGetLastError());
  return ADSCF_OK;
}

// forward 3D transform of a real field (Real2Fourier: scaled 1/N), returns the
// r2c half spectrum [gz][gy][gx/2+1] interleaved on the host
template <typename T>
int r2c_t(adscf_ctx* ctx, const double* d_prop, double* h_half) {
  BulkDev<T>& I = hb<T>(ctx);
  const BulkDev<T>* d = static_cast<const BulkDev<T>*>(ctx->d_inst);
  const cplx<T>* tw = static_cast<const cplx<T>*>(ctx->d_tw);
  const T* fk = static_cast<const T*>(ctx->d_fk);
  const double2* tw64 = static_cast<const double2*>(ctx->d_tw64);
  const double* g64 = ctx->d_g64;
  cudaStream_t s = ctx->stream;
  const size_t n = (size_t)ctx->npts;
  T* tp = reinterpret_cast<T*>(I.slices);
  const int gb = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
  k_convert<T, double><<<gb, 256, 0, s>>>(d_prop, tp, n);
  XAux a{tp, nullptr, nullptr};
  launch_x<T>(ctx, 0, XM_R2S, a);
  launch_s<T>(ctx, 0, 0);
  launch_s<T>(ctx, 0, 3);
  double2* full = reinterpret_cast<double2*>(ctx->d_tmp);  // needs 2*npts doubles
  k_spec_to_f64<T><<<gb, 256, 0, s>>>(I.spec, full, n, 1.0 / (double)n);
  CK(cudaGetLastError());
  std::vector<double2> h(n);
  CK(cudaMemcpyAsync(h.data(), full, n * sizeof(double2), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  const int hx = ctx->gx / 2 + 1;
  for (int z = 0; z < ctx->gz; ++z)
    for (int y = 0; y < ctx->gy; ++y)
      for (int x = 0; x < hx; ++x) {
        const double2 v = h[((size_t)z * ctx->gy + y) * ctx->gx + x];
        const size_t o = ((size_t)z * ctx->gy + y) * hx + x;
        h_half[2 * o] = v.x;
        h_half[2 * o + 1] = v.y;
      }
  return ADSCF_OK;
}

// Fourier2Real: unnormalised inverse of a Hermitian half spectrum
template <typename T>
int c2r_t(adscf_ctx* ctx, const double* h_half, double* d_prop) {
  BulkDev<T>& I = hb<T>(ctx);
  const BulkDev<T>* d = static_cast<const BulkDev<T>*>(ctx->d_inst);
  const cplx<T>* tw = static_cast<const cplx<T>*>(ctx->d_tw);
  const T* fk = static_cast<const T*>(ctx->d_fk);
  const double2* tw64 = static_cast<const double2*>(ctx->d_tw64);
  const double* g64 = ctx->d_g64;
  cudaStream_t s = ctx->stream;
  const size_t n = (size_t)ctx->npts;
  const int gx = ctx->gx, gy = ctx->gy, gz = ctx->gz, hx = gx / 2 + 1;
  std::vector<double2> h(n);
  for (int z = 0; z < gz; ++z)
    for (int y = 0; y < gy; ++y)
      for (int x = 0; x < gx; ++x) {
        double2 v;
        if (x < hx) {
          const size_t o = ((size_t)z * gy + y) * hx + x;
          v = make_double2(h_half[2 * o], h_half[2 * o + 1]);
        } else {  // Hermitian completion X(-k) = conj X(k)
          const int xs = gx - x, ys = (gy - y) % gy, zs = (gz - z) % gz;
          const size_t o = ((size_t)zs * gy + ys) * hx + xs;
          v = make_double2(h_half[2 * o], -h_half[2 * o + 1]);
        }
        h[((size_t)z * gy + y) * gx + x] = v;
      }
  double2* full = reinterpret_cast<double2*>(ctx->d_tmp);
  CK(cudaMemcpyAsync(full, h.data(), n * sizeof(double2), cudaMemcpyHostToDevice, s));
  const int gb = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
  k_f64_to_spec<T><<<gb, 256, 0, s>>>(full, I.spec, n);
  launch_s<T>(ctx, 0, 4);
  launch_s<T>(ctx, 0, 1);
  T* tp = reinterpret_cast<T*>(I.slices);
  XAux b{nullptr, tp, nullptr};
  launch_x<T>(ctx, 0, XM_S2R, b);
  k_convert<double, T><<<gb, 256, 0, s>>>(tp, d_prop, n);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s));
  return ADSCF_OK;
}

template <typename T>
int mix_e_t(adscf_ctx* ctx) {
  k_mix<T><<<ctx->mix_blocks, SCF_THREADS, 0, ctx->stream>>>(ctx->S, hb<T>(ctx).E, ctx->p.ds);
  CK(cudaGetLastError());
  return ADSCF_OK;
}

// new box side lengths: recompute the k-space tables in place (same sizes,
// same device buffers, so captured kernels keep valid pointers)
template <typename T>
int set_box_t(adscf_ctx* ctx) {
  std::vector<T> fk;
  std::vector<double> g64;
  int gxy_off = 0, gz_off = 0, g64_off = 0;
  bulkhost::append_tables<T>(ctx->gx, ctx->gy, ctx->gz, ctx->p.sizex, ctx->p.sizey, ctx->p.sizez,
                             ctx->p.ds, fk, g64, gxy_off, gz_off, g64_off);
  CK(cudaStreamSynchronize(ctx->stream));
  CK(cudaMemcpy(ctx->d_fk, fk.data(), fk.size() * sizeof(T), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(ctx->d_g64, g64.data(), g64.size() * sizeof(double), cudaMemcpyHostToDevice));
  return ADSCF_OK;
}

}  // namespace

int bulk_set_box(adscf_ctx* ctx) {
  return ctx->prec == ADSCF_SPLIT ? set_box_t<float>(ctx) : set_box_t<double>(ctx);
}

int bulk_create(adscf_ctx* ctx) {
  return ctx->prec == ADSCF_SPLIT ? create_t<float>(ctx) : create_t<double>(ctx);
}

void bulk_destroy(adscf_ctx* ctx) {
  if (ctx->prec == ADSCF_SPLIT) {
    cudaFree(ctx->hb32.spec); cudaFree(ctx->hb32.slices); cudaFree(ctx->hb32.E);
  } else {
    cudaFree(ctx->hb64.spec); cudaFree(ctx->hb64.slices); cudaFree(ctx->hb64.E);
  }
  cudaFree(ctx->d_wtab);
  cudaFree(ctx->d_inst); cudaFree(ctx->d_tw); cudaFree(ctx->d_fk);
  cudaFree(ctx->d_tw64); cudaFree(ctx->d_g64); cudaFree(ctx->d_flags); cudaFree(ctx->d_dcin);
  cudaFree(ctx->d_work_x); cudaFree(ctx->d_work_y); cudaFree(ctx->d_work_z);
  cudaFree(ctx->d_qpart);
}

static int slices_released(adscf_ctx* ctx) {
  return set_err(ctx, ADSCF_E_STATE, "the propagator slices are released while adjoint checkpointing is on");
}
int bulk_enqueue_propagate(adscf_ctx* ctx) {
  if (!ctx->slices_full) return slices_released(ctx);
  return ctx->prec == ADSCF_SPLIT ? propagate_t<float>(ctx) : propagate_t<double>(ctx);
}
int bulk_enqueue_chains(adscf_ctx* ctx) {
  if (!ctx->slices_full) return slices_released(ctx);
  return ctx->prec == ADSCF_SPLIT ? chains_t<float>(ctx) : chains_t<double>(ctx);
}
int bulk_enqueue_contour(adscf_ctx* ctx) {
  if (!ctx->slices_full) return slices_released(ctx);
  return ctx->prec == ADSCF_SPLIT ? contour_t<float>(ctx) : contour_t<double>(ctx);
}
// Slice storage of an FP64 context: all Ns + 1 nodes, or two nodes of scratch
// (the conversions of the single-step entry points stage through the slice
// buffer) while checkpointed adjoint passes recompute their nodes elsewhere.
// The new buffer is allocated before the old one is freed, so a failed
// allocation leaves the context as it was.
int bulk_hold_slices(adscf_ctx* ctx, bool full) {
  if (ctx->prec != ADSCF_FP64) return set_err(ctx, ADSCF_E_STATE, "slice release applies to FP64 contexts");
  if (full == ctx->slices_full) return ADSCF_OK;
  const size_t bytes = (size_t)(full ? ctx->ns + 1 : 2) * ctx->npts * sizeof(double2);
  double2* p = nullptr;
  CK(cudaStreamSynchronize(ctx->stream));
  if (cudaMalloc(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return set_err(ctx, ADSCF_E_OOM, "propagator slice storage");
  }
  cudaFree(ctx->hb64.slices);
  ctx->hb64.slices = p;
  CK(cudaMemcpy(ctx->d_inst, &ctx->hb64, sizeof(ctx->hb64), cudaMemcpyHostToDevice));
  ctx->slices_full = full;
  // captured graphs replay the full chains: capture again on next use
  if (ctx->g_iter) { cudaGraphExecDestroy(ctx->g_iter); ctx->g_iter = nullptr; }
  if (ctx->g_prop) { cudaGraphExecDestroy(ctx->g_prop); ctx->g_prop = nullptr; }
  return ADSCF_OK;
}
// bound of the TMA passes' pipeline waits (0: every wait gives up at once)
int bulk_set_wait_polls(adscf_ctx* ctx, int polls) {
  CK(cudaStreamSynchronize(ctx->stream));
  if (ctx->prec == ADSCF_SPLIT) {
    ctx->hb32.wait_polls = polls;
    CK(cudaMemcpy(ctx->d_inst, &ctx->hb32, sizeof(ctx->hb32), cudaMemcpyHostToDevice));
  } else {
    ctx->hb64.wait_polls = polls;
    CK(cudaMemcpy(ctx->d_inst, &ctx->hb64, sizeof(ctx->hb64), cudaMemcpyHostToDevice));
  }
  return ADSCF_OK;
}
int bulk_enqueue_expfield(adscf_ctx* ctx, const double* d_w) {
  return ctx->prec == ADSCF_SPLIT ? expfield_t<float>(ctx, d_w) : expfield_t<double>(ctx, d_w);
}
int bulk_step_single(adscf_ctx* ctx, double* d_prop, const double* d_e) {
  return ctx->prec == ADSCF_SPLIT ? step_single_t<float>(ctx, d_prop, d_e) : step_single_t<double>(ctx, d_prop, d_e);
}
int bulk_r2c(adscf_ctx* ctx, const double* d_prop, double* h_half) {
  return ctx->prec == ADSCF_SPLIT ? r2c_t<float>(ctx, d_prop, h_half) : r2c_t<double>(ctx, d_prop, h_half);
}
int bulk_c2r(adscf_ctx* ctx, const double* h_half, double* d_prop) {
  return ctx->prec == ADSCF_SPLIT ? c2r_t<float>(ctx, h_half, d_prop) : c2r_t<double>(ctx, h_half, d_prop);
}
int bulk_mix_e(adscf_ctx* ctx) {
  return ctx->prec == ADSCF_SPLIT ? mix_e_t<float>(ctx) : mix_e_t<double>(ctx);
}
