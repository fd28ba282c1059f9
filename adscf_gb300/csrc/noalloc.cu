// noalloc.cu -- allocation-free variant of the bulk propagator step.
//
// Who needs it: callers that must not allocate device memory on the hot path
// -- a host whose memory is fully pre-partitioned between tenants, a Fortran
// driver that hands the library device buffers it owns, or code that runs
// where a cudaMalloc would synchronise the device or fail under a memory
// quota.  adscf_propagate_step_noalloc does one FP64 Propagate_Step on the
// caller's device buffers and takes every piece of working memory (plan,
// tables, work lists, spectrum) from one file-scope static device array of
// fixed size.
//
// The array belongs to the loaded library: it is reserved on a device when
// the library's device code is loaded there -- with CUDA's default lazy
// module loading, at the first call on that device -- and held until the
// process exits.  A caller on a tightly budgeted GPU should therefore make
// one call during its set-up (or run with CUDA_MODULE_LOADING=EAGER); when
// the reservation fails the call returns ADSCF_E_OOM.  All calls on one
// device share the array and it keeps the last call's contents, so two calls
// whose kernels overlap on the GPU (different streams without ordering, or
// different host threads) race and corrupt each other.  Calls must be
// ordered on the device, e.g. issued to one stream.
//
// Set-up and table rebuilds: the first call on each device takes the array's
// device address with cudaGetSymbolAddress (with that device current) and
// raises the shared-memory limit of the FFT kernels; a call with a new grid,
// box or ds rewrites the plan, tables and work lists in the array and
// synchronises its stream.  Both return ADSCF_E_STATE instead when the
// stream is capturing, so make the first call, and every call with new
// parameters, before any stream capture.  A rewrite replaces the tables that
// work enqueued or recorded earlier will read when it runs.
#include <cmath>
#include <cstring>
#include <mutex>

#include "internal.h"
#include "bulk_host.h"

// sizes the static scratch is laid out for
#define NOALLOC_MAX_POINTS 262144   // e.g. 64^3
#define NOALLOC_MAX_LINE 512        // longest axis
#define NOALLOC_MAX_PLANE 65536     // gx*gy
#define NOALLOC_MAX_TILES 65536     // work-list entries per pass

namespace {

constexpr size_t kInstBytes = 1024;
constexpr size_t kWorkBytes = 3 * (size_t)NOALLOC_MAX_TILES * sizeof(int2);
constexpr size_t kTwBytes = 3 * (size_t)NOALLOC_MAX_LINE * sizeof(double2);
constexpr size_t kFkBytes = (2 * (size_t)NOALLOC_MAX_PLANE + 2 * NOALLOC_MAX_LINE) * sizeof(double);
constexpr size_t kSpecBytes = (size_t)NOALLOC_MAX_POINTS * sizeof(double2);
constexpr size_t kOffWork = kInstBytes;
constexpr size_t kOffTw = kOffWork + kWorkBytes;
constexpr size_t kOffFk = kOffTw + kTwBytes;
constexpr size_t kOffSpec = ((kOffFk + kFkBytes + 255) / 256) * 256;
constexpr size_t kTotal = kOffSpec + kSpecBytes;
// the instance header sits in front of the work lists
static_assert(sizeof(BulkDev<double>) <= kInstBytes, "BulkDev<double> outgrew its scratch slot");
static_assert(kInstBytes % alignof(int2) == 0 && kInstBytes % alignof(BulkDev<double>) == 0,
              "work lists and header must stay aligned");

}  // namespace

#define ADSCF_NOALLOC_SCRATCH_BYTES kTotal

// The scratch itself.  Host code must never hand this symbol to a kernel:
// on the host it names a stand-in, not device memory; its device address
// comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kTotal];

namespace {

struct DevState {
  bool ready = false;
  unsigned char* base = nullptr;  // device address of g_noalloc_scratch
  // parameters the tables currently in the array were built for
  int gx = 0, gy = 0, gz = 0;
  double lx = 0, ly = 0, lz = 0, ds = 0;
  int nwx = 0, nwy = 0, nwz = 0;
  size_t smx = 0, smy = 0, smz = 0;
};

std::mutex g_mu;
DevState g_dev[64];
// host staging for the tables (file scope, so a call allocates nothing)
double2 h_tw[3 * NOALLOC_MAX_LINE];
double h_fk[2 * (size_t)NOALLOC_MAX_PLANE + 2 * NOALLOC_MAX_LINE];
int2 h_work[3 * (size_t)NOALLOC_MAX_TILES];

// (re)build plan, tables and work lists inside the scratch for this problem
int build_tables(DevState& D, int gx, int gy, int gz, double lx, double ly, double lz,
                 double ds, cudaStream_t s) {
  BulkDev<double> I{};
  I.gx = gx; I.gy = gy; I.gz = gz;
  I.npts = gx * gy * gz;
  I.ns = 0; I.na = 0; I.nb = 0;
  if (!bulkhost::make_plan(gx, I.px) || !bulkhost::make_plan(gy, I.py) || !bulkhost::make_plan(gz, I.pz)) return ADSCF_E_ARG;
  const int ns3[3] = {gx, gy, gz};
  int offs[3];
  int ntw = 0;
  for (int d = 0; d < 3; ++d) {
    offs[d] = ntw;
    for (int m = 0; m < ns3[d]; ++m) {
      const double a = -2.0 * M_PI * (double)m / (double)ns3[d];
      h_tw[ntw++] = make_double2(std::cos(a), std::sin(a));
    }
  }
  I.px.tw_off = offs[0]; I.py.tw_off = offs[1]; I.pz.tw_off = offs[2];
  const int nxy = gx * gy;
  double* fk = h_fk;
  const size_t nfk = 2 * (size_t)nxy + 2 * (size_t)gz;
  std::memset(fk, 0, nfk * sizeof(double));
  I.gxy_off = 0;
  I.gz_off = 2 * nxy;
  for (int y = 0; y < gy; ++y) {
    const double ky = bulkhost::wavenum(y, gy, ly);
    for (int x = 0; x < gx; ++x) {
      const double kx = bulkhost::wavenum(x, gx, lx);
      fk[(size_t)y * gx + x] = std::exp(-ds * kx * kx) * std::exp(-ds * ky * ky);
    }
  }
  const double invn = 1.0 / ((double)gx * gy * gz);
  for (int z = 0; z < gz; ++z) {
    const double kz = bulkhost::wavenum(z, gz, lz);
    fk[I.gz_off + z] = std::exp(-ds * kz * kz) * invn;
  }
  I.tw64_off = 0;
  I.g64_off = 0;
  I.spec = reinterpret_cast<double2*>(D.base + kOffSpec);
  I.slices = nullptr;
  I.E = nullptr;
  const int nwx = (gy * gz + I.px.lpc - 1) / I.px.lpc;
  const int nwy = (gx * gz + I.py.lpc - 1) / I.py.lpc;
  const int nwz = (gx * gy + I.pz.lpc - 1) / I.pz.lpc;
  if (nwx > NOALLOC_MAX_TILES || nwy > NOALLOC_MAX_TILES || nwz > NOALLOC_MAX_TILES) return ADSCF_E_TOO_LARGE;
  int2* work = h_work;
  for (int i = 0; i < nwx; ++i) work[i] = make_int2(0, i);
  for (int i = 0; i < nwy; ++i) work[NOALLOC_MAX_TILES + i] = make_int2(0, i);
  for (int i = 0; i < nwz; ++i) work[2 * (size_t)NOALLOC_MAX_TILES + i] = make_int2(0, i);
  if (cudaMemcpyAsync(D.base, &I, sizeof(I), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(D.base + kOffWork, work, 3 * (size_t)NOALLOC_MAX_TILES * sizeof(int2), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(D.base + kOffTw, h_tw, ntw * sizeof(double2), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(D.base + kOffFk, fk, nfk * sizeof(double), cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return ADSCF_E_CUDA;
  D.gx = gx; D.gy = gy; D.gz = gz; D.lx = lx; D.ly = ly; D.lz = lz; D.ds = ds;
  D.nwx = nwx; D.nwy = nwy; D.nwz = nwz;
  D.smx = bulkhost::plan_smem<double>(I.px);
  D.smy = bulkhost::plan_smem<double>(I.py);
  D.smz = bulkhost::plan_smem<double>(I.pz);
  return ADSCF_OK;
}

}  // namespace

extern "C" int adscf_propagate_step_noalloc(int gx, int gy, int gz, double sizex, double sizey,
                                            double sizez, double ds, double* d_prop,
                                            const double* d_expfield, void* stream) {
  if (!d_prop || !d_expfield || gx < 1 || gy < 1 || gz < 1 || !(ds > 0) ||
      !(sizex > 0 && sizey > 0 && sizez > 0))
    return ADSCF_E_ARG;
  if ((long long)gx * gy * gz > NOALLOC_MAX_POINTS || gx > NOALLOC_MAX_LINE ||
      gy > NOALLOC_MAX_LINE || gz > NOALLOC_MAX_LINE || (long long)gx * gy > NOALLOC_MAX_PLANE)
    return ADSCF_E_TOO_LARGE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return ADSCF_E_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::lock_guard<std::mutex> lock(g_mu);
  DevState& D = g_dev[dev];
  const bool rebuild = D.gx != gx || D.gy != gy || D.gz != gz || D.lx != sizex ||
                       D.ly != sizey || D.lz != sizez || D.ds != ds;
  if (!D.ready || rebuild) {
    // set-up and table rebuilds synchronise the stream: not while it captures
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) return ADSCF_E_CUDA;
    if (cs != cudaStreamCaptureStatusNone) return ADSCF_E_STATE;
  }
  if (!D.ready) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e == cudaErrorMemoryAllocation) {
      cudaGetLastError();
      return ADSCF_E_OOM;   // the array could not be reserved on this device
    }
    if (e != cudaSuccess || !p) return ADSCF_E_CUDA;
    D.base = static_cast<unsigned char*>(p);
    if (cudaFuncSetAttribute(k_bulk_xpass<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) != cudaSuccess ||
        cudaFuncSetAttribute(k_bulk_strided<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) != cudaSuccess)
      return ADSCF_E_CUDA;
    D.ready = true;
  }
  if (rebuild) {
    D.gx = 0;  // tables invalid until rebuilt
    const int rc = build_tables(D, gx, gy, gz, sizex, sizey, sizez, ds, s);
    if (rc) return rc;
  }
  if (D.smx > 227 * 1024 || D.smy > 227 * 1024 || D.smz > 227 * 1024) return ADSCF_E_TOO_LARGE;
  const BulkDev<double>* inst = reinterpret_cast<const BulkDev<double>*>(D.base);
  const int2* wx = reinterpret_cast<const int2*>(D.base + kOffWork);
  const int2* wy = wx + NOALLOC_MAX_TILES;
  const int2* wz = wx + 2 * NOALLOC_MAX_TILES;
  const double2* tw = reinterpret_cast<const double2*>(D.base + kOffTw);
  const double* fk = reinterpret_cast<const double*>(D.base + kOffFk);
  // prop <- E IFFT(exp(-ds k^2) FFT(E prop)) (mod_propagate.f90:56-64)
  XAux a{d_prop, nullptr, d_expfield};
  k_bulk_xpass<double><<<D.nwx, BULK_THREADS, D.smx, s>>>(inst, wx, tw, 0, XM_R2S, a);
  k_bulk_strided<double><<<D.nwy, BULK_THREADS, D.smy, s>>>(inst, wy, tw, fk, nullptr, nullptr, 0, 0);
  k_bulk_strided<double><<<D.nwz, BULK_THREADS, D.smz, s>>>(inst, wz, tw, fk, nullptr, nullptr, 0, 2);
  k_bulk_strided<double><<<D.nwy, BULK_THREADS, D.smy, s>>>(inst, wy, tw, fk, nullptr, nullptr, 0, 1);
  XAux b{nullptr, d_prop, d_expfield};
  k_bulk_xpass<double><<<D.nwx, BULK_THREADS, D.smx, s>>>(inst, wx, tw, 0, XM_S2R, b);
  return cudaGetLastError() == cudaSuccess ? ADSCF_OK : ADSCF_E_CUDA;
}
