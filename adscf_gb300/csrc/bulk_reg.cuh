// bulk_reg.cuh -- register-FFT passes of the bulk propagator (power-of-two axes).
//
// Same pipeline and arithmetic as bulk_kernels.cuh (X, Yf, Z, Yi passes per
// double step), with every line transform held in registers (RegFFT): one
// in-warp exchange per 1D transform, power-of-two index arithmetic, and
// global loads/stores issued straight from the register distributions.
#pragma once
#include "bulk_kernels.cuh"
#include "fft_reg.cuh"

namespace regk {

template <int N>
struct Cfg;
template <> struct Cfg<24> { static constexpr int R1 = 12, TPL = 2; };
template <> struct Cfg<32> { static constexpr int R1 = 8, TPL = 4; };
template <> struct Cfg<40> { static constexpr int R1 = 20, TPL = 2; };
template <> struct Cfg<48> { static constexpr int R1 = 12, TPL = 4; };
template <> struct Cfg<64> { static constexpr int R1 = 8, TPL = 8; };
template <> struct Cfg<128> { static constexpr int R1 = 16, TPL = 8; };
template <> struct Cfg<256> { static constexpr int R1 = 16, TPL = 16; };

template <typename T, int N>
struct Layout {
  using F = RegFFT<T, Cfg<N>::R1, Cfg<N>::TPL>;
  static constexpr int LPC = BULK_THREADS / F::TPL;
  // shared memory: twiddles [N] | z factors hi,lo [2N] (T) | scratch [LPC*LS] | dc [N] double2
  static constexpr size_t tw_bytes = N * sizeof(cplx<T>);
  static constexpr size_t gz_bytes = 2 * N * sizeof(T);
  static constexpr size_t sc_off = ((tw_bytes + gz_bytes + 15) / 16) * 16;
  static constexpr size_t sc_bytes = (size_t)LPC * F::LS * sizeof(cplx<T>);
  static constexpr size_t dc_off = ((sc_off + sc_bytes + 15) / 16) * 16;
  static constexpr size_t bytes = dc_off + 3 * N * sizeof(float2);
};

__device__ __forceinline__ int ilog2(int v) { return __ffs(v) - 1; }
constexpr bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// line L = o * gx + x of a strided pass -> offset of its first point:
// shifts for power-of-two line lengths (with a power-of-two gx), a division
// for the others (cubic grids, gx = N)
template <int N>
__device__ __forceinline__ size_t line_base(int L, int gx, int lgx, size_t ostride) {
  if constexpr (pow2(N)) return (size_t)(L >> lgx) * ostride + (L & (gx - 1));
  else {
    const int o = L / gx;
    return (size_t)o * ostride + (L - o * gx);
  }
}

}  // namespace regk

// ---------------------------------------------------------------------------
// X pass (rows along x).  Modes as k_bulk_xpass.
// ---------------------------------------------------------------------------
template <typename T, int N>
__device__ __forceinline__ void rx_tile(const BulkDev<T>* __restrict__ insts, const int2 w,
                                        const cplx<T>* __restrict__ gtw, int t, int mode, XAux aux,
                                        unsigned char* smraw) {
  using LY = regk::Layout<T, N>;
  using F = typename LY::F;
  constexpr int R1 = F::R1, TPL = F::TPL, LPC = LY::LPC;
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smraw);
  cplx<T>* scr = reinterpret_cast<cplx<T>*>(smraw + LY::sc_off);
  const BulkDev<T>& I = insts[w.x];
  const int ns = I.ns;
  if (mode == XM_STEP && t > ns) return;
  const int npts = I.npts;
  const int nrows = I.gy * I.gz;
  const int tw_off = I.px.tw_off;
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = gtw[tw_off + i];
  __syncthreads();
  const int line = threadIdx.x / TPL, lt = threadIdx.x % TPL;
  const int row0 = w.y * LPC + line;
  const bool valid = row0 < nrows;
  const int row = valid ? row0 : nrows - 1;
  cplx<T>* sc = scr + line * F::LS;
  const size_t base = (size_t)row * N;
  cplx<T>* spec = I.spec;
  cplx<T> v[R1];

  if (mode == XM_INIT || mode == XM_R2S) {
    if (mode == XM_INIT) {
      const bool fA = chain_type_fwd(I, 1) == 0, bA = chain_type_bwd(I, 1) == 0;
      cplx<T>* s0 = I.slices;
#pragma unroll
      for (int m = 0; m < R1; ++m) {
        const size_t g = base + F::in_index(lt, m);
        const EPt<T> ev = load_ept(I.E, g);
        v[m] = mk<T>(fA ? ev.a : ev.b, bA ? ev.a : ev.b);
        if (valid) s0[g] = mk<T>((T)1, (T)1);
      }
    } else {
      const T* in = static_cast<const T*>(aux.in);
      const T* ee = static_cast<const T*>(aux.e);
#pragma unroll
      for (int m = 0; m < R1; ++m) {
        const size_t g = base + F::in_index(lt, m);
        T x = in[g];
        if (ee) x *= ee[g];
        v[m] = mk<T>(x, (T)0);
      }
    }
    F::forward(v, sc, tw, lt);
    if (valid) {
#pragma unroll
      for (int r = 0; r < R1; ++r) spec[base + F::out_index(lt, r)] = v[r];
    }
    return;
  }
  // XM_STEP / XM_S2R: inverse x of the spectrum row
#pragma unroll
  for (int r = 0; r < R1; ++r) v[r] = spec[base + F::out_index(lt, r)];
  F::inverse(v, sc, tw, lt);
  if (mode == XM_S2R) {
    T* out = static_cast<T*>(aux.out);
    const T* ee = static_cast<const T*>(aux.e);
    if (valid) {
#pragma unroll
      for (int m = 0; m < R1; ++m) {
        const size_t g = base + F::in_index(lt, m);
        T x = v[m].x;
        if (ee) x *= ee[g];
        out[g] = x;
      }
    }
    return;
  }
  // A or B factor per chain and step (forward A then B, backward B then A)
  const bool fA = chain_type_fwd(I, t) == 0, bA = chain_type_bwd(I, t) == 0;
  const bool more = t < ns;
  const bool fA2 = chain_type_fwd(I, t + 1) == 0, bA2 = chain_type_bwd(I, t + 1) == 0;
  cplx<T>* sl = I.slices + (size_t)t * npts;
#pragma unroll
  for (int m = 0; m < R1; ++m) {
    const size_t g = base + F::in_index(lt, m);
    const EPt<T> ev = load_ept(I.E, g);
    const cplx<T> q = mk<T>(emul(v[m].x, fA ? ev.a : ev.b, fA ? ev.al : ev.bl),
                            emul(v[m].y, bA ? ev.a : ev.b, bA ? ev.al : ev.bl));
    if (valid) sl[g] = q;
    if (more)
      v[m] = mk<T>(emul(q.x, fA2 ? ev.a : ev.b, fA2 ? ev.al : ev.bl),
                   emul(q.y, bA2 ? ev.a : ev.b, bA2 ? ev.al : ev.bl));
  }
  if (!more) return;
  F::forward(v, sc, tw, lt);
  if (valid) {
#pragma unroll
    for (int r = 0; r < R1; ++r) spec[base + F::out_index(lt, r)] = v[r];
  }
}

template <typename T, int N>
__global__ void __launch_bounds__(BULK_THREADS)
k_rx(const BulkDev<T>* __restrict__ insts, const int2* __restrict__ work,
     const cplx<T>* __restrict__ gtw, int t, int mode, XAux aux) {
  extern __shared__ __align__(16) unsigned char smraw[];
  rx_tile<T, N>(insts, work[blockIdx.x], gtw, t, mode, aux, smraw);
}

// ---------------------------------------------------------------------------
// Strided passes (Y: KIND 0 fwd / 1 inv; Z: KIND 2 fwd*G*inv, 3 fwd, 4 inv).
// Flattened lines L = o*gx + x; LPC consecutive lines per CTA.
// ---------------------------------------------------------------------------
template <typename T, int N, int KIND>
__device__ __forceinline__ void rs_tile(const BulkDev<T>* __restrict__ insts, const int2 w,
                                        const cplx<T>* __restrict__ gtw, const T* __restrict__ fk,
                                        const double2* __restrict__ gtw64,
                                        const double* __restrict__ g64, int t, unsigned char* smraw) {
  using LY = regk::Layout<T, N>;
  using F = typename LY::F;
  constexpr int R1 = F::R1, TPL = F::TPL, LPC = LY::LPC;
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smraw);
  T* gzs = reinterpret_cast<T*>(smraw + LY::tw_bytes);
  cplx<T>* scr = reinterpret_cast<cplx<T>*>(smraw + LY::sc_off);
  const BulkDev<T>& I = insts[w.x];
  if (t > I.ns) return;
  constexpr bool zdir = KIND >= 2;
  const int gx = I.gx, gy = I.gy;
  const int lgx = regk::ilog2(gx);
  const int tw_off = zdir ? I.pz.tw_off : I.py.tw_off;
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = gtw[tw_off + i];
  if constexpr (KIND == 2) {
    const T* gzt = fk + I.gz_off;
    for (int i = threadIdx.x; i < 2 * N; i += blockDim.x) gzs[i] = gzt[i];
  }
  __syncthreads();
  const int nlines = gx * (zdir ? gy : I.gz);
  const int line = threadIdx.x / TPL, lt = threadIdx.x % TPL;
  const int L0 = w.y * LPC;
  const int Lr = L0 + line;
  const bool valid = Lr < nlines;
  const int L = valid ? Lr : nlines - 1;
  const size_t es = zdir ? (size_t)gx * gy : (size_t)gx;
  const size_t ostride = zdir ? (size_t)gx : (size_t)gx * gy;
  const size_t base = regk::line_base<N>(L, gx, lgx, ostride);
  cplx<T>* sc = scr + line * F::LS;
  cplx<T>* spec = I.spec;
  cplx<T> v[R1];
  constexpr bool in_dout = (KIND == 1 || KIND == 4);  // inverse-only passes start in D_out
  if constexpr (in_dout) {
#pragma unroll
    for (int r = 0; r < R1; ++r) v[r] = spec[base + (size_t)F::out_index(lt, r) * es];
    F::inverse(v, sc, tw, lt);
#pragma unroll
    for (int m = 0; m < R1; ++m)
      if (valid) spec[base + (size_t)F::in_index(lt, m) * es] = v[m];
    return;
  }
  // (0, 0) pencil in float-float (CTA of tile 0), read before it is overwritten
  constexpr bool dc64 = sizeof(T) == 4 && KIND == 2;
  const bool dcline = dc64 && L0 == 0;
  float2* dcf = reinterpret_cast<float2*>(smraw + LY::dc_off);
  const DcPencil dcp{dcf, dcf + N, dcf + 2 * N};
  if (dcline) {
    dc_pencil_load<T>(spec, es, N, g64 + I.g64_off, dcp);
    __syncthreads();
    dc_pencil_apply(N, dcp);
  }
#pragma unroll
  for (int m = 0; m < R1; ++m) v[m] = spec[base + (size_t)F::in_index(lt, m) * es];
  F::forward(v, sc, tw, lt);
  if constexpr (KIND == 0 || KIND == 3) {
    if (valid) {
#pragma unroll
      for (int r = 0; r < R1; ++r) spec[base + (size_t)F::out_index(lt, r) * es] = v[r];
    }
    return;
  }
  // exp(-ds k^2)/N, one rounding (compensated hi/lo product in FP32)
  if constexpr (KIND == 2) {
    const T* gxy = fk + I.gxy_off;
    const int nxy = gx * gy;
    const T ah = gxy[L];
    const T al = gxy[nxy + L];
#pragma unroll
    for (int r = 0; r < R1; ++r) {
      const int kz = F::out_index(lt, r);
      if constexpr (sizeof(T) == 4) {
        const float bh = gzs[kz], bl = gzs[N + kz];
        const float gh = ah * bh;
        const float gl = fmaf(ah, bh, -gh) + fmaf(ah, bl, al * bh);
        v[r] = mk<T>(fmaf(v[r].x, gh, v[r].x * gl), fmaf(v[r].y, gh, v[r].y * gl));
      } else {
        const T f = ah * gzs[kz];
        v[r] = mk<T>(v[r].x * f, v[r].y * f);
      }
    }
  }
  F::inverse(v, sc, tw, lt);
  if (valid) {
#pragma unroll
    for (int m = 0; m < R1; ++m) spec[base + (size_t)F::in_index(lt, m) * es] = v[m];
  }
  if (dcline) {
    __syncthreads();
    dc_pencil_store<T>(spec, es, N, dcp);
  }
}

template <typename T, int N, int KIND>
__global__ void __launch_bounds__(BULK_THREADS, KIND == 2 ? 2 : 3)
k_rs(const BulkDev<T>* __restrict__ insts, const int2* __restrict__ work,
     const cplx<T>* __restrict__ gtw, const T* __restrict__ fk,
     const double2* __restrict__ gtw64, const double* __restrict__ g64, int t) {
  extern __shared__ __align__(16) unsigned char smraw[];
  rs_tile<T, N, KIND>(insts, work[blockIdx.x], gtw, fk, gtw64, g64, t, smraw);
}

// ---------------------------------------------------------------------------
// Persistent, software-pipelined variants (one instance, power-of-two axes):
// each CTA walks tiles blockIdx.x, blockIdx.x + gridDim.x, ... and loads the
// next tile's registers before transforming the current one, so the memory
// latency of tile i+1 overlaps the FFT of tile i.
// ---------------------------------------------------------------------------
template <typename T, int N, int KIND>
__global__ void __launch_bounds__(BULK_THREADS, 2)
k_rs_p(const BulkDev<T>* __restrict__ insts, int ntiles, const cplx<T>* __restrict__ gtw,
       const T* __restrict__ fk, const double2* __restrict__ gtw64,
       const double* __restrict__ g64, int t) {
  using LY = regk::Layout<T, N>;
  using F = typename LY::F;
  constexpr int R1 = F::R1, TPL = F::TPL, LPC = LY::LPC;
  constexpr bool zdir = KIND >= 2;
  constexpr bool in_dout = (KIND == 1);
  constexpr bool out_dout = (KIND == 0);
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smraw);
  T* gzs = reinterpret_cast<T*>(smraw + LY::tw_bytes);
  cplx<T>* scr = reinterpret_cast<cplx<T>*>(smraw + LY::sc_off);
  const BulkDev<T>& I = insts[0];
  if (t > I.ns) return;
  const int gx = I.gx, gy = I.gy;
  const int lgx = regk::ilog2(gx);
  const int tw_off = zdir ? I.pz.tw_off : I.py.tw_off;
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = gtw[tw_off + i];
  if constexpr (KIND == 2) {
    const T* gzt = fk + I.gz_off;
    for (int i = threadIdx.x; i < 2 * N; i += blockDim.x) gzs[i] = gzt[i];
  }
  __syncthreads();
  const int nlines = gx * (zdir ? gy : I.gz);
  const int line = threadIdx.x / TPL, lt = threadIdx.x % TPL;
  const size_t es = zdir ? (size_t)gx * gy : (size_t)gx;
  const size_t ostride = zdir ? (size_t)gx : (size_t)gx * gy;
  cplx<T>* sc = scr + line * F::LS;
  cplx<T>* spec = I.spec;
  const T* gxy = fk + I.gxy_off;
  auto line_of = [&](int tile) { return min(tile * LPC + line, nlines - 1); };
  auto base_of = [&](int L) { return (size_t)(L >> lgx) * ostride + (L & (gx - 1)); };
  // (0, 0) pencil in float-float: read before CTA 0 overwrites it (tile 0)
  constexpr bool dc64 = sizeof(T) == 4 && KIND == 2;
  float2* dcf = reinterpret_cast<float2*>(smraw + LY::dc_off);
  const DcPencil dcp{dcf, dcf + N, dcf + 2 * N};
  const bool dcblk = dc64 && blockIdx.x == 0;
  if (dcblk) {
    dc_pencil_load<T>(spec, es, N, g64 + I.g64_off, dcp);
    __syncthreads();
    dc_pencil_apply(N, dcp);
  }
  cplx<T> nx[R1];
  int tile = blockIdx.x;
  if (tile < ntiles) {
    const size_t b = base_of(line_of(tile));
#pragma unroll
    for (int r = 0; r < R1; ++r)
      nx[r] = spec[b + (size_t)(in_dout ? F::out_index(lt, r) : F::in_index(lt, r)) * es];
  }
  for (; tile < ntiles; tile += gridDim.x) {
    const int Lr = tile * LPC + line;
    const bool valid = Lr < nlines;
    const int L = valid ? Lr : nlines - 1;
    const size_t base = base_of(L);
    cplx<T> v[R1];
#pragma unroll
    for (int r = 0; r < R1; ++r) v[r] = nx[r];
    const int nxt = tile + gridDim.x;
    if (nxt < ntiles) {
      const size_t b = base_of(line_of(nxt));
#pragma unroll
      for (int r = 0; r < R1; ++r)
        nx[r] = spec[b + (size_t)(in_dout ? F::out_index(lt, r) : F::in_index(lt, r)) * es];
    }
    if constexpr (KIND == 1) {
      F::inverse(v, sc, tw, lt);
    } else if constexpr (KIND == 0) {
      F::forward(v, sc, tw, lt);
    } else {
      F::forward(v, sc, tw, lt);
      const T ah = gxy[L];
      const T al = gxy[gx * gy + L];
#pragma unroll
      for (int r = 0; r < R1; ++r) {
        const int kz = F::out_index(lt, r);
        if constexpr (sizeof(T) == 4) {
          const float bh = gzs[kz], bl = gzs[N + kz];
          const float gh = ah * bh;
          const float gl = fmaf(ah, bh, -gh) + fmaf(ah, bl, al * bh);
          v[r] = mk<T>(fmaf(v[r].x, gh, v[r].x * gl), fmaf(v[r].y, gh, v[r].y * gl));
        } else {
          const T f = ah * gzs[kz];
          v[r] = mk<T>(v[r].x * f, v[r].y * f);
        }
      }
      F::inverse(v, sc, tw, lt);
    }
    if (valid) {
#pragma unroll
      for (int r = 0; r < R1; ++r)
        spec[base + (size_t)(out_dout ? F::out_index(lt, r) : F::in_index(lt, r)) * es] = v[r];
    }
  }
  if (dcblk) {
    __syncthreads();
    dc_pencil_store<T>(spec, es, N, dcp);
  }
}

// X pass, XM_STEP only, persistent with the next spectrum row prefetched
template <typename T, int N>
__global__ void __launch_bounds__(BULK_THREADS, 2)
k_rx_p(const BulkDev<T>* __restrict__ insts, int ntiles, const cplx<T>* __restrict__ gtw, int t) {
  using LY = regk::Layout<T, N>;
  using F = typename LY::F;
  constexpr int R1 = F::R1, TPL = F::TPL, LPC = LY::LPC;
  extern __shared__ __align__(16) unsigned char smraw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smraw);
  cplx<T>* scr = reinterpret_cast<cplx<T>*>(smraw + LY::sc_off);
  const BulkDev<T>& I = insts[0];
  const int ns = I.ns;
  if (t > ns) return;
  const int npts = I.npts;
  const int nrows = I.gy * I.gz;
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = gtw[I.px.tw_off + i];
  __syncthreads();
  const int line = threadIdx.x / TPL, lt = threadIdx.x % TPL;
  cplx<T>* sc = scr + line * F::LS;
  cplx<T>* spec = I.spec;
  // A or B factor per chain and step (forward A then B, backward B then A)
  const bool fA = chain_type_fwd(I, t) == 0, bA = chain_type_bwd(I, t) == 0;
  const bool more = t < ns;
  const bool fA2 = chain_type_fwd(I, t + 1) == 0, bA2 = chain_type_bwd(I, t + 1) == 0;
  cplx<T>* sl = I.slices + (size_t)t * npts;
  cplx<T> nx[R1];
  int tile = blockIdx.x;
  if (tile < ntiles) {
    const size_t b = (size_t)min(tile * LPC + line, nrows - 1) * N;
#pragma unroll
    for (int r = 0; r < R1; ++r) nx[r] = spec[b + F::out_index(lt, r)];
  }
  for (; tile < ntiles; tile += gridDim.x) {
    const int row0 = tile * LPC + line;
    const bool valid = row0 < nrows;
    const size_t base = (size_t)(valid ? row0 : nrows - 1) * N;
    cplx<T> v[R1];
#pragma unroll
    for (int r = 0; r < R1; ++r) v[r] = nx[r];
    const int nxt = tile + gridDim.x;
    if (nxt < ntiles) {
      const size_t b = (size_t)min(nxt * LPC + line, nrows - 1) * N;
#pragma unroll
      for (int r = 0; r < R1; ++r) nx[r] = spec[b + F::out_index(lt, r)];
    }
    F::inverse(v, sc, tw, lt);
#pragma unroll
    for (int m = 0; m < R1; ++m) {
      const size_t g = base + F::in_index(lt, m);
      const EPt<T> ev = load_ept(I.E, g);
      const cplx<T> q = mk<T>(emul(v[m].x, fA ? ev.a : ev.b, fA ? ev.al : ev.bl),
                              emul(v[m].y, bA ? ev.a : ev.b, bA ? ev.al : ev.bl));
      if (valid) sl[g] = q;
      if (more)
        v[m] = mk<T>(emul(q.x, fA2 ? ev.a : ev.b, fA2 ? ev.al : ev.bl),
                     emul(q.y, bA2 ? ev.a : ev.b, bA2 ? ev.al : ev.bl));
    }
    if (!more) continue;
    F::forward(v, sc, tw, lt);
    if (valid) {
#pragma unroll
      for (int r = 0; r < R1; ++r) spec[base + F::out_index(lt, r)] = v[r];
    }
  }
}
