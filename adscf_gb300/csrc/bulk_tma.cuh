// bulk_tma.cuh -- TMA-fed strided passes (Y and Z) of the FP32 bulk propagator.
//
// The strided passes read and write lines that run across rows of the
// spectrum; issued from the threads, every warp access touches eight rows and
// the L1/LSU pipe becomes the limit.  Here the tiles move between global and
// shared memory by TMA (cp.async.bulk.tensor), off the LSU pipe:
//   - a tile is LPC = 32 consecutive x-lines x N points, fetched as two
//     16-line boxes {16, N, 1} (Y) or {16, 1, N} (Z) of 8-byte complex values;
//   - boxes land 128-byte swizzled: the 16-byte chunk index of row j is XORed
//     with j mod 8, so the eight lanes of one line (rows t + 8m) hit eight
//     different chunks -- conflict-free column reads;
//   - persistent CTAs run a two-stage pipeline: thread 0 prefetches tile i+1
//     (mbarrier with transaction bytes) while the CTA transforms tile i in
//     registers (RegFFT), writes it back in place and TMA-stores it;
//   - every mbarrier wait is bounded; on expiry the CTA sets an error flag,
//     drains its bulk copies and returns (no hang).
#pragma once
#include <cuda.h>

#include "bulk_reg.cuh"

namespace tmak {

// prefetch the 128-byte line holding p into L1 (a hint: no register, no wait)
__device__ __forceinline__ void prefetch_l1(const void* p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}


__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: false when the phase did not complete within `limit` polls
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int limit) {
  for (int i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x,
                                            int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, const void* src, int x, int y,
                                             int z) {
  asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(map),
               "r"(x), "r"(y), "r"(z), "r"(smem_u32(src))
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read0() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// Programmatic dependent launch: the two passes of a double step are launched
// with programmatic stream serialisation, so the next pass's CTAs may start
// (and load their constant tables) while this one finishes.  launch_dependents
// lets them start; wait blocks until the previous grid has completed and its
// memory is visible.  Without such a launch both return at once.
__device__ __forceinline__ void pdl_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// element offset of (row j, column c) in a 16-column box with 128-byte swizzle
__device__ __forceinline__ int swz(int j, int c) {
  return j * 16 + ((((c >> 1) ^ (j & 7)) << 1) | (c & 1));
}

// One output z of the float-float (0, 0) pencil convolution
// sum_d c[d] in[z - d mod n] that a z pass's pencil CTA evaluates for all z
// (dc_pencil_apply).  Lanes 0-7 of the calling
// warp run the eight real-part chains ((d mod 8) = lane), lanes 8-15 the
// imaginary ones, each summing its terms in increasing d; the chains are then
// combined pairwise as ((0+1) + (2+3)) + ((4+5) + (6+7)) -- the operations
// of the pencil CTA in the same order, so the result is bit for bit the
// same.  Every lane of the warp calls it; the value is returned in lane 0.
__device__ __forceinline__ float2 dc_point(const float2* in, const float2* c, int n, int z) {
  const int lane = threadIdx.x & 31;
  const int u = lane & (kDcChains - 1);
  const bool im = lane & kDcChains;
  float sh = 0.f, sl = 0.f;
  if (lane < 2 * kDcChains) {
    for (int d = u; d < n; d += kDcChains) {
      int zz = z - d;
      if (zz < 0) zz += n;
      const float2 p = in[zz];
      const float2 cc = c[d];
      ff_fma(sh, sl, cc.x, cc.y, im ? p.y : p.x);
    }
  }
#pragma unroll
  for (int st = 1; st < kDcChains; st *= 2) {
    const float oh = __shfl_down_sync(0xffffffffu, sh, st);
    const float ol = __shfl_down_sync(0xffffffffu, sl, st);
    if ((u & (2 * st - 1)) == 0) ff_add(sh, sl, oh, ol);
  }
  const float r = sh + sl;
  const float ri = __shfl_down_sync(0xffffffffu, r, kDcChains);
  return make_float2(r, ri);
}

constexpr int kBoxCols = 16;           // 16 x 8 B = 128 B inner box
// default bound of one pipeline mbarrier wait (BulkDev::wait_polls, settable
// per context) and the fixed bound of the drain waits at kernel exit
constexpr int kWaitPolls = 1 << 22;

template <int N>
struct TmaLayout {
  using F = RegFFT<float, regk::Cfg<N>::R1, regk::Cfg<N>::TPL>;
  static constexpr int LPC = BULK_THREADS / F::TPL;     // lines per tile
  static constexpr int NB = LPC / kBoxCols;             // boxes per tile
  static constexpr int box_elems = N * kBoxCols;
  static constexpr int tile_elems = NB * box_elems;
  static constexpr uint32_t tile_bytes = tile_elems * 8;
  // [buf0 | buf1] (1024-aligned) | twiddles N | z factors 2N | exchange | dc 3N | 2 barriers
  static constexpr size_t buf_off = 0;
  static constexpr size_t tw_off = 2 * (size_t)tile_bytes;
  static constexpr size_t gz_off = tw_off + N * sizeof(float2);
  static constexpr size_t ex_off = ((gz_off + 2 * N * sizeof(float) + 15) / 16) * 16;
  static constexpr size_t dc_off = ex_off + (size_t)LPC * F::LS * sizeof(float2);
  static constexpr size_t bar_off = ((dc_off + 3 * N * sizeof(float2) + 15) / 16) * 16;
  static constexpr size_t bytes = bar_off + 2 * sizeof(uint64_t) + 1024;  // + alignment slack
  static_assert(LPC % kBoxCols == 0, "tile must be whole boxes");
};

}  // namespace tmak

// KIND 0: forward y, 1: inverse y, 2: z (forward, exp(-ds k^2)/N, inverse).
// One instance, gx a multiple of 32, every line length N.
template <int N, int KIND>
__global__ void __launch_bounds__(BULK_THREADS, 2)
k_rs_tma(const BulkDev<float>* __restrict__ insts, const __grid_constant__ CUtensorMap tmap,
         int ntiles, const float2* __restrict__ gtw, const float* __restrict__ fk,
         const double* __restrict__ g64, int t, int dc, const float2* __restrict__ dcin,
         float2* __restrict__ dcout, int* __restrict__ err) {
  using LY = tmak::TmaLayout<N>;
  using F = typename LY::F;
  constexpr int R1 = F::R1, TPL = F::TPL, LPC = LY::LPC;
  constexpr bool zdir = KIND == 2;
  constexpr bool in_dout = KIND == 1;
  constexpr bool out_dout = KIND == 0;
  extern __shared__ __align__(1024) unsigned char smraw_[];
  // 1024-byte alignment of the swizzled boxes
  unsigned char* smraw = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smraw_) + 1023) & ~uintptr_t(1023));
  float2* buf = reinterpret_cast<float2*>(smraw + LY::buf_off);
  float2* tw = reinterpret_cast<float2*>(smraw + LY::tw_off);
  float* gzs = reinterpret_cast<float*>(smraw + LY::gz_off);
  float2* ex = reinterpret_cast<float2*>(smraw + LY::ex_off);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smraw + LY::bar_off);
  const BulkDev<float>& I = insts[0];
  if (t > I.ns) return;
  const int gx = I.gx, gy = I.gy;
  const int lgx = regk::ilog2(gx);
  const int tw_off = zdir ? I.pz.tw_off : I.py.tw_off;
  auto coords = [&](int tile, int b, int& cx, int& cy, int& cz) {
    const int L0 = tile * LPC;
    const int o = L0 >> lgx, x0 = (L0 & (gx - 1)) + b * tmak::kBoxCols;
    cx = x0;
    if (zdir) { cy = o; cz = 0; } else { cy = 0; cz = o; }
  };
  auto issue_load = [&](int tile, int s) {
    tmak::mbar_expect_tx(&bar[s], LY::tile_bytes);
    for (int b = 0; b < LY::NB; ++b) {
      int cx, cy, cz;
      coords(tile, b, cx, cy, cz);
      tmak::tma_load_3d(buf + (size_t)s * LY::tile_elems + b * LY::box_elems, &tmap, &bar[s], cx, cy, cz);
    }
  };
  // loads issued / completed, in issue order (load k uses stage k & 1 with
  // phase (k >> 1) & 1), to drain on an early exit
  int issued = 0, done = 0;
  tmak::pdl_launch_dependents();
  // the first tile's load is issued as soon as the previous pass is complete;
  // the other threads load the constant tables meanwhile
  if (threadIdx.x == 0) {
    tmak::mbar_init(&bar[0], 1);
    tmak::mbar_init(&bar[1], 1);
    tmak::fence_mbar_init();
    tmak::pdl_wait();
    if (blockIdx.x < ntiles) { issue_load(blockIdx.x, 0); issued = 1; }
  }
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = gtw[tw_off + i];
  if constexpr (KIND == 2) {
    const float* gzt = fk + I.gz_off;
    for (int i = threadIdx.x; i < 2 * N; i += blockDim.x) gzs[i] = gzt[i];
  }
  tmak::pdl_wait();
  const size_t es = zdir ? (size_t)gx * gy : (size_t)gx;
  float2* spec = I.spec;
  // (0, 0) pencil in float-float.  dc = 1: CTA 0 convolves the whole pencil
  // before its first tile (tile 0, which holds the pencil) and stores it with
  // that tile.  dc = 0 (fused plan): the CTAs with the fewest tiles each
  // convolve outputs z = k, k + nlight, ... after their tiles, from the pencil
  // the previous plane pass kept (dcin), into dcout; the plane pass that
  // follows puts dcout[z] into its plane.
  const bool dcblk = zdir && dc && blockIdx.x == 0;
  const int G = gridDim.x;
  const int nlight = ntiles % G == 0 ? G : G - ntiles % G;
  const int klight = (int)blockIdx.x - (G - nlight);
  const bool dcsplit = zdir && !dc && klight >= 0 && klight < N;
  float2* dcf = reinterpret_cast<float2*>(smraw + LY::dc_off);
  const DcPencil dcp{dcf, dcf + N, dcf + 2 * N};
  if (dcsplit) {
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      dcp.in[i] = dcin[(t & 1) * N + i];
      const double c = g64[I.g64_off + i];
      const float h = (float)c;
      dcp.c[i] = make_float2(h, (float)(c - (double)h));
    }
  }
  __syncthreads();
  if (dcblk) {
    dc_pencil_load<float>(spec, es, N, g64 + I.g64_off, dcp);
    __syncthreads();
    dc_pencil_apply(N, dcp);
  }
  const int line = threadIdx.x / TPL, lt = threadIdx.x % TPL;
  const int box = line / tmak::kBoxCols, col = line % tmak::kBoxCols;
  float2* sc = ex + line * F::LS;
  const float* gxy = fk + I.gxy_off;
  int it = 0;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int s = it & 1;
    const int nxt = tile + gridDim.x;
    if (threadIdx.x == 0 && nxt < ntiles) {
      tmak::bulk_wait_read0();  // the store of the tile last held in stage s^1 has read it
      issue_load(nxt, s ^ 1);
      ++issued;
    }
    // this line's k-space factor is read while the tile is in flight
    float ah = 0.f, al = 0.f;
    if constexpr (KIND == 2) {
      const int L = tile * LPC + line;
      ah = gxy[L];
      al = gxy[gx * gy + L];
    }
    const bool got = tmak::mbar_wait_bounded(&bar[s], (it >> 1) & 1, I.wait_polls);
    if (!__syncthreads_and(got)) {
      if (threadIdx.x == 0) atomicOr(err, 2);
      break;
    }
    ++done;
    float2* tb = buf + (size_t)s * LY::tile_elems + box * LY::box_elems;
    float2 v[R1];
#pragma unroll
    for (int r = 0; r < R1; ++r) {
      const int j = in_dout ? F::out_index(lt, r) : F::in_index(lt, r);
      v[r] = tb[tmak::swz(j, col)];
    }
    if constexpr (KIND == 1) {
      F::inverse(v, sc, tw, lt);
    } else if constexpr (KIND == 0) {
      F::forward(v, sc, tw, lt);
    } else {
      F::forward(v, sc, tw, lt);
#pragma unroll
      for (int r = 0; r < R1; ++r) {
        const int kz = F::out_index(lt, r);
        const float bh = gzs[kz], bl = gzs[N + kz];
        const float gh = ah * bh;
        const float gl = fmaf(ah, bh, -gh) + fmaf(ah, bl, al * bh);
        v[r] = make_float2(fmaf(v[r].x, gh, v[r].x * gl), fmaf(v[r].y, gh, v[r].y * gl));
      }
      F::inverse(v, sc, tw, lt);
    }
#pragma unroll
    for (int r = 0; r < R1; ++r) {
      const int j = out_dout ? F::out_index(lt, r) : F::in_index(lt, r);
      tb[tmak::swz(j, col)] = v[r];
    }
    if (dcblk && tile == 0) {
      __syncthreads();
      float2* t0 = buf + (size_t)s * LY::tile_elems;  // line 0 = box 0, column 0
      for (int j = threadIdx.x; j < N; j += blockDim.x) t0[tmak::swz(j, 0)] = dcp.out[j];
    }
    tmak::fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int b = 0; b < LY::NB; ++b) {
        int cx, cy, cz;
        coords(tile, b, cx, cy, cz);
        tmak::tma_store_3d(&tmap, buf + (size_t)s * LY::tile_elems + b * LY::box_elems, cx, cy, cz);
      }
      tmak::bulk_commit();
    }
  }
  if (dcsplit && (threadIdx.x >> 5) == 1) {   // warp 1, while thread 0 drains the stores
    for (int z = klight; z < N; z += nlight) {
      const float2 o = tmak::dc_point(dcp.in, dcp.c, N, z);
      if ((threadIdx.x & 31) == 0) dcout[z] = o;
    }
  }
  if (threadIdx.x == 0) {
    // loads still in flight after an early exit land before shared memory is released
    for (int k = done; k < issued; ++k)
      tmak::mbar_wait_bounded(&bar[k & 1], (k >> 1) & 1, tmak::kWaitPolls);
    tmak::bulk_wait0();
  }
}

// ---------------------------------------------------------------------------
// Fused XY pass: one z-plane per CTA, whole plane in shared memory.
//
// A 128 x 128 FP32 plane is 128 KB, so the three passes that run inside one
// plane -- inverse y (Yi of step t), the x pass of step t, and forward y (Yf
// of step t+1) -- fuse into one kernel: the plane arrives by TMA as N/16
// swizzled 16-column boxes (the Y pass's tensor map), is transformed in
// place, and leaves by TMA.  A double step becomes two launches, Z and XY,
// and the spectrum crosses L2 twice per step instead of four times.
//   phase 1: inverse y on the N columns (lines of D_out -> D_in)
//   phase 2: inverse x on the N rows, q_t = E(t) z, slice store,
//            z = E(t+1) q_t, forward x
//   phase 3: forward y on the columns
// t = 0 (initial): slice 0 = (1, 1), z = E(1), forward x, forward y.
// t = Ns: phase 2 stores the last slice only.  Same arithmetic, element for
// element, as the separate passes.  The mbarrier wait is bounded (error flag
// 8); a CTA that gives up drains its copy before returning.
// ---------------------------------------------------------------------------
namespace tmak {

template <int N>
struct XYLayout {
  using F = RegFFT<float, regk::Cfg<N>::R1, regk::Cfg<N>::TPL>;
  static constexpr int THREADS = 512;
  static constexpr int LINES = THREADS / F::TPL;            // lines per round
  static constexpr int NB = N / kBoxCols;                   // boxes per plane
  static constexpr int box_elems = N * kBoxCols;
  static constexpr uint32_t plane_bytes = (uint32_t)N * N * 8;
  static constexpr size_t sc_off = plane_bytes;             // plane at 0 (1024-aligned)
  static constexpr size_t tw_off = sc_off + (size_t)LINES * F::LS * sizeof(float2);
  static constexpr size_t bar_off = ((tw_off + N * sizeof(float2) + 15) / 16) * 16;
  static constexpr size_t bytes = bar_off + 2 * sizeof(uint64_t) + 1024;   // + alignment slack
  // the plane arrives and leaves as two halves of NB / 2 boxes (columns
  // [0, N/2) and [N/2, N)), one mbarrier each, so that phase 1 starts on the
  // first half while the second is in flight and the first half is stored
  // while phase 3 transforms the second
  static constexpr int HB = NB / 2;
  static constexpr uint32_t half_bytes = plane_bytes / 2;
  static constexpr bool split = LINES < N;   // rounds of phases 1 and 3 cover one half each
  static_assert(!split || LINES == N / 2, "a round covers one half of the plane");
  static_assert(N % LINES == 0 || LINES % N == 0, "rounds of whole lines");
};

// element (row j, column x) of a plane held as N/16 swizzled 16-column boxes
template <int N>
__device__ __forceinline__ int plane_at(int j, int x) {
  return (x >> 4) * (N * kBoxCols) + swz(j, x & 15);
}

}  // namespace tmak

template <int N>
__global__ void __launch_bounds__(512, 1)
k_xy_tma(const BulkDev<float>* __restrict__ insts, const __grid_constant__ CUtensorMap tmap,
         const float2* __restrict__ gtw, const float2* __restrict__ dcout,
         float2* __restrict__ dcin, int t, int* __restrict__ err) {
  using LY = tmak::XYLayout<N>;
  using F = typename LY::F;
  constexpr int R1 = F::R1, TPL = F::TPL, LINES = LY::LINES;
  extern __shared__ __align__(1024) unsigned char smraw_[];
  unsigned char* smraw = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smraw_) + 1023) & ~uintptr_t(1023));
  float2* plane = reinterpret_cast<float2*>(smraw);
  float2* scr = reinterpret_cast<float2*>(smraw + LY::sc_off);
  float2* tw = reinterpret_cast<float2*>(smraw + LY::tw_off);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smraw + LY::bar_off);
  const BulkDev<float>& I = insts[0];
  if (t > I.ns) return;
  const bool init = t == 0;
  const bool more = init || t < I.ns;
  const int gz = I.gz;
  int it = 0, issued = 0, done0 = 0, done1 = 0;
  auto issue_plane = [&](int z) {
    for (int h = 0; h < 2; ++h) {
      tmak::mbar_expect_tx(&bar[h], LY::half_bytes);
      for (int b = h * LY::HB; b < (h + 1) * LY::HB; ++b)
        tmak::tma_load_3d(plane + b * LY::box_elems, &tmap, &bar[h], b * tmak::kBoxCols, 0, z);
    }
    ++issued;
  };
  auto store_half = [&](int h, int z) {
    for (int b = h * LY::HB; b < (h + 1) * LY::HB; ++b)
      tmak::tma_store_3d(&tmap, plane + b * LY::box_elems, b * tmak::kBoxCols, 0, z);
    tmak::bulk_commit();
  };
  // bounded wait for half h of plane iteration `it`; false (flag 8 set) when
  // it expired in any thread of the CTA
  auto wait_half = [&](int h) {
    const bool got = tmak::mbar_wait_bounded(&bar[h], (uint32_t)(it & 1), I.wait_polls);
    if (!__syncthreads_and(got)) {
      if (threadIdx.x == 0) atomicOr(err, 8);
      return false;
    }
    if (h == 0) ++done0; else ++done1;
    return true;
  };
  tmak::pdl_launch_dependents();
  // the first plane's load is issued as soon as the previous pass is
  // complete; the other threads load the constant tables meanwhile
  if (threadIdx.x == 0) {
    tmak::mbar_init(&bar[0], 1);
    tmak::mbar_init(&bar[1], 1);
    tmak::fence_mbar_init();
    tmak::pdl_wait();
    if (!init && (int)blockIdx.x < gz) issue_plane(blockIdx.x);
  }
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw[i] = gtw[I.px.tw_off + i];
  tmak::pdl_wait();
  __syncthreads();
  const int line = threadIdx.x / TPL, lt = threadIdx.x % TPL;
  const bool active = line < N;          // N = 64 leaves no idle line; kept for clarity
  float2* sc = scr + line * F::LS;
  // Boltzmann factor choice: node t of each chain, then node t+1
  const int tt = init ? 1 : t;
  const bool fA = chain_type_fwd(I, tt) == 0, bA = chain_type_bwd(I, tt) == 0;
  const bool fA2 = chain_type_fwd(I, t + 1) == 0, bA2 = chain_type_bwd(I, t + 1) == 0;
  float2* sl = I.slices + (size_t)t * I.npts;
  for (int z = blockIdx.x; z < gz; z += gridDim.x, ++it) {
    const size_t pbase = (size_t)z * N * N;
    if (!init) {
      if (threadIdx.x == 0 && it > 0) {
        tmak::bulk_wait_read0();          // the previous plane's stores have read the buffer
        issue_plane(z);
      }
      // (0, 0) entry: after the TMA z pass of the fused plan (dcout set) it is
      // in FP32, and its float-float value comes from dcout (read while the
      // plane is in flight); the other z kernels store the float-float value
      // themselves.  Column 0 is read in phase 1 by lanes 0-7 of warp 0 only,
      // so a warp barrier orders the write.
      float2 dco = make_float2(0.f, 0.f);
      if (dcout && threadIdx.x == 0) dco = dcout[z];
      if (!wait_half(0)) break;
      if (!LY::split && !wait_half(1)) break;
      if (dcout && threadIdx.x == 0) plane[tmak::plane_at<N>(0, 0)] = dco;
      __syncwarp();
      // phase 1: inverse y, columns x (with split halves, the round of the
      // second half waits for its boxes)
      bool ok = true;
      for (int c0 = 0; c0 < N; c0 += LINES) {
        if (LY::split && c0 > 0 && !(ok = wait_half(1))) break;
        const int x = c0 + line;
        if (active && x < N) {
          float2 v[R1];
#pragma unroll
          for (int r = 0; r < R1; ++r) v[r] = plane[tmak::plane_at<N>(F::out_index(lt, r), x)];
          F::inverse(v, sc, tw, lt);
#pragma unroll
          for (int r = 0; r < R1; ++r) plane[tmak::plane_at<N>(F::in_index(lt, r), x)] = v[r];
        }
      }
      if (!ok) break;
      __syncthreads();
    } else {
      if (threadIdx.x == 0) tmak::bulk_wait_read0();
      __syncthreads();
    }
    // phase 2: rows j
    for (int r0 = 0; r0 < N; r0 += LINES) {
      const int j = r0 + line;
      if (!(active && j < N)) continue;
      const size_t rbase = pbase + (size_t)j * N;
      float2 v[R1];
      if (!init) {
        // the Boltzmann factors of the first half of the row's points are
        // loaded before its inverse x transform, so their latency overlaps
        // it (all sixteen would leave too few registers for the transform);
        // the second half is prefetched into L1, which takes no registers
        constexpr int HP = R1 / 2;
#pragma unroll
        for (int m = HP; m < R1; ++m)
          tmak::prefetch_l1(reinterpret_cast<const float4*>(I.E) + rbase + F::in_index(lt, m));
        EPt<float> epre[HP];
#pragma unroll
        for (int m = 0; m < HP; ++m) epre[m] = load_ept(I.E, rbase + F::in_index(lt, m));
#pragma unroll
        for (int r = 0; r < R1; ++r) v[r] = plane[tmak::plane_at<N>(j, F::out_index(lt, r))];
        F::inverse(v, sc, tw, lt);
#pragma unroll
        for (int m = 0; m < R1; ++m) {
          const size_t g = rbase + F::in_index(lt, m);
          const EPt<float> ev = m < HP ? epre[m % HP] : load_ept(I.E, g);
          const float2 q = make_float2(emul(v[m].x, fA ? ev.a : ev.b, fA ? ev.al : ev.bl),
                                       emul(v[m].y, bA ? ev.a : ev.b, bA ? ev.al : ev.bl));
          sl[g] = q;
          if (more)
            v[m] = make_float2(emul(q.x, fA2 ? ev.a : ev.b, fA2 ? ev.al : ev.bl),
                               emul(q.y, bA2 ? ev.a : ev.b, bA2 ? ev.al : ev.bl));
        }
      } else {
#pragma unroll
        for (int m = 0; m < R1; ++m) {
          const size_t g = rbase + F::in_index(lt, m);
          const EPt<float> ev = load_ept(I.E, g);
          v[m] = make_float2(fA ? ev.a : ev.b, bA ? ev.a : ev.b);
          sl[g] = make_float2(1.f, 1.f);
        }
      }
      if (more) {
        F::forward(v, sc, tw, lt);
#pragma unroll
        for (int r = 0; r < R1; ++r) plane[tmak::plane_at<N>(j, F::out_index(lt, r))] = v[r];
      }
    }
    __syncthreads();
    if (!more) continue;                  // last step: nothing goes back to the spectrum
    // phase 3: forward y, columns x; each half leaves as soon as its columns
    // are done
    for (int c0 = 0; c0 < N; c0 += LINES) {
      const int x = c0 + line;
      if (active && x < N) {
        float2 v[R1];
#pragma unroll
        for (int r = 0; r < R1; ++r) v[r] = plane[tmak::plane_at<N>(F::in_index(lt, r), x)];
        F::forward(v, sc, tw, lt);
#pragma unroll
        for (int r = 0; r < R1; ++r) plane[tmak::plane_at<N>(F::out_index(lt, r), x)] = v[r];
      }
      if (LY::split) {
        tmak::fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) store_half(c0 == 0 ? 0 : 1, z);
      }
    }
    if (!LY::split) {
      tmak::fence_async_smem();
      __syncthreads();
      if (threadIdx.x == 0) { store_half(0, z); store_half(1, z); }
    }
    if (threadIdx.x == 0)
      dcin[((t + 1) & 1) * N + z] = plane[tmak::plane_at<N>(0, 0)];   // the next z pass's pencil
  }
  if (threadIdx.x == 0) {
    // loads still in flight after an early exit land before shared memory is released
    for (int k = done0; k < issued; ++k) tmak::mbar_wait_bounded(&bar[0], (uint32_t)(k & 1), tmak::kWaitPolls);
    for (int k = done1; k < issued; ++k) tmak::mbar_wait_bounded(&bar[1], (uint32_t)(k & 1), tmak::kWaitPolls);
    tmak::bulk_wait0();
  }
}
