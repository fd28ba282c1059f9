// film_adi.cu -- launches of the warp-cooperative FP32 Douglas ADI sweeps
// (film_warp.cuh) for Film_3D contexts in split precision.
#include "film_warp.cuh"
#include "internal.h"

#include <algorithm>
#include <vector>

namespace {

bool pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }

template <int G, int K>
struct XW { static void go(dim3 g, cudaStream_t s, const FilmDev<float>& D, int st) { k_adi_x_w<G, K><<<g, 128, 0, s>>>(D, st); } };
template <int G, int K>
struct YW { static void go(dim3 g, cudaStream_t s, const FilmDev<float>& D, int st) { k_adi_y_w<G, K><<<g, 128, 0, s>>>(D, st); } };
template <int G, int K>
struct ZW { static void go(dim3 g, cudaStream_t s, const FilmDev<float>& D, int st) { k_adi_z_w<G, K><<<g, 128, 0, s>>>(D, st); } };
template <int G, int K>
struct YS {
  static void go(dim3 g, cudaStream_t s, const FilmDev<float>& D, int st) {
    k_adi_yz_s<G, K, false><<<g, 128, adi_staged_smem(D.gy, false), s>>>(D, st);
  }
};
template <int G, int K>
struct ZS {
  static void go(dim3 g, cudaStream_t s, const FilmDev<float>& D, int st) {
    k_adi_yz_s<G, K, true><<<g, 128, adi_staged_smem(D.gz + 1, true), s>>>(D, st);
  }
};

// instantiated shapes: G in {2, .., 32} with K in {2, 3, 4} (K = 3 for the
// Dirichlet sweep only), and K in 5..8 for the Dirichlet sweep on 8, 16 or 32
// lanes
template <template <int, int> class W, int K>
void by_g(int G, dim3 g, cudaStream_t s, const FilmDev<float>& D, int st) {
  switch (G) {
    case 2: W<2, K>::go(g, s, D, st); break;
    case 4: W<4, K>::go(g, s, D, st); break;
    case 8: W<8, K>::go(g, s, D, st); break;
    case 16: W<16, K>::go(g, s, D, st); break;
    default: W<32, K>::go(g, s, D, st); break;
  }
}
template <template <int, int> class W, int K>
void by_g_wide(int G, dim3 g, cudaStream_t s, const FilmDev<float>& D, int st) {
  switch (G) {
    case 8: W<8, K>::go(g, s, D, st); break;
    case 16: W<16, K>::go(g, s, D, st); break;
    default: W<32, K>::go(g, s, D, st); break;
  }
}

template <template <int, int> class W, int K>
void by_g4(int G, dim3 g, cudaStream_t s, const FilmDev<float>& D, int st) {
  switch (G) {
    case 4: W<4, K>::go(g, s, D, st); break;
    case 8: W<8, K>::go(g, s, D, st); break;
    case 16: W<16, K>::go(g, s, D, st); break;
    default: W<32, K>::go(g, s, D, st); break;
  }
}

// staged shapes keep their tile (and the block's static coefficients) within
// the default 48 KB of shared memory
constexpr size_t kStagedSmemMax = 46 * 1024;

// blocks of 4 warps, 32 / G lines per warp
dim3 grid_for(int lines, int G, int chains) {
  const int per_block = 4 * (32 / G);
  return dim3((lines + per_block - 1) / per_block, chains);
}

}  // namespace

// Warp-solver shapes (G lanes per line, K points per lane) that fit the lines
// of sweep `dim` (0: x, 1: y, periodic lines of gx or gy points with G K = n;
// 2: z, Dirichlet lines of gz + 1 rows padded to G K).
std::vector<AdiShape> adi_shapes(int dim, const FilmDev<float>& D) {
  std::vector<AdiShape> v;
  if (dim < 2) {
    const int n = dim == 0 ? D.gx : D.gy;
    for (int k : {2, 4}) {
      if (n % k) continue;
      const int g = n / k;
      if (g >= 2 && g <= 32 && pow2(g)) v.push_back({g, k, 0});
    }
  } else {
    const int n = D.gz + 1;
    if (n < 2 || n > 256) return v;
    for (int g = 2; g <= 32; g *= 2) {
      const int k = std::max(2, (n + g - 1) / g);
      if (k <= 4 || (k <= 8 && g >= 8)) v.push_back({g, k, 0});
    }
  }
  // the same shapes staged through shared memory (y and z sweeps, G >= 4)
  if (dim > 0) {
    const int n = dim == 1 ? D.gy : D.gz + 1;
    const size_t nv = v.size();
    for (size_t i = 0; i < nv; ++i)
      if (v[i].g >= 4 && adi_staged_smem(n, dim == 2) <= kStagedSmemMax) v.push_back({v[i].g, v[i].k, 1});
  }
  return v;
}

// The shape used without timing: periodic lines K = 4 before K = 2;
// Dirichlet lines the fewest lanes with K <= 4, else 32 lanes; {0, 0} (one
// thread per line) when no shape fits.
AdiShape adi_default_shape(int dim, const FilmDev<float>& D) {
  const std::vector<AdiShape> v = adi_shapes(dim, D);
  if (v.empty()) return {0, 0, 0};
  if (dim < 2) return v[v.size() > 1 && v[1].k == 4 ? 1 : 0];
  for (const AdiShape& a : v)
    if (a.k <= 4) return a;
  return v.back();
}

// The fused x + y plane sweep (k_adi_xy_p) exists for square planes whose x
// and y sweeps share one unstaged shape of these sizes (N G <= 1024 threads).
bool adi_fused_ok(AdiShape x, AdiShape y, const FilmDev<float>& D) {
  if (x.g != y.g || x.k != y.k || x.staged || y.staged || D.gx != D.gy || D.gx != x.g * x.k) return false;
  return (x.g == 16 && (x.k == 4 || x.k == 2)) || (x.g == 8 && (x.k == 4 || x.k == 2));
}

void adi_fused_sweep(AdiShape sh, const FilmDev<float>& D, int step, int chains, cudaStream_t s) {
  const dim3 g(D.gz - 1, chains);
  const int nt = sh.g * sh.g * sh.k;
  if (sh.g == 16 && sh.k == 4) k_adi_xy_p<16, 4><<<g, nt, 0, s>>>(D, step);
  else if (sh.g == 16) k_adi_xy_p<16, 2><<<g, nt, 0, s>>>(D, step);
  else if (sh.k == 4) k_adi_xy_p<8, 4><<<g, nt, 0, s>>>(D, step);
  else k_adi_xy_p<8, 2><<<g, nt, 0, s>>>(D, step);
}

void adi_warp_sweep(int dim, AdiShape sh, const FilmDev<float>& D, int step, int chains, cudaStream_t s) {
  const int G = sh.g, K = sh.k;
  if (dim == 0) {
    const dim3 g = grid_for(D.gy * (D.gz - 1), G, chains);
    if (K == 4) by_g<XW, 4>(G, g, s, D, step);
    else by_g<XW, 2>(G, g, s, D, step);
  } else if (dim == 1 && sh.staged) {
    const dim3 g(((D.gx + kAdiTile - 1) / kAdiTile) * (D.gz - 1), chains);
    if (K == 4) by_g4<YS, 4>(G, g, s, D, step);
    else by_g4<YS, 2>(G, g, s, D, step);
  } else if (dim == 1) {
    const dim3 g = grid_for(D.gx * (D.gz - 1), G, chains);
    if (K == 4) by_g<YW, 4>(G, g, s, D, step);
    else by_g<YW, 2>(G, g, s, D, step);
  } else if (sh.staged) {
    const dim3 g((D.nlines + kAdiTile - 1) / kAdiTile, chains);
    switch (K) {
      case 2: by_g4<ZS, 2>(G, g, s, D, step); break;
      case 3: by_g4<ZS, 3>(G, g, s, D, step); break;
      case 4: by_g4<ZS, 4>(G, g, s, D, step); break;
      case 5: by_g_wide<ZS, 5>(G, g, s, D, step); break;
      case 6: by_g_wide<ZS, 6>(G, g, s, D, step); break;
      case 7: by_g_wide<ZS, 7>(G, g, s, D, step); break;
      default: by_g_wide<ZS, 8>(G, g, s, D, step); break;
    }
  } else {
    const dim3 g = grid_for(D.nlines, G, chains);
    switch (K) {
      case 2: by_g<ZW, 2>(G, g, s, D, step); break;
      case 3: by_g<ZW, 3>(G, g, s, D, step); break;
      case 4: by_g<ZW, 4>(G, g, s, D, step); break;
      case 5: by_g_wide<ZW, 5>(G, g, s, D, step); break;
      case 6: by_g_wide<ZW, 6>(G, g, s, D, step); break;
      case 7: by_g_wide<ZW, 7>(G, g, s, D, step); break;
      default: by_g_wide<ZW, 8>(G, g, s, D, step); break;
    }
  }
}
