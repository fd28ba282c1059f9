// film_adi.cu -- launches of the warp-cooperative FP32 Douglas ADI sweeps
// (film_warp.cuh) for Film_3D contexts in split precision.
#include "film_warp.cuh"
#include "internal.h"

namespace {

bool pow2(int v) { return v > 0 && (v & (v - 1)) == 0; }

// (G, K) for a periodic line of n points: K in {4, 2} with n = G K and G a
// power of two in [2, 32]; false when neither fits
bool periodic_shape(int n, int& G, int& K) {
  for (int k : {4, 2}) {
    if (n % k) continue;
    const int g = n / k;
    if (g >= 2 && g <= 32 && pow2(g)) { G = g; K = k; return true; }
  }
  return false;
}

// (G, K) for a Dirichlet line of n rows: the fewest lanes with K <= 4 (G a
// power of two in [2, 32]), K up to 8 on 32 lanes
bool dirichlet_shape(int n, int& G, int& K) {
  if (n < 2 || n > 256) return false;
  G = 2;
  while (G < 32 && 4 * G < n) G *= 2;
  K = (n + G - 1) / G;
  if (K < 2) K = 2;
  return K <= 8;
}

template <template <int, int> class Kern, int K>
struct ByG;

template <int G, int K>
struct XW { static void go(dim3 g, cudaStream_t s, const FilmDev<float>& D, int st) { k_adi_x_w<G, K><<<g, 128, 0, s>>>(D, st); } };
template <int G, int K>
struct YW { static void go(dim3 g, cudaStream_t s, const FilmDev<float>& D, int st) { k_adi_y_w<G, K><<<g, 128, 0, s>>>(D, st); } };
template <int G, int K>
struct ZW { static void go(dim3 g, cudaStream_t s, const FilmDev<float>& D, int st) { k_adi_z_w<G, K><<<g, 128, 0, s>>>(D, st); } };

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

// blocks of 4 warps, 32 / G lines per warp
dim3 grid_for(int lines, int G, int chains) {
  const int per_block = 4 * (32 / G);
  return dim3((lines + per_block - 1) / per_block, chains);
}

}  // namespace

// Which ADI sweeps of this context run on the warp solver (bits 1: x, 2: y,
// 4: z); the others keep the one-thread-per-line kernels.
int adi_warp_mask(const FilmDev<float>& D) {
  int G, K, m = 0;
  if (periodic_shape(D.gx, G, K)) m |= 1;
  if (periodic_shape(D.gy, G, K)) m |= 2;
  if (dirichlet_shape(D.gz + 1, G, K)) m |= 4;
  return m;
}

void adi_x_warp(const FilmDev<float>& D, int step, int chains, cudaStream_t s) {
  int G = 2, K = 2;
  periodic_shape(D.gx, G, K);
  const dim3 g = grid_for(D.gy * (D.gz - 1), G, chains);
  if (K == 4) by_g<XW, 4>(G, g, s, D, step);
  else by_g<XW, 2>(G, g, s, D, step);
}

void adi_y_warp(const FilmDev<float>& D, int step, int chains, cudaStream_t s) {
  int G = 2, K = 2;
  periodic_shape(D.gy, G, K);
  const dim3 g = grid_for(D.gx * (D.gz - 1), G, chains);
  if (K == 4) by_g<YW, 4>(G, g, s, D, step);
  else by_g<YW, 2>(G, g, s, D, step);
}

void adi_z_warp(const FilmDev<float>& D, int step, int chains, cudaStream_t s) {
  int G = 2, K = 2;
  dirichlet_shape(D.gz + 1, G, K);
  const dim3 g = grid_for(D.nlines, G, chains);
  switch (K) {
    case 2: by_g<ZW, 2>(G, g, s, D, step); break;
    case 3: by_g<ZW, 3>(G, g, s, D, step); break;
    case 4: by_g<ZW, 4>(G, g, s, D, step); break;
    case 5: ZW<32, 5>::go(g, s, D, step); break;
    case 6: ZW<32, 6>::go(g, s, D, step); break;
    case 7: ZW<32, 7>::go(g, s, D, step); break;
    default: ZW<32, 8>::go(g, s, D, step); break;
  }
}
