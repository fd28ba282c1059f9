// bulk_host.h -- host-side plans and k-space tables of the bulk propagator,
// shared by the single-instance context (bulk.cu) and the batch (batch.cu).
//
// Calculate_Laplace (Bulk_3D_FFT/Geometry_Modules/Bulk/mod_fourier.f90:
// 165-198): explaplace = exp(-ds (kx^2 + ky^2 + kz^2)) with the wrapped wave
// numbers of :178-186.  Here the factor is kept separable -- g_xy[y][x] and
// g_z[z]/N -- each as T plus its rounding residue, and the (kx, ky) = (0, 0)
// z pencil additionally as the FP64 circulant kernel of its convolution.
#pragma once
#include <cmath>
#include <cstring>
#include <utility>
#include <vector>

#include "bulk_kernels.cuh"

namespace bulkhost {

inline int pow2_floor(int v) {
  int p = 1;
  while (p * 2 <= v) p *= 2;
  return p;
}

// mixed-radix plan of an n-point line (radices 8, 4, 2, 3, 5)
inline bool make_plan(int n, Plan1D& P) {
  std::memset(&P, 0, sizeof(P));
  P.n = n;
  int m = n;
  while (m % 8 == 0 && P.nst < ADSCF_MAX_STAGES) { P.rad[P.nst++] = 8; m /= 8; }
  while (m % 4 == 0 && P.nst < ADSCF_MAX_STAGES) { P.rad[P.nst++] = 4; m /= 4; }
  while (m % 2 == 0 && P.nst < ADSCF_MAX_STAGES) { P.rad[P.nst++] = 2; m /= 2; }
  while (m % 3 == 0 && P.nst < ADSCF_MAX_STAGES) { P.rad[P.nst++] = 3; m /= 3; }
  while (m % 5 == 0 && P.nst < ADSCF_MAX_STAGES) { P.rad[P.nst++] = 5; m /= 5; }
  if (m != 1) return false;
  int tpl = pow2_floor(n / 8 > 0 ? n / 8 : 1);
  if (tpl > 64) tpl = 64;
  P.tpl = tpl;
  P.lpc = BULK_THREADS / tpl;
  P.ld = n + 1;
  return true;
}

// signed wave number of index i (mod_fourier.f90:178-186)
inline double wavenum(int i, int n, double L) {
  double m = (i > n / 2) ? double(i - n) : double(i);
  return 2.0 * M_PI * m / L;
}

// dynamic shared memory of the generic passes: twiddles + two line buffers
template <typename T>
size_t plan_smem(const Plan1D& P) {
  size_t twn = (P.n + 1) & ~1;
  return (twn + 2 * (size_t)P.lpc * P.ld) * sizeof(cplx<T>);
}

// the generic z pass also holds the float-float (0,0) pencil
template <typename T>
size_t plan_smem_z(const Plan1D& P) {
  return plan_smem<T>(P) + 16 + (((P.n + 1) & ~1) + 2 * (size_t)P.ld) * sizeof(double2);
}

// W_n^m = exp(-2 pi i m / n) for m < n, appended once per distinct n
template <typename T>
int twiddle_offset(int n, std::vector<cplx<T>>& tw, std::vector<std::pair<int, int>>& seen) {
  for (const auto& s : seen)
    if (s.first == n) return s.second;
  const int off = (int)tw.size();
  for (int m = 0; m < n; ++m) {
    const double a = -2.0 * M_PI * (double)m / (double)n;
    tw.push_back(mk<T>((T)std::cos(a), (T)std::sin(a)));
  }
  seen.push_back({n, off});
  return off;
}

// Appends the diffusion tables of one gx x gy x gz box of side lengths
// (lx, ly, lz) at contour step ds: fk gets g_xy hi/lo ([gy][gx] each) and
// g_z/N hi/lo ([gz] each); g64 gets the circulant kernel c(d) = sum_kz
// G(kz) cos(2 pi kz d / gz) of the (0,0) pencil (FP64, phase index reduced
// mod gz before the cosine).
template <typename T>
void append_tables(int gx, int gy, int gz, double lx, double ly, double lz, double ds,
                   std::vector<T>& fk, std::vector<double>& g64, int& gxy_off, int& gz_off,
                   int& g64_off) {
  const double invn = 1.0 / ((double)gx * gy * gz);
  const size_t nxy = (size_t)gx * gy;
  gxy_off = (int)fk.size();
  fk.resize(fk.size() + 2 * nxy + 2 * (size_t)gz);
  gz_off = gxy_off + (int)(2 * nxy);
  for (int y = 0; y < gy; ++y) {
    const double ky = wavenum(y, gy, ly);
    for (int x = 0; x < gx; ++x) {
      const double kx = wavenum(x, gx, lx);
      const double g = std::exp(-ds * kx * kx) * std::exp(-ds * ky * ky);
      const T h = (T)g;
      fk[gxy_off + (size_t)y * gx + x] = h;
      fk[gxy_off + nxy + (size_t)y * gx + x] = (T)(g - (double)h);
    }
  }
  std::vector<double> gzd(gz);
  for (int z = 0; z < gz; ++z) {
    const double kz = wavenum(z, gz, lz);
    const double g = std::exp(-ds * kz * kz) * invn;
    const T h = (T)g;
    fk[gz_off + z] = h;
    fk[gz_off + gz + z] = (T)(g - (double)h);
    gzd[z] = g;
  }
  g64_off = (int)g64.size();
  for (int d = 0; d < gz; ++d) {
    double s = 0.0;
    for (int k = 0; k < gz; ++k) {
      const long long m = ((long long)k * d) % gz;
      s += gzd[k] * std::cos(2.0 * M_PI * (double)m / (double)gz);
    }
    g64.push_back(s);
  }
}

}  // namespace bulkhost
