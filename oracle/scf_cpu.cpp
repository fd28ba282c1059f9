// scf_cpu.cpp -- FP64 C++17/OpenMP restatement of one bulk SCF iteration:
// the timed CPU baseline of the GPU library, and test infrastructure (the
// tests check it against the numpy oracle; no product code calls it).
//
// It restates, on the host cores:
//   Propagate_Step      Bulk_3D_FFT/General_Routines/mod_propagate.f90:40-68
//                       (E FFT^-1[exp(-ds k^2) FFT[E q]], Real2Fourier's 1/N,
//                       Geometry_Modules/Bulk/mod_fourier.f90:94-105)
//   Calculate_Laplace   mod_fourier.f90:165-198 (wrapped wave numbers)
//   Propagate_Diblock   Bulk_3D_FFT/Polymer_Modules/mod_diblock.f90:100-173
//                       (all Ns+1 slices of both chains kept, Q = dvol sum
//                       q_N, block trapezoid, canonical closure)
//   Check_Accuracy      Main_Diblock_Melt/main_diblock.f90:380-390
//   Calculate_Mean_Fields / Interaction_Energy
//                       Interaction_Modules/mod_FloryHuggins.f90:74-129
//   Mixing_Anderson + ludcmp/lubksb
//                       General_Routines/mod_iterate.f90:92-150,232-337
//                       (history depth m as a parameter, warm-up step
//                       lam_warm for iter <= warm_iters, persistent history)
// The free energy of iterate k is Calculate_Energy (main_diblock.f90:295-307)
// at that iterate, over rho V.
//
// The reference calls FFTW's r2c/c2r once per chain and step.  Both chains
// are real and exp(-ds k^2) is real and even, so here one complex FFT of
// E_f q + i E_b q-dagger advances both chains one step -- the same
// arithmetic cost as two r2c/c2r pairs.  The FFT is this file's own:
// mixed-radix (4, 2, 3, 5) Stockham stages over batches of B lines held as
// separate real and imaginary planes [n][B], so the inner loops run over
// the B lines with unit stride.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int kB = 16;   // lines per FFT batch

struct Stage {
  int p = 0;                  // radix
  int m = 0;                  // butterflies per sub-transform (n_cur / p)
  int s = 0;                  // stride (product of the earlier radices)
  std::vector<double> wr, wi; // twiddles [m][p-1]: exp(-2 pi i k j / n_cur)
};

struct Plan {
  int n = 0;
  std::vector<Stage> st;
};

bool make_plan(int n, Plan& P) {
  P.n = n;
  P.st.clear();
  int rem = n, s = 1;
  while (rem > 1) {
    int p = rem % 4 == 0 ? 4 : rem % 2 == 0 ? 2 : rem % 3 == 0 ? 3 : rem % 5 == 0 ? 5 : 0;
    if (!p) return false;
    Stage S;
    S.p = p;
    S.m = rem / p;
    S.s = s;
    S.wr.resize((size_t)S.m * (p - 1));
    S.wi.resize((size_t)S.m * (p - 1));
    for (int j = 0; j < S.m; ++j)
      for (int k = 1; k < p; ++k) {
        // exponent k*j reduced mod rem before the angle is formed
        const long long e = ((long long)k * j) % rem;
        const double a = -2.0 * M_PI * (double)e / (double)rem;
        S.wr[(size_t)j * (p - 1) + k - 1] = std::cos(a);
        S.wi[(size_t)j * (p - 1) + k - 1] = std::sin(a);
      }
    P.st.push_back(std::move(S));
    rem /= p;
    s *= p;
  }
  return true;
}

// One Stockham DIF stage on B lanes: input x[q + s (j + r m)], output
// y[q + s (p j + k)] = (sum_r x_r w_p^{rk}) * w^{k j}; sg = +1 forward
// (exp(-i...)), -1 inverse.
template <int P>
void stage_fixed(const Stage& S, int B, const double* xr, const double* xi, double* yr, double* yi,
                 int sg) {
  const int m = S.m, s = S.s;
  // DFT matrix of the radices without a hand-written butterfly (5)
  double dmr[P][P], dmi[P][P];
  for (int k = 0; k < P; ++k)
    for (int r = 0; r < P; ++r) {
      const double a = -2.0 * M_PI * (double)((r * k) % P) / (double)P;
      dmr[k][r] = std::cos(a);
      dmi[k][r] = sg * std::sin(a);
    }
  for (int j = 0; j < m; ++j) {
    double twr[P], twi[P];
    twr[0] = 1.0; twi[0] = 0.0;
    for (int k = 1; k < P; ++k) {
      twr[k] = S.wr[(size_t)j * (P - 1) + k - 1];
      twi[k] = sg * S.wi[(size_t)j * (P - 1) + k - 1];
    }
    for (int q = 0; q < s; ++q) {
      const double* ar[P];
      const double* ai[P];
      double* br[P];
      double* bi[P];
      for (int r = 0; r < P; ++r) {
        ar[r] = xr + (size_t)(q + s * (j + r * m)) * B;
        ai[r] = xi + (size_t)(q + s * (j + r * m)) * B;
        br[r] = yr + (size_t)(q + s * (P * j + r)) * B;
        bi[r] = yi + (size_t)(q + s * (P * j + r)) * B;
      }
#pragma omp simd
      for (int b = 0; b < B; ++b) {
        double cr[P], ci[P];
        if constexpr (P == 2) {
          cr[0] = ar[0][b] + ar[1][b]; ci[0] = ai[0][b] + ai[1][b];
          cr[1] = ar[0][b] - ar[1][b]; ci[1] = ai[0][b] - ai[1][b];
        } else if constexpr (P == 4) {
          const double t0r = ar[0][b] + ar[2][b], t0i = ai[0][b] + ai[2][b];
          const double t1r = ar[0][b] - ar[2][b], t1i = ai[0][b] - ai[2][b];
          const double t2r = ar[1][b] + ar[3][b], t2i = ai[1][b] + ai[3][b];
          // (a1 - a3) * (-i sg)
          const double dr = ar[1][b] - ar[3][b], di = ai[1][b] - ai[3][b];
          const double t3r = sg * di, t3i = -sg * dr;
          cr[0] = t0r + t2r; ci[0] = t0i + t2i;
          cr[2] = t0r - t2r; ci[2] = t0i - t2i;
          cr[1] = t1r + t3r; ci[1] = t1i + t3i;
          cr[3] = t1r - t3r; ci[3] = t1i - t3i;
        } else if constexpr (P == 3) {
          const double h = 0.86602540378443864676;   // sqrt(3)/2
          const double sr = ar[1][b] + ar[2][b], si = ai[1][b] + ai[2][b];
          const double dr = ar[1][b] - ar[2][b], di = ai[1][b] - ai[2][b];
          const double mr = ar[0][b] - 0.5 * sr, mi = ai[0][b] - 0.5 * si;
          cr[0] = ar[0][b] + sr; ci[0] = ai[0][b] + si;
          // X1 = m - i sg h d, X2 = m + i sg h d
          cr[1] = mr + sg * h * di; ci[1] = mi - sg * h * dr;
          cr[2] = mr - sg * h * di; ci[2] = mi + sg * h * dr;
        } else {
          for (int k = 0; k < P; ++k) {
            double zr = 0.0, zi = 0.0;
            for (int r = 0; r < P; ++r) {
              zr += ar[r][b] * dmr[k][r] - ai[r][b] * dmi[k][r];
              zi += ar[r][b] * dmi[k][r] + ai[r][b] * dmr[k][r];
            }
            cr[k] = zr; ci[k] = zi;
          }
        }
        br[0][b] = cr[0]; bi[0][b] = ci[0];
        for (int k = 1; k < P; ++k) {
          br[k][b] = cr[k] * twr[k] - ci[k] * twi[k];
          bi[k][b] = cr[k] * twi[k] + ci[k] * twr[k];
        }
      }
    }
  }
}

// transform B lines held as planes re/im [n][B]; result lands back in re/im
// (tr/ti scratch of the same size)
void fft_lines(const Plan& P, int B, double* re, double* im, double* tr, double* ti, int sg) {
  double *xr = re, *xi = im, *yr = tr, *yi = ti;
  for (const Stage& S : P.st) {
    switch (S.p) {
      case 4: stage_fixed<4>(S, B, xr, xi, yr, yi, sg); break;
      case 2: stage_fixed<2>(S, B, xr, xi, yr, yi, sg); break;
      case 3: stage_fixed<3>(S, B, xr, xi, yr, yi, sg); break;
      default: stage_fixed<5>(S, B, xr, xi, yr, yi, sg); break;
    }
    std::swap(xr, yr);
    std::swap(xi, yi);
  }
  if (xr != re) {
    std::memcpy(re, xr, sizeof(double) * (size_t)P.n * B);
    std::memcpy(im, xi, sizeof(double) * (size_t)P.n * B);
  }
}

int nint(double v) { return (int)std::lround(v); }

struct Scratch {
  std::vector<double> re, im, tr, ti;
  explicit Scratch(int n) : re((size_t)n * kB), im((size_t)n * kB), tr((size_t)n * kB), ti((size_t)n * kB) {}
};

// NR ludcmp + lubksb (mod_iterate.f90:232-337), row-major a[n][n], in place
void lu_solve(std::vector<double>& a, std::vector<double>& b, int n) {
  std::vector<int> indx(n);
  std::vector<double> vv(n);
  const double tiny = 1.0e-20;
  for (int i = 0; i < n; ++i) {
    double big = 0.0;
    for (int j = 0; j < n; ++j) big = std::fmax(big, std::fabs(a[i * n + j]));
    vv[i] = 1.0 / big;
  }
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < j; ++i) {
      double s = a[i * n + j];
      for (int k = 0; k < i; ++k) s -= a[i * n + k] * a[k * n + j];
      a[i * n + j] = s;
    }
    double big = 0.0;
    int imax = j;
    for (int i = j; i < n; ++i) {
      double s = a[i * n + j];
      for (int k = 0; k < j; ++k) s -= a[i * n + k] * a[k * n + j];
      a[i * n + j] = s;
      const double dum = vv[i] * std::fabs(s);
      if (dum >= big) { imax = i; big = dum; }
    }
    if (j != imax) {
      for (int k = 0; k < n; ++k) std::swap(a[imax * n + k], a[j * n + k]);
      vv[imax] = vv[j];
    }
    indx[j] = imax;
    if (a[j * n + j] == 0.0) a[j * n + j] = tiny;
    if (j != n - 1) {
      const double dum = 1.0 / a[j * n + j];
      for (int i = j + 1; i < n; ++i) a[i * n + j] *= dum;
    }
  }
  int ii = -1;
  for (int i = 0; i < n; ++i) {
    const int ll = indx[i];
    double s = b[ll];
    b[ll] = b[i];
    if (ii >= 0) {
      for (int j = ii; j < i; ++j) s -= a[i * n + j] * b[j];
    } else if (s != 0.0) {
      ii = i;
    }
    b[i] = s;
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = b[i];
    for (int j = i + 1; j < n; ++j) s -= a[i * n + j] * b[j];
    b[i] = s / a[i * n + i];
  }
}

struct Ctx {
  int gx = 0, gy = 0, gz = 0;
  size_t N = 0;
  double lx = 0, ly = 0, lz = 0, ds = 0, volume = 0, dvol = 0;
  int na = 0, nb = 0, ns = 0;
  double kappa = 0, chi = 0, rho = 1.0;
  int m = 2, warm = 2;
  double lam = 0.1, lam_warm = 1e-3;
  Plan px, py, pz;
  std::vector<double> gxy, gzf;   // exp(-ds k^2) separable: [gy][gx] and [gz] / N
  std::vector<double> sr, si;     // slices [ns+1][N]: q (re) and q-dagger (im)
  std::vector<double> fr, fi;     // work field [N]
  std::vector<double> E;          // [2][N] exp(-ds w / 2)
  std::vector<double> w;          // current field x_k [2][N]
  std::vector<double> dens, dens_old, newf;
  std::vector<double> hx, hr;     // Anderson history [m+1][2N] (ring)
  int iter = 0;                   // iterations done
  double Qsum = 0, logQ = 0, mu = 0, energy = 0, F = 0, acc = 0;
};

double wavenum(int i, int n, double L) {
  const double m = (i > n / 2) ? double(i - n) : double(i);
  return 2.0 * M_PI * m / L;
}

// Propagator step t of both chains: slice t-1 -> slice t.  ef / eb are the
// Boltzmann factors of the chains' blocks at step t.
void chain_step(Ctx& c, int t, const double* ef, const double* eb) {
  const int gx = c.gx, gy = c.gy, gz = c.gz;
  const double* qr = c.sr.data() + (size_t)(t - 1) * c.N;
  const double* qi = c.si.data() + (size_t)(t - 1) * c.N;
  double* fr = c.fr.data();
  double* fi = c.fi.data();
  const int nrows = gy * gz;
  const int nxc = (gx + kB - 1) / kB;
  // X forward: pack E_f q + i E_b q-dagger, rows in batches of B
#pragma omp parallel
  {
    Scratch S(std::max(gx, std::max(gy, gz)));
#pragma omp for schedule(static)
    for (int r0 = 0; r0 < nrows; r0 += kB) {
      const int B = std::min(kB, nrows - r0);
      for (int b = 0; b < B; ++b) {
        const size_t base = (size_t)(r0 + b) * gx;
        for (int x = 0; x < gx; ++x) {
          S.re[(size_t)x * B + b] = ef[base + x] * qr[base + x];
          S.im[(size_t)x * B + b] = eb[base + x] * qi[base + x];
        }
      }
      fft_lines(c.px, B, S.re.data(), S.im.data(), S.tr.data(), S.ti.data(), 1);
      for (int b = 0; b < B; ++b) {
        const size_t base = (size_t)(r0 + b) * gx;
        for (int x = 0; x < gx; ++x) {
          fr[base + x] = S.re[(size_t)x * B + b];
          fi[base + x] = S.im[(size_t)x * B + b];
        }
      }
    }
    // Y forward: per z plane, B consecutive x
#pragma omp for schedule(static) collapse(2)
    for (int z = 0; z < gz; ++z)
      for (int xc = 0; xc < nxc; ++xc) {
        const int x0 = xc * kB, B = std::min(kB, gx - x0);
        for (int y = 0; y < gy; ++y) {
          const size_t g = ((size_t)z * gy + y) * gx + x0;
          for (int b = 0; b < B; ++b) { S.re[(size_t)y * B + b] = fr[g + b]; S.im[(size_t)y * B + b] = fi[g + b]; }
        }
        fft_lines(c.py, B, S.re.data(), S.im.data(), S.tr.data(), S.ti.data(), 1);
        for (int y = 0; y < gy; ++y) {
          const size_t g = ((size_t)z * gy + y) * gx + x0;
          for (int b = 0; b < B; ++b) { fr[g + b] = S.re[(size_t)y * B + b]; fi[g + b] = S.im[(size_t)y * B + b]; }
        }
      }
    // Z: forward, exp(-ds k^2)/N, inverse
#pragma omp for schedule(static) collapse(2)
    for (int y = 0; y < gy; ++y)
      for (int xc = 0; xc < nxc; ++xc) {
        const int x0 = xc * kB, B = std::min(kB, gx - x0);
        for (int z = 0; z < gz; ++z) {
          const size_t g = ((size_t)z * gy + y) * gx + x0;
          for (int b = 0; b < B; ++b) { S.re[(size_t)z * B + b] = fr[g + b]; S.im[(size_t)z * B + b] = fi[g + b]; }
        }
        fft_lines(c.pz, B, S.re.data(), S.im.data(), S.tr.data(), S.ti.data(), 1);
        for (int z = 0; z < gz; ++z) {
          const double gzv = c.gzf[z];
          for (int b = 0; b < B; ++b) {
            const double g = c.gxy[(size_t)y * gx + x0 + b] * gzv;
            S.re[(size_t)z * B + b] *= g;
            S.im[(size_t)z * B + b] *= g;
          }
        }
        fft_lines(c.pz, B, S.re.data(), S.im.data(), S.tr.data(), S.ti.data(), -1);
        for (int z = 0; z < gz; ++z) {
          const size_t g = ((size_t)z * gy + y) * gx + x0;
          for (int b = 0; b < B; ++b) { fr[g + b] = S.re[(size_t)z * B + b]; fi[g + b] = S.im[(size_t)z * B + b]; }
        }
      }
    // Y inverse
#pragma omp for schedule(static) collapse(2)
    for (int z = 0; z < gz; ++z)
      for (int xc = 0; xc < nxc; ++xc) {
        const int x0 = xc * kB, B = std::min(kB, gx - x0);
        for (int y = 0; y < gy; ++y) {
          const size_t g = ((size_t)z * gy + y) * gx + x0;
          for (int b = 0; b < B; ++b) { S.re[(size_t)y * B + b] = fr[g + b]; S.im[(size_t)y * B + b] = fi[g + b]; }
        }
        fft_lines(c.py, B, S.re.data(), S.im.data(), S.tr.data(), S.ti.data(), -1);
        for (int y = 0; y < gy; ++y) {
          const size_t g = ((size_t)z * gy + y) * gx + x0;
          for (int b = 0; b < B; ++b) { fr[g + b] = S.re[(size_t)y * B + b]; fi[g + b] = S.im[(size_t)y * B + b]; }
        }
      }
    // X inverse: unpack, E, store slice t
    double* sr = c.sr.data() + (size_t)t * c.N;
    double* si = c.si.data() + (size_t)t * c.N;
#pragma omp for schedule(static)
    for (int r0 = 0; r0 < nrows; r0 += kB) {
      const int B = std::min(kB, nrows - r0);
      for (int b = 0; b < B; ++b) {
        const size_t base = (size_t)(r0 + b) * gx;
        for (int x = 0; x < gx; ++x) {
          S.re[(size_t)x * B + b] = fr[base + x];
          S.im[(size_t)x * B + b] = fi[base + x];
        }
      }
      fft_lines(c.px, B, S.re.data(), S.im.data(), S.tr.data(), S.ti.data(), -1);
      for (int b = 0; b < B; ++b) {
        const size_t base = (size_t)(r0 + b) * gx;
        for (int x = 0; x < gx; ++x) {
          sr[base + x] = ef[base + x] * S.re[(size_t)x * B + b];
          si[base + x] = eb[base + x] * S.im[(size_t)x * B + b];
        }
      }
    }
  }
}

// Propagate_Diblock at the context's E: slices, Q, densities by type
void propagate(Ctx& c) {
  const size_t N = c.N;
  const double* eA = c.E.data();
  const double* eB = c.E.data() + N;
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < N; ++i) { c.sr[i] = 1.0; c.si[i] = 1.0; }
  for (int t = 1; t <= c.ns; ++t) {
    const double* ef = t <= c.na ? eA : eB;   // forward: A then B
    const double* eb = t <= c.nb ? eB : eA;   // backward: B then A
    chain_step(c, t, ef, eb);
  }
  const int ns = c.ns, na = c.na;
  const double* qN = c.sr.data() + (size_t)ns * N;
  double qs = 0.0;
#pragma omp parallel for reduction(+ : qs) schedule(static)
  for (size_t i = 0; i < N; ++i) qs += qN[i];
  c.Qsum = c.dvol * qs;
  // block trapezoid (mod_diblock.f90:143-154)
  const double ds = c.ds;
  const size_t blk = 2048;
#pragma omp parallel for schedule(static)
  for (size_t i0 = 0; i0 < N; i0 += blk) {
    const size_t n = std::min(blk, N - i0);
    double da[blk], db[blk];
    for (size_t k = 0; k < n; ++k) { da[k] = 0.0; db[k] = 0.0; }
    for (int s = 0; s <= ns; ++s) {
      const double* q = c.sr.data() + (size_t)s * N + i0;
      const double* qd = c.si.data() + (size_t)(ns - s) * N + i0;
      double wa = 0.0, wb = 0.0;
      if (s <= na) wa = (s == 0 || s == na) ? 0.5 * ds : ds;
      if (s >= na) wb = (s == na || s == ns) ? 0.5 * ds : ds;
      if (wa != 0.0)
        for (size_t k = 0; k < n; ++k) da[k] += wa * q[k] * qd[k];
      if (wb != 0.0)
        for (size_t k = 0; k < n; ++k) db[k] += wb * q[k] * qd[k];
    }
    // canonical closure (mod_diblock.f90:156-159)
    const double f = c.rho * c.volume / c.Qsum;
    for (size_t k = 0; k < n; ++k) {
      c.dens[i0 + k] = f * da[k];
      c.dens[N + i0 + k] = f * db[k];
    }
  }
  c.mu = std::log(c.rho * c.volume / c.Qsum);
  c.energy = c.rho * c.volume * (c.mu - 1.0);
  c.logQ = std::log(c.Qsum);
}

void set_expfield(Ctx& c) {
  const size_t n2 = 2 * c.N;
  const double h = -0.5 * c.ds;
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < n2; ++i) c.E[i] = std::exp(h * c.w[i]);
}

// one Calculate_Saddle_Point loop body (main_diblock.f90:410-429)
void iterate_once(Ctx& c) {
  const size_t N = c.N, n2 = 2 * N;
  const int it = ++c.iter;
  set_expfield(c);
  propagate(c);
  // accuracy, mean fields, energy terms
  double acc = 0.0, phiw = 0.0, e2 = 0.0, ex = 0.0;
  const double kap = c.kappa, chi = c.chi;
#pragma omp parallel for reduction(+ : acc, phiw, e2, ex) schedule(static)
  for (size_t i = 0; i < N; ++i) {
    const double a = c.dens[i], b = c.dens[N + i];
    const double da = c.dens_old[i] - a, db = c.dens_old[N + i] - b;
    acc += da * da + db * db;
    phiw += a * c.w[i] + b * c.w[N + i];
    const double tot = a + b - 1.0;
    e2 += tot * tot;
    ex += a * b;
    c.newf[i] = kap * tot + chi * b;
    c.newf[N + i] = kap * tot + chi * a;
  }
  c.acc = acc;
  const double eint = 0.5 * kap * c.dvol * e2 + chi * c.dvol * ex;
  c.F = (c.energy - c.dvol * phiw + eint) / (c.rho * c.volume);
  // Anderson mixing, history as a ring of m+1 slots (slot of iterate j: j mod (m+1))
  const int m = c.m, slots = m + 1;
  const int cur = it % slots;
  double* x0 = c.hx.data() + (size_t)cur * n2;
  double* r0 = c.hr.data() + (size_t)cur * n2;
#pragma omp parallel for schedule(static)
  for (size_t i = 0; i < n2; ++i) {
    x0[i] = c.w[i];
    r0[i] = c.newf[i] - c.w[i];
  }
  if (it > c.warm) {
    std::vector<const double*> xi(m), ri(m);
    for (int i = 0; i < m; ++i) {
      const int sl = ((it - 1 - i) % slots + slots) % slots;
      xi[i] = c.hx.data() + (size_t)sl * n2;
      ri[i] = c.hr.data() + (size_t)sl * n2;
    }
    // v_i = <d_i, r0>, U_ij = <d_i, d_j> with d_i = r0 - r_i (:112-121)
    const int nu = m * (m + 1) / 2;
    std::vector<double> acc_v(m, 0.0), acc_u(nu, 0.0);
#pragma omp parallel
    {
      std::vector<double> v(m, 0.0), u(nu, 0.0), d(m);
#pragma omp for schedule(static)
      for (size_t k = 0; k < n2; ++k) {
        const double r = r0[k];
        for (int i = 0; i < m; ++i) d[i] = r - ri[i][k];
        int o = 0;
        for (int i = 0; i < m; ++i) {
          v[i] += d[i] * r;
          for (int j = 0; j <= i; ++j) u[o++] += d[i] * d[j];
        }
      }
#pragma omp critical
      {
        for (int i = 0; i < m; ++i) acc_v[i] += v[i];
        for (int i = 0; i < nu; ++i) acc_u[i] += u[i];
      }
    }
    std::vector<double> U((size_t)m * m), b(acc_v);
    int o = 0;
    for (int i = 0; i < m; ++i)
      for (int j = 0; j <= i; ++j) { U[i * m + j] = acc_u[o]; U[j * m + i] = acc_u[o]; ++o; }
    lu_solve(U, b, m);
    const double lam = c.lam;
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n2; ++k) {
      double xm = x0[k], rm = r0[k];
      for (int i = 0; i < m; ++i) {
        xm -= b[i] * (x0[k] - xi[i][k]);
        rm -= b[i] * (r0[k] - ri[i][k]);
      }
      c.w[k] = xm + lam * rm;
    }
  } else {
    const double lam = c.lam_warm;
#pragma omp parallel for schedule(static)
    for (size_t k = 0; k < n2; ++k) c.w[k] = x0[k] + lam * r0[k];
  }
  std::swap(c.dens_old, c.dens);
}

bool init(Ctx& c, const int* grid, const double* box, double ds, double fA, double kappa, double chi,
          int m, double lam, double lam_warm, int warm) {
  c.gx = grid[0]; c.gy = grid[1]; c.gz = grid[2];
  c.N = (size_t)c.gx * c.gy * c.gz;
  c.lx = box[0]; c.ly = box[1]; c.lz = box[2];
  c.ds = ds;
  c.volume = c.lx * c.ly * c.lz;
  c.dvol = c.volume / (double)c.N;
  c.na = nint(fA / ds);
  c.nb = nint((1.0 - fA) / ds);
  c.ns = c.na + c.nb;
  c.kappa = kappa; c.chi = chi;
  c.m = m < 1 ? 1 : m;
  c.warm = warm < c.m ? c.m : warm;
  c.lam = lam; c.lam_warm = lam_warm;
  if (!make_plan(c.gx, c.px) || !make_plan(c.gy, c.py) || !make_plan(c.gz, c.pz)) return false;
  c.gxy.resize((size_t)c.gx * c.gy);
  for (int y = 0; y < c.gy; ++y)
    for (int x = 0; x < c.gx; ++x) {
      const double kx = wavenum(x, c.gx, c.lx), ky = wavenum(y, c.gy, c.ly);
      c.gxy[(size_t)y * c.gx + x] = std::exp(-ds * kx * kx) * std::exp(-ds * ky * ky);
    }
  c.gzf.resize(c.gz);
  for (int z = 0; z < c.gz; ++z) {
    const double kz = wavenum(z, c.gz, c.lz);
    c.gzf[z] = std::exp(-ds * kz * kz) / (double)c.N;
  }
  const size_t N = c.N;
  c.sr.assign((size_t)(c.ns + 1) * N, 0.0);
  c.si.assign((size_t)(c.ns + 1) * N, 0.0);
  c.fr.assign(N, 0.0);
  c.fi.assign(N, 0.0);
  c.E.assign(2 * N, 1.0);
  c.w.assign(2 * N, 0.0);
  c.dens.assign(2 * N, 0.0);
  c.dens_old.assign(2 * N, 0.0);
  c.newf.assign(2 * N, 0.0);
  c.hx.assign((size_t)(c.m + 1) * 2 * N, 0.0);
  c.hr.assign((size_t)(c.m + 1) * 2 * N, 0.0);
  return true;
}

}  // namespace

extern "C" {

// threads of the OpenMP runtime (the count used by every call)
int scfcpu_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void scfcpu_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// canonical bulk diblock melt (rho = 1), Anderson mixing with history m
void* scfcpu_create(const int* grid, const double* box, double ds, double fA, double kappa,
                    double chi, int m, double lam, double lam_warm, int warm_iters) {
  Ctx* c = new (std::nothrow) Ctx;
  if (!c) return nullptr;
  try {
    if (!init(*c, grid, box, ds, fA, kappa, chi, m, lam, lam_warm, warm_iters)) {
      delete c;
      return nullptr;
    }
  } catch (...) {
    delete c;
    return nullptr;
  }
  return c;
}
void scfcpu_destroy(void* h) { delete static_cast<Ctx*>(h); }

int scfcpu_contour_steps(void* h) { return static_cast<Ctx*>(h)->ns; }

// x_1 = field [2][N]; resets the iteration count and the density history
void scfcpu_set_field(void* h, const double* field) {
  Ctx& c = *static_cast<Ctx*>(h);
  std::memcpy(c.w.data(), field, sizeof(double) * 2 * c.N);
  std::fill(c.dens_old.begin(), c.dens_old.end(), 0.0);
  c.iter = 0;
}
void scfcpu_get_field(void* h, double* field) {
  Ctx& c = *static_cast<Ctx*>(h);
  std::memcpy(field, c.w.data(), sizeof(double) * 2 * c.N);
}
// densities of the last iteration
void scfcpu_get_density(void* h, double* density) {
  Ctx& c = *static_cast<Ctx*>(h);
  std::memcpy(density, c.dens_old.data(), sizeof(double) * 2 * c.N);
}

// n SCF iterations; out[0..3] = accuracy, free energy per chain, log Q,
// iteration index of the last one
void scfcpu_iterate(void* h, int n, double* out) {
  Ctx& c = *static_cast<Ctx*>(h);
  for (int k = 0; k < n; ++k) iterate_once(c);
  if (out) { out[0] = c.acc; out[1] = c.F; out[2] = c.logQ; out[3] = c.iter; }
}

// Propagate_Diblock at `field`: density [2][N]; out[0..3] = Qsum, log Q,
// mu, chain energy (canonical)
void scfcpu_propagate(void* h, const double* field, double* density, double* out) {
  Ctx& c = *static_cast<Ctx*>(h);
  std::vector<double> keep(c.w);
  std::memcpy(c.w.data(), field, sizeof(double) * 2 * c.N);
  set_expfield(c);
  propagate(c);
  std::memcpy(density, c.dens.data(), sizeof(double) * 2 * c.N);
  c.w.swap(keep);
  if (out) { out[0] = c.Qsum; out[1] = c.logQ; out[2] = c.mu; out[3] = c.energy; }
}

// In-place 3D complex FFT of data [gz][gy][gx] (interleaved re, im);
// sign -1 forward (exp(-i...)), +1 inverse, unnormalised.  Returns 0, or 1
// for a length with a prime factor above 5.
int scfcpu_fft3d(int gx, int gy, int gz, double* data, int sign) {
  Plan px, py, pz;
  if (!make_plan(gx, px) || !make_plan(gy, py) || !make_plan(gz, pz)) return 1;
  const int sg = sign < 0 ? 1 : -1;
  Scratch S(std::max(gx, std::max(gy, gz)));
  auto run = [&](const Plan& P, int n, size_t stride, size_t base, int B, size_t bstride) {
    for (int i = 0; i < n; ++i)
      for (int b = 0; b < B; ++b) {
        const size_t g = 2 * (base + i * stride + b * bstride);
        S.re[(size_t)i * B + b] = data[g];
        S.im[(size_t)i * B + b] = data[g + 1];
      }
    fft_lines(P, B, S.re.data(), S.im.data(), S.tr.data(), S.ti.data(), sg);
    for (int i = 0; i < n; ++i)
      for (int b = 0; b < B; ++b) {
        const size_t g = 2 * (base + i * stride + b * bstride);
        data[g] = S.re[(size_t)i * B + b];
        data[g + 1] = S.im[(size_t)i * B + b];
      }
  };
  for (int z = 0; z < gz; ++z)
    for (int y = 0; y < gy; ++y) run(px, gx, 1, ((size_t)z * gy + y) * gx, 1, 0);
  for (int z = 0; z < gz; ++z)
    for (int x = 0; x < gx; ++x) run(py, gy, gx, (size_t)z * gy * gx + x, 1, 0);
  for (int y = 0; y < gy; ++y)
    for (int x = 0; x < gx; ++x) run(pz, gz, (size_t)gx * gy, (size_t)y * gx + x, 1, 0);
  return 0;
}

}  // extern "C"
