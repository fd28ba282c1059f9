// film_host.h -- host-side mesh coefficients, integration weights and contour
// schedules of films and brushes, shared by the film context (film.cu) and
// film batches (batch.cu).
#pragma once
#include <algorithm>
#include <string>
#include <vector>

#include "../../include/adscf.h"

struct FilmTables {
  std::vector<double> al, be, ga;   // [gz+1] a_z = -ds al, c_z = -ds ga, b_z = ds be
  std::vector<double> wz;           // [gz+1] integration weights dx dy w_z
  std::vector<double> dss;          // [ns+1] contour steps, dss[0] = 0 unless given
  std::vector<double> wA, wB;       // [ns+1] contour weights per block
  double max_ratio = 1.0;           // largest neighbour spacing ratio of the mesh
  double chain_len = 0.0;           // sum of the contour steps
};

// geometry, grid (gz intervals), dz[0..gz], box (dx = sizex/gx, dy = sizey/gy),
// integrator choice, contour steps ns / A-block steps na, and either
// dss[0..ns] or a uniform ds.
inline int film_tables(const adscf_params& p, int ns, int na, FilmTables& T, std::string& why) {
  const int gz = p.gz;
  if (gz < 2) { why = "films need gz >= 2 intervals"; return ADSCF_E_ARG; }
  if (!p.dz) { why = "films need dz"; return ADSCF_E_ARG; }
  for (int i = 1; i <= gz; ++i)
    if (!(p.dz[i] > 0)) { why = "dz[1..gz] must be positive"; return ADSCF_E_ARG; }
  const double* dz = p.dz;
  // z coefficients: Film_1D / Brush form b = ds (h1+h2)/h1/h2/(h1+h2)
  // (Film_1D/.../mod_realspace.f90:36-43), Film_3D form b = ds/h1/h2 (:70-76)
  T.al.assign(gz + 1, 0.0); T.be.assign(gz + 1, 0.0); T.ga.assign(gz + 1, 0.0);
  T.max_ratio = 1.0;
  for (int z = 1; z < gz; ++z) {
    const double h1 = dz[z], h2 = dz[z + 1];
    T.al[z] = 1.0 / h1 / (h1 + h2);
    T.ga[z] = 1.0 / h2 / (h1 + h2);
    T.be[z] = p.geometry == ADSCF_FILM_3D ? 1.0 / h1 / h2 : (h1 + h2) / h1 / h2 / (h1 + h2);
    T.max_ratio = std::max(T.max_ratio, std::max(h1 / h2, h2 / h1));
  }
  // integrator weights dx dy w_z (Film_3D/.../mod_realspace.f90:267-281 for
  // span 0, Film_1D :201-218 and Brush mod_adaptive.f90:124-143 for span 1)
  const double dx = p.sizex / p.gx, dy = p.sizey / p.gy;
  T.wz.assign(gz + 1, 0.0);
  if (p.int_scheme == 0) {
    const int lo = p.int_span == 0 ? 0 : 1;
    for (int i = lo; i <= gz - 1; ++i) T.wz[i] += dz[i];
  } else {
    const int hi = p.int_span == 0 ? gz : gz - 1;
    for (int i = 1; i <= hi; ++i) { T.wz[i - 1] += 0.5 * dz[i]; T.wz[i] += 0.5 * dz[i]; }
  }
  for (double& v : T.wz) v *= dx * dy;
  // contour schedule dss[0..ns]
  T.dss.assign(ns + 1, 0.0);
  if (p.dss) {
    for (int s = 0; s <= ns; ++s) T.dss[s] = p.dss[s];
  } else {
    for (int s = 1; s <= ns; ++s) T.dss[s] = p.ds;
  }
  T.chain_len = 0.0;
  for (int s = 1; s <= ns; ++s) T.chain_len += T.dss[s];
  // contour weights: diblock = trapezoid per block with the step sizes
  // (mod_diblock.f90:143-154 for uniform steps); brush = the
  // 1/2 (dss_s + dss_{s+1}) rule of mod_homopolymer.f90:231-239
  T.wA.assign(ns + 1, 0.0); T.wB.assign(ns + 1, 0.0);
  if (p.geometry == ADSCF_BRUSH) {
    T.wA[0] = 0.5 * T.dss[0];
    for (int s = 1; s < ns; ++s) T.wA[s] = 0.5 * (T.dss[s] + T.dss[s + 1]);
    T.wA[ns] = 0.5 * T.dss[ns];
  } else {
    for (int s = 0; s < na; ++s) { T.wA[s] += 0.5 * T.dss[s + 1]; T.wA[s + 1] += 0.5 * T.dss[s + 1]; }
    for (int s = na; s < ns; ++s) { T.wB[s] += 0.5 * T.dss[s + 1]; T.wB[s + 1] += 0.5 * T.dss[s + 1]; }
  }
  return ADSCF_OK;
}

// split precision keeps the Thomas sweep in FP64 on meshes graded past a
// neighbour spacing ratio of 1.5
inline bool film_sweep_fp64(int precision, double max_ratio) {
  return !(precision == ADSCF_SPLIT && max_ratio <= 1.5);
}
