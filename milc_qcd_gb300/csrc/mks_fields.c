/* mks_fields.c -- host-side lattice geometry, staggered phases and the
 * seeded synthetic fields of the C ABI (mks_gen_*, defined in mks_synth.h,
 * which the CPU oracle compiles too).
 *
 * Geometry follows MILC's single-node layout (generic/layout_hyper_prime.c:
 * 509-520): lexicographic i = x + nx*(y + ny*(z + nz*t)); even sites
 * ((x+y+z+t) even) are stored first at i/2, odd sites at (i+V)/2.
 *
 * Staggered phases follow generic_ks/rephase.c:53-96 (eta_t = 1,
 * eta_x = (-1)^t, eta_y = (-1)^(t+x), eta_z = (-1)^(t+x+y), with an extra
 * minus sign on t-links of the t = nt-1 slice for antiperiodic time BC).
 *
 * This file runs on the host only; it prepares inputs and never touches
 * the device.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <stddef.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/milc_ks_gb300.h"
#include "mks_synth.h"

/* ---------------- geometry ---------------- */
void mks_site_coords(const int dims[4], size_t index, int xyzt[4]) { synth_site_coords(dims, index, xyzt); }

size_t mks_site_index(const int dims[4], const int xyzt[4]) {
  size_t V = (size_t)dims[0] * dims[1] * dims[2] * dims[3];
  size_t i = synth_lex(dims, xyzt);
  if (((xyzt[0] + xyzt[1] + xyzt[2] + xyzt[3]) & 1) == 0) return i / 2;
  return (i + V) / 2;
}

double mks_staggered_phase(const int dims[4], const int xyzt[4], int dir) {
  int x = xyzt[0], y = xyzt[1], t = xyzt[3];
  double px = (t & 1) ? -1.0 : 1.0;
  double py = (x & 1) ? -px : px;
  double pz = (y & 1) ? -py : py;
  double pt = (t == dims[3] - 1) ? -1.0 : 1.0;
  switch (dir) {
  case 0: return px;
  case 1: return py;
  case 2: return pz;
  default: return pt;
  }
}

/* ---------------- seeded synthetic fields ---------------- */
int mks_gen_thin_links(const int dims[4], uint64_t seed, double a, double *links) {
  if (!synth_dims_ok(dims) || !links) return MKS_ERR_ARG;
  synth_thin_links(dims, seed, a, links);
  return MKS_OK;
}

int mks_apply_phases(const int dims[4], double *links, int sign) {
  if (!dims || !links) return MKS_ERR_ARG;
  (void)sign; /* phases are +-1: folding in and out are the same product */
  size_t V = (size_t)dims[0] * dims[1] * dims[2] * dims[3];
  long long n = (long long)V;
#pragma omp parallel for schedule(static)
  for (long long idx = 0; idx < n; idx++) {
    int c[4];
    mks_site_coords(dims, (size_t)idx, c);
    for (int dir = 0; dir < 4; dir++) {
      double ph = mks_staggered_phase(dims, c, dir);
      double *m = links + ((size_t)idx * 4 + dir) * 18;
      for (int k = 0; k < 18; k++) m[k] *= ph;
    }
  }
  return MKS_OK;
}

int mks_gen_vector(const int dims[4], uint64_t seed, int parity, double *vec) {
  if (!dims || !vec) return MKS_ERR_ARG;
  synth_vector(dims, seed, parity, vec);
  return MKS_OK;
}

int mks_gen_momenta(const int dims[4], uint64_t seed, double *mom) {
  if (!dims || !mom) return MKS_ERR_ARG;
  synth_momenta(dims, seed, mom);
  return MKS_OK;
}
