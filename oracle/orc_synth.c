/* orc_synth.c -- the seeded synthetic inputs, exported by the oracle library.
 *
 * TEST INFRASTRUCTURE ONLY.  The generators are defined once, in
 * milc_qcd_gb300/csrc/mks_synth.h, and compiled both here and into the
 * product library (mks_gen_*), so a process that must not load the product
 * library -- the CPU reference arm of the benchmark -- builds the same
 * links, sources and momenta bit for bit.  Staggered phases for these links
 * come from orc_rephase (milc_oracle.c).
 */
#include "../milc_qcd_gb300/csrc/mks_synth.h"

int orc_gen_thin_links(const int dims[4], uint64_t seed, double a, double *links) {
  if (!synth_dims_ok(dims) || !links) return -1;
  synth_thin_links(dims, seed, a, links);
  return 0;
}

int orc_gen_vector(const int dims[4], uint64_t seed, int parity, double *vec) {
  if (!synth_dims_ok(dims) || !vec) return -1;
  synth_vector(dims, seed, parity, vec);
  return 0;
}

int orc_gen_momenta(const int dims[4], uint64_t seed, double *mom) {
  if (!synth_dims_ok(dims) || !mom) return -1;
  synth_momenta(dims, seed, mom);
  return 0;
}
