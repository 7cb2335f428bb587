/*
 * ggem_workloads.h -- seeded synthetic inputs for tests and benchmarks.
 *
 * These generators are not part of the reference's interface: the reference
 * reads LAMMPS-style data files (polymer_chain.C:61-226) produced by an
 * external packer.  They stand in for those inputs with the shapes of the
 * benchmark configurations: random sequential non-overlapping beads and
 * self-avoiding bead-spring chains in a periodic cube.
 */
#ifndef GGEM_WORKLOADS_H
#define GGEM_WORKLOADS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* n beads of `radius`, no two closer than 2*radius, volume fraction phi in a
 * periodic cube [0, L)^3; writes xyz[3n] and L */
int ggem_make_suspension(uint64_t seed, int64_t n, double phi, double radius, double *xyz,
                         double *box_length);
/* n_chains self-avoiding random-walk chains of beads_per_chain beads, bond
 * length `bond`, beads no closer than 2*radius (bonded pairs excepted) */
int ggem_make_chains(uint64_t seed, int64_t n_chains, int beads_per_chain, double bond,
                     double phi, double radius, double *xyz, double *box_length);
/* n iid N(0,1) values */
/* n_chains chains of beads_per_chain beads (grown as in ggem_make_chains)
 * followed by n_free free beads placed by random sequential addition, all
 * non-overlapping, in the periodic cube of volume fraction phi; beads
 * [0, n_chains * beads_per_chain) are the chains */
int ggem_make_mixture(uint64_t seed, int64_t n_chains, int beads_per_chain, int64_t n_free,
                      double bond, double phi, double radius, double *xyz, double *box_length);
int ggem_make_normals(uint64_t seed, int64_t n, double *out);

#ifdef __cplusplus
}
#endif
#endif
