/*
 * ggem_io.h -- particle input and output in the reference's file formats,
 * so that COPSS inputs feed the GPU path and trajectories come out as the
 * reference writes them.
 *
 *   ggem_read_polymer_data   PolymerChain::read_particles_data
 *                            (polymer_chain.C:61-226, LAMMPS-style data file)
 *   ggem_read_polymer_vtk    PolymerChain::read_data_vtk (polymer_chain.C:396-494)
 *   ggem_write_polymer_vtk   PolymerChain::write_polymer_trajectory
 *                            (polymer_chain.C:1096-1154, output_polymer_<k>.vtk)
 *   ggem_write_bead_csv      PolymerChain::write_bead_trajectory
 *                            (polymer_chain.C:1340-1378, output_bead_<k>.csv)
 *   ggem_write_petsc_vec /   the restart vectors vector_RIN.dat / _ROUT.dat
 *   ggem_read_petsc_vec      (copss.C:1391-1414): PETSc's binary Vec format,
 *                            big-endian int32 class id 1211214, int32 length,
 *                            then the values as big-endian float64
 *
 * Host code only; ids in memory are 0-based (the data file's are 1-based).
 */
#ifndef GGEM_IO_H
#define GGEM_IO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ggem_polymer_data {
  int64_t n_beads, n_bonds;
  int n_bead_types, n_bond_types, n_chains;
  int has_box;                 /* the "xlo xhi" lines were present */
  double box_lo[3], box_hi[3];
  double *xyz;                 /* [n_beads][3] */
  int32_t *chain_id;           /* [n_beads], 0-based */
  int32_t *bead_type;          /* [n_beads], 0-based */
  double *rot;                 /* [n_beads][3] rotation-vector columns */
  double *const_force;         /* [n_beads][3] */
  double *charge;              /* [n_beads] */
  double *mass;                /* [n_bead_types] */
  int64_t *bonds;              /* [n_bonds][2], 0-based bead ids */
  int32_t *bond_type;          /* [n_bonds], 0-based */
} ggem_polymer_data;

/* 0 or GGEM_ERR_BAD_ARG (unreadable or malformed file); arrays are
 * allocated by the library and released by ggem_free_polymer_data */
int ggem_read_polymer_data(const char *path, ggem_polymer_data *out);
int ggem_read_polymer_vtk(const char *path, ggem_polymer_data *out);
void ggem_free_polymer_data(ggem_polymer_data *d);

/* positions with `precision` fixed decimals (the reference uses 6) */
int ggem_write_polymer_vtk(const char *path, int64_t n, const double *xyz, int64_t m,
                           const int64_t *bonds, const int32_t *chain_id, int precision);
/* velocity and force may be NULL (written as 0) */
int ggem_write_bead_csv(const char *path, int64_t n, const double *xyz, const double *vel,
                        const double *force, int precision);

int ggem_write_petsc_vec(const char *path, int64_t n, const double *v);
/* n_expected < 0 accepts any length; *n_read gets the file's length; v may
 * be NULL to query it */
int ggem_read_petsc_vec(const char *path, int64_t n_expected, double *v, int64_t *n_read);

#ifdef __cplusplus
}
#endif
#endif
