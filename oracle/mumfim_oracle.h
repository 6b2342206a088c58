/*
 * mumfim_oracle.h -- CPU restatement of MuMFiM's batched explicit
 * fiber-network RVE solve.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker the GPU library is compared
 * against (tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg);
 * nothing in the product links, loads or calls it.
 *
 * The arithmetic follows the reference's batched path operation by operation
 * (file:line citations in mumfim_oracle.cpp), with the serial accumulation
 * order of a TEAM_SIZE=1 host build. It is compiled with -ffp-contract=off so
 * that no multiply-add is fused.
 *
 * The input/output structs are the product's (include/mumfim_gpu.h) so the
 * two take identical arguments.
 */
#ifndef MUMFIM_ORACLE_H
#define MUMFIM_ORACLE_H
#include <stdint.h>
#include "mumfim_gpu.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_batch orc_batch;

orc_batch* orc_batch_create(const mfg_network* nets, const mfg_strategy* ss, int32_t n_rve);
void orc_batch_destroy(orc_batch* b);
/* n_threads > 1 solves RVEs concurrently, one RVE per thread at a time (the
 * structure of a Kokkos host build with TEAM_SIZE=1), each thread taking the
 * next unsolved RVE. */
int32_t orc_batch_run(orc_batch* b, const double* F, int32_t n_F, double* sigma,
                      int32_t update_coords, mfg_rve_status* status, int32_t n_threads);
int32_t orc_batch_material_stiffness(orc_batch* b, double* C, int32_t n_threads);
int32_t orc_batch_orientation_3d(orc_batch* b, double* omega);
int32_t orc_batch_orientation_2d(orc_batch* b, const double* normal, double* omega);
int32_t orc_batch_get_displacements(orc_batch* b, int32_t rve, double* u);
int32_t orc_batch_get_coordinates(orc_batch* b, int32_t rve, double* x);
int32_t orc_batch_get_current_stress(orc_batch* b, double* sigma);

/* Setup pieces, exposed for known-answer tests. */
/* Boundary-last permutation old id -> new id (BatchedReorderMesh.h:54-73). */
void orc_reorder_permutation(int32_t n_vert, const int32_t* fixed, int32_t n_fixed,
                             int32_t* perm);
/* Boundary node ids of a network in mesh order (RVE.h:86-103), returns count. */
int32_t orc_boundary_nodes(int32_t n_nodes, const double* coords, int32_t* out);
/* Scale conversion 1 / d^2 of the multiscale coupling
 * (MultiscaleCoupling.cc:7-23). */
double orc_scale_conversion(int32_t n_nodes, const double* coords, int32_t n_fibers,
                            const int32_t* conn, double fiber_radius, double volume_fraction);
/* Row-sum lumped nodal mass (MassIntegrator.cc:16-56), original order. */
void orc_nodal_mass(int32_t n_nodes, const double* coords, int32_t n_fibers,
                    const int32_t* conn, double density, double area, double* mass);

#ifdef __cplusplus
}
#endif
#endif
