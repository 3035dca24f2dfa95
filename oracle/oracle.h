/*
 * oracle.h - CPU oracle of the rod collision-and-constraint step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is an FP64 C++/OpenMP restatement of the
 * published method that SimToolbox's SylinderSystem::runStep implements
 * (aLENS: Yan et al., eLife 11:e74160 (2022); constraint formulation and
 * BBPGD: Yan, Zhang, Shelley, J. Chem. Phys. 150:064109 (2019)).  Only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark may load
 * it; the GPU library never does.
 *
 * Parity with SimToolbox itself is UNPINNED: the SimToolbox submodule is
 * empty in the reference checkout (.gitmodules:1-6) and the reference ships
 * no tests or golden outputs for this path.
 *
 * The API mirrors include/alens_gpu.h for a single system.
 */
#ifndef ALENS_ORACLE_H
#define ALENS_ORACLE_H

#include "../include/alens_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OrcCtx OrcCtx;

int orc_create(const AlensConfig *cfg, OrcCtx **out);
int orc_destroy(OrcCtx *ctx);
int orc_set_rods(OrcCtx *ctx, int n, const int64_t *gid, const double *pos,
                 const double *orientation, const double *length,
                 const double *radius, const int32_t *immovable);
int orc_update_rods(OrcCtx *ctx, int n, const double *pos,
                    const double *orientation);
int orc_get_rods(OrcCtx *ctx, int n, double *pos, double *orientation);
int orc_get_velocity(OrcCtx *ctx, int n, double *vel, double *omega);
int orc_add_bilateral(OrcCtx *ctx, int n, const AlensBlock *blocks);
int orc_set_initial_gamma(OrcCtx *ctx, int n, const double *gamma);
int orc_set_boundaries(OrcCtx *ctx, int n, const AlensBoundary *boundaries);
int orc_set_links(OrcCtx *ctx, int n, const int32_t *indexI, const int32_t *indexJ, const double *sI,
                  const double *sJ, const double *restLength, const double *kappa);
int orc_step(OrcCtx *ctx, AlensStepStats *stats);
int orc_detect(OrcCtx *ctx, AlensStepStats *stats);
int orc_solve(OrcCtx *ctx, AlensStepStats *stats);
int orc_advance(OrcCtx *ctx, AlensStepStats *stats);
int orc_get_num_constraints(OrcCtx *ctx, int *nCollision, int *nBilateral);
int orc_get_constraints(OrcCtx *ctx, int cap, int32_t *indexI,
                        int32_t *indexJ, int32_t *image, double *delta0,
                        double *gamma, double *jac);
int orc_get_con_stress(OrcCtx *ctx, double *stress9);
int orc_get_known_velocity(OrcCtx *ctx, int n, double *vel6);
int orc_get_step_count(OrcCtx *ctx, int64_t *count);
/* q and diag(A) of the current constraints (after detect). */
int orc_get_solver_data(OrcCtx *ctx, int cap, double *q, double *diag);
int orc_get_operator(OrcCtx *ctx, int capNnz, int *nnz, int32_t *rowPtr, int32_t *cols, double *vals);
int orc_set_threads(int nthreads);

/* Protein binding step (oracle_kmc.cpp), mirroring alens_set_protein_types,
 * alens_set_proteins, alens_get_proteins and alens_protein_bind_step. */
int orc_set_protein_types(OrcCtx *ctx, int n, const AlensProteinType *types, double KBT, double rodDiameter);
int orc_set_proteins(OrcCtx *ctx, int n, const AlensProtein *proteins);
int orc_get_proteins(OrcCtx *ctx, int cap, int *n, AlensProtein *proteins);
int orc_protein_bind_step(OrcCtx *ctx, AlensKmcStats *stats);
int orc_protein_motion_step(OrcCtx *ctx, AlensKmcStats *stats);
void orc_normal_pair(uint32_t wa, uint32_t wb, double *z0, double *z1);
double orc_kmc_exp(double x);
float orc_kmc_expf(float x);
double orc_kmc_sd_integral(const AlensProteinType *t, double KBT, double D, double dt, double d2, double sA,
                           double sB);
double orc_kmc_sd_invert(const AlensProteinType *t, double KBT, double D, double dt, double d2, double sA,
                         double sB, double target);
double orc_kmc_bind_volume(const AlensProteinType *t, double KBT, double D);
double orc_kmc_binding_factor_sd(const AlensProteinType *t, int end, const double dirBound[3],
                                 const double dirRod[3]);
void orc_kmc_type_constants(const AlensProteinType *t, double KBT, double D, double dt, double out[12]);

/* Building blocks exposed for known-answer tests. */
void orc_dcp(const double c1[3], const double u1[3], double h1,
             const double c2[3], const double u2[3], double h2,
             double *s, double *t, double P[3], double Q[3], double *dist);
double orc_log(double x);
void orc_sincos(double x, double *s, double *c);
void orc_philox4x32(const uint32_t ctr[4], const uint32_t key[2],
                    uint32_t out[4]);
void orc_normals6(uint64_t seed, int64_t gid, int64_t step, double z[6]);
double orc_canon_sum(const double *v, int64_t n);
void orc_mobility(double length, double radius, double viscosity,
                  double out3[3]);

#ifdef __cplusplus
}
#endif

#endif
