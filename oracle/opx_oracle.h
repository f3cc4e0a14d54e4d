/*
 * opx_oracle.h -- CPU FP64 oracle for the OpenPixi temporal-gauge Yang-Mills
 * leapfrog, its CPIC (NGP) coupling and the field reductions.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: only the test suite,
 * the smoke check and the CPU-baseline leg of the benchmark load it.  The GPU
 * product never links or calls it.
 *
 * It restates, operation by operation, the sequential (one-thread) behaviour of
 * the Java reference (paths relative to pixi/src/main/java/org/openpixi/pixi):
 *   math/SU2GroupElement.java, math/SU2AlgebraElement.java,
 *   math/SU3GroupElement.java, math/SU3AlgebraElement.java,
 *   physics/grid/Grid.java, physics/grid/Cell.java,
 *   physics/fields/FastTYMSolver.java,
 *   physics/measurements/FieldMeasurements.java,
 *   diagnostics/methods/{BulkQuantitiesInTime,EnergyDensity,
 *                        ProjectedEnergyDensity,GaussConstraintRestoration}.java,
 *   physics/grid/CGCParticleInterpolationNGP.java,
 *   physics/movement/solver/CGCParticleSolver.java,
 *   physics/particles/YangMillsParticle.java, physics/util/GridFunctions.java.
 *
 * Pinning: the reference ships no golden vectors.  The oracle is pinned by the
 * reference's own property tests (SU2MatrixTest, SU2FieldTest,
 * SU3EverythingTest, GridTest, GaussConstraintTest), restated in tests/, and by
 * an independent matrix-library check (numpy/scipy) of every group operation.
 * Step-level trajectories are not pinned by the reference ("parity unpinned"
 * at the trajectory level); golden fixtures produced by this oracle pin it
 * against regressions.
 *
 * Layout ("reference layout", the per-Cell object layout flattened):
 *   U, Unext : [V][3][ng]   ng = 4 (SU(2) quaternion e0..e3) or 18 (SU(3): 9 re, 9 im)
 *   E, J     : [V][3][na]   na = 3 (SU(2) v0..v2) or 9 (SU(3) hermitian entries v[9])
 *   rho      : [V][na]
 *   active, eval : [V] uint8
 * Site index = ((x0*N1)+x1)*N2+x2 (dimension 0 slowest), Grid.java:757-770.
 *
 * Compiled with -ffp-contract=off so that no multiply-add is fused, as in Java.
 */
#ifndef OPX_ORACLE_H
#define OPX_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nc;          /* number of colours: 2 or 3 */
    int n[3];        /* lattice cells per direction */
    double a[3];     /* lattice spacing per direction */
    double dt;       /* temporal spacing */
    double g;        /* gauge coupling */
} orc_params;

int orc_ng(int nc);
int orc_na(int nc);

/* ---- group / algebra math (math package) ---- */
void orc_group_mult(int nc, const double *l, const double *r, double *out);
void orc_group_adj(int nc, const double *u, double *out);
void orc_group_proj(int nc, const double *u, double *alg);
void orc_alg_getlink(int nc, const double *alg, double *u);
void orc_alg_act(int nc, const double *alg, const double *g, double *out);
double orc_alg_square(int nc, const double *alg);
void orc_alg_to_gen(int nc, const double *alg, double *gen);
void orc_gen_to_alg(int nc, const double *gen, double *alg);

/* ---- grid (physics/grid/Grid.java) ---- */
long orc_shift(const orc_params *p, long index, int dir, int orient);
void orc_staple_sum(const orc_params *p, const double *U, long index, int d, double *S);
void orc_plaquette(const orc_params *p, const double *U, long index, int d1, int d2,
                   int o1, int o2, double *out);
void orc_get_b(const orc_params *p, const double *U, long index, int dir, double *alg);
void orc_gauss_constraint(const orc_params *p, const double *U, const double *E,
                          const double *rho, long index, double *alg);

/* ---- leapfrog (physics/fields/FastTYMSolver.java) ---- */
void orc_update_grid(const orc_params *p, const double *U, double *E, const double *J,
                     double *Unext, const uint8_t *active);
/* TemporalYangMillsSolver.step: the plaquette form, E pass then link pass */
void orc_update_grid_tym(const orc_params *p, const double *U, double *E, const double *J,
                         double *Unext, const uint8_t *active);
void orc_update_links(const orc_params *p, const double *U, const double *E,
                      double *Unext, const uint8_t *active);
/* Same algorithm split over host threads (OpenMP); timed CPU baseline only. */
void orc_update_grid_omp(const orc_params *p, const double *U, double *E, const double *J,
                         double *Unext, const uint8_t *active, int nthreads);
void orc_update_grid_range_omp(const orc_params *p, const double *U, double *E, const double *J,
                               double *Unext, const uint8_t *active, long s0, long s1, int nthreads);
int orc_max_threads(void);

/* ---- reductions (FieldMeasurements / BulkQuantitiesInTime) ----
 * out[0..2]  = E^2 per direction (getSum(dir): divided by V)
 * out[3..5]  = B^2 per direction (average of U and Unext plaquettes, divided by V)
 * out[6..8]  = P_x, P_y, P_z
 * out[9]     = mean Gauss violation squared
 * out[10]    = sqrt(sum rho^2)/V  (TotalChargeSquared.getSum)
 * out[11]    = E^2 total (sum over directions), out[12] = B^2 total          */
void orc_bulk(const orc_params *p, const double *U, const double *Unext, const double *E,
              const double *rho, const uint8_t *eval, double *out);
void orc_energy_density(const orc_params *p, const double *U, const double *Unext,
                        const double *E, const uint8_t *eval, double *out);
/* out: 4 rows of N[dir]: T_el, T_mag, L_el, L_mag (ProjectedEnergyDensity order) */
void orc_projected_energy(const orc_params *p, const double *U, const double *Unext,
                          const double *E, const uint8_t *eval, int dir, double *out);
/* out: 2 rows of N[dir]: Poynting averaged, time-averaged (SU(2); -1 for SU(3)) */
int orc_projected_poynting(const orc_params *p, const double *U, const double *Unext,
                           const double *E, int dir, double *out);
void orc_gauss_field(const orc_params *p, const double *U, const double *E,
                     const double *rho, double *out /* [V][na] */);

/* ---- CPIC NGP (CGCParticleInterpolationNGP / CGCParticleSolver) ----
 * Particles in the reference's object semantics, as structure of arrays:
 *   pos0,pos1,vel : [n][3];  Q0,Q1 : [n][na];  dir : [n];  flag : [n] (updateCharge)
 *   Ulink : [n][ng] (the cached P.U of the particle)                         */
void orc_cpic_reassign(int nc, long np, double *pos0, double *pos1, double *Q0, double *Q1);
void orc_cpic_charge_density(const orc_params *p, long np, const double *pos0,
                             const double *Q0, double *rho);
void orc_cpic_update_positions(const orc_params *p, long np, const double *pos0,
                               double *pos1, const double *vel);
void orc_cpic_to_particle(const orc_params *p, long np, const double *pos0,
                          const double *pos1, const double *vel, const int32_t *dir,
                          const double *Unext, double *Ulink, uint8_t *flag);
void orc_cpic_update_charges(int nc, long np, double *Q0, double *Q1,
                             const double *Ulink, uint8_t *flag);
void orc_cpic_to_grid(const orc_params *p, long np, const double *pos0,
                      const double *pos1, const double *vel, const int32_t *dir,
                      const double *Q0, const double *Q1, double *J);
void orc_ngp(const orc_params *p, const double *pos, int32_t *cell3);

/* ---- seeded synthetic initial conditions ---- */
double orc_normal(uint64_t seed, uint64_t ctr);
void orc_random_gen(uint64_t seed, uint64_t stream, long count, double sigma, double *out);
void orc_random_fields(const orc_params *p, uint64_t seed, double sigma_a, double sigma_e,
                       double *U, double *E);
/* Covariant Gauss projection by conjugate gradients on div(divT mu) = rho - div E.
 * Returns iterations used; *final_g2 = mean G^2 afterwards. */
int orc_gauss_project_cg(const orc_params *p, const double *U, double *E, const double *rho,
                         double tol_g2, int maxit, double *final_g2);
/* GaussConstraintRestoration.iterateRestorationAlgorithm (hep-ph/9603384 iteration). */
int orc_gauss_restoration(const orc_params *p, double *U, double *Unext, double *E,
                          const double *rho, double gamma, int maxit, double absval,
                          double *final_violation);

/* ---- CGC initial conditions (physics/initial/CGC) ---- */
/* java.util.Random(seed): kind 0 nextGaussian, 1 nextDouble, 2 nextInt */
void orc_java_random(int64_t seed, int kind, long count, double *out);
/* StrictMath.log (fdlibm) */
double orc_strict_log(double x);
/* MVModel.initialize before regulation: out [ncomp][V] generator components */
void orc_mv_charges(const orc_params *p, int direction, double location, double width, double mu,
                    int64_t seed, double *out);
/* LightConePoissonSolverImproved.solve after the Poisson solves */
void orc_cgc_solve(const orc_params *p, int direction, int orientation, const double *phi,
                   double *U, double *Unext, double *E, const uint8_t *active, double *gauss, double *vt);
/* SU3GroupElement.getAlgebraElement in generator components (own eigen-decomposition) */
void orc_su3_log_gen(const double *u, double *gen);
void orc_su3_pow(const double *u, double x, double *out);
/* WilsonLineObservables (vt: V at the boundary behind the nucleus, [ntr][ng]) */
double orc_wilson_tadpole(int nc, const double *vt, long ntr);
int orc_wilson_dipole(int nc, const double *vt, int n1, int n2, double a1, double a2, double *out, double *ds_out);
/* LightConeNGPParticleCreator.initializeParticles (beam direction 0) */
long orc_cgc_particles(const orc_params *p, const double *gauss, int orientation, long cap,
                       double *pos0, double *pos1, double *vel, double *Q);

/* ---- super particles (temporal optimized cgc ngp) ---- */
long orc_super_create(const orc_params *p, const double *gauss, long *base_out, double *Q);
void orc_super_cin(const orc_params *p, int ngroups, const int *orient, const long *n, const long *base,
                   double *const *Q, int nthreads, long t, double *rho);
void orc_super_jin(const orc_params *p, int ngroups, const int *orient, const long *n, const long *base,
                   double *const *Q, int nthreads, long t, const double *Unext, double *J);

/* ---- Coulomb gauge and occupation numbers (SU(2)) ---- */
double orc_coulomb_divergence(const orc_params *p, const double *U, double *div);
void orc_coulomb_apply(const orc_params *p, const double *psi, double *U, double *Unext, double *E);
void orc_occupation_fields(const orc_params *p, const double *U, const double *Unext, const double *E,
                           double gainv, double *Ef, double *A);

/* ---- ImplicitTYMSolver.step (SU(2); -1 for SU(3)) ---- */
int orc_implicit_update_grid(const orc_params *p, const double *U, double *E, const double *J, double *Unext,
                             const uint8_t *active, int iterations, double damping);

#ifdef __cplusplus
}
#endif
#endif
