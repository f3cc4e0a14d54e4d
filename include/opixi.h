/*
 * opixi.h -- C ABI of libopixi_gpu.so, the GB300 (sm_103a) implementation of
 * OpenPixi's temporal-gauge Yang-Mills leapfrog, its CPIC (NGP) coupling and
 * the energy / Gauss-law reductions.
 *
 * The reference is Java and has no native boundary.  Each entry point below
 * names the Java method it stands in for (paths relative to
 * pixi/src/main/java/org/openpixi/pixi/).  A Java drop-in (JNI or Panama FFM)
 * binds these symbols one to one.
 *
 * Conventions
 *  - Every function returns an int status: OPX_OK (0) or a negative OPX_ERR_*.
 *    opx_last_error() gives the message of the last failure on a handle (or the
 *    last failure of opx_create when called with NULL).  No C++ exception
 *    crosses this boundary.
 *  - Host buffers are caller-owned and copied; the library owns device memory.
 *  - A handle is used by one host thread at a time; all work of a handle is
 *    queued on its own CUDA stream.
 *  - Host data are always doubles (the reference is FP64).  An OPX_F32 handle
 *    stores links and fields in FP32 on the device and converts on transfer.
 *  - Host layout OPX_LAYOUT_REF is the reference's per-cell layout:
 *      U, Unext : [V][3][ng]  ng = 4  (SU(2) e0..e3, SU2GroupElement.java:3-14)
 *                             ng = 18 (SU(3) 9 real then 9 imaginary parts,
 *                                      SU3GroupElement.java:3-11)
 *      E, J     : [V][3][na]  na = 3  (SU(2) v0..v2, SU2AlgebraElement.java)
 *                             na = 9  (SU(3) hermitian entries v[9],
 *                                      SU3AlgebraElement.java:3-11)
 *      rho      : [V][na]
 *    OPX_LAYOUT_GEN is the same but with E, J, rho given as generator
 *    components (SU3AlgebraElement.get(a), :117-129): 3 (SU(2)) or 8 (SU(3)).
 *    Site index = ((x0*N1)+x1)*N2+x2, dimension 0 slowest (Grid.java:757-770).
 */
#ifndef OPIXI_H
#define OPIXI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OPX_OK 0
#define OPX_ERR_INVALID (-1)     /* bad argument, size or handle */
#define OPX_ERR_CUDA (-2)        /* CUDA runtime / launch failure */
#define OPX_ERR_NOMEM (-3)       /* device or pinned allocation failed */
#define OPX_ERR_NUMERIC (-4)     /* device status word: NaN/Inf or bound exceeded */
#define OPX_ERR_UNSUPPORTED (-5) /* combination not provided (e.g. CPIC on FP32) */
#define OPX_ERR_TIMEOUT (-6)     /* a bounded device wait gave up */

#define OPX_F64 0
#define OPX_F32 1

#define OPX_FIELD_U 0
#define OPX_FIELD_UNEXT 1
#define OPX_FIELD_E 2
#define OPX_FIELD_J 3
#define OPX_FIELD_RHO 4

#define OPX_LAYOUT_REF 0
#define OPX_LAYOUT_GEN 1

/* Phase indices of opx_phase_times (the PerformanceTimer laps of
 * physics/Simulation.java:392-433, plus reductions and reunitarisation). */
#define OPX_PHASE_EOM 0   /* storeFields + updateGrid (E and Unext) */
#define OPX_PHASE_CPIC 1  /* CIN+PUP+PIN+CUP+JIN: the particle phases */
#define OPX_PHASE_DIA 2   /* reductions / diagnostics */
#define OPX_PHASE_LINKS 3 /* stepLinks */
#define OPX_NUM_PHASES 4

typedef struct opx_ctx opx_ctx;

/* Settings subset that the field solver reads (physics/Settings.java:43-104,
 * physics/grid/Grid.java:443-473). */
typedef struct {
    int ncolors;       /* 2 or 3 (Settings.numberOfColors) */
    int dims[3];       /* grid cells per direction (Settings.gridCells) */
    double a[3];       /* lattice spacing per direction (Settings.gridStep[s]) */
    double dt;         /* temporal spacing (Settings.timeStep) */
    double g;          /* gauge coupling (Settings.couplingConstant) */
    int precision;     /* OPX_F64 or OPX_F32 */
    int reunit_every;  /* OPX_F32: re-unitarise links every k steps (0 = never) */
    int device;        /* CUDA device ordinal */
    int flags;         /* reserved, 0 */
} opx_config;

/* BulkQuantitiesInTime columns (diagnostics/methods/BulkQuantitiesInTime.java:83-121),
 * computed as FieldMeasurements does (physics/measurements/FieldMeasurements.java:68-231),
 * accumulated in FP64 with compensated sums. */
typedef struct {
    double e2[3];      /* EFieldSquared.getSum(dir) */
    double b2[3];      /* BFieldSquared.getSum(dir): mean of U and Unext plaquettes */
    double px, py, pz; /* pressures */
    double gauss;      /* GaussLaw.getSum(): mean squared Gauss violation */
    double rho2;       /* TotalChargeSquared.getSum(): sqrt(sum rho^2)/V */
    double e2_total;   /* E^2 column */
    double b2_total;   /* B^2 column */
} opx_observables;

/* CGC particle list (physics/particles/CGCParticle.java, YangMillsParticle.java:13-25)
 * as host arrays: pos0, pos1, vel : [n][3]; Q0, Q1 : [n][na] (reference algebra
 * layout); dir : [n]; update_charge : [n]. */
typedef struct {
    long n;
    double *pos0, *pos1, *vel, *Q0, *Q1;
    int32_t *dir;
    uint8_t *update_charge;
} opx_particles;

/* ---- lifetime ---- */
/* new Grid(settings) + FieldSolver selection (Grid.java:443-473,
 * Settings.applySimulationTypeSetting :540-581).  Links start as identity,
 * fields at zero, every cell active and evaluatable (Cell.java:49-74). */
int opx_create(const opx_config *cfg, opx_ctx **out);
void opx_destroy(opx_ctx *ctx);
const char *opx_last_error(const opx_ctx *ctx);
int opx_version(void);

/* ---- host <-> device (the Grid getters/setters, Grid.java:126-261) ----
 * host holds count doubles in the reference's per-cell layout (OPX_LAYOUT_REF)
 * or generator components (OPX_LAYOUT_GEN).  A page-locked buffer
 * (opx_host_alloc, cudaMallocHost, cudaHostRegister) is read or written by the
 * conversion kernels directly; a pageable one goes through a device staging
 * copy (allocated on first use, kept by the handle).  Both return after the
 * transfer is complete. */
int opx_upload(opx_ctx *ctx, int field, const double *host, size_t count, int layout);
int opx_download(opx_ctx *ctx, int field, double *host, size_t count, int layout);
/* Cell.isActive / Cell.isEvaluatable masks; NULL resets to all-true
 * (Grid.setActiveRegion / setEvaluationRegion, Grid.java:978-1004). */
int opx_set_active(opx_ctx *ctx, const uint8_t *mask, size_t count);
int opx_set_evaluatable(opx_ctx *ctx, const uint8_t *mask, size_t count);

/* ---- leapfrog (physics/fields/FastTYMSolver.java) ---- */
/* FieldSolver.stepLinks -> UpdateLinks: Unext = exp(-i dt E) U (FastTYMSolver.java:34-38,65-84) */
int opx_step_links(opx_ctx *ctx);
/* FieldSolver.step -> CombinedUpdate (FastTYMSolver.java:24-63) */
int opx_update_grid(opx_ctx *ctx);
/* Field solver of opx_update_grid / opx_step (Settings.applySimulationTypeSetting,
 * physics/Settings.java:540-581): FastTYMSolver (the default), or
 * ImplicitTYMSolver(implicitSolverIterations, implicitSolverDamping)
 * (physics/fields/ImplicitTYMSolver.java:35-58; SU(2), SU(3)) for the implicit CGC types. */
#define OPX_SOLVER_FAST 0
#define OPX_SOLVER_IMPLICIT 1
int opx_set_field_solver(opx_ctx *ctx, int kind, int iterations, double damping);
/* Grid.storeFields -> Cell.reassignLinks (Grid.java:591-593, Cell.java:173-177) */
int opx_store_fields(opx_ctx *ctx);
/* Simulation.initialize (Simulation.java:318-352) */
int opx_initialize(opx_ctx *ctx);
/* nsteps x Simulation.step without diagnostics (Simulation.java:373-435) */
int opx_step(opx_ctx *ctx, int nsteps);
/* Re-unitarise U and Unext (FP32 form; no counterpart in the reference). */
int opx_reunitarize(opx_ctx *ctx);
int opx_synchronize(opx_ctx *ctx);
long opx_steps_done(const opx_ctx *ctx);

/* ---- reductions / diagnostics ---- */
int opx_reduce(opx_ctx *ctx, opx_observables *out);
/* nsteps x {Simulation.step; BulkQuantitiesInTime.calculate} (MainBatch's loop
 * with BulkQuantitiesInTime every step, Simulation.java:373-435,
 * BulkQuantitiesInTime.java:83-121): out[k] holds what opx_reduce returns after
 * the (k+1)-th step.  For SU(3) FP32 handles with the FastTYMSolver, no current,
 * no masks and no particles, each step's kernel also forms the per-site
 * BulkQuantities terms it can from what it loads (E^2 of the new E, B^2 of its
 * input links, the transported E of the Gauss law, whose sum the next step
 * forms) and one reduction follows the last step; the values agree with
 * opx_step + opx_reduce to FP32 rounding of the per-site terms (the plaquettes
 * are multiplied in another order, the sums run in another order).  Otherwise,
 * and for nsteps = 1, it is exactly opx_step(ctx, 1) + opx_reduce per step.
 * OPX_ERR_NUMERIC (non-finite values): the rows before the first non-finite one
 * are filled; the fused form has made all nsteps steps, the step + reduce form
 * stops after the step of that row. */
int opx_step_measured(opx_ctx *ctx, int nsteps, opx_observables *out);
/* EnergyDensity.ComponentComputation (diagnostics/methods/EnergyDensity.java:119-166): V doubles */
int opx_energy_density(opx_ctx *ctx, double *host_out, size_t count);
/* ProjectedEnergyDensity.EnergyDensityComputation (ProjectedEnergyDensity.java:114-179):
 * 4 rows of dims[dir] doubles: T_el, T_mag, L_el, L_mag */
int opx_projected_energy(opx_ctx *ctx, int dir, double *host_out, size_t count);
/* Grid.getGaussConstraint at every cell (Grid.java:944-968), generator components [V][ngen] */
/* ProjectedEnergyDensity.PoyntingComputation (ProjectedEnergyDensity.java:182-279):
 * out [2][dims[dir]]: the longitudinal Poynting vector averaged in space and
 * time, and only time-averaged.  SU(2) handles (the reference's SU(3) algebra
 * has no scalar product and throws); every cell counts, as in the reference. */
int opx_projected_poynting(opx_ctx *ctx, int dir, double *host_out, size_t count);
int opx_gauss_field(opx_ctx *ctx, double *host_out, size_t count);

/* ---- CPIC (physics/grid/CGCParticleInterpolationNGP.java,
 *             physics/movement/solver/CGCParticleSolver.java) ---- */
int opx_particles_upload(opx_ctx *ctx, const opx_particles *p);
int opx_particles_download(opx_ctx *ctx, opx_particles *p);
/* Number of particles attached to the handle (s.particles.size()). */
long opx_particles_count(const opx_ctx *ctx);
/* Particle phases of one Simulation.step (reassign != 0) or of
 * Simulation.initialize (reassign == 0): charge density, positions, transport,
 * charges, currents (Simulation.java:398-421, 329-347).  With super particles:
 * their charge density and current at the handle's step count. */
int opx_cpic_phases(opx_ctx *ctx, int reassign);

/* ---- CGC initial conditions (physics/initial/CGC/CGCInitialCondition.java:55-93) ----
 * One MV-model nucleus (MVModel.java constructor arguments, YAML keys of
 * ui/util/yaml/initial/YamlMVModel.java). */
typedef struct {
    int direction;       /* beam axis (0) */
    int orientation;     /* +1 or -1 */
    double location;     /* longitudinalLocation */
    double width;        /* longitudinalWidth */
    double mu;           /* MV parameter mu */
    int use_seed;        /* randomSeed given */
    int seed;            /* java.util.Random seed */
    double uvt;          /* ultravioletCutoffTransverse */
    double coherence;    /* longitudinalCoherenceLength */
    double ir;           /* infraredCoefficient */
} opx_mv_nucleus;
/* Applies the nuclei in order: MV charges (java.util.Random stream), 3D
 * momentum-space regulation and 2D Poisson solves (cuFFT), Wilson lines,
 * links U and Unext (improved, M = 20), E from the temporal plaquette, and the
 * NGP particles of LightConeNGPParticleCreator (round(aL/dt) per cell, 100+100
 * refinement sweeps), appended to the handle's particle list.  The Gauss
 * violation that seeds the particles is taken with zero grid charge, as before
 * Simulation.initialize.  use_seed == 0 draws an unseeded stream.  OPX_F64
 * handles, beam along direction 0.  Call opx_initialize afterwards. */
int opx_cgc_mv(opx_ctx *ctx, const opx_mv_nucleus *nuclei, int n);

/* WilsonLineObservables (physics/initial/CGC/WilsonLineObservables.java:37-131)
 * of nucleus k of the last opx_cgc_mv / opx_cgc_mv_super call, from the
 * Poisson solver's Wilson lines V at the longitudinal boundary behind the
 * nucleus (LightConePoissonSolverImproved.getV, :125-136, :231):
 * computeTadpole's mean of Re tr V over the transverse cells, and
 * computeDipole's mean of Re tr(V(x) V(y)^dagger) over all pairs of transverse
 * cells binned by their periodic distance, (int) sqrt(n1 n2) / 2 bins of width
 * min(n1 a1, n2 a2) / 2 / nbins (empty bins NaN, as in the reference).
 * tadpole, dipole (nbins values) and bin_width may each be NULL. */
int opx_cgc_wilson_lines(opx_ctx *ctx, int nucleus, double *tadpole, double *dipole, size_t nbins,
                         double *bin_width);

/* ---- occupation numbers (diagnostics/methods/OccupationNumbersInTime.java:172-297) ----
 * On copies of the handle's fields: the Coulomb gauge iteration of
 * CoulombGauge.applyGaugeTransformation (physics/gauge/CoulombGauge.java:56-194;
 * at most max_iter iterations, until the summed squared divergence of
 * A = log U falls below accuracy_goal; the reference uses 100 and 1e-18),
 * then the occupation numbers n [V][N^2 - 1] (momentum index in cell order, colour
 * inner) and the energy density from them.  n_out may be
 * NULL.  SU(2) and SU(3) (the SU(3) gauge field from the matrix logarithm of
 * SU3GroupElement.getAlgebraElement), one lattice spacing.
 * opx_occupation_numbers_ex adds the mirrored grid and the cone windows. */
int opx_occupation_numbers(opx_ctx *ctx, int max_iter, double accuracy_goal, double *n_out, size_t count,
                           double *energy_density, int *iterations, double *last_divergence);

/* The diagnostic's options (OccupationNumbersInTime.java:92-115, applied in
 * calculate :164-201): the Coulomb gauge fixed on the grid mirrored along
 * mirrored_direction (MirroredGrid :655-686; -1 for none) and cut back
 * (UnmirroredGrid :688-703), then the windows in the order Gaussian
 * (:555-599), Tukey (:601-653), cone (:506-553), each when its flag is set.
 * The cone of axis d (cone_velocity[d] != 0) at the grid's time t = steps x dt
 * spans -/+ |t - collision_time| cone_velocity[d] + collision_position[d]. */
#define OPX_WINDOW_GAUSSIAN 1
#define OPX_WINDOW_TUKEY 2
#define OPX_WINDOW_CONE 4
typedef struct {
    int mirrored_direction;
    int windows;
    double collision_time;
    double collision_position[3];
    double cone_velocity[3];
    double tukey_width;
} opx_occupation_options;
int opx_occupation_numbers_ex(opx_ctx *ctx, const opx_occupation_options *options, int max_iter,
                              double accuracy_goal, double *n_out, size_t count, double *energy_density,
                              int *iterations, double *last_divergence);

/* ---- super particles: simulationType "temporal optimized cgc ngp"
 *      (Settings.java:566-571: CGCSuperParticleSolver + CGCSuperParticleInterpolationNGP;
 *      physics/particles/CGCSuperParticle.java) ----
 * The nuclei's particles are created by LightConeNGPSuperParticleCreator
 * (physics/initial/CGC/LightConeNGPSuperParticleCreator.java:102-241): per nucleus
 * a group of round(aL/dt) super particles k, each a block of charges over the
 * particle block [base, base + n) of global cell indices, moving along
 * direction 0.  opx_initialize / opx_step then run the charge density and
 * current of CGCSuperParticleInterpolationNGP (:19-93) instead of the NGP
 * particle phases.  OPX_F64 handles, beam along direction 0; a handle holds
 * either NGP particles or super particles. */
int opx_cgc_mv_super(opx_ctx *ctx, const opx_mv_nucleus *nuclei, int n);
/* number of super-particle groups on the handle */
int opx_super_groups(const opx_ctx *ctx);
/* group g: orientation, n, base and (Q != NULL) the charges Q[k][i][na_ref]
 * (reference layout; count = round(aL/dt) * n * na_ref) */
int opx_super_download(opx_ctx *ctx, int group, int *orientation, long *n, long *base, double *Q, size_t count);
/* appends a group with charges Q[k][i][na_ref] (the layout of opx_super_download) */
int opx_super_upload(opx_ctx *ctx, int orientation, long n, long base, const double *Q);

/* ---- seeded synthetic initial conditions (no counterpart in the reference) ---- */
/* U_i(x) = exp(i A_i^a(x) t_a), A ~ N(0, sigma_a^2); E_i^a(x) ~ N(0, sigma_e^2);
 * same counter-based generator as the oracle. */
int opx_init_random(opx_ctx *ctx, uint64_t seed, double sigma_a, double sigma_e);
/* Project E onto Gauss's law by conjugate gradients (FP64 on the device):
 * div(divT mu) = rho - div E, E <- E + divT mu. */
int opx_gauss_project(opx_ctx *ctx, double tol_g2, int maxit, int *iters, double *final_g2);

/* ---- timing (Simulation PerformanceTimer laps as CUDA events on the handle's stream) ---- */
int opx_set_profiling(opx_ctx *ctx, int on);
/* per phase: accumulated milliseconds and launch counts since profiling was enabled */
int opx_phase_times(opx_ctx *ctx, double *ms, long *counts, int nphases);
/* Time nsteps x opx_step with CUDA events recorded on the handle's stream. */
int opx_time_steps(opx_ctx *ctx, int nsteps, double *ms);
/* Number of kernels this handle has launched since creation. */
long opx_kernel_launches(const opx_ctx *ctx);

/* ---- differentiation form (SU(2); no counterpart in the reference) ----
 * Objective J = mean over the box lo..hi (inclusive cell coordinates; NULL =
 * whole lattice) of the per-cell energy density of
 * EnergyDensity.ComponentComputation (diagnostics/methods/EnergyDensity.java:119-166)
 * after nsteps x Simulation.step from the handle's current U and E (as
 * before opx_initialize).  The handle's fields are not modified.
 * Host direction / gradient arrays: [V][3][3] generator components of E. */
/* J at E + h*dE (dE may be NULL), from an FP64 forward run: finite differences */
int opx_energy_objective(opx_ctx *ctx, int nsteps, const int *lo, const int *hi, const double *dE, double h,
                         double *J);
/* FP64 tangent-linear run: J and dJ along dE (the forward kernels on dual numbers) */
int opx_energy_tangent(opx_ctx *ctx, int nsteps, const int *lo, const int *hi, const double *dE, double *J,
                       double *dJ);
/* Adjoint: dJ/dE_0 for every link.  The forward runs in the handle's precision
 * with FP64 checkpoints every ckpt steps (about sqrt(nsteps)); the reverse
 * sweep recomputes each segment in FP64 and applies the reverse step. */
int opx_energy_gradient(opx_ctx *ctx, int nsteps, int ckpt, const int *lo, const int *hi, double *J,
                        double *grad, size_t count);

/* The general form: an objective selector and the charge density as a second
 * input.
 *   OPX_OBJ_ENERGY     the mean EnergyDensity over the box (as above);
 *   OPX_OBJ_ANISOTROPY the pressure anisotropy P_L / P_T over the box from the
 *     components of ProjectedEnergyDensity (diagnostics/methods/
 *     ProjectedEnergyDensity.java:18-41, 114-179) with `direction` the
 *     longitudinal axis: per cell and direction j, eps_j = [E_j^2/2 +
 *     (|B_j(U)|^2 + |B_j(Unext)|^2)/4] / (g a_j)^2, eps_L = eps_direction,
 *     eps_T = the other two, P_L = eps_T - eps_L, P_T = eps_L, and
 *     J = sum_box P_L / sum_box P_T.
 * Inputs: OPX_WRT_E, the initial E ([V][3][3] generator components); or
 * OPX_WRT_RHO, the colour-charge density ([V][3]) through Gauss's law
 * (Grid.getGaussConstraint, physics/grid/Grid.java:944-968): the initial E is
 * the projection of the handle's E onto div E = rho (opx_gauss_project), so a
 * change d of rho moves E_0 by divT K^+ d (K = div divT on the handle's links)
 * and dJ/drho = K^+ div dJ/dE_0.  The handle's E must satisfy Gauss's law for
 * its rho (e.g. after opx_gauss_project).  SU(2) only; the handle's fields are
 * not modified. */
#define OPX_OBJ_ENERGY 0
#define OPX_OBJ_ANISOTROPY 1
#define OPX_WRT_E 0
#define OPX_WRT_RHO 1
typedef struct {
    int kind;       /* OPX_OBJ_ENERGY or OPX_OBJ_ANISOTROPY */
    int direction;  /* longitudinal axis of OPX_OBJ_ANISOTROPY (0, 1 or 2) */
    int lo[3], hi[3];  /* the box of cells, inclusive */
} opx_objective;
/* J with E_0 moved by h (dE + divT K^+ drho) (dE, drho may be NULL): finite differences */
int opx_objective_value(opx_ctx *ctx, const opx_objective *obj, int nsteps, const double *dE, const double *drho,
                        double h, double *J);
/* FP64 tangent-linear run along dE + divT K^+ drho (at least one non-NULL) */
int opx_objective_tangent(opx_ctx *ctx, const opx_objective *obj, int nsteps, const double *dE, const double *drho,
                          double *J, double *dJ);
/* Adjoint gradient with respect to OPX_WRT_E (count = V*3*3) or OPX_WRT_RHO (count = V*3) */
int opx_objective_gradient(opx_ctx *ctx, const opx_objective *obj, int nsteps, int ckpt, int wrt, double *J,
                           double *grad, size_t count);

/* ---- batching form: many independent lattices ("events") in one launch ----
 * The reference runs one Simulation per event (a loop over independent
 * Simulation objects); here the events advance together under one of two
 * schedules, both captured in a CUDA graph: one persistent launch of
 * thread-block clusters, each cluster owning a load-balanced set of events for
 * every step (cluster size 1-8), or the flat schedule (cluster size 0), one
 * launch per step over the sites of all events.  Events are pure Yang-Mills
 * (no particles).
 * dims: [nevents][3]; a: [nevents][3] lattice spacings or NULL (all 1). */
typedef struct opx_batch opx_batch;
int opx_batch_create(int ncolors, int nevents, const int *dims, const double *a, double dt, double g,
                     int precision, int reunit_every, int device, opx_batch **out);
void opx_batch_destroy(opx_batch *b);
const char *opx_batch_last_error(const opx_batch *b);
/* Seeded Gaussian links / E per event (seeds[nevents]), E projected onto
 * Gauss's law to mean G^2 <= tol_g2 (tol_g2 <= 0: no projection). */
int opx_batch_init_random(opx_batch *b, const uint64_t *seeds, double sigma_a, double sigma_e, double tol_g2);
int opx_batch_upload(opx_batch *b, int event, int field, const double *host, size_t count, int layout);
int opx_batch_download(opx_batch *b, int event, int field, double *host, size_t count, int layout);
/* Simulation.initialize (stepLinks) for every event */
int opx_batch_initialize(opx_batch *b);
/* Pick the schedule (cluster size 0 = flat, or 1, 2, 4, 8) and block size by
 * timing `steps` steps of each candidate on the batch itself (the fields are
 * restored afterwards). */
int opx_batch_autotune(opx_batch *b, int steps, int *cluster, int *block);
/* Set the schedule directly: cluster 0 (flat) or 1, 2, 4, 8 with block 128 or
 * 256; OPX_ERR_UNSUPPORTED if that launch does not fit (SU(3) FP32: block 128). */
int opx_batch_set_schedule(opx_batch *b, int cluster, int block);
/* nsteps x Simulation.step (no diagnostics) of every event: one launch
 * (clusters) or nsteps launches (flat); use_graph != 0 replays a captured CUDA
 * graph of them. */
int opx_batch_run(opx_batch *b, int nsteps, int use_graph);
int opx_batch_time_run(opx_batch *b, int nsteps, int use_graph, double *ms);
/* BulkQuantities of every event (out[nevents]), FP64 compensated sums */
int opx_batch_reduce(opx_batch *b, opx_observables *out);
int opx_batch_config(const opx_batch *b, int *cluster, int *block, int *nclusters);
long opx_batch_kernel_launches(const opx_batch *b);

/* Allocation-free BulkQuantities reductions over caller-owned device fields
 * (no counterpart in the reference).  For callers that cannot allocate device
 * memory themselves or through this library: hosts whose device memory is
 * owned by another allocator (a framework's caching allocator, a JVM or
 * service with a fixed GPU budget) or code that must not stall on the device
 * synchronisation of cudaMalloc/cudaFree.  Computes what opx_reduce computes
 * and writes one opx_observables record to out_device (device memory), queued
 * on `stream` (a cudaStream_t; NULL = the default stream).  Fields are device
 * pointers in the handle's layout: SU(3) links U, Unext in warp-sized site
 * blocks [3][ceil(V/32)][18][32], SU(2) links as [3][32 ceil(V/32)][4]
 * (quaternion components contiguous), algebra fields as planes E [3][ngen][V],
 * rho [ngen][V] (NULL = zero charge), eval [V] (NULL = all cells), elements
 * double (OPX_F64) or float (OPX_F32).  U and Unext must be 16-byte aligned
 * (OPX_ERR_INVALID otherwise; cudaMalloc'd buffers are).
 * Calls no cudaMalloc/cudaFree: its scratch is a fixed 77,824-byte __device__
 * array of the library, held by every GPU that loads the library until exit.
 * Limit: V <= 2^29 sites (larger lattices return OPX_ERR_INVALID).  The first
 * call on a device looks up the scratch address and should come before any
 * stream capture; after cudaDeviceReset of a device the looked-up address is
 * stale, so do not call it on that device again.  Calls share the scratch, so
 * calls that overlap on the GPU race.  Non-finite field values are not
 * detected (opx_reduce returns OPX_ERR_NUMERIC for them): they reach the record
 * as NaN or Inf, and the caller checks it.  OPX_ERR_CUDA reports a launch
 * failure of this call only; an error left pending by earlier work is neither
 * reported nor cleared. */
int opx_reduce_noalloc(int ncolors, int precision, const int *dims, const double *a, double g,
                       const void *U, const void *Unext, const void *E, const void *rho,
                       const uint8_t *eval, opx_observables *out_device, void *stream);

/* Page-locked host memory for transfers (cudaMallocHost / cudaFreeHost). */
void *opx_host_alloc(size_t bytes);
void opx_host_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
