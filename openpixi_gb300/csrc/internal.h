// internal.h -- handle state and kernel launchers shared by the translation units
// of libopixi_gpu.so.  Not part of the public ABI (include/opixi.h is).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/opixi.h"
#include "lattice.cuh"

namespace opx {

// Device status word bits (read back by the host after each API call that
// checks numerics).
enum : unsigned {
    STATUS_NAN = 1u,        // a NaN/Inf was produced
    STATUS_CG_DIVERGED = 2u,
};

struct Particles {
    long n = 0, cap = 0;
    double *pos0 = nullptr, *pos1 = nullptr, *vel = nullptr;  // [3][n] each
    double *q0 = nullptr, *q1 = nullptr;                        // [na_ref][n]
    int8_t *dir = nullptr;
    // deposition scratch
    int *key_rho = nullptr, *key_j = nullptr;                   // [n]
    double *val_rho = nullptr, *val_j = nullptr;                // [na_ref][n]
    int *count = nullptr, *offset = nullptr;                    // [4V + 1]: bucket sizes (zero between steps), their scan
    int *slots = nullptr;                                       // [2n]
    int *scan_tmp = nullptr;
    long scan_tmp_len = 0;
};

// Super particles (CGCSuperParticle, temporal optimized cgc ngp): one group per
// nucleus, ppc layers k of charges over the particle block [base, base + n)
// of global cell indices; Q is [ppc][na_ref][n] on the device.
struct SuperGroup {
    int orientation = 1;
    long n = 0, base = 0;
    double *Q = nullptr;
};

struct Ctx {
    opx_config cfg;
    Lat L;
    int nc = 2, ng = 4, na = 3, na_ref = 3;  // reals per link / generator comps / reference algebra reals
    int prec = OPX_F64;
    size_t rsize = 8;  // bytes per real on the device
    cudaStream_t stream = nullptr;
    void *U = nullptr, *Unext = nullptr, *E = nullptr, *J = nullptr, *rho = nullptr;
    uint8_t *active = nullptr, *eval = nullptr;  // null = all true
    bool j_nonzero = false;
    // rho has been written (an upload or the particle phases); until then it is
    // zero and the kernels that subtract it from the Gauss law skip its loads
    bool rho_nonzero = false;
    // SU(3) FP32 leapfrog and reduction with two sites per thread in paired FP32
    // instructions (environment OPX_ONE_SITE_FP32=1 selects the
    // one-site-per-thread forms)
    bool pair_kernel = true;
    // 32-bit site and element offsets in the leapfrog kernels while every link
    // and E offset fits (SU(3): 54 V < 2^31); OPX_LONG_OFFSETS=1 selects the
    // 64-bit forms at any size, so that tests can compare them on small lattices
    bool int_offsets = true;
    // opt-in (OPX_STREAM_FP32=1): the SU(3) FP32 leapfrog in plaquette form
    // streamed along dimension 0 (su3_stream.cuh), where the lattice tiles
    // (N1 % 8 == 0, N2 % 32 == 0) and there is no current or activity mask.
    // st_grid: its resident-wave grid (0 = not yet computed for this handle's
    // device)
    bool stream_kernel = false;
    int st_grid = 0;
    double *staging = nullptr;
    size_t staging_len = 0;  // doubles
    double *red_part = nullptr;
    int red_blocks = 0;
    double *red_out = nullptr;     // device
    unsigned *red_count = nullptr; // device: blocks of the running reduction that have finished
    double *red_host = nullptr;    // pinned
    unsigned *status = nullptr;    // device status word
    unsigned *status_host = nullptr;
    long steps = 0;
    long launches = 0;
    // Reuse of B^2 across reductions: a reduction after one opx_step(ctx, 1)
    // that followed a reduction takes B^2 of U from that reduction's B^2 of Unext
    // (the same links after the swap).  api_calls counts the entry-point calls
    // that may change the fields or the masks (all but the read-only ones:
    // downloads, reductions, diagnostics, profiling), so that any other such call
    // in between (an upload, an initial condition, a gauge transformation ...)
    // disables the reuse.
    long api_calls = 0;
    long step1_call = -1;  // api_calls value of the last opx_step(ctx, 1)
    struct {
        long calls = -1, steps = -1;
        const void *unext = nullptr;
        double bn[3] = {0, 0, 0};  // B^2 of Unext, per direction, summed over the sites
    } bcache;
    // the same for ProjectedEnergyDensity, per direction: the Unext magnetic
    // rows (T then L, dims[dir] each) of the last call
    struct {
        long calls = -1, steps = -1;
        const void *unext = nullptr;
        std::vector<double> mag_next;
    } pcache[3];
    Particles P;
    // field solver: FastTYMSolver (imp_solver false) or ImplicitTYMSolver
    bool imp_solver = false;
    int imp_iterations = 0;
    double imp_damping = 0.0;
    void *imp_Ua = nullptr, *imp_Ub = nullptr, *imp_E = nullptr;  // the implicit grid's links and E
    std::vector<SuperGroup> sg;  // super-particle groups in list order
    // Wilson lines at the longitudinal boundary behind each nucleus of the last
    // opx_cgc_mv / opx_cgc_mv_super call ([n1 n2][ng], reference layout)
    std::vector<double *> cgc_vt;
    int sg_ppc = 0;
    // opx_step_measured: the second E buffer (the measured step writes the new
    // E there and the pointers swap), the transported Gauss-law terms of the
    // last and the next step, the block partials and the per-step rows
    void *E_alt = nullptr, *W_in = nullptr, *W_out = nullptr;
    // per-site B_d^2 of Unext [3][V] (FP64) written by the generic BulkQuantities
    // pass (null: not written), and the state it belongs to: ProjectedEnergyDensity
    // after opx_reduce on the same state reads them instead of forming the
    // plaquettes again
    double *bn_site = nullptr;
    struct {
        long calls = -1, steps = -1;
        const void *unext = nullptr;
    } bnsite;
    double *meas_part = nullptr, *meas_rows = nullptr, *meas_host = nullptr;  // rows: device and pinned
    int meas_rows_cap = 0, meas_chunk = 0;  // steps whose partials meas_part holds
    bool profiling = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double phase_ms[OPX_NUM_PHASES] = {0, 0, 0, 0};
    long phase_n[OPX_NUM_PHASES] = {0, 0, 0, 0};
    std::string err;
};

// ---- launchers (field_kernels.cu) ----
void launch_update_grid(Ctx &c, bool reunit);
int launch_implicit_update(Ctx &c);  // ImplicitTYMSolver.step in place of launch_update_grid
void launch_update_links(Ctx &c);
void launch_reunit(Ctx &c, void *links);
// the measured step (SU(3) FP32 paired form, FastTYMSolver, no current, no
// masks, no particles): row[0..6] = E^2 of the new E [3] (x (g a_i)^-2),
// B^2 of the step's input links [3] (x (g a_i)^-2 / 2), G^2 of the state
// before the step (from the previous step's transported terms)
constexpr int MEAS_ROW = 7;
bool measured_step_fusable(const Ctx &c);
int measured_blocks(const Ctx &c);
int measured_parts(const Ctx &c);
void launch_update_measure(Ctx &c, bool reunit, void *Eout, const void *Win, void *Wout, double *part);
void launch_measure_combine(Ctx &c, const double *part, int nsteps, double *rows);  // rows[nsteps][8]
// ---- reductions (reduce_kernels.cu) ----
// result in c.red_out[0..10]: E^2[3], B^2 of U [3] (zero with skip_u), G^2, rho^2, B^2 of Unext [3]
constexpr int BULK_COLUMNS = 11;
void launch_bulk(Ctx &c, int skip_u);
int reduction_blocks(long V);
void launch_energy_density(Ctx &c, double *dev_out);
// six rows of dims[dir]: T_el, T_mag(U), L_el, L_mag(U), T_mag(Unext), L_mag(Unext)
// (the U rows zero with skip_u); with bn_site the per-site B^2 of Unext come
// from that buffer instead of the plaquettes
void launch_projected_energy(Ctx &c, int dir, int skip_u, const double *bn_site, double *dev_out);
int launch_projected_poynting(Ctx &c, int dir, double *dev_out);  // SU(2) only
void launch_gauss_field(Ctx &c, double *dev_out);
// ---- conversions (convert_kernels.cu) ----
void launch_links_from_ref(Ctx &c, const double *src, void *dst);
void launch_links_to_ref(Ctx &c, const void *src, double *dst);
void launch_alg_from_host(Ctx &c, const double *src, void *dst, int ndir, int layout);
void launch_alg_to_host(Ctx &c, const void *src, double *dst, int ndir, int layout);
// ---- initial conditions (ic_kernels.cu) ----
int ic_init_random(Ctx &c, uint64_t seed, double sigma_a, double sigma_e);
int ic_gauss_project(Ctx &c, double tol, int maxit, int *iters, double *final_g2);
// FP64 covariant divergence of a link-algebra field and its transpose (ic_kernels.cu):
//   (div E)(x) = sum_i c_i [E_i(x) - Ad(U_i(x-i)^dag) E_i(x-i)],  (divT l)_i(x) = c_i [l(x) - Ad(U_i(x)) l(x+i)]
void ic_div(Ctx &c, const double *U64, const double *El, double *o);
void ic_divT(Ctx &c, const double *U64, const double *l, double *o, int acc);
// x = K^+ b, K = div divT, by conjugate gradients (|r| <= tol_rel |b|)
int ic_covariant_solve(Ctx &c, const double *U64, const double *b, double *x, double tol_rel, int maxit, int *iters);
// ---- CPIC (cpic_kernels.cu) ----
int cpic_alloc(Ctx &c, long n);
void cpic_free(Ctx &c);
void launch_cpic_phases(Ctx &c, int reassign);
void launch_super_phases(Ctx &c, long t);  // CGCSuperParticleInterpolationNGP CIN + JIN at step t
void super_free(Ctx &c);
void cgc_vt_free(Ctx &c);  // cgc_kernels.cu

int grid_for(long n, int block);

// the handle behind an opx_ctx (api.cu)
Ctx &ctx_of(opx_ctx *h);

}  // namespace opx
