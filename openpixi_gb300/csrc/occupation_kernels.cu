// occupation_kernels.cu -- Coulomb gauge fixing and gluon occupation numbers (SU(2)).
//
// Restates, on copies of the handle's fields (the handle is not modified):
//   CoulombGauge.applyGaugeTransformation / iterateCoulombGauge
//     (physics/gauge/CoulombGauge.java:56-194): divergence of the gauge field
//     A = log U per colour, Poisson solve with the lattice Laplacian in
//     momentum space (cuFFT, three colours in one batched transform),
//     g = exp(-i psi) and GaugeTransformation's action on U, Unext and E
//     (physics/gauge/GaugeTransformation.java:57-90); repeated until the
//     summed squared divergence is below the accuracy goal;
//   OccupationNumbersInTime.calculate (diagnostics/methods/OccupationNumbersInTime.java:172-297):
//     Fourier transforms of E and of A averaged over U and Unext (18 fields in
//     one batched transform), occupation numbers per momentum and colour with
//     the abelian lattice dispersion, and the energy density from them.
//   the diagnostic's options (:92-115, :164-201): the mirrored grid (MirroredGrid,
//     :655-686) on which the Coulomb gauge is fixed before the grid is cut back
//     (UnmirroredGrid, :688-703), and the Gaussian, Tukey and cone windows
//     (:555-653, :506-553) applied after the gauge fixing, in that order.
// Work is in FP64 whatever the handle's precision.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fftlib.h"
#include "internal.h"
#include "ksum.cuh"

namespace opx {

// SU2GroupElement.getAlgebraElement (math/SU2GroupElement.java:234-252)
__device__ __forceinline__ void su2_log(const double *u, double *v) {
    double norm = u[1] * u[1] + u[2] * u[2] + u[3] * u[3];
    norm = sqrt(norm);
    if (norm < 1.E-15) {
        v[0] = 2 * u[1]; v[1] = 2 * u[2]; v[2] = 2 * u[3];
        return;
    }
    const double f = 2.0 * asin(norm) / norm;
    v[0] = f * u[1]; v[1] = f * u[2]; v[2] = f * u[3];
}

// SU2AlgebraElement.getLink in the reference's own form (math/SU2AlgebraElement.java:140-152)
__device__ __forceinline__ void su2_link_ref(const double *v, double *u) {
    const double sum = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    const double mod = sqrt(sum) / 2;
    const double sinfakt = mod < 1.E-20 ? 0.0 : 0.5 / mod * sin(mod);
    u[0] = cos(mod); u[1] = v[0] * sinfakt; u[2] = v[1] * sinfakt; u[3] = v[2] * sinfakt;
}

__device__ __forceinline__ void q_mul(const double *x, const double *a, double *b) {
    // SU2GroupElement.mult (math/SU2GroupElement.java:206-217)
    const double b0 = x[0] * a[0] - x[1] * a[1] - x[2] * a[2] - x[3] * a[3];
    const double b1 = x[0] * a[1] + x[1] * a[0] - x[2] * a[3] + x[3] * a[2];
    const double b2 = x[0] * a[2] + x[2] * a[0] - x[3] * a[1] + x[1] * a[3];
    const double b3 = x[0] * a[3] + x[3] * a[0] - x[1] * a[2] + x[2] * a[1];
    b[0] = b0; b[1] = b1; b[2] = b2; b[3] = b3;
}

template <typename R>
__global__ void k_occ_copy(const R *__restrict__ U, const R *__restrict__ Un, const R *__restrict__ E, Lat L,
                           double *__restrict__ Uc, double *__restrict__ Unc, double *__restrict__ Ec) {
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    const LinkPlanes<SU2<R>, R> Up{const_cast<R *>(U), L.V}, Unp{const_cast<R *>(Un), L.V};
    const LinkPlanes<SU2<double>, double> Uo{Uc, L.V}, Uno{Unc, L.V};
    for (int d = 0; d < 3; d++) {
        const Q2<R> a = Up.load(d, s), b = Unp.load(d, s);
        Uo.store(d, s, Q2<double>{{(double)a.e[0], (double)a.e[1], (double)a.e[2], (double)a.e[3]}});
        Uno.store(d, s, Q2<double>{{(double)b.e[0], (double)b.e[1], (double)b.e[2], (double)b.e[3]}});
        for (int a2 = 0; a2 < 3; a2++) Ec[((long)d * 3 + a2) * L.V + s] = (double)E[((long)d * 3 + a2) * L.V + s];
    }
}

// MirroredGrid (:655-686): the grid doubled along md, every cell copied to its
// own position and to the mirrored one (2 N - 1 - x), and the mirrored copy's
// link along md taken from the cell one step back (x - 1, or x itself at x = 0)
template <typename R>
__global__ void k_occ_copy_mirror(const R *__restrict__ U, const R *__restrict__ Un, const R *__restrict__ E, Lat L,
                                  Lat Lm, int md, double *__restrict__ Uc, double *__restrict__ Unc,
                                  double *__restrict__ Ec) {
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    int x[3];
    site_coords(L, s, x);
    int y[3] = {x[0], x[1], x[2]};
    y[md] = 2 * L.n[md] - x[md] - 1;
    const long s1 = ((long)x[0] * Lm.n[1] + x[1]) * Lm.n[2] + x[2];
    const long s2 = ((long)y[0] * Lm.n[1] + y[1]) * Lm.n[2] + y[2];
    int z[3] = {x[0], x[1], x[2]};
    if (z[md] > 0) z[md]--;
    const long sh = ((long)z[0] * L.n[1] + z[1]) * L.n[2] + z[2];
    const LinkPlanes<SU2<R>, R> Up{const_cast<R *>(U), L.V}, Unp{const_cast<R *>(Un), L.V};
    const LinkPlanes<SU2<double>, double> Uo{Uc, Lm.V}, Uno{Unc, Lm.V};
    auto wide = [](const Q2<R> &a) { return Q2<double>{{(double)a.e[0], (double)a.e[1], (double)a.e[2], (double)a.e[3]}}; };
    for (int d = 0; d < 3; d++) {
        const Q2<double> a = wide(Up.load(d, s)), b = wide(Unp.load(d, s));
        Uo.store(d, s1, a);
        Uo.store(d, s2, d == md ? wide(Up.load(d, sh)) : a);
        Uno.store(d, s1, b);
        Uno.store(d, s2, b);
        for (int c = 0; c < 3; c++) {
            const double e = (double)E[((long)d * 3 + c) * L.V + s];
            Ec[((long)d * 3 + c) * Lm.V + s1] = e;
            Ec[((long)d * 3 + c) * Lm.V + s2] = e;
        }
    }
}

// UnmirroredGrid (:688-703): the cells of the first half, at their own positions
__global__ void k_occ_unmirror(const double *__restrict__ Ucm, const double *__restrict__ Uncm,
                               const double *__restrict__ Ecm, Lat Lm, Lat L, double *__restrict__ Uc,
                               double *__restrict__ Unc, double *__restrict__ Ec) {
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    int x[3];
    site_coords(L, s, x);
    const long sm = ((long)x[0] * Lm.n[1] + x[1]) * Lm.n[2] + x[2];
    const LinkPlanes<SU2<double>, double> Ui{const_cast<double *>(Ucm), Lm.V}, Uni{const_cast<double *>(Uncm), Lm.V};
    const LinkPlanes<SU2<double>, double> Uo{Uc, L.V}, Uno{Unc, L.V};
    for (int d = 0; d < 3; d++) {
        Uo.store(d, s, Ui.load(d, sm));
        Uno.store(d, s, Uni.load(d, sm));
        for (int c = 0; c < 3; c++) Ec[((long)d * 3 + c) * L.V + s] = Ecm[((long)d * 3 + c) * Lm.V + sm];
    }
}

// SU2GroupElement.pow(x) = getLink(x getAlgebraElement()) (math/SU2GroupElement.java:269-271)
__device__ __forceinline__ Q2<double> su2_pow_ref(const Q2<double> &u, double f) {
    double v[3];
    su2_log(u.e, v);
    for (int c = 0; c < 3; c++) v[c] *= f;
    Q2<double> r;
    su2_link_ref(v, r.e);
    return r;
}

struct OccWindow {
    int flags;            // OPX_WINDOW_GAUSSIAN | OPX_WINDOW_TUKEY | OPX_WINDOW_CONE
    double time, ctime;   // the grid's time (steps x dt) and the collision time
    double tukey;         // Tukey width
    double pos[3], vel[3];  // collision position, cone velocity (0: no restriction on the axis)
};

// GaussianConeRestrictedGrid (:555-599), TukeyConeRestrictedGrid (:601-653) and
// ConeRestrictedGrid (:506-553), in the order calculate applies them (:194-202).
// On every axis with a cone velocity the cone spans [minPos, maxPos] with
// minPos/maxPos = -/+ |t - t_c| v + x_c.  The windows scale E and take U and
// Unext to the power of their suppression factor; the cone replaces the cells
// outside it by fresh cells (identity links, E = 0).
__global__ void k_occ_window(double *__restrict__ U, double *__restrict__ Un, double *__restrict__ E, Lat L,
                             OccWindow w) {
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    int x[3];
    site_coords(L, s, x);
    const double two_sqrt_log_two = 2 * sqrt(log(2.0));
    const double pi = 3.141592653589793;
    const LinkPlanes<SU2<double>, double> Up{U, L.V}, Unp{Un, L.V};
    for (int pass = 0; pass < 3; pass++) {
        const int flag = pass == 0 ? OPX_WINDOW_GAUSSIAN : (pass == 1 ? OPX_WINDOW_TUKEY : OPX_WINDOW_CONE);
        if (!(w.flags & flag)) continue;
        double factor = 1.0;
        bool inside = true;
        for (int d = 0; d < 3; d++) {
            if (w.vel[d] == 0) continue;
            const double pos = x[d] * L.a[d];
            const double minTime = -fabs(w.time - w.ctime), maxTime = fabs(w.time - w.ctime);
            const double minPos = minTime * w.vel[d] + w.pos[d], maxPos = maxTime * w.vel[d] + w.pos[d];
            if (flag == OPX_WINDOW_GAUSSIAN) {
                const double sigma = (maxPos - minPos) / two_sqrt_log_two;
                const double z = (pos - w.pos[d]) / sigma;
                factor *= exp(-(z * z));
            } else if (flag == OPX_WINDOW_TUKEY) {
                const double xx = (pos - w.pos[d]) / (maxPos - minPos), tw = w.tukey;
                double sup;
                if ((xx > -.5 - .5 * tw) && (xx <= -.5 + .5 * tw)) sup = 0.5 * (1 + sin(pi * (xx + 0.5) / tw));
                else if ((xx > -.5 + .5 * tw) && (xx <= .5 - 0.5 * tw)) sup = 1;
                else if ((xx > 0.5 - 0.5 * tw) && (xx < 0.5 + 0.5 * tw)) sup = 0.5 * (1 - sin(pi * (xx - 0.5) / tw));
                else sup = 0;
                factor *= sup;
            } else if ((pos < minPos) || (pos > maxPos)) {
                inside = false;
            }
        }
        for (int d = 0; d < 3; d++) {
            if (flag == OPX_WINDOW_CONE) {
                if (inside) continue;
                Up.store(d, s, Q2<double>{{1.0, 0.0, 0.0, 0.0}});
                Unp.store(d, s, Q2<double>{{1.0, 0.0, 0.0, 0.0}});
                for (int c = 0; c < 3; c++) E[((long)d * 3 + c) * L.V + s] = 0.0;
            } else {
                for (int c = 0; c < 3; c++) E[((long)d * 3 + c) * L.V + s] *= factor;
                Up.store(d, s, su2_pow_ref(Up.load(d, s), factor));
                Unp.store(d, s, su2_pow_ref(Unp.load(d, s), factor));
            }
        }
    }
}

// CoulombGauge.CalculateDivergence (:148-166) for the three colours; block
// partial sums of the squares, per colour.
__global__ void __launch_bounds__(256) k_coulomb_div(const double *__restrict__ U, Lat L,
                                                     cufftDoubleComplex *__restrict__ f, double *__restrict__ part) {
    const LinkPlanes<SU2<double>, double> Up{const_cast<double *>(U), L.V};
    KSum acc[3] = {{0, 0}, {0, 0}, {0, 0}};
    for (long s = (long)blockIdx.x * blockDim.x + threadIdx.x; s < L.V; s += (long)gridDim.x * blockDim.x) {
        int x[3];
        site_coords(L, s, x);
        const Nbr nb = neighbours(L, s, x);
        double dv[3] = {0.0, 0.0, 0.0};
        for (int d = 0; d < 3; d++) {
            const Q2<double> u = Up.load(d, s), w = Up.load(d, nb.bwd[d]);
            double a[3], b[3];
            su2_log(u.e, a);
            su2_log(w.e, b);
            for (int c = 0; c < 3; c++) dv[c] += a[c] - b[c];
        }
        for (int c = 0; c < 3; c++) {
            f[(long)c * L.V + s] = make_cuDoubleComplex(dv[c], 0.0);
            two_sum_add(acc[c], dv[c] * dv[c]);
        }
    }
    int q;
    KSum v = block_reduce<3>(acc, q);
    if (q >= 0) { part[((long)blockIdx.x * 3 + q) * 2] = v.s; part[((long)blockIdx.x * 3 + q) * 2 + 1] = v.c; }
}

// CoulombGauge.InverseLaplaceOperator (:169-193) on the three colours' spectra
__global__ void k_inverse_laplace(cufftDoubleComplex *__restrict__ f, Lat L) {
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    int k[3];
    site_coords(L, s, k);
    double inv = 0.0;
    if (!(k[0] == 0 && k[1] == 0 && k[2] == 0)) {
        const double pi = 3.141592653589793;
        inv = -0.5 / ((cos(2 * pi * k[0] / (double)L.n[0]) + cos(2 * pi * k[1] / (double)L.n[1]) +
                       cos(2 * pi * k[2] / (double)L.n[2])) - 3.);
    }
    for (int c = 0; c < 3; c++) {
        const cufftDoubleComplex z = f[(long)c * L.V + s];
        f[(long)c * L.V + s] = make_cuDoubleComplex(z.x * inv, z.y * inv);
    }
}

// g(x) = getLink(-psi(x)), psi = Re(inverse transform) / V (CoulombGauge.java:95-122)
__device__ __forceinline__ void coulomb_g(const cufftDoubleComplex *__restrict__ f, long V, long s, double *g) {
    const double inv = 1.0 / (double)V;
    const double v[3] = {(f[s].x * inv) * -1, (f[V + s].x * inv) * -1, (f[2 * V + s].x * inv) * -1};
    su2_link_ref(v, g);
}

// GaugeTransformation's action (:57-90): U -> g U g^dagger(x+i), Unext likewise,
// E -> proj(g getLinearizedLink(E) g^dagger)
__global__ void k_coulomb_apply(const cufftDoubleComplex *__restrict__ f, Lat L, double *__restrict__ U,
                                double *__restrict__ Un, double *__restrict__ E) {
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    const LinkPlanes<SU2<double>, double> Up{U, L.V}, Unp{Un, L.V};
    int x[3];
    site_coords(L, s, x);
    const Nbr nb = neighbours(L, s, x);
    double g[4], ga[4];
    coulomb_g(f, L.V, s, g);
    ga[0] = g[0]; ga[1] = -g[1]; ga[2] = -g[2]; ga[3] = -g[3];
    for (int d = 0; d < 3; d++) {
        double gs[4], gd[4], t[4], r[4];
        coulomb_g(f, L.V, nb.fwd[d], gs);
        gd[0] = gs[0]; gd[1] = -gs[1]; gd[2] = -gs[2]; gd[3] = -gs[3];
        Q2<double> u = Up.load(d, s);
        q_mul(g, u.e, t);
        q_mul(t, gd, r);
        Up.store(d, s, Q2<double>{{r[0], r[1], r[2], r[3]}});
        u = Unp.load(d, s);
        q_mul(g, u.e, t);
        q_mul(t, gd, r);
        Unp.store(d, s, Q2<double>{{r[0], r[1], r[2], r[3]}});
        double *e = E + (long)d * 3 * L.V + s;
        const double e0 = e[0], e1 = e[L.V], e2 = e[2 * L.V];
        const double sum = (e0 * e0 + e1 * e1 + e2 * e2) / 4;
        const double lin[4] = {sqrt(1.0 - sum), e0 / 2, e1 / 2, e2 / 2};
        q_mul(g, lin, t);
        q_mul(t, ga, r);
        e[0] = 2 * r[1]; e[L.V] = 2 * r[2]; e[2 * L.V] = 2 * r[3];
    }
}

// OccupationNumbersInTime.calculate (:203-225): fields into the 18 transform inputs,
// F[0..8] = E_j^k gainv, F[9..17] = A_j^k gainv averaged over U and Unext
__global__ void k_occ_fields(const double *__restrict__ U, const double *__restrict__ Un, const double *__restrict__ E,
                             Lat L, double gainv, cufftDoubleComplex *__restrict__ F) {
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    const LinkPlanes<SU2<double>, double> Up{const_cast<double *>(U), L.V}, Unp{const_cast<double *>(Un), L.V};
    for (int j = 0; j < 3; j++) {
        double a0[3], a1[3];
        su2_log(Up.load(j, s).e, a0);
        su2_log(Unp.load(j, s).e, a1);
        for (int k = 0; k < 3; k++) {
            F[(long)(j * 3 + k) * L.V + s] = make_cuDoubleComplex(E[((long)j * 3 + k) * L.V + s] * gainv, 0.0);
            F[(long)(9 + j * 3 + k) * L.V + s] = make_cuDoubleComplex(0.5 * (a0[k] * gainv + a1[k] * gainv), 0.0);
        }
    }
}

// occupation numbers n[i][k] (:230-263) and block partial sums of their total
__global__ void __launch_bounds__(256) k_occupation(const cufftDoubleComplex *__restrict__ F, Lat L, double a,
                                                    double conv, double *__restrict__ n, double *__restrict__ part) {
    KSum acc[1] = {{0, 0}};
    const double pi = 3.141592653589793;
    for (long s = (long)blockIdx.x * blockDim.x + threadIdx.x; s < L.V; s += (long)gridDim.x * blockDim.x) {
        int x[3];
        site_coords(L, s, x);
        double w2 = 0.0;
        for (int i = 0; i < 3; i++) {
            const double delta = x[i] / ((double)L.n[i]);
            const double k = delta < 0.5 ? 2.0 * delta * pi / a : 2.0 * (delta - 1.0) * pi / a;
            w2 += 2.0 * (1.0 - cos(k * a)) / (a * a);
        }
        const double w = sqrt(w2);
        for (int k = 0; k < 3; k++) {
            double e2 = 0.0, a2 = 0.0, mixed = 0.0;
            for (int j = 0; j < 3; j++) {
                const cufftDoubleComplex ef = F[(long)(j * 3 + k) * L.V + s], af = F[(long)(9 + j * 3 + k) * L.V + s];
                e2 += ef.x * ef.x + ef.y * ef.y;
                a2 += (af.x * af.x + af.y * af.y);
                mixed -= 2.0 * (-af.y * ef.x + af.x * ef.y);
            }
            const double v = (e2 + w * w * a2 + w * mixed) * conv;
            if (n) n[s * 3 + k] = v;
            two_sum_add(acc[0], v);
        }
    }
    int q;
    KSum v = block_reduce<1>(acc, q);
    if (q >= 0) { part[(long)blockIdx.x * 2] = v.s; part[(long)blockIdx.x * 2 + 1] = v.c; }
}

}  // namespace opx

using namespace opx;

extern "C" int opx_occupation_numbers_ex(opx_ctx *ctx, const opx_occupation_options *opt, int max_iter,
                                         double accuracy_goal, double *n_out, size_t count, double *energy_density,
                                         int *iterations, double *last_divergence) {
    if (!ctx) return OPX_ERR_INVALID;
    Ctx &c = ctx_of(ctx);
    const int md = opt ? opt->mirrored_direction : -1;
    const int wflags = opt ? opt->windows : 0;
    if (md < -1 || md > 2 || (wflags & ~(OPX_WINDOW_GAUSSIAN | OPX_WINDOW_TUKEY | OPX_WINDOW_CONE))) {
        c.err = "opx_occupation_numbers_ex: mirrored_direction -1..2, windows a combination of OPX_WINDOW_*";
        return OPX_ERR_INVALID;
    }
    if (c.nc != 2) {
        c.err = "opx_occupation_numbers: SU(2) only (the SU(3) gauge-field logarithm is not provided)";
        return OPX_ERR_UNSUPPORTED;
    }
    const long V = c.L.V;
    if (n_out && count != (size_t)V * 3) { c.err = "opx_occupation_numbers: n must hold 3*V doubles"; return OPX_ERR_INVALID; }
    if (max_iter < 1) { c.err = "opx_occupation_numbers: max_iter >= 1"; return OPX_ERR_INVALID; }
    if (!(c.L.a[0] == c.L.a[1] && c.L.a[1] == c.L.a[2])) {
        c.err = "opx_occupation_numbers: isotropic lattice spacing only (the reference uses one spacing)";
        return OPX_ERR_UNSUPPORTED;
    }
    if (!fft_lib().load(c.err)) return OPX_ERR_UNSUPPORTED;
    // the lattice the Coulomb gauge is fixed on: the handle's, or the mirrored one
    int dm[3] = {c.L.n[0], c.L.n[1], c.L.n[2]};
    if (md >= 0) dm[md] *= 2;
    const Lat Lm = make_lat(dm, c.L.a, c.L.dt, c.L.g);
    const long Vm = Lm.V;
    const size_t nU = (size_t)link_elems(V, 4), nUm = (size_t)link_elems(Vm, 4);
    double *Uc = nullptr, *Unc = nullptr, *Ec = nullptr, *part = nullptr, *nd = nullptr;
    double *Ucm = nullptr, *Uncm = nullptr, *Ecm = nullptr;
    cufftDoubleComplex *F = nullptr;
    const int B = 256, nb = (int)std::min<long>(grid_for(Vm, B), 4L * 152);
    bool ok = cudaMalloc(&Uc, sizeof(double) * nU) == cudaSuccess && cudaMalloc(&Unc, sizeof(double) * nU) == cudaSuccess &&
              cudaMalloc(&Ec, sizeof(double) * 9 * V) == cudaSuccess &&
              cudaMalloc(&F, sizeof(cufftDoubleComplex) * std::max(18 * V, 3 * Vm)) == cudaSuccess &&
              cudaMalloc(&part, sizeof(double) * 6 * nb) == cudaSuccess &&
              (!n_out || cudaMalloc(&nd, sizeof(double) * 3 * V) == cudaSuccess);
    if (md >= 0)
        ok = ok && cudaMalloc(&Ucm, sizeof(double) * nUm) == cudaSuccess &&
             cudaMalloc(&Uncm, sizeof(double) * nUm) == cudaSuccess && cudaMalloc(&Ecm, sizeof(double) * 9 * Vm) == cudaSuccess;
    int rc = OPX_OK;
    FFTPlan p3, p18;
    int dims[3] = {c.L.n[0], c.L.n[1], c.L.n[2]};
    if (ok) ok = p3.make(3, dm, 3, c.stream) && p18.make(3, dims, 18, c.stream);
    if (!ok) {
        cudaGetLastError();
        c.err = "opx_occupation_numbers: out of device memory or cuFFT plan failure";
        rc = OPX_ERR_NOMEM;
    }
    std::vector<double> hp(6 * nb);
    int it = 0;
    double s = 0.0;
    // the buffers the gauge is fixed in
    double *Ug = md >= 0 ? Ucm : Uc, *Ung = md >= 0 ? Uncm : Unc, *Eg = md >= 0 ? Ecm : Ec;
    if (!rc) {
        if (md >= 0) {
            if (c.prec == OPX_F64)
                k_occ_copy_mirror<double><<<grid_for(V, B), B, 0, c.stream>>>(
                    (const double *)c.U, (const double *)c.Unext, (const double *)c.E, c.L, Lm, md, Ug, Ung, Eg);
            else
                k_occ_copy_mirror<float><<<grid_for(V, B), B, 0, c.stream>>>(
                    (const float *)c.U, (const float *)c.Unext, (const float *)c.E, c.L, Lm, md, Ug, Ung, Eg);
        } else if (c.prec == OPX_F64) {
            k_occ_copy<double><<<grid_for(V, B), B, 0, c.stream>>>((const double *)c.U, (const double *)c.Unext,
                                                                   (const double *)c.E, c.L, Uc, Unc, Ec);
        } else {
            k_occ_copy<float><<<grid_for(V, B), B, 0, c.stream>>>((const float *)c.U, (const float *)c.Unext,
                                                                  (const float *)c.E, c.L, Uc, Unc, Ec);
        }
        c.launches++;
        // CoulombGauge.applyGaugeTransformation (:56-75)
        while (it < max_iter && !rc) {
            k_coulomb_div<<<nb, B, 0, c.stream>>>(Ug, Lm, F, part);
            cudaMemcpyAsync(hp.data(), part, sizeof(double) * 6 * nb, cudaMemcpyDeviceToHost, c.stream);
            if (fft_lib().execZ2Z(p3.h, F, F, CUFFT_FORWARD) != CUFFT_SUCCESS) rc = OPX_ERR_CUDA;
            k_inverse_laplace<<<grid_for(Vm, B), B, 0, c.stream>>>(F, Lm);
            if (fft_lib().execZ2Z(p3.h, F, F, CUFFT_INVERSE) != CUFFT_SUCCESS) rc = OPX_ERR_CUDA;
            k_coulomb_apply<<<grid_for(Vm, B), B, 0, c.stream>>>(F, Lm, Ug, Ung, Eg);
            c.launches += 5;
            cudaError_t e = cudaStreamSynchronize(c.stream);
            if (e != cudaSuccess) { c.err = std::string("opx_occupation_numbers: ") + cudaGetErrorString(e); rc = OPX_ERR_CUDA; break; }
            // colour by colour, blocks in index order
            s = 0.0;
            for (int col = 0; col < 3; col++) {
                KSum v{0.0, 0.0};
                for (int b = 0; b < nb; b++) ksum_merge(v, KSum{hp[((size_t)b * 3 + col) * 2], hp[((size_t)b * 3 + col) * 2 + 1]});
                s += v.s + v.c;
            }
            it++;
            if (s < accuracy_goal) break;
        }
        if (rc && c.err.empty()) c.err = "opx_occupation_numbers: cuFFT execution failed";
    }
    if (!rc && md >= 0) {
        k_occ_unmirror<<<grid_for(V, B), B, 0, c.stream>>>(Ucm, Uncm, Ecm, Lm, c.L, Uc, Unc, Ec);
        c.launches++;
    }
    if (!rc && wflags) {
        OccWindow w;
        w.flags = wflags;
        w.time = (double)c.steps * c.L.dt;  // grid.getSimulationSteps() * grid.getTemporalSpacing()
        w.ctime = opt->collision_time;
        w.tukey = opt->tukey_width;
        for (int d = 0; d < 3; d++) { w.pos[d] = opt->collision_position[d]; w.vel[d] = opt->cone_velocity[d]; }
        k_occ_window<<<grid_for(V, B), B, 0, c.stream>>>(Uc, Unc, Ec, c.L, w);
        c.launches++;
    }
    double energy = 0.0;
    if (!rc) {
        const double a = c.L.a[0];
        const double gainv = 1.0 / (a * c.L.g);
        int deff = 0;
        double box = 1.0;
        for (int i = 0; i < 3; i++)
            if (c.L.n[i] > 1) { deff++; box *= c.L.n[i] * c.L.a[i]; }
        const double conv = std::pow(a, 2 * deff);
        k_occ_fields<<<grid_for(V, B), B, 0, c.stream>>>(Uc, Unc, Ec, c.L, gainv, F);
        if (fft_lib().execZ2Z(p18.h, F, F, CUFFT_FORWARD) != CUFFT_SUCCESS) rc = OPX_ERR_CUDA;
        k_occupation<<<nb, B, 0, c.stream>>>(F, c.L, a, conv, nd, part);
        c.launches += 2;
        cudaMemcpyAsync(hp.data(), part, sizeof(double) * 2 * nb, cudaMemcpyDeviceToHost, c.stream);
        if (n_out) cudaMemcpyAsync(n_out, nd, sizeof(double) * 3 * V, cudaMemcpyDeviceToHost, c.stream);
        cudaError_t e = cudaStreamSynchronize(c.stream);
        if (e != cudaSuccess) { c.err = std::string("opx_occupation_numbers: ") + cudaGetErrorString(e); rc = OPX_ERR_CUDA; }
        if (!rc) {
            KSum v{0.0, 0.0};
            for (int b = 0; b < nb; b++) ksum_merge(v, KSum{hp[(size_t)b * 2], hp[(size_t)b * 2 + 1]});
            energy = (v.s + v.c) * (1.0 / (2.0 * box * box));
        }
    }
    void *bufs[] = {Uc, Unc, Ec, F, part, nd, Ucm, Uncm, Ecm};
    for (void *b : bufs) if (b) cudaFree(b);
    if (rc) return rc;
    if (energy_density) *energy_density = energy;
    if (iterations) *iterations = it;
    if (last_divergence) *last_divergence = s;
    return OPX_OK;
}

extern "C" int opx_occupation_numbers(opx_ctx *ctx, int max_iter, double accuracy_goal, double *n_out, size_t count,
                                      double *energy_density, int *iterations, double *last_divergence) {
    return opx_occupation_numbers_ex(ctx, nullptr, max_iter, accuracy_goal, n_out, count, energy_density, iterations,
                                     last_divergence);
}
