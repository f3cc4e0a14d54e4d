// occupation_kernels.cu -- Coulomb gauge fixing and gluon occupation numbers (SU(2), SU(3)).
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
#include "su3_log.cuh"

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

// Per-group operations of the occupation numbers, FP64 links.  NCOMP is the
// number of generator components (the reference's numberOfComponents).
template <int NC> struct OccG;
template <> struct OccG<2> {
    using M = Q2<double>;
    static constexpr int NCOMP = 3;
    // getAlgebraElement (SU2GroupElement.java:234-252)
    __device__ static void log_gen(const M &u, double *x) { su2_log(u.e, x); }
    // getLink in the reference's own form (SU2AlgebraElement.java:140-152)
    __device__ static M link(const double *x) {
        M u;
        su2_link_ref(x, u.e);
        return u;
    }
    // g U h^dagger
    __device__ static M conj2(const M &g, const M &u, const M &h) { return SU2<double>::mul(SU2<double>::mul(g, u), SU2<double>::adj(h)); }
    // proj(g getLinearizedLink(E) g^dagger) (SU2AlgebraElement.java:133-138)
    __device__ static void act_lin(const M &g, double *e) {
        const double sum = (e[0] * e[0] + e[1] * e[1] + e[2] * e[2]) / 4;
        const double lin[4] = {sqrt(1.0 - sum), e[0] / 2, e[1] / 2, e[2] / 2};
        double t[4], r[4], ga[4] = {g.e[0], -g.e[1], -g.e[2], -g.e[3]};
        q_mul(g.e, lin, t);
        q_mul(t, ga, r);
        e[0] = 2 * r[1]; e[1] = 2 * r[2]; e[2] = 2 * r[3];
    }
};
template <> struct OccG<3> {
    using M = M3<double>;
    static constexpr int NCOMP = 8;
    __device__ static void log_gen(const M &u, double *x) { su3_log_gen(u, x); }
    __device__ static M link(const double *x) { return SU3<double>::expi(x); }
    __device__ static M conj2(const M &g, const M &u, const M &h) { return SU3<double>::mul_adj(SU3<double>::mul(g, u), h); }
    // proj(g getLinearizedLink(E) g^dagger) = the components of g E g^dagger
    // (SU3AlgebraElement.java:402-405: getLinearizedLink = I + i E)
    __device__ static void act_lin(const M &g, double *e) {
        double o[8];
        SU3<double>::act(e, g, o);
        for (int a = 0; a < 8; a++) e[a] = o[a];
    }
};
template <typename R> __device__ __forceinline__ Q2<double> widen(const Q2<R> &a) {
    return Q2<double>{{(double)a.e[0], (double)a.e[1], (double)a.e[2], (double)a.e[3]}};
}
template <typename R> __device__ __forceinline__ M3<double> widen(const M3<R> &a) {
    M3<double> m;
    for (int k = 0; k < 9; k++) { m.r[k] = (double)a.r[k]; m.i[k] = (double)a.i[k]; }
    return m;
}

template <int NC, typename R>
__global__ void k_occ_copy(const R *__restrict__ U, const R *__restrict__ Un, const R *__restrict__ E, Lat L,
                           double *__restrict__ Uc, double *__restrict__ Unc, double *__restrict__ Ec) {
    using G = typename GroupOf<NC, R>::T;
    constexpr int NA = OccG<NC>::NCOMP;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    const LinkPlanes<G, R> Up{const_cast<R *>(U), L.V}, Unp{const_cast<R *>(Un), L.V};
    const LinkPlanes<typename GroupOf<NC, double>::T, double> Uo{Uc, L.V}, Uno{Unc, L.V};
    for (int d = 0; d < 3; d++) {
        Uo.store(d, s, widen(Up.load(d, s)));
        Uno.store(d, s, widen(Unp.load(d, s)));
        for (int a2 = 0; a2 < NA; a2++) Ec[((long)d * NA + a2) * L.V + s] = (double)E[((long)d * NA + a2) * L.V + s];
    }
}

// MirroredGrid (:655-686): the grid doubled along md, every cell copied to its
// own position and to the mirrored one (2 N - 1 - x), and the mirrored copy's
// link along md taken from the cell one step back (x - 1, or x itself at x = 0)
template <int NC, typename R>
__global__ void k_occ_copy_mirror(const R *__restrict__ U, const R *__restrict__ Un, const R *__restrict__ E, Lat L,
                                  Lat Lm, int md, double *__restrict__ Uc, double *__restrict__ Unc,
                                  double *__restrict__ Ec) {
    using G = typename GroupOf<NC, R>::T;
    constexpr int NA = OccG<NC>::NCOMP;
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
    const LinkPlanes<G, R> Up{const_cast<R *>(U), L.V}, Unp{const_cast<R *>(Un), L.V};
    const LinkPlanes<typename GroupOf<NC, double>::T, double> Uo{Uc, Lm.V}, Uno{Unc, Lm.V};
    for (int d = 0; d < 3; d++) {
        const auto a = widen(Up.load(d, s)), b = widen(Unp.load(d, s));
        Uo.store(d, s1, a);
        Uo.store(d, s2, d == md ? widen(Up.load(d, sh)) : a);
        Uno.store(d, s1, b);
        Uno.store(d, s2, b);
        for (int c = 0; c < NA; c++) {
            const double e = (double)E[((long)d * NA + c) * L.V + s];
            Ec[((long)d * NA + c) * Lm.V + s1] = e;
            Ec[((long)d * NA + c) * Lm.V + s2] = e;
        }
    }
}

// UnmirroredGrid (:688-703): the cells of the first half, at their own positions
template <int NC>
__global__ void k_occ_unmirror(const double *__restrict__ Ucm, const double *__restrict__ Uncm,
                               const double *__restrict__ Ecm, Lat Lm, Lat L, double *__restrict__ Uc,
                               double *__restrict__ Unc, double *__restrict__ Ec) {
    using G = typename GroupOf<NC, double>::T;
    constexpr int NA = OccG<NC>::NCOMP;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    int x[3];
    site_coords(L, s, x);
    const long sm = ((long)x[0] * Lm.n[1] + x[1]) * Lm.n[2] + x[2];
    const LinkPlanes<G, double> Ui{const_cast<double *>(Ucm), Lm.V}, Uni{const_cast<double *>(Uncm), Lm.V};
    const LinkPlanes<G, double> Uo{Uc, L.V}, Uno{Unc, L.V};
    for (int d = 0; d < 3; d++) {
        Uo.store(d, s, Ui.load(d, sm));
        Uno.store(d, s, Uni.load(d, sm));
        for (int c = 0; c < NA; c++) Ec[((long)d * NA + c) * L.V + s] = Ecm[((long)d * NA + c) * Lm.V + sm];
    }
}

// GroupElement.pow(x) = getLink(x getAlgebraElement()) (SU2GroupElement.java:269-271,
// SU3GroupElement.java:516-518)
template <int NC>
__device__ __forceinline__ typename OccG<NC>::M group_pow(const typename OccG<NC>::M &u, double f) {
    double v[OccG<NC>::NCOMP];
    OccG<NC>::log_gen(u, v);
    for (int c = 0; c < OccG<NC>::NCOMP; c++) v[c] *= f;
    return OccG<NC>::link(v);
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
template <int NC>
__global__ void k_occ_window(double *__restrict__ U, double *__restrict__ Un, double *__restrict__ E, Lat L,
                             OccWindow w) {
    using G = typename GroupOf<NC, double>::T;
    constexpr int NA = OccG<NC>::NCOMP;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    int x[3];
    site_coords(L, s, x);
    const double two_sqrt_log_two = 2 * sqrt(log(2.0));
    const double pi = 3.141592653589793;
    const LinkPlanes<G, double> Up{U, L.V}, Unp{Un, L.V};
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
                const double zero[NA] = {};
                Up.store(d, s, OccG<NC>::link(zero));
                Unp.store(d, s, OccG<NC>::link(zero));
                for (int c = 0; c < NA; c++) E[((long)d * NA + c) * L.V + s] = 0.0;
            } else {
                for (int c = 0; c < NA; c++) E[((long)d * NA + c) * L.V + s] *= factor;
                Up.store(d, s, group_pow<NC>(Up.load(d, s), factor));
                Unp.store(d, s, group_pow<NC>(Unp.load(d, s), factor));
            }
        }
    }
}

// CoulombGauge.CalculateDivergence (:148-166) for every colour; block partial
// sums of the squares, per colour.  f: [NCOMP][V]
template <int NC>
__global__ void __launch_bounds__(256) k_coulomb_div(const double *__restrict__ U, Lat L,
                                                     cufftDoubleComplex *__restrict__ f, double *__restrict__ part) {
    using G = typename GroupOf<NC, double>::T;
    constexpr int NA = OccG<NC>::NCOMP;
    const LinkPlanes<G, double> Up{const_cast<double *>(U), L.V};
    KSum acc[NA];
    for (int c = 0; c < NA; c++) acc[c] = KSum{0, 0};
    for (long s = (long)blockIdx.x * blockDim.x + threadIdx.x; s < L.V; s += (long)gridDim.x * blockDim.x) {
        int x[3];
        site_coords(L, s, x);
        const Nbr nb = neighbours(L, s, x);
        double dv[NA];
        for (int c = 0; c < NA; c++) dv[c] = 0.0;
        for (int d = 0; d < 3; d++) {
            double a[NA], b[NA];
            OccG<NC>::log_gen(Up.load(d, s), a);
            OccG<NC>::log_gen(Up.load(d, nb.bwd[d]), b);
            for (int c = 0; c < NA; c++) dv[c] += a[c] - b[c];
        }
        for (int c = 0; c < NA; c++) {
            f[(long)c * L.V + s] = make_cuDoubleComplex(dv[c], 0.0);
            two_sum_add(acc[c], dv[c] * dv[c]);
        }
    }
    int q;
    KSum v = block_reduce<NA>(acc, q);
    if (q >= 0) { part[((long)blockIdx.x * NA + q) * 2] = v.s; part[((long)blockIdx.x * NA + q) * 2 + 1] = v.c; }
}

// CoulombGauge.InverseLaplaceOperator (:169-193) on the colours' spectra
__global__ void k_inverse_laplace(cufftDoubleComplex *__restrict__ f, Lat L, int ncomp) {
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
    for (int c = 0; c < ncomp; c++) {
        const cufftDoubleComplex z = f[(long)c * L.V + s];
        f[(long)c * L.V + s] = make_cuDoubleComplex(z.x * inv, z.y * inv);
    }
}

// g(x) = getLink(-psi(x)), psi = Re(inverse transform) / V (CoulombGauge.java:95-122)
template <int NC>
__device__ __forceinline__ typename OccG<NC>::M coulomb_g(const cufftDoubleComplex *__restrict__ f, long V, long s) {
    const double inv = 1.0 / (double)V;
    double v[OccG<NC>::NCOMP];
    for (int c = 0; c < OccG<NC>::NCOMP; c++) v[c] = (f[(long)c * V + s].x * inv) * -1;
    return OccG<NC>::link(v);
}

// GaugeTransformation's action (:57-90): U -> g U g^dagger(x+i), Unext likewise,
// E -> proj(g getLinearizedLink(E) g^dagger)
template <int NC>
__global__ void k_coulomb_apply(const cufftDoubleComplex *__restrict__ f, Lat L, double *__restrict__ U,
                                double *__restrict__ Un, double *__restrict__ E) {
    using G = typename GroupOf<NC, double>::T;
    constexpr int NA = OccG<NC>::NCOMP;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    const LinkPlanes<G, double> Up{U, L.V}, Unp{Un, L.V};
    int x[3];
    site_coords(L, s, x);
    const Nbr nb = neighbours(L, s, x);
    const auto g = coulomb_g<NC>(f, L.V, s);
    for (int d = 0; d < 3; d++) {
        const auto gs = coulomb_g<NC>(f, L.V, nb.fwd[d]);
        Up.store(d, s, OccG<NC>::conj2(g, Up.load(d, s), gs));
        Unp.store(d, s, OccG<NC>::conj2(g, Unp.load(d, s), gs));
        double e[NA];
        for (int c = 0; c < NA; c++) e[c] = E[((long)d * NA + c) * L.V + s];
        OccG<NC>::act_lin(g, e);
        for (int c = 0; c < NA; c++) E[((long)d * NA + c) * L.V + s] = e[c];
    }
}

// OccupationNumbersInTime.calculate (:203-225): fields into the 6 NCOMP transform
// inputs, F[j NCOMP + k] = E_j^k gainv, F[(3 + j) NCOMP + k] = A_j^k gainv averaged
// over U and Unext
template <int NC>
__global__ void k_occ_fields(const double *__restrict__ U, const double *__restrict__ Un, const double *__restrict__ E,
                             Lat L, double gainv, cufftDoubleComplex *__restrict__ F) {
    using G = typename GroupOf<NC, double>::T;
    constexpr int NA = OccG<NC>::NCOMP;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    const LinkPlanes<G, double> Up{const_cast<double *>(U), L.V}, Unp{const_cast<double *>(Un), L.V};
    for (int j = 0; j < 3; j++) {
        double a0[NA], a1[NA];
        OccG<NC>::log_gen(Up.load(j, s), a0);
        OccG<NC>::log_gen(Unp.load(j, s), a1);
        for (int k = 0; k < NA; k++) {
            F[(long)(j * NA + k) * L.V + s] = make_cuDoubleComplex(E[((long)j * NA + k) * L.V + s] * gainv, 0.0);
            F[(long)((3 + j) * NA + k) * L.V + s] = make_cuDoubleComplex(0.5 * (a0[k] * gainv + a1[k] * gainv), 0.0);
        }
    }
}

// occupation numbers n[i][k] (:230-263) and block partial sums of their total
template <int NC>
__global__ void __launch_bounds__(256) k_occupation(const cufftDoubleComplex *__restrict__ F, Lat L, double a,
                                                    double conv, double *__restrict__ n, double *__restrict__ part) {
    constexpr int NA = OccG<NC>::NCOMP;
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
        for (int k = 0; k < NA; k++) {
            double e2 = 0.0, a2 = 0.0, mixed = 0.0;
            for (int j = 0; j < 3; j++) {
                const cufftDoubleComplex ef = F[(long)(j * NA + k) * L.V + s], af = F[(long)((3 + j) * NA + k) * L.V + s];
                e2 += ef.x * ef.x + ef.y * ef.y;
                a2 += (af.x * af.x + af.y * af.y);
                mixed -= 2.0 * (-af.y * ef.x + af.x * ef.y);
            }
            const double v = (e2 + w * w * a2 + w * mixed) * conv;
            if (n) n[s * NA + k] = v;
            two_sum_add(acc[0], v);
        }
    }
    int q;
    KSum v = block_reduce<1>(acc, q);
    if (q >= 0) { part[(long)blockIdx.x * 2] = v.s; part[(long)blockIdx.x * 2 + 1] = v.c; }
}

}  // namespace opx

using namespace opx;

template <int NC>
static int occupation_t(Ctx &c, const opx_occupation_options *opt, int max_iter, double accuracy_goal, double *n_out,
                        size_t count, double *energy_density, int *iterations, double *last_divergence) {
    constexpr int NA = OccG<NC>::NCOMP;
    const int ng = NC == 2 ? 4 : 18;
    const int md = opt ? opt->mirrored_direction : -1;
    const int wflags = opt ? opt->windows : 0;
    if (md < -1 || md > 2 || (wflags & ~(OPX_WINDOW_GAUSSIAN | OPX_WINDOW_TUKEY | OPX_WINDOW_CONE))) {
        c.err = "opx_occupation_numbers_ex: mirrored_direction -1..2, windows a combination of OPX_WINDOW_*";
        return OPX_ERR_INVALID;
    }
    const long V = c.L.V;
    if (n_out && count != (size_t)V * NA) {
        c.err = "opx_occupation_numbers: n must hold V * (N^2 - 1) doubles";
        return OPX_ERR_INVALID;
    }
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
    const size_t nU = (size_t)link_elems(V, ng), nUm = (size_t)link_elems(Vm, ng);
    double *Uc = nullptr, *Unc = nullptr, *Ec = nullptr, *part = nullptr, *nd = nullptr;
    double *Ucm = nullptr, *Uncm = nullptr, *Ecm = nullptr;
    cufftDoubleComplex *F = nullptr;
    const int B = 256, nb = (int)std::min<long>(grid_for(Vm, B), 4L * 152);
    bool ok = cudaMalloc(&Uc, sizeof(double) * nU) == cudaSuccess && cudaMalloc(&Unc, sizeof(double) * nU) == cudaSuccess &&
              cudaMalloc(&Ec, sizeof(double) * 3 * NA * V) == cudaSuccess &&
              cudaMalloc(&F, sizeof(cufftDoubleComplex) * std::max(6L * NA * V, (long)NA * Vm)) == cudaSuccess &&
              cudaMalloc(&part, sizeof(double) * 2 * NA * nb) == cudaSuccess &&
              (!n_out || cudaMalloc(&nd, sizeof(double) * NA * V) == cudaSuccess);
    if (md >= 0)
        ok = ok && cudaMalloc(&Ucm, sizeof(double) * nUm) == cudaSuccess &&
             cudaMalloc(&Uncm, sizeof(double) * nUm) == cudaSuccess &&
             cudaMalloc(&Ecm, sizeof(double) * 3 * NA * Vm) == cudaSuccess;
    int rc = OPX_OK;
    FFTPlan p3, p18;
    int dims[3] = {c.L.n[0], c.L.n[1], c.L.n[2]};
    if (ok) ok = p3.make(3, dm, NA, c.stream) && p18.make(3, dims, 6 * NA, c.stream);
    if (!ok) {
        cudaGetLastError();
        c.err = "opx_occupation_numbers: out of device memory or cuFFT plan failure";
        rc = OPX_ERR_NOMEM;
    }
    std::vector<double> hp(2 * NA * nb);
    int it = 0;
    double s = 0.0;
    // the buffers the gauge is fixed in
    double *Ug = md >= 0 ? Ucm : Uc, *Ung = md >= 0 ? Uncm : Unc, *Eg = md >= 0 ? Ecm : Ec;
    if (!rc) {
        if (md >= 0) {
            if (c.prec == OPX_F64)
                k_occ_copy_mirror<NC, double><<<grid_for(V, B), B, 0, c.stream>>>(
                    (const double *)c.U, (const double *)c.Unext, (const double *)c.E, c.L, Lm, md, Ug, Ung, Eg);
            else
                k_occ_copy_mirror<NC, float><<<grid_for(V, B), B, 0, c.stream>>>(
                    (const float *)c.U, (const float *)c.Unext, (const float *)c.E, c.L, Lm, md, Ug, Ung, Eg);
        } else if (c.prec == OPX_F64) {
            k_occ_copy<NC, double><<<grid_for(V, B), B, 0, c.stream>>>((const double *)c.U, (const double *)c.Unext,
                                                                       (const double *)c.E, c.L, Uc, Unc, Ec);
        } else {
            k_occ_copy<NC, float><<<grid_for(V, B), B, 0, c.stream>>>((const float *)c.U, (const float *)c.Unext,
                                                                      (const float *)c.E, c.L, Uc, Unc, Ec);
        }
        c.launches++;
        // CoulombGauge.applyGaugeTransformation (:56-75)
        while (it < max_iter && !rc) {
            k_coulomb_div<NC><<<nb, B, 0, c.stream>>>(Ug, Lm, F, part);
            cudaMemcpyAsync(hp.data(), part, sizeof(double) * 2 * NA * nb, cudaMemcpyDeviceToHost, c.stream);
            if (fft_lib().execZ2Z(p3.h, F, F, CUFFT_FORWARD) != CUFFT_SUCCESS) rc = OPX_ERR_CUDA;
            k_inverse_laplace<<<grid_for(Vm, B), B, 0, c.stream>>>(F, Lm, NA);
            if (fft_lib().execZ2Z(p3.h, F, F, CUFFT_INVERSE) != CUFFT_SUCCESS) rc = OPX_ERR_CUDA;
            k_coulomb_apply<NC><<<grid_for(Vm, B), B, 0, c.stream>>>(F, Lm, Ug, Ung, Eg);
            c.launches += 5;
            cudaError_t e = cudaStreamSynchronize(c.stream);
            if (e != cudaSuccess) { c.err = std::string("opx_occupation_numbers: ") + cudaGetErrorString(e); rc = OPX_ERR_CUDA; break; }
            // colour by colour, blocks in index order
            s = 0.0;
            for (int col = 0; col < NA; col++) {
                KSum v{0.0, 0.0};
                for (int b = 0; b < nb; b++) ksum_merge(v, KSum{hp[((size_t)b * NA + col) * 2], hp[((size_t)b * NA + col) * 2 + 1]});
                s += v.s + v.c;
            }
            it++;
            if (s < accuracy_goal) break;
        }
        if (rc && c.err.empty()) c.err = "opx_occupation_numbers: cuFFT execution failed";
    }
    if (!rc && md >= 0) {
        k_occ_unmirror<NC><<<grid_for(V, B), B, 0, c.stream>>>(Ucm, Uncm, Ecm, Lm, c.L, Uc, Unc, Ec);
        c.launches++;
    }
    if (!rc && wflags) {
        OccWindow w;
        w.flags = wflags;
        w.time = (double)c.steps * c.L.dt;  // grid.getSimulationSteps() * grid.getTemporalSpacing()
        w.ctime = opt->collision_time;
        w.tukey = opt->tukey_width;
        for (int d = 0; d < 3; d++) { w.pos[d] = opt->collision_position[d]; w.vel[d] = opt->cone_velocity[d]; }
        k_occ_window<NC><<<grid_for(V, B), B, 0, c.stream>>>(Uc, Unc, Ec, c.L, w);
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
        k_occ_fields<NC><<<grid_for(V, B), B, 0, c.stream>>>(Uc, Unc, Ec, c.L, gainv, F);
        if (fft_lib().execZ2Z(p18.h, F, F, CUFFT_FORWARD) != CUFFT_SUCCESS) rc = OPX_ERR_CUDA;
        k_occupation<NC><<<nb, B, 0, c.stream>>>(F, c.L, a, conv, nd, part);
        c.launches += 2;
        cudaMemcpyAsync(hp.data(), part, sizeof(double) * 2 * nb, cudaMemcpyDeviceToHost, c.stream);
        if (n_out) cudaMemcpyAsync(n_out, nd, sizeof(double) * NA * V, cudaMemcpyDeviceToHost, c.stream);
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

extern "C" int opx_occupation_numbers_ex(opx_ctx *ctx, const opx_occupation_options *opt, int max_iter,
                                         double accuracy_goal, double *n_out, size_t count, double *energy_density,
                                         int *iterations, double *last_divergence) {
    if (!ctx) return OPX_ERR_INVALID;
    Ctx &c = ctx_of(ctx);
    if (c.nc == 2)
        return occupation_t<2>(c, opt, max_iter, accuracy_goal, n_out, count, energy_density, iterations, last_divergence);
    return occupation_t<3>(c, opt, max_iter, accuracy_goal, n_out, count, energy_density, iterations, last_divergence);
}

extern "C" int opx_occupation_numbers(opx_ctx *ctx, int max_iter, double accuracy_goal, double *n_out, size_t count,
                                      double *energy_density, int *iterations, double *last_divergence) {
    return opx_occupation_numbers_ex(ctx, nullptr, max_iter, accuracy_goal, n_out, count, energy_density, iterations,
                                     last_divergence);
}
