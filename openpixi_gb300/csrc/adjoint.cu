// adjoint.cu -- differentiation form of the SU(2) leapfrog.
//
// Objectives, over a box of cells after N steps of Simulation.step:
//   OPX_OBJ_ENERGY: the mean of the per-cell energy density
//     (EnergyDensity.ComponentComputation, diagnostics/methods/EnergyDensity.java:119-166),
//     J = mean_x sum_d [E_d^2/2 + |B_d(U) + B_d(Unext)|^2/4] / (g a_0)^2;
//   OPX_OBJ_ANISOTROPY: the pressure anisotropy P_L / P_T of the projected
//     energy density components (ProjectedEnergyDensity.java:18-41, 114-179):
//     per cell and direction j, eps_j = [E_j^2/2 + (|B_j(U)|^2 + |B_j(Unext)|^2)/4] / (g a_j)^2,
//     eps_L = eps_l (l the longitudinal direction), eps_T = the other two,
//     P_L = eps_T - eps_L, P_T = eps_L, J = sum_box P_L / sum_box P_T.
// Inputs: the initial electric field E_0 (the links at t = 0 fixed), or the
// colour-charge density rho through Gauss's law: the initial E is the
// projection of the handle's E onto div E = rho (Grid.getGaussConstraint),
// E_0(rho) = E + divT K^+ (rho - div E) with K = div divT, so a change d of rho
// moves E_0 by divT K^+ d and dJ/drho = K^+ div (dJ/dE_0).
//
// Forward model (FastTYMSolver, physics/fields/FastTYMSolver.java:40-84):
//     W_0 = exp(-i dt E_0) U                       (initialize: stepLinks)
//     E_n = E_{n-1} + dt proj(W_{n-1} S(W_{n-1}))  (CombinedUpdate, E part)
//     W_n = exp(-i dt E_n) W_{n-1}                 (CombinedUpdate, Unext)
// with J evaluated on (E_N, W_{N-1}, W_N).
//
// Three entry points:
//   * opx_energy_objective : J from a forward run (finite differences use it);
//   * opx_energy_tangent   : the FP64 tangent-linear model, i.e. the forward
//     kernels instantiated on dual numbers (dual.cuh), giving dJ along a direction;
//   * opx_energy_gradient  : the adjoint.  The forward runs in the handle's
//     precision and stores FP64 checkpoints of (W_n, E_n) every `ckpt` steps;
//     the reverse sweep recomputes each segment in FP64 from its checkpoint and
//     runs the hand-written reverse step below, segment by segment from the end.
//
// Reverse of one step, per link l = (x, i), in the ambient coordinates of the
// quaternions (e0..e3) with the Euclidean pairing (the reference's own
// representation, SU2GroupElement.java:3-14): for q = a b the cotangents are
// abar = qbar b^*, bbar = a^* qbar (^* = SU2GroupElement.adj).
//   W_n = X W_{n-1}, X = exp(i v.sigma/2), v = -dt E_n:
//       Wbar_{n-1} += X^* Wbar_n,  Xbar = Wbar_n W_{n-1}^*,
//       vbar_b = -(s/4) Xbar_0 v_b + (s/2) Xbar_b + (q/8) v_b (Xbar . v),
//       s = sin m / m, q = (m cos m - sin m) / m^3, m = |v|/2,
//       Ebar_n += -dt vbar
//   E_n = E_{n-1} + dt proj(M), M = W_i(x) S, proj(M) = 2 (M_1, M_2, M_3):
//       Ebar_{n-1} = Ebar_n,  Mbar = 2 dt (0, Ebar_n),
//       Wbar_i(x) += Mbar S^*,  Sbar = W_i(x)^* Mbar
//   S = sum_j c_j [A_j + B_j], A = P Q^* R^*, B = P^* Q^* R (Grid.getStapleSum,
//       Grid.java:675-696), c_j = 1/a_j^2: the cotangents of the staple links
//       are gathered by each link from the (up to) twelve staples it enters.
// SU(2) only.
#include <algorithm>
#include <vector>

#include "dual.cuh"
#include "internal.h"
#include "ksum.cuh"
#include "leapfrog.cuh"
#include "observables.cuh"

namespace opx {

using Q = Q2<double>;
using G2 = SU2<double>;

__device__ __forceinline__ double value_of(double x) { return x; }
__device__ __forceinline__ double tangent_of(double) { return 0.0; }
__device__ __forceinline__ double value_of(Dual x) { return x.v; }
__device__ __forceinline__ double tangent_of(Dual x) { return x.d; }

__device__ __forceinline__ Q qmul(const Q &a, const Q &b) { return G2::mul(a, b); }
__device__ __forceinline__ Q qadj(const Q &a) { return G2::adj(a); }
__device__ __forceinline__ Q qscale(const Q &a, double s) { return Q{{a.e[0] * s, a.e[1] * s, a.e[2] * s, a.e[3] * s}}; }
__device__ __forceinline__ void qacc(Q &a, const Q &b) {
#pragma unroll
    for (int k = 0; k < 4; k++) a.e[k] += b.e[k];
}

// cotangent of v in X = exp(i v.sigma/2) given the cotangent of X
__device__ __forceinline__ void expi_adjoint(const double *v, const Q &Xb, double *vb) {
    const double m2 = (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) * 0.25;
    double s, q;
    if (m2 < 0.01) {
        s = 1 + m2 * (-1.0 / 6 + m2 * (1.0 / 120 + m2 * (-1.0 / 5040 + m2 * (1.0 / 362880 + m2 * (-1.0 / 39916800)))));
        // q = sum_{k>=1} (-1)^k 2k/(2k+1)! m^(2k-2)
        q = -1.0 / 3 + m2 * (1.0 / 30 + m2 * (-1.0 / 840 + m2 * (1.0 / 45360 + m2 * (-1.0 / 3991680))));
    } else {
        const double m = sqrt(m2);
        double sn, cs;
        sincos(m, &sn, &cs);
        s = sn / m;
        q = (m * cs - sn) / (m2 * m);
    }
    const double xv = Xb.e[1] * v[0] + Xb.e[2] * v[1] + Xb.e[3] * v[2];
    for (int b = 0; b < 3; b++) vb[b] = -(s * 0.25) * Xb.e[0] * v[b] + 0.5 * s * Xb.e[1 + b] + 0.125 * q * v[b] * xv;
}

// staple sum S_i(x) (the same expression as leapfrog.cuh, FP64)
__device__ __forceinline__ Q staple_sum(const LinkPlanes<G2, double> &W, const Lat &L, long s, const int *x, int i) {
    Q S = G2::zero();
    const long s_pi = shift_d(L, s, pick(x[0], x[1], x[2], i), i, +1);
    for (int jj = 1; jj < 3; jj++) {
        const int j = (i + jj) % 3;
        const int xj = pick(x[0], x[1], x[2], j);
        const long s_pj = shift_d(L, s, xj, j, +1), s_mj = shift_d(L, s, xj, j, -1);
        const long s_pimj = shift_d(L, s_pi, xj, j, -1);
        Q F = G2::mul_adj(G2::mul_adj(W.load(j, s_pi), W.load(i, s_pj)), W.load(j, s));
        const Q C = G2::mul(W.load(i, s_mj), W.load(j, s_pimj));
        G2::add(F, G2::adj_mul(C, W.load(j, s_mj)));
        G2::scale(F, LatR<double>::inva2(L, j));
        G2::add(S, F);
    }
    return S;
}

// Pass 1 of the reverse step: per link, the local cotangents.
__global__ void k_adj_local(const double *__restrict__ Wprev, const double *__restrict__ Enew,
                            const double *__restrict__ Wbar_new, const double *__restrict__ Ebar_new, Lat L,
                            double *__restrict__ Sbar, double *__restrict__ Uown, double *__restrict__ Ebar_prev) {
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    const LinkPlanes<G2, double> W{const_cast<double *>(Wprev), L.V}, Wb{const_cast<double *>(Wbar_new), L.V};
    const LinkPlanes<G2, double> SB{Sbar, L.V}, UO{Uown, L.V};
    const AlgPlanes<3, double> En{const_cast<double *>(Enew), L.V}, Eb{const_cast<double *>(Ebar_new), L.V};
    const AlgPlanes<3, double> Ep{Ebar_prev, L.V};
    int x[3];
    site_coords(L, s, x);
    const double dt = L.dt;
    for (int i = 0; i < 3; i++) {
        const Q Ui = W.load(i, s);
        double e[3], v[3], eb[3], vb[3];
        En.load_ro(i, s, e);
        for (int a = 0; a < 3; a++) v[a] = -dt * e[a];
        const Q X = G2::expi(v);
        const Q Wn_b = Wb.load(i, s);
        Q own = qmul(qadj(X), Wn_b);
        expi_adjoint(v, qmul(Wn_b, qadj(Ui)), vb);
        Eb.load_ro(i, s, eb);
        for (int a = 0; a < 3; a++) eb[a] += -dt * vb[a];
        const Q Mb{{0.0, 2 * dt * eb[0], 2 * dt * eb[1], 2 * dt * eb[2]}};
        const Q S = staple_sum(W, L, s, x, i);
        qacc(own, qmul(Mb, qadj(S)));
        SB.store(i, s, qmul(qadj(Ui), Mb));
        UO.store(i, s, own);
        Ep.store(i, s, eb);
    }
}

// Pass 2: each link gathers the cotangents from the staples it belongs to.
__global__ void k_adj_gather(const double *__restrict__ Wprev, const double *__restrict__ Sbar,
                             const double *__restrict__ Uown, Lat L, double *__restrict__ Wbar_prev) {
    const long y = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= L.V) return;
    const LinkPlanes<G2, double> W{const_cast<double *>(Wprev), L.V}, SB{const_cast<double *>(Sbar), L.V};
    const LinkPlanes<G2, double> UO{const_cast<double *>(Uown), L.V}, OUT{Wbar_prev, L.V};
    int x[3];
    site_coords(L, y, x);
    for (int k = 0; k < 3; k++) {
        Q acc = UO.load(k, y);
        const int xk = pick(x[0], x[1], x[2], k);
        const long y_pk = shift_d(L, y, xk, k, +1);
        const double ck = LatR<double>::inva2(L, k);
        for (int ii = 1; ii < 3; ii++) {
            const int i = (k + ii) % 3;  // the other direction (i for the A/B-term P,R roles; j for Q roles)
            const int xi = pick(x[0], x[1], x[2], i);
            const long y_mi = shift_d(L, y, xi, i, -1);
            const long y_pi = shift_d(L, y, xi, i, +1);
            const long y_mi_pk = shift_d(L, y_mi, xk, k, +1);
            const long y_pk_pi = shift_d(L, y_pk, xi, i, +1);  // unused placeholder for symmetry
            (void)y_pk_pi;
            const double ci = LatR<double>::inva2(L, i);
            // A-term, role P: l = (y - i, i), plane k: += c_k Sbar_l U_k(y-i) U_i(y-i+k)
            qacc(acc, qscale(qmul(qmul(SB.load(i, y_mi), W.load(k, y_mi)), W.load(i, y_mi_pk)), ck));
            // A-term, role Q: l = (y - j, k), plane j=i: += c_j (U_j(y-j+k)^* Sbar_l U_j(y-j))^*
            {
                const Q P = W.load(i, y_mi_pk), R = W.load(i, y_mi);
                qacc(acc, qscale(qadj(qmul(qmul(qadj(P), SB.load(k, y_mi)), R)), ci));
            }
            // A-term, role R: l = (y, i), plane k: += c_k (U_i(y+k) U_k(y+i)^* Sbar_l)^*
            {
                const Q Qv = W.load(i, y_pk), P = W.load(k, y_pi);
                qacc(acc, qscale(qadj(qmul(qmul(Qv, qadj(P)), SB.load(i, y))), ck));
            }
            // B-term, role P: l = (y - i + k, i), plane k: += c_k (Sbar_l U_k(y-i)^* U_i(y-i))^*
            qacc(acc, qscale(qadj(qmul(qmul(SB.load(i, y_mi_pk), qadj(W.load(k, y_mi))), W.load(i, y_mi))), ck));
            // B-term, role Q: l = (y + j, k), plane j=i: += c_j (U_j(y+k) Sbar_l U_j(y)^*)^*
            {
                const long y_pj = y_pi;
                const Q P = W.load(i, y_pk), R = W.load(i, y);
                qacc(acc, qscale(qadj(qmul(qmul(P, SB.load(k, y_pj)), qadj(R))), ci));
            }
            // B-term, role R: l = (y + k, i), plane k: += c_k U_i(y) U_k(y+i) Sbar_l
            qacc(acc, qscale(qmul(qmul(W.load(i, y), W.load(k, y_pi)), SB.load(i, y_pk)), ck));
        }
        OUT.store(k, y, acc);
    }
}

__device__ __forceinline__ void atomic_add_link(double *base, long V, int d, long s, const Q &q) {
#pragma unroll
    for (int k = 0; k < 4; k++) atomicAdd(base + link_offset(V, 4, d, k, s), q.e[k]);
}

__device__ __forceinline__ bool in_box(const int *x, const int *lo, const int *hi) {
    return x[0] >= lo[0] && x[0] <= hi[0] && x[1] >= lo[1] && x[1] <= hi[1] && x[2] >= lo[2] && x[2] <= hi[2];
}

struct Box {
    int lo[3], hi[3];
    double inv_n;
};

// Cotangents of J with respect to E_N, W_{N-1} and W_N.
__global__ void k_adj_objective(const double *__restrict__ Wm, const double *__restrict__ Wn,
                                const double *__restrict__ En, Lat L, Box bx, double *__restrict__ Wm_b,
                                double *__restrict__ Wn_b, double *__restrict__ En_b) {
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    int x[3];
    site_coords(L, s, x);
    const AlgPlanes<3, double> E{const_cast<double *>(En), L.V}, Eb{En_b, L.V};
    const double uf = 1.0 / ((L.g * L.a[0]) * (L.g * L.a[0]));
    if (!in_box(x, bx.lo, bx.hi)) {
        const double z[3] = {0, 0, 0};
        for (int d = 0; d < 3; d++) Eb.store(d, s, z);
        return;
    }
    const Nbr nb = neighbours(L, s, x);
    const LinkPlanes<G2, double> U0{const_cast<double *>(Wm), L.V}, U1{const_cast<double *>(Wn), L.V};
    for (int d = 0; d < 3; d++) {
        double e[3], eb[3];
        E.load_ro(d, s, e);
        for (int a = 0; a < 3; a++) eb[a] = e[a] * uf * bx.inv_n;
        Eb.store(d, s, eb);
        const int j = (d + 1) % 3, k = (d + 2) % 3;
        double b0[3], b1[3];
        field_b<G2, double>(U0, L, s, nb, d, b0);
        field_b<G2, double>(U1, L, s, nb, d, b1);
        const double f = L.a[d] / (L.a[j] * L.a[k]);
        for (int t = 0; t < 2; t++) {
            const LinkPlanes<G2, double> &Ut = t ? U1 : U0;
            double *Wb = t ? Wn_b : Wm_b;
            // dJ/dB = (B(U) + B(Unext)) uf / (2 n); P = A1 A2 A3^* A4^*, B = 2 f vec(P)
            Q Pb{{0.0, 0.0, 0.0, 0.0}};
            for (int a = 0; a < 3; a++) Pb.e[1 + a] = 2 * f * 0.5 * (b0[a] + b1[a]) * uf * bx.inv_n;
            const Q A1 = Ut.load(j, s), A2 = Ut.load(k, nb.fwd[j]), A3 = Ut.load(j, nb.fwd[k]), A4 = Ut.load(k, s);
            const Q A3s = qadj(A3), A4s = qadj(A4);
            atomic_add_link(Wb, L.V, j, s, qmul(Pb, qadj(qmul(qmul(A2, A3s), A4s))));
            atomic_add_link(Wb, L.V, k, nb.fwd[j], qmul(qmul(qadj(A1), Pb), qadj(qmul(A3s, A4s))));
            atomic_add_link(Wb, L.V, j, nb.fwd[k], qadj(qmul(qmul(qmul(qadj(A2), qadj(A1)), Pb), A4)));
            atomic_add_link(Wb, L.V, k, s, qadj(qmul(qadj(qmul(qmul(A1, A2), A3s)), Pb)));
        }
    }
}

// W_0 = exp(-i dt E_0) U: Ebar_0 += -dt vbar(Xbar = Wbar_0 U^*)
__global__ void k_adj_init_links(const double *__restrict__ Uinit, const double *__restrict__ E0,
                                 const double *__restrict__ W0_b, Lat L, double *__restrict__ E0_b) {
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    const LinkPlanes<G2, double> U{const_cast<double *>(Uinit), L.V}, Wb{const_cast<double *>(W0_b), L.V};
    const AlgPlanes<3, double> E{const_cast<double *>(E0), L.V}, Eb{E0_b, L.V};
    for (int i = 0; i < 3; i++) {
        double e[3], v[3], vb[3], eb[3];
        E.load_ro(i, s, e);
        for (int a = 0; a < 3; a++) v[a] = -L.dt * e[a];
        expi_adjoint(v, qmul(Wb.load(i, s), qadj(U.load(i, s))), vb);
        Eb.load(i, s, eb);
        for (int a = 0; a < 3; a++) eb[a] += -L.dt * vb[a];
        Eb.store(i, s, eb);
    }
}

// J (value, and tangent for duals) over the box
template <typename R>
__device__ __forceinline__ R energy_cell(const LinkPlanes<SU2<R>, R> &U0, const LinkPlanes<SU2<R>, R> &U1,
                                         const AlgPlanes<3, R> &E, const Lat &L, long s, const Nbr &nb) {
    using GG = SU2<R>;
    const R uf = R(1.0 / ((L.g * L.a[0]) * (L.g * L.a[0])));
    R en = R(0.0);
    for (int d = 0; d < 3; d++) {
        R e[3], b0[3], b1[3];
        E.load_ro(d, s, e);
        field_b<GG, R>(U0, L, s, nb, d, b0);
        field_b<GG, R>(U1, L, s, nb, d, b1);
        R e2 = R(0.0), bb = R(0.0);
        for (int a = 0; a < 3; a++) {
            e2 += e[a] * e[a];
            const R t = b0[a] + b1[a];
            bb += t * t;
        }
        en += (R(0.5) * e2 + R(0.25) * bb) * uf;
    }
    return en;
}

struct Obj {
    int kind;  // OPX_OBJ_ENERGY or OPX_OBJ_ANISOTROPY
    int dir;   // longitudinal direction of the anisotropy
    Box box;
};

// The per-cell terms of the objective: (a, b) = (energy density, 0) or (P_L, P_T)
template <typename R>
__device__ __forceinline__ void obj_cell(const LinkPlanes<SU2<R>, R> &U0, const LinkPlanes<SU2<R>, R> &U1,
                                         const AlgPlanes<3, R> &E, const Lat &L, long s, const Nbr &nb,
                                         const Obj &ob, R &a, R &b) {
    using GG = SU2<R>;
    if (ob.kind == OPX_OBJ_ENERGY) {
        a = energy_cell<R>(U0, U1, E, L, s, nb);
        b = R(0.0);
        return;
    }
    R eL = R(0.0), eT = R(0.0);
    for (int d = 0; d < 3; d++) {
        R e[3], b0[3], b1[3];
        E.load_ro(d, s, e);
        field_b<GG, R>(U0, L, s, nb, d, b0);
        field_b<GG, R>(U1, L, s, nb, d, b1);
        R e2 = R(0.0), bb = R(0.0);
        for (int q = 0; q < 3; q++) {
            e2 += e[q] * e[q];
            bb += b0[q] * b0[q] + b1[q] * b1[q];
        }
        const R t = (R(0.5) * e2 + R(0.25) * bb) * R(1.0 / ((L.g * L.a[d]) * (L.g * L.a[d])));
        if (d == ob.dir) eL += t; else eT += t;
    }
    a = eT - eL;
    b = eL;
}

// Box sums of a and b: values and (dual numbers) tangents
template <typename R>
__global__ void k_obj_box(const R *__restrict__ Wm, const R *__restrict__ Wn, const R *__restrict__ En, Lat L,
                          Obj ob, double *__restrict__ part) {
    const LinkPlanes<SU2<R>, R> U0{const_cast<R *>(Wm), L.V}, U1{const_cast<R *>(Wn), L.V};
    const AlgPlanes<3, R> E{const_cast<R *>(En), L.V};
    KSum acc[4] = {{0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}, {0.0, 0.0}};
    for (long s = (long)blockIdx.x * blockDim.x + threadIdx.x; s < L.V; s += (long)gridDim.x * blockDim.x) {
        int x[3];
        site_coords(L, s, x);
        if (!in_box(x, ob.box.lo, ob.box.hi)) continue;
        const Nbr nb = neighbours(L, s, x);
        R a, b;
        obj_cell<R>(U0, U1, E, L, s, nb, ob, a, b);
        two_sum_add(acc[0], value_of(a));
        two_sum_add(acc[1], tangent_of(a));
        two_sum_add(acc[2], value_of(b));
        two_sum_add(acc[3], tangent_of(b));
    }
    int q;
    KSum v = block_reduce<4>(acc, q);
    if (q >= 0) { part[2 * (blockIdx.x * 4 + q)] = v.s; part[2 * (blockIdx.x * 4 + q) + 1] = v.c; }
}

__global__ void k_obj_box_final(const double *__restrict__ part, int nb, double *__restrict__ out) {
    if (threadIdx.x >= 4) return;
    KSum v{0.0, 0.0};
    for (int b = 0; b < nb; b++) ksum_merge(v, KSum{part[2 * (b * 4 + threadIdx.x)], part[2 * (b * 4 + threadIdx.x) + 1]});
    out[threadIdx.x] = v.s + v.c;
}

// Cotangents of the anisotropy J = A / B with respect to E_N, W_{N-1} and W_N:
// dJ = (dA - J dB) / B, i.e. per direction the weight wT = 1/B (transverse) or
// wL = (-1 - J)/B (longitudinal) on d eps_j.
__global__ void k_adj_aniso(const double *__restrict__ Wm, const double *__restrict__ Wn,
                            const double *__restrict__ En, Lat L, Obj ob, double wT, double wL,
                            double *__restrict__ Wm_b, double *__restrict__ Wn_b, double *__restrict__ En_b) {
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    int x[3];
    site_coords(L, s, x);
    const AlgPlanes<3, double> E{const_cast<double *>(En), L.V}, Eb{En_b, L.V};
    if (!in_box(x, ob.box.lo, ob.box.hi)) {
        const double z[3] = {0, 0, 0};
        for (int d = 0; d < 3; d++) Eb.store(d, s, z);
        return;
    }
    const Nbr nb = neighbours(L, s, x);
    const LinkPlanes<G2, double> U0{const_cast<double *>(Wm), L.V}, U1{const_cast<double *>(Wn), L.V};
    for (int d = 0; d < 3; d++) {
        const double w = (d == ob.dir ? wL : wT) / ((L.g * L.a[d]) * (L.g * L.a[d]));
        double e[3], eb[3];
        E.load_ro(d, s, e);
        for (int a = 0; a < 3; a++) eb[a] = w * e[a];
        Eb.store(d, s, eb);
        const int j = (d + 1) % 3, k = (d + 2) % 3;
        const double f = L.a[d] / (L.a[j] * L.a[k]);
        for (int t = 0; t < 2; t++) {
            const LinkPlanes<G2, double> &Ut = t ? U1 : U0;
            double *Wb = t ? Wn_b : Wm_b;
            double bt[3];
            field_b<G2, double>(Ut, L, s, nb, d, bt);
            // d(w |B_t|^2 / 4)/dB_t = w B_t / 2; B = 2 f vec(P)
            Q Pb{{0.0, 0.0, 0.0, 0.0}};
            for (int a = 0; a < 3; a++) Pb.e[1 + a] = 2 * f * 0.5 * bt[a] * w;
            const Q A1 = Ut.load(j, s), A2 = Ut.load(k, nb.fwd[j]), A3 = Ut.load(j, nb.fwd[k]), A4 = Ut.load(k, s);
            const Q A3s = qadj(A3), A4s = qadj(A4);
            atomic_add_link(Wb, L.V, j, s, qmul(Pb, qadj(qmul(qmul(A2, A3s), A4s))));
            atomic_add_link(Wb, L.V, k, nb.fwd[j], qmul(qmul(qadj(A1), Pb), qadj(qmul(A3s, A4s))));
            atomic_add_link(Wb, L.V, j, nb.fwd[k], qadj(qmul(qmul(qmul(qadj(A2), qadj(A1)), Pb), A4)));
            atomic_add_link(Wb, L.V, k, s, qadj(qmul(qadj(qmul(qmul(A1, A2), A3s)), Pb)));
        }
    }
}

template <int NC, typename R, bool REUNIT>
__global__ void __launch_bounds__(128) k_step_plain(const R *__restrict__ U, R *__restrict__ E, R *__restrict__ Un, Lat L) {
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    update_site<NC, R, false, REUNIT>(U, E, nullptr, Un, L, s);
}

template <int NC, typename R>
__global__ void __launch_bounds__(128) k_links_plain(const R *__restrict__ U, const R *__restrict__ E, R *__restrict__ Un, Lat L) {
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    update_links_site<NC, R>(U, E, Un, L, s);
}

__global__ void k_make_dual(const double *__restrict__ v, const double *__restrict__ t, Dual *__restrict__ out, long n) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = Dual(v[k], t ? t[k] : 0.0);
}
__global__ void k_widen(const float *__restrict__ src, double *__restrict__ dst, long n) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dst[k] = (double)src[k];
}
__global__ void k_axpy_d(double *__restrict__ y, const double *__restrict__ x, double a, long n) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) y[k] += a * x[k];
}

}  // namespace opx


// ------------------------------------------------------------------ host side
using namespace opx;

namespace {

struct DevBuf {
    std::vector<void *> ptrs;
    bool ok = true;
    template <typename T> T *get(size_t n) {
        void *p = nullptr;
        if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) { ok = false; cudaGetLastError(); return nullptr; }
        ptrs.push_back(p);
        return (T *)p;
    }
    ~DevBuf() { for (void *p : ptrs) cudaFree(p); }
};

struct ObjArgs {
    Obj ob;
    int ok;
};

ObjArgs make_obj(const Ctx &c, int kind, int dir, const int *lo, const int *hi) {
    ObjArgs a{};
    a.ok = (kind == OPX_OBJ_ENERGY || kind == OPX_OBJ_ANISOTROPY) && (kind == OPX_OBJ_ENERGY || (dir >= 0 && dir < 3));
    a.ob.kind = kind;
    a.ob.dir = dir;
    long n = 1;
    for (int i = 0; i < 3; i++) {
        a.ob.box.lo[i] = lo ? lo[i] : 0;
        a.ob.box.hi[i] = hi ? hi[i] : c.L.n[i] - 1;
        if (a.ob.box.lo[i] < 0 || a.ob.box.hi[i] >= c.L.n[i] || a.ob.box.lo[i] > a.ob.box.hi[i]) a.ok = 0;
        n *= (a.ob.box.hi[i] - a.ob.box.lo[i] + 1);
    }
    a.ob.box.inv_n = 1.0 / (double)n;
    return a;
}

// handle fields in FP64 (a copy; the handle is not modified)
void widen_state(Ctx &c, double *U64, double *E64) {
    const long nU = link_elems(c.L.V, c.ng), nE = c.L.V * 3 * c.na;
    if (c.prec == OPX_F64) {
        cudaMemcpyAsync(U64, c.U, nU * 8, cudaMemcpyDeviceToDevice, c.stream);
        cudaMemcpyAsync(E64, c.E, nE * 8, cudaMemcpyDeviceToDevice, c.stream);
    } else {
        k_widen<<<grid_for(nU, 256), 256, 0, c.stream>>>((const float *)c.U, U64, nU);
        k_widen<<<grid_for(nE, 256), 256, 0, c.stream>>>((const float *)c.E, E64, nE);
        c.launches += 2;
    }
}

// J (and with dual numbers dJ) of the objective on (W_{N-1}, W_N, E_N); *A_B
// receives the box sums (A, B) of the values
template <typename R>
double objective_value(Ctx &c, const R *Wm, const R *Wn, const R *E, const Obj &ob, double *part, double *out4,
                       double *dJ, double *A_B = nullptr) {
    const int nb = 304;
    k_obj_box<R><<<nb, 256, 0, c.stream>>>(Wm, Wn, E, c.L, ob, part);
    k_obj_box_final<<<1, 32, 0, c.stream>>>(part, nb, out4);
    c.launches += 2;
    double h[4] = {0, 0, 0, 0};
    cudaMemcpyAsync(h, out4, 4 * sizeof(double), cudaMemcpyDeviceToHost, c.stream);
    cudaStreamSynchronize(c.stream);
    if (A_B) { A_B[0] = h[0]; A_B[1] = h[2]; }
    if (ob.kind == OPX_OBJ_ENERGY) {
        if (dJ) *dJ = h[1] * ob.box.inv_n;
        return h[0] * ob.box.inv_n;
    }
    if (dJ) *dJ = (h[1] * h[2] - h[0] * h[3]) / (h[2] * h[2]);
    return h[0] / h[2];
}

template <typename R>
void fwd_steps(Ctx &c, R *Wa, R *Wb, R *E, int n, R **last, R **prev) {
    R *cur = Wa, *nxt = Wb;
    for (int k = 0; k < n; k++) {
        k_step_plain<2, R, false><<<grid_for(c.L.V, 128), 128, 0, c.stream>>>(cur, E, nxt, c.L);
        c.launches++;
        std::swap(cur, nxt);
    }
    *last = cur;
    *prev = nxt;
}

int check_su2(Ctx &c, int nsteps, const char *where) {
    if (c.nc != 2) { c.err = std::string(where) + ": the differentiation form is provided for SU(2)"; return OPX_ERR_UNSUPPORTED; }
    if (nsteps < 1) { c.err = std::string(where) + ": nsteps must be >= 1"; return OPX_ERR_INVALID; }
    return OPX_OK;
}

int finish(Ctx &c, const char *where) {
    cudaError_t e = cudaStreamSynchronize(c.stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) { c.err = std::string(where) + ": " + cudaGetErrorString(e); return OPX_ERR_CUDA; }
    return OPX_OK;
}

// host [V][3][3] (link, direction, component) <-> device planes [3][3][V]
void to_planes(const double *h, long V, double *t) {
    for (long s = 0; s < V; s++)
        for (int d = 0; d < 3; d++)
            for (int a = 0; a < 3; a++) t[(d * 3 + a) * V + s] = h[(s * 3 + d) * 3 + a];
}

// The initial-E direction of an input direction: dE (host, [V][3][3] or NULL)
// plus divT K^+ drho (host, [V][3] or NULL), into dev (planes); U64 the
// handle's links in FP64.  Returns OPX_OK or an error status.
int input_direction(Ctx &c, const double *U64, const double *dE, const double *drho, double *dev, const char *where) {
    const long V = c.L.V, nE = V * 9, nr = V * 3;
    std::vector<double> t(nE, 0.0);
    if (dE) to_planes(dE, V, t.data());
    cudaMemcpyAsync(dev, t.data(), nE * 8, cudaMemcpyHostToDevice, c.stream);
    cudaStreamSynchronize(c.stream);
    if (!drho) return OPX_OK;
    DevBuf B;
    double *r = B.get<double>(nr), *mu = B.get<double>(nr);
    if (!B.ok) { c.err = std::string(where) + ": out of device memory"; return OPX_ERR_NOMEM; }
    std::vector<double> tr(nr);
    for (long s = 0; s < V; s++)
        for (int a = 0; a < 3; a++) tr[a * V + s] = drho[s * 3 + a];
    cudaMemcpyAsync(r, tr.data(), nr * 8, cudaMemcpyHostToDevice, c.stream);
    int rc = ic_covariant_solve(c, U64, r, mu, 1e-13, 20000, nullptr);
    if (rc) { c.err = std::string(where) + ": " + c.err; return rc; }
    ic_divT(c, U64, mu, dev, 1);
    return OPX_OK;
}

int objective_value_impl(Ctx &c, const ObjArgs &ar, int nsteps, const double *dE, const double *drho, double h,
                         double *J, const char *where) {
    const long V = c.L.V, nU = link_elems(V, 4), nE = V * 9;
    DevBuf B;
    double *U0 = B.get<double>(nU), *Wa = B.get<double>(nU), *Wb = B.get<double>(nU), *E = B.get<double>(nE);
    double *dEd = B.get<double>(nE), *part = B.get<double>(8 * 304), *out4 = B.get<double>(4);
    if (!B.ok) { c.err = std::string(where) + ": out of device memory"; return OPX_ERR_NOMEM; }
    widen_state(c, U0, E);
    if ((dE || drho) && h != 0.0) {
        int rc = input_direction(c, U0, dE, drho, dEd, where);
        if (rc) return rc;
        k_axpy_d<<<grid_for(nE, 256), 256, 0, c.stream>>>(E, dEd, h, nE);
        c.launches++;
    }
    k_links_plain<2, double><<<grid_for(V, 128), 128, 0, c.stream>>>(U0, E, Wa, c.L);
    c.launches++;
    double *last, *prev;
    fwd_steps<double>(c, Wa, Wb, E, nsteps, &last, &prev);
    *J = objective_value<double>(c, prev, last, E, ar.ob, part, out4, nullptr);
    return finish(c, where);
}

int objective_tangent_impl(Ctx &c, const ObjArgs &ar, int nsteps, const double *dE, const double *drho, double *J,
                           double *dJ, const char *where) {
    const long V = c.L.V, nU = link_elems(V, 4), nE = V * 9;
    DevBuf B;
    double *U0 = B.get<double>(nU), *E0 = B.get<double>(nE), *dEd = B.get<double>(nE);
    Dual *Ud = B.get<Dual>(nU), *Wa = B.get<Dual>(nU), *Wb = B.get<Dual>(nU), *Ed = B.get<Dual>(nE);
    double *part = B.get<double>(8 * 304), *out4 = B.get<double>(4);
    if (!B.ok) { c.err = std::string(where) + ": out of device memory"; return OPX_ERR_NOMEM; }
    widen_state(c, U0, E0);
    int rc = input_direction(c, U0, dE, drho, dEd, where);
    if (rc) return rc;
    k_make_dual<<<grid_for(nU, 256), 256, 0, c.stream>>>(U0, nullptr, Ud, nU);
    k_make_dual<<<grid_for(nE, 256), 256, 0, c.stream>>>(E0, dEd, Ed, nE);
    k_links_plain<2, Dual><<<grid_for(V, 128), 128, 0, c.stream>>>(Ud, Ed, Wa, c.L);
    c.launches += 3;
    Dual *last, *prev;
    fwd_steps<Dual>(c, Wa, Wb, Ed, nsteps, &last, &prev);
    *J = objective_value<Dual>(c, prev, last, Ed, ar.ob, part, out4, dJ);
    return finish(c, where);
}

int objective_gradient_impl(Ctx &c, const ObjArgs &ar, int nsteps, int ckpt, int wrt, double *J, double *grad,
                            size_t count, const char *where) {
    const long V = c.L.V, nU = link_elems(V, 4), nE = V * 9;
    if (ckpt < 1) { c.err = std::string(where) + ": ckpt must be >= 1"; return OPX_ERR_INVALID; }
    if (wrt != OPX_WRT_E && wrt != OPX_WRT_RHO) { c.err = std::string(where) + ": unknown input"; return OPX_ERR_INVALID; }
    const size_t want = wrt == OPX_WRT_E ? (size_t)nE : (size_t)V * 3;
    if (count != want) {
        c.err = std::string(where) + (wrt == OPX_WRT_E ? ": gradient must hold V*3*3 doubles" : ": gradient must hold V*3 doubles");
        return OPX_ERR_INVALID;
    }
    const int nseg = (nsteps + ckpt - 1) / ckpt;
    const int rs = c.prec == OPX_F64 ? 8 : 4;
    DevBuf B;
    // forward in the handle's precision
    char *Ur0 = B.get<char>(nU * rs), *Wra = B.get<char>(nU * rs), *Wrb = B.get<char>(nU * rs), *Er = B.get<char>(nE * rs);
    double *U64 = B.get<double>(nU), *E64 = B.get<double>(nE);
    std::vector<double *> ckW(nseg), ckE(nseg);
    for (int k = 0; k < nseg; k++) { ckW[k] = B.get<double>(nU); ckE[k] = B.get<double>(nE); }
    std::vector<double *> segW(ckpt + 1), segE(ckpt + 1);
    for (int m = 0; m <= ckpt; m++) { segW[m] = B.get<double>(nU); segE[m] = B.get<double>(nE); }
    double *Wbar[2] = {B.get<double>(nU), B.get<double>(nU)}, *Ebar[2] = {B.get<double>(nE), B.get<double>(nE)};
    double *Wm_b = B.get<double>(nU), *Sbar = B.get<double>(nU), *Uown = B.get<double>(nU);
    double *part = B.get<double>(8 * 304), *out4 = B.get<double>(4);
    if (!B.ok) { c.err = std::string(where) + ": out of device memory"; return OPX_ERR_NOMEM; }
    cudaMemcpyAsync(Ur0, c.U, nU * rs, cudaMemcpyDeviceToDevice, c.stream);
    cudaMemcpyAsync(Er, c.E, nE * rs, cudaMemcpyDeviceToDevice, c.stream);
    widen_state(c, U64, E64);
    const dim3 gs(grid_for(V, 128));
    auto store_ckpt = [&](int k, char *W) {
        if (c.prec == OPX_F64) {
            cudaMemcpyAsync(ckW[k], W, nU * 8, cudaMemcpyDeviceToDevice, c.stream);
            cudaMemcpyAsync(ckE[k], Er, nE * 8, cudaMemcpyDeviceToDevice, c.stream);
        } else {
            k_widen<<<grid_for(nU, 256), 256, 0, c.stream>>>((const float *)W, ckW[k], nU);
            k_widen<<<grid_for(nE, 256), 256, 0, c.stream>>>((const float *)Er, ckE[k], nE);
            c.launches += 2;
        }
    };
    char *cur = Wra, *nxt = Wrb;
    if (c.prec == OPX_F64) k_links_plain<2, double><<<gs, 128, 0, c.stream>>>((double *)Ur0, (double *)Er, (double *)cur, c.L);
    else k_links_plain<2, float><<<gs, 128, 0, c.stream>>>((float *)Ur0, (float *)Er, (float *)cur, c.L);
    c.launches++;
    store_ckpt(0, cur);
    for (int n = 1; n < nsteps; n++) {
        const bool reunit = c.prec == OPX_F32 && c.cfg.reunit_every > 0 && n % c.cfg.reunit_every == 0;
        if (c.prec == OPX_F64) k_step_plain<2, double, false><<<gs, 128, 0, c.stream>>>((double *)cur, (double *)Er, (double *)nxt, c.L);
        else if (reunit) k_step_plain<2, float, true><<<gs, 128, 0, c.stream>>>((float *)cur, (float *)Er, (float *)nxt, c.L);
        else k_step_plain<2, float, false><<<gs, 128, 0, c.stream>>>((float *)cur, (float *)Er, (float *)nxt, c.L);
        c.launches++;
        std::swap(cur, nxt);
        if (n % ckpt == 0) store_ckpt(n / ckpt, cur);
    }
    // reverse sweep, segment by segment, in FP64
    int wb = 0;
    double Jv = 0.0;
    for (int k = nseg - 1; k >= 0; k--) {
        const int start = k * ckpt, len = std::min(ckpt, nsteps - start);
        cudaMemcpyAsync(segW[0], ckW[k], nU * 8, cudaMemcpyDeviceToDevice, c.stream);
        cudaMemcpyAsync(segE[0], ckE[k], nE * 8, cudaMemcpyDeviceToDevice, c.stream);
        for (int m = 1; m <= len; m++) {
            cudaMemcpyAsync(segE[m], segE[m - 1], nE * 8, cudaMemcpyDeviceToDevice, c.stream);
            k_step_plain<2, double, false><<<gs, 128, 0, c.stream>>>(segW[m - 1], segE[m], segW[m], c.L);
            c.launches++;
        }
        if (k == nseg - 1) {
            double AB[2];
            Jv = objective_value<double>(c, segW[len - 1], segW[len], segE[len], ar.ob, part, out4, nullptr, AB);
            cudaMemsetAsync(Wm_b, 0, nU * 8, c.stream);
            cudaMemsetAsync(Wbar[wb], 0, nU * 8, c.stream);
            if (ar.ob.kind == OPX_OBJ_ENERGY) {
                k_adj_objective<<<gs, 128, 0, c.stream>>>(segW[len - 1], segW[len], segE[len], c.L, ar.ob.box, Wm_b,
                                                          Wbar[wb], Ebar[wb]);
            } else {
                const double wT = 1.0 / AB[1], wL = (-1.0 - Jv) / AB[1];
                k_adj_aniso<<<gs, 128, 0, c.stream>>>(segW[len - 1], segW[len], segE[len], c.L, ar.ob, wT, wL, Wm_b,
                                                      Wbar[wb], Ebar[wb]);
            }
            c.launches++;
        }
        for (int m = len; m >= 1; m--) {
            const int n = start + m;
            k_adj_local<<<gs, 128, 0, c.stream>>>(segW[m - 1], segE[m], Wbar[wb], Ebar[wb], c.L, Sbar, Uown,
                                                  Ebar[wb ^ 1]);
            k_adj_gather<<<gs, 128, 0, c.stream>>>(segW[m - 1], Sbar, Uown, c.L, Wbar[wb ^ 1]);
            c.launches += 2;
            if (n == nsteps) {
                k_axpy_d<<<grid_for(nU, 256), 256, 0, c.stream>>>(Wbar[wb ^ 1], Wm_b, 1.0, nU);
                c.launches++;
            }
            wb ^= 1;
        }
    }
    // W_0 = exp(-i dt E_0) U
    k_adj_init_links<<<gs, 128, 0, c.stream>>>(U64, E64, Wbar[wb], c.L, Ebar[wb]);
    c.launches++;
    int rc = finish(c, where);
    if (rc) return rc;
    if (wrt == OPX_WRT_E) {
        std::vector<double> t(nE);
        cudaMemcpyAsync(t.data(), Ebar[wb], nE * 8, cudaMemcpyDeviceToHost, c.stream);
        rc = finish(c, where);
        if (rc) return rc;
        for (long s = 0; s < V; s++)
            for (int d = 0; d < 3; d++)
                for (int a = 0; a < 3; a++) grad[(s * 3 + d) * 3 + a] = t[(d * 3 + a) * V + s];
    } else {
        // dJ/drho = K^+ div (dJ/dE_0)
        double *r = Sbar, *nu = Uown;  // site fields ([3][V]) in the free cotangent buffers
        ic_div(c, U64, Ebar[wb], r);
        rc = ic_covariant_solve(c, U64, r, nu, 1e-13, 20000, nullptr);
        if (rc) { c.err = std::string(where) + ": " + c.err; return rc; }
        std::vector<double> t(V * 3);
        cudaMemcpyAsync(t.data(), nu, V * 3 * 8, cudaMemcpyDeviceToHost, c.stream);
        rc = finish(c, where);
        if (rc) return rc;
        for (long s = 0; s < V; s++)
            for (int a = 0; a < 3; a++) grad[s * 3 + a] = t[a * V + s];
    }
    *J = Jv;
    return OPX_OK;
}

}  // namespace

extern "C" {

int opx_objective_value(opx_ctx *ctx, const opx_objective *obj, int nsteps, const double *dE, const double *drho,
                        double h, double *J) {
    if (!ctx || !obj || !J) return OPX_ERR_INVALID;
    Ctx &c = ctx_of(ctx);
    int rc = check_su2(c, nsteps, "opx_objective_value");
    if (rc) return rc;
    ObjArgs ar = make_obj(c, obj->kind, obj->direction, obj->lo, obj->hi);
    if (!ar.ok) { c.err = "opx_objective_value: unknown objective or box outside the lattice"; return OPX_ERR_INVALID; }
    return objective_value_impl(c, ar, nsteps, dE, drho, h, J, "opx_objective_value");
}

int opx_objective_tangent(opx_ctx *ctx, const opx_objective *obj, int nsteps, const double *dE, const double *drho,
                          double *J, double *dJ) {
    if (!ctx || !obj || !J || !dJ || (!dE && !drho)) return OPX_ERR_INVALID;
    Ctx &c = ctx_of(ctx);
    int rc = check_su2(c, nsteps, "opx_objective_tangent");
    if (rc) return rc;
    ObjArgs ar = make_obj(c, obj->kind, obj->direction, obj->lo, obj->hi);
    if (!ar.ok) { c.err = "opx_objective_tangent: unknown objective or box outside the lattice"; return OPX_ERR_INVALID; }
    return objective_tangent_impl(c, ar, nsteps, dE, drho, J, dJ, "opx_objective_tangent");
}

int opx_objective_gradient(opx_ctx *ctx, const opx_objective *obj, int nsteps, int ckpt, int wrt, double *J,
                           double *grad, size_t count) {
    if (!ctx || !obj || !J || !grad) return OPX_ERR_INVALID;
    Ctx &c = ctx_of(ctx);
    int rc = check_su2(c, nsteps, "opx_objective_gradient");
    if (rc) return rc;
    ObjArgs ar = make_obj(c, obj->kind, obj->direction, obj->lo, obj->hi);
    if (!ar.ok) { c.err = "opx_objective_gradient: unknown objective or box outside the lattice"; return OPX_ERR_INVALID; }
    return objective_gradient_impl(c, ar, nsteps, ckpt, wrt, J, grad, count, "opx_objective_gradient");
}

int opx_energy_objective(opx_ctx *ctx, int nsteps, const int *lo, const int *hi, const double *dE, double h,
                         double *J) {
    if (!ctx || !J) return OPX_ERR_INVALID;
    Ctx &c = ctx_of(ctx);
    int rc = check_su2(c, nsteps, "opx_energy_objective");
    if (rc) return rc;
    ObjArgs ar = make_obj(c, OPX_OBJ_ENERGY, 0, lo, hi);
    if (!ar.ok) { c.err = "opx_energy_objective: box outside the lattice"; return OPX_ERR_INVALID; }
    return objective_value_impl(c, ar, nsteps, dE, nullptr, h, J, "opx_energy_objective");
}

int opx_energy_tangent(opx_ctx *ctx, int nsteps, const int *lo, const int *hi, const double *dE, double *J,
                       double *dJ) {
    if (!ctx || !J || !dJ || !dE) return OPX_ERR_INVALID;
    Ctx &c = ctx_of(ctx);
    int rc = check_su2(c, nsteps, "opx_energy_tangent");
    if (rc) return rc;
    ObjArgs ar = make_obj(c, OPX_OBJ_ENERGY, 0, lo, hi);
    if (!ar.ok) { c.err = "opx_energy_tangent: box outside the lattice"; return OPX_ERR_INVALID; }
    return objective_tangent_impl(c, ar, nsteps, dE, nullptr, J, dJ, "opx_energy_tangent");
}

int opx_energy_gradient(opx_ctx *ctx, int nsteps, int ckpt, const int *lo, const int *hi, double *J, double *grad,
                        size_t count) {
    if (!ctx || !J || !grad) return OPX_ERR_INVALID;
    Ctx &c = ctx_of(ctx);
    int rc = check_su2(c, nsteps, "opx_energy_gradient");
    if (rc) return rc;
    ObjArgs ar = make_obj(c, OPX_OBJ_ENERGY, 0, lo, hi);
    if (!ar.ok) { c.err = "opx_energy_gradient: box outside the lattice"; return OPX_ERR_INVALID; }
    return objective_gradient_impl(c, ar, nsteps, ckpt, OPX_WRT_E, J, grad, count, "opx_energy_gradient");
}

}  // extern "C"
