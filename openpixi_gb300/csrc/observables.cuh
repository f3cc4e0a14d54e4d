// observables.cuh -- per-site field-strength and Gauss-law helpers shared by
// the reduction kernels.
#pragma once
#include "ksum.cuh"
#include "lattice.cuh"

namespace opx {

// B_d(x) = proj(P_jk(x)) a_d / (a_j a_k) with (d, j, k) cyclic (Grid.getB, Grid.java:901-920)
template <class G, typename R>
__device__ __forceinline__ void field_b(const LinkPlanes<G, R> &Up, const Lat &L, long s, const Nbr &nb,
                                        int d, R *b) {
    const int j = (d + 1) % 3, k = (d + 2) % 3;
    // U_j(x) U_k(x+j) U_j(x+k)^dagger U_k(x)^dagger (Grid.getPlaquette, Grid.java:609-642)
    auto P = G::mul_adj(G::mul_adj(G::mul(Up.load(j, s), Up.load(k, nb.fwd[j])), Up.load(j, nb.fwd[k])),
                        Up.load(k, s));
    G::proj(P, b);
    const R f = LatR<R>::bfac(L, d);
#pragma unroll
    for (int a = 0; a < G::NA; a++) b[a] *= f;
}

// G(x) = sum_i [E_i(x) - U_i(x-i)^dagger E_i(x-i) U_i(x-i)] / (a_i g a_i) - rho(x)
template <class G, typename R>
__device__ __forceinline__ void gauss_site(const LinkPlanes<G, R> &Up, const AlgPlanes<G::NA, R> &Ep,
                                           const R *rho, const Lat &L, long s, const Nbr &nb, R *gs) {
    constexpr int NA = G::NA;
#pragma unroll
    for (int a = 0; a < NA; a++) gs[a] = R(0);
#pragma unroll
    for (int i = 0; i < 3; i++) {
        R e0[NA], e1[NA], t[NA];
        Ep.load_ro(i, s, e0);
        Ep.load_ro(i, nb.bwd[i], e1);
        G::act(e1, G::adj(Up.load(i, nb.bwd[i])), t);
        const R f = LatR<R>::gfac(L, i);
#pragma unroll
        for (int a = 0; a < NA; a++) gs[a] += (e0[a] - t[a]) * f;
    }
    if (rho) {
#pragma unroll
        for (int a = 0; a < NA; a++) gs[a] -= __ldg(rho + (long)a * L.V + s);
    }
}

template <typename R, int NA>
__device__ __forceinline__ double sq(const R *x) {
    double s = 0.0;
#pragma unroll
    for (int a = 0; a < NA; a++) s += (double)x[a] * (double)x[a];
    return s;
}
constexpr int NQ = 8;  // E2[3], B2[3], G2, rho2

// Sum of squares in the storage precision (the per-site value the reference
// forms), widened once.
template <typename R, int NA>
__device__ __forceinline__ double sqr(const R *x) {
    R s = R(0);
#pragma unroll
    for (int a = 0; a < NA; a++) s += x[a] * x[a];
    return (double)s;
}

// Per-thread compensated FP64 sums of the BulkQuantities columns over the sites
// first, first + stride, ... (FieldMeasurements EFieldSquared/BFieldSquared/
// GaussLaw/TotalChargeSquared, physics/measurements/FieldMeasurements.java:68-231).
// Runs of 32 sites are summed plainly in FP64 and folded into the compensated
// sums, so the error stays at the compensated level while the FP64 work per
// site is one addition per column.
template <int NC, typename R>
__device__ __forceinline__ void bulk_accumulate(const R *__restrict__ U, const R *__restrict__ Unext,
                                                const R *__restrict__ E, const R *__restrict__ rho,
                                                const uint8_t *__restrict__ eval, const Lat &L, KSum *acc,
                                                long first, long stride) {
    using G = typename GroupOf<NC, R>::T;
    constexpr int NA = G::NA;
    const LinkPlanes<G, R> Up{const_cast<R *>(U), L.V}, Unp{const_cast<R *>(Unext), L.V};
    const AlgPlanes<NA, R> Ep{const_cast<R *>(E), L.V};
#pragma unroll
    for (int q = 0; q < NQ; q++) acc[q] = KSum{0.0, 0.0};
    double p[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) p[q] = 0.0;
    int run = 0;
    for (long s = first; s < L.V; s += stride) {
        if (eval && !eval[s]) continue;
        int x[3];
        site_coords(L, s, x);
        const Nbr nb = neighbours(L, s, x);
#pragma unroll 1
        for (int i = 0; i < 3; i++) {
            R e[NA];
            Ep.load_ro(i, s, e);
            const double ev = sqr<R, NA>(e);
            R b0[NA], b1[NA];
            field_b<G, R>(Up, L, s, nb, i, b0);
            field_b<G, R>(Unp, L, s, nb, i, b1);
            const double bv = sqr<R, NA>(b0) + sqr<R, NA>(b1);
            if (i == 0) { p[0] += ev; p[3] += bv; }
            else if (i == 1) { p[1] += ev; p[4] += bv; }
            else { p[2] += ev; p[5] += bv; }
        }
        R gs[NA];
        gauss_site<G, R>(Up, Ep, rho, L, s, nb, gs);
        p[6] += sqr<R, NA>(gs);
        if (rho) {
            R r[NA];
#pragma unroll
            for (int a = 0; a < NA; a++) r[a] = __ldg(rho + (long)a * L.V + s);
            p[7] += sqr<R, NA>(r);
        }
        if (++run == 32) {
#pragma unroll
            for (int q = 0; q < NQ; q++) { two_sum_add(acc[q], p[q]); p[q] = 0.0; }
            run = 0;
        }
    }
#pragma unroll
    for (int q = 0; q < NQ; q++) two_sum_add(acc[q], p[q]);
    // the constant unit factors (g a_i)^-2, and 1/2 for the U / Unext average of B^2
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const double uf = 1.0 / ((L.g * L.a[i]) * (L.g * L.a[i]));
        acc[i].s *= uf; acc[i].c *= uf;
        acc[3 + i].s *= 0.5 * uf; acc[3 + i].c *= 0.5 * uf;
    }
}

}  // namespace opx
