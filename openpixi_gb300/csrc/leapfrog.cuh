// leapfrog.cuh -- one site of the temporal-gauge leapfrog, shared by the
// single-lattice kernel (field_kernels.cu) and the batched persistent kernel
// (batch_kernels.cu).
//
// FastTYMSolver.CombinedUpdate (physics/fields/FastTYMSolver.java:40-63) with
// Grid.getStapleSum (physics/grid/Grid.java:675-696):
//     E_i(x) += dt proj(U_i(x) S_i(x)) - g a_i dt J_i(x)
//     Unext_i(x) = exp(-i dt E_i(x)) U_i(x)
//
// Register and instruction budget: the SU(3) products are unrolled (108 FMA
// each) but the loops over the link direction i and the staple plane j stay
// rolled, with runtime indices resolved by selects, so that the body fits the
// instruction cache and a thread keeps one staple in flight.
#pragma once
#include "lattice.cuh"

namespace opx {

// I is the type of the site and element offsets: int where they fit (the
// 64-bit divisions and address arithmetic of long cost issue slots).
template <int NC, typename R, bool HAS_J, bool REUNIT, typename I = long>
__device__ __forceinline__ void update_site(const R *__restrict__ U, R *__restrict__ E, const R *__restrict__ J,
                                            R *__restrict__ Unext, const Lat &L, I s) {
    using G = typename GroupOf<NC, R>::T;
    using M = typename G::M;
    constexpr int NA = G::NA;
    int x[3];
    site_coords<I>(L, s, x);
    const Deltas<I> D = deltas<I>(L, x);
    const LinkPlanes<G, R, I> Up{const_cast<R *>(U), (I)L.V};
    const LinkPlanes<G, R, I> Un{Unext, (I)L.V};
    const AlgPlanes<NA, R, I> Ep{E, (I)L.V};
    const AlgPlanes<NA, R, I> Jp{const_cast<R *>(J), (I)L.V};
    const R dt = LatR<R>::dt(L);

#pragma unroll 1
    for (int i = 0; i < 3; i++) {
        const I s_pi = s + D.f(i);  // x + i
        M S = G::zero();
#pragma unroll 1
        for (int jj = 1; jj < 3; jj++) {
            const int j = i + jj >= 3 ? i + jj - 3 : i + jj;
            const I bj = D.b(j);
            const I s_pj = s + D.f(j);  // x + j
            const I s_mj = s + bj;      // x - j
            const I s_pimj = s_pi + bj; // x + i - j
            // U_j(x+i) U_i(x+j)^dagger U_j(x)^dagger
            M F = G::mul_adj(G::mul_adj(Up.load(j, s_pi), Up.load(i, s_pj)), Up.load(j, s));
            // (U_i(x-j) U_j(x+i-j))^dagger U_j(x-j)
            const M C = G::mul(Up.load(i, s_mj), Up.load(j, s_pimj));
            G::add(F, G::adj_mul(C, Up.load(j, s_mj)));
            G::scale(F, LatR<R>::inva2(L, j));
            G::add(S, F);
        }
        const M Ui = Up.load(i, s);
        R pr[NA], e[NA];
        G::proj(G::mul(Ui, S), pr);
        Ep.load(i, s, e);
#pragma unroll
        for (int a = 0; a < NA; a++) e[a] += pr[a] * dt;
        if (HAS_J) {
            R jv[NA];
            Jp.load_ro(i, s, jv);
            const R jf = LatR<R>::jfac(L, i);
#pragma unroll
            for (int a = 0; a < NA; a++) e[a] += jv[a] * jf;
        }
        Ep.store(i, s, e);
        R v[NA];
#pragma unroll
        for (int a = 0; a < NA; a++) v[a] = -dt * e[a];
        M Vn = G::mul(G::expi(v), Ui);
        if (REUNIT) G::reunit(Vn);
        Un.store(i, s, Vn);
    }
}

// SU(2): the same update with the staple sums of all three links formed plane
// by plane, so that the two forward staples of a plane share one product:
// with T = U_j(x+i) U_i(x+j)^dagger, link i's forward staple is T U_j(x)^dagger
// and link j's is T^dagger U_i(x)^dagger (21 instead of 24 quaternion products
// per site; the SU(2) state of three sums fits in registers).  Each link's sum
// receives its planes in the order of getStapleSum (j ascending), forward plus
// backward staple scaled by 1/a_j^2, as update_site forms it.
template <typename R, bool HAS_J, bool REUNIT, typename I = long>
__device__ __forceinline__ void update_site_su2_planes(const R *__restrict__ U, R *__restrict__ E,
                                                       const R *__restrict__ J, R *__restrict__ Unext, const Lat &L,
                                                       I s) {
    using G = SU2<R>;
    using M = typename G::M;
    int x[3];
    site_coords<I>(L, s, x);
    const Deltas<I> D = deltas<I>(L, x);
    const LinkPlanes<G, R, I> Up{const_cast<R *>(U), (I)L.V};
    const LinkPlanes<G, R, I> Un{Unext, (I)L.V};
    const AlgPlanes<3, R, I> Ep{E, (I)L.V};
    const AlgPlanes<3, R, I> Jp{const_cast<R *>(J), (I)L.V};
    const R dt = LatR<R>::dt(L);
    M S0 = G::zero(), S1 = G::zero(), S2 = G::zero();
#pragma unroll
    for (int pl = 0; pl < 3; pl++) {
        const int i = pl == 2 ? 1 : 0, j = pl == 0 ? 1 : 2;
        const I pi = s + D.f(i), pj = s + D.f(j), mi = s + D.b(i), mj = s + D.b(j);
        const M T = G::mul_adj(Up.load(j, pi), Up.load(i, pj));
        M Fi = G::mul_adj(T, Up.load(j, s));
        M Fj = G::mul_adj(G::adj(T), Up.load(i, s));
        // (U_i(x-j) U_j(x+i-j))^dagger U_j(x-j) and (U_j(x-i) U_i(x+j-i))^dagger U_i(x-i)
        G::add(Fi, G::adj_mul(G::mul(Up.load(i, mj), Up.load(j, pi + D.b(j))), Up.load(j, mj)));
        G::add(Fj, G::adj_mul(G::mul(Up.load(j, mi), Up.load(i, pj + D.b(i))), Up.load(i, mi)));
        G::scale(Fi, LatR<R>::inva2(L, j));
        G::scale(Fj, LatR<R>::inva2(L, i));
        if (pl == 0) { G::add(S0, Fi); G::add(S1, Fj); }
        else if (pl == 1) { G::add(S0, Fi); G::add(S2, Fj); }
        else { G::add(S1, Fi); G::add(S2, Fj); }
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const M &S = i == 0 ? S0 : (i == 1 ? S1 : S2);
        const M Ui = Up.load(i, s);
        R pr[3], e[3];
        G::proj(G::mul(Ui, S), pr);
        Ep.load(i, s, e);
#pragma unroll
        for (int a = 0; a < 3; a++) e[a] += pr[a] * dt;
        if (HAS_J) {
            R jv[3];
            Jp.load_ro(i, s, jv);
            const R jf = LatR<R>::jfac(L, i);
#pragma unroll
            for (int a = 0; a < 3; a++) e[a] += jv[a] * jf;
        }
        Ep.store(i, s, e);
        R v[3];
#pragma unroll
        for (int a = 0; a < 3; a++) v[a] = -dt * e[a];
        M Vn = G::mul(G::expi(v), Ui);
        if (REUNIT) G::reunit(Vn);
        Un.store(i, s, Vn);
    }
}

// FastTYMSolver.UpdateLinks (:65-84): Unext = exp(-i dt E) U at one site
template <int NC, typename R>
__device__ __forceinline__ void update_links_site(const R *__restrict__ U, const R *__restrict__ E,
                                                  R *__restrict__ Unext, const Lat &L, long s) {
    using G = typename GroupOf<NC, R>::T;
    constexpr int NA = G::NA;
    const LinkPlanes<G, R> Up{const_cast<R *>(U), L.V};
    const LinkPlanes<G, R> Un{Unext, L.V};
    const AlgPlanes<NA, R> Ep{const_cast<R *>(E), L.V};
#pragma unroll 1
    for (int k = 0; k < 3; k++) {
        R e[NA], v[NA];
        Ep.load_ro(k, s, e);
#pragma unroll
        for (int a = 0; a < NA; a++) v[a] = -LatR<R>::dt(L) * e[a];
        Un.store(k, s, G::mul(G::expi(v), Up.load(k, s)));
    }
}

}  // namespace opx
