// field_kernels.cu -- the temporal-gauge leapfrog on the device.
//
//   k_update_grid : FastTYMSolver.CombinedUpdate (physics/fields/FastTYMSolver.java:40-63)
//                   with Grid.getStapleSum (physics/grid/Grid.java:675-696):
//       E_i(x) += dt proj(U_i(x) S_i(x)) - g a_i dt J_i(x)
//       Unext_i(x) = exp(-i dt E_i(x)) U_i(x)
//   k_update_links: FastTYMSolver.UpdateLinks (:65-84): Unext = exp(-i dt E) U
//   k_reunit      : re-unitarisation of FP32 links (no counterpart in the reference)
//
// One thread owns one site and updates its three links, so U_i(x) and the
// site's own links are read once and reused for all staples.  Compulsory HBM
// traffic per link update: read U_i(x), E_i(x) [, J_i(x)], write E_i(x),
// Unext_i(x); the 12 neighbour links of the staples are served from L1/L2
// (consecutive blocks cover consecutive sites, so the +-1 planes of dimension
// 0 are resident in L2 while a block works on its plane).
#include "internal.h"

namespace opx {

int grid_for(long n, int block) { return (int)((n + block - 1) / block); }

// Register and instruction budget: the SU(3) products are unrolled (108 FMA
// each) but the loops over the link direction i and the staple plane j stay
// rolled, with runtime indices resolved by selects, so that the kernel body
// fits the instruction cache and a thread keeps one staple in flight.
template <int NC, typename R> struct UpdateBounds { static constexpr int minb = 4; };
template <> struct UpdateBounds<3, float> { static constexpr int minb = 4; };
template <> struct UpdateBounds<3, double> { static constexpr int minb = 3; };

template <int NC, typename R, bool HAS_J, bool REUNIT>
__global__ void __launch_bounds__(128, UpdateBounds<NC, R>::minb)
k_update_grid(const R *__restrict__ U, R *__restrict__ E, const R *__restrict__ J, R *__restrict__ Unext,
              const uint8_t *__restrict__ active, Lat L) {
    using G = typename GroupOf<NC, R>::T;
    using M = typename G::M;
    constexpr int NA = G::NA;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    if (active && !active[s]) return;  // Cell.isActive gate (FastTYMSolver.java:51)
    int x[3];
    site_coords(L, s, x);
    const int x0 = x[0], x1 = x[1], x2 = x[2];
    const LinkPlanes<G, R> Up{const_cast<R *>(U), L.V};
    const LinkPlanes<G, R> Un{Unext, L.V};
    const AlgPlanes<NA, R> Ep{E, L.V};
    const AlgPlanes<NA, R> Jp{const_cast<R *>(J), L.V};
    const R dt = R(L.dt);

#pragma unroll 1
    for (int i = 0; i < 3; i++) {
        const int xi = pick(x0, x1, x2, i);
        const long s_pi = shift_d(L, s, xi, i, +1);  // x + i
        M S = G::zero();
#pragma unroll 1
        for (int jj = 1; jj < 3; jj++) {
            const int j = i + jj >= 3 ? i + jj - 3 : i + jj;
            const int xj = pick(x0, x1, x2, j);
            const long s_pj = shift_d(L, s, xj, j, +1);     // x + j
            const long s_mj = shift_d(L, s, xj, j, -1);     // x - j
            const long s_pimj = shift_d(L, s_pi, xj, j, -1);  // x + i - j
            // U_j(x+i) U_i(x+j)^dagger U_j(x)^dagger
            M F = G::mul_adj(G::mul_adj(Up.load(j, s_pi), Up.load(i, s_pj)), Up.load(j, s));
            // (U_i(x-j) U_j(x+i-j))^dagger U_j(x-j)
            const M C = G::mul(Up.load(i, s_mj), Up.load(j, s_pimj));
            G::add(F, G::adj_mul(C, Up.load(j, s_mj)));
            const R aj = R(pickd(L.a[0], L.a[1], L.a[2], j));
            G::scale(F, R(1) / (aj * aj));
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
            const R jf = R(-(L.g * pickd(L.a[0], L.a[1], L.a[2], i)) * L.dt);
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

template <int NC, typename R>
__global__ void __launch_bounds__(128) k_update_links(const R *__restrict__ U, const R *__restrict__ E,
                                                      R *__restrict__ Unext, const uint8_t *__restrict__ active,
                                                      Lat L) {
    using G = typename GroupOf<NC, R>::T;
    constexpr int NA = G::NA;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    if (active && !active[s]) return;
    const LinkPlanes<G, R> Up{const_cast<R *>(U), L.V};
    const LinkPlanes<G, R> Un{Unext, L.V};
    const AlgPlanes<NA, R> Ep{const_cast<R *>(E), L.V};
    for (int k = 0; k < 3; k++) {
        R e[NA], v[NA];
        Ep.load_ro(k, s, e);
#pragma unroll
        for (int a = 0; a < NA; a++) v[a] = -R(L.dt) * e[a];
        Un.store(k, s, G::mul(G::expi(v), Up.load(k, s)));
    }
}

template <int NC, typename R>
__global__ void k_reunit(R *__restrict__ U, Lat L) {
    using G = typename GroupOf<NC, R>::T;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    const LinkPlanes<G, R> Up{U, L.V};
    for (int k = 0; k < 3; k++) {
        auto m = Up.load(k, s);
        G::reunit(m);
        Up.store(k, s, m);
    }
}

template <int NC, typename R>
static void update_grid_t(Ctx &c, bool reunit) {
    const int B = 128;
    dim3 grid(grid_for(c.L.V, B));
    const R *U = (const R *)c.U;
    R *E = (R *)c.E, *Un = (R *)c.Unext;
    const R *J = (const R *)c.J;
    if (c.j_nonzero) {
        if (reunit) k_update_grid<NC, R, true, true><<<grid, B, 0, c.stream>>>(U, E, J, Un, c.active, c.L);
        else k_update_grid<NC, R, true, false><<<grid, B, 0, c.stream>>>(U, E, J, Un, c.active, c.L);
    } else {
        if (reunit) k_update_grid<NC, R, false, true><<<grid, B, 0, c.stream>>>(U, E, J, Un, c.active, c.L);
        else k_update_grid<NC, R, false, false><<<grid, B, 0, c.stream>>>(U, E, J, Un, c.active, c.L);
    }
    c.launches++;
}

void launch_update_grid(Ctx &c, bool reunit) {
    if (c.nc == 2) {
        if (c.prec == OPX_F64) update_grid_t<2, double>(c, reunit); else update_grid_t<2, float>(c, reunit);
    } else {
        if (c.prec == OPX_F64) update_grid_t<3, double>(c, reunit); else update_grid_t<3, float>(c, reunit);
    }
}

template <int NC, typename R>
static void update_links_t(Ctx &c) {
    const int B = 128;
    k_update_links<NC, R><<<grid_for(c.L.V, B), B, 0, c.stream>>>((const R *)c.U, (const R *)c.E,
                                                                   (R *)c.Unext, c.active, c.L);
    c.launches++;
}

void launch_update_links(Ctx &c) {
    if (c.nc == 2) {
        if (c.prec == OPX_F64) update_links_t<2, double>(c); else update_links_t<2, float>(c);
    } else {
        if (c.prec == OPX_F64) update_links_t<3, double>(c); else update_links_t<3, float>(c);
    }
}

template <int NC, typename R>
static void reunit_t(Ctx &c, void *links) {
    const int B = 256;
    k_reunit<NC, R><<<grid_for(c.L.V, B), B, 0, c.stream>>>((R *)links, c.L);
    c.launches++;
}

void launch_reunit(Ctx &c, void *links) {
    if (c.nc == 2) {
        if (c.prec == OPX_F64) reunit_t<2, double>(c, links); else reunit_t<2, float>(c, links);
    } else {
        if (c.prec == OPX_F64) reunit_t<3, double>(c, links); else reunit_t<3, float>(c, links);
    }
}

}  // namespace opx
