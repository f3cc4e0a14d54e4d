// field_kernels.cu -- the temporal-gauge leapfrog on the device.
//
//   k_update_grid : FastTYMSolver.CombinedUpdate (physics/fields/FastTYMSolver.java:40-63)
//                   with Grid.getStapleSum (physics/grid/Grid.java:675-696):
//       E_i(x) += dt proj(U_i(x) S_i(x)) - g a_i dt J_i(x)
//       Unext_i(x) = exp(-i dt E_i(x)) U_i(x)
//   k_update_links: FastTYMSolver.UpdateLinks (:65-84): Unext = exp(-i dt E) U
//   k_reunit      : re-unitarisation of FP32 links (no counterpart in the reference)
//
// The per-site arithmetic is in leapfrog.cuh.  One thread owns one site and updates its three links, so U_i(x) and the
// site's own links are read once and reused for all staples.  Compulsory HBM
// traffic per link update: read U_i(x), E_i(x) [, J_i(x)], write E_i(x),
// Unext_i(x); the 12 neighbour links of the staples are served from L1/L2
// (consecutive blocks cover consecutive sites, so the +-1 planes of dimension
// 0 are resident in L2 while a block works on its plane).
#include "internal.h"
#include "leapfrog.cuh"
#include "su3_pair.cuh"

namespace opx {

int grid_for(long n, int block) { return (int)((n + block - 1) / block); }

template <int NC, typename R> struct UpdateBounds { static constexpr int minb = 4; };
template <> struct UpdateBounds<3, double> { static constexpr int minb = 3; };

template <int NC, typename R, bool HAS_J, bool REUNIT>
__global__ void __launch_bounds__(128, UpdateBounds<NC, R>::minb)
k_update_grid(const R *__restrict__ U, R *__restrict__ E, const R *__restrict__ J, R *__restrict__ Unext,
              const uint8_t *__restrict__ active, Lat L) {
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    if (active && !active[s]) return;  // Cell.isActive gate (FastTYMSolver.java:51)
    update_site<NC, R, HAS_J, REUNIT>(U, E, J, Unext, L, s);
}

// SU(3) FP32: two sites per thread in paired FP32 instructions.  Warp w
// covers sites [64 w, 64 w + 64): lane l takes site 64 w + l and the site 32
// further, so both halves of a warp read whole warp-sized link blocks.
// I = int when every link offset fits in 32 bits.
template <typename I, bool HAS_J, bool REUNIT>
__global__ void __launch_bounds__(128, 3)
k_update_grid_su3f_pair(const float *__restrict__ U, float *__restrict__ E, const float *__restrict__ J,
                        float *__restrict__ Unext, const uint8_t *__restrict__ active, Lat L) {
    const I t = (I)blockIdx.x * (I)blockDim.x + (I)threadIdx.x;
    const I sa = ((t >> 5) << 6) + (t & 31);
    if (sa >= (I)L.V) return;
    I sb = sa + 32;
    bool vb = sb < (I)L.V;
    if (!vb) sb = sa;
    const bool va = !active || active[sa];
    vb = vb && (!active || active[sb]);
    if (!va && !vb) return;  // Cell.isActive gate (FastTYMSolver.java:51)
    update_site_pair<I, HAS_J, REUNIT>(U, E, J, Unext, L, sa, sb, va, vb);
}

template <int NC, typename R>
__global__ void __launch_bounds__(128) k_update_links(const R *__restrict__ U, const R *__restrict__ E,
                                                      R *__restrict__ Unext, const uint8_t *__restrict__ active,
                                                      Lat L) {
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    if (active && !active[s]) return;
    update_links_site<NC, R>(U, E, Unext, L, s);
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

template <typename I>
static void update_grid_su3f_pair_i(Ctx &c, bool reunit) {
    const int B = 128;
    const long threads = ((c.L.V + 63) / 64) * 32;
    dim3 grid(grid_for(threads, B));
    const float *U = (const float *)c.U, *J = (const float *)c.J;
    float *E = (float *)c.E, *Un = (float *)c.Unext;
    if (c.j_nonzero) {
        if (reunit) k_update_grid_su3f_pair<I, true, true><<<grid, B, 0, c.stream>>>(U, E, J, Un, c.active, c.L);
        else k_update_grid_su3f_pair<I, true, false><<<grid, B, 0, c.stream>>>(U, E, J, Un, c.active, c.L);
    } else {
        if (reunit) k_update_grid_su3f_pair<I, false, true><<<grid, B, 0, c.stream>>>(U, E, J, Un, c.active, c.L);
        else k_update_grid_su3f_pair<I, false, false><<<grid, B, 0, c.stream>>>(U, E, J, Un, c.active, c.L);
    }
    c.launches++;
}

static void update_grid_su3f_pair(Ctx &c, bool reunit) {
    // 32-bit offsets while the largest link offset (3 blocks x 576 floats) fits
    if (link_elems(c.L.V, 18) < (1L << 31) - 64) update_grid_su3f_pair_i<int>(c, reunit);
    else update_grid_su3f_pair_i<long>(c, reunit);
}

template <int NC, typename R>
static void update_grid_t(Ctx &c, bool reunit) {
    if (NC == 3 && sizeof(R) == 4 && c.pair_kernel) {
        update_grid_su3f_pair(c, reunit);
        return;
    }
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
