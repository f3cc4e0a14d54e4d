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
#include <algorithm>
#include <cstdlib>

#include "internal.h"
#include "leapfrog.cuh"
#include "su3_log.cuh"
#include "su3_pair.cuh"
#include "su3_stream.cuh"

namespace opx {

int grid_for(long n, int block) { return (int)((n + block - 1) / block); }

template <int NC, typename R> struct UpdateBounds { static constexpr int minb = 4; };
template <> struct UpdateBounds<3, double> { static constexpr int minb = 3; };
// SU(2) FP32 is latency-bound on its link loads: the plane-by-plane staple sums
// at 8 blocks per SM (64 registers) take a 128^3 step in 0.081 ms (0.085 ms
// for the per-link sums at 12 blocks and 40 registers, 0.092 ms at 56)
template <> struct UpdateBounds<2, float> { static constexpr int minb = 8; };

template <int NC, typename R, bool HAS_J, bool REUNIT, typename I, bool PLANES = false>
__global__ void __launch_bounds__(128, UpdateBounds<NC, R>::minb)
k_update_grid(const R *__restrict__ U, R *__restrict__ E, const R *__restrict__ J, R *__restrict__ Unext,
              const uint8_t *__restrict__ active, Lat L) {
    const I s = (I)blockIdx.x * (I)blockDim.x + (I)threadIdx.x;
    if (s >= (I)L.V) return;
    if (active && !active[s]) return;  // Cell.isActive gate (FastTYMSolver.java:51)
    if constexpr (NC == 2) {
        if (PLANES) {
            update_site_su2_planes<R, HAS_J, REUNIT, I>(U, E, J, Unext, L, s);
            return;
        }
    }
    update_site<NC, R, HAS_J, REUNIT, I>(U, E, J, Unext, L, s);
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
    {
        // L2 prefetch of the warp's E lines (3 links x 8 components x the two
        // 32-site halves), which the thread reads only after its staple sums:
        // their DRAM latency then overlaps the staples (0.5 % per 128^3 step)
        const int lane = threadIdx.x & 31;
        const I s0 = sa - (I)lane + (I)((lane & 1) << 5);
        if (lane < 16 && s0 < (I)L.V) {
            const float *e = E + (I)(lane >> 1) * (I)L.V + s0;
            asm volatile("prefetch.global.L2 [%0];" ::"l"(e));
            asm volatile("prefetch.global.L2 [%0];" ::"l"(e + (I)8 * (I)L.V));
            asm volatile("prefetch.global.L2 [%0];" ::"l"(e + (I)16 * (I)L.V));
        }
    }
    if (sa >= (I)L.V) return;
    I sb = sa + 32;
    bool vb = sb < (I)L.V;
    if (!vb) sb = sa;
    const bool va = !active || active[sa];
    vb = vb && (!active || active[sb]);
    if (!va && !vb) return;  // Cell.isActive gate (FastTYMSolver.java:51)
    update_site_pair<I, HAS_J, REUNIT>(U, E, J, Unext, L, sa, sb, va, vb);
}

// The measured step: the update above plus the per-site BulkQuantities terms
// it can form from what it loads (update_site_pair with MEAS) and the Gauss
// law of the previous state from the previous step's transported terms Win
// (gauss_w_pair); it stores its own in Wout.  Every thread reaches the warp
// reduction, so no thread returns early.  Partials: FP32 warp sums, one row per
// warp, part[block * MEAS_THREADS / 32 + warp][MEAS_COLS].  There is no block
// barrier: a warp that has finished leaves, and the next block can start on
// its SM without waiting for the block's last warp (3 % per 128^3 measured
// step against block partials combined after a barrier).
template <typename I, bool REUNIT>
__global__ void __launch_bounds__(MEAS_THREADS, 3)
k_update_measure_su3f_pair(const float *__restrict__ U, float *__restrict__ E, float *__restrict__ Eout,
                           const float *__restrict__ Win, float *__restrict__ Wout, const float *__restrict__ rho,
                           float *__restrict__ Unext, Lat L, double *__restrict__ part) {
    __shared__ float slots[MEAS_COLS * MEAS_THREADS];
    float *slot = slots + threadIdx.x;
#pragma unroll
    for (int q = 0; q < MEAS_COLS; q++) slot[q * MEAS_THREADS] = 0.f;
    const I t = (I)blockIdx.x * (I)blockDim.x + (I)threadIdx.x;
    const I sa = ((t >> 5) << 6) + (t & 31);
    if (sa < (I)L.V) {
        I sb = sa + 32;
        const bool vb = sb < (I)L.V;
        if (!vb) sb = sa;
        slot[6 * MEAS_THREADS] = pr::lanes(gauss_w_pair<I>(E, Win, rho, L, sa, sb), true, vb);
        update_site_pair<I, false, REUNIT, true>(U, E, nullptr, Unext, L, sa, sb, true, vb, Eout, slot, Wout);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    double *pw = part + ((long)blockIdx.x * (MEAS_THREADS / 32) + w) * MEAS_COLS;
#pragma unroll
    for (int q = 0; q < MEAS_COLS; q++) {
        float v = slot[q * MEAS_THREADS];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) pw[q] = (double)v;
    }
}

// Column sums of the warp partials in a fixed order (block (q, k): column q
// of step k of the chunk), with the unit factors of the BulkQuantities
// columns: (g a_i)^-2 for E^2, (g a_i)^-2 / 2 for B^2 (the U / Unext
// average).  part[k][nparts][MEAS_COLS] -> rows[k][8].
__global__ void __launch_bounds__(256) k_measure_combine(const double *__restrict__ part, int nparts, Lat L,
                                                         double *__restrict__ rows) {
    __shared__ double ws[8];
    const int q = blockIdx.x;
    const double *pk = part + (long)blockIdx.y * nparts * MEAS_COLS;
    double *row = rows + 8 * blockIdx.y;
    double v = 0.0;
    for (int b = threadIdx.x; b < nparts; b += blockDim.x) v += pk[(long)b * MEAS_COLS + q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += ws[k];
        if (q < 6) {
            const int i = q % 3;
            const double uf = 1.0 / ((L.g * L.a[i]) * (L.g * L.a[i]));
            s *= q < 3 ? uf : 0.5 * uf;
        }
        row[q] = s;
    }
}

bool measured_step_fusable(const Ctx &c) {
    return c.nc == 3 && c.prec == OPX_F32 && c.pair_kernel && !c.imp_solver && !c.j_nonzero && !c.active &&
           !c.eval && c.P.n == 0 && c.sg.empty();
}

// the host sizes the partials by MEAS_ROW, the kernel writes MEAS_COLS per warp
static_assert(MEAS_ROW == MEAS_COLS, "measured-step row width");
int measured_blocks(const Ctx &c) { return grid_for(((c.L.V + 63) / 64) * 32, MEAS_THREADS); }
// rows of partials per measured step (one per warp)
int measured_parts(const Ctx &c) { return measured_blocks(c) * (MEAS_THREADS / 32); }

// One measured step, warp partials into part[measured_parts][MEAS_COLS]:
// reads c.U, c.E and Win, writes c.Unext, Eout and Wout (the caller swaps Eout
// into c.E and Wout into Win).
void launch_update_measure(Ctx &c, bool reunit, void *Eout, const void *Win, void *Wout, double *part) {
    const int nb = measured_blocks(c);
    const float *U = (const float *)c.U, *rho = c.rho_nonzero ? (const float *)c.rho : nullptr;
    const float *Wi = (const float *)Win;
    float *E = (float *)c.E, *Eo = (float *)Eout, *Un = (float *)c.Unext, *Wo = (float *)Wout;
    if (c.int_offsets) {
        if (reunit) k_update_measure_su3f_pair<int, true><<<nb, MEAS_THREADS, 0, c.stream>>>(U, E, Eo, Wi, Wo, rho, Un, c.L, part);
        else k_update_measure_su3f_pair<int, false><<<nb, MEAS_THREADS, 0, c.stream>>>(U, E, Eo, Wi, Wo, rho, Un, c.L, part);
    } else {
        if (reunit) k_update_measure_su3f_pair<long, true><<<nb, MEAS_THREADS, 0, c.stream>>>(U, E, Eo, Wi, Wo, rho, Un, c.L, part);
        else k_update_measure_su3f_pair<long, false><<<nb, MEAS_THREADS, 0, c.stream>>>(U, E, Eo, Wi, Wo, rho, Un, c.L, part);
    }
    c.launches += 1;
}

// The rows of nsteps measured steps from their consecutive partials.
void launch_measure_combine(Ctx &c, const double *part, int nsteps, double *rows) {
    k_measure_combine<<<dim3(MEAS_COLS, nsteps), 256, 0, c.stream>>>(part, measured_parts(c), c.L, rows);
    c.launches += 1;
}

// ---------------------------------------------------------------- implicit solver
// ImplicitTYMSolver (physics/fields/ImplicitTYMSolver.java), SU(2).  The
// implicit grid is a copy: Ui its links (the latest estimate after its
// storeFields), Uin its next links, Ei its E.

// SU2GroupElement.pow(x) = exp(x log u) (math/SU2GroupElement.java:234-271)
template <typename R>
__device__ __forceinline__ Q2<R> group_pow(const Q2<R> &u, R x) {
    R norm = u.e[1] * u.e[1] + u.e[2] * u.e[2] + u.e[3] * u.e[3];
    norm = Real<R>::sqrt_(norm);
    R v[3];
    if (norm < R(1.E-15)) {
        v[0] = R(2) * u.e[1]; v[1] = R(2) * u.e[2]; v[2] = R(2) * u.e[3];
    } else {
        const R f = R(2) * asin(norm) / norm;
        v[0] = f * u.e[1]; v[1] = f * u.e[2]; v[2] = f * u.e[3];
    }
    for (int c = 0; c < 3; c++) v[c] *= x;
    return SU2<R>::expi(v);
}
// SU3GroupElement.pow(x) = getAlgebraElement().mult(x).getLink() (math/SU3GroupElement.java:516-518);
// the logarithm in FP64 (su3_log.cuh)
template <typename R>
__device__ __forceinline__ M3<R> group_pow(const M3<R> &u, R x) {
    M3<double> ud;
    for (int k = 0; k < 9; k++) { ud.r[k] = (double)u.r[k]; ud.i[k] = (double)u.i[k]; }
    double g[8];
    su3_log_gen(ud, g);
    R v[8];
    for (int a = 0; a < 8; a++) v[a] = (R)(g[a] * (double)x);
    return SU3<R>::expi(v);
}

// ImplicitStep.getPlaquetteSum (:136-177): links of direction i / d at time
// -1 (Wm: the grid's Unext slot = the previous links), 0 (W0 = grid U) or +1
// (Wp = Ui), implicit time in the transverse plane and along the beam (0).
template <class G, typename R>
__device__ __forceinline__ typename G::M implicit_psum(const LinkPlanes<G, R> &Wm, const LinkPlanes<G, R> &W0,
                                                       const LinkPlanes<G, R> &Wp, const Lat &L, long s, const int *x,
                                                       int d, int time) {
    using M = typename G::M;
    M S = G::zero();
    const int beam = 0;
    const long ci1 = shift_d(L, s, x[d], d, +1);
    int x1[3] = {x[0], x[1], x[2]};
    x1[d] = x[d] == L.n[d] - 1 ? 0 : x[d] + 1;
#pragma unroll 1
    for (int i = 0; i < 3; i++) {
        if (i == d) continue;
        const bool inT = (i != beam) && (d != beam);
        int td = 0, ti = 0;
        if (inT) { td = time; ti = time; }
        else { if (d == beam) td = time; else if (i == beam) ti = time; }
        const LinkPlanes<G, R> &Wd = td < 0 ? Wm : (td > 0 ? Wp : W0);
        const LinkPlanes<G, R> &Wi = ti < 0 ? Wm : (ti > 0 ? Wp : W0);
        const long ci2 = shift_d(L, s, x[i], i, +1), ci3 = shift_d(L, ci1, x1[i], i, -1),
                   ci4 = shift_d(L, s, x[i], i, -1);
        M U1 = G::mul_adj(G::mul_adj(Wi.load(i, ci1), Wd.load(d, ci2)), Wi.load(i, s));
        const M U2 = G::adj_mul(G::mul(Wd.load(d, ci4), Wi.load(i, ci3)), Wi.load(i, ci4));
        G::add(U1, U2);
        U1 = G::mul(Wd.load(d, s), U1);
        G::scale(U1, LatR<R>::inva2(L, i));
        G::add(S, U1);
    }
    return S;
}

// ImplicitStep (:103-131) fused with ImplicitDamping (:195-207) for the three links of a site
template <int NC, typename R, bool HAS_J>
__global__ void __launch_bounds__(128) k_implicit_step(const R *__restrict__ U, const R *__restrict__ Uprev,
                                                       const R *__restrict__ Ui, const R *__restrict__ E,
                                                       const R *__restrict__ J, R *__restrict__ Ei,
                                                       R *__restrict__ Uin, const uint8_t *__restrict__ active, Lat L,
                                                       R damping) {
    using G = typename GroupOf<NC, R>::T;
    constexpr int NA = G::NA;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    if (active && !active[s]) return;
    const LinkPlanes<G, R> Wm{const_cast<R *>(Uprev), L.V}, W0{const_cast<R *>(U), L.V}, Wp{const_cast<R *>(Ui), L.V},
        Wn{Uin, L.V};
    const AlgPlanes<NA, R> Ep{const_cast<R *>(E), L.V}, Eo{Ei, L.V}, Jp{const_cast<R *>(J), L.V};
    int x[3];
    site_coords(L, s, x);
    const R dt = LatR<R>::dt(L), hdt = dt * R(0.5);
#pragma unroll 1
    for (int i = 0; i < 3; i++) {
        R e[NA], pr[NA];
        Ep.load_ro(i, s, e);
        G::proj(implicit_psum<G, R>(Wm, W0, Wp, L, s, x, i, +1), pr);
        for (int c = 0; c < NA; c++) e[c] += pr[c] * hdt;
        G::proj(implicit_psum<G, R>(Wm, W0, Wp, L, s, x, i, -1), pr);
        for (int c = 0; c < NA; c++) e[c] += pr[c] * hdt;
        if (HAS_J) {
            R jv[NA];
            Jp.load_ro(i, s, jv);
            const R jf = LatR<R>::jfac(L, i);
            for (int c = 0; c < NA; c++) e[c] += jv[c] * jf;
        }
        Eo.store(i, s, e);
        R v[NA];
        for (int c = 0; c < NA; c++) v[c] = -dt * e[c];
        const auto Vn = G::mul(G::expi(v), W0.load(i, s));
        Wn.store(i, s, G::mul(group_pow(Wp.load(i, s), damping), group_pow(Vn, R(1) - damping)));
    }
}

// ImplicitEnd (:217-226): E and Unext of the active cells from the implicit grid
template <int NC, typename R>
__global__ void k_implicit_end(const R *__restrict__ Ei, const R *__restrict__ Uin, R *__restrict__ E,
                               R *__restrict__ Un, const uint8_t *__restrict__ active, Lat L) {
    using G = typename GroupOf<NC, R>::T;
    constexpr int NA = G::NA;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    if (active && !active[s]) return;
    const LinkPlanes<G, R> A{const_cast<R *>(Uin), L.V}, B{Un, L.V};
    for (int d = 0; d < 3; d++) {
        B.store(d, s, A.load(d, s));
        for (int a = 0; a < NA; a++) E[((long)d * NA + a) * L.V + s] = Ei[((long)d * NA + a) * L.V + s];
    }
}

template <int NC, typename R>
static int implicit_update_t(Ctx &c) {
    const long V = c.L.V;
    const size_t nU = (size_t)link_elems(V, c.ng) * sizeof(R), nE = (size_t)V * 3 * c.na * sizeof(R);
    if (!c.imp_Ua) {
        if (cudaMalloc(&c.imp_Ua, nU) != cudaSuccess || cudaMalloc(&c.imp_Ub, nU) != cudaSuccess ||
            cudaMalloc(&c.imp_E, nE) != cudaSuccess) {
            cudaGetLastError();
            c.err = "implicit solver: out of device memory";
            return OPX_ERR_NOMEM;
        }
    }
    R *Ui = (R *)c.imp_Ua, *Uin = (R *)c.imp_Ub, *Ei = (R *)c.imp_E;
    // Grid(grid): the implicit grid starts as a copy
    cudaMemcpyAsync(Ui, c.U, nU, cudaMemcpyDeviceToDevice, c.stream);
    cudaMemcpyAsync(Uin, c.Unext, nU, cudaMemcpyDeviceToDevice, c.stream);
    cudaMemcpyAsync(Ei, c.E, nE, cudaMemcpyDeviceToDevice, c.stream);
    // ImplicitBegin (:68-90): the explicit combined update into the implicit grid
    const int B = 128;
    const dim3 grid(grid_for(V, B));
    if (c.j_nonzero) k_update_grid<NC, R, true, false, long><<<grid, B, 0, c.stream>>>((const R *)c.U, Ei, (const R *)c.J, Uin, c.active, c.L);
    else k_update_grid<NC, R, false, false, long><<<grid, B, 0, c.stream>>>((const R *)c.U, Ei, (const R *)c.J, Uin, c.active, c.L);
    c.launches++;
    for (int it = 0; it < c.imp_iterations; it++) {
        std::swap(Ui, Uin);  // implicitGrid.storeFields()
        if (c.j_nonzero)
            k_implicit_step<NC, R, true><<<grid, B, 0, c.stream>>>((const R *)c.U, (const R *)c.Unext, Ui, (const R *)c.E,
                                                               (const R *)c.J, Ei, Uin, c.active, c.L, (R)c.imp_damping);
        else
            k_implicit_step<NC, R, false><<<grid, B, 0, c.stream>>>((const R *)c.U, (const R *)c.Unext, Ui, (const R *)c.E,
                                                                (const R *)c.J, Ei, Uin, c.active, c.L, (R)c.imp_damping);
        c.launches++;
    }
    k_implicit_end<NC, R><<<grid, B, 0, c.stream>>>(Ei, Uin, (R *)c.E, (R *)c.Unext, c.active, c.L);
    c.launches++;
    return OPX_OK;
}

int launch_implicit_update(Ctx &c) {
    if (c.nc == 2) return c.prec == OPX_F64 ? implicit_update_t<2, double>(c) : implicit_update_t<2, float>(c);
    return c.prec == OPX_F64 ? implicit_update_t<3, double>(c) : implicit_update_t<3, float>(c);
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

// The plaquette form streamed along dimension 0 (su3_stream.cuh): one wave of
// resident blocks, each with an equal share of the (tile, x0) units.
static bool stream_eligible(const Ctx &c) {
    return c.stream_kernel && c.int_offsets && !c.j_nonzero && !c.active && c.L.n[1] % st::T1 == 0 &&
           c.L.n[2] % st::T2 == 0;
}

static void update_grid_su3f_stream(Ctx &c, bool reunit) {
    const int smem = (int)sizeof(st::Smem);
    if (!c.st_grid) {
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(st::k_update_grid_su3f_stream<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        cudaFuncSetAttribute(st::k_update_grid_su3f_stream<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, st::k_update_grid_su3f_stream<false>, st::THREADS, smem);
        const long units = (long)(c.L.n[1] / st::T1) * (c.L.n[2] / st::T2) * c.L.n[0];
        long grid = (long)std::max(1, per_sm) * std::max(1, sms);
        // OPX_STREAM_BLOCKS=n: n blocks instead of one resident wave (tests use
        // a few blocks so that each walks long ranges across tile boundaries)
        if (const char *v = std::getenv("OPX_STREAM_BLOCKS")) grid = std::max(1L, std::atol(v));
        c.st_grid = (int)std::max(1L, std::min<long>(units, grid));
    }
    const float *U = (const float *)c.U;
    float *E = (float *)c.E, *Un = (float *)c.Unext;
    if (reunit) st::k_update_grid_su3f_stream<true><<<c.st_grid, st::THREADS, smem, c.stream>>>(U, E, Un, c.L);
    else st::k_update_grid_su3f_stream<false><<<c.st_grid, st::THREADS, smem, c.stream>>>(U, E, Un, c.L);
    c.launches++;
}

static void update_grid_su3f_pair(Ctx &c, bool reunit) {
    if (stream_eligible(c)) {
        update_grid_su3f_stream(c, reunit);
        return;
    }
    // 32-bit offsets while the largest link offset (3 blocks x 576 floats) fits
    if (c.int_offsets) update_grid_su3f_pair_i<int>(c, reunit);
    else update_grid_su3f_pair_i<long>(c, reunit);
}

template <int NC, typename R, typename I>
static void launch_update_grid_i(Ctx &c, bool reunit, dim3 grid, int B, const R *U, R *E, const R *J, R *Un) {
    // SU(2): the plane-by-plane staple sums (update_site_su2_planes: 6 % faster
    // in FP64, 5 % in FP32)
    if (NC == 2) {
        if (c.j_nonzero) {
            if (reunit) k_update_grid<NC, R, true, true, I, true><<<grid, B, 0, c.stream>>>(U, E, J, Un, c.active, c.L);
            else k_update_grid<NC, R, true, false, I, true><<<grid, B, 0, c.stream>>>(U, E, J, Un, c.active, c.L);
        } else {
            if (reunit) k_update_grid<NC, R, false, true, I, true><<<grid, B, 0, c.stream>>>(U, E, J, Un, c.active, c.L);
            else k_update_grid<NC, R, false, false, I, true><<<grid, B, 0, c.stream>>>(U, E, J, Un, c.active, c.L);
        }
        return;
    }
    if (c.j_nonzero) {
        if (reunit) k_update_grid<NC, R, true, true, I><<<grid, B, 0, c.stream>>>(U, E, J, Un, c.active, c.L);
        else k_update_grid<NC, R, true, false, I><<<grid, B, 0, c.stream>>>(U, E, J, Un, c.active, c.L);
    } else {
        if (reunit) k_update_grid<NC, R, false, true, I><<<grid, B, 0, c.stream>>>(U, E, J, Un, c.active, c.L);
        else k_update_grid<NC, R, false, false, I><<<grid, B, 0, c.stream>>>(U, E, J, Un, c.active, c.L);
    }
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
    if (c.int_offsets) launch_update_grid_i<NC, R, int>(c, reunit, grid, B, U, E, J, Un);
    else launch_update_grid_i<NC, R, long>(c, reunit, grid, B, U, E, J, Un);
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
