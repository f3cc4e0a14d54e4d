// reduce_kernels.cu -- whole-lattice reductions and per-cell diagnostics.
//
//   k_bulk_partial(_su3f_pair) : FieldMeasurements E^2, B^2, Gauss, rho^2
//       (physics/measurements/FieldMeasurements.java:68-231) as used by
//       BulkQuantitiesInTime.calculate (diagnostics/methods/BulkQuantitiesInTime.java:83-121).
//       One pass computes all of them (the reference makes six lattice passes).
//       Per-site values are formed in the storage precision; each thread
//       accumulates them in FP64 with compensated (Neumaier/TwoSum) sums (FP64
//       storage) or in FP32 Kahan runs added to an FP64 sum (FP32 storage); a
//       block adds its threads in a fixed FP64 tree and the block partials are
//       combined by one block in a fixed order, so results are deterministic.
//   k_energy_density   : EnergyDensity.ComponentComputation (EnergyDensity.java:119-166)
//   k_projected_energy : ProjectedEnergyDensity.EnergyDensityComputation (:114-179)
//   k_gauss_field      : Grid.getGaussConstraint (Grid.java:944-968) at every cell
#include <algorithm>

#include "internal.h"
#include "ksum.cuh"
#include "observables.cuh"
#include "su3_pair.cuh"

namespace opx {

// Register caps for 128-thread reduction blocks: 4 blocks per SM (128
// registers), SU(3) FP64 2 (255).
template <int NC, typename R> struct RedBounds { static constexpr int minb = 4; };
template <> struct RedBounds<3, float> { static constexpr int minb = 4; };
template <> struct RedBounds<3, double> { static constexpr int minb = 2; };
constexpr int RED_THREADS = 128;

// Columns of the partial sums: E^2[3], B^2 from U [3], G^2, rho^2, B^2 from
// Unext [3].  B^2 of U and of Unext are kept apart so that a reduction right
// after one step can take B^2 of U from the previous reduction's B^2 of Unext
// (the same links; skip_u).
constexpr int NQS = BULK_COLUMNS;

// The last block of a reduction to finish combines the block partials: warp w
// takes columns w, w + nwarps, ...; its lanes stride over the blocks with
// compensated sums and a fixed shuffle tree adds the lanes.  So a reduction is
// one launch.  Each block publishes its partials, fences and draws a ticket;
// the block that draws the last ticket reads every partial (through L2) and
// resets the counter for the next launch on the stream.  No block waits on
// another.
template <int NQ>
__device__ __forceinline__ void last_block_combine(const double *part, unsigned *count, double *out) {
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(count, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
    for (int q = warp; q < NQ; q += nw) {
        KSum v{0.0, 0.0};
        for (int b = lane; b < (int)gridDim.x; b += 32)
            ksum_merge(v, KSum{__ldcg(part + ((long)b * NQ + q) * 2), __ldcg(part + ((long)b * NQ + q) * 2 + 1)});
        for (int o = 16; o > 0; o >>= 1) {
            KSum w{__shfl_down_sync(0xffffffffu, v.s, o), __shfl_down_sync(0xffffffffu, v.c, o)};
            ksum_merge(v, w);
        }
        if (lane == 0) out[q] = v.s + v.c;
    }
    if (threadIdx.x == 0) *count = 0u;
}

template <int NC, typename R>
__global__ void __launch_bounds__(RED_THREADS, RedBounds<NC, R>::minb)
    k_bulk_partial(const R *__restrict__ U, const R *__restrict__ Unext, const R *__restrict__ E,
                   const R *__restrict__ rho, const uint8_t *__restrict__ eval, Lat L, int skip_u,
                   double *__restrict__ part, unsigned *__restrict__ count, double *__restrict__ out,
                   double *__restrict__ bn_site) {
    using G = typename GroupOf<NC, R>::T;
    constexpr int NA = G::NA;
    const LinkPlanes<G, R> Up{const_cast<R *>(U), L.V}, Unp{const_cast<R *>(Unext), L.V};
    const AlgPlanes<NA, R> Ep{const_cast<R *>(E), L.V};
    __shared__ double2 acc_sh[NQS * RED_THREADS];
    const SharedKSums<NQS, RED_THREADS> sacc{acc_sh};
    sacc.zero();
    double p[NQS];
#pragma unroll
    for (int q = 0; q < NQS; q++) p[q] = 0.0;
    int run = 0;
    for (long s = (long)blockIdx.x * blockDim.x + threadIdx.x; s < L.V; s += (long)gridDim.x * blockDim.x) {
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
            double bu = 0.0;
            if (!skip_u) {
                field_b<G, R>(Up, L, s, nb, i, b0);
                bu = sqr<R, NA>(b0);
            }
            field_b<G, R>(Unp, L, s, nb, i, b1);
            const double bn = sqr<R, NA>(b1);
            if (bn_site) bn_site[(long)i * L.V + s] = bn;
            if (i == 0) { p[0] += ev; p[3] += bu; p[8] += bn; }
            else if (i == 1) { p[1] += ev; p[4] += bu; p[9] += bn; }
            else { p[2] += ev; p[5] += bu; p[10] += bn; }
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
            sacc.add(p);
#pragma unroll
            for (int q = 0; q < NQS; q++) p[q] = 0.0;
            run = 0;
        }
    }
    sacc.add(p);
    KSum acc[NQS];
    sacc.load(acc);
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const double uf = 1.0 / ((L.g * L.a[i]) * (L.g * L.a[i]));
        acc[i].s *= uf; acc[i].c *= uf;
        acc[3 + i].s *= 0.5 * uf; acc[3 + i].c *= 0.5 * uf;
        acc[8 + i].s *= 0.5 * uf; acc[8 + i].c *= 0.5 * uf;
    }
    int q;
    KSum v = block_reduce<NQS>(acc, q);
    if (q >= 0) {
        part[((long)blockIdx.x * NQS + q) * 2] = v.s;
        part[((long)blockIdx.x * NQS + q) * 2 + 1] = v.c;
    }
    last_block_combine<NQS>(part, count, out);
}

int reduction_blocks(long V) { return (int)std::min<long>(grid_for(V, RED_THREADS), 8L * 152); }

// SU(3) FP32: two sites per thread in paired FP32 instructions (the
// arithmetic of bulk_accumulate for sites sa and sb = sa + 32).  The per-site
// values are FP32; a thread sums the two lanes and runs of 32 pair-iterations
// (64 sites) in FP32 with Kahan compensation (every value is a sum of squares,
// so the running sum dominates each term), then adds each run to a plain FP64
// sum.  The FP64 pipe is narrow on this part: one FP64 add per column per site
// kept it half busy.
template <typename I>
__global__ void __launch_bounds__(RED_THREADS, 3)
    k_bulk_partial_su3f_pair(const float *__restrict__ U, const float *__restrict__ Unext,
                             const float *__restrict__ E, const float *__restrict__ rho,
                             const uint8_t *__restrict__ eval, Lat L, int skip_u, double *__restrict__ part,
                             unsigned *__restrict__ count, double *__restrict__ out) {
    using namespace pr;
    const I V = (I)L.V, nblk = (I)((L.V + 31) >> 5);
    const I npairs = (I)(((L.V + 63) >> 6) << 5);
    __shared__ double acc_sh[NQS * RED_THREADS];
    const SharedSums<NQS, RED_THREADS> sacc{acc_sh};
    sacc.zero();
    float rs[NQS], rc[NQS];  // FP32 Kahan run sums and their compensations
#pragma unroll
    for (int q = 0; q < NQS; q++) { rs[q] = 0.f; rc[q] = 0.f; }
    auto kadd = [&](int q, float x) {
        const float y = x - rc[q];
        const float t = rs[q] + y;
        rc[q] = (t - rs[q]) - y;
        rs[q] = t;
    };
    auto flush = [&]() {
#pragma unroll
        for (int q = 0; q < NQS; q++) {
            sacc.add1(q, (double)rs[q] - (double)rc[q]);
            rs[q] = 0.f;
            rc[q] = 0.f;
        }
    };
    int run = 0;
    for (I t = (I)blockIdx.x * blockDim.x + threadIdx.x; t < npairs; t += (I)gridDim.x * blockDim.x) {
        const I sa = ((t >> 5) << 6) + (t & 31);
        if (sa >= V) continue;
        I sb = sa + 32;
        bool vb = sb < V;
        if (!vb) sb = sa;
        const bool wa = !eval || eval[sa];
        const bool wb = vb && (!eval || eval[sb]);
        if (!wa && !wb) continue;
        int xa[3], xb[3];
        coords<I>(L, sa, xa);
        coords<I>(L, sb, xb);
        auto lanes = [&](P v) { return (wa ? v.x : 0.f) + (wb ? v.y : 0.f); };
#pragma unroll 1
        for (int d = 0; d < 3; d++) {
            // B_d from U and Unext: U_j(x) U_k(x+j) U_j(x+k)^dagger U_k(x)^dagger, (d, j, k) cyclic
            const int j = d + 1 >= 3 ? d - 2 : d + 1, k = d + 2 >= 3 ? d - 1 : d + 2;
            const I pja = shift<I>(L, sa, pick(xa[0], xa[1], xa[2], j), j, +1);
            const I pjb = shift<I>(L, sb, pick(xb[0], xb[1], xb[2], j), j, +1);
            const I pka = shift<I>(L, sa, pick(xa[0], xa[1], xa[2], k), k, +1);
            const I pkb = shift<I>(L, sb, pick(xb[0], xb[1], xb[2], k), k, +1);
            const P bf = bc(LatR<float>::bfac(L, d));
            P sbu = zero2(), sbn = zero2();
#pragma unroll 1
            for (int tt = skip_u ? 1 : 0; tt < 2; tt++) {
                const float *W = tt == 0 ? U : Unext;
                const M Pq = mul_adj(mul_adj(mul(load<I>(W, nblk, j, sa, sb), load<I>(W, nblk, k, pja, pjb)),
                                             load<I>(W, nblk, j, pka, pkb)),
                                     load<I>(W, nblk, k, sa, sb));
                P b[8];
                proj(Pq, b);
                P sb2 = zero2();
#pragma unroll
                for (int a = 0; a < 8; a++) { b[a] = mul2(b[a], bf); sb2 = fma2(b[a], b[a], sb2); }
                if (tt == 0) sbu = sb2; else sbn = sb2;
            }
            // constant indices keep the run sums in registers
            const float bu = lanes(sbu), bn = lanes(sbn);
            if (d == 0) { if (!skip_u) kadd(3, bu); kadd(8, bn); }
            else if (d == 1) { if (!skip_u) kadd(4, bu); kadd(9, bn); }
            else { if (!skip_u) kadd(5, bu); kadd(10, bn); }
        }
        // Gauss: sum_i [E_i(x) - U_i(x-i)^dagger E_i(x-i) U_i(x-i)] gfac_i - rho(x)
        P gs[8];
#pragma unroll
        for (int a = 0; a < 8; a++) gs[a] = zero2();
        // the three directions unrolled: their loads interleave (5 % faster after a step)
#pragma unroll
        for (int i = 0; i < 3; i++) {
            const I mia = shift<I>(L, sa, pick(xa[0], xa[1], xa[2], i), i, -1);
            const I mib = shift<I>(L, sb, pick(xb[0], xb[1], xb[2], i), i, -1);
            const I eo = (I)i * 8 * V;
            P e0[8], e1[8], tv[8];
#pragma unroll
            for (int a = 0; a < 8; a++) {
                e0[a] = pp(__ldg(E + eo + (I)a * V + sa), __ldg(E + eo + (I)a * V + sb));
                e1[a] = pp(__ldg(E + eo + (I)a * V + mia), __ldg(E + eo + (I)a * V + mib));
            }
            // E^2 of link i at x
            P se = mul2(e0[0], e0[0]);
#pragma unroll
            for (int a = 1; a < 8; a++) se = fma2(e0[a], e0[a], se);
            const float ev = lanes(se);
            if (i == 0) kadd(0, ev);
            else if (i == 1) kadd(1, ev);
            else kadd(2, ev);
            const M Ub = load<I>(U, nblk, i, mia, mib);
            act_adj_gen(Ub, e1, tv);
            const P gf = bc(LatR<float>::gfac(L, i));
#pragma unroll
            for (int a = 0; a < 8; a++) gs[a] = fma2(sub2(e0[a], tv[a]), gf, gs[a]);
        }
        if (rho) {
            P r2 = zero2();
#pragma unroll
            for (int a = 0; a < 8; a++) {
                const P r = pp(__ldg(rho + (I)a * V + sa), __ldg(rho + (I)a * V + sb));
                gs[a] = sub2(gs[a], r);
                r2 = fma2(r, r, r2);
            }
            kadd(7, lanes(r2));
        }
        P g2 = mul2(gs[0], gs[0]);
#pragma unroll
        for (int a = 1; a < 8; a++) g2 = fma2(gs[a], gs[a], g2);
        kadd(6, lanes(g2));
        if (++run == 32) {
            flush();
            run = 0;
        }
    }
    flush();
    KSum acc[NQS];
    sacc.load(acc);
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const double uf = 1.0 / ((L.g * L.a[i]) * (L.g * L.a[i]));
        acc[i].s *= uf; acc[i].c *= uf;
        acc[3 + i].s *= 0.5 * uf; acc[3 + i].c *= 0.5 * uf;
        acc[8 + i].s *= 0.5 * uf; acc[8 + i].c *= 0.5 * uf;
    }
    int q;
    KSum v = block_reduce<NQS>(acc, q);
    if (q >= 0) {
        part[((long)blockIdx.x * NQS + q) * 2] = v.s;
        part[((long)blockIdx.x * NQS + q) * 2 + 1] = v.c;
    }
    last_block_combine<NQS>(part, count, out);
}


// Blocks of one kernel resident on the whole device at once: the grid-stride
// reductions then run in a single wave with equal work per thread.
template <typename K>
static int resident_blocks(K kernel) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, RED_THREADS, 0);
    return std::max(1, per_sm) * std::max(1, sms);
}

template <int NC, typename R>
static void bulk_t(Ctx &c, int skip_u) {
    int nb = c.red_blocks;
    if (NC == 3 && sizeof(R) == 4 && c.pair_kernel) {
        if (c.int_offsets) {
            static const int wave = resident_blocks(k_bulk_partial_su3f_pair<int>);
            nb = std::min(nb, wave);
            k_bulk_partial_su3f_pair<int><<<nb, RED_THREADS, 0, c.stream>>>(
                (const float *)c.U, (const float *)c.Unext, (const float *)c.E, (const float *)(c.rho_nonzero ? c.rho : nullptr), c.eval, c.L,
                skip_u, c.red_part, c.red_count, c.red_out);
        } else {
            static const int wave = resident_blocks(k_bulk_partial_su3f_pair<long>);
            nb = std::min(nb, wave);
            k_bulk_partial_su3f_pair<long><<<nb, RED_THREADS, 0, c.stream>>>(
                (const float *)c.U, (const float *)c.Unext, (const float *)c.E, (const float *)(c.rho_nonzero ? c.rho : nullptr), c.eval, c.L,
                skip_u, c.red_part, c.red_count, c.red_out);
        }
    } else {
        static const int wave = resident_blocks(k_bulk_partial<NC, R>);
        nb = std::min(nb, wave);
        k_bulk_partial<NC, R><<<nb, RED_THREADS, 0, c.stream>>>((const R *)c.U, (const R *)c.Unext, (const R *)c.E,
                                                               (const R *)(c.rho_nonzero ? c.rho : nullptr), c.eval, c.L, skip_u, c.red_part,
                                                               c.red_count, c.red_out, c.bn_site);
    }
    c.launches += 1;
}

void launch_bulk(Ctx &c, int skip_u) {
    if (c.nc == 2) {
        if (c.prec == OPX_F64) bulk_t<2, double>(c, skip_u); else bulk_t<2, float>(c, skip_u);
    } else {
        if (c.prec == OPX_F64) bulk_t<3, double>(c, skip_u); else bulk_t<3, float>(c, skip_u);
    }
}

// EnergyDensity: sum_d [0.5 E_d^2 + 0.25 (B_d(U) + B_d(Unext))^2] / (g a_0)^2
// (the direction-0 unit factor for every d and B summed before squaring, as the
// reference does: EnergyDensity.java:136,154-158)
template <int NC, typename R>
__global__ void k_energy_density(const R *__restrict__ U, const R *__restrict__ Unext, const R *__restrict__ E,
                                 const uint8_t *__restrict__ eval, Lat L, double *__restrict__ out) {
    using G = typename GroupOf<NC, R>::T;
    constexpr int NA = G::NA;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    if (eval && !eval[s]) { out[s] = 0.0; return; }
    const LinkPlanes<G, R> Up{const_cast<R *>(U), L.V}, Unp{const_cast<R *>(Unext), L.V};
    const AlgPlanes<NA, R> Ep{const_cast<R *>(E), L.V};
    int x[3];
    site_coords(L, s, x);
    const Nbr nb = neighbours(L, s, x);
    const double uf = 1.0 / ((L.g * L.a[0]) * (L.g * L.a[0]));
    double en = 0.0;
    for (int d = 0; d < 3; d++) {
        R e[NA], b0[NA], b1[NA];
        Ep.load_ro(d, s, e);
        field_b<G, R>(Up, L, s, nb, d, b0);
        field_b<G, R>(Unp, L, s, nb, d, b1);
#pragma unroll
        for (int a = 0; a < NA; a++) b0[a] += b1[a];
        en += (0.5 * sq<R, NA>(e) + 0.25 * sq<R, NA>(b0)) * uf;
    }
    out[s] = en;
}

// Block (k, part) sums slice x_dir = k over its share of the transverse sites;
// six sums per block (PROJ_COLUMNS): T_el, T_mag of U, L_el, L_mag of U, T_mag
// of Unext, L_mag of Unext, combined per slice in a fixed order by
// k_projected_final.  The magnetic sums of U and Unext stay apart so that a
// call after one step can take U's from the previous call's Unext (skip_u).
constexpr int PROJ_COLUMNS = 6;
template <int NC, typename R>
__global__ void __launch_bounds__(RED_THREADS, RedBounds<NC, R>::minb)
    k_projected_energy(const R *__restrict__ U, const R *__restrict__ Unext, const R *__restrict__ E,
                       const uint8_t *__restrict__ eval, Lat L, int dir, int skip_u,
                       const double *__restrict__ bn_site, double *__restrict__ part) {
    using G = typename GroupOf<NC, R>::T;
    constexpr int NA = G::NA;
    const LinkPlanes<G, R> Up{const_cast<R *>(U), L.V}, Unp{const_cast<R *>(Unext), L.V};
    const AlgPlanes<NA, R> Ep{const_cast<R *>(E), L.V};
    const int k = blockIdx.x, nsplit = gridDim.y;
    const int o1 = (dir + 1) % 3, o2 = (dir + 2) % 3;
    const long nt = L.V / L.n[dir];
    const double area = (double)L.V / (double)L.n[dir];
    // a thread's sites of the slice are summed plainly in FP64 (a handful per
    // thread: nt / (nsplit * blockDim) of them), the block's threads with
    // compensation; the FP64 pipe is narrow on this part
    double p[PROJ_COLUMNS];
#pragma unroll
    for (int q = 0; q < PROJ_COLUMNS; q++) p[q] = 0.0;
    for (long t = (long)blockIdx.y * blockDim.x + threadIdx.x; t < nt; t += (long)nsplit * blockDim.x) {
        int x[3];
        x[dir] = k;
        const int lo = (o1 > o2) ? o1 : o2, hi = (o1 > o2) ? o2 : o1;  // hi = slower of the two
        x[lo] = (int)(t % L.n[lo]);
        x[hi] = (int)(t / L.n[lo]);
        const long s = x[0] * L.stride[0] + x[1] * L.stride[1] + x[2];
        if (eval && !eval[s]) continue;
        const Nbr nb = neighbours(L, s, x);
        double el_t = 0, el_l = 0, mu_t = 0, mu_l = 0, mn_t = 0, mn_l = 0;
#pragma unroll 1
        for (int j = 0; j < 3; j++) {
            const double uf = 1.0 / ((L.g * L.a[j]) * (L.g * L.a[j])) / area;
            R e[NA], b0[NA], b1[NA];
            Ep.load_ro(j, s, e);
            double mu = 0.0;
            if (!skip_u) {
                field_b<G, R>(Up, L, s, nb, j, b0);
                mu = 0.25 * sqr<R, NA>(b0) * uf;
            }
            double bn;
            if (bn_site) {
                bn = __ldg(bn_site + (long)j * L.V + s);
            } else {
                field_b<G, R>(Unp, L, s, nb, j, b1);
                bn = sqr<R, NA>(b1);
            }
            const double el = 0.5 * sqr<R, NA>(e) * uf;
            const double mn = 0.25 * bn * uf;
            if (j == dir) { el_l += el; mu_l += mu; mn_l += mn; } else { el_t += el; mu_t += mu; mn_t += mn; }
        }
        p[0] += el_t;
        p[2] += el_l;
        p[4] += mn_t;
        p[5] += mn_l;
        if (!skip_u) {
            p[1] += mu_t;
            p[3] += mu_l;
        }
    }
    KSum acc[PROJ_COLUMNS];
#pragma unroll
    for (int q = 0; q < PROJ_COLUMNS; q++) acc[q] = KSum{p[q], 0.0};
    int q;
    KSum v = block_reduce<PROJ_COLUMNS>(acc, q);
    if (q >= 0) {
        const long o = (((long)k * nsplit + blockIdx.y) * PROJ_COLUMNS + q) * 2;
        part[o] = v.s;
        part[o + 1] = v.c;
    }
}

// out[q][k] for the six columns of slice k
__global__ void k_projected_final(const double *__restrict__ part, int nslices, int nsplit, double *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // i = q * nslices + k
    if (i >= PROJ_COLUMNS * nslices) return;
    const int q = i / nslices, k = i % nslices;
    KSum v{0.0, 0.0};
    for (int b = 0; b < nsplit; b++) {
        const long o = (((long)k * nsplit + b) * PROJ_COLUMNS + q) * 2;
        ksum_merge(v, KSum{part[o], part[o + 1]});
    }
    out[(long)q * nslices + k] = v.s + v.c;
}

// ProjectedEnergyDensity.PoyntingComputation (diagnostics/methods/ProjectedEnergyDensity.java:182-279),
// SU(2): per cell the averaged longitudinal Poynting vector (E averaged over
// the link and its transported neighbour, F from the eight plaquettes of the
// (dir, i) plane at U and Unext) and the time-averaged one (E x B with B
// averaged over U and Unext).  Every cell counts, as in the reference.
template <typename R>
__device__ __forceinline__ Q2<R> link_o(const LinkPlanes<SU2<R>, R> &Up, const Lat &L, const int *x, int d, int o) {
    // Grid.getLink: U_d(x) for o > 0, U_d(x - d)^dagger for o < 0
    int y[3] = {x[0], x[1], x[2]};
    if (o < 0) y[d] = y[d] == 0 ? L.n[d] - 1 : y[d] - 1;
    const long s = ((long)y[0] * L.n[1] + y[1]) * L.n[2] + y[2];
    const Q2<R> u = Up.load(d, s);
    return o < 0 ? SU2<R>::adj(u) : u;
}
__device__ __forceinline__ void step_pos(const Lat &L, int *x, int d, int o) {
    x[d] = o > 0 ? (x[d] == L.n[d] - 1 ? 0 : x[d] + 1) : (x[d] == 0 ? L.n[d] - 1 : x[d] - 1);
}
// Grid.getPlaquette(index, d1, d2, o1, o2): U1 U2 U3 U4 around x -> x+o1 d1 -> +o2 d2 -> -o1 d1
template <typename R>
__device__ __forceinline__ Q2<R> plaq_o(const LinkPlanes<SU2<R>, R> &Up, const Lat &L, const int *x, int d1, int d2,
                                        int o1, int o2) {
    int y[3] = {x[0], x[1], x[2]};
    Q2<R> P = link_o(Up, L, y, d1, o1);
    step_pos(L, y, d1, o1);
    P = SU2<R>::mul(P, link_o(Up, L, y, d2, o2));
    step_pos(L, y, d2, o2);
    P = SU2<R>::mul(P, link_o(Up, L, y, d1, -o1));
    step_pos(L, y, d1, -o1);
    return SU2<R>::mul(P, link_o(Up, L, y, d2, -o2));
}

template <typename R>
__global__ void __launch_bounds__(RED_THREADS) k_projected_poynting(const R *__restrict__ U, const R *__restrict__ Unext,
                                                                    const R *__restrict__ E, Lat L, int dir,
                                                                    double *__restrict__ part) {
    using G = SU2<R>;
    const LinkPlanes<G, R> Up{const_cast<R *>(U), L.V}, Unp{const_cast<R *>(Unext), L.V};
    const AlgPlanes<3, R> Ep{const_cast<R *>(E), L.V};
    const int k = blockIdx.x, nsplit = gridDim.y;
    const int o1 = (dir + 1) % 3, o2 = (dir + 2) % 3;
    const long nt = L.V / L.n[dir];
    const double area = (double)L.V / (double)L.n[dir];
    const double sa = sqrt(area);
    KSum acc[2] = {{0, 0}, {0, 0}};
    for (long t = (long)blockIdx.y * blockDim.x + threadIdx.x; t < nt; t += (long)nsplit * blockDim.x) {
        int x[3];
        x[dir] = k;
        const int lo = (o1 > o2) ? o1 : o2, hi = (o1 > o2) ? o2 : o1;
        x[lo] = (int)(t % L.n[lo]);
        x[hi] = (int)(t / L.n[lo]);
        const long s = x[0] * L.stride[0] + x[1] * L.stride[1] + x[2];
        const Nbr nb = neighbours(L, s, x);
        double lavg = 0.0;
#pragma unroll 1
        for (int i = 0; i < 3; i++) {
            if (i == dir) continue;
            Q2<R> FG = G::zero();
#pragma unroll 1
            for (int tt = 0; tt < 2; tt++) {
                const LinkPlanes<G, R> &W = tt == 0 ? Up : Unp;
                G::add(FG, plaq_o(W, L, x, dir, i, 1, 1));
                G::add(FG, plaq_o(W, L, x, i, dir, -1, 1));
                G::add(FG, plaq_o(W, L, x, i, dir, 1, -1));
                G::add(FG, plaq_o(W, L, x, dir, i, -1, -1));
            }
            R F[3], e1[3], e2[3], e2t[3];
            G::proj(FG, F);
            const double ufF = 1.0 / ((L.a[i] * L.a[dir]) * L.g * sa);
            const double ufEB = 1.0 / ((L.g * L.a[i]) * sa);
            Ep.load_ro(i, s, e1);
            Ep.load_ro(i, nb.bwd[i], e2);
            G::act(e2, G::adj(Up.load(i, nb.bwd[i])), e2t);
            double dot = 0.0;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const double fv = (double)F[c] * (ufF / 8.0);
                const double ev = ((double)e1[c] + (double)e2t[c]) * (0.5 * ufEB);
                dot += ev * fv;
            }
            lavg += dot;
        }
        const int d1 = (dir + 1) % 3, d2 = (dir + 2) % 3;
        const double uf1 = 1.0 / ((L.g * L.a[d1]) * sa), uf2 = 1.0 / ((L.g * L.a[d2]) * sa);
        R E1[3], E2[3], b10[3], b11[3], b20[3], b21[3];
        Ep.load_ro(d1, s, E1);
        Ep.load_ro(d2, s, E2);
        field_b<G, R>(Up, L, s, nb, d1, b10);
        field_b<G, R>(Unp, L, s, nb, d1, b11);
        field_b<G, R>(Up, L, s, nb, d2, b20);
        field_b<G, R>(Unp, L, s, nb, d2, b21);
        double p12 = 0.0, p21 = 0.0;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const double B1 = ((double)b10[c] + (double)b11[c]) * (uf1 * 0.5);
            const double B2 = ((double)b20[c] + (double)b21[c]) * (uf2 * 0.5);
            p12 += ((double)E1[c] * uf1) * B2;
            p21 += ((double)E2[c] * uf2) * B1;
        }
        two_sum_add(acc[0], lavg);
        two_sum_add(acc[1], p12 - p21);
    }
    int q;
    KSum v = block_reduce<2>(acc, q);
    if (q >= 0) {
        const long o = (((long)k * nsplit + blockIdx.y) * 2 + q) * 2;
        part[o] = v.s;
        part[o + 1] = v.c;
    }
}

__global__ void k_poynting_final(const double *__restrict__ part, int nslices, int nsplit, double *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // i = q * nslices + k
    if (i >= 2 * nslices) return;
    const int q = i / nslices, k = i % nslices;
    KSum v{0.0, 0.0};
    for (int b = 0; b < nsplit; b++) {
        const long o = (((long)k * nsplit + b) * 2 + q) * 2;
        ksum_merge(v, KSum{part[o], part[o + 1]});
    }
    out[(long)q * nslices + k] = v.s + v.c;
}

int launch_projected_poynting(Ctx &c, int dir, double *out) {
    if (c.nc != 2) return OPX_ERR_UNSUPPORTED;
    const int ns = c.L.n[dir];
    const long nt = c.L.V / ns;
    int nsplit = (int)std::max<long>(1, std::min<long>(c.red_blocks / ns, nt / RED_THREADS));
    nsplit = std::max(1, std::min(nsplit, (int)(c.red_blocks * 4 / ns)));  // 4 doubles per (slice, split)
    if (c.prec == OPX_F64)
        k_projected_poynting<double><<<dim3(ns, nsplit), RED_THREADS, 0, c.stream>>>(
            (const double *)c.U, (const double *)c.Unext, (const double *)c.E, c.L, dir, c.red_part);
    else
        k_projected_poynting<float><<<dim3(ns, nsplit), RED_THREADS, 0, c.stream>>>(
            (const float *)c.U, (const float *)c.Unext, (const float *)c.E, c.L, dir, c.red_part);
    k_poynting_final<<<grid_for(2L * ns, 128), 128, 0, c.stream>>>(c.red_part, ns, nsplit, out);
    c.launches += 2;
    return OPX_OK;
}

template <int NC, typename R>
__global__ void k_gauss_field(const R *__restrict__ U, const R *__restrict__ E, const R *__restrict__ rho, Lat L,
                              double *__restrict__ out) {
    using G = typename GroupOf<NC, R>::T;
    constexpr int NA = G::NA;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    const LinkPlanes<G, R> Up{const_cast<R *>(U), L.V};
    const AlgPlanes<NA, R> Ep{const_cast<R *>(E), L.V};
    int x[3];
    site_coords(L, s, x);
    const Nbr nb = neighbours(L, s, x);
    R gs[NA];
    gauss_site<G, R>(Up, Ep, rho, L, s, nb, gs);
#pragma unroll
    for (int a = 0; a < NA; a++) out[s * NA + a] = (double)gs[a];
}

#define OPX_DISPATCH(fn, ...)                                              \
    do {                                                                   \
        if (c.nc == 2) {                                                   \
            if (c.prec == OPX_F64) fn<2, double>(__VA_ARGS__);             \
            else fn<2, float>(__VA_ARGS__);                                \
        } else {                                                           \
            if (c.prec == OPX_F64) fn<3, double>(__VA_ARGS__);             \
            else fn<3, float>(__VA_ARGS__);                                \
        }                                                                  \
    } while (0)

template <int NC, typename R>
static void energy_density_t(Ctx &c, double *out) {
    k_energy_density<NC, R><<<grid_for(c.L.V, 128), 128, 0, c.stream>>>((const R *)c.U, (const R *)c.Unext,
                                                                        (const R *)c.E, c.eval, c.L, out);
    c.launches++;
}
void launch_energy_density(Ctx &c, double *out) { OPX_DISPATCH(energy_density_t, c, out); }

template <int NC, typename R>
static void projected_energy_t(Ctx &c, int dir, int skip_u, const double *bn_site, double *out) {
    // split each slice over enough blocks to fill the GPU, within the partial
    // buffer (2 * BULK_COLUMNS * max(red_blocks, 2 (n0 + n1 + n2)) doubles; 12
    // doubles per (slice, split))
    const int ns = c.L.n[dir];
    const long nt = c.L.V / ns;
    const long cap = 2L * BULK_COLUMNS * std::max(c.red_blocks, 2 * c.L.n[0] + 2 * c.L.n[1] + 2 * c.L.n[2]);
    int nsplit = (int)std::max<long>(1, std::min<long>(c.red_blocks / ns, nt / RED_THREADS));
    nsplit = (int)std::min<long>(nsplit, cap / (2L * PROJ_COLUMNS * ns));
    nsplit = std::max(nsplit, 1);
    k_projected_energy<NC, R><<<dim3(ns, nsplit), RED_THREADS, 0, c.stream>>>(
        (const R *)c.U, (const R *)c.Unext, (const R *)c.E, c.eval, c.L, dir, skip_u, bn_site, c.red_part);
    k_projected_final<<<grid_for((long)PROJ_COLUMNS * ns, 128), 128, 0, c.stream>>>(c.red_part, ns, nsplit, out);
    c.launches += 2;
}
void launch_projected_energy(Ctx &c, int dir, int skip_u, const double *bn_site, double *out) {
    OPX_DISPATCH(projected_energy_t, c, dir, skip_u, bn_site, out);
}

template <int NC, typename R>
static void gauss_field_t(Ctx &c, double *out) {
    k_gauss_field<NC, R><<<grid_for(c.L.V, 128), 128, 0, c.stream>>>((const R *)c.U, (const R *)c.E,
                                                                     (const R *)c.rho, c.L, out);
    c.launches++;
}
void launch_gauss_field(Ctx &c, double *out) { OPX_DISPATCH(gauss_field_t, c, out); }

}  // namespace opx
