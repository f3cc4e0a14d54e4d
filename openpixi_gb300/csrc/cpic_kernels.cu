// cpic_kernels.cu -- CPIC particle phases of one step on the device, bit-exact
// with the sequential reference.  Compiled with --fmad=false: every product and
// sum is rounded separately, in the reference's order, as Java evaluates it.
//
// Reference (physics/Simulation.java:386-421 for step, :318-347 for initialize):
//   reassign        YangMillsParticle.reassignValues (particles/YangMillsParticle.java:117-125)
//   charge density  CGCParticleInterpolationNGP.interpolateChargedensity (grid/CGCParticleInterpolationNGP.java:52-68)
//   positions       CGCParticleSolver.updatePosition (movement/solver/CGCParticleSolver.java:15-21),
//                   absorbing boundary is a no-op (AbsorbingParticleBoundaryConditions.java:31-40)
//   transport       CGCParticleInterpolationNGP.interpolateToParticle (:70-104)
//   charges         CGCParticleSolver.updateCharge (:24-36)
//   currents        CGCParticleInterpolationNGP.interpolateToGrid (:15-50)
//
// k_cpic_push does all per-particle work in one pass and emits (key, value)
// deposits.  The reference adds deposits into rho and J in particle-list order
// (synchronized adds, one thread).  To reproduce that order exactly the
// deposits are bucketed by key with a counting sort (count, exclusive scan,
// scatter), each bucket is put back into ascending particle order, and one
// thread per key sums its bucket sequentially starting from 0.0 (resetCharge /
// resetCurrent).  No floating-point atomics are used.
#include <cmath>

#include "internal.h"

namespace opx {

// Term order of SU3GroupElement.mult (math/SU3GroupElement.java:183-208):
// entry k of l*r is the left-to-right sum of sign * r[ai] * l[ei].
__constant__ signed char c_su3_terms[18][6][3] = {
    {{1, 0, 0}, {1, 3, 1}, {-1, 12, 10}, {-1, 15, 11}, {1, 6, 2}, {-1, 9, 9}},
    {{1, 1, 0}, {1, 4, 1}, {-1, 13, 10}, {-1, 16, 11}, {1, 7, 2}, {-1, 10, 9}},
    {{1, 2, 0}, {1, 5, 1}, {-1, 14, 10}, {-1, 17, 11}, {1, 8, 2}, {-1, 11, 9}},
    {{-1, 9, 12}, {-1, 12, 13}, {-1, 15, 14}, {1, 0, 3}, {1, 3, 4}, {1, 6, 5}},
    {{-1, 10, 12}, {-1, 13, 13}, {-1, 16, 14}, {1, 1, 3}, {1, 4, 4}, {1, 7, 5}},
    {{-1, 11, 12}, {-1, 14, 13}, {-1, 17, 14}, {1, 2, 3}, {1, 5, 4}, {1, 8, 5}},
    {{-1, 9, 15}, {-1, 12, 16}, {-1, 15, 17}, {1, 0, 6}, {1, 3, 7}, {1, 6, 8}},
    {{-1, 10, 15}, {-1, 13, 16}, {-1, 16, 17}, {1, 1, 6}, {1, 4, 7}, {1, 7, 8}},
    {{-1, 11, 15}, {-1, 14, 16}, {-1, 17, 17}, {1, 2, 6}, {1, 5, 7}, {1, 8, 8}},
    {{1, 9, 0}, {1, 12, 1}, {1, 3, 10}, {1, 6, 11}, {1, 15, 2}, {1, 0, 9}},
    {{1, 10, 0}, {1, 13, 1}, {1, 4, 10}, {1, 7, 11}, {1, 16, 2}, {1, 1, 9}},
    {{1, 11, 0}, {1, 14, 1}, {1, 5, 10}, {1, 8, 11}, {1, 17, 2}, {1, 2, 9}},
    {{1, 0, 12}, {1, 3, 13}, {1, 6, 14}, {1, 9, 3}, {1, 12, 4}, {1, 15, 5}},
    {{1, 1, 12}, {1, 4, 13}, {1, 7, 14}, {1, 10, 3}, {1, 13, 4}, {1, 16, 5}},
    {{1, 2, 12}, {1, 5, 13}, {1, 8, 14}, {1, 11, 3}, {1, 14, 4}, {1, 17, 5}},
    {{1, 0, 15}, {1, 3, 16}, {1, 6, 17}, {1, 9, 6}, {1, 12, 7}, {1, 15, 8}},
    {{1, 1, 15}, {1, 4, 16}, {1, 7, 17}, {1, 10, 6}, {1, 13, 7}, {1, 16, 8}},
    {{1, 2, 15}, {1, 5, 16}, {1, 8, 17}, {1, 11, 6}, {1, 14, 7}, {1, 17, 8}},
};

__device__ void ref_su3_mult(const double *l, const double *r, double *out) {
    for (int k = 0; k < 18; k++) {
        const signed char *t = c_su3_terms[k][0];
        double acc = (t[0] < 0 ? -r[t[1]] : r[t[1]]) * l[t[2]];
        for (int m = 1; m < 6; m++) {
            const signed char *u = c_su3_terms[k][m];
            double prod = r[u[1]] * l[u[2]];
            acc = u[0] < 0 ? acc - prod : acc + prod;
        }
        out[k] = acc;
    }
}

__device__ void ref_su3_adj(const double *e, double *b) {
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            b[3 * i + j] = e[3 * j + i];
            b[9 + 3 * i + j] = -e[9 + 3 * j + i];
        }
}

// SU3AlgebraElement.act (math/SU3AlgebraElement.java:144-168) on the 9-entry layout
__device__ void ref_su3_act(const double *v, const double *a, double *f) {
    double temp[18] = {v[0], v[1], v[2], v[1], v[4], v[5], v[2], v[5], v[8],
                       0, -v[3], -v[6], v[3], 0, -v[7], v[6], v[7], 0};
    double aadj[18], t1[18], t2[18];
    ref_su3_adj(a, aadj);
    ref_su3_mult(temp, aadj, t1);
    ref_su3_mult(a, t1, t2);
    f[0] = t2[0];
    f[4] = t2[4];
    f[8] = t2[8];
    f[1] = (t2[1] + t2[3]) / 2;
    f[2] = (t2[2] + t2[6]) / 2;
    f[5] = (t2[5] + t2[7]) / 2;
    f[3] = (t2[12] - t2[10]) / 2;
    f[6] = (t2[15] - t2[11]) / 2;
    f[7] = (t2[16] - t2[14]) / 2;
}

// SU2GroupElement.mult (math/SU2GroupElement.java:206-217)
__device__ void ref_su2_mult(const double *x, const double *a, double *b) {
    double b0 = x[0] * a[0] - x[1] * a[1] - x[2] * a[2] - x[3] * a[3];
    double b1 = x[0] * a[1] + x[1] * a[0] - x[2] * a[3] + x[3] * a[2];
    double b2 = x[0] * a[2] + x[2] * a[0] - x[3] * a[1] + x[1] * a[3];
    double b3 = x[0] * a[3] + x[3] * a[0] - x[1] * a[2] + x[2] * a[1];
    b[0] = b0; b[1] = b1; b[2] = b2; b[3] = b3;
}

// SU2AlgebraElement.act (math/SU2AlgebraElement.java:159-172)
__device__ void ref_su2_act(const double *v, const double *u, double *out) {
    double xm[4] = {0.0, v[0] / 2, v[1] / 2, v[2] / 2};
    double ua[4] = {u[0], -u[1], -u[2], -u[3]};
    double t[4], r[4];
    ref_su2_mult(xm, ua, t);
    ref_su2_mult(u, t, r);
    out[0] = 2 * r[1];
    out[1] = 2 * r[2];
    out[2] = 2 * r[3];
}

// Grid.getCellIndex with the periodic wrap (physics/grid/Grid.java:779-786)
__device__ __forceinline__ int cpic_cell(const Lat &L, int c0, int c1, int c2) {
    int r0 = c0 % L.n[0], r1 = c1 % L.n[1], r2 = c2 % L.n[2];
    r0 += r0 < 0 ? L.n[0] : 0;
    r1 += r1 < 0 ? L.n[1] : 0;
    r2 += r2 < 0 ? L.n[2] : 0;
    return (r0 * L.n[1] + r1) * L.n[2] + r2;
}

// (int) Math.rint(p / a) (GridFunctions.nearestGridPoint, physics/util/GridFunctions.java:67-73)
// with the correctly rounded quotient, dividing only where it can matter.  For
// a = 1 the quotient is p.  Otherwise q = p * (1/a) is within 3.01 u |q| of the
// correctly rounded p / a (u = 2^-53: one rounding in 1/a, one in the product,
// against one in the quotient); rint maps every value strictly between two
// consecutive half-integers to the same integer, so rint(q) is the reference's
// result unless a half-integer lies within that distance of q (the fraction
// itself is formed with an error below u), and then the quotient is formed.
// GB300's FP64 division is a dozen FP64 instructions at 1/64 of the FP32 rate.
__device__ __forceinline__ int ngp_index(double p, double a, double inv_a) {
    if (a == 1.0) return (int)rint(p);
    const double q = p * inv_a;
    const double h = fabs((q - floor(q)) - 0.5);
    if (h > 1e-15 * (fabs(q) + 1.0)) return (int)rint(q);
    return (int)rint(p / a);
}

__device__ __forceinline__ int sel3(int a0, int a1, int a2, int d) { return d == 0 ? a0 : (d == 1 ? a1 : a2); }
__device__ __forceinline__ double sel3(double a0, double a1, double a2, int d) {
    return d == 0 ? a0 : (d == 1 ? a1 : a2);
}

// Per-direction constants of the push, formed on the host with the same IEEE
// divisions the reference makes: 1/a_i, and a_d / dt of the current
// (CGCParticleInterpolationNGP.java:43,46; (-a)/dt = -(a/dt) exactly).
struct CpicConst {
    double inv_a[3], a_dt[3];
};

template <int NC>
__global__ void __launch_bounds__(256) k_cpic_push(Particles P, const double *__restrict__ Unext, Lat L,
                                                   CpicConst K, int reassign) {
    constexpr int NG = NC == 3 ? 18 : 4;
    constexpr int NAR = NC == 3 ? 9 : 3;
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long n = P.n;
    if (k >= n) return;
    const double *__restrict__ pin = reassign ? P.pos1 : P.pos0;
    const double *__restrict__ qa = reassign ? P.q1 : P.q0;
    const double *__restrict__ qb = reassign ? P.q0 : P.q1;
    double p0[3], p1[3], vel[3], q0[NAR], q1[NAR];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        p0[i] = pin[i * n + k];
        vel[i] = P.vel[i * n + k];
    }
#pragma unroll
    for (int a = 0; a < NAR; a++) {
        q0[a] = qa[a * n + k];
        q1[a] = qb[a * n + k];
    }
    const int d = P.dir[k];
    // nearest grid points before and after the move
    int o[3], m[3];
#pragma unroll
    for (int i = 0; i < 3; i++) o[i] = ngp_index(p0[i], L.a[i], K.inv_a[i]);
#pragma unroll
    for (int i = 0; i < 3; i++) p1[i] = p0[i] + vel[i] * L.dt;
#pragma unroll
    for (int i = 0; i < 3; i++) m[i] = ngp_index(p1[i], L.a[i], K.inv_a[i]);
    const int cell_old = cpic_cell(L, o[0], o[1], o[2]);
    P.key_rho[k] = cell_old;
#pragma unroll
    for (int a = 0; a < NAR; a++) P.val_rho[a * n + k] = q0[a];
    double Q0n[NAR], Q1n[NAR];
    int keyj = -1;
    if (sel3(o[0], o[1], o[2], d) != sel3(m[0], m[1], m[2], d)) {
        const int cell_new = cpic_cell(L, m[0], m[1], m[2]);
        const double vd = sel3(vel[0], vel[1], vel[2], d);
        // P.U: Unext(old) for v > 0, Unext(new)^dagger otherwise; the charge
        // update uses U^dagger, i.e. Unext(old)^dagger or Unext(new).
        double Uadj[NG], U[NG];
        const long cl = vd > 0 ? cell_old : cell_new;
#pragma unroll
        for (int c = 0; c < NG; c++) U[c] = Unext[link_offset(L.V, NG, d, c, cl)];
        if (vd > 0) {
            if (NC == 3) ref_su3_adj(U, Uadj);
            else { Uadj[0] = U[0]; Uadj[1] = -U[1]; Uadj[2] = -U[2]; Uadj[3] = -U[3]; }
        } else {
            // (U^dagger)^dagger = U exactly
#pragma unroll
            for (int c = 0; c < NG; c++) Uadj[c] = U[c];
        }
#pragma unroll
        for (int a = 0; a < NAR; a++) Q0n[a] = q0[a];
        if (NC == 3) ref_su3_act(q0, Uadj, Q1n);
        else ref_su2_act(q0, Uadj, Q1n);
        const double f = sel3(K.a_dt[0], K.a_dt[1], K.a_dt[2], d);
        if (vd > 0) {
            keyj = cell_old * 3 + d;
#pragma unroll
            for (int a = 0; a < NAR; a++) P.val_j[a * n + k] = Q0n[a] * f;
        } else {
            keyj = cell_new * 3 + d;
#pragma unroll
            for (int a = 0; a < NAR; a++) P.val_j[a * n + k] = Q1n[a] * -f;
        }
    } else {
        // no cell change: Q0 and Q1 swap back (CGCParticleSolver.java:30-35)
#pragma unroll
        for (int a = 0; a < NAR; a++) { Q0n[a] = q1[a]; Q1n[a] = q0[a]; }
    }
    P.key_j[k] = keyj;
    // bucket sizes of the counting sort (the buckets are empty on entry)
    atomicAdd(&P.count[cell_old], 1);
    if (keyj >= 0) atomicAdd(&P.count[L.V + keyj], 1);
#pragma unroll
    for (int i = 0; i < 3; i++) { P.pos0[i * n + k] = p0[i]; P.pos1[i * n + k] = p1[i]; }
#pragma unroll
    for (int a = 0; a < NAR; a++) { P.q0[a * n + k] = Q0n[a]; P.q1[a * n + k] = Q1n[a]; }
}

// Places each particle in its buckets: bucket sizes count down to zero, so
// they are empty again for the next step, and a bucket's entries fill
// [offset[key], offset[key + 1]) in some order (the segmented sum restores
// the particle order).
__global__ void k_cpic_scatter(Particles P, long V) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.n) return;
    const int kr = P.key_rho[k];
    P.slots[P.offset[kr] + atomicSub(&P.count[kr], 1) - 1] = (int)k;
    const int kj = P.key_j[k];
    if (kj >= 0) P.slots[P.offset[V + kj] + atomicSub(&P.count[V + kj], 1) - 1] = (int)k;
}

// one thread per key: keys [0,V) are rho cells, [V, 4V) are (cell*3 + dir) of J
template <int NC>
__global__ void k_cpic_segsum(Particles P, long V, double *__restrict__ rho, double *__restrict__ J) {
    constexpr int NAR = NC == 3 ? 9 : 3;
    constexpr int NA = NC == 3 ? 8 : 3;
    const long key = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (key >= 4 * V) return;
    const int beg = P.offset[key], cnt = P.offset[key + 1] - beg;
    int *seg = P.slots + beg;
    // ascending particle index (buckets hold a handful of entries)
    for (int i = 1; i < cnt; i++) {
        int v = seg[i], j = i - 1;
        while (j >= 0 && seg[j] > v) { seg[j + 1] = seg[j]; j--; }
        seg[j + 1] = v;
    }
    const bool is_rho = key < V;
    const double *val = is_rho ? P.val_rho : P.val_j;
    double acc[NAR];
    for (int a = 0; a < NAR; a++) acc[a] = 0.0;
    for (int i = 0; i < cnt; i++) {
        const long k = seg[i];
        for (int a = 0; a < NAR; a++) acc[a] = acc[a] + val[a * P.n + k];
    }
    double g[NA];
    if (NC == 3) {
        // SU3AlgebraElement.get(a) (math/SU3AlgebraElement.java:117-129)
        const double s3 = 1.7320508075688772;
        g[0] = 2 * acc[1]; g[1] = 2 * acc[3]; g[2] = acc[0] - acc[4]; g[3] = 2 * acc[2];
        g[4] = 2 * acc[6]; g[5] = 2 * acc[5]; g[6] = 2 * acc[7];
        g[NA - 1] = (acc[0] + acc[4] - 2 * acc[8]) / s3;
    } else {
        for (int a = 0; a < NA; a++) g[a] = acc[a];
    }
    if (is_rho) {
        for (int a = 0; a < NA; a++) rho[(long)a * V + key] = g[a];
    } else {
        const long kk = key - V, cell = kk / 3;
        const int d = (int)(kk - cell * 3);
        for (int a = 0; a < NA; a++) J[((long)d * NA + a) * V + cell] = g[a];
    }
}

// ---- exclusive scan of int counts (three phases) ----
// A block scans SCAN_B * 4 counts, four per thread: each thread's four, then
// the threads' totals by warp shuffles and the warps' totals in shared memory.
constexpr int SCAN_B = 1024, SCAN_PER = 4, SCAN_TILE = SCAN_B * SCAN_PER;

// exclusive prefix of v over the block (all SCAN_B threads take part); total = the block's sum
__device__ __forceinline__ int block_exclusive_scan(int v, int &total) {
    __shared__ int warp_tot[SCAN_B / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        warp_tot[lane] = t;  // inclusive over warps
    }
    __syncthreads();
    total = warp_tot[SCAN_B / 32 - 1];
    const int before = w > 0 ? warp_tot[w - 1] : 0;
    __syncthreads();  // warp_tot is reused by the next call
    return before + x - v;
}

__global__ void __launch_bounds__(SCAN_B) k_scan_block(const int *__restrict__ in, int *__restrict__ out,
                                                       int *__restrict__ sums, long n) {
    const long base = (long)blockIdx.x * SCAN_TILE + (long)threadIdx.x * SCAN_PER;
    int v[SCAN_PER], t = 0;
#pragma unroll
    for (int j = 0; j < SCAN_PER; j++) {
        v[j] = base + j < n ? in[base + j] : 0;
        t += v[j];
    }
    int total;
    int run = block_exclusive_scan(t, total);
#pragma unroll
    for (int j = 0; j < SCAN_PER; j++) {
        if (base + j < n) out[base + j] = run;
        run += v[j];
    }
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// one block: exclusive scan of the block sums, in chunks of SCAN_TILE with a carry
__global__ void __launch_bounds__(SCAN_B) k_scan_sums(int *__restrict__ sums, long nb) {
    int carry = 0;
    for (long chunk = 0; chunk < nb; chunk += SCAN_TILE) {
        const long base = chunk + (long)threadIdx.x * SCAN_PER;
        int v[SCAN_PER], t = 0;
#pragma unroll
        for (int j = 0; j < SCAN_PER; j++) {
            v[j] = base + j < nb ? sums[base + j] : 0;
            t += v[j];
        }
        int total;
        int run = carry + block_exclusive_scan(t, total);
#pragma unroll
        for (int j = 0; j < SCAN_PER; j++) {
            if (base + j < nb) sums[base + j] = run;
            run += v[j];
        }
        carry += total;
    }
}

__global__ void __launch_bounds__(SCAN_B) k_scan_add(int *__restrict__ out, const int *__restrict__ sums, long n) {
    const int add = sums[blockIdx.x];
    const long base = (long)blockIdx.x * SCAN_TILE + threadIdx.x;
#pragma unroll
    for (int j = 0; j < SCAN_PER; j++) {
        const long i = base + (long)j * SCAN_B;
        if (i < n) out[i] += add;
    }
}

int cpic_alloc(Ctx &c, long n) {
    Particles &P = c.P;
    const long V = c.L.V;
    if (n <= P.cap && P.count) { P.n = n; return OPX_OK; }
    cpic_free(c);
    const long cap = n > 0 ? n : 1;
    const int nar = c.na_ref;
    bool ok = true;
    auto al = [&](void **p, size_t bytes) { if (cudaMalloc(p, bytes) != cudaSuccess) { ok = false; *p = nullptr; } };
    al((void **)&P.pos0, sizeof(double) * 3 * cap);
    al((void **)&P.pos1, sizeof(double) * 3 * cap);
    al((void **)&P.vel, sizeof(double) * 3 * cap);
    al((void **)&P.q0, sizeof(double) * nar * cap);
    al((void **)&P.q1, sizeof(double) * nar * cap);
    al((void **)&P.dir, sizeof(int8_t) * cap);
    al((void **)&P.key_rho, sizeof(int) * cap);
    al((void **)&P.key_j, sizeof(int) * cap);
    al((void **)&P.val_rho, sizeof(double) * nar * cap);
    al((void **)&P.val_j, sizeof(double) * nar * cap);
    // bucket sizes (zero between steps) and their exclusive scan over 4V + 1 keys
    al((void **)&P.count, sizeof(int) * (4 * V + 1));
    al((void **)&P.offset, sizeof(int) * (4 * V + 1));
    al((void **)&P.slots, sizeof(int) * 2 * cap);
    P.scan_tmp_len = (4 * V + 1 + SCAN_TILE - 1) / SCAN_TILE;
    al((void **)&P.scan_tmp, sizeof(int) * P.scan_tmp_len);
    if (ok && cudaMemset(P.count, 0, sizeof(int) * (4 * V + 1)) != cudaSuccess) ok = false;
    if (!ok) { cpic_free(c); c.err = "particle buffers: out of device memory"; return OPX_ERR_NOMEM; }
    P.cap = cap;
    P.n = n;
    return OPX_OK;
}

void cpic_free(Ctx &c) {
    Particles &P = c.P;
    void *ptrs[] = {P.pos0, P.pos1, P.vel, P.q0, P.q1, P.dir, P.key_rho, P.key_j, P.val_rho,
                    P.val_j, P.count, P.offset, P.slots, P.scan_tmp};
    for (void *p : ptrs) if (p) cudaFree(p);
    P = Particles{};
}

void launch_cpic_phases(Ctx &c, int reassign) {
    Particles &P = c.P;
    c.rho_nonzero = true;
    const long V = c.L.V;
    const int B = 256;
    if (P.n == 0) {
        cudaMemsetAsync(c.rho, 0, sizeof(double) * c.na * V, c.stream);
        cudaMemsetAsync(c.J, 0, sizeof(double) * c.na * 3 * V, c.stream);
        return;
    }
    const int gp = grid_for(P.n, B);
    CpicConst K;
    for (int i = 0; i < 3; i++) {
        K.inv_a[i] = 1.0 / c.L.a[i];
        K.a_dt[i] = c.L.a[i] / c.L.dt;
    }
    if (c.nc == 3) k_cpic_push<3><<<gp, B, 0, c.stream>>>(P, (const double *)c.Unext, c.L, K, reassign);
    else k_cpic_push<2><<<gp, B, 0, c.stream>>>(P, (const double *)c.Unext, c.L, K, reassign);
    const long n4 = 4 * V;
    const long nb = (n4 + 1 + SCAN_TILE - 1) / SCAN_TILE;
    k_scan_block<<<(int)nb, SCAN_B, 0, c.stream>>>(P.count, P.offset, P.scan_tmp, n4 + 1);
    k_scan_sums<<<1, SCAN_B, 0, c.stream>>>(P.scan_tmp, nb);
    k_scan_add<<<(int)nb, SCAN_B, 0, c.stream>>>(P.offset, P.scan_tmp, n4 + 1);
    k_cpic_scatter<<<gp, B, 0, c.stream>>>(P, V);
    if (c.nc == 3) k_cpic_segsum<3><<<grid_for(n4, B), B, 0, c.stream>>>(P, V, (double *)c.rho, (double *)c.J);
    else k_cpic_segsum<2><<<grid_for(n4, B), B, 0, c.stream>>>(P, V, (double *)c.rho, (double *)c.J);
    c.launches += 6;
    c.j_nonzero = true;
}

// ---------------------------------------------------------------- super particles
// CGCSuperParticleInterpolationNGP (physics/grid/CGCSuperParticleInterpolationNGP.java):
// the particles move along direction 0 with fixed relative positions; super
// particle k of a group is a block of charges whose global cell index is
// offset_k(t) + j.  The reference adds the super particles into rho and J in
// list order (group by group, and within a group subdivision by subdivision,
// k = 0 .. ppc-1); every cell then receives its terms in (group, k) order, the
// order of the loops below, whatever the subdivision.  One thread per cell sums
// them from 0.0, so the deposits are bit-exact.
constexpr int SUPER_MAX = 64;
struct SuperStep {
    int m;                       // entries = groups x ppc, list order
    long off[SUPER_MAX];         // offset_k(t) (current, or NGP for the charge density)
    long n[SUPER_MAX];
    const double *Q[SUPER_MAX];  // [na_ref][n] of this (group, k)
    int orient[SUPER_MAX];
    int upd[SUPER_MAX];          // needsUpdate(t)
};

template <int NC>
__device__ __forceinline__ void ref_to_gen(const double *acc, double *g) {
    if (NC == 3) {
        // SU3AlgebraElement.get(a) (math/SU3AlgebraElement.java:117-129)
        const double s3 = 1.7320508075688772;
        g[0] = 2 * acc[1]; g[1] = 2 * acc[3]; g[2] = acc[0] - acc[4]; g[3] = 2 * acc[2];
        g[4] = 2 * acc[6]; g[5] = 2 * acc[5]; g[6] = 2 * acc[7];
        g[7] = (acc[0] + acc[4] - 2 * acc[8]) / s3;
    } else {
        g[0] = acc[0]; g[1] = acc[1]; g[2] = acc[2];
    }
}

template <int NC>
__device__ __forceinline__ void ref_act(const double *v, const double *u, double *out) {
    if (NC == 3) ref_su3_act(v, u, out); else ref_su2_act(v, u, out);
}
template <int NC>
__device__ __forceinline__ void ref_adj(const double *u, double *out) {
    if (NC == 3) ref_su3_adj(u, out);
    else { out[0] = u[0]; out[1] = -u[1]; out[2] = -u[2]; out[3] = -u[3]; }
}

// interpolateChargedensity (:75-93)
template <int NC>
__global__ void k_super_cin(SuperStep S, long V, double *__restrict__ rho) {
    constexpr int NAR = NC == 3 ? 9 : 3, NA = NC == 3 ? 8 : 3;
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= V) return;
    double acc[NAR];
    for (int a = 0; a < NAR; a++) acc[a] = 0.0;
    for (int e = 0; e < S.m; e++) {
        const long j = c - S.off[e];
        if (j < 0 || j >= S.n[e]) continue;
        for (int a = 0; a < NAR; a++) acc[a] = acc[a] + S.Q[e][(long)a * S.n[e] + j];
    }
    double g[NA];
    ref_to_gen<NC>(acc, g);
    for (int a = 0; a < NA; a++) rho[(long)a * V + c] = g[a];
}

// interpolateToGrid (:19-73), the current along direction 0.  Orientation +1:
// J(index + quickfix) += Q (as/at) with Q before its transport; orientation -1:
// J(index) += (U Q U^dagger) (-as/at), U = Unext_0(index).  quickfix = one
// plane when one particle sits in a cell (ppc = 1), and the last quickfix
// cells are excluded for both orientations, as in the reference.
template <int NC>
__global__ void k_super_jin(SuperStep S, long V, long qf, double f, const double *__restrict__ Unext,
                            double *__restrict__ J) {
    constexpr int NAR = NC == 3 ? 9 : 3, NA = NC == 3 ? 8 : 3, NG = NC == 3 ? 18 : 4;
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= V) return;
    double acc[NAR];
    for (int a = 0; a < NAR; a++) acc[a] = 0.0;
    for (int e = 0; e < S.m; e++) {
        if (!S.upd[e]) continue;
        if (S.orient[e] > 0) {
            const long index = c - qf, j = index - S.off[e];
            if (j < 0 || j >= S.n[e] || index < 0 || index >= V - qf) continue;
            for (int a = 0; a < NAR; a++) acc[a] = acc[a] + S.Q[e][(long)a * S.n[e] + j] * f;
        } else {
            const long index = c, j = index - S.off[e];
            if (j < 0 || j >= S.n[e] || index >= V - qf) continue;
            double q[NAR], u[NG], t[NAR];
            for (int a = 0; a < NAR; a++) q[a] = S.Q[e][(long)a * S.n[e] + j];
            for (int k = 0; k < NG; k++) u[k] = Unext[link_offset(V, NG, 0, k, index)];
            ref_act<NC>(q, u, t);
            for (int a = 0; a < NAR; a++) acc[a] = acc[a] + t[a] * -f;
        }
    }
    double g[NA];
    ref_to_gen<NC>(acc, g);
    for (int a = 0; a < NA; a++) J[(long)a * V + c] = g[a];
}

// the parallel transport of the charges that crossed (:59-60, :66-67)
template <int NC>
__global__ void k_super_transport(double *__restrict__ Q, long n, long off, int orientation, long V, long qf,
                                  const double *__restrict__ Unext) {
    constexpr int NAR = NC == 3 ? 9 : 3, NG = NC == 3 ? 18 : 4;
    const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const long index = off + j;
    if (index < 0 || index >= V - qf) return;
    double q[NAR], u[NG], ua[NG], t[NAR];
    for (int a = 0; a < NAR; a++) q[a] = Q[(long)a * n + j];
    for (int k = 0; k < NG; k++) u[k] = Unext[link_offset(V, NG, 0, k, index)];
    if (orientation > 0) {
        ref_adj<NC>(u, ua);
        ref_act<NC>(q, ua, t);
    } else {
        ref_act<NC>(q, u, t);
    }
    for (int a = 0; a < NAR; a++) Q[(long)a * n + j] = t[a];
}

// CGCSuperParticle.getCurrentOffset / getCurrentNGPOffset / needsUpdate (:71-105)
static long super_offset(int orientation, long base, int shift, int ppc, long ppp, long t) {
    if (orientation > 0) return base + ((t + shift) / ppc) * ppp;
    return base + (long)std::floor((-t + shift) / (1.0 * ppc)) * ppp;
}
static long super_ngp_offset(int orientation, long base, int shift, int ppc, long ppp, long t) {
    const long cur = super_offset(orientation, base, shift, ppc, ppp, t);
    if (orientation > 0) return cur + ((((t + shift) % ppc) < ppc / 2) ? 0 : ppp);
    return cur + ((((t - shift + ppc + ppc / 2 - 1) % ppc) < ppc / 2) ? 0 : ppp);
}
static bool super_needs_update(int orientation, int shift, int ppc, long t) {
    if (orientation > 0) return 0 == (t + shift + ppc / 2 + 1) % ppc;
    return 0 == (t - shift + ppc / 2) % ppc;
}

void launch_super_phases(Ctx &c, long t) {
    c.rho_nonzero = true;
    const long V = c.L.V, ntr = V / c.L.n[0];
    const int ppc = c.sg_ppc, nar = c.na_ref;
    SuperStep cin{}, jin{};
    int m = 0;
    for (const SuperGroup &G : c.sg)
        for (int k = 0; k < ppc && m < SUPER_MAX; k++, m++) {
            const double *Qk = G.Q + (size_t)k * nar * G.n;
            cin.off[m] = super_ngp_offset(G.orientation, G.base, k, ppc, ntr, t);
            jin.off[m] = super_offset(G.orientation, G.base, k, ppc, ntr, t);
            cin.n[m] = jin.n[m] = G.n;
            cin.Q[m] = jin.Q[m] = Qk;
            cin.orient[m] = jin.orient[m] = G.orientation;
            cin.upd[m] = 1;
            jin.upd[m] = super_needs_update(G.orientation, k, ppc, t) ? 1 : 0;
        }
    cin.m = jin.m = m;
    const int B = 256;
    const long qf = ppc == 1 ? ntr : 0;
    const double f = c.L.a[0] / c.L.dt;
    double *rho = (double *)c.rho, *J = (double *)c.J;
    const double *Un = (const double *)c.Unext;
    // resetCharge + interpolateChargedensity
    if (c.nc == 3) k_super_cin<3><<<grid_for(V, B), B, 0, c.stream>>>(cin, V, rho);
    else k_super_cin<2><<<grid_for(V, B), B, 0, c.stream>>>(cin, V, rho);
    // resetCurrent + interpolateToGrid: J_0 from the crossing charges, then their transport
    cudaMemsetAsync(J + (size_t)c.na * V, 0, sizeof(double) * 2 * c.na * V, c.stream);
    if (c.nc == 3) k_super_jin<3><<<grid_for(V, B), B, 0, c.stream>>>(jin, V, qf, f, Un, J);
    else k_super_jin<2><<<grid_for(V, B), B, 0, c.stream>>>(jin, V, qf, f, Un, J);
    c.launches += 2;
    int e = 0;
    for (SuperGroup &G : c.sg)
        for (int k = 0; k < ppc && e < SUPER_MAX; k++, e++) {
            if (!jin.upd[e]) continue;
            double *Qk = G.Q + (size_t)k * nar * G.n;
            if (c.nc == 3)
                k_super_transport<3><<<grid_for(G.n, B), B, 0, c.stream>>>(Qk, G.n, jin.off[e], G.orientation, V, qf, Un);
            else
                k_super_transport<2><<<grid_for(G.n, B), B, 0, c.stream>>>(Qk, G.n, jin.off[e], G.orientation, V, qf, Un);
            c.launches++;
        }
    c.j_nonzero = true;
}

void super_free(Ctx &c) {
    for (SuperGroup &G : c.sg)
        if (G.Q) cudaFree(G.Q);
    c.sg.clear();
    c.sg_ppc = 0;
}

}  // namespace opx
