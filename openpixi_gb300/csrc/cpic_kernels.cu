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

__device__ __forceinline__ long cpic_cell(const Lat &L, const int *c) {
    long idx = 0;
    for (int i = 0; i < 3; i++) {
        long r = ((long)c[i] % L.n[i] + L.n[i]) % L.n[i];
        idx = i == 0 ? r : idx * L.n[i] + r;
    }
    return idx;
}

template <int NC>
__global__ void k_cpic_push(Particles P, const double *__restrict__ Unext, Lat L, int reassign) {
    constexpr int NG = NC == 3 ? 18 : 4;
    constexpr int NAR = NC == 3 ? 9 : 3;
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long n = P.n;
    if (k >= n) return;
    double p0[3], p1[3], vel[3], q0[NAR], q1[NAR];
    for (int i = 0; i < 3; i++) {
        p0[i] = reassign ? P.pos1[i * n + k] : P.pos0[i * n + k];
        vel[i] = P.vel[i * n + k];
    }
    for (int a = 0; a < NAR; a++) {
        q0[a] = reassign ? P.q1[a * n + k] : P.q0[a * n + k];
        q1[a] = reassign ? P.q0[a * n + k] : P.q1[a * n + k];
    }
    // nearest grid points: (int) Math.rint(pos / a) (physics/util/GridFunctions.java:67-73)
    int o[3], m[3];
    for (int i = 0; i < 3; i++) o[i] = (int)rint(p0[i] / L.a[i]);
    const long cell_old = cpic_cell(L, o);
    P.key_rho[k] = (int)cell_old;
    for (int a = 0; a < NAR; a++) P.val_rho[a * n + k] = q0[a];
    for (int i = 0; i < 3; i++) p1[i] = p0[i] + vel[i] * L.dt;
    for (int i = 0; i < 3; i++) m[i] = (int)rint(p1[i] / L.a[i]);
    const int d = P.dir[k];
    double Q0n[NAR], Q1n[NAR];
    int keyj = -1;
    if (o[d] != m[d]) {
        const long cell_new = cpic_cell(L, m);
        // P.U: Unext(old) for v > 0, Unext(new)^dagger otherwise; the charge
        // update uses U^dagger, i.e. Unext(old)^dagger or Unext(new).
        double Uadj[NG], U[NG];
        const long cl = P.vel[d * n + k] > 0 ? cell_old : cell_new;
        for (int c = 0; c < NG; c++) U[c] = Unext[link_offset(L.V, NG, d, c, cl)];
        if (vel[d] > 0) {
            if (NC == 3) ref_su3_adj(U, Uadj);
            else { Uadj[0] = U[0]; Uadj[1] = -U[1]; Uadj[2] = -U[2]; Uadj[3] = -U[3]; }
        } else {
            // (U^dagger)^dagger = U exactly
            for (int c = 0; c < NG; c++) Uadj[c] = U[c];
        }
        for (int a = 0; a < NAR; a++) Q0n[a] = q0[a];
        if (NC == 3) ref_su3_act(q0, Uadj, Q1n);
        else ref_su2_act(q0, Uadj, Q1n);
        if (vel[d] > 0) {
            const double f = L.a[d] / L.dt;
            keyj = (int)(cell_old * 3 + d);
            for (int a = 0; a < NAR; a++) P.val_j[a * n + k] = Q0n[a] * f;
        } else {
            const double f = -L.a[d] / L.dt;
            keyj = (int)(cell_new * 3 + d);
            for (int a = 0; a < NAR; a++) P.val_j[a * n + k] = Q1n[a] * f;
        }
    } else {
        // no cell change: Q0 and Q1 swap back (CGCParticleSolver.java:30-35)
        for (int a = 0; a < NAR; a++) { Q0n[a] = q1[a]; Q1n[a] = q0[a]; }
    }
    P.key_j[k] = keyj;
    for (int i = 0; i < 3; i++) { P.pos0[i * n + k] = p0[i]; P.pos1[i * n + k] = p1[i]; }
    for (int a = 0; a < NAR; a++) { P.q0[a * n + k] = Q0n[a]; P.q1[a * n + k] = Q1n[a]; }
}

__global__ void k_cpic_count(Particles P, long V) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.n) return;
    atomicAdd(&P.count[P.key_rho[k]], 1);
    if (P.key_j[k] >= 0) atomicAdd(&P.count[V + P.key_j[k]], 1);
}

__global__ void k_cpic_scatter(Particles P, long V) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.n) return;
    const int kr = P.key_rho[k];
    P.slots[P.offset[kr] + atomicAdd(&P.cursor[kr], 1)] = (int)k;
    const int kj = P.key_j[k];
    if (kj >= 0) P.slots[P.offset[V + kj] + atomicAdd(&P.cursor[V + kj], 1)] = (int)k;
}

// one thread per key: keys [0,V) are rho cells, [V, 4V) are (cell*3 + dir) of J
template <int NC>
__global__ void k_cpic_segsum(Particles P, long V, double *__restrict__ rho, double *__restrict__ J) {
    constexpr int NAR = NC == 3 ? 9 : 3;
    constexpr int NA = NC == 3 ? 8 : 3;
    const long key = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (key >= 4 * V) return;
    const int beg = P.offset[key], cnt = P.count[key];
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
constexpr int SCAN_B = 1024;
__global__ void k_scan_block(const int *__restrict__ in, int *__restrict__ out, int *__restrict__ sums, long n) {
    __shared__ int sh[SCAN_B];
    const long i = (long)blockIdx.x * SCAN_B + threadIdx.x;
    int v = i < n ? in[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < SCAN_B; o <<= 1) {
        int t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) out[i] = sh[threadIdx.x] - v;  // exclusive
    if (threadIdx.x == SCAN_B - 1) sums[blockIdx.x] = sh[SCAN_B - 1];
}
__global__ void k_scan_sums(int *__restrict__ sums, long nb) {
    // single block: exclusive scan of block sums with a running carry
    __shared__ int sh[SCAN_B];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (long base = 0; base < nb; base += SCAN_B) {
        const long i = base + threadIdx.x;
        int v = i < nb ? sums[i] : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < SCAN_B; o <<= 1) {
            int t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < nb) sums[i] = carry + sh[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == SCAN_B - 1) carry += sh[SCAN_B - 1];
        __syncthreads();
    }
}
__global__ void k_scan_add(int *__restrict__ out, const int *__restrict__ sums, long n) {
    const long i = (long)blockIdx.x * SCAN_B + threadIdx.x;
    if (i < n) out[i] += sums[blockIdx.x];
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
    al((void **)&P.count, sizeof(int) * 4 * V);
    al((void **)&P.offset, sizeof(int) * 4 * V);
    al((void **)&P.cursor, sizeof(int) * 4 * V);
    al((void **)&P.slots, sizeof(int) * 2 * cap);
    P.scan_tmp_len = (4 * V + SCAN_B - 1) / SCAN_B;
    al((void **)&P.scan_tmp, sizeof(int) * P.scan_tmp_len);
    if (!ok) { cpic_free(c); c.err = "particle buffers: out of device memory"; return OPX_ERR_NOMEM; }
    P.cap = cap;
    P.n = n;
    return OPX_OK;
}

void cpic_free(Ctx &c) {
    Particles &P = c.P;
    void *ptrs[] = {P.pos0, P.pos1, P.vel, P.q0, P.q1, P.dir, P.key_rho, P.key_j, P.val_rho,
                    P.val_j, P.count, P.offset, P.cursor, P.slots, P.scan_tmp};
    for (void *p : ptrs) if (p) cudaFree(p);
    P = Particles{};
}

void launch_cpic_phases(Ctx &c, int reassign) {
    Particles &P = c.P;
    const long V = c.L.V;
    const int B = 256;
    if (P.n == 0) {
        cudaMemsetAsync(c.rho, 0, sizeof(double) * c.na * V, c.stream);
        cudaMemsetAsync(c.J, 0, sizeof(double) * c.na * 3 * V, c.stream);
        return;
    }
    const int gp = grid_for(P.n, B);
    if (c.nc == 3) k_cpic_push<3><<<gp, B, 0, c.stream>>>(P, (const double *)c.Unext, c.L, reassign);
    else k_cpic_push<2><<<gp, B, 0, c.stream>>>(P, (const double *)c.Unext, c.L, reassign);
    cudaMemsetAsync(P.count, 0, sizeof(int) * 4 * V, c.stream);
    cudaMemsetAsync(P.cursor, 0, sizeof(int) * 4 * V, c.stream);
    k_cpic_count<<<gp, B, 0, c.stream>>>(P, V);
    const long n4 = 4 * V;
    const long nb = (n4 + SCAN_B - 1) / SCAN_B;
    k_scan_block<<<(int)nb, SCAN_B, 0, c.stream>>>(P.count, P.offset, P.scan_tmp, n4);
    k_scan_sums<<<1, SCAN_B, 0, c.stream>>>(P.scan_tmp, nb);
    k_scan_add<<<(int)nb, SCAN_B, 0, c.stream>>>(P.offset, P.scan_tmp, n4);
    k_cpic_scatter<<<gp, B, 0, c.stream>>>(P, V);
    if (c.nc == 3) k_cpic_segsum<3><<<grid_for(n4, B), B, 0, c.stream>>>(P, V, (double *)c.rho, (double *)c.J);
    else k_cpic_segsum<2><<<grid_for(n4, B), B, 0, c.stream>>>(P, V, (double *)c.rho, (double *)c.J);
    c.launches += 7;
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
