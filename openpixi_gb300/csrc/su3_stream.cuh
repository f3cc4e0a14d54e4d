// su3_stream.cuh -- the SU(3) FP32 leapfrog in plaquette form, streamed along
// dimension 0 (FastTYMSolver.CombinedUpdate, physics/fields/FastTYMSolver.java:40-63,
// with Grid.getStapleSum, physics/grid/Grid.java:675-696).
//
// The force on link i at x is proj(U_i(x) S_i(x)) with the staple sum S_i of
// getStapleSum.  Since proj is linear and commutes with conjugation by a
// unitary matrix, each staple's term is a plaquette term:
//   forward staple : proj(U_i(x) U_j(x+i) U_i(x+j)^dag U_j(x)^dag) = proj(P_ij(x))
//   backward staple: proj(U_i(x) (U_i(x-j) U_j(x+i-j))^dag U_j(x-j))
//                    = -Ad(U_j(x-j)^dag) proj(P_ij(x-j))
// with P_ij(x) = U_i(x) U_j(x+i) U_i(x+j)^dag U_j(x)^dag (Grid.getPlaquette),
// P_ji = P_ij^dag and Ad(g) X the generator components of g H(X) g^dag.  So
// for each site x and plane i < j, with X = proj(P_ij(x)) / a^2 factors:
//   F_i(x)   += X / a_j^2          F_j(x)   -= X / a_i^2
//   F_i(x+j) -= Ad(U_j(x)^dag) X / a_j^2
//   F_j(x+i) += Ad(U_i(x)^dag) X / a_i^2
// Per site: three plaquettes (three products, the last one only as far as
// proj reads it) and six transports, against eight staple products per link in
// the staple form: about 2.6 k instead of 3.9 k FMAs per site, and 9 link loads
// instead of 36.  E_i(x) += dt F_i(x) and Unext_i(x) = exp(-i dt E_i(x)) U_i(x)
// then follow as in the staple form.  Same physics, other FP32 rounding order.
//
// Work layout.  A block owns a tile of 8 (x1) x 32 (x2) columns and walks along
// x0 over a contiguous range of (tile, x0) units, the ranges of all blocks
// covering the lattice once (one wave of resident blocks, equal shares).  Per
// x0 plane, warps 0-3 take two tile sites each (rows w and w + 4, column =
// lane; links read as whole warp-sized blocks) and warp 4 takes the halo: row
// x1 = tile start - 1 (for the transports that cross into the tile along 1)
// and column x2 = tile start - 1 (along 2).  The transports cross into their
// neighbours through shared memory: along 1 and 2 within the plane (one
// barrier), along 0 into the same thread's next plane (its own slots, so no
// barrier).  A range starts with a prologue that forms the transports of the
// plane before it.  Sites are updated by exactly one block; E is read and
// written only at its own site, U is only read and Unext only written.
//
// Measured on GB300 (SU(3) FP32, 128^3): 0.72 ms per step against 0.44 ms for
// the paired staple form, with 20 % fewer instructions.  Each x0 step is a
// chain of dependent DRAM loads between two block barriers, and 10 resident
// warps per SM do not cover it (FMA pipe 26 %, long-scoreboard stalls 5.1 per
// issue).  The links of the next plane are re-read one step later, after the
// whole GPU has streamed about 50 MB through L2, and the tile edges are read
// by two blocks at different times, so DRAM reads are 2.5x the compulsory
// bytes.  It is therefore an opt-in form (OPX_STREAM_FP32=1), kept with its
// tests as the plaquette formulation of the update.
#pragma once
#include <cuda_runtime.h>

#include "su3_pair.cuh"

namespace opx {
namespace st {
using namespace pr;

constexpr int T1 = 8;    // tile rows (x1)
constexpr int T2 = 32;   // tile columns (x2): one warp-sized link block
constexpr int THREADS = 160;  // four warps of tile sites, one of halo sites

// Shared memory of one block (76.3 KB): the transports into the next site
// along 1 and 2 (written in the first phase of a plane, read after the
// barrier), each tile site's transports into its next plane along 0, and the
// tile sites' forces.
struct Smem {
    // W for x + 1: kind 0 = Ad(U_1(x)^dag) X_01(x), kind 1 = Ad(U_1(x)^dag) X_12(x);
    // index row + 1 holds tile row `row`, index 0 the halo row
    float wx1[2][8][T1 + 1][T2];
    // W for x + 2: kind 0 = Ad(U_2(x)^dag) X_02(x), kind 1 = Ad(U_2(x)^dag) X_12(x);
    // index col + 1 holds tile column `col`, index 0 the halo column
    float wx2[2][8][T1][T2 + 1];
    // W for x + 0: kind 0 = Ad(U_0(x)^dag) X_01(x), kind 1 = Ad(U_0(x)^dag) X_02(x)
    float carry[2][8][T1][T2];
    // the force F_i of each tile site, accumulated over the plane's terms
    float fs[3][8][T1][T2];
};

// Links of the two lanes' sites, each lane with its own direction.
__device__ __forceinline__ M load_dd(const float *__restrict__ U, int nblk, int da, int sa, int db, int sb) {
    const float *a = U + loff<int>(nblk, da, sa);
    const float *b = U + loff<int>(nblk, db, sb);
    M m;
#pragma unroll
    for (int k = 0; k < 9; k++) {
        m.r[k] = pp(__ldg(a + 32 * k), __ldg(b + 32 * k));
        m.i[k] = pp(__ldg(a + 32 * (9 + k)), __ldg(b + 32 * (9 + k)));
    }
    return m;
}

// x = proj(a b^dagger): the imaginary diagonal and the six off-diagonal
// entries; the positive and negative terms of each imaginary part accumulate
// separately and meet in one subtraction.
__device__ __forceinline__ void proj_mul_adj(const M &a, const M &b, P *x) {
    P dp[3], dn[3];
#pragma unroll
    for (int r = 0; r < 3; r++) {
        // Im (a b^dag)_rr = sum_k a.i[rk] b.r[rk] - a.r[rk] b.i[rk]
        P vp = mul2(a.i[3 * r], b.r[3 * r]), vn = mul2(a.r[3 * r], b.i[3 * r]);
#pragma unroll
        for (int k = 1; k < 3; k++) {
            vp = fma2(a.i[3 * r + k], b.r[3 * r + k], vp);
            vn = fma2(a.r[3 * r + k], b.i[3 * r + k], vn);
        }
        dp[r] = vp;
        dn[r] = vn;
    }
    // (a b^dag)_rq = sum_k a_rk conj(b_qk): re, and im as (ip - in)
    auto ent = [&](int r, int q, P &re, P &ip, P &in) {
        P vr = mul2(a.r[3 * r], b.r[3 * q]), vp = mul2(a.i[3 * r], b.r[3 * q]), vn = mul2(a.r[3 * r], b.i[3 * q]);
        vr = fma2(a.i[3 * r], b.i[3 * q], vr);
#pragma unroll
        for (int k = 1; k < 3; k++) {
            vr = fma2(a.r[3 * r + k], b.r[3 * q + k], vr);
            vr = fma2(a.i[3 * r + k], b.i[3 * q + k], vr);
            vp = fma2(a.i[3 * r + k], b.r[3 * q + k], vp);
            vn = fma2(a.r[3 * r + k], b.i[3 * q + k], vn);
        }
        re = vr;
        ip = vp;
        in = vn;
    };
    P r01, p01, n01, r10, p10, n10, r02, p02, n02, r20, p20, n20, r12, p12, n12, r21, p21, n21;
    ent(0, 1, r01, p01, n01);
    ent(1, 0, r10, p10, n10);
    ent(0, 2, r02, p02, n02);
    ent(2, 0, r20, p20, n20);
    ent(1, 2, r12, p12, n12);
    ent(2, 1, r21, p21, n21);
    x[0] = sub2(add2(p01, p10), add2(n01, n10));
    x[1] = sub2(r01, r10);
    x[2] = sub2(add2(dp[0], dn[1]), add2(dn[0], dp[1]));
    x[3] = sub2(add2(p02, p20), add2(n02, n20));
    x[4] = sub2(r02, r20);
    x[5] = sub2(add2(p12, p21), add2(n12, n21));
    x[6] = sub2(r12, r21);
    // (d0 + d1 - 2 d2) / sqrt(3)
    const P dsum = sub2(add2(add2(dp[0], dp[1]), add2(dn[2], dn[2])), add2(add2(dn[0], dn[1]), add2(dp[2], dp[2])));
    x[7] = mul2(dsum, bc(0.57735026918962576451f));
}

// w = generator components of u^dagger H u, H = x^a lambda_a / 2: H's real
// diagonal and the hermitian result as in pr::act_adj_gen, with the negated
// imaginary parts of H formed once and the negative terms of the result's
// imaginary parts accumulated apart.
__device__ __forceinline__ void act_adj(const M &u, const P *x, P *w) {
    const P half = bc(0.5f), mhalf = bc(-0.5f), c2s3 = bc(0.28867513459481288225f);
    P hd[3], hr[3], hi[3], nhi[3];  // diagonal; off-diagonal (0,1), (0,2), (1,2): H_rk = hr + i hi for r < k
    hd[0] = fma2(half, x[2], mul2(c2s3, x[7]));
    hd[1] = sub2(mul2(c2s3, x[7]), mul2(half, x[2]));
    hd[2] = mul2(bc(-0.57735026918962576451f), x[7]);
    hr[0] = mul2(half, x[0]); hi[0] = mul2(mhalf, x[1]); nhi[0] = mul2(half, x[1]);
    hr[1] = mul2(half, x[3]); hi[1] = mul2(mhalf, x[4]); nhi[1] = mul2(half, x[4]);
    hr[2] = mul2(half, x[5]); hi[2] = mul2(mhalf, x[6]); nhi[2] = mul2(half, x[6]);
    // A = H u
    M A;
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int q = 0; q < 3; q++) {
            P re = mul2(hd[r], u.r[3 * r + q]), im = mul2(hd[r], u.i[3 * r + q]);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                if (k == r) continue;
                const int o = (r == 0 || k == 0) ? (r + k - 1) : 2;
                const P a = hr[o], b = r < k ? hi[o] : nhi[o], nb = r < k ? nhi[o] : hi[o];
                re = fma2(a, u.r[3 * k + q], fma2(nb, u.i[3 * k + q], re));
                im = fma2(a, u.i[3 * k + q], fma2(b, u.r[3 * k + q], im));
            }
            A.r[3 * r + q] = re;
            A.i[3 * r + q] = im;
        }
    // W = u^dagger A: real diagonal and upper triangle
    P wd[3], wr[3], wi[3];
#pragma unroll
    for (int r = 0; r < 3; r++) {
        P d = mul2(u.r[r], A.r[r]);
        d = fma2(u.i[r], A.i[r], d);
#pragma unroll
        for (int k = 1; k < 3; k++) { d = fma2(u.r[3 * k + r], A.r[3 * k + r], d); d = fma2(u.i[3 * k + r], A.i[3 * k + r], d); }
        wd[r] = d;
    }
#pragma unroll
    for (int o = 0; o < 3; o++) {
        const int r = o == 2 ? 1 : 0, q = o == 0 ? 1 : 2;
        P re = mul2(u.r[r], A.r[q]), ip = mul2(u.r[r], A.i[q]), in = mul2(u.i[r], A.r[q]);
        re = fma2(u.i[r], A.i[q], re);
#pragma unroll
        for (int k = 1; k < 3; k++) {
            re = fma2(u.r[3 * k + r], A.r[3 * k + q], fma2(u.i[3 * k + r], A.i[3 * k + q], re));
            ip = fma2(u.r[3 * k + r], A.i[3 * k + q], ip);
            in = fma2(u.i[3 * k + r], A.r[3 * k + q], in);
        }
        wr[o] = re;
        wi[o] = sub2(in, ip);  // minus the imaginary part
    }
    const P two = bc(2.f);
    w[0] = mul2(two, wr[0]);
    w[1] = mul2(two, wi[0]);
    w[2] = sub2(wd[0], wd[1]);
    w[3] = mul2(two, wr[1]);
    w[4] = mul2(two, wi[1]);
    w[5] = mul2(two, wr[2]);
    w[6] = mul2(two, wi[2]);
    w[7] = mul2(sub2(add2(wd[0], wd[1]), add2(wd[2], wd[2])), bc(0.57735026918962576451f));
}

// X = proj(P_ij(x)) for the two lanes' sites (directions per lane):
// P_ij(x) = U_i(x) U_j(x+i) U_i(x+j)^dag U_j(x)^dag.  s = x, si = x + i, sj = x + j.
__device__ __forceinline__ void plaq(const float *__restrict__ U, int nblk, int ia, int ja, int ib, int jb, int sa,
                                     int sia, int sja, int sb, int sib, int sjb, P *X) {
    const M A = mul(load_dd(U, nblk, ia, sa, ib, sb), load_dd(U, nblk, ja, sia, jb, sib));
    const M C = mul_adj(A, load_dd(U, nblk, ia, sja, ib, sjb));
    proj_mul_adj(C, load_dd(U, nblk, ja, sa, jb, sb), X);
}

__device__ __forceinline__ void put_w(float *base, int stride_a, const P *w, bool va, bool vb, int off_b) {
    if (va) {
#pragma unroll
        for (int a = 0; a < 8; a++) base[a * stride_a] = w[a].x;
    }
    if (vb) {
#pragma unroll
        for (int a = 0; a < 8; a++) base[a * stride_a + off_b] = w[a].y;
    }
}

// Plane and in-plane offsets of the two lanes' sites and of their neighbours
// along 1 and 2 (periodic), for the tile starting at (t1s, t2s).
struct Cols {
    int pa, pb;    // x
    int p1a, p1b;  // x + 1
    int p2a, p2b;  // x + 2
};

__device__ __forceinline__ int col_off(const Lat &L, int x1, int x2) { return x1 * L.n[2] + x2; }
__device__ __forceinline__ void set_cols(const Lat &L, int x1a, int x2a, int x1b, int x2b, Cols &c) {
    const int n1 = L.n[1], n2 = L.n[2];
    c.pa = col_off(L, x1a, x2a);
    c.pb = col_off(L, x1b, x2b);
    c.p1a = col_off(L, x1a + 1 == n1 ? 0 : x1a + 1, x2a);
    c.p1b = col_off(L, x1b + 1 == n1 ? 0 : x1b + 1, x2b);
    c.p2a = col_off(L, x1a, x2a + 1 == n2 ? 0 : x2a + 1);
    c.p2b = col_off(L, x1b, x2b + 1 == n2 ? 0 : x2b + 1);
}

// Force accumulator of a tile site in shared memory: F_i^a of the site at tile
// (row, col) is fs[i][a][row][col]; each thread reads and writes only its own.
__device__ __forceinline__ void fs_set(float *f, const P *v) {
#pragma unroll
    for (int a = 0; a < 8; a++) { f[a * T1 * T2] = v[a].x; f[a * T1 * T2 + 4 * T2] = v[a].y; }
}
__device__ __forceinline__ void fs_get(const float *f, P *v) {
#pragma unroll
    for (int a = 0; a < 8; a++) v[a] = pp(f[a * T1 * T2], f[a * T1 * T2 + 4 * T2]);
}

template <bool REUNIT>
__global__ void __launch_bounds__(THREADS, 2)
k_update_grid_su3f_stream(const float *__restrict__ U, float *__restrict__ E, float *__restrict__ Unext, Lat L) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem &sm = *reinterpret_cast<Smem *>(smem_raw);
    const int N0 = L.n[0], N1 = L.n[1], N2 = L.n[2];
    const int plane = N1 * N2, V = (int)L.V, nblk = (V + 31) >> 5;
    const int nt2 = N2 / T2, ntiles = (N1 / T1) * nt2;
    const long units = (long)ntiles * N0;
    const int u0 = (int)(units * blockIdx.x / gridDim.x), u1 = (int)(units * (blockIdx.x + 1) / gridDim.x);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const bool halo = warp == 4;
    const float ia0 = L.inva2f[0], ia1 = L.inva2f[1], ia2 = L.inva2f[2];
    const P dt = bc(L.dtf), mdt = bc(-L.dtf);
    // halo lanes: a = the halo row (transports along 1), b = the halo column
    // (transports along 2; lanes 0-7 store, the others repeat a column site)
    const bool vb_h = lane < T1;
    // this thread's slots (tile sites only)
    const int own = (halo ? 0 : warp) * T2 + lane;
    float *fs0 = &sm.fs[0][0][0][0] + own, *fs1 = &sm.fs[1][0][0][0] + own, *fs2 = &sm.fs[2][0][0][0] + own;
    float *cy0 = &sm.carry[0][0][0][0] + own, *cy1 = &sm.carry[1][0][0][0] + own;
    Cols cl;
    int tile = -1;
    for (int u = u0; u < u1; u++) {
        const int t = u / N0, x0 = u - t * N0;
        if (t != tile) {
            tile = t;
            const int t1s = (t / nt2) * T1, t2s = (t - (t / nt2) * nt2) * T2;
            if (!halo) set_cols(L, t1s + warp, t2s + lane, t1s + warp + 4, t2s + lane, cl);
            else set_cols(L, t1s == 0 ? N1 - 1 : t1s - 1, t2s + lane, t1s + (lane & 7), t2s == 0 ? N2 - 1 : t2s - 1, cl);
        }
        const int xn = x0 + 1 == N0 ? 0 : x0 + 1;
        if (!halo && (u == u0 || x0 == 0)) {
            // prologue: the transports along 0 out of the plane before x0
            const int xm = x0 == 0 ? N0 - 1 : x0 - 1;
            const int sa = xm * plane + cl.pa, sb = xm * plane + cl.pb;
            const int s0a = x0 * plane + cl.pa, s0b = x0 * plane + cl.pb;
            P X[8], w[8];
            plaq(U, nblk, 0, 1, 0, 1, sa, s0a, xm * plane + cl.p1a, sb, s0b, xm * plane + cl.p1b, X);
            act_adj(load_dd(U, nblk, 0, sa, 0, sb), X, w);
            fs_set(cy0, w);
            plaq(U, nblk, 0, 2, 0, 2, sa, s0a, xm * plane + cl.p2a, sb, s0b, xm * plane + cl.p2b, X);
            act_adj(load_dd(U, nblk, 0, sa, 0, sb), X, w);
            fs_set(cy1, w);
        }
        const int base = x0 * plane;
        const int sa = base + cl.pa, sb = base + cl.pb;
        const int s0a = xn * plane + cl.pa, s0b = xn * plane + cl.pb;  // x + 0
        const int s1a = base + cl.p1a, s1b = base + cl.p1b;            // x + 1
        const int s2a = base + cl.p2a, s2b = base + cl.p2b;            // x + 2
        if (!halo) {
            P X[8], w[8], f[8];
            // plane (0,1): F_0 = X / a1^2, F_1 = (W_carry - X) / a0^2
            plaq(U, nblk, 0, 1, 0, 1, sa, s0a, s1a, sb, s0b, s1b, X);
            fs_get(cy0, f);
#pragma unroll
            for (int a = 0; a < 8; a++) { f[a] = mul2(sub2(f[a], X[a]), bc(ia0)); w[a] = mul2(X[a], bc(ia1)); }
            fs_set(fs1, f);
            fs_set(fs0, w);
            act_adj(load_dd(U, nblk, 0, sa, 0, sb), X, w);
            fs_set(cy0, w);
            act_adj(load_dd(U, nblk, 1, sa, 1, sb), X, w);
            put_w(&sm.wx1[0][0][warp + 1][lane], (T1 + 1) * T2, w, true, true, 4 * T2);
            // plane (0,2): F_0 += X / a2^2, F_2 = (W_carry - X) / a0^2
            plaq(U, nblk, 0, 2, 0, 2, sa, s0a, s2a, sb, s0b, s2b, X);
            fs_get(cy1, f);
#pragma unroll
            for (int a = 0; a < 8; a++) f[a] = mul2(sub2(f[a], X[a]), bc(ia0));
            fs_set(fs2, f);
            fs_get(fs0, f);
#pragma unroll
            for (int a = 0; a < 8; a++) f[a] = fma2(X[a], bc(ia2), f[a]);
            fs_set(fs0, f);
            act_adj(load_dd(U, nblk, 0, sa, 0, sb), X, w);
            fs_set(cy1, w);
            act_adj(load_dd(U, nblk, 2, sa, 2, sb), X, w);
            put_w(&sm.wx2[0][0][warp][lane + 1], T1 * (T2 + 1), w, true, true, 4 * (T2 + 1));
            // plane (1,2): F_1 += X / a2^2, F_2 -= X / a1^2
            plaq(U, nblk, 1, 2, 1, 2, sa, s1a, s2a, sb, s1b, s2b, X);
            fs_get(fs1, f);
#pragma unroll
            for (int a = 0; a < 8; a++) f[a] = fma2(X[a], bc(ia2), f[a]);
            fs_set(fs1, f);
            fs_get(fs2, f);
#pragma unroll
            for (int a = 0; a < 8; a++) f[a] = fma2(X[a], bc(-ia1), f[a]);
            fs_set(fs2, f);
            act_adj(load_dd(U, nblk, 1, sa, 1, sb), X, w);
            put_w(&sm.wx1[1][0][warp + 1][lane], (T1 + 1) * T2, w, true, true, 4 * T2);
            act_adj(load_dd(U, nblk, 2, sa, 2, sb), X, w);
            put_w(&sm.wx2[1][0][warp][lane + 1], T1 * (T2 + 1), w, true, true, 4 * (T2 + 1));
        } else {
            // halo: lane a (row x1 - 1) plane (0,1) and Ad(U_1^dag); lane b
            // (column x2 - 1) plane (0,2) and Ad(U_2^dag); then plane (1,2)
            P X[8], w[8];
            plaq(U, nblk, 0, 1, 0, 2, sa, s0a, s1a, sb, s0b, s2b, X);
            act_adj(load_dd(U, nblk, 1, sa, 2, sb), X, w);
#pragma unroll
            for (int a = 0; a < 8; a++) sm.wx1[0][a][0][lane] = w[a].x;
            if (vb_h) {
#pragma unroll
                for (int a = 0; a < 8; a++) sm.wx2[0][a][lane][0] = w[a].y;
            }
            plaq(U, nblk, 1, 2, 1, 2, sa, s1a, s2a, sb, s1b, s2b, X);
            act_adj(load_dd(U, nblk, 1, sa, 2, sb), X, w);
#pragma unroll
            for (int a = 0; a < 8; a++) sm.wx1[1][a][0][lane] = w[a].x;
            if (vb_h) {
#pragma unroll
                for (int a = 0; a < 8; a++) sm.wx2[1][a][lane][0] = w[a].y;
            }
        }
        __syncthreads();
        if (!halo) {
            // the transports into x from x - 1 and x - 2
#pragma unroll
            for (int a = 0; a < 8; a++) {
                const int o = a * T1 * T2, o4 = o + 4 * T2;
                const P w10 = pp(sm.wx1[0][a][warp][lane], sm.wx1[0][a][warp + 4][lane]);
                const P w11 = pp(sm.wx1[1][a][warp][lane], sm.wx1[1][a][warp + 4][lane]);
                const P w20 = pp(sm.wx2[0][a][warp][lane], sm.wx2[0][a][warp + 4][lane]);
                const P w21 = pp(sm.wx2[1][a][warp][lane], sm.wx2[1][a][warp + 4][lane]);
                P f0 = pp(fs0[o], fs0[o4]), f1 = pp(fs1[o], fs1[o4]), f2 = pp(fs2[o], fs2[o4]);
                f0 = fma2(w10, bc(-ia1), f0);
                f0 = fma2(w20, bc(-ia2), f0);
                f1 = fma2(w21, bc(-ia2), f1);
                f2 = fma2(w11, bc(ia1), f2);
                fs0[o] = f0.x; fs0[o4] = f0.y;
                fs1[o] = f1.x; fs1[o4] = f1.y;
                fs2[o] = f2.x; fs2[o4] = f2.y;
            }
        }
        __syncthreads();  // the exchange buffers are free for the next plane
        if (!halo) {
#pragma unroll 1
            for (int i = 0; i < 3; i++) {
                P f[8], e[8];
                fs_get(&sm.fs[i][0][0][0] + own, f);
                float *ea = E + (i * 8) * V + sa, *eb = E + (i * 8) * V + sb;
#pragma unroll
                for (int a = 0; a < 8; a++) e[a] = fma2(f[a], dt, pp(ea[a * V], eb[a * V]));
#pragma unroll
                for (int a = 0; a < 8; a++) { ea[a * V] = e[a].x; eb[a * V] = e[a].y; }
                P v[8];
#pragma unroll
                for (int a = 0; a < 8; a++) v[a] = mul2(mdt, e[a]);
                M Vn = mul(expi(v), load_dd(U, nblk, i, sa, i, sb));
                if (REUNIT) reunit(Vn);
                store<int>(Unext, nblk, i, sa, sb, true, true, Vn);
            }
        }
    }
}

}  // namespace st
}  // namespace opx
