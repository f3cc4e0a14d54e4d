// su3_pair.cuh -- SU(3) FP32 arithmetic on two sites at once.
//
// Every value is a float2 whose lanes belong to two different lattice sites
// (site A in .x, site B in .y), and every operation is one paired FP32
// instruction (fma/mul/add .f32x2) for both sites.  The SU(3) leapfrog is
// issue-bound in scalar FP32 (the FMA pipe is not saturated), so executing the
// same arithmetic for two sites per instruction halves the issue slots the
// arithmetic takes.  Control flow is uniform over the two lanes: the
// exponential's series runs until both lanes have converged and both lanes use
// the larger scaling exponent.
//
// Matrices are 3x3 complex, row-major, real and imaginary parts in separate
// arrays (the storage order of the links).
#pragma once
#include <cuda_runtime.h>

#include "lattice.cuh"

namespace opx {
namespace pr {

typedef float2 P;

__device__ __forceinline__ P pp(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ P bc(float a) { return make_float2(a, a); }
__device__ __forceinline__ P fma2(P a, P b, P c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ P mul2(P a, P b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ P add2(P a, P b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ P neg2(P a) { return make_float2(-a.x, -a.y); }
// a - b in one paired instruction (sub.rn.f32x2; the same bits as a + (-b))
__device__ __forceinline__ P sub2(P a, P b) {
    unsigned long long ra, rb, rc;
    memcpy(&ra, &a, 8);
    memcpy(&rb, &b, 8);
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(rc) : "l"(ra), "l"(rb));
    P c;
    memcpy(&c, &rc, 8);
    return c;
}
__device__ __forceinline__ P zero2() { return make_float2(0.f, 0.f); }
__device__ __forceinline__ float maxl(P a) { return fmaxf(a.x, a.y); }
// the sum of the lanes whose site counts
__device__ __forceinline__ float lanes(P a, bool va, bool vb) { return (va ? a.x : 0.f) + (vb ? a.y : 0.f); }

struct M {
    P r[9], i[9];
};

__device__ __forceinline__ M mzero() {
    M m;
#pragma unroll
    for (int k = 0; k < 9; k++) { m.r[k] = zero2(); m.i[k] = zero2(); }
    return m;
}

// (a b)_{rq} real and imaginary parts; positive and negative products are
// accumulated separately so that no operand needs a sign change.
__device__ __forceinline__ void e_mul(const M &a, const M &b, int r, int q, P &re, P &im) {
    P rp = mul2(a.r[3 * r], b.r[q]);
    rp = fma2(a.r[3 * r + 1], b.r[3 + q], rp);
    rp = fma2(a.r[3 * r + 2], b.r[6 + q], rp);
    P rn = mul2(a.i[3 * r], b.i[q]);
    rn = fma2(a.i[3 * r + 1], b.i[3 + q], rn);
    rn = fma2(a.i[3 * r + 2], b.i[6 + q], rn);
    P ii = mul2(a.r[3 * r], b.i[q]);
    ii = fma2(a.r[3 * r + 1], b.i[3 + q], ii);
    ii = fma2(a.r[3 * r + 2], b.i[6 + q], ii);
    ii = fma2(a.i[3 * r], b.r[q], ii);
    ii = fma2(a.i[3 * r + 1], b.r[3 + q], ii);
    ii = fma2(a.i[3 * r + 2], b.r[6 + q], ii);
    re = sub2(rp, rn);
    im = ii;
}
__device__ __forceinline__ P e_mul_im(const M &a, const M &b, int r, int q) {
    P ii = mul2(a.r[3 * r], b.i[q]);
    ii = fma2(a.r[3 * r + 1], b.i[3 + q], ii);
    ii = fma2(a.r[3 * r + 2], b.i[6 + q], ii);
    ii = fma2(a.i[3 * r], b.r[q], ii);
    ii = fma2(a.i[3 * r + 1], b.r[3 + q], ii);
    ii = fma2(a.i[3 * r + 2], b.r[6 + q], ii);
    return ii;
}

// The products below run k-outer: every k adds one term to all nine output
// entries, so eighteen independent accumulator chains interleave and the FMA
// latency is covered within one thread.  One operand's sign-flipped copy
// replaces the subtractions.

// a b
__device__ __forceinline__ M mul(const M &a, const M &b) {
    M c;
    P nai[9];
#pragma unroll
    for (int k = 0; k < 9; k++) nai[k] = neg2(a.i[k]);
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int q = 0; q < 3; q++) {
            c.r[3 * r + q] = fma2(nai[3 * r], b.i[q], mul2(a.r[3 * r], b.r[q]));
            c.i[3 * r + q] = fma2(a.i[3 * r], b.r[q], mul2(a.r[3 * r], b.i[q]));
        }
#pragma unroll
    for (int k = 1; k < 3; k++)
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
            for (int q = 0; q < 3; q++) {
                c.r[3 * r + q] = fma2(nai[3 * r + k], b.i[3 * k + q], fma2(a.r[3 * r + k], b.r[3 * k + q], c.r[3 * r + q]));
                c.i[3 * r + q] = fma2(a.i[3 * r + k], b.r[3 * k + q], fma2(a.r[3 * r + k], b.i[3 * k + q], c.i[3 * r + q]));
            }
    return c;
}

// a b^dagger: (b^dagger)_{kq} = conj(b_{qk})
__device__ __forceinline__ M mul_adj(const M &a, const M &b) {
    M c;
    P nbi[9];
#pragma unroll
    for (int k = 0; k < 9; k++) nbi[k] = neg2(b.i[k]);
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int q = 0; q < 3; q++) {
            c.r[3 * r + q] = fma2(a.i[3 * r], b.i[3 * q], mul2(a.r[3 * r], b.r[3 * q]));
            c.i[3 * r + q] = fma2(a.r[3 * r], nbi[3 * q], mul2(a.i[3 * r], b.r[3 * q]));
        }
#pragma unroll
    for (int k = 1; k < 3; k++)
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
            for (int q = 0; q < 3; q++) {
                c.r[3 * r + q] = fma2(a.i[3 * r + k], b.i[3 * q + k], fma2(a.r[3 * r + k], b.r[3 * q + k], c.r[3 * r + q]));
                c.i[3 * r + q] = fma2(a.r[3 * r + k], nbi[3 * q + k], fma2(a.i[3 * r + k], b.r[3 * q + k], c.i[3 * r + q]));
            }
    return c;
}

// a^dagger b: (a^dagger)_{rk} = conj(a_{kr})
__device__ __forceinline__ M adj_mul(const M &a, const M &b) {
    M c;
    P nai[9];
#pragma unroll
    for (int k = 0; k < 9; k++) nai[k] = neg2(a.i[k]);
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int q = 0; q < 3; q++) {
            c.r[3 * r + q] = fma2(a.i[r], b.i[q], mul2(a.r[r], b.r[q]));
            c.i[3 * r + q] = fma2(nai[r], b.r[q], mul2(a.r[r], b.i[q]));
        }
#pragma unroll
    for (int k = 1; k < 3; k++)
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
            for (int q = 0; q < 3; q++) {
                c.r[3 * r + q] = fma2(a.i[3 * k + r], b.i[3 * k + q], fma2(a.r[3 * k + r], b.r[3 * k + q], c.r[3 * r + q]));
                c.i[3 * r + q] = fma2(nai[3 * k + r], b.r[3 * k + q], fma2(a.r[3 * k + r], b.i[3 * k + q], c.i[3 * r + q]));
            }
    return c;
}

__device__ __forceinline__ void madd(M &acc, const M &b) {
#pragma unroll
    for (int k = 0; k < 9; k++) { acc.r[k] = add2(acc.r[k], b.r[k]); acc.i[k] = add2(acc.i[k], b.i[k]); }
}
// acc += f b
__device__ __forceinline__ void maxpy(M &acc, P f, const M &b) {
#pragma unroll
    for (int k = 0; k < 9; k++) { acc.r[k] = fma2(f, b.r[k], acc.r[k]); acc.i[k] = fma2(f, b.i[k], acc.i[k]); }
}

// x = proj(a b), proj_a(M) = Im tr(lambda_a M); only the entries proj reads
// are formed: the imaginary diagonal and the six off-diagonal entries.
__device__ __forceinline__ void proj_mul(const M &a, const M &b, P *x) {
    const P d0 = e_mul_im(a, b, 0, 0), d1 = e_mul_im(a, b, 1, 1), d2 = e_mul_im(a, b, 2, 2);
    P r01, i01, r10, i10, r02, i02, r20, i20, r12, i12, r21, i21;
    e_mul(a, b, 0, 1, r01, i01);
    e_mul(a, b, 1, 0, r10, i10);
    e_mul(a, b, 0, 2, r02, i02);
    e_mul(a, b, 2, 0, r20, i20);
    e_mul(a, b, 1, 2, r12, i12);
    e_mul(a, b, 2, 1, r21, i21);
    x[0] = add2(i01, i10);
    x[1] = sub2(r01, r10);
    x[2] = sub2(d0, d1);
    x[3] = add2(i02, i20);
    x[4] = sub2(r02, r20);
    x[5] = add2(i12, i21);
    x[6] = sub2(r12, r21);
    x[7] = mul2(sub2(add2(d0, d1), add2(d2, d2)), bc(0.57735026918962576451f));
}

// exp(i H), H = x^a lambda_a / 2, by the Cayley-Hamilton reduction
// exp(iH) = f0 + f1 H + f2 H^2 with the scalar series of the scalar SU(3) code
// (H^3 = c1 H + c0, c1 = tr(H^2)/2, c0 = det H), scaling and squaring above
// ||H||_F^2 = 1.  H^2 uses the hermitian structure (six distinct entries).
__device__ __forceinline__ M expi(const P *x) {
    const P half = bc(0.5f), c2s3 = bc(0.28867513459481288225f);
    // H: real diagonal d, off-diagonal u = H01, v = H02, w = H12
    P d0 = fma2(half, x[2], mul2(c2s3, x[7]));
    P d1 = sub2(mul2(c2s3, x[7]), mul2(half, x[2]));
    P d2 = mul2(bc(-0.57735026918962576451f), x[7]);
    P ur = mul2(half, x[0]), ui = mul2(bc(-0.5f), x[1]);
    P vr = mul2(half, x[3]), vi = mul2(bc(-0.5f), x[4]);
    P wr = mul2(half, x[5]), wi = mul2(bc(-0.5f), x[6]);
    P c1 = mul2(x[0], x[0]);
#pragma unroll
    for (int a = 1; a < 8; a++) c1 = fma2(x[a], x[a], c1);
    c1 = mul2(c1, bc(0.25f));
    int s = 0;
    float sc = 1.f;
    const float c1m = maxl(c1);
    while (2.f * c1m * sc * sc > 1.f && s < 30) { sc *= 0.5f; s++; }
    if (s) {
        const P S = bc(sc), S2 = bc(sc * sc);
        d0 = mul2(d0, S); d1 = mul2(d1, S); d2 = mul2(d2, S);
        ur = mul2(ur, S); ui = mul2(ui, S); vr = mul2(vr, S); vi = mul2(vi, S); wr = mul2(wr, S); wi = mul2(wi, S);
        c1 = mul2(c1, S2);
    }
    const P uu = fma2(ur, ur, mul2(ui, ui)), vv = fma2(vr, vr, mul2(vi, vi)), ww = fma2(wr, wr, mul2(wi, wi));
    // det H = d0 (d1 d2 - |w|^2) - d1 |v|^2 - d2 |u|^2 + 2 Re(u w conj(v))
    P c0 = mul2(d0, sub2(mul2(d1, d2), ww));
    c0 = sub2(c0, mul2(d1, vv));
    c0 = sub2(c0, mul2(d2, uu));
    P re_uwv = fma2(ur, fma2(wr, vr, mul2(wi, vi)), mul2(ui, sub2(mul2(wr, vi), mul2(wi, vr))));
    c0 = fma2(bc(2.f), re_uwv, c0);
    // series
    P al = bc(1.f), be = zero2(), ga = zero2();
    float t = 1.f;
    P f0r = bc(1.f), f0i = zero2(), f1r = zero2(), f1i = zero2(), f2r = zero2(), f2i = zero2();
    const P two_c1 = add2(c1, c1);
    const P nrm = pp(sqrtf(two_c1.x), sqrtf(two_c1.y));
    P bound = bc(1.f);
    const P nrm2 = mul2(nrm, nrm), nrm4 = mul2(nrm2, nrm2);
    // four terms per pass, i^k fixed within a pass (k = 1, 2, 3, 0 mod 4), the
    // stopping test after the fourth
    for (int k = 1; k < 40; k += 4) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const P nal = mul2(c0, ga), nbe = fma2(c1, ga, al);
            ga = be;
            al = nal;
            be = nbe;
            t = t * c_inv_k32[k + u];
            const P T = bc((u == 1 || u == 2) ? -t : t);
            if (u & 1) { f0r = fma2(T, al, f0r); f1r = fma2(T, be, f1r); f2r = fma2(T, ga, f2r); }
            else { f0i = fma2(T, al, f0i); f1i = fma2(T, be, f1i); f2i = fma2(T, ga, f2i); }
        }
        bound = mul2(bound, nrm4);
        if (maxl(bound) * t < 5.9604645e-08f * 0.01f) break;
    }
    // Q = H^2 (hermitian)
    const P q00 = add2(fma2(d0, d0, uu), vv), q11 = add2(fma2(d1, d1, uu), ww), q22 = add2(fma2(d2, d2, vv), ww);
    const P s01 = add2(d0, d1), s02 = add2(d0, d2), s12 = add2(d1, d2);
    // Q01 = u (d0 + d1) + v conj(w)
    const P q01r = fma2(ur, s01, fma2(vr, wr, mul2(vi, wi)));
    const P q01i = fma2(ui, s01, sub2(mul2(vi, wr), mul2(vr, wi)));
    // Q02 = v (d0 + d2) + u w
    const P q02r = fma2(vr, s02, sub2(mul2(ur, wr), mul2(ui, wi)));
    const P q02i = fma2(vi, s02, fma2(ur, wi, mul2(ui, wr)));
    // Q12 = w (d1 + d2) + conj(u) v
    const P q12r = fma2(wr, s12, fma2(ur, vr, mul2(ui, vi)));
    const P q12i = fma2(wi, s12, sub2(mul2(ur, vi), mul2(ui, vr)));
    M W;
    // diagonal: f0 + f1 d + f2 q
    W.r[0] = fma2(f2r, q00, fma2(f1r, d0, f0r));
    W.i[0] = fma2(f2i, q00, fma2(f1i, d0, f0i));
    W.r[4] = fma2(f2r, q11, fma2(f1r, d1, f0r));
    W.i[4] = fma2(f2i, q11, fma2(f1i, d1, f0i));
    W.r[8] = fma2(f2r, q22, fma2(f1r, d2, f0r));
    W.i[8] = fma2(f2i, q22, fma2(f1i, d2, f0i));
    // upper entry z = f1 h + f2 q, lower entry f1 conj(h) + f2 conj(q)
    auto off = [&](P hr, P hi, P qr, P qi, P &ur_, P &ui_, P &lr_, P &li_) {
        const P a = fma2(f1r, hr, mul2(f2r, qr));  // f1r hr + f2r qr
        const P b = fma2(f1i, hi, mul2(f2i, qi));  // f1i hi + f2i qi
        const P c = fma2(f1r, hi, mul2(f2r, qi));  // f1r hi + f2r qi
        const P e = fma2(f1i, hr, mul2(f2i, qr));  // f1i hr + f2i qr
        ur_ = sub2(a, b);
        ui_ = add2(c, e);
        lr_ = add2(a, b);
        li_ = sub2(e, c);
    };
    off(ur, ui, q01r, q01i, W.r[1], W.i[1], W.r[3], W.i[3]);
    off(vr, vi, q02r, q02i, W.r[2], W.i[2], W.r[6], W.i[6]);
    off(wr, wi, q12r, q12i, W.r[5], W.i[5], W.r[7], W.i[7]);
    for (int k = 0; k < s; k++) W = mul(W, W);
    return W;
}

// Gram-Schmidt on rows 0 and 1; row 2 = conj(row0 x row1)
__device__ __forceinline__ void reunit_gs(M &m) {
    P n0 = mul2(m.r[0], m.r[0]);
    n0 = fma2(m.i[0], m.i[0], n0);
#pragma unroll
    for (int k = 1; k < 3; k++) { n0 = fma2(m.r[k], m.r[k], n0); n0 = fma2(m.i[k], m.i[k], n0); }
    const P inv0 = pp(1.f / sqrtf(n0.x), 1.f / sqrtf(n0.y));
#pragma unroll
    for (int k = 0; k < 3; k++) { m.r[k] = mul2(m.r[k], inv0); m.i[k] = mul2(m.i[k], inv0); }
    P pr_ = zero2(), pip = zero2(), pin = zero2();
#pragma unroll
    for (int k = 0; k < 3; k++) {
        pr_ = fma2(m.r[k], m.r[3 + k], pr_);
        pr_ = fma2(m.i[k], m.i[3 + k], pr_);
        pip = fma2(m.r[k], m.i[3 + k], pip);
        pin = fma2(m.i[k], m.r[3 + k], pin);
    }
    const P pi_ = sub2(pip, pin), npr = neg2(pr_), npi = neg2(pi_);
#pragma unroll
    for (int k = 0; k < 3; k++) {
        // row1 -= p row0
        const P nr = fma2(npr, m.r[k], fma2(pi_, m.i[k], m.r[3 + k]));
        const P ni = fma2(npr, m.i[k], fma2(npi, m.r[k], m.i[3 + k]));
        m.r[3 + k] = nr;
        m.i[3 + k] = ni;
    }
    P n1 = mul2(m.r[3], m.r[3]);
    n1 = fma2(m.i[3], m.i[3], n1);
#pragma unroll
    for (int k = 4; k < 6; k++) { n1 = fma2(m.r[k], m.r[k], n1); n1 = fma2(m.i[k], m.i[k], n1); }
    const P inv1 = pp(1.f / sqrtf(n1.x), 1.f / sqrtf(n1.y));
#pragma unroll
    for (int k = 3; k < 6; k++) { m.r[k] = mul2(m.r[k], inv1); m.i[k] = mul2(m.i[k], inv1); }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int a = (k + 1) % 3, b = (k + 2) % 3;
        const P xr = sub2(sub2(mul2(m.r[a], m.r[3 + b]), mul2(m.i[a], m.i[3 + b])),
                          sub2(mul2(m.r[b], m.r[3 + a]), mul2(m.i[b], m.i[3 + a])));
        const P xi = sub2(fma2(m.r[a], m.i[3 + b], mul2(m.i[a], m.r[3 + b])),
                          fma2(m.r[b], m.i[3 + a], mul2(m.i[b], m.r[3 + a])));
        m.r[6 + k] = xr;
        m.i[6 + k] = neg2(xi);
    }
}

// H = m^dagger m: real diagonal hd, upper entries (0,1), (0,2), (1,2) as hr + i hi;
// returns the largest |H - 1| entry of the two lanes.
__device__ __forceinline__ float gram(const M &m, P *hd, P *hr, P *hi) {
#pragma unroll
    for (int c = 0; c < 3; c++) {
        P d = mul2(m.r[c], m.r[c]);
        d = fma2(m.i[c], m.i[c], d);
#pragma unroll
        for (int k = 1; k < 3; k++) { d = fma2(m.r[3 * k + c], m.r[3 * k + c], d); d = fma2(m.i[3 * k + c], m.i[3 * k + c], d); }
        hd[c] = d;
    }
#pragma unroll
    for (int o = 0; o < 3; o++) {
        const int r = o == 2 ? 1 : 0, c = o == 0 ? 1 : 2;
        P re = mul2(m.r[r], m.r[c]), ip = mul2(m.r[r], m.i[c]), in = mul2(m.i[r], m.r[c]);
        re = fma2(m.i[r], m.i[c], re);
#pragma unroll
        for (int k = 1; k < 3; k++) {
            re = fma2(m.r[3 * k + r], m.r[3 * k + c], fma2(m.i[3 * k + r], m.i[3 * k + c], re));
            ip = fma2(m.r[3 * k + r], m.i[3 * k + c], ip);
            in = fma2(m.i[3 * k + r], m.r[3 * k + c], in);
        }
        hr[o] = re;
        hi[o] = sub2(ip, in);
    }
    float dev = 0.f;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        dev = fmaxf(dev, fmaxf(fabsf(hd[c].x - 1.f), fabsf(hd[c].y - 1.f)));
        dev = fmaxf(dev, fmaxf(fmaxf(fabsf(hr[c].x), fabsf(hr[c].y)), fmaxf(fabsf(hi[c].x), fabsf(hi[c].y))));
    }
    return dev;
}

// One Newton-Schulz step toward the unitary factor of m's polar decomposition:
// m <- m (3 - m^dagger m) / 2, given H = m^dagger m.
__device__ __forceinline__ void newton_schulz(M &m, const P *hd, const P *hr, const P *hi) {
    const P h3 = bc(1.5f), mh = bc(-0.5f);
    P kd[3], kr[3], ki[3];  // K = (3 - H) / 2, hermitian
#pragma unroll
    for (int c = 0; c < 3; c++) { kd[c] = fma2(mh, hd[c], h3); kr[c] = mul2(mh, hr[c]); ki[c] = mul2(mh, hi[c]); }
    M n;
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            P re = mul2(m.r[3 * r + c], kd[c]), im = mul2(m.i[3 * r + c], kd[c]);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                if (k == c) continue;
                // K_kc: stored upper entries, lower ones their conjugates
                const int o = (k == 0 || c == 0) ? (k + c - 1) : 2;
                const P a = kr[o], b = k < c ? ki[o] : neg2(ki[o]);
                re = fma2(m.r[3 * r + k], a, fma2(neg2(m.i[3 * r + k]), b, re));
                im = fma2(m.r[3 * r + k], b, fma2(m.i[3 * r + k], a, im));
            }
            n.r[3 * r + c] = re;
            n.i[3 * r + c] = im;
        }
    m = n;
}

// Reunitarisation of the FP32 form: the nearest unitary matrix (polar factor by
// Newton-Schulz steps: the deviations met between reunitarisations are ~1e-6,
// which one step removes to FP32 rounding; a second step above 1e-3), then the determinant's
// phase spread evenly over the rows (det = 1 to first order in the phase).
// Unlike Gram-Schmidt, which rotates the link by an amount of the order of its
// deviation from unitarity, the polar factor only removes the deviation, so the
// reunitarisation adds no systematic drift to the energy.  Far from unitary
// (an entry of m^dagger m off by more than 0.25), Gram-Schmidt comes first.
__device__ __forceinline__ void reunit(M &m) {
    P hd[3], hr[3], hi[3];
    float dev = gram(m, hd, hr, hi);
    if (dev > 0.25f) {
        reunit_gs(m);
        dev = gram(m, hd, hr, hi);
    }
    newton_schulz(m, hd, hr, hi);
    if (dev > 1e-3f) {
        // a second step where the first leaves more than FP32 rounding
        gram(m, hd, hr, hi);
        newton_schulz(m, hd, hr, hi);
    }
    // Im det m, from the cofactors of row 0
    const P c0r = sub2(sub2(mul2(m.r[4], m.r[8]), mul2(m.i[4], m.i[8])), sub2(mul2(m.r[5], m.r[7]), mul2(m.i[5], m.i[7])));
    const P c0i = sub2(add2(mul2(m.r[4], m.i[8]), mul2(m.i[4], m.r[8])), add2(mul2(m.r[5], m.i[7]), mul2(m.i[5], m.r[7])));
    const P c1r = sub2(sub2(mul2(m.r[5], m.r[6]), mul2(m.i[5], m.i[6])), sub2(mul2(m.r[3], m.r[8]), mul2(m.i[3], m.i[8])));
    const P c1i = sub2(add2(mul2(m.r[5], m.i[6]), mul2(m.i[5], m.r[6])), add2(mul2(m.r[3], m.i[8]), mul2(m.i[3], m.r[8])));
    const P c2r = sub2(sub2(mul2(m.r[3], m.r[7]), mul2(m.i[3], m.i[7])), sub2(mul2(m.r[4], m.r[6]), mul2(m.i[4], m.i[6])));
    const P c2i = sub2(add2(mul2(m.r[3], m.i[7]), mul2(m.i[3], m.r[7])), add2(mul2(m.r[4], m.i[6]), mul2(m.i[4], m.r[6])));
    P di = mul2(m.r[0], c0i);
    di = fma2(m.i[0], c0r, di);
    di = fma2(m.r[1], c1i, di);
    di = fma2(m.i[1], c1r, di);
    di = fma2(m.r[2], c2i, di);
    di = fma2(m.i[2], c2r, di);
    // m <- m (1 - i phi / 3), phi = Im det
    const P t = mul2(di, bc(1.f / 3.f)), nt = neg2(t);
#pragma unroll
    for (int k = 0; k < 9; k++) {
        const P re = fma2(t, m.i[k], m.r[k]);
        m.i[k] = fma2(nt, m.r[k], m.i[k]);
        m.r[k] = re;
    }
}

// H = x^a lambda_a / 2 as a matrix, and its generator components x^a = tr(lambda_a H)
__device__ __forceinline__ M herm(const P *x) {
    const P half = bc(0.5f), mhalf = bc(-0.5f), c2s3 = bc(0.28867513459481288225f);
    M h;
    h.r[0] = fma2(half, x[2], mul2(c2s3, x[7]));
    h.r[4] = sub2(mul2(c2s3, x[7]), mul2(half, x[2]));
    h.r[8] = mul2(bc(-0.57735026918962576451f), x[7]);
    h.i[0] = h.i[4] = h.i[8] = zero2();
    h.r[1] = h.r[3] = mul2(half, x[0]);
    h.i[1] = mul2(mhalf, x[1]); h.i[3] = mul2(half, x[1]);
    h.r[2] = h.r[6] = mul2(half, x[3]);
    h.i[2] = mul2(mhalf, x[4]); h.i[6] = mul2(half, x[4]);
    h.r[5] = h.r[7] = mul2(half, x[5]);
    h.i[5] = mul2(mhalf, x[6]); h.i[7] = mul2(half, x[6]);
    return h;
}
__device__ __forceinline__ void herm_gen(const M &h, P *x) {
    x[0] = add2(h.r[1], h.r[3]);
    x[1] = sub2(h.i[3], h.i[1]);
    x[2] = sub2(h.r[0], h.r[4]);
    x[3] = add2(h.r[2], h.r[6]);
    x[4] = sub2(h.i[6], h.i[2]);
    x[5] = add2(h.r[5], h.r[7]);
    x[6] = sub2(h.i[7], h.i[5]);
    x[7] = mul2(sub2(add2(h.r[0], h.r[4]), add2(h.r[8], h.r[8])), bc(0.57735026918962576451f));
}
// w = generator components of u^dagger H u, H = x^a lambda_a / 2 (the parallel
// transport of SU3AlgebraElement.act with g = u^dagger).  Uses the structure:
// H has a real diagonal, and the result is hermitian, so only its real
// diagonal and upper triangle are formed.
__device__ __forceinline__ void act_adj_gen(const M &u, const P *x, P *w) {
    const P half = bc(0.5f), mhalf = bc(-0.5f), c2s3 = bc(0.28867513459481288225f);
    P hd[3], hr[3], hi[3];  // diagonal; off-diagonal (0,1), (0,2), (1,2)
    hd[0] = fma2(half, x[2], mul2(c2s3, x[7]));
    hd[1] = sub2(mul2(c2s3, x[7]), mul2(half, x[2]));
    hd[2] = mul2(bc(-0.57735026918962576451f), x[7]);
    hr[0] = mul2(half, x[0]); hi[0] = mul2(mhalf, x[1]);
    hr[1] = mul2(half, x[3]); hi[1] = mul2(mhalf, x[4]);
    hr[2] = mul2(half, x[5]); hi[2] = mul2(mhalf, x[6]);
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
                // H_rk: upper entries stored, lower ones their conjugates
                const int o = (r == 0 || k == 0) ? (r + k - 1) : 2;
                const P a = hr[o], b = r < k ? hi[o] : neg2(hi[o]);
                re = fma2(a, u.r[3 * k + q], fma2(neg2(b), u.i[3 * k + q], re));
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
        P re = mul2(u.r[r], A.r[q]), im = mul2(u.r[r], A.i[q]);
        re = fma2(u.i[r], A.i[q], re);
        im = fma2(neg2(u.i[r]), A.r[q], im);
#pragma unroll
        for (int k = 1; k < 3; k++) {
            re = fma2(u.r[3 * k + r], A.r[3 * k + q], fma2(u.i[3 * k + r], A.i[3 * k + q], re));
            im = fma2(u.r[3 * k + r], A.i[3 * k + q], fma2(neg2(u.i[3 * k + r]), A.r[3 * k + q], im));
        }
        wr[o] = re;
        wi[o] = im;
    }
    const P two = bc(2.f), mtwo = bc(-2.f);
    w[0] = mul2(two, wr[0]);
    w[1] = mul2(mtwo, wi[0]);
    w[2] = sub2(wd[0], wd[1]);
    w[3] = mul2(two, wr[1]);
    w[4] = mul2(mtwo, wi[1]);
    w[5] = mul2(two, wr[2]);
    w[6] = mul2(mtwo, wi[2]);
    w[7] = mul2(sub2(add2(wd[0], wd[1]), add2(wd[2], wd[2])), bc(0.57735026918962576451f));
}

// proj(M) for a whole matrix
__device__ __forceinline__ void proj(const M &m, P *x) {
    x[0] = add2(m.i[1], m.i[3]);
    x[1] = sub2(m.r[1], m.r[3]);
    x[2] = sub2(m.i[0], m.i[4]);
    x[3] = add2(m.i[2], m.i[6]);
    x[4] = sub2(m.r[2], m.r[6]);
    x[5] = add2(m.i[5], m.i[7]);
    x[6] = sub2(m.r[5], m.r[7]);
    x[7] = mul2(sub2(add2(m.i[0], m.i[4]), add2(m.i[8], m.i[8])), bc(0.57735026918962576451f));
}

// Warp-blocked link loads and stores for the two sites (layout of lattice.cuh).
// I is the index type: 32-bit when every link offset fits (54 V < 2^31).
template <typename I> __device__ __forceinline__ I loff(I nblk, int d, I s) {
    return ((I)d * nblk + (s >> 5)) * (I)576 + (s & 31);
}
template <typename I>
__device__ __forceinline__ M load(const float *__restrict__ U, I nblk, int d, I sa, I sb) {
    const float *a = U + loff<I>(nblk, d, sa);
    const float *b = U + loff<I>(nblk, d, sb);
    M m;
#pragma unroll
    for (int k = 0; k < 9; k++) {
        m.r[k] = pp(__ldg(a + 32 * k), __ldg(b + 32 * k));
        m.i[k] = pp(__ldg(a + 32 * (9 + k)), __ldg(b + 32 * (9 + k)));
    }
    return m;
}
template <typename I>
__device__ __forceinline__ void store(float *__restrict__ U, I nblk, int d, I sa, I sb, bool va, bool vb, const M &m) {
    float *a = U + loff<I>(nblk, d, sa);
    float *b = U + loff<I>(nblk, d, sb);
    if (va) {
#pragma unroll
        for (int k = 0; k < 9; k++) { a[32 * k] = m.r[k].x; a[32 * (9 + k)] = m.i[k].x; }
    }
    if (vb) {
#pragma unroll
        for (int k = 0; k < 9; k++) { b[32 * k] = m.r[k].y; b[32 * (9 + k)] = m.i[k].y; }
    }
}

// acc += f a b^dagger (the forward staple's last product folded into the sum)
__device__ __forceinline__ void acc_mul_adj(M &acc, P f, const M &a, const M &b) {
    const M c = mul_adj(a, b);
    maxpy(acc, f, c);
}
// acc += f a^dagger b
__device__ __forceinline__ void acc_adj_mul(M &acc, P f, const M &a, const M &b) {
    const M c = adj_mul(a, b);
    maxpy(acc, f, c);
}

// Periodic shift by one in direction d (runtime), orientation o, given the
// coordinate xd of s along d.
template <typename I> __device__ __forceinline__ I shift(const Lat &L, I s, int xd, int d, int o) {
    const int nd = d == 0 ? L.n[0] : (d == 1 ? L.n[1] : L.n[2]);
    const I st = d == 0 ? (I)L.stride[0] : (d == 1 ? (I)L.stride[1] : (I)1);
    if (o > 0) return xd == nd - 1 ? s - (I)(nd - 1) * st : s + st;
    return xd == 0 ? s + (I)(nd - 1) * st : s - st;
}
template <typename I> __device__ __forceinline__ void coords(const Lat &L, I s, int *x) { site_coords<I>(L, s, x); }

}  // namespace pr

// Per-thread measurement columns of the measured step (MEAS below), FP32
// slots in shared memory, column q of thread t at slot[q * MEAS_THREADS]:
// E^2 of the new E per direction, |B_d|^2 of the step's input links per
// direction, the Gauss-law square of the previous state.
constexpr int MEAS_THREADS = 128;
constexpr int MEAS_COLS = 7;

// FastTYMSolver.CombinedUpdate for SU(3) FP32 at sites sa and sb; a lane
// whose flag (va, vb) is false computes but stores nothing (a site past the end
// of the lattice or an inactive cell).  Same equations and staple order as
// update_site in leapfrog.cuh.
//
// MEAS: the step also measures (FieldMeasurements, the per-site terms of the
// BulkQuantities pass).  The new E goes to Eout (E is only read), E^2 of the
// new E is added to slot columns 0-2, and the squared magnetic field of each
// plane is formed from a forward staple that the update computes anyway:
// U_i(x) (U_j(x+i) U_i(x+j)^dagger U_j(x)^dagger) with j = i + 1 is the
// plaquette P_ij(x) of Grid.getPlaquette, so |proj(P_ij) a_d/(a_i a_j)|^2 with
// d = i + 2 goes to column 3 + d (one plane per link, each plane once).  For the Gauss law of the new state the step
// stores W_i(x) = U_i(x)^dagger E_i(x) U_i(x) (its input link, the new E) in
// Wout: the transported term that the next step reads at x + i.
template <typename I, bool HAS_J, bool REUNIT, bool MEAS = false>
__device__ __forceinline__ void update_site_pair(const float *__restrict__ U, float *__restrict__ E,
                                                 const float *__restrict__ J, float *__restrict__ Unext,
                                                 const Lat &L, I sa, I sb, bool va, bool vb,
                                                 float *__restrict__ Eout = nullptr, float *slot = nullptr,
                                                 float *__restrict__ Wout = nullptr) {
    using namespace pr;
    const I V = (I)L.V, nblk = (I)((L.V + 31) >> 5);
    int xa[3], xb[3];
    coords<I>(L, sa, xa);
    coords<I>(L, sb, xb);
    const Deltas<I> Da = deltas<I>(L, xa), Db = deltas<I>(L, xb);
    const P dt = bc(L.dtf), mdt = bc(-L.dtf);
#pragma unroll 1
    for (int i = 0; i < 3; i++) {
        const I pia = sa + Da.f(i), pib = sb + Db.f(i);  // x + i
        M S = mzero();
        [[maybe_unused]] M Pl;  // MEAS: the forward staple of plane i + 1
        // the two staple planes unrolled: their loads and products interleave
        // (1 % faster than the rolled loop at 128^3, same registers).  Plane
        // i + 2 before plane i + 1, each backward staple before the forward
        // one, so that the last staple formed is the forward staple of plane
        // i + 1, whose product with U_i(x) is the plaquette P_{i,i+1}(x).
#pragma unroll
        for (int jj = 2; jj >= 1; jj--) {
            const int j = i + jj >= 3 ? i + jj - 3 : i + jj;
            const P f = bc(LatR<float>::inva2(L, j));
            {
                // (U_i(x-j) U_j(x+i-j))^dagger U_j(x-j)
                const I bja = Da.b(j), bjb = Db.b(j);
                const I mja = sa + bja, mjb = sb + bjb;
                const I pimja = pia + bja, pimjb = pib + bjb;
                const M C = mul(load<I>(U, nblk, i, mja, mjb), load<I>(U, nblk, j, pimja, pimjb));
                acc_adj_mul(S, f, C, load<I>(U, nblk, j, mja, mjb));
            }
            {
                // U_j(x+i) U_i(x+j)^dagger U_j(x)^dagger
                const I pja = sa + Da.f(j), pjb = sb + Db.f(j);
                const M T = mul_adj(load<I>(U, nblk, j, pia, pib), load<I>(U, nblk, i, pja, pjb));
                if constexpr (MEAS) {
                    const M c = mul_adj(T, load<I>(U, nblk, j, sa, sb));
                    maxpy(S, f, c);
                    if (jj == 1) Pl = c;
                } else {
                    acc_mul_adj(S, f, T, load<I>(U, nblk, j, sa, sb));
                }
            }
        }
        const M Ui = load<I>(U, nblk, i, sa, sb);
        P p[8], e[8];
        proj_mul(Ui, S, p);
        if constexpr (MEAS) {
            // |B_d|^2, d = i + 2: P_{i,i+1}(x) is Grid.getPlaquette of B_d with (d, j, k) cyclic
            P b[8];
            proj_mul(Ui, Pl, b);
            const int d = i == 0 ? 2 : i - 1;
            const P bf = bc(LatR<float>::bfac(L, d));
            P b2 = zero2();
#pragma unroll
            for (int a = 0; a < 8; a++) { b[a] = mul2(b[a], bf); b2 = fma2(b[a], b[a], b2); }
            slot[(3 + d) * MEAS_THREADS] += lanes(b2, va, vb);
        }
        const I eo = (I)i * 8 * V;
        const float *ea = E + eo + sa, *eb = E + eo + sb;
#pragma unroll
        for (int a = 0; a < 8; a++) e[a] = fma2(p[a], dt, pp(ea[(I)a * V], eb[(I)a * V]));
        if (HAS_J) {
            const float *ja = J + eo + sa, *jb = J + eo + sb;
            const P jf = bc(LatR<float>::jfac(L, i));
#pragma unroll
            for (int a = 0; a < 8; a++) e[a] = fma2(pp(__ldg(ja + (I)a * V), __ldg(jb + (I)a * V)), jf, e[a]);
        }
        float *wa = (MEAS ? Eout : E) + eo + sa, *wb = (MEAS ? Eout : E) + eo + sb;
        if constexpr (MEAS) {
            P e2 = mul2(e[0], e[0]);
#pragma unroll
            for (int a = 1; a < 8; a++) e2 = fma2(e[a], e[a], e2);
            slot[i * MEAS_THREADS] += lanes(e2, va, vb);
            P w[8];
            act_adj_gen(Ui, e, w);
            float *xa = Wout + eo + sa, *xb = Wout + eo + sb;
            if (va) {
#pragma unroll
                for (int a = 0; a < 8; a++) xa[(I)a * V] = w[a].x;
            }
            if (vb) {
#pragma unroll
                for (int a = 0; a < 8; a++) xb[(I)a * V] = w[a].y;
            }
        }
        if (va) {
#pragma unroll
            for (int a = 0; a < 8; a++) wa[(I)a * V] = e[a].x;
        }
        if (vb) {
#pragma unroll
            for (int a = 0; a < 8; a++) wb[(I)a * V] = e[a].y;
        }
        P v[8];
#pragma unroll
        for (int a = 0; a < 8; a++) v[a] = mul2(mdt, e[a]);
        M Vn = mul(expi(v), Ui);
        if (REUNIT) reunit(Vn);
        store<I>(Unext, nblk, i, sa, sb, va, vb, Vn);
    }
}

// Gauss-law square of the state before a step (Grid.getGaussConstraintSquared,
// Grid.java:944-968):
//   G(x) = sum_i [E_i(x) - W_i(x-i)] gfac_i - rho(x),  W_i(y) = U_i(y)^dagger E_i(y) U_i(y)
// with E the step's input E and W the previous step's transported terms.
template <typename I>
__device__ __forceinline__ pr::P gauss_w_pair(const float *__restrict__ E, const float *__restrict__ W,
                                              const float *__restrict__ rho, const Lat &L, I sa, I sb) {
    using namespace pr;
    const I V = (I)L.V;
    int xa[3], xb[3];
    coords<I>(L, sa, xa);
    coords<I>(L, sb, xb);
    const Deltas<I> Da = deltas<I>(L, xa), Db = deltas<I>(L, xb);
    P gs[8];
#pragma unroll
    for (int a = 0; a < 8; a++) gs[a] = zero2();
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const I mia = sa + Da.b(i), mib = sb + Db.b(i);
        const I eo = (I)i * 8 * V;
        const P gf = bc(LatR<float>::gfac(L, i));
#pragma unroll
        for (int a = 0; a < 8; a++) {
            const P e0 = pp(__ldg(E + eo + (I)a * V + sa), __ldg(E + eo + (I)a * V + sb));
            const P w = pp(__ldg(W + eo + (I)a * V + mia), __ldg(W + eo + (I)a * V + mib));
            gs[a] = fma2(sub2(e0, w), gf, gs[a]);
        }
    }
    if (rho) {
#pragma unroll
        for (int a = 0; a < 8; a++) gs[a] = sub2(gs[a], pp(__ldg(rho + (I)a * V + sa), __ldg(rho + (I)a * V + sb)));
    }
    P g2 = mul2(gs[0], gs[0]);
#pragma unroll
    for (int a = 1; a < 8; a++) g2 = fma2(gs[a], gs[a], g2);
    return g2;
}

}  // namespace opx
