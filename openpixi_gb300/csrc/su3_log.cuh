// su3_log.cuh -- the SU(3) logarithm on the device (FP64).
//
// SU3GroupElement.getAlgebraElement (math/SU3GroupElement.java:476-490) returns
// the hermitian H with exp(i H) = U.  The reference solves the characteristic
// cubic, builds eigenvectors and falls back to a Taylor series near the
// identity and for degenerate eigenvalues; here:
//   * inverse scaling and squaring: principal square roots (Denman-Beavers
//     iteration) halve U's eigenphases until ||U' - I||_F <= 0.5, then
//     log U' = 2 atanh(Z), Z = (U' - I)(U' + I)^-1, by its odd power series,
//     and log U = 2^k log U' -- the principal logarithm, accurate near the
//     identity and for coincident eigenvalues;
//   * when the principal logarithm's trace is not 0 (the eigenphases add up to
//     +-2 pi), the eigen-decomposition: the eigenvalues from the cubic
//     l^3 - a l^2 + b l - det U (Cardano, two Newton steps), the eigenvector of
//     an eigenvalue the largest column of (U - l_i)(U - l_j), and, as in the
//     reference, the phase sum taken off the first eigenvalue's phase.
// The result is returned in generator components x (H = x_a lambda_a / 2).
#pragma once
#include "group.cuh"

namespace opx {
namespace lg {

struct cd {
    double x, y;
};
__device__ __forceinline__ cd mk(double x, double y) { return cd{x, y}; }
__device__ __forceinline__ cd add(cd a, cd b) { return cd{a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ cd sub(cd a, cd b) { return cd{a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ cd mul(cd a, cd b) { return cd{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ cd scl(cd a, double s) { return cd{a.x * s, a.y * s}; }
__device__ __forceinline__ cd conj(cd a) { return cd{a.x, -a.y}; }
__device__ __forceinline__ double abs2(cd a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ double cabs(cd a) { return hypot(a.x, a.y); }
__device__ __forceinline__ cd cdiv(cd a, cd b) {
    const double d = abs2(b);
    return cd{(a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d};
}
__device__ __forceinline__ double arg(cd a) { return atan2(a.y, a.x); }
__device__ __forceinline__ cd polar(double r, double t) {
    double s, c;
    sincos(t, &s, &c);
    return cd{r * c, r * s};
}
__device__ __forceinline__ cd csqrt(cd a) { return polar(sqrt(cabs(a)), 0.5 * arg(a)); }
__device__ __forceinline__ cd ccbrt(cd a) { return polar(cbrt(cabs(a)), arg(a) / 3.0); }

struct CM {
    cd m[3][3];
};
__device__ __forceinline__ CM cm_mul(const CM &a, const CM &b) {
    CM c;
    for (int r = 0; r < 3; r++)
        for (int q = 0; q < 3; q++) {
            cd t = mk(0, 0);
            for (int k = 0; k < 3; k++) t = add(t, mul(a.m[r][k], b.m[k][q]));
            c.m[r][q] = t;
        }
    return c;
}
// inverse by the adjugate
__device__ __forceinline__ CM cm_inv(const CM &A) {
    const auto &a = A.m;
    CM T;
    T.m[0][0] = sub(mul(a[1][1], a[2][2]), mul(a[1][2], a[2][1]));
    T.m[0][1] = sub(mul(a[0][2], a[2][1]), mul(a[0][1], a[2][2]));
    T.m[0][2] = sub(mul(a[0][1], a[1][2]), mul(a[0][2], a[1][1]));
    T.m[1][0] = sub(mul(a[1][2], a[2][0]), mul(a[1][0], a[2][2]));
    T.m[1][1] = sub(mul(a[0][0], a[2][2]), mul(a[0][2], a[2][0]));
    T.m[1][2] = sub(mul(a[0][2], a[1][0]), mul(a[0][0], a[1][2]));
    T.m[2][0] = sub(mul(a[1][0], a[2][1]), mul(a[1][1], a[2][0]));
    T.m[2][1] = sub(mul(a[0][1], a[2][0]), mul(a[0][0], a[2][1]));
    T.m[2][2] = sub(mul(a[0][0], a[1][1]), mul(a[0][1], a[1][0]));
    const cd det = add(add(mul(a[0][0], T.m[0][0]), mul(a[0][1], T.m[1][0])), mul(a[0][2], T.m[2][0]));
    for (int r = 0; r < 3; r++)
        for (int q = 0; q < 3; q++) T.m[r][q] = cdiv(T.m[r][q], det);
    return T;
}
__device__ __forceinline__ double cm_dist_id(const CM &a) {
    double n = 0;
    for (int r = 0; r < 3; r++)
        for (int q = 0; q < 3; q++) n += abs2(sub(a.m[r][q], mk(r == q ? 1.0 : 0.0, 0.0)));
    return sqrt(n);
}

// hermitian matrix (as 9 complex entries) -> generator components, through the
// 9 hermiticized values (SU3GroupElement.hermiticize :468-474) and
// SU3AlgebraElement.get (math/SU3AlgebraElement.java:117-129)
__device__ __forceinline__ void herm_to_gen(const CM &H, double *g) {
    const double v0 = H.m[0][0].x, v4 = H.m[1][1].x, v8 = H.m[2][2].x;
    const double v1 = (H.m[0][1].x + H.m[1][0].x) / 2, v2 = (H.m[0][2].x + H.m[2][0].x) / 2;
    const double v5 = (H.m[1][2].x + H.m[2][1].x) / 2;
    const double v3 = (H.m[1][0].y - H.m[0][1].y) / 2, v6 = (H.m[2][0].y - H.m[0][2].y) / 2;
    const double v7 = (H.m[2][1].y - H.m[1][2].y) / 2;
    g[0] = 2 * v1;
    g[1] = 2 * v3;
    g[2] = v0 - v4;
    g[3] = 2 * v2;
    g[4] = 2 * v6;
    g[5] = 2 * v5;
    g[6] = 2 * v7;
    g[7] = (v0 + v4 - 2 * v8) / sqrt(3.0);
}

__device__ inline void log_eigen(const CM &M, double *gen) {
    const auto &m = M.m;
    const cd a = add(add(m[0][0], m[1][1]), m[2][2]);
    cd tr2 = mk(0, 0);
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) tr2 = add(tr2, mul(m[i][k], m[k][i]));
    const cd b = scl(sub(mul(a, a), tr2), 0.5);
    const cd det = add(sub(mul(m[0][0], sub(mul(m[1][1], m[2][2]), mul(m[1][2], m[2][1]))),
                           mul(m[0][1], sub(mul(m[1][0], m[2][2]), mul(m[1][2], m[2][0])))),
                       mul(m[0][2], sub(mul(m[1][0], m[2][1]), mul(m[1][1], m[2][0]))));
    const cd a3 = scl(a, 1.0 / 3.0);
    const cd p = sub(b, mul(a, a3));
    const cd q = sub(add(scl(mul(mul(a, a), a), -2.0 / 27.0), scl(mul(a, b), 1.0 / 3.0)), det);
    const cd disc = add(scl(mul(q, q), 0.25), scl(mul(mul(p, p), p), 1.0 / 27.0));
    const cd sq = csqrt(disc);
    cd w3 = add(scl(q, -0.5), sq);
    const cd w3b = sub(scl(q, -0.5), sq);
    if (cabs(w3b) > cabs(w3)) w3 = w3b;
    cd lam[3];
    if (cabs(w3) < 1e-300) {
        for (int k = 0; k < 3; k++) lam[k] = a3;
    } else {
        cd w = ccbrt(w3);
        const cd om = polar(1.0, 2.0 * 3.141592653589793 / 3.0);
        for (int k = 0; k < 3; k++) {
            lam[k] = add(sub(w, cdiv(p, scl(w, 3.0))), a3);
            w = mul(w, om);
        }
    }
    for (int k = 0; k < 3; k++)
        for (int it = 0; it < 2; it++) {
            const cd l = lam[k];
            const cd f = sub(mul(add(mul(sub(l, a), l), b), l), det);
            const cd df = add(mul(sub(scl(l, 3.0), scl(a, 2.0)), l), b);
            if (cabs(df) > 1e-300) lam[k] = sub(l, cdiv(f, df));
        }
    double th[3];
    for (int k = 0; k < 3; k++) th[k] = arg(lam[k]);
    th[0] -= th[0] + th[1] + th[2];
    CM H;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) H.m[r][c] = mk(0, 0);
    // coincident eigenvalues: the pair shares the projector I - v v^dagger of the
    // simple one, which carries the phase-sum correction; three: a multiple of I
    const bool s01 = cabs(sub(lam[0], lam[1])) < 1e-9, s02 = cabs(sub(lam[0], lam[2])) < 1e-9,
               s12 = cabs(sub(lam[1], lam[2])) < 1e-9;
    if (s01 && s02) {
        const double t = arg(scl(add(add(lam[0], lam[1]), lam[2]), 1.0 / 3.0));
        for (int r = 0; r < 3; r++) H.m[r][r] = mk(t, 0);
        herm_to_gen(H, gen);
        return;
    }
    int ks = -1, kd0 = -1, kd1 = -1;
    if (s01) { ks = 2; kd0 = 0; kd1 = 1; }
    else if (s02) { ks = 1; kd0 = 0; kd1 = 2; }
    else if (s12) { ks = 0; kd0 = 1; kd1 = 2; }
    for (int k = 0; k < 3; k++) {
        if (ks >= 0 && k != ks) continue;
        const int i = (k + 1) % 3, j = (k + 2) % 3;
        CM A, B;
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) {
                A.m[r][c] = r == c ? sub(m[r][c], lam[i]) : m[r][c];
                B.m[r][c] = r == c ? sub(m[r][c], lam[j]) : m[r][c];
            }
        const CM P = cm_mul(A, B);
        int best = 0;
        double bn = -1;
        for (int c = 0; c < 3; c++) {
            double n = 0;
            for (int r = 0; r < 3; r++) n += abs2(P.m[r][c]);
            if (n > bn) { bn = n; best = c; }
        }
        const double nrm = sqrt(bn);
        cd v[3];
        for (int r = 0; r < 3; r++) v[r] = nrm > 0 ? scl(P.m[r][best], 1.0 / nrm) : mk(r == k ? 1.0 : 0.0, 0.0);
        if (ks < 0) {
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) H.m[r][c] = add(H.m[r][c], scl(mul(v[r], conj(v[c])), th[k]));
        } else {
            double ts = arg(lam[ks]);
            const double td = arg(scl(add(lam[kd0], lam[kd1]), 0.5));
            ts -= ts + 2 * td;
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) {
                    const cd pr = mul(v[r], conj(v[c]));
                    H.m[r][c] = add(scl(pr, ts), scl(sub(mk(r == c ? 1.0 : 0.0, 0.0), pr), td));
                }
        }
    }
    herm_to_gen(H, gen);
}

}  // namespace lg

// generator components x of the hermitian H with exp(i H) = U
__device__ inline void su3_log_gen(const M3<double> &U, double *gen) {
    using namespace lg;
    CM Y, Z, M0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Y.m[i][j] = mk(U.r[3 * i + j], U.i[3 * i + j]);
    M0 = Y;
    int k = 0;
    while (cm_dist_id(Y) > 0.5 && k < 30) {
        // Denman-Beavers: Y -> sqrt(Y)
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) Z.m[r][c] = mk(r == c ? 1.0 : 0.0, 0.0);
        for (int it = 0; it < 50; it++) {
            const CM Yi = cm_inv(Y), Zi = cm_inv(Z);
            double change = 0;
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) {
                    const cd yn = scl(add(Y.m[r][c], Zi.m[r][c]), 0.5);
                    Z.m[r][c] = scl(add(Z.m[r][c], Yi.m[r][c]), 0.5);
                    change += cabs(sub(yn, Y.m[r][c]));
                    Y.m[r][c] = yn;
                }
            if (change < 1e-13) break;  // quadratic convergence: the next step is below rounding
        }
        k++;
    }
    // log Y = 2 atanh(Z), Z = (Y - I)(Y + I)^-1
    CM A, B;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            A.m[r][c] = sub(Y.m[r][c], mk(r == c ? 1.0 : 0.0, 0.0));
            B.m[r][c] = add(Y.m[r][c], mk(r == c ? 1.0 : 0.0, 0.0));
        }
    Z = cm_mul(A, cm_inv(B));
    const CM Z2 = cm_mul(Z, Z);
    CM term = Z, L = Z;
    for (int n = 3; n < 200; n += 2) {
        term = cm_mul(term, Z2);
        double tn = 0;
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) {
                L.m[r][c] = add(L.m[r][c], scl(term.m[r][c], 1.0 / n));
                tn += cabs(term.m[r][c]);
            }
        if (tn / n < 1e-18) break;
    }
    const double scale = 2.0 * ldexp(1.0, k);
    const double trim = L.m[0][0].y + L.m[1][1].y + L.m[2][2].y;
    if (fabs(trim * scale) > 1.0) {  // eigenphases adding up to +-2 pi
        log_eigen(M0, gen);
        return;
    }
    // H = -i log U
    CM H;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) H.m[r][c] = mk(L.m[r][c].y * scale, -L.m[r][c].x * scale);
    herm_to_gen(H, gen);
}

}  // namespace opx
