/*
 * opx_oracle.c -- CPU FP64 oracle (test infrastructure only; see opx_oracle.h).
 *
 * Every function names the reference file:line it restates.  Reference paths
 * are relative to pixi/src/main/java/org/openpixi/pixi/.
 */
#include "opx_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NG_MAX 18
#define NA_MAX 9

int orc_ng(int nc) { return nc == 3 ? 18 : 4; }
int orc_na(int nc) { return nc == 3 ? 9 : 3; }

/* ------------------------------------------------------------------------- */
/* SU(2): quaternion e0 + i e_a sigma_a (math/SU2GroupElement.java:3-14)      */
/* ------------------------------------------------------------------------- */

/* SU2GroupElement.mult, math/SU2GroupElement.java:206-217 */
static void su2_mult(const double *x, const double *a, double *b)
{
    double b0 = x[0] * a[0] - x[1] * a[1] - x[2] * a[2] - x[3] * a[3];
    double b1 = x[0] * a[1] + x[1] * a[0] - x[2] * a[3] + x[3] * a[2];
    double b2 = x[0] * a[2] + x[2] * a[0] - x[3] * a[1] + x[1] * a[3];
    double b3 = x[0] * a[3] + x[3] * a[0] - x[1] * a[2] + x[2] * a[1];
    b[0] = b0; b[1] = b1; b[2] = b2; b[3] = b3;
}

/* SU2AlgebraElement.getLink, math/SU2AlgebraElement.java:140-152 */
static void su2_getlink(const double *v, double *u)
{
    double sum = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    double mod = sqrt(sum) / 2;
    double sinfakt;
    if (mod < 1.E-20)
        sinfakt = 0.0;
    else
        sinfakt = 0.5 / mod * sin(mod);
    u[0] = cos(mod);
    u[1] = v[0] * sinfakt;
    u[2] = v[1] * sinfakt;
    u[3] = v[2] * sinfakt;
}

/* SU2AlgebraElement.act, math/SU2AlgebraElement.java:159-172: proj(u X u^dagger) */
static void su2_act(const double *v, const double *u, double *out)
{
    double xm[4] = {0.0, v[0] / 2, v[1] / 2, v[2] / 2};
    double ua[4] = {u[0], -u[1], -u[2], -u[3]};
    double t[4], r[4];
    su2_mult(xm, ua, t);
    su2_mult(u, t, r);
    out[0] = 2 * r[1];
    out[1] = 2 * r[2];
    out[2] = 2 * r[3];
}

/* ------------------------------------------------------------------------- */
/* SU(3): 3x3 complex, e[0..8] real parts, e[9..17] imaginary parts, row-major */
/* (math/SU3GroupElement.java:3-11)                                            */
/* ------------------------------------------------------------------------- */

/* Term order of SU3GroupElement.mult (math/SU3GroupElement.java:183-208).
 * Entry k of l*r is the left-to-right sum of sign * r[ai] * l[ei] over the six
 * (sign, ai, ei) triplets below.  The order is kept because the CPIC colour
 * charge transport must be bit-identical to the reference. */
static const signed char SU3_TERMS[18][6][3] = {
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

static void su3_mult(const double *l, const double *r, double *out)
{
    double b[18];
    for (int k = 0; k < 18; k++) {
        const signed char(*t)[3] = SU3_TERMS[k];
        double acc = (t[0][0] < 0 ? -r[t[0][1]] : r[t[0][1]]) * l[t[0][2]];
        for (int m = 1; m < 6; m++) {
            double prod = r[t[m][1]] * l[t[m][2]];
            acc = t[m][0] < 0 ? acc - prod : acc + prod;
        }
        b[k] = acc;
    }
    memcpy(out, b, sizeof(b));
}

/* SU3GroupElement.adj, math/SU3GroupElement.java:101-131 */
static void su3_adj(const double *e, double *b)
{
    double t[18];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            t[3 * i + j] = e[3 * j + i];
            t[9 + 3 * i + j] = -e[9 + 3 * j + i];
        }
    memcpy(b, t, sizeof(t));
}

/* SU3GroupElement.proj, math/SU3GroupElement.java:494-505 */
static void su3_proj(const double *e, double *v)
{
    double f[9];
    f[0] = (2 * e[9] - e[13] - e[17]) / 3;
    f[1] = (e[10] + e[12]) / 2;
    f[2] = (e[11] + e[15]) / 2;
    f[3] = (e[1] - e[3]) / 2;
    f[4] = (2 * e[13] - e[17] - e[9]) / 3;
    f[5] = (e[14] + e[16]) / 2;
    f[6] = (e[2] - e[6]) / 2;
    f[7] = (e[5] - e[7]) / 2;
    f[8] = (2 * e[17] - e[9] - e[13]) / 3;
    memcpy(v, f, sizeof(f));
}

/* SU3AlgebraElement hermiticize step shared by act and the log
 * (math/SU3AlgebraElement.java:155-165) */
static void su3_hermiticize(const double *values, double *f)
{
    f[0] = values[0];
    f[4] = values[4];
    f[8] = values[8];
    f[1] = (values[1] + values[3]) / 2;
    f[2] = (values[2] + values[6]) / 2;
    f[5] = (values[5] + values[7]) / 2;
    f[3] = (values[12] - values[10]) / 2;
    f[6] = (values[15] - values[11]) / 2;
    f[7] = (values[16] - values[14]) / 2;
}

/* SU3AlgebraElement.act, math/SU3AlgebraElement.java:144-168 */
static void su3_act(const double *v, const double *a, double *out)
{
    double temp[18] = {v[0], v[1], v[2], v[1], v[4], v[5], v[2], v[5], v[8],
                       0, -v[3], -v[6], v[3], 0, -v[7], v[6], v[7], 0};
    double aadj[18], t1[18], t2[18], f[9];
    su3_adj(a, aadj);
    su3_mult(temp, aadj, t1);
    su3_mult(a, t1, t2);
    su3_hermiticize(t2, f);
    memcpy(out, f, sizeof(f));
}

/* SU3AlgebraElement.square, math/SU3AlgebraElement.java:174-176 */
static double su3_square(const double *v)
{
    return 2 * (v[0] * v[0] + v[4] * v[4] + v[8] * v[8] +
                 2 * (v[1] * v[1] + v[2] * v[2] + v[3] * v[3] + v[5] * v[5] + v[6] * v[6] +
                      v[7] * v[7]));
}

static int su3_normalize(double *vec)
{
    double norm = 0;
    for (int i = 0; i < 6; i++) norm += vec[i] * vec[i];
    norm = sqrt(norm);
    if (fabs(norm) < 1.E-12) return 0;
    for (int i = 0; i < 6; i++) vec[i] /= norm;
    return 1;
}

/* SU3AlgebraElement.groupElementTaylorSeries, math/SU3AlgebraElement.java:389-400 */
static void su3_getlink_taylor(const double *v, int iterations, double *out)
{
    double result[18] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    double inter[18] = {1, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    double mult[18] = {0, v[3], v[6], -v[3], 0, v[7], -v[6], -v[7], 0,
                       v[0], v[1], v[2], v[1], v[4], v[5], v[2], v[5], v[8]};
    for (int i = 1; i <= iterations; i++) {
        double t[18];
        su3_mult(inter, mult, t);
        double s = 1.0 / i;
        for (int k = 0; k < 18; k++) inter[k] = t[k] * s;
        for (int k = 0; k < 18; k++) result[k] = result[k] + inter[k];
    }
    memcpy(out, result, sizeof(result));
}

/* SU3AlgebraElement.groupElementDecompositionMethod + getLink,
 * math/SU3AlgebraElement.java:240-417.  Returns 0 if the Taylor branch must be
 * used with *iters iterations. */
static int su3_getlink_decomp(const double *v, double *out, int *iters)
{
    double trSq = su3_square(v) / 2;
    if (trSq <= 1.E-0) { *iters = 15; return 0; }
    double det = -v[2] * v[2] * v[4] + v[6] * (2 * v[3] * v[5] - v[4] * v[6] + 2 * v[1] * v[7]) +
                 2 * v[2] * (v[1] * v[5] - v[3] * v[7]) - (v[1] * v[1] + v[3] * v[3]) * v[8] -
                 v[0] * (v[5] * v[5] + v[7] * v[7] - v[4] * v[8]);
    double linTerm = -trSq / 2;
    double preRad = det * det + pow(linTerm, 3) * 4 / 27;
    if (preRad > 0) preRad = 0;
    double radIm = sqrt(-preRad);
    double preOmegaRe = det / 2, preOmegaIm = radIm / 2;
    double th = atan2(preOmegaIm, preOmegaRe);
    double r = pow(preOmegaRe * preOmegaRe + preOmegaIm * preOmegaIm, 1. / 6);
    double ths[3], ph[3];
    for (int i = 0; i < 3; i++) ths[i] = (th + 2 * M_PI * i) / 3;
    for (int i = 0; i < 3; i++) {
        if (fabs(r) == 0)
            ph[i] = 0;
        else
            ph[i] = r * cos(ths[i]) - (linTerm * cos(ths[i])) / (3 * r);
    }
    const double dc = 1.E-2;
    if (fabs(1 - ph[0] / ph[1]) < dc || fabs(1 - ph[0] / ph[2]) < dc ||
        fabs(1 - ph[1] / ph[2]) < dc) {
        *iters = 25;
        return 0;
    }
    double vec[3][6];
    for (int i = 0; i < 3; i++) {
        double opp = ph[(i + 1) % 3] * ph[(i + 2) % 3];
        double ops = ph[0] + ph[1] + ph[2] - ph[i];
        double *w = vec[i];
        w[0] = v[0] * v[0] + v[1] * v[1] + v[2] * v[2] + v[3] * v[3] + v[6] * v[6] + opp - v[0] * ops;
        w[1] = v[2] * v[5] + v[6] * v[7] + v[1] * (v[0] + v[4] - ops);
        w[2] = v[1] * v[5] - v[3] * v[7] + v[2] * (v[0] + v[8] - ops);
        w[3] = 0;
        w[4] = v[5] * v[6] - v[2] * v[7] + v[3] * (v[0] + v[4] - ops);
        w[5] = v[3] * v[5] + v[1] * v[7] + v[6] * (v[0] + v[8] - ops);
        if (!su3_normalize(w)) {
            w[0] = v[2] * v[5] + v[6] * v[7] + v[1] * (v[0] + v[4] - ops);
            w[1] = v[1] * v[1] + v[3] * v[3] + v[4] * v[4] + v[5] * v[5] + v[7] * v[7] + opp - v[4] * ops;
            w[2] = v[1] * v[2] + v[3] * v[6] + v[5] * (v[4] + v[8] - ops);
            w[3] = v[2] * v[7] - v[5] * v[6] - v[3] * (v[0] + v[4] - ops);
            w[4] = 0;
            w[5] = v[1] * v[6] - v[2] * v[3] + v[7] * (v[4] + v[8] - ops);
            if (!su3_normalize(w)) {
                w[0] = v[1] * v[5] - v[3] * v[7] + v[2] * (v[0] + v[8] - ops);
                w[1] = v[1] * v[2] + v[3] * v[6] + v[5] * (v[4] + v[8] - ops);
                w[2] = v[2] * v[2] + v[5] * v[5] + v[6] * v[6] + v[7] * v[7] + v[8] * v[8] + opp - v[8] * ops;
                w[3] = -v[3] * v[5] - v[1] * v[7] - v[6] * (v[0] + v[8] - ops);
                w[4] = -v[1] * v[6] + v[2] * v[3] - v[7] * (v[4] + v[8] - ops);
                w[5] = 0;
                if (!su3_normalize(w)) {
                    for (int j = 0; j < 6; j++) w[j] = 0;
                    w[i] = 1;
                }
            }
        }
    }
    double unit[18] = {vec[0][0], vec[1][0], vec[2][0], vec[0][1], vec[1][1], vec[2][1],
                       vec[0][2], vec[1][2], vec[2][2], vec[0][3], vec[1][3], vec[2][3],
                       vec[0][4], vec[1][4], vec[2][4], vec[0][5], vec[1][5], vec[2][5]};
    double diag[18] = {cos(ph[0]), 0, 0, 0, cos(ph[1]), 0, 0, 0, cos(ph[2]),
                       sin(ph[0]), 0, 0, 0, sin(ph[1]), 0, 0, 0, sin(ph[2])};
    double t1[18], ua[18];
    su3_mult(unit, diag, t1);
    su3_adj(unit, ua);
    su3_mult(t1, ua, out);
    return 1;
}

static void su3_getlink(const double *v, double *out)
{
    int iters = 15;
    if (!su3_getlink_decomp(v, out, &iters)) su3_getlink_taylor(v, iters, out);
}

/* SU3AlgebraElement.get(j), math/SU3AlgebraElement.java:117-129 */
static void su3_to_gen(const double *v, double *g)
{
    double s3 = sqrt(3);
    g[0] = 2 * v[1];
    g[1] = 2 * v[3];
    g[2] = v[0] - v[4];
    g[3] = 2 * v[2];
    g[4] = 2 * v[6];
    g[5] = 2 * v[5];
    g[6] = 2 * v[7];
    g[7] = (v[0] + v[4] - 2 * v[8]) / s3;
}

/* SU3AlgebraElement(double[8]) -> set(j, value) for j=0..7 from zero,
 * math/SU3AlgebraElement.java:36-49, 93-115 */
static void su3_from_gen(const double *gen, double *v)
{
    double w[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int j = 0; j < 8; j++) {
        double g[8];
        su3_to_gen(w, g);
        double diff = (gen[j] - g[j]) / 2;
        switch (j) {
        case 0: w[1] += diff; break;
        case 1: w[3] += diff; break;
        case 2: w[0] += diff; w[4] -= diff; break;
        case 3: w[2] += diff; break;
        case 4: w[6] += diff; break;
        case 5: w[5] += diff; break;
        case 6: w[7] += diff; break;
        case 7:
            w[0] += diff / sqrt(3);
            w[4] += diff / sqrt(3);
            w[8] -= 2 * diff / sqrt(3);
            break;
        }
    }
    memcpy(v, w, sizeof(w));
}

/* SU3GroupElement.getAlgebraElement (math/SU3GroupElement.java:476-490): the
 * hermitian H with exp(i H) = U, restated with methods of our own (the
 * reference solves the characteristic cubic, builds eigenvectors and falls
 * back to a Taylor series near the identity and for degenerate eigenvalues).
 *
 * su3_log: inverse scaling and squaring.  Principal square roots (the
 * Denman-Beavers iteration) halve U's eigenphases until ||U' - I||_F <= 0.5,
 * then log U' = 2 atanh(Z), Z = (U' - I)(U' + I)^-1, by its odd power series,
 * and log U = 2^k log U'.  This is the principal logarithm; when its trace is
 * not 0 (the eigenphases add up to +-2 pi) the reference instead takes the
 * phase sum off one eigenvalue, which su3_log_eigen does.
 *
 * su3_log_eigen: the eigenvalues are the roots of l^3 - a l^2 + b l - det U
 * (Cardano in complex arithmetic, two Newton steps), the eigenvector of a
 * simple eigenvalue the largest column of (U - l_i)(U - l_j); the phase sum is
 * taken off the first phase.  Accurate for well separated eigenvalues. */
static void su3_log_eigen(const double *u, double *v)
{
    double complex M[3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) M[i][j] = u[3 * i + j] + I * u[9 + 3 * i + j];
    double complex a = M[0][0] + M[1][1] + M[2][2], tr2 = 0;
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) tr2 += M[i][k] * M[k][i];
    double complex b = (a * a - tr2) / 2;
    double complex det = M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) -
                         M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
                         M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
    double complex p = b - a * a / 3, q = -2.0 * a * a * a / 27 + a * b / 3 - det;
    double complex disc = q * q / 4 + p * p * p / 27, sq = csqrt(disc);
    double complex w3 = -q / 2 + sq;
    if (cabs(-q / 2 - sq) > cabs(w3)) w3 = -q / 2 - sq;
    double complex lam[3];
    if (cabs(w3) < 1e-300) {
        for (int k = 0; k < 3; k++) lam[k] = a / 3;
    } else {
        double complex w = cpow(w3, 1.0 / 3.0), om = cexp(2.0 * M_PI * I / 3.0);
        for (int k = 0; k < 3; k++) {
            lam[k] = w - p / (3.0 * w) + a / 3;
            w *= om;
        }
    }
    for (int k = 0; k < 3; k++)
        for (int it = 0; it < 2; it++) {
            double complex l = lam[k];
            double complex f = ((l - a) * l + b) * l - det, df = (3.0 * l - 2.0 * a) * l + b;
            if (cabs(df) > 1e-300) lam[k] = l - f / df;
        }
    double th[3];
    for (int k = 0; k < 3; k++) th[k] = carg(lam[k]);
    th[0] -= th[0] + th[1] + th[2];
    /* coincident eigenvalues */
    int same01 = cabs(lam[0] - lam[1]) < 1e-9, same02 = cabs(lam[0] - lam[2]) < 1e-9,
        same12 = cabs(lam[1] - lam[2]) < 1e-9;
    double complex H[3][3] = {{0}};
    if (same01 && same02) {
        double t = carg((lam[0] + lam[1] + lam[2]) / 3.0);
        for (int i = 0; i < 3; i++) H[i][i] = t;
    } else {
        int simple[3] = {1, 1, 1}, ks = -1, kd0 = -1, kd1 = -1;
        if (same01) { simple[0] = simple[1] = 0; ks = 2; kd0 = 0; kd1 = 1; }
        else if (same02) { simple[0] = simple[2] = 0; ks = 1; kd0 = 0; kd1 = 2; }
        else if (same12) { simple[1] = simple[2] = 0; ks = 0; kd0 = 1; kd1 = 2; }
        double complex vec[3][3];
        for (int k = 0; k < 3; k++) {
            if (!simple[k] && k != ks) continue;
            int i = (k + 1) % 3, j = (k + 2) % 3;
            double complex A[3][3], B[3][3], P[3][3];
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) {
                    A[r][c] = M[r][c] - (r == c ? lam[i] : 0);
                    B[r][c] = M[r][c] - (r == c ? lam[j] : 0);
                }
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) {
                    P[r][c] = 0;
                    for (int m = 0; m < 3; m++) P[r][c] += A[r][m] * B[m][c];
                }
            int best = 0;
            double bn = -1;
            for (int c = 0; c < 3; c++) {
                double n = 0;
                for (int r = 0; r < 3; r++) n += creal(P[r][c] * conj(P[r][c]));
                if (n > bn) { bn = n; best = c; }
            }
            double nrm = sqrt(bn);
            for (int r = 0; r < 3; r++) vec[k][r] = nrm > 0 ? P[r][best] / nrm : (r == k ? 1.0 : 0.0);
        }
        if (ks < 0) {
            for (int k = 0; k < 3; k++)
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++) H[r][c] += th[k] * vec[k][r] * conj(vec[k][c]);
        } else {
            /* the simple eigenvalue's phase carries the trace correction of th[0] */
            double ts = th[ks], td = carg((lam[kd0] + lam[kd1]) / 2.0);
            double sum = ts + 2 * td;
            ts -= sum;
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) {
                    double complex pr = vec[ks][r] * conj(vec[ks][c]);
                    H[r][c] = ts * pr + td * ((r == c ? 1.0 : 0.0) - pr);
                }
        }
    }
    double vals[18];
    for (int i = 0; i < 9; i++) { vals[i] = creal(H[i / 3][i % 3]); vals[9 + i] = cimag(H[i / 3][i % 3]); }
    su3_hermiticize(vals, v);
}

typedef double complex cm3[3][3];

static void cm3_mul(const cm3 A, const cm3 B, cm3 C)
{
    cm3 T;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            double complex t = 0;
            for (int m = 0; m < 3; m++) t += A[r][m] * B[m][c];
            T[r][c] = t;
        }
    memcpy(C, T, sizeof(cm3));
}

/* inverse by the adjugate */
static void cm3_inv(const cm3 A, cm3 B)
{
    cm3 T;
    T[0][0] = A[1][1] * A[2][2] - A[1][2] * A[2][1];
    T[0][1] = A[0][2] * A[2][1] - A[0][1] * A[2][2];
    T[0][2] = A[0][1] * A[1][2] - A[0][2] * A[1][1];
    T[1][0] = A[1][2] * A[2][0] - A[1][0] * A[2][2];
    T[1][1] = A[0][0] * A[2][2] - A[0][2] * A[2][0];
    T[1][2] = A[0][2] * A[1][0] - A[0][0] * A[1][2];
    T[2][0] = A[1][0] * A[2][1] - A[1][1] * A[2][0];
    T[2][1] = A[0][1] * A[2][0] - A[0][0] * A[2][1];
    T[2][2] = A[0][0] * A[1][1] - A[0][1] * A[1][0];
    double complex det = A[0][0] * T[0][0] + A[0][1] * T[1][0] + A[0][2] * T[2][0];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) B[r][c] = T[r][c] / det;
}

static double cm3_dist_id(const cm3 A)
{
    double n = 0;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            double complex d = A[r][c] - (r == c ? 1.0 : 0.0);
            n += creal(d * conj(d));
        }
    return sqrt(n);
}

static void su3_log(const double *u, double *v)
{
    cm3 Y, Z, Yi, Zi, L;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) Y[i][j] = u[3 * i + j] + I * u[9 + 3 * i + j];
    int k = 0;
    while (cm3_dist_id(Y) > 0.5 && k < 30) {
        /* Denman-Beavers: Y -> sqrt(Y) */
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) Z[r][c] = r == c ? 1.0 : 0.0;
        for (int it = 0; it < 50; it++) {
            cm3_inv(Y, Yi);
            cm3_inv(Z, Zi);
            double change = 0;
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++) {
                    double complex yn = 0.5 * (Y[r][c] + Zi[r][c]);
                    Z[r][c] = 0.5 * (Z[r][c] + Yi[r][c]);
                    change += cabs(yn - Y[r][c]);
                    Y[r][c] = yn;
                }
            if (change < 1e-13) break;  /* quadratic convergence: the next step is below rounding */
        }
        k++;
    }
    /* log Y = 2 atanh(Z), Z = (Y - I)(Y + I)^-1 */
    cm3 A, B, Z2, term;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) {
            A[r][c] = Y[r][c] - (r == c ? 1.0 : 0.0);
            B[r][c] = Y[r][c] + (r == c ? 1.0 : 0.0);
        }
    cm3_inv(B, B);
    cm3_mul(A, B, Z);
    cm3_mul(Z, Z, Z2);
    memcpy(term, Z, sizeof(cm3));
    memcpy(L, Z, sizeof(cm3));
    for (int n = 3; n < 200; n += 2) {
        cm3_mul(term, Z2, term);
        double tn = 0;
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) {
                L[r][c] += term[r][c] / n;
                tn += cabs(term[r][c]);
            }
        if (tn / n < 1e-18) break;
    }
    double scale = 2.0 * ldexp(1.0, k);
    double complex tr = 0;
    for (int r = 0; r < 3; r++) tr += L[r][r];
    if (fabs(cimag(tr) * scale) > 1.0) {  /* eigenphases adding up to +-2 pi */
        su3_log_eigen(u, v);
        return;
    }
    double vals[18];
    /* H = -i log U */
    for (int i = 0; i < 9; i++) {
        double complex h = -I * L[i / 3][i % 3] * scale;
        vals[i] = creal(h);
        vals[9 + i] = cimag(h);
    }
    su3_hermiticize(vals, v);
}

/* the generator components of getAlgebraElement (SU(3)) */
void orc_su3_log_gen(const double *u, double *gen)
{
    double v[9];
    su3_log(u, v);
    su3_to_gen(v, gen);
}

/* SU3GroupElement.pow(x) = getAlgebraElement().mult(x).getLink() (math/SU3GroupElement.java:516-518) */
void orc_su3_pow(const double *u, double x, double *out)
{
    double v[9];
    su3_log(u, v);
    for (int k = 0; k < 9; k++) v[k] *= x;
    su3_getlink(v, out);
}

/* ---- generic dispatch ---- */
void orc_group_mult(int nc, const double *l, const double *r, double *out)
{
    if (nc == 3) su3_mult(l, r, out); else su2_mult(l, r, out);
}
void orc_group_adj(int nc, const double *u, double *out)
{
    if (nc == 3) { su3_adj(u, out); return; }
    out[0] = u[0]; out[1] = -u[1]; out[2] = -u[2]; out[3] = -u[3];
}
void orc_group_proj(int nc, const double *u, double *alg)
{
    if (nc == 3) { su3_proj(u, alg); return; }
    /* SU2GroupElement.proj, math/SU2GroupElement.java:254-263 */
    alg[0] = 2 * u[1]; alg[1] = 2 * u[2]; alg[2] = 2 * u[3];
}
void orc_alg_getlink(int nc, const double *alg, double *u)
{
    if (nc == 3) su3_getlink(alg, u); else su2_getlink(alg, u);
}
void orc_alg_act(int nc, const double *alg, const double *g, double *out)
{
    if (nc == 3) su3_act(alg, g, out); else su2_act(alg, g, out);
}
double orc_alg_square(int nc, const double *alg)
{
    if (nc == 3) return su3_square(alg);
    return alg[0] * alg[0] + alg[1] * alg[1] + alg[2] * alg[2];
}
void orc_alg_to_gen(int nc, const double *alg, double *gen)
{
    if (nc == 3) { su3_to_gen(alg, gen); return; }
    gen[0] = alg[0]; gen[1] = alg[1]; gen[2] = alg[2];
}
void orc_gen_to_alg(int nc, const double *gen, double *alg)
{
    if (nc == 3) { su3_from_gen(gen, alg); return; }
    alg[0] = gen[0]; alg[1] = gen[1]; alg[2] = gen[2];
}

/* Bilinear form 2 tr(XY) in the algebra layout (the polarisation of square()). */
static double alg_dot(int nc, const double *x, const double *y)
{
    if (nc == 3)
        return 2 * (x[0] * y[0] + x[4] * y[4] + x[8] * y[8] +
                    2 * (x[1] * y[1] + x[2] * y[2] + x[3] * y[3] + x[5] * y[5] + x[6] * y[6] +
                         x[7] * y[7]));
    return x[0] * y[0] + x[1] * y[1] + x[2] * y[2];
}

/* ------------------------------------------------------------------------- */
/* Grid (physics/grid/Grid.java)                                              */
/* ------------------------------------------------------------------------- */
static long vol(const orc_params *p) { return (long)p->n[0] * p->n[1] * p->n[2]; }

/* Grid.shift, physics/grid/Grid.java:802-823 (cummulatedCellCount :534-538) */
long orc_shift(const orc_params *p, long index, int direction, int orientation)
{
    long ccc[4];
    ccc[3] = 1;
    for (int i = 2; i >= 0; i--) ccc[i] = ccc[i + 1] * p->n[i];
    long result = index;
    long directionIndex = index / ccc[direction + 1];
    long within = directionIndex % p->n[direction];
    if (orientation > 0) {
        if (within == p->n[direction] - 1) result -= ccc[direction];
        result += ccc[direction + 1];
    } else if (orientation < 0) {
        if (within == 0) result += ccc[direction];
        result -= ccc[direction + 1];
    }
    return result;
}

static inline const double *link(const orc_params *p, const double *U, long index, int dir)
{
    return U + ((size_t)index * 3 + dir) * orc_ng(p->nc);
}

/* Grid.getLink, physics/grid/Grid.java:712-727 */
static void get_link(const orc_params *p, const double *U, long index, int dir, int orient,
                     double *out)
{
    int ng = orc_ng(p->nc);
    if (orient < 0)
        orc_group_adj(p->nc, link(p, U, orc_shift(p, index, dir, orient), dir), out);
    else
        memcpy(out, link(p, U, index, dir), sizeof(double) * ng);
}

static void group_identity(int nc, double *u)
{
    int ng = orc_ng(nc);
    memset(u, 0, sizeof(double) * ng);
    if (nc == 3) { u[0] = u[4] = u[8] = 1; } else u[0] = 1;
}

/* Grid.getStapleSum, physics/grid/Grid.java:675-696 */
void orc_staple_sum(const orc_params *p, const double *U, long index, int d, double *S)
{
    int nc = p->nc, ng = orc_ng(nc);
    double U1[NG_MAX], U2[NG_MAX], t[NG_MAX], adj[NG_MAX];
    memset(S, 0, sizeof(double) * ng);
    long ci1 = orc_shift(p, index, d, 1);
    for (int i = 0; i < 3; i++) {
        if (i == d) continue;
        long ci2 = orc_shift(p, index, i, 1);
        long ci3 = orc_shift(p, ci1, i, -1);
        long ci4 = orc_shift(p, index, i, -1);
        orc_group_adj(nc, link(p, U, ci2, d), adj);
        orc_group_mult(nc, link(p, U, ci1, i), adj, U1);
        orc_group_adj(nc, link(p, U, index, i), adj);
        orc_group_mult(nc, U1, adj, t);
        memcpy(U1, t, sizeof(double) * ng);
        orc_group_mult(nc, link(p, U, ci4, d), link(p, U, ci3, i), U2);
        orc_group_adj(nc, U2, t);
        orc_group_mult(nc, t, link(p, U, ci4, i), U2);
        double areaFactor = 1.0 / pow(p->a[i], 2);
        for (int k = 0; k < ng; k++) U1[k] = U1[k] + U2[k];
        for (int k = 0; k < ng; k++) U1[k] = U1[k] * areaFactor;
        for (int k = 0; k < ng; k++) S[k] = S[k] + U1[k];
    }
}

/* Grid.getPlaquette, physics/grid/Grid.java:609-642 */
void orc_plaquette(const orc_params *p, const double *U, long index, int d1, int d2, int o1,
                   int o2, double *out)
{
    int nc = p->nc, ng = orc_ng(nc);
    long x1 = index;
    long x2 = orc_shift(p, x1, d1, o1);
    long x3 = orc_shift(p, x2, d2, o2);
    long x4 = orc_shift(p, x3, d1, -o1);
    double L[4][NG_MAX], A[NG_MAX], T[NG_MAX];
    get_link(p, U, x1, d1, o1, L[0]);
    get_link(p, U, x2, d2, o2, L[1]);
    get_link(p, U, x3, d1, -o1, L[2]);
    get_link(p, U, x4, d2, -o2, L[3]);
    group_identity(nc, A);
    for (int k = 0; k < 4; k++) {
        orc_group_mult(nc, A, L[k], T);
        memcpy(A, T, sizeof(double) * ng);
    }
    memcpy(out, A, sizeof(double) * ng);
}

/* Grid.getB, physics/grid/Grid.java:901-920 */
void orc_get_b(const orc_params *p, const double *U, long index, int dir, double *alg)
{
    int j = 0, k = 0, na = orc_na(p->nc);
    switch (dir) {
    case 0: j = 1; k = 2; break;
    case 1: j = 2; k = 0; break;
    case 2: j = 0; k = 1; break;
    }
    double P[NG_MAX];
    orc_plaquette(p, U, index, j, k, 1, 1, P);
    orc_group_proj(p->nc, P, alg);
    double f = p->a[dir] / (p->a[j] * p->a[k]);
    for (int c = 0; c < na; c++) alg[c] = alg[c] * f;
}

/* Grid.getGaussConstraint, physics/grid/Grid.java:944-968 */
void orc_gauss_constraint(const orc_params *p, const double *U, const double *E,
                          const double *rho, long index, double *alg)
{
    int nc = p->nc, na = orc_na(nc);
    double gauss[NA_MAX] = {0}, e[NA_MAX], g[NG_MAX];
    for (int i = 0; i < 3; i++) {
        double unitFactor = p->g * p->a[i];
        long sh = orc_shift(p, index, i, -1);
        get_link(p, U, index, i, -1, g);
        orc_alg_act(nc, E + ((size_t)sh * 3 + i) * na, g, e);
        for (int c = 0; c < na; c++) e[c] = e[c] * -1.0;
        for (int c = 0; c < na; c++) e[c] = e[c] + E[((size_t)index * 3 + i) * na + c];
        double f = 1.0 / (p->a[i] * unitFactor);
        for (int c = 0; c < na; c++) e[c] = e[c] * f;
        for (int c = 0; c < na; c++) gauss[c] = gauss[c] + e[c];
    }
    for (int c = 0; c < na; c++) alg[c] = gauss[c] - rho[(size_t)index * na + c];
}

/* ------------------------------------------------------------------------- */
/* FastTYMSolver (physics/fields/FastTYMSolver.java)                          */
/* ------------------------------------------------------------------------- */

/* CombinedUpdate.execute, physics/fields/FastTYMSolver.java:50-62 (the unit
 * factor -g*a_i*dt is set in step(), :25-32) */
static void combined_update_site(const orc_params *p, const double *U, double *E,
                                 const double *J, double *Unext, long index)
{
    int nc = p->nc, ng = orc_ng(nc), na = orc_na(nc);
    double S[NG_MAX], temp[NG_MAX], pr[NA_MAX], ve[NA_MAX], V[NG_MAX], t[NG_MAX];
    for (int i = 0; i < 3; i++) {
        double unitFactor = -(p->g * p->a[i]) * p->dt;
        const double *Ui = link(p, U, index, i);
        double *Ei = E + ((size_t)index * 3 + i) * na;
        const double *Ji = J + ((size_t)index * 3 + i) * na;
        orc_staple_sum(p, U, index, i, S);
        orc_group_mult(nc, Ui, S, temp);
        orc_group_proj(nc, temp, pr);
        for (int c = 0; c < na; c++) Ei[c] = Ei[c] + pr[c] * p->dt;
        for (int c = 0; c < na; c++) Ei[c] = Ei[c] + Ji[c] * unitFactor;
        for (int c = 0; c < na; c++) ve[c] = Ei[c] * -p->dt;
        orc_alg_getlink(nc, ve, V);
        orc_group_mult(nc, V, Ui, t);
        memcpy(Unext + ((size_t)index * 3 + i) * ng, t, sizeof(double) * ng);
    }
}

void orc_update_grid(const orc_params *p, const double *U, double *E, const double *J,
                     double *Unext, const uint8_t *active)
{
    long V = vol(p);
    for (long x = 0; x < V; x++)
        if (!active || active[x]) combined_update_site(p, U, E, J, Unext, x);
}

void orc_update_grid_omp(const orc_params *p, const double *U, double *E, const double *J,
                         double *Unext, const uint8_t *active, int nthreads)
{
    long V = vol(p);
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (long x = 0; x < V; x++)
        if (!active || active[x]) combined_update_site(p, U, E, J, Unext, x);
    (void)nthreads;
}

/* The same over the site range [s0, s1) (a bounded sample of a large lattice). */
void orc_update_grid_range_omp(const orc_params *p, const double *U, double *E, const double *J,
                               double *Unext, const uint8_t *active, long s0, long s1, int nthreads)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (long x = s0; x < s1; x++)
        if (!active || active[x]) combined_update_site(p, U, E, J, Unext, x);
    (void)nthreads;
}

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* UpdateLinks.execute, physics/fields/FastTYMSolver.java:73-83 */
void orc_update_links(const orc_params *p, const double *U, const double *E, double *Unext,
                      const uint8_t *active)
{
    int nc = p->nc, ng = orc_ng(nc), na = orc_na(nc);
    long Vn = vol(p);
    for (long x = 0; x < Vn; x++) {
        if (active && !active[x]) continue;
        for (int k = 0; k < 3; k++) {
            double ve[NA_MAX], V[NG_MAX], t[NG_MAX];
            const double *Ek = E + ((size_t)x * 3 + k) * na;
            for (int c = 0; c < na; c++) ve[c] = Ek[c] * -p->dt;
            orc_alg_getlink(nc, ve, V);
            orc_group_mult(nc, V, link(p, U, x, k), t);
            memcpy(Unext + ((size_t)x * 3 + k) * ng, t, sizeof(double) * ng);
        }
    }
}

/* TemporalYangMillsSolver.step (physics/fields/TemporalYangMillsSolver.java:24-40):
 * the same equations as FastTYMSolver in plaquette form, in two passes over
 * the cells.  UpdateFields.execute (:58-73): for each direction i,
 * temp = sum_{j != i} [getPlaquette(x, i, j, 1, 1, 0) + getPlaquette(x, i, j, 1, -1, 0)]
 * * (dt / a_j^2), then E_i += proj(temp) and E_i += J_i * (-dt * g a_i);
 * UpdateLinks.execute (:83-93) as FastTYMSolver's. */
void orc_update_grid_tym(const orc_params *p, const double *U, double *E, const double *J,
                         double *Unext, const uint8_t *active)
{
    int nc = p->nc, ng = orc_ng(nc), na = orc_na(nc);
    long Vn = vol(p);
    double plaquetteFactor[3], unitFactor[3];
    for (int j = 0; j < 3; j++) {
        plaquetteFactor[j] = p->dt / pow(p->a[j], 2);
        unitFactor[j] = -p->dt * (p->g * p->a[j]);
    }
    for (long x = 0; x < Vn; x++) {
        if (active && !active[x]) continue;
        for (int i = 0; i < 3; i++) {
            double temp[NG_MAX], P[NG_MAX], pr[NA_MAX];
            memset(temp, 0, sizeof(double) * ng);
            for (int j = 0; j < 3; j++) {
                if (j == i) continue;
                orc_plaquette(p, U, x, i, j, 1, 1, P);
                for (int k = 0; k < ng; k++) P[k] = P[k] * plaquetteFactor[j];
                for (int k = 0; k < ng; k++) temp[k] = temp[k] + P[k];
                orc_plaquette(p, U, x, i, j, 1, -1, P);
                for (int k = 0; k < ng; k++) P[k] = P[k] * plaquetteFactor[j];
                for (int k = 0; k < ng; k++) temp[k] = temp[k] + P[k];
            }
            double *Ei = E + ((size_t)x * 3 + i) * na;
            const double *Ji = J + ((size_t)x * 3 + i) * na;
            orc_group_proj(nc, temp, pr);
            for (int c = 0; c < na; c++) Ei[c] = Ei[c] + pr[c];
            for (int c = 0; c < na; c++) Ei[c] = Ei[c] + Ji[c] * unitFactor[i];
        }
    }
    orc_update_links(p, U, E, Unext, active);
}

/* ------------------------------------------------------------------------- */
/* Reductions                                                                 */
/* ------------------------------------------------------------------------- */

/* FieldMeasurements EFieldSquared/BFieldSquared/GaussLaw/TotalChargeSquared
 * (physics/measurements/FieldMeasurements.java:68-231) combined as
 * BulkQuantitiesInTime.calculate does (diagnostics/methods/BulkQuantitiesInTime.java:83-121) */
void orc_bulk(const orc_params *p, const double *U, const double *Unext, const double *E,
              const double *rho, const uint8_t *eval, double *out)
{
    int nc = p->nc, na = orc_na(nc);
    long V = vol(p);
    double ev[3] = {0, 0, 0}, bv[3] = {0, 0, 0}, gsum = 0.0, charge = 0.0;
    double uf[3];
    for (int i = 0; i < 3; i++) uf[i] = pow(p->g * p->a[i], -2);
    for (long x = 0; x < V; x++) {
        if (eval && !eval[x]) continue;
        double b0[NA_MAX], b1[NA_MAX], gg[NA_MAX];
        for (int i = 0; i < 3; i++) {
            double r = 0.0;
            r += orc_alg_square(nc, E + ((size_t)x * 3 + i) * na) * uf[i];
            ev[i] += r;
        }
        for (int i = 0; i < 3; i++) {
            orc_get_b(p, U, x, i, b0);
            orc_get_b(p, Unext, x, i, b1);
            double r = 0.0;
            r += 0.5 * (orc_alg_square(nc, b0) + orc_alg_square(nc, b1)) * uf[i];
            bv[i] += r;
        }
        orc_gauss_constraint(p, U, E, rho, x, gg);
        gsum += orc_alg_square(nc, gg);
        charge += orc_alg_square(nc, rho + (size_t)x * na);
    }
    double es[3], bs[3];
    for (int i = 0; i < 3; i++) { es[i] = ev[i] / V; bs[i] = bv[i] / V; }
    out[0] = es[0]; out[1] = es[1]; out[2] = es[2];
    out[3] = bs[0]; out[4] = bs[1]; out[5] = bs[2];
    out[6] = -es[0] + es[1] + es[2] - bs[0] + bs[1] + bs[2];
    out[7] = +es[0] - es[1] + es[2] + bs[0] - bs[1] + bs[2];
    out[8] = +es[0] + es[1] - es[2] + bs[0] + bs[1] - bs[2];
    out[9] = gsum / V;
    out[10] = sqrt(charge) / V;
    out[11] = es[0] + es[1] + es[2];
    out[12] = bs[0] + bs[1] + bs[2];
}

/* EnergyDensity.ComponentComputation, diagnostics/methods/EnergyDensity.java:119-166.
 * Kept as in the reference: the unit factor of direction 0 for every d, and B
 * summed over U and Unext before squaring. */
void orc_energy_density(const orc_params *p, const double *U, const double *Unext,
                        const double *E, const uint8_t *eval, double *out)
{
    int nc = p->nc, na = orc_na(nc);
    long V = vol(p);
    double uf = pow(p->g * p->a[0], -2);
    for (long x = 0; x < V; x++) {
        out[x] = 0.0;
        if (eval && !eval[x]) continue;
        for (int d = 0; d < 3; d++) {
            double b0[NA_MAX], b1[NA_MAX];
            orc_get_b(p, U, x, d, b0);
            orc_get_b(p, Unext, x, d, b1);
            for (int c = 0; c < na; c++) b0[c] = b0[c] + b1[c];
            double Esq = 0.5 * orc_alg_square(nc, E + ((size_t)x * 3 + d) * na);
            double Bsq = 0.25 * orc_alg_square(nc, b0);
            out[x] += (Esq + Bsq) * uf;
        }
    }
}

static void cell_pos(const orc_params *p, long index, int *pos)
{
    for (int i = 2; i >= 0; i--) {
        pos[i] = (int)(index % p->n[i]);
        index -= pos[i];
        index /= p->n[i];
    }
}

/* ProjectedEnergyDensity.EnergyDensityComputation,
 * diagnostics/methods/ProjectedEnergyDensity.java:114-179 */
void orc_projected_energy(const orc_params *p, const double *U, const double *Unext,
                          const double *E, const uint8_t *eval, int dir, double *out)
{
    int nc = p->nc, na = orc_na(nc);
    long V = vol(p);
    int N = p->n[dir];
    double *T_el = out, *T_mag = out + N, *L_el = out + 2 * N, *L_mag = out + 3 * N;
    for (int i = 0; i < 4 * N; i++) out[i] = 0.0;
    double areaFactor = V / ((double)N);
    double uf[3];
    for (int i = 0; i < 3; i++) uf[i] = pow(p->g * p->a[i], -2) / areaFactor;
    for (long x = 0; x < V; x++) {
        if (eval && !eval[x]) continue;
        int pos[3];
        cell_pos(p, x, pos);
        int pi = pos[dir];
        double eTel = 0.0, eLel = 0.0, eTmag = 0.0, eLmag = 0.0;
        for (int j = 0; j < 3; j++) {
            double b0[NA_MAX], b1[NA_MAX];
            double electric = 0.5 * orc_alg_square(nc, E + ((size_t)x * 3 + j) * na) * uf[j];
            orc_get_b(p, U, x, j, b0);
            orc_get_b(p, Unext, x, j, b1);
            double magnetic = 0.25 * (orc_alg_square(nc, b0) + orc_alg_square(nc, b1)) * uf[j];
            if (j == dir) { eLel += electric; eLmag += magnetic; }
            else { eTel += electric; eTmag += magnetic; }
        }
        T_el[pi] += eTel;
        T_mag[pi] += eTmag;
        L_el[pi] += eLel;
        L_mag[pi] += eLmag;
    }
}

/* ProjectedEnergyDensity.PoyntingComputation (diagnostics/methods/ProjectedEnergyDensity.java:182-279),
 * SU(2) only (SU3AlgebraElement.mult(AlgebraElement) throws in the reference).
 * Every cell counts (the computation has no isEvaluatable test).
 * out: 2 rows of N[dir]: Poynting vector averaged, and only time-averaged. */
int orc_projected_poynting(const orc_params *p, const double *U, const double *Unext,
                           const double *E, int dir, double *out)
{
    if (p->nc != 2) return -1;
    const int na = 3, ng = 4;
    long V = vol(p);
    int N = p->n[dir];
    double *avg = out, *tavg = out + N;
    for (int i = 0; i < 2 * N; i++) out[i] = 0.0;
    double areaFactor = V / ((double)N);
    double ufF[3], ufEB[3];
    for (int i = 0; i < 3; i++) {
        ufF[i] = 1.0 / ((p->a[i] * p->a[dir]) * p->g * sqrt(areaFactor));
        ufEB[i] = 1.0 / ((p->g * p->a[i]) * sqrt(areaFactor));
    }
    const int d = dir;
    for (long x = 0; x < V; x++) {
        double lavg = 0.0, ltavg = 0.0;
        for (int i = 0; i < 3; i++) {
            if (i == d) continue;
            double FG[NG_MAX] = {0}, P[NG_MAX];
            for (int t = 0; t < 2; t++) {
                const double *W = t ? Unext : U;
                orc_plaquette(p, W, x, d, i, 1, 1, P);
                for (int c = 0; c < ng; c++) FG[c] += P[c];
                orc_plaquette(p, W, x, i, d, -1, 1, P);
                for (int c = 0; c < ng; c++) FG[c] += P[c];
                orc_plaquette(p, W, x, i, d, 1, -1, P);
                for (int c = 0; c < ng; c++) FG[c] += P[c];
                orc_plaquette(p, W, x, d, i, -1, -1, P);
                for (int c = 0; c < ng; c++) FG[c] += P[c];
            }
            double F[NA_MAX], E1[NA_MAX], E2[NA_MAX], g[NG_MAX], Ev[NA_MAX];
            orc_group_proj(2, FG, F);
            for (int c = 0; c < na; c++) F[c] = F[c] * (ufF[i] / 8.0);
            long sh = orc_shift(p, x, i, -1);
            memcpy(E1, E + ((size_t)x * 3 + i) * na, sizeof(double) * na);
            get_link(p, U, x, i, -1, g);
            orc_alg_act(2, E + ((size_t)sh * 3 + i) * na, g, E2);
            for (int c = 0; c < na; c++) Ev[c] = (E1[c] + E2[c]) * (0.5 * ufEB[i]);
            lavg += Ev[0] * F[0] + Ev[1] * F[1] + Ev[2] * F[2];
        }
        int dir1 = (d + 1) % 3, dir2 = (d + 2) % 3;
        double e1[NA_MAX], e2[NA_MAX], b10[NA_MAX], b11[NA_MAX], b20[NA_MAX], b21[NA_MAX], B1[NA_MAX], B2[NA_MAX];
        for (int c = 0; c < na; c++) {
            e1[c] = E[((size_t)x * 3 + dir1) * na + c] * ufEB[dir1];
            e2[c] = E[((size_t)x * 3 + dir2) * na + c] * ufEB[dir2];
        }
        orc_get_b(p, U, x, dir1, b10);
        orc_get_b(p, Unext, x, dir1, b11);
        orc_get_b(p, U, x, dir2, b20);
        orc_get_b(p, Unext, x, dir2, b21);
        for (int c = 0; c < na; c++) {
            B1[c] = (b10[c] + b11[c]) * (ufEB[dir1] * 0.5);
            B2[c] = (b20[c] + b21[c]) * (ufEB[dir2] * 0.5);
        }
        ltavg = (e1[0] * B2[0] + e1[1] * B2[1] + e1[2] * B2[2]) - (e2[0] * B1[0] + e2[1] * B1[1] + e2[2] * B1[2]);
        int pos[3];
        cell_pos(p, x, pos);
        avg[pos[d]] += lavg;
        tavg[pos[d]] += ltavg;
    }
    return 0;
}

void orc_gauss_field(const orc_params *p, const double *U, const double *E, const double *rho,
                     double *out)
{
    int na = orc_na(p->nc);
    long V = vol(p);
    for (long x = 0; x < V; x++) orc_gauss_constraint(p, U, E, rho, x, out + (size_t)x * na);
}

/* ------------------------------------------------------------------------- */
/* CPIC NGP                                                                   */
/* ------------------------------------------------------------------------- */

/* GridFunctions.nearestGridPoint, physics/util/GridFunctions.java:67-73 ((int) Math.rint) */
void orc_ngp(const orc_params *p, const double *pos, int32_t *c)
{
    for (int i = 0; i < 3; i++) c[i] = (int32_t)rint(pos[i] / p->a[i]);
}

/* Grid.getCellIndex + periodic, physics/grid/Grid.java:757-786 */
static long cell_index(const orc_params *p, const int32_t *c)
{
    long idx = 0;
    for (int i = 0; i < 3; i++) {
        long r = ((long)c[i] % p->n[i] + p->n[i]) % p->n[i];
        idx = i == 0 ? r : idx * p->n[i] + r;
    }
    return idx;
}

/* YangMillsParticle.reassignValues, physics/particles/YangMillsParticle.java:117-125 */
void orc_cpic_reassign(int nc, long np, double *pos0, double *pos1, double *Q0, double *Q1)
{
    int na = orc_na(nc);
    for (long k = 0; k < np; k++) {
        for (int i = 0; i < 3; i++) {
            double t = pos0[k * 3 + i]; pos0[k * 3 + i] = pos1[k * 3 + i]; pos1[k * 3 + i] = t;
        }
        for (int c = 0; c < na; c++) {
            double t = Q0[k * na + c]; Q0[k * na + c] = Q1[k * na + c]; Q1[k * na + c] = t;
        }
    }
}

/* CGCParticleInterpolationNGP.interpolateChargedensity, physics/grid/CGCParticleInterpolationNGP.java:52-68 */
void orc_cpic_charge_density(const orc_params *p, long np, const double *pos0, const double *Q0,
                             double *rho)
{
    int na = orc_na(p->nc);
    for (long k = 0; k < np; k++) {
        int32_t c[3];
        orc_ngp(p, pos0 + k * 3, c);
        long ci = cell_index(p, c);
        for (int m = 0; m < na; m++) rho[ci * na + m] = rho[ci * na + m] + Q0[k * na + m];
    }
}

/* CGCParticleSolver.updatePosition, physics/movement/solver/CGCParticleSolver.java:15-21;
 * AbsorbingParticleBoundaryConditions.applyOnParticle is a no-op (:31-40). */
void orc_cpic_update_positions(const orc_params *p, long np, const double *pos0, double *pos1,
                               const double *vel)
{
    for (long k = 0; k < np; k++)
        for (int i = 0; i < 3; i++) pos1[k * 3 + i] = pos0[k * 3 + i] + vel[k * 3 + i] * p->dt;
}

/* CGCParticleInterpolationNGP.interpolateToParticle, :70-104 */
void orc_cpic_to_particle(const orc_params *p, long np, const double *pos0, const double *pos1,
                          const double *vel, const int32_t *dir, const double *Unext,
                          double *Ulink, uint8_t *flag)
{
    int nc = p->nc, ng = orc_ng(nc);
    for (long k = 0; k < np; k++) {
        int32_t o[3], n[3];
        int d = dir[k];
        orc_ngp(p, pos0 + k * 3, o);
        orc_ngp(p, pos1 + k * 3, n);
        if (o[d] == n[d]) continue;
        long co = cell_index(p, o), cn = cell_index(p, n);
        if (vel[k * 3 + d] > 0)
            memcpy(Ulink + k * ng, link(p, Unext, co, d), sizeof(double) * ng);
        else
            orc_group_adj(nc, link(p, Unext, cn, d), Ulink + k * ng);
        flag[k] = 1;
    }
}

/* CGCParticleSolver.updateCharge, physics/movement/solver/CGCParticleSolver.java:24-36 */
void orc_cpic_update_charges(int nc, long np, double *Q0, double *Q1, const double *Ulink,
                             uint8_t *flag)
{
    int na = orc_na(nc), ng = orc_ng(nc);
    for (long k = 0; k < np; k++) {
        if (flag[k]) {
            double ua[NG_MAX];
            orc_group_adj(nc, Ulink + k * ng, ua);
            orc_alg_act(nc, Q0 + k * na, ua, Q1 + k * na);
            flag[k] = 0;
        } else {
            for (int c = 0; c < na; c++) {
                double t = Q1[k * na + c]; Q1[k * na + c] = Q0[k * na + c]; Q0[k * na + c] = t;
            }
        }
    }
}

/* CGCParticleInterpolationNGP.interpolateToGrid, :15-50 */
void orc_cpic_to_grid(const orc_params *p, long np, const double *pos0, const double *pos1,
                      const double *vel, const int32_t *dir, const double *Q0, const double *Q1,
                      double *J)
{
    int na = orc_na(p->nc);
    double at = p->dt;
    for (long k = 0; k < np; k++) {
        int32_t o[3], n[3];
        int d = dir[k];
        orc_ngp(p, pos0 + k * 3, o);
        orc_ngp(p, pos1 + k * 3, n);
        if (o[d] == n[d]) continue;
        long co = cell_index(p, o), cn = cell_index(p, n);
        if (vel[k * 3 + d] > 0) {
            double f = p->a[d] / at;
            double *Jd = J + ((size_t)co * 3 + d) * na;
            for (int c = 0; c < na; c++) Jd[c] = Jd[c] + Q0[k * na + c] * f;
        } else {
            double f = -p->a[d] / at;
            double *Jd = J + ((size_t)cn * 3 + d) * na;
            for (int c = 0; c < na; c++) Jd[c] = Jd[c] + Q1[k * na + c] * f;
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Seeded synthetic initial conditions                                        */
/* ------------------------------------------------------------------------- */

/* Counter-based generator: splitmix64 finaliser of (seed, counter); two 53-bit
 * uniforms per normal (Box-Muller, cosine branch).  The same integer recipe is
 * used by the GPU initial-condition kernels. */
static inline uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static inline double unif(uint64_t seed, uint64_t ctr)
{
    uint64_t h = mix64(seed ^ mix64(ctr));
    return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
double orc_normal(uint64_t seed, uint64_t ctr)
{
    double u1 = unif(seed, 2 * ctr), u2 = unif(seed, 2 * ctr + 1);
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}
void orc_random_gen(uint64_t seed, uint64_t stream, long count, double sigma, double *out)
{
    uint64_t base = stream << 40;
    for (long k = 0; k < count; k++) out[k] = sigma * orc_normal(seed, base + (uint64_t)k);
}

/* Seeded links U = getLink(A) and fields E (reference layout) for a whole lattice:
 * the loops of OracleGrid.random_links / random_e done in C for large lattices. */
void orc_random_fields(const orc_params *p, uint64_t seed, double sigma_a, double sigma_e,
                       double *U, double *E)
{
    int nc = p->nc, ng = orc_ng(nc), na = orc_na(nc), k = nc == 3 ? 8 : 3;
    long n = vol(p) * 3;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long m = 0; m < n; m++) {
        double ga[8], ge[8], alg[NA_MAX];
        for (int a = 0; a < k; a++) {
            ga[a] = sigma_a * orc_normal(seed, (0ULL << 40) + (uint64_t)(m * k + a));
            ge[a] = sigma_e * orc_normal(seed, (1ULL << 40) + (uint64_t)(m * k + a));
        }
        orc_gen_to_alg(nc, ga, alg);
        orc_alg_getlink(nc, alg, U + m * ng);
        orc_gen_to_alg(nc, ge, E + m * na);
    }
}

/* div E (x) = sum_i c_i [E_i(x) - Ad(U_i(x-i)^dagger) E_i(x-i)], c_i = 1/(a_i g a_i):
 * the E part of Grid.getGaussConstraint (Grid.java:944-968). */
static void op_div(const orc_params *p, const double *U, const double *E, double *out)
{
    int nc = p->nc, na = orc_na(nc);
    long V = vol(p);
    for (long x = 0; x < V; x++) {
        double acc[NA_MAX] = {0}, e[NA_MAX], g[NG_MAX];
        for (int i = 0; i < 3; i++) {
            double ci = 1.0 / (p->a[i] * p->g * p->a[i]);
            long sh = orc_shift(p, x, i, -1);
            orc_group_adj(nc, link(p, U, sh, i), g);
            orc_alg_act(nc, E + ((size_t)sh * 3 + i) * na, g, e);
            for (int c = 0; c < na; c++)
                acc[c] += ci * (E[((size_t)x * 3 + i) * na + c] - e[c]);
        }
        memcpy(out + (size_t)x * na, acc, sizeof(double) * na);
    }
}
/* The adjoint of op_div: (divT l)_i(x) = c_i [l(x) - Ad(U_i(x)) l(x+i)]. */
static void op_divT(const orc_params *p, const double *U, const double *l, double *out)
{
    int nc = p->nc, na = orc_na(nc);
    long V = vol(p);
    for (long x = 0; x < V; x++)
        for (int i = 0; i < 3; i++) {
            double ci = 1.0 / (p->a[i] * p->g * p->a[i]), e[NA_MAX];
            long sh = orc_shift(p, x, i, 1);
            orc_alg_act(nc, l + (size_t)sh * na, link(p, U, x, i), e);
            for (int c = 0; c < na; c++)
                out[((size_t)x * 3 + i) * na + c] = ci * (l[(size_t)x * na + c] - e[c]);
        }
}

static double field_dot(int nc, long n, const double *x, const double *y)
{
    int na = orc_na(nc);
    double s = 0.0;
    for (long k = 0; k < n; k++) s += alg_dot(nc, x + k * na, y + k * na);
    return s;
}

int orc_gauss_project_cg(const orc_params *p, const double *U, double *E, const double *rho,
                         double tol_g2, int maxit, double *final_g2)
{
    int nc = p->nc, na = orc_na(nc);
    long V = vol(p);
    size_t ns = (size_t)V * na, nl = ns * 3;
    double *r = malloc(ns * sizeof(double)), *pp = malloc(ns * sizeof(double));
    double *Ap = malloc(ns * sizeof(double)), *mu = calloc(ns, sizeof(double));
    double *tl = malloc(nl * sizeof(double));
    /* r = rho - div E */
    op_div(p, U, E, r);
    for (size_t k = 0; k < ns; k++) r[k] = rho[k] - r[k];
    memcpy(pp, r, ns * sizeof(double));
    double rr = field_dot(nc, V, r, r);
    int it = 0;
    while (it < maxit && rr / V > tol_g2 * 1e-4) {
        op_divT(p, U, pp, tl);
        op_div(p, U, tl, Ap);
        double pAp = field_dot(nc, V, pp, Ap);
        if (!(pAp > 0)) break;
        double alpha = rr / pAp;
        for (size_t k = 0; k < ns; k++) { mu[k] += alpha * pp[k]; r[k] -= alpha * Ap[k]; }
        double rr2 = field_dot(nc, V, r, r);
        double beta = rr2 / rr;
        rr = rr2;
        for (size_t k = 0; k < ns; k++) pp[k] = r[k] + beta * pp[k];
        it++;
    }
    /* E <- E + divT mu */
    op_divT(p, U, mu, tl);
    for (size_t k = 0; k < nl; k++) E[k] += tl[k];
    double g2 = 0.0;
    for (long x = 0; x < V; x++) {
        double gg[NA_MAX];
        orc_gauss_constraint(p, U, E, rho, x, gg);
        g2 += orc_alg_square(nc, gg);
    }
    if (final_g2) *final_g2 = g2 / V;
    free(r); free(pp); free(Ap); free(mu); free(tl);
    return it;
}

/* GaussConstraintRestoration.computeGaussViolation,
 * diagnostics/methods/GaussConstraintRestoration.java:117-139 */
static double restoration_violation(const orc_params *p, const double *U, const double *Unext,
                                    const double *rho, double *gv)
{
    int nc = p->nc, ng = orc_ng(nc), na = orc_na(nc);
    long V = vol(p);
    double factor = 1.0 / (p->dt * p->a[0]);
    double total = 0.0;
    for (long i = 0; i < V; i++) {
        double C[NG_MAX] = {0}, C1[NG_MAX], C2[NG_MAX], t[NG_MAX], pr[NA_MAX];
        for (int j = 0; j < 3; j++) {
            long k = orc_shift(p, i, j, -1);
            orc_group_adj(nc, link(p, U, i, j), t);
            orc_group_mult(nc, link(p, Unext, i, j), t, C1);
            orc_group_adj(nc, link(p, U, k, j), t);
            orc_group_mult(nc, t, link(p, Unext, k, j), C2);
            for (int c = 0; c < ng; c++) C[c] = C[c] + (C1[c] - C2[c]);
        }
        for (int c = 0; c < ng; c++) gv[(size_t)i * ng + c] = C[c] * factor;
        orc_group_proj(nc, gv + (size_t)i * ng, pr);
        for (int c = 0; c < na; c++) pr[c] = pr[c] - rho[(size_t)i * na + c];
        total += orc_alg_square(nc, pr);
    }
    return total / V;
}

/* GaussConstraintRestoration.applyCorrection, :146-163 */
static void restoration_correct(const orc_params *p, const double *U, double *Unext, double *E,
                                const double *gv, double gamma)
{
    int nc = p->nc, ng = orc_ng(nc), na = orc_na(nc);
    long V = vol(p);
    double factor2 = -0.5 * p->a[0] * gamma;
    for (long i = 0; i < V; i++)
        for (int j = 0; j < 3; j++) {
            long k = orc_shift(p, i, j, 1);
            double t[NG_MAX], C1[NG_MAX], ua[NG_MAX], pr[NA_MAX];
            orc_group_mult(nc, link(p, U, i, j), gv + (size_t)k * ng, t);
            orc_group_adj(nc, link(p, U, i, j), ua);
            orc_group_mult(nc, t, ua, C1);
            for (int c = 0; c < ng; c++) C1[c] = C1[c] - gv[(size_t)i * ng + c];
            orc_group_proj(nc, C1, pr);
            double *Ej = E + ((size_t)i * 3 + j) * na;
            for (int c = 0; c < na; c++) Ej[c] = Ej[c] + pr[c] * factor2;
        }
    orc_update_links(p, U, E, Unext, NULL);
}

/* GaussConstraintRestoration.iterateRestorationAlgorithm, :78-110 */
int orc_gauss_restoration(const orc_params *p, double *U, double *Unext, double *E,
                          const double *rho, double gamma, int maxit, double absval,
                          double *final_violation)
{
    int nc = p->nc, ng = orc_ng(nc), na = orc_na(nc);
    long V = vol(p);
    size_t nlg = (size_t)V * 3 * ng, nla = (size_t)V * 3 * na;
    double *gv = malloc((size_t)V * ng * sizeof(double));
    double *bE = malloc(nla * sizeof(double)), *bUn = malloc(nlg * sizeof(double));
    double total = restoration_violation(p, U, Unext, rho, gv);
    double old = total;
    int i;
    for (i = 0; i < maxit; i++) {
        if (total < absval) break;
        memcpy(bE, E, nla * sizeof(double));
        memcpy(bUn, Unext, nlg * sizeof(double));
        restoration_correct(p, U, Unext, E, gv, gamma);
        total = restoration_violation(p, U, Unext, rho, gv);
        if (old - total < 0) {
            memcpy(E, bE, nla * sizeof(double));
            memcpy(Unext, bUn, nlg * sizeof(double));
            total = old;
            break;
        }
        old = total;
    }
    if (final_violation) *final_violation = total;
    free(gv); free(bE); free(bUn);
    return i;
}

/* ------------------------------------------------------------------------- */
/* CGC initial conditions (physics/initial/CGC)                               */
/* ------------------------------------------------------------------------- */

/* java.util.Random as the Java SE API documentation specifies it: 48-bit LCG
 * (multiplier 0x5DEECE66D, addend 0xB), nextDouble from 26 + 27 bits,
 * nextGaussian by the polar method with one cached deviate. */
typedef struct { uint64_t seed; int have; double next; } jrand;

/* StrictMath.log: the fdlibm algorithm (e_log.c, the method Java specifies for
 * StrictMath): x = 2^k (1+f) with sqrt(2)/2 < 1+f < sqrt(2), s = f/(2+f),
 * log(1+f) = f - s (f - R(s^2)) with a degree-14 even minimax polynomial R,
 * and k ln2 split into a high and a low part.  Finite x > 0 only.
 * The constants and steps are fdlibm's e_log.c, which carries this notice:
 * ====================================================
 * Copyright (C) 1993 by Sun Microsystems, Inc. All rights reserved.
 *
 * Developed at SunSoft, a Sun Microsystems, Inc. business.
 * Permission to use, copy, modify, and distribute this
 * software is freely granted, provided that this notice
 * is preserved.
 * ==================================================== */
static double strict_log(double x)
{
    static const double ln2_hi = 6.93147180369123816490e-01, ln2_lo = 1.90821492927058770002e-10,
                        two54 = 1.80143985094819840000e+16,
                        Lg1 = 6.666666666666735130e-01, Lg2 = 3.999999999940941908e-01,
                        Lg3 = 2.857142874366239149e-01, Lg4 = 2.222219843214978396e-01,
                        Lg5 = 1.818357216161805012e-01, Lg6 = 1.531383769920937332e-01,
                        Lg7 = 1.479819860511658591e-01;
    uint64_t bits;
    memcpy(&bits, &x, 8);
    int32_t hx = (int32_t)(bits >> 32);
    uint32_t lx = (uint32_t)bits;
    int32_t k = 0;
    if (hx < 0x00100000) { /* subnormal */
        (void)lx;
        k -= 54;
        x *= two54;
        memcpy(&bits, &x, 8);
        hx = (int32_t)(bits >> 32);
    }
    k += (hx >> 20) - 1023;
    hx &= 0x000fffff;
    int32_t i = (hx + 0x95f64) & 0x100000;
    bits = ((uint64_t)(uint32_t)(hx | (i ^ 0x3ff00000)) << 32) | (bits & 0xffffffffULL);
    memcpy(&x, &bits, 8);
    k += (i >> 20);
    double f = x - 1.0, dk, R;
    if ((0x000fffff & (2 + hx)) < 3) {
        if (f == 0.0) {
            if (k == 0) return 0.0;
            dk = (double)k;
            return dk * ln2_hi + dk * ln2_lo;
        }
        R = f * f * (0.5 - 0.33333333333333333 * f);
        if (k == 0) return f - R;
        dk = (double)k;
        return dk * ln2_hi - ((R - dk * ln2_lo) - f);
    }
    double s = f / (2.0 + f);
    dk = (double)k;
    double z = s * s;
    i = hx - 0x6147a;
    double w = z * z;
    int32_t j = 0x6b851 - hx;
    double t1 = w * (Lg2 + w * (Lg4 + w * Lg6));
    double t2 = z * (Lg1 + w * (Lg3 + w * (Lg5 + w * Lg7)));
    i |= j;
    R = t2 + t1;
    if (i > 0) {
        double hfsq = 0.5 * f * f;
        if (k == 0) return f - (hfsq - s * (hfsq + R));
        return dk * ln2_hi - ((hfsq - (s * (hfsq + R) + dk * ln2_lo)) - f);
    }
    if (k == 0) return f - s * (f - R);
    return dk * ln2_hi - ((s * (f - R) - dk * ln2_lo) - f);
}

static void jrand_seed(jrand *r, int64_t s)
{
    r->seed = ((uint64_t)s ^ 0x5DEECE66DULL) & ((1ULL << 48) - 1);
    r->have = 0;
}
static int32_t jrand_next(jrand *r, int bits)
{
    r->seed = (r->seed * 0x5DEECE66DULL + 0xBULL) & ((1ULL << 48) - 1);
    return (int32_t)(int64_t)(r->seed >> (48 - bits));
}
static double jrand_double(jrand *r)
{
    int64_t hi = (int64_t)jrand_next(r, 26), lo = (int64_t)jrand_next(r, 27);
    return (double)((hi << 27) + lo) * 0x1.0p-53;
}
static double jrand_gaussian(jrand *r)
{
    if (r->have) { r->have = 0; return r->next; }
    double v1, v2, s;
    do {
        v1 = 2 * jrand_double(r) - 1;
        v2 = 2 * jrand_double(r) - 1;
        s = v1 * v1 + v2 * v2;
    } while (s >= 1 || s == 0);
    double m = sqrt(-2 * strict_log(s) / s);
    r->next = v2 * m;
    r->have = 1;
    return v1 * m;
}

double orc_strict_log(double x) { return strict_log(x); }

void orc_java_random(int64_t seed, int kind, long count, double *out)
{
    jrand r;
    jrand_seed(&r, seed);
    for (long i = 0; i < count; i++) {
        if (kind == 0) out[i] = jrand_gaussian(&r);
        else if (kind == 1) out[i] = jrand_double(&r);
        else out[i] = (double)jrand_next(&r, 32);
    }
}

/* MVModel.initialize, random part (physics/initial/CGC/MVModel.java:113-132):
 * one java.util.Random stream over all components in site order, scaled by
 * g mu / sqrt(aL aT^2) and the square root of the longitudinal Gaussian profile
 * (org.apache.commons.math3.analysis.function.Gaussian 3.5: norm * exp(-d*d*i2s2),
 * norm = 1/(sigma sqrt(2 pi)), i2s2 = 0.5 (1/sigma)^2).  out: [ncomp][V]. */
void orc_mv_charges(const orc_params *p, int direction, double location, double width, double mu,
                    int64_t seed, double *out)
{
    long V = vol(p);
    int ncomp = p->nc > 1 ? p->nc * p->nc - 1 : 1;
    double aL = p->a[direction], aT = p->a[(direction + 1) % 3];
    double is = 1.0 / width, i2s2 = 0.5 * is * is;
    double norm = 1.0 / (width * sqrt(2.0 * M_PI));
    double colorWidth = mu * p->g / sqrt(aL * aT * aT);
    jrand r;
    jrand_seed(&r, seed);
    for (int j = 0; j < ncomp; j++)
        for (long i = 0; i < V; i++) {
            int pos[3];
            cell_pos(p, i, pos);
            double longPos = pos[direction] * p->a[direction];
            double d = longPos - location;
            double profile = sqrt(norm * exp(-d * d * i2s2));
            out[(size_t)j * V + i] = jrand_gaussian(&r) * colorWidth * profile;
        }
}

/* LightConePoissonSolverImproved.solve after the 2D Poisson solves
 * (physics/initial/CGC/LightConePoissonSolverImproved.java:92-220).
 * phi: [ncomp][V] generator components (phi0[i].set(c, .)); U, Unext, E are
 * updated in place (reference layout); gauss: [V][na], the Gauss violation of
 * the nucleus alone (grid copy with its own links, rho of the grid = 0). */
void orc_cgc_solve(const orc_params *p, int direction, int orientation, const double *phi,
                   double *U, double *Unext, double *E, const uint8_t *active, double *gauss, double *vt)
{
    int nc = p->nc, ng = orc_ng(nc), na = orc_na(nc);
    int ncomp = nc > 1 ? nc * nc - 1 : 1;
    long V = vol(p);
    int nL = p->n[direction];
    long ntr = V / nL;
    double aL = p->a[direction];
    double *Vw = malloc((size_t)V * ng * sizeof(double));
    double *phiA = malloc((size_t)V * na * sizeof(double));
    double *Uc = malloc((size_t)V * 3 * ng * sizeof(double));
    double *Unc = malloc((size_t)V * 3 * ng * sizeof(double));
    double *Ec = malloc((size_t)V * 3 * na * sizeof(double));
    double zero[NA_MAX] = {0};
    for (long i = 0; i < V; i++) {
        double gen[8];
        for (int c = 0; c < ncomp; c++) gen[c] = phi[(size_t)c * V + i];
        orc_gen_to_alg(nc, gen, phiA + (size_t)i * na);
        group_identity(nc, Vw + (size_t)i * ng);
    }
    /* grid copy: every cell copied from the grid (Grid(Grid), Cell.copyFrom) */
    memcpy(Uc, U, (size_t)V * 3 * ng * sizeof(double));
    memcpy(Unc, Unext, (size_t)V * 3 * ng * sizeof(double));
    memcpy(Ec, E, (size_t)V * 3 * na * sizeof(double));
    /* Wilson lines (:100-124); the transverse index runs over the other two
     * dimensions in order, so for direction 0 it is the site's offset within the sheet */
    double gaugeFactor = -p->g * aL;
    for (int k = 0; k < nL; k++) {
        int z = orientation < 0 ? k : nL - k - 1;
        for (long t = 0; t < ntr; t++) {
            /* transverse cell position -> grid position with the longitudinal slot z */
            int pos[3], tp[2], dims_t[2], m = 0;
            for (int d = 0; d < 3; d++) if (d != direction) dims_t[m++] = p->n[d];
            tp[0] = (int)(t / dims_t[1]);
            tp[1] = (int)(t % dims_t[1]);
            m = 0;
            for (int d = 0; d < 3; d++) pos[d] = d == direction ? z : tp[m++];
            long index = ((long)pos[0] * p->n[1] + pos[1]) * p->n[2] + pos[2];
            long indexL = orc_shift(p, index, direction, orientation);
            double a[NA_MAX], W[NG_MAX], t2[NG_MAX];
            const double *src = phiA + (size_t)(orientation == -1 ? indexL : index) * na;
            for (int c = 0; c < na; c++) a[c] = src[c] * gaugeFactor;
            orc_alg_getlink(nc, a, W);
            orc_group_mult(nc, Vw + (size_t)indexL * ng, W, t2);
            memcpy(Vw + (size_t)index * ng, t2, sizeof(double) * ng);
        }
    }
    /* VT: V at the longitudinal boundary behind the nucleus (:125-136), per transverse cell */
    if (vt) {
        int zb = orientation > 0 ? 0 : nL - 1;
        for (long t = 0; t < ntr; t++) {
            int pos[3], tp[2], dims_t[2], m = 0;
            for (int d = 0; d < 3; d++) if (d != direction) dims_t[m++] = p->n[d];
            tp[0] = (int)(t / dims_t[1]);
            tp[1] = (int)(t % dims_t[1]);
            m = 0;
            for (int d = 0; d < 3; d++) pos[d] = d == direction ? zb : tp[m++];
            long index = ((long)pos[0] * p->n[1] + pos[1]) * p->n[2] + pos[2];
            memcpy(vt + (size_t)t * ng, Vw + (size_t)index * ng, sizeof(double) * ng);
        }
    }
    /* links at t = -dt/2 (:143-157) */
    for (long i = 0; i < V; i++)
        for (int d = 0; d < 3; d++) {
            if (d == direction) continue;
            long is = orc_shift(p, i, d, 1);
            double adj[NG_MAX], t1[NG_MAX];
            orc_group_adj(nc, Vw + (size_t)is * ng, adj);
            orc_group_mult(nc, Vw + (size_t)i * ng, U + ((size_t)i * 3 + d) * ng, t1);
            orc_group_mult(nc, t1, adj, U + ((size_t)i * 3 + d) * ng);
            orc_group_mult(nc, Vw + (size_t)i * ng, adj, Uc + ((size_t)i * 3 + d) * ng);
        }
    /* improved V at t = dt/2 (:160-185), M = 20 path-ordered factors */
    const int M = 20;
    for (long i = 0; i < V; i++) {
        double IW[NG_MAX], W[NG_MAX], t1[NG_MAX], ph[NA_MAX];
        group_identity(nc, IW);
        long is = orc_shift(p, i, direction, -1);
        for (int m = 0; m < M; m++) {
            double z = (m + 0.5) / ((double)2 * M);
            double FL = orientation == 1 ? +z + 0.5 : -z + 0.5;
            double FR = orientation == 1 ? -z + 0.5 : +z + 0.5;
            for (int c = 0; c < na; c++)
                ph[c] = phiA[(size_t)is * na + c] * FL + phiA[(size_t)i * na + c] * FR;
            double f = -p->g * p->dt / ((double)M);
            for (int c = 0; c < na; c++) ph[c] = ph[c] * f;
            orc_alg_getlink(nc, ph, W);
            orc_group_mult(nc, IW, W, t1);
            memcpy(IW, t1, sizeof(double) * ng);
        }
        orc_group_mult(nc, Vw + (size_t)i * ng, IW, t1);
        memcpy(Vw + (size_t)i * ng, t1, sizeof(double) * ng);
    }
    /* links at t = dt/2 (:188-202) */
    for (long i = 0; i < V; i++)
        for (int d = 0; d < 3; d++) {
            if (d == direction) continue;
            long is = orc_shift(p, i, d, 1);
            double adj[NG_MAX], t1[NG_MAX];
            orc_group_adj(nc, Vw + (size_t)is * ng, adj);
            orc_group_mult(nc, Vw + (size_t)i * ng, Unext + ((size_t)i * 3 + d) * ng, t1);
            orc_group_mult(nc, t1, adj, Unext + ((size_t)i * 3 + d) * ng);
            orc_group_mult(nc, Vw + (size_t)i * ng, adj, Unc + ((size_t)i * 3 + d) * ng);
        }
    /* E at t = 0 from the temporal plaquette (:205-210, Grid.getEFromLinks) */
    for (long i = 0; i < V; i++)
        for (int j = 0; j < 3; j++) {
            double adj[NG_MAX], pl[NG_MAX], v[NA_MAX];
            orc_group_adj(nc, U + ((size_t)i * 3 + j) * ng, adj);
            orc_group_mult(nc, Unext + ((size_t)i * 3 + j) * ng, adj, pl);
            orc_group_proj(nc, pl, v);
            for (int c = 0; c < na; c++) E[((size_t)i * 3 + j) * na + c] = v[c] * (-1.0 / p->dt);
            orc_group_adj(nc, Uc + ((size_t)i * 3 + j) * ng, adj);
            orc_group_mult(nc, Unc + ((size_t)i * 3 + j) * ng, adj, pl);
            orc_group_proj(nc, pl, v);
            for (int c = 0; c < na; c++) Ec[((size_t)i * 3 + j) * na + c] = v[c] * (-1.0 / p->dt);
        }
    /* Gauss violation of the copy (:213-220) */
    double *rho0 = calloc((size_t)V * na, sizeof(double));
    for (long i = 0; i < V; i++) {
        if (!active || active[i]) orc_gauss_constraint(p, Uc, Ec, rho0, i, gauss + (size_t)i * na);
        else memcpy(gauss + (size_t)i * na, zero, sizeof(double) * na);
    }
    free(rho0); free(Vw); free(phiA); free(Uc); free(Unc); free(Ec);
}

static long ring(long i, long n) { return (i % n + n) % n; }

/* LightConeNGPParticleCreator.initializeParticles (physics/initial/CGC/
 * LightConeNGPParticleCreator.java:110-235) for beam direction 0.
 * Returns the number of particles; the arrays are filled when cap >= that
 * number: pos0, pos1, vel [np][3], Q [np][na] (Q0 = Q1). */
long orc_cgc_particles(const orc_params *p, const double *gauss, int orientation, long cap,
                       double *pos0, double *pos1, double *vel, double *Q)
{
    int nc = p->nc, na = orc_na(nc);
    const int direction = 0;
    long V = vol(p);
    int lnum = p->n[0];
    long ntr = V / lnum;
    int ppc = (int)lround(p->a[direction] / p->dt);
    if (ppc < 1) return -1;
    double *maxCharges = malloc(sizeof(double) * lnum), globalMax = 0.0;
    for (int z = 0; z < lnum; z++) {
        double mx = 0.0;
        for (long j = 0; j < ntr; j++) {
            double charge = sqrt(orc_alg_square(nc, gauss + (size_t)(z * ntr + j) * na));
            if (mx < charge) mx = charge;
        }
        maxCharges[z] = mx;
        if (globalMax < mx) globalMax = mx;
    }
    double cutoff = globalMax * 10E-10;
    int zStart = 0, zEnd = lnum - 1;
    for (int z = 0; z < lnum; z++) if (maxCharges[z] > cutoff) { zStart = z; break; }
    for (int z = zEnd - 1; z >= 0; z--) if (maxCharges[z] > cutoff) { zEnd = z; break; }
    free(maxCharges);
    long np = (long)(zEnd - zStart + 1) * ntr * ppc;
    if (cap < np) return np;
    long k = 0;
    for (int z = zStart; z <= zEnd; z++)
        for (long i = 0; i < ntr; i++) {
            int gp[3] = {z, (int)(i / p->n[2]), (int)(i % p->n[2])};
            for (int j = 0; j < ppc; j++, k++) {
                double x = (1.0 * j - ppc / 2) / (ppc);
                double dz = x * p->a[direction];
                for (int d = 0; d < 3; d++) {
                    double fix = 10E-12 * p->a[d];
                    pos0[k * 3 + d] = gp[d] * p->a[d] + fix;
                    pos1[k * 3 + d] = gp[d] * p->a[d] + fix;
                    if (d == direction) {
                        pos0[k * 3 + d] += 0.0 * orientation + dz;
                        pos1[k * 3 + d] += (0.0 + p->dt) * orientation + dz;
                    }
                    vel[k * 3 + d] = d == direction ? 1.0 * orientation : 0.0;
                }
                int32_t c[3];
                orc_ngp(p, pos0 + k * 3, c);
                const double *gsrc = gauss + (size_t)cell_index(p, c) * na;
                for (int a = 0; a < na; a++) Q[k * na + a] = gsrc[a] * (1.0 / ppc);
            }
        }
    /* charge refinement per transverse column (:211-227, refine2 :237-262,
     * refine4 :265-296); the column's list runs over z, then over j */
    long n = (long)(zEnd - zStart + 1) * ppc;
    for (long t = 0; t < ntr; t++) {
#define PIDX(ii) ((((ring((ii), n)) / ppc) * ntr + t) * ppc + (ring((ii), n)) % ppc)
        for (int it = 0; it < 100; it++)
            for (long i = 0; i < n; i++) {
                long jm = i % ppc;
                if (!(jm >= 0 && jm < ppc - 1)) continue;
                double *Q0 = Q + PIDX(i - 1) * na, *Q1 = Q + PIDX(i) * na, *Q2 = Q + PIDX(i + 1) * na,
                       *Q3 = Q + PIDX(i + 2) * na;
                for (int a = 0; a < na; a++) {
                    double DQ = Q0[a] * -1;
                    DQ = DQ + Q1[a] * 3;
                    DQ = DQ + Q2[a] * -3;
                    DQ = DQ + Q3[a] * 1;
                    DQ = DQ * (1.0 / 4.0);
                    Q1[a] = Q1[a] + DQ * -1.0;
                    Q2[a] = Q2[a] + DQ * 1.0;
                }
            }
        for (int it = 0; it < 100; it++)
            for (long i = 0; i < n; i++) {
                long jm = i % ppc;
                if (!(jm >= 0 && jm < ppc - 1)) continue;
                double *Q0 = Q + PIDX(i - 2) * na, *Q1 = Q + PIDX(i - 1) * na, *Q2 = Q + PIDX(i) * na,
                       *Q3 = Q + PIDX(i + 1) * na, *Q4 = Q + PIDX(i + 2) * na, *Q5 = Q + PIDX(i + 3) * na;
                for (int a = 0; a < na; a++) {
                    double DQ = Q0[a] * 1;
                    DQ = DQ + Q1[a] * -5;
                    DQ = DQ + Q2[a] * 10;
                    DQ = DQ + Q3[a] * -10;
                    DQ = DQ + Q4[a] * 5;
                    DQ = DQ + Q5[a] * -1;
                    DQ = DQ * (1.0 / 12.0);
                    Q2[a] = Q2[a] + DQ * -1.0;
                    Q3[a] = Q3[a] + DQ * 1.0;
                }
            }
#undef PIDX
    }
    return np;
}

/* ------------------------------------------------------------------------- */
/* Super particles (physics/particles/CGCSuperParticle.java,                  */
/* physics/grid/CGCSuperParticleInterpolationNGP.java,                        */
/* physics/initial/CGC/LightConeNGPSuperParticleCreator.java)                 */
/* ------------------------------------------------------------------------- */

/* LightConeNGPSuperParticleCreator.initializeParticles (:102-241) for the
 * beam along direction 0.  The charges of super particle k (k < ppc) over the
 * whole particle block, index i = global cell index - base, are written to
 * Q[k][i][na]; the block is [base, base + n) with base = zStart * ntr and
 * n = (zEnd - zStart) * ntr.  The subdivision of the block into
 * numberOfThreads pieces only splits these arrays (orc_super_cin/jin take it
 * as a parameter).  Returns n (Q filled when Q != NULL); *base_out = base. */
long orc_super_create(const orc_params *p, const double *gauss, long *base_out, double *Q)
{
    int nc = p->nc, na = orc_na(nc);
    long V = vol(p);
    int lnum = p->n[0];
    long ntr = V / lnum;
    int ppc = (int)lround(p->a[0] / p->dt);
    if (ppc < 1) return -1;
    double *maxCharges = malloc(sizeof(double) * lnum), globalMax = 0.0;
    for (int z = 0; z < lnum; z++) {
        double mx = 0.0;
        for (long j = 0; j < ntr; j++) {
            double charge = sqrt(orc_alg_square(nc, gauss + (size_t)(z * ntr + j) * na));
            if (mx < charge) mx = charge;
        }
        maxCharges[z] = mx;
        if (globalMax < mx) globalMax = mx;
    }
    double cutoff = globalMax * 10E-10;
    int zStart = 0, zEnd = lnum - 1;
    for (int z = 0; z < lnum; z++) if (maxCharges[z] > cutoff) { zStart = z; break; }
    for (int z = zEnd - 1; z >= 0; z--) if (maxCharges[z] > cutoff) { zEnd = z; break; }
    free(maxCharges);
    long blockWidth = zEnd - zStart, n = blockWidth * ntr;
    long base = (long)zStart * ntr;
    if (base_out) *base_out = base;
    if (!Q) return n;
    for (long i = 0; i < n; i++) {
        long index = base + i;
        for (int k = 0; k < ppc; k++) {
            long ngp = (k < ppc / 2) ? index : orc_shift(p, index, 0, 1);
            for (int a = 0; a < na; a++)
                Q[((size_t)k * n + i) * na + a] = gauss[(size_t)ngp * na + a] * (1.0 / ppc);
        }
    }
    /* refinement over each transverse column's longitudinal list
     * (:200-240): entry (zrel * ppc + k) is charge i = zrel * ntr + t of super particle k */
    long len = blockWidth * ppc;
    for (long t = 0; t < ntr && len > 0; t++) {
#define SQ(ii) (Q + ((size_t)(ring((ii), len) % ppc) * n + (ring((ii), len) / ppc) * ntr + t) * na)
        for (int it = 0; it < 100; it++)
            for (long i = 0; i < len; i++) {
                long jm = (i + ppc / 2) % ppc;
                if (!(jm >= 0 && jm < ppc - 1)) continue;
                double *Q0 = SQ(i - 1), *Q1 = SQ(i), *Q2 = SQ(i + 1), *Q3 = SQ(i + 2);
                for (int a = 0; a < na; a++) {
                    double DQ = Q0[a] * -1;
                    DQ = DQ + Q1[a] * 3;
                    DQ = DQ + Q2[a] * -3;
                    DQ = DQ + Q3[a] * 1;
                    DQ = DQ * (1.0 / 4.0);
                    Q1[a] = Q1[a] + DQ * -1.0;
                    Q2[a] = Q2[a] + DQ * 1.0;
                }
            }
        for (int it = 0; it < 100; it++)
            for (long i = 0; i < len; i++) {
                long jm = (i + ppc / 2) % ppc;
                if (!(jm >= 0 && jm < ppc - 1)) continue;
                double *Q0 = SQ(i - 2), *Q1 = SQ(i - 1), *Q2 = SQ(i), *Q3 = SQ(i + 1), *Q4 = SQ(i + 2),
                       *Q5 = SQ(i + 3);
                for (int a = 0; a < na; a++) {
                    double DQ = Q0[a] * 1;
                    DQ = DQ + Q1[a] * -5;
                    DQ = DQ + Q2[a] * 10;
                    DQ = DQ + Q3[a] * -10;
                    DQ = DQ + Q4[a] * 5;
                    DQ = DQ + Q5[a] * -1;
                    DQ = DQ * (1.0 / 12.0);
                    Q2[a] = Q2[a] + DQ * -1.0;
                    Q3[a] = Q3[a] + DQ * 1.0;
                }
            }
#undef SQ
    }
    return n;
}

/* One super particle as the reference holds it. */
typedef struct {
    int orientation, numberOfParticles, particlesPerPlane, subLatticeShift, particlePerCell;
    long indexOffset;
    double *Q; /* [numberOfParticles][na] */
} super_particle;

/* CGCSuperParticle.getCurrentOffset / getCurrentNGPOffset / needsUpdate (:71-105) */
static long sp_offset(const super_particle *P, long t)
{
    if (P->orientation > 0)
        return P->indexOffset + ((t + P->subLatticeShift) / P->particlePerCell) * P->particlesPerPlane;
    long shift = (long)floor((-t + P->subLatticeShift) / (1.0 * P->particlePerCell)) * P->particlesPerPlane;
    return P->indexOffset + shift;
}
static long sp_ngp_offset(const super_particle *P, long t)
{
    long cur = sp_offset(P, t);
    int ppc = P->particlePerCell;
    if (P->orientation > 0)
        return cur + ((((t + P->subLatticeShift) % ppc) < ppc / 2) ? 0 : P->particlesPerPlane);
    return cur + ((((t - P->subLatticeShift + ppc + ppc / 2 - 1) % ppc) < ppc / 2) ? 0 : P->particlesPerPlane);
}
static int sp_needs_update(const super_particle *P, long t)
{
    int ppc = P->particlePerCell;
    if (P->orientation > 0) return 0 == (t + P->subLatticeShift + ppc / 2 + 1) % ppc;
    return 0 == (t - P->subLatticeShift + ppc / 2) % ppc;
}

/* The super particles of one group (one nucleus) in the reference's list
 * order for numberOfThreads = nthreads (:153-195): subdivision j of the block,
 * then k = 0 .. ppc-1.  Returns the count written to out (<= cap). */
static int sp_list(const orc_params *p, int orientation, long n, long base, double *Q, int nthreads,
                   super_particle *out, int cap)
{
    int na = orc_na(p->nc);
    long ntr = vol(p) / p->n[0];
    int ppc = (int)lround(p->a[0] / p->dt);
    long blockWidth = n / ntr;
    if (blockWidth <= 0) return 0;
    long nsub = nthreads < blockWidth ? nthreads : blockWidth;
    long ws = blockWidth / nsub, wl = blockWidth / nsub + 1;
    long ps = ws * ntr, pl = wl * ntr;
    long nl = blockWidth - nsub * ws;
    long off = 0;
    int m = 0;
    for (long j = 0; j < nsub; j++) {
        long cnt = j < nl ? pl : ps;
        for (int k = 0; k < ppc && m < cap; k++, m++) {
            super_particle *P = out + m;
            P->orientation = orientation;
            P->numberOfParticles = (int)cnt;
            P->indexOffset = base + off;
            P->particlesPerPlane = (int)ntr;
            P->subLatticeShift = k;
            P->particlePerCell = ppc;
            P->Q = Q + ((size_t)k * n + off) * na;
        }
        off += cnt;
    }
    return m;
}

/* CGCSuperParticleInterpolationNGP.interpolateChargedensity (:75-93) over all
 * groups in list order.  Groups: orient[g], n[g], base[g], Q[g] ([ppc][n][na]). */
void orc_super_cin(const orc_params *p, int ngroups, const int *orient, const long *n, const long *base,
                   double *const *Q, int nthreads, long t, double *rho)
{
    int na = orc_na(p->nc);
    long V = vol(p);
    super_particle list[4096];
    for (int g = 0; g < ngroups; g++) {
        int m = sp_list(p, orient[g], n[g], base[g], Q[g], nthreads, list, 4096);
        for (int q = 0; q < m; q++) {
            const super_particle *P = list + q;
            long indexOffset = sp_ngp_offset(P, t);
            long imin = (indexOffset < 0) ? -indexOffset : 0;
            long hi = indexOffset + P->numberOfParticles < V ? indexOffset + P->numberOfParticles : V;
            long imax = hi - indexOffset > 0 ? hi - indexOffset : 0;
            long ireg = imax - imin;
            for (long i = 0; i < ireg; i++) {
                long j = i + imin, index = indexOffset + j;
                for (int a = 0; a < na; a++)
                    rho[(size_t)index * na + a] = rho[(size_t)index * na + a] + P->Q[(size_t)j * na + a];
            }
        }
    }
}

/* CGCSuperParticleInterpolationNGP.interpolateToGrid (:19-73): for the super
 * particles that cross an NGP boundary in the next step, the current along
 * direction 0 and the parallel transport of their charges by Unext. */
void orc_super_jin(const orc_params *p, int ngroups, const int *orient, const long *n, const long *base,
                   double *const *Q, int nthreads, long t, const double *Unext, double *J)
{
    int nc = p->nc, na = orc_na(nc), ng = orc_ng(nc);
    long V = vol(p);
    double at = p->dt, as = p->a[0];
    super_particle list[4096];
    for (int g = 0; g < ngroups; g++) {
        int m = sp_list(p, orient[g], n[g], base[g], Q[g], nthreads, list, 4096);
        for (int q = 0; q < m; q++) {
            const super_particle *P = list + q;
            if (!sp_needs_update(P, t)) continue;
            long indexOffset = sp_offset(P, t);
            long quickfix = P->particlePerCell == 1 ? P->particlesPerPlane : 0;
            long imin = (indexOffset < 0) ? -indexOffset : 0;
            long hi = indexOffset + P->numberOfParticles < V - quickfix ? indexOffset + P->numberOfParticles
                                                                        : V - quickfix;
            long imax = hi - indexOffset > 0 ? hi - indexOffset : 0;
            long ireg = imax - imin;
            for (long i = 0; i < ireg; i++) {
                long j = i + imin, index = indexOffset + j;
                double *Qj = P->Q + (size_t)j * na, tmp[NA_MAX], g2[NG_MAX];
                const double *Ul = Unext + ((size_t)index * 3 + 0) * ng;
                if (P->orientation > 0) {
                    double *Jc = J + ((size_t)(index + quickfix) * 3 + 0) * na;
                    for (int a = 0; a < na; a++) Jc[a] = Jc[a] + Qj[a] * (as / at);
                    orc_group_adj(nc, Ul, g2);
                    orc_alg_act(nc, Qj, g2, tmp);
                    memcpy(Qj, tmp, sizeof(double) * na);
                } else {
                    orc_alg_act(nc, Qj, Ul, tmp);
                    memcpy(Qj, tmp, sizeof(double) * na);
                    double *Jc = J + ((size_t)index * 3 + 0) * na;
                    for (int a = 0; a < na; a++) Jc[a] = Jc[a] + Qj[a] * (-as / at);
                }
            }
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Coulomb gauge and occupation numbers, SU(2) (physics/gauge/CoulombGauge.java, */
/* physics/gauge/GaugeTransformation.java,                                    */
/* diagnostics/methods/OccupationNumbersInTime.java)                          */
/* ------------------------------------------------------------------------- */

/* SU2GroupElement.getAlgebraElement (math/SU2GroupElement.java:234-252) */
static void su2_log(const double *u, double *v)
{
    double norm = u[1] * u[1] + u[2] * u[2] + u[3] * u[3];
    norm = sqrt(norm);
    if (norm < 1.E-15) {
        v[0] = 2 * u[1]; v[1] = 2 * u[2]; v[2] = 2 * u[3];
        return;
    }
    v[0] = 2.0 * asin(norm) / norm * u[1];
    v[1] = 2.0 * asin(norm) / norm * u[2];
    v[2] = 2.0 * asin(norm) / norm * u[3];
}

/* SU2AlgebraElement.getLink in the reference's own form (math/SU2AlgebraElement.java:140-152) */
static void su2_link_ref(const double *v, double *u)
{
    double sum = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    double mod = sqrt(sum) / 2;
    double sinfakt = mod < 1.E-20 ? 0.0 : 0.5 / mod * sin(mod);
    u[0] = cos(mod); u[1] = v[0] * sinfakt; u[2] = v[1] * sinfakt; u[3] = v[2] * sinfakt;
}

/* CoulombGauge.CalculateDivergence (:148-166) for every colour: div[c][x] =
 * sum_dir A_c(U_dir(x)) - A_c(U_dir(x - dir)); returns the sum of squares in the
 * reference's order (colour by colour, cells in sequence). */
/* generator components of getAlgebraElement (SU(2): 2 asin|e| e_a/|e|; SU(3): su3_log) */
static int link_log_gen(int nc, const double *u, double *g)
{
    if (nc == 2) { su2_log(u, g); return 3; }
    orc_su3_log_gen(u, g);
    return 8;
}

/* CoulombGauge.CalculateDivergence (CoulombGauge.java:148-166) per colour c of
 * the gauge field A = getAlgebraElement(U) (generator components); div: [ncomp][V] */
double orc_coulomb_divergence(const orc_params *p, const double *U, double *div)
{
    long V = vol(p);
    int nc = p->nc, ng = orc_ng(nc), ncomp = nc == 2 ? 3 : 8;
    double *A = malloc(sizeof(double) * (size_t)V * 3 * ncomp);
    for (long x = 0; x < V; x++)
        for (int dir = 0; dir < 3; dir++) link_log_gen(nc, U + ((size_t)x * 3 + dir) * ng, A + ((size_t)x * 3 + dir) * ncomp);
    double total = 0.0;
    for (int c = 0; c < ncomp; c++) {
        double s = 0.0;
        for (long x = 0; x < V; x++) {
            double d = 0.0;
            for (int dir = 0; dir < 3; dir++) {
                long xs = orc_shift(p, x, dir, -1);
                d += A[((size_t)x * 3 + dir) * ncomp + c] - A[((size_t)xs * 3 + dir) * ncomp + c];
            }
            div[(size_t)c * V + x] = d;
            s += d * d;
        }
        total += s;
    }
    free(A);
    return total;
}

/* g(x) = getLink(-psi(x)) (CoulombGauge.java:114-122) and GaugeTransformation's
 * action (GaugeTransformation.java:57-90) on U, Unext and E.  psi: [ncomp][V]. */
void orc_coulomb_apply(const orc_params *p, const double *psi, double *U, double *Unext, double *E)
{
    long V = vol(p);
    int nc = p->nc, ng = orc_ng(nc), na = orc_na(nc), ncomp = nc == 2 ? 3 : 8;
    double *g = malloc(sizeof(double) * ng * V);
    for (long x = 0; x < V; x++) {
        double v[8], alg[9];
        for (int c = 0; c < ncomp; c++) v[c] = psi[(size_t)c * V + x] * -1;
        if (nc == 2) su2_link_ref(v, g + 4 * x);
        else { su3_from_gen(v, alg); su3_getlink(alg, g + 18 * x); }
    }
    for (long x = 0; x < V; x++)
        for (int dir = 0; dir < 3; dir++) {
            double gd[NG_MAX], t[NG_MAX], r[NG_MAX];
            long xs = orc_shift(p, x, dir, 1);
            const double *gx = g + (size_t)ng * x;
            orc_group_adj(nc, g + (size_t)ng * xs, gd);
            double *u = U + ((size_t)x * 3 + dir) * ng;
            orc_group_mult(nc, gx, u, t);
            orc_group_mult(nc, t, gd, r);
            memcpy(u, r, sizeof(double) * ng);
            u = Unext + ((size_t)x * 3 + dir) * ng;
            orc_group_mult(nc, gx, u, t);
            orc_group_mult(nc, t, gd, r);
            memcpy(u, r, sizeof(double) * ng);
            /* E -> proj(g getLinearizedLink(E) g^dagger) (SU2AlgebraElement.java:133-138,
             * SU3AlgebraElement.java:402-405) */
            double *e = E + ((size_t)x * 3 + dir) * na;
            double Lk[NG_MAX], ga[NG_MAX];
            if (nc == 2) {
                double sum = (e[0] * e[0] + e[1] * e[1] + e[2] * e[2]) / 4;
                Lk[0] = sqrt(1.0 - sum); Lk[1] = e[0] / 2; Lk[2] = e[1] / 2; Lk[3] = e[2] / 2;
            } else {
                double w[18] = {1, e[3], e[6], -e[3], 1, e[7], -e[6], -e[7], 1,
                                e[0], e[1], e[2], e[1], e[4], e[5], e[2], e[5], e[8]};
                memcpy(Lk, w, sizeof(w));
            }
            orc_group_adj(nc, gx, ga);
            orc_group_mult(nc, gx, Lk, t);
            orc_group_mult(nc, t, ga, r);
            orc_group_proj(nc, r, e);
        }
    free(g);
}

/* The gauge field of OccupationNumbersInTime.calculate (:203-225):
 * A[dir][c][x] = 0.5 (A_c(U_dir(x)) + A_c(Unext_dir(x))) * gainv and
 * Ef[dir][c][x] = E_dir(x).get(c) * gainv, c over the ncomp generator components. */
void orc_occupation_fields(const orc_params *p, const double *U, const double *Unext, const double *E,
                           double gainv, double *Ef, double *A)
{
    long V = vol(p);
    int nc = p->nc, ng = orc_ng(nc), na = orc_na(nc), ncomp = nc == 2 ? 3 : 8;
    for (long x = 0; x < V; x++)
        for (int j = 0; j < 3; j++) {
            double a0[8], a1[8], eg[8];
            link_log_gen(nc, U + ((size_t)x * 3 + j) * ng, a0);
            link_log_gen(nc, Unext + ((size_t)x * 3 + j) * ng, a1);
            orc_alg_to_gen(nc, E + ((size_t)x * 3 + j) * na, eg);
            for (int k = 0; k < ncomp; k++) {
                Ef[((size_t)j * ncomp + k) * V + x] = eg[k] * gainv;
                A[((size_t)j * ncomp + k) * V + x] = 0.5 * (a0[k] * gainv + a1[k] * gainv);
            }
        }
}

/* ------------------------------------------------------------------------- */
/* ImplicitTYMSolver.step (physics/fields/ImplicitTYMSolver.java:35-58), SU(2) and SU(3) */
/* ------------------------------------------------------------------------- */

/* SU2GroupElement.pow(x) = getAlgebraElement().mult(x).getLink() (math/SU2GroupElement.java:269-271) */
static void su2_pow(const double *u, double x, double *out)
{
    double v[3];
    su2_log(u, v);
    for (int c = 0; c < 3; c++) v[c] = v[c] * x;
    su2_link_ref(v, out);
}

static void group_pow(int nc, const double *u, double x, double *out)
{
    if (nc == 2) su2_pow(u, x, out); else orc_su3_pow(u, x, out);
}

/* ImplicitStep.getPlaquetteSum (:136-177): plaquettes closed along the central
 * link, with the links of direction i / d taken at time -1 (W_m, the grid's
 * Unext slot, which holds the previous U), 0 (W_0 = grid U) or +1 (W_p = the
 * implicit grid's U), implicit time in the transverse plane and along the beam. */
static void implicit_plaquette_sum(const orc_params *p, const double *Wm, const double *W0, const double *Wp,
                                   long index, int d, int beam, int time, double *S)
{
    const int nc = p->nc, ng = orc_ng(nc);
    memset(S, 0, sizeof(double) * ng);
    long ci1 = orc_shift(p, index, d, 1);
    for (int i = 0; i < 3; i++) {
        if (i == d) continue;
        int inT = (i != beam) && (d != beam);
        int td = 0, ti = 0;
        if (inT) { td = time; ti = time; }
        else { if (d == beam) td = time; else if (i == beam) ti = time; }
        const double *Wd = td < 0 ? Wm : (td > 0 ? Wp : W0);
        const double *Wi = ti < 0 ? Wm : (ti > 0 ? Wp : W0);
        long ci2 = orc_shift(p, index, i, 1), ci3 = orc_shift(p, ci1, i, -1), ci4 = orc_shift(p, index, i, -1);
        double U1[NG_MAX], U2[NG_MAX], t[NG_MAX], adj[NG_MAX];
        orc_group_adj(nc, link(p, Wd, ci2, d), adj);
        orc_group_mult(nc, link(p, Wi, ci1, i), adj, U1);
        orc_group_adj(nc, link(p, Wi, index, i), adj);
        orc_group_mult(nc, U1, adj, t);
        memcpy(U1, t, sizeof(double) * ng);
        orc_group_mult(nc, link(p, Wd, ci4, d), link(p, Wi, ci3, i), U2);
        orc_group_adj(nc, U2, t);
        orc_group_mult(nc, t, link(p, Wi, ci4, i), U2);
        double areaFactor = 1.0 / pow(p->a[i], 2);
        for (int k = 0; k < ng; k++) U1[k] = U1[k] + U2[k];
        orc_group_mult(nc, link(p, Wd, index, d), U1, t);
        for (int k = 0; k < ng; k++) U1[k] = t[k] * areaFactor;
        for (int k = 0; k < ng; k++) S[k] = S[k] + U1[k];
    }
}

/* In place of orc_update_grid for the implicit solver: U current links, Unext
 * the previous links (the slot after storeFields), E, J; writes E and Unext of
 * the active cells. */
int orc_implicit_update_grid(const orc_params *p, const double *U, double *E, const double *J, double *Unext,
                             const uint8_t *active, int iterations, double damping)
{
    const int nc = p->nc, ng = orc_ng(nc), na = orc_na(nc), beam = 0;
    long V = vol(p);
    size_t nl = (size_t)V * 3 * ng, ne = (size_t)V * 3 * na;
    /* Grid(grid): the implicit grid is a copy */
    double *Ui = malloc(sizeof(double) * nl), *Uin = malloc(sizeof(double) * nl), *Ei = malloc(sizeof(double) * ne);
    memcpy(Ui, U, sizeof(double) * nl);
    memcpy(Uin, Unext, sizeof(double) * nl);
    memcpy(Ei, E, sizeof(double) * ne);
    /* ImplicitBegin (:68-90) */
    for (long x = 0; x < V; x++) {
        if (active && !active[x]) continue;
        for (int i = 0; i < 3; i++) {
            double S[NG_MAX], temp[NG_MAX], pr[NA_MAX], ve[NA_MAX], Vl[NG_MAX], t[NG_MAX];
            double unitFactor = -(p->g * p->a[i]) * p->dt;
            orc_staple_sum(p, U, x, i, S);
            orc_group_mult(nc, link(p, U, x, i), S, temp);
            orc_group_proj(nc, temp, pr);
            double *e = Ei + ((size_t)x * 3 + i) * na;
            const double *j = J + ((size_t)x * 3 + i) * na;
            for (int c = 0; c < na; c++) e[c] = e[c] + pr[c] * p->dt;
            for (int c = 0; c < na; c++) e[c] = e[c] + j[c] * unitFactor;
            for (int c = 0; c < na; c++) ve[c] = e[c] * -p->dt;
            orc_alg_getlink(nc, ve, Vl);
            orc_group_mult(nc, Vl, link(p, U, x, i), t);
            memcpy(Uin + ((size_t)x * 3 + i) * ng, t, sizeof(double) * ng);
        }
    }
    for (int it = 0; it < iterations; it++) {
        double *sw = Ui; Ui = Uin; Uin = sw; /* implicitGrid.storeFields() */
        /* ImplicitStep (:103-131) */
        for (long x = 0; x < V; x++) {
            if (active && !active[x]) continue;
            for (int i = 0; i < 3; i++) {
                double S[NG_MAX], pr[NA_MAX], ve[NA_MAX], Vl[NG_MAX], t[NG_MAX];
                double unitFactor = -(p->g * p->a[i]) * p->dt;
                double *e = Ei + ((size_t)x * 3 + i) * na;
                const double *j = J + ((size_t)x * 3 + i) * na;
                memcpy(e, E + ((size_t)x * 3 + i) * na, sizeof(double) * na);
                implicit_plaquette_sum(p, Unext, U, Ui, x, i, beam, +1, S);
                orc_group_proj(nc, S, pr);
                for (int c = 0; c < na; c++) e[c] = e[c] + pr[c] * (p->dt * 0.5);
                implicit_plaquette_sum(p, Unext, U, Ui, x, i, beam, -1, S);
                orc_group_proj(nc, S, pr);
                for (int c = 0; c < na; c++) e[c] = e[c] + pr[c] * (p->dt * 0.5);
                for (int c = 0; c < na; c++) e[c] = e[c] + j[c] * unitFactor;
                for (int c = 0; c < na; c++) ve[c] = e[c] * -p->dt;
                orc_alg_getlink(nc, ve, Vl);
                orc_group_mult(nc, Vl, link(p, U, x, i), t);
                memcpy(Uin + ((size_t)x * 3 + i) * ng, t, sizeof(double) * ng);
            }
        }
        /* ImplicitDamping (:195-207) */
        for (long x = 0; x < V; x++) {
            if (active && !active[x]) continue;
            for (int i = 0; i < 3; i++) {
                double U1[NG_MAX], U2[NG_MAX], t[NG_MAX];
                group_pow(nc, Uin + ((size_t)x * 3 + i) * ng, 1 - damping, U1);
                group_pow(nc, Ui + ((size_t)x * 3 + i) * ng, damping, U2);
                orc_group_mult(nc, U2, U1, t);
                memcpy(Uin + ((size_t)x * 3 + i) * ng, t, sizeof(double) * ng);
            }
        }
    }
    /* ImplicitEnd (:217-226) */
    for (long x = 0; x < V; x++) {
        if (active && !active[x]) continue;
        memcpy(E + (size_t)x * 3 * na, Ei + (size_t)x * 3 * na, sizeof(double) * 3 * na);
        memcpy(Unext + (size_t)x * 3 * ng, Uin + (size_t)x * 3 * ng, sizeof(double) * 3 * ng);
    }
    free(Ui); free(Uin); free(Ei);
    return 0;
}


/* ---- Wilson-line observables (physics/initial/CGC/WilsonLineObservables.java) ---- */

static double group_retrace(int nc, const double *u)
{
    /* GroupElement.getRealTrace: SU(2) 2 e0; SU(3) Re tr */
    return nc == 2 ? 2.0 * u[0] : u[0] + u[4] + u[8];
}

/* computeTadpole (:37-59): the mean of Re tr V over the transverse cells, summed in cell order */
double orc_wilson_tadpole(int nc, const double *vt, long ntr)
{
    int ng = orc_ng(nc);
    double s = 0.0;
    for (long i = 0; i < ntr; i++) s += group_retrace(nc, vt + (size_t)i * ng);
    return s / (double)ntr;
}

/* computeDipole (:67-131): Re tr(V(x) V(y)^dagger) binned by the periodic
 * transverse distance; nb = (int) sqrt(cells) / 2 bins of width ds =
 * min(n1 a1, n2 a2) / 2 / nb, i outer and j inner as in the reference.
 * Returns nb; out (nb values) and ds may be NULL. */
int orc_wilson_dipole(int nc, const double *vt, int n1, int n2, double a1, double a2, double *out, double *ds_out)
{
    int ng = orc_ng(nc);
    long total = (long)n1 * n2;
    int nb = (int)sqrt((double)total) / 2;
    if (!out) return nb;
    double *sum = calloc((size_t)(nb > 0 ? nb : 1), sizeof(double));
    long *cnt = calloc((size_t)(nb > 0 ? nb : 1), sizeof(long));
    double maxd = fmin(n1 * a1, n2 * a2) * 0.5;
    double ds = maxd / (double)nb;
    int nn[2] = {n1, n2};
    double as[2] = {a1, a2};
    for (long i = 0; i < total; i++) {
        int x[2] = {(int)(i / n2), (int)(i % n2)};
        for (long j = 0; j < total; j++) {
            int y[2] = {(int)(j / n2), (int)(j % n2)};
            double dist = 0.0;
            for (int k = 0; k < 2; k++) {
                double d = fabs((double)(x[k] - y[k]));
                if (d > nn[k] / 2) d -= nn[k];
                dist += d * d * as[k] * as[k];
            }
            dist = sqrt(dist);
            int bin = (int)(dist / ds);
            if (bin < nb) {
                double adj[NG_MAX], prod[NG_MAX];
                orc_group_adj(nc, vt + (size_t)j * ng, adj);
                orc_group_mult(nc, vt + (size_t)i * ng, adj, prod);
                sum[bin] += group_retrace(nc, prod);
                cnt[bin]++;
            }
        }
    }
    for (int b = 0; b < nb; b++) out[b] = sum[b] / (double)cnt[b];
    if (ds_out) *ds_out = ds;
    free(sum);
    free(cnt);
    return nb;
}
