// group.cuh -- SU(2) and SU(3) arithmetic for the device kernels.
//
// Representations (the reference's, so that values move between host and
// device without conversion of the links):
//   SU(2): quaternion (e0, e1, e2, e3), U = e0 + i e_a sigma_a
//          (math/SU2GroupElement.java:3-14).  Products follow the quaternion
//          product of SU2GroupElement.mult (:206-217).
//   SU(3): 3x3 complex matrix, 9 real parts then 9 imaginary parts, row major
//          (math/SU3GroupElement.java:3-11).
// Algebra elements on the device are generator components X^a with
// X = X^a t_a, t_a = sigma_a/2 (SU(2)) or lambda_a/2 (SU(3)); this is the basis
// of SU3AlgebraElement.get(a) (math/SU3AlgebraElement.java:117-129) and the
// native basis of SU2AlgebraElement.  With it,
//   proj_a(M) = Im tr(lambda_a M)   (SU2GroupElement.proj :254-263, SU3GroupElement.proj :494-505)
//   square(X) = sum_a (X^a)^2       (SU2AlgebraElement.square, SU3AlgebraElement.square :174-176)
//   getLink(X) = exp(i X^a t_a)     (SU2AlgebraElement.getLink :140-152, SU3AlgebraElement.getLink :407-417)
//   act(X, g) = g X g^dagger        (SU2AlgebraElement.act :159-172, SU3AlgebraElement.act :144-168)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#define OPX_HD __host__ __device__
#define OPX_INLINE __forceinline__

namespace opx {

template <typename R> struct Real;
template <> struct Real<double> {
    static constexpr double eps = 1.1102230246251565e-16;
    OPX_HD static double sqrt_(double x) { return sqrt(x); }
    OPX_HD static double abs_(double x) { return fabs(x); }
    OPX_HD static double max_(double a, double b) { return fmax(a, b); }
    OPX_HD static void sincos_(double x, double *s, double *c) {
#ifdef __CUDA_ARCH__
        sincos(x, s, c);
#else
        *s = ::sin(x); *c = ::cos(x);
#endif
    }
};
template <> struct Real<float> {
    static constexpr float eps = 5.9604645e-08f;
    OPX_HD static float sqrt_(float x) { return sqrtf(x); }
    OPX_HD static float abs_(float x) { return fabsf(x); }
    OPX_HD static float max_(float a, float b) { return fmaxf(a, b); }
    OPX_HD static void sincos_(float x, float *s, float *c) {
#ifdef __CUDA_ARCH__
        sincosf(x, s, c);
#else
        *s = ::sinf(x); *c = ::cosf(x);
#endif
    }
};

// 1/k for the exponential series (t_k = t_(k-1) / k), k < 44: read from a
// table on the device (a product instead of a division per term; the index is
// uniform across a warp), computed on the host, the same correctly rounded values
static __constant__ double c_inv_k64[44] = {
    0.0, 1.0, 1.0 / 2, 1.0 / 3, 1.0 / 4, 1.0 / 5, 1.0 / 6, 1.0 / 7,
    1.0 / 8, 1.0 / 9, 1.0 / 10, 1.0 / 11, 1.0 / 12, 1.0 / 13, 1.0 / 14, 1.0 / 15,
    1.0 / 16, 1.0 / 17, 1.0 / 18, 1.0 / 19, 1.0 / 20, 1.0 / 21, 1.0 / 22, 1.0 / 23,
    1.0 / 24, 1.0 / 25, 1.0 / 26, 1.0 / 27, 1.0 / 28, 1.0 / 29, 1.0 / 30, 1.0 / 31,
    1.0 / 32, 1.0 / 33, 1.0 / 34, 1.0 / 35, 1.0 / 36, 1.0 / 37, 1.0 / 38, 1.0 / 39,
    1.0 / 40, 1.0 / 41, 1.0 / 42, 1.0 / 43};
static __constant__ float c_inv_k32[44] = {
    0.f, 1.f, 1.f / 2, 1.f / 3, 1.f / 4, 1.f / 5, 1.f / 6, 1.f / 7,
    1.f / 8, 1.f / 9, 1.f / 10, 1.f / 11, 1.f / 12, 1.f / 13, 1.f / 14, 1.f / 15,
    1.f / 16, 1.f / 17, 1.f / 18, 1.f / 19, 1.f / 20, 1.f / 21, 1.f / 22, 1.f / 23,
    1.f / 24, 1.f / 25, 1.f / 26, 1.f / 27, 1.f / 28, 1.f / 29, 1.f / 30, 1.f / 31,
    1.f / 32, 1.f / 33, 1.f / 34, 1.f / 35, 1.f / 36, 1.f / 37, 1.f / 38, 1.f / 39,
    1.f / 40, 1.f / 41, 1.f / 42, 1.f / 43};
template <typename R> OPX_HD OPX_INLINE R inv_k(int k) { return R(1) / R(k); }
template <> OPX_HD OPX_INLINE double inv_k<double>(int k) {
#ifdef __CUDA_ARCH__
    return c_inv_k64[k];
#else
    return 1.0 / k;
#endif
}
template <> OPX_HD OPX_INLINE float inv_k<float>(int k) {
#ifdef __CUDA_ARCH__
    return c_inv_k32[k];
#else
    return 1.f / (float)k;
#endif
}

// ------------------------------------------------------------------------ SU(2)
template <typename R> struct Q2 {
    R e[4];
};

template <typename R> struct SU2 {
    static constexpr int NG = 4;  // reals per link
    static constexpr int NA = 3;  // generator components
    using M = Q2<R>;

    OPX_HD OPX_INLINE static M identity() { return M{{R(1), R(0), R(0), R(0)}}; }
    OPX_HD OPX_INLINE static M zero() { return M{{R(0), R(0), R(0), R(0)}}; }

    // a * b  (SU2GroupElement.mult)
    OPX_HD OPX_INLINE static M mul(const M &x, const M &a) {
        M b;
        b.e[0] = x.e[0] * a.e[0] - x.e[1] * a.e[1] - x.e[2] * a.e[2] - x.e[3] * a.e[3];
        b.e[1] = x.e[0] * a.e[1] + x.e[1] * a.e[0] - x.e[2] * a.e[3] + x.e[3] * a.e[2];
        b.e[2] = x.e[0] * a.e[2] + x.e[2] * a.e[0] - x.e[3] * a.e[1] + x.e[1] * a.e[3];
        b.e[3] = x.e[0] * a.e[3] + x.e[3] * a.e[0] - x.e[1] * a.e[2] + x.e[2] * a.e[1];
        return b;
    }
    OPX_HD OPX_INLINE static M adj(const M &a) { return M{{a.e[0], -a.e[1], -a.e[2], -a.e[3]}}; }
    OPX_HD OPX_INLINE static M mul_adj(const M &a, const M &b) { return mul(a, adj(b)); }
    OPX_HD OPX_INLINE static M adj_mul(const M &a, const M &b) { return mul(adj(a), b); }
    OPX_HD OPX_INLINE static void add(M &acc, const M &b) {
#pragma unroll
        for (int k = 0; k < 4; k++) acc.e[k] += b.e[k];
    }
    OPX_HD OPX_INLINE static void scale(M &a, R s) {
#pragma unroll
        for (int k = 0; k < 4; k++) a.e[k] *= s;
    }
    // proj_a(M) = 2 e_a
    OPX_HD OPX_INLINE static void proj(const M &m, R *x) {
        x[0] = R(2) * m.e[1];
        x[1] = R(2) * m.e[2];
        x[2] = R(2) * m.e[3];
    }
    // Re tr M
    OPX_HD OPX_INLINE static R retrace(const M &m) { return R(2) * m.e[0]; }

    // exp(i v_a sigma_a / 2) = (cos m, v_a sin(m)/(2m)), m = |v|/2.  For
    // m^2 < 0.01 the cosine and sin(m)/m come from their Taylor series
    // (truncation below 1e-21); otherwise from sincos.
    OPX_HD OPX_INLINE static M expi(const R *v) {
        R m2 = (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) * R(0.25);
        R c, s;
        if (m2 < R(0.01)) {
            // cos m = sum (-1)^k m^2k/(2k)!,  sin m / m = sum (-1)^k m^2k/(2k+1)!
            c = R(1) + m2 * (R(-1.0 / 2) + m2 * (R(1.0 / 24) + m2 * (R(-1.0 / 720) +
                m2 * (R(1.0 / 40320) + m2 * (R(-1.0 / 3628800))))));
            s = R(1) + m2 * (R(-1.0 / 6) + m2 * (R(1.0 / 120) + m2 * (R(-1.0 / 5040) +
                m2 * (R(1.0 / 362880) + m2 * (R(-1.0 / 39916800))))));
        } else {
            R m = Real<R>::sqrt_(m2), sn;
            Real<R>::sincos_(m, &sn, &c);
            s = sn / m;
        }
        R h = R(0.5) * s;
        return M{{c, v[0] * h, v[1] * h, v[2] * h}};
    }
    // g X g^dagger with X = x_a sigma_a/2
    OPX_HD OPX_INLINE static void act(const R *x, const M &g, R *out) {
        M X{{R(0), x[0] * R(0.5), x[1] * R(0.5), x[2] * R(0.5)}};
        M t = mul(g, mul(X, adj(g)));
        proj(t, out);
    }
    OPX_HD OPX_INLINE static void reunit(M &m) {
        R n = m.e[0] * m.e[0] + m.e[1] * m.e[1] + m.e[2] * m.e[2] + m.e[3] * m.e[3];
        R inv = R(1) / Real<R>::sqrt_(n);
        scale(m, inv);
    }
};

// ------------------------------------------------------------------------ SU(3)
template <typename R> struct M3 {
    R r[9], i[9];
};

template <typename R> struct SU3 {
    static constexpr int NG = 18;
    static constexpr int NA = 8;
    using M = M3<R>;

    OPX_HD OPX_INLINE static M zero() {
        M m;
#pragma unroll
        for (int k = 0; k < 9; k++) { m.r[k] = R(0); m.i[k] = R(0); }
        return m;
    }
    OPX_HD OPX_INLINE static M identity() {
        M m = zero();
        m.r[0] = m.r[4] = m.r[8] = R(1);
        return m;
    }
    // a * b
    OPX_HD OPX_INLINE static M mul(const M &a, const M &b) {
        M c;
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
            for (int q = 0; q < 3; q++) {
                R re = R(0), im = R(0);
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    re += a.r[3 * r + k] * b.r[3 * k + q] - a.i[3 * r + k] * b.i[3 * k + q];
                    im += a.r[3 * r + k] * b.i[3 * k + q] + a.i[3 * r + k] * b.r[3 * k + q];
                }
                c.r[3 * r + q] = re;
                c.i[3 * r + q] = im;
            }
        return c;
    }
    // a * b^dagger
    OPX_HD OPX_INLINE static M mul_adj(const M &a, const M &b) {
        M c;
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
            for (int q = 0; q < 3; q++) {
                R re = R(0), im = R(0);
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    // (b^dagger)_{kq} = conj(b_{qk})
                    re += a.r[3 * r + k] * b.r[3 * q + k] + a.i[3 * r + k] * b.i[3 * q + k];
                    im += a.i[3 * r + k] * b.r[3 * q + k] - a.r[3 * r + k] * b.i[3 * q + k];
                }
                c.r[3 * r + q] = re;
                c.i[3 * r + q] = im;
            }
        return c;
    }
    // a^dagger * b
    OPX_HD OPX_INLINE static M adj_mul(const M &a, const M &b) {
        M c;
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
            for (int q = 0; q < 3; q++) {
                R re = R(0), im = R(0);
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    // (a^dagger)_{rk} = conj(a_{kr})
                    re += a.r[3 * k + r] * b.r[3 * k + q] + a.i[3 * k + r] * b.i[3 * k + q];
                    im += a.r[3 * k + r] * b.i[3 * k + q] - a.i[3 * k + r] * b.r[3 * k + q];
                }
                c.r[3 * r + q] = re;
                c.i[3 * r + q] = im;
            }
        return c;
    }
    OPX_HD OPX_INLINE static M adj(const M &a) {
        M c;
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
            for (int q = 0; q < 3; q++) {
                c.r[3 * r + q] = a.r[3 * q + r];
                c.i[3 * r + q] = -a.i[3 * q + r];
            }
        return c;
    }
    OPX_HD OPX_INLINE static void add(M &acc, const M &b) {
#pragma unroll
        for (int k = 0; k < 9; k++) { acc.r[k] += b.r[k]; acc.i[k] += b.i[k]; }
    }
    OPX_HD OPX_INLINE static void scale(M &a, R s) {
#pragma unroll
        for (int k = 0; k < 9; k++) { a.r[k] *= s; a.i[k] *= s; }
    }
    OPX_HD OPX_INLINE static R retrace(const M &m) { return m.r[0] + m.r[4] + m.r[8]; }

    // proj_a(M) = Im tr(lambda_a M)
    OPX_HD OPX_INLINE static void proj(const M &m, R *x) {
        const R inv_s3 = R(0.57735026918962576451);
        x[0] = m.i[1] + m.i[3];
        x[1] = m.r[1] - m.r[3];
        x[2] = m.i[0] - m.i[4];
        x[3] = m.i[2] + m.i[6];
        x[4] = m.r[2] - m.r[6];
        x[5] = m.i[5] + m.i[7];
        x[6] = m.r[5] - m.r[7];
        x[7] = (m.i[0] + m.i[4] - R(2) * m.i[8]) * inv_s3;
    }

    // Hermitian H = x^a lambda_a / 2 as a matrix
    OPX_HD OPX_INLINE static M herm(const R *x) {
        const R inv_2s3 = R(0.28867513459481288225);
        M h;
        h.r[0] = R(0.5) * x[2] + inv_2s3 * x[7];
        h.r[4] = -R(0.5) * x[2] + inv_2s3 * x[7];
        h.r[8] = -R(2) * inv_2s3 * x[7];
        h.i[0] = h.i[4] = h.i[8] = R(0);
        h.r[1] = R(0.5) * x[0]; h.i[1] = -R(0.5) * x[1];
        h.r[3] = R(0.5) * x[0]; h.i[3] = R(0.5) * x[1];
        h.r[2] = R(0.5) * x[3]; h.i[2] = -R(0.5) * x[4];
        h.r[6] = R(0.5) * x[3]; h.i[6] = R(0.5) * x[4];
        h.r[5] = R(0.5) * x[5]; h.i[5] = -R(0.5) * x[6];
        h.r[7] = R(0.5) * x[5]; h.i[7] = R(0.5) * x[6];
        return h;
    }
    // generator components of a hermitian matrix: x^a = tr(lambda_a H)
    OPX_HD OPX_INLINE static void herm_gen(const M &h, R *x) {
        const R inv_s3 = R(0.57735026918962576451);
        x[0] = h.r[1] + h.r[3];
        x[1] = h.i[3] - h.i[1];
        x[2] = h.r[0] - h.r[4];
        x[3] = h.r[2] + h.r[6];
        x[4] = h.i[6] - h.i[2];
        x[5] = h.r[5] + h.r[7];
        x[6] = h.i[7] - h.i[5];
        x[7] = (h.r[0] + h.r[4] - R(2) * h.r[8]) * inv_s3;
    }

    // exp(i H), H = x^a lambda_a/2 hermitian traceless.
    // Cayley-Hamilton: H^3 = c1 H + c0 with c1 = tr(H^2)/2, c0 = det H, so
    // H^k = al_k + be_k H + ga_k H^2 with al_{k+1} = c0 ga_k,
    // be_{k+1} = al_k + c1 ga_k, ga_{k+1} = be_k; the exponential series then
    // reduces to exp(iH) = f0 + f1 H + f2 H^2 with scalar series f_j.  The
    // series stops when the next term is below the working precision.
    // For ||H||_F^2 = 2 c1 > 1 the argument is halved s times and the result
    // squared s times (scaling and squaring).
    OPX_HD static M expi(const R *x) {
        M h = herm(x);
        R c1 = R(0);
#pragma unroll
        for (int a = 0; a < 8; a++) c1 += x[a] * x[a];
        c1 *= R(0.25);  // tr(H^2)/2 = sum x_a^2 / 4
        int s = 0;
        R sc = R(1);
        while (R(2) * c1 * sc * sc > R(1) && s < 30) { sc *= R(0.5); s++; }
        if (s) scale(h, sc);
        c1 *= sc * sc;
        // det of hermitian h (real): abc - a|w|^2 - b|v|^2 - c|u|^2 + 2 Re(u w conj(v)),
        // u = h01, v = h02, w = h12
        const R da = h.r[0], db = h.r[4], dc = h.r[8];
        const R ur = h.r[1], ui = h.i[1], vr = h.r[2], vi = h.i[2], wr = h.r[5], wi = h.i[5];
        R c0 = da * (db * dc - (wr * wr + wi * wi)) - db * (vr * vr + vi * vi) - dc * (ur * ur + ui * ui)
             + R(2) * (ur * (wr * vr + wi * vi) + ui * (wr * vi - wi * vr));
        // series: f = sum_k i^k/k! (al_k, be_k, ga_k)
        R al = R(1), be = R(0), ga = R(0), t = R(1);
        R f0r = R(1), f0i = R(0), f1r = R(0), f1i = R(0), f2r = R(0), f2i = R(0);
        R nrm = Real<R>::sqrt_(R(2) * c1);  // ||H||_F bounds the spectral radius
        R bound = R(1);
        const R nrm4 = (nrm * nrm) * (nrm * nrm);
        // four terms per pass, i^k fixed within a pass (k = 1, 2, 3, 0 mod 4),
        // the stopping test after the fourth
        for (int k = 1; k < 40; k += 4) {
#pragma unroll
            for (int u = 0; u < 4; u++) {
                R nal = c0 * ga, nbe = al + c1 * ga, nga = be;
                al = nal; be = nbe; ga = nga;
                t = t * inv_k<R>(k + u);
                if (u == 0) { f0i += t * al; f1i += t * be; f2i += t * ga; }
                else if (u == 1) { f0r -= t * al; f1r -= t * be; f2r -= t * ga; }
                else if (u == 2) { f0i -= t * al; f1i -= t * be; f2i -= t * ga; }
                else { f0r += t * al; f1r += t * be; f2r += t * ga; }
            }
            bound *= nrm4;
            if (bound * t < Real<R>::eps * R(0.01)) break;
        }
        // H^2
        M h2 = mul(h, h);
        M w;
#pragma unroll
        for (int k = 0; k < 9; k++) {
            R hr = h.r[k], hi = h.i[k], qr = h2.r[k], qi = h2.i[k];
            w.r[k] = f1r * hr - f1i * hi + f2r * qr - f2i * qi;
            w.i[k] = f1r * hi + f1i * hr + f2r * qi + f2i * qr;
        }
        w.r[0] += f0r; w.r[4] += f0r; w.r[8] += f0r;
        w.i[0] += f0i; w.i[4] += f0i; w.i[8] += f0i;
        for (int k = 0; k < s; k++) w = mul(w, w);
        return w;
    }

    // g X g^dagger for X = x^a lambda_a/2
    OPX_HD OPX_INLINE static void act(const R *x, const M &g, R *out) {
        M h = herm(x);
        M t = mul(g, h);
        M y = mul_adj(t, g);
        herm_gen(y, out);
    }

    // Gram-Schmidt on rows 0 and 1; row 2 = conj(row0 x row1)
    // Gram-Schmidt on rows 0 and 1; row 2 = conj(row0 x row1)
    OPX_HD OPX_INLINE static void reunit_gs(M &m) {
        R n0 = R(0);
#pragma unroll
        for (int k = 0; k < 3; k++) n0 += m.r[k] * m.r[k] + m.i[k] * m.i[k];
        R inv0 = R(1) / Real<R>::sqrt_(n0);
#pragma unroll
        for (int k = 0; k < 3; k++) { m.r[k] *= inv0; m.i[k] *= inv0; }
        // p = <row0, row1> = sum conj(r0_k) r1_k
        R pr = R(0), pi = R(0);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            pr += m.r[k] * m.r[3 + k] + m.i[k] * m.i[3 + k];
            pi += m.r[k] * m.i[3 + k] - m.i[k] * m.r[3 + k];
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
            m.r[3 + k] -= pr * m.r[k] - pi * m.i[k];
            m.i[3 + k] -= pr * m.i[k] + pi * m.r[k];
        }
        R n1 = R(0);
#pragma unroll
        for (int k = 0; k < 3; k++) n1 += m.r[3 + k] * m.r[3 + k] + m.i[3 + k] * m.i[3 + k];
        R inv1 = R(1) / Real<R>::sqrt_(n1);
#pragma unroll
        for (int k = 0; k < 3; k++) { m.r[3 + k] *= inv1; m.i[3 + k] *= inv1; }
        // row2 = conj(row0 x row1)
#pragma unroll
        for (int k = 0; k < 3; k++) {
            int a = (k + 1) % 3, b = (k + 2) % 3;
            R xr = (m.r[a] * m.r[3 + b] - m.i[a] * m.i[3 + b]) - (m.r[b] * m.r[3 + a] - m.i[b] * m.i[3 + a]);
            R xi = (m.r[a] * m.i[3 + b] + m.i[a] * m.r[3 + b]) - (m.r[b] * m.i[3 + a] + m.i[b] * m.r[3 + a]);
            m.r[6 + k] = xr;
            m.i[6 + k] = -xi;
        }
    }
    // H = m^dagger m (real diagonal, upper entries); returns the largest |H - 1| entry
    OPX_HD OPX_INLINE static R gram(const M &m, R *hd, R *hr, R *hi) {
        R dev = R(0);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            R d = R(0);
#pragma unroll
            for (int k = 0; k < 3; k++) d += m.r[3 * k + c] * m.r[3 * k + c] + m.i[3 * k + c] * m.i[3 * k + c];
            hd[c] = d;
            dev = Real<R>::max_(dev, Real<R>::abs_(d - R(1)));
        }
#pragma unroll
        for (int o = 0; o < 3; o++) {
            const int r = o == 2 ? 1 : 0, c = o == 0 ? 1 : 2;
            R re = R(0), im = R(0);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                re += m.r[3 * k + r] * m.r[3 * k + c] + m.i[3 * k + r] * m.i[3 * k + c];
                im += m.r[3 * k + r] * m.i[3 * k + c] - m.i[3 * k + r] * m.r[3 * k + c];
            }
            hr[o] = re;
            hi[o] = im;
            dev = Real<R>::max_(dev, Real<R>::max_(Real<R>::abs_(re), Real<R>::abs_(im)));
        }
        return dev;
    }
    // m <- m (3 - H) / 2, one Newton-Schulz step toward the polar factor
    OPX_HD OPX_INLINE static void newton_schulz(M &m, const R *hd, const R *hr, const R *hi) {
        M n;
#pragma unroll
        for (int r = 0; r < 3; r++)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const R kd = R(1.5) - R(0.5) * hd[c];
                R re = m.r[3 * r + c] * kd, im = m.i[3 * r + c] * kd;
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    if (k == c) continue;
                    const int o = (k == 0 || c == 0) ? (k + c - 1) : 2;
                    const R a = R(-0.5) * hr[o], b = R(-0.5) * (k < c ? hi[o] : -hi[o]);
                    re += m.r[3 * r + k] * a - m.i[3 * r + k] * b;
                    im += m.r[3 * r + k] * b + m.i[3 * r + k] * a;
                }
                n.r[3 * r + c] = re;
                n.i[3 * r + c] = im;
            }
        m = n;
    }
    // The nearest unitary matrix (polar factor: Newton-Schulz steps from a
    // near-unitary m), then the determinant's phase spread evenly over the
    // rows; Gram-Schmidt first when m is far from unitary (an entry of
    // m^dagger m off by more than 0.25).  The polar factor removes the
    // deviation from unitarity without rotating the link, so periodic
    // reunitarisation of the FP32 form adds no systematic energy drift.
    OPX_HD OPX_INLINE static void reunit(M &m) {
        R hd[3], hr[3], hi[3];
        R dev = gram(m, hd, hr, hi);
        if (dev > R(0.25)) {
            reunit_gs(m);
            dev = gram(m, hd, hr, hi);
        }
        newton_schulz(m, hd, hr, hi);
        // further steps while the last one left more than rounding
        for (int it = 0; it < 4 && dev > R(1e-3); it++) {
            dev = gram(m, hd, hr, hi);
            newton_schulz(m, hd, hr, hi);
        }
        // Im det m from the cofactors of row 0
        const R c0r = (m.r[4] * m.r[8] - m.i[4] * m.i[8]) - (m.r[5] * m.r[7] - m.i[5] * m.i[7]);
        const R c0i = (m.r[4] * m.i[8] + m.i[4] * m.r[8]) - (m.r[5] * m.i[7] + m.i[5] * m.r[7]);
        const R c1r = (m.r[5] * m.r[6] - m.i[5] * m.i[6]) - (m.r[3] * m.r[8] - m.i[3] * m.i[8]);
        const R c1i = (m.r[5] * m.i[6] + m.i[5] * m.r[6]) - (m.r[3] * m.i[8] + m.i[3] * m.r[8]);
        const R c2r = (m.r[3] * m.r[7] - m.i[3] * m.i[7]) - (m.r[4] * m.r[6] - m.i[4] * m.i[6]);
        const R c2i = (m.r[3] * m.i[7] + m.i[3] * m.r[7]) - (m.r[4] * m.i[6] + m.i[4] * m.r[6]);
        const R t = (m.r[0] * c0i + m.i[0] * c0r + m.r[1] * c1i + m.i[1] * c1r + m.r[2] * c2i + m.i[2] * c2r) / R(3);
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const R re = m.r[k] + t * m.i[k];
            m.i[k] = m.i[k] - t * m.r[k];
            m.r[k] = re;
        }
    }
};

template <int NC, typename R> struct GroupOf;
template <typename R> struct GroupOf<2, R> { using T = SU2<R>; };
template <typename R> struct GroupOf<3, R> { using T = SU3<R>; };

}  // namespace opx
