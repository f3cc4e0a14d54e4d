// dual.cuh -- forward-mode dual numbers (value, tangent) in FP64.
//
// Instantiating the leapfrog templates (group.cuh, leapfrog.cuh) with this
// element type runs the tangent-linear model of the exact same arithmetic: the
// value part is the FP64 trajectory and the tangent part its directional
// derivative.  Branches (Taylor or sincos in the SU(2) exponential) are taken
// on the value part.
#pragma once
#include <math.h>

#include "group.cuh"
#include "lattice.cuh"

namespace opx {

struct Dual {
    double v, d;
    Dual() = default;
    OPX_HD constexpr Dual(double x) : v(x), d(0.0) {}
    OPX_HD constexpr Dual(double x, double y) : v(x), d(y) {}
};

OPX_HD inline Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
OPX_HD inline Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
OPX_HD inline Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
OPX_HD inline Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
OPX_HD inline Dual operator/(Dual a, Dual b) {
    const double q = a.v / b.v;
    return Dual(q, (a.d - q * b.d) / b.v);
}
OPX_HD inline Dual &operator+=(Dual &a, Dual b) { a = a + b; return a; }
OPX_HD inline Dual &operator-=(Dual &a, Dual b) { a = a - b; return a; }
OPX_HD inline Dual &operator*=(Dual &a, Dual b) { a = a * b; return a; }
OPX_HD inline bool operator<(Dual a, Dual b) { return a.v < b.v; }
OPX_HD inline bool operator>(Dual a, Dual b) { return a.v > b.v; }

template <> struct Real<Dual> {
    static constexpr double eps = 1.1102230246251565e-16;
    OPX_HD static Dual sqrt_(Dual x) {
        const double r = sqrt(x.v);
        return Dual(r, r > 0.0 ? x.d / (2.0 * r) : 0.0);
    }
    OPX_HD static void sincos_(Dual x, Dual *s, Dual *c) {
        double sv, cv;
#ifdef __CUDA_ARCH__
        sincos(x.v, &sv, &cv);
#else
        sv = ::sin(x.v);
        cv = ::cos(x.v);
#endif
        *s = Dual(sv, cv * x.d);
        *c = Dual(cv, -sv * x.d);
    }
};

template <> struct LatR<Dual> {
    __device__ __forceinline__ static Dual inva2(const Lat &L, int d) { return Dual(LatR<double>::inva2(L, d)); }
    __device__ __forceinline__ static Dual jfac(const Lat &L, int d) { return Dual(LatR<double>::jfac(L, d)); }
    __device__ __forceinline__ static Dual dt(const Lat &L) { return Dual(L.dt); }
    __device__ __forceinline__ static Dual bfac(const Lat &L, int d) { return Dual(LatR<double>::bfac(L, d)); }
    __device__ __forceinline__ static Dual gfac(const Lat &L, int d) { return Dual(LatR<double>::gfac(L, d)); }
};

}  // namespace opx
