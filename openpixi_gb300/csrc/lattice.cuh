// lattice.cuh -- lattice geometry and the structure-of-arrays field layout.
//
// Site index s = ((x0*N1)+x1)*N2+x2, dimension 0 slowest (Grid.java:757-770),
// so dimension 2 is contiguous and a warp reads 32 consecutive sites.
// SU(3) links are stored in warp-sized blocks of 32 consecutive sites,
//   U[d][s/32][c][s%32]   (c < 18),
// so that component c of 32 consecutive sites is one 128-byte (FP32) or
// 256-byte (FP64) line, and the 18 components of one link sit at fixed
// 32-element strides from one address (one address computation per link).
// SU(2) links keep their four quaternion components together, U[d][s][4]
// (one vector load per link), with the site count padded to 32.
// Algebra fields are plain planes, one contiguous array of V values per
// component:
//   fields E[d][a][s]  (a < NA: 3 for SU(2), 8 for SU(3), generator components)
//   rho    [a][s]
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "group.cuh"

namespace opx {

struct Lat {
    int n[3];
    long V;
    long stride[3];  // n1*n2, n2, 1
    double a[3];
    double dt, g;
    // the staple area factors 1/a_j^2 and current factors -g a_i dt, in both
    // precisions, so that FP32 kernels do no FP64 arithmetic or conversions
    double inva2[3], jfac[3];
    float inva2f[3], jfacf[3], dtf;
    // Grid.getB area factor a_d / (a_j a_k) and Gauss-law factor 1 / (a_i g a_i)
    double bfac[3], gfac[3];
    float bfacf[3], gfacf[3];
    // division by N2 (k = 0) and N1 (k = 1) of site indices below 2^31 as a
    // multiply and a shift: s / N = (s * dmul[k]) >> dsh[k] (div_n)
    unsigned dmul[2];
    int dsh[2];
};

// m = ceil(2^(31 + l) / n), l = ceil(log2 n): then floor(s m / 2^(31 + l)) =
// floor(s / n) for every s < 2^31 (the round-up method of Granlund and
// Montgomery: s m / 2^(31 + l) exceeds s / n by less than 1 / n), and m < 2^32.
__host__ inline void div_magic(int n, unsigned *m, int *sh) {
    int l = 0;
    while ((1L << l) < n) l++;
    const unsigned long long p = 1ULL << (31 + l);
    *m = (unsigned)((p + (unsigned long long)n - 1) / (unsigned long long)n);
    *sh = 31 + l;
}

__host__ inline Lat make_lat(const int *dims, const double *a, double dt, double g) {
    Lat L;
    for (int i = 0; i < 3; i++) { L.n[i] = dims[i]; L.a[i] = a[i]; }
    L.V = (long)dims[0] * dims[1] * dims[2];
    L.stride[2] = 1;
    L.stride[1] = dims[2];
    L.stride[0] = (long)dims[1] * dims[2];
    L.dt = dt;
    L.g = g;
    for (int i = 0; i < 3; i++) {
        L.inva2[i] = 1.0 / (a[i] * a[i]);
        L.jfac[i] = -(g * a[i]) * dt;
        L.inva2f[i] = (float)L.inva2[i];
        L.jfacf[i] = (float)L.jfac[i];
    }
    L.dtf = (float)dt;
    for (int d = 0; d < 3; d++) {
        const int j = (d + 1) % 3, k = (d + 2) % 3;
        L.bfac[d] = a[d] / (a[j] * a[k]);
        L.gfac[d] = 1.0 / (a[d] * (g * a[d]));
        L.bfacf[d] = (float)L.bfac[d];
        L.gfacf[d] = (float)L.gfac[d];
    }
    div_magic(dims[2], &L.dmul[0], &L.dsh[0]);
    div_magic(dims[1], &L.dmul[1], &L.dsh[1]);
    return L;
}

template <typename R> struct LatR;
template <> struct LatR<double> {
    __device__ __forceinline__ static double inva2(const Lat &L, int d) {
        return d == 0 ? L.inva2[0] : (d == 1 ? L.inva2[1] : L.inva2[2]);
    }
    __device__ __forceinline__ static double jfac(const Lat &L, int d) {
        return d == 0 ? L.jfac[0] : (d == 1 ? L.jfac[1] : L.jfac[2]);
    }
    __device__ __forceinline__ static double dt(const Lat &L) { return L.dt; }
    __device__ __forceinline__ static double bfac(const Lat &L, int d) {
        return d == 0 ? L.bfac[0] : (d == 1 ? L.bfac[1] : L.bfac[2]);
    }
    __device__ __forceinline__ static double gfac(const Lat &L, int d) {
        return d == 0 ? L.gfac[0] : (d == 1 ? L.gfac[1] : L.gfac[2]);
    }
};
template <> struct LatR<float> {
    __device__ __forceinline__ static float inva2(const Lat &L, int d) {
        return d == 0 ? L.inva2f[0] : (d == 1 ? L.inva2f[1] : L.inva2f[2]);
    }
    __device__ __forceinline__ static float jfac(const Lat &L, int d) {
        return d == 0 ? L.jfacf[0] : (d == 1 ? L.jfacf[1] : L.jfacf[2]);
    }
    __device__ __forceinline__ static float dt(const Lat &L) { return L.dtf; }
    __device__ __forceinline__ static float bfac(const Lat &L, int d) {
        return d == 0 ? L.bfacf[0] : (d == 1 ? L.bfacf[1] : L.bfacf[2]);
    }
    __device__ __forceinline__ static float gfac(const Lat &L, int d) {
        return d == 0 ? L.gfacf[0] : (d == 1 ? L.gfacf[1] : L.gfacf[2]);
    }
};

// Periodic neighbour offsets of site s (Grid.shift, Grid.java:802-823).
struct Nbr {
    long fwd[3];  // index of x + d
    long bwd[3];  // index of x - d
};

// floor(s / N2) (k = 0) or floor(s / N1) (k = 1) for 0 <= s < 2^31
OPX_HD OPX_INLINE int div_n(const Lat &L, int k, int s) {
    return (int)(((unsigned long long)(unsigned)s * (unsigned long long)L.dmul[k]) >> L.dsh[k]);
}
// Coordinates of site s; I = int where the site index fits (then without a
// division: div_n), 64-bit divisions otherwise.
template <typename I>
__device__ __forceinline__ void site_coords(const Lat &L, I s, int *x) {
    I t, u;
    if constexpr (sizeof(I) == 4) t = (I)div_n(L, 0, (int)s);
    else t = s / (I)L.n[2];
    x[2] = (int)(s - t * (I)L.n[2]);
    if constexpr (sizeof(I) == 4) u = (I)div_n(L, 1, (int)t);
    else u = t / (I)L.n[1];
    x[1] = (int)(t - u * (I)L.n[1]);
    x[0] = (int)u;
}

__device__ __forceinline__ Nbr neighbours(const Lat &L, long s, const int *x) {
    Nbr nb;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        long st = L.stride[d];
        long wrap = (long)(L.n[d] - 1) * st;
        nb.fwd[d] = x[d] == L.n[d] - 1 ? s - wrap : s + st;
        nb.bwd[d] = x[d] == 0 ? s + wrap : s - st;
    }
    return nb;
}

// Shift by one unit in direction d (runtime) with orientation o, given the
// coordinate xd of s along d.  Selects instead of indexed arrays keep
// everything in registers when d is not a compile-time constant.
__device__ __forceinline__ long shift_d(const Lat &L, long s, int xd, int d, int o) {
    const int nd = d == 0 ? L.n[0] : (d == 1 ? L.n[1] : L.n[2]);
    const long st = d == 0 ? L.stride[0] : (d == 1 ? L.stride[1] : 1L);
    if (o > 0) return xd == nd - 1 ? s - (long)(nd - 1) * st : s + st;
    return xd == 0 ? s + (long)(nd - 1) * st : s - st;
}
__device__ __forceinline__ int pick(int a0, int a1, int a2, int d) { return d == 0 ? a0 : (d == 1 ? a1 : a2); }
template <typename T> __device__ __forceinline__ T pick3(T a0, T a1, T a2, int d) {
    return d == 0 ? a0 : (d == 1 ? a1 : a2);
}

// Periodic neighbour offsets of a site, computed once: s + f_d is x + d,
// s + b_d is x - d; and x + i - j is s + f_i + b_j for i != j (the j
// coordinate of x + i is that of x).
template <typename I> struct Deltas {
    I f0, f1, f2, b0, b1, b2;
    __device__ __forceinline__ I f(int d) const { return pick3(f0, f1, f2, d); }
    __device__ __forceinline__ I b(int d) const { return pick3(b0, b1, b2, d); }
};
template <typename I> __device__ __forceinline__ Deltas<I> deltas(const Lat &L, const int *x) {
    Deltas<I> D;
    const I st0 = (I)L.stride[0], st1 = (I)L.stride[1];
    const I w0 = (I)(L.n[0] - 1) * st0, w1 = (I)(L.n[1] - 1) * st1, w2 = (I)(L.n[2] - 1);
    D.f0 = x[0] == L.n[0] - 1 ? -w0 : st0;
    D.b0 = x[0] == 0 ? w0 : -st0;
    D.f1 = x[1] == L.n[1] - 1 ? -w1 : st1;
    D.b1 = x[1] == 0 ? w1 : -st1;
    D.f2 = x[2] == L.n[2] - 1 ? -w2 : (I)1;
    D.b2 = x[2] == 0 ? w2 : (I)-1;
    return D;
}
__device__ __forceinline__ double pickd(double a0, double a1, double a2, int d) { return d == 0 ? a0 : (d == 1 ? a1 : a2); }

// Read-only loads through the non-coherent cache for built-in element types;
// other element types (the dual numbers of the tangent-linear form) load plainly.
template <typename R> __device__ __forceinline__ R ld(const R *p) { return *p; }
template <> __device__ __forceinline__ float ld<float>(const float *p) { return __ldg(p); }
template <> __device__ __forceinline__ double ld<double>(const double *p) { return __ldg(p); }

// Link layouts.  SU(3) (NG = 18): warp-blocked, component c of 32 consecutive
// sites contiguous.  SU(2) (NG = 4): the four quaternion components of a link
// contiguous (one 16-byte vector load in FP32, two in FP64), links of
// consecutive sites consecutive.  Both pad the site count to a multiple of 32.
__host__ __device__ __forceinline__ long link_blocks(long V) { return (V + 31) >> 5; }
// Element offset of component c of link (s, d); I = int where every offset fits.
template <typename I>
__host__ __device__ __forceinline__ I link_offset_t(I V, int NG, int d, int c, I s) {
    const I nb = (V + 31) >> 5;
    if (NG == 4) return ((I)d * (nb << 5) + s) * 4 + c;
    return (((I)d * nb + (s >> 5)) * NG + c) * 32 + (s & 31);
}
__host__ __device__ __forceinline__ long link_offset(long V, int NG, int d, int c, long s) {
    return link_offset_t<long>(V, NG, d, c, s);
}
__host__ __device__ __forceinline__ long link_elems(long V, int NG) { return 3L * link_blocks(V) * 32 * NG; }

// Structure-of-arrays views; I is the type of the site and element offsets.
template <class G, typename R, typename I = long> struct LinkPlanes {
    R *p;
    I V;
    __device__ __forceinline__ typename G::M load(int d, I s) const;
    __device__ __forceinline__ void store(int d, I s, const typename G::M &m) const;
};

// Four contiguous reals: vector loads and stores for the built-in types.
template <typename R> __device__ __forceinline__ void ld4(const R *b, R *e) {
    e[0] = b[0]; e[1] = b[1]; e[2] = b[2]; e[3] = b[3];
}
template <> __device__ __forceinline__ void ld4<float>(const float *b, float *e) {
    const float4 v = __ldg(reinterpret_cast<const float4 *>(b));
    e[0] = v.x; e[1] = v.y; e[2] = v.z; e[3] = v.w;
}
template <> __device__ __forceinline__ void ld4<double>(const double *b, double *e) {
    const double2 v0 = __ldg(reinterpret_cast<const double2 *>(b));
    const double2 v1 = __ldg(reinterpret_cast<const double2 *>(b) + 1);
    e[0] = v0.x; e[1] = v0.y; e[2] = v1.x; e[3] = v1.y;
}
template <typename R> __device__ __forceinline__ void st4(R *b, const R *e) {
    b[0] = e[0]; b[1] = e[1]; b[2] = e[2]; b[3] = e[3];
}
template <> __device__ __forceinline__ void st4<float>(float *b, const float *e) {
    *reinterpret_cast<float4 *>(b) = make_float4(e[0], e[1], e[2], e[3]);
}
template <> __device__ __forceinline__ void st4<double>(double *b, const double *e) {
    reinterpret_cast<double2 *>(b)[0] = make_double2(e[0], e[1]);
    reinterpret_cast<double2 *>(b)[1] = make_double2(e[2], e[3]);
}

template <typename R, typename I> struct LinkPlanes<SU2<R>, R, I> {
    R *p;
    I V;
    __device__ __forceinline__ Q2<R> load(int d, I s) const {
        Q2<R> q;
        ld4<R>(p + link_offset_t<I>(V, 4, d, 0, s), q.e);
        return q;
    }
    __device__ __forceinline__ void store(int d, I s, const Q2<R> &m) const {
        st4<R>(p + link_offset_t<I>(V, 4, d, 0, s), m.e);
    }
};

template <typename R, typename I> struct LinkPlanes<SU3<R>, R, I> {
    R *p;
    I V;
    __device__ __forceinline__ M3<R> load(int d, I s) const {
        const R *b = p + link_offset_t<I>(V, 18, d, 0, s);
        M3<R> m;
#pragma unroll
        for (int k = 0; k < 9; k++) { m.r[k] = ld(b + k * 32); m.i[k] = ld(b + (9 + k) * 32); }
        return m;
    }
    __device__ __forceinline__ void store(int d, I s, const M3<R> &m) const {
        R *b = p + link_offset_t<I>(V, 18, d, 0, s);
#pragma unroll
        for (int k = 0; k < 9; k++) { b[k * 32] = m.r[k]; b[(9 + k) * 32] = m.i[k]; }
    }
};

// Algebra-valued link field E[d][a][s] (or site field with d = 0).
template <int NA, typename R, typename I = long> struct AlgPlanes {
    R *p;
    I V;
    __device__ __forceinline__ void load(int d, I s, R *x) const {
        const R *b = p + ((I)d * NA * V + s);
#pragma unroll
        for (int a = 0; a < NA; a++) x[a] = b[a * V];
    }
    __device__ __forceinline__ void load_ro(int d, I s, R *x) const {
        const R *b = p + ((I)d * NA * V + s);
#pragma unroll
        for (int a = 0; a < NA; a++) x[a] = ld(b + a * V);
    }
    __device__ __forceinline__ void store(int d, I s, const R *x) const {
        R *b = p + ((I)d * NA * V + s);
#pragma unroll
        for (int a = 0; a < NA; a++) b[a * V] = x[a];
    }
};

}  // namespace opx
