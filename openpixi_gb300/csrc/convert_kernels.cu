// convert_kernels.cu -- transposes between the reference's per-cell layout (host,
// FP64) and the device's structure-of-arrays planes (FP64 or FP32).
//
// The host-layout side is either a device staging copy or the caller's
// page-locked host buffer itself, read or written over the host link.  A block
// moves a contiguous span of XB host rows (one link, or one algebra element)
// through shared memory, so that the host side is read and written in whole
// lines whatever the row width.
//
// Links keep their components (SU(2) e0..e3, SU(3) 9 re + 9 im).  SU(3) algebra
// fields in the reference layout are the 9 entries of a hermitian matrix
// (math/SU3AlgebraElement.java:3-11); on the device they are the 8 generator
// components, converted with SU3AlgebraElement.get(a) (:117-129) on upload and
// with the set(a) sequence of the double[8] constructor (:36-49, :93-115) on
// download.
#include "internal.h"

namespace opx {

constexpr int XB = 128;  // host rows per block
constexpr int XW = 19;   // shared-memory row stride (doubles): the widest row (18) + 1

// Copies rows [r0, r0 + nr) of width w from the host layout into sh (stride XW).
__device__ __forceinline__ void rows_in(const double *__restrict__ src, long r0, int nr, int w, double *sh) {
    const double *s0 = src + r0 * w;
    for (int k = threadIdx.x; k < nr * w; k += XB) {
        const int l = k / w;
        sh[l * XW + (k - l * w)] = s0[k];
    }
}
__device__ __forceinline__ void rows_out(double *__restrict__ dst, long r0, int nr, int w, const double *sh) {
    double *d0 = dst + r0 * w;
    for (int k = threadIdx.x; k < nr * w; k += XB) {
        const int l = k / w;
        d0[k] = sh[l * XW + (k - l * w)];
    }
}

template <typename R>
__global__ void __launch_bounds__(XB) k_links_from_ref(const double *__restrict__ src, R *__restrict__ dst, long V, int ng) {
    __shared__ double sh[XB * XW];
    const long t0 = (long)blockIdx.x * XB;
    const int nl = (int)min((long)XB, 3 * V - t0);
    rows_in(src, t0, nl, ng, sh);
    __syncthreads();
    if ((int)threadIdx.x >= nl) return;
    const long t = t0 + threadIdx.x, s = t / 3;
    const int d = (int)(t - s * 3);
    for (int c = 0; c < ng; c++) dst[link_offset(V, ng, d, c, s)] = (R)sh[threadIdx.x * XW + c];
}

template <typename R>
__global__ void __launch_bounds__(XB) k_links_to_ref(const R *__restrict__ src, double *__restrict__ dst, long V, int ng) {
    __shared__ double sh[XB * XW];
    const long t0 = (long)blockIdx.x * XB;
    const int nl = (int)min((long)XB, 3 * V - t0);
    if ((int)threadIdx.x < nl) {
        const long t = t0 + threadIdx.x, s = t / 3;
        const int d = (int)(t - s * 3);
        for (int c = 0; c < ng; c++) sh[threadIdx.x * XW + c] = (double)src[link_offset(V, ng, d, c, s)];
    }
    __syncthreads();
    rows_out(dst, t0, nl, ng, sh);
}

// SU3AlgebraElement.get(j)
__device__ __forceinline__ void herm9_to_gen(const double *v, double *g) {
    const double s3 = 1.7320508075688772;
    g[0] = 2 * v[1];
    g[1] = 2 * v[3];
    g[2] = v[0] - v[4];
    g[3] = 2 * v[2];
    g[4] = 2 * v[6];
    g[5] = 2 * v[5];
    g[6] = 2 * v[7];
    g[7] = (v[0] + v[4] - 2 * v[8]) / s3;
}

// new SU3AlgebraElement(double[8]): set(j, value) for j = 0..7 from zero
__device__ __forceinline__ void gen_to_herm9(const double *g, double *v) {
    const double s3 = 1.7320508075688772;
    for (int k = 0; k < 9; k++) v[k] = 0.0;
    v[1] += g[0] / 2;
    v[3] += g[1] / 2;
    {
        double d = g[2] / 2;
        v[0] += d;
        v[4] -= d;
    }
    v[2] += g[3] / 2;
    v[6] += g[4] / 2;
    v[5] += g[5] / 2;
    v[7] += g[6] / 2;
    {
        double cur = (v[0] + v[4] - 2 * v[8]) / s3;
        double d = (g[7] - cur) / 2;
        v[0] += d / s3;
        v[4] += d / s3;
        v[8] -= 2 * d / s3;
    }
}

// host [V][ndir][na_host] -> device planes [ndir][NA][V]
template <typename R>
__global__ void __launch_bounds__(XB) k_alg_from_host(const double *__restrict__ src, R *__restrict__ dst, long V,
                                                      int ndir, int NA, int herm9) {
    __shared__ double sh[XB * XW];
    const long t0 = (long)blockIdx.x * XB;
    const int nr = (int)min((long)XB, V * ndir - t0);
    const int w = herm9 ? 9 : NA;
    rows_in(src, t0, nr, w, sh);
    __syncthreads();
    if ((int)threadIdx.x >= nr) return;
    const long t = t0 + threadIdx.x, s = t / ndir;
    const int d = (int)(t - s * ndir);
    const double *row = sh + threadIdx.x * XW;
    if (herm9) {
        double g[8];
        herm9_to_gen(row, g);
        for (int a = 0; a < 8; a++) dst[((long)d * 8 + a) * V + s] = (R)g[a];
    } else {
        for (int a = 0; a < NA; a++) dst[((long)d * NA + a) * V + s] = (R)row[a];
    }
}

template <typename R>
__global__ void __launch_bounds__(XB) k_alg_to_host(const R *__restrict__ src, double *__restrict__ dst, long V,
                                                    int ndir, int NA, int herm9) {
    __shared__ double sh[XB * XW];
    const long t0 = (long)blockIdx.x * XB;
    const int nr = (int)min((long)XB, V * ndir - t0);
    const int w = herm9 ? 9 : NA;
    if ((int)threadIdx.x < nr) {
        const long t = t0 + threadIdx.x, s = t / ndir;
        const int d = (int)(t - s * ndir);
        double *row = sh + threadIdx.x * XW;
        if (herm9) {
            double g[8];
            for (int a = 0; a < 8; a++) g[a] = (double)src[((long)d * 8 + a) * V + s];
            gen_to_herm9(g, row);
        } else {
            for (int a = 0; a < NA; a++) row[a] = (double)src[((long)d * NA + a) * V + s];
        }
    }
    __syncthreads();
    rows_out(dst, t0, nr, w, sh);
}

void launch_links_from_ref(Ctx &c, const double *src, void *dst) {
    const int B = XB;
    if (c.prec == OPX_F64) k_links_from_ref<double><<<grid_for(c.L.V * 3, B), B, 0, c.stream>>>(src, (double *)dst, c.L.V, c.ng);
    else k_links_from_ref<float><<<grid_for(c.L.V * 3, B), B, 0, c.stream>>>(src, (float *)dst, c.L.V, c.ng);
    c.launches++;
}

void launch_links_to_ref(Ctx &c, const void *src, double *dst) {
    const int B = XB;
    if (c.prec == OPX_F64) k_links_to_ref<double><<<grid_for(c.L.V * 3, B), B, 0, c.stream>>>((const double *)src, dst, c.L.V, c.ng);
    else k_links_to_ref<float><<<grid_for(c.L.V * 3, B), B, 0, c.stream>>>((const float *)src, dst, c.L.V, c.ng);
    c.launches++;
}

void launch_alg_from_host(Ctx &c, const double *src, void *dst, int ndir, int layout) {
    const int B = XB;
    const int herm9 = (c.nc == 3 && layout == OPX_LAYOUT_REF) ? 1 : 0;
    if (c.prec == OPX_F64) k_alg_from_host<double><<<grid_for(c.L.V * ndir, B), B, 0, c.stream>>>(src, (double *)dst, c.L.V, ndir, c.na, herm9);
    else k_alg_from_host<float><<<grid_for(c.L.V * ndir, B), B, 0, c.stream>>>(src, (float *)dst, c.L.V, ndir, c.na, herm9);
    c.launches++;
}

void launch_alg_to_host(Ctx &c, const void *src, double *dst, int ndir, int layout) {
    const int B = XB;
    const int herm9 = (c.nc == 3 && layout == OPX_LAYOUT_REF) ? 1 : 0;
    if (c.prec == OPX_F64) k_alg_to_host<double><<<grid_for(c.L.V * ndir, B), B, 0, c.stream>>>((const double *)src, dst, c.L.V, ndir, c.na, herm9);
    else k_alg_to_host<float><<<grid_for(c.L.V * ndir, B), B, 0, c.stream>>>((const float *)src, dst, c.L.V, ndir, c.na, herm9);
    c.launches++;
}

}  // namespace opx
