// ic_kernels.cu -- seeded synthetic initial conditions on the device.
//
// The reference has no Gauss-projecting initializer; the synthetic benchmark
// lattices need one.  Links U_i(x) = exp(i A_i^a(x) t_a) with A ~ N(0, sigma_a^2)
// per generator component, E_i^a(x) ~ N(0, sigma_e^2), then E is projected onto
// Gauss's law (Grid.getGaussConstraint, Grid.java:944-968) by conjugate
// gradients on the covariant Laplacian:
//     div(divT mu) = rho - div E,   E <- E + divT mu,
// (div E)(x)   = sum_i c_i [E_i(x) - Ad(U_i(x-i)^dagger) E_i(x-i)],
// (divT l)_i(x) = c_i [l(x) - Ad(U_i(x)) l(x+i)],  c_i = 1/(a_i g a_i),
// divT being the adjoint of div.  Everything here runs in FP64; an FP32 handle
// receives the rounded result.  The random numbers use the same counter-based
// recipe as the CPU oracle (splitmix64 finaliser, Box-Muller), so both sides
// draw the same A and E.
#include <vector>

#include "internal.h"
#include "ksum.cuh"

namespace opx {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double unif(uint64_t seed, uint64_t ctr) {
    uint64_t h = mix64(seed ^ mix64(ctr));
    return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
__device__ __forceinline__ double normal(uint64_t seed, uint64_t ctr) {
    double u1 = unif(seed, 2 * ctr), u2 = unif(seed, 2 * ctr + 1);
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

template <int NC>
__global__ void k_init_random(double *__restrict__ U, double *__restrict__ E, Lat L, uint64_t seed, double sa,
                              double se) {
    using G = typename GroupOf<NC, double>::T;
    constexpr int NA = G::NA;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;  // t = s*3 + d
    if (t >= L.V * 3) return;
    const long s = t / 3;
    const int d = (int)(t - s * 3);
    double A[NA], e[NA];
    const uint64_t baseA = 0ull << 40, baseE = 1ull << 40;
#pragma unroll
    for (int a = 0; a < NA; a++) {
        A[a] = sa * normal(seed, baseA + (uint64_t)(t * NA + a));
        e[a] = se * normal(seed, baseE + (uint64_t)(t * NA + a));
    }
    const LinkPlanes<G, double> Up{U, L.V};
    const AlgPlanes<NA, double> Ep{E, L.V};
    Up.store(d, s, G::expi(A));
    Ep.store(d, s, e);
}

template <int NC>
__global__ void k_div(const double *__restrict__ U, const double *__restrict__ El, Lat L, double *__restrict__ out) {
    using G = typename GroupOf<NC, double>::T;
    constexpr int NA = G::NA;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    const LinkPlanes<G, double> Up{const_cast<double *>(U), L.V};
    const AlgPlanes<NA, double> Ep{const_cast<double *>(El), L.V};
    int x[3];
    site_coords(L, s, x);
    const Nbr nb = neighbours(L, s, x);
    double acc[NA];
#pragma unroll
    for (int a = 0; a < NA; a++) acc[a] = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const double ci = 1.0 / (L.a[i] * L.g * L.a[i]);
        double e0[NA], e1[NA], t[NA];
        Ep.load_ro(i, s, e0);
        Ep.load_ro(i, nb.bwd[i], e1);
        G::act(e1, G::adj(Up.load(i, nb.bwd[i])), t);
#pragma unroll
        for (int a = 0; a < NA; a++) acc[a] += ci * (e0[a] - t[a]);
    }
    const AlgPlanes<NA, double> Op{out, L.V};
    Op.store(0, s, acc);
}

template <int NC>
__global__ void k_divT(const double *__restrict__ U, const double *__restrict__ l, Lat L, double *__restrict__ out,
                       int accumulate) {
    using G = typename GroupOf<NC, double>::T;
    constexpr int NA = G::NA;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    const LinkPlanes<G, double> Up{const_cast<double *>(U), L.V};
    const AlgPlanes<NA, double> Lp{const_cast<double *>(l), L.V};
    const AlgPlanes<NA, double> Op{out, L.V};
    int x[3];
    site_coords(L, s, x);
    const Nbr nb = neighbours(L, s, x);
    double l0[NA];
    Lp.load_ro(0, s, l0);
#pragma unroll
    for (int i = 0; i < 3; i++) {
        const double ci = 1.0 / (L.a[i] * L.g * L.a[i]);
        double l1[NA], t[NA], o[NA];
        Lp.load_ro(0, nb.fwd[i], l1);
        G::act(l1, Up.load(i, s), t);
        if (accumulate) Op.load(i, s, o);
#pragma unroll
        for (int a = 0; a < NA; a++) o[a] = (accumulate ? o[a] : 0.0) + ci * (l0[a] - t[a]);
        Op.store(i, s, o);
    }
}

__global__ void k_dot_partial(const double *__restrict__ a, const double *__restrict__ b, long n,
                              double *__restrict__ part) {
    KSum acc[1] = {{0.0, 0.0}};
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
        two_sum_add(acc[0], a[k] * b[k]);
    int q;
    KSum v = block_reduce<1>(acc, q);
    if (q == 0) { part[2 * blockIdx.x] = v.s; part[2 * blockIdx.x + 1] = v.c; }
}

__global__ void k_dot_final(const double *__restrict__ part, int nb, double *__restrict__ out) {
    if (threadIdx.x != 0) return;
    KSum v{0.0, 0.0};
    for (int b = 0; b < nb; b++) ksum_merge(v, KSum{part[2 * b], part[2 * b + 1]});
    *out = v.s + v.c;
}

// y = a*x + y ; optionally p = r + beta*p
__global__ void k_axpy(double *__restrict__ y, const double *__restrict__ x, double a, long n) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) y[k] += a * x[k];
}
__global__ void k_xpby(double *__restrict__ p, const double *__restrict__ r, double b, long n) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) p[k] = r[k] + b * p[k];
}
__global__ void k_sub_from(double *__restrict__ r, const double *__restrict__ rho, long n) {
    // r = rho - r (rho may be null)
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) r[k] = (rho ? rho[k] : 0.0) - r[k];
}
__global__ void k_to_float(const double *__restrict__ src, float *__restrict__ dst, long n) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dst[k] = (float)src[k];
}
__global__ void k_to_double(const float *__restrict__ src, double *__restrict__ dst, long n) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) dst[k] = (double)src[k];
}

struct Dot {
    Ctx &c;
    double *part = nullptr, *out = nullptr;
    int nb = 0;
    explicit Dot(Ctx &c_) : c(c_) {
        nb = 4 * 152;
        cudaMalloc(&part, sizeof(double) * 2 * nb);
        cudaMalloc(&out, sizeof(double));
    }
    ~Dot() { cudaFree(part); cudaFree(out); }
    double operator()(const double *a, const double *b, long n) {
        k_dot_partial<<<nb, 256, 0, c.stream>>>(a, b, n, part);
        k_dot_final<<<1, 32, 0, c.stream>>>(part, nb, out);
        c.launches += 2;
        double h = 0.0;
        cudaMemcpyAsync(&h, out, sizeof(double), cudaMemcpyDeviceToHost, c.stream);
        cudaStreamSynchronize(c.stream);
        return h;
    }
};

int ic_init_random(Ctx &c, uint64_t seed, double sigma_a, double sigma_e) {
    const long V = c.L.V;
    const size_t nU = (size_t)link_elems(V, c.ng), nE = (size_t)V * 3 * c.na;
    double *U64 = nullptr, *E64 = nullptr;
    const bool f32 = c.prec == OPX_F32;
    if (f32) {
        if (cudaMalloc(&U64, nU * 8) != cudaSuccess || cudaMalloc(&E64, nE * 8) != cudaSuccess) {
            cudaFree(U64);
            c.err = "opx_init_random: cannot allocate FP64 scratch";
            return OPX_ERR_NOMEM;
        }
    } else {
        U64 = (double *)c.U;
        E64 = (double *)c.E;
    }
    const int B = 256;
    if (c.nc == 2) k_init_random<2><<<grid_for(V * 3, B), B, 0, c.stream>>>(U64, E64, c.L, seed, sigma_a, sigma_e);
    else k_init_random<3><<<grid_for(V * 3, B), B, 0, c.stream>>>(U64, E64, c.L, seed, sigma_a, sigma_e);
    c.launches++;
    if (f32) {
        k_to_float<<<grid_for((long)nU, B), B, 0, c.stream>>>(U64, (float *)c.U, (long)nU);
        k_to_float<<<grid_for((long)nE, B), B, 0, c.stream>>>(E64, (float *)c.E, (long)nE);
        c.launches += 2;
        cudaStreamSynchronize(c.stream);
        cudaFree(U64);
        cudaFree(E64);
    }
    return OPX_OK;
}

// div and divT on FP64 fields with the FP64 links U64 (NA components per site)
void ic_div(Ctx &c, const double *U64, const double *El, double *o) {
    if (c.nc == 2) k_div<2><<<grid_for(c.L.V, 128), 128, 0, c.stream>>>(U64, El, c.L, o);
    else k_div<3><<<grid_for(c.L.V, 128), 128, 0, c.stream>>>(U64, El, c.L, o);
    c.launches++;
}
void ic_divT(Ctx &c, const double *U64, const double *l, double *o, int acc) {
    if (c.nc == 2) k_divT<2><<<grid_for(c.L.V, 128), 128, 0, c.stream>>>(U64, l, c.L, o, acc);
    else k_divT<3><<<grid_for(c.L.V, 128), 128, 0, c.stream>>>(U64, l, c.L, o, acc);
    c.launches++;
}

// x = K^+ b for the covariant Laplacian K = div divT of the links U64, by
// conjugate gradients from x = 0 until |r| <= tol_rel |b| (b in the range of
// div, so the iterates stay orthogonal to K's null space).
int ic_covariant_solve(Ctx &c, const double *U64, const double *b, double *x, double tol_rel, int maxit,
                       int *iters) {
    const long ns = c.L.V * c.na, nl = ns * 3;
    const int B = 256;
    std::vector<double *> bufs;
    auto alloc = [&](size_t n) -> double * {
        double *p = nullptr;
        if (cudaMalloc(&p, n * sizeof(double)) != cudaSuccess) return nullptr;
        bufs.push_back(p);
        return p;
    };
    double *r = alloc(ns), *p = alloc(ns), *Ap = alloc(ns), *tl = alloc(nl);
    if (!r || !p || !Ap || !tl) {
        for (double *q : bufs) cudaFree(q);
        cudaGetLastError();
        c.err = "covariant Laplacian solve: out of device memory";
        return OPX_ERR_NOMEM;
    }
    Dot dot(c);
    cudaMemsetAsync(x, 0, ns * sizeof(double), c.stream);
    cudaMemcpyAsync(r, b, ns * sizeof(double), cudaMemcpyDeviceToDevice, c.stream);
    cudaMemcpyAsync(p, b, ns * sizeof(double), cudaMemcpyDeviceToDevice, c.stream);
    double rr = dot(r, r, ns);
    const double stop = tol_rel * tol_rel * rr;
    int it = 0;
    while (it < maxit && rr > stop && rr > 0) {
        ic_divT(c, U64, p, tl, 0);
        ic_div(c, U64, tl, Ap);
        const double pAp = dot(p, Ap, ns);
        if (!(pAp > 0)) break;
        const double alpha = rr / pAp;
        k_axpy<<<grid_for(ns, B), B, 0, c.stream>>>(x, p, alpha, ns);
        k_axpy<<<grid_for(ns, B), B, 0, c.stream>>>(r, Ap, -alpha, ns);
        const double rr2 = dot(r, r, ns);
        k_xpby<<<grid_for(ns, B), B, 0, c.stream>>>(p, r, rr2 / rr, ns);
        c.launches += 3;
        rr = rr2;
        it++;
    }
    cudaError_t e = cudaStreamSynchronize(c.stream);
    for (double *q : bufs) cudaFree(q);
    if (iters) *iters = it;
    if (e != cudaSuccess) { c.err = std::string("covariant Laplacian solve: ") + cudaGetErrorString(e); return OPX_ERR_CUDA; }
    if (rr > stop && rr > 0) { c.err = "covariant Laplacian solve: no convergence"; return OPX_ERR_NUMERIC; }
    return OPX_OK;
}

int ic_gauss_project(Ctx &c, double tol, int maxit, int *iters, double *final_g2) {
    const long V = c.L.V;
    const int NA = c.na;
    const long ns = V * NA, nl = ns * 3;
    const size_t nU = (size_t)link_elems(V, c.ng);
    const bool f32 = c.prec == OPX_F32;
    std::vector<double *> bufs;
    auto alloc = [&](size_t n) -> double * {
        double *p = nullptr;
        if (cudaMalloc(&p, n * sizeof(double)) != cudaSuccess) return nullptr;
        bufs.push_back(p);
        return p;
    };
    auto release = [&]() { for (double *p : bufs) cudaFree(p); };
    double *U64, *E64, *rho64 = nullptr;
    const int B = 256;
    if (f32) {
        U64 = alloc(nU);
        E64 = alloc(nl);
        rho64 = alloc(ns);
        if (!U64 || !E64 || !rho64) { release(); c.err = "opx_gauss_project: out of device memory"; return OPX_ERR_NOMEM; }
        k_to_double<<<grid_for((long)nU, B), B, 0, c.stream>>>((const float *)c.U, U64, (long)nU);
        k_to_double<<<grid_for(nl, B), B, 0, c.stream>>>((const float *)c.E, E64, nl);
        k_to_double<<<grid_for(ns, B), B, 0, c.stream>>>((const float *)c.rho, rho64, ns);
        c.launches += 3;
    } else {
        U64 = (double *)c.U;
        E64 = (double *)c.E;
        rho64 = (double *)c.rho;
    }
    double *r = alloc(ns), *p = alloc(ns), *Ap = alloc(ns), *mu = alloc(ns), *tl = alloc(nl);
    if (!r || !p || !Ap || !mu || !tl) { release(); c.err = "opx_gauss_project: out of device memory"; return OPX_ERR_NOMEM; }
    Dot dot(c);
    auto div = [&](const double *El, double *o) {
        if (c.nc == 2) k_div<2><<<grid_for(V, 128), 128, 0, c.stream>>>(U64, El, c.L, o);
        else k_div<3><<<grid_for(V, 128), 128, 0, c.stream>>>(U64, El, c.L, o);
        c.launches++;
    };
    auto divT = [&](const double *l, double *o, int acc) {
        if (c.nc == 2) k_divT<2><<<grid_for(V, 128), 128, 0, c.stream>>>(U64, l, c.L, o, acc);
        else k_divT<3><<<grid_for(V, 128), 128, 0, c.stream>>>(U64, l, c.L, o, acc);
        c.launches++;
    };
    cudaMemsetAsync(mu, 0, ns * sizeof(double), c.stream);
    div(E64, r);
    k_sub_from<<<grid_for(ns, B), B, 0, c.stream>>>(r, rho64, ns);
    cudaMemcpyAsync(p, r, ns * sizeof(double), cudaMemcpyDeviceToDevice, c.stream);
    double rr = dot(r, r, ns);
    int it = 0;
    while (it < maxit && rr / V > tol * 1e-4) {
        divT(p, tl, 0);
        div(tl, Ap);
        double pAp = dot(p, Ap, ns);
        if (!(pAp > 0)) break;
        double alpha = rr / pAp;
        k_axpy<<<grid_for(ns, B), B, 0, c.stream>>>(mu, p, alpha, ns);
        k_axpy<<<grid_for(ns, B), B, 0, c.stream>>>(r, Ap, -alpha, ns);
        c.launches += 2;
        double rr2 = dot(r, r, ns);
        double beta = rr2 / rr;
        rr = rr2;
        k_xpby<<<grid_for(ns, B), B, 0, c.stream>>>(p, r, beta, ns);
        c.launches++;
        it++;
    }
    divT(mu, E64, 1);
    // final residual, recomputed from the projected field
    div(E64, r);
    k_sub_from<<<grid_for(ns, B), B, 0, c.stream>>>(r, rho64, ns);
    c.launches++;
    double g2 = dot(r, r, ns) / V;
    if (f32) {
        k_to_float<<<grid_for(nl, B), B, 0, c.stream>>>(E64, (float *)c.E, nl);
        c.launches++;
    }
    cudaError_t e = cudaStreamSynchronize(c.stream);
    release();
    if (iters) *iters = it;
    if (final_g2) *final_g2 = g2;
    if (e != cudaSuccess) { c.err = std::string("opx_gauss_project: ") + cudaGetErrorString(e); return OPX_ERR_CUDA; }
    return OPX_OK;
}

}  // namespace opx
