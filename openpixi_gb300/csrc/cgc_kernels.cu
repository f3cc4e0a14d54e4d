// cgc_kernels.cu -- colour-glass-condensate initial conditions (MV model) on the device.
//
// Restates physics/initial/CGC/CGCInitialCondition.java:55-93 for one MV
// nucleus at a time (a list of nuclei is applied in order, as the YAML list of
// MVModel entries is):
//   1. MVModel.initialize (physics/initial/CGC/MVModel.java:101-157): Gaussian
//      colour charges rho^a(x) ~ N(0, (g mu / sqrt(aL aT^2))^2) * sqrt(pdf(x_L)),
//      drawn from java.util.Random(seed) in site order per component (the
//      generator's published algorithm: 48-bit LCG, polar Gaussian; restated
//      on the host because the stream is sequential), then regulated in 3D
//      momentum space (FourierFunctions.regulateChargeDensityGaussian, :86-132)
//      and cut to the longitudinal window around the nucleus;
//   2. LightConePoissonSolverImproved.solve (:42-221): 2D Poisson solve per
//      longitudinal sheet in momentum space (FourierFunctions.solvePoisson2D,
//      :147-172), path-ordered Wilson lines V along the beam axis, links
//      U <- V U V^dagger(x+i), the improved Unext with M = 20 path-ordered
//      factors, E from the temporal plaquette (Grid.getEFromLinks, Grid.java:877-879)
//      and the Gauss violation of this nucleus alone;
//   3. LightConeNGPParticleCreator.initializeParticles (:110-235): round(aL/dt)
//      NGP particles per cell carrying the Gauss violation, refined by 100
//      second- and 100 fourth-order smoothing sweeps per transverse column.
// FFTs use cuFFT (double complex), loaded at run time so that the rest of the
// library does not depend on it.  Beam direction 0 (the particle creator of the
// reference assumes it too).
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include <cufft.h>

#include "fftlib.h"
#include "internal.h"
#include "java_random.h"
#include "ksum.cuh"

namespace opx {



// ---------------------------------------------------------------- kernels
// V = identity in the direction-0 slot of a link-shaped buffer
template <int NC>
__global__ void k_identity0(double *__restrict__ Vl, long V) {
    using G = typename GroupOf<NC, double>::T;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= V) return;
    const LinkPlanes<G, double> Vp{Vl, V};
    Vp.store(0, s, G::identity());
}

__global__ void k_to_complex(const double *__restrict__ r, cufftDoubleComplex *__restrict__ c, long n) {
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) c[k] = make_cuDoubleComplex(r[k], 0.0);
}

// FourierFunctions.regulateChargeDensityGaussian, momentum-space part
__global__ void k_regulate(cufftDoubleComplex *__restrict__ f, int n0, int n1, int n2, double UVT, double longWidth,
                           double IR, double aT, double aL) {
    const long V = (long)n0 * n1 * n2;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= V) return;
    const int z = (int)(s / ((long)n1 * n2)), t1 = (int)((s / n2) % n1), t2 = (int)(s % n2);
    if (s == 0) { f[0] = make_cuDoubleComplex(0.0, 0.0); return; }
    const double pi = 3.141592653589793;
    double kTeff2 = 4.0 - 2.0 * cos(2.0 * pi * t1 / n1) - 2.0 * cos(2.0 * pi * t2 / n2);
    kTeff2 /= aT * aT;
    double k1 = (t1 < n1 / 2) ? 2 * pi * t1 / (aT * n1) : 2 * pi * (n1 - t1) / (aT * n1);
    double k2 = (t2 < n2 / 2) ? 2 * pi * t2 / (aT * n2) : 2 * pi * (n2 - t2) / (aT * n2);
    const double kT2 = k1 * k1 + k2 * k2;
    const double delta = z / (double)n0;
    const double kL = fabs(delta < 0.5 ? 2.0 * delta * pi / aL : 2.0 * (delta - 1.0) * pi / aL);
    if (kT2 <= UVT * UVT && kT2 > 0) {
        const double reg = kTeff2 / (kTeff2 + IR * IR) * exp(-0.25 * kL * kL * longWidth * longWidth);
        f[s] = make_cuDoubleComplex(f[s].x * reg, f[s].y * reg);
    } else {
        f[s] = make_cuDoubleComplex(0.0, 0.0);
    }
}

// FourierFunctions.solvePoisson2D on every sheet (batch index = longitudinal z)
__global__ void k_poisson2d(cufftDoubleComplex *__restrict__ f, int n0, int n1, int n2, double aT) {
    const long V = (long)n0 * n1 * n2;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= V) return;
    const int t1 = (int)((s / n2) % n1), t2 = (int)(s % n2);
    if (t1 == 0 && t2 == 0) { f[s] = make_cuDoubleComplex(0.0, 0.0); return; }
    const double pi = 3.141592653589793;
    double kTeff2 = 4.0 - 2.0 * cos(2.0 * pi * t1 / n1) - 2.0 * cos(2.0 * pi * t2 / n2);
    kTeff2 /= aT * aT;
    f[s] = make_cuDoubleComplex(f[s].x * (1.0 / kTeff2), f[s].y * (1.0 / kTeff2));
}

// real part / N into component c of a generator-component field, optionally masked
__global__ void k_from_complex(const cufftDoubleComplex *__restrict__ f, double scale, double *__restrict__ out,
                               int comp, int ncomp, long V, int n0, int lmin, int lmax, const uint8_t *__restrict__ active) {
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= V) return;
    const int z = (int)(s / (V / n0));
    double v = f[s].x * scale;
    if (lmin >= 0) {
        const bool keep = lmin < z && z < lmax && (!active || active[s]);
        v = keep ? v : 0.0;
    }
    out[(long)comp * V + s] = v;
}

// Wilson lines V along the beam axis: one thread per transverse site, the scan
// runs over the longitudinal sheets in the order of LightConePoissonSolverImproved.solve.
template <int NC>
__global__ void k_wilson_scan(const double *__restrict__ phi, double *__restrict__ Vl, int n0, long ntr,
                              int orientation, double gaugeFactor) {
    using G = typename GroupOf<NC, double>::T;
    constexpr int NA = G::NA;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntr) return;
    const long V = (long)n0 * ntr;
    const LinkPlanes<G, double> Vp{Vl, V};  // direction slot 0 holds V
    // each sheet's V is the previous sheet's (kept in registers: the loads of
    // LinkPlanes go through the read-only cache, which must not see this
    // kernel's own stores) times one exponential; the first reads the identity
    const int z0 = orientation < 0 ? 0 : n0 - 1;
    auto prev = Vp.load(0, (long)(((z0 + orientation) % n0 + n0) % n0) * ntr + t);
    for (int k = 0; k < n0; k++) {
        const int z = orientation < 0 ? k : (n0 - k - 1);
        const long idx = (long)z * ntr + t;
        const int zl = ((z + orientation) % n0 + n0) % n0;
        const long idxL = (long)zl * ntr + t;
        const long src = orientation == -1 ? idxL : idx;
        double x[NA];
        for (int a = 0; a < NA; a++) x[a] = phi[(long)a * V + src] * gaugeFactor;
        prev = G::mul(prev, G::expi(x));
        Vp.store(0, idx, prev);
    }
}

// U_i(x) <- V(x) U_i(x) V(x+i)^dagger for the transverse directions; the copy holds V V^dagger(x+i)
template <int NC>
__global__ void k_gauge_links(const double *__restrict__ Vl, double *__restrict__ U, double *__restrict__ Uc, Lat L,
                              int direction) {
    using G = typename GroupOf<NC, double>::T;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    const LinkPlanes<G, double> Vp{const_cast<double *>(Vl), L.V}, Up{U, L.V}, Cp{Uc, L.V};
    int x[3];
    site_coords(L, s, x);
    const Nbr nb = neighbours(L, s, x);
    for (int d = 0; d < 3; d++) {
        // the copy's longitudinal links are the grid's own (Grid(Grid) copies every cell)
        if (d == direction) { Cp.store(d, s, Up.load(d, s)); continue; }
        const auto V1 = Vp.load(0, s), V2 = Vp.load(0, nb.fwd[d]);
        Up.store(d, s, G::mul_adj(G::mul(V1, Up.load(d, s)), V2));
        Cp.store(d, s, G::mul_adj(V1, V2));
    }
}

// V(x) <- V(x) prod_m exp(-g dt phi_m / M), phi_m linear between phi(x - L) and phi(x)
template <int NC>
__global__ void k_improved_w(const double *__restrict__ phi, double *__restrict__ Vl, Lat L, int direction,
                             int orientation, int M) {
    using G = typename GroupOf<NC, double>::T;
    constexpr int NA = G::NA;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    int x[3];
    site_coords(L, s, x);
    const Nbr nb = neighbours(L, s, x);
    const long is = nb.bwd[direction];
    const LinkPlanes<G, double> Vp{Vl, L.V};
    auto W = G::identity();
    for (int m = 0; m < M; m++) {
        const double z = (m + 0.5) / ((double)2 * M);
        const double FL = orientation == 1 ? z + 0.5 : -z + 0.5;
        const double FR = orientation == 1 ? -z + 0.5 : z + 0.5;
        double p[NA];
        for (int a = 0; a < NA; a++)
            p[a] = (phi[(long)a * L.V + is] * FL + phi[(long)a * L.V + s] * FR) * (-L.g * L.dt / (double)M);
        W = G::mul(W, G::expi(p));
    }
    Vp.store(0, s, G::mul(Vp.load(0, s), W));
}

// E_j(x) = proj(Unext_j(x) U_j(x)^dagger) (-1/dt) (Grid.getEFromLinks)
template <int NC>
__global__ void k_e_from_links(const double *__restrict__ U, const double *__restrict__ Un, double *__restrict__ E, Lat L) {
    using G = typename GroupOf<NC, double>::T;
    constexpr int NA = G::NA;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    const LinkPlanes<G, double> Up{const_cast<double *>(U), L.V}, Unp{const_cast<double *>(Un), L.V};
    const AlgPlanes<NA, double> Ep{E, L.V};
    for (int j = 0; j < 3; j++) {
        double e[NA];
        G::proj(G::mul_adj(Unp.load(j, s), Up.load(j, s)), e);
        for (int a = 0; a < NA; a++) e[a] *= -1.0 / L.dt;
        Ep.store(j, s, e);
    }
}

// Gauss violation of the nucleus alone (Grid.getGaussConstraint with rho = 0), 0 where inactive
template <int NC>
__global__ void k_gauss_copy(const double *__restrict__ Uc, const double *__restrict__ Ec, const uint8_t *__restrict__ active,
                             Lat L, double *__restrict__ Gout) {
    using G = typename GroupOf<NC, double>::T;
    constexpr int NA = G::NA;
    const long s = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.V) return;
    int x[3];
    site_coords(L, s, x);
    const Nbr nb = neighbours(L, s, x);
    const LinkPlanes<G, double> Up{const_cast<double *>(Uc), L.V};
    const AlgPlanes<NA, double> Ep{const_cast<double *>(Ec), L.V};
    double gs[NA];
    for (int a = 0; a < NA; a++) gs[a] = 0.0;
    if (!active || active[s]) {
        for (int i = 0; i < 3; i++) {
            double e0[NA], e1[NA], t[NA];
            Ep.load_ro(i, s, e0);
            Ep.load_ro(i, nb.bwd[i], e1);
            G::act(e1, G::adj(Up.load(i, nb.bwd[i])), t);
            const double f = 1.0 / (L.a[i] * (L.g * L.a[i]));
            for (int a = 0; a < NA; a++) gs[a] += (e0[a] - t[a]) * f;
        }
    }
    for (int a = 0; a < NA; a++) Gout[(long)a * L.V + s] = gs[a];
}

// max over the transverse sheet of |G| per longitudinal z
__global__ void k_sheet_max(const double *__restrict__ Gf, int NA, long V, long ntr, double *__restrict__ out) {
    const int z = blockIdx.x;
    __shared__ double sh[256];
    double m = 0.0;
    for (long t = threadIdx.x; t < ntr; t += blockDim.x) {
        const long s = (long)z * ntr + t;
        double q = 0.0;
        for (int a = 0; a < NA; a++) q += Gf[(long)a * V + s] * Gf[(long)a * V + s];
        m = fmax(m, sqrt(q));
    }
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[z] = sh[0];
}

// LightConeNGPParticleCreator.initializeParticles (:159-214): particle k of this
// nucleus, k = ((z - zStart) ntr + t) ppc + j, charge = G(ngp(pos0)) / ppc.
template <int NC>
__global__ void k_cgc_particles(const double *__restrict__ Gv, Lat L, int zStart, long ntr, int ppc, int direction,
                                int orientation, long np, double *__restrict__ pos0, double *__restrict__ pos1,
                                double *__restrict__ vel, double *__restrict__ q) {
    constexpr int NA = NC == 3 ? 8 : 3;
    constexpr int NAR = NC == 3 ? 9 : 3;
    const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= np) return;
    const int j = (int)(k % ppc);
    const long t = (k / ppc) % ntr;
    const int z = zStart + (int)(k / (ppc * ntr));
    const int pos[3] = {z, (int)(t / L.n[2]), (int)(t % L.n[2])};
    const double xr = (1.0 * j - ppc / 2) / ppc;
    const double dz = xr * L.a[direction];
    int g[3];
    for (int d = 0; d < 3; d++) {
        const double fix = 10E-12 * L.a[d];
        double p0 = pos[d] * L.a[d] + fix, p1 = pos[d] * L.a[d] + fix;
        if (d == direction) {
            p0 += 0.0 * orientation + dz;
            p1 += (0.0 + L.dt) * orientation + dz;
        }
        pos0[d * np + k] = p0;
        pos1[d * np + k] = p1;
        vel[d * np + k] = d == direction ? 1.0 * orientation : 0.0;
        g[d] = (int)rint(p0 / L.a[d]);
    }
    long ci = 0;
    for (int d = 0; d < 3; d++) {
        const long r = ((long)g[d] % L.n[d] + L.n[d]) % L.n[d];
        ci = d == 0 ? r : ci * L.n[d] + r;
    }
    double gen[NA], ref[NAR];
    for (int a = 0; a < NA; a++) gen[a] = Gv[(long)a * L.V + ci];
    if (NC == 3) {
        // generator components -> the reference's 9-entry layout (SU3AlgebraElement(double[8]))
        const double s3 = 1.7320508075688772;
        for (int a = 0; a < NAR; a++) ref[a] = 0.0;
        ref[1] += gen[0] / 2;
        ref[3] += gen[1] / 2;
        { const double dd = gen[2] / 2; ref[0] += dd; ref[4] -= dd; }
        ref[2] += gen[3] / 2;
        ref[6] += gen[4] / 2;
        ref[5] += gen[5] / 2;
        ref[7] += gen[6] / 2;
        { const double cur = (ref[0] + ref[4] - 2 * ref[8]) / s3; const double dd = (gen[NA - 1] - cur) / 2;
          ref[0] += dd / s3; ref[4] += dd / s3; ref[8] -= 2 * dd / s3; }
    } else {
        for (int a = 0; a < NAR; a++) ref[a] = gen[a];
    }
    for (int a = 0; a < NAR; a++) q[a * np + k] = ref[a] * (1.0 / ppc);
}

// refine2 / refine4 sweeps (:216-305), 100 each, one thread per transverse
// column; the column's list runs over z, then over the particles of a cell.
__global__ void k_cgc_refine(double *__restrict__ q, int nar, long np, long ntr, int ppc, int nz) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntr) return;
    const int n = nz * ppc;
    auto P = [&](int i) -> long {
        const int ii = ((i % n) + n) % n;
        return ((long)(ii / ppc) * ntr + t) * ppc + (ii % ppc);
    };
    for (int it = 0; it < 100; it++)
        for (int i = 0; i < n; i++) {
            const int jm = i % ppc;
            if (!(jm >= 0 && jm < ppc - 1)) continue;
            const long i0 = P(i - 1), i1 = P(i), i2 = P(i + 1), i3 = P(i + 2);
            for (int a = 0; a < nar; a++) {
                double DQ = q[a * np + i0] * -1;
                DQ += q[a * np + i1] * 3;
                DQ += q[a * np + i2] * -3;
                DQ += q[a * np + i3] * 1;
                DQ *= 1.0 / 4.0;
                q[a * np + i1] += DQ * -1.0;
                q[a * np + i2] += DQ * 1.0;
            }
        }
    for (int it = 0; it < 100; it++)
        for (int i = 0; i < n; i++) {
            const int jm = i % ppc;
            if (!(jm >= 0 && jm < ppc - 1)) continue;
            const long i0 = P(i - 2), i1 = P(i - 1), i2 = P(i), i3 = P(i + 1), i4 = P(i + 2), i5 = P(i + 3);
            for (int a = 0; a < nar; a++) {
                double DQ = q[a * np + i0] * 1;
                DQ += q[a * np + i1] * -5;
                DQ += q[a * np + i2] * 10;
                DQ += q[a * np + i3] * -10;
                DQ += q[a * np + i4] * 5;
                DQ += q[a * np + i5] * -1;
                DQ *= 1.0 / 12.0;
                q[a * np + i2] += DQ * -1.0;
                q[a * np + i3] += DQ * 1.0;
            }
        }
}

// LightConeNGPSuperParticleCreator.initializeParticles (:150-199): charge i of
// super particle k is G(ngp)/ppc with ngp = index (k < ppc/2) or index + one
// plane, index = base + i; stored as Q[k][a][i] in the reference layout.
template <int NC>
__global__ void k_super_init(const double *__restrict__ Gv, long V, long ntr, long base, long n, int ppc,
                             double *__restrict__ Q) {
    constexpr int NA = NC == 3 ? 8 : 3;
    constexpr int NAR = NC == 3 ? 9 : 3;
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long index = base + i;
    for (int k = 0; k < ppc; k++) {
        const long ngp = (k < ppc / 2) ? index : (index + ntr >= V ? index + ntr - V : index + ntr);
        double gen[NA], ref[NAR];
        for (int a = 0; a < NA; a++) gen[a] = Gv[(long)a * V + ngp];
        if (NC == 3) {
            const double s3 = 1.7320508075688772;
            for (int a = 0; a < NAR; a++) ref[a] = 0.0;
            ref[1] += gen[0] / 2;
            ref[3] += gen[1] / 2;
            { const double dd = gen[2] / 2; ref[0] += dd; ref[4] -= dd; }
            ref[2] += gen[3] / 2;
            ref[6] += gen[4] / 2;
            ref[5] += gen[5] / 2;
            ref[7] += gen[6] / 2;
            { const double cur = (ref[0] + ref[4] - 2 * ref[8]) / s3; const double dd = (gen[NA - 1] - cur) / 2;
              ref[0] += dd / s3; ref[4] += dd / s3; ref[8] -= 2 * dd / s3; }
        } else {
            for (int a = 0; a < NAR; a++) ref[a] = gen[a];
        }
        for (int a = 0; a < NAR; a++) Q[((long)k * NAR + a) * n + i] = ref[a] * (1.0 / ppc);
    }
}

// refine2 / refine4 (:200-302) on each transverse column's list: entry ii is
// charge (ii / ppc) * ntr + t of super particle ii % ppc; the sweeps skip
// entries with (ii + ppc/2) % ppc == ppc - 1.
__global__ void k_super_refine(double *__restrict__ Q, int nar, long n, long ntr, int ppc, long len) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntr || len <= 0) return;
    auto P = [&](long i, int a) -> double & {
        const long ii = ((i % len) + len) % len;
        return Q[((long)(ii % ppc) * nar + a) * n + (ii / ppc) * ntr + t];
    };
    for (int it = 0; it < 100; it++)
        for (long i = 0; i < len; i++) {
            const long jm = (i + ppc / 2) % ppc;
            if (!(jm >= 0 && jm < ppc - 1)) continue;
            for (int a = 0; a < nar; a++) {
                double DQ = P(i - 1, a) * -1;
                DQ += P(i, a) * 3;
                DQ += P(i + 1, a) * -3;
                DQ += P(i + 2, a) * 1;
                DQ *= 1.0 / 4.0;
                P(i, a) += DQ * -1.0;
                P(i + 1, a) += DQ * 1.0;
            }
        }
    for (int it = 0; it < 100; it++)
        for (long i = 0; i < len; i++) {
            const long jm = (i + ppc / 2) % ppc;
            if (!(jm >= 0 && jm < ppc - 1)) continue;
            for (int a = 0; a < nar; a++) {
                double DQ = P(i - 2, a) * 1;
                DQ += P(i - 1, a) * -5;
                DQ += P(i, a) * 10;
                DQ += P(i + 1, a) * -10;
                DQ += P(i + 2, a) * 5;
                DQ += P(i + 3, a) * -1;
                DQ *= 1.0 / 12.0;
                P(i, a) += DQ * -1.0;
                P(i + 1, a) += DQ * 1.0;
            }
        }
}

}  // namespace opx

using namespace opx;


// Host driver; returns the particles created for this nucleus (reference layout, host).
// ---- Wilson-line observables (physics/initial/CGC/WilsonLineObservables.java) ----

__device__ __forceinline__ void put_ref(const Q2<double> &m, double *o) {
    for (int k = 0; k < 4; k++) o[k] = m.e[k];
}
__device__ __forceinline__ void put_ref(const M3<double> &m, double *o) {
    for (int k = 0; k < 9; k++) { o[k] = m.r[k]; o[9 + k] = m.i[k]; }
}
// Re tr V (GroupElement.getRealTrace) and Re tr(A B^dagger) of reference-layout elements
template <int NC> __device__ __forceinline__ double retr(const double *a) {
    return NC == 2 ? 2.0 * a[0] : a[0] + a[4] + a[8];
}
template <int NC> __device__ __forceinline__ double retr_adj(const double *a, const double *b) {
    double s = 0.0;
    for (int k = 0; k < (NC == 2 ? 4 : 18); k++) s = fma(a[k], b[k], s);
    return NC == 2 ? 2.0 * s : s;
}

// VT: V at the longitudinal boundary behind the nucleus, z = 0 for orientation
// +1 and n0 - 1 for -1 (LightConePoissonSolverImproved.solve :125-136), taken
// before the improved links modify V
template <int NC>
__global__ void k_extract_vt(const double *__restrict__ Vl, double *__restrict__ vt, long V, long ntr, int zb) {
    using G = typename GroupOf<NC, double>::T;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntr) return;
    const LinkPlanes<G, double> Vp{const_cast<double *>(Vl), V};
    put_ref(Vp.load(0, (long)zb * ntr + t), vt + t * G::NG);
}

// WilsonLineObservables.computeTadpole (:37-59): one block, cells strided over
// the threads, a fixed-order block sum
template <int NC>
__global__ void k_tadpole(const double *__restrict__ vt, long ntr, double *__restrict__ out) {
    constexpr int NG = NC == 2 ? 4 : 18;
    KSum acc[1] = {{0.0, 0.0}};
    for (long t = threadIdx.x; t < ntr; t += blockDim.x) two_sum_add(acc[0], retr<NC>(vt + t * NG));
    int q;
    const KSum v = block_reduce<1>(acc, q);
    if (q == 0) out[0] = (v.s + v.c) / (double)ntr;
}

// WilsonLineObservables.computeDipole (:67-131): block i takes cell x_i against
// every cell y (threads stride over y); Re tr(V(x) V(y)^dagger) goes to the bin
// of the periodic transverse distance, exactly as the reference forms it
// (integer coordinate differences wrapped at n/2, sqrt, truncation by ds).
// Each thread keeps its own column of bins in shared memory; the block adds the
// columns in order into part[i][bin], and k_dipole_final adds the cells in order.
template <int NC>
__global__ void k_dipole(const double *__restrict__ vt, int n1, int n2, double a1, double a2, int nb, double ds,
                         double *__restrict__ part, long long *__restrict__ cnt) {
    constexpr int NG = NC == 2 ? 4 : 18;
    extern __shared__ double dsh[];  // [nb][blockDim] sums, then [nb][blockDim] counts
    const int B = blockDim.x, tid = threadIdx.x;
    double *sum = dsh;
    long long *num = reinterpret_cast<long long *>(dsh + (size_t)nb * B);
    for (int b = 0; b < nb; b++) { sum[b * B + tid] = 0.0; num[b * B + tid] = 0; }
    const long ntr = (long)n1 * n2, i = blockIdx.x;
    const int x0 = (int)(i / n2), x1 = (int)(i % n2);
    double vi[NG];
    for (int k = 0; k < NG; k++) vi[k] = vt[i * NG + k];
    for (long j = tid; j < ntr; j += B) {
        const int y0 = (int)(j / n2), y1 = (int)(j % n2);
        double d0 = fabs((double)(x0 - y0)), d1 = fabs((double)(x1 - y1));
        if (d0 > n1 / 2) d0 -= n1;
        if (d1 > n2 / 2) d1 -= n2;
        double dist = 0.0;
        dist += d0 * d0 * a1 * a1;
        dist += d1 * d1 * a2 * a2;
        dist = sqrt(dist);
        const int bin = (int)(dist / ds);
        if (bin < nb) {
            sum[bin * B + tid] += retr_adj<NC>(vi, vt + j * NG);
            num[bin * B + tid] += 1;
        }
    }
    __syncthreads();
    for (int b = tid; b < nb; b += B) {
        double s = 0.0;
        long long c = 0;
        for (int t = 0; t < B; t++) { s += sum[b * B + t]; c += num[b * B + t]; }
        part[i * nb + b] = s;
        cnt[i * nb + b] = c;
    }
}

__global__ void k_dipole_final(const double *__restrict__ part, const long long *__restrict__ cnt, long ntr, int nb,
                               double *__restrict__ out) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    KSum v{0.0, 0.0};
    long long c = 0;
    for (long i = 0; i < ntr; i++) { two_sum_add(v, part[i * nb + b]); c += cnt[i * nb + b]; }
    out[b] = (v.s + v.c) / (double)c;  // 0/0 = NaN for an empty bin, as in the reference
}

void opx::cgc_vt_free(Ctx &c) {
    for (double *p : c.cgc_vt) if (p) cudaFree(p);
    c.cgc_vt.clear();
}

static int cgc_nucleus(Ctx &c, const opx_mv_nucleus &nu, std::vector<double> &ppos0, std::vector<double> &ppos1,
                       std::vector<double> &pvel, std::vector<double> &pq, std::vector<int32_t> &pdir,
                       SuperGroup *sg) {
    const int n0 = c.L.n[0], n1 = c.L.n[1], n2 = c.L.n[2];
    const long V = c.L.V, ntr = (long)n1 * n2;
    const int NA = c.na, nc = c.nc;
    const int direction = nu.direction, orientation = nu.orientation;
    const double aL = c.L.a[direction], aT = c.L.a[(direction + 1) % 3];
    // device buffers
    double *rho = nullptr, *phi = nullptr, *Vl = nullptr, *Uc = nullptr, *Unc = nullptr, *Ec = nullptr, *Gv = nullptr,
           *smax = nullptr;
    cufftDoubleComplex *f = nullptr;
    const size_t nU = (size_t)link_elems(V, c.ng);
    bool ok = true;
    auto al = [&](void **p, size_t b) { if (ok && cudaMalloc(p, b) != cudaSuccess) { ok = false; *p = nullptr; } };
    al((void **)&rho, sizeof(double) * NA * V);
    al((void **)&phi, sizeof(double) * NA * V);
    al((void **)&f, sizeof(cufftDoubleComplex) * V);
    al((void **)&Vl, sizeof(double) * nU);
    al((void **)&Uc, sizeof(double) * nU);
    al((void **)&Unc, sizeof(double) * nU);
    al((void **)&Ec, sizeof(double) * 3 * NA * V);
    al((void **)&Gv, sizeof(double) * NA * V);
    al((void **)&smax, sizeof(double) * n0);
    double *vt = nullptr;  // kept on the handle for opx_cgc_wilson_lines
    al((void **)&vt, sizeof(double) * ntr * c.ng);
    if (vt) c.cgc_vt.push_back(vt);
    int rc = OPX_OK;
    FFTPlan p3, p2;
    if (ok) {
        int dims3[3] = {n0, n1, n2}, dims2[2] = {n1, n2};
        p3.make(3, dims3, 1, c.stream);
        p2.make(2, dims2, n0, c.stream);
    }
    if (!ok || !p3.ok || !p2.ok) {
        c.err = "opx_cgc_mv: out of device memory or cuFFT plan failure";
        rc = OPX_ERR_NOMEM;
    }
    const int B = 256;
    if (!rc) {
        // 1. MV charges (host random stream, MVModel.java:114-131)
        JavaRandom rand((int64_t)nu.seed);
        const double width = nu.mu * c.L.g / std::sqrt(aL * aT * aT);
        // org.apache.commons.math3.analysis.function.Gaussian(mean, sigma).value:
        // norm * exp(-d * d * i2s2), norm = 1/(sigma sqrt(2 pi)), i2s2 = 0.5 (1/sigma)^2
        const double norm = 1.0 / (nu.width * std::sqrt(2.0 * 3.141592653589793));
        const double is = 1.0 / nu.width, i2s2 = 0.5 * is * is;
        std::vector<double> tmp(V);
        const double box = n0 * aL;
        const double zmin = std::max(nu.location - box / 2.0, 0.0), zmax = std::min(nu.location + box / 2.0, box);
        const int lmin = (int)std::floor(zmin / aL), lmax = (int)std::ceil(zmax / aL);
        for (int comp = 0; comp < NA && !rc; comp++) {
            for (long s = 0; s < V; s++) {
                const int z = (int)(s / ntr);
                const double d = z * aL - nu.location;
                const double profile = std::sqrt(norm * std::exp(-d * d * i2s2));
                tmp[s] = rand.next_gaussian() * width * profile;
            }
            cudaMemcpyAsync(phi, tmp.data(), sizeof(double) * V, cudaMemcpyHostToDevice, c.stream);
            k_to_complex<<<grid_for(V, B), B, 0, c.stream>>>(phi, f, V);
            if (fft_lib().execZ2Z(p3.h, f, f, CUFFT_FORWARD) != CUFFT_SUCCESS) rc = OPX_ERR_CUDA;
            k_regulate<<<grid_for(V, B), B, 0, c.stream>>>(f, n0, n1, n2, nu.uvt, nu.coherence, nu.ir, aT, aL);
            if (fft_lib().execZ2Z(p3.h, f, f, CUFFT_INVERSE) != CUFFT_SUCCESS) rc = OPX_ERR_CUDA;
            k_from_complex<<<grid_for(V, B), B, 0, c.stream>>>(f, 1.0 / V, rho, comp, NA, V, n0, lmin, lmax, c.active);
            cudaStreamSynchronize(c.stream);
            c.launches += 4;
        }
        // 2. Poisson 2D per sheet (LightConePoissonSolverImproved.java:69-95)
        for (int comp = 0; comp < NA && !rc; comp++) {
            k_to_complex<<<grid_for(V, B), B, 0, c.stream>>>(rho + (long)comp * V, f, V);
            if (fft_lib().execZ2Z(p2.h, f, f, CUFFT_FORWARD) != CUFFT_SUCCESS) rc = OPX_ERR_CUDA;
            k_poisson2d<<<grid_for(V, B), B, 0, c.stream>>>(f, n0, n1, n2, aT);
            if (fft_lib().execZ2Z(p2.h, f, f, CUFFT_INVERSE) != CUFFT_SUCCESS) rc = OPX_ERR_CUDA;
            k_from_complex<<<grid_for(V, B), B, 0, c.stream>>>(f, 1.0 / ntr, phi, comp, NA, V, n0, -1, -1, nullptr);
            c.launches += 4;
        }
        if (rc) c.err = "opx_cgc_mv: cuFFT execution failed";
    }
    if (!rc) {
        // 3. Wilson lines, links, improved Unext, E, Gauss violation
        const Lat L = c.L;
        if (nc == 2) {
            k_identity0<2><<<grid_for(V, 128), 128, 0, c.stream>>>(Vl, V);
            k_wilson_scan<2><<<grid_for(ntr, 128), 128, 0, c.stream>>>(phi, Vl, n0, ntr, orientation, -L.g * aL);
            if (vt) k_extract_vt<2><<<grid_for(ntr, 128), 128, 0, c.stream>>>(Vl, vt, V, ntr, orientation > 0 ? 0 : n0 - 1);
            k_gauge_links<2><<<grid_for(V, 128), 128, 0, c.stream>>>(Vl, (double *)c.U, Uc, L, direction);
            k_improved_w<2><<<grid_for(V, 128), 128, 0, c.stream>>>(phi, Vl, L, direction, orientation, 20);
            k_gauge_links<2><<<grid_for(V, 128), 128, 0, c.stream>>>(Vl, (double *)c.Unext, Unc, L, direction);
            k_e_from_links<2><<<grid_for(V, 128), 128, 0, c.stream>>>((double *)c.U, (double *)c.Unext, (double *)c.E, L);
            k_e_from_links<2><<<grid_for(V, 128), 128, 0, c.stream>>>(Uc, Unc, Ec, L);
            k_gauss_copy<2><<<grid_for(V, 128), 128, 0, c.stream>>>(Uc, Ec, c.active, L, Gv);
        } else {
            k_identity0<3><<<grid_for(V, 128), 128, 0, c.stream>>>(Vl, V);
            k_wilson_scan<3><<<grid_for(ntr, 128), 128, 0, c.stream>>>(phi, Vl, n0, ntr, orientation, -L.g * aL);
            if (vt) k_extract_vt<3><<<grid_for(ntr, 128), 128, 0, c.stream>>>(Vl, vt, V, ntr, orientation > 0 ? 0 : n0 - 1);
            k_gauge_links<3><<<grid_for(V, 128), 128, 0, c.stream>>>(Vl, (double *)c.U, Uc, L, direction);
            k_improved_w<3><<<grid_for(V, 128), 128, 0, c.stream>>>(phi, Vl, L, direction, orientation, 20);
            k_gauge_links<3><<<grid_for(V, 128), 128, 0, c.stream>>>(Vl, (double *)c.Unext, Unc, L, direction);
            k_e_from_links<3><<<grid_for(V, 128), 128, 0, c.stream>>>((double *)c.U, (double *)c.Unext, (double *)c.E, L);
            k_e_from_links<3><<<grid_for(V, 128), 128, 0, c.stream>>>(Uc, Unc, Ec, L);
            k_gauss_copy<3><<<grid_for(V, 128), 128, 0, c.stream>>>(Uc, Ec, c.active, L, Gv);
        }
        k_sheet_max<<<n0, 256, 0, c.stream>>>(Gv, NA, V, ntr, smax);
        c.launches += 8;
    }
    std::vector<double> mx(n0);
    if (!rc) {
        cudaMemcpyAsync(mx.data(), smax, sizeof(double) * n0, cudaMemcpyDeviceToHost, c.stream);
        cudaError_t e = cudaStreamSynchronize(c.stream);
        if (e != cudaSuccess) { c.err = std::string("opx_cgc_mv: ") + cudaGetErrorString(e); rc = OPX_ERR_CUDA; }
    }
    // 4b. super particles (LightConeNGPSuperParticleCreator.initializeParticles, :102-241)
    if (!rc && sg) {
        const int ppc = (int)std::lround(aL / c.L.dt);
        double gmax = 0.0;
        for (int z = 0; z < n0; z++) gmax = std::max(gmax, mx[z]);
        const double cutoff = gmax * 10E-10;
        int zStart = 0, zEnd = n0 - 1;
        for (int z = 0; z < n0; z++) if (mx[z] > cutoff) { zStart = z; break; }
        for (int z = zEnd - 1; z >= 0; z--) if (mx[z] > cutoff) { zEnd = z; break; }
        const long n = (long)(zEnd - zStart) * ntr;
        const int nar = c.na_ref;
        sg->orientation = orientation;
        sg->base = (long)zStart * ntr;
        sg->n = n;
        sg->Q = nullptr;
        if (ppc < 1) {
            c.err = "opx_cgc_mv_super: round(aL/dt) particles per cell must be >= 1";
            rc = OPX_ERR_INVALID;
        } else if (n > 0 && cudaMalloc(&sg->Q, sizeof(double) * (size_t)ppc * nar * n) != cudaSuccess) {
            cudaGetLastError();
            sg->Q = nullptr;
            c.err = "opx_cgc_mv_super: out of device memory";
            rc = OPX_ERR_NOMEM;
        } else if (n > 0) {
            if (nc == 2) k_super_init<2><<<grid_for(n, 128), 128, 0, c.stream>>>(Gv, V, ntr, sg->base, n, ppc, sg->Q);
            else k_super_init<3><<<grid_for(n, 128), 128, 0, c.stream>>>(Gv, V, ntr, sg->base, n, ppc, sg->Q);
            k_super_refine<<<grid_for(ntr, 64), 64, 0, c.stream>>>(sg->Q, nar, n, ntr, ppc, (long)(zEnd - zStart) * ppc);
            c.launches += 2;
            cudaError_t e = cudaStreamSynchronize(c.stream);
            if (e != cudaSuccess) { c.err = std::string("opx_cgc_mv_super: ") + cudaGetErrorString(e); rc = OPX_ERR_CUDA; }
        }
    }
    // 4. particles (LightConeNGPParticleCreator.initializeParticles, :110-235)
    if (!rc && !sg) {
        const int ppc = (int)std::lround(aL / c.L.dt);
        double gmax = 0.0;
        for (int z = 0; z < n0; z++) gmax = std::max(gmax, mx[z]);
        const double cutoff = gmax * 10E-10;
        int zStart = 0, zEnd = n0 - 1;
        for (int z = 0; z < n0; z++) if (mx[z] > cutoff) { zStart = z; break; }
        for (int z = zEnd - 1; z >= 0; z--) if (mx[z] > cutoff) { zEnd = z; break; }
        const int nar = c.na_ref, nz = zEnd - zStart + 1;
        const long np = (long)nz * ntr * ppc;
        double *d0 = nullptr, *d1 = nullptr, *dv = nullptr, *dq = nullptr;
        bool ok2 = cudaMalloc(&d0, sizeof(double) * 3 * np) == cudaSuccess && cudaMalloc(&d1, sizeof(double) * 3 * np) == cudaSuccess &&
                   cudaMalloc(&dv, sizeof(double) * 3 * np) == cudaSuccess && cudaMalloc(&dq, sizeof(double) * nar * np) == cudaSuccess;
        if (!ok2 || ppc < 1) {
            cudaGetLastError();
            c.err = ppc < 1 ? "opx_cgc_mv: round(aL/dt) particles per cell must be >= 1" : "opx_cgc_mv: out of device memory";
            rc = ppc < 1 ? OPX_ERR_INVALID : OPX_ERR_NOMEM;
        } else {
            if (nc == 2) k_cgc_particles<2><<<grid_for(np, 128), 128, 0, c.stream>>>(Gv, c.L, zStart, ntr, ppc, direction, orientation, np, d0, d1, dv, dq);
            else k_cgc_particles<3><<<grid_for(np, 128), 128, 0, c.stream>>>(Gv, c.L, zStart, ntr, ppc, direction, orientation, np, d0, d1, dv, dq);
            k_cgc_refine<<<grid_for(ntr, 64), 64, 0, c.stream>>>(dq, nar, np, ntr, ppc, nz);
            c.launches += 2;
            // append to the host-side list (reference per-particle layout)
            std::vector<double> h0(3 * np), h1(3 * np), hv(3 * np), hq(nar * np);
            cudaMemcpyAsync(h0.data(), d0, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost, c.stream);
            cudaMemcpyAsync(h1.data(), d1, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost, c.stream);
            cudaMemcpyAsync(hv.data(), dv, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost, c.stream);
            cudaMemcpyAsync(hq.data(), dq, sizeof(double) * nar * np, cudaMemcpyDeviceToHost, c.stream);
            cudaError_t e = cudaStreamSynchronize(c.stream);
            if (e != cudaSuccess) { c.err = std::string("opx_cgc_mv: ") + cudaGetErrorString(e); rc = OPX_ERR_CUDA; }
            const long first = (long)pdir.size();
            ppos0.resize((first + np) * 3);
            ppos1.resize((first + np) * 3);
            pvel.resize((first + np) * 3);
            pq.resize((first + np) * nar);
            pdir.resize(first + np, direction);
            for (long k = 0; k < np; k++) {
                for (int d = 0; d < 3; d++) {
                    ppos0[(first + k) * 3 + d] = h0[d * np + k];
                    ppos1[(first + k) * 3 + d] = h1[d * np + k];
                    pvel[(first + k) * 3 + d] = hv[d * np + k];
                }
                for (int a = 0; a < nar; a++) pq[(first + k) * nar + a] = hq[a * np + k];
            }
        }
        if (d0) cudaFree(d0);
        if (d1) cudaFree(d1);
        if (dv) cudaFree(dv);
        if (dq) cudaFree(dq);
    }
    void *bufs[] = {rho, phi, f, Vl, Uc, Unc, Ec, Gv, smax};
    for (void *b : bufs) if (b) cudaFree(b);
    return rc;
}

extern "C" int opx_cgc_mv(opx_ctx *ctx, const opx_mv_nucleus *nuclei, int n) {
    if (!ctx || !nuclei || n < 1) return OPX_ERR_INVALID;
    Ctx &c = ctx_of(ctx);
    if (c.prec != OPX_F64) { c.err = "opx_cgc_mv: CGC initial conditions need an OPX_F64 handle"; return OPX_ERR_UNSUPPORTED; }
    for (int q = 0; q < n; q++) {
        if (nuclei[q].direction != 0) { c.err = "opx_cgc_mv: the beam must run along direction 0"; return OPX_ERR_UNSUPPORTED; }
        if (nuclei[q].orientation != 1 && nuclei[q].orientation != -1) { c.err = "opx_cgc_mv: orientation must be +1 or -1"; return OPX_ERR_INVALID; }
        if (!(nuclei[q].width > 0) || !(nuclei[q].uvt >= 0)) { c.err = "opx_cgc_mv: width must be > 0 and the UV cutoff >= 0"; return OPX_ERR_INVALID; }
    }
    if (!fft_lib().load(c.err)) return OPX_ERR_UNSUPPORTED;
    if (!c.sg.empty()) { c.err = "opx_cgc_mv: the handle holds super particles (optimized CGC type)"; return OPX_ERR_INVALID; }
    cudaStreamSynchronize(c.stream);
    cgc_vt_free(c);
    // particles already on the handle stay first in the list (s.particles.add appends)
    const long n0 = c.P.n;
    const int nar = c.na_ref;
    std::vector<double> p0(3 * n0), p1(3 * n0), v(3 * n0), q0((size_t)nar * n0), q1((size_t)nar * n0);
    std::vector<int32_t> d(n0);
    if (n0 > 0) {
        opx_particles cur{n0, p0.data(), p1.data(), v.data(), q0.data(), q1.data(), d.data(), nullptr};
        int rc = opx_particles_download(ctx, &cur);
        if (rc) return rc;
    }
    for (int k = 0; k < n; k++) {
        opx_mv_nucleus nu = nuclei[k];
        // MVModel without randomSeed draws from an unseeded java.util.Random
        if (!nu.use_seed) nu.seed = (int)std::random_device{}();
        int rc = cgc_nucleus(c, nu, p0, p1, v, q0, d, nullptr);
        if (rc) return rc;
    }
    // Q1 = Q0 for the new particles (LightConeNGPParticleCreator.java:229-234)
    q1.insert(q1.end(), q0.begin() + (size_t)nar * n0, q0.end());
    opx_particles P{(long)d.size(), p0.data(), p1.data(), v.data(), q0.data(), q1.data(), d.data(), nullptr};
    return opx_particles_upload(ctx, &P);
}

extern "C" int opx_cgc_mv_super(opx_ctx *ctx, const opx_mv_nucleus *nuclei, int n) {
    if (!ctx || !nuclei || n < 1) return OPX_ERR_INVALID;
    Ctx &c = ctx_of(ctx);
    if (c.prec != OPX_F64) { c.err = "opx_cgc_mv_super: CGC initial conditions need an OPX_F64 handle"; return OPX_ERR_UNSUPPORTED; }
    if (c.P.n > 0) { c.err = "opx_cgc_mv_super: the handle holds NGP particles (cgc ngp type)"; return OPX_ERR_INVALID; }
    for (int q = 0; q < n; q++) {
        if (nuclei[q].direction != 0) { c.err = "opx_cgc_mv_super: the beam must run along direction 0"; return OPX_ERR_UNSUPPORTED; }
        if (nuclei[q].orientation != 1 && nuclei[q].orientation != -1) { c.err = "opx_cgc_mv_super: orientation must be +1 or -1"; return OPX_ERR_INVALID; }
        if (!(nuclei[q].width > 0) || !(nuclei[q].uvt >= 0)) { c.err = "opx_cgc_mv_super: width must be > 0 and the UV cutoff >= 0"; return OPX_ERR_INVALID; }
    }
    if ((int)c.sg.size() + n > 32) { c.err = "opx_cgc_mv_super: at most 32 nuclei"; return OPX_ERR_INVALID; }
    if (!fft_lib().load(c.err)) return OPX_ERR_UNSUPPORTED;
    const int ppc = (int)std::lround(c.L.a[0] / c.L.dt);
    if (ppc < 1 || (int)(c.sg.size() + n) * ppc > 64) {
        c.err = "opx_cgc_mv_super: round(aL/dt) must be >= 1 and nuclei x round(aL/dt) <= 64";
        return OPX_ERR_INVALID;
    }
    std::vector<double> p0, p1, v, q0;
    std::vector<int32_t> d;
    cudaStreamSynchronize(c.stream);
    cgc_vt_free(c);
    for (int k = 0; k < n; k++) {
        opx_mv_nucleus nu = nuclei[k];
        if (!nu.use_seed) nu.seed = (int)std::random_device{}();
        SuperGroup G;
        int rc = cgc_nucleus(c, nu, p0, p1, v, q0, d, &G);
        if (rc) { if (G.Q) cudaFree(G.Q); return rc; }
        c.sg.push_back(G);
    }
    c.sg_ppc = ppc;
    return OPX_OK;
}

extern "C" int opx_cgc_wilson_lines(opx_ctx *ctx, int nucleus, double *tadpole, double *dipole, size_t nbins,
                                    double *bin_width) {
    if (!ctx) return OPX_ERR_INVALID;
    Ctx &c = ctx_of(ctx);
    if (nucleus < 0 || nucleus >= (int)c.cgc_vt.size()) {
        c.err = "opx_cgc_wilson_lines: no such nucleus in the last CGC initial condition";
        return OPX_ERR_INVALID;
    }
    const int n1 = c.L.n[1], n2 = c.L.n[2];
    const long ntr = (long)n1 * n2;
    const int nb = (int)std::sqrt((double)ntr) / 2;
    if (dipole && nbins != (size_t)nb) {
        c.err = "opx_cgc_wilson_lines: the dipole has (int) sqrt(n1 n2) / 2 = " + std::to_string(nb) + " bins";
        return OPX_ERR_INVALID;
    }
    const double *vt = c.cgc_vt[nucleus];
    double *dev = nullptr;
    double *part = nullptr;
    long long *cnt = nullptr;
    const size_t nout = 1 + (dipole ? (size_t)nb : 0);
    bool ok = cudaMalloc(&dev, sizeof(double) * nout) == cudaSuccess;
    const double a1 = c.L.a[1], a2 = c.L.a[2];
    const double ds = std::min(n1 * a1, n2 * a2) * 0.5 / (double)nb;
    const int B = 64;
    const size_t smem = (size_t)nb * B * (sizeof(double) + sizeof(long long));
    if (dipole && nb > 0) {
        ok = ok && cudaMalloc(&part, sizeof(double) * ntr * nb) == cudaSuccess;
        ok = ok && cudaMalloc(&cnt, sizeof(long long) * ntr * nb) == cudaSuccess;
        if (smem > 200 * 1024) ok = false;
    }
    if (!ok) {
        cudaGetLastError();
        if (dev) cudaFree(dev);
        if (part) cudaFree(part);
        if (cnt) cudaFree(cnt);
        c.err = "opx_cgc_wilson_lines: out of device memory (or too many dipole bins for shared memory)";
        return OPX_ERR_NOMEM;
    }
    if (c.nc == 2) k_tadpole<2><<<1, 256, 0, c.stream>>>(vt, ntr, dev);
    else k_tadpole<3><<<1, 256, 0, c.stream>>>(vt, ntr, dev);
    c.launches++;
    if (dipole && nb > 0) {
        if (c.nc == 2) {
            cudaFuncSetAttribute(k_dipole<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            k_dipole<2><<<(unsigned)ntr, B, smem, c.stream>>>(vt, n1, n2, a1, a2, nb, ds, part, cnt);
        } else {
            cudaFuncSetAttribute(k_dipole<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            k_dipole<3><<<(unsigned)ntr, B, smem, c.stream>>>(vt, n1, n2, a1, a2, nb, ds, part, cnt);
        }
        k_dipole_final<<<grid_for(nb, 128), 128, 0, c.stream>>>(part, cnt, ntr, nb, dev + 1);
        c.launches += 2;
    }
    std::vector<double> host(nout);
    cudaMemcpyAsync(host.data(), dev, sizeof(double) * nout, cudaMemcpyDeviceToHost, c.stream);
    cudaError_t e = cudaStreamSynchronize(c.stream);
    cudaFree(dev);
    if (part) cudaFree(part);
    if (cnt) cudaFree(cnt);
    if (e != cudaSuccess) { c.err = std::string("opx_cgc_wilson_lines: ") + cudaGetErrorString(e); return OPX_ERR_CUDA; }
    if (tadpole) *tadpole = host[0];
    if (dipole) for (int b = 0; b < nb; b++) dipole[b] = host[1 + b];
    if (bin_width) *bin_width = ds;
    return OPX_OK;
}
