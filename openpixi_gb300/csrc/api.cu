// api.cu -- the C ABI of libopixi_gpu.so (declared in include/opixi.h).
//
// A handle is one lattice on one GPU with its own CUDA stream: the device
// counterpart of physics/grid/Grid.java plus the FastTYMSolver selected by
// physics/Settings.java:540-581, the CGC particle list and the diagnostics.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <cstdlib>

#include "internal.h"

using namespace opx;

struct opx_ctx {
    Ctx c;
};

static std::string g_create_error;

Ctx &opx::ctx_of(opx_ctx *h) {
    h->c.api_calls++;
    return h->c;
}

// API_CHECK for entry points that may change the fields or the masks (counted,
// so that the B^2 reuse of opx_reduce sees them); API_CHECK_RO for the ones
// that only read.
#define API_CHECK(ctx)                                   \
    do {                                                 \
        if (!(ctx)) return OPX_ERR_INVALID;              \
        (ctx)->c.api_calls++;                            \
    } while (0)
#define API_CHECK_RO(ctx)                                \
    do {                                                 \
        if (!(ctx)) return OPX_ERR_INVALID;              \
    } while (0)

static int cuda_fail(Ctx &c, const char *where, cudaError_t e) {
    c.err = std::string(where) + ": " + cudaGetErrorString(e);
    return OPX_ERR_CUDA;
}

// Check for launch errors of the work queued so far (cheap, no sync).
static int check_launch(Ctx &c, const char *where) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(c, where, e);
    return OPX_OK;
}

static int sync_check(Ctx &c, const char *where) {
    cudaError_t e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return cuda_fail(c, where, e);
    return check_launch(c, where);
}

template <typename R>
__global__ void k_fill_identity(R *U, long V, int ng, int nc) {
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;  // over the blocked link array
    if (t >= link_elems(V, ng)) return;
    // component index of element t in the link layout (lattice.cuh)
    const int c = ng == 4 ? (int)(t & 3) : (int)((t >> 5) % ng);
    const bool one = nc == 3 ? (c == 0 || c == 4 || c == 8) : (c == 0);
    U[t] = one ? R(1) : R(0);
}

static void fill_identity(Ctx &c, void *U) {
    const long n = link_elems(c.L.V, c.ng);
    if (c.prec == OPX_F64) k_fill_identity<double><<<grid_for(n, 256), 256, 0, c.stream>>>((double *)U, c.L.V, c.ng, c.nc);
    else k_fill_identity<float><<<grid_for(n, 256), 256, 0, c.stream>>>((float *)U, c.L.V, c.ng, c.nc);
    c.launches++;
}

static void release(Ctx &c) {
    cpic_free(c);
    super_free(c);
    cgc_vt_free(c);
    void *dev[] = {c.U, c.Unext, c.E, c.J, c.rho, c.active, c.eval, c.staging, c.red_part, c.red_out, c.red_count, c.status,
                   c.imp_Ua, c.imp_Ub, c.imp_E, c.E_alt, c.W_in, c.W_out, c.meas_part, c.meas_rows, c.bn_site};
    for (void *p : dev) if (p) cudaFree(p);
    if (c.red_host) cudaFreeHost(c.red_host);
    if (c.meas_host) cudaFreeHost(c.meas_host);
    if (c.status_host) cudaFreeHost(c.status_host);
    if (c.ev0) cudaEventDestroy(c.ev0);
    if (c.ev1) cudaEventDestroy(c.ev1);
    if (c.stream) cudaStreamDestroy(c.stream);
}

extern "C" {

int opx_version(void) { return 10000; }

const char *opx_last_error(const opx_ctx *ctx) {
    if (!ctx) return g_create_error.c_str();
    return ctx->c.err.c_str();
}

int opx_create(const opx_config *cfg, opx_ctx **out) {
    if (!cfg || !out) { g_create_error = "opx_create: null argument"; return OPX_ERR_INVALID; }
    *out = nullptr;
    if (cfg->ncolors != 2 && cfg->ncolors != 3) { g_create_error = "opx_create: ncolors must be 2 or 3"; return OPX_ERR_INVALID; }
    if (cfg->precision != OPX_F64 && cfg->precision != OPX_F32) { g_create_error = "opx_create: precision must be OPX_F64 or OPX_F32"; return OPX_ERR_INVALID; }
    long V = 1;
    for (int i = 0; i < 3; i++) {
        if (cfg->dims[i] < 1) { g_create_error = "opx_create: dims must be >= 1"; return OPX_ERR_INVALID; }
        if (!(cfg->a[i] > 0)) { g_create_error = "opx_create: lattice spacings must be > 0"; return OPX_ERR_INVALID; }
        V *= cfg->dims[i];
    }
    if (V * 4 > 2147483647L) { g_create_error = "opx_create: lattice too large (4*V must fit in int32)"; return OPX_ERR_INVALID; }
    if (!(cfg->dt > 0) || !(cfg->g > 0)) { g_create_error = "opx_create: dt and g must be > 0"; return OPX_ERR_INVALID; }
    if (cfg->reunit_every < 0) { g_create_error = "opx_create: reunit_every must be >= 0"; return OPX_ERR_INVALID; }
    cudaError_t e = cudaSetDevice(cfg->device);
    if (e != cudaSuccess) { g_create_error = std::string("opx_create: ") + cudaGetErrorString(e); return OPX_ERR_CUDA; }
    opx_ctx *h = new (std::nothrow) opx_ctx();
    if (!h) { g_create_error = "opx_create: host allocation failed"; return OPX_ERR_NOMEM; }
    Ctx &c = h->c;
    c.cfg = *cfg;
    c.L = make_lat(cfg->dims, cfg->a, cfg->dt, cfg->g);
    c.nc = cfg->ncolors;
    c.ng = c.nc == 3 ? 18 : 4;
    c.na = c.nc == 3 ? 8 : 3;
    c.na_ref = c.nc == 3 ? 9 : 3;
    c.prec = cfg->precision;
    c.pair_kernel = std::getenv("OPX_ONE_SITE_FP32") == nullptr;
    c.stream_kernel = std::getenv("OPX_STREAM_FP32") != nullptr;
    c.int_offsets = std::getenv("OPX_LONG_OFFSETS") == nullptr && link_elems(V, c.ng) < (1L << 31) - 64 &&
                    3L * c.na * V < (1L << 31);
    c.rsize = c.prec == OPX_F64 ? 8 : 4;
    bool ok = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) == cudaSuccess;
    auto al = [&](void **p, size_t bytes) { if (ok && cudaMalloc(p, bytes) != cudaSuccess) { ok = false; *p = nullptr; } };
    const size_t nU = (size_t)link_elems(V, c.ng), nE = (size_t)V * 3 * c.na;
    al(&c.U, nU * c.rsize);
    al(&c.Unext, nU * c.rsize);
    al(&c.E, nE * c.rsize);
    // J and rho are FP64 when particles can be attached (FP64 handles), storage precision otherwise
    al(&c.J, nE * c.rsize);
    al(&c.rho, (size_t)V * c.na * c.rsize);
    c.red_blocks = reduction_blocks(V);
    // 16 doubles per block: the bulk partials, or 2 (slice, split) partials of the projected energy
    al((void **)&c.red_part,
       sizeof(double) * 2 * BULK_COLUMNS * std::max(c.red_blocks, 2 * c.L.n[0] + 2 * c.L.n[1] + 2 * c.L.n[2]));
    al((void **)&c.red_out, sizeof(double) * 16);
    al((void **)&c.red_count, sizeof(unsigned));
    al((void **)&c.status, sizeof(unsigned));
    if (ok && cudaMallocHost((void **)&c.red_host, sizeof(double) * 16) != cudaSuccess) ok = false;
    if (ok && cudaMallocHost((void **)&c.status_host, sizeof(unsigned)) != cudaSuccess) ok = false;
    if (ok && (cudaEventCreate(&c.ev0) != cudaSuccess || cudaEventCreate(&c.ev1) != cudaSuccess)) ok = false;
    if (!ok) {
        release(c);
        delete h;
        g_create_error = "opx_create: out of device memory";
        cudaGetLastError();
        return OPX_ERR_NOMEM;
    }
    fill_identity(c, c.U);
    fill_identity(c, c.Unext);
    cudaMemsetAsync(c.E, 0, nE * c.rsize, c.stream);
    cudaMemsetAsync(c.J, 0, nE * c.rsize, c.stream);
    cudaMemsetAsync(c.rho, 0, (size_t)V * c.na * c.rsize, c.stream);
    cudaMemsetAsync(c.status, 0, sizeof(unsigned), c.stream);
    if (c.red_count) cudaMemsetAsync(c.red_count, 0, sizeof(unsigned), c.stream);
    if (sync_check(c, "opx_create") != OPX_OK) {
        g_create_error = c.err;
        release(c);
        delete h;
        return OPX_ERR_CUDA;
    }
    *out = h;
    return OPX_OK;
}

void opx_destroy(opx_ctx *ctx) {
    if (!ctx) return;
    cudaStreamSynchronize(ctx->c.stream);
    release(ctx->c);
    delete ctx;
}

static int ensure_staging(Ctx &c, size_t ndoubles) {
    if (c.staging_len >= ndoubles) return OPX_OK;
    if (c.staging) cudaFree(c.staging);
    c.staging = nullptr;
    c.staging_len = 0;
    if (cudaMalloc(&c.staging, ndoubles * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        c.err = "staging buffer: out of device memory";
        return OPX_ERR_NOMEM;
    }
    c.staging_len = ndoubles;
    return OPX_OK;
}

static int field_count(const Ctx &c, int field, int layout, size_t *n, int *ndir) {
    const int na_host = (layout == OPX_LAYOUT_REF) ? c.na_ref : c.na;
    switch (field) {
    case OPX_FIELD_U:
    case OPX_FIELD_UNEXT: *n = (size_t)c.L.V * 3 * c.ng; *ndir = 3; return OPX_OK;
    case OPX_FIELD_E:
    case OPX_FIELD_J: *n = (size_t)c.L.V * 3 * na_host; *ndir = 3; return OPX_OK;
    case OPX_FIELD_RHO: *n = (size_t)c.L.V * na_host; *ndir = 1; return OPX_OK;
    }
    return OPX_ERR_INVALID;
}

// The device address of a page-locked host buffer of n doubles (cudaMallocHost
// or cudaHostRegister memory, both ends mapped at one offset), or null for
// pageable memory.  The conversion kernels read and write page-locked buffers
// directly over the host link; pageable ones go through the staging copy.
static double *device_view(const void *host, size_t n) {
    cudaPointerAttributes a0, a1;
    const char *first = (const char *)host, *last = first + n * sizeof(double) - 1;
    if (cudaPointerGetAttributes(&a0, first) != cudaSuccess || cudaPointerGetAttributes(&a1, last) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer || !a1.devicePointer)
        return nullptr;
    if ((const char *)a1.devicePointer - (const char *)a0.devicePointer != last - first) return nullptr;
    return (double *)a0.devicePointer;
}

int opx_upload(opx_ctx *ctx, int field, const double *host, size_t count, int layout) {
    API_CHECK(ctx);
    Ctx &c = ctx->c;
    size_t n;
    int ndir;
    if (!host || (layout != OPX_LAYOUT_REF && layout != OPX_LAYOUT_GEN) || field_count(c, field, layout, &n, &ndir)) {
        c.err = "opx_upload: invalid field, layout or null buffer";
        return OPX_ERR_INVALID;
    }
    if (count != n) {
        c.err = "opx_upload: count " + std::to_string(count) + " != expected " + std::to_string(n);
        return OPX_ERR_INVALID;
    }
    const double *src = device_view(host, n);
    if (!src) {
        int rc = ensure_staging(c, n);
        if (rc) return rc;
        cudaError_t e = cudaMemcpyAsync(c.staging, host, n * sizeof(double), cudaMemcpyHostToDevice, c.stream);
        if (e != cudaSuccess) return cuda_fail(c, "opx_upload", e);
        src = c.staging;
    }
    switch (field) {
    case OPX_FIELD_U: launch_links_from_ref(c, src, c.U); break;
    case OPX_FIELD_UNEXT: launch_links_from_ref(c, src, c.Unext); break;
    case OPX_FIELD_E: launch_alg_from_host(c, src, c.E, 3, layout); break;
    case OPX_FIELD_J: launch_alg_from_host(c, src, c.J, 3, layout); c.j_nonzero = true; break;
    case OPX_FIELD_RHO: launch_alg_from_host(c, src, c.rho, 1, layout); c.rho_nonzero = true; break;
    }
    return sync_check(c, "opx_upload");
}

int opx_download(opx_ctx *ctx, int field, double *host, size_t count, int layout) {
    API_CHECK_RO(ctx);
    Ctx &c = ctx->c;
    size_t n;
    int ndir;
    if (!host || (layout != OPX_LAYOUT_REF && layout != OPX_LAYOUT_GEN) || field_count(c, field, layout, &n, &ndir)) {
        c.err = "opx_download: invalid field, layout or null buffer";
        return OPX_ERR_INVALID;
    }
    if (count != n) {
        c.err = "opx_download: count " + std::to_string(count) + " != expected " + std::to_string(n);
        return OPX_ERR_INVALID;
    }
    double *dst = device_view(host, n);
    const bool direct = dst != nullptr;
    if (!direct) {
        int rc = ensure_staging(c, n);
        if (rc) return rc;
        dst = c.staging;
    }
    switch (field) {
    case OPX_FIELD_U: launch_links_to_ref(c, c.U, dst); break;
    case OPX_FIELD_UNEXT: launch_links_to_ref(c, c.Unext, dst); break;
    case OPX_FIELD_E: launch_alg_to_host(c, c.E, dst, 3, layout); break;
    case OPX_FIELD_J: launch_alg_to_host(c, c.J, dst, 3, layout); break;
    case OPX_FIELD_RHO: launch_alg_to_host(c, c.rho, dst, 1, layout); break;
    }
    if (!direct) {
        cudaError_t e = cudaMemcpyAsync(host, c.staging, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream);
        if (e != cudaSuccess) return cuda_fail(c, "opx_download", e);
    }
    return sync_check(c, "opx_download");
}

static int set_mask(Ctx &c, uint8_t **dst, const uint8_t *mask, size_t count, const char *where) {
    if (!mask) {
        if (*dst) { cudaStreamSynchronize(c.stream); cudaFree(*dst); }
        *dst = nullptr;
        return OPX_OK;
    }
    if (count != (size_t)c.L.V) { c.err = std::string(where) + ": count must equal the number of cells"; return OPX_ERR_INVALID; }
    if (!*dst && cudaMalloc((void **)dst, c.L.V) != cudaSuccess) { cudaGetLastError(); c.err = std::string(where) + ": out of device memory"; return OPX_ERR_NOMEM; }
    cudaError_t e = cudaMemcpyAsync(*dst, mask, c.L.V, cudaMemcpyHostToDevice, c.stream);
    if (e != cudaSuccess) return cuda_fail(c, where, e);
    return sync_check(c, where);
}

int opx_set_active(opx_ctx *ctx, const uint8_t *mask, size_t count) {
    API_CHECK(ctx);
    return set_mask(ctx->c, &ctx->c.active, mask, count, "opx_set_active");
}

int opx_set_evaluatable(opx_ctx *ctx, const uint8_t *mask, size_t count) {
    API_CHECK(ctx);
    return set_mask(ctx->c, &ctx->c.eval, mask, count, "opx_set_evaluatable");
}

static void phase_begin(Ctx &c) {
    if (c.profiling) cudaEventRecord(c.ev0, c.stream);
}
static void phase_end(Ctx &c, int phase) {
    if (!c.profiling) return;
    cudaEventRecord(c.ev1, c.stream);
    cudaEventSynchronize(c.ev1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c.ev0, c.ev1);
    c.phase_ms[phase] += ms;
    c.phase_n[phase] += 1;
}

int opx_step_links(opx_ctx *ctx) {
    API_CHECK(ctx);
    Ctx &c = ctx->c;
    phase_begin(c);
    launch_update_links(c);
    phase_end(c, OPX_PHASE_LINKS);
    return check_launch(c, "opx_step_links");
}

int opx_update_grid(opx_ctx *ctx) {
    API_CHECK(ctx);
    Ctx &c = ctx->c;
    phase_begin(c);
    if (c.imp_solver) {
        int rc = launch_implicit_update(c);
        if (rc) return rc;
    } else {
        launch_update_grid(c, false);
    }
    phase_end(c, OPX_PHASE_EOM);
    return check_launch(c, "opx_update_grid");
}

int opx_store_fields(opx_ctx *ctx) {
    API_CHECK(ctx);
    std::swap(ctx->c.U, ctx->c.Unext);
    return OPX_OK;
}

int opx_reunitarize(opx_ctx *ctx) {
    API_CHECK(ctx);
    Ctx &c = ctx->c;
    launch_reunit(c, c.U);
    launch_reunit(c, c.Unext);
    return check_launch(c, "opx_reunitarize");
}

static int cpic_ok(Ctx &c, const char *where) {
    if (c.prec != OPX_F64) {
        c.err = std::string(where) + ": particles require an OPX_F64 handle";
        return OPX_ERR_UNSUPPORTED;
    }
    return OPX_OK;
}

int opx_cpic_phases(opx_ctx *ctx, int reassign) {
    API_CHECK(ctx);
    Ctx &c = ctx->c;
    int rc = cpic_ok(c, "opx_cpic_phases");
    if (rc) return rc;
    phase_begin(c);
    if (!c.sg.empty()) launch_super_phases(c, c.steps);  // the step counter is the simulation step t
    else launch_cpic_phases(c, reassign);
    phase_end(c, OPX_PHASE_CPIC);
    return check_launch(c, "opx_cpic_phases");
}

int opx_initialize(opx_ctx *ctx) {
    API_CHECK(ctx);
    Ctx &c = ctx->c;
    int rc = opx_step_links(ctx);
    if (rc) return rc;
    if (c.P.n > 0) return opx_cpic_phases(ctx, 0);
    if (!c.sg.empty()) {
        launch_super_phases(c, c.steps);
        return check_launch(c, "opx_initialize");
    }
    return OPX_OK;
}

static int one_step(Ctx &c) {
    c.steps++;
    std::swap(c.U, c.Unext);  // storeFields
    const bool reunit = c.prec == OPX_F32 && c.cfg.reunit_every > 0 && (c.steps % c.cfg.reunit_every) == 0;
    phase_begin(c);
    if (c.imp_solver) {
        int rc = launch_implicit_update(c);
        if (rc) return rc;
    } else {
        launch_update_grid(c, reunit);
    }
    phase_end(c, OPX_PHASE_EOM);
    if (c.P.n > 0) {
        phase_begin(c);
        launch_cpic_phases(c, 1);
        phase_end(c, OPX_PHASE_CPIC);
    } else if (!c.sg.empty()) {
        phase_begin(c);
        launch_super_phases(c, c.steps);
        phase_end(c, OPX_PHASE_CPIC);
    }
    return OPX_OK;
}

int opx_step(opx_ctx *ctx, int nsteps) {
    API_CHECK(ctx);
    Ctx &c = ctx->c;
    if (nsteps < 0) { c.err = "opx_step: nsteps < 0"; return OPX_ERR_INVALID; }
    c.step1_call = nsteps == 1 ? c.api_calls : -1;
    for (int k = 0; k < nsteps; k++) {
        int rc = one_step(c);
        if (rc) return rc;
    }
    return check_launch(c, "opx_step");
}

int opx_set_field_solver(opx_ctx *ctx, int kind, int iterations, double damping) {
    API_CHECK(ctx);
    Ctx &c = ctx->c;
    if (kind == OPX_SOLVER_FAST) { c.imp_solver = false; return OPX_OK; }
    if (kind != OPX_SOLVER_IMPLICIT || iterations < 0 || !(damping >= 0 && damping <= 1)) {
        c.err = "opx_set_field_solver: kind FAST or IMPLICIT, iterations >= 0, 0 <= damping <= 1";
        return OPX_ERR_INVALID;
    }
    c.imp_solver = true;
    c.imp_iterations = iterations;
    c.imp_damping = damping;
    return OPX_OK;
}

int opx_synchronize(opx_ctx *ctx) {
    API_CHECK_RO(ctx);
    return sync_check(ctx->c, "opx_synchronize");
}

long opx_steps_done(const opx_ctx *ctx) { return ctx ? ctx->c.steps : -1; }

// BulkQuantitiesInTime's row from the column sums r (the layout of
// c.red_out) with B^2 of U taken from bu (BulkQuantitiesInTime.java:83-121)
static int fill_observables(Ctx &c, const double *r, const double *bu, const char *where, opx_observables *out) {
    const double V = (double)c.L.V;
    for (int q = 0; q < BULK_COLUMNS; q++)
        if (!std::isfinite(q >= 3 && q < 6 ? bu[q - 3] : r[q])) {
            c.err = std::string(where) + ": non-finite field values (NaN/Inf) on the lattice";
            return OPX_ERR_NUMERIC;
        }
    double es[3], bs[3];
    for (int i = 0; i < 3; i++) {
        es[i] = r[i] / V;
        bs[i] = (bu[i] + r[8 + i]) / V;
        out->e2[i] = es[i];
        out->b2[i] = bs[i];
    }
    out->px = -es[0] + es[1] + es[2] - bs[0] + bs[1] + bs[2];
    out->py = +es[0] - es[1] + es[2] + bs[0] - bs[1] + bs[2];
    out->pz = +es[0] + es[1] - es[2] + bs[0] + bs[1] - bs[2];
    out->gauss = r[6] / V;
    out->rho2 = std::sqrt(r[7]) / V;
    out->e2_total = es[0] + es[1] + es[2];
    out->b2_total = bs[0] + bs[1] + bs[2];
    return OPX_OK;
}

int opx_reduce(opx_ctx *ctx, opx_observables *out) {
    API_CHECK_RO(ctx);
    Ctx &c = ctx->c;
    if (!out) { c.err = "opx_reduce: null output"; return OPX_ERR_INVALID; }
    // the only call since the last reduction that could change the fields was
    // opx_step(ctx, 1): U now is the Unext that reduction summed B^2 over
    const bool reuse = c.bcache.calls >= 0 && c.api_calls == c.bcache.calls + 1 && c.step1_call == c.api_calls &&
                       c.steps == c.bcache.steps + 1 && c.U == c.bcache.unext;
    c.bcache.calls = -1;
    // the generic pass also leaves the per-site B^2 of Unext for ProjectedEnergyDensity
    const bool generic = !(c.nc == 3 && c.prec == OPX_F32 && c.pair_kernel);
    if (generic && !c.bn_site && cudaMalloc((void **)&c.bn_site, sizeof(double) * 3 * c.L.V) != cudaSuccess) {
        cudaGetLastError();
        c.bn_site = nullptr;  // no cache: ProjectedEnergyDensity forms the plaquettes
    }
    c.bnsite.calls = -1;
    phase_begin(c);
    launch_bulk(c, reuse ? 1 : 0);
    cudaMemcpyAsync(c.red_host, c.red_out, sizeof(double) * BULK_COLUMNS, cudaMemcpyDeviceToHost, c.stream);
    int rc = sync_check(c, "opx_reduce");
    phase_end(c, OPX_PHASE_DIA);
    if (rc) return rc;
    const double *r = c.red_host;
    double bu[3];
    for (int i = 0; i < 3; i++) bu[i] = reuse ? c.bcache.bn[i] : r[3 + i];
    rc = fill_observables(c, r, bu, "opx_reduce", out);
    if (rc) return rc;
    c.bcache.calls = c.api_calls;
    c.bcache.steps = c.steps;
    c.bcache.unext = c.Unext;
    for (int i = 0; i < 3; i++) c.bcache.bn[i] = r[8 + i];
    if (generic && c.bn_site) {
        c.bnsite.calls = c.api_calls;
        c.bnsite.steps = c.steps;
        c.bnsite.unext = c.Unext;
    }
    return OPX_OK;
}

static int ensure_measure_buffers(Ctx &c, int nsteps) {
    const size_t nE = (size_t)c.L.V * 3 * c.na;
    bool ok = true;
    if (!c.E_alt) ok = cudaMalloc(&c.E_alt, nE * c.rsize) == cudaSuccess;
    for (void **w : {&c.W_in, &c.W_out})
        if (ok && !*w) {
            ok = cudaMalloc(w, nE * c.rsize) == cudaSuccess;
            if (ok) cudaMemsetAsync(*w, 0, nE * c.rsize, c.stream);  // the first step's Gauss term is unused
        }
    if (ok && !c.meas_part) {
        // the partials of up to 64 steps (at most 64 MB): their rows are formed
        // with one launch per chunk of steps
        const size_t per_step = sizeof(double) * MEAS_ROW * measured_parts(c);
        c.meas_chunk = (int)std::max<size_t>(1, std::min<size_t>(64, ((size_t)64 << 20) / per_step));
        ok = cudaMalloc((void **)&c.meas_part, per_step * c.meas_chunk) == cudaSuccess;
        if (!ok) c.meas_chunk = 0;
    }
    if (ok && c.meas_rows_cap < nsteps) {
        if (c.meas_rows) cudaFree(c.meas_rows);
        if (c.meas_host) cudaFreeHost(c.meas_host);
        c.meas_rows = c.meas_host = nullptr;
        c.meas_rows_cap = 0;
        ok = cudaMalloc((void **)&c.meas_rows, sizeof(double) * 8 * nsteps) == cudaSuccess &&
             cudaMallocHost((void **)&c.meas_host, sizeof(double) * 8 * nsteps) == cudaSuccess;
        if (ok) c.meas_rows_cap = nsteps;
    }
    if (!ok) {
        cudaGetLastError();
        c.err = "opx_step_measured: out of device memory";
        return OPX_ERR_NOMEM;
    }
    return OPX_OK;
}

int opx_step_measured(opx_ctx *ctx, int nsteps, opx_observables *out) {
    API_CHECK(ctx);
    Ctx &c = ctx->c;
    if (nsteps < 0 || (nsteps > 0 && !out)) { c.err = "opx_step_measured: nsteps < 0 or null output"; return OPX_ERR_INVALID; }
    if (nsteps == 0) return OPX_OK;
    if (nsteps == 1 || !measured_step_fusable(c)) {
        for (int k = 0; k < nsteps; k++) {
            int rc = opx_step(ctx, 1);
            if (!rc) rc = opx_reduce(ctx, &out[k]);
            if (rc) return rc;
        }
        return OPX_OK;
    }
    int rc = ensure_measure_buffers(c, nsteps);
    if (rc) return rc;
    c.bcache.calls = -1;
    const size_t per_step = (size_t)MEAS_ROW * measured_parts(c);
    for (int k0 = 0; k0 < nsteps; k0 += c.meas_chunk) {
        const int nk = std::min(c.meas_chunk, nsteps - k0);
        phase_begin(c);
        for (int k = 0; k < nk; k++) {
            c.steps++;
            std::swap(c.U, c.Unext);  // storeFields
            const bool reunit = c.cfg.reunit_every > 0 && (c.steps % c.cfg.reunit_every) == 0;
            launch_update_measure(c, reunit, c.E_alt, c.W_in, c.W_out, c.meas_part + per_step * k);
            std::swap(c.E, c.E_alt);
            std::swap(c.W_in, c.W_out);
        }
        launch_measure_combine(c, c.meas_part, nk, c.meas_rows + 8 * k0);
        phase_end(c, OPX_PHASE_EOM);
        // the chunk's rows to the host
        cudaMemcpyAsync(c.meas_host + 8 * k0, c.meas_rows + 8 * k0, sizeof(double) * 8 * nk, cudaMemcpyDeviceToHost,
                        c.stream);
    }
    // the last state: B^2 of its next links, its Gauss law and rho^2
    phase_begin(c);
    launch_bulk(c, 1);
    cudaMemcpyAsync(c.red_host, c.red_out, sizeof(double) * BULK_COLUMNS, cudaMemcpyDeviceToHost, c.stream);
    rc = sync_check(c, "opx_step_measured");
    phase_end(c, OPX_PHASE_DIA);
    if (rc) return rc;
    const double *red = c.red_host;
    for (int k = 0; k < nsteps; k++) {
        // step k's kernel: E^2 and B^2 of its input links (this state's U);
        // step k + 1's kernel (or the last reduction): B^2 of Unext and the Gauss law
        const double *m = c.meas_host + 8 * k, *mn = k + 1 < nsteps ? c.meas_host + 8 * (k + 1) : nullptr;
        double r[BULK_COLUMNS], bu[3];
        for (int i = 0; i < 3; i++) {
            r[i] = m[i];
            r[3 + i] = 0.0;
            bu[i] = m[3 + i];
            r[8 + i] = mn ? mn[3 + i] : red[8 + i];
        }
        r[6] = mn ? mn[6] : red[6];
        r[7] = red[7];
        rc = fill_observables(c, r, bu, "opx_step_measured", &out[k]);
        if (rc) return rc;
    }
    // a following opx_step(ctx, 1) + opx_reduce may reuse B^2 of Unext
    c.bcache.calls = c.api_calls;
    c.bcache.steps = c.steps;
    c.bcache.unext = c.Unext;
    for (int i = 0; i < 3; i++) c.bcache.bn[i] = red[8 + i];
    return OPX_OK;
}

int opx_energy_density(opx_ctx *ctx, double *host_out, size_t count) {
    API_CHECK_RO(ctx);
    Ctx &c = ctx->c;
    if (!host_out || count != (size_t)c.L.V) { c.err = "opx_energy_density: output must hold V doubles"; return OPX_ERR_INVALID; }
    int rc = ensure_staging(c, c.L.V);
    if (rc) return rc;
    phase_begin(c);
    launch_energy_density(c, c.staging);
    cudaMemcpyAsync(host_out, c.staging, sizeof(double) * c.L.V, cudaMemcpyDeviceToHost, c.stream);
    rc = sync_check(c, "opx_energy_density");
    phase_end(c, OPX_PHASE_DIA);
    return rc;
}

int opx_projected_energy(opx_ctx *ctx, int dir, double *host_out, size_t count) {
    API_CHECK_RO(ctx);
    Ctx &c = ctx->c;
    if (dir < 0 || dir > 2) { c.err = "opx_projected_energy: dir must be 0, 1 or 2"; return OPX_ERR_INVALID; }
    const int ns = c.L.n[dir];
    const size_t n = 4 * (size_t)ns;
    if (!host_out || count != n) { c.err = "opx_projected_energy: output must hold 4*dims[dir] doubles"; return OPX_ERR_INVALID; }
    int rc = ensure_staging(c, 6 * (size_t)ns);
    if (rc) return rc;
    // as in opx_reduce: after one opx_step(ctx, 1) since the last call for this
    // direction, the magnetic rows of U are that call's rows of Unext
    auto &pc = c.pcache[dir];
    const bool reuse = pc.calls >= 0 && c.api_calls == pc.calls + 1 && c.step1_call == c.api_calls &&
                       c.steps == pc.steps + 1 && c.U == pc.unext;
    pc.calls = -1;
    // B^2 of Unext per site from the last opx_reduce when nothing changed since
    const bool sites = c.bn_site && c.bnsite.calls == c.api_calls && c.bnsite.steps == c.steps &&
                       c.bnsite.unext == c.Unext;
    std::vector<double> rows(6 * (size_t)ns);
    phase_begin(c);
    launch_projected_energy(c, dir, reuse ? 1 : 0, sites ? c.bn_site : nullptr, c.staging);
    cudaMemcpyAsync(rows.data(), c.staging, sizeof(double) * rows.size(), cudaMemcpyDeviceToHost, c.stream);
    rc = sync_check(c, "opx_projected_energy");
    phase_end(c, OPX_PHASE_DIA);
    if (rc) return rc;
    for (int k = 0; k < ns; k++) {
        // magnetic T and L of U: this call's rows, or the last call's Unext rows
        const double tu = reuse ? pc.mag_next[k] : rows[ns + k];
        const double lu = reuse ? pc.mag_next[ns + k] : rows[3 * (size_t)ns + k];
        host_out[k] = rows[k];                                    // T_el
        host_out[ns + k] = tu + rows[4 * (size_t)ns + k];         // T_mag
        host_out[2 * (size_t)ns + k] = rows[2 * (size_t)ns + k];  // L_el
        host_out[3 * (size_t)ns + k] = lu + rows[5 * (size_t)ns + k];  // L_mag
    }
    pc.mag_next.assign(rows.begin() + 4 * (size_t)ns, rows.end());
    pc.calls = c.api_calls;
    pc.steps = c.steps;
    pc.unext = c.Unext;
    return OPX_OK;
}

int opx_projected_poynting(opx_ctx *ctx, int dir, double *host_out, size_t count) {
    API_CHECK_RO(ctx);
    Ctx &c = ctx->c;
    if (dir < 0 || dir > 2) { c.err = "opx_projected_poynting: dir must be 0, 1 or 2"; return OPX_ERR_INVALID; }
    if (c.nc != 2) {
        c.err = "opx_projected_poynting: SU(2) only (the reference's SU(3) algebra has no scalar product)";
        return OPX_ERR_UNSUPPORTED;
    }
    const size_t n = 2 * (size_t)c.L.n[dir];
    if (!host_out || count != n) { c.err = "opx_projected_poynting: output must hold 2*dims[dir] doubles"; return OPX_ERR_INVALID; }
    int rc = ensure_staging(c, n);
    if (rc) return rc;
    rc = launch_projected_poynting(c, dir, c.staging);
    if (rc) return rc;
    cudaMemcpyAsync(host_out, c.staging, sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream);
    return sync_check(c, "opx_projected_poynting");
}

int opx_gauss_field(opx_ctx *ctx, double *host_out, size_t count) {
    API_CHECK_RO(ctx);
    Ctx &c = ctx->c;
    const size_t n = (size_t)c.L.V * c.na;
    if (!host_out || count != n) { c.err = "opx_gauss_field: output must hold V*ngen doubles"; return OPX_ERR_INVALID; }
    int rc = ensure_staging(c, n);
    if (rc) return rc;
    phase_begin(c);
    launch_gauss_field(c, c.staging);
    cudaMemcpyAsync(host_out, c.staging, sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream);
    rc = sync_check(c, "opx_gauss_field");
    phase_end(c, OPX_PHASE_DIA);
    return rc;
}

int opx_particles_upload(opx_ctx *ctx, const opx_particles *p) {
    API_CHECK(ctx);
    Ctx &c = ctx->c;
    int rc = cpic_ok(c, "opx_particles_upload");
    if (rc) return rc;
    if (!p || p->n < 0) { c.err = "opx_particles_upload: invalid particle list"; return OPX_ERR_INVALID; }
    if (!c.sg.empty()) { c.err = "opx_particles_upload: the handle holds super particles"; return OPX_ERR_INVALID; }
    const long n = p->n;
    if (n > 0 && (!p->pos0 || !p->pos1 || !p->vel || !p->Q0 || !p->Q1 || !p->dir)) {
        c.err = "opx_particles_upload: null array";
        return OPX_ERR_INVALID;
    }
    if (n >= 2147483647L / 2) { c.err = "opx_particles_upload: too many particles"; return OPX_ERR_INVALID; }
    for (long k = 0; k < n; k++)
        if (p->dir[k] < 0 || p->dir[k] > 2) { c.err = "opx_particles_upload: direction must be 0, 1 or 2"; return OPX_ERR_INVALID; }
    rc = cpic_alloc(c, n);
    if (rc) return rc;
    if (n == 0) return OPX_OK;
    const int nar = c.na_ref;
    std::vector<double> t(3 * n);
    auto put3 = [&](const double *src, double *dst) {
        for (long k = 0; k < n; k++) for (int i = 0; i < 3; i++) t[i * n + k] = src[k * 3 + i];
        return cudaMemcpy(dst, t.data(), sizeof(double) * 3 * n, cudaMemcpyHostToDevice);
    };
    std::vector<double> tq((size_t)nar * n);
    auto putq = [&](const double *src, double *dst) {
        for (long k = 0; k < n; k++) for (int a = 0; a < nar; a++) tq[a * n + k] = src[k * nar + a];
        return cudaMemcpy(dst, tq.data(), sizeof(double) * nar * n, cudaMemcpyHostToDevice);
    };
    std::vector<int8_t> d8(n);
    for (long k = 0; k < n; k++) d8[k] = (int8_t)p->dir[k];
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = put3(p->pos0, c.P.pos0);
    if (e == cudaSuccess) e = put3(p->pos1, c.P.pos1);
    if (e == cudaSuccess) e = put3(p->vel, c.P.vel);
    if (e == cudaSuccess) e = putq(p->Q0, c.P.q0);
    if (e == cudaSuccess) e = putq(p->Q1, c.P.q1);
    if (e == cudaSuccess) e = cudaMemcpy(c.P.dir, d8.data(), n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(c, "opx_particles_upload", e);
    return OPX_OK;
}

int opx_particles_download(opx_ctx *ctx, opx_particles *p) {
    API_CHECK_RO(ctx);
    Ctx &c = ctx->c;
    if (!p || p->n != c.P.n) { c.err = "opx_particles_download: n must equal the uploaded count"; return OPX_ERR_INVALID; }
    const long n = p->n;
    if (n == 0) return OPX_OK;
    int rc = sync_check(c, "opx_particles_download");
    if (rc) return rc;
    const int nar = c.na_ref;
    std::vector<double> t(3 * n), tq((size_t)nar * n);
    auto get3 = [&](const double *src, double *dst) {
        cudaError_t e = cudaMemcpy(t.data(), src, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost);
        for (long k = 0; k < n; k++) for (int i = 0; i < 3; i++) dst[k * 3 + i] = t[i * n + k];
        return e;
    };
    auto getq = [&](const double *src, double *dst) {
        cudaError_t e = cudaMemcpy(tq.data(), src, sizeof(double) * nar * n, cudaMemcpyDeviceToHost);
        for (long k = 0; k < n; k++) for (int a = 0; a < nar; a++) dst[k * nar + a] = tq[a * n + k];
        return e;
    };
    cudaError_t e = cudaSuccess;
    if (p->pos0 && e == cudaSuccess) e = get3(c.P.pos0, p->pos0);
    if (p->pos1 && e == cudaSuccess) e = get3(c.P.pos1, p->pos1);
    if (p->vel && e == cudaSuccess) e = get3(c.P.vel, p->vel);
    if (p->Q0 && e == cudaSuccess) e = getq(c.P.q0, p->Q0);
    if (p->Q1 && e == cudaSuccess) e = getq(c.P.q1, p->Q1);
    if (p->dir && e == cudaSuccess) {
        std::vector<int8_t> d8(n);
        e = cudaMemcpy(d8.data(), c.P.dir, n, cudaMemcpyDeviceToHost);
        for (long k = 0; k < n; k++) p->dir[k] = d8[k];
    }
    if (p->update_charge) std::memset(p->update_charge, 0, n);
    if (e != cudaSuccess) return cuda_fail(c, "opx_particles_download", e);
    return OPX_OK;
}

long opx_particles_count(const opx_ctx *ctx) { return ctx ? ctx->c.P.n : -1; }

int opx_super_groups(const opx_ctx *ctx) { return ctx ? (int)ctx->c.sg.size() : -1; }

int opx_super_download(opx_ctx *ctx, int group, int *orientation, long *n, long *base, double *Q, size_t count) {
    API_CHECK_RO(ctx);
    Ctx &c = ctx->c;
    if (group < 0 || group >= (int)c.sg.size()) { c.err = "opx_super_download: no such group"; return OPX_ERR_INVALID; }
    const SuperGroup &G = c.sg[group];
    if (orientation) *orientation = G.orientation;
    if (n) *n = G.n;
    if (base) *base = G.base;
    if (!Q) return OPX_OK;
    const int nar = c.na_ref, ppc = c.sg_ppc;
    const size_t tot = (size_t)ppc * G.n * nar;
    if (count != tot) { c.err = "opx_super_download: Q must hold ppc*n*na_ref doubles"; return OPX_ERR_INVALID; }
    int rc = sync_check(c, "opx_super_download");
    if (rc) return rc;
    std::vector<double> t(tot);
    cudaError_t e = tot ? cudaMemcpy(t.data(), G.Q, sizeof(double) * tot, cudaMemcpyDeviceToHost) : cudaSuccess;
    if (e != cudaSuccess) return cuda_fail(c, "opx_super_download", e);
    // device [k][a][n] -> host [k][n][a]
    for (int k = 0; k < ppc; k++)
        for (long i = 0; i < G.n; i++)
            for (int a = 0; a < nar; a++) Q[((size_t)k * G.n + i) * nar + a] = t[((size_t)k * nar + a) * G.n + i];
    return OPX_OK;
}

int opx_super_upload(opx_ctx *ctx, int orientation, long n, long base, const double *Q) {
    API_CHECK(ctx);
    Ctx &c = ctx->c;
    if (c.prec != OPX_F64) { c.err = "opx_super_upload: super particles require an OPX_F64 handle"; return OPX_ERR_UNSUPPORTED; }
    if (c.P.n > 0) { c.err = "opx_super_upload: the handle holds NGP particles"; return OPX_ERR_INVALID; }
    const int ppc = (int)std::lround(c.L.a[0] / c.L.dt);
    if ((orientation != 1 && orientation != -1) || n < 0 || (n > 0 && !Q) || ppc < 1 ||
        (int)(c.sg.size() + 1) * ppc > 64) {
        c.err = "opx_super_upload: orientation +-1, n >= 0, round(a0/dt) >= 1, groups x round(a0/dt) <= 64";
        return OPX_ERR_INVALID;
    }
    SuperGroup G;
    G.orientation = orientation;
    G.n = n;
    G.base = base;
    const int nar = c.na_ref;
    const size_t tot = (size_t)ppc * n * nar;
    if (tot) {
        if (cudaMalloc(&G.Q, sizeof(double) * tot) != cudaSuccess) {
            cudaGetLastError();
            c.err = "opx_super_upload: out of device memory";
            return OPX_ERR_NOMEM;
        }
        std::vector<double> t(tot);
        for (int k = 0; k < ppc; k++)
            for (long i = 0; i < n; i++)
                for (int a = 0; a < nar; a++) t[((size_t)k * nar + a) * n + i] = Q[((size_t)k * n + i) * nar + a];
        cudaError_t e = cudaMemcpy(G.Q, t.data(), sizeof(double) * tot, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) { cudaFree(G.Q); return cuda_fail(c, "opx_super_upload", e); }
    }
    c.sg.push_back(G);
    c.sg_ppc = ppc;
    return OPX_OK;
}

int opx_init_random(opx_ctx *ctx, uint64_t seed, double sigma_a, double sigma_e) {
    API_CHECK(ctx);
    Ctx &c = ctx->c;
    if (!(sigma_a >= 0) || !(sigma_e >= 0)) { c.err = "opx_init_random: sigmas must be >= 0"; return OPX_ERR_INVALID; }
    int rc = ic_init_random(c, seed, sigma_a, sigma_e);
    if (rc) return rc;
    return sync_check(c, "opx_init_random");
}

int opx_gauss_project(opx_ctx *ctx, double tol_g2, int maxit, int *iters, double *final_g2) {
    API_CHECK(ctx);
    Ctx &c = ctx->c;
    if (!(tol_g2 > 0) || maxit < 0) { c.err = "opx_gauss_project: tol must be > 0 and maxit >= 0"; return OPX_ERR_INVALID; }
    return ic_gauss_project(c, tol_g2, maxit, iters, final_g2);
}

int opx_set_profiling(opx_ctx *ctx, int on) {
    API_CHECK_RO(ctx);
    Ctx &c = ctx->c;
    c.profiling = on != 0;
    for (int k = 0; k < OPX_NUM_PHASES; k++) { c.phase_ms[k] = 0; c.phase_n[k] = 0; }
    return OPX_OK;
}

int opx_phase_times(opx_ctx *ctx, double *ms, long *counts, int nphases) {
    API_CHECK_RO(ctx);
    Ctx &c = ctx->c;
    for (int k = 0; k < nphases && k < OPX_NUM_PHASES; k++) {
        if (ms) ms[k] = c.phase_ms[k];
        if (counts) counts[k] = c.phase_n[k];
    }
    return OPX_OK;
}

int opx_time_steps(opx_ctx *ctx, int nsteps, double *ms) {
    API_CHECK(ctx);
    Ctx &c = ctx->c;
    if (nsteps < 0 || !ms) { c.err = "opx_time_steps: invalid arguments"; return OPX_ERR_INVALID; }
    const bool prof = c.profiling;
    c.profiling = false;
    cudaEventRecord(c.ev0, c.stream);
    for (int k = 0; k < nsteps; k++) one_step(c);
    cudaEventRecord(c.ev1, c.stream);
    cudaError_t e = cudaEventSynchronize(c.ev1);
    c.profiling = prof;
    if (e != cudaSuccess) return cuda_fail(c, "opx_time_steps", e);
    float f = 0.f;
    cudaEventElapsedTime(&f, c.ev0, c.ev1);
    *ms = f;
    return check_launch(c, "opx_time_steps");
}

long opx_kernel_launches(const opx_ctx *ctx) { return ctx ? ctx->c.launches : -1; }

void *opx_host_alloc(size_t bytes) {
    void *p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) { cudaGetLastError(); return nullptr; }
    return p;
}

void opx_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

}  // extern "C"
