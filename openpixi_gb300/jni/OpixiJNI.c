/* OpixiJNI.c -- JNI binding of libopixi_gpu.so for the Java reference
 * (class org.openpixi.pixi.gpu.Opixi, Opixi.java beside this file).
 *
 * Build (any JDK):
 *   gcc -O2 -shared -fPIC -I$JAVA_HOME/include -I$JAVA_HOME/include/linux \
 *       -I<repo>/include OpixiJNI.c -L<repo>/openpixi_gb300/lib -lopixi_gpu \
 *       -Wl,-rpath,<repo>/openpixi_gb300/lib -o libOpixiJNI.so
 *
 * Handles.  A Java handle (long) points to a jhandle: the library handle and a
 * page-locked staging buffer (opx_host_alloc) that is kept and grown on demand.
 *
 * Transfers.  Field arrays on the Java heap move through the staging buffer in
 * chunks of Get/SetDoubleArrayRegion: no JNI critical region is held while the
 * device copies, so the garbage collector is never stalled by a transfer, and
 * the library reads or writes page-locked memory directly (its fast path).  A
 * direct ByteBuffer from Opixi.hostAlloc is page-locked already and is passed
 * through without a copy (uploadDirect / downloadDirect).  Smaller arrays
 * (masks, particles, diagnostics rows) use Get/Release<Type>ArrayElements.
 *
 * Errors.  Every library status other than OPX_OK raises
 * java.lang.RuntimeException with opx_last_error's message; the call returns
 * with the exception pending.  Threading: a handle is used by one thread at a
 * time, as Simulation.step does. */
#include <jni.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "opixi.h"

typedef struct {
    opx_ctx *ctx;
    double *stage;
    size_t stage_len; /* doubles */
} jhandle;

#define CHUNK ((jsize)(1 << 20)) /* doubles per region copy */

static jhandle *H(jlong h) { return (jhandle *)(intptr_t)h; }

static void throw_rt(JNIEnv *env, const char *msg) {
    jclass c = (*env)->FindClass(env, "java/lang/RuntimeException");
    if (c) (*env)->ThrowNew(env, c, msg ? msg : "opixi: error");
}

/* 1 when rc is OPX_OK, else raises and returns 0 */
static int ok(JNIEnv *env, jhandle *h, int rc) {
    if (rc == OPX_OK) return 1;
    throw_rt(env, opx_last_error(h ? h->ctx : NULL));
    return 0;
}

static double *stage(JNIEnv *env, jhandle *h, size_t n) {
    if (h->stage_len < n) {
        if (h->stage) opx_host_free(h->stage);
        h->stage = (double *)opx_host_alloc(n * sizeof(double));
        h->stage_len = h->stage ? n : 0;
        if (!h->stage) {
            throw_rt(env, "opixi: page-locked staging allocation failed");
            return NULL;
        }
    }
    return h->stage;
}

/* Java heap array -> dst (n doubles), region by region */
static int from_heap(JNIEnv *env, jdoubleArray a, double *dst, jsize n) {
    for (jsize k = 0; k < n; k += CHUNK) {
        const jsize m = n - k < CHUNK ? n - k : CHUNK;
        (*env)->GetDoubleArrayRegion(env, a, k, m, (jdouble *)(dst + k));
        if ((*env)->ExceptionCheck(env)) return 0;
    }
    return 1;
}

static int to_heap(JNIEnv *env, const double *src, jdoubleArray a, jsize n) {
    for (jsize k = 0; k < n; k += CHUNK) {
        const jsize m = n - k < CHUNK ? n - k : CHUNK;
        (*env)->SetDoubleArrayRegion(env, a, k, m, (const jdouble *)(src + k));
        if ((*env)->ExceptionCheck(env)) return 0;
    }
    return 1;
}

/* ---------------------------------------------------------------- handles */

JNIEXPORT jlong JNICALL Java_org_openpixi_pixi_gpu_Opixi_create(JNIEnv *env, jclass cls, jint ncolors,
                                                               jintArray dims, jdoubleArray a, jdouble dt,
                                                               jdouble g, jint precision, jint reunitEvery,
                                                               jint device) {
    (void)cls;
    opx_config c;
    memset(&c, 0, sizeof c);
    c.ncolors = ncolors;
    (*env)->GetIntArrayRegion(env, dims, 0, 3, (jint *)c.dims);
    (*env)->GetDoubleArrayRegion(env, a, 0, 3, (jdouble *)c.a);
    if ((*env)->ExceptionCheck(env)) return 0;
    c.dt = dt;
    c.g = g;
    c.precision = precision;
    c.reunit_every = reunitEvery;
    c.device = device;
    jhandle *h = (jhandle *)calloc(1, sizeof(jhandle));
    if (!h) {
        throw_rt(env, "opixi: out of host memory");
        return 0;
    }
    if (opx_create(&c, &h->ctx) != OPX_OK) {
        throw_rt(env, opx_last_error(NULL));
        free(h);
        return 0;
    }
    return (jlong)(intptr_t)h;
}

JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_destroy(JNIEnv *env, jclass cls, jlong hh) {
    (void)env;
    (void)cls;
    jhandle *h = H(hh);
    if (!h) return;
    opx_destroy(h->ctx);
    if (h->stage) opx_host_free(h->stage);
    free(h);
}

/* ---------------------------------------------------------------- fields */

/* Grid setters (Grid.java:126-261): the whole field, reference layout
 * (OPX_LAYOUT_REF) or generator components (OPX_LAYOUT_GEN) */
JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_upload(JNIEnv *env, jclass cls, jlong hh, jint field,
                                                              jdoubleArray data, jint layout) {
    (void)cls;
    jhandle *h = H(hh);
    const jsize n = (*env)->GetArrayLength(env, data);
    double *st = stage(env, h, (size_t)n);
    if (!st || !from_heap(env, data, st, n)) return;
    ok(env, h, opx_upload(h->ctx, field, st, (size_t)n, layout));
}

/* Grid getters: getU / getUnext / getE / getJ / getRho for every cell */
JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_download(JNIEnv *env, jclass cls, jlong hh, jint field,
                                                                jdoubleArray out, jint layout) {
    (void)cls;
    jhandle *h = H(hh);
    const jsize n = (*env)->GetArrayLength(env, out);
    double *st = stage(env, h, (size_t)n);
    if (!st) return;
    if (!ok(env, h, opx_download(h->ctx, field, st, (size_t)n, layout))) return;
    to_heap(env, st, out, n);
}

/* a direct ByteBuffer over Opixi.hostAlloc memory: no copy on the host */
JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_uploadDirect(JNIEnv *env, jclass cls, jlong hh, jint field,
                                                                    jobject buf, jlong count, jint layout) {
    (void)cls;
    jhandle *h = H(hh);
    const double *p = (const double *)(*env)->GetDirectBufferAddress(env, buf);
    if (!p || (*env)->GetDirectBufferCapacity(env, buf) < count * (jlong)sizeof(double)) {
        throw_rt(env, "opixi: uploadDirect needs a direct buffer of count doubles");
        return;
    }
    ok(env, h, opx_upload(h->ctx, field, p, (size_t)count, layout));
}

JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_downloadDirect(JNIEnv *env, jclass cls, jlong hh, jint field,
                                                                      jobject buf, jlong count, jint layout) {
    (void)cls;
    jhandle *h = H(hh);
    double *p = (double *)(*env)->GetDirectBufferAddress(env, buf);
    if (!p || (*env)->GetDirectBufferCapacity(env, buf) < count * (jlong)sizeof(double)) {
        throw_rt(env, "opixi: downloadDirect needs a direct buffer of count doubles");
        return;
    }
    ok(env, h, opx_download(h->ctx, field, p, (size_t)count, layout));
}

JNIEXPORT jobject JNICALL Java_org_openpixi_pixi_gpu_Opixi_hostAlloc(JNIEnv *env, jclass cls, jlong bytes) {
    (void)cls;
    void *p = opx_host_alloc((size_t)bytes);
    if (!p) {
        throw_rt(env, "opixi: page-locked allocation failed");
        return NULL;
    }
    return (*env)->NewDirectByteBuffer(env, p, bytes);
}

JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_hostFree(JNIEnv *env, jclass cls, jobject buf) {
    (void)cls;
    void *p = (*env)->GetDirectBufferAddress(env, buf);
    if (p) opx_host_free(p);
}

/* Grid.setActiveRegion / setEvaluationRegion: one byte per cell, null = all cells */
static void set_mask(JNIEnv *env, jlong hh, jbyteArray mask, int evaluatable) {
    jhandle *h = H(hh);
    if (!mask) {
        ok(env, h, evaluatable ? opx_set_evaluatable(h->ctx, NULL, 0) : opx_set_active(h->ctx, NULL, 0));
        return;
    }
    const jsize n = (*env)->GetArrayLength(env, mask);
    jbyte *m = (*env)->GetByteArrayElements(env, mask, NULL);
    if (!m) return;
    const int rc = evaluatable ? opx_set_evaluatable(h->ctx, (const uint8_t *)m, (size_t)n)
                               : opx_set_active(h->ctx, (const uint8_t *)m, (size_t)n);
    (*env)->ReleaseByteArrayElements(env, mask, m, JNI_ABORT);
    ok(env, h, rc);
}

JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_setActive(JNIEnv *env, jclass cls, jlong hh, jbyteArray mask) {
    (void)cls;
    set_mask(env, hh, mask, 0);
}

JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_setEvaluatable(JNIEnv *env, jclass cls, jlong hh,
                                                                      jbyteArray mask) {
    (void)cls;
    set_mask(env, hh, mask, 1);
}

/* ---------------------------------------------------------------- solver */

/* FieldSolver.stepLinks (FastTYMSolver.java:34-38) */
JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_stepLinks(JNIEnv *env, jclass cls, jlong hh) {
    (void)cls;
    ok(env, H(hh), opx_step_links(H(hh)->ctx));
}

/* FieldSolver.step (FastTYMSolver.java:24-32) */
JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_updateGrid(JNIEnv *env, jclass cls, jlong hh) {
    (void)cls;
    ok(env, H(hh), opx_update_grid(H(hh)->ctx));
}

/* Grid.storeFields (Grid.java:591-593) */
JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_storeFields(JNIEnv *env, jclass cls, jlong hh) {
    (void)cls;
    ok(env, H(hh), opx_store_fields(H(hh)->ctx));
}

/* Simulation.initialize / step (Simulation.java:318-435) */
JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_initialize(JNIEnv *env, jclass cls, jlong hh) {
    (void)cls;
    ok(env, H(hh), opx_initialize(H(hh)->ctx));
}

JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_step(JNIEnv *env, jclass cls, jlong hh, jint n) {
    (void)cls;
    ok(env, H(hh), opx_step(H(hh)->ctx, n));
}

JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_setFieldSolver(JNIEnv *env, jclass cls, jlong hh, jint kind,
                                                                      jint iterations, jdouble damping) {
    (void)cls;
    ok(env, H(hh), opx_set_field_solver(H(hh)->ctx, kind, iterations, damping));
}

/* ---------------------------------------------------------------- diagnostics */

/* BulkQuantitiesInTime / FieldMeasurements: 13 doubles in opx_observables order */
JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_reduce(JNIEnv *env, jclass cls, jlong hh,
                                                              jdoubleArray out13) {
    (void)cls;
    opx_observables o;
    if (!ok(env, H(hh), opx_reduce(H(hh)->ctx, &o))) return;
    (*env)->SetDoubleArrayRegion(env, out13, 0, 13, (const jdouble *)&o);
}

/* MainBatch's loop with BulkQuantitiesInTime every step: n rows of 13 doubles */
JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_stepMeasured(JNIEnv *env, jclass cls, jlong hh, jint n,
                                                                    jdoubleArray rows) {
    (void)cls;
    jhandle *h = H(hh);
    opx_observables *o = (opx_observables *)malloc(sizeof(opx_observables) * (size_t)(n > 0 ? n : 1));
    if (!o) {
        throw_rt(env, "opixi: out of host memory");
        return;
    }
    if (ok(env, h, opx_step_measured(h->ctx, n, o)))
        (*env)->SetDoubleArrayRegion(env, rows, 0, 13 * n, (const jdouble *)o);
    free(o);
}

/* EnergyDensity (V doubles), ProjectedEnergyDensity (4 x dims[dir]), Poynting
 * rows (2 x dims[dir]), Gauss law per cell (V x ngen): out sized by the caller */
JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_energyDensity(JNIEnv *env, jclass cls, jlong hh,
                                                                     jdoubleArray out) {
    (void)cls;
    jhandle *h = H(hh);
    const jsize n = (*env)->GetArrayLength(env, out);
    double *st = stage(env, h, (size_t)n);
    if (!st || !ok(env, h, opx_energy_density(h->ctx, st, (size_t)n))) return;
    to_heap(env, st, out, n);
}

JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_projectedEnergy(JNIEnv *env, jclass cls, jlong hh, jint dir,
                                                                       jdoubleArray out) {
    (void)cls;
    jhandle *h = H(hh);
    const jsize n = (*env)->GetArrayLength(env, out);
    double *st = stage(env, h, (size_t)n);
    if (!st || !ok(env, h, opx_projected_energy(h->ctx, dir, st, (size_t)n))) return;
    to_heap(env, st, out, n);
}

JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_projectedPoynting(JNIEnv *env, jclass cls, jlong hh, jint dir,
                                                                         jdoubleArray out) {
    (void)cls;
    jhandle *h = H(hh);
    const jsize n = (*env)->GetArrayLength(env, out);
    double *st = stage(env, h, (size_t)n);
    if (!st || !ok(env, h, opx_projected_poynting(h->ctx, dir, st, (size_t)n))) return;
    to_heap(env, st, out, n);
}

JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_gaussField(JNIEnv *env, jclass cls, jlong hh,
                                                                  jdoubleArray out) {
    (void)cls;
    jhandle *h = H(hh);
    const jsize n = (*env)->GetArrayLength(env, out);
    double *st = stage(env, h, (size_t)n);
    if (!st || !ok(env, h, opx_gauss_field(h->ctx, st, (size_t)n))) return;
    to_heap(env, st, out, n);
}

/* ---------------------------------------------------------------- particles */

/* The CGC particle list (CGCParticle: pos0, pos1, vel [n][3], Q0, Q1
 * [n][na_ref], direction [n]); InterpolatorAlgorithm / ParticleSolver run on
 * the device in opx_step (or cpicPhases). */
/* the six (or seven) particle arrays, pinned or copied by the JVM one by one;
 * on failure the ones obtained are released and an exception is pending */
typedef struct {
    jdoubleArray a[5];
    jdouble *p[5];
    jintArray dir;
    jint *pdir;
    jbyteArray upd;
    jbyte *pupd;
} particle_arrays;

static void release_particles(JNIEnv *env, particle_arrays *q, jint mode) {
    for (int k = 0; k < 5; k++)
        if (q->p[k]) (*env)->ReleaseDoubleArrayElements(env, q->a[k], q->p[k], mode);
    if (q->pdir) (*env)->ReleaseIntArrayElements(env, q->dir, q->pdir, mode);
    if (q->pupd) (*env)->ReleaseByteArrayElements(env, q->upd, q->pupd, mode);
}

static int get_particles(JNIEnv *env, particle_arrays *q) {
    for (int k = 0; k < 5; k++) {
        q->p[k] = (*env)->GetDoubleArrayElements(env, q->a[k], NULL);
        if (!q->p[k]) return 0;
    }
    q->pdir = (*env)->GetIntArrayElements(env, q->dir, NULL);
    if (!q->pdir) return 0;
    if (q->upd) {
        q->pupd = (*env)->GetByteArrayElements(env, q->upd, NULL);
        if (!q->pupd) return 0;
    }
    return 1;
}

/* The CGC particle list (CGCParticle: pos0, pos1, vel [n][3], Q0, Q1
 * [n][na_ref], direction [n]); InterpolatorAlgorithm / ParticleSolver run on
 * the device in opx_step (or cpicPhases). */
JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_particlesUpload(JNIEnv *env, jclass cls, jlong hh,
                                                                       jdoubleArray pos0, jdoubleArray pos1,
                                                                       jdoubleArray vel, jdoubleArray q0,
                                                                       jdoubleArray q1, jintArray dir) {
    (void)cls;
    jhandle *h = H(hh);
    particle_arrays q;
    memset(&q, 0, sizeof q);
    q.a[0] = pos0; q.a[1] = pos1; q.a[2] = vel; q.a[3] = q0; q.a[4] = q1;
    q.dir = dir;
    if (!get_particles(env, &q)) {
        release_particles(env, &q, JNI_ABORT);
        return;
    }
    opx_particles p;
    memset(&p, 0, sizeof p);
    p.n = (long)(*env)->GetArrayLength(env, dir);
    p.pos0 = q.p[0]; p.pos1 = q.p[1]; p.vel = q.p[2]; p.Q0 = q.p[3]; p.Q1 = q.p[4];
    p.dir = (int32_t *)q.pdir;
    const int rc = opx_particles_upload(h->ctx, &p);
    release_particles(env, &q, JNI_ABORT);
    ok(env, h, rc);
}

JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_particlesDownload(JNIEnv *env, jclass cls, jlong hh,
                                                                         jdoubleArray pos0, jdoubleArray pos1,
                                                                         jdoubleArray vel, jdoubleArray q0,
                                                                         jdoubleArray q1, jintArray dir,
                                                                         jbyteArray updateCharge) {
    (void)cls;
    jhandle *h = H(hh);
    particle_arrays q;
    memset(&q, 0, sizeof q);
    q.a[0] = pos0; q.a[1] = pos1; q.a[2] = vel; q.a[3] = q0; q.a[4] = q1;
    q.dir = dir;
    q.upd = updateCharge;
    if (!get_particles(env, &q)) {
        release_particles(env, &q, JNI_ABORT);
        return;
    }
    opx_particles p;
    memset(&p, 0, sizeof p);
    p.n = (long)(*env)->GetArrayLength(env, dir);
    p.pos0 = q.p[0]; p.pos1 = q.p[1]; p.vel = q.p[2]; p.Q0 = q.p[3]; p.Q1 = q.p[4];
    p.dir = (int32_t *)q.pdir;
    p.update_charge = (uint8_t *)q.pupd;
    const int rc = opx_particles_download(h->ctx, &p);
    release_particles(env, &q, rc == OPX_OK ? 0 : JNI_ABORT);  /* copy back a complete download only */
    ok(env, h, rc);
}

JNIEXPORT jlong JNICALL Java_org_openpixi_pixi_gpu_Opixi_particlesCount(JNIEnv *env, jclass cls, jlong hh) {
    (void)env;
    (void)cls;
    return (jlong)opx_particles_count(H(hh)->ctx);
}

/* the particle phases of Simulation.step (reassign = 1) or initialize (0) */
JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_cpicPhases(JNIEnv *env, jclass cls, jlong hh, jint reassign) {
    (void)cls;
    ok(env, H(hh), opx_cpic_phases(H(hh)->ctx, reassign));
}

/* CGCInitialCondition with MVModel entries (YamlMVModel): per nucleus
 * ints {direction, orientation, useSeed, seed} and reals {location, width, mu,
 * ultravioletCutoffTransverse, longitudinalCoherenceLength, infraredCoefficient} */
JNIEXPORT void JNICALL Java_org_openpixi_pixi_gpu_Opixi_cgcMV(JNIEnv *env, jclass cls, jlong hh, jintArray ints,
                                                             jdoubleArray reals, jint n) {
    (void)cls;
    jhandle *h = H(hh);
    opx_mv_nucleus *nu = (opx_mv_nucleus *)calloc((size_t)(n > 0 ? n : 1), sizeof(opx_mv_nucleus));
    jint *iv = (jint *)malloc(sizeof(jint) * 4 * (size_t)(n > 0 ? n : 1));
    jdouble *rv = (jdouble *)malloc(sizeof(jdouble) * 6 * (size_t)(n > 0 ? n : 1));
    if (!nu || !iv || !rv) {
        free(nu);
        free(iv);
        free(rv);
        throw_rt(env, "opixi: out of host memory");
        return;
    }
    (*env)->GetIntArrayRegion(env, ints, 0, 4 * n, iv);
    (*env)->GetDoubleArrayRegion(env, reals, 0, 6 * n, rv);
    if (!(*env)->ExceptionCheck(env)) {
        for (jint k = 0; k < n; k++) {
            nu[k].direction = iv[4 * k];
            nu[k].orientation = iv[4 * k + 1];
            nu[k].use_seed = iv[4 * k + 2];
            nu[k].seed = iv[4 * k + 3];
            nu[k].location = rv[6 * k];
            nu[k].width = rv[6 * k + 1];
            nu[k].mu = rv[6 * k + 2];
            nu[k].uvt = rv[6 * k + 3];
            nu[k].coherence = rv[6 * k + 4];
            nu[k].ir = rv[6 * k + 5];
        }
        ok(env, h, opx_cgc_mv(h->ctx, nu, n));
    }
    free(nu);
    free(iv);
    free(rv);
}

/* ---------------------------------------------------------------- gradients */

/* The Java gradient API (no counterpart in the reference): objective kind
 * (Opixi.OBJ_ENERGY / OBJ_ANISOTROPY), longitudinal direction, box lo..hi. */
static int fill_objective(JNIEnv *env, opx_objective *o, jint kind, jint direction, jintArray lo, jintArray hi) {
    memset(o, 0, sizeof *o);
    o->kind = kind;
    o->direction = direction;
    (*env)->GetIntArrayRegion(env, lo, 0, 3, (jint *)o->lo);
    (*env)->GetIntArrayRegion(env, hi, 0, 3, (jint *)o->hi);
    return !(*env)->ExceptionCheck(env);
}

/* an optional direction array on the host (NULL when absent) */
static double *opt_array(JNIEnv *env, jdoubleArray a) {
    return a ? (*env)->GetDoubleArrayElements(env, a, NULL) : NULL;
}
static void release_opt(JNIEnv *env, jdoubleArray a, double *p) {
    if (a && p) (*env)->ReleaseDoubleArrayElements(env, a, p, JNI_ABORT);
}

JNIEXPORT jdouble JNICALL Java_org_openpixi_pixi_gpu_Opixi_objectiveValue(JNIEnv *env, jclass cls, jlong hh, jint kind,
                                                                         jint direction, jintArray lo, jintArray hi,
                                                                         jint nsteps, jdoubleArray dE,
                                                                         jdoubleArray drho, jdouble step) {
    (void)cls;
    jhandle *h = H(hh);
    opx_objective o;
    if (!fill_objective(env, &o, kind, direction, lo, hi)) return 0.0;
    double *e = opt_array(env, dE), *r = opt_array(env, drho);
    double J = 0.0;
    const int rc = opx_objective_value(h->ctx, &o, nsteps, e, r, step, &J);
    release_opt(env, dE, e);
    release_opt(env, drho, r);
    ok(env, h, rc);
    return J;
}

/* returns {J, dJ} */
JNIEXPORT jdoubleArray JNICALL Java_org_openpixi_pixi_gpu_Opixi_objectiveTangent(JNIEnv *env, jclass cls, jlong hh,
                                                                                jint kind, jint direction,
                                                                                jintArray lo, jintArray hi,
                                                                                jint nsteps, jdoubleArray dE,
                                                                                jdoubleArray drho) {
    (void)cls;
    jhandle *h = H(hh);
    opx_objective o;
    if (!fill_objective(env, &o, kind, direction, lo, hi)) return NULL;
    double *e = opt_array(env, dE), *r = opt_array(env, drho);
    double v[2] = {0.0, 0.0};
    const int rc = opx_objective_tangent(h->ctx, &o, nsteps, e, r, &v[0], &v[1]);
    release_opt(env, dE, e);
    release_opt(env, drho, r);
    if (!ok(env, h, rc)) return NULL;
    jdoubleArray out = (*env)->NewDoubleArray(env, 2);
    if (out) (*env)->SetDoubleArrayRegion(env, out, 0, 2, v);
    return out;
}

/* fills grad (V*3*ngen doubles for Opixi.WRT_E, V*ngen for WRT_RHO), returns J */
JNIEXPORT jdouble JNICALL Java_org_openpixi_pixi_gpu_Opixi_objectiveGradient(JNIEnv *env, jclass cls, jlong hh,
                                                                            jint kind, jint direction, jintArray lo,
                                                                            jintArray hi, jint nsteps, jint ckpt,
                                                                            jint wrt, jdoubleArray grad) {
    (void)cls;
    jhandle *h = H(hh);
    opx_objective o;
    if (!fill_objective(env, &o, kind, direction, lo, hi)) return 0.0;
    const jsize n = (*env)->GetArrayLength(env, grad);
    double *st = stage(env, h, (size_t)n);
    if (!st) return 0.0;
    double J = 0.0;
    if (!ok(env, h, opx_objective_gradient(h->ctx, &o, nsteps, ckpt, wrt, &J, st, (size_t)n))) return 0.0;
    to_heap(env, st, grad, n);
    return J;
}
