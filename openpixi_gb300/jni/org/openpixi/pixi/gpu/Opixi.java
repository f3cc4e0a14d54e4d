package org.openpixi.pixi.gpu;

import java.nio.ByteBuffer;

/**
 * JNI declarations of libopixi_gpu.so (OpixiJNI.c; the C ABI is include/opixi.h).
 * A handle is one lattice on one GPU; its fields stay on the device between
 * calls.  Every method raises RuntimeException with the library's message when
 * the library reports an error.  Arrays are sized by the caller:
 * links V*3*ng (ng = 4 for SU(2), 18 for SU(3)), E and J V*3*na_ref (reference
 * layout) or V*3*ngen (LAYOUT_GEN), rho V*na_ref or V*ngen, masks V bytes.
 */
public final class Opixi {
    static { System.loadLibrary("OpixiJNI"); }

    private Opixi() {}

    public static final int F64 = 0, F32 = 1;
    public static final int FIELD_U = 0, FIELD_UNEXT = 1, FIELD_E = 2, FIELD_J = 3, FIELD_RHO = 4;
    public static final int LAYOUT_REF = 0, LAYOUT_GEN = 1;
    public static final int SOLVER_FAST = 0, SOLVER_IMPLICIT = 1;
    public static final int OBJ_ENERGY = 0, OBJ_ANISOTROPY = 1;
    public static final int WRT_E = 0, WRT_RHO = 1;

    // handles (Grid construction: Settings.gridCells, gridStep, timeStep, couplingConstant)
    public static native long create(int ncolors, int[] dims, double[] a, double dt, double g, int precision,
                                     int reunitEvery, int device);
    public static native void destroy(long h);

    // fields (Grid getters and setters for every cell)
    public static native void upload(long h, int field, double[] data, int layout);
    public static native void download(long h, int field, double[] out, int layout);
    /** page-locked host memory: a direct ByteBuffer (native byte order) for uploadDirect / downloadDirect */
    public static native ByteBuffer hostAlloc(long bytes);
    public static native void hostFree(ByteBuffer buf);
    public static native void uploadDirect(long h, int field, ByteBuffer buf, long count, int layout);
    public static native void downloadDirect(long h, int field, ByteBuffer buf, long count, int layout);
    /** Grid.setActiveRegion / setEvaluationRegion: one byte per cell, null = every cell */
    public static native void setActive(long h, byte[] mask);
    public static native void setEvaluatable(long h, byte[] mask);

    // solver (FieldSolver.step / stepLinks, Grid.storeFields, Simulation.initialize / step)
    public static native void stepLinks(long h);
    public static native void updateGrid(long h);
    public static native void storeFields(long h);
    public static native void initialize(long h);
    public static native void step(long h, int n);
    public static native void setFieldSolver(long h, int kind, int iterations, double damping);

    // diagnostics
    /** BulkQuantitiesInTime / FieldMeasurements: e2[3], b2[3], px, py, pz, gauss, rho2, e2 total, b2 total */
    public static native void reduce(long h, double[] out13);
    /** n steps with the BulkQuantities row of each: 13 n doubles */
    public static native void stepMeasured(long h, int n, double[] rows13n);
    public static native void energyDensity(long h, double[] outV);
    /** 4 rows of dims[dir]: T_el, T_mag, L_el, L_mag */
    public static native void projectedEnergy(long h, int dir, double[] out4n);
    public static native void projectedPoynting(long h, int dir, double[] out2n);
    public static native void gaussField(long h, double[] out);

    // particles (CGCParticle list; InterpolatorAlgorithm and ParticleSolver run on the device)
    public static native void particlesUpload(long h, double[] pos0, double[] pos1, double[] vel, double[] q0,
                                              double[] q1, int[] dir);
    public static native void particlesDownload(long h, double[] pos0, double[] pos1, double[] vel, double[] q0,
                                                double[] q1, int[] dir, byte[] updateCharge);
    public static native long particlesCount(long h);
    public static native void cpicPhases(long h, int reassign);
    /** MVModel nuclei: ints {direction, orientation, useSeed, seed} and reals {location, width, mu,
     *  ultravioletCutoffTransverse, longitudinalCoherenceLength, infraredCoefficient} per nucleus */
    public static native void cgcMV(long h, int[] ints, double[] reals, int n);

    // gradients (SU(2); no counterpart in the reference)
    /** J with the initial E moved by step * (dE + the Gauss-law response to drho); dE, drho may be null */
    public static native double objectiveValue(long h, int kind, int direction, int[] lo, int[] hi, int nsteps,
                                               double[] dE, double[] drho, double step);
    /** {J, dJ} of the FP64 tangent-linear run along dE and drho */
    public static native double[] objectiveTangent(long h, int kind, int direction, int[] lo, int[] hi, int nsteps,
                                                   double[] dE, double[] drho);
    /** fills grad (V*3*3 for WRT_E, V*3 for WRT_RHO) and returns J */
    public static native double objectiveGradient(long h, int kind, int direction, int[] lo, int[] hi, int nsteps,
                                                  int ckpt, int wrt, double[] grad);
}
