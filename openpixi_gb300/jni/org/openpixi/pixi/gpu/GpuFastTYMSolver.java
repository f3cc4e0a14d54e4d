package org.openpixi.pixi.gpu;

import org.openpixi.pixi.math.AlgebraElement;
import org.openpixi.pixi.math.GroupElement;
import org.openpixi.pixi.math.SU2GroupElement;
import org.openpixi.pixi.math.SU3GroupElement;
import org.openpixi.pixi.physics.fields.FieldSolver;
import org.openpixi.pixi.physics.grid.Grid;

/**
 * FastTYMSolver on the GPU as a FieldSolver drop-in (physics/fields/FieldSolver.java:63-69)
 * with the host Grid authoritative: every step copies U, E and J to the device
 * and E and Unext back (Grid.getU/getE/getJ/getUnext, Grid.java:126-261).  A
 * simulation whose fields can stay on the device calls Opixi.step on a handle
 * instead and downloads only for diagnostics.  The handle is created on the
 * first call from the grid's shape, spacings, coupling and time step, and its
 * activity mask from Grid.isActive.
 */
public class GpuFastTYMSolver extends FieldSolver {
    private long handle = 0;
    private int nc, ng, V;
    private double[] links, alg;

    private void ensure(Grid g, double timeStep) {
        if (handle != 0) return;
        nc = g.getNumberOfColors();
        ng = nc == 2 ? 4 : 18;
        V = g.getTotalNumberOfCells();
        int[] dims = g.getNumCells();
        double[] a = {g.getLatticeSpacing(0), g.getLatticeSpacing(1), g.getLatticeSpacing(2)};
        handle = Opixi.create(nc, dims, a, timeStep, g.getGaugeCoupling(), Opixi.F64, 0, 0);
        links = new double[V * 3 * ng];
        alg = new double[V * 3 * (nc * nc - 1)];
        byte[] active = new byte[V];
        boolean all = true;
        for (int s = 0; s < V; s++) {
            active[s] = (byte) (g.isActive(s) ? 1 : 0);
            all &= g.isActive(s);
        }
        Opixi.setActive(handle, all ? null : active);
    }

    private static double linkComponent(GroupElement u, int c, int nc) {
        return nc == 2 ? ((SU2GroupElement) u).get(c) : ((SU3GroupElement) u).get(c);
    }

    private static void setLinkComponent(GroupElement u, int c, double v, int nc) {
        if (nc == 2) ((SU2GroupElement) u).set(c, v);
        else ((SU3GroupElement) u).set(c, v);
    }

    private void uploadLinks(Grid g) {
        for (int s = 0, k = 0; s < V; s++)
            for (int d = 0; d < 3; d++) {
                GroupElement u = g.getU(s, d);
                for (int c = 0; c < ng; c++) links[k++] = linkComponent(u, c, nc);
            }
        Opixi.upload(handle, Opixi.FIELD_U, links, Opixi.LAYOUT_REF);
    }

    private void uploadAlgebra(Grid g, int field) {
        final int na = nc * nc - 1;
        for (int s = 0, k = 0; s < V; s++)
            for (int d = 0; d < 3; d++) {
                AlgebraElement e = field == Opixi.FIELD_E ? g.getE(s, d) : g.getJ(s, d);
                for (int a = 0; a < na; a++) alg[k++] = e.get(a);
            }
        Opixi.upload(handle, field, alg, Opixi.LAYOUT_GEN);
    }

    private void downloadE(Grid g) {
        final int na = nc * nc - 1;
        Opixi.download(handle, Opixi.FIELD_E, alg, Opixi.LAYOUT_GEN);
        for (int s = 0, k = 0; s < V; s++)
            for (int d = 0; d < 3; d++) {
                AlgebraElement e = g.getE(s, d);
                for (int a = 0; a < na; a++) e.set(a, alg[k++]);
            }
    }

    private void downloadUnext(Grid g) {
        Opixi.download(handle, Opixi.FIELD_UNEXT, links, Opixi.LAYOUT_REF);
        for (int s = 0, k = 0; s < V; s++)
            for (int d = 0; d < 3; d++) {
                GroupElement u = g.getUnext(s, d);
                for (int c = 0; c < ng; c++) setLinkComponent(u, c, links[k++], nc);
            }
    }

    @Override
    public void step(Grid g, double timeStep) {
        ensure(g, timeStep);
        uploadLinks(g);
        uploadAlgebra(g, Opixi.FIELD_E);
        uploadAlgebra(g, Opixi.FIELD_J);
        Opixi.updateGrid(handle);
        downloadE(g);
        downloadUnext(g);
    }

    @Override
    public void stepLinks(Grid g, double timeStep) {
        ensure(g, timeStep);
        uploadLinks(g);
        uploadAlgebra(g, Opixi.FIELD_E);
        Opixi.stepLinks(handle);
        downloadUnext(g);
    }

    @Override
    public FieldSolver clone() {
        return new GpuFastTYMSolver();
    }

    /** releases the device fields */
    public void close() {
        if (handle != 0) Opixi.destroy(handle);
        handle = 0;
    }
}
