/*
 * Fused GB300 entry points for fairSIM's Java code (natives in jni/fsim_jni.cpp, over the C
 * ABI include/fairsim_gb300.h). The vector path needs no new Java: the reference's accel
 * classes (org.fairsim.accel.AccelVector*) load the same library and call its
 * Java_org_fairsim_accel_* symbols. This class adds what the reference lacks: a whole
 * reconstruction per call, batches, and the parameter fit on the device.
 *
 * Typical use, replacing SimAlgorithm.runReconstruction (SimAlgorithm.java:268):
 *
 *   FusedSim.Plan plan = FusedSim.plan(param, w, 1.4, 525, 1.0, FusedSim.PATH_OFFLINE,
 *                                      FusedSim.INPUT_F32, 10, 0.0);
 *   float [] out = new float[4*w*w];
 *   plan.reconstruct(rawStack, out);     // nDirs*nPhases*w*w floats in, 2w x 2w out
 *   plan.close();
 */
package org.fairsim.gb300;

import org.fairsim.sim_algorithm.SimParam;

public final class FusedSim {

    public static final int PATH_OFFLINE = 0;   // SimAlgorithm.runReconstruction
    public static final int PATH_LIVE = 1;      // ReconstructionRunner's per-stack work
    public static final int INPUT_F32 = 0;
    public static final int INPUT_U16 = 1;

    static {
	System.loadLibrary("fairsim_gb300_jni");
    }

    private FusedSim() {}

    /** The flat records the natives take, filled from a SimParam (SimParam.java:191-607). */
    static int [] geometry(SimParam p, int w) {
	return new int [] { w, p.nrDir(), p.nrBand(), p.dir(0).nrPha(),
	    (p.otf() != null && p.otf().isAttenuate()) ? 1 : 0 };
    }

    static double [] optics(SimParam p, int w, double na, double lambdaNm, double otfA) {
	double att = 0, fwhm = 0;
	if (p.otf() != null) {
	    att = p.otf().getAttStr(0);
	    fwhm = p.otf().getAttFWHM(0);
	}
	return new double [] { 1.0 / (w * p.pxlSizeCyclesMicron()), na, lambdaNm, otfA, att, fwhm,
	    p.getWienerFilter(), p.getApoCutoff(), 0.9 };
    }

    static double [] directions(SimParam p) {
	int nb = p.nrBand();
	double [] d = new double[p.nrDir() * (3 + nb)];
	for (int i = 0; i < p.nrDir(); i++) {
	    SimParam.Dir dir = p.dir(i);
	    d[i*(3+nb)+0] = dir.px(1);
	    d[i*(3+nb)+1] = dir.py(1);
	    d[i*(3+nb)+2] = dir.getPhaOff();
	    double [] m = dir.getModulations();
	    for (int b = 0; b < nb; b++) d[i*(3+nb)+3+b] = m[b];
	}
	return d;
    }

    /** A parameter set's resident filters on the device. */
    public static final class Plan implements AutoCloseable {
	long handle;
	final int w;
	Plan(long h, int w) { this.handle = h; this.w = w; }

	/** raw: float[] (INPUT_F32) or short[] (INPUT_U16); out: float[4*w*w] */
	public void reconstruct(Object raw, float [] out) { reconstruct(handle, raw, out); }

	/** The reconstruction plus runReconstruction's "Widefield" and "filtered Widefield"
	 *  images (SimAlgorithm.java:533-576; offline plans): wf, fwf float[4*w*w], either null */
	public void reconstruct(Object raw, float [] out, float [] wf, float [] fwf) {
	    reconstructWidefield(handle, raw, out, wf, fwf);
	}

	/** New shifts / phases / modulations (same geometry). */
	public void update(SimParam p, double na, double lambdaNm, double otfA) {
	    planUpdate(handle, geometry(p, w), optics(p, w, na, lambdaNm, otfA), directions(p));
	}

	@Override public void close() {
	    if (handle != 0) planDestroy(handle);
	    handle = 0;
	}
    }

    public static Plan plan(SimParam p, int w, double na, double lambdaNm, double otfA,
	int path, int inputType, int fadePx, double background) {
	return new Plan(planCreate(geometry(p, w), optics(p, w, na, lambdaNm, otfA), directions(p),
	    path, inputType, fadePx, background), w);
    }

    /** Many stacks in one call; uploads, passes and downloads overlap. */
    public static void reconstructBatch(Plan [] plans, Object [] raws, float [][] outs) {
	long [] h = new long[plans.length];
	for (int i = 0; i < h.length; i++) h[i] = plans[i].handle;
	reconstructBatch(h, raws, outs);
    }

    /** SimAlgorithm.estimateParameters (SimAlgorithm.java:37) on a raw float stack; the
     *  fitted shifts, phases and modulations are written into p. */
    public static void estimateParameters(SimParam p, int w, double na, double lambdaNm, double otfA,
	float [] raw, int fadePx, int fitBand, double fitExclude) {
	double [] d = directions(p);
	estimate(geometry(p, w), optics(p, w, na, lambdaNm, otfA), d, raw, fadePx, fitBand, fitExclude);
	int nb = p.nrBand();
	for (int i = 0; i < p.nrDir(); i++) {
	    SimParam.Dir dir = p.dir(i);
	    dir.setPxPy(d[i*(3+nb)+0] * (nb - 1), d[i*(3+nb)+1] * (nb - 1));
	    dir.setPhaOff(d[i*(3+nb)+2]);
	    for (int b = 1; b < nb; b++) dir.setModulation(b, d[i*(3+nb)+3+b]);
	}
    }

    static native long planCreate(int [] geom, double [] optics, double [] dirs, int path,
	int inputType, int fadePx, double bgr);
    static native void planUpdate(long plan, int [] geom, double [] optics, double [] dirs);
    static native void planDestroy(long plan);
    static native void reconstruct(long plan, Object raw, float [] out);
    static native void reconstructWidefield(long plan, Object raw, float [] out, float [] wf, float [] fwf);
    static native void reconstructBatch(long [] plans, Object [] raws, float [][] outs);
    static native void estimate(int [] geom, double [] optics, double [] dirs, float [] raw,
	int fadePx, int fitBand, double fitExclude);
}
