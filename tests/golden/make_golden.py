"""Regenerates the golden fixtures in this folder from the oracle (oracle/refcpu, the CPU
restatement of the reference's Java path) on seeded synthetic stacks:

  offline_64.npz   64^2 3x3 float32 stack -> 128^2 (SimAlgorithm.runReconstruction, fade 10)
  offline_128.npz  128^2 3x3 float32 stack -> 256^2, the float64 oracle's image (stored as
                   float32), and the shifts, phases and modulations that estimateParameters
                   fits on the same stack
  live_64.npz      64^2 3x3 uint16 stack -> 128^2 and the widefield (ReconstructionThread)

Each file holds the raw stack, the parameters (px/py of the highest band in display
coordinates, phase offsets, modulation, optics) and the expected outputs. The reference
itself (Java) cannot run here, so these pin the oracle and the GPU path against drift; they
are not reference outputs. Run: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def params_of(truth):
    return dict(pxpy=np.array(truth["pxpy"], np.float64), phi0=np.array(truth["phi0"], np.float64),
                modulation=np.float64(truth["modulation"]), na=np.float64(truth["na"]),
                em_wavelength=np.float64(truth["em_wavelength"]), pxl_um=np.float64(truth["pxl_um"]),
                otf_a=np.float64(truth["otf_a"]))


def main():
    import __graft_entry__ as g
    from oracle import refcpu

    fs = g.load_package()
    refcpu.build()
    refcpu.set_threads(1)
    rng_seeds = {"offline_64": 11, "offline_128": 12, "live_64": 13}

    raw, truth = fs.synth.make_dataset(n=64, seed=rng_seeds["offline_64"])
    sp = fs.synth.sim_param_for(truth, 64)
    np.savez_compressed(os.path.join(HERE, "offline_64.npz"), raw=raw, out=refcpu.recon_raw(sp, raw, fade=10),
                        **params_of(truth))

    raw, truth = fs.synth.make_dataset(n=128, seed=rng_seeds["offline_128"])
    sp = fs.synth.sim_param_for(truth, 128)
    out = refcpu.recon_raw(sp, raw, fade=10)
    out64 = refcpu.recon_raw(sp, raw.astype(np.float64), fade=10, dtype=np.float64).astype(np.float32)
    spe = fs.synth.sim_param_for(truth, 128)
    spe.directions = [fs.Dir(2, 3) for _ in range(3)]
    est, peaks, _ = refcpu.estimate(spe, refcpu.prepare_raw(spe, raw), 1, 0.6)
    np.savez_compressed(os.path.join(HERE, "offline_128.npz"), raw=raw, out=out, out64=out64,
                        est_px=np.array(est["pX"][:3]), est_py=np.array(est["pY"][:3]),
                        est_pha=np.array(est["phaOff"][:3]), est_mod=np.array([m[1] for m in est["modulations"][:3]]),
                        **params_of(truth))

    raw, truth = fs.synth.make_dataset(n=64, seed=rng_seeds["live_64"], as_u16=True)
    sp = fs.synth.sim_param_for(truth, 64)
    rec, wf = refcpu.live_recon(sp, raw)
    np.savez_compressed(os.path.join(HERE, "live_64.npz"), raw=raw, out=rec[0], widefield=wf[0], **params_of(truth))



if __name__ == "__main__":
    main()
