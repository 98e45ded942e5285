"""Regenerates tests/golden/stdc_vector_ops.npz from the reference's own standard-C vector
backend (accel/stdC_cplx.c, accel/stdC_real.c: the JNI natives of AccelVectorCplx /
AccelVectorReal when the accel factory runs on the CPU), built from a reference checkout by
oracle/Makefile (`make ref`) and called through oracle/stdc_ref.py.

The fixture holds seeded inputs and the reference's outputs of every compute native that
needs no JNI environment: complex add, axpy, times (plain and conjugate), times-real, scal,
norm2 and copy-from-real; real add, axpy, times, scal, sum and norm2; pasteFreq (zero
padding with offsets) and fourierShift. tests/test_ref_stdc.py pins the oracle to it (and,
where the reference is at hand, checks the fixture against a fresh run), and
tests/test_gpu_vector_api.py checks the library's device kernels against it.

Run: FSIM_REFERENCE_ROOT=<reference checkout> python tests/golden/make_stdc_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

AXPY_A = complex(0.5, -0.25)
SCAL_A = complex(-1.25, 0.75)
REAL_A = 0.375
PASTE = [(16, 32, 0, 0), (16, 32, 5, -7), (24, 48, -3, 2), (32, 32, 3, 1)]  # wi, wo, xoff, yoff
SHIFTS = [(32, 3.3, -7.7), (48, 20.9, 13.1), (64, -0.37, 0.81)]          # N, kx, ky


def inputs():
    rng = np.random.default_rng(20251204)
    n = 32
    c = lambda *s: (rng.standard_normal(s) + 1j * rng.standard_normal(s)).astype(np.complex64)  # noqa: E731
    d = dict(a=c(n, n), b=c(n, n), r=rng.standard_normal((n, n)).astype(np.float32),
             s=rng.standard_normal((n, n)).astype(np.float32))
    for i, (wi, wo, xo, yo) in enumerate(PASTE):
        d["paste_in_%d" % i] = c(wi, wi)
    for i, (N, kx, ky) in enumerate(SHIFTS):
        d["shift_in_%d" % i] = c(N, N)
    return d


def outputs(S, d):
    a, b, r, s = d["a"], d["b"], d["r"], d["s"]
    o = dict(c_add=S.cplx_add(a, b), c_axpy=S.cplx_axpy(AXPY_A, a, b), c_times=S.cplx_times(a, b),
             c_times_conj=S.cplx_times(a, b, conj=True), c_times_real=S.cplx_times_real(a, r),
             c_scal=S.cplx_scal(a, SCAL_A), c_norm2=np.float64(S.cplx_norm2(a)), c_from_real=S.cplx_from_real(r),
             r_add=S.real_add(r, s), r_axpy=S.real_axpy(REAL_A, r, s), r_times=S.real_times(r, s),
             r_scal=S.real_scal(r, REAL_A), r_sum=np.float64(S.real_reduce(r, False)),
             r_norm2=np.float64(S.real_reduce(r, True)))
    for i, (wi, wo, xo, yo) in enumerate(PASTE):
        o["paste_out_%d" % i] = S.paste_freq(d["paste_in_%d" % i], wo, wo, xo, yo)
    for i, (N, kx, ky) in enumerate(SHIFTS):
        o["shift_out_%d" % i] = S.fourier_shift(d["shift_in_%d" % i], kx, ky)
    return o


def main():
    from oracle import stdc_ref as S
    if not S.build():
        sys.exit("set FSIM_REFERENCE_ROOT to a reference checkout (its accel/stdC_*.c are compiled)")
    d = inputs()
    np.savez_compressed(os.path.join(HERE, "stdc_vector_ops.npz"), **d, **outputs(S, d))
    print("wrote stdc_vector_ops.npz")


if __name__ == "__main__":
    main()
