"""Pins the oracle's vector operations to the reference's own code (no GPU).

The fixture tests/golden/stdc_vector_ops.npz holds outputs of the reference's standard-C
vector backend (accel/stdC_cplx.c, accel/stdC_real.c), made by
tests/golden/make_stdc_golden.py. The oracle's pasteFreq must equal them bit for bit and its
fourierShift (float phase, as linalg/BasicVectors.java:309-339) must agree to float rounding.
Where a reference checkout is at hand (FSIM_REFERENCE_ROOT), the backend is compiled
(oracle/Makefile, `make ref`) and the fixture is checked against a fresh run of it, and the
oracle against it on further sizes."""
import os
import sys

import numpy as np
import pytest

from conftest import rel_l2

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_stdc_golden as G  # noqa: E402

FIX = os.path.join(HERE, "golden", "stdc_vector_ops.npz")


@pytest.fixture(scope="module")
def fx():
    return dict(np.load(FIX))


def test_oracle_paste_freq_equals_reference(fx, oracle):
    for i, (wi, wo, xo, yo) in enumerate(G.PASTE):
        got = oracle.paste_freq(fx["paste_in_%d" % i], wo, wo, xo, yo).astype(np.complex64)
        assert np.array_equal(got, fx["paste_out_%d" % i]), i


def test_oracle_fourier_shift_agrees_with_reference(fx, oracle):
    for i, (N, kx, ky) in enumerate(G.SHIFTS):
        z = fx["shift_in_%d" % i]
        ref = fx["shift_out_%d" % i]
        # both round the phase to float before sin/cos; they differ in the sin/cos rounding only
        assert rel_l2(oracle.fourier_shift(z, kx, ky, dtype=np.float32), ref) < 1e-6, i
        # against exact phases the reference's own float phase error shows (grows with |k|)
        assert rel_l2(oracle.fourier_shift(z.astype(np.complex128), kx, ky, dtype=np.float64), ref) < 1e-5, i


def test_fixture_elementwise_follow_float_arithmetic(fx):
    """The reference's element-wise natives are plain float arithmetic in a fixed order: the
    formulas the library's kernels (and the oracle's Java restatement) implement."""
    a, b, r, s = fx["a"], fx["b"], fx["r"], fx["s"]
    ar, ai, br, bi = a.real, a.imag, b.real, b.imag
    c = np.complex64(G.AXPY_A)
    assert np.array_equal(fx["c_add"], a + b)
    exp = (ar + (c.real * br - c.imag * bi)) + 1j * (ai + (c.imag * br + c.real * bi))
    assert np.array_equal(fx["c_axpy"], exp.astype(np.complex64))
    assert np.array_equal(fx["c_times"], ((ar * br - ai * bi) + 1j * (ar * bi + ai * br)).astype(np.complex64))
    assert np.array_equal(fx["c_times_conj"], ((ar * br + ai * bi) + 1j * (ai * br - ar * bi)).astype(np.complex64))
    assert np.array_equal(fx["c_times_real"], (ar * r + 1j * (ai * r)).astype(np.complex64))
    assert np.array_equal(fx["c_from_real"], r.astype(np.complex64))
    assert abs(fx["c_norm2"] - np.sum(ar.astype(np.float64) ** 2 + ai.astype(np.float64) ** 2)) < 1e-9 * fx["c_norm2"]
    assert np.array_equal(fx["r_add"], r + s)
    assert np.array_equal(fx["r_axpy"], r + np.float32(G.REAL_A) * s)
    assert np.array_equal(fx["r_times"], r * s)
    assert np.array_equal(fx["r_scal"], r * np.float32(G.REAL_A))


def test_fixture_reproduced_by_reference_backend(fx, oracle):
    from oracle import stdc_ref as S
    if not S.available():
        pytest.skip("FSIM_REFERENCE_ROOT unset: the reference's stdC backend cannot be built")
    d = {k: fx[k] for k in G.inputs()}
    for k, v in G.outputs(S, d).items():
        assert np.array_equal(np.asarray(v), fx[k]), k
    # further sizes: pasteFreq bit for bit, fourierShift to float rounding, straight against
    # the reference's code
    rng = np.random.default_rng(3)
    for wi, wo, xo, yo in ((128, 256, 11, -40), (96, 192, 0, 0), (256, 256, -9, 17)):
        z = (rng.standard_normal((wi, wi)) + 1j * rng.standard_normal((wi, wi))).astype(np.complex64)
        assert np.array_equal(oracle.paste_freq(z, wo, wo, xo, yo).astype(np.complex64), S.paste_freq(z, wo, wo, xo, yo))
    for N, kx, ky in ((256, 85.7, -6.7), (384, 12.3, 44.1)):
        z = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))).astype(np.complex64)
        assert rel_l2(oracle.fourier_shift(z, kx, ky, dtype=np.float32), S.fourier_shift(z, kx, ky)) < 1e-6
