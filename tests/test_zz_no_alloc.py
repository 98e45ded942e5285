"""The allocation-free correlation sweep (fsim_corr_grid_noalloc), called through the C ABI.

Callers that cannot allocate device memory mid-run (real-time acquisition threads, work
captured into a CUDA graph, processes with pre-partitioned device memory) use this entry
point; its scratch is a static device array. Its grid must equal the first iteration grid
of the allocating fit (fsim_fit_peak) on the same bands, on two calls in a row (the second
call reuses the scratch the first one left behind). This file is collected last so that a
run stopping at the first failure has run every other test before it."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_grid_matches_fit_peak_twice(fs, oracle):
    N_ = fs.native
    N_.init(0)
    V, A = fs.vectors, fs.algorithm
    n = 256
    raw, truth = fs.synth.make_dataset(n=n, seed=123)
    sp = fs.synth.sim_param_for(truth, n, known=False)
    spec = oracle.prepare_raw(sp, raw)
    sep = oracle.separate_bands(sp, 0, spec[:3])
    k = truth["pxpy"][0]
    kx, ky, search = -round(k[0]), -round(k[1]), 2.5

    def cvec(z):
        v = V.Vec2dCplx(n, n)
        v.setData(z.astype(np.complex64))
        return v

    # reference: the allocating fit, first iteration's 10 x 10 grid
    grid = np.zeros((3, 10, 10, 2))
    A.Correlation.fitPeak(cvec(sep[0]), cvec(sep[1]), 0, 1, sp, kx, ky, 0.05, search, grid)
    expect = grid[0, ..., 0] + 1j * grid[0, ..., 1]
    # the same bands prepared by the caller: common region, inverse FFT, normaliser
    b0, b1 = cvec(sep[0]), cvec(sep[1])
    A.Correlation.commonRegion(b0, b1, 0, 1, sp, kx, ky, 0.15, 0.05, True)
    b0.fft2d(True)
    b1.fft2d(True)
    N_.check(N_.lib().fsim_sync())
    scal = 1.0 / b0.norm2()
    kxs = np.array([kx + ((i - 4.5) / 4.5) * search for i in range(10)])
    kys = np.array([ky + ((i - 4.5) / 4.5) * search for i in range(10)])
    for call in range(2):
        out = np.zeros((10, 10, 2))
        rc = N_.lib().fsim_corr_grid_noalloc(
            C.c_void_p(b0.device_ptr()), C.c_void_p(b1.device_ptr()), n,
            kxs.ctypes.data_as(C.c_void_p), 10, kys.ctypes.data_as(C.c_void_p), 10,
            C.c_double(scal), out.ctypes.data_as(C.c_void_p), None)
        N_.check(rc)
        got = out[..., 0] + 1j * out[..., 1]
        assert np.abs(got - expect).max() <= 1e-12 * np.abs(expect).max(), call


def test_noalloc_rejects_sizes_beyond_scratch(fs):
    N_ = fs.native
    N_.init(0)
    k = np.zeros(10)
    out = np.zeros(200)
    dummy = C.c_void_p(1)
    rc = N_.lib().fsim_corr_grid_noalloc(dummy, dummy, 4096, k.ctypes.data_as(C.c_void_p), 10,
                                         k.ctypes.data_as(C.c_void_p), 10, C.c_double(1.0),
                                         out.ctypes.data_as(C.c_void_p), None)
    assert rc == N_.FSIM_EINVAL
    assert b"static scratch" in N_.lib().fsim_last_error()
