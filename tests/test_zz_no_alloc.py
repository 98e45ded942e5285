"""The allocation-free correlation sweep (fsim_corr_grid_noalloc), called through the C ABI.

Callers that cannot allocate device memory mid-run use this entry point: a real-time
acquisition thread, whose latency budget has no room for the allocator, or a process whose
device memory was partitioned up front. Its scratch is a static device array. Its grid must
equal the first iteration grid of the allocating fit (fsim_fit_peak) on the same bands, bit
for bit, on two calls in a row (the second call reuses the scratch the first one left
behind); smaller grids and the largest size are checked against a direct FP64 evaluation.
This file is collected last so that a run stopping at the first failure has run every other
test before it."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(N_, b0_ptr, b1_ptr, n, kxs, kys, scal):
    kxs = np.ascontiguousarray(kxs, dtype=np.float64)
    kys = np.ascontiguousarray(kys, dtype=np.float64)
    out = np.zeros((len(kys), len(kxs), 2))
    rc = N_.lib().fsim_corr_grid_noalloc(
        C.c_void_p(b0_ptr), C.c_void_p(b1_ptr), n, kxs.ctypes.data_as(C.c_void_p), len(kxs),
        kys.ctypes.data_as(C.c_void_p), len(kys), C.c_double(scal), out.ctypes.data_as(C.c_void_p), None)
    N_.check(rc)
    return out[..., 0] + 1j * out[..., 1]


def _grid_fp64(b0, b1, kxs, kys, scal):
    """scal * sum_{x,y} b1 conj(b0) exp(+2 pi i (kx x - ky y)/n), separably in FP64."""
    n = b0.shape[0]
    p = b1.astype(np.complex128) * np.conj(b0.astype(np.complex128))
    x = np.arange(n)
    tx = np.exp(2j * np.pi * np.outer(kxs, x) / n)   # [jx][x]
    ty = np.exp(-2j * np.pi * np.outer(kys, x) / n)  # [jy][y]
    return scal * (ty @ (p @ tx.T))                   # [jy][jx]


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
        got = _noalloc(N_, b0.device_ptr(), b1.device_ptr(), n, kxs, kys, scal)
        assert np.array_equal(got, expect), call
    # grids narrower than 10 (1 x 1, 3 x 7) right after a 10 x 10 call, whose ramps and row
    # sums are still in the scratch, against a direct FP64 evaluation
    h0, h1 = b0.vectorData(), b1.vectorData()
    for gx, gy in ((1, 1), (3, 7), (7, 3)):
        _noalloc(N_, b0.device_ptr(), b1.device_ptr(), n, kxs, kys, scal)
        got = _noalloc(N_, b0.device_ptr(), b1.device_ptr(), n, kxs[:gx], kys[:gy], scal)
        ref = _grid_fp64(h0, h1, kxs[:gx], kys[:gy], scal)
        assert got.shape == (gy, gx)
        assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max(), (gx, gy)


def test_noalloc_largest_size_vs_fp64(fs, torch_cuda):
    """n = 2048, the largest size the static scratch holds, twice in a row."""
    torch = torch_cuda
    N_ = fs.native
    N_.init(0)
    n = 2048
    rng = np.random.default_rng(7)
    b0 = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))).astype(np.complex64)
    b1 = (0.5 * np.roll(b0, (3, -5), axis=(0, 1)) + 0.1 * rng.standard_normal((n, n))).astype(np.complex64)
    d0 = torch.from_numpy(b0.view(np.float32)).cuda()
    d1 = torch.from_numpy(b1.view(np.float32)).cuda()
    kxs = np.array([5.0 + (i - 4.5) / 4.5 * 0.5 for i in range(10)])
    kys = np.array([-3.0 + (i - 4.5) / 4.5 * 0.5 for i in range(10)])
    scal = 1.0 / float(np.sum(np.abs(b0.astype(np.complex128)) ** 2))
    ref = _grid_fp64(b0, b1, kxs, kys, scal)
    for call in range(2):
        got = _noalloc(N_, d0.data_ptr(), d1.data_ptr(), n, kxs, kys, scal)
        assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max(), call


def test_noalloc_rejects_sizes_beyond_scratch(fs):
    N_ = fs.native
    N_.init(0)
    k = np.zeros(11)
    out = np.zeros(242)
    dummy = C.c_void_p(1)
    for n, nx, ny in ((4096, 10, 10), (256, 11, 10), (256, 10, 0)):
        rc = N_.lib().fsim_corr_grid_noalloc(dummy, dummy, n, k.ctypes.data_as(C.c_void_p), nx,
                                             k.ctypes.data_as(C.c_void_p), ny, C.c_double(1.0),
                                             out.ctypes.data_as(C.c_void_p), None)
        assert rc == N_.FSIM_EINVAL
        assert b"static scratch" in N_.lib().fsim_last_error()
