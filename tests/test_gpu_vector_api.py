"""GPU parity of the Vector API kernels (the replacements of the reference's JNI vector
natives, org/fairsim/accel/AccelVectorCplx.java:296-331) and of the SIM building blocks,
called through the C ABI and checked against the oracle (float instantiation = the
reference's semantics) or numpy. This follows the reference's own agreement harness
(org/fairsim/accel/TestAccel.java:399-443), with thresholds."""
import math

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def V(fs):
    fs.native.init(0)
    return fs.vectors


def cvec(V, z):
    v = V.Vec2dCplx(z.shape[1], z.shape[0])
    v.setData(z.astype(np.complex64))
    return v


def rvec(V, a):
    v = V.Vec2dReal(a.shape[1], a.shape[0])
    v.setData(a.astype(np.float32))
    return v


@pytest.mark.parametrize("w,h", [(64, 64), (96, 96), (128, 256), (384, 384), (512, 512), (768, 768),
                                 (1024, 1024), (2048, 2048), (1536, 1536), (4096, 4096)])
def test_fft2d_vs_numpy(V, w, h):
    rng = np.random.default_rng(w + h)
    z = (rng.standard_normal((h, w)) + 1j * rng.standard_normal((h, w))).astype(np.complex64)
    v = cvec(V, z)
    v.fft2d(False)
    assert rel_l2(v.vectorData(), np.fft.fft2(z.astype(np.complex128))) < 3e-6
    v.fft2d(True)
    assert rel_l2(v.vectorData(), z) < 3e-6


def test_elementwise_ops(V):
    rng = np.random.default_rng(1)
    n = 96
    a = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))).astype(np.complex64)
    b = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))).astype(np.complex64)
    r = rng.standard_normal((n, n)).astype(np.float32)
    va, vb, vr = cvec(V, a), cvec(V, b), rvec(V, r)
    va.axpy(0.5 - 0.25j, vb)
    c = np.complex64(0.5 - 0.25j)
    exp = a.copy()
    exp.real = a.real + (np.float32(c.real) * b.real - np.float32(c.imag) * b.imag)
    exp.imag = a.imag + (np.float32(c.imag) * b.real + np.float32(c.real) * b.imag)
    assert np.array_equal(va.vectorData(), exp)  # AbstractVectorCplx.axpy rounding, bit-exact
    va.setData(a)
    va.timesConj(vb)
    assert rel_l2(va.vectorData(), a * np.conj(b)) < 1e-7
    va.setData(a)
    va.times(vr)
    assert np.array_equal(va.vectorData(), a * r)
    va.setData(a)
    assert abs(va.norm2() - float(np.sum(a.real.astype(np.float32) ** 2 + a.imag.astype(np.float32) ** 2, dtype=np.float64))) < 1e-9 * va.norm2()
    s = va.sumElements()
    assert abs(s - complex(np.sum(a.astype(np.complex128)))) < 1e-9 * abs(s) + 1e-9
    d = va.dot(vb)
    assert abs(d - complex(np.vdot(a.astype(np.complex128), b.astype(np.complex128)))) < 1e-5 * abs(d)
    vr2 = V.Vec2dReal(n, n)
    vr2.copy(va)
    assert np.array_equal(vr2.vectorData(), a.real)
    va.scal(2.0)
    assert np.array_equal(va.vectorData(), a * np.float32(2))


def test_set_from_16bit_pixels(V):
    rng = np.random.default_rng(2)
    u = rng.integers(0, 65535, (64, 64), dtype=np.uint16)
    v = V.Vec2dCplx(64, 64)
    v.setFrom16bitPixels(u)
    assert np.array_equal(v.vectorData(), u.astype(np.float32).astype(np.complex64))


@pytest.mark.parametrize("wi,wo,xo,yo", [(64, 128, 0, 0), (64, 128, 5, -7), (48, 96, -3, 2), (64, 64, 3, 1)])
def test_paste_freq_vs_oracle(V, oracle, wi, wo, xo, yo):
    rng = np.random.default_rng(wi + wo)
    z = (rng.standard_normal((wi, wi)) + 1j * rng.standard_normal((wi, wi))).astype(np.complex64)
    vin, vout = cvec(V, z), V.Vec2dCplx(wo, wo)
    vout.pasteFreq(vin, xo, yo)
    assert np.array_equal(vout.vectorData(), oracle.paste_freq(z, wo, wo, xo, yo).astype(np.complex64))


@pytest.mark.parametrize("n,kx,ky", [(512, 185.7, -6.7), (1024, -100.9, 155.9), (384, 12.3, 44.1), (1024, 0.37, -0.81)])
def test_fourier_shift_vs_oracle(V, oracle, n, kx, ky):
    rng = np.random.default_rng(n)
    z = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))).astype(np.complex64)
    v = cvec(V, z)
    v.fourierShift(kx, ky)
    got = v.vectorData()
    f64 = oracle.fourier_shift(z.astype(np.complex128), kx, ky, dtype=np.float64)
    f32 = oracle.fourier_shift(z, kx, ky, dtype=np.float32)
    # phase reduced exactly before sin/cos: close to FP64; the reference's float phase is within 1e-4
    assert rel_l2(got, f64) < 2e-7
    assert rel_l2(got, f32) < 1e-4


def test_otf_vectors_vs_oracle(V, oracle, fs):
    n = 256
    otf = fs.OtfProvider.fromEstimate(1.4, 525, 0.4)
    otf.setAttenuation(0.95, 1.4)
    otf.switchAttenuation(True)
    sp = fs.SimParam.create(2, 3, 3, n, 0.08, otf)
    A = fs.algorithm.OtfVectors
    for (kx, ky, which, write, att) in [(0, 0, 0, True, False), (37.2, -81.6, 0, True, False),
                                        (12.5, 9.25, 1, True, True)]:
        v = V.Vec2dCplx(n, n)
        A.otfToVector(sp, v, 0, kx, ky, att, write)
        exp = oracle.otf_vector(sp, np.zeros((n, n), complex), kx, ky, which=which)
        assert np.array_equal(v.vectorData(), exp.astype(np.complex64))
    rng = np.random.default_rng(3)
    z = (rng.standard_normal((2 * n, 2 * n)) + 1j * rng.standard_normal((2 * n, 2 * n))).astype(np.complex64)
    v = cvec(V, z)
    A.applyOtf(sp, v, 0, 100.5, -40.25)
    assert np.array_equal(v.vectorData(), oracle.otf_vector(sp, z, 100.5, -40.25, which=2).astype(np.complex64))
    ra = V.Vec2dReal(2 * n, 2 * n)
    A.writeApoVector(sp, ra, 0.9, 2.0)
    assert rel_l2(ra.vectorData(), oracle.apo_vector(sp, 2 * n, 2 * n, 0.9, 2.0)) < 1e-7
    rt = V.Vec2dReal(n, n)
    cut = otf.getCutoff()
    A.writeAttenuationVector(sp, rt, 0.99, 0.15 * cut, 0, 0)
    assert rel_l2(rt.vectorData(), oracle.attenuation_vector(sp, n, n, 0.99, 0.15 * cut)) < 1e-7


def test_wiener_denominator_vs_oracle(V, oracle, fs):
    n = 256
    raw, truth = fs.synth.make_dataset(n=n, seed=3)
    sp = fs.synth.sim_param_for(truth, n)
    for att in (False, True):
        sp.otf().switchAttenuation(att)
        wd = fs.algorithm.WienerFilter(sp).getDenominator(sp.getWienerFilter())
        exp = oracle.wiener_denominator(sp)
        assert rel_l2(wd.vectorData(), exp) < 1e-7


def test_separate_bands_vs_oracle(V, oracle, fs):
    n = 128
    raw, truth = fs.synth.make_dataset(n=n, seed=5)
    sp = fs.synth.sim_param_for(truth, n)
    spec = oracle.prepare_raw(sp, raw)
    inv = [cvec(V, spec[p]) for p in range(3)]
    out = [V.Vec2dCplx(n, n) for _ in range(3)]
    d = sp.dir(0)
    fs.algorithm.BandSeparation.separateBands(inv, out, d.getPhases(), 2, d.getModulations())
    exp = oracle.separate_bands(sp, 0, spec[:3])
    for i in range(3):
        assert np.array_equal(out[i].vectorData(), exp[i].astype(np.complex64))


def test_correlation_fit_vs_oracle(V, oracle, fs):
    n = 256
    raw, truth = fs.synth.make_dataset(n=n, seed=6)
    sp = fs.synth.sim_param_for(truth, n, known=False)
    spec = oracle.prepare_raw(sp, raw)
    sep = oracle.separate_bands(sp, 0, spec[:3])  # phases 0, 2pi/3.. with modulation 1 -> fac .5
    k = truth["pxpy"][0]
    # commonRegion
    g0, g1 = cvec(V, sep[0]), cvec(V, sep[1])
    fs.algorithm.Correlation.commonRegion(g0, g1, 0, 1, sp, -k[0], -k[1], 0.15, 0.05, True)
    e0, e1 = oracle.common_region(sp, sep[0], sep[1], -k[0], -k[1])
    # the OTF weights come from float-float table positions: the same samples and cuts as the
    # reference's double precision, the interpolation weight at most a last bit apart, which
    # can move a divided value by an ulp
    for g, e in ((g0.vectorData(), e0.astype(np.complex64)), (g1.vectorData(), e1.astype(np.complex64))):
        d = g != e
        assert np.count_nonzero(d) <= 1e-4 * d.size
        assert np.all(np.abs(g[d] - e[d]) <= 3e-7 * np.abs(e[d]))
    # fitPeak: the grid maxima and therefore the fitted k must agree
    b0, b1 = cvec(V, sep[0]), cvec(V, sep[1])
    start = (-round(k[0]), -round(k[1]))
    grid = np.zeros((3, 10, 10, 2))
    got = fs.algorithm.Correlation.fitPeak(b0, b1, 0, 1, sp, start[0], start[1], 0.05, 2.5, grid)
    exp, egrid = oracle.fit_peak(sp, sep[0], sep[1], start[0], start[1])
    assert abs(got[0] - exp[0]) < 1e-9 and abs(got[1] - exp[1]) < 1e-9
    gg = grid[..., 0] + 1j * grid[..., 1]
    assert rel_l2(gg, egrid) < 1e-4
    assert abs(got[3] - exp[3]) < 1e-4 * abs(exp[3])
    p = fs.algorithm.Correlation.getPeak(b0, b1, 0, 1, sp, exp[0], exp[1], 0.05)
    ep = oracle.get_peak(sp, sep[0], sep[1], exp[0], exp[1])
    assert abs(p - ep) < 1e-4 * abs(ep)


@pytest.mark.parametrize("n", [256, 512])
def test_estimate_parameters_vs_oracle(V, oracle, fs, n):
    raw, truth = fs.synth.make_dataset(n=n, seed=8)
    sp = fs.synth.sim_param_for(truth, n, known=False)
    spec = oracle.prepare_raw(sp, raw)
    est, epeaks, _ = oracle.estimate(sp, spec, 1, 0.6)
    inFFT = [[cvec(V, spec[a * 3 + p]) for p in range(3)] for a in range(3)]
    gpeaks = fs.algorithm.SimAlgorithm.estimateParameters(sp, inFFT, 1, 0.6)
    for d in range(3):
        # same fitted k0 (the grid search picks the same point) and the same pixel
        assert abs(sp.dir(d).pX - est["pX"][d]) < 1e-9 and abs(sp.dir(d).pY - est["pY"][d]) < 1e-9
        assert round(sp.dir(d).pX) == round(truth["pxpy"][d][0]) and round(sp.dir(d).pY) == round(truth["pxpy"][d][1])
        assert abs(sp.dir(d).phaOff - est["phaOff"][d]) < 1e-4
        assert abs(sp.dir(d).modul[1] - est["modulations"][d][1]) < 1e-4


@pytest.mark.parametrize("n", [128, 512])
def test_run_reconstruction_op_by_op_vs_oracle(V, oracle, fs, n):
    raw, truth = fs.synth.make_dataset(n=n, seed=9)
    sp = fs.synth.sim_param_for(truth, n)
    spec = oracle.prepare_raw(sp, raw)
    exp32 = oracle.recon(sp, spec)
    exp64 = oracle.recon(sp, spec.astype(np.complex128), dtype=np.float64)
    inFFT = [[cvec(V, spec[a * 3 + p]) for p in range(3)] for a in range(3)]
    out = fs.algorithm.SimAlgorithm.runReconstruction(sp, inFFT, False, 0).vectorData()
    assert rel_l2(out, exp32) < 1e-4   # vs the reference's float semantics
    assert rel_l2(out, exp64) < 1e-5   # vs the FP64 oracle


@pytest.mark.parametrize("clip", [1, 2])
def test_run_reconstruction_clip_scale_vs_oracle(V, oracle, fs, clip):
    """runReconstruction's CLIPSCALE.CLIP and .BOTH outputs (SimUtils.spatial ->
    clipAndScale, S/SimUtils.java:146-153,244-264; BOTH is the reference's default)."""
    n = 256
    raw, truth = fs.synth.make_dataset(n=n, seed=19)
    sp = fs.synth.sim_param_for(truth, n)
    spec = oracle.prepare_raw(sp, raw)
    exp = oracle.recon(sp, spec, clip_scale=clip)
    inFFT = [[cvec(V, spec[a * 3 + p]) for p in range(3)] for a in range(3)]
    out = fs.algorithm.SimAlgorithm.runReconstruction(sp, inFFT, False, clip).vectorData()
    assert out.min() >= 0
    assert rel_l2(out, exp) < 1e-4
    if clip == 2:
        assert abs(out.max() - 255.0) < 1e-3 and abs(exp.max() - 255.0) < 1e-3


def test_accel_natives_set_get_reshape_plan_buffers(fs, V):
    """The remaining accel natives: nativeSet/nativeGet (element access), vectors allocated
    by element count and shaped by the call that needs a shape, nativeCreatePlan2d, and
    the factory's raw device / pinned host buffers."""
    import ctypes as C

    lib = fs.native.lib()
    rng = np.random.default_rng(9)
    z = (rng.standard_normal((64, 32)) + 1j * rng.standard_normal((64, 32))).astype(np.complex64)
    v = V.Vec2dCplx(64 * 32, 1)  # allocated by element count, like AccelVectorCplx.alloc
    fs.native.check(lib.fsim_vec_reshape(v.handle, 32, 64))
    v.setData(z)
    re, im = C.c_float(), C.c_float()
    fs.native.check(lib.fsim_vec_get_elem(v.handle, 5 + 7 * 32, C.byref(re), C.byref(im)))
    assert (re.value, im.value) == (float(z[7, 5].real), float(z[7, 5].imag))
    fs.native.check(lib.fsim_vec_set_elem(v.handle, 3 + 2 * 32, 1.5, -2.25))
    z[2, 3] = 1.5 - 2.25j
    plan = C.c_int64()
    fs.native.check(lib.fsim_fft_plan_2d(32, 64, C.byref(plan)))
    assert (plan.value >> 32, plan.value & 0xffffffff) == (32, 64)
    v.fft2d(False)
    assert rel_l2(v.vectorData().reshape(64, 32), np.fft.fft2(z.astype(np.complex128))) < 3e-6
    assert lib.fsim_vec_reshape(v.handle, 33, 64) == fs.native.FSIM_EINVAL
    assert lib.fsim_vec_set_elem(v.handle, 64 * 32, 0.0, 0.0) == fs.native.FSIM_EINVAL
    for host in (0, 1):
        p = C.c_void_p()
        fs.native.check(lib.fsim_buffer_alloc(8 << 20, host, C.byref(p)))
        assert p.value
        fs.native.check(lib.fsim_buffer_free(p, host))
    fs.native.check(lib.fsim_profiler(1))
    fs.native.check(lib.fsim_profiler(0))


# (512, 512, 6) and (256, 512, 12): the 512-point column pass with cp.async-pipelined tiles
# (at least two tiles per SM); the others the plain column pass
@pytest.mark.parametrize("w,h,batch", [(64, 64, 3), (384, 384, 2), (512, 256, 4), (512, 512, 6), (256, 512, 12)])
def test_fft2d_batch_on_device_buffers(fs, V, w, h, batch):
    import ctypes as C

    import torch

    rng = np.random.default_rng(w * h + batch)
    z = (rng.standard_normal((batch, h, w)) + 1j * rng.standard_normal((batch, h, w))).astype(np.complex64)
    d = torch.from_numpy(z).cuda()
    lib = fs.native.lib()
    fs.native.check(lib.fsim_fft2d_batch(C.c_void_p(d.data_ptr()), w, h, batch, 0, None))
    torch.cuda.synchronize()
    assert rel_l2(d.cpu().numpy(), np.fft.fft2(z.astype(np.complex128))) < 3e-6
    fs.native.check(lib.fsim_fft2d_batch(C.c_void_p(d.data_ptr()), w, h, batch, 1, None))
    torch.cuda.synchronize()
    assert rel_l2(d.cpu().numpy(), z) < 3e-6
    assert lib.fsim_fft2d_batch(C.c_void_p(d.data_ptr()), 100, h, batch, 0, None) == fs.native.FSIM_EINVAL


def test_rl_deconvolution_and_auto_correlation(fs, oracle, V):
    """RLDeconvolution.deconvolve and Correlation.autoCorrelation (Wicker) on device vectors
    against the oracle's float restatement (S/RLDeconvolution.java:45-103,
    S/Correlation.java:294-325)."""
    n = 128
    rng = np.random.default_rng(12)
    img = rng.uniform(50, 150, (n, n))
    k = np.fft.fftfreq(n)
    otf = (np.exp(-(k[None, :] ** 2 + k[:, None] ** 2) * 40) + 0j).astype(np.complex64)
    spec = np.fft.fft2(img).astype(np.complex64)
    v, o = cvec(V, spec), cvec(V, otf)
    fs.algorithm.RLDeconvolution.deconvolve(v, o, 5, True)
    exp = oracle.rl_deconvolve(spec, otf, 5, True)
    assert rel_l2(v.vectorData(), exp) < 1e-5
    band = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))).astype(np.complex64)
    got = fs.algorithm.Correlation.autoCorrelation(cvec(V, band), 7.3, -11.6)
    ref = oracle.auto_correlation(band, 7.3, -11.6)
    ref64 = oracle.auto_correlation(band, 7.3, -11.6, dtype=np.float64)
    assert abs(got - ref) < 1e-5 * abs(ref)
    assert abs(got - ref64) < 1e-5 * abs(ref64)


@pytest.mark.parametrize("style", [1, 2, 3])
def test_run_reconstruction_rl_styles_vs_oracle(fs, oracle, V, style):
    """runReconstruction with RL on the input, the output, or both (the op-by-op device path)
    against the oracle in float and FP64; raw frames carry a camera offset (RL divides by the
    blurred estimate and needs positive data to be well conditioned)."""
    n = 128
    raw, truth = fs.synth.make_dataset(n=n, seed=91)
    raw = raw + 200.0
    sp = fs.synth.sim_param_for(truth, n)
    sp.setFilterStyle(style)
    sp.setRLiterations(3)
    spec = oracle.prepare_raw(sp, raw)
    exp32 = oracle.recon(sp, spec)
    exp64 = oracle.recon(sp, spec.astype(np.complex128), dtype=np.float64)
    inFFT = [[cvec(V, spec[a * 3 + p]) for p in range(3)] for a in range(3)]
    out = fs.algorithm.SimAlgorithm.runReconstruction(sp, inFFT, False, 0).vectorData()
    assert rel_l2(out, exp32) < 1e-4
    assert rel_l2(out, exp64) < 1e-4
    with pytest.raises(ValueError):  # live plans take estimated OTFs only
        fs.plan.ReconPlan(sp, path=fs.native.PATH_LIVE, input_type=fs.native.INPUT_U16, fade_px=10)


def measured_otf(fs, samples=300, bands=2, spacing=256, na=1.4, lam=525.0, a=0.3):
    """A complex multi-band measured OTF (OtfProvider with band data): the estimate's shape
    with a per-band gain and a slow phase, `spacing` samples up to the cutoff."""
    cut = 1000 / (lam / na / 2)
    v = np.clip(np.arange(samples) / spacing, 0, 1)
    base = (2 / np.pi) * (np.arccos(v) - v * np.sqrt(1 - v * v)) * a ** v
    b = [(base * (1 - 0.1 * k) * np.exp(1j * 0.3 * (k + 1) * v)).tolist() for k in range(bands)]
    return fs.OtfProvider.fromMeasured(na, lam, b, cut / spacing)


@pytest.mark.parametrize("samples", [300, 200])
def test_measured_otf_reconstruction_and_filters_vs_oracle(V, oracle, fs, samples):
    """Measured two-band complex OTFs (OtfProvider.loadFromConfig with band data) through the
    op-by-op path: the band-1 OTF vector with and without attenuation, the Wiener
    denominator and the reconstruction against the oracle."""
    n = 128
    raw, truth = fs.synth.make_dataset(n=n, seed=41)
    sp = fs.synth.sim_param_for(truth, n)
    sp.setOtf(measured_otf(fs, samples=samples))
    sp.otf().setAttenuation(0.97, 1.1)
    sp.otf().switchAttenuation(True)
    for which, att in ((0, False), (1, True)):  # writeOtfVector, writeOtfWithAttVector
        v = V.Vec2dCplx(2 * n, 2 * n)
        fs.algorithm.OtfVectors.otfToVector(sp, v, 1, 10.5, -3.25, att, True)
        exp = oracle.otf_vector(sp, np.zeros((2 * n, 2 * n), complex), 10.5, -3.25, which=which, band=1)
        assert rel_l2(v.vectorData(), exp) < 1e-6
    # getAttVal reads past a table that ends inside the cutoff (the reference throws there)
    sp.otf().switchAttenuation(samples * sp.otf().measured["cycles"] >= sp.otf().getCutoff())
    wd = fs.algorithm.WienerFilter(sp).getDenominator(sp.wiener)
    assert rel_l2(wd.vectorData(), oracle.wiener_denominator(sp)) < 1e-6
    spec = oracle.prepare_raw(sp, raw)
    inFFT = [[cvec(V, spec[a * 3 + p]) for p in range(3)] for a in range(3)]
    out = fs.algorithm.SimAlgorithm.runReconstruction(sp, inFFT, False, 0).vectorData()
    assert rel_l2(out, oracle.recon(sp, spec)) < 1e-4
    assert rel_l2(out, oracle.recon(sp, spec.astype(np.complex128), dtype=np.float64)) < 1e-5


def test_measured_otf_estimation_vs_oracle(V, oracle, fs):
    """estimateParameters with a measured two-band OTF: commonRegion weights and divisions
    by the complex band-0 / band-1 values; the same fitted k0 as the oracle."""
    n = 256
    raw, truth = fs.synth.make_dataset(n=n, seed=42)
    sp = fs.synth.sim_param_for(truth, n, known=False)
    sp.setOtf(measured_otf(fs))
    spec = oracle.prepare_raw(sp, raw)
    est, _, _ = oracle.estimate(sp, spec, 1, 0.6)
    inFFT = [[cvec(V, spec[a * 3 + p]) for p in range(3)] for a in range(3)]
    fs.algorithm.SimAlgorithm.estimateParameters(sp, inFFT, 1, 0.6)
    for d in range(3):
        assert abs(sp.dir(d).pX - est["pX"][d]) < 1e-9 and abs(sp.dir(d).pY - est["pY"][d]) < 1e-9
        assert abs(sp.dir(d).phaOff - est["phaOff"][d]) < 1e-4
        assert abs(sp.dir(d).modul[1] - est["modulations"][d][1]) < 1e-4


def test_vector_ops_vs_reference_stdc_fixture(V):
    """The device kernels against the reference's own standard-C vector backend
    (accel/stdC_cplx.c, accel/stdC_real.c; outputs in tests/golden/stdc_vector_ops.npz, made
    by tests/golden/make_stdc_golden.py): element-wise ops and pasteFreq bit for bit,
    reductions to float-square rounding, fourierShift to the reference's float-phase
    rounding."""
    import os
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, "golden"))
    import make_stdc_golden as G
    fx = dict(np.load(os.path.join(here, "golden", "stdc_vector_ops.npz")))
    a, b, r, s = fx["a"], fx["b"], fx["r"], fx["s"]

    def run_c(op):
        v = cvec(V, a)
        op(v)
        return v.vectorData()

    assert np.array_equal(run_c(lambda v: v.add(cvec(V, b))), fx["c_add"])
    assert np.array_equal(run_c(lambda v: v.axpy(G.AXPY_A, cvec(V, b))), fx["c_axpy"])
    assert np.array_equal(run_c(lambda v: v.times(cvec(V, b))), fx["c_times"])
    assert np.array_equal(run_c(lambda v: v.timesConj(cvec(V, b))), fx["c_times_conj"])
    assert np.array_equal(run_c(lambda v: v.times(rvec(V, r))), fx["c_times_real"])
    assert np.array_equal(run_c(lambda v: v.scal(G.SCAL_A)), fx["c_scal"])
    # squares in float as AbstractVectorCplx.norm2 (linalg/AbstractVectorCplx.java:241-247);
    # the stdC backend squares in double
    assert abs(cvec(V, a).norm2() - fx["c_norm2"]) <= 1e-6 * fx["c_norm2"]
    vc = V.Vec2dCplx(a.shape[1], a.shape[0])
    vc.copy(rvec(V, r))
    assert np.array_equal(vc.vectorData(), fx["c_from_real"])

    def run_r(op):
        v = rvec(V, r)
        op(v)
        return v.vectorData()

    assert np.array_equal(run_r(lambda v: v.add(rvec(V, s))), fx["r_add"])
    assert np.array_equal(run_r(lambda v: v.axpy(G.REAL_A, rvec(V, s))), fx["r_axpy"])
    assert np.array_equal(run_r(lambda v: v.times(rvec(V, s))), fx["r_times"])
    assert np.array_equal(run_r(lambda v: v.scal(G.REAL_A)), fx["r_scal"])
    assert abs(rvec(V, r).sumElements() - fx["r_sum"]) <= 1e-9 * np.abs(r).sum()
    assert abs(rvec(V, r).norm2() - fx["r_norm2"]) <= 1e-6 * fx["r_norm2"]
    for i, (wi, wo, xo, yo) in enumerate(G.PASTE):
        out = V.Vec2dCplx(wo, wo)
        out.pasteFreq(cvec(V, fx["paste_in_%d" % i]), xo, yo)
        assert np.array_equal(out.vectorData(), fx["paste_out_%d" % i]), i
    for i, (N, kx, ky) in enumerate(G.SHIFTS):
        v = cvec(V, fx["shift_in_%d" % i])
        v.fourierShift(kx, ky)
        # the library reduces the phase modulo one turn in double; the reference rounds it
        # to float first (an error that grows with |k|)
        assert rel_l2(v.vectorData(), fx["shift_out_%d" % i]) < 1e-5, i
