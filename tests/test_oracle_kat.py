"""Known-answer tests that pin the CPU restatement (the oracle) of fairSIM's Java path.

The reference has no test suite and no golden data, so these tests pin each building
block against mathematics it must satisfy, following the reference's own self-checks
(org/fairsim/linalg/MTool.java:80-92, org/fairsim/linalg/MatrixComplex.java:307-327)."""
import math

import numpy as np
import pytest

from conftest import rel_l2


@pytest.mark.parametrize("n", [64, 96, 128, 384])
@pytest.mark.parametrize("dtype,tol", [(np.float32, 2e-6), (np.float64, 1e-13)])
def test_fft2d_matches_numpy(oracle, n, dtype, tol):
    rng = np.random.default_rng(n)
    z = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    f = oracle.fft2d(z, inverse=False, dtype=dtype)
    assert rel_l2(f, np.fft.fft2(z)) < tol
    g = oracle.fft2d(z, inverse=True, dtype=dtype)  # JTransforms complexInverse(scale=true)
    assert rel_l2(g, np.fft.ifft2(z)) < tol


def test_fft2d_non_square(oracle):
    rng = np.random.default_rng(3)
    z = rng.standard_normal((48, 80)) + 1j * rng.standard_normal((48, 80))
    assert rel_l2(oracle.fft2d(z, dtype=np.float64), np.fft.fft2(z)) < 1e-13


def test_fsin_error_bound(oracle):
    # MTool.fsin documents 5.4e-9 max error; the reference's main() scans +-6 pi in 0.01 steps
    worst = 0.0
    for r in np.arange(-6 * math.pi, 6 * math.pi, 0.01):
        worst = max(worst, abs(oracle.fsin(r) - math.sin(r)), abs(oracle.fcos(r) - math.cos(r)))
    assert worst <= 5.5e-9


def test_matrix_inverse_identity(oracle):
    rng = np.random.default_rng(7)
    for n in (3, 5):
        M = rng.uniform(-1, 1, (n, n)) + 1j * rng.uniform(-1, 1, (n, n))
        inv = oracle.matrix_inverse(M)
        assert np.abs(inv @ M - np.eye(n)).max() < 1e-10
    A = rng.uniform(-1, 1, (5, 3)) + 1j * rng.uniform(-1, 1, (5, 3))
    pinv = oracle.matrix_inverse(A, pseudo=True)
    assert np.abs(pinv - np.linalg.pinv(A)).max() < 1e-10


@pytest.mark.parametrize("n_pha,bands", [(3, 2), (5, 2), (5, 3)])
def test_band_separation_recovers_bands(oracle, fs, n_pha, bands):
    n = 32
    rng = np.random.default_rng(11)
    nc = 2 * bands - 1
    truth = rng.standard_normal((nc, n, n)) + 1j * rng.standard_normal((nc, n, n))
    phases = [2 * math.pi * p / n_pha + 0.3 for p in range(n_pha)]
    mod = [1.0] + [0.7] * (bands - 1)
    fac = [mod[0]] + [0.5 * m for m in mod[1:]]
    mixed = []
    for p in range(n_pha):
        img = fac[0] * truth[0]
        for j in range(bands - 1):
            ph = phases[p] * (j + 1)
            img = img + fac[j + 1] * np.exp(1j * ph) * truth[2 * j + 1] + fac[j + 1] * np.exp(-1j * ph) * truth[2 * j + 2]
        mixed.append(img)
    otf = fs.OtfProvider.fromEstimate(1.4, 525, 1.0)
    sp = fs.SimParam.create(bands, 1, n_pha, n, 0.08, otf)
    sp.dir(0).setPhaOff(0.3)
    for b in range(1, bands):
        sp.dir(0).setModulation(b, 0.7)
    sep = oracle.separate_bands(sp, 0, np.array(mixed), dtype=np.float64)
    assert rel_l2(sep, truth) < 1e-10


def test_integer_fourier_shift_is_roll(oracle):
    n = 64
    rng = np.random.default_rng(5)
    z = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    # SimUtils.fourierShift(v, kx, ky): ifft, times exp(i 2pi (kx x - ky y)/N), fft
    real = np.fft.ifft2(z)
    real = oracle.fourier_shift(real, 5.0, -(-3.0), dtype=np.float64)
    shifted = np.fft.fft2(real)
    assert rel_l2(shifted, np.roll(np.roll(z, 5, axis=1), 3, axis=0)) < 1e-12


def test_paste_freq_layout(oracle):
    z = np.arange(16, dtype=np.float64).reshape(4, 4) + 0j
    out = oracle.paste_freq(z, 8, 8, dtype=np.float64)
    # x<wi/2 stays, x>=wi/2 moves by wo/2 (org/fairsim/linalg/BasicVectors.java:275-283)
    assert out[0, 0] == 0 and out[0, 1] == 1 and out[0, 6] == 2 and out[0, 7] == 3
    assert out[6, 0] == 8 and out[7, 7] == 15 and out[2, 2] == 0
    off = oracle.paste_freq(z, 8, 8, 1, -1, dtype=np.float64)
    assert off[7, 1] == 0 and off[0, 2] == 5


def test_otf_lookup_is_floor_indexed(oracle, fs):
    # getOtfVal returns vals[floor(pos)] (S/OtfProvider.java:208-219)
    n = 64
    otf = fs.OtfProvider.fromEstimate(1.4, 525, 0.3)
    sp = fs.SimParam.create(2, 1, 3, n, 0.08, otf)
    v = oracle.otf_vector(sp, np.zeros((n, n), complex), 0, 0, which=0, dtype=np.float64)
    cut = 1000 / (525 / 1.4 / 2)
    cpm = 1 / (n * 0.08)
    step = cut / 512
    for x in (1, 3, 7, 11):
        pos = x * cpm / step
        d = math.floor(pos) / 512
        ideal = (2 / math.pi) * (math.acos(d) - d * math.sqrt(1 - d * d)) * 0.3 ** d
        assert abs(v[0, x].real - ideal) < 1e-12


def test_estimation_recovers_seeded_k0(oracle, fs):
    n = 256
    raw, truth = fs.synth.make_dataset(n=n, seed=4)
    sp = fs.synth.sim_param_for(truth, n, known=False)
    spec = oracle.prepare_raw(sp, raw)
    est, peaks, coarse = oracle.estimate(sp, spec, 1, 0.6)
    for d in range(3):
        assert abs(est["pX"][d] - truth["pxpy"][d][0]) < 0.1
        assert abs(est["pY"][d] - truth["pxpy"][d][1]) < 0.1
        assert abs(est["modulations"][d][1] - truth["modulation"]) < 0.15


@pytest.mark.parametrize("n,n_phases,n_bands", [(64, 3, 2), (128, 3, 2), (128, 5, 2), (128, 5, 3)])
def test_float_oracle_against_fp64_oracle(oracle, fs, n, n_phases, n_bands):
    """The reference's float semantics (float phases, MTool.fsin/fcos, float vectors) stay
    within the parity tolerance of the same algorithm in double precision; the error is
    printed (the GPU path is compared against both)."""
    raw, truth = fs.synth.make_dataset(n=n, seed=50 + n + n_phases, n_phases=n_phases, n_bands=n_bands)
    sp = fs.synth.sim_param_for(truth, n, n_phases=n_phases, n_bands=n_bands)
    f32 = oracle.recon_raw(sp, raw, fade=10)
    f64 = oracle.recon_raw(sp, raw.astype(np.float64), fade=10, dtype=np.float64)
    err = float(np.linalg.norm(f32 - f64) / np.linalg.norm(f64))
    print("oracle float vs FP64 at %d^2, %d phases, %d bands: rel-L2 %.2e" % (n, n_phases, n_bands, err))
    assert err < 1e-4


def test_widefield_outputs_match_numpy(oracle, fs):
    """runReconstruction's widefield side outputs (S/SimAlgorithm.java:533-576) against the
    same steps in numpy: the band-0 spectra of every direction pasted at 2w and summed, then
    (filtered) times OTF_0 / (2 OTF_0^2 + w^2) inside the OTF support."""
    n = 64
    raw, truth = fs.synth.make_dataset(n=n, seed=21)
    sp = fs.synth.sim_param_for(truth, n)
    wf, fwf = oracle.widefield_raw(sp, raw.astype(np.float64), fade=10, dtype=np.float64)
    spec = oracle.prepare_raw(sp, raw.astype(np.float64), fade=10, dtype=np.float64)
    n_dirs, n_pha = sp.nrDirs, sp.nrPhases
    placed = np.zeros((2 * n, 2 * n), complex)
    lo = np.r_[0:n // 2]
    hi = np.r_[n // 2:n]
    for a in range(n_dirs):
        b0 = oracle.separate_bands(sp, a, spec[a * n_pha:(a + 1) * n_pha], dtype=np.float64)[0]
        for ys, yd in ((lo, lo), (hi, hi + n)):
            for xs, xd in ((lo, lo), (hi, hi + n)):
                placed[np.ix_(yd, xd)] += b0[np.ix_(ys, xs)]
    assert rel_l2(wf, np.fft.ifft2(placed).real) < 1e-12
    W = 2 * n
    xh = np.where(np.arange(W) < n, np.arange(W), np.arange(W) - W)
    yh = np.where(np.arange(W) < n, -np.arange(W), W - np.arange(W))
    cpm = 1 / (n * sp.micronsPerPixel)
    cycl = np.hypot(xh[None, :], yh[:, None]) * cpm
    otfp = sp.otf()
    cut = otfp.getCutoff()
    pos = cycl / (cut / 512)
    dd = np.clip(np.floor(pos) / 512, 0, 1)
    otf = (2 / np.pi) * (np.arccos(dd) - dd * np.sqrt(1 - dd * dd)) * otfp.a ** dd
    otf = np.where((cycl < cut) & (np.ceil(pos) < 512), otf, 0.0)  # getOtfVal's two zero tests
    filt = otf / (2 * otf * otf + sp.wienerFilterParameter ** 2)
    filt[cycl > cut] = 0
    assert rel_l2(fwf, np.fft.ifft2(placed * filt).real) < 1e-12
    f32 = oracle.widefield_raw(sp, raw, fade=10)
    for a64, a32 in zip((wf, fwf), f32):
        assert rel_l2(a32, a64) < 1e-5


def test_rl_deconvolution_matches_numpy(oracle):
    """RLDeconvolution.deconvolve (S/RLDeconvolution.java:45-103) against the same iteration
    in numpy (FP64), and the float oracle against FP64."""
    n = 64
    rng = np.random.default_rng(5)
    img = rng.uniform(1, 2, (n, n)) + 0j
    k = np.fft.fftfreq(n)
    otf = np.exp(-(k[None, :] ** 2 + k[:, None] ** 2) * 30) + 0j
    spec = np.fft.fft2(img)
    got = oracle.rl_deconvolve(spec, otf, 4, True, dtype=np.float64)
    d = np.fft.ifft2(spec)
    u = d.copy()
    for _ in range(4):
        nx = np.fft.ifft2(np.fft.fft2(u) * otf)
        nx = d / nx
        nx = np.fft.ifft2(np.fft.fft2(nx) * otf)
        u = nx * u
    assert rel_l2(got, np.fft.fft2(u)) < 1e-12
    assert rel_l2(oracle.rl_deconvolve(spec, otf, 4, True), got) < 1e-5


def test_auto_correlation_matches_numpy(oracle):
    """Correlation.autoCorrelation (S/Correlation.java:294-325) in FP64 against numpy."""
    n = 32
    rng = np.random.default_rng(9)
    band = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    kx, ky = 3.3, -5.7
    got = oracle.auto_correlation(band, kx, ky, dtype=np.float64)
    N = 2 * n
    a = oracle.paste_freq(band, N, N, dtype=np.float64)
    X, Y = np.meshgrid(np.arange(N), np.arange(N))
    b = np.fft.fft2(np.fft.ifft2(a) * np.exp(2j * np.pi * (kx * X - ky * Y) / N))
    exp = np.sum(a * np.conj(b)) / np.sum(np.abs(a) ** 2)
    assert abs(got - exp) < 1e-10 * abs(exp)
    assert abs(oracle.auto_correlation(band, kx, ky) - got) < 1e-5 * abs(got)


@pytest.mark.parametrize("style", [1, 2, 3])
def test_rl_filter_styles_float_vs_fp64(oracle, fs, style):
    """runReconstruction with RL on the input, the output, or both (S/SimAlgorithm.java:318-361,
    587-641): the float oracle within the parity bound of FP64; the result differs from the
    Wiener result (it is a different filter)."""
    n = 64
    raw, truth = fs.synth.make_dataset(n=n, seed=77)
    # a camera offset keeps the raw frames positive: RL divides by the blurred estimate, and
    # with the generator's zero-mean read noise in dark pixels that division is ill-conditioned
    # (float and double then part ways in the reference's algorithm itself)
    raw = raw + 200.0
    sp = fs.synth.sim_param_for(truth, n)
    sp.setFilterStyle(style)
    sp.setRLiterations(3)
    f32 = oracle.recon_raw(sp, raw, fade=10)
    f64 = oracle.recon_raw(sp, raw.astype(np.float64), fade=10, dtype=np.float64)
    err = rel_l2(f32, f64)
    print("RL style %d: float vs FP64 rel-L2 %.2e" % (style, err))
    assert err < 1e-4
    sp.setFilterStyle(0)
    assert rel_l2(f64, oracle.recon_raw(sp, raw.astype(np.float64), fade=10, dtype=np.float64)) > 1e-2


def measured_bands(na=1.4, lam=525.0, samples=300, bands=2, a=0.3, spacing=256):
    """Synthetic measured OTF bands: the estimate's shape with a per-band gain and a slow
    complex phase (as a bead measurement gives), `spacing` samples up to the cutoff."""
    cut = 1000 / (lam / na / 2)
    v = np.arange(samples) / spacing
    vc = np.clip(v, 0, 1)
    base = (2 / np.pi) * (np.arccos(vc) - vc * np.sqrt(1 - vc * vc)) * a ** vc
    return [(base * (1 - 0.1 * b) * np.exp(1j * 0.3 * (b + 1) * vc)).tolist() for b in range(bands)], cut / spacing


def test_measured_otf_equal_to_estimate_gives_estimate_result(oracle, fs):
    """OtfProvider built from band data (S/OtfProvider.java:588-621) holding the estimate's own
    512 samples reconstructs like the estimate: the measured-OTF code path is the estimate's."""
    n = 64
    raw, truth = fs.synth.make_dataset(n=n, seed=33)
    sp = fs.synth.sim_param_for(truth, n)
    est = oracle.recon_raw(sp, raw, fade=10, dtype=np.float64)
    o = sp.otf()
    v = np.arange(512) / 512
    vals = (2 / np.pi) * (np.arccos(v) - v * np.sqrt(1 - v * v)) * o.a ** v
    sp2 = sp.duplicate()
    sp2.setOtf(fs.OtfProvider.fromMeasured(o.na, o.emWavelength, [vals.astype(np.float32).tolist()],
                                           o.getCutoff() / 512))
    meas = oracle.recon_raw(sp2, raw, fade=10, dtype=np.float64)
    assert rel_l2(meas, est) < 1e-6


@pytest.mark.parametrize("samples", [300, 200])
def test_measured_multiband_otf_float_vs_fp64(oracle, fs, samples):
    """A complex two-band measured OTF (200 samples ends the table inside the cutoff): the
    float oracle within the parity bound of FP64, and different from the estimate."""
    n = 64
    raw, truth = fs.synth.make_dataset(n=n, seed=34)
    sp = fs.synth.sim_param_for(truth, n)
    bands, cyc = measured_bands(samples=samples)
    est = oracle.recon_raw(sp, raw.astype(np.float64), fade=10, dtype=np.float64)
    sp.setOtf(fs.OtfProvider.fromMeasured(1.4, 525.0, bands, cyc))
    f32 = oracle.recon_raw(sp, raw, fade=10)
    f64 = oracle.recon_raw(sp, raw.astype(np.float64), fade=10, dtype=np.float64)
    assert rel_l2(f32, f64) < 1e-4
    assert rel_l2(f64, est) > 1e-3
