"""The identities the fused offline passes are built on, checked in double precision with
numpy (no GPU, no library). The reference shifts a band by pasting its N-point spectrum onto
the 2N grid and multiplying the real-space image by a phase ramp there
(sim_algorithm/SimUtils.java:43-50 with linalg/BasicVectors.java:259-339):
    F = FFT_W(r * iFFT_W(paste(FFT_N(z)))),  W = 2N.
The passes evaluate it with N-point transforms only, and transform only the neg component of
each conjugate band pair (csrc/recon_kernels.cuh, passes A, G, B); the image is real, so the
column pass forms only the Hermitian half of the spectrum and the row pass C completes it."""
import numpy as np
import pytest


def paste_src(X, N):
    """Source index in the N-point spectrum of output index X of pasteFreq onto 2N, or -1."""
    return X if X < N // 2 else (X - N if X >= 3 * N // 2 else -1)


def paste(Z, N):
    W = 2 * N
    P = np.zeros(W, complex)
    for X in range(W):
        m = paste_src(X, N)
        if m >= 0:
            P[X] = Z[m]
    return P


def shifted_spectrum(z, k):
    """1D: FFT_W(r * iFFT_W(paste(FFT_N(z)))) with r[n] = exp(2 pi i k n / W)."""
    N = len(z)
    W = 2 * N
    r = np.exp(2j * np.pi * k * np.arange(W) / W)
    return np.fft.fft(r * np.fft.ifft(paste(np.fft.fft(z), N)))


def shifted_spectrum_2d(z, kx, ky):
    """The same along x (axis 1) then along y (axis 0)."""
    rows = np.array([shifted_spectrum(z[y], kx) for y in range(z.shape[0])])
    return np.array([shifted_spectrum(rows[:, X], ky) for X in range(rows.shape[1])]).T


@pytest.mark.parametrize("N,k", [(16, 3.25), (32, -7.6), (48, 11.0), (64, 20.37)])
def test_even_odd_split_of_the_2n_shift(N, k):
    """u = iFFT_W(paste(Z)) has u[2n] = z[n]/2 and u[2n+1] = iFFT_N(Z * s)[n] / 2 with
    s(m) = exp(i pi m~/N) (m~ the pasted signed frequency; numpy's iFFT carries 1/N), and
    FFT_W(r u)[X] = E[X mod N] + exp(-2 pi i X/W) O[X mod N] with E, O the N-point
    transforms of the even and odd samples of r u."""
    rng = np.random.default_rng(1)
    z = rng.normal(size=N) + 1j * rng.normal(size=N)
    W = 2 * N
    Z = np.fft.fft(z)
    u = np.fft.ifft(paste(Z, N))
    m = np.arange(N)
    ms = np.where(m < N // 2, m, m - N)
    s = np.exp(1j * np.pi * ms / N)
    assert np.allclose(u[0::2], z / 2, atol=1e-13)
    assert np.allclose(u[1::2], np.fft.ifft(Z * s) / 2, atol=1e-13)
    r = np.exp(2j * np.pi * k * np.arange(W) / W)
    E = np.fft.fft(r[0::2] * u[0::2])
    O = np.fft.fft(r[1::2] * u[1::2])
    X = np.arange(W)
    assert np.allclose(shifted_spectrum(z, k), E[X % N] + np.exp(-2j * np.pi * X / W) * O[X % N], atol=1e-11)


@pytest.mark.parametrize("N,k", [(16, 3.25), (32, -7.6), (64, 20.37)])
def test_conjugate_pair_along_one_axis(N, k):
    """z_pos = conj(z_neg) with the opposite shift gives
    F_pos[X] = conj(F_neg[-X]) + exp(-2 pi i X/W) Q[X mod N] d, d = -2i conj(Z_neg[N/2]),
    Q = FFT_N((-1)^n r_pos[2n+1]) / W: the pasted Nyquist bin, whose half-sample phase
    s(N/2) = -i is not conjugate-symmetric, is the only asymmetry."""
    rng = np.random.default_rng(2)
    z = rng.normal(size=N) + 1j * rng.normal(size=N)
    W = 2 * N
    F_neg = shifted_spectrum(z, k)
    F_pos = shifted_spectrum(np.conj(z), -k)
    d = -2j * np.conj(np.fft.fft(z)[N // 2])
    r_pos = np.exp(-2j * np.pi * k * np.arange(W) / W)
    Q = np.fft.fft((-1.0) ** np.arange(N) * r_pos[1::2]) / W
    X = np.arange(W)
    pred = np.conj(F_neg[(-X) % W]) + np.exp(-2j * np.pi * X / W) * Q[X % N] * d
    assert np.allclose(F_pos, pred, atol=1e-11)
    # without the Nyquist term the pair is not mirror-symmetric
    assert not np.allclose(F_pos, np.conj(F_neg[(-X) % W]), atol=1e-6)


@pytest.mark.parametrize("N,kx,ky", [(16, 3.25, -2.5), (32, -7.6, 5.1)])
def test_conjugate_pair_in_two_dimensions(N, kx, ky):
    """F_pos[Y][X] = conj(F_neg[-Y][-X]) + exp(-2 pi i Y/W) d'(-X) Qy[Y mod N]
                     + exp(-2 pi i X/W) Qx[X mod N] G[Y]
    with d(y) the row Nyquist terms of the neg component (pass A), G their y transform with
    the pos shift (pass G) and d'(X) the Nyquist term of the neg x-transformed column X
    (pass B); pass B forms the pos component from these and the mirrored neg window."""
    rng = np.random.default_rng(3)
    z = rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))
    W = 2 * N
    F_neg = shifted_spectrum_2d(z, kx, ky)
    F_pos = shifted_spectrum_2d(np.conj(z), -kx, -ky)
    n = np.arange(N)
    rx_pos = np.exp(-2j * np.pi * kx * np.arange(W) / W)
    ry_pos = np.exp(-2j * np.pi * ky * np.arange(W) / W)
    Qx = np.fft.fft((-1.0) ** n * rx_pos[1::2]) / W
    Qy = np.fft.fft((-1.0) ** n * ry_pos[1::2]) / W
    d = -2j * np.conj(np.fft.fft(z, axis=1)[:, N // 2])  # per real-space row y
    G = shifted_spectrum(d, -ky)  # along y with the pos shift
    rows_neg = np.array([shifted_spectrum(z[y], kx) for y in range(N)])  # x pass of neg
    dcol = -2j * np.conj(np.fft.fft(rows_neg, axis=0)[N // 2, :])  # per x-transformed column X
    X = np.arange(W)[None, :]
    Y = np.arange(W)[:, None]
    pred = (np.conj(F_neg[(-Y) % W, (-X) % W])
            + np.exp(-2j * np.pi * Y / W) * dcol[(-X) % W] * Qy[Y % N]
            + np.exp(-2j * np.pi * X / W) * Qx[X % N] * G[Y])
    assert np.allclose(F_pos, pred, atol=1e-10)


def test_band_zero_sum_over_angles_is_one_transform():
    """Band separation and the row FFT are linear, so summing band 0 over the angles before
    the transform (pass A's extra row block) equals transforming each angle's band 0."""
    rng = np.random.default_rng(4)
    nA, nP, N = 3, 3, 32
    raw = rng.normal(size=(nA, nP, N))
    c0 = rng.normal(size=(nA, nP)) + 1j * rng.normal(size=(nA, nP))
    per_angle = sum(np.fft.fft(np.tensordot(c0[a], raw[a], axes=1)) for a in range(nA))
    folded = np.fft.fft(np.einsum("ap,apn->n", c0, raw))
    assert np.allclose(per_angle, folded, atol=1e-12)


@pytest.mark.parametrize("N", [16, 48, 64])
def test_real_output_row_from_hermitian_halves(N):
    """The widefield output pass (csrc/widefield.cu, WC) keeps only the real part of the
    2N-point inverse of a pasted row V: its even samples are Re(iFFT_N(a))/2 with a = V, its
    odd samples Re(iFFT_N(b))/2 with b = V * s. Re(iFFT(a)) = iFFT(Ha) with the Hermitian
    half Ha[k] = (a[k] + conj(a[-k]))/2, so one transform of Ha + i Hb gives both rows."""
    rng = np.random.default_rng(5)
    V = rng.normal(size=N) + 1j * rng.normal(size=N)
    m = np.arange(N)
    s = np.exp(1j * np.pi * np.where(m < N // 2, m, m - N) / N)
    full = np.real(np.fft.ifft(paste(V, N)))
    a, b = V, V * s
    herm = lambda c: (c + np.conj(c[(-m) % N])) / 2  # noqa: E731
    y = np.fft.ifft(herm(a) + 1j * herm(b)) / 2
    assert np.allclose(full[0::2], y.real, atol=1e-13)
    assert np.allclose(full[1::2], y.imag, atol=1e-13)


@pytest.mark.parametrize("N,kx,ky", [(16, 3.25, -2.5), (32, -7.6, 5.1)])
def test_hermitian_half_of_a_band_pair(N, kx, ky):
    """Pass B stores H = (F(k) + conj F(-k))/2 (the image Re iFFT2(F) = iFFT2(H)) for the
    columns 0..N only. For a pair with mirror-image masks (mask_neg(-k) = mask_pos(k)) and
    F = mask_neg F_neg + mask_pos F_pos, with F_pos(k) = conj(F_neg(-k)) + n1(k):
        H(k) = mask_neg(k) (A + conj(n2)/2) + mask_pos(k) (conj(B) + n1/2),
    A = F_neg(k), B = F_neg(-k), n2(k) = n1(-k). Band 0 (a symmetric mask) adds
    mask_0(k) (T0(k) + conj T0(-k)) / 2."""
    rng = np.random.default_rng(6)
    W = 2 * N
    z = rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))
    F_neg = shifted_spectrum_2d(z, kx, ky)
    F_pos = shifted_spectrum_2d(np.conj(z), -kx, -ky)
    Yi, Xi = np.meshgrid(np.arange(W), np.arange(W), indexing="ij")
    mir = lambda a: a[(-Yi) % W, (-Xi) % W]  # noqa: E731  a(-k)
    n1 = F_pos - np.conj(mir(F_neg))
    m_pos = rng.uniform(size=(W, W))  # any real mask; the neg mask is its mirror image
    m_neg = mir(m_pos)
    m0 = rng.uniform(size=(W, W))
    m0 = (m0 + mir(m0)) / 2  # band 0: symmetric
    T0 = np.fft.fft2(rng.normal(size=(W, W)) + 1j * rng.normal(size=(W, W)))
    F = m_neg * F_neg + m_pos * F_pos + m0 * T0
    H_direct = (F + np.conj(mir(F))) / 2
    A, B, n2 = F_neg, mir(F_neg), mir(n1)
    H_pass_b = m_neg * (A + np.conj(n2) / 2) + m_pos * (np.conj(B) + n1 / 2) + m0 * (T0 + np.conj(mir(T0))) / 2
    assert np.allclose(H_pass_b, H_direct, atol=1e-10)
    assert np.allclose(np.real(np.fft.ifft2(F)), np.fft.ifft2(H_direct), atol=1e-12)


@pytest.mark.parametrize("N", [8, 24, 64])
def test_complex_to_real_row_from_half_spectrum(N):
    """Pass C: a real row out[x] = sum_X H[X] exp(+2 pi i x X/W) of a Hermitian H
    (H[W-X] = conj H[X]) from its half H[0..N] by one N-point inverse transform of
    Z[k] = (H[k] + conj H[N-k]) + i exp(+2 pi i k/W) (H[k] - conj H[N-k]):
    iFFT_N(Z)[n] N = out[2n] + i out[2n+1]."""
    rng = np.random.default_rng(7)
    W = 2 * N
    h = np.fft.fft(rng.normal(size=W))  # Hermitian
    out = np.fft.ifft(h).real * W        # unnormalised inverse
    k = np.arange(N)
    hk, hm = h[k], np.conj(h[N - k])
    Z = (hk + hm) + 1j * np.exp(2j * np.pi * k / W) * (hk - hm)
    z = np.fft.ifft(Z) * N
    assert np.allclose(z.real, out[0::2], atol=1e-10)
    assert np.allclose(z.imag, out[1::2], atol=1e-10)
