"""Seeded synthetic SIM datasets.

The reference publishes no dataset for this path; these seeded stacks stand in for real
camera data with the sizes and value distributions of the benchmark configurations:

* object: ``n_points`` Poisson-placed point emitters (brightness lognormal(0, 0.5)) plus
  ``n_filaments`` random-walk filaments;
* illumination ``1 + m cos(2 pi k.r + phi_p)`` at ``n_dirs`` angles (0, 60, 120 deg plus a seeded
  offset below 5 deg), phases ``2 pi p / n_phases + phi0``, ``|k0| = k0_frac * cutoff``;
* optics: the analytic widefield OTF of ``OtfProvider.fromEstimate(NA, lambda, a)``
  (org/fairsim/sim_algorithm/OtfProvider.java:74-78, 96-120);
* noise: Poisson at ``photons`` peak plus Gaussian ``gauss`` counts.

The returned ``truth`` dict holds the generating parameters converted to the SimParam
convention: ``setPxPy`` takes the highest band's shift in display coordinates (x right, y
flipped up: S/OtfProvider.java:345-346), which for a pattern ``cos(2 pi (kx x + ky y)/n)``
in array-index coordinates is ``(kx, -ky)``.
"""
from __future__ import annotations

import math

import numpy as np


def ideal_otf(d):
    d = np.clip(np.asarray(d, dtype=np.float64), 0, None)
    out = np.zeros_like(d)
    m = d <= 1
    dm = d[m]
    out[m] = (2 / math.pi) * (np.arccos(dm) - dm * np.sqrt(1 - dm * dm))
    return out


def cutoff_cycles_per_micron(na, em_wavelength):
    return 1000.0 / (em_wavelength / na / 2.0)


def make_object(n, rng, n_points=2000, n_filaments=40, scale=1.0):
    obj = np.zeros((n, n), dtype=np.float64)
    npts = int(round(n_points * scale))
    xs = rng.uniform(0, n, npts)
    ys = rng.uniform(0, n, npts)
    br = rng.lognormal(0.0, 0.5, npts)
    np.add.at(obj, (ys.astype(int) % n, xs.astype(int) % n), br)
    nfil = int(round(n_filaments * scale))
    steps = max(64, n // 2)
    for _ in range(nfil):
        x, y = rng.uniform(0, n), rng.uniform(0, n)
        ang = rng.uniform(0, 2 * math.pi)
        amp = rng.lognormal(-1.0, 0.3)
        for _s in range(steps):
            ang += rng.normal(0, 0.15)
            x = (x + math.cos(ang)) % n
            y = (y + math.sin(ang)) % n
            obj[int(y) % n, int(x) % n] += amp
    return obj


def make_dataset(n=512, n_dirs=3, n_phases=3, n_bands=2, seed=0, na=1.4, em_wavelength=525.0,
                 pxl_um=0.08, otf_a=1.0, k0_frac=0.85, modulation=0.8, photons=500.0,
                 gauss=2.0, angles_deg=None, angle_jitter_deg=5.0, n_points=2000,
                 n_filaments=40, dtype=np.float32, as_u16=False):
    """Return (raw stack (n_dirs*n_phases, n, n), truth dict)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    if angles_deg is None:
        angles_deg = [180.0 * d / n_dirs for d in range(n_dirs)]
    area = (n / 512.0) ** 2
    obj = make_object(n, rng, n_points, n_filaments, scale=area)

    cut_um = cutoff_cycles_per_micron(na, em_wavelength)
    cut_px = cut_um * n * pxl_um
    k0 = k0_frac * cut_px
    fy = np.fft.fftfreq(n) * n
    fx = np.fft.fftfreq(n) * n
    rr = np.sqrt(fx[None, :] ** 2 + fy[:, None] ** 2)
    otf = ideal_otf(rr / cut_px) * np.power(otf_a, np.clip(rr / cut_px, 0, 1))

    yy, xx = np.mgrid[0:n, 0:n].astype(np.float64)
    frames = []
    kvec = []
    phi0 = []
    for d in range(n_dirs):
        th = math.radians(angles_deg[d] + rng.uniform(0, angle_jitter_deg))
        kx, ky = k0 * math.cos(th), k0 * math.sin(th)
        p0 = rng.uniform(0, 2 * math.pi)
        kvec.append((kx, ky))
        phi0.append(p0)
        for p in range(n_phases):
            phi = 2 * math.pi * p / n_phases + p0
            pat = 1.0 + modulation * np.cos(2 * math.pi * (kx * xx + ky * yy) / n + phi)
            for b in range(2, n_bands):  # higher harmonics for 3-beam data
                pat += modulation * 0.5 * np.cos(b * (2 * math.pi * (kx * xx + ky * yy) / n + phi))
            img = np.fft.ifft2(np.fft.fft2(obj * pat) * otf).real
            frames.append(img)
    frames = np.array(frames)
    frames = np.clip(frames, 0, None)
    frames *= photons / frames.max()
    noisy = rng.poisson(frames).astype(np.float64) + rng.normal(0, gauss, frames.shape)
    if as_u16:
        raw = np.clip(np.rint(noisy), 0, 65535).astype(np.uint16)
    else:
        raw = noisy.astype(dtype)
    # shift of the highest band in display coordinates (y flipped), band b shift = b*k/(nB-1)
    hb = n_bands - 1
    truth = dict(
        kx=[k[0] for k in kvec], ky=[k[1] for k in kvec],
        pxpy=[(hb * k[0], -hb * k[1]) for k in kvec],
        phi0=phi0, modulation=modulation, cutoff_px=cut_px, k0_px=k0,
        na=na, em_wavelength=em_wavelength, pxl_um=pxl_um, otf_a=otf_a,
    )
    return raw, truth


def sim_param_for(truth, n, n_dirs=3, n_phases=3, n_bands=2, known=True):
    """SimParam mirror filled with the generator's true parameters."""
    from .sim_param import OtfProvider, SimParam

    otf = OtfProvider.fromEstimate(truth["na"], truth["em_wavelength"], truth["otf_a"])
    sp = SimParam.create(n_bands, n_dirs, n_phases, n, truth["pxl_um"], otf)
    if known:
        for d in range(n_dirs):
            sp.dir(d).setPxPy(*truth["pxpy"][d])
            sp.dir(d).setPhaOff(truth["phi0"][d])
            for b in range(1, n_bands):
                sp.dir(d).setModulation(b, truth["modulation"])
    return sp


def synthetic_params(n, n_dirs=3, n_phases=3, n_bands=2, na=1.4, em_wavelength=525.0, pxl_um=0.08, k0_frac=0.85,
                     modulation=0.8, seed=0):
    """SimParam mirror with the generator's geometry, without generating images (for
    launch-shape tuning and timing, where the pixel values do not matter)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cut_px = cutoff_cycles_per_micron(na, em_wavelength) * n * pxl_um
    k0 = k0_frac * cut_px
    hb = n_bands - 1
    pxpy, phi0 = [], []
    for d in range(n_dirs):
        th = math.radians(180.0 * d / n_dirs + rng.uniform(0, 5.0))
        pxpy.append((hb * k0 * math.cos(th), -hb * k0 * math.sin(th)))
        phi0.append(rng.uniform(0, 2 * math.pi))
    truth = dict(pxpy=pxpy, phi0=phi0, modulation=modulation, na=na, em_wavelength=em_wavelength, pxl_um=pxl_um,
                 otf_a=1.0)
    return sim_param_for(truth, n, n_dirs, n_phases, n_bands)
