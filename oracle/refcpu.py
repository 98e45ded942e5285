"""ORACLE — test infrastructure only.

ctypes binding of ``oracle/_build/librefcpu.so`` (the C++ restatement of fairSIM's Java
2D SIM path in ``refcpu.hpp``).  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module; the product library never does.

Parity status: unpinned against the Java reference's own outputs (no JVM here and the
reference ships no golden vectors); pinned by known-answer tests in ``tests/``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "librefcpu.so")

MAXD, MAXB, MAXP = 8, 4, 16


class RefParam(C.Structure):
    _fields_ = [
        ("w", C.c_int),
        ("nrDirs", C.c_int),
        ("nrBands", C.c_int),
        ("nrPhases", C.c_int),
        ("micronsPerPixel", C.c_double),
        ("na", C.c_double),
        ("lambda_", C.c_double),
        ("otfA", C.c_double),
        ("useAtt", C.c_int),
        ("attStr", C.c_double),
        ("attFWHM", C.c_double),
        ("wiener", C.c_double),
        ("apoCutoff", C.c_double),
        ("apoBend", C.c_double),
        ("pX", C.c_double * MAXD),
        ("pY", C.c_double * MAXD),
        ("phaOff", C.c_double * MAXD),
        ("modul", (C.c_double * MAXB) * MAXD),
        ("hasPhases", C.c_int),
        ("phases", (C.c_double * MAXP) * MAXD),
        ("filterStyle", C.c_int),
        ("rlIterations", C.c_int),
        ("otfData", C.c_void_p),
        ("otfBands", C.c_int),
        ("otfSamples", C.c_int),
        ("otfCycles", C.c_double),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++ only)."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
        os.path.getmtime(os.path.join(_HERE, f)) for f in ("refcpu.hpp", "refcpu_capi.cpp")
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.ref_last_error.restype = C.c_char_p
        L.ref_fsin.restype = C.c_double
        L.ref_fsin.argtypes = [C.c_double]
        L.ref_fcos.restype = C.c_double
        L.ref_fcos.argtypes = [C.c_double]
        _lib = L
    return _lib


def _chk(rc):
    if rc != 0:
        raise RuntimeError("oracle: " + lib().ref_last_error().decode())


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _suf(dtype):
    return "f32" if np.dtype(dtype) == np.float32 else "f64"


def set_threads(n: int) -> int:
    return lib().ref_set_threads(int(n))


def make_param(p) -> RefParam:
    """Convert a parameter description (object with the SimParam mirror's fields or a dict)."""
    g = (lambda k: p[k]) if isinstance(p, dict) else (lambda k: getattr(p, k))
    r = RefParam()
    r.w = g("w")
    r.nrDirs, r.nrBands, r.nrPhases = g("nrDirs"), g("nrBands"), g("nrPhases")
    r.micronsPerPixel = g("micronsPerPixel")
    r.na, r.lambda_, r.otfA = g("na"), g("emWavelength"), g("otfA")
    r.useAtt = int(g("useAttenuation"))
    r.attStr, r.attFWHM = g("attStrength"), g("attFWHM")
    r.wiener, r.apoCutoff, r.apoBend = g("wiener"), g("apoCutoff"), g("apoBend")
    px, py, po, mod = g("pX"), g("pY"), g("phaOff"), g("modulations")
    for d in range(r.nrDirs):
        r.pX[d], r.pY[d], r.phaOff[d] = px[d], py[d], po[d]
        for b in range(r.nrBands):
            r.modul[d][b] = mod[d][b]
    ph = g("phases")
    if ph is not None:
        r.hasPhases = 1
        for d in range(r.nrDirs):
            for i in range(r.nrPhases):
                r.phases[d][i] = ph[d][i]
    if isinstance(p, dict):
        r.filterStyle, r.rlIterations = int(p.get("filterStyle", 0)), int(p.get("rlIterations", 5))
    else:
        r.filterStyle, r.rlIterations = int(getattr(p, "filterStyle", 0)), int(getattr(p, "rlIterations", 5))
        otf = p.otf() if callable(getattr(p, "otf", None)) else None
        m = getattr(otf, "measured", None) if otf is not None else None
        if m is not None:  # measured OTF bands (OtfProvider.loadFromConfig with data)
            arr = np.array([[(z.real, z.imag) for z in band] for band in m["bands"]], dtype=np.float32)
            r._keep = arr
            r.otfData = arr.ctypes.data
            r.otfBands, r.otfSamples = arr.shape[0], arr.shape[1]
            r.otfCycles = float(m["cycles"])
    return r


def read_param(r: RefParam):
    n = r.nrDirs
    return dict(
        pX=[r.pX[d] for d in range(n)],
        pY=[r.pY[d] for d in range(n)],
        phaOff=[r.phaOff[d] for d in range(n)],
        modulations=[[r.modul[d][b] for b in range(r.nrBands)] for d in range(n)],
    )


def as_cplx_planes(a, dtype):
    """complex array (..., h, w) -> interleaved float array of the same layout."""
    a = np.ascontiguousarray(a)
    if np.iscomplexobj(a):
        out = np.empty(a.shape + (2,), dtype=dtype)
        out[..., 0] = a.real
        out[..., 1] = a.imag
        return out
    return np.ascontiguousarray(a, dtype=dtype)


def from_interleaved(a):
    return a[..., 0] + 1j * a[..., 1]


def fft2d(z, inverse=False, dtype=np.float32):
    d = as_cplx_planes(z, dtype)
    h, w = d.shape[-3], d.shape[-2]
    _chk(getattr(lib(), "ref_fft2d_" + _suf(dtype))(_ptr(d), w, h, int(inverse)))
    return from_interleaved(d)


def fourier_shift(z, kx, ky, dtype=np.float32):
    d = as_cplx_planes(z, dtype)
    n = d.shape[0]
    _chk(getattr(lib(), "ref_fourier_shift_" + _suf(dtype))(_ptr(d), n, C.c_double(kx), C.c_double(ky)))
    return from_interleaved(d)


def paste_freq(z, wo, ho, xoff=0, yoff=0, dtype=np.float32):
    d = as_cplx_planes(z, dtype)
    hi, wi = d.shape[0], d.shape[1]
    out = np.zeros((ho, wo, 2), dtype=dtype)
    _chk(getattr(lib(), "ref_paste_freq_" + _suf(dtype))(_ptr(out), wo, ho, _ptr(d), wi, hi, xoff, yoff))
    return from_interleaved(out)


def separation_matrix(phases, bands, modul=None):
    nP = len(phases)
    nc = 2 * bands - 1
    out = np.zeros((nc, nP, 2))
    ph = np.ascontiguousarray(phases, dtype=np.float64)
    m = None if modul is None else np.ascontiguousarray(modul, dtype=np.float64)
    _chk(lib().ref_separation_matrix(_ptr(ph), nP, bands, None if m is None else _ptr(m), _ptr(out)))
    return from_interleaved(out)


def matrix_inverse(M, pseudo=False):
    M = np.asarray(M, dtype=np.complex128)
    m, n = M.shape
    d = as_cplx_planes(M, np.float64)
    out = np.zeros((n, m, 2)) if pseudo else np.zeros((n, n, 2))
    _chk(lib().ref_matrix_inverse(_ptr(d), n, _ptr(out), int(pseudo), m))
    return from_interleaved(out)


def separate_bands(p, d, spectra, dtype=np.float32):
    r = make_param(p)
    sp = as_cplx_planes(spectra, dtype)
    nc = 2 * r.nrBands - 1
    out = np.zeros((nc, r.w, r.w, 2), dtype=dtype)
    _chk(getattr(lib(), "ref_separate_bands_" + _suf(dtype))(C.byref(r), d, _ptr(sp), _ptr(out)))
    return from_interleaved(out)


def otf_vector(p, vec, kx=0.0, ky=0.0, which=0, dtype=np.float32, band=0):
    """which: 0 writeOtfVector, 1 writeOtfWithAttVector, 2 applyOtf, 3 maskOtf (of `band`)."""
    r = make_param(p)
    d = as_cplx_planes(vec, dtype)
    h, w = d.shape[0], d.shape[1]
    _chk(getattr(lib(), "ref_otf_vector_" + _suf(dtype))(C.byref(r), _ptr(d), w, h, C.c_double(kx), C.c_double(ky), which,
                                                         int(band)))
    return from_interleaved(d)


def apo_vector(p, w, h, bend, cutoff, dtype=np.float32):
    r = make_param(p)
    out = np.zeros((h, w), dtype=dtype)
    _chk(getattr(lib(), "ref_apo_vector_" + _suf(dtype))(C.byref(r), _ptr(out), w, h, C.c_double(bend), C.c_double(cutoff)))
    return out


def attenuation_vector(p, w, h, strength, fwhm, kx=0.0, ky=0.0, dtype=np.float32):
    r = make_param(p)
    out = np.zeros((h, w), dtype=dtype)
    _chk(getattr(lib(), "ref_attenuation_vector_" + _suf(dtype))(
        C.byref(r), _ptr(out), w, h, C.c_double(strength), C.c_double(fwhm), C.c_double(kx), C.c_double(ky)))
    return out


def wiener_denominator(p, dtype=np.float32):
    r = make_param(p)
    out = np.zeros((2 * r.w, 2 * r.w), dtype=dtype)
    _chk(getattr(lib(), "ref_wiener_denominator_" + _suf(dtype))(C.byref(r), _ptr(out)))
    return out


def prepare_raw(p, raw, bgr=0.0, fade=10, dtype=np.float32):
    r = make_param(p)
    raw = np.ascontiguousarray(raw, dtype=dtype)
    out = np.zeros((r.nrDirs * r.nrPhases, r.w, r.w, 2), dtype=dtype)
    _chk(getattr(lib(), "ref_prepare_raw_" + _suf(dtype))(C.byref(r), _ptr(raw), C.c_double(bgr), fade, _ptr(out)))
    return from_interleaved(out)


def recon(p, spectra, otf_before_shift=False, clip_scale=0, dtype=np.float32):
    r = make_param(p)
    sp = as_cplx_planes(spectra, dtype)
    out = np.zeros((2 * r.w, 2 * r.w), dtype=dtype)
    _chk(getattr(lib(), "ref_recon_" + _suf(dtype))(C.byref(r), _ptr(sp), int(otf_before_shift), clip_scale, _ptr(out)))
    return out


def recon_raw(p, raw, bgr=0.0, fade=10, clip_scale=0, dtype=np.float32):
    r = make_param(p)
    raw = np.ascontiguousarray(raw, dtype=dtype)
    out = np.zeros((2 * r.w, 2 * r.w), dtype=dtype)
    _chk(getattr(lib(), "ref_recon_raw_" + _suf(dtype))(C.byref(r), _ptr(raw), C.c_double(bgr), fade, clip_scale, _ptr(out)))
    return out


def rl_deconvolve(img, otf, steps, in_freq=True, dtype=np.float32):
    """RLDeconvolution.deconvolve on a copy of img (complex, h x w) with the complex otf."""
    d = as_cplx_planes(img, dtype)
    o = as_cplx_planes(otf, dtype)
    h, w = d.shape[0], d.shape[1]
    _chk(getattr(lib(), "ref_rl_deconvolve_" + _suf(dtype))(_ptr(d), _ptr(o), w, h, int(steps), int(in_freq)))
    return from_interleaved(d)


def auto_correlation(band, kx, ky, dtype=np.float32):
    """Correlation.autoCorrelation: complex (double) for a square band spectrum."""
    d = as_cplx_planes(band, dtype)
    out = np.zeros(2)
    _chk(getattr(lib(), "ref_auto_correlation_" + _suf(dtype))(_ptr(d), d.shape[0], C.c_double(kx), C.c_double(ky),
                                                               _ptr(out)))
    return complex(out[0], out[1])


def widefield_raw(p, raw, bgr=0.0, fade=10, clip_scale=0, dtype=np.float32):
    """(widefield, filtered widefield), both 2w x 2w, of runReconstruction's Wiener path."""
    r = make_param(p)
    raw = np.ascontiguousarray(raw, dtype=dtype)
    wf = np.zeros((2 * r.w, 2 * r.w), dtype=dtype)
    fwf = np.zeros((2 * r.w, 2 * r.w), dtype=dtype)
    _chk(getattr(lib(), "ref_widefield_raw_" + _suf(dtype))(C.byref(r), _ptr(raw), C.c_double(bgr), fade,
                                                            clip_scale, _ptr(wf), _ptr(fwf)))
    return wf, fwf


def estimate(p, spectra, fit_band=1, fit_exclude=0.6, dtype=np.float32):
    """Returns (params dict, peaks [nDir,4], coarse [nDir,2])."""
    r = make_param(p)
    sp = as_cplx_planes(spectra, dtype)
    peaks = np.zeros((r.nrDirs, 4))
    coarse = np.zeros((r.nrDirs, 2))
    _chk(getattr(lib(), "ref_estimate_" + _suf(dtype))(C.byref(r), _ptr(sp), fit_band, C.c_double(fit_exclude), _ptr(peaks), _ptr(coarse)))
    return read_param(r), peaks, coarse


def common_region(p, b0, b1, kx, ky, dist=0.15, weight_limit=0.05, divide=True, dtype=np.float32):
    r = make_param(p)
    d0, d1 = as_cplx_planes(b0, dtype), as_cplx_planes(b1, dtype)
    _chk(getattr(lib(), "ref_common_region_" + _suf(dtype))(
        C.byref(r), _ptr(d0), _ptr(d1), C.c_double(kx), C.c_double(ky), C.c_double(dist), C.c_double(weight_limit), int(divide)))
    return from_interleaved(d0), from_interleaved(d1)


def locate_peak(vec, kmin, dtype=np.float32):
    d = as_cplx_planes(vec, dtype)
    out = np.zeros(4)
    _chk(getattr(lib(), "ref_locate_peak_" + _suf(dtype))(_ptr(d), d.shape[1], d.shape[0], C.c_double(kmin), _ptr(out)))
    return out


def fit_peak(p, band0, band1, kx, ky, weight_limit=0.05, search=2.5, dtype=np.float32):
    r = make_param(p)
    d0, d1 = as_cplx_planes(band0, dtype), as_cplx_planes(band1, dtype)
    out = np.zeros(4)
    grid = np.zeros((3, 10, 10, 2))
    _chk(getattr(lib(), "ref_fit_peak_" + _suf(dtype))(
        C.byref(r), _ptr(d0), _ptr(d1), C.c_double(kx), C.c_double(ky), C.c_double(weight_limit), C.c_double(search), _ptr(out), _ptr(grid)))
    return out, from_interleaved(grid)


def get_peak(p, band0, band1, kx, ky, weight_limit=0.05, dtype=np.float32):
    r = make_param(p)
    d0, d1 = as_cplx_planes(band0, dtype), as_cplx_planes(band1, dtype)
    out = np.zeros(2)
    _chk(getattr(lib(), "ref_get_peak_" + _suf(dtype))(
        C.byref(r), _ptr(d0), _ptr(d1), C.c_double(kx), C.c_double(ky), C.c_double(weight_limit), _ptr(out)))
    return out[0] + 1j * out[1]


def live_recon(p, raw_u16, dtype=np.float32):
    """raw_u16: (nStacks, nDir*nPha, w, w) uint16 -> (recon (nStacks,2w,2w), widefield (nStacks,w,w))."""
    r = make_param(p)
    raw = np.ascontiguousarray(raw_u16, dtype=np.uint16)
    if raw.ndim == 3:
        raw = raw[None]
    ns = raw.shape[0]
    out = np.zeros((ns, 2 * r.w, 2 * r.w), dtype=dtype)
    wf = np.zeros((ns, r.w, r.w), dtype=dtype)
    _chk(getattr(lib(), "ref_live_recon_" + _suf(dtype))(C.byref(r), _ptr(raw), ns, _ptr(out), _ptr(wf)))
    return out, wf


def live_refit(p, raw_u16, dtype=np.float32):
    r = make_param(p)
    raw = np.ascontiguousarray(raw_u16, dtype=np.uint16)
    peaks = np.zeros((r.nrDirs, 4))
    _chk(getattr(lib(), "ref_live_refit_" + _suf(dtype))(C.byref(r), _ptr(raw), _ptr(peaks)))
    return read_param(r), peaks


def fsin(x):
    return lib().ref_fsin(float(x))


def fcos(x):
    return lib().ref_fcos(float(x))
