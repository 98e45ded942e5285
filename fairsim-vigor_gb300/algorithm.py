"""SIM-algorithm call surface over the native library, mirroring the reference's static
classes: ``SimAlgorithm`` (S/SimAlgorithm.java:27), ``BandSeparation``
(S/BandSeparation.java:27), ``SimUtils`` (S/SimUtils.java:26), ``Correlation``
(S/Correlation.java:26), ``WienerFilter`` (S/WienerFilter.java:26) and the vector writers
of ``OtfProvider`` (S/OtfProvider.java:331-559). Arguments keep the reference's meaning
and order; every call runs in the native library on the GPU.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import native as N
from .vectors import Vec2dCplx, Vec2dReal, handles


def _cp(param):
    return N.to_c_param(param)


class OtfVectors:
    """OtfProvider's vector writers; ``param`` supplies the OTF and the vector pixel size."""

    @staticmethod
    def otfToVector(param, vec, band, kx, ky, useAtt, write):
        c = _cp(param)
        N.check(N.lib().fsim_otf_to_vector(vec.handle, C.byref(c), int(band), float(kx), float(ky), int(useAtt), int(write)))

    @staticmethod
    def applyOtf(param, vec, band, kx=0.0, ky=0.0):
        OtfVectors.otfToVector(param, vec, band, kx, ky, param.otf().isAttenuate(), False)

    @staticmethod
    def writeOtfVector(param, vec, band, kx, ky):
        OtfVectors.otfToVector(param, vec, band, kx, ky, False, True)

    @staticmethod
    def writeOtfWithAttVector(param, vec, band, kx, ky):
        OtfVectors.otfToVector(param, vec, band, kx, ky, param.otf().isAttenuate(), True)

    @staticmethod
    def writeApoVector(param, vec, bend, cutOff):
        N.check(N.lib().fsim_apo_vector(vec.handle, C.byref(_cp(param)), float(bend), float(cutOff)))

    @staticmethod
    def writeAttenuationVector(param, vec, strength, fwhm, kx, ky):
        N.check(N.lib().fsim_attenuation_vector(vec.handle, C.byref(_cp(param)), float(strength), float(fwhm), float(kx), float(ky)))

    @staticmethod
    def maskOtf(param, vec, kx, ky):
        N.check(N.lib().fsim_mask_otf(vec.handle, C.byref(_cp(param)), float(kx), float(ky)))


class WienerFilter:
    def __init__(self, sp):
        self.sp = sp

    def getDenominator(self, wParam: float) -> Vec2dReal:
        out = Vec2dReal(2 * self.sp.w, 2 * self.sp.w)
        N.check(N.lib().fsim_wiener_denominator(out.handle, C.byref(_cp(self.sp)), float(wParam)))
        return out


class BandSeparation:
    @staticmethod
    def createSeparationMatrix(phases, bands, fac=None) -> np.ndarray:
        """createSeparationMatrix (BandSeparation.java:40-114): the inverse (or pseudo-inverse)
        phase matrix, (2*bands-1) x nPhases complex. ``phases``: the phases of band 1, or the
        reference's per-band rows [bands-1][nPhases], whose band-b row must be b times the
        first (the only form separateBands builds)."""
        ph = np.asarray(phases, dtype=np.float64)
        if ph.ndim == 2:
            if ph.shape[0] != bands - 1:
                raise ValueError("#factors or #phases+1 != #bands")
            for b in range(1, bands - 1):
                if not np.allclose(ph[b], (b + 1) * ph[0], rtol=0, atol=1e-12):
                    raise ValueError("band %d phases are not %d times the first band's" % (b + 1, b + 1))
            ph = ph[0]
        ph = np.ascontiguousarray(ph)
        if fac is not None and len(fac) != bands:
            raise ValueError("#factors or #phases+1 != #bands")
        fa = None if fac is None else np.ascontiguousarray(fac, dtype=np.float64)
        out = np.zeros((2 * bands - 1, len(ph), 2), dtype=np.float64)
        N.check(N.lib().fsim_separation_matrix(ph.ctypes.data_as(C.c_void_p), len(ph), int(bands),
                                               None if fa is None else fa.ctypes.data_as(C.c_void_p),
                                               out.ctypes.data_as(C.c_void_p)))
        return out[..., 0] + 1j * out[..., 1]

    @staticmethod
    def separateBands(inp, out, phases, bands, fac=None):
        """separateBands(in, out, phases[] | phaOff, bands, fac) (BandSeparation.java:131-197)."""
        if np.isscalar(phases):
            n = len(inp)
            phases = [(2 * math.pi * p) / n + float(phases) for p in range(n)]
        if len(inp) != len(phases):
            raise IndexError("#input images != phases per band")
        if len(out) != 2 * bands - 1:
            raise IndexError("#output images != #bands*2-1")
        ph = np.ascontiguousarray(phases, dtype=np.float64)
        fa = None if fac is None else np.ascontiguousarray(fac, dtype=np.float64)
        N.check(N.lib().fsim_separate_bands(handles(inp), len(inp), handles(out), len(out),
                                            ph.ctypes.data_as(C.c_void_p), int(bands),
                                            None if fa is None else fa.ctypes.data_as(C.c_void_p)))


class SimUtils:
    @staticmethod
    def placeFreq(inV, outV):
        outV.pasteFreq(inV)

    @staticmethod
    def fourierShift(inV, kx, ky):
        inV.fft2d(True)
        inV.fourierShift(kx, -ky)
        inV.fft2d(False)

    @staticmethod
    def pasteAndFourierShift(inV, outV, kx, ky, doFastShift):
        if not doFastShift:
            outV.pasteFreq(inV, 0, 0)
            outV.fft2d(True)
            outV.fourierShift(kx, -ky)
            outV.fft2d(False)
        else:
            xFrac = kx - math.floor(kx)
            yFrac = -ky - math.floor(-ky)
            inV.fft2d(True)
            inV.fourierShift(xFrac, yFrac)
            inV.fft2d(False)
            outV.pasteFreq(inV, int(math.floor(kx)), int(math.floor(-ky)))

    @staticmethod
    def spatial(inV) -> Vec2dReal:
        tmp = inV.duplicate()
        tmp.fft2d(True)
        out = Vec2dReal(inV.w, inV.h)
        out.copy(tmp)
        return out


class Correlation:
    @staticmethod
    def commonRegion(band0, band1, bn0, bn1, otf_param, kx, ky, dist, weightLimit, divideByOtf):
        N.check(N.lib().fsim_common_region(band0.handle, band1.handle, C.byref(_cp(otf_param)), float(kx), float(ky),
                                           float(dist), float(weightLimit), int(divideByOtf)))

    @staticmethod
    def locatePeak(vec, kMin):
        out = (C.c_double * 4)()
        N.check(N.lib().fsim_locate_peak(vec.handle, float(kMin), out))
        return list(out)

    @staticmethod
    def fitPeak(band0, band1, bn0, bn1, otf_param, kx, ky, weightLimit, search, grid=None):
        out = (C.c_double * 4)()
        g = (C.c_double * 600)() if grid is not None else None
        N.check(N.lib().fsim_fit_peak(band0.handle, band1.handle, C.byref(_cp(otf_param)), float(kx), float(ky),
                                      float(weightLimit), float(search), out, g))
        if grid is not None:
            grid[:] = np.array(list(g)).reshape(3, 10, 10, 2)
        return list(out)

    @staticmethod
    def autoCorrelation(inV, kx, ky):
        """Correlation.autoCorrelation (S/Correlation.java:294-325): Wicker's phase estimate."""
        re, im = C.c_double(), C.c_double()
        N.check(N.lib().fsim_auto_correlation(inV.handle, float(kx), float(ky), C.byref(re), C.byref(im)))
        return complex(re.value, im.value)

    @staticmethod
    def getPeak(band0, band1, bn0, bn1, otf_param, kx, ky, weightLimit):
        out = (C.c_double * 2)()
        N.check(N.lib().fsim_get_peak(band0.handle, band1.handle, C.byref(_cp(otf_param)), float(kx), float(ky),
                                      float(weightLimit), out))
        return complex(out[0], out[1])


class RLDeconvolution:
    @staticmethod
    def deconvolve(img, otf, steps, inputIsInFreqSpace=False):
        """RLDeconvolution.deconvolve (S/RLDeconvolution.java:45-103) on device vectors."""
        N.check(N.lib().fsim_rl_deconvolve(img.handle, otf.handle, int(steps), int(bool(inputIsInFreqSpace))))


class SimAlgorithm:
    @staticmethod
    def runReconstruction(param, inFFT, otfBeforeShift=False, clipScale=0) -> Vec2dReal:
        """runReconstruction (SimAlgorithm.java:268): inFFT[dir][phase] spectra; CLIPSCALE 0/1/2
        = NONE/CLIP/BOTH. Runs op by op on device vectors (the plain, one-dataset GPU form)."""
        flat = [v for d in inFFT for v in d]
        out = Vec2dReal(2 * param.w, 2 * param.w)
        N.check(N.lib().fsim_run_reconstruction(C.byref(_cp(param)), handles(flat), out.handle,
                                                int(bool(otfBeforeShift)), int(clipScale)))
        return out

    @staticmethod
    def estimateParameters(param, inFFT, fitBand=1, fitExclude=0.6):
        """estimateParameters (SimAlgorithm.java:37): writes shifts, phase offsets and
        modulations into ``param``; returns the fitted [kx, ky, phase, mag] per direction."""
        flat = [v for d in inFFT for v in d]
        c = _cp(param)
        peaks = (C.c_double * (4 * param.nrDirs))()
        N.check(N.lib().fsim_estimate_parameters(C.byref(c), handles(flat), int(fitBand), float(fitExclude), peaks))
        param.set_from(N.from_c_param(c))
        return np.array(list(peaks)).reshape(param.nrDirs, 4)
