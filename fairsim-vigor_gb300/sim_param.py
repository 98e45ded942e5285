"""Host-side mirror of fairSIM's ``SimParam`` / ``SimParam.Dir`` / ``OtfProvider``.

Field meanings follow the reference:
  * ``SimParam.create(bands, dirs, phases, size, micronsPerPxl, otf)``
    (org/fairsim/sim_algorithm/SimParam.java:118-124);
  * ``Dir.setPxPy`` stores the highest-band shift divided by (nBands-1), ``px(b) = pX*b``
    (SimParam.java:536-562);
  * phases ``2*pi*i/nPhases + phaOff`` (SimParam.java:463-477);
  * modulations clamped to [0.3, 1.1] by ``getModulations`` (SimParam.java:598-607);
  * ``OtfProvider.fromEstimate(na, lambda, a)`` with cutoff ``1000/(lambda/na/2)`` cycles/micron
    (OtfProvider.java:96-127), attenuation defaults 0.99 / 1.2 (OtfProvider.java:64);
  * ``loadConfig`` / ``saveConfig`` / ``loadFromConfig`` read and write the reference's
    configuration folders (conf.py; SimParam.java:645-726, OtfProvider.java:575-676).

These are plain parameter records: every computation on them runs in the native library.
"""
from __future__ import annotations

import copy
import math
from dataclasses import dataclass, field
from typing import List, Optional


# SimParam.FilterStyle (S/SimParam.java:33-43), by ordinal
FILTER_WIENER, FILTER_RL_IN, FILTER_RL_OUT, FILTER_RL_BOTH = 0, 1, 2, 3
FILTER_STYLES = ["Wiener", "RLin", "RLout", "RLboth"]


class OtfProvider:
    """``OtfProvider.fromEstimate`` parameters (S/OtfProvider.java:96-127)."""

    def __init__(self, na: float, em_wavelength: float, a: float):
        if a < 0 or a > 1 or na < 0.3 or na > 2.2 or em_wavelength < 300 or em_wavelength > 1500:
            raise ValueError("unphysical input parameters")
        self.na = float(na)
        self.emWavelength = float(em_wavelength)
        self.a = float(a)
        self.attStrength = 0.99
        self.attFWHM = 1.2
        self.useAttenuation = False

    @staticmethod
    def fromEstimate(na: float, em_wavelength: float, a: float) -> "OtfProvider":
        return OtfProvider(na, em_wavelength, a)

    def getCutoff(self) -> float:
        return 1000.0 / (self.emWavelength / self.na / 2.0)

    def setAttenuation(self, strength: float, fwhm: float) -> None:
        self.attStrength = float(strength)
        self.attFWHM = float(fwhm)

    def switchAttenuation(self, on: bool) -> None:
        self.useAttenuation = bool(on)

    def isAttenuate(self) -> bool:
        return self.useAttenuation

    def duplicate(self) -> "OtfProvider":
        return copy.deepcopy(self)

    # measured OTFs (OtfProvider.loadFromConfig with a "data" folder) keep their samples
    # here: per band, complex values at cyclesPerMicron spacing
    isEstimate = True
    measured = None  # dict(bands=[[complex, ...], ...], cycles=float) or None

    @staticmethod
    def fromMeasured(na: float, em_wavelength: float, bands, cycles_per_sample: float) -> "OtfProvider":
        """A measured OTF as loadFromConfig builds it from band data (S/OtfProvider.java:588-621):
        ``bands`` holds one sequence of complex samples per band, ``cycles_per_sample`` their
        spacing in cycles/micron; attenuation defaults 0.99 / 1.2, switched off."""
        ret = OtfProvider.__new__(OtfProvider)
        ret.na, ret.emWavelength, ret.a = float(na), float(em_wavelength), 1.0
        ret.attStrength, ret.attFWHM, ret.useAttenuation = 0.99, 1.2, False
        ret.isEstimate = False
        ret.measured = dict(bands=[[complex(z) for z in b] for b in bands], cycles=float(cycles_per_sample))
        return ret

    @staticmethod
    def loadFromConfig(cfg) -> "OtfProvider":
        """OtfProvider.loadFromConfig (S/OtfProvider.java:575-633): the "otf2d" folder;
        an estimate (NA, emission, a-estimate) or measured band data, then attenuation."""
        from .conf import from_bytes

        fld = cfg.cd("otf2d")
        if not fld.contains("data"):
            ret = OtfProvider.fromEstimate(fld.getDbl("NA").val(), fld.getInt("emission").val(),
                                           fld.getDbl("a-estimate").val())
        else:
            data = fld.cd("data")
            nb, ns = data.getInt("bands").val(), data.getInt("samples").val()
            bands = []
            for b in range(nb):
                v = from_bytes(data.getData("band-%d" % b).val())
                bands.append([complex(v[2 * i], v[2 * i + 1]) for i in range(ns)])
            ret = OtfProvider.fromMeasured(fld.getDbl("NA").val(), fld.getInt("emission").val(), bands,
                                           data.getDbl("cycles").val())
        if fld.contains("attenuation"):
            att = fld.cd("attenuation")
            ret.setAttenuation(att.getDbl("strength").val(), att.getDbl("FWHM").val())
            ret.switchAttenuation(True)
        return ret

    # ---- the reference's instance API: sample tables, scalar lookups, vector writers ------

    SAMPLES_ESTIMATE = 512  # samplesLateral of an estimated OTF (S/OtfProvider.java:45)
    vecCyclesPerMicron = -1.0

    @staticmethod
    def valIdealOTF(dist: float) -> float:
        """OtfProvider.valIdealOTF (S/OtfProvider.java:74-78): the OTF of an aberration-free
        lens with a circular pupil, dist in [0, 1] of the cutoff (0 outside)."""
        if dist < 0 or dist > 1:
            return 0.0
        return (2 / math.pi) * (math.acos(dist) - dist * math.sqrt(1 - dist * dist))

    @staticmethod
    def valAttenuation(dist: float, strength: float, fwhm: float) -> float:
        """OtfProvider.valAttenuation (S/OtfProvider.java:238-240), a float in the reference."""
        import numpy as np

        return float(np.float32(1 - strength * math.exp(-(dist ** 2) / (2 * (fwhm / 2.355) ** 2))))

    def setPixelSize(self, cyclesPerMicron: float) -> None:
        """OtfProvider.setPixelSize (S/OtfProvider.java:226-230): frequency spacing of the
        vectors the writers below fill, in cycles/micron."""
        if cyclesPerMicron <= 0:
            raise ValueError("pxl size must be positive")
        self.vecCyclesPerMicron = float(cyclesPerMicron)

    def setAttenuationStrength(self, strength: float) -> None:
        self.setAttenuation(strength, self.attFWHM)

    def setAttenuationFWHM(self, fwhm: float) -> None:
        self.setAttenuation(self.attStrength, fwhm)

    def getAttStr(self, band: int = 0) -> float:
        return self.attStrength

    def getAttFWHM(self, band: int = 0) -> float:
        return self.attFWHM

    def isMultiBand(self) -> bool:
        return self.measured is not None and len(self.measured["bands"]) > 1

    def _tables(self):
        """(cycles per sample, vals, valsOnlyAtt, valsAtt) as float32 arrays [band][sample]:
        fromEstimate's samples (S/OtfProvider.java:105-120) or the measured bands, and the
        attenuation cache of setAttenuation (:276-287)."""
        import numpy as np

        if self.measured is None:
            ns = self.SAMPLES_ESTIMATE
            cps = self.getCutoff() / ns
            v = np.array([[np.float32(self.valIdealOTF(i / ns) * (self.a ** (i / ns))) for i in range(ns)]],
                         dtype=np.complex64)
        else:
            cps = self.measured["cycles"]
            v = np.array(self.measured["bands"], dtype=np.complex64)
        only = np.array([[self.valAttenuation(i * cps, self.attStrength, self.attFWHM) for i in range(v.shape[1])]],
                        dtype=np.float32).repeat(v.shape[0], axis=0)
        att = (v.real * only + 1j * (v.imag * only)).astype(np.complex64)
        return cps, v, only, att

    def _band(self, band: int, nbands: int) -> int:
        if not self.isMultiBand():
            band = 0
        if band >= nbands or band < 0:
            raise IndexError("band idx too high or <0")
        return band

    def getOtfVal(self, band: int, cycl: float, att: bool) -> complex:
        """OtfProvider.getOtfVal (S/OtfProvider.java:189-222): the sample at floor(pos)
        (its 'interpolation' weighs the lower sample twice: (1-f)*v + f*v in float)."""
        import numpy as np

        cps, v, _, va = self._tables()
        band = self._band(band, v.shape[0])
        if cycl < 0:
            raise IndexError("cylc negative!")
        if cycl >= self.getCutoff():
            return 0j
        pos = cycl / cps
        if math.ceil(pos) >= v.shape[1]:
            return 0j
        lpos = int(math.floor(pos))
        f = np.float32(pos - lpos)
        z = (va if att else v)[band][lpos]
        lo = np.complex64(complex(np.float32(z.real * (np.float32(1) - f)), np.float32(z.imag * (np.float32(1) - f))))
        hi = np.complex64(complex(np.float32(z.real * f), np.float32(z.imag * f)))
        return complex(np.float32(lo.real + hi.real), np.float32(lo.imag + hi.imag))

    def getAttVal(self, band: int, cycl: float) -> float:
        """OtfProvider.getAttVal (S/OtfProvider.java:246-269): 1 beyond the cutoff, else the
        attenuation sample at floor(pos) weighed f + (1-f) in float."""
        import numpy as np

        cps, v, only, _ = self._tables()
        band = self._band(band, v.shape[0])
        if cycl < 0:
            raise IndexError("cylc negative!")
        if cycl >= self.getCutoff():
            return 1.0
        pos = cycl / cps
        lpos = int(math.floor(pos))
        f = np.float32(pos - lpos)
        s = only[band][lpos]
        return float(np.float32(np.float32(s * f) + np.float32(s * (np.float32(1) - f))))

    def printState(self, html: bool = False) -> str:
        """OtfProvider.printState (S/OtfProvider.java:165-176)."""
        lam = "λ<sub>em</sub>" if html else "lambda"
        ret = "NA %4.2f, %s %4.0f, " % (self.na, lam, self.emWavelength)
        return ret + ("(est., a=%4.2f)" % self.a if self.isEstimate else "(from file)")

    def _vector_param(self, vec):
        """A parameter record that gives the library this OTF and a vector frequency spacing
        of vecCyclesPerMicron (the library's spacing is 1/(w * micronsPerPixel))."""
        if self.vecCyclesPerMicron <= 0:
            raise RuntimeError("Vector pixel size not initialized")
        nb = max(2, len(self.measured["bands"]) if self.isMultiBand() else 2)
        return SimParam.create(nb, 1, 2 * nb - 1, vec.w, 1.0 / (vec.w * self.vecCyclesPerMicron), self)

    def otfToVector(self, vec, band: int, kx: float, ky: float, useAtt: bool, write: bool) -> None:
        """OtfProvider.otfToVector (S/OtfProvider.java:331-373), in the library."""
        from .algorithm import OtfVectors

        OtfVectors.otfToVector(self._vector_param(vec), vec, band, kx, ky, useAtt, write)

    def applyOtf(self, vec, band: int, kx: float = 0.0, ky: float = 0.0) -> None:
        self.otfToVector(vec, band, kx, ky, self.useAttenuation, False)

    def writeOtfVector(self, vec, band: int, kx: float, ky: float) -> None:
        self.otfToVector(vec, band, kx, ky, False, True)

    def writeOtfWithAttVector(self, vec, band: int, kx: float, ky: float) -> None:
        self.otfToVector(vec, band, kx, ky, self.useAttenuation, True)

    def writeApoVector(self, vec, bend: float, cutOff: float) -> None:
        """OtfProvider.writeApoVector (S/OtfProvider.java:437-492), in the library."""
        from .algorithm import OtfVectors

        OtfVectors.writeApoVector(self._vector_param(vec), vec, bend, cutOff)

    def writeAttenuationVector(self, vec, strength: float, fwhm: float, kx: float, ky: float) -> None:
        """OtfProvider.writeAttenuationVector (S/OtfProvider.java:503-529), in the library."""
        from .algorithm import OtfVectors

        OtfVectors.writeAttenuationVector(self._vector_param(vec), vec, strength, fwhm, kx, ky)

    def maskOtf(self, vec, kx: float, ky: float) -> None:
        """OtfProvider.maskOtf (S/OtfProvider.java:538-559), in the library."""
        from .algorithm import OtfVectors

        OtfVectors.maskOtf(self._vector_param(vec), vec, kx, ky)

    def saveConfig(self, cfg) -> None:
        """OtfProvider.saveConfig (S/OtfProvider.java:636-676) into folder ``cfg``."""
        from .conf import to_bytes

        fld = cfg.mk("otf2d")
        fld.newDbl("NA").setVal(self.na)
        fld.newInt("emission").setVal(int(self.emWavelength))
        if self.isEstimate:
            fld.newDbl("a-estimate").setVal(self.a)
        else:
            data = fld.mk("data")
            bands = self.measured["bands"]
            data.newInt("bands").setVal(len(bands))
            data.newInt("samples").setVal(len(bands[0]))
            data.newDbl("cycles").setVal(self.measured["cycles"])
            for b, vals in enumerate(bands):
                flat = []
                for z in vals:
                    flat += [z.real, z.imag]
                data.newData("band-%d" % b).setVal(to_bytes(flat))
        if self.useAttenuation:
            att = fld.mk("attenuation")
            att.newDbl("strength").setVal(self.attStrength)
            att.newDbl("FWHM").setVal(self.attFWHM)


@dataclass
class Dir:
    nrBands: int
    nrPhases: int
    pX: float = 0.0
    pY: float = 0.0
    phaOff: float = 0.0
    phases: Optional[List[float]] = None  # individual phases (None = equidistant)
    modul: List[float] = field(default_factory=list)

    def __post_init__(self):
        if self.nrBands < 2:
            raise ValueError("bands < 2, not useful")
        if self.nrPhases < 2 * self.nrBands - 1:
            raise ValueError("not enough phases for bands")
        if not self.modul:
            self.modul = [1.0] * self.nrBands

    def setPxPy(self, x: float, y: float) -> None:
        self.pX = x / (self.nrBands - 1)
        self.pY = y / (self.nrBands - 1)

    def px(self, band: int) -> float:
        return self.pX * band

    def py(self, band: int) -> float:
        return self.pY * band

    def setPhaOff(self, p: float) -> None:
        self.phaOff = float(p)

    def getPhaOff(self) -> float:
        return self.phaOff

    def setPhases(self, pha, reset: bool) -> None:
        if len(pha) != self.nrPhases:
            raise ValueError("Length mismatch")
        if reset:
            self.phaOff = 0.0
        self.phases = [float(p) for p in pha]

    def getPhases(self) -> List[float]:
        base = self.phases or [(2 * math.pi / self.nrPhases) * i for i in range(self.nrPhases)]
        return [b + self.phaOff for b in base]

    def setModulation(self, b: int, m: float) -> bool:
        self.modul[b] = float(m)
        return 0.3 < m < 1.1

    def getModulations(self) -> List[float]:
        return [min(max(m, 0.3), 1.1) for m in self.modul]

    def nrComp(self) -> int:
        return 2 * self.nrBands - 1

    def nrBand(self) -> int:
        return self.nrBands

    def nrPha(self) -> int:
        return self.nrPhases

    def _fail_band(self, b: int) -> None:
        if b < 0 or b >= self.nrBands:  # Dir.failBand (S/SimParam.java:429-432)
            raise IndexError("Wrong band index")

    def getPhase(self, i: int) -> float:
        """Phase i without the offset (S/SimParam.java:485-487)."""
        base = self.phases or [(2 * math.pi / self.nrPhases) * k for k in range(self.nrPhases)]
        return base[i]

    def resetPhases(self) -> None:
        """Back to equidistant phases (S/SimParam.java:463-467)."""
        self.phases = None

    def getPxPyAngle(self, band: int) -> float:
        """atan2 of band's shift (S/SimParam.java:573-576)."""
        self._fail_band(band)
        return math.atan2(self.pY * band, self.pX * band)

    def getPxPyLen(self, band: int) -> float:
        """Length of band's shift (S/SimParam.java:584-587)."""
        self._fail_band(band)
        return math.hypot(self.pY * band, self.pX * band)

    def getRawModulations(self) -> List[float]:
        """Modulations without the [0.3, 1.1] clamp (S/SimParam.java:609-613)."""
        return list(self.modul)


class SimParam:
    """2D subset of ``SimParam`` (S/SimParam.java:31-615)."""

    def __init__(self, bands: int, dirs: int, phases: int, size: int, microns_per_pxl: float,
                 otf: Optional[OtfProvider]):
        if dirs < 1:
            raise ValueError("dirs < 1, not useful")
        self.nrDirs = int(dirs)
        self.nrBands = int(bands)
        self.nrPhases = int(phases)
        self.directions = [Dir(bands, phases) for _ in range(dirs)]
        self.imgSize = int(size)
        self.micronsPerPixel = float(microns_per_pxl)
        self._otf = otf
        self.wienerFilterParameter = 0.05
        self.apoCutOff = 2.0
        self.apoBend = 0.9  # runReconstruction's fixed bend (SimAlgorithm.java:277)
        self.filterStyle = FILTER_WIENER  # SimParam.FilterStyle ordinal
        self.rlIterations = 5
        self.imgSeq = "PAZ"  # IMGSEQ name (input order of the raw frames, stored only)
        self.clipScale = "BOTH"  # CLIPSCALE name (BOTH, CLIP, NONE), stored only (S/SimParam.java:62-63)
        self.paramDate = 0   # "timestamp" of the parameter set, ms since 1970

    @staticmethod
    def create(bands, dirs, phases, size, microns_per_pxl, otf) -> "SimParam":
        return SimParam(bands, dirs, phases, size, microns_per_pxl, otf)

    def dir(self, i: int) -> Dir:
        return self.directions[i]

    def nrDir(self) -> int:
        return self.nrDirs

    def nrBand(self) -> int:
        return self.nrBands

    def otf(self) -> OtfProvider:
        return self._otf

    def setFilterStyle(self, style) -> None:
        """SimParam.setFilterStyle: FILTER_WIENER, FILTER_RL_IN, FILTER_RL_OUT, FILTER_RL_BOTH
        (or their names "Wiener", "RLin", "RLout", "RLboth")."""
        if isinstance(style, str):
            style = FILTER_STYLES.index(style)
        if style not in range(4):
            raise ValueError("unknown filter style %r" % (style,))
        self.filterStyle = int(style)

    def getFilterStyle(self) -> int:
        return self.filterStyle

    def getImgSeq(self) -> str:
        return self.imgSeq

    def setImgSeq(self, seq: str) -> "SimParam":
        """SimParam.setImgSeq: "PAZ", "PZA" or "ZAP" (S/SimParam.java:223-226, 753-756)."""
        if seq not in ("PAZ", "PZA", "ZAP"):
            raise ValueError("unknown image order %r" % (seq,))
        self.imgSeq = seq
        return self

    def getClipScale(self) -> str:
        return self.clipScale

    def setClipScale(self, mode: str) -> "SimParam":
        """SimParam.setClipScale: "BOTH", "CLIP" or "NONE" (S/SimParam.java:234-237, 735-738);
        runReconstruction takes it as 2 / 1 / 0."""
        if mode not in ("BOTH", "CLIP", "NONE"):
            raise ValueError("unknown clip/scale mode %r" % (mode,))
        self.clipScale = mode
        return self

    def useWienerFilter(self) -> bool:
        return self.filterStyle in (FILTER_WIENER, FILTER_RL_IN)

    def useRLonInput(self) -> bool:
        return self.filterStyle in (FILTER_RL_BOTH, FILTER_RL_IN)

    def useRLonOutput(self) -> bool:
        return self.filterStyle in (FILTER_RL_BOTH, FILTER_RL_OUT)

    def setRLiterations(self, n: int) -> None:
        self.rlIterations = int(n)

    def getRLiterations(self) -> int:
        return self.rlIterations

    def setOtf(self, otf: OtfProvider) -> "SimParam":
        """SimParam.otf(OtfProvider): attach the OTF."""
        self._otf = otf
        return self

    def saveConfig(self, cfg) -> None:
        """SimParam.saveConfig (S/SimParam.java:645-672): a "sim-param" folder in ``cfg``."""
        fd = cfg.mk("sim-param")
        fd.newInt("nr-angles").setVal(self.nrDirs)
        fd.newInt("nr-bands").setVal(self.nrBands)
        fd.newInt("nr-phases").setVal(self.nrPhases)
        fd.newStr("img-seq").setVal(self.imgSeq)
        fd.newInt("img-size-pxl").setVal(self.imgSize)
        fd.newDbl("microns-per-pxl").setVal(self.micronsPerPixel)
        fd.newDbl("wiener-parameter").setVal(self.wienerFilterParameter)
        fd.newDbl("apodization-cutoff").setVal(self.apoCutOff)
        fd.newTDE("timestamp").set(self.paramDate)
        for d, dr in enumerate(self.directions):
            df = fd.mk("dir-%d" % d)
            df.newDbl("shift").setVal(dr.pX * (dr.nrBands - 1), dr.pY * (dr.nrBands - 1))
            df.newDbl("phase-offset").setVal(dr.phaOff)
            df.newDbl("modulations").setVal(*dr.modul)
            if dr.phases is not None:
                df.newDbl("phases").setVal(*dr.phases)

    @staticmethod
    def loadConfig(cfg, otf: Optional[OtfProvider] = None) -> "SimParam":
        """SimParam.loadConfig (S/SimParam.java:675-726) from the "sim-param" folder of
        ``cfg``; the OTF is attached separately (``setOtf`` / OtfProvider.loadFromConfig)."""
        fd = cfg.cd("sim-param")
        ret = SimParam(fd.getInt("nr-bands").val(), fd.getInt("nr-angles").val(), fd.getInt("nr-phases").val(),
                       fd.getInt("img-size-pxl").val(), fd.getDbl("microns-per-pxl").val(), otf)
        if fd.contains("timestamp"):
            ret.paramDate = fd.getTDE("timestamp").val()
        ret.imgSeq = fd.getStr("img-seq").val().strip()
        ret.setWienerFilter(fd.getDbl("wiener-parameter").val())
        ret.setApoCutoff(fd.getDbl("apodization-cutoff").val())
        for d in range(ret.nrDirs):
            df = fd.cd("dir-%d" % d)
            dr = ret.dir(d)
            sh = df.getDbl("shift").vals()
            if len(sh) < 2:
                raise ValueError("Array too short")
            dr.setPxPy(sh[0], sh[1])
            dr.setPhaOff(df.getDbl("phase-offset").val())
            for i, m in enumerate(df.getDbl("modulations").vals()):
                dr.setModulation(i, m)
            if df.contains("phases"):
                dr.setPhases(df.getDbl("phases").vals(), False)
        return ret

    def pxlSizeCyclesMicron(self) -> float:
        return 1.0 / (self.imgSize * self.micronsPerPixel)

    def setPxlSize(self, size: int, microns: Optional[float] = None) -> "SimParam":
        self.imgSize = int(size)
        if microns is not None:
            self.micronsPerPixel = float(microns)
        return self

    def setWienerFilter(self, w: float) -> "SimParam":
        self.wienerFilterParameter = float(w)
        return self

    def getWienerFilter(self) -> float:
        return self.wienerFilterParameter

    def setApoCutoff(self, a: float) -> "SimParam":
        self.apoCutOff = float(a)
        return self

    def getApoCutoff(self) -> float:
        return self.apoCutOff

    def vectorWidth(self) -> int:
        return self.imgSize

    def vectorHeight(self) -> int:
        return self.imgSize

    def duplicate(self) -> "SimParam":
        return copy.deepcopy(self)

    # flat views used by the native bindings (and by the oracle's ctypes struct)
    @property
    def w(self):
        return self.imgSize

    @property
    def na(self):
        return self._otf.na

    @property
    def emWavelength(self):
        return self._otf.emWavelength

    @property
    def otfA(self):
        return self._otf.a

    @property
    def useAttenuation(self):
        return self._otf.useAttenuation

    @property
    def attStrength(self):
        return self._otf.attStrength

    @property
    def attFWHM(self):
        return self._otf.attFWHM

    @property
    def wiener(self):
        return self.wienerFilterParameter

    @property
    def apoCutoff(self):
        return self.apoCutOff

    @property
    def pX(self):
        return [d.pX for d in self.directions]

    @property
    def pY(self):
        return [d.pY for d in self.directions]

    @property
    def phaOff(self):
        return [d.phaOff for d in self.directions]

    @property
    def modulations(self):
        return [list(d.modul) for d in self.directions]

    @property
    def phases(self):
        if all(d.phases is None for d in self.directions):
            return None
        return [d.phases or [(2 * math.pi / d.nrPhases) * i for i in range(d.nrPhases)] for d in self.directions]

    def set_from(self, vals: dict) -> None:
        for d in range(self.nrDirs):
            self.directions[d].pX = vals["pX"][d]
            self.directions[d].pY = vals["pY"][d]
            self.directions[d].phaOff = vals["phaOff"][d]
            self.directions[d].modul = list(vals["modulations"][d])
