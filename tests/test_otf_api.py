"""OtfProvider's instance API on the host (S/OtfProvider.java:67-287): the ideal OTF, the
attenuation, the floor-indexed sample lookups getOtfVal / getAttVal, checked against the
oracle's otfToVector (which writes getOtfVal at every pixel), and the argument checks of
the vector writers, which run before anything reaches the library."""
import math

import numpy as np
import pytest


def param(fs, n=64, pxl=0.08, a=0.3, att=None, otf=None):
    otf = otf or fs.OtfProvider.fromEstimate(1.4, 525, a)
    if att:
        otf.setAttenuation(*att)
        otf.switchAttenuation(True)
    return fs.SimParam.create(2, 3, 3, n, pxl, otf)


def test_ideal_otf_and_attenuation_values(fs):
    O = fs.OtfProvider
    assert O.valIdealOTF(0.0) == 1.0 and O.valIdealOTF(1.0) == 0.0
    assert O.valIdealOTF(-0.1) == 0.0 and O.valIdealOTF(1.1) == 0.0
    d = 0.37
    assert O.valIdealOTF(d) == pytest.approx((2 / math.pi) * (math.acos(d) - d * math.sqrt(1 - d * d)), rel=1e-15)
    v = O.valAttenuation(1.1, 0.95, 1.3)
    assert v == float(np.float32(1 - 0.95 * math.exp(-(1.1 ** 2) / (2 * (1.3 / 2.355) ** 2))))
    assert O.valAttenuation(0.0, 0.95, 1.3) == pytest.approx(0.05, abs=1e-7)


@pytest.mark.parametrize("a,att", [(1.0, None), (0.3, None), (0.3, (0.95, 1.3))])
def test_get_otf_val_matches_the_oracle_vectors(fs, oracle, a, att):
    n, pxl = 64, 0.08
    sp = param(fs, n, pxl, a, att)
    otf = sp.otf()
    cpm = 1 / (n * pxl)
    for which, use_att in ((0, False), (1, True)):  # writeOtfVector, writeOtfWithAttVector
        vec = oracle.otf_vector(sp, np.zeros((n, n), complex), 0.0, 0.0, which=which)
        for x in range(n // 2):
            got = np.complex64(otf.getOtfVal(0, x * cpm, use_att and otf.isAttenuate()))
            assert got == vec[0, x], (which, x)
    # beyond the cutoff: zero; negative radius and bad band: errors as in the reference
    assert otf.getOtfVal(0, otf.getCutoff(), False) == 0
    with pytest.raises(IndexError):
        otf.getOtfVal(0, -1.0, False)
    assert otf.getOtfVal(5, 1.0, False) == otf.getOtfVal(0, 1.0, False)  # one band: index ignored


def test_get_otf_val_of_measured_bands(fs, oracle):
    n, pxl = 64, 0.08
    rng = np.random.default_rng(7)
    bands = [[complex(*rng.normal(size=2)) for _ in range(300)] for _ in range(2)]
    otf = fs.OtfProvider.fromMeasured(1.4, 525, bands, 0.02)
    assert otf.isMultiBand()
    sp = param(fs, n, pxl, otf=otf)
    cpm = 1 / (n * pxl)
    for band in (0, 1):
        vec = oracle.otf_vector(sp, np.zeros((n, n), complex), 0.0, 0.0, which=0, band=band)
        for x in range(n // 2):
            assert np.complex64(otf.getOtfVal(band, x * cpm, False)) == vec[0, x], (band, x)
    with pytest.raises(IndexError):
        otf.getOtfVal(2, 1.0, False)


def test_get_att_val(fs):
    otf = fs.OtfProvider.fromEstimate(1.4, 525, 0.3)
    otf.setAttenuation(0.9, 1.5)
    cut = otf.getCutoff()
    assert otf.getAttVal(0, cut) == 1.0 and otf.getAttVal(0, cut + 1) == 1.0
    for c in (0.0, 0.5, 1.0, 2.0, 4.0):
        assert otf.getAttVal(0, c) == pytest.approx(fs.OtfProvider.valAttenuation(c, 0.9, 1.5), abs=2e-3)
    assert (otf.getAttStr(), otf.getAttFWHM()) == (0.9, 1.5)
    otf.setAttenuationStrength(0.8)
    otf.setAttenuationFWHM(1.1)
    assert (otf.getAttStr(0), otf.getAttFWHM(0)) == (0.8, 1.1)


def test_vector_writers_need_a_pixel_size(fs):
    otf = fs.OtfProvider.fromEstimate(1.4, 525, 0.3)
    with pytest.raises(ValueError):
        otf.setPixelSize(0)

    class Vec:  # only the size is read before the library call
        w = h = 64

    for call in (lambda v: otf.applyOtf(v, 0), lambda v: otf.writeOtfVector(v, 0, 1.0, 2.0),
                 lambda v: otf.writeApoVector(v, 0.9, 2.0), lambda v: otf.maskOtf(v, 0.0, 0.0),
                 lambda v: otf.writeAttenuationVector(v, 0.9, 1.2, 0.0, 0.0)):
        with pytest.raises(RuntimeError, match="pixel size"):
            call(Vec())
    otf.setPixelSize(0.2)
    p = otf._vector_param(Vec())
    assert p.w == 64 and 1 / (p.w * p.micronsPerPixel) == pytest.approx(0.2, rel=1e-15)
    assert p.otf() is otf


def test_print_state(fs):
    otf = fs.OtfProvider.fromEstimate(1.4, 525, 0.3)
    assert otf.printState() == "NA 1.40, lambda  525, (est., a=0.30)"


def test_dir_and_param_accessors(fs):
    """SimParam.Dir's shift, phase and modulation accessors (S/SimParam.java:429-613) and the
    stored image order / clip-scale settings (:219-237)."""
    sp = param(fs)
    d = sp.dir(0)
    d.setPxPy(30.0, -40.0)  # stored per band step: /(nBands - 1)
    assert (d.nrBand(), d.nrPha(), d.nrComp()) == (2, 3, 3)
    assert d.getPxPyLen(1) == pytest.approx(50.0) and d.getPxPyAngle(1) == pytest.approx(math.atan2(-40, 30))
    assert d.getPxPyLen(0) == 0.0
    with pytest.raises(IndexError):
        d.getPxPyLen(2)
    d.setPhaOff(0.5)
    assert d.getPhase(1) == pytest.approx(2 * math.pi / 3) and d.getPhases()[1] == pytest.approx(2 * math.pi / 3 + 0.5)
    d.setPhases([0.1, 2.0, 4.1], False)
    assert d.getPhase(2) == 4.1
    d.resetPhases()
    assert d.getPhase(2) == pytest.approx(4 * math.pi / 3)
    d.setModulation(1, 1.7)
    assert d.getRawModulations() == [1.0, 1.7] and d.getModulations() == [1.0, 1.1]
    assert sp.getImgSeq() == "PAZ" and sp.getClipScale() == "BOTH"
    assert sp.setImgSeq("ZAP").getImgSeq() == "ZAP" and sp.setClipScale("NONE").getClipScale() == "NONE"
    with pytest.raises(ValueError):
        sp.setImgSeq("XYZ")
    with pytest.raises(ValueError):
        sp.setClipScale("SOME")


@pytest.mark.parametrize("n_pha,bands,fac", [(3, 2, None), (5, 2, [1.0, 0.7]), (5, 3, [1.0, 0.8, 0.6])])
def test_separation_matrix_host_entry_vs_oracle(fs, oracle, n_pha, bands, fac):
    """BandSeparation.createSeparationMatrix through the host-only C entry (no device):
    equal to the oracle's restatement, and its inverse property."""
    rng = np.random.default_rng(11)
    phases = [2 * math.pi * i / n_pha + 0.3 + 0.01 * rng.normal() for i in range(n_pha)]
    got = fs.algorithm.BandSeparation.createSeparationMatrix(phases, bands, fac)
    exp = oracle.separation_matrix(phases, bands, fac)
    assert got.shape == (2 * bands - 1, n_pha)
    assert np.allclose(got, exp, rtol=0, atol=1e-12)
    per_band = [[(b + 1) * p for p in phases] for b in range(bands - 1)]  # the reference's 2D form
    assert np.array_equal(fs.algorithm.BandSeparation.createSeparationMatrix(per_band, bands, fac), got)
    with pytest.raises(ValueError):
        fs.algorithm.BandSeparation.createSeparationMatrix(phases[:2 * bands - 2], bands, fac)
