"""fairSIM / VIGOR configuration files (no GPU): the reference's Conf text formats
(org/fairsim/utils/Conf.java), SimParam.saveConfig / loadConfig
(org/fairsim/sim_algorithm/SimParam.java:645-726), OtfProvider.loadFromConfig /
saveConfig (org/fairsim/sim_algorithm/OtfProvider.java:575-676) and the live mode's channel
settings; the configuration files the reference ships are read where they are present."""
import glob
import math
import os
import re

import pytest

# the reference project's root (its shipped configuration files), when a checkout is at hand
REF = os.environ.get("FSIM_REFERENCE_ROOT", "")


def sample_param(fs):
    otf = fs.OtfProvider.fromEstimate(1.4, 525, 0.3)
    otf.setAttenuation(0.98, 1.3)
    otf.switchAttenuation(True)
    sp = fs.SimParam.create(2, 3, 3, 512, 0.078, otf)
    sp.setWienerFilter(0.07).setApoCutoff(1.8)
    sp.paramDate = 1481205767740
    for d in range(3):
        sp.dir(d).setPxPy(137.478 - 50 * d, -106.278 + 20 * d)
        sp.dir(d).setPhaOff(-0.307837 + d)
        sp.dir(d).setModulation(1, 0.639470 - 0.1 * d)
    sp.dir(2).setPhases([0.1, 2.2, 4.3], False)
    return sp


def test_entry_text_formats(fs):
    C = fs.conf
    assert C.IntEntry().setVal(3, -4).text() == " 3 -4 "
    assert C.DoubleEntry().setVal(0.05, -23.7889).text() == " 5.00000e-02 -2.37889e+01 "
    e = C.DoubleEntry().setVal(math.pi, 1e-300)
    e.setExactOutput(True)
    back = C.DoubleEntry.from_text(e.text())
    assert back.vals() == [math.pi, 1e-300]  # big-endian doubles in BASE64, exact
    assert C.IntEntry.from_text("  12 13 x 14").vals() == [12, 13]  # Scanner stops at "x"
    assert C.DoubleEntry.from_text(" 1.5e+00 2 ").vals() == [1.5, 2.0]
    assert C.to_bytes([1.0]) == b"\x3f\x80\x00\x00"  # Conf.toByte: big-endian floats
    assert C.from_bytes(C.to_bytes([0.25, -2.0])) == [0.25, -2.0]
    assert C.TimeDateEntry.from_text(" 1481205767740 ").val() == 1481205767740


def test_sim_param_and_otf_roundtrip(fs, tmp_path):
    sp = sample_param(fs)
    cfg = fs.conf.Conf("fairsim")
    sp.saveConfig(cfg.r())
    sp.otf().saveConfig(cfg.r())
    path = tmp_path / "param.xml"
    cfg.saveFile(path)
    txt = path.read_text()
    assert '<nr-angles type="int"> 3 </nr-angles>' in txt
    assert '<shift type="decimal"> 1.37478e+02 -1.06278e+02 </shift>' in txt
    back = fs.conf.Conf.loadFile(path).r()
    lp = fs.SimParam.loadConfig(back)
    lp.setOtf(fs.OtfProvider.loadFromConfig(back))
    assert (lp.nrDirs, lp.nrBands, lp.nrPhases, lp.imgSize) == (3, 2, 3, 512)
    assert lp.paramDate == sp.paramDate and lp.imgSeq == sp.imgSeq
    for a, b in ((lp.micronsPerPixel, 0.078), (lp.wiener, 0.07), (lp.apoCutOff, 1.8)):
        assert abs(a - b) <= 1e-5 * abs(b)
    for d in range(3):  # %8.5e keeps 6 significant digits
        for a, b in ((lp.dir(d).pX, sp.dir(d).pX), (lp.dir(d).pY, sp.dir(d).pY),
                     (lp.dir(d).phaOff, sp.dir(d).phaOff), (lp.dir(d).modul[1], sp.dir(d).modul[1])):
            assert abs(a - b) <= 1e-5 * max(abs(b), 1e-3)
    assert lp.dir(0).phases is None and lp.dir(2).phases == pytest.approx([0.1, 2.2, 4.3], rel=1e-5)
    o = lp.otf()
    assert (o.na, o.emWavelength, o.a, o.useAttenuation) == (1.4, 525.0, 0.3, True)
    assert (o.attStrength, o.attFWHM) == (0.98, 1.3)


def test_measured_otf_roundtrip_and_fused_refusal(fs, tmp_path):
    cfg = fs.conf.Conf("fairsim")
    fld = cfg.r().mk("otf2d")
    fld.newDbl("NA").setVal(1.4)
    fld.newInt("emission").setVal(525)
    data = fld.mk("data")
    data.newInt("bands").setVal(2)
    data.newInt("samples").setVal(4)
    data.newDbl("cycles").setVal(0.0125)
    bands = [[1.0, 0.0, 0.75, 0.125, 0.5, 0.25, 0.0, 0.0], [0.5, -0.5, 0.25, 0.0, 0.125, 0.0, 0.0, 0.0]]
    for b, v in enumerate(bands):
        data.newData("band-%d" % b).setVal(fs.conf.to_bytes(v))
    path = tmp_path / "otf.xml"
    cfg.saveFile(path)
    otf = fs.OtfProvider.loadFromConfig(fs.conf.Conf.loadFile(path).r())
    assert not otf.isEstimate
    assert otf.measured["cycles"] == 0.0125
    assert otf.measured["bands"][0][1] == complex(0.75, 0.125)
    assert otf.measured["bands"][1][0] == complex(0.5, -0.5)
    cfg2 = fs.conf.Conf("fairsim")
    otf.saveConfig(cfg2.r())
    d2 = cfg2.r().cd("otf2d").cd("data")
    assert d2.getData("band-1").val() == fs.conf.to_bytes(bands[1])
    sp = fs.SimParam.create(2, 3, 3, 256, 0.08, otf)
    c = fs.native.to_c_param(sp)  # the record carries the bands to the library
    assert (c.otf_bands, c.otf_samples, c.otf_cycles) == (2, 4, 0.0125)
    with pytest.raises(ValueError):  # live plans take estimated OTFs only (checked before any device work)
        fs.plan.ReconPlan(sp, path=fs.native.PATH_LIVE, input_type=fs.native.INPUT_U16, fade_px=10)


@pytest.mark.skipif(not REF or not os.path.isdir(REF), reason="FSIM_REFERENCE_ROOT unset or not a directory")
def test_reference_configs_load(fs):
    files = sorted(glob.glob(os.path.join(REF, "vigor-*.xml")))
    assert files
    for f in files:
        root = fs.conf.Conf.loadFile(f).r()
        settings = root.cd("vigor-settings")
        chans, stream = fs.conf.load_vigor_channels(settings)
        txt = open(f).read()
        assert stream["sync_mode"] == int(re.search(r'<SyncMode type="int">\s*(\d+)', txt).group(1))
        assert stream["raws_per_recon"] == (int(re.search(r'<NrAngles type="int">\s*(\d+)', txt).group(1))
                                            * int(re.search(r'<NrPhases type="int">\s*(\d+)', txt).group(1)))
        for ch in chans:
            block = re.search(r"<channel-%s>(.*?)</channel-%s>" % (ch.name, ch.name), txt, re.S).group(1)
            shift = re.search(r"<dir-0>.*?<shift[^>]*>([^<]*)</shift>", block, re.S).group(1).split()
            nb = int(re.search(r'<nr-bands type="int">\s*(\d+)', block).group(1))
            assert ch.param.dir(0).pX == pytest.approx(float(shift[0]) / (nb - 1), rel=1e-12)
            assert ch.param.dir(0).pY == pytest.approx(float(shift[1]) / (nb - 1), rel=1e-12)
            em = int(re.search(r'<emission type="int">\s*(\d+)', block).group(1))
            assert ch.param.otf().emWavelength == em
            assert ch.number == int(re.search(r'<ChannelNumber type="int">\s*(\d+)', block).group(1))
            assert ch.param.imgSize == stream["width"]
            fs.native.to_c_param(ch.param)  # estimated OTFs: the device path takes them
