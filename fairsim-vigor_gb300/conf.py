"""Configuration files of fairSIM / VIGOR (the reference's ``utils/Conf``): an XML tree of
folders (elements without a ``type`` attribute) and typed entries, read and written with
the reference's text formats (org/fairsim/utils/Conf.java:86-640):

* ``int``: whitespace-separated integers, written as " 1 2 ";
* ``decimal``: whitespace-separated numbers, written "%8.5e " each after a leading space,
  or " BASE64:...:END64 " holding big-endian IEEE doubles ("exact" entries);
* ``string``: the text as is;
* ``data``: " BASE64:...:END64 " bytes (``Conf.toByte`` / ``fromByte`` hold big-endian
  floats, e.g. measured OTF bands);
* ``timepoint``: milliseconds since 1970, written " ms ".

On top of it: ``load_vigor_channels`` builds the per-channel SimParam / OtfProvider and the
stream-sync settings the reference's live mode reads (livemode/ReconstructionRunner.java:
86-101,160-196; livemode/SimSequenceExtractor.java:60-68)."""
from __future__ import annotations

import base64
import re
import struct
import xml.etree.ElementTree as ET
from typing import Dict, List, Optional


class EntryNotFound(KeyError):
    """Conf.EntryNotFoundException."""


class Entry:
    type = ""

    def text(self) -> str:
        raise NotImplementedError


class IntEntry(Entry):
    type = "int"

    def __init__(self, vals=(0,)):
        self._v = [int(v) for v in vals]

    def val(self) -> int:
        return self._v[0]

    def vals(self) -> List[int]:
        return list(self._v)

    def setVal(self, *v) -> "IntEntry":
        if not v:
            raise ValueError("Array empty!")
        self._v = [int(x) for x in v]
        return self

    def text(self) -> str:
        return " " + "".join("%d " % v for v in self._v)

    @staticmethod
    def from_text(t: str) -> "IntEntry":
        vals = []
        for tok in t.split():  # Scanner.hasNextInt: stops at the first non-integer token
            if not re.fullmatch(r"[+-]?\d+", tok):
                break
            vals.append(int(tok))
        return IntEntry(vals)


def _b64(b: bytes) -> str:
    return " BASE64:" + base64.b64encode(b).decode("ascii") + ":END64 "


def _unb64(t: str, start_marker: str) -> bytes:
    a = t.index(start_marker) + len(start_marker)
    return base64.b64decode(t[a:t.index(":END64")].strip())


class DoubleEntry(Entry):
    type = "decimal"

    def __init__(self, vals=(0.0,), exact=False):
        self._v = [float(v) for v in vals]
        self.exact = exact

    def val(self) -> float:
        return self._v[0]

    def vals(self) -> List[float]:
        return list(self._v)

    def setVal(self, *v) -> "DoubleEntry":
        if len(v) == 1 and isinstance(v[0], (list, tuple)):
            v = tuple(v[0])
        if not v:
            raise ValueError("Array empty")
        self._v = [float(x) for x in v]
        return self

    def setExactOutput(self, s: bool) -> None:
        self.exact = bool(s)

    def text(self) -> str:
        if self.exact:
            return _b64(struct.pack(">%dd" % len(self._v), *self._v))
        return " " + "".join("%8.5e " % v for v in self._v)

    @staticmethod
    def from_text(t: str) -> "DoubleEntry":
        if "BASE64:" in t:
            # the reference cuts from the first ':' (the one of "BASE64:")
            raw = base64.b64decode(t[t.index(":") + 1:t.index(":END64")].strip())
            if len(raw) % 8:
                raise ValueError("Wrong base64 len for double")
            return DoubleEntry(struct.unpack(">%dd" % (len(raw) // 8), raw), exact=True)
        vals = []
        for tok in t.split():  # Scanner.hasNextDouble (Locale.US)
            try:
                vals.append(float(tok))
            except ValueError:
                break
        return DoubleEntry(vals)


class StringEntry(Entry):
    type = "string"

    def __init__(self, v: str = ""):
        self._v = v

    def val(self) -> str:
        return self._v

    def setVal(self, v: str) -> "StringEntry":
        self._v = str(v)
        return self

    def text(self) -> str:
        return self._v


class DataEntry(Entry):
    type = "data"

    def __init__(self, data: bytes = b""):
        self._v = bytes(data)

    def val(self) -> bytes:
        return self._v

    def setVal(self, b: bytes) -> "DataEntry":
        self._v = bytes(b)
        return self

    def text(self) -> str:
        return _b64(self._v)


class TimeDateEntry(Entry):
    type = "timepoint"

    def __init__(self, ms: int = 0):
        self._v = int(ms)

    def val(self) -> int:
        return self._v

    def set(self, ms: int) -> "TimeDateEntry":
        self._v = int(ms)
        return self

    def text(self) -> str:
        return " %d " % self._v

    @staticmethod
    def from_text(t: str) -> "TimeDateEntry":
        toks = t.split()
        try:
            return TimeDateEntry(int(toks[0]) if toks else 0)
        except ValueError:
            return TimeDateEntry(0)


def to_bytes(floats) -> bytes:
    """Conf.toByte: big-endian IEEE floats."""
    return struct.pack(">%df" % len(floats), *floats)


def from_bytes(b: bytes) -> List[float]:
    """Conf.fromByte."""
    if len(b) % 4:
        raise ValueError("Array size not a multiple of 4")
    return list(struct.unpack(">%df" % (len(b) // 4), b))


class Folder(Entry):
    """Conf.Folder: named entries and sub-folders."""

    def __init__(self, name: str):
        self.name = name
        self.sub: Dict[str, Entry] = {}

    # -- structure --
    def mk(self, name: str) -> "Folder":
        f = Folder(name)
        self.sub[name] = f
        return f

    def cd(self, name: str) -> "Folder":
        return self._get(name, Folder)

    def contains(self, name: str) -> bool:
        return name in self.sub

    def names(self) -> List[str]:
        return list(self.sub)

    def _get(self, name, cls):
        e = self.sub.get(name)
        if not isinstance(e, cls):
            raise EntryNotFound("%s (in %s)" % (name, self.name))
        return e

    # -- typed access (Conf.Folder.getInt / getDbl / getStr / getData / getTDE) --
    def getInt(self, name) -> IntEntry:
        return self._get(name, IntEntry)

    def getDbl(self, name) -> DoubleEntry:
        return self._get(name, DoubleEntry)

    def getStr(self, name) -> StringEntry:
        return self._get(name, StringEntry)

    def getData(self, name) -> DataEntry:
        return self._get(name, DataEntry)

    def getTDE(self, name) -> TimeDateEntry:
        return self._get(name, TimeDateEntry)

    def _new(self, name, e):
        self.sub[name] = e
        return e

    def newInt(self, name) -> IntEntry:
        return self._new(name, IntEntry())

    def newDbl(self, name) -> DoubleEntry:
        return self._new(name, DoubleEntry())

    def newStr(self, name) -> StringEntry:
        return self._new(name, StringEntry())

    def newData(self, name) -> DataEntry:
        return self._new(name, DataEntry())

    def newTDE(self, name) -> TimeDateEntry:
        return self._new(name, TimeDateEntry())

    # -- XML --
    def to_element(self) -> ET.Element:
        el = ET.Element(self.name)
        for n, e in self.sub.items():
            if isinstance(e, Folder):
                el.append(e.to_element())
            else:
                s = ET.SubElement(el, n, {"type": e.type})
                s.text = e.text()
        return el

    def import_element(self, xml: ET.Element) -> None:
        """Conf.importXmlElement (:678-735): untyped elements are folders; unknown types
        are skipped."""
        for e in xml:
            if not isinstance(e.tag, str):  # comments, processing instructions
                continue
            t = e.get("type", "")
            c = "".join(e.itertext())
            if t == "":
                self.mk(e.tag).import_element(e)
            elif t == "int":
                self.sub[e.tag] = IntEntry.from_text(c)
            elif t == "decimal":
                self.sub[e.tag] = DoubleEntry.from_text(c)
            elif t == "string":
                self.sub[e.tag] = StringEntry(c)
            elif t == "data":
                self.sub[e.tag] = DataEntry(_unb64(c, "BASE64:"))
            elif t == "timepoint":
                self.sub[e.tag] = TimeDateEntry.from_text(c)


class Conf:
    """A configuration: one root folder (Conf.java)."""

    def __init__(self, name: str):
        self.root = Folder(name)

    def r(self) -> Folder:
        return self.root

    @staticmethod
    def loadFile(path) -> "Conf":
        with open(path, "rb") as fh:
            data = fh.read()
        # the reference's configs carry comments such as "<!--- ... -->", which a strict
        # parser rejects ("--" inside a comment); Java's parser reads them as comments
        data = re.sub(rb"<!--.*?-->", b"", data, flags=re.S)
        root = ET.fromstring(data)
        cfg = Conf(root.tag)
        cfg.root.import_element(root)
        return cfg

    def saveFile(self, path) -> bool:
        el = self.root.to_element()
        ET.indent(el)
        with open(path, "wb") as fh:
            fh.write(ET.tostring(el, encoding="utf-8"))
        return True


# ---- live-mode settings ---------------------------------------------------------------------

class VigorChannel:
    """One channel folder of a VIGOR configuration (ReconstructionRunner.PerChannel)."""

    def __init__(self, name: str, number: int, offset: float, param):
        self.name, self.number, self.offset, self.param = name, number, offset, param


def load_vigor_channels(settings: Folder, channels: Optional[List[str]] = None):
    """From the ``vigor-settings`` folder: (channels, stream) where channels are
    VigorChannel records whose SimParam carries the channel's OTF and the raw pixel size
    (ReconstructionRunner.java:86-101,175-196), and stream holds the sequence-detection
    settings (SimSequenceExtractor.java:60-68) for ``ingest.SequenceExtractor``."""
    from .sim_param import OtfProvider, SimParam

    if channels is None:
        channels = [n[len("channel-"):] for n in settings.names() if n.startswith("channel-")]
    size = settings.getInt("RawPxlCount").val()
    microns = settings.getDbl("RawPxlSize").val()
    out = []
    for ch in channels:
        fld = settings.cd("channel-" + ch)
        sp = SimParam.loadConfig(fld)
        sp.setPxlSize(size, microns)
        sp.setOtf(OtfProvider.loadFromConfig(fld))
        out.append(VigorChannel(ch, fld.getInt("ChannelNumber").val(), fld.getDbl("offset").val(), sp))
    stream = dict(channel_numbers=[c.number for c in out],
                  raws_per_recon=settings.getInt("NrAngles").val() * settings.getInt("NrPhases").val(),
                  width=size, height=size, sync_mode=settings.getInt("SyncMode").val(),
                  sync_frame_freq=settings.getInt("SyncFrameFreq").val(),
                  sync_frame_avr=settings.getInt("SyncFrameAvr").val(),
                  sync_frame_delay=settings.getInt("SyncFrameDelay").val())
    return out, stream
