"""ORACLE - test infrastructure only (tests/ and nothing else import it).

A plain-Python restatement of the reference's live-stream ingest, the oracle the tests
compare the library's fsim_livesim_* / fsim_seqx_* entry points against:

* LIVESIM header write / parse: org/fairsim/transport/ImageWrapper.java:418-478
  (little endian, header-definition.md), pixels: getPixels (:265-278, Java's signed byte
  for 8-bit frames);
* per-channel SIM sequence detection: org/fairsim/livemode/SimSequenceExtractor.java,
  PerChannelBuffer (:212-516) with its blocking thread restated as a generator: every
  ``rawImgs.take()`` of the reference is a ``yield`` until a frame is queued, and the
  recursion getSorted -> sortFromQueue -> getSorted is kept as written;
* ImageSorter (:155-180) and JoinedChannelBuffer (:185-204) as ``Extractor.push`` and
  ``Extractor.pop``.

Where the reference ends its thread with an exception (a second frame with a buffered
sequence number, a full sort buffer when a mode-0 sync frame is put back), the restatement
counts the event and drops the frame, as the library does.
"""
from __future__ import annotations

import collections
import struct

HEADER = 128
SORT_SLOTS = 20  # SortBuffer(20)
SYNCJITTER = 50  # PerChannelBuffer.SYNCJITTER


def write_header(seq_nr=0, width=0, height=0, bytes_per_pixel=2, pos_a=0, pos_b=0, pos0=0, pos1=0, pos2=0,
                 time_camera=0, time_capture=0, time_record=0):
    """ImageWrapper.writeHeader (:422-443)."""
    b = bytearray(HEADER)
    struct.pack_into("<q", b, 0, seq_nr)
    struct.pack_into("<i", b, 12, width * height)
    struct.pack_into("<b", b, 16, 1)
    struct.pack_into("<b", b, 17, bytes_per_pixel)
    struct.pack_into("<hhhh", b, 32, width, height, pos_a, pos_b)
    struct.pack_into("<hh", b, 40, pos0, pos1)
    struct.pack_into("<i", b, 44, pos2)
    struct.pack_into("<qqq", b, 48, time_camera, time_capture, time_record)
    return bytes(b)


def parse_header(b, max_w, max_h):
    """ImageWrapper.parseHeader (:445-478); ValueError where it throws BrokenHeaderException."""
    h = dict(seq_nr=struct.unpack_from("<q", b, 0)[0], payload_offset=struct.unpack_from("<i", b, 8)[0],
             payload_len=struct.unpack_from("<i", b, 12)[0], version=struct.unpack_from("<b", b, 16)[0],
             bytes_per_pixel=struct.unpack_from("<b", b, 17)[0])
    (h["width"], h["height"], h["pos_a"], h["pos_b"], h["pos0"], h["pos1"]) = struct.unpack_from("<hhhhhh", b, 32)
    h["pos2"] = struct.unpack_from("<i", b, 44)[0]
    h["time_camera"], h["time_capture"], h["time_record"] = struct.unpack_from("<qqq", b, 48)
    if h["width"] > max_w or h["height"] > max_h or h["width"] < 0 or h["height"] < 0:
        raise ValueError("Image too large")
    if h["payload_len"] != h["width"] * h["height"]:
        raise ValueError("Width x Height != Len")
    if h["bytes_per_pixel"] not in (1, 2):
        raise ValueError("bpp neither 1 nor 2")
    if h["version"] != 1:
        raise ValueError("unsupported version")
    return h


def get_pixels(frame, h):
    """ImageWrapper.getPixels as unsigned 16-bit values: u16 little endian, or each byte
    widened as Java's signed byte (b >= 128 -> 0xFF00 + b)."""
    n = h["width"] * h["height"]
    p = frame[HEADER:]
    if h["bytes_per_pixel"] == 2:
        return list(struct.unpack_from("<%dH" % n, p, 0))
    return [(v if v < 128 else v + 0xFF00) for v in p[:n]]


class Frame:
    __slots__ = ("seq", "t_cam", "px")

    def __init__(self, seq, t_cam, px):
        self.seq, self.t_cam, self.px = seq, t_cam, px


def avr_ushort(px):
    """MTool.avr_ushort (linalg/MTool.java:68-76)."""
    return float(sum(px)) / len(px)


class PerChannelBuffer:
    """SimSequenceExtractor.PerChannelBuffer: queue, sort buffer, and the run() thread."""

    def __init__(self, raws_per_recon, sync_mode, seq_count, sync_avr, sync_delay, queue_size):
        self.raws = raws_per_recon
        self.sync_mode, self.seq_count = sync_mode, seq_count
        self.sync_avr, self.sync_delay = sync_avr, sync_delay
        self.queue_size = queue_size
        self.raw = collections.deque()
        self.sim = collections.deque()
        self.sort = {}
        self.seqNr = 0
        self.missed_raw = self.missed_sim = self.syncs = self.resyncs = self.dups = 0
        self.gen = self.run()
        next(self.gen)  # start the thread: it blocks in setSeqNr for the first frame

    def push(self, f):  # pushImg (:249-255)
        if len(self.raw) >= self.queue_size:
            self.missed_raw += 1
            return
        self.raw.append(f)
        next(self.gen)  # wake the thread: it runs until its next take() finds nothing

    def take(self):  # rawImgs.take(), blocking
        while not self.raw:
            yield
        return self.raw.popleft()

    def sort_add(self, f):  # SortBuffer.add (:500-509), overflow checked by the callers
        if f.seq in self.sort:
            self.dups += 1
            return
        self.sort[f.seq] = f

    def get_sorted(self):  # :262-276
        if not self.sort:
            return (yield from self.sort_from_queue())
        f = self.sort.pop(self.seqNr, None)
        if f is not None:
            self.seqNr += 1
            return f
        return (yield from self.sort_from_queue())

    def sort_from_queue(self):  # :283-298
        f = yield from self.take()
        if f.seq == self.seqNr:
            self.seqNr += 1
            return f
        if len(self.sort) < SORT_SLOTS:
            self.sort_add(f)
        else:  # BufferOverflowException
            self.seqNr += 1
            self.resyncs += 1
            yield from self.set_seq_nr()
        return (yield from self.get_sorted())

    def set_seq_nr(self):  # :312-338
        self.sort.clear()
        self.seqNr = 1 << 63
        while len(self.sort) < self.raws:
            f = yield from self.take()
            self.sort_add(f)
            if f.seq < self.seqNr:
                self.seqNr = f.seq

    def run(self):  # :397-477
        nraw = self.raws
        yield from self.set_seq_nr()
        last = cur = 0
        while True:
            counter = 0
            while True:
                f = yield from self.get_sorted()
                cur = f.t_cam
                if self.sync_mode == 0:
                    if cur - last > self.sync_delay:
                        if len(self.sort) < SORT_SLOTS:
                            self.sort_add(f)
                            self.seqNr -= 1
                        self.syncs += 1
                        break
                else:
                    if abs(cur - last - self.sync_delay) < SYNCJITTER:
                        self.syncs += 1
                        break
                    if avr_ushort(f.px) > self.sync_avr:
                        self.syncs += 1
                        yield from self.get_sorted()  # ignore the next frame
                        break
                last = cur
                counter += 1
                if counter >= nraw * self.seq_count:
                    counter = 0
            for _ in range(self.seq_count):
                seq, first = [], None
                for _ in range(nraw):
                    f = yield from self.get_sorted()
                    if first is None:
                        first = f.seq
                    seq.append(f.px)
                    cur = f.t_cam
                    last = cur
                if len(self.sim) < self.queue_size:
                    self.sim.append((first, seq))
                else:
                    self.missed_sim += 1


class Extractor:
    """ImageSorter + PerChannelBuffers + JoinedChannelBuffer."""

    def __init__(self, channel_numbers, raws_per_recon, width, height, sync_mode=0, sync_frame_freq=1,
                 sync_frame_avr=7000, sync_frame_delay=5000, queue_size=None):
        q = queue_size or raws_per_recon * raws_per_recon * 10
        self.numbers = list(channel_numbers)
        self.w, self.h = width, height
        self.ch = [PerChannelBuffer(raws_per_recon, sync_mode, sync_frame_freq, sync_frame_avr, sync_frame_delay, q)
                   for _ in self.numbers]
        self.unknown = 0

    def push(self, frame):
        h = parse_header(frame, self.w, self.h)
        if h["pos1"] not in self.numbers:
            self.unknown += 1
            return False
        c = self.ch[self.numbers.index(h["pos1"])]
        c.push(Frame(h["seq_nr"], h["time_camera"], get_pixels(frame, h)))
        return True

    def pop(self):
        if any(not c.sim for c in self.ch):
            return None
        return [c.sim.popleft() for c in self.ch]
