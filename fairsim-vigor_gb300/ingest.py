"""Live stream ingest: LIVESIM frame headers and the per-channel SIM sequence detection of
the reference's live mode (transport/ImageWrapper.java, transport/ImageReceiver.java,
livemode/SimSequenceExtractor.java), over the library's fsim_livesim_* / fsim_seqx_* C ABI.
Host work only; complete multi-channel stacks go to a ``plan.Server`` (``LiveIngest``)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native as N

HEADER_BYTES = N.LIVESIM_HEADER_BYTES
_FIELDS = [f for f, _ in N.LiveSimHeader._fields_]


def parse_header(data, max_width: int, max_height: int) -> dict:
    """ImageWrapper.parseHeader on the first 128 bytes: a dict of the header fields;
    ValueError for a broken header."""
    b = bytes(data[:HEADER_BYTES])
    if len(b) < HEADER_BYTES:
        raise ValueError("header shorter than %d bytes" % HEADER_BYTES)
    h = N.LiveSimHeader()
    N.check(N.lib().fsim_livesim_parse(b, int(max_width), int(max_height), C.byref(h)))
    return {f: getattr(h, f) for f in _FIELDS}


def write_header(**fields) -> bytes:
    """ImageWrapper.writeHeader: 128 bytes from the given fields (seq_nr, width, height,
    bytes_per_pixel, pos_a, pos_b, pos0, pos1, pos2, time_camera, time_capture, time_record)."""
    h = N.LiveSimHeader()
    h.bytes_per_pixel = 2
    for k, v in fields.items():
        if k not in _FIELDS:
            raise KeyError(k)
        setattr(h, k, int(v))
    out = C.create_string_buffer(HEADER_BYTES)
    N.check(N.lib().fsim_livesim_write(C.byref(h), out))
    return out.raw


def make_frame(pixels, **fields) -> bytes:
    """A complete frame: header + little-endian payload (uint16, or uint8 with
    bytes_per_pixel=1)."""
    px = np.asarray(pixels)
    bpp = 1 if px.dtype == np.uint8 else 2
    h, w = px.shape
    hdr = write_header(width=w, height=h, bytes_per_pixel=bpp, **fields)
    return hdr + px.astype("<u2" if bpp == 2 else np.uint8).tobytes()


class SequenceExtractor:
    """SimSequenceExtractor without threads: push frames (or feed raw TCP bytes) of any
    channel in any order; pop() returns the next stack holding one SIM sequence of every
    channel, shaped (channels, raws_per_recon, height, width) uint16, or None."""

    def __init__(self, channel_numbers, raws_per_recon, width, height, sync_mode=0, sync_frame_freq=1,
                 sync_frame_avr=7000, sync_frame_delay=5000, raw_queue=0, sim_queue=0):
        cfg = N.SeqxConfig()
        cfg.n_channels = len(channel_numbers)
        if cfg.n_channels > N.MAX_CHANNELS:
            raise ValueError("at most %d channels" % N.MAX_CHANNELS)
        for i, c in enumerate(channel_numbers):
            cfg.channel_numbers[i] = int(c)
        cfg.raws_per_recon, cfg.width, cfg.height = int(raws_per_recon), int(width), int(height)
        cfg.sync_mode, cfg.sync_frame_freq = int(sync_mode), int(sync_frame_freq)
        cfg.sync_frame_avr, cfg.sync_frame_delay = int(sync_frame_avr), int(sync_frame_delay)
        cfg.raw_queue, cfg.sim_queue = int(raw_queue), int(sim_queue)
        h = C.c_void_p()
        N.check(N.lib().fsim_seqx_create(C.byref(h), C.byref(cfg)))
        self._h = h
        self.n_channels, self.raws = cfg.n_channels, cfg.raws_per_recon
        self.width, self.height = cfg.width, cfg.height

    def push(self, frame) -> None:
        """One frame (header + payload). Unknown channels raise FsimNotFound (the frame
        is counted and dropped); broken headers raise ValueError."""
        b = frame if isinstance(frame, bytes) else bytes(frame)
        N.check(N.lib().fsim_seqx_push(self._h, b, len(b)))

    def feed(self, data) -> None:
        """TCP stream bytes in any pieces."""
        b = data if isinstance(data, bytes) else bytes(data)
        N.check(N.lib().fsim_seqx_feed(self._h, b, len(b)))

    def pop(self, with_seq: bool = False):
        out = np.empty((self.n_channels, self.raws, self.height, self.width), np.uint16)
        first = (C.c_int64 * self.n_channels)()
        rc = N.lib().fsim_seqx_pop(self._h, out.ctypes.data_as(C.c_void_p), first)
        if rc == N.FSIM_ENOTFOUND:
            return None
        N.check(rc)
        return (out, list(first)) if with_seq else out

    def stats(self) -> dict:
        s = N.SeqxStats()
        N.check(N.lib().fsim_seqx_stats_get(self._h, C.byref(s)))
        n = self.n_channels
        return {"frames": s.frames, "bytes": s.bytes, "unknown_channel": s.unknown_channel,
                "missed_raw": list(s.missed_raw)[:n], "missed_sim": list(s.missed_sim)[:n],
                "sync_frames": list(s.sync_frames)[:n], "resyncs": list(s.resyncs)[:n],
                "duplicates": list(s.duplicates)[:n], "sequences": s.sequences}

    def reset(self) -> None:
        N.check(N.lib().fsim_seqx_reset(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().fsim_seqx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LiveIngest:
    """Camera stream -> reconstruction: every stack the extractor completes is submitted to
    the server, one channel at a time (the JoinedChannelBuffer -> ReconstructionRunner
    hand-over, livemode/SimSequenceExtractor.java:185-204). Returns the server's tickets."""

    def __init__(self, extractor: SequenceExtractor, server):
        self.x, self.server = extractor, server
        self.dropped = 0

    def _drain(self):
        tickets = []
        while True:
            stack = self.x.pop()
            if stack is None:
                return tickets
            for c in range(stack.shape[0]):
                t = self.server.try_submit(c, stack[c])
                if t is None:
                    self.dropped += 1
                else:
                    tickets.append((c, t))

    def feed(self, data):
        self.x.feed(data)
        return self._drain()

    def push(self, frame):
        self.x.push(frame)
        return self._drain()
