"""Live stream ingest (no GPU): the library's LIVESIM header, TCP framing and SIM sequence
detection (fsim_livesim_* / fsim_seqx_*) against the oracle's restatement of
org/fairsim/transport/ImageWrapper.java and org/fairsim/livemode/SimSequenceExtractor.java
(oracle/seqx_ref.py), on seeded camera streams with reordered, lost, duplicated and
late frames, both sync modes, two channels, and unknown channels."""
import numpy as np
import pytest

from oracle import seqx_ref

W = H = 4
CHANNELS = [488, 568]


def ingest(fs):
    return fs.ingest


def frame_px(seq, bright=False):
    if bright:
        return np.full((H, W), 60000, np.uint16)
    return ((np.arange(W * H, dtype=np.int64) * 131 + seq * 7) & 0xFFFF).astype(np.uint16).reshape(H, W)


def channel_stream(rng, ch, nraw, seq_count, mode, n_groups, delay=5000):
    """Frames of one camera: [(seq, t_cam, pixels)] with a sync marker before each group of
    seq_count sequences (mode 0: a time gap on the group's first frame; mode 1: an extra
    frame after a gap of `delay`, or a bright frame plus one frame to skip), then lost,
    duplicated, swapped and late frames."""
    out, seq, t = [], int(rng.integers(0, 1000)), int(rng.integers(10 ** 6, 10 ** 7))
    lead = int(rng.integers(0, nraw))  # the stream starts inside a sequence
    for _ in range(lead):
        out.append([seq, t, frame_px(seq)])
        seq += 1
        t += 1000
    for g in range(n_groups):
        if mode == 0:
            t += delay + 1000
        elif rng.random() < 0.5:
            t += delay - 1000 + int(rng.integers(-40, 40))  # delay +- 40 after the previous frame
            out.append([seq, t, frame_px(seq)])  # sync frame by time stamp
            seq += 1
            t += 1000
        else:
            out.append([seq, t, frame_px(seq, bright=True)])  # bright frame, then one skipped
            seq += 1
            t += 1000
            out.append([seq, t, frame_px(seq)])
            seq += 1
            t += 1000
        for _ in range(nraw * seq_count):
            out.append([seq, t, frame_px(seq)])
            seq += 1
            t += 1000
    # perturbations
    i = 0
    res = []
    while i < len(out):
        r = rng.random()
        if r < 0.01:  # lost (the sort buffer then stalls until it overflows and re-sorts)
            i += 1
            continue
        if r < 0.02:  # duplicated
            res.append(out[i])
        if r < 0.08 and i + 1 < len(out):  # swapped with the next
            res.append(out[i + 1])
            res.append(out[i])
            i += 2
            continue
        res.append(out[i])
        i += 1
    if len(res) > 60 and rng.random() < 0.7:  # one frame arrives 25 frames late: sort-buffer overflow
        k = int(rng.integers(5, len(res) - 30))
        res.insert(k + 25, res.pop(k))
    return [(s, tc, px, ch) for s, tc, px in res]


def build_stream(rng, nraw, seq_count, mode, n_groups, unknown=True):
    per = [channel_stream(rng, ch, nraw, seq_count, mode, n_groups) for ch in CHANNELS]
    idx = [0] * len(per)
    merged = []
    while any(i < len(p) for i, p in zip(idx, per)):
        c = int(rng.integers(len(per)))
        if idx[c] < len(per[c]):
            merged.append(per[c][idx[c]])
            idx[c] += 1
        if unknown and rng.random() < 0.01:
            merged.append((5, 0, frame_px(5), 999))
    return [seqx_ref.write_header(seq_nr=s, width=W, height=H, pos1=ch, time_camera=tc) + px.astype("<u2").tobytes()
            for s, tc, px, ch in merged]


def drain_lib(x):
    out = []
    while True:
        r = x.pop(with_seq=True)
        if r is None:
            return out
        out.append(r)


def drain_ref(x):
    out = []
    while True:
        r = x.pop()
        if r is None:
            return out
        out.append(r)


def same(lib_pops, ref_pops, nraw):
    assert len(lib_pops) == len(ref_pops)
    for (stack, first), ref in zip(lib_pops, ref_pops):
        for c, (rfirst, rseq) in enumerate(ref):
            assert first[c] == rfirst
            assert np.array_equal(stack[c].reshape(nraw, -1), np.array(rseq, np.uint16))


def test_header_roundtrip_and_checks(fs):
    ig = ingest(fs)
    rng = np.random.default_rng(1)
    for _ in range(50):
        f = dict(seq_nr=int(rng.integers(-2 ** 62, 2 ** 62)), width=int(rng.integers(1, 2048)),
                 height=int(rng.integers(1, 2048)), bytes_per_pixel=int(rng.integers(1, 3)),
                 pos_a=int(rng.integers(0, 32767)), pos_b=int(rng.integers(0, 32767)),
                 pos0=int(rng.integers(0, 32767)), pos1=int(rng.integers(0, 32767)),
                 pos2=int(rng.integers(0, 2 ** 31 - 1)), time_camera=int(rng.integers(0, 2 ** 62)),
                 time_capture=-1, time_record=0)
        b = ig.write_header(**f)
        assert b == seqx_ref.write_header(**f)
        got, exp = ig.parse_header(b, 2048, 2048), seqx_ref.parse_header(b, 2048, 2048)
        assert got == exp
        for k, v in f.items():
            assert got[k] == v
        assert got["payload_len"] == f["width"] * f["height"] and got["version"] == 1
    good = seqx_ref.write_header(seq_nr=1, width=64, height=32)
    bad = {
        "too large": good,
        "len": good[:12] + (7).to_bytes(4, "little") + good[16:],
        "bpp": good[:17] + bytes([3]) + good[18:],
        "version": good[:16] + bytes([2]) + good[17:],
    }
    for name, b in bad.items():
        limit = 32 if name == "too large" else 64
        with pytest.raises(ValueError):
            seqx_ref.parse_header(b, limit, limit)
        with pytest.raises(ValueError):
            ig.parse_header(b, limit, limit)


def test_eight_bit_pixels_widen_as_java_bytes(fs):
    ig = ingest(fs)
    x = ig.SequenceExtractor([1], 1, 4, 1, sync_mode=0, sync_frame_delay=5)
    px = np.array([[0, 127, 128, 255]], np.uint8)
    x.push(ig.make_frame(px, seq_nr=0, pos1=1, time_camera=100))  # fills the initial sort
    x.push(ig.make_frame(px, seq_nr=1, pos1=1, time_camera=200))
    stack = x.pop()
    assert stack is not None
    assert stack.reshape(-1).tolist() == [0, 127, 0xFF80, 0xFFFF]
    h = seqx_ref.parse_header(ig.make_frame(px, seq_nr=0, pos1=1), 4, 1)
    assert seqx_ref.get_pixels(ig.make_frame(px, seq_nr=0, pos1=1), h) == [0, 127, 0xFF80, 0xFFFF]
    x.close()


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("seq_count", [1, 2])
@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_sequences_match_oracle(fs, mode, seq_count, seed):
    ig = ingest(fs)
    nraw = 9
    rng = np.random.default_rng(100 * seed + 10 * mode + seq_count)
    frames = build_stream(rng, nraw, seq_count, mode, n_groups=16)
    kw = dict(sync_mode=mode, sync_frame_freq=seq_count, sync_frame_avr=7000, sync_frame_delay=5000)
    ref = seqx_ref.Extractor(CHANNELS, nraw, W, H, **kw)
    lib = ig.SequenceExtractor(CHANNELS, nraw, W, H, **kw)
    unknown = 0
    for f in frames:
        ref.push(f)
        try:
            lib.push(f)
        except fs.native.FsimNotFound:
            unknown += 1
    ref_pops, lib_pops = drain_ref(ref), drain_lib(lib)
    assert len(ref_pops) >= 4  # the stream does produce sequences
    same(lib_pops, ref_pops, nraw)
    st = lib.stats()
    assert st["unknown_channel"] == ref.unknown == unknown
    assert st["sync_frames"] == [c.syncs for c in ref.ch]
    assert st["resyncs"] == [c.resyncs for c in ref.ch]
    assert st["duplicates"] == [c.dups for c in ref.ch]
    assert st["sequences"] == len(lib_pops)
    # the same bytes as one TCP stream, cut at random places
    lib2 = ig.SequenceExtractor(CHANNELS, nraw, W, H, **kw)
    blob = b"".join(frames)
    at = 0
    while at < len(blob):
        n = int(rng.integers(1, 700))
        lib2.feed(blob[at:at + n])
        at += n
    same(drain_lib(lib2), ref_pops, nraw)
    assert lib2.stats()["bytes"] == len(blob)
    lib.close()
    lib2.close()


def test_interleaved_pops_and_full_sequence_queue(fs):
    """Popping while frames arrive gives the same stacks; a sequence queue of 3 drops the
    sequences the reference's offer() would drop."""
    ig = ingest(fs)
    nraw = 9
    rng = np.random.default_rng(7)
    frames = build_stream(rng, nraw, 1, 0, n_groups=10, unknown=False)
    ref = seqx_ref.Extractor(CHANNELS, nraw, W, H, queue_size=3)
    lib = ig.SequenceExtractor(CHANNELS, nraw, W, H, raw_queue=3, sim_queue=3)
    for f in frames:
        ref.push(f)
        lib.push(f)
    same(drain_lib(lib), drain_ref(ref), nraw)
    assert lib.stats()["missed_sim"] == [c.missed_sim for c in ref.ch]
    assert sum(lib.stats()["missed_sim"]) > 0
    ref2 = seqx_ref.Extractor(CHANNELS, nraw, W, H)
    lib2 = ig.SequenceExtractor(CHANNELS, nraw, W, H)
    got, exp = [], []
    for i, f in enumerate(frames):
        ref2.push(f)
        lib2.push(f)
        if i % 5 == 0:
            got += drain_lib(lib2)
            exp += drain_ref(ref2)
    got += drain_lib(lib2)
    exp += drain_ref(ref2)
    same(got, exp, nraw)


def test_broken_header_closes_stream_until_reset(fs):
    ig = ingest(fs)
    x = ig.SequenceExtractor([1], 1, W, H)
    good = ig.make_frame(frame_px(0), seq_nr=0, pos1=1, time_camera=1)
    broken = bytearray(ig.make_frame(frame_px(1), seq_nr=1, pos1=1, time_camera=2))
    broken[16] = 2  # protocol version 2
    x.feed(good)
    with pytest.raises(ValueError):
        x.feed(bytes(broken))
    with pytest.raises(ValueError):
        x.feed(good)
    x.reset()
    x.feed(good)
    with pytest.raises(ValueError):  # a frame larger than the configured size is a broken header
        x.push(ig.make_frame(np.zeros((H, W + 1), np.uint16), seq_nr=3, pos1=1))
    with pytest.raises(fs.native.FsimNotFound):
        x.push(ig.make_frame(frame_px(4), seq_nr=4, pos1=2))
    with pytest.raises(ValueError):  # bad configurations
        ig.SequenceExtractor([1, 1], 9, W, H)
    with pytest.raises(ValueError):
        ig.SequenceExtractor([1], 25, W, H)
    with pytest.raises(ValueError):
        ig.SequenceExtractor([1], 9, W, H, sync_mode=2)
    x.close()


def test_concurrent_receivers_and_consumer(fs):
    """One receiving thread per channel pushing frames while a consumer pops stacks (the
    reference's ImageSorter / PerChannelBuffer / JoinedChannelBuffer threads): every stack
    comes out once, in order, identical to the single-threaded result."""
    import threading

    ig = ingest(fs)
    nraw = 9
    rng = np.random.default_rng(17)
    frames = build_stream(rng, nraw, 1, 0, n_groups=20, unknown=False)
    by_ch = {c: [f for f in frames if seqx_ref.parse_header(f, W, H)["pos1"] == c] for c in CHANNELS}
    ref = ig.SequenceExtractor(CHANNELS, nraw, W, H)
    for f in frames:
        ref.push(f)
    expected = drain_lib(ref)
    x = ig.SequenceExtractor(CHANNELS, nraw, W, H)
    got, done = [], threading.Event()

    def consumer():
        while True:
            finished = done.is_set()  # read before the pop: nothing arrives after it is set
            r = x.pop(with_seq=True)
            if r is not None:
                got.append(r)
            elif finished:
                return

    def receiver(c):
        for f in by_ch[c]:
            x.push(f)

    cons = threading.Thread(target=consumer)
    cons.start()
    recv = [threading.Thread(target=receiver, args=(c,)) for c in CHANNELS]
    for t in recv:
        t.start()
    for t in recv:
        t.join()
    done.set()
    cons.join(timeout=30)
    assert not cons.is_alive()
    assert len(got) == len(expected) >= 5
    for (s1, f1), (s2, f2) in zip(got, expected):
        assert f1 == f2 and np.array_equal(s1, s2)
    x.close()
    ref.close()
