"""GPU tests of the served form (fsim_serve_*), the continuous-batching replacement of
ReconstructionRunner (org/fairsim/livemode/ReconstructionRunner.java:140-593):
  * each result is identical alone and in a mix of concurrent requests from several
    channels and sizes (continuous batching must not change a reconstruction);
  * admission refuses work beyond the slot budget with FSIM_EBUSY (no silent drops);
  * refits run on the device every N stacks and swap in parameters that match the
    oracle's ParameterRefitThread.doRefit on the same stack."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def channel(fs, n, seed, lam=525.0, n_phases=3):
    raw, truth = fs.synth.make_dataset(n=n, seed=seed, em_wavelength=lam, as_u16=True, n_phases=n_phases)
    return raw, fs.synth.sim_param_for(truth, n, n_phases=n_phases)


def test_results_identical_alone_and_in_mix(fs):
    specs = [(256, 1, 488.0), (256, 2, 525.0), (512, 3, 600.0), (384, 4, 525.0)]
    chans = [channel(fs, n, s, lam) for n, s, lam in specs]
    alone = []
    for raw, sp in chans:
        plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_LIVE, input_type=fs.native.INPUT_U16, fade_px=10)
        alone.append(plan.reconstruct_host(raw))
    srv = fs.plan.Server([sp for _, sp in chans], max_batch=8, max_inflight=32, streams=3, refit_every=0)
    order = [0, 1, 2, 3, 2, 1, 0, 3, 3, 0, 1, 2, 0, 0, 2, 1]
    tickets = [(srv.submit(c, chans[c][0]), c) for c in order]
    for tk, c in tickets:
        n = chans[c][1].w
        out = np.empty((2 * n, 2 * n), np.float32)
        lat = srv.wait(tk, out)
        assert lat > 0
        assert np.array_equal(out, alone[c])
    st = srv.stats()
    assert st["completed"] == len(order) and st["rejected"] == 0
    srv.close()


def test_fifteen_frame_stacks_identical_alone_and_in_mix(fs, oracle):
    """15-frame (3 x 5) and 9-frame channels served together: each result equals its plan's
    result alone, and the 15-frame results match the oracle's live reconstruction."""
    specs = [(256, 21, 488.0, 5), (512, 22, 525.0, 5), (256, 23, 600.0, 3)]
    chans = [channel(fs, n, s, lam, nph) for n, s, lam, nph in specs]
    alone = []
    for raw, sp in chans:
        plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_LIVE, input_type=fs.native.INPUT_U16, fade_px=10)
        alone.append(plan.reconstruct_host(raw))
    for (raw, sp), a, (_, _, _, nph) in zip(chans, alone, specs):
        if nph == 5:
            exp, _ = oracle.live_recon(sp, raw)
            assert np.linalg.norm(a - exp[0]) / np.linalg.norm(exp[0]) < 1e-4
    srv = fs.plan.Server([sp for _, sp in chans], max_batch=8, max_inflight=32, streams=3, refit_every=0)
    order = [0, 1, 2, 1, 0, 2, 2, 1, 0, 0, 1]
    tickets = [(srv.submit(c, chans[c][0]), c) for c in order]
    for tk, c in tickets:
        n = chans[c][1].w
        out = np.empty((2 * n, 2 * n), np.float32)
        srv.wait(tk, out)
        assert np.array_equal(out, alone[c])
    assert srv.stats()["completed"] == len(order)
    srv.close()


def test_admission_refuses_when_slots_are_full(fs):
    raw, sp = channel(fs, 256, 7)
    srv = fs.plan.Server([sp], max_batch=2, max_inflight=3, streams=1, refit_every=0)
    got = [srv.try_submit(0, raw) for _ in range(3)]
    assert all(t is not None for t in got)
    assert srv.try_submit(0, raw) is None  # every slot is taken until a result is collected
    out = np.empty((512, 512), np.float32)
    srv.wait(got[0], out)
    assert srv.try_submit(0, raw) is not None
    assert srv.stats()["rejected"] == 1
    srv.close()


def test_admission_by_size_class(fs):
    """Slots are sized per channel size, max_inflight of them per class: a full 1024^2 class
    refuses with FSIM_EBUSY while 512^2 stacks are still admitted, and every admitted stack
    reconstructs as it does alone."""
    raw5, sp5 = channel(fs, 512, 31)
    raw10, sp10 = channel(fs, 1024, 32)
    srv = fs.plan.Server([sp5, sp10], max_batch=2, max_inflight=2, streams=2, refit_every=0)
    assert srv.capacity(0) == {"slots": 2, "free": 2} and srv.capacity(1) == {"slots": 2, "free": 2}
    t10 = [srv.try_submit(1, raw10) for _ in range(2)]
    assert all(t is not None for t in t10)
    assert srv.try_submit(1, raw10) is None  # every 1024^2 slot is taken until a result is collected
    t5 = [srv.try_submit(0, raw5) for _ in range(2)]
    assert all(t is not None for t in t5)  # the 512^2 class still admits
    assert srv.try_submit(0, raw5) is None
    alone = {}
    for c, (raw, sp) in enumerate(((raw5, sp5), (raw10, sp10))):
        plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_LIVE, input_type=fs.native.INPUT_U16, fade_px=10)
        alone[c] = plan.reconstruct_host(raw)
    for c, tickets in ((1, t10), (0, t5)):
        n = (sp5, sp10)[c].w
        for tk in tickets:
            out = np.empty((2 * n, 2 * n), np.float32)
            srv.wait(tk, out)
            assert np.array_equal(out, alone[c])
    assert srv.capacity(0)["free"] == 2 and srv.capacity(1)["free"] == 2
    assert srv.stats()["rejected"] == 2
    srv.close()


def test_slots_follow_the_hbm_budget(fs):
    """Within a device-memory budget the classes take equal shares of bytes: the class of
    small stacks gets more slots than the class of large ones."""
    raw5, sp5 = channel(fs, 256, 33)
    raw10, sp10 = channel(fs, 1024, 34)
    srv = fs.plan.Server([sp5, sp10], max_batch=1, max_inflight=64, streams=1, refit_every=0,
                         hbm_budget_bytes=1 << 30)
    small, large = srv.capacity(0)["slots"], srv.capacity(1)["slots"]
    assert 1 <= large < small <= 64
    srv.close()


def test_refit_on_device_matches_oracle(fs, oracle):
    raw, sp = channel(fs, 512, 11)
    # start from deliberately wrong parameters; the refit must recover them from the stack
    sp0 = sp.duplicate()
    for d in range(3):
        sp0.dir(d).pX += 0.7
        sp0.dir(d).pY -= 0.4
    srv = fs.plan.Server([sp0], max_batch=4, max_inflight=8, streams=2, refit_every=4)
    out = np.empty((1024, 1024), np.float32)
    for _ in range(4):
        srv.wait(srv.submit(0, raw), out)
    deadline = time.time() + 30
    while srv.stats()["refits"] < 1 and time.time() < deadline:
        time.sleep(0.05)
    assert srv.stats()["refits"] >= 1
    got = srv.channel_params(0)
    exp, _ = oracle.live_refit(sp0, raw)
    for d in range(3):
        assert abs(got["pX"][d] - exp["pX"][d]) < 1e-9 and abs(got["pY"][d] - exp["pY"][d]) < 1e-9
    srv.close()


def test_livesim_stream_to_served_reconstructions(fs):
    """A two-channel LIVESIM camera stream (128-byte headers, u16 frames, a sync gap before
    every sequence, neighbouring frames swapped) cut into TCP-sized pieces, through the
    sequence extractor into the server: every stack reconstructs to the bits of that
    channel's stack reconstructed alone."""
    ig = fs.ingest
    specs = [(488, 256, 21, 488.0), (568, 256, 22, 600.0)]
    chans = [channel(fs, n, s, lam) for _, n, s, lam in specs]
    alone = []
    for raw, sp in chans:
        plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_LIVE, input_type=fs.native.INPUT_U16, fade_px=10)
        alone.append(plan.reconstruct_host(raw))
    rng = np.random.default_rng(5)
    n_seq, nraw = 6, 9
    per = []
    for (num, n, _, _), (raw, sp) in zip(specs, chans):
        frames, seq, t = [], 0, 10 ** 6
        for _ in range(n_seq):
            t += 8000  # sync gap (SyncFrameDelay 5000 us)
            for i in range(nraw):
                frames.append(ig.make_frame(raw[i], seq_nr=seq, pos1=num, time_camera=t))
                seq += 1
                t += 1000
        for i in range(1, len(frames) - 1, 7):  # out-of-order arrivals
            frames[i], frames[i + 1] = frames[i + 1], frames[i]
        per.append(frames)
    blob = b"".join(f for pair in zip(*per) for f in pair)
    x = ig.SequenceExtractor([s[0] for s in specs], nraw, 256, 256, sync_mode=0, sync_frame_delay=5000)
    srv = fs.plan.Server([sp for _, sp in chans], max_batch=8, max_inflight=32, streams=2, refit_every=0)
    live = ig.LiveIngest(x, srv)
    tickets = []
    at = 0
    while at < len(blob):
        k = int(rng.integers(1000, 300000))
        tickets += live.feed(blob[at:at + k])
        at += k
    assert len(tickets) == 2 * n_seq and live.dropped == 0
    out = np.empty((512, 512), np.float32)
    for c, tk in tickets:
        srv.wait(tk, out)
        assert np.array_equal(out, alone[c])
    assert x.stats()["sync_frames"] == [n_seq, n_seq]
    srv.close()
    x.close()


def test_vigor_config_drives_ingest_and_server(fs, tmp_path):
    """A VIGOR configuration (vigor-settings: raw size, angles, phases, sync settings, one
    folder per channel with its sim-param and otf2d, as the reference's vigor-*.xml files
    hold them) written, read back and used to set up the sequence extractor and the server;
    a camera stream then reconstructs to the bits of plans built from the loaded channels."""
    cfg = fs.conf.Conf("fairsim")
    vs = cfg.r().mk("vigor-settings")
    vs.newInt("RawPxlCount").setVal(256)
    vs.newDbl("RawPxlSize").setVal(0.08)
    vs.newInt("NrPhases").setVal(3)
    vs.newInt("NrAngles").setVal(3)
    vs.newInt("NrBands").setVal(2)
    for k, v in (("SyncMode", 0), ("SyncFrameFreq", 1), ("SyncFrameAvr", 7000), ("SyncFrameDelay", 5000)):
        vs.newInt(k).setVal(v)
    raws = {}
    for num, seed, lam in ((488, 31, 488.0), (568, 32, 600.0)):
        raw, sp = channel(fs, 256, seed, lam)
        raws[num] = raw
        ch = vs.mk("channel-%d" % num)
        ch.newDbl("offset").setVal(140.0)
        ch.newInt("ChannelNumber").setVal(num)
        sp.saveConfig(ch)
        sp.otf().saveConfig(ch)
    cfg.saveFile(tmp_path / "vigor.xml")
    chans, stream = fs.conf.load_vigor_channels(fs.conf.Conf.loadFile(tmp_path / "vigor.xml").r().cd("vigor-settings"))
    assert [c.number for c in chans] == [488, 568] and stream["raws_per_recon"] == 9
    ig = fs.ingest
    x = ig.SequenceExtractor(**stream)
    srv = fs.plan.Server([c.param for c in chans], max_batch=4, max_inflight=16, streams=2, refit_every=0)
    live = ig.LiveIngest(x, srv)
    frames = []
    for c in chans:
        t, seq = 10 ** 6, 0
        for _ in range(2):
            t += 9000
            for i in range(9):
                frames.append(ig.make_frame(raws[c.number][i], seq_nr=seq, pos1=c.number, time_camera=t))
                seq += 1
                t += 1000
    tickets = []
    for f in frames:
        tickets += live.push(f)
    assert len(tickets) == 4
    out = np.empty((512, 512), np.float32)
    for ci, tk in tickets:
        c = chans[ci]
        srv.wait(tk, out)
        plan = fs.plan.ReconPlan(c.param, path=fs.native.PATH_LIVE, input_type=fs.native.INPUT_U16, fade_px=10)
        assert np.array_equal(out, plan.reconstruct_host(raws[c.number]))
    srv.close()
    x.close()
