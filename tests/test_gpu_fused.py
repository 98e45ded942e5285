"""GPU parity of the fused, batched reconstruction (fsim_plan_* / fsim_recon_batch through
the C ABI) against the oracle's restatement of the reference:
  * offline path = SimAlgorithm.runReconstruction with the GUI's input preparation
    (org/fairsim/sim_gui/ImageControl.java:819-836), CLIPSCALE.NONE;
  * live path = ReconstructionThread.run (org/fairsim/livemode/ReconstructionRunner.java:434-542).
Tolerance: relative L2 <= 1e-4 against the reference's float semantics (the parity bound),
and the error against the FP64 oracle is checked to stay below 1e-5."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def device_alone(fs, torch, plan, raw, widefield=False, filtered=False):
    """One job alone through the device batch entry (fsim_recon_batch): the bits every other
    entry (host buffers, batches, graphs, the served mix) must reproduce."""
    n = plan.w
    d_raw = torch.from_numpy(raw.view(np.int16) if raw.dtype == np.uint16 else raw).cuda()
    dev = lambda: torch.zeros((2 * n, 2 * n), dtype=torch.float32, device="cuda")  # noqa: E731
    out, wf, fwf = dev(), dev() if widefield else None, dev() if filtered else None
    ws = torch.empty(fs.plan.batch_workspace_bytes([plan]), dtype=torch.uint8, device="cuda")
    ptr = lambda t: t.data_ptr() if t is not None else None  # noqa: E731
    fs.plan.recon_batch([(plan, d_raw.data_ptr(), out.data_ptr(), ptr(wf), ptr(fwf))], ws.data_ptr(), ws.numel())
    torch.cuda.synchronize()
    res = [t.cpu().numpy() if t is not None else None for t in (out, wf, fwf)]
    return res[0] if not (widefield or filtered) else res


def make(fs, n, seed, **kw):
    raw, truth = fs.synth.make_dataset(n=n, seed=seed, **kw)
    sp = fs.synth.sim_param_for(truth, n, n_dirs=kw.get("n_dirs", 3), n_phases=kw.get("n_phases", 3),
                                n_bands=kw.get("n_bands", 2))
    return raw, truth, sp


@pytest.mark.parametrize("n", [64, 128, 192, 256, 384, 512, 768, 1024])
def test_offline_fused_vs_oracle(fs, oracle, n):
    """Every offline size up to 1024^2 (the 3*2^k sizes run radix-3 line plans) within 1e-4
    of the float oracle and 1e-5 of the FP64 oracle (the float oracle itself is 4e-6 from
    it at 768^2 and 8e-6 at 1024^2: the reference rounds the shift phase to float)."""
    raw, truth, sp = make(fs, n, seed=20 + n)
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10)
    got = plan.reconstruct_host(raw)
    exp32 = oracle.recon_raw(sp, raw, fade=10)
    assert rel_l2(got, exp32) < 1e-4
    exp64 = oracle.recon_raw(sp, raw.astype(np.float64), fade=10, dtype=np.float64)
    assert rel_l2(got, exp64) < 1e-5


@pytest.mark.parametrize("clip", [1, 2])
def test_offline_fused_clip_scale_vs_oracle(fs, oracle, torch_cuda, clip):
    """CLIPSCALE.CLIP and .BOTH (the reference's default; SimUtils.clipAndScale,
    S/SimUtils.java:244-264) on the fused plans, alone and in a batch with NONE jobs."""
    torch = torch_cuda
    n = 256
    raw, truth, sp = make(fs, n, seed=27)
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10)
    plan.setClipScale(clip)
    got = plan.reconstruct_host(raw)
    exp = oracle.recon_raw(sp, raw, fade=10, clip_scale=clip)
    assert got.min() >= 0
    assert rel_l2(got, exp) < 1e-4
    if clip == 2:
        assert abs(got.max() - 255.0) < 1e-3
    # in one batch with an unscaled job of the same size: each keeps its own scaling
    plain = fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10)
    d_raw = torch.from_numpy(raw).cuda()
    d_out = [torch.empty((2 * n, 2 * n), dtype=torch.float32, device="cuda") for _ in range(2)]
    ws = torch.empty(fs.plan.batch_workspace_bytes([plan, plain]), dtype=torch.uint8, device="cuda")
    fs.plan.recon_batch([(plan, d_raw.data_ptr(), d_out[0].data_ptr()), (plain, d_raw.data_ptr(), d_out[1].data_ptr())],
                        ws.data_ptr(), ws.numel())
    torch.cuda.synchronize()
    assert np.array_equal(d_out[0].cpu().numpy(), got)
    assert np.array_equal(d_out[1].cpu().numpy(), plain.reconstruct_host(raw))
    assert rel_l2(d_out[1].cpu().numpy(), oracle.recon_raw(sp, raw, fade=10)) < 1e-4


@pytest.mark.parametrize("n", [256, 384, 512, 1024])
def test_b2_bulk_staging_matches_plain_loads(fs, torch_cuda, n):
    """Pass B2 staged through shared memory by bulk copies (cp.async.bulk into an
    mbarrier-tracked ring, where two stages fit) gives the same bits as the variant with plain
    loads, alone and in a batch with another wavelength's window size, and no bounded wait
    expires (device status word)."""
    torch = torch_cuda
    N_ = fs.native
    raw, truth, sp = make(fs, n, seed=51 + n)
    raw2, truth2, sp2 = make(fs, n, seed=52 + n, em_wavelength=600.0)
    plans = [fs.plan.ReconPlan(p, path=N_.PATH_OFFLINE, input_type=N_.INPUT_F32, fade_px=10) for p in (sp, sp2)]
    st, prev = C.c_int(), C.c_int()
    detail = (C.c_int * 3)()
    N_.check(N_.lib().fsim_device_status(C.byref(st), None, 1))

    def run():
        d_raw = [torch.from_numpy(r).cuda() for r in (raw, raw2)]
        d_out = [torch.empty((2 * n, 2 * n), dtype=torch.float32, device="cuda") for _ in range(2)]
        ws = torch.empty(fs.plan.batch_workspace_bytes(plans), dtype=torch.uint8, device="cuda")
        fs.plan.recon_batch([(p, r.data_ptr(), o.data_ptr()) for p, r, o in zip(plans, d_raw, d_out)],
                            ws.data_ptr(), ws.numel())
        torch.cuda.synchronize()
        return [plans[0].reconstruct_host(raw)] + [o.cpu().numpy() for o in d_out]

    N_.check(N_.lib().fsim_debug_b2_staging(1, C.byref(prev)))
    try:
        staged = run()
        N_.check(N_.lib().fsim_debug_b2_staging(0, None))
        plain = run()
    finally:
        N_.check(N_.lib().fsim_debug_b2_staging(prev.value, None))
    N_.check(N_.lib().fsim_device_status(C.byref(st), detail, 1))
    assert st.value == 0, (st.value, [hex(d & 0xffffffff) for d in detail])
    for a, b in zip(staged, plain):
        assert np.array_equal(a, b)
    assert np.array_equal(staged[0], staged[1])


@pytest.mark.parametrize("n,kind,att", [(256, "est", False), (512, "est", True), (1024, "est", False),
                                        (384, "est", True), (256, "measured", True), (256, "live", True),
                                        (512, "live", False)])
def test_plan_filter_table_vs_oracle(fs, oracle, n, kind, att):
    """The plans' resident Wiener x apodization tables (table positions in float-float, the
    apodization from its octant table) against the oracle's double-precision
    getDenominator times writeApoVector: within 1e-7 relative L2, every element within a few
    float ulps, and nearly all of them bit-equal."""
    from test_gpu_vector_api import measured_otf
    raw, truth, sp = make(fs, n, seed=31 + n)
    if kind == "measured":
        sp.setOtf(measured_otf(fs, samples=300))
    sp.otf().setAttenuation(0.97, 1.1)
    sp.otf().switchAttenuation(att)
    live = kind == "live"
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_LIVE if live else fs.native.PATH_OFFLINE,
                             input_type=fs.native.INPUT_U16 if live else fs.native.INPUT_F32, fade_px=10)
    got = plan.filter_table()
    bend, cut = (1.0, 2.0) if live else (sp.apoBend, sp.apoCutOff)
    exp = (oracle.wiener_denominator(sp) * oracle.apo_vector(sp, 2 * n, 2 * n, bend, cut)).astype(np.float32)
    exp = exp[:, :got.shape[1]]
    assert rel_l2(got, exp) < 1e-7
    rel = np.abs(got.astype(np.float64) - exp) / np.maximum(np.abs(exp), 1e-30)
    assert rel.max() < 5e-7
    assert np.count_nonzero(got != exp) <= 1e-3 * got.size


# (with attenuation on, the table must reach the cutoff: the reference indexes beyond its
# arrays otherwise, and the oracle stops there)
@pytest.mark.parametrize("n,samples,att", [(256, 300, False), (512, 300, True), (384, 200, False)])
def test_offline_fused_measured_otf_vs_oracle(fs, oracle, torch_cuda, n, samples, att):
    """Measured two-band complex OTFs (OtfProvider.loadFromConfig with band data) on the fused
    offline plans: complex masks of each component's band and the band-aware Wiener
    denominator, within 1e-4 of the oracle; in one batch with an estimated-OTF plan of the
    same size, each keeps its own result."""
    from test_gpu_vector_api import measured_otf
    torch = torch_cuda
    raw, truth, sp = make(fs, n, seed=23 + n)
    sp.setOtf(measured_otf(fs, samples=samples))
    if att:
        sp.otf().setAttenuation(0.97, 1.1)
        sp.otf().switchAttenuation(True)
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10)
    got = plan.reconstruct_host(raw)
    exp = oracle.recon_raw(sp, raw, fade=10)
    assert rel_l2(got, exp) < 1e-4
    raw2, truth2, sp2 = make(fs, n, seed=24 + n)
    est = fs.plan.ReconPlan(sp2, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10)
    d_raw = [torch.from_numpy(r).cuda() for r in (raw, raw2)]
    d_out = [torch.empty((2 * n, 2 * n), dtype=torch.float32, device="cuda") for _ in range(2)]
    ws = torch.empty(fs.plan.batch_workspace_bytes([plan, est]), dtype=torch.uint8, device="cuda")
    fs.plan.recon_batch([(plan, d_raw[0].data_ptr(), d_out[0].data_ptr()), (est, d_raw[1].data_ptr(), d_out[1].data_ptr())],
                        ws.data_ptr(), ws.numel())
    torch.cuda.synchronize()
    assert np.array_equal(d_out[0].cpu().numpy(), got)
    assert np.array_equal(d_out[1].cpu().numpy(), est.reconstruct_host(raw2))


@pytest.mark.parametrize("variant", ["bgr_att", "five_phases", "three_bands"])
def test_offline_fused_variants(fs, oracle, variant):
    n = 256
    kw = {}
    if variant == "five_phases":
        kw = dict(n_phases=5)
    if variant == "three_bands":
        kw = dict(n_phases=5, n_bands=3)
    raw, truth, sp = make(fs, n, seed=31, **kw)
    bgr = 0.0
    if variant == "bgr_att":
        sp.otf().setAttenuation(0.98, 1.3)
        sp.otf().switchAttenuation(True)
        bgr = 3.0
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10, bgr=bgr)
    got = plan.reconstruct_host(raw)
    exp = oracle.recon_raw(sp, raw, bgr=bgr, fade=10)
    assert rel_l2(got, exp) < 1e-4


@pytest.mark.parametrize("n", [128, 256, 512, 1024])
def test_live_fused_vs_oracle(fs, oracle, n):
    raw, truth, sp = make(fs, n, seed=40 + n, as_u16=True)
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_LIVE, input_type=fs.native.INPUT_U16, fade_px=10)
    got = plan.reconstruct_host(raw)
    exp, _ = oracle.live_recon(sp, raw)
    assert rel_l2(got, exp[0]) < 1e-4


@pytest.mark.parametrize("n", [256, 512])
def test_live_fused_fifteen_frames_vs_oracle(fs, oracle, n):
    """Live path on 3 angles x 5 phases (15-frame stacks, pseudo-inverse separation)."""
    raw, truth, sp = make(fs, n, seed=45 + n, as_u16=True, n_phases=5)
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_LIVE, input_type=fs.native.INPUT_U16, fade_px=10)
    got = plan.reconstruct_host(raw)
    exp, _ = oracle.live_recon(sp, raw)
    assert rel_l2(got, exp[0]) < 1e-4


def test_mixed_batch_datasets_vs_oracle(fs, oracle, torch_cuda):
    """The ragged batch of the mixed workload (sizes 256^2-1024^2, emission 488/525/600 nm,
    per-dataset k0 and modulation 0.5-0.9, 1-3 channels) in one call: one dataset per (size,
    wavelength) against the oracle, not only against its own single run."""
    torch = torch_cuda
    rng = np.random.default_rng(5)
    plans, raws, sps = [], [], []
    for i, n in enumerate((256, 384, 512, 768, 1024)):
        for j, lam in enumerate((488.0, 525.0, 600.0)):
            mod = float(rng.uniform(0.5, 0.9))
            raw, truth = fs.synth.make_dataset(n=n, seed=300 + 3 * i + j, em_wavelength=lam, modulation=mod,
                                               k0_frac=float(rng.uniform(0.75, 0.9)))
            sp = fs.synth.sim_param_for(truth, n)
            plans.append(fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32,
                                           fade_px=10))
            raws.append(raw)
            sps.append(sp)
    d_raw = [torch.from_numpy(r).cuda() for r in raws]
    d_out = [torch.empty((2 * p.w, 2 * p.w), dtype=torch.float32, device="cuda") for p in plans]
    ws = torch.empty(fs.plan.batch_workspace_bytes(plans), dtype=torch.uint8, device="cuda")
    order = rng.permutation(len(plans))  # sizes interleaved in the job table
    fs.plan.recon_batch([(plans[k], d_raw[k].data_ptr(), d_out[k].data_ptr()) for k in order],
                        ws.data_ptr(), ws.numel())
    torch.cuda.synchronize()
    for k in range(len(plans)):
        exp = oracle.recon_raw(sps[k], raws[k], fade=10)
        assert rel_l2(d_out[k].cpu().numpy(), exp) < 1e-4, (plans[k].w, k)


def test_live_widefield_and_attenuation(fs, oracle, torch_cuda):
    torch = torch_cuda
    n = 256
    raw, truth, sp = make(fs, n, seed=51, as_u16=True)
    sp.otf().setAttenuation(0.99, 1.5)
    sp.otf().switchAttenuation(True)
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_LIVE, input_type=fs.native.INPUT_U16, fade_px=10)
    d_raw = torch.from_numpy(raw.view(np.int16)).cuda()
    d_out = torch.empty((2 * n, 2 * n), dtype=torch.float32, device="cuda")
    d_wf = torch.empty((n, n), dtype=torch.float32, device="cuda")
    ws = torch.empty(fs.plan.batch_workspace_bytes([plan]), dtype=torch.uint8, device="cuda")
    fs.plan.recon_batch([(plan, d_raw.data_ptr(), d_out.data_ptr(), d_wf.data_ptr())], ws.data_ptr(), ws.numel())
    torch.cuda.synchronize()
    exp, wf = oracle.live_recon(sp, raw)
    assert rel_l2(d_out.cpu().numpy(), exp[0]) < 1e-4
    assert np.array_equal(d_wf.cpu().numpy(), wf[0])  # float adds in the reference's order


def test_batched_mixed_sizes_identical_to_single(fs, torch_cuda):
    """Ragged batch: datasets of different sizes and parameter sets in one call give the
    same bits as each dataset reconstructed alone."""
    torch = torch_cuda
    specs = [(256, 60), (512, 61), (384, 62), (256, 63), (128, 64), (512, 65)]
    plans, raws, singles = [], [], []
    for n, seed in specs:
        raw, truth, sp = make(fs, n, seed)
        p = fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10)
        plans.append(p)
        raws.append(raw)
        singles.append(device_alone(fs, torch, p, raw))
        # the host-buffer entry runs the same passes: the same bits
        assert np.array_equal(p.reconstruct_host(raw), singles[-1])
    d_raw = [torch.from_numpy(r).cuda() for r in raws]
    d_out = [torch.empty((2 * p.w, 2 * p.w), dtype=torch.float32, device="cuda") for p in plans]
    ws = torch.empty(fs.plan.batch_workspace_bytes(plans), dtype=torch.uint8, device="cuda")
    fs.plan.recon_batch([(p, r.data_ptr(), o.data_ptr()) for p, r, o in zip(plans, d_raw, d_out)],
                        ws.data_ptr(), ws.numel())
    torch.cuda.synchronize()
    for o, s in zip(d_out, singles):
        assert np.array_equal(o.cpu().numpy(), s)


def test_plan_update_changes_parameters(fs, oracle):
    n = 256
    raw, truth, sp = make(fs, n, seed=70)
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10)
    sp2 = sp.duplicate()
    for d in range(3):
        sp2.dir(d).setPhaOff(sp.dir(d).getPhaOff() + 0.3)
        sp2.dir(d).setModulation(1, 0.6)
    plan.update(sp2)
    assert rel_l2(plan.reconstruct_host(raw), oracle.recon_raw(sp2, raw, fade=10)) < 1e-4


def test_estimate_raw_on_device_vs_oracle(fs, oracle, torch_cuda):
    import ctypes as C
    torch = torch_cuda
    n = 512
    raw, truth, sp = make(fs, n, seed=80)
    sp.directions = [fs.Dir(2, 3) for _ in range(3)]
    spec = oracle.prepare_raw(sp, raw)
    est, peaks, _ = oracle.estimate(sp, spec, 1, 0.6)
    c = fs.native.to_c_param(sp)
    d_raw = torch.from_numpy(raw).cuda()
    out = (C.c_double * 12)()
    fs.native.check(fs.native.lib().fsim_estimate_raw(C.byref(c), C.c_void_p(d_raw.data_ptr()), fs.native.INPUT_F32,
                                                      10, 1, C.c_double(0.6), out))
    got = fs.native.from_c_param(c)
    for d in range(3):
        assert abs(got["pX"][d] - est["pX"][d]) < 1e-9 and abs(got["pY"][d] - est["pY"][d]) < 1e-9
        assert abs(got["phaOff"][d] - est["phaOff"][d]) < 1e-4


def test_live_refit_vs_oracle(fs, oracle, torch_cuda):
    import ctypes as C
    torch = torch_cuda
    n = 512
    raw, truth, sp = make(fs, n, seed=90, as_u16=True)
    est, peaks = oracle.live_refit(sp, raw)
    c = fs.native.to_c_param(sp)
    d_raw = torch.from_numpy(raw.view(np.int16)).cuda()
    out = (C.c_double * 12)()
    fs.native.check(fs.native.lib().fsim_live_refit(C.byref(c), C.c_void_p(d_raw.data_ptr()), out))
    got = fs.native.from_c_param(c)
    for d in range(3):
        assert abs(got["pX"][d] - est["pX"][d]) < 1e-9 and abs(got["pY"][d] - est["pY"][d]) < 1e-9
        assert abs(got["modulations"][d][1] - est["modulations"][d][1]) < 1e-4


@pytest.mark.parametrize("n", [384, 512, 1024])
def test_every_tuned_variant_matches_oracle(fs, oracle, n):
    """The autotuner may pick any launch-shape variant: each must give the same result."""
    import ctypes as C
    lib = fs.native.lib()
    raw, truth, sp = make(fs, n, seed=100 + n)
    exp = oracle.recon_raw(sp, raw, fade=10)
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10)
    v, cnt = C.c_int(), C.c_int()
    saved = []
    for p in (0, 1, 2):
        fs.native.check(lib.fsim_tune_get(n, fs.native.PATH_OFFLINE, p, C.byref(v), C.byref(cnt)))
        saved.append((v.value, cnt.value))
    try:
        # every variant of each pass, the other passes at their tuned choice
        for p in (0, 1, 2):
            for var in range(saved[p][1]):
                fs.native.check(lib.fsim_tune_set(n, fs.native.PATH_OFFLINE, p, var))
                assert rel_l2(plan.reconstruct_host(raw), exp) < 1e-4, (p, var)
            fs.native.check(lib.fsim_tune_set(n, fs.native.PATH_OFFLINE, p, saved[p][0]))
    finally:
        for p in (0, 1, 2):
            fs.native.check(lib.fsim_tune_set(n, fs.native.PATH_OFFLINE, p, saved[p][0]))


def test_batch_graph_replays_match_batch(fs, torch_cuda):
    """A batch recorded as a CUDA graph gives the same bits as the direct batch call, reads
    the raw buffers' current contents on each replay, and picks up plan updates."""
    torch = torch_cuda
    specs = [(256, 110), (512, 111), (384, 112), (256, 113)]
    plans, raws = [], []
    for n, seed in specs:
        raw, truth, sp = make(fs, n, seed)
        plans.append(fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10))
        raws.append(raw)
    d_raw = [torch.from_numpy(r).cuda() for r in raws]
    d_out = [torch.empty((2 * p.w, 2 * p.w), dtype=torch.float32, device="cuda") for p in plans]
    ws = torch.empty(fs.plan.batch_workspace_bytes(plans), dtype=torch.uint8, device="cuda")
    jobs = [(p, r.data_ptr(), o.data_ptr()) for p, r, o in zip(plans, d_raw, d_out)]
    fs.plan.recon_batch(jobs, ws.data_ptr(), ws.numel())
    torch.cuda.synchronize()
    direct = [o.cpu().numpy().copy() for o in d_out]
    g = fs.plan.BatchGraph(jobs, ws.data_ptr(), ws.numel())
    assert g.info() == {"jobs": 4, "kernels": 16}  # the job table, three size classes x passes A, G, B1, B2, C
    for o in d_out:
        o.zero_()
    g.launch()
    torch.cuda.synchronize()
    for o, e in zip(d_out, direct):
        assert np.array_equal(o.cpu().numpy(), e)
    # new pixels in a raw buffer and new parameters in a plan reach the next replay
    raw2, _, _ = make(fs, 256, 114)
    d_raw[0].copy_(torch.from_numpy(raw2))
    sp3 = plans[1].sp.duplicate()
    for d in range(3):
        sp3.dir(d).setPhaOff(sp3.dir(d).getPhaOff() + 0.2)
    plans[1].update(sp3)
    g.launch()
    torch.cuda.synchronize()
    assert np.array_equal(d_out[0].cpu().numpy(), device_alone(fs, torch, plans[0], raw2))
    assert np.array_equal(d_out[1].cpu().numpy(), device_alone(fs, torch, plans[1], raws[1]))
    g.close()


def test_misaligned_workspace_refused_before_device_work(fs, torch_cuda):
    """The job table is written to the workspace head with 16-byte stores: a workspace that
    is not 256-byte aligned is refused (EINVAL) before anything is launched."""
    torch = torch_cuda
    raw, truth, sp = make(fs, 64, 160)
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=4)
    d_raw = torch.from_numpy(raw).cuda()
    d_out = torch.zeros((128, 128), dtype=torch.float32, device="cuda")
    need = fs.plan.batch_workspace_bytes([plan])
    ws = torch.empty(need + 256, dtype=torch.uint8, device="cuda")
    with pytest.raises(ValueError, match="aligned"):
        fs.plan.recon_batch([(plan, d_raw.data_ptr(), d_out.data_ptr())], ws.data_ptr() + 16, need + 240)
    fs.plan.recon_batch([(plan, d_raw.data_ptr(), d_out.data_ptr())], ws.data_ptr(), need + 256)
    torch.cuda.synchronize()
    assert np.array_equal(d_out.cpu().numpy(), device_alone(fs, torch, plan, raw))


def test_job_table_over_several_parameter_blocks(fs, torch_cuda):
    """A batch whose job table exceeds one launch-parameter block (400 jobs, about 70 KB of
    descriptors) is written by several table launches: every job's result equals its
    result alone, through the batch entry and through a recorded graph."""
    torch = torch_cuda
    n, n_jobs = 64, 400
    plans, raws = [], []
    for seed in (150, 151, 152):
        raw, truth, sp = make(fs, n, seed)
        plans.append(fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=4))
        raws.append(raw)
    alone = [device_alone(fs, torch, p, r) for p, r in zip(plans, raws)]
    d_raw = [torch.from_numpy(r).cuda() for r in raws]
    d_out = torch.zeros((n_jobs, 2 * n, 2 * n), dtype=torch.float32, device="cuda")
    job_plans = [plans[k % 3] for k in range(n_jobs)]
    ws = torch.empty(fs.plan.batch_workspace_bytes(job_plans), dtype=torch.uint8, device="cuda")
    jobs = [(job_plans[k], d_raw[k % 3].data_ptr(), d_out[k].data_ptr()) for k in range(n_jobs)]
    fs.plan.recon_batch(jobs, ws.data_ptr(), ws.numel())
    torch.cuda.synchronize()
    out = d_out.cpu().numpy()
    for k in range(n_jobs):
        assert np.array_equal(out[k], alone[k % 3]), k
    d_out.zero_()
    g = fs.plan.BatchGraph(jobs, ws.data_ptr(), ws.numel())
    g.launch()
    torch.cuda.synchronize()
    out = d_out.cpu().numpy()
    for k in range(n_jobs):
        assert np.array_equal(out[k], alone[k % 3]), k
    g.close()


@pytest.mark.parametrize("pinned", [True, False])
def test_recon_batch_host_matches_single(fs, torch_cuda, pinned):
    """Host-buffer batches (overlapped upload / passes / download in chunks) give the same
    bits as each stack reconstructed alone, for mixed sizes, paths and input types."""
    torch = torch_cuda
    specs = [(256, 120, "off"), (512, 121, "live"), (384, 122, "off"), (256, 123, "live"), (512, 124, "off")]
    plans, raws, singles, wfs = [], [], [], []
    for n, seed, kind in specs:
        live = kind == "live"
        raw, truth, sp = make(fs, n, seed, as_u16=live)
        p = fs.plan.ReconPlan(sp, path=fs.native.PATH_LIVE if live else fs.native.PATH_OFFLINE,
                              input_type=fs.native.INPUT_U16 if live else fs.native.INPUT_F32, fade_px=10)
        plans.append(p)
        raws.append(raw)
        singles.append(p.reconstruct_host(raw))
    if pinned:
        h_raw = [torch.from_numpy(r.view(np.int16) if r.dtype == np.uint16 else r).pin_memory() for r in raws]
        h_out = [torch.empty((2 * p.w, 2 * p.w), dtype=torch.float32).pin_memory() for p in plans]
        ptr = lambda t: t.data_ptr()  # noqa: E731
        get = lambda t: t.numpy()  # noqa: E731
    else:
        h_raw = [np.ascontiguousarray(r) for r in raws]
        h_out = [np.empty((2 * p.w, 2 * p.w), np.float32) for p in plans]
        ptr = lambda a: a.ctypes.data  # noqa: E731
        get = lambda a: a  # noqa: E731
    h_wf = [np.empty((p.w, p.w), np.float32) if p.path == fs.native.PATH_LIVE else None for p in plans]
    jobs = [(p, ptr(r), ptr(o), w.ctypes.data if w is not None else None) for p, r, o, w in zip(plans, h_raw, h_out, h_wf)]
    fs.plan.recon_batch_host(jobs, chunk=2)
    for o, s in zip(h_out, singles):
        assert np.array_equal(get(o), s)
    for p, w, r in zip(plans, h_wf, raws):
        if w is not None:
            d_raw = torch.from_numpy(r.view(np.int16)).cuda()
            d_out = torch.empty((2 * p.w, 2 * p.w), dtype=torch.float32, device="cuda")
            d_wf = torch.empty((p.w, p.w), dtype=torch.float32, device="cuda")
            ws = torch.empty(fs.plan.batch_workspace_bytes([p]), dtype=torch.uint8, device="cuda")
            fs.plan.recon_batch([(p, d_raw.data_ptr(), d_out.data_ptr(), d_wf.data_ptr())], ws.data_ptr(), ws.numel())
            torch.cuda.synchronize()
            assert np.array_equal(w, d_wf.cpu().numpy())


def test_offline_large_five_phase_vs_oracle(fs, oracle):
    """2048^2, 3 angles x 5 phases (pseudo-inverse separation), |k0| = 0.9 cutoff,
    modulation 0.6, 200 photons, reconstructed to 4096^2: within 1e-4 relative L2 of the
    float oracle; the error against the FP64 oracle is recorded."""
    n = 2048
    raw, truth, sp = make(fs, n, seed=130, n_phases=5, k0_frac=0.9, modulation=0.6, photons=200.0)
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10)
    got = plan.reconstruct_host(raw)
    exp32 = oracle.recon_raw(sp, raw, fade=10)
    e32 = rel_l2(got, exp32)
    exp64 = oracle.recon_raw(sp, raw.astype(np.float64), fade=10, dtype=np.float64)
    e64 = rel_l2(got, exp64)
    print("2048^2 3x5: rel-L2 vs float oracle %.3e, vs FP64 oracle %.3e (oracle float vs FP64 %.3e)"
          % (e32, e64, rel_l2(exp32, exp64)))
    assert e32 < 1e-4
    assert e64 < 1e-4


def test_estimate_raw_1024_vs_oracle(fs, oracle, torch_cuda):
    """Full parameter fit at 1024^2 (locatePeak, fitPeak 3 x 10 x 10, getPeak): the fitted
    shifts equal the oracle's and land on the generator's k0 pixel."""
    import ctypes as C
    torch = torch_cuda
    n = 1024
    raw, truth, sp = make(fs, n, seed=140)
    sp.directions = [fs.Dir(2, 3) for _ in range(3)]
    spec = oracle.prepare_raw(sp, raw)
    est, peaks, _ = oracle.estimate(sp, spec, 1, 0.6)
    c = fs.native.to_c_param(sp)
    d_raw = torch.from_numpy(raw).cuda()
    out = (C.c_double * 12)()
    fs.native.check(fs.native.lib().fsim_estimate_raw(C.byref(c), C.c_void_p(d_raw.data_ptr()), fs.native.INPUT_F32,
                                                      10, 1, C.c_double(0.6), out))
    got = fs.native.from_c_param(c)
    for d in range(3):
        assert abs(got["pX"][d] - est["pX"][d]) < 1e-9 and abs(got["pY"][d] - est["pY"][d]) < 1e-9
        assert abs(got["phaOff"][d] - est["phaOff"][d]) < 1e-4
        assert abs(got["pX"][d] - truth["pxpy"][d][0]) < 0.1 and abs(got["pY"][d] - truth["pxpy"][d][1]) < 0.1


@pytest.mark.parametrize("n", [64, 128, 192, 256, 384, 512, 768, 1024])
def test_offline_widefield_outputs_vs_oracle(fs, oracle, n):
    """The "Widefield" and "filtered Widefield" side outputs of runReconstruction
    (S/SimAlgorithm.java:533-576), computed on the device after the passes, against the
    oracle; the reconstruction itself is unchanged by asking for them."""
    raw, truth, sp = make(fs, n, seed=60 + n)
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10)
    img, wf, fwf = plan.reconstruct_host_widefield(raw)
    assert np.array_equal(img, plan.reconstruct_host(raw))
    e_wf, e_fwf = oracle.widefield_raw(sp, raw, fade=10)
    assert rel_l2(wf, e_wf) < 1e-4
    assert rel_l2(fwf, e_fwf) < 1e-4
    if n <= 512:
        d_wf, d_fwf = oracle.widefield_raw(sp, raw.astype(np.float64), fade=10, dtype=np.float64)
        assert rel_l2(wf, d_wf) < 1e-5
        assert rel_l2(fwf, d_fwf) < 1e-5


@pytest.mark.parametrize("variant", ["u16_bgr_att", "five_phases", "three_bands", "2048"])
def test_offline_widefield_variants(fs, oracle, variant):
    """u16 input with background and an attenuated OTF (the widefield filter is never
    attenuated), 5 phases (pseudo-inverse separation), 3 bands, and the largest size."""
    n, kw, bgr = 256, {}, 0.0
    if variant == "u16_bgr_att":
        kw = dict(as_u16=True)
    if variant == "five_phases":
        kw = dict(n_phases=5)
    if variant == "three_bands":
        kw = dict(n_phases=5, n_bands=3)
    if variant == "2048":
        n = 2048
    raw, truth, sp = make(fs, n, seed=71, **kw)
    u16 = raw.dtype == np.uint16
    if u16:
        sp.otf().setAttenuation(0.98, 1.3)
        sp.otf().switchAttenuation(True)
        bgr = 3.0
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE,
                             input_type=fs.native.INPUT_U16 if u16 else fs.native.INPUT_F32, fade_px=10, bgr=bgr)
    img, wf, fwf = plan.reconstruct_host_widefield(raw)
    e_wf, e_fwf = oracle.widefield_raw(sp, raw.astype(np.float32), bgr=bgr, fade=10)
    assert rel_l2(wf, e_wf) < 1e-4
    assert rel_l2(fwf, e_fwf) < 1e-4
    assert rel_l2(img, oracle.recon_raw(sp, raw.astype(np.float32), bgr=bgr, fade=10)) < 1e-4


def test_widefield_in_batches_and_graphs(fs, torch_cuda):
    """Widefield outputs for some jobs of a mixed batch: the same bits as each job alone, no
    change to the jobs that do not ask, the same bits again from a CUDA-graph replay (three
    more launches per size class that asks), and EINVAL for a filtered widefield on a live plan."""
    torch = torch_cuda
    specs = [(256, 130, 2), (512, 131, 0), (384, 132, 1), (256, 133, 0)]  # 2: both, 1: widefield only
    plans, raws = [], []
    for n, seed, _ in specs:
        raw, truth, sp = make(fs, n, seed)
        plans.append(fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10))
        raws.append(raw)
    dev = lambda shape: torch.zeros(shape, dtype=torch.float32, device="cuda")  # noqa: E731
    d_raw = [torch.from_numpy(r).cuda() for r in raws]
    d_out = [dev((2 * p.w, 2 * p.w)) for p in plans]
    d_wf = [dev((2 * p.w, 2 * p.w)) if s[2] >= 1 else None for p, s in zip(plans, specs)]
    d_fwf = [dev((2 * p.w, 2 * p.w)) if s[2] == 2 else None for p, s in zip(plans, specs)]
    ws = torch.empty(fs.plan.batch_workspace_bytes(plans), dtype=torch.uint8, device="cuda")
    ptr = lambda t: t.data_ptr() if t is not None else None  # noqa: E731
    jobs = [(p, ptr(r), ptr(o), ptr(w), ptr(f)) for p, r, o, w, f in zip(plans, d_raw, d_out, d_wf, d_fwf)]
    fs.plan.recon_batch(jobs, ws.data_ptr(), ws.numel())
    torch.cuda.synchronize()
    for i, (p, r) in enumerate(zip(plans, raws)):
        img, wf, fwf = device_alone(fs, torch, p, r, widefield=True, filtered=True)
        assert np.array_equal(d_out[i].cpu().numpy(), img)
        if d_wf[i] is not None:
            assert np.array_equal(d_wf[i].cpu().numpy(), wf)
        if d_fwf[i] is not None:
            assert np.array_equal(d_fwf[i].cpu().numpy(), fwf)
    first = [[t.cpu().numpy().copy() if t is not None else None for t in ts] for ts in (d_out, d_wf, d_fwf)]
    g = fs.plan.BatchGraph(jobs, ws.data_ptr(), ws.numel())
    assert g.info() == {"jobs": 4, "kernels": 16 + 3 * 2}  # the 256 and 384 classes ask
    for ts in (d_out, d_wf, d_fwf):
        for t in ts:
            if t is not None:
                t.zero_()
    g.launch()
    torch.cuda.synchronize()
    for ts, fs_ in zip((d_out, d_wf, d_fwf), first):
        for t, e in zip(ts, fs_):
            if t is not None:
                assert np.array_equal(t.cpu().numpy(), e)
    g.close()
    live_raw, _, live_sp = make(fs, 256, 134, as_u16=True)
    live = fs.plan.ReconPlan(live_sp, path=fs.native.PATH_LIVE, input_type=fs.native.INPUT_U16, fade_px=10)
    lr = torch.from_numpy(live_raw.view(np.int16)).cuda()
    lo, lw, lf = dev((512, 512)), dev((256, 256)), dev((512, 512))
    ws2 = torch.empty(fs.plan.batch_workspace_bytes([live]), dtype=torch.uint8, device="cuda")
    with pytest.raises(ValueError):
        fs.plan.recon_batch([(live, lr.data_ptr(), lo.data_ptr(), lw.data_ptr(), lf.data_ptr())],
                            ws2.data_ptr(), ws2.numel())


def test_recon_batch_host_widefield(fs, torch_cuda):
    """Host-buffer batches carry the offline widefield outputs (2w x 2w) and the live one (w x w)."""
    torch = torch_cuda
    specs = [(256, 140, "off"), (512, 141, "live"), (384, 142, "off")]
    plans, raws = [], []
    for n, seed, kind in specs:
        live = kind == "live"
        raw, truth, sp = make(fs, n, seed, as_u16=live)
        plans.append(fs.plan.ReconPlan(sp, path=fs.native.PATH_LIVE if live else fs.native.PATH_OFFLINE,
                                       input_type=fs.native.INPUT_U16 if live else fs.native.INPUT_F32, fade_px=10))
        raws.append(raw)
    pin = lambda shape: torch.empty(shape, dtype=torch.float32).pin_memory()  # noqa: E731
    h_raw = [torch.from_numpy(r.view(np.int16) if r.dtype == np.uint16 else r).pin_memory() for r in raws]
    h_out = [pin((2 * p.w, 2 * p.w)) for p in plans]
    h_wf = [pin((p.w, p.w)) if p.path == fs.native.PATH_LIVE else pin((2 * p.w, 2 * p.w)) for p in plans]
    h_fwf = [pin((2 * p.w, 2 * p.w)) if p.path == fs.native.PATH_OFFLINE else None for p in plans]
    jobs = [(p, r.data_ptr(), o.data_ptr(), w.data_ptr(), f.data_ptr() if f is not None else None)
            for p, r, o, w, f in zip(plans, h_raw, h_out, h_wf, h_fwf)]
    fs.plan.recon_batch_host(jobs, chunk=2)
    for p, r, o, w, f in zip(plans, raws, h_out, h_wf, h_fwf):
        single = p.reconstruct_host_widefield(r)
        assert np.array_equal(o.numpy(), single[0])
        assert np.array_equal(w.numpy(), single[1])
        if f is not None:
            assert np.array_equal(f.numpy(), single[2])


@pytest.mark.parametrize("layout", ["one_array", "separate"])
def test_recon_batch_host_merged_copies(fs, torch_cuda, layout):
    """Stacks whose host buffers are one page-locked array move as one copy per chunk and
    direction; buffers in separate allocations (adjacent or not) are copied one by one. Both
    give the same bits as each stack reconstructed alone."""
    torch = torch_cuda
    n, B = 256, 6
    raw0, truth, sp = make(fs, n, seed=150)
    p = fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10)
    g = np.random.default_rng(150)
    raws = [np.ascontiguousarray(raw0 * np.float32(1 + 0.1 * i) + g.random(raw0.shape, np.float32)) for i in range(B)]
    singles = [p.reconstruct_host(r) for r in raws]
    if layout == "one_array":
        h_raw_all = torch.from_numpy(np.stack(raws)).pin_memory()
        h_out_all = torch.empty((B, 2 * n, 2 * n), dtype=torch.float32).pin_memory()
        h_raw, h_out = list(h_raw_all), list(h_out_all)
    else:
        h_raw = [torch.from_numpy(r).pin_memory() for r in raws]
        h_out = [torch.empty((2 * n, 2 * n), dtype=torch.float32).pin_memory() for _ in range(B)]
    fs.plan.recon_batch_host([(p, r.data_ptr(), o.data_ptr()) for r, o in zip(h_raw, h_out)], chunk=3)
    for o, s in zip(h_out, singles):
        assert np.array_equal(o.numpy(), s)


def test_plan_from_saved_config(fs, oracle, tmp_path):
    """A parameter set written as the reference's XML (SimParam.saveConfig,
    OtfProvider.saveConfig), read back and used for a plan: the reconstruction matches the
    oracle on the loaded parameters."""
    raw, truth, sp = make(fs, 256, seed=80)
    sp.otf().setAttenuation(0.98, 1.3)
    sp.otf().switchAttenuation(True)
    cfg = fs.conf.Conf("fairsim")
    sp.saveConfig(cfg.r())
    sp.otf().saveConfig(cfg.r())
    cfg.saveFile(tmp_path / "param.xml")
    root = fs.conf.Conf.loadFile(tmp_path / "param.xml").r()
    lp = fs.SimParam.loadConfig(root)
    lp.setOtf(fs.OtfProvider.loadFromConfig(root))
    plan = fs.plan.ReconPlan(lp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10)
    assert rel_l2(plan.reconstruct_host(raw), oracle.recon_raw(lp, raw, fade=10)) < 1e-4
