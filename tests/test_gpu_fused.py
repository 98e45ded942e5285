"""GPU parity of the fused, batched reconstruction (fsim_plan_* / fsim_recon_batch through
the C ABI) against the oracle's restatement of the reference:
  * offline path = SimAlgorithm.runReconstruction with the GUI's input preparation
    (org/fairsim/sim_gui/ImageControl.java:819-836), CLIPSCALE.NONE;
  * live path = ReconstructionThread.run (org/fairsim/livemode/ReconstructionRunner.java:434-542).
Tolerance: relative L2 <= 1e-4 against the reference's float semantics (spec bound),
and the error against the FP64 oracle is checked to stay below 1e-5."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def make(fs, n, seed, **kw):
    raw, truth = fs.synth.make_dataset(n=n, seed=seed, **kw)
    sp = fs.synth.sim_param_for(truth, n, n_dirs=kw.get("n_dirs", 3), n_phases=kw.get("n_phases", 3),
                                n_bands=kw.get("n_bands", 2))
    return raw, truth, sp


@pytest.mark.parametrize("n", [64, 128, 256, 384, 512, 1024])
def test_offline_fused_vs_oracle(fs, oracle, n):
    raw, truth, sp = make(fs, n, seed=20 + n)
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10)
    got = plan.reconstruct_host(raw)
    exp32 = oracle.recon_raw(sp, raw, fade=10)
    assert rel_l2(got, exp32) < 1e-4
    if n <= 512:
        exp64 = oracle.recon_raw(sp, raw.astype(np.float64), fade=10, dtype=np.float64)
        assert rel_l2(got, exp64) < 1e-5


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
        singles.append(p.reconstruct_host(raw))
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
    for p in (0, 1):
        fs.native.check(lib.fsim_tune_get(n, fs.native.PATH_OFFLINE, p, C.byref(v), C.byref(cnt)))
        saved.append((v.value, cnt.value))
    try:
        for va in range(saved[0][1]):
            for vb in range(saved[1][1]):
                fs.native.check(lib.fsim_tune_set(n, fs.native.PATH_OFFLINE, 0, va))
                fs.native.check(lib.fsim_tune_set(n, fs.native.PATH_OFFLINE, 1, vb))
                assert rel_l2(plan.reconstruct_host(raw), exp) < 1e-4, (va, vb)
    finally:
        fs.native.check(lib.fsim_tune_set(n, fs.native.PATH_OFFLINE, 0, saved[0][0]))
        fs.native.check(lib.fsim_tune_set(n, fs.native.PATH_OFFLINE, 1, saved[1][0]))
