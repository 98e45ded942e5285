"""Golden fixtures (tests/golden/, made by tests/golden/make_golden.py from the oracle):
the oracle must still reproduce them (CPU), and the GPU path must match them within the
parity tolerance (1e-4 relative L2 on images; fitted shifts to 1e-9 px)."""
import os

import numpy as np
import pytest

from conftest import rel_l2

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLD, name + ".npz")))


def sim_param(fs, d, n):
    truth = {"pxpy": [tuple(v) for v in d["pxpy"]], "phi0": list(d["phi0"]), "modulation": float(d["modulation"]),
             "na": float(d["na"]), "em_wavelength": float(d["em_wavelength"]), "pxl_um": float(d["pxl_um"]),
             "otf_a": float(d["otf_a"])}
    return fs.synth.sim_param_for(truth, n)


@pytest.mark.parametrize("name,n", [("offline_64", 64), ("offline_128", 128)])
def test_oracle_reproduces_offline_golden(fs, oracle, name, n):
    d = load(name)
    got = oracle.recon_raw(sim_param(fs, d, n), d["raw"], fade=10)
    assert rel_l2(got, d["out"]) < 1e-6


def test_oracle_reproduces_live_golden(fs, oracle):
    d = load("live_64")
    rec, wf = oracle.live_recon(sim_param(fs, d, 64), d["raw"])
    assert rel_l2(rec[0], d["out"]) < 1e-6
    assert rel_l2(wf[0], d["widefield"]) < 1e-7


def test_oracle_reproduces_estimate_golden(fs, oracle):
    d = load("offline_128")
    sp = sim_param(fs, d, 128)
    sp.directions = [fs.Dir(2, 3) for _ in range(3)]
    est, _, _ = oracle.estimate(sp, oracle.prepare_raw(sp, d["raw"]), 1, 0.6)
    assert np.allclose(est["pX"][:3], d["est_px"], atol=1e-9, rtol=0)
    assert np.allclose(est["pY"][:3], d["est_py"], atol=1e-9, rtol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("name,n", [("offline_64", 64), ("offline_128", 128)])
def test_gpu_matches_offline_golden(fs, name, n):
    d = load(name)
    plan = fs.plan.ReconPlan(sim_param(fs, d, n), path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32,
                             fade_px=10)
    got = plan.reconstruct_host(d["raw"])
    assert rel_l2(got, d["out"]) < 1e-4
    if "out64" in d:
        assert rel_l2(got, d["out64"]) < 1e-5


@pytest.mark.gpu
def test_gpu_matches_live_golden(fs, torch_cuda):
    torch = torch_cuda
    d = load("live_64")
    plan = fs.plan.ReconPlan(sim_param(fs, d, 64), path=fs.native.PATH_LIVE, input_type=fs.native.INPUT_U16,
                             fade_px=10)
    d_raw = torch.from_numpy(d["raw"].view(np.int16)).cuda()
    d_out = torch.empty((128, 128), dtype=torch.float32, device="cuda")
    d_wf = torch.empty((64, 64), dtype=torch.float32, device="cuda")
    ws = torch.empty(fs.plan.batch_workspace_bytes([plan]), dtype=torch.uint8, device="cuda")
    fs.plan.recon_batch([(plan, d_raw.data_ptr(), d_out.data_ptr(), d_wf.data_ptr())], ws.data_ptr(), ws.numel())
    torch.cuda.synchronize()
    assert rel_l2(d_out.cpu().numpy(), d["out"]) < 1e-4
    assert rel_l2(d_wf.cpu().numpy(), d["widefield"]) < 1e-7


@pytest.mark.gpu
def test_gpu_matches_estimate_golden(fs, torch_cuda):
    import ctypes as C

    torch = torch_cuda
    d = load("offline_128")
    sp = sim_param(fs, d, 128)
    sp.directions = [fs.Dir(2, 3) for _ in range(3)]
    c = fs.native.to_c_param(sp)
    d_raw = torch.from_numpy(d["raw"]).cuda()
    out = (C.c_double * 12)()
    fs.native.check(fs.native.lib().fsim_estimate_raw(C.byref(c), C.c_void_p(d_raw.data_ptr()), fs.native.INPUT_F32,
                                                      10, 1, C.c_double(0.6), out))
    got = fs.native.from_c_param(c)
    assert np.allclose(got["pX"][:3], d["est_px"], atol=1e-9, rtol=0)
    assert np.allclose(got["pY"][:3], d["est_py"], atol=1e-9, rtol=0)
    assert np.allclose(got["phaOff"][:3], d["est_pha"], atol=1e-4, rtol=0)
