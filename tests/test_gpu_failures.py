"""Failure handling on the GPU, injected on the host only (no GPU fault, trap or hang):
  * forced device-allocation failures (fsim_debug_fail_alloc) at every allocation of plan
    creation, host-buffer batches, the parameter fit and server start-up return FSIM_EOOM
    (MemoryError), leave nothing half-built, and the next call succeeds;
  * a malformed stack size is refused at submission (ValueError) and counted nowhere;
  * cancelled requests free their slots (queued, finished, or still on the GPU) and cannot
    be waited on; the other requests in the mix are unaffected;
  * a slow consumer that does not collect results makes admission refuse new stacks
    (FSIM_EBUSY) instead of dropping or overwriting finished results."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _disarm(fs):
    yield
    fs.native.lib().fsim_debug_fail_alloc(0)


def _data(fs, n=256, seed=3, u16=False):
    raw, truth = fs.synth.make_dataset(n=n, seed=seed, as_u16=u16)
    return raw, fs.synth.sim_param_for(truth, n)


def test_plan_create_survives_every_allocation_failure(fs, oracle):
    raw, sp = _data(fs)
    fs.native.init()
    failures = 0
    for k in range(1, 12):
        fs.native.lib().fsim_debug_fail_alloc(k)
        try:
            plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10)
            got = plan.reconstruct_host(raw)  # an allocation here may be the k-th one
        except MemoryError:
            failures += 1
            continue
        finally:
            fs.native.lib().fsim_debug_fail_alloc(0)
        assert np.array_equal(got, plan.reconstruct_host(raw))
    assert failures >= 2
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10)
    exp = oracle.recon_raw(sp, raw, fade=10)
    got = plan.reconstruct_host(raw)
    assert np.linalg.norm(got - exp) / np.linalg.norm(exp) < 1e-4


def test_host_batch_allocation_failure_then_success(fs):
    raw, sp = _data(fs, n=384, seed=4)
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_OFFLINE, input_type=fs.native.INPUT_F32, fade_px=10)
    ref = plan.reconstruct_host(raw)
    out = np.empty_like(ref)
    fs.native.lib().fsim_debug_fail_alloc(1)
    with pytest.raises(MemoryError):
        fs.plan.recon_batch_host([(plan, raw.ctypes.data, out.ctypes.data)])
    fs.native.lib().fsim_debug_fail_alloc(0)
    fs.plan.recon_batch_host([(plan, raw.ctypes.data, out.ctypes.data)])
    assert np.array_equal(out, ref)


def test_estimate_allocation_failure_then_success(fs, torch_cuda):
    torch = torch_cuda
    raw, sp = _data(fs, n=256, seed=5)
    sp.directions = [fs.Dir(2, 3) for _ in range(3)]
    d_raw = torch.from_numpy(raw).cuda()
    lib = fs.native.lib()
    out = (C.c_double * 12)()
    results = []
    for k in (1, 2, 3, 5, 8, 0):
        c = fs.native.to_c_param(sp)
        lib.fsim_debug_fail_alloc(k)
        rc = lib.fsim_estimate_raw(C.byref(c), C.c_void_p(d_raw.data_ptr()), fs.native.INPUT_F32, 10, 1,
                                   C.c_double(0.6), out)
        lib.fsim_debug_fail_alloc(0)
        assert rc in (fs.native.FSIM_OK, fs.native.FSIM_EOOM)
        if rc == fs.native.FSIM_OK:
            results.append([fs.native.from_c_param(c)["pX"][d] for d in range(3)])
    assert len(results) >= 1 and all(r == results[-1] for r in results)


def test_server_open_survives_allocation_failures(fs):
    raw, sp = _data(fs, u16=True)
    for k in range(1, 10):
        fs.native.lib().fsim_debug_fail_alloc(k)
        try:
            srv = fs.plan.Server([sp], max_batch=2, max_inflight=4, streams=2, refit_every=0)
        except MemoryError:
            continue
        finally:
            fs.native.lib().fsim_debug_fail_alloc(0)
        srv.close()
    srv = fs.plan.Server([sp], max_batch=2, max_inflight=4, streams=2, refit_every=0)
    out = np.empty((512, 512), np.float32)
    srv.wait(srv.submit(0, raw), out)
    srv.close()


def test_malformed_stack_is_refused(fs):
    raw, sp = _data(fs, u16=True)
    srv = fs.plan.Server([sp], max_batch=2, max_inflight=4, streams=1, refit_every=0)
    with pytest.raises(ValueError):
        srv.submit(0, raw[:8])  # 8 of 9 frames
    with pytest.raises(ValueError):
        srv.submit(0, raw.astype(np.float32).view(np.uint16))  # twice the bytes
    with pytest.raises(ValueError):
        srv.submit(3, raw)  # no such channel
    st = srv.stats()
    assert st["submitted"] == 0 and st["rejected"] == 0
    out = np.empty((512, 512), np.float32)
    srv.wait(srv.submit(0, raw), out)
    srv.close()


def test_cancelled_requests_free_their_slots(fs):
    raw, sp = _data(fs, u16=True)
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_LIVE, input_type=fs.native.INPUT_U16, fade_px=10)
    ref = plan.reconstruct_host(raw)
    srv = fs.plan.Server([sp], max_batch=2, max_inflight=6, streams=1, refit_every=0)
    tickets = [srv.submit(0, raw) for _ in range(6)]
    assert srv.try_submit(0, raw) is None  # full
    for t in tickets[::2]:
        srv.cancel(t)  # queued, running or done: each is released
    with pytest.raises(KeyError):
        srv.cancel(tickets[0])
    out = np.empty((512, 512), np.float32)
    for t in tickets[1::2]:
        srv.wait(t, out)
        assert np.array_equal(out, ref)
    with pytest.raises(KeyError):
        srv.wait(tickets[0], out, timeout_ms=100)
    # every slot comes back once the cancelled work has left the GPU
    import time

    deadline = time.time() + 10
    again = []
    while len(again) < 6 and time.time() < deadline:
        t = srv.try_submit(0, raw)
        if t is None:
            time.sleep(0.01)
        else:
            again.append(t)
    assert len(again) == 6
    for t in again:
        srv.wait(t, out)
        assert np.array_equal(out, ref)
    st = srv.stats()
    assert st["cancelled"] == 3
    srv.close()


def test_slow_consumer_gets_busy_not_dropped_results(fs):
    raw, sp = _data(fs, u16=True)
    plan = fs.plan.ReconPlan(sp, path=fs.native.PATH_LIVE, input_type=fs.native.INPUT_U16, fade_px=10)
    ref = plan.reconstruct_host(raw)
    srv = fs.plan.Server([sp], max_batch=4, max_inflight=4, streams=2, refit_every=0)
    tickets = [srv.submit(0, raw) for _ in range(4)]
    import time

    time.sleep(0.5)  # all four finish on the GPU; nobody collects them
    refused = sum(srv.try_submit(0, raw) is None for _ in range(10))
    assert refused == 10
    out = np.empty((512, 512), np.float32)
    for t in tickets:  # the finished results are all still there, unchanged
        srv.wait(t, out)
        assert np.array_equal(out, ref)
    assert srv.stats()["rejected"] == 10
    srv.close()
