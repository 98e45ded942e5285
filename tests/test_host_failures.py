"""Host-side failure handling of the C ABI, without a GPU: malformed arguments are refused
with FSIM_EINVAL (mapped to ValueError, the reference's Vec.failSize / IllegalArgument
behaviour) before any device work, and every failure leaves a message for the calling
thread. These run before the library touches a device, so they hold on a CPU-only host."""
import ctypes as C

import numpy as np
import pytest


def _param(fs, n=256, **kw):
    sp = fs.synth.synthetic_params(n)
    c = fs.native.to_c_param(sp)
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def _create(fs, c, path=0, input_type=0, fade=10):
    h = C.c_void_p()
    return fs.native.lib().fsim_plan_create(C.byref(h), C.byref(c), path, input_type, fade, 0.0), h


@pytest.mark.parametrize("field,value", [("w", 100), ("w", 4), ("nr_phases", 2), ("nr_bands", 5), ("na", 0.1),
                                         ("em_wavelength", 5000.0), ("otf_a", 1.5), ("microns_per_pixel", 0.0)])
def test_plan_create_rejects_malformed_parameters(fs, field, value):
    rc, h = _create(fs, _param(fs, **{field: value}))
    assert rc == fs.native.FSIM_EINVAL
    assert h.value is None
    assert fs.native.lib().fsim_last_error()


def test_plan_create_rejects_bad_path_type_and_fade(fs):
    c = _param(fs)
    assert _create(fs, c, path=7)[0] == fs.native.FSIM_EINVAL
    assert _create(fs, c, input_type=3)[0] == fs.native.FSIM_EINVAL
    assert _create(fs, c, fade=200)[0] == fs.native.FSIM_EINVAL
    assert _create(fs, c, path=fs.native.PATH_LIVE, fade=-1)[0] == fs.native.FSIM_EINVAL


def test_python_mirror_raises_value_error(fs):
    sp = fs.synth.synthetic_params(100)
    with pytest.raises(ValueError):
        fs.plan.ReconPlan(sp)


def test_batch_entries_reject_empty_batches(fs):
    lib = fs.native.lib()
    assert lib.fsim_recon_batch(None, 0, None, 0, None) == fs.native.FSIM_EINVAL
    assert lib.fsim_recon_batch_host(None, 0, 0) == fs.native.FSIM_EINVAL
    g = C.c_void_p()
    assert lib.fsim_batch_graph_create(C.byref(g), None, 0, None, 0, None) == fs.native.FSIM_EINVAL
    assert lib.fsim_batch_graph_launch(None, None) == fs.native.FSIM_EINVAL
    assert lib.fsim_batch_graph_destroy(None) == fs.native.FSIM_OK


def _serve_open(fs, cfg, params):
    arr = (fs.native.SimParamC * len(params))(*params)
    h = C.c_void_p()
    return fs.native.lib().fsim_serve_open(C.byref(h), C.byref(cfg), arr, len(params)), h


@pytest.mark.parametrize("cfg_args", [(0, 8, 2, 0, 1, 10, 1 << 30), (4, 0, 2, 0, 1, 10, 1 << 30),
                                      (4, 8, 0, 0, 1, 10, 1 << 30), (4, 8, 2, 0, 9, 10, 1 << 30)])
def test_serve_open_rejects_bad_config(fs, cfg_args):
    rc, h = _serve_open(fs, fs.native.ServeConfig(*cfg_args), [_param(fs)])
    assert rc == fs.native.FSIM_EINVAL and h.value is None


def test_serve_open_rejects_bad_channel(fs):
    cfg = fs.native.ServeConfig(4, 8, 2, 0, 1, 10, 1 << 30)
    assert _serve_open(fs, cfg, [_param(fs), _param(fs, w=100)])[0] == fs.native.FSIM_EINVAL
    assert _serve_open(fs, cfg, [_param(fs, nr_dirs=0)])[0] == fs.native.FSIM_EINVAL


def test_serve_calls_on_null_server(fs):
    lib = fs.native.lib()
    t = C.c_uint64()
    raw = np.zeros(16, np.uint16)
    assert lib.fsim_serve_submit(None, 0, raw.ctypes.data_as(C.c_void_p), raw.nbytes, C.byref(t)) == fs.native.FSIM_EINVAL
    assert lib.fsim_serve_cancel(None, 1) == fs.native.FSIM_EINVAL
    assert lib.fsim_serve_close(None) == fs.native.FSIM_OK


def test_fail_alloc_hook_arms_and_disarms(fs):
    lib = fs.native.lib()
    assert lib.fsim_debug_fail_alloc(-1) == fs.native.FSIM_EINVAL
    assert lib.fsim_debug_fail_alloc(3) == fs.native.FSIM_OK
    assert lib.fsim_debug_fail_alloc(0) == fs.native.FSIM_OK


def test_status_codes_map_to_exception_types(fs):
    N = fs.native
    with pytest.raises(ValueError):
        N.check(N.FSIM_EINVAL)
    with pytest.raises(MemoryError):
        N.check(N.FSIM_EOOM)
    with pytest.raises(TimeoutError):
        N.check(N.FSIM_ETIMEOUT)
    with pytest.raises(N.FsimBusy):
        N.check(N.FSIM_EBUSY)
    with pytest.raises(N.FsimError):
        N.check(N.FSIM_ECUDA)


def test_fft_plan_checks_sizes_without_a_device(fs):
    lib = fs.native.lib()
    h = C.c_int64()
    assert lib.fsim_fft_plan_2d(100, 64, C.byref(h)) == fs.native.FSIM_EINVAL
    assert lib.fsim_fft_plan_2d(512, 384, C.byref(h)) == fs.native.FSIM_OK
    assert (h.value >> 32, h.value & 0xffffffff) == (512, 384)
