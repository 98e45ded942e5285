"""CPU checks of the drop-in boundary: the C-ABI library loads without a GPU and exports
every function that include/fairsim_gb300.h declares; calls made without a device fail
with a status code instead of crashing."""
import ctypes
import os

import pytest


def test_library_exports_every_declared_symbol(fs):
    lib = fs.native.lib()
    names = fs.native.header_functions()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, "declared but not exported: %s" % missing


def test_param_struct_layout_matches_oracle(fs):
    from oracle import refcpu

    assert ctypes.sizeof(fs.native.SimParamC) == ctypes.sizeof(refcpu.RefParam)
    for (a, _), (b, _) in zip(fs.native.SimParamC._fields_, refcpu.RefParam._fields_):
        assert getattr(fs.native.SimParamC, a).offset == getattr(refcpu.RefParam, b).offset


def test_calls_without_device_return_status(fs):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = fs.native.lib()
    rc = lib.fsim_init(0)
    assert rc == fs.native.FSIM_ENODEV
    assert b"device" in lib.fsim_last_error()
