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


def test_jni_shim_defines_every_reference_native():
    """The JNI shim must export the symbol of every `native` method the reference's accel
    classes declare (list in tests/golden/jni_natives.txt, made by make_jni_natives.py), so
    that those classes load the GB300 library unchanged. Checked on the source: no jni.h
    is installed here to compile it."""
    import re

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    want = open(os.path.join(root, "tests", "golden", "jni_natives.txt")).read().split()
    src = open(os.path.join(root, "fairsim-vigor_gb300", "jni", "fsim_jni.cpp")).read()
    have = {"Java_org_fairsim_accel_%s_%s" % m for m in re.findall(r"JFN\(\w+,\s*(\w+),\s*(\w+)\)", src)}
    assert len(want) == 38
    assert sorted(set(want) - have) == []


def test_jni_shim_calls_only_declared_functions(fs):
    import re

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = open(os.path.join(root, "fairsim-vigor_gb300", "jni", "fsim_jni.cpp")).read()
    declared = set(fs.native.header_functions())
    used = set(re.findall(r"\b(fsim_\w+)\(", src))
    assert used and used <= declared, sorted(used - declared)
