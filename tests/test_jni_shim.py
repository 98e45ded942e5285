"""The JNI shim (fairsim-vigor_gb300/jni/fsim_jni.cpp) on a machine without a JDK:
  * it type-checks against the JNI declarations of tests/jni_stub/jni.h (g++ -fsyntax-only);
  * it exports a function for every native method of the Java wrapper it ships
    (org/fairsim/gb300/FusedSim.java) and, where the reference's sources are present, for
    every native method of the reference's accel classes (org/fairsim/accel/*.java), under
    the Java_<package>_<class>_<method> names the JVM looks up, so that those classes load
    the library unchanged."""
import glob
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SHIM = os.path.join(ROOT, "fairsim-vigor_gb300", "jni", "fsim_jni.cpp")
WRAPPER = os.path.join(ROOT, "fairsim-vigor_gb300", "jni", "org", "fairsim", "gb300", "FusedSim.java")
REF_ACCEL = "/root/reference/org/fairsim/accel"


def exported_symbols():
    """Java_* names the shim defines, with its JFN / GFN macros expanded."""
    src = open(SHIM).read()
    names = set(re.findall(r"\bJava_\w+", src))
    for cls, meth in re.findall(r"\bJFN\(\s*\w+\s*,\s*(\w+)\s*,\s*(\w+)\s*\)", src):
        names.add("Java_org_fairsim_accel_%s_%s" % (cls, meth))
    for meth in re.findall(r"\bGFN\(\s*\w+\s*,\s*(\w+)\s*\)", src):
        names.add("Java_org_fairsim_gb300_FusedSim_%s" % meth)
    return names


def native_methods(path, package):
    """JNI names of the native methods declared in a Java source file: the owner is the
    innermost class whose body holds the declaration (nested classes joined with the
    JNI encoding of '$', _00024)."""
    text = re.sub(r"/\*.*?\*/", "", open(path).read(), flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    text = re.sub(r'"(?:\\.|[^"\\])*"', '""', text)
    spans = []
    for m in re.finditer(r"\bclass\s+(\w+)", text):
        open_at = text.index("{", m.end())
        depth, i = 0, open_at
        while True:
            depth += {"{": 1, "}": -1}.get(text[i], 0)
            if depth == 0:
                break
            i += 1
        spans.append((open_at, i, m.group(1)))
    out = []
    for m in re.finditer(r"\bnative\b[^;{(]*?\b(\w+)\s*\(", text):
        chain = [name for lo, hi, name in sorted(spans) if lo < m.start() < hi]
        if chain:
            out.append("Java_%s_%s_%s" % (package.replace(".", "_"), "_00024".join(chain), m.group(1)))
    return out


@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_shim_type_checks_against_jni_declarations():
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-Werror",
                        "-I", os.path.join(HERE, "jni_stub"), SHIM], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_shim_exports_every_native_of_its_wrapper():
    want = native_methods(WRAPPER, "org.fairsim.gb300")
    assert len(want) >= 7
    missing = sorted(set(want) - exported_symbols())
    assert not missing, missing


@pytest.mark.skipif(not os.path.isdir(REF_ACCEL), reason="reference sources not present")
def test_shim_exports_every_native_of_the_reference_accel_classes():
    files = [f for f in glob.glob(os.path.join(REF_ACCEL, "*.java")) if not os.path.basename(f).startswith("Test")]
    want = set()
    for f in files:
        want.update(native_methods(f, "org.fairsim.accel"))
    assert len(want) >= 30
    missing = sorted(want - exported_symbols())
    assert not missing, missing
