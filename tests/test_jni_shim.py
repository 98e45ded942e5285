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
# the reference project's accel sources, when a checkout is at hand (FSIM_REFERENCE_ROOT)
REF_ACCEL = os.path.join(os.environ.get("FSIM_REFERENCE_ROOT", "/nonexistent"), "org", "fairsim", "accel")


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


@pytest.mark.skipif(not os.path.isdir(REF_ACCEL), reason="FSIM_REFERENCE_ROOT unset or without the accel sources")
def test_shim_exports_every_native_of_the_reference_accel_classes():
    files = [f for f in glob.glob(os.path.join(REF_ACCEL, "*.java")) if not os.path.basename(f).startswith("Test")]
    want = set()
    for f in files:
        want.update(native_methods(f, "org.fairsim.accel"))
    assert len(want) >= 30
    missing = sorted(want - exported_symbols())
    assert not missing, missing


JNI_OF = {"void": {"void"}, "boolean": {"jboolean"}, "byte": {"jbyte"}, "char": {"jchar"}, "short": {"jshort"},
          "int": {"jint"}, "long": {"jlong"}, "float": {"jfloat"}, "double": {"jdouble"}}


def jni_types_for(java_type):
    """JNI parameter / return types that match a Java type at the call boundary."""
    if java_type in JNI_OF:
        return JNI_OF[java_type]
    if java_type.endswith("[]"):
        base = java_type[:-2]
        if base in JNI_OF and base != "void" and not base.endswith("[]"):
            return {"j%sArray" % base, "jarray", "jobject"}
        return {"jobjectArray", "jarray", "jobject"}
    return {"jobject", "jarray", "jclass", "jstring"}  # a reference to any object


def java_natives_with_signatures(path, package):
    """{JNI name: (is_static, return type, [parameter types])} of a Java source file."""
    text = re.sub(r"/\*.*?\*/", "", open(path).read(), flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    names = native_methods(path, package)
    modifiers = {"static", "final", "synchronized", "public", "private", "protected"}
    decls = []
    for m in re.finditer(r"((?:\b\w+\s+)*)\bnative\b([^;{(]*)\(([^)]*)\)", text):
        toks = m.group(2).replace("[", " [").replace("]", "] ").split()
        mods = set(m.group(1).split()) | {t for t in toks if t in modifiers}
        rest = [t for t in toks if t not in modifiers]
        decls.append(("static" in mods, "".join(rest[:-1]), rest[-1], m.group(3)))
    out = {}
    for name, (static, ret, meth, params) in zip(names, decls):
        assert name.endswith("_" + meth)
        types = []
        for p in [q.strip() for q in params.split(",") if q.strip()]:
            toks = p.replace("[", " [").replace("]", "] ").split()
            toks = [t for t in toks if t != "final"][:-1]  # drop the parameter name
            types.append("".join(toks))
        out[name] = (static, ret, types)
    return out


def shim_signatures():
    """{JNI name: (return type, [parameter types])} of the shim's definitions."""
    src = open(SHIM).read()
    out = {}
    pat = r"\b(JFN|GFN)\(\s*(\w+)\s*,\s*(\w+)\s*(?:,\s*(\w+)\s*)?\)\s*\("
    for m in re.finditer(pat, src):
        kind, ret, a, b = m.groups()
        name = ("Java_org_fairsim_accel_%s_%s" % (a, b)) if kind == "JFN" else ("Java_org_fairsim_gb300_FusedSim_%s" % a)
        depth, i = 1, m.end()
        while depth:
            depth += {"(": 1, ")": -1}.get(src[i], 0)
            i += 1
        params = [q.strip() for q in src[m.end():i - 1].split(",")]
        out[name] = (ret, [q.replace("*", "* ").split()[0].replace(" ", "") for q in params])
    return out


def check_signatures(java):
    shim = shim_signatures()
    bad = []
    for name, (static, ret, ptypes) in java.items():
        got_ret, got = shim[name]
        if got_ret not in jni_types_for(ret):
            bad.append((name, "return", ret, got_ret))
        if len(got) != 2 + len(ptypes) or got[0] != "JNIEnv*":
            bad.append((name, "arity", ptypes, got))
            continue
        if got[1] not in ({"jclass", "jobject"} if static else {"jobject"}):
            bad.append((name, "receiver", "static" if static else "instance", got[1]))
        for jt, ct in zip(ptypes, got[2:]):
            if ct not in jni_types_for(jt):
                bad.append((name, jt, ct))
    return bad


def test_shim_signatures_match_its_wrapper():
    java = java_natives_with_signatures(WRAPPER, "org.fairsim.gb300")
    assert len(java) >= 7
    assert check_signatures(java) == []


@pytest.mark.skipif(not os.path.isdir(REF_ACCEL), reason="FSIM_REFERENCE_ROOT unset or without the accel sources")
def test_shim_signatures_match_the_reference_accel_classes():
    java = {}
    for f in glob.glob(os.path.join(REF_ACCEL, "*.java")):
        if not os.path.basename(f).startswith("Test"):
            java.update(java_natives_with_signatures(f, "org.fairsim.accel"))
    assert len(java) >= 30
    assert check_signatures(java) == []
