"""Writes jni_natives.txt: the JNI symbol of every `native` method the reference's accel Java
classes declare (org/fairsim/accel/*.java), which the shim (fairsim-vigor_gb300/jni/
fsim_jni.cpp) must export so that those classes load the GB300 library unchanged.
Run where the reference source is present: python tests/golden/make_jni_natives.py REF_ROOT
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    accel = os.path.join(ref_root, "org", "fairsim", "accel")
    syms = set()
    for fn in sorted(os.listdir(accel)):
        if not fn.endswith(".java"):
            continue
        src = open(os.path.join(accel, fn)).read()
        src = re.sub(r"//[^\n]*", "", src)
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        # class bodies as brace ranges; a method belongs to the innermost class around it
        # (nested classes appear in JNI names as Outer_00024Inner)
        spans = []
        for m in re.finditer(r"\bclass\s+(\w+)[^{]*\{", src):
            depth, i = 1, m.end()
            while depth and i < len(src):
                depth += {"{": 1, "}": -1}.get(src[i], 0)
                i += 1
            spans.append((m.start(), i, m.group(1)))
        for m in re.finditer(r"\bnative\b[^;(]*?\b(\w+)\s*\(", src):
            chain = [c for a, b, c in spans if a < m.start() < b]
            syms.add("Java_org_fairsim_accel_%s_%s" % ("_00024".join(chain), m.group(1)))
    with open(os.path.join(HERE, "jni_natives.txt"), "w") as f:
        f.write("\n".join(sorted(syms)) + "\n")
    return sorted(syms)


if __name__ == "__main__":
    print("\n".join(main(sys.argv[1] if len(sys.argv) > 1 else ".")))
