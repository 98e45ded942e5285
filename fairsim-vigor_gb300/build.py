"""Builds ``lib/libfairsim_gb300.so`` from ``csrc/`` with nvcc for sm_103a only.

One nvcc invocation per translation unit, run in parallel, then one shared-object link.
Objects go to ``_build/`` (git-ignored); the library goes to ``lib/`` (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libfairsim_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
# host code keeps Java's separate double roundings (no FMA contraction on aarch64 either)
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr",
          "-I" + os.path.join(HERE, "..", "include")]


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
                  + glob.glob(os.path.join(HERE, "..", "include", "*.h")))


def _compile(src, verbose=False, extra=()):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    newest_dep = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in _headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest_dep and not extra:
        return obj, ""
    cmd = [NVCC] + ARCH + COMMON + list(extra) + ["-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [NVCC] + COMMON + ["-x", "c++", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr[-6000:]))
    return obj, r.stderr


def build(verbose: bool = False, jobs: int | None = None, ptxas_info: bool = False) -> str:
    """FSIM_NVCC_FLAGS (environment) adds nvcc flags to every translation unit, e.g. the
    register budgets -DFSIM_PA_REGS=80 (every unit is then recompiled)."""
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = _sources()
    extra = (("-Xptxas", "-v") if ptxas_info else ()) + tuple(os.environ.get("FSIM_NVCC_FLAGS", "").split())
    jobs = jobs or min(len(srcs), max(2, os.cpu_count() or 2))
    objs, logs = [], []
    with cf.ThreadPoolExecutor(jobs) as ex:
        for obj, log in ex.map(lambda s: _compile(s, verbose, extra), srcs):
            objs.append(obj)
            logs.append(log)
    if verbose or ptxas_info:
        for l in logs:
            if l:
                sys.stderr.write(l)
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    return LIB


def find_jni_include():
    """Include folders of a JDK's jni.h (JAVA_HOME, then /usr/lib/jvm), or None."""
    cands = []
    if os.environ.get("JAVA_HOME"):
        cands.append(os.path.join(os.environ["JAVA_HOME"], "include"))
    cands += sorted(glob.glob("/usr/lib/jvm/*/include"))
    for inc in cands:
        if os.path.exists(os.path.join(inc, "jni.h")):
            return [inc] + [os.path.dirname(h) for h in glob.glob(os.path.join(inc, "*", "jni_md.h"))]
    return None


def build_jni(verbose: bool = False):
    """Builds lib/libfairsim_gb300_jni.so (jni/fsim_jni.cpp) when a JDK is installed; returns
    its path, or None without a jni.h (the C ABI library is complete without it)."""
    inc = find_jni_include()
    if not inc:
        return None
    lib = build(verbose)
    out = os.path.join(LIBDIR, "libfairsim_gb300_jni.so")
    cmd = (["g++", "-O2", "-std=c++17", "-shared", "-fPIC"] + ["-I" + i for i in inc]
           + [os.path.join(HERE, "jni", "fsim_jni.cpp"), "-L" + LIBDIR, "-lfairsim_gb300",
              "-Wl,-rpath,$ORIGIN", "-o", out])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("JNI shim build failed:\n" + r.stderr[-4000:])
    return out if lib else None


if __name__ == "__main__":
    import time

    t = time.time()
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
    print("built in %.1fs" % (time.time() - t))
