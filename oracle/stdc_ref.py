"""ctypes binding of the reference's own standard-C vector backend (accel/stdC_cplx.c and
accel/stdC_real.c, the JNI natives behind org/fairsim/accel/AccelVectorCplx.java:296-331 and
AccelVectorReal.java:218-247 when the accel factory runs on the CPU), compiled from the
reference checkout by ``make ref`` (oracle/Makefile) into oracle/_ref/libstdc_ref.so.

TEST INFRASTRUCTURE ONLY: it pins the oracle's vector operations, and through the committed
fixture tests/golden/stdc_vector_ops.npz the library's device kernels, to the reference's
code. The natives are called directly with a NULL JNIEnv; only those that never touch the
JNI environment are bound (element-wise ops, reductions, pasteFreq, fourierShift).

The reference checkout is located by FSIM_REFERENCE_ROOT; without it (or without a C
compiler) ``available()`` is False and the tests that need the live library skip."""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libstdc_ref.so")
_lib = None


def reference_root():
    return os.environ.get("FSIM_REFERENCE_ROOT", "")


def build() -> bool:
    """Builds oracle/_ref/libstdc_ref.so from the reference checkout; True when it exists."""
    root = reference_root()
    if root and os.path.isfile(os.path.join(root, "accel", "stdC_cplx.c")):
        r = subprocess.run(["make", "-C", HERE, "ref", "REFERENCE_ROOT=" + root], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("building the reference's stdC backend failed:\n" + r.stdout + r.stderr)
    return os.path.isfile(LIB)


def available() -> bool:
    try:
        return build()
    except (OSError, RuntimeError):
        return False


def lib():
    global _lib
    if _lib is None:
        if not build():
            raise RuntimeError("oracle/_ref/libstdc_ref.so is not built (FSIM_REFERENCE_ROOT unset?)")
        L = C.CDLL(LIB)
        V, P, I, F, D, B = None, C.c_int64, C.c_int32, C.c_float, C.c_double, C.c_uint8
        null = [C.c_void_p, C.c_void_p]  # JNIEnv*, jobject
        sig = {
            "Java_org_fairsim_accel_AccelVectorCplx_nativeAdd": (V, [P, P, I]),
            "Java_org_fairsim_accel_AccelVectorCplx_nativeAXPY": (V, [F, F, P, P, I]),
            "Java_org_fairsim_accel_AccelVectorCplx_nativeTIMES": (V, [P, P, I, B]),
            "Java_org_fairsim_accel_AccelVectorCplx_nativeTIMESREAL": (V, [P, P, I]),
            "Java_org_fairsim_accel_AccelVectorCplx_nativeScal": (V, [P, I, F, F]),
            "Java_org_fairsim_accel_AccelVectorCplx_nativeREDUCE": (D, [P, I, B]),
            "Java_org_fairsim_accel_AccelVectorCplx_nativeCOPYREAL": (V, [P, P, I]),
            "Java_org_fairsim_accel_AccelVectorCplx2d_nativePasteFreq": (V, [P, I, I, P, I, I, I, I]),
            "Java_org_fairsim_accel_AccelVectorCplx2d_nativeFourierShift": (V, [P, I, D, D]),
            "Java_org_fairsim_accel_AccelVectorReal_nativeAdd": (V, [P, P, I]),
            "Java_org_fairsim_accel_AccelVectorReal_nativeAXPY": (V, [F, P, P, I]),
            "Java_org_fairsim_accel_AccelVectorReal_nativeTIMES": (V, [P, P, I]),
            "Java_org_fairsim_accel_AccelVectorReal_nativeScal": (V, [P, I, F]),
            "Java_org_fairsim_accel_AccelVectorReal_nativeREDUCE": (D, [P, I, B]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = null + args
        _lib = L
    return _lib


def _p(a):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def _c(a):
    return np.ascontiguousarray(a, dtype=np.complex64).copy()


def _r(a):
    return np.ascontiguousarray(a, dtype=np.float32).copy()


def _f(name):
    return getattr(lib(), "Java_org_fairsim_accel_" + name)


# ---- complex vectors (AccelVectorCplx natives) ------------------------------------------
def cplx_add(y, x):
    y, x = _c(y), _c(x)
    _f("AccelVectorCplx_nativeAdd")(None, None, _p(y), _p(x), y.size)
    return y


def cplx_axpy(a, y, x):
    y, x = _c(y), _c(x)
    a = complex(a)
    _f("AccelVectorCplx_nativeAXPY")(None, None, a.real, a.imag, _p(y), _p(x), y.size)
    return y


def cplx_times(y, x, conj=False):
    y, x = _c(y), _c(x)
    _f("AccelVectorCplx_nativeTIMES")(None, None, _p(y), _p(x), y.size, 1 if conj else 0)
    return y


def cplx_times_real(y, r):
    y, r = _c(y), _r(r)
    _f("AccelVectorCplx_nativeTIMESREAL")(None, None, _p(y), _p(r), y.size)
    return y


def cplx_scal(y, a):
    y = _c(y)
    a = complex(a)
    _f("AccelVectorCplx_nativeScal")(None, None, _p(y), y.size, a.real, a.imag)
    return y


def cplx_norm2(y):
    y = _c(y)
    return _f("AccelVectorCplx_nativeREDUCE")(None, None, _p(y), y.size, 1)


def cplx_from_real(r):
    r = _r(r)
    y = np.zeros(r.shape, np.complex64)
    _f("AccelVectorCplx_nativeCOPYREAL")(None, None, _p(y), _p(r), y.size)
    return y


def paste_freq(z, wo, ho, xoff=0, yoff=0):
    """nativePasteFreq: z (hi x wi) placed into a zeroed ho x wo spectrum."""
    z = _c(z)
    hi, wi = z.shape
    out = np.empty((ho, wo), np.complex64)
    _f("AccelVectorCplx2d_nativePasteFreq")(None, None, _p(out), wo, ho, _p(z), wi, hi, xoff, yoff)
    return out


def fourier_shift(z, kx, ky):
    """nativeFourierShift: z (N x N) times exp(i 2 pi (kx x + ky y)/N)."""
    z = _c(z)
    _f("AccelVectorCplx2d_nativeFourierShift")(None, None, _p(z), z.shape[0], float(kx), float(ky))
    return z


# ---- real vectors (AccelVectorReal natives) ---------------------------------------------
def real_add(y, x):
    y, x = _r(y), _r(x)
    _f("AccelVectorReal_nativeAdd")(None, None, _p(y), _p(x), y.size)
    return y


def real_axpy(a, y, x):
    y, x = _r(y), _r(x)
    _f("AccelVectorReal_nativeAXPY")(None, None, float(a), _p(y), _p(x), y.size)
    return y


def real_times(y, x):
    y, x = _r(y), _r(x)
    _f("AccelVectorReal_nativeTIMES")(None, None, _p(y), _p(x), y.size)
    return y


def real_scal(y, a):
    y = _r(y)
    _f("AccelVectorReal_nativeScal")(None, None, _p(y), y.size, float(a))
    return y


def real_reduce(y, sqr):
    y = _r(y)
    return _f("AccelVectorReal_nativeREDUCE")(None, None, _p(y), y.size, 1 if sqr else 0)
