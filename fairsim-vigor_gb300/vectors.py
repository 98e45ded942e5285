"""The Vector API over device memory: the GB300 counterpart of the reference's
``AccelVectorFactory`` / ``AccelVectorReal2d`` / ``AccelVectorCplx2d``
(org/fairsim/accel/AccelVectorFactory.java:31-149, AccelVectorCplx.java:29-496,
AccelVectorReal.java:28-342) behind the ``VectorFactory`` seam
(org/fairsim/linalg/VectorFactory.java:28-171).

Method names and argument meaning follow ``Vec2d.Real`` / ``Vec2d.Cplx``
(org/fairsim/linalg/Vec2d.java:115-221). Data lives on the device; ``vectorData()`` copies
it to a host numpy array (the reference's readyBuffer), ``setData()`` copies back
(syncBuffer). Size mismatches raise like ``Vec.failSize``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native as N


def _vp(a):
    return a.ctypes.data_as(C.c_void_p)


class _Vec2d:
    is_complex = False

    def __init__(self, w: int, h: int):
        N.init()
        h_ = C.c_void_p()
        N.check(N.lib().fsim_vec_create(C.byref(h_), int(w), int(h), int(self.is_complex)))
        self._h = h_
        self.w, self.h = int(w), int(h)

    # -- lifetime --
    def close(self):
        if getattr(self, "_h", None):
            N.lib().fsim_vec_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def device_ptr(self) -> int:
        p = C.c_void_p()
        N.check(N.lib().fsim_vec_info(self._h, None, None, None, C.byref(p)))
        return p.value

    # -- Vec2d.Size --
    def vectorWidth(self):
        return self.w

    def vectorHeight(self):
        return self.h

    def vectorSize(self):
        return self.w * self.h

    def _fail_size(self, *others):
        for o in others:
            if o.w * o.h != self.w * self.h:
                raise ValueError("Vector size mismatch %d != %d" % (self.w * self.h, o.w * o.h))

    # -- element-wise ops (AccelVectorCplx.java:150-291) --
    def zero(self):
        N.check(N.lib().fsim_vec_zero(self._h))

    def add(self, *vs):
        for v in vs:
            self._fail_size(v)
            N.check(N.lib().fsim_vec_add(self._h, v._h))

    def times(self, v):
        self._fail_size(v)
        N.check(N.lib().fsim_vec_times(self._h, v._h, 0))

    def norm2(self) -> float:
        r = C.c_double()
        N.check(N.lib().fsim_vec_norm2(self._h, C.byref(r)))
        return r.value

    def reciproc(self):
        N.check(N.lib().fsim_vec_reciproc(self._h))

    def syncConcurrent(self):
        N.check(N.lib().fsim_sync())


class Vec2dReal(_Vec2d):
    is_complex = False

    def duplicate(self):
        r = Vec2dReal(self.w, self.h)
        r.copy(self)
        return r

    def copy(self, src):
        """copy(Vec.Real) or copy(Vec.Cplx): real part (AbstractVectorReal.java:90-106)."""
        self._fail_size(src)
        N.check(N.lib().fsim_vec_copy(self._h, src._h))

    def addConst(self, a: float):
        N.check(N.lib().fsim_vec_addconst(self._h, float(a), 0.0))

    def axpy(self, a: float, x):
        self._fail_size(x)
        N.check(N.lib().fsim_vec_axpy(self._h, float(a), 0.0, x._h))

    def scal(self, a: float):
        N.check(N.lib().fsim_vec_scal(self._h, float(a), 0.0))

    def sumElements(self) -> float:
        re, im = C.c_double(), C.c_double()
        N.check(N.lib().fsim_vec_sum(self._h, C.byref(re), C.byref(im)))
        return re.value

    def vectorData(self) -> np.ndarray:
        out = np.empty((self.h, self.w), dtype=np.float32)
        N.check(N.lib().fsim_vec_download(self._h, _vp(out)))
        return out

    def setData(self, a):
        a = np.ascontiguousarray(a, dtype=np.float32).reshape(self.h, self.w)
        N.check(N.lib().fsim_vec_upload(self._h, _vp(a)))

    def setFrom16bitPixels(self, a):
        a = np.ascontiguousarray(a, dtype=np.uint16).reshape(self.h, self.w)
        N.check(N.lib().fsim_vec_upload_u16(self._h, _vp(a)))


class Vec2dCplx(_Vec2d):
    is_complex = True

    def duplicate(self):
        r = Vec2dCplx(self.w, self.h)
        r.copy(self)
        return r

    def copy(self, src):
        """copy(Vec.Cplx) or copy(Vec.Real) with imaginary part 0."""
        self._fail_size(src)
        N.check(N.lib().fsim_vec_copy(self._h, src._h))

    def addConst(self, a):
        a = complex(a)
        N.check(N.lib().fsim_vec_addconst(self._h, a.real, a.imag))

    def axpy(self, a, x):
        self._fail_size(x)
        a = complex(a)
        N.check(N.lib().fsim_vec_axpy(self._h, a.real, a.imag, x._h))

    def timesConj(self, v):
        self._fail_size(v)
        N.check(N.lib().fsim_vec_times(self._h, v._h, 1))

    def scal(self, a):
        a = complex(a)
        N.check(N.lib().fsim_vec_scal(self._h, a.real, a.imag))

    def sumElements(self) -> complex:
        re, im = C.c_double(), C.c_double()
        N.check(N.lib().fsim_vec_sum(self._h, C.byref(re), C.byref(im)))
        return complex(re.value, im.value)

    def dot(self, y) -> complex:
        self._fail_size(y)
        re, im = C.c_double(), C.c_double()
        N.check(N.lib().fsim_vec_dot(self._h, y._h, C.byref(re), C.byref(im)))
        return complex(re.value, im.value)

    def fft2d(self, inverse: bool):
        N.check(N.lib().fsim_vec_fft2d(self._h, int(bool(inverse))))

    def fourierShift(self, kx: float, ky: float):
        N.check(N.lib().fsim_vec_fourier_shift(self._h, float(kx), float(ky)))

    def pasteFreq(self, src, xOffset: int = 0, yOffset: int = 0):
        N.check(N.lib().fsim_vec_paste_freq(self._h, src._h, int(xOffset), int(yOffset)))

    def vectorData(self) -> np.ndarray:
        out = np.empty((self.h, self.w), dtype=np.complex64)
        N.check(N.lib().fsim_vec_download(self._h, _vp(out)))
        return out

    def setData(self, a):
        a = np.ascontiguousarray(a, dtype=np.complex64).reshape(self.h, self.w)
        N.check(N.lib().fsim_vec_upload(self._h, _vp(a)))

    def setFrom16bitPixels(self, a):
        a = np.ascontiguousarray(a, dtype=np.uint16).reshape(self.h, self.w)
        N.check(N.lib().fsim_vec_upload_u16(self._h, _vp(a)))


class AccelVectorFactory:
    """``VectorFactory`` returning device-resident vectors (VectorFactory.java:31-169)."""

    _instance = None

    @classmethod
    def getFactory(cls):
        if cls._instance is None:
            cls._instance = cls()
        return cls._instance

    def createReal2D(self, w, h):
        return Vec2dReal(w, h)

    def createCplx2D(self, w, h):
        return Vec2dCplx(w, h)

    def createArrayReal2D(self, n, w, h):
        return [Vec2dReal(w, h) for _ in range(n)]

    def createArrayCplx2D(self, n, w, h):
        return [Vec2dCplx(w, h) for _ in range(n)]

    def syncConcurrent(self):
        N.check(N.lib().fsim_sync())


def handles(vs):
    arr = (C.c_void_p * len(vs))()
    for i, v in enumerate(vs):
        arr[i] = v.handle
    return arr
