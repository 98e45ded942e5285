"""Fused, batched reconstruction plans (C ABI: fsim_plan_* / fsim_recon_batch) and the
served form (fsim_serve_*), which replaces ``ReconstructionRunner``
(org/fairsim/livemode/ReconstructionRunner.java:140-593) with continuous batching.

A plan holds one parameter set's resident filters (separation coefficients, shift ramps,
OTF masks, Wiener x apodization, border damping). ``PATH_OFFLINE`` reproduces
``SimAlgorithm.runReconstruction`` with the GUI's input preparation (background clip,
``fadeBorderCos``, FFT); ``PATH_LIVE`` reproduces the live ``ReconstructionThread``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native as N


class ReconPlan:
    def __init__(self, sp, path=N.PATH_OFFLINE, input_type=N.INPUT_F32, fade_px=10, bgr=0.0):
        self.sp = sp
        self.path, self.input_type = path, input_type
        h = C.c_void_p()
        self._c = N.to_c_param(sp)
        if N._device is None:
            # the library checks the arguments before it touches a device: malformed
            # parameters raise ValueError even on a host without a GPU
            N.check(N.lib().fsim_plan_create(C.byref(h), C.byref(self._c), int(path), int(input_type), int(fade_px),
                                             float(bgr)))
            self._h = h
            N.init()
        else:
            N.init()
            N.check(N.lib().fsim_plan_create(C.byref(h), C.byref(self._c), int(path), int(input_type), int(fade_px),
                                             float(bgr)))
            self._h = h

    @property
    def handle(self):
        return self._h

    @property
    def w(self):
        return self.sp.w

    def update(self, sp):
        self.sp = sp
        self._c = N.to_c_param(sp)
        N.check(N.lib().fsim_plan_update(self._h, C.byref(self._c)))

    def setClipScale(self, clip_scale: int):
        """Output scaling of the reconstruction, SimParam.CLIPSCALE ordinal: 0 NONE (default),
        1 CLIP, 2 BOTH (scaled to 255 at the maximum, then clipped; SimUtils.clipAndScale)."""
        N.check(N.lib().fsim_plan_set_clip_scale(self._h, int(clip_scale)))
        return self

    def workspace_bytes(self) -> int:
        return int(N.lib().fsim_plan_workspace_bytes(self._h))

    def filter_bytes(self) -> int:
        return int(N.lib().fsim_plan_filter_bytes(self._h))

    def filter_table(self) -> np.ndarray:
        """The resident Wiener x apodization table: 2w rows of w + 1 columns (offline, the
        Hermitian half) or 2w (live), in the reference's vector layout."""
        W = 2 * self.sp.imgSize
        nc = W if self.path == N.PATH_LIVE else W // 2 + 1
        out = np.zeros((W, nc), np.float32)
        got = C.c_int()
        N.check(N.lib().fsim_plan_filter_table(self._h, out.ctypes.data_as(C.c_void_p), out.size, C.byref(got)))
        assert got.value == nc
        return out

    def raw_dtype(self):
        return np.uint16 if self.input_type == N.INPUT_U16 else np.float32

    def reconstruct_host(self, raw) -> np.ndarray:
        """Host buffers in and out: H2D copy, fused reconstruction, D2H copy."""
        raw = np.ascontiguousarray(raw, dtype=self.raw_dtype())
        n = self.sp.w
        if raw.size != self.sp.nrDirs * self.sp.nrPhases * n * n:
            raise ValueError("raw stack size mismatch")
        out = np.empty((2 * n, 2 * n), dtype=np.float32)
        N.check(N.lib().fsim_recon_host(self._h, raw.ctypes.data_as(C.c_void_p), out.ctypes.data_as(C.c_void_p)))
        return out

    def reconstruct_host_widefield(self, raw):
        """The reconstruction with its widefield side outputs, host buffers in and out.
        Offline plans: (image, widefield, filtered widefield), each 2w x 2w, as
        runReconstruction's "Widefield" and "filtered Widefield" (SimAlgorithm.java:533-576);
        live plans: (image, w x w widefield)."""
        raw = np.ascontiguousarray(raw, dtype=self.raw_dtype())
        n = self.sp.w
        if raw.size != self.sp.nrDirs * self.sp.nrPhases * n * n:
            raise ValueError("raw stack size mismatch")
        out = np.empty((2 * n, 2 * n), dtype=np.float32)
        ptr = lambda a: a.ctypes.data  # noqa: E731
        if self.path == N.PATH_LIVE:
            wf = np.empty((n, n), dtype=np.float32)
            recon_batch_host([(self, ptr(raw), ptr(out), ptr(wf))])
            return out, wf
        wf = np.empty((2 * n, 2 * n), dtype=np.float32)
        fwf = np.empty((2 * n, 2 * n), dtype=np.float32)
        recon_batch_host([(self, ptr(raw), ptr(out), ptr(wf), ptr(fwf))])
        return out, wf, fwf

    def close(self):
        if getattr(self, "_h", None):
            N.lib().fsim_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_workspace_bytes(plans) -> int:
    # the library keeps one internal job descriptor (< 256 bytes) per job at the head
    job_table = (len(plans) * 256 + 255) // 256 * 256
    return job_table + sum((p.workspace_bytes() + 255) // 256 * 256 for p in plans)


def _job_array(jobs):
    jobs = list(jobs)
    arr = (N.Job * len(jobs))()
    for i, j in enumerate(jobs):
        arr[i].plan = j[0].handle
        arr[i].raw = j[1]
        arr[i].out = j[2]
        arr[i].widefield = j[3] if len(j) > 3 else None
        arr[i].filtered_widefield = j[4] if len(j) > 4 else None
    return arr


def recon_batch(jobs, workspace_ptr: int, workspace_bytes: int, stream_ptr: int = 0):
    """jobs: iterable of (plan, raw_device_ptr, out_device_ptr[, widefield_device_ptr
    [, filtered_widefield_device_ptr]]). The widefield is w x w on live plans and 2w x 2w on
    offline plans; the filtered widefield (2w x 2w) exists on offline plans only."""
    arr = _job_array(jobs)
    N.check(N.lib().fsim_recon_batch(arr, len(arr), C.c_void_p(workspace_ptr), C.c_size_t(workspace_bytes),
                                     C.c_void_p(stream_ptr) if stream_ptr else None))


def recon_batch_host(jobs, chunk: int = 0):
    """Host-buffer batch (fsim_recon_batch_host): jobs is an iterable of
    (plan, raw_host_ptr, out_host_ptr[, widefield_host_ptr[, filtered_widefield_host_ptr]]),
    sized as in ``recon_batch``; uploads, passes and downloads
    of successive chunks overlap, and the call returns when every output is on the host."""
    arr = _job_array(jobs)
    N.check(N.lib().fsim_recon_batch_host(arr, len(arr), int(chunk)))


class BatchGraph:
    """A fixed batch recorded once as a CUDA graph (fsim_batch_graph_*); ``launch()``
    replays the job-table copy and every size class's passes in one call."""

    def __init__(self, jobs, workspace_ptr: int, workspace_bytes: int, stream_ptr: int = 0):
        arr = _job_array(jobs)
        h = C.c_void_p()
        N.check(N.lib().fsim_batch_graph_create(C.byref(h), arr, len(arr), C.c_void_p(workspace_ptr),
                                                C.c_size_t(workspace_bytes),
                                                C.c_void_p(stream_ptr) if stream_ptr else None))
        self._h = h

    def launch(self, stream_ptr: int = 0):
        N.check(N.lib().fsim_batch_graph_launch(self._h, C.c_void_p(stream_ptr) if stream_ptr else None))

    def info(self):
        nj, nk = C.c_int(), C.c_int()
        N.check(N.lib().fsim_batch_graph_info(self._h, C.byref(nj), C.byref(nk)))
        return {"jobs": nj.value, "kernels": nk.value}

    def close(self):
        if getattr(self, "_h", None):
            N.lib().fsim_batch_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching live reconstruction over several channels (fsim_serve_*)."""

    def __init__(self, channel_params, max_batch=16, max_inflight=64, streams=3, refit_every=50,
                 input_type=N.INPUT_U16, fade_px=10, hbm_budget_bytes=8 << 30):
        N.init()
        cfg = N.ServeConfig(max_batch, max_inflight, streams, refit_every, input_type, fade_px, hbm_budget_bytes)
        self.params = list(channel_params)
        arr = (N.SimParamC * len(self.params))()
        for i, p in enumerate(self.params):
            arr[i] = N.to_c_param(p)
        h = C.c_void_p()
        N.check(N.lib().fsim_serve_open(C.byref(h), C.byref(cfg), arr, len(self.params)))
        self._h = h
        self.input_type = input_type

    def submit(self, channel: int, raw) -> int:
        raw = np.ascontiguousarray(raw, dtype=np.uint16 if self.input_type == N.INPUT_U16 else np.float32)
        t = C.c_uint64()
        N.check(N.lib().fsim_serve_submit(self._h, int(channel), raw.ctypes.data_as(C.c_void_p), raw.nbytes,
                                          C.byref(t)))
        return t.value

    def try_submit(self, channel: int, raw):
        """submit(), or None when admission refuses the stack (FSIM_EBUSY)."""
        raw = np.ascontiguousarray(raw, dtype=np.uint16 if self.input_type == N.INPUT_U16 else np.float32)
        t = C.c_uint64()
        rc = N.lib().fsim_serve_submit(self._h, int(channel), raw.ctypes.data_as(C.c_void_p), raw.nbytes, C.byref(t))
        if rc == N.FSIM_EBUSY:
            return None
        N.check(rc)
        return t.value

    def cancel(self, ticket: int):
        N.check(N.lib().fsim_serve_cancel(self._h, C.c_uint64(ticket)))

    def wait(self, ticket: int, out=None, timeout_ms=10000):
        n = None
        lat = C.c_double()
        if out is None:
            raise ValueError("out buffer required")
        N.check(N.lib().fsim_serve_wait(self._h, C.c_uint64(ticket), out.ctypes.data_as(C.c_void_p), int(timeout_ms),
                                        C.byref(lat)))
        return lat.value

    def stats(self) -> dict:
        s = N.ServeStats()
        N.check(N.lib().fsim_serve_stats_get(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in N.ServeStats._fields_}

    def capacity(self, ch: int) -> dict:
        """Slots of the channel's size class: allocated, and free now."""
        tot, free = C.c_int(), C.c_int()
        N.check(N.lib().fsim_serve_capacity(self._h, int(ch), C.byref(tot), C.byref(free)))
        return {"slots": tot.value, "free": free.value}

    def channel_params(self, ch: int) -> dict:
        c = N.SimParamC()
        N.check(N.lib().fsim_serve_params(self._h, int(ch), C.byref(c)))
        return N.from_c_param(c)

    def close(self):
        if getattr(self, "_h", None):
            N.check(N.lib().fsim_serve_close(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
