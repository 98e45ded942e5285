"""ctypes binding of ``lib/libfairsim_gb300.so`` (the C ABI declared in include/fairsim_gb300.h).

The library is the product: every call here runs native code. There is no Python or CPU
fallback; a missing library or a failing CUDA call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libfairsim_gb300.so")
HEADER = os.path.join(_HERE, "..", "include", "fairsim_gb300.h")

FSIM_OK, FSIM_EINVAL, FSIM_EOOM, FSIM_ECUDA, FSIM_ETIMEOUT, FSIM_EBUSY, FSIM_ENOTFOUND, FSIM_ENODEV = 0, -1, -2, -3, -4, -5, -6, -7
PATH_OFFLINE, PATH_LIVE = 0, 1
INPUT_F32, INPUT_U16 = 0, 1
MAXD, MAXB, MAXP = 8, 4, 16


class FsimError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("fsim error %d: %s" % (code, msg))
        self.code = code


# Status codes map to exception types the way the reference's JNI layer maps failures to
# Java exceptions: bad sizes/arguments -> IllegalArgument/RuntimeException (Vec.failSize),
# allocation failure -> OutOfMemoryError (AccelVectorCplx.java:51-54).
class FsimInvalidArgument(FsimError, ValueError):
    pass


class FsimOutOfMemory(FsimError, MemoryError):
    pass


class FsimTimeout(FsimError, TimeoutError):
    pass


class FsimBusy(FsimError):
    pass


class FsimNotFound(FsimError, KeyError):
    pass


_ERRORS = {-1: FsimInvalidArgument, -2: FsimOutOfMemory, -4: FsimTimeout, -5: FsimBusy, -6: FsimNotFound}


class SimParamC(C.Structure):
    _fields_ = [
        ("w", C.c_int32),
        ("nr_dirs", C.c_int32),
        ("nr_bands", C.c_int32),
        ("nr_phases", C.c_int32),
        ("microns_per_pixel", C.c_double),
        ("na", C.c_double),
        ("em_wavelength", C.c_double),
        ("otf_a", C.c_double),
        ("use_attenuation", C.c_int32),
        ("att_strength", C.c_double),
        ("att_fwhm", C.c_double),
        ("wiener", C.c_double),
        ("apo_cutoff", C.c_double),
        ("apo_bend", C.c_double),
        ("px", C.c_double * MAXD),
        ("py", C.c_double * MAXD),
        ("pha_off", C.c_double * MAXD),
        ("modulation", (C.c_double * MAXB) * MAXD),
        ("has_phases", C.c_int32),
        ("phases", (C.c_double * MAXP) * MAXD),
        ("filter_style", C.c_int32),
        ("rl_iterations", C.c_int32),
        ("otf_data", C.c_void_p),
        ("otf_bands", C.c_int32),
        ("otf_samples", C.c_int32),
        ("otf_cycles", C.c_double),
    ]


class Job(C.Structure):
    _fields_ = [("plan", C.c_void_p), ("raw", C.c_void_p), ("out", C.c_void_p), ("widefield", C.c_void_p),
                ("filtered_widefield", C.c_void_p)]


HostJob = Job  # fsim_host_job: same four pointer fields, host addresses


class ServeConfig(C.Structure):
    _fields_ = [
        ("max_batch", C.c_int32),
        ("max_inflight", C.c_int32),
        ("streams", C.c_int32),
        ("refit_every", C.c_int32),
        ("input_type", C.c_int32),
        ("fade_px", C.c_int32),
        ("hbm_budget_bytes", C.c_size_t),
    ]


class ServeStats(C.Structure):
    _fields_ = [
        ("submitted", C.c_uint64),
        ("completed", C.c_uint64),
        ("rejected", C.c_uint64),
        ("refits", C.c_uint64),
        ("p50_ms", C.c_double),
        ("p99_ms", C.c_double),
        ("mean_ms", C.c_double),
        ("max_ms", C.c_double),
        ("recon_per_s", C.c_double),
        ("wall_s", C.c_double),
        ("cancelled", C.c_uint64),
    ]


MAX_CHANNELS = 8
LIVESIM_HEADER_BYTES = 128


class LiveSimHeader(C.Structure):
    _fields_ = [("seq_nr", C.c_int64), ("payload_offset", C.c_int32), ("payload_len", C.c_int32),
                ("version", C.c_int32), ("bytes_per_pixel", C.c_int32), ("width", C.c_int32),
                ("height", C.c_int32), ("pos_a", C.c_int32), ("pos_b", C.c_int32), ("pos0", C.c_int32),
                ("pos1", C.c_int32), ("pos2", C.c_int32), ("time_camera", C.c_int64),
                ("time_capture", C.c_int64), ("time_record", C.c_int64)]


class SeqxConfig(C.Structure):
    _fields_ = [("n_channels", C.c_int32), ("channel_numbers", C.c_int32 * MAX_CHANNELS),
                ("raws_per_recon", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
                ("sync_mode", C.c_int32), ("sync_frame_freq", C.c_int32), ("sync_frame_avr", C.c_int32),
                ("sync_frame_delay", C.c_int64), ("raw_queue", C.c_int32), ("sim_queue", C.c_int32)]


class SeqxStats(C.Structure):
    _fields_ = [("frames", C.c_uint64), ("bytes", C.c_uint64), ("unknown_channel", C.c_uint64),
                ("missed_raw", C.c_uint64 * MAX_CHANNELS), ("missed_sim", C.c_uint64 * MAX_CHANNELS),
                ("sync_frames", C.c_uint64 * MAX_CHANNELS), ("resyncs", C.c_uint64 * MAX_CHANNELS),
                ("duplicates", C.c_uint64 * MAX_CHANNELS), ("sequences", C.c_uint64)]


def to_c_param(p) -> SimParamC:
    """SimParam mirror (or dict) -> the C record."""
    g = (lambda k: p[k]) if isinstance(p, dict) else (lambda k: getattr(p, k))
    otf = None if isinstance(p, dict) else p.otf()
    c = SimParamC()
    m = getattr(otf, "measured", None) if otf is not None else None
    if m is not None:  # measured OTF bands (OtfProvider.loadFromConfig with data)
        arr = np.ascontiguousarray([[(z.real, z.imag) for z in band] for band in m["bands"]], dtype=np.float32)
        c._keep = arr  # the record points into it; it lives as long as the record
        c.otf_data = arr.ctypes.data
        c.otf_bands, c.otf_samples = arr.shape[0], arr.shape[1]
        c.otf_cycles = float(m["cycles"])
    c.w = g("w")
    c.nr_dirs, c.nr_bands, c.nr_phases = g("nrDirs"), g("nrBands"), g("nrPhases")
    c.microns_per_pixel = g("micronsPerPixel")
    c.na, c.em_wavelength, c.otf_a = g("na"), g("emWavelength"), g("otfA")
    c.use_attenuation = int(g("useAttenuation"))
    c.att_strength, c.att_fwhm = g("attStrength"), g("attFWHM")
    c.wiener, c.apo_cutoff, c.apo_bend = g("wiener"), g("apoCutoff"), g("apoBend")
    if isinstance(p, dict):
        c.filter_style, c.rl_iterations = int(p.get("filterStyle", 0)), int(p.get("rlIterations", 5))
    else:
        c.filter_style, c.rl_iterations = int(getattr(p, "filterStyle", 0)), int(getattr(p, "rlIterations", 5))
    for d in range(c.nr_dirs):
        c.px[d], c.py[d], c.pha_off[d] = g("pX")[d], g("pY")[d], g("phaOff")[d]
        for b in range(c.nr_bands):
            c.modulation[d][b] = g("modulations")[d][b]
    ph = g("phases")
    if ph is not None:
        c.has_phases = 1
        for d in range(c.nr_dirs):
            for i in range(c.nr_phases):
                c.phases[d][i] = ph[d][i]
    return c


def from_c_param(c: SimParamC) -> dict:
    n = c.nr_dirs
    return dict(pX=[c.px[d] for d in range(n)], pY=[c.py[d] for d in range(n)],
                phaOff=[c.pha_off[d] for d in range(n)],
                modulations=[[c.modulation[d][b] for b in range(c.nr_bands)] for d in range(n)])


_lib = None
VP, I32, F32, F64, PTR = C.c_void_p, C.c_int, C.c_float, C.c_double, C.c_void_p
_SIGS = {
    "fsim_last_error": (C.c_char_p, []),
    "fsim_init": (I32, [I32]),
    "fsim_sync": (I32, []),
    "fsim_version": (I32, []),
    "fsim_buffer_alloc": (I32, [C.c_size_t, I32, C.POINTER(VP)]),
    "fsim_buffer_free": (I32, [VP, I32]),
    "fsim_profiler": (I32, [I32]),
    "fsim_fft_plan_2d": (I32, [I32, I32, C.POINTER(C.c_int64)]),
    "fsim_vec_reshape": (I32, [VP, I32, I32]),
    "fsim_fft2d_batch": (I32, [VP, I32, I32, I32, I32, VP]),
    "fsim_vec_set_elem": (I32, [VP, C.c_size_t, C.c_float, C.c_float]),
    "fsim_vec_get_elem": (I32, [VP, C.c_size_t, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "fsim_set_stream": (I32, [VP]),
    "fsim_vec_create": (I32, [C.POINTER(VP), I32, I32, I32]),
    "fsim_vec_destroy": (I32, [VP]),
    "fsim_vec_info": (I32, [VP, C.POINTER(I32), C.POINTER(I32), C.POINTER(I32), C.POINTER(VP)]),
    "fsim_vec_upload": (I32, [VP, VP]),
    "fsim_vec_download": (I32, [VP, VP]),
    "fsim_vec_upload_u16": (I32, [VP, VP]),
    "fsim_vec_zero": (I32, [VP]),
    "fsim_vec_add": (I32, [VP, VP]),
    "fsim_vec_addconst": (I32, [VP, F32, F32]),
    "fsim_vec_axpy": (I32, [VP, F32, F32, VP]),
    "fsim_vec_times": (I32, [VP, VP, I32]),
    "fsim_vec_scal": (I32, [VP, F32, F32]),
    "fsim_vec_copy": (I32, [VP, VP]),
    "fsim_vec_reciproc": (I32, [VP]),
    "fsim_vec_norm2": (I32, [VP, C.POINTER(F64)]),
    "fsim_vec_sum": (I32, [VP, C.POINTER(F64), C.POINTER(F64)]),
    "fsim_vec_dot": (I32, [VP, VP, C.POINTER(F64), C.POINTER(F64)]),
    "fsim_vec_fft2d": (I32, [VP, I32]),
    "fsim_vec_fourier_shift": (I32, [VP, F64, F64]),
    "fsim_vec_paste_freq": (I32, [VP, VP, I32, I32]),
    "fsim_otf_to_vector": (I32, [VP, VP, I32, F64, F64, I32, I32]),
    "fsim_apo_vector": (I32, [VP, VP, F64, F64]),
    "fsim_attenuation_vector": (I32, [VP, VP, F64, F64, F64, F64]),
    "fsim_mask_otf": (I32, [VP, VP, F64, F64]),
    "fsim_wiener_denominator": (I32, [VP, VP, F64]),
    "fsim_separate_bands": (I32, [VP, I32, VP, I32, VP, I32, VP]),
    "fsim_separation_matrix": (I32, [VP, I32, I32, VP, VP]),
    "fsim_common_region": (I32, [VP, VP, VP, F64, F64, F64, F64, I32]),
    "fsim_locate_peak": (I32, [VP, F64, VP]),
    "fsim_fit_peak": (I32, [VP, VP, VP, F64, F64, F64, F64, VP, VP]),
    "fsim_get_peak": (I32, [VP, VP, VP, F64, F64, F64, VP]),
    "fsim_run_reconstruction": (I32, [VP, VP, VP, I32, I32]),
    "fsim_estimate_parameters": (I32, [VP, VP, I32, F64, VP]),
    "fsim_plan_create": (I32, [C.POINTER(VP), VP, I32, I32, I32, F64]),
    "fsim_plan_update": (I32, [VP, VP]),
    "fsim_plan_destroy": (I32, [VP]),
    "fsim_plan_workspace_bytes": (C.c_size_t, [VP]),
    "fsim_plan_filter_bytes": (C.c_size_t, [VP]),
    "fsim_plan_info": (I32, [VP, C.POINTER(I32), C.POINTER(I32), C.POINTER(I32)]),
    "fsim_plan_filter_table": (I32, [VP, VP, C.c_size_t, C.POINTER(I32)]),
    "fsim_device_status": (I32, [C.POINTER(I32), VP, I32]),
    "fsim_plan_set_clip_scale": (I32, [VP, I32]),
    "fsim_recon_batch": (I32, [VP, I32, VP, C.c_size_t, VP]),
    "fsim_recon_batch_host": (I32, [VP, I32, I32]),
    "fsim_batch_graph_create": (I32, [VP, VP, I32, VP, C.c_size_t, VP]),
    "fsim_batch_graph_launch": (I32, [VP, VP]),
    "fsim_batch_graph_info": (I32, [VP, VP, VP]),
    "fsim_batch_graph_destroy": (I32, [VP]),
    "fsim_recon_host": (I32, [VP, VP, VP]),
    "fsim_tune_set": (I32, [I32, I32, I32, I32]),
    "fsim_tune_get": (I32, [I32, I32, I32, C.POINTER(I32), C.POINTER(I32)]),
    "fsim_profile_enable": (I32, [I32]),
    "fsim_profile_read": (I32, [VP, I32, C.POINTER(I32)]),
    "fsim_estimate_raw": (I32, [VP, VP, I32, I32, I32, F64, VP]),
    "fsim_live_refit": (I32, [VP, VP, VP]),
    "fsim_corr_grid_noalloc": (I32, [VP, VP, I32, VP, I32, VP, I32, F64, VP, VP]),
    "fsim_serve_open": (I32, [C.POINTER(VP), VP, VP, I32]),
    "fsim_serve_submit": (I32, [VP, I32, VP, C.c_size_t, C.POINTER(C.c_uint64)]),
    "fsim_serve_cancel": (I32, [VP, C.c_uint64]),
    "fsim_debug_fail_alloc": (I32, [I32]),
    "fsim_debug_b2_staging": (I32, [I32, C.POINTER(I32)]),
    "fsim_serve_wait": (I32, [VP, C.c_uint64, VP, I32, C.POINTER(F64)]),
    "fsim_serve_stats_get": (I32, [VP, VP]),
    "fsim_serve_params": (I32, [VP, I32, VP]),
    "fsim_serve_capacity": (I32, [VP, I32, C.POINTER(I32), C.POINTER(I32)]),
    "fsim_serve_close": (I32, [VP]),
    "fsim_rl_deconvolve": (I32, [VP, VP, I32, I32]),
    "fsim_auto_correlation": (I32, [VP, F64, F64, C.POINTER(F64), C.POINTER(F64)]),
    "fsim_livesim_parse": (I32, [VP, I32, I32, VP]),
    "fsim_livesim_write": (I32, [VP, VP]),
    "fsim_seqx_create": (I32, [C.POINTER(VP), VP]),
    "fsim_seqx_push": (I32, [VP, VP, C.c_size_t]),
    "fsim_seqx_feed": (I32, [VP, VP, C.c_size_t]),
    "fsim_seqx_pop": (I32, [VP, VP, VP]),
    "fsim_seqx_stats_get": (I32, [VP, VP]),
    "fsim_seqx_reset": (I32, [VP]),
    "fsim_seqx_destroy": (I32, [VP]),
}


def header_functions():
    """Names of every function the public header declares."""
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fsim_[a-z0-9_]+)\s*\(", txt)))


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("native library missing: %s (run __graft_entry__.build())" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name, None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc):
    if rc != FSIM_OK:
        msg = lib().fsim_last_error()
        raise _ERRORS.get(rc, FsimError)(rc, msg.decode() if msg else "")
    return rc


_tuned = False


def apply_tuning(path=None):
    """Apply the autotuner's table (tuning.json) to the library (fsim_tune_set)."""
    import json

    global _tuned
    path = path or os.path.join(_HERE, "tuning.json")
    if not os.path.exists(path):
        return False
    with open(path) as f:
        t = json.load(f)
    for n, v in t.get("offline", {}).items():
        check(lib().fsim_tune_set(int(n), PATH_OFFLINE, 0, int(v["a"])))
        check(lib().fsim_tune_set(int(n), PATH_OFFLINE, 1, int(v["b"])))
        check(lib().fsim_tune_set(int(n), PATH_OFFLINE, 2, int(v.get("b2", v["b"]))))
    _tuned = True
    return True


_device = None


def init(device=None, apply_tuning=True):
    """Initialise the library on `device` (None: the device chosen before, else 0) and apply
    the autotuner's launch shapes once."""
    global _device
    if device is None:
        device = _device if _device is not None else 0
    check(lib().fsim_init(device))
    _device = device
    if apply_tuning and not _tuned:
        globals()["apply_tuning"]()
    return FSIM_OK
