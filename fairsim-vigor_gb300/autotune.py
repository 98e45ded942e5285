"""Autotuner for the fused reconstruction's launch shapes.

For every image size it times each variant of the row pass (elements per thread, i.e. the
radix plan and threads per line) and of the column passes (elements per thread x interleaved
columns per block) with the library's per-pass CUDA events on a batch of datasets larger
than L2, picks the fastest of each, and writes ``tuning.json`` next to this file.
``native.init()`` applies the table (fsim_tune_set). Variants change launch shapes only;
every variant computes the same reconstruction (covered by tests/test_gpu_fused.py).

Run on the GPU: ``python fairsim-vigor_gb300/autotune.py [sizes...]``.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TUNING = os.path.join(HERE, "tuning.json")


def _pkg():
    sys.path.insert(0, os.path.dirname(HERE))
    import __graft_entry__ as g

    return g.load_package()


def tune(sizes=(256, 384, 512, 768, 1024), reps=5, target_bytes=1 << 30, verbose=True):
    import torch

    fs = _pkg()
    N_ = fs.native
    N_.init(0, apply_tuning=False)
    lib = N_.lib()
    result = {}
    for n in sizes:
        sp = fs.synth.synthetic_params(n)
        plan = fs.plan.ReconPlan(sp, path=N_.PATH_OFFLINE, input_type=N_.INPUT_F32, fade_px=10)
        frame_bytes = 9 * n * n * 4
        B = int(max(4, min(128, target_bytes // frame_bytes)))
        raw = torch.rand((B, 9, n, n), device="cuda", dtype=torch.float32) * 500
        out = torch.empty((B, 2 * n, 2 * n), device="cuda", dtype=torch.float32)
        ws_bytes = fs.plan.batch_workspace_bytes([plan] * B)
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
        jobs = [(plan, raw[i].data_ptr(), out[i].data_ptr()) for i in range(B)]
        stream = torch.cuda.Stream()

        def measure():
            arr = (C.c_float * 8)()
            cnt = C.c_int()
            lib.fsim_profile_enable(1)
            ms = []
            with torch.cuda.stream(stream):
                for r in range(reps + 2):
                    fs.plan.recon_batch(jobs, ws.data_ptr(), ws_bytes, stream.cuda_stream)
                    N_.check(lib.fsim_profile_read(arr, 8, C.byref(cnt)))
                    if r >= 2:
                        ms.append([arr[i] for i in range(cnt.value)])
            lib.fsim_profile_enable(0)
            return np.median(np.array(ms), axis=0)

        na, nb = C.c_int(), C.c_int()
        v, cnt = C.c_int(), C.c_int()
        N_.check(lib.fsim_tune_get(n, N_.PATH_OFFLINE, 0, C.byref(v), C.byref(cnt)))
        nva = cnt.value
        N_.check(lib.fsim_tune_get(n, N_.PATH_OFFLINE, 1, C.byref(v), C.byref(cnt)))
        nvb = cnt.value
        a_ms, b_ms = [], []
        N_.check(lib.fsim_tune_set(n, N_.PATH_OFFLINE, 1, 0))
        for va in range(nva):
            N_.check(lib.fsim_tune_set(n, N_.PATH_OFFLINE, 0, va))
            a_ms.append(float(measure()[0]))
        best_a = int(np.argmin(a_ms))
        N_.check(lib.fsim_tune_set(n, N_.PATH_OFFLINE, 0, best_a))
        for vb in range(nvb):
            N_.check(lib.fsim_tune_set(n, N_.PATH_OFFLINE, 1, vb))
            m = measure()
            b_ms.append(float(sum(m[1:-1])))  # the column passes (G+B1, B2)
        best_b = int(np.argmin(b_ms))
        N_.check(lib.fsim_tune_set(n, N_.PATH_OFFLINE, 1, best_b))
        result[str(n)] = {"a": best_a, "b": best_b, "batch": B, "a_ms": a_ms, "b_ms": b_ms,
                          "us_per_dataset": float(sum(measure())) * 1000 / B}
        if verbose:
            print(n, result[str(n)], flush=True)
        del raw, out, ws
        plan.close()
    meta = {"device": torch.cuda.get_device_name(0), "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}
    with open(TUNING, "w") as f:
        json.dump({"meta": meta, "offline": result}, f, indent=1)
    return result


if __name__ == "__main__":
    sizes = [int(a) for a in sys.argv[1:]] or [256, 384, 512, 768, 1024]
    tune(sizes)
