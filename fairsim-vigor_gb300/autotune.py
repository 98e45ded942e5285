"""Autotuner for the fused reconstruction's launch shapes.

For every image size it times each variant of the row pass (elements per thread, i.e. the
radix plan and threads per line) and of each of the two column passes (elements per thread x
interleaved columns per block) with the library's per-pass CUDA events on a batch of datasets larger
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

        v, cnt = C.c_int(), C.c_int()
        counts = []
        for p in range(3):
            N_.check(lib.fsim_tune_get(n, N_.PATH_OFFLINE, p, C.byref(v), C.byref(cnt)))
            counts.append(cnt.value)
        for p in range(3):
            N_.check(lib.fsim_tune_set(n, N_.PATH_OFFLINE, p, 0))
        # one pass at a time, the others at their best so far; the per-pass CUDA events give
        # [A, G+B1, B2, C]
        timed_index = {0: 0, 1: 1, 2: 2}
        best, times = [], []
        for p in range(3):
            ms = []
            for var in range(counts[p]):
                N_.check(lib.fsim_tune_set(n, N_.PATH_OFFLINE, p, var))
                ms.append(float(measure()[timed_index[p]]))
            b = int(np.argmin(ms))
            N_.check(lib.fsim_tune_set(n, N_.PATH_OFFLINE, p, b))
            best.append(b)
            times.append(ms)
        result[str(n)] = {"a": best[0], "b": best[1], "b2": best[2], "batch": B, "a_ms": times[0],
                          "b1_ms": times[1], "b2_ms": times[2],
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
