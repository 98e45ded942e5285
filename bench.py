"""Benchmark of the fused, batched 2D SIM reconstruction on GB300.

Workload (one "step"): a batch of B independent 512x512 datasets, 3 angles x 3 phases
(float32 raw, seeded synthetic), reconstructed to 1024x1024 with known parameters,
Wiener 0.05, apodization cutoff 2.0 (SimAlgorithm.runReconstruction semantics with the
GUI's input preparation: fadeBorderCos(10), FFT). The raw batch (B * 9 MiB) is larger
than L2, so no flush is needed between steps.

  value      recon/s with inputs resident in HBM, device-timed (CUDA events on the launch stream)
  e2e        recon/s through the C ABI with host buffers (pinned H2D + batch + D2H every step)
  roofline   the dominant pass's algorithmic bytes / its event-timed duration vs measured HBM peak
  cpu_baseline  the oracle (CPU restatement of the reference's Java path), all host threads
  plain_gpu  the op-by-op device path (fsim_run_reconstruction, one dataset at a time)
  serve      live served form: Poisson arrivals, 3 channels, p50/p99 latency

`--impl reference` times the reference path's CPU implementation (the oracle port; the Java
reference cannot run here) on the same workload and prints the same JSON line.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SIM recon/s at 512² 3×3 batched+served vs plain GPU; p50/p99 live latency"
N = 512
NA, NP, NB = 3, 3, 2
WORKLOAD = "offline 2D SIM reconstruction, 512x512 x (3 angles x 3 phases) f32 -> 1024x1024, known params, wiener 0.05, apo cutoff 2.0, fade 10"


def load_package():
    import __graft_entry__ as g

    return g.load_package()


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self, wait_first_s=3.0):
        """Start sampling every 100 ms and wait for the first sample, so that the samples
        cover the region timed next."""
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.time()
            while not self.lines and time.time() - t0 < wait_first_s:
                time.sleep(0.02)
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_datasets(fs, n_distinct, seed0=1000):
    out = []
    for i in range(n_distinct):
        raw, truth = fs.synth.make_dataset(n=N, seed=seed0 + i)
        sp = fs.synth.sim_param_for(truth, N)
        out.append((raw, sp))
    return out


def cpu_recon_rate(fs, datasets, min_seconds=10.0, max_recons=40):
    """Oracle (CPU restatement of the reference Java path) with every host thread."""
    from oracle import refcpu

    cores = os.cpu_count() or 1
    refcpu.set_threads(cores)
    raw, sp = datasets[0]
    refcpu.recon_raw(sp, raw, fade=10)  # warm-up (thread pool, plans)
    t0 = time.perf_counter()
    n = 0
    while n < max_recons and (time.perf_counter() - t0 < min_seconds or n < 2):
        raw, sp = datasets[n % len(datasets)]
        refcpu.recon_raw(sp, raw, fade=10)
        n += 1
    dt = time.perf_counter() - t0
    return n / dt, cores, n, dt


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    fs = load_package()
    from oracle import refcpu

    refcpu.build()
    ds = make_datasets(fs, 2)
    cores = os.cpu_count() or 1
    refcpu.set_threads(cores)
    for i in range(args.warmup):
        raw, sp = ds[i % len(ds)]
        refcpu.recon_raw(sp, raw, fade=10)
    t0 = time.perf_counter()
    for i in range(args.steps):
        raw, sp = ds[i % len(ds)]
        refcpu.recon_raw(sp, raw, fade=10)
    dt = time.perf_counter() - t0
    v = args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "recon/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "batch": 1, "n": N,
                   "note": "each step is one dataset of the batched workload (bounded CPU sample)"},
        "cpu_baseline": {"value": v, "unit": "recon/s", "cores": cores, "kind": "port",
                         "sample": "%d reconstructions of 512x512 3x3 -> 1024x1024 (oracle, C++ restatement of the "
                                   "reference Java path; the Java reference and its JTransforms jar cannot run here)"
                                   % args.steps},
        "e2e": {"value": v, "unit": "recon/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# DRAM bytes (read + write) per dataset of each pass at 512^2 3x3, from single-kernel ncu
# captures (dram__bytes_read.sum + dram__bytes_write.sum; `ncu --set full -k regex:<pass>
# -s 2 -c 1` of `bench.py --batch 16 --steps 3 --warmup 3 --no-extras`, raw 151 MB, larger than
# L2); per-launch traffic = this x the batch size. G+B1 counts B1 (G moves 0.04 MB). Pass C is
# left out: at batch 16 its input, the Hermitian halves pass B2 has just written (67 MB), is
# still in L2, so the capture does not show its DRAM traffic at batch 64.
TRAFFIC_PER_DATASET = {"k_pass_a<512>": 15.99e6, "k_pass_g+k_pass_b1<512>": 11.21e6, "k_pass_b2<512>": 14.20e6,
                       "k_pass_c<512>": None}
PASS_NAMES = ["k_pass_a<512>", "k_pass_g+k_pass_b1<512>", "k_pass_b2<512>", "k_pass_c<512>"]


def pass_bytes(n=N, n_dirs=NA, n_phases=NP, n_bands=NB, na=1.4, lam=525.0, pxl=0.08):
    """Algorithmic bytes per dataset of the offline passes (each input read once, each output
    written once):
      A      raw frames in; row-transformed OTF-support windows I out (band 0 of all angles
             summed, once; each angle's pair neg components), plus one Nyquist term per row (D)
      G+B1   D in, one column per angle and pair out (G); I in, the column-transformed windows
             Tw (band 0, neg of every pair) and one Nyquist term per neg column (Dy) out
      B2     over the Hermitian half's columns 0..N: Tw (each neg window column once: at X for
             the neg component, at -X for the pos one; band 0 half a window), the OTF masks
             (a pair's neg and pos windows are mirror images, so together they cover one
             window's columns; band 0 half a window), the Wiener x apodization table, G, Dy
             in; the W x (N+1) Hermitian half out
      C      the Hermitian half in, the W x W image out"""
    npair = n_bands - 1
    W = 2 * n
    R = (2 * na / (lam / 1000.0)) / (1.0 / (n * pxl))
    nwin = min(W, ((2 * int(np.ceil(R)) + 6) // 4) * 4 + 4)
    I = (1 + n_dirs * npair) * nwin * n * 8  # band 0 summed over the angles in pass A
    D = n_dirs * npair * n * 8
    G = n_dirs * npair * nwin * 8
    Tw = (1 + n_dirs * npair) * nwin * nwin * 8
    Dy = n_dirs * npair * nwin * 8
    masks = (0.5 + n_dirs * npair) * nwin * nwin * 4
    OH = W * (n + 1) * 8
    a = n_dirs * n_phases * n * n * 4 + I + D
    b1 = D + G + I + Tw + Dy
    b2 = (0.5 + n_dirs * npair) * nwin * nwin * 8 + masks + (n + 1) * W * 4 + G + Dy + OH
    c = OH + W * W * 4
    return [a, b1, b2, c]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--distinct", type=int, default=16)
    ap.add_argument("--no-extras", action="store_true", help="skip plain-GPU, serve, mixed, large and CPU legs")
    ap.add_argument("--only", choices=["live", "fft", "estimate", "mixed", "large", "serve", "widefield", "ingest"],
                    help="run one extra leg alone and print its JSON (profiling of its kernels)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.only:
        return run_only(args)

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    fs = load_package()
    N_ = fs.native
    N_.init(local)

    B = args.batch
    datasets = make_datasets(fs, args.distinct, seed0=1000 + 97 * rank)
    plans = [fs.plan.ReconPlan(sp, path=N_.PATH_OFFLINE, input_type=N_.INPUT_F32, fade_px=10) for _, sp in datasets]
    job_plans = [plans[i % len(plans)] for i in range(B)]
    raw_host = torch.empty((B, NA * NP, N, N), dtype=torch.float32).pin_memory()
    for i in range(B):
        raw_host[i].copy_(torch.from_numpy(datasets[i % len(datasets)][0]))
    raw_dev = raw_host.cuda()
    out_dev = torch.empty((B, 2 * N, 2 * N), dtype=torch.float32, device="cuda")
    out_host = torch.empty((B, 2 * N, 2 * N), dtype=torch.float32).pin_memory()
    ws_bytes = fs.plan.batch_workspace_bytes(job_plans)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    sp_ = stream.cuda_stream
    jobs = [(job_plans[i], raw_dev[i].data_ptr(), out_dev[i].data_ptr()) for i in range(B)]
    graph = fs.plan.BatchGraph(jobs, ws.data_ptr(), ws_bytes, sp_)
    kernels_per_step = graph.info()["kernels"]

    def step():
        graph.launch(sp_)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def timed(fn, k):
        with torch.cuda.stream(stream):
            barrier()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(k):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            barrier()
            ms = e0.elapsed_time(e1)
        if world > 1:
            t = torch.tensor([ms], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    def wall(fn, k):
        """Host wall time of k calls that return with their results on the host."""
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(k):
            fn()
        torch.cuda.synchronize()
        barrier()
        ms = (time.perf_counter() - t0) * 1000.0
        if world > 1:
            t = torch.tensor([ms], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    clocks = ClockSampler(local)
    clocks.start()
    # ---- resident (device) throughput: the batch replayed as one CUDA graph ----
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ms = timed(step, args.steps)
    value = B * args.steps * world / (ms / 1000.0)

    # ---- end to end through the C ABI with host buffers: pinned raw in, pinned image out ----
    host_jobs = [(job_plans[i], raw_host[i].data_ptr(), out_host[i].data_ptr()) for i in range(B)]

    def e2e_step():
        fs.plan.recon_batch_host(host_jobs)

    for _ in range(2):
        e2e_step()
    e2e_steps = max(3, args.steps // 2)
    # three timed repetitions, the median reported: single wall-clock runs of the host path
    # occasionally lose half their rate to the host (measured on GB300: 6.7k and 7.6k
    # between neighbours at 13.3-13.7k)
    e2e_runs = sorted(wall(e2e_step, e2e_steps) for _ in range(3))
    e2e_ms = e2e_runs[1]
    e2e_value = B * e2e_steps * world / (e2e_ms / 1000.0)
    h2d = B * NA * NP * N * N * 4
    d2h = B * 4 * N * N * 4
    clk = clocks.stop()
    # the host link alone: one pinned upload of the raw batch and one download of the images
    with torch.cuda.stream(stream):
        raw_dev.copy_(raw_host, non_blocking=True)
        out_host.copy_(out_dev, non_blocking=True)
    h2d_ms = timed(lambda: raw_dev.copy_(raw_host, non_blocking=True), 2) / 2
    d2h_ms = timed(lambda: out_host.copy_(out_dev, non_blocking=True), 2) / 2

    # ---- per-pass timing (CUDA events between the passes of the direct batch call) ----
    import ctypes as C

    N_.check(N_.lib().fsim_profile_enable(1))
    pass_ms = []
    with torch.cuda.stream(stream):
        for _ in range(3):
            fs.plan.recon_batch(jobs, ws.data_ptr(), ws_bytes, sp_)
            arr = (C.c_float * 8)()
            n = C.c_int()
            N_.check(N_.lib().fsim_profile_read(arr, 8, C.byref(n)))
            pass_ms.append([arr[i] for i in range(n.value)])
    N_.check(N_.lib().fsim_profile_enable(0))
    pm = np.median(np.array(pass_ms), axis=0)
    algo = pass_bytes()
    names = PASS_NAMES
    dom = int(np.argmax(pm))
    peak, peak_kind = peaks()
    achieved = algo[dom] * B / (pm[dom] / 1000.0) / 1e9
    passes = {names[i]: {"ms": float(pm[i]), "algorithmic_MB_per_dataset": algo[i] / 1e6,
                         "GB_per_s": algo[i] * B / (pm[i] / 1000.0) / 1e9,
                         "frac_of_measured_hbm": algo[i] * B / (pm[i] / 1000.0) / 1e9 / peak}
              for i in range(len(pm))}
    traffic = TRAFFIC_PER_DATASET.get(names[dom])
    traffic = traffic * B if traffic else None

    extras = {}
    if rank == 0 and not args.no_extras:
        extras["plain_gpu"] = plain_gpu_leg(fs, datasets[0])
        extras["plain_gpu_rl_both"] = plain_gpu_leg(fs, datasets[0], k=3, style=3)
        extras["speedup_batched_vs_plain"] = value / extras["plain_gpu"]["value"]
        extras["speedup_e2e_vs_plain"] = e2e_value / extras["plain_gpu"]["value"]
        extras["fused_batch1"] = fused_batch1_leg(fs, datasets[0])
        extras["speedup_batched_vs_fused_batch1"] = value / extras["fused_batch1"]["value"]
        extras["speedup_e2e_vs_fused_batch1"] = e2e_value / extras["fused_batch1"]["value"]
        extras["serve"] = serve_leg(fs, seconds=3.0)
        extras["serve_saturated"] = serve_capacity_leg(fs)
        extras["serve_saturated"]["speedup_vs_plain"] = (extras["serve_saturated"]["recon_per_s"]
                                                         / extras["plain_gpu"]["value"])
        extras["mixed_batch"] = mixed_leg(fs, torch, stream, timed)
        extras["live_batch"] = live_leg(fs, torch, stream, timed)
        extras["widefield_outputs"] = widefield_leg(fs, torch, stream, timed)
        extras["livesim_ingest"] = ingest_leg(fs)
        extras["large_3x5_2048"] = large_leg(fs, torch, stream, timed)
        extras["estimate_1024"] = estimate_leg(fs, torch)
        extras["fft2d_vs_cufft"] = [fft_leg(fs, torch, stream, timed, n, b) for n, b in ((512, 64), (1024, 16))]
        rate, cores, n, dt = cpu_recon_rate(fs, datasets)
        extras["cpu_baseline"] = {"value": rate, "unit": "recon/s", "cores": cores, "kind": "port",
                                  "sample": "%d reconstructions of one 512x512 3x3 dataset in %.1f s (oracle: C++ "
                                            "restatement of the reference Java path, %d threads)" % (n, dt, cores)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "recon/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded: 2000 lognormal points + 40 filaments, cos patterns m=0.8, |k0|=0.85 cutoff, "
                    "500 photons + N(0,2)); %d distinct datasets tiled to the batch" % args.distinct,
            "config": {"workload": WORKLOAD, "batch": B, "n": N, "out": 2 * N, "path": "offline (runReconstruction)",
                       "form": "batch recorded as one CUDA graph (fsim_batch_graph), replayed per step",
                       "l2": "inputs larger than L2 (%.0f MiB raw per step)" % (h2d / 2 ** 20),
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "e2e": {"value": e2e_value, "unit": "recon/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "call": "fsim_recon_batch_host (pinned host buffers; chunked upload/passes/download overlapped)",
                    "repetitions_recon_per_s": [B * e2e_steps * world / (m / 1000.0) for m in e2e_runs],
                    "statistic": "median of 3 timed repetitions",
                    "h2d_GB_per_s_alone": h2d / (h2d_ms / 1000) / 1e9, "d2h_GB_per_s_alone": d2h / (d2h_ms / 1000) / 1e9},
            "roofline": {"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                         "algorithmic_bytes_per_launch": algo[dom] * B},
            "passes": passes,
            "e2e_fraction_of_hbm": (18874368 * value) / (peak * 1e9),
            "clocks": clk,
            "gpu_launches": kernels_per_step * args.steps,
        }
        if "cpu_baseline" in extras:
            line["cpu_baseline"] = extras.pop("cpu_baseline")
        line.update(extras)
        print(json.dumps(line))
    graph.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_only(args):
    """One extra leg on its own (GPU 0), e.g. to capture its kernels with ncu."""
    import torch

    fs = load_package()
    fs.native.init(0)
    stream = torch.cuda.Stream()

    def timed(fn, k):
        with torch.cuda.stream(stream):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(k):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            return e0.elapsed_time(e1)

    if args.only == "live":
        res = live_leg(fs, torch, stream, timed, batch=args.batch, steps=args.steps)
    elif args.only == "fft":
        res = [fft_leg(fs, torch, stream, timed, n, b, steps=args.steps) for n, b in ((512, 64), (1024, 16))]
    elif args.only == "estimate":
        res = estimate_leg(fs, torch, reps=max(1, args.steps))
    elif args.only == "mixed":
        res = mixed_leg(fs, torch, stream, timed, steps=args.steps)
    elif args.only == "large":
        res = large_leg(fs, torch, stream, timed, steps=args.steps)
    elif args.only == "ingest":
        res = ingest_leg(fs)
    elif args.only == "widefield":
        res = widefield_leg(fs, torch, stream, timed, batch=args.batch, steps=args.steps)
    else:
        res = {"poisson": serve_leg(fs), "saturated": serve_capacity_leg(fs)}
    print(json.dumps({args.only: res}))
    return 0


def plain_gpu_leg(fs, dataset, k=5, style=0):
    """The plain GPU form: one dataset at a time through the op-by-op device vector path
    (the reference's accel-backed Java pipeline, one library call per vector op); style:
    SimParam.FilterStyle (0 Wiener; 3 RL on the input and the output, 5 iterations each)."""
    V = fs.vectors
    raw, sp = dataset
    if style:
        sp = sp.duplicate()
        sp.setFilterStyle(style)
        sp.setRLiterations(5)
    spec_vecs = [[V.Vec2dCplx(N, N) for _ in range(NP)] for _ in range(NA)]
    fade = V.Vec2dReal(N, N)
    fade.setData(np.ones((N, N), np.float32))
    host_raw = [raw[i] for i in range(NA * NP)]

    def plain():
        for a in range(NA):
            for p in range(NP):
                v = spec_vecs[a][p]
                v.setData(host_raw[a * NP + p].astype(np.complex64))
                v.times(fade)
                v.fft2d(False)
        out = fs.algorithm.SimAlgorithm.runReconstruction(sp, spec_vecs, False, 0)
        out.vectorData()

    plain()
    t0 = time.perf_counter()
    for _ in range(k):
        plain()
    return {"value": k / (time.perf_counter() - t0), "unit": "recon/s", "filter_style": style,
            "note": "op-by-op device vector path (fsim_vec_* + fsim_run_reconstruction), one dataset at a time, "
                    "host buffers"}


def fused_batch1_leg(fs, dataset, k=200):
    """One dataset at a time through the fused plan from host buffers (fsim_recon_host: the raw
    stack uploaded, the passes, the image downloaded, one C call per dataset): the
    one-at-a-time GPU form without per-op calls, beside the op-by-op plain GPU form."""
    N_ = fs.native
    raw, sp = dataset
    plan = fs.plan.ReconPlan(sp, path=N_.PATH_OFFLINE, input_type=N_.INPUT_F32, fade_px=10)
    for _ in range(3):
        plan.reconstruct_host(raw)
    t0 = time.perf_counter()
    for _ in range(k):
        plan.reconstruct_host(raw)
    return {"value": k / (time.perf_counter() - t0), "unit": "recon/s",
            "note": "fused plan, one dataset per call from pageable host memory (fsim_recon_host), %d calls" % k}


def mixed_leg(fs, torch, stream, timed, n_datasets=64, steps=5, seed=77):
    """64 datasets, sizes uniform over {256, 384, 512, 768, 1024}, each with 1-3 channels
    (emission 488 / 525 / 600 nm, separate OTFs), 3x3 stacks, per-dataset seeded k0 angle and
    modulation in [0.5, 0.9]; all channels of all datasets in one CUDA-graph replay."""
    N_ = fs.native
    rng = np.random.default_rng(seed)
    sizes = [256, 384, 512, 768, 1024]
    lams = [488.0, 525.0, 600.0]
    # one generated stack per (size, emission) supplies the pixels; each dataset's channels
    # get their own seeded parameters (the work per stack does not depend on pixel values)
    pix = {}
    for n in sizes:
        for lam in lams:
            raw, _ = fs.synth.make_dataset(n=n, seed=300 + n + int(lam), em_wavelength=lam)
            pix[(n, lam)] = torch.from_numpy(raw).cuda()
    plans, raws, outs = [], [], []
    n_stacks = 0
    for d in range(n_datasets):
        n = sizes[rng.integers(len(sizes))]
        nch = int(rng.integers(1, 4))
        for ch in range(nch):
            lam = lams[ch]
            sp = fs.synth.synthetic_params(n, em_wavelength=lam, modulation=float(rng.uniform(0.5, 0.9)),
                                           seed=int(rng.integers(1 << 30)))
            plans.append(fs.plan.ReconPlan(sp, path=N_.PATH_OFFLINE, input_type=N_.INPUT_F32, fade_px=10))
            raws.append(pix[(n, lam)].clone())
            outs.append(torch.empty((2 * n, 2 * n), dtype=torch.float32, device="cuda"))
            n_stacks += 1
    ws = torch.empty(fs.plan.batch_workspace_bytes(plans), dtype=torch.uint8, device="cuda")
    jobs = [(p, r.data_ptr(), o.data_ptr()) for p, r, o in zip(plans, raws, outs)]
    g = fs.plan.BatchGraph(jobs, ws.data_ptr(), ws.numel(), stream.cuda_stream)
    for _ in range(3):
        g.launch(stream.cuda_stream)
    ms = timed(lambda: g.launch(stream.cuda_stream), steps)
    info = g.info()
    g.close()
    hist = {n: sum(1 for p in plans if p.w == n) for n in sizes}
    res = {"datasets_per_s": n_datasets * steps / (ms / 1000.0), "stacks_per_s": n_stacks * steps / (ms / 1000.0),
           "ms_per_batch": ms / steps, "datasets": n_datasets, "stacks": n_stacks, "stacks_per_size": hist,
           "kernels_per_replay": info["kernels"],
           "raw_MB_per_batch": sum(r.numel() * 4 for r in raws) / 1e6}
    for p in plans:
        p.close()
    return res


def widefield_leg(fs, torch, stream, timed, batch=64, steps=10, n=512, seed=88):
    """The offline batch of the headline (64 x 512^2 3x3 stacks) with and without the two
    widefield side outputs (runReconstruction's "Widefield" and "filtered Widefield",
    2w x 2w each): the added time per batch, and the widefield passes' algorithmic bytes
    (raw read + band-0 rows + filter + column outputs + images, per dataset) over that time."""
    N_ = fs.native
    raw, truth = fs.synth.make_dataset(n=n, seed=seed)
    sp = fs.synth.sim_param_for(truth, n)
    plan = fs.plan.ReconPlan(sp, path=N_.PATH_OFFLINE, input_type=N_.INPUT_F32, fade_px=10)
    d_raw = [torch.from_numpy(raw).cuda() for _ in range(batch)]
    img = lambda: torch.empty((2 * n, 2 * n), dtype=torch.float32, device="cuda")  # noqa: E731
    d_out, d_wf, d_fwf = [img() for _ in range(batch)], [img() for _ in range(batch)], [img() for _ in range(batch)]
    ws = torch.empty(fs.plan.batch_workspace_bytes([plan] * batch), dtype=torch.uint8, device="cuda")
    res = {}
    for key, with_wf in (("without", False), ("with", True)):
        jobs = [(plan, r.data_ptr(), o.data_ptr()) + ((w.data_ptr(), f.data_ptr()) if with_wf else ())
                for r, o, w, f in zip(d_raw, d_out, d_wf, d_fwf)]
        g = fs.plan.BatchGraph(jobs, ws.data_ptr(), ws.numel(), stream.cuda_stream)
        for _ in range(3):
            g.launch(stream.cuda_stream)
        ms = timed(lambda: g.launch(stream.cuda_stream), steps) / steps
        res[key] = {"ms_per_batch": ms, "recon_per_s": batch / (ms / 1000.0), "kernels": g.info()["kernels"]}
        g.close()
    nf = NA * NP
    wf_bytes = (nf * 4 * n * n + 8 * n * n) + (8 * n * n + 4 * n * n + 2 * 16 * n * n) + 2 * (16 * n * n + 16 * n * n)
    added = res["with"]["ms_per_batch"] - res["without"]["ms_per_batch"]
    res.update({"added_ms_per_batch": added, "algorithmic_MB_per_dataset": wf_bytes / 1e6,
                "widefield_GB_per_s": wf_bytes * batch / (added / 1000.0) / 1e9 if added > 0 else None})
    plan.close()
    return res


def ingest_leg(fs, n=512, n_seq=20, chunk=1 << 20, seed=91):
    """Live stream ingest (host): a two-channel LIVESIM byte stream of 512^2 u16 frames
    (3x3 per sequence, a sync gap before each) cut into 1 MiB pieces, through the sequence
    extractor alone (frames/s, GB/s of stream), then into the server as well (stacks/s
    reconstructed end to end, p50/p99 from submission to result)."""
    ig = fs.ingest
    nraw = NA * NP
    chans = []
    for k, lam in enumerate((488.0, 568.0)):
        raw, truth = fs.synth.make_dataset(n=n, seed=seed + k, em_wavelength=lam, as_u16=True)
        chans.append((int(lam), raw, fs.synth.sim_param_for(truth, n)))
    per = []
    for num, raw, _ in chans:
        frames, seq, t = [], 0, 10 ** 6
        for _ in range(n_seq):
            t += 8000
            for i in range(nraw):
                frames.append(ig.make_frame(raw[i], seq_nr=seq, pos1=num, time_camera=t))
                seq += 1
                t += 1000
        per.append(frames)
    blob = b"".join(f for pair in zip(*per) for f in pair)
    pieces = [blob[at:at + chunk] for at in range(0, len(blob), chunk)]

    def extractor():
        return ig.SequenceExtractor([c[0] for c in chans], nraw, n, n, sync_mode=0, sync_frame_delay=5000)

    x = extractor()
    t0 = time.perf_counter()
    for piece in pieces:
        x.feed(piece)
    popped = 0
    while x.pop() is not None:
        popped += 1
    dt = time.perf_counter() - t0
    frames = 2 * n_seq * nraw
    res = {"frames_per_s": frames / dt, "stream_GB_per_s": len(blob) / dt / 1e9, "stacks": popped,
           "note": "host only: header parse, sort, sync search, sequence copy"}
    x.close()
    srv = fs.plan.Server([c[2] for c in chans], max_batch=8, max_inflight=64, streams=3, refit_every=0)
    live = ig.LiveIngest(extractor(), srv)
    out = np.empty((2 * n, 2 * n), np.float32)
    t0 = time.perf_counter()
    tickets = []
    for piece in pieces:
        tickets += live.feed(piece)
    lat = [srv.wait(tk, out) for _, tk in tickets]
    dt = time.perf_counter() - t0
    res.update({"e2e_stacks_per_s": len(tickets) / dt, "e2e_p50_ms": float(np.percentile(lat, 50)),
                "e2e_p99_ms": float(np.percentile(lat, 99)), "e2e_stacks": len(tickets), "dropped": live.dropped})
    srv.close()
    live.x.close()
    return res


def live_leg(fs, torch, stream, timed, batch=64, steps=10):
    """The live path's kernels (ReconstructionThread semantics: u16 frames, damping, OTF
    before the fast shift, apodization bend 1) on a device-resident batch of 512^2 stacks
    from 3 channels, one CUDA-graph replay per step: the device throughput behind the
    served form."""
    N_ = fs.native
    chans = []
    for ch, lam in enumerate([488.0, 525.0, 600.0]):
        raw, truth = fs.synth.make_dataset(n=N, seed=700 + ch, em_wavelength=lam, as_u16=True)
        plan = fs.plan.ReconPlan(fs.synth.sim_param_for(truth, N), path=N_.PATH_LIVE, input_type=N_.INPUT_U16,
                                 fade_px=10)
        chans.append((plan, torch.from_numpy(raw.view(np.int16)).cuda()))
    plans = [chans[i % 3][0] for i in range(batch)]
    raws = [chans[i % 3][1].clone() for i in range(batch)]
    outs = torch.empty((batch, 2 * N, 2 * N), dtype=torch.float32, device="cuda")
    wfs = torch.empty((batch, N, N), dtype=torch.float32, device="cuda")
    ws = torch.empty(fs.plan.batch_workspace_bytes(plans), dtype=torch.uint8, device="cuda")
    jobs = [(p, r.data_ptr(), outs[i].data_ptr(), wfs[i].data_ptr()) for i, (p, r) in enumerate(zip(plans, raws))]
    g = fs.plan.BatchGraph(jobs, ws.data_ptr(), ws.numel(), stream.cuda_stream)
    for _ in range(3):
        g.launch(stream.cuda_stream)
    ms = timed(lambda: g.launch(stream.cuda_stream), steps)
    g.close()
    for p, _ in chans:
        p.close()
    return {"recon_per_s": batch * steps / (ms / 1000.0), "ms_per_batch": ms / steps, "batch": batch,
            "workload": "live path, 512^2 3x3 u16 -> 1024^2 + widefield, 3 channels"}


def large_leg(fs, torch, stream, timed, steps=5):
    """2048^2 raw, 3 angles x 5 phases (phases 2 pi k/5, pseudo-inverse separation),
    |k0| = 0.9 cutoff, modulation 0.6, 200 photons, reconstructed to 4096^2; throughput
    against the 20 stacks/s stream, and rel-L2 against the float and FP64 oracles."""
    from oracle import refcpu

    N_ = fs.native
    n = 2048
    raw, truth = fs.synth.make_dataset(n=n, n_phases=5, seed=500, k0_frac=0.9, modulation=0.6, photons=200.0)
    sp = fs.synth.sim_param_for(truth, n, n_phases=5)
    plan = fs.plan.ReconPlan(sp, path=N_.PATH_OFFLINE, input_type=N_.INPUT_F32, fade_px=10)
    d_raw = torch.from_numpy(raw).cuda()
    d_out = torch.empty((2 * n, 2 * n), dtype=torch.float32, device="cuda")
    ws = torch.empty(fs.plan.batch_workspace_bytes([plan]), dtype=torch.uint8, device="cuda")
    g = fs.plan.BatchGraph([(plan, d_raw.data_ptr(), d_out.data_ptr())], ws.data_ptr(), ws.numel(),
                           stream.cuda_stream)
    for _ in range(3):
        g.launch(stream.cuda_stream)
    ms = timed(lambda: g.launch(stream.cuda_stream), steps)
    got = d_out.cpu().numpy()
    g.close()
    t0 = time.perf_counter()
    got_host = plan.reconstruct_host(raw)
    host_ms = (time.perf_counter() - t0) * 1000
    refcpu.set_threads(os.cpu_count() or 1)
    exp32 = refcpu.recon_raw(sp, raw, fade=10)
    exp64 = refcpu.recon_raw(sp, raw.astype(np.float64), fade=10, dtype=np.float64)
    rl = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))  # noqa: E731
    plan.close()
    return {"stacks_per_s": 1000.0 / (ms / steps), "ms_per_stack": ms / steps,
            "host_call_ms": host_ms, "stream_target_stacks_per_s": 20.0,
            "rel_l2_vs_oracle_f32": rl(got, exp32), "rel_l2_vs_oracle_f64": rl(got, exp64),
            "oracle_f32_vs_f64": rl(exp32, exp64), "device_vs_host_call_identical": bool(np.array_equal(got, got_host))}


def fft_leg(fs, torch, stream, timed, n, batch, steps=10):
    """The library's 2D FFT (fsim_fft2d_batch: row pass + column pass, Stockham line FFTs)
    against cuFFT (torch.fft.fft2), as a comparator only, on `batch` n x n complex64 planes."""
    import ctypes as C

    lib = fs.native.lib()
    g = torch.Generator(device="cuda").manual_seed(n)
    x = torch.randn((batch, n, n), dtype=torch.complex64, device="cuda", generator=g)
    y = x.clone()
    sp = C.c_void_p(stream.cuda_stream)

    def ours():
        fs.native.check(lib.fsim_fft2d_batch(C.c_void_p(y.data_ptr()), n, n, batch, 0, sp))

    with torch.cuda.stream(stream):
        ours()
        ref = torch.fft.fft2(x)
        torch.cuda.synchronize()
        err = float((torch.linalg.vector_norm(y - ref) / torch.linalg.vector_norm(ref)).item())
        for _ in range(3):
            ours()
            torch.fft.fft2(x)
    ms_ours = timed(ours, steps) / steps
    with torch.cuda.stream(stream):
        ms_cufft = timed(lambda: torch.fft.fft2(x), steps) / steps
    byts = 16.0 * batch * n * n  # one read and one write of every complex64 element
    return {"n": n, "batch": batch, "ms": ms_ours, "cufft_ms": ms_cufft, "rel_l2_vs_cufft": err,
            "GB_per_s": byts / (ms_ours / 1000) / 1e9, "cufft_GB_per_s": byts / (ms_cufft / 1000) / 1e9}


def estimate_leg(fs, torch, reps=3):
    """Full parameter fit at 1024^2 on the device (fade, FFT, locatePeak, fitPeak 3 x 10 x
    10, getPeak per angle), with the fitted k0 compared to the generator's."""
    import ctypes as C

    N_ = fs.native
    n = 1024
    raw, truth = fs.synth.make_dataset(n=n, seed=600)
    sp = fs.synth.sim_param_for(truth, n)
    sp.directions = [fs.Dir(NB, NP) for _ in range(NA)]  # start from no knowledge of the shifts
    d_raw = torch.from_numpy(raw).cuda()
    out = (C.c_double * 12)()
    ts = []
    for _ in range(reps + 1):
        c = N_.to_c_param(sp)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        N_.check(N_.lib().fsim_estimate_raw(C.byref(c), C.c_void_p(d_raw.data_ptr()), N_.INPUT_F32, 10, 1,
                                            C.c_double(0.6), out))
        ts.append((time.perf_counter() - t0) * 1000)
    got = N_.from_c_param(c)
    err = max(max(abs(got["pX"][d] - truth["pxpy"][d][0]), abs(got["pY"][d] - truth["pxpy"][d][1]))
              for d in range(NA))
    return {"ms_per_fit": float(np.median(ts[1:])), "max_k0_error_px": err}


def serve_leg(fs, seconds=3.0, rate_per_channel=100.0, seed=5):
    """Poisson arrivals from 3 channels at 512^2 (u16) plus their 1024^2 stacks (10%)."""
    N_ = fs.native
    rng = np.random.default_rng(seed)
    chans, stacks = [], []
    for ch, lam in enumerate([488.0, 525.0, 600.0]):
        for n in (512, 1024):
            raw, truth = fs.synth.make_dataset(n=n, seed=200 + 10 * ch + n // 512, em_wavelength=lam, as_u16=True)
            chans.append(fs.synth.sim_param_for(truth, n))
            stacks.append(raw)
    srv = fs.plan.Server(chans, max_batch=16, max_inflight=96, streams=3, refit_every=50,
                         input_type=N_.INPUT_U16, fade_px=10)
    outs = {n: np.empty((2 * n, 2 * n), np.float32) for n in (512, 1024)}
    # arrival schedule
    events = []
    for ch in range(3):
        t = 0.0
        while t < seconds:
            t += rng.exponential(1.0 / rate_per_channel)
            big = rng.random() < 0.1
            events.append((t, 2 * ch + (1 if big else 0)))
    events.sort()
    tickets = []
    t0 = time.perf_counter()
    rejected = 0
    for t, c in events:
        while time.perf_counter() - t0 < t:
            time.sleep(0.0002)
        tk = srv.try_submit(c, stacks[c])
        if tk is None:
            rejected += 1
            continue
        tickets.append((tk, c))
        # collect finished results opportunistically to free slots
        while len(tickets) > 64:
            tk0, c0 = tickets.pop(0)
            srv.wait(tk0, outs[chans[c0].w])
    for tk, c in tickets:
        srv.wait(tk, outs[chans[c].w])
    st = srv.stats()
    srv.close()
    return {"p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"], "max_ms": st["max_ms"],
            "recon_per_s": st["completed"] / max(1e-9, time.perf_counter() - t0), "completed": st["completed"],
            "rejected": st["rejected"], "refits": st["refits"],
            "arrivals": "Poisson, 3 channels x %.0f stacks/s, 10%% at 1024^2, u16, %.1f s" % (rate_per_channel, seconds)}


def serve_capacity_leg(fs, seconds=2.0, seed=6):
    """Served form at saturation: a closed loop keeps the slots of 3 channels at 512^2 (u16)
    full, so completions per second measure the serving capacity; latencies are those of
    stacks queued behind a full device."""
    N_ = fs.native
    chans, stacks = [], []
    for ch, lam in enumerate([488.0, 525.0, 600.0]):
        raw, truth = fs.synth.make_dataset(n=N, seed=400 + ch, em_wavelength=lam, as_u16=True)
        chans.append(fs.synth.sim_param_for(truth, N))
        stacks.append(raw)
    srv = fs.plan.Server(chans, max_batch=32, max_inflight=192, streams=3, refit_every=0,
                         input_type=N_.INPUT_U16, fade_px=10)
    out = np.empty((2 * N, 2 * N), np.float32)
    from collections import deque

    q = deque()
    k = 0
    t0 = time.perf_counter()
    done = 0
    while time.perf_counter() - t0 < seconds:
        while True:
            tk = srv.try_submit(k % 3, stacks[k % 3])
            if tk is None:
                break
            q.append(tk)
            k += 1
        for _ in range(min(32, len(q))):
            srv.wait(q.popleft(), out)
            done += 1
    while q:
        srv.wait(q.popleft(), out)
        done += 1
    dt = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    return {"recon_per_s": done / dt, "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "completed": done,
            "load": "closed loop, 3 channels x 512^2 u16, up to 192 stacks in flight, batches of up to 32"}


if __name__ == "__main__":
    sys.exit(main())
