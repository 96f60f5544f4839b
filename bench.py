"""Benchmark: eSRRF input Mpx*frames/s on one GB300 (and N independent replicas).

Workload (default): the large single eSRRF -- 500 frames x 512 x 512 float32
(seeded blinking emitters, 400 emitters), magnification 5, radius 1.5,
sensitivity 2, VAR and TAC2 correlations, 100 frames per timepoint,
macro-pixel correction; output 2 x 5 x 2560 x 2560 float32.

* ``value``: device-resident throughput (input already in HBM): one step = the
  full reconstruction of the stack (fused frame-loop kernel + temporal
  finalisation + macro-pixel correction), CUDA events on the launching stream.
* ``e2e``: the same reconstruction through the public API ``nanopyx_gb300.eSRRF``
  with NumPy host buffers in and out (H2D + D2H inside the timed region).
* ``roofline``: the fused kernel's algorithmic FP32 FLOP/s over the measured
  FP32 FMA peak of this GPU (the path is FP32-compute bound; no tensor cores).
* ``cpu_baseline``: the reference's own compiled CPU path (``oracle/_ref``) on a
  bounded sample of the same workload, all host threads.

``--impl reference`` times the reference CPU path alone (rank 0 only).
Inputs (524 MB) are larger than L2 (129 MB), so no L2 flush is needed.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

CFG = dict(T=500, H=512, W=512, emitters=400, m=5, radius=1.5, sensitivity=2.0,
           correlations=("VAR", "TAC2"), fpt=100, mpc=True, seed=1)
# profiling case: same kernel and frame size, 160 frames (168 MB input, still > L2)
SMALL = dict(T=160, fpt=80)
# DRAM bytes of one fused launch, dram__bytes_read.sum + dram__bytes_write.sum from a
# 1-pass ncu capture of that launch (large: the full 500-frame launch; small: 160 frames)
TRAFFIC_BYTES = {"large": 531373568 + 603790336, "small": 168473856 + 207223296}
METRIC = "eSRRF input Mpx*frames/s"
# frames per reference step: eSRRF_ST and the temporal step scale with the frame
# count; the per-timepoint macro-pixel correction (2 x ~30 ms on 2560^2) is <1 %
# of an 8-frame step, so treating the sample as one timepoint keeps the rate
# within ~1 % of the 100-frame-timepoint workload's
REF_SAMPLE_FRAMES = 8


def _workload_name():
    return (f"single eSRRF {CFG['T']}x{CFG['H']}x{CFG['W']} m={CFG['m']} R={CFG['radius']} "
            f"s={CFG['sensitivity']:g} VAR+TAC2 fpt={CFG['fpt']} MPC")


def _mpx_frames(T, H, W):
    return T * H * W / 1e6


def make_stack():
    from nanopyx_gb300.synthetic import blinking_stack

    return blinking_stack(CFG["T"], CFG["H"], CFG["W"], CFG["emitters"], seed=CFG["seed"])


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed
    region runs (read through a pipe; nothing is written to disk)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, command=None):
        self.gpu = gpu_index
        self.proc = None
        self.thread = None
        self.lines = []
        self.command = command or ["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.Q}",
                                   "--format=csv,noheader,nounits", "-lms", "100"]

    def _read(self, ready):
        for line in self.proc.stdout:
            self.lines.append(line)
            ready.set()

    def __enter__(self):
        import threading

        try:
            self.proc = subprocess.Popen(self.command, stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            ready = threading.Event()
            self.thread = threading.Thread(target=self._read, args=(ready,), daemon=True)
            self.thread.start()
            # nvidia-smi takes a moment to start: hold the timed region until it samples
            ready.wait(1.0)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            if self.thread is not None:
                self.thread.join(timeout=5)

    def summary(self):
        rows = [r.strip().split(", ") for r in list(self.lines) if r.strip()]
        rows = [r for r in rows if len(r) >= 9]
        if not rows:
            return None
        try:
            sm = [float(r[1]) for r in rows]
            mx = max(float(r[2]) for r in rows)
        except ValueError:
            return None
        busy = [x for x in sm if x > 0.5 * mx] or sm
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(busy), "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------------------
# algorithmic work of the fused kernel
# ---------------------------------------------------------------------------
def samples_per_output(m, radius):
    """Mean number of in-radius RGC samples per output pixel, S(m, R)."""
    import ctypes

    from nanopyx_gb300 import _native

    L = _native.lib()
    cap = m * m * 64 * 64
    buf = np.zeros(cap, dtype=np.float32)
    J = L.nx_esrrf_weight_table(m, float(radius), buf.ctypes.data_as(ctypes.c_void_p), cap)
    W2 = 2 * J + 1
    w = buf[: m * m * W2 * W2]
    return float((w > 0).sum()) / (m * m)


def fused_flops(T, H, W, m, radius):
    """FLOP = sum_frames [H W m^2 (10 S(m,R) + 20) + 60 H W]."""
    S = samples_per_output(m, radius)
    return T * (H * W * m * m * (10.0 * S + 20.0) + 60.0 * H * W), S


def measure_fp32_peak(device, packed=False):
    """Best FP32 FMA throughput of an FMA-only loop (TFLOP/s); ``packed`` uses f32x2."""
    import torch

    from nanopyx_gb300 import _native

    L = _native.lib()
    probe = L.nx_probe_ffma2 if packed else L.nx_probe_ffma
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    blocks = sms * 8
    iters = 4096
    sink = torch.empty(blocks * 256, dtype=torch.float32, device=device)
    s = torch.cuda.current_stream(device)
    for _ in range(2):
        _native.check(probe(sink.data_ptr(), blocks, iters, s.cuda_stream))
    torch.cuda.synchronize(device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 0.0
    for _ in range(5):
        e0.record(s)
        _native.check(probe(sink.data_ptr(), blocks, iters, s.cuda_stream))
        e1.record(s)
        torch.cuda.synchronize(device)
        flops = blocks * 256 * iters * 16 * 8 * 2.0
        best = max(best, flops / (e0.elapsed_time(e1) * 1e-3))
    return best / 1e12


# ---------------------------------------------------------------------------
# CPU baseline: the reference's compiled path on a bounded sample
# ---------------------------------------------------------------------------
def reference_step(R, sample):
    """eSRRF_ST + VAR + TAC2 + macro-pixel correction on one sample block."""
    st = R["eSRRF_ST"](verbose=False).run(sample, magnification=CFG["m"], radius=CFG["radius"],
                                          sensitivity=CFG["sensitivity"], run_type="Threaded")
    outs = []
    for corr in CFG["correlations"]:
        tc = R["calculate_eSRRF_temporal_correlations"](st, corr)
        outs.append(R["macro_pixel_corrector"](np.expand_dims(np.asarray(tc), 0),
                                               magnification=CFG["m"]))
    return outs


def cpu_reference_available():
    try:
        from oracle import ref_build

        if not ref_build.available():
            ref_build.build()
        return ref_build.available()
    except Exception:
        return False


def time_cpu_baseline(stack, frames=REF_SAMPLE_FRAMES):
    """Returns the cpu_baseline dict (reference if buildable here, else the FP64 port)."""
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    sample = np.ascontiguousarray(stack[:frames])
    if cpu_reference_available():
        from oracle import ref_build

        R = ref_build.load()
        reference_step(R, sample[:2])  # warm-up (thread pool, pages)
        t0 = time.perf_counter()
        reference_step(R, sample)
        dt = time.perf_counter() - t0
        kind = "reference"
        desc = (f"{frames} frames of the {CFG['H']}x{CFG['W']} stack as one timepoint (the "
                f"workload's timepoints hold {CFG['fpt']} frames; the per-timepoint macro-pixel "
                f"correction is <1 % of the sample's time): compiled reference "
                f"eSRRF_ST(Threaded) + VAR + TAC2 + macro_pixel_corrector")
    else:
        from oracle import esrrf_np

        frames = 1
        cores = 1
        t0 = time.perf_counter()
        esrrf_np.esrrf_st(sample[:1], CFG["m"], CFG["radius"], CFG["sensitivity"])
        dt = time.perf_counter() - t0
        kind = "port"
        desc = "1 frame of the stack through the FP64 NumPy oracle (reference not buildable)"
    return {"value": _mpx_frames(frames, CFG["H"], CFG["W"]) / dt, "unit": "Mpx*frames/s",
            "cores": int(os.environ.get("OMP_NUM_THREADS", cores)) if kind == "reference" else 1,
            "kind": kind, "sample": desc, "seconds": dt}


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------
def run_reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(cores)
    from nanopyx_gb300.synthetic import blinking_stack

    frames = REF_SAMPLE_FRAMES
    stack = blinking_stack(frames, CFG["H"], CFG["W"], CFG["emitters"], seed=CFG["seed"])
    line = {"impl": "reference", "metric": METRIC, "unit": "Mpx*frames/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": _workload_name(), "parallelism": "cpu"}}
    if not cpu_reference_available():
        from oracle import esrrf_np

        kind, cores_used = "port", 1
        fn = lambda: esrrf_np.esrrf_st(stack[:1], CFG["m"], CFG["radius"], CFG["sensitivity"])  # noqa: E731
        frames = 1
        sample = "1 frame per step through the FP64 NumPy oracle (reference not buildable here)"
    else:
        from oracle import ref_build

        R = ref_build.load()
        kind, cores_used = "reference", cores
        fn = lambda: reference_step(R, stack)  # noqa: E731
        sample = (f"{frames} frames of the {CFG['H']}x{CFG['W']} stack per step as one timepoint "
                  f"(the workload's timepoints hold {CFG['fpt']} frames; the per-timepoint "
                  "macro-pixel correction is <1 % of a step): eSRRF_ST(Threaded) + VAR + TAC2 + "
                  "macro_pixel_corrector")
    for _ in range(args.warmup):
        fn()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        fn()
        times.append(time.perf_counter() - t0)
    ms = 1e3 * sum(times) / len(times)
    value = _mpx_frames(frames, CFG["H"], CFG["W"]) / (ms / 1e3)
    line.update({"value": value, "ms_per_step": ms,
                 "cpu_baseline": {"value": value, "unit": "Mpx*frames/s", "cores": cores_used,
                                  "kind": kind, "sample": sample},
                 "e2e": {"value": value, "unit": "Mpx*frames/s", "h2d_bytes_per_step": 0,
                         "d2h_bytes_per_step": 0}})
    print(json.dumps(line), flush=True)
    return 0


def max_over_ranks(value_ms: float, device=None) -> float:
    """Largest timing over all ranks (every rank gets it); no-op without a process group."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value_ms)
    t = torch.tensor([float(value_ms)], dtype=torch.float64,
                     device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_gpu_arm(args):
    import torch

    import nanopyx_gb300 as nx
    from nanopyx_gb300 import _device, _native

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)

    stack_np = make_stack()
    T, H, W = stack_np.shape
    m, R, s = CFG["m"], CFG["radius"], CFG["sensitivity"]
    fpt = CFG["fpt"]
    L = _native.lib()
    stream = torch.cuda.current_stream(dev)
    x = torch.from_numpy(stack_np).to(dev)
    plan = _device.get_plan(H, W, m, R, s, True)
    mask = _native.NX_CORR_VAR | _native.NX_CORR_TAC2
    ws = _device.workspace(L.nx_esrrf_workspace_bytes(plan.handle, T, fpt, mask), dev)
    n_tp = (T + fpt - 1) // fpt
    out = torch.empty((2, n_tp, H * m, W * m), dtype=torch.float32, device=dev)

    def step(ev0=None, ev1=None):
        if ev0 is not None:
            ev0.record(stream)
        _native.check(L.nx_esrrf_run_stage1(plan.handle, x.data_ptr(), T, fpt, mask,
                                            ws.data_ptr(), ws.numel(), stream.cuda_stream))
        if ev1 is not None:
            ev1.record(stream)
        _native.check(L.nx_esrrf_run_stage2(plan.handle, T, fpt, mask, 1, out.data_ptr(),
                                            ws.data_ptr(), ws.numel(), stream.cuda_stream))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    _native.check(L.nx_workspace_status(ws.data_ptr(), stream.cuda_stream), "warm-up")

    k_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            for _ in range(args.steps)]
    t_start, t_stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        t_start.record(stream)
        for i in range(args.steps):
            step(*k_ev[i])
        t_stop.record(stream)
        torch.cuda.synchronize(dev)
    if dist is not None:
        dist.barrier()
    _native.check(L.nx_workspace_status(ws.data_ptr(), stream.cuda_stream), "timed steps")
    total_ms = t_start.elapsed_time(t_stop)
    kern_ms = sum(a.elapsed_time(b) for a, b in k_ev) / args.steps
    total_ms = max_over_ranks(total_ms, dev)
    ms_per_step = total_ms / args.steps
    mpxf = _mpx_frames(T, H, W)
    value = world * mpxf / (ms_per_step / 1e3)

    # kernel roofline (FP32 FMA bound)
    flops, S = fused_flops(T, H, W, m, R)
    achieved = flops / (kern_ms * 1e-3) / 1e12
    peak_scalar = measure_fp32_peak(dev)
    peak_packed = measure_fp32_peak(dev, packed=True)
    peak = max(peak_scalar, peak_packed)
    clocks = clk.summary()

    # end to end through the public API with host buffers
    e2e_times = []
    res = None
    for i in range(max(1, min(args.steps, 3)) + 1):
        # the previous call's result (262 MB at the full size) is released
        # before the clock starts, not inside the next call's timing
        res = None
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        res = nx.eSRRF(stack_np, magnification=m, radius=R, sensitivity=s,
                       frames_per_timepoint=fpt, temporal_correlation=CFG["correlations"])
        t1 = time.perf_counter()
        if i > 0:
            e2e_times.append(t1 - t0)
    e2e_s = statistics.median(e2e_times)
    out_bytes = sum(r.nbytes for r in res)

    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "value": value, "unit": "Mpx*frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded blinking emitters)",
        "config": {"workload": _workload_name(), "T": T, "H": H, "W": W, "magnification": m,
                   "radius": R, "sensitivity": s, "correlations": list(CFG["correlations"]),
                   "frames_per_timepoint": fpt, "macro_pixel_correction": True,
                   "parallelism": f"replicas{world}" if world > 1 else "single GPU",
                   "l2": f"input {stack_np.nbytes / 1e6:.0f} MB > 129 MB L2; no flush"},
        "e2e": {"value": mpxf / e2e_s, "unit": "Mpx*frames/s", "seconds": e2e_s,
                "h2d_bytes_per_step": int(stack_np.nbytes), "d2h_bytes_per_step": int(out_bytes)},
        "gpu_launches": args.steps * (1 + n_tp + 2),
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak,
                     "traffic": TRAFFIC_BYTES.get(args.workload),
                     "traffic_unit": "bytes per launch (ncu DRAM read + write)",
                     "kernel": f"esrrf_fused_kernel<m={m},J={int(2 * R)},FULL>",
                     "kernel_ms": kern_ms,
                     "flops_per_launch": flops, "samples_per_output": S,
                     "peak_scalar_ffma": peak_scalar, "peak_packed_ffma2": peak_packed,
                     "peak_source": "measured FMA-loop throughput on this GPU, best of scalar FFMA "
                                    "and packed f32x2 FFMA2 (no FP32 figure in MEASURED_PEAKS.json)"},
        "clocks": clocks,
    }
    if not args.no_extras and args.workload == "large" and world == 1:
        del x, out, ws
        torch.cuda.empty_cache()
        line["batched"] = bench_uneven_batch(dev)
        torch.cuda.empty_cache()
        line["sweep"] = bench_sweep(dev)
        torch.cuda.empty_cache()
        line["sweep_scored"] = bench_scored_sweep(dev)
        torch.cuda.empty_cache()
        line["esrrf3d"] = bench_esrrf3d(dev)
        torch.cuda.empty_cache()
        # arrival-rate sweep of the served stream (rates bracket the device's
        # capacity for this request mix); "served" is the highest rate
        blocks = served_blocks([64, 90, 128, 181, 256, 362, 512, 724, 1024])
        rates = SERVED_RATES if args.served_rates is None else tuple(args.served_rates)
        sweep = [bench_served(dev, n_requests=args.served_requests, rate=r, blocks=blocks)
                 for r in rates]
        line["served_sweep"] = [{"rate_per_s": r, "served": x["served"], "plain": x["plain"],
                                 "throughput_ratio": x["throughput_ratio"]}
                                for r, x in zip(rates, sweep)]
        line["served"] = sweep[-1]
        torch.cuda.empty_cache()
        line["srrf"] = bench_srrf(dev, stack_np, peak=peak)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = time_cpu_baseline(stack_np)
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# batched, sweep and served workloads (reported beside the headline line)
# ---------------------------------------------------------------------------
def _base_stacks(sizes, frames=25, density=0.006, seed=11):
    from nanopyx_gb300.synthetic import blinking_stack, emitters_for_density

    return {H: blinking_stack(frames, H, H, emitters_for_density(H, H, density), seed=seed + H)
            for H in sizes}


def _tile_frames(base, T):
    reps = -(-T // base.shape[0])
    return np.ascontiguousarray(np.concatenate([base] * reps)[:T])


def bench_uneven_batch(dev, n_stacks=64, seed=3, repeats=2):
    """64 stacks, H=W in {64,128,256,512}, T in [50,500], m in {2,4,5}, AVG/VAR/TAC2."""
    import torch

    import nanopyx_gb300 as nx
    from nanopyx_gb300 import engine

    rng = np.random.default_rng(seed)
    sizes = [64, 128, 256, 512]
    bases = _base_stacks(sizes)
    stacks, params, mpxf = [], [], 0.0
    for _ in range(n_stacks):
        H = int(rng.choice(sizes))
        T = int(rng.integers(50, 501))
        x = torch.from_numpy(_tile_frames(bases[H], T)).to(dev)
        stacks.append(x)
        params.append(dict(magnification=int(rng.choice([2, 4, 5])), radius=1.5, sensitivity=1,
                           temporal_correlation=str(rng.choice(["AVG", "VAR", "TAC2"]))))
        mpxf += T * H * H / 1e6
    def build(tiles):
        bb = engine.EsrrfBatch(dev, tiles=tiles)
        for x, kw in zip(stacks, params):
            bb.add(x, **kw)
        return bb

    # the tiling autotuner times each kernel key's tilings on this batch
    tuned = engine.tune_tiling(build)
    b = build(None)
    b.run(graph=True)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(repeats):
        b.run(graph=True, check=False)
    e1.record()
    torch.cuda.synchronize(dev)
    t_batch = e0.elapsed_time(e1) / repeats / 1e3
    # plain per-stack GPU path: one eSRRF call per stack, in turn
    for x, kw in zip(stacks[:2], params[:2]):
        nx.esrrf_device(x, kw["magnification"], kw["radius"], kw["sensitivity"], 0,
                        kw["temporal_correlation"], check_status=False)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for x, kw in zip(stacks, params):
        nx.esrrf_device(x, kw["magnification"], kw["radius"], kw["sensitivity"], 0,
                        kw["temporal_correlation"], check_status=False)
        torch.cuda.synchronize(dev)
    t_plain = time.perf_counter() - t0
    return {"workload": f"{n_stacks} uneven stacks, H=W in {{64,128,256,512}}, T in [50,500], "
                        "m in {2,4,5}, R=1.5, s=1, AVG/VAR/TAC2 (one persistent launch per "
                        "kernel class, CUDA graph); each stack's frames repeat one seeded "
                        "25-frame block per frame size (kernel time does not depend on the "
                        "pixel values)",
            "mpx_frames": mpxf, "batched_value": mpxf / t_batch, "plain_value": mpxf / t_plain,
            "unit": "Mpx*frames/s", "batched_s": t_batch, "plain_s": t_plain,
            "speedup": t_plain / t_batch,
            "tiling": {"autotuned": tuned,
                       "used": {f"m{m}_J{J}": v for (m, J), v in sorted(b.tiling.items())}}}


def bench_sweep(dev, repeats=3):
    """200 x 256 x 256, m=4, R in {1,1.5,2,2.5} x s in {1,2,3,4}, AVG: 16 outputs.

    The grid is planned and captured once (outside the timed region); the
    timed region replays its CUDA graph.  The plain comparison is 16 separate
    eSRRF calls on the resident stack, as the reference's sweep makes 16 runs."""
    import torch

    import nanopyx_gb300 as nx
    from nanopyx_gb300 import engine
    from nanopyx_gb300.synthetic import blinking_stack

    x = torch.from_numpy(blinking_stack(200, 256, 256, 150, seed=2)).to(dev)
    sens, radii = [1, 2, 3, 4], [1.0, 1.5, 2.0, 2.5]
    tuned = engine.tune_tiling(lambda t: engine.SweepGrid(x, 4, sens, radii, tiles=t,
                                                          plan=False).batch)
    grid = engine.SweepGrid(x, 4, sens, radii)
    grid.run(graph=True)
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(repeats):
        grid.run(graph=True, check=False)
    e1.record()
    torch.cuda.synchronize(dev)
    t_sweep = e0.elapsed_time(e1) / repeats / 1e3
    for s in sens[:1]:
        nx.esrrf_device(x, 4, 1.5, s, 0, "AVG", macro_pixel_correction=False, check_status=False)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for s in sens:
        for r in radii:
            nx.esrrf_device(x, 4, r, s, 0, "AVG", macro_pixel_correction=False, check_status=False)
    torch.cuda.synchronize(dev)
    t_plain = time.perf_counter() - t0
    mpxf = 200 * 256 * 256 / 1e6
    return {"workload": "sweep 200x256x256, m=4, R in {1,1.5,2,2.5} x s in {1,2,3,4}, AVG "
                        "(16 outputs; one RGC pass per radius shared by 4 sensitivities; "
                        "CUDA-graph replay, planning outside the timed region)",
            "sweep_s": t_sweep, "plain_16_calls_s": t_plain, "speedup": t_plain / t_sweep,
            "value": mpxf / t_sweep, "unit": "input Mpx*frames/s for the whole grid",
            "tiling": {"autotuned": tuned,
                       "used": {f"m{m}_J{J}": v
                                for (m, J), v in sorted(grid.batch.tiling.items())}}}


def bench_scored_sweep(dev, repeats=3, with_reference=True):
    """The scored sweep of the same grid: ParameterSweep.run -- reconstructions
    over all, odd and even frames, ErrorMap RSP of all 16 pairs (one lockstep
    Brent search), FRC of all 16 pairs (one batch of FFTs), QnR.

    Beside it, the compiled reference on bounded samples of the same work: its
    eSRRF_ST on 4 frames and its ErrorMap + FIRECalculator on one pair's
    1024 x 1024 images (inputs: this engine's reconstructions of that pair);
    the reference's whole sweep is extrapolated from those two timings
    (16 x (200 frames x per-frame time + scoring time)), and the pair's RSP and
    FRC resolution are compared with this engine's."""
    import torch

    import nanopyx_gb300 as nx
    from nanopyx_gb300 import scoring
    from nanopyx_gb300.synthetic import blinking_stack

    x_np = blinking_stack(200, 256, 256, 150, seed=2)
    x = torch.from_numpy(x_np).to(dev)
    sens, radii = [1, 2, 3, 4], [1.0, 1.5, 2.0, 2.5]
    ps = nx.ParameterSweep()
    ps.run(x, 4, sens, radii)  # warm-up: plans, kernels, tuned tilings
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(repeats):
        q = ps.run(x, 4, sens, radii)
    torch.cuda.synchronize(dev)
    t_sweep = (time.perf_counter() - t0) / repeats
    t0 = time.perf_counter()
    rec = ps.reconstructions(x, 4, sens, radii)
    torch.cuda.synchronize(dev)
    t1 = time.perf_counter()
    H, W = rec[0].shape[-2:]
    em = scoring.error_maps(scoring._frame_mean(x), rec[0][:, :, 0].reshape(16, H, W))
    torch.cuda.synchronize(dev)
    t2 = time.perf_counter()
    frc = ps._fire_grid(rec[1], rec[2])
    t3 = time.perf_counter()
    img = rec[0][1, 1, 0].contiguous()  # s = 2, R = 1.5
    nx.DecorrAnalysis().run_analysis(img)
    torch.cuda.synchronize(dev)
    t4 = time.perf_counter()
    dec_gpu = nx.DecorrAnalysis().run_analysis(img)
    torch.cuda.synchronize(dev)
    t_dec = time.perf_counter() - t4
    out = {"workload": "scored sweep: 200x256x256, m=4, R in {1,1.5,2,2.5} x s in {1,2,3,4}, "
                       "AVG; reconstructions (all/odd/even frames), RSP, FRC, QnR",
           "seconds": t_sweep, "reconstructions_s": t1 - t0, "error_maps_s": t2 - t1,
           "frc_s": t3 - t2, "brent_evaluations": int(sum(em["evaluations"])),
           "qnr_best": [sens[int(np.argmax(q)) // 4], radii[int(np.argmax(q)) % 4]],
           "decorrelation_1024x1024_s": t_dec}
    if with_reference and cpu_reference_available():
        from oracle import ref_build

        R = ref_build.load()
        R["eSRRF_ST"](verbose=False).run(x_np[:2], magnification=4, radius=1.5, sensitivity=1,
                                         run_type="Threaded")
        t0 = time.perf_counter()
        R["eSRRF_ST"](verbose=False).run(x_np[:4], magnification=4, radius=1.5, sensitivity=1,
                                         run_type="Threaded")
        t_frame = (time.perf_counter() - t0) / 4
        si, ri = 1, 1  # s = 2, R = 1.5
        ref_img = np.mean(x_np, axis=0)
        t0 = time.perf_counter()
        emr = R["ErrorMap"]()
        emr.optimise(ref_img, rec[0][si, ri, 0].cpu().numpy())
        t1 = time.perf_counter()
        fire_ref = R["FIRECalculator"]().calculate_fire_number(rec[1][si, ri, 0].cpu().numpy(),
                                                               rec[2][si, ri, 0].cpu().numpy())
        t2 = time.perf_counter()
        t_score = t2 - t0
        dcr = R["DecorrAnalysis"]()
        t3 = time.perf_counter()
        dcr.run_analysis(img.cpu().numpy())
        t_dec_ref = time.perf_counter() - t3
        est = 16 * (200 * t_frame + t_score)
        out["reference"] = {
            "kind": "reference", "cores": os.cpu_count(),
            "sample": "compiled reference: eSRRF_ST(Threaded) of 4 frames at m=4; ErrorMap + "
                      "FIRECalculator of one pair (s=2, R=1.5) at 1024x1024",
            "esrrf_st_s_per_frame": t_frame, "error_map_s": t1 - t0, "frc_s": t2 - t1,
            "sweep_s_extrapolated": est,
            # the reference's Pearson correlation sums 1M pixels in float32 per
            # OpenMP thread: its RSP at this size depends on the thread count
            "omp_threads": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)),
            "pair_parity": {"sigma_gpu": em["sigma"][si * 4 + ri],
                            "sigma_reference": emr.get_sigma(),
                            "rsp_gpu": em["rsp"][si * 4 + ri], "rsp_reference": emr.getRSP(),
                            "fire_gpu": float(frc[si, ri]), "fire_reference": float(fire_ref),
                            "decorrelation_gpu": dec_gpu,
                            "decorrelation_reference": float(dcr.resolution)},
            "decorrelation_s": t_dec_ref}
        out["speedup_vs_reference_extrapolated"] = est / t_sweep
    return out


def bench_esrrf3d(dev, T=20, S=16, H=128, W=128, repeats=3, with_reference=True):
    """eSRRF-3D of a (20, 16, 128, 128) stack at magnification 2 x 2 (R = 1.5,
    PSF ratio 2.8, voxel ratio 4, average), inputs resident on the device;
    beside it the compiled reference's eSRRF3D_ST on 2 frames of the stack."""
    import torch

    import nanopyx_gb300 as nx

    rng = np.random.default_rng(1)
    x_np = (rng.random((T, S, H, W)) * 200 + 20).astype(np.float32)
    x = torch.from_numpy(x_np).to(dev)
    op = nx.eSRRF3D_ST(verbose=False)
    op.run(x[:2])
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(repeats):
        out = op.run(x)
    e1.record()
    torch.cuda.synchronize(dev)
    t = e0.elapsed_time(e1) / repeats / 1e3
    vox = int(out.numel()) * T
    res = {"workload": f"eSRRF-3D {T}x{S}x{H}x{W}, m_xy=2, m_z=2, R=1.5, average",
           "seconds": t, "value": vox / t / 1e6, "unit": "output Mvoxel*frames/s"}
    if with_reference and cpu_reference_available():
        from oracle import ref_build

        R = ref_build.load()
        t0 = time.perf_counter()
        R["eSRRF3D_ST"](verbose=False).run(x_np[:2], run_type="Threaded")
        tr = (time.perf_counter() - t0) / 2
        res["reference"] = {"kind": "reference", "cores": os.cpu_count(),
                            "sample": "compiled reference eSRRF3D_ST(Threaded), 2 frames",
                            "seconds_per_frame": tr, "value": vox / T / tr / 1e6}
        res["speedup_vs_reference"] = tr * T / t
    return res


SERVED_RATES = (5.0, 10.0, 20.0, 30.0)


def bench_served(dev, n_requests=200, rate=8.0, block_interval=0.01, seed=9, blocks=None):
    """Poisson arrivals; H=W log-uniform 64..1024; 1-10 blocks of 100 frames; m in {2,4,5}.

    Every request's blocks repeat one seeded 100-frame block of its frame size
    (one per size, generated once): the kernels' time does not depend on the
    pixel values, and 200 requests of distinct frames would need ~80 GB of
    host memory."""
    import threading

    import torch

    from nanopyx_gb300.serve import ESRRFServer, serve_plain

    rng = np.random.default_rng(seed)
    sizes = [64, 90, 128, 181, 256, 362, 512, 724, 1024]
    blocks100 = blocks if blocks is not None else served_blocks(sizes)
    reqs, t = [], 0.0
    for _ in range(n_requests):
        t += rng.exponential(1.0 / rate)
        H = int(sizes[rng.integers(0, len(sizes))])
        reqs.append(dict(t=t, H=H, nb=int(rng.integers(1, 11)), m=int(rng.choice([2, 4, 5]))))
    total = sum(r["nb"] * 100 * r["H"] ** 2 / 1e6 for r in reqs)
    # warm-up: plans and kernels of every (m, window) used
    for m in (2, 4, 5):
        serve_plain([[blocks100[64][:10]]], [dict(magnification=m)])
    torch.cuda.synchronize(dev)

    def run_served():
        srv = ESRRFServer(n_streams=8, max_active=16)
        handles = [None] * len(reqs)
        events = sorted((r["t"] + k * block_interval, i, k) for i, r in enumerate(reqs)
                        for k in range(r["nb"]))
        t0 = time.perf_counter()

        def feeder():
            for ta, i, k in events:
                dt = t0 + ta - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
                if handles[i] is None:
                    r = reqs[i]
                    handles[i] = srv.submit(r["H"], r["H"], r["nb"], magnification=r["m"])
                srv.push(handles[i], blocks100[reqs[i]["H"]])

        th = threading.Thread(target=feeder)
        th.start()
        th.join()
        for h in handles:
            h.result(timeout=600)
        srv.close()
        t_end = max(h.t_done for h in handles) - t0
        return t_end, [h.latency for h in handles], [h.first_latency for h in handles]

    def run_plain():
        t0 = time.perf_counter()
        lat, first, done = [], [], 0.0
        for r in sorted(reqs, key=lambda r: r["t"]):
            last = r["t"] + (r["nb"] - 1) * block_interval
            dt = t0 + last - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            serve_plain([[blocks100[r["H"]]] * r["nb"]], [dict(magnification=r["m"])])
            done = time.perf_counter() - t0
            lat.append(done - last)
            first.append(done - r["t"])
        return done, lat, first

    t_srv, lat_srv, first_srv = run_served()
    t_pl, lat_pl, first_pl = run_plain()
    pct = lambda a, q: float(np.percentile(np.asarray(a) * 1e3, q))  # noqa: E731

    def stats(t_all, lat, first):
        return {"value": total / t_all, "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99),
                "first_arrival_p50_ms": pct(first, 50), "first_arrival_p99_ms": pct(first, 99)}

    return {"workload": f"{n_requests} requests, Poisson {rate:g}/s, H=W log-uniform 64..1024, "
                        f"1-10 blocks of 100 frames every {block_interval * 1e3:g} ms (each block a "
                        "repeat of one seeded 100-frame block per frame size), m in {2,4,5}, R=1.5, "
                        "s=1, AVG+MPC; latency = last block arrival -> result on host, "
                        "first_arrival = first block arrival -> result on host",
            "mpx_frames": total, "served": stats(t_srv, lat_srv, first_srv),
            "plain": stats(t_pl, lat_pl, first_pl), "unit": "Mpx*frames/s",
            "throughput_ratio": t_pl / t_srv}


def served_blocks(sizes, seed=11, density=0.006):
    from nanopyx_gb300.synthetic import blinking_stack, emitters_for_density

    return {H: blinking_stack(100, H, H, emitters_for_density(H, H, density), seed=seed + H)
            for H in sizes}


def srrf_flops(T, H, W, m):
    """FLOP = sum_frames H W m^2 (12 (2 * 32 + 12) + 20): 12 ring points, two
    16-tap Catmull-Rom interpolations of the gradient (32 FLOP each) and ~12
    FLOP of radiality per point, plus ~20 per output for the intensity and
    normalisation."""
    return T * H * W * m * m * (12.0 * (2 * 32 + 12) + 20.0)


def bench_srrf(dev, stack_np, frames=None, fpt=100, peak=None):
    """SRRF (ring 0.5, 12 ring points, m=5) + per-frame macro-pixel correction
    on the stack, then the order-1 temporal mean per 100-frame timepoint -- the
    reference's SRRF() followed by calculate_SRRF_temporal_correlations, one
    timepoint block at a time on the device."""
    import torch

    import nanopyx_gb300 as nx
    from nanopyx_gb300 import _native as N
    from nanopyx_gb300._device import workspace

    T = stack_np.shape[0] if frames is None else frames
    H, W = stack_np.shape[1:]
    m = 5
    x = torch.from_numpy(np.ascontiguousarray(stack_np[:T])).to(dev)
    blocks = [(a, min(T, a + fpt)) for a in range(0, T, fpt)]

    def one():
        return [nx.calculate_SRRF_temporal_correlations(
            nx.SRRF(x[a:b], magnification=m, ringRadius=0.5), 1) for a, b in blocks]

    one()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    one()
    torch.cuda.synchronize(dev)
    dt = time.perf_counter() - t0
    res = {"workload": f"SRRF {T}x{H}x{W}, m={m}, ring 0.5 (12 points), per-frame MPC, "
                       f"order-1 mean per {fpt}-frame timepoint (device-resident input)",
           "value": T * H * W / 1e6 / dt, "unit": "Mpx*frames/s", "seconds": dt}
    # the fused radiality kernel alone, per timepoint block (CUDA events)
    L = N.lib()
    s = torch.cuda.current_stream(dev)
    nb = max(b - a for a, b in blocks)
    out = torch.empty((nb, H * m, W * m), dtype=torch.float32, device=dev)
    ws = workspace(L.nx_radiality_workspace_bytes(nb, H, W), dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in blocks]
    for (a, b), (e0, e1) in zip(blocks, ev):
        e0.record(s)
        N.check(L.nx_radiality(x[a:b].data_ptr(), None, b - a, H, W, m, 0.5, 0, 1, 1,
                               out.data_ptr(), ws.data_ptr(), ws.numel(), s.cuda_stream),
                "radiality")
        e1.record(s)
    torch.cuda.synchronize(dev)
    kern_ms = sum(e0.elapsed_time(e1) for e0, e1 in ev)
    flops = srrf_flops(T, H, W, m)
    achieved = flops / (kern_ms * 1e-3) / 1e12
    res["roofline"] = {"bound": "fp32", "kernel": "srrf_fused_kernel<5>", "kernel_ms": kern_ms,
                       "flops": flops, "achieved": achieved, "unit": "TFLOP/s",
                       "peak": peak, "frac": (achieved / peak) if peak else None}
    del out, ws
    if cpu_reference_available():
        from oracle import ref_build

        R = ref_build.load()
        smp = np.ascontiguousarray(stack_np[:4])
        R["Radiality"](verbose=False).run(smp[:1], R["CRShiftAndMagnify"](verbose=False).run(
            smp[:1], 0, 0, m, m, run_type="Threaded"), magnification=m, ringRadius=0.5,
            run_type="Threaded")  # warm-up
        t0 = time.perf_counter()
        mag = R["CRShiftAndMagnify"](verbose=False).run(smp, 0, 0, m, m, run_type="Threaded")
        rad = R["Radiality"](verbose=False).run(smp, mag, magnification=m, ringRadius=0.5,
                                                run_type="Threaded")
        R["calculate_SRRF_temporal_correlations"](R["macro_pixel_corrector"](
            rad, magnification=m), 1)
        cdt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": 4 * H * W / 1e6 / cdt, "unit": "Mpx*frames/s",
                               "cores": os.cpu_count(), "kind": "reference",
                               "sample": "4 frames as one timepoint: compiled reference "
                                         "CRShiftAndMagnify + Radiality (Threaded) + "
                                         "macro_pixel_corrector + order-1 mean"}
    return res


def bench_standalone_ops(dev, T=100):
    """HBM throughput of the standalone ops off the fused path: Catmull-Rom
    ShiftAndMagnify (T x 512 x 512, m=5) and the eSRRF temporal correlations
    of a T x 2560 x 2560 stack, against the measured HBM copy bandwidth."""
    import torch

    from nanopyx_gb300 import _native as N

    L = N.lib()
    s = torch.cuda.current_stream(dev)
    H, W, m = 512, 512, 5
    x = torch.rand((T, H, W), device=dev)
    zr = torch.zeros(T, device=dev)
    out = torch.empty((T, H * m, W * m), device=dev)
    stack = torch.rand((T, H * m * W * m), device=dev)
    res = torch.empty(H * m * W * m, device=dev)

    def timeit(f, n=5):
        for _ in range(2):
            f()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(n):
            f()
        e1.record(s)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / n

    try:
        peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except (OSError, KeyError, ValueError):
        peak = 6800.0  # fallback figure for a GB300
    rows = []
    ms = timeit(lambda: N.check(L.nx_cr_shift_magnify(
        x.data_ptr(), T, H, W, zr.data_ptr(), zr.data_ptr(), 5.0, 5.0, out.data_ptr(),
        s.cuda_stream), "cr"))
    b = (x.numel() + out.numel()) * 4
    rows.append({"op": f"cr_shift_magnify {T}x512x512 m=5", "ms": ms, "gbs": b / ms / 1e6})
    # write ceiling of that output: a library fill of the same buffer (torch's
    # own kernel, not ours; reported only to bound the write-dominated op)
    ms = timeit(lambda: out.fill_(1.0))
    rows.append({"op": f"write-only fill of the {T}x2560x2560 output (torch fill_, ceiling)",
                 "ms": ms, "gbs": out.numel() * 4 / ms / 1e6})
    for name, c in (("AVG", 1), ("VAR", 2), ("TAC2", 4)):
        ms = timeit(lambda: N.check(L.nx_temporal_correlation(
            stack.data_ptr(), T, H * m * W * m, c, res.data_ptr(), s.cuda_stream), "tc"))
        b = (stack.numel() + res.numel()) * 4
        rows.append({"op": f"temporal {name} {T}x2560x2560", "ms": ms, "gbs": b / ms / 1e6})
    for r in rows:
        r["frac_of_measured_hbm"] = r["gbs"] / peak
    return {"hbm_peak_gbs": peak, "ops": rows}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--srrf-only", action="store_true",
                    help="only the SRRF measurement (profiling the radiality kernel)")
    ap.add_argument("--srrf-frames", type=int, default=100)
    ap.add_argument("--ops-only", action="store_true",
                    help="only the HBM throughput of the standalone ShiftAndMagnify and "
                         "temporal-correlation kernels")
    ap.add_argument("--ops-frames", type=int, default=100,
                    help="frames of the standalone-op measurement")
    ap.add_argument("--scored-sweep-only", action="store_true",
                    help="only the scored parameter sweep (RSP / FRC / QnR)")
    ap.add_argument("--esrrf3d-only", action="store_true", help="only the eSRRF-3D measurement")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the uneven-batch, sweep and served-stream measurements")
    ap.add_argument("--served-requests", type=int, default=200,
                    help="requests per arrival rate of the served-stream measurement")
    ap.add_argument("--served-rates", type=float, nargs="*", default=None,
                    help="arrival rates (requests/s) of the served-stream measurement")
    ap.add_argument("--workload", default="large", choices=["large", "small"],
                    help="small: 160 frames, 80 per timepoint (for ncu captures)")
    args = ap.parse_args()
    if args.workload == "small":
        CFG.update(SMALL)
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.ops_only:
        import torch

        torch.cuda.set_device(0)
        print(json.dumps(bench_standalone_ops(torch.device("cuda", 0), T=args.ops_frames)),
              flush=True)
        return 0
    if args.scored_sweep_only or args.esrrf3d_only:
        import torch

        torch.cuda.set_device(0)
        dev = torch.device("cuda", 0)
        fn = bench_scored_sweep if args.scored_sweep_only else bench_esrrf3d
        print(json.dumps(fn(dev, with_reference=not args.no_cpu_baseline)), flush=True)
        return 0
    if args.srrf_only:
        import torch

        from nanopyx_gb300.synthetic import blinking_stack

        torch.cuda.set_device(0)
        st = blinking_stack(args.srrf_frames, CFG["H"], CFG["W"], CFG["emitters"], seed=CFG["seed"])
        dev = torch.device("cuda", 0)
        peak = max(measure_fp32_peak(dev), measure_fp32_peak(dev, packed=True))
        print(json.dumps(bench_srrf(dev, st, frames=args.srrf_frames, peak=peak)), flush=True)
        return 0
    return run_gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
