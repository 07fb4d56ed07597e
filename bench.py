"""Benchmark: frames/s of the structure-factor chain at 256x256x128, 200k atoms.

Workload (one step): the seeded columnar system -- 200,000 atoms in a
16.0 x 13.856 x 8.0 nm box, 100 frames of float32 positions (320 MB as
float4, more than L2) -- through histogram deposit -> R2C FFT -> |F|^2 ->
FP64 frame sum, then get_dplot and the Ewald slices at lambda = 0.154 nm.

  value       frames/s of the step captured once in a CUDA graph and replayed,
              inputs resident in HBM.
  e2e         the same step through the public API from pinned HOST buffers:
              H2D of the step's positions (streamed on a side stream), the
              chain, get_dplot, the Ewald slices, and the D2H of sf and of the
              three slices, all inside the timed region.
  roofline    the dominant kernel, timed live with CUDA events over a pass
              of the same workload driven stage by stage.
  cpu_baseline the numpy oracle (histogramdd + rfftn, one core) on a bounded
              sample of frames of the same workload.
  config.errors  max and RMS error of S(q) / max(S) against the FP64 numpy
              oracle for the five workloads (the headline on the very sf the
              timed step produced), computed after the timing in a spawn
              pool on the host cores.

The plan's tuning comes from the autotuner (mdsf.tune): the cached tuning of
the grid shape on this GPU, tuned at start-up when the cache has none; the
line says which (``tuning``).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
N>1 runs under torchrun: every rank processes its own trajectory (frames
shard with no exchange until one FP64 sum of sf per step).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "md-structure-factor_gb300"))
sys.path.insert(0, ROOT)

DIMS = (256, 256, 128)
N_ATOMS = 200_000
FRAMES = 100
BOX = (16.0, 13.856, 8.0)
WAVELENGTH = 0.154
METRIC = "frames/s at 256^2x128 grid, 200k atoms (batched, graph-captured hist->FFT->|F|^2->FP64 sum)"
WORKLOAD = ("columnar 200k atoms, 16.0x13.856x8.0 nm, 256x256x128 grid, 100 frames/step, f32 positions, "
            "get_dplot + Ewald lambda=0.154 nm")
# source-level FP32 operation counts of one (atom, q) pair of the direct sum
# (msf_direct.cu): the phase in turns from hi + lo parts of q/2pi with FMA
# residuals (3 x [FMUL, 2 FFMA, FRND, 2 FADD], 2 FADD), the turn-based
# sin/cos whose quadrant rounding also removes the whole turns (FMUL, FRND,
# FFMA, FMUL, 4 + 4 polynomial FMA/FMUL, F2I, LOP, 2 selects, 2 sign selects:
# 17), then the accumulation (forward: 2 FFMA and the grouped compensated
# sum, ~0.5 per pair; adjoint: the weight, 3 gradient and 2 weight-gradient
# FMAs: 7)
DIRECT_FP32_OPS = {"fwd": 39.5, "bwd": 44}
SM_COUNT_FALLBACK = 152
FP32_LANES_PER_SM = 128


def config(world):
    """The workload description both arms print (identical by construction)."""
    return {"workload": WORKLOAD, "frames_per_step": FRAMES, "n_atoms": N_ATOMS, "grid": list(DIMS),
            "l2": "inputs larger than L2 (320 MB of float4 positions per step)",
            "arithmetic": "int32 grid (FP32 binning exact vs FP64 edges), FP32 FFT, FP64 frame sum",
            "parallelism": f"frames sharded x{world}"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def algorithmic_bytes_per_frame(n_atoms=N_ATOMS, dims=DIMS):
    V = dims[0] * dims[1] * dims[2]
    Vh = dims[0] * dims[1] * (dims[2] // 2 + 1)
    return 16 * n_atoms + 8 * V + 16 * Vh


def moved_bytes_per_frame(n_atoms=N_ATOMS, dims=DIMS, batch=64):
    """Bytes the bucketed chain moves per frame: positions, bucket entries
    written / read / compacted (8 B each way), the half spectrum written and
    read once, and the FP64 sf read + written once per kPowerFlush-capped
    pass of `batch` frames."""
    Vh = dims[0] * dims[1] * (dims[2] // 2 + 1)
    flushes = -(-batch // 32)
    return 16 * n_atoms + 32 * n_atoms + 16 * Vh + 16 * Vh * flushes / batch


# ------------------------------------------------------------------ clocks
class Clocks:
    """SM clock, power and clock-event reasons sampled every 10 ms through
    NVML (read-only queries, libnvidia-ml via ctypes) while the timed region
    runs; nvidia-smi at 100 ms when NVML cannot be opened."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, torch, dev, period=0.01):
        self.period = period
        self.samples = []
        self.nv = None
        self.handle = None
        self.smi = None
        self.t0 = self.t1 = None
        try:
            nv = ctypes.CDLL("libnvidia-ml.so.1")
            if nv.nvmlInit_v2() != 0:
                raise OSError("nvmlInit failed")
            h = ctypes.c_void_p()
            ok = False
            try:
                uuid = "GPU-" + str(torch.cuda.get_device_properties(dev).uuid)
                ok = nv.nvmlDeviceGetHandleByUUID(uuid.encode(), ctypes.byref(h)) == 0
            except Exception:
                ok = False
            if not ok:
                cnt = ctypes.c_uint()
                nv.nvmlDeviceGetCount_v2(ctypes.byref(cnt))
                idx = dev.index if cnt.value > 1 else 0
                ok = nv.nvmlDeviceGetHandleByIndex_v2(idx, ctypes.byref(h)) == 0
            if not ok:
                raise OSError("no NVML handle")
            self.nv, self.handle = nv, h
            mx = ctypes.c_uint()
            self.max_mhz = float(mx.value) if nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0 else None
            self._reasons = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                nv.nvmlDeviceGetCurrentClocksThrottleReasons
        except Exception:
            self.nv = None

    def _sample(self):
        mhz, mw, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        self.nv.nvmlDeviceGetClockInfo(self.handle, 1, ctypes.byref(mhz))
        self.nv.nvmlDeviceGetPowerUsage(self.handle, ctypes.byref(mw))
        self._reasons(self.handle, ctypes.byref(rs))
        return time.time(), float(mhz.value), mw.value / 1000.0, int(rs.value)

    def _loop(self):
        while not self._stop.is_set():
            try:
                self.samples.append(self._sample())
            except Exception:
                return
            self._stop.wait(self.period)

    def start(self):
        self.samples = []
        if self.nv is not None:
            self._stop = threading.Event()
            self._th = threading.Thread(target=self._loop, daemon=True)
            self._th.start()
        else:
            self.path = os.path.join(tempfile.gettempdir(), "clocks_bench.csv")
            try:
                self.f = open(self.path, "w")
                self.smi = subprocess.Popen(
                    ["nvidia-smi", "--query-gpu=timestamp,clocks.sm,clocks.max.sm,power.draw,"
                     "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                     "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                     "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
                time.sleep(0.2)
            except Exception:
                self.smi = None
        self.t0 = time.time()

    def stop(self):
        self.t1 = time.time()
        if self.nv is not None:
            self._stop.set()
            self._th.join()
        elif self.smi is not None:
            time.sleep(0.15)
            self.smi.terminate()
            self.smi.wait()
            self.f.close()

    def summary(self):
        sm, pw, reasons = [], [], set()
        mx = None
        if self.nv is not None:
            mx = self.max_mhz
            for t, mhz, w, rs in self.samples:
                sm.append(mhz)
                pw.append(w)
                reasons |= {n for bit, n in self.REASONS.items() if rs & bit}
            source = "nvml, 10 ms"
        elif self.smi is not None:
            import datetime
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 8:
                    continue
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                if not self.t0 <= ts <= self.t1:
                    continue
                sm.append(float(f[1]))
                mx = float(f[2])
                pw.append(float(f[3]))
                reasons |= {n for n, v in zip(names, f[4:8]) if v.lower().startswith("active")}
            source = "nvidia-smi, 100 ms"
        else:
            return None
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "samples": 0, "reasons": [], "source": source}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "samples": len(sm), "sm_mhz_min": min(sm),
                "power_w_max": max(pw) if pw else None, "reasons": sorted(reasons), "source": source}


# ------------------------------------------------------------- reference arm
def _ref_worker(args):
    seed, frames = args
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    from mdsf import synth
    from oracle import hist as ohist
    pos, box, w = synth.columnar(n_atoms=N_ATOMS, box=BOX, frames=frames, seed=seed)
    t0 = time.perf_counter()
    sf = np.zeros((DIMS[0], DIMS[1], DIMS[2] // 2 + 1))
    for t in range(frames):
        sf += ohist.power(ohist.hist_grid(pos[t], box, w, DIMS))
    return frames, time.perf_counter() - t0, float(sf[0, 0, 0])


def run_reference(args):
    """--impl reference: the reference's CPU method (the oracle port: the
    reference is pure Python and cannot run on the GPU host) on all host cores."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return 0
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    frames_per_worker = 2
    ctx = mp.get_context("spawn")
    times = []
    with ctx.Pool(cores) as pool:
        for step in range(args.warmup + args.steps):
            res = pool.map(_ref_worker, [(1000 + step * cores + i, frames_per_worker) for i in range(cores)])
            # workers run side by side; the step lasts as long as the slowest
            # worker's compute (input generation is outside each worker's clock)
            dt = max(r[1] for r in res)
            if step >= args.warmup:
                times.append((sum(r[0] for r in res), dt))
    frames = sum(t[0] for t in times)
    total = sum(t[1] for t in times)
    value = frames / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded columnar system (no dataset in the reference)",
            "config": config(world),
            "cpu_baseline": {"value": value, "unit": "frames/s", "cores": cores, "kind": "port",
                             "sample": f"{frames_per_worker} frames per process per step, {cores} spawn processes, "
                                       "numpy histogramdd + numpy.fft.rfftn + |F|^2 + FP64 sum (the reference has no "
                                       "GPU-host-runnable code: it is pure Python and absent on the GPU host)"},
            "e2e": {"value": value, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------- CPU side
def cpu_port_baseline(pos, box, w, budget_s=12.0, min_frames=2):
    """Oracle port (numpy histogramdd + rfftn + |F|^2, FP64) on one core."""
    from oracle import hist as ohist
    sf = np.zeros((DIMS[0], DIMS[1], DIMS[2] // 2 + 1))
    t0 = time.perf_counter()
    n = 0
    while n < pos.shape[0] and (n < min_frames or time.perf_counter() - t0 < budget_s):
        sf += ohist.power(ohist.hist_grid(pos[n], box, w, DIMS))
        n += 1
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": "frames/s", "cores": 1, "kind": "port",
            "sample": f"{n} frames of the same workload, numpy histogramdd + numpy.fft.rfftn + |F|^2 + FP64 sum, "
                      f"single thread ({dt:.1f} s)"}


def _errors(got, ref):
    m = float(np.abs(ref).max())
    return {"max": float(np.abs(got - ref).max() / m), "rms": float(np.sqrt(np.mean((got - ref) ** 2)) / m)}


def pool_hist_sf(pool, jobs, frames_per_job=8):
    """FP64 oracle sums of several (pos, box, w, dims) systems, frames split
    over the pool."""
    from oracle import hist as ohist
    tasks, owner = [], []
    for i, (pos, box, w, dims) in enumerate(jobs):
        for a in range(0, pos.shape[0], frames_per_job):
            tasks.append((np.ascontiguousarray(pos[a:a + frames_per_job]), np.asarray(box), w, tuple(dims)))
            owner.append(i)
    parts = pool.starmap(ohist.hist_sf, tasks, chunksize=1)
    out = [None] * len(jobs)
    for i, p in zip(owner, parts):
        out[i] = p if out[i] is None else out[i] + p
    return out


# ----------------------------------------------------------------- tuning
def resolve_tuning(args, dev):
    """(plan tuning, record): command-line knobs, else the autotuner's
    cached tuning of DIMS on this GPU, tuned now when the cache has none."""
    explicit = {}
    if args.batch:
        explicit["batch"] = args.batch
    if args.variant:
        explicit["variant"] = args.variant
    if args.tile_w:
        explicit["tile_w"] = args.tile_w
    if args.no_overlap:
        explicit["options"] = 1
    if explicit:
        return explicit, {"source": "command line"}
    if args.no_tune:
        return {}, {"source": "plan defaults (--no-tune)"}
    from mdsf import tune
    source = "autotuner cache"
    t0 = time.perf_counter()
    if tune.lookup(DIMS) is None:
        tune.tune(DIMS, n_atoms=N_ATOMS, frames=128, device=dev)
        source = "autotuned at start-up"
    e = tune.entry(DIMS)
    rec = {"source": source, "cache_key": tune.key(DIMS), "cache": tune.cache_path(),
           "candidates_timed": e["tried"], "ms_per_frame_tuned": e["ms_per_frame"],
           "tuning_s": time.perf_counter() - t0,
           "runner_up": e["results"][1] if len(e.get("results", [])) > 1 else None}
    return dict(e["tuning"]), rec


# ------------------------------------------------------------------- main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 200 for the chain; 5 for --impl reference; 3 for --batched-only)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=0)
    ap.add_argument("--variant", type=int, default=0)
    ap.add_argument("--tile-w", type=int, default=0)
    ap.add_argument("--no-overlap", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="plan defaults instead of the autotuner's tuning")
    ap.add_argument("--post-only", action="store_true",
                    help="only the post-processing rows (radial, (r, z) histograms, nearest node)")
    ap.add_argument("--zero-copy", action="store_true",
                    help="e2e: the kernels read the pinned host positions in place instead of staged copies")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--no-errors", action="store_true", help="skip the per-configuration oracle errors")
    ap.add_argument("--stream-chunk", type=int, default=0,
                    help="frames per host->device chunk of the e2e path (0: the API default: a quarter-batch lead chunk, then near-equal chunks of at most one batch)")
    ap.add_argument("--stress-only", action="store_true",
                    help="only the 512^3 stress grid (1M atoms, 200 frames from pinned host memory)")
    ap.add_argument("--stress-frames", type=int, default=200)
    ap.add_argument("--batched-only", action="store_true",
                    help="only the 64 uneven batched systems (one graph, 2 warm-up + `--steps` replays)")
    ap.add_argument("--direct-only", action="store_true", help="only the direct-sum forward + adjoint")
    ap.add_argument("--gauss-only", action="store_true", help="only the Gaussian drop-in (water box, 64^3)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.steps is None:
        args.steps = 5 if args.impl == "reference" else (3 if args.batched_only or args.stress_only else 200)
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import torch.distributed as dist

    import mdsf
    from mdsf import synth
    from mdsf._lib import c_p, call
    from mdsf.api import _ptr

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.batched_only:
        print(json.dumps({"metric": "batched systems frames/s (64 uneven systems, one graph)",
                          **batched_systems(torch, dev, args.steps)}))
        return 0
    if args.stress_only:
        print(json.dumps({"metric": "frames/s of the 512^3 stress grid (1M atoms, streamed from host)",
                          **stress_512(torch, dev, frames=args.stress_frames, steps=args.steps)}))
        return 0
    if args.direct_only:
        print(json.dumps({"metric": "direct-sum forward + adjoint", **direct_extra(torch, dev)}))
        return 0
    if args.gauss_only:
        print(json.dumps({"metric": "Gaussian drop-in compute_sf frames/s", **gauss_extra(torch, dev)}))
        return 0
    if args.post_only:
        return run_post_only(torch, dev, args)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    pos, box, w = synth.columnar(n_atoms=N_ATOMS, box=BOX, frames=FRAMES, seed=2 + 7919 * rank)
    pos4_h = torch.from_numpy(synth.pack_float4(pos, w)).pin_memory()
    pos4 = pos4_h.to(dev)
    tuning, tuning_rec = resolve_tuning(args, dev)
    plan = mdsf.get_plan(DIMS, box, device=dev, max_atoms=N_ATOMS, **tuning)
    tuning_rec["plan"] = plan.tuning()
    st = torch.cuda.current_stream(dev)
    sf = torch.zeros(plan.half_shape, dtype=torch.float64, device=dev)
    X, Y, Z = mdsf.plot_axes(plan.half_shape, box)
    Xd, Yd, Zd = (torch.from_numpy(a).to(dev) for a in (X, Y, Z))
    D = torch.empty((DIMS[0] - 2, DIMS[1] - 2, 2 * plan.nh - 3), dtype=torch.float64, device=dev)
    ew = [torch.empty(s, dtype=torch.float64, device=dev) for s in
          ((D.shape[0], D.shape[1]), (D.shape[0], D.shape[2]), (D.shape[1], D.shape[2]))]
    K = 2.0 * np.pi / WAVELENGTH

    def post(out, sp):
        call("msf_sfplt", _ptr(out), DIMS[0], DIMS[1], plan.nh, _ptr(D), sp)
        call("msf_ewald", _ptr(D), D.shape[0], D.shape[1], D.shape[2], _ptr(Xd), _ptr(Yd), _ptr(Zd), K,
             _ptr(ew[0]), _ptr(ew[1]), _ptr(ew[2]), sp)

    def step_body():
        sf.zero_()
        sp = c_p(torch.cuda.current_stream(dev).cuda_stream)   # the capture stream inside graph capture
        call("msf_hist_sf_f32", plan.handle, _ptr(pos4), N_ATOMS, FRAMES, c_p(0), 0, _ptr(sf), sp)
        if world > 1:
            dist.all_reduce(sf)
        post(sf, sp)

    batches = (FRAMES + plan.batch - 1) // plan.batch
    launches_per_step = batches * {1: 3, 2: 4, 3: 5, 4: 4}[plan.variant] + 2

    # warm-up (also primes one-time kernel attributes before graph capture)
    for _ in range(2):
        step_body()
    torch.cuda.synchronize()
    graph = None
    if world == 1:
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            step_body()
        run = graph.replay
    else:
        run = step_body
    for _ in range(args.warmup):
        run()
    torch.cuda.synchronize()

    def timed(fn, steps, join=()):
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        for js in join:   # the end event follows the work of these streams too
            torch.cuda.current_stream().wait_stream(js)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        if world > 1:
            t = torch.tensor([ms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
            dist.barrier()
        return ms

    clk = Clocks(torch, dev)
    clk.start()
    ms = timed(run, args.steps)
    clk.stop()
    clocks = clk.summary()
    ms_per_step = ms / args.steps
    value = FRAMES * world * args.steps / (ms / 1000.0)
    # the timed output: sf of the last replayed step (100 frames), checked
    # below against the oracle (config.errors) and here by its DC term
    sf_timed = sf.cpu().numpy()
    dc_ref = FRAMES * world * float(np.sum(w, dtype=np.float64)) ** 2
    assert abs(sf_timed[0, 0, 0] - dc_ref) < 1e-5 * dc_ref, (sf_timed[0, 0, 0], dc_ref)

    # ---- e2e: public API from pinned host buffers, then get_dplot + Ewald on
    # the device, D2H of sf and of the three slices in the timed region
    sf_h = torch.empty(plan.half_shape, dtype=torch.float64).pin_memory()
    ew_h = [torch.empty(t.shape, dtype=torch.float64).pin_memory() for t in ew]
    d2h_stream = torch.cuda.Stream(dev)

    def e2e_step():
        out = mdsf.structure_factor(pos4_h, box, None, DIMS, device=dev, tuning=tuning,
                                    stream_chunk=args.stream_chunk or None, zero_copy=args.zero_copy)
        if world > 1:
            dist.all_reduce(out)
        post(out, c_p(torch.cuda.current_stream(dev).cuda_stream))
        # the read-back on its own stream, so that the next step's kernels do
        # not queue behind it (the timed region ends after it)
        done = torch.cuda.Event()
        done.record()
        with torch.cuda.stream(d2h_stream):
            d2h_stream.wait_event(done)
            sf_h.copy_(out, non_blocking=True)
            for h, d in zip(ew_h, ew):
                h.copy_(d, non_blocking=True)
            out.record_stream(d2h_stream)
    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    clk_e = Clocks(torch, dev)
    clk_e.start()
    ms_e2e = timed(e2e_step, args.steps, join=(d2h_stream,))
    clk_e.stop()
    e2e_value = FRAMES * world * args.steps / (ms_e2e / 1000.0)

    # ---- roofline: each stage timed live with events around its launches
    stage_ms = {1: [], 2: [], 4: []}
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    sf.zero_()
    sp = c_p(st.cuda_stream)
    torch.cuda.synchronize()
    for f0 in range(0, FRAMES, plan.batch):
        k = min(plan.batch, FRAMES - f0)
        p = c_p(pos4.data_ptr() + f0 * N_ATOMS * 16)
        ev[0].record()
        call("msf_hist_batch_stages", plan.handle, 1, 0, p, c_p(0), N_ATOMS, k, c_p(0), 0, _ptr(sf), sp)
        ev[1].record()
        call("msf_hist_batch_stages", plan.handle, 2, 0, p, c_p(0), N_ATOMS, k, c_p(0), 0, _ptr(sf), sp)
        ev[2].record()
        call("msf_hist_batch_stages", plan.handle, 4, 0, p, c_p(0), N_ATOMS, k, c_p(0), 0, _ptr(sf), sp)
        ev[3].record()
        torch.cuda.synchronize()
        for s, (a, b) in zip((1, 2, 4), ((0, 1), (1, 2), (2, 3))):
            stage_ms[s].append((ev[a].elapsed_time(ev[b]), k))
    V = DIMS[0] * DIMS[1] * DIMS[2]
    Vh = DIMS[0] * DIMS[1] * plan.nh
    B = plan.batch
    # compulsory bytes of each stage for one launch of `k` frames
    if plan.variant == 3:
        stage_bytes = {
            # positions read, bucket entries written, then read and written once more compacted
            1: lambda k: 16 * N_ATOMS * k + 8 * N_ATOMS * k + 16 * N_ATOMS * k,
            2: lambda k: 8 * N_ATOMS * k + 8 * Vh * k,              # bucket read, spectrum written
            4: lambda k: 8 * Vh * k + 16 * Vh * -(-k // 32),       # spectrum read, sf read + written per 32 frames
        }
        stage_names = {1: "k_bucket_sort+scan+compact", 2: "k_plane_ct",
                       4: "k_xpower_tma" if plan.tma else "k_xpower_ct"}
    else:
        stage_bytes = {
            1: lambda k: 16 * N_ATOMS * k + 4 * V * k,             # positions read, grid written
            2: lambda k: 4 * V * k + 4 * V * k + 8 * Vh * k,        # grid read, grid zeroed, spectrum written
            4: lambda k: 8 * Vh * k + 16 * Vh * -(-k // 32),       # spectrum read, sf read + written per 32 frames
        }
        stage_names = {1: "k_hist_deposit", 2: {1: "k_plane", 2: "k_zrows+k_ycols", 4: "k_zs+k_ys"}[plan.variant],
                       4: "k_xs" if plan.variant == 4 else "k_xpower"}
    totals = {s: sum(t for t, _ in v) for s, v in stage_ms.items()}
    dom = max(totals, key=totals.get)
    full = [(t, k) for t, k in stage_ms[dom] if k == B] or stage_ms[dom]
    avg_ms = float(np.mean([t for t, _ in full]))
    kfull = full[0][1]
    achieved = stage_bytes[dom](kfull) / (avg_ms / 1000.0) / 1e9
    peak, peak_kind = peaks()
    # DRAM bytes per launch of the dominant kernel from the committed ncu
    # capture of this workload (profiles/dram_traffic.txt), when it matches
    # (a capture at another frame count per launch is scaled by the frames: the
    # kernel's traffic is per frame plus nothing per launch)
    traffic, traffic_note = None, None
    try:
        with open(os.path.join(ROOT, "profiles", "dram_traffic.txt")) as f:
            rows = [ln.split() for ln in f if not ln.startswith("#")]
        rows = [r for r in rows if len(r) == 4 and r[0] == stage_names[dom] and r[1] == "x".join(map(str, DIMS))]
        exact = [r for r in rows if int(r[2]) == kfull]
        if exact:
            traffic = int(exact[0][3])
        elif rows:
            r = max(rows, key=lambda r: int(r[2]))
            traffic = int(int(r[3]) * kfull / int(r[2]))
            traffic_note = f"ncu capture at {r[2]} frames per launch, scaled to {kfull}"
    except (OSError, ValueError):
        pass
    chain_gbs = algorithmic_bytes_per_frame() * value / world / 1e9
    moved_gbs = moved_bytes_per_frame(batch=B) * value / world / 1e9 if plan.variant == 3 else None

    extras = {}
    if not args.no_extras and rank == 0:
        extras = run_extras(mdsf, torch, dev, pos4, box, args)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_port_baseline(pos, box, w)

    errors = None
    if rank == 0 and not args.no_errors:
        errors = config_errors(torch, dev, sf_timed, pos, box, w, extras.get("_direct_S"))
    extras.pop("_direct_S", None)

    if rank == 0:
        cfg = config(world)
        if errors is not None:
            cfg["errors"] = errors
        line = {
            "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded columnar system (no dataset in the reference)",
            "config": cfg,
            "tuning": tuning_rec, "graph": world == 1,
            "roofline": {"bound": "hbm", "kernel": stage_names[dom], "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": traffic, "traffic_note": traffic_note,
                         "peak_kind": peak_kind, "avg_launch_ms": avg_ms, "frames_per_launch": kfull,
                         "stage_ms_per_frame": {stage_names[s]: totals[s] / FRAMES for s in totals},
                         "chain_algorithmic_gbs": chain_gbs, "chain_frac": chain_gbs / peak,
                         "chain_moved_gbs": moved_gbs, "chain_moved_frac": moved_gbs / peak if moved_gbs else None},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "frames/s", "h2d_bytes_per_step": int(pos4_h.numel() * 4),
                    "d2h_bytes_per_step": int(sf_h.numel() * 8 + sum(h.numel() * 8 for h in ew_h)),
                    "work": "structure_factor (chain) + get_dplot + Ewald slices, sf and slices read back",
                    "h2d": ("kernels read the pinned host positions in place (mapped memory, NVLink-C2C)"
                            if args.zero_copy else "chunked copies from pinned host memory on a side stream"),
                    "clocks": clk_e.summary()},
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clocks,
            "extras": extras,
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()
    return 0


# ------------------------------------------------------------------ errors
def config_errors(torch, dev, sf_timed, pos, box, w, direct_S=None):
    """Max and RMS error of S(q) / max(S) against the FP64 oracle, per
    workload, computed in a spawn pool on the host cores."""
    import multiprocessing as mp
    from mdsf import synth
    import mdsf
    out = {}
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(max(1, min(16, os.cpu_count() or 1))) as pool:
        jobs, names, gots = [], [], []
        # configuration 2: the very sf the timed graph replay produced
        jobs.append((pos, box, w, DIMS))
        names.append("config2")
        gots.append(sf_timed)
        # configuration 1: 1,500 waters, 10 float64 frames, 64^3
        p1, b1, w1 = synth.water_box(n_waters=1500, L=2.5, frames=10, seed=1)
        gots.append(mdsf.structure_factor(p1, b1, w1, (64, 64, 64), device=dev).cpu().numpy())
        jobs.append((p1, b1, w1, (64, 64, 64)))
        names.append("config1")
        # configuration 3: 8 of the 64 uneven systems (the largest atom count
        # and grid among them), 2 frames each, one graph
        from mdsf.batch import BatchedSystems, random_batch
        systems = random_batch(64, seed=5, device=dev)
        pick = sorted(set([max(range(64), key=lambda i: systems[i]["pos_w"].shape[1]),
                           max(range(64), key=lambda i: int(np.prod(systems[i]["dims"])))] + list(range(6))))
        sub = [dict(systems[i], pos_w=systems[i]["pos_w"][:2].contiguous()) for i in pick]
        del systems
        b = BatchedSystems(sub, n_streams=4, device=dev)
        b.run()
        for i, s in enumerate(sub):
            p = s["pos_w"].cpu().numpy()
            jobs.append((p[..., :3], np.asarray(s["box"], np.float64), p[0, :, 3].astype(np.int32), tuple(s["dims"])))
            names.append("config3")
            gots.append(b.sf[i].cpu().numpy())
        del b, sub
        # configuration 5: 1M atoms, 512^3, 2 frames
        p5, b5, w5 = synth.columnar(n_atoms=1_000_000, box=(25.0, 25.0, 25.0), n_cols=(6, 6), lattice=25.0 / 6,
                                    frames=2, seed=11)
        gots.append(mdsf.structure_factor(synth.pack_float4(p5, w5), b5, None, (512, 512, 512),
                                          device=dev).cpu().numpy())
        jobs.append((p5, b5, w5, (512, 512, 512)))
        names.append("config5")
        torch.cuda.empty_cache()
        refs = pool_hist_sf(pool, jobs, frames_per_job=8)
        agg = {}
        for n, g, r in zip(names, gots, refs):
            e = _errors(g, r)
            a = agg.setdefault(n, {"max": 0.0, "rms": 0.0})
            a["max"], a["rms"] = max(a["max"], e["max"]), max(a["rms"], e["rms"])
        out.update(agg)
        out["config1"]["sample"] = "the whole workload (10 frames)"
        out["config2"]["sample"] = "the sf of the timed step (100 frames, two 50-frame batches)"
        out["config3"]["sample"] = (f"{len(pick)} of the 64 systems (incl. the most atoms and the largest grid), "
                                    "2 frames each, one graph; worst system")
        out["config5"]["sample"] = "2 frames of the 1M-atom system on 512^3"
        # configuration 4: the direct sum of system 0 of the bench's batch, on
        # every 16th q vector (4,096), against the FP64 direct sum
        if direct_S is not None:
            from oracle import direct as odirect
            r, f, q, S = direct_S
            sel = np.arange(0, len(q), 16)
            parts = pool.starmap(odirect.amplitudes, [(r, f, q[sel[a:a + 256]]) for a in range(0, len(sel), 256)],
                                 chunksize=1)
            A = np.concatenate([p[0] for p in parts])
            Bv = np.concatenate([p[1] for p in parts])
            S64 = A * A + Bv * Bv
            e = _errors(S[sel], S64)
            e["norm"] = float(np.linalg.norm(S[sel] - S64) / np.linalg.norm(S64))
            e["sample"] = "system 0 of the 32, every 16th of the 65,536 q vectors, forward S(q) in FP32"
            out["config4"] = e
    out["seconds"] = time.perf_counter() - t0
    return out


# ------------------------------------------------------------------ extras
def run_extras(mdsf, torch, dev, pos4, box, args):
    """Plain one-frame-per-launch path, the direct sum, the Gaussian drop-in,
    the batched uneven systems, the 512^3 stress grid and the post-processing
    rows."""
    from mdsf._lib import c_p, call
    from mdsf.api import _ptr
    out = {}
    plan1 = mdsf.get_plan(DIMS, box, device=dev, batch=1, max_atoms=N_ATOMS)
    sf = torch.zeros(plan1.half_shape, dtype=torch.float64, device=dev)
    st = torch.cuda.current_stream(dev)

    def plain_step():
        sp = c_p(st.cuda_stream)
        for t in range(FRAMES):
            call("msf_hist_sf_f32", plan1.handle, c_p(pos4.data_ptr() + t * N_ATOMS * 16), N_ATOMS, 1, c_p(0), 0,
                 _ptr(sf), sp)
            torch.cuda.synchronize()
    plain_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plain_step()
    torch.cuda.synchronize()
    out["plain_frames_per_s"] = FRAMES / (time.perf_counter() - t0)
    out["plain_note"] = "plan batch=1, one host call + synchronize per frame, no graph"
    del plan1, sf

    out.update(direct_extra(torch, dev, keep=out))
    out.update(gauss_extra(torch, dev))
    out.update(batched_systems(torch, dev, 2, prefix="batched_systems_"))
    torch.cuda.empty_cache()
    out.update(stress_512(torch, dev, frames=args.stress_frames, prefix="stress_512_"))
    out.update(radial_extra(torch, dev))
    out.update(rz_extra(torch, dev))
    out.update(nearest_extra(torch, dev))
    out.update(gro_ingest())
    return out


def _sm_count(torch, dev):
    try:
        return torch.cuda.get_device_properties(dev).multi_processor_count
    except Exception:
        return SM_COUNT_FALLBACK


def direct_extra(torch, dev, keep=None):
    """Direct sum at the differentiable workload's size: 32 systems x 20,000
    atoms (6 nm cube) x 65,536 q (three Ewald-sphere slices + a 5-15 nm^-1
    shell), target from positions perturbed by 0.05 nm, loss MSE(log1p S).
    Forward and adjoint timed separately with CUDA events; each rate against
    the FP32-issue and MUFU ceilings of the SMs at the sampled clock."""
    import mdsf
    from mdsf import synth
    S_, N = 32, 20_000
    rs, fs, ts = zip(*[synth.direct_system(N, 6.0, seed=100 + s) for s in range(S_)])
    q_np = synth.ewald_q_set(65_536)
    M = len(q_np)
    r = torch.from_numpy(np.stack(rs)).to(dev)
    f = torch.from_numpy(np.stack(fs)).to(dev)
    q = torch.from_numpy(q_np).to(dev)
    with torch.no_grad():
        target = mdsf.direct_sf(torch.from_numpy(np.stack(ts)).to(dev), f, q)

    def fwd():
        return mdsf.direct_sf(rr, f, q)
    rr = r.clone().requires_grad_(True)
    S = fwd()
    loss = torch.mean((torch.log1p(S) - torch.log1p(target)) ** 2, dim=-1).sum()
    g, = torch.autograd.grad(loss, rr)
    torch.cuda.synchronize()
    reps = 3
    clk = Clocks(torch, dev)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    fwd_ms = bwd_ms = tot_ms = 0.0
    clk.start()
    for _ in range(reps):
        e[0].record()
        S = fwd()
        e[1].record()
        loss = torch.mean((torch.log1p(S) - torch.log1p(target)) ** 2, dim=-1).sum()
        e[2].record()
        g, = torch.autograd.grad(loss, rr)
        e[3].record()
        torch.cuda.synchronize()
        fwd_ms += e[0].elapsed_time(e[1])
        bwd_ms += e[2].elapsed_time(e[3])
        tot_ms += e[0].elapsed_time(e[3])
    clk.stop()
    c = clk.summary() or {}
    mhz = c.get("sm_mhz") or c.get("sm_max_mhz") or 2070.0
    sms = _sm_count(torch, dev)
    pairs = S_ * N * M
    res = {"grad_evals_per_s": S_ / (tot_ms / reps / 1000.0),
           "grad_note": f"systems/s: forward + loss + adjoint of {S_} systems x {N} atoms x {M} q per launch pair",
           "direct_pairs_per_s": 2 * pairs / (tot_ms / reps / 1000.0)}
    for name, ms in (("fwd", fwd_ms / reps), ("bwd", bwd_ms / reps)):
        rate = pairs / (ms / 1000.0)
        fp32_ceiling = sms * FP32_LANES_PER_SM * mhz * 1e6 / DIRECT_FP32_OPS[name]
        res[f"direct_{name}_pairs_per_s"] = rate
        res[f"direct_{name}_frac_fp32_issue"] = rate / fp32_ceiling
    res["direct_roofline_note"] = (
        f"ceiling at {mhz:.0f} MHz x {sms} SMs: FP32 issue = 128 lanes/SM / FP32 ops per pair "
        f"({DIRECT_FP32_OPS['fwd']} forward, {DIRECT_FP32_OPS['bwd']} adjoint, source-level count; sin/cos are "
        f"polynomials in turns on the FP32 pipe, no SFU)")
    # one system alone (config 4's base case): the kernels switch to smaller
    # blocks so that 20k atoms / 65,536 q still cover the SMs
    r1 = r[0].clone().requires_grad_(True)
    f1, t1 = f[0], target[0]

    def one():
        S1 = mdsf.direct_sf(r1, f1, q)
        l1 = torch.mean((torch.log1p(S1) - torch.log1p(t1)) ** 2)
        return torch.autograd.grad(l1, r1)[0]
    one()
    torch.cuda.synchronize()
    e[0].record()
    for _ in range(reps):
        one()
    e[1].record()
    torch.cuda.synchronize()
    res["grad_evals_single_system_per_s"] = reps / (e[0].elapsed_time(e[1]) / 1000.0)
    if keep is not None:
        keep["_direct_S"] = (rs[0], fs[0], q_np, S[0].detach().cpu().numpy().astype(np.float64))
    del r, f, q, rr, S, g, target, r1
    torch.cuda.empty_cache()
    return res


def gauss_extra(torch, dev, frames=10):
    """The reference's own method through the drop-in: mdsf.dens.compute_sf
    (mode "gauss") on the 1,500-water box (4,500 O/H atoms, 25 A, 64^3),
    host rescale/wrap, H2D, FP64 Gaussian deposit + fold (k_gauss_sep), FFT,
    |F|^2, get_dplot, D2H and the kgrid tables; beside it the oracle's
    restatement of the reference's Python loop on one host core."""
    from mdsf import dens as mdens
    from mdsf import synth
    from mdsf._lib import c_p, call
    from mdsf.api import _ptr, to_device
    pos, box, _ = synth.water_box(n_waters=1500, L=2.5, frames=frames, seed=1)
    r0 = pos * 10.0
    L0 = np.tile(box * 10.0, (frames, 1))
    typ = np.array(["O", "H", "H"] * 1500, dtype=object)
    # electrons and Gaussian widths (Angstrom) of O and H in the reference's
    # radii table (8 e, 60 pm; 1 e, 53 pm)
    rad = {"O": (8.0, 0.60), "H": (1.0, 0.53)}
    Sres = 25.0 / 64
    mdens.compute_sf_arrays(r0.copy(), L0.copy(), typ, rad, np.eye(3), Sres, device=dev)
    torch.cuda.synchronize()
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        mdens.compute_sf_arrays(r0.copy(), L0.copy(), typ, rad, np.eye(3), Sres, device=dev)
    torch.cuda.synchronize()
    wall = (time.perf_counter() - t0) / reps
    # the deposit kernel alone, timed with events over the same frames
    r = r0.copy()
    r, Lm = mdens.rescale(r, L0.copy())
    N = mdens.grid_dims(Lm, Sres)
    dr = np.divide(Lm, N)
    mdens.wrap_positions(r, Lm)
    dims = tuple(int(n) for n in N)
    plan = mdens.get_plan(dims, Lm, device=dev, max_atoms=r.shape[1])
    names, tidx, tab, nborder = mdens._type_table(rad, typ, dr)
    geom = np.zeros(16)
    geom[0:3] = dr
    geom[3:12] = np.eye(3).reshape(9)
    geom[12] = nborder
    geom[13] = 2 * int(tab[:, 2:5].max())
    td, tabd = to_device(tidx, dev), to_device(tab, dev)
    rd = to_device(np.ascontiguousarray(r, np.float64), dev)
    grid = torch.empty(dims, dtype=torch.float64, device=dev)
    sp = c_p(torch.cuda.current_stream(dev).cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    call("msf_gauss_grid_f64", plan.handle, _ptr(rd[0]), _ptr(td), r.shape[1], _ptr(tabd), len(names),
         c_p(geom.ctypes.data), _ptr(grid), sp)
    e0.record()
    for t in range(frames):
        call("msf_gauss_grid_f64", plan.handle, _ptr(rd[t]), _ptr(td), r.shape[1], _ptr(tabd), len(names),
             c_p(geom.ctypes.data), _ptr(grid), sp)
    e1.record()
    torch.cuda.synchronize()
    dep_ms = e0.elapsed_time(e1) / frames
    A = tab[:, 2:5].astype(int)
    per_type = {n: int(np.prod(2 * A[i])) for i, n in enumerate(names)}
    updates = sum(per_type[t] for t in typ)
    # the reference's method on the CPU: the oracle restatement of its loop
    from oracle import dens as odens
    t1 = time.perf_counter()
    odens.compute_sf(r0[:1].copy(), L0[:1].copy(), typ, rad, np.eye(3), Sres)
    cpu_s = time.perf_counter() - t1
    return {"gauss_frames_per_s": frames / wall,
            "gauss_note": f"mdsf.dens.compute_sf_arrays (mode gauss), 4,500 atoms, 64^3, {frames} frames per call, "
                          "wall time incl. host rescale/wrap, H2D, get_dplot, D2H and kgrid",
            "gauss_deposit_ms_per_frame": dep_ms,
            "gauss_deposit_voxel_updates_per_s": updates / (dep_ms / 1000.0),
            "gauss_deposit_note": f"k_gauss_sep: {updates} FP64 voxel updates per frame (separable factors, "
                                  "FP64 atomics into the L2-resident 2 MB grid): bound by L2 atomic throughput",
            "gauss_cpu_frames_per_s": 1.0 / cpu_s,
            "gauss_cpu_note": "the oracle's restatement of the reference's Python loop (dens.py:283-318), "
                              "1 frame, 1 core"}


def batched_systems(torch, dev, runs, prefix=""):
    """64 independent systems of uneven size (random_batch(64, seed=5):
    log-uniform 5k-300k atoms, boxes 3-16 nm, 2^a 3^b 5^c grids in 48-256,
    20-200 frames) in one CUDA graph over 8 streams, each system on the
    autotuner's tuning of its grid shape (shapes missing from the cache are
    tuned first, 4 candidates each)."""
    from mdsf.batch import BatchedSystems, random_batch
    systems = random_batch(64, seed=5, device=dev)
    frames = sum(int(s["pos_w"].shape[0]) for s in systems)
    t0 = time.perf_counter()
    b = BatchedSystems(systems, n_streams=8, device=dev, autotune=True)
    setup_s = time.perf_counter() - t0
    b.run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(runs):
        b.run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / runs
    variants = [b.tuning(i)["variant"] for i in range(len(systems))]
    res = {"frames_per_s": frames / (ms / 1000.0), "frames_per_run": frames, "ms_per_run": ms,
           "note": (f"64 systems, {frames} frames, one graph launch per run ({variants.count(3)} on the bucketed "
                    f"power-of-two chain, {variants.count(4)} on the smooth mixed-radix chain); "
                    f"{b.tuned_shapes} grid shapes autotuned at set-up ({setup_s:.1f} s incl. capture)")}
    del b, systems
    torch.cuda.empty_cache()
    return {prefix + k: v for k, v in res.items()}


def stress_512(torch, dev, frames=200, steps=1, prefix=""):
    """1M atoms in a 25 nm cube (6 x 6 columns) on the 512^3 grid: `frames`
    frames streamed from pinned host memory through mdsf.structure_factor,
    then get_dplot and the Ewald slices of the result on the GPU and the D2H
    of sf and the slices (end to end)."""
    import mdsf
    from mdsf import synth
    from mdsf.plan import clear_plans
    pos5, box5, w5 = synth.columnar(n_atoms=1_000_000, box=(25.0, 25.0, 25.0), n_cols=(6, 6), lattice=25.0 / 6,
                                    frames=frames, seed=11)
    p5 = torch.from_numpy(synth.pack_float4(pos5, w5)).pin_memory()
    del pos5
    dims = (512, 512, 512)

    def run():
        sf5 = mdsf.structure_factor(p5, box5, None, dims, device=dev)
        xy, xz, yz = mdsf.ewald_from_sf(sf5, box5, WAVELENGTH)
        return sf5, [sf5.cpu(), xy.cpu(), xz.cpu(), yz.cpu()]
    run()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        sf5, host = run()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / steps
    dc = float(host[0][0, 0, 0])
    assert abs(dc - frames * float(np.sum(w5, dtype=np.float64)) ** 2) < 1e-5 * dc
    plan5 = mdsf.get_plan(dims, box5, device=dev, max_atoms=1_000_000)
    res = {"frames_per_s": frames / dt,
           "note": (f"1M atoms, 25 nm cube, 6x6 columns, 512^3 grid, {frames} frames streamed from pinned host "
                    f"memory ({p5.numel() * 4 / 1e9:.1f} GB) + get_dplot + Ewald slices (lambda {WAVELENGTH} nm) on "
                    f"the GPU + D2H of sf and slices; wall time per call (variant {plan5.tuning()['variant']}, "
                    f"batch {plan5.batch})")}
    del sf5, p5, plan5, host
    clear_plans()
    torch.cuda.empty_cache()
    return {prefix + k: v for k, v in res.items()}


def radial_extra(torch, dev, shape=(254, 254, 255), nbins=750, reps=5):
    """radial_integrate (the |q|^2 float16 histogram) over the kgridplt of
    the 256x256x128 grid: the (..., 4) array form (range pass + bin pass,
    32 B read per voxel each) and the grid form (8 B per voxel)."""
    from mdsf import radial as mrad
    from mdsf.api import plot_axes
    X, Y, Z = plot_axes((shape[0] + 2, shape[1] + 2, (shape[2] + 3) // 2), np.array([160.0, 138.56, 80.0]))
    g = torch.Generator(device=dev).manual_seed(3)
    S = torch.rand(shape, dtype=torch.float64, device=dev, generator=g) * 100
    D = torch.empty(shape + (4,), dtype=torch.float64, device=dev)
    D[..., 0] = torch.from_numpy(X).to(dev)[:, None, None]
    D[..., 1] = torch.from_numpy(Y).to(dev)[None, :, None]
    D[..., 2] = torch.from_numpy(Z).to(dev)[None, None, :]
    D[..., 3] = S
    nv = S.numel()
    res = {}
    for name, fn, bytes_per in (("points", lambda: mrad.radial_histograms(D, nbins), 64),
                                ("grid", lambda: mrad.radial_histograms_grid(S, X, Y, Z, nbins), 8)):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / reps
        res[f"radial_{name}_voxels_per_s"] = nv / dt
        res[f"radial_{name}_gbs"] = nv * bytes_per / dt / 1e9
    res["radial_note"] = (f"{shape} voxels, {nbins} bins, float16 R and bin search as numpy; wall time per call "
                          "incl. host range/edges and the D2H of the histograms")
    del D, S
    torch.cuda.empty_cache()
    return res


def rz_extra(torch, dev, shape=(254, 254, 255), reps=3):
    """(r, z) histograms of measure_intensity.py over the kgridplt of the
    256x256x128 grid in the 120-degree cell: shear, trilinear interpolation,
    r/z bin search and FP64 atomics per voxel."""
    from mdsf import rz as mrz
    from mdsf.api import plot_axes
    X, Y, Z = plot_axes((shape[0] + 2, shape[1] + 2, (shape[2] + 3) // 2), np.array([160.0, 138.56, 80.0]))
    g = torch.Generator(device=dev).manual_seed(4)
    S = torch.rand(shape, dtype=torch.float64, device=dev, generator=g) * 100
    th = 120 * np.pi / 180.0
    ucell = np.array([[1, 0, 0], [np.cos(th), np.sin(th), 0], [0, 0, 1]])
    mrz.rz_histogram(S, X, Y, Z, ucell)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        mrz.rz_histogram(S, X, Y, Z, ucell)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / reps
    del S
    return {"rz_voxels_per_s": shape[0] * shape[1] * shape[2] / dt,
            "rz_note": f"{shape} voxels, r/z edges = the x/z axes, theta = 120 deg cell, linear weights; wall time "
                       "per call incl. the D2H of the two histograms"}


def nearest_extra(torch, dev, shape=(254, 254, 255), m=4_000_000, reps=3):
    """Nearest node of the sheared 120-degree kgridplt grid (plot2d.py's
    NearestNDInterpolator branch) for 4M random queries inside the sheared
    grid (uniform fractional lattice indices)."""
    from mdsf import rz as mrz
    from mdsf.api import plot_axes
    X, Y, Z = plot_axes((shape[0] + 2, shape[1] + 2, (shape[2] + 3) // 2), np.array([160.0, 138.56, 80.0]))
    th = 120 * np.pi / 180.0
    ucell = np.array([[1, 0, 0], [np.cos(th), np.sin(th), 0], [0, 0, 1]])
    g = torch.Generator(device=dev).manual_seed(5)
    S = torch.rand(shape, dtype=torch.float64, device=dev, generator=g)
    b = torch.from_numpy(mrz.reciprocal_rows(ucell)).to(dev)
    f = torch.rand((m, 3), dtype=torch.float64, device=dev, generator=g) * torch.tensor(
        [shape[0] - 1, shape[1] - 1, shape[2] - 1], dtype=torch.float64, device=dev)
    ax = [torch.tensor([a[0], (a[-1] - a[0]) / (len(a) - 1)], dtype=torch.float64, device=dev) for a in (X, Y, Z)]
    q = sum((ax[i][0] + f[:, i:i + 1] * ax[i][1]) * b[i] for i in range(3)).contiguous()
    mrz.nearest_sheared(S, X, Y, Z, ucell, q)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        mrz.nearest_sheared(S, X, Y, Z, ucell, q)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / reps
    del S, q
    return {"nearest_queries_per_s": m / dt,
            "nearest_note": f"{m} queries inside the {shape} grid in the 120-degree cell, wall time per call "
                            "(Fincke-Pohst enumeration of the lattice points within the distance bound)"}


def run_post_only(torch, dev, args):
    """The post-processing rows alone (radial_integrate, the (r, z)
    histograms, the sheared-grid nearest node), for launch lists and ncu."""
    out = {}
    out.update(radial_extra(torch, dev))
    out.update(rz_extra(torch, dev))
    out.update(nearest_extra(torch, dev))
    print(json.dumps({"metric": "post-processing rows on the 254x254x255 kgridplt", **out}))
    return 0


def gro_ingest(frames=8, atoms=N_ATOMS):
    """Host trajectory ingest: the native multithreaded .gro reader on a
    synthetic 200k-atom, 8-frame file (3 decimals, cubic box)."""
    from mdsf import traj
    rng = np.random.default_rng(9)
    xyz = rng.uniform(0, 12.0, (atoms, 3))
    body = "".join("%5d%-5s%5s%5d%8.3f%8.3f%8.3f\n" % ((i // 3 + 1) % 100000, "SOL", ("OW", "HW1", "HW2")[i % 3],
                                                      (i + 1) % 100000, *xyz[i]) for i in range(atoms))
    with tempfile.NamedTemporaryFile("w", suffix=".gro", delete=False) as f:
        for t in range(frames):
            f.write("synthetic water t= %d\n%5d\n%s  12.00000  12.00000  12.00000\n" % (t, atoms, body))
        path = f.name
    try:
        size = os.path.getsize(path)
        traj.read_gro(path)
        best = min(_timed_read(traj, path) for _ in range(3))
    finally:
        os.remove(path)
    return {"gro_ingest_frames_per_s": frames / best, "gro_ingest_mb_per_s": size / best / 1e6,
            "gro_ingest_note": f"{frames} frames x {atoms} atoms ({size / 1e6:.0f} MB) from page cache, "
                               f"scan + parse, {os.cpu_count()} host threads"}


def _timed_read(traj, path):
    t0 = time.perf_counter()
    traj.read_gro(path)
    return time.perf_counter() - t0


if __name__ == "__main__":
    sys.exit(main())
