"""Benchmark: frames/s of the structure-factor chain at 256x256x128, 200k atoms.

Workload (one step): the seeded columnar system -- 200,000 atoms in a
16.0 x 13.856 x 8.0 nm box, 100 frames of float32 positions (320 MB as
float4, more than L2) -- through histogram deposit -> R2C FFT -> |F|^2 ->
FP64 frame sum, then get_dplot and the Ewald slices at lambda = 0.154 nm.

  value       frames/s of the batched chain captured once in a CUDA graph
              and replayed per step, inputs resident in HBM.
  e2e         the same through the public API from pinned HOST buffers:
              H2D of the step's positions (streamed on a side stream) and
              D2H of sf inside the timed region.
  roofline    the dominant kernel, timed live with CUDA events over a pass
              of the same workload driven stage by stage.
  cpu_baseline the numpy oracle (histogramdd + rfftn, one core) on a bounded
              sample of frames of the same workload.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
N>1 runs under torchrun: every rank processes its own trajectory (frames
shard with no exchange until one FP64 sum of sf per step).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
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
WORKLOAD = "columnar 200k atoms, 16.0x13.856x8.0 nm, 256x256x128 grid, 100 frames/step, f32 positions, Ewald lambda=0.154 nm"


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


class Clocks:
    """nvidia-smi sampled every 100 ms; only the samples stamped inside the
    timed region (between mark_start and mark_end) are summarised.  The
    sampler is started, and its first sample awaited, before the region."""

    def __init__(self, index=0):
        self.proc = None
        self.path = os.path.join(os.environ.get("MSF_BENCH_DIR", tempfile.gettempdir()), "clocks_bench.csv")
        self.index = index
        self.t0 = self.t1 = None

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
            deadline = time.time() + 5.0
            while time.time() < deadline and os.path.getsize(self.path) == 0:
                time.sleep(0.02)
        except Exception:
            self.proc = None
        return self

    def mark_start(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.15)   # let the sample after the region land
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return None
        import datetime
        sm, mx, reasons, total = [], [], set(), 0
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 10:
                    continue
                total += 1
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                if self.t0 is not None and not (self.t0 <= ts <= self.t1):
                    continue
                sm.append(float(f[2]))
                mx.append(float(f[3]))
                for n, v in zip(names, f[6:10]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        except Exception:
            return None
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "samples": 0, "reasons": [],
                    "note": f"no sample inside the timed region ({total} around it): region shorter than "
                            "the 100 ms sampling period"}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "samples": len(sm),
                "reasons": sorted(reasons)}


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
            "data": "synthetic (seeded columnar system)",
            "config": {"workload": WORKLOAD, "sample_per_step": f"{frames_per_worker} frames x {cores} processes"},
            "cpu_baseline": {"value": value, "unit": "frames/s", "cores": cores, "kind": "port",
                             "sample": f"{frames_per_worker} frames per process per step, {cores} spawn processes, "
                                       "numpy histogramdd + numpy.fft.rfftn + |F|^2 + FP64 sum (the reference has no "
                                       "GPU-host-runnable code: it is pure Python and absent on the GPU host)"},
            "e2e": {"value": value, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_batched_only(torch, dev, args):
    """The batched-systems workload alone (for launch lists and ncu captures)."""
    from mdsf.batch import BatchedSystems, random_batch
    systems = random_batch(64, seed=5, device=dev)
    frames = sum(int(s["pos_w"].shape[0]) for s in systems)
    b = BatchedSystems(systems, n_streams=8, device=dev)
    for _ in range(2):
        b.run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        b.run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    variants = [b.tuning(i)["variant"] for i in range(len(systems))]
    print(json.dumps({"metric": "batched systems frames/s (64 uneven systems, one graph)",
                      "value": frames / (ms / 1000.0), "unit": "frames/s", "frames_per_run": frames,
                      "ms_per_run": ms, "variants": {str(v): variants.count(v) for v in sorted(set(variants))}}))
    return 0


def stress_512(torch, dev, steps=1, frames=40):
    """1M atoms in a 25 nm cube (6 x 6 columns) on the 512^3 grid, `frames`
    frames streamed from pinned host memory through mdsf.structure_factor;
    returns (frames/s, note)."""
    import mdsf
    from mdsf import synth
    from mdsf.plan import clear_plans
    pos5, box5, w5 = synth.columnar(n_atoms=1_000_000, box=(25.0, 25.0, 25.0), n_cols=(6, 6), lattice=25.0 / 6,
                                    frames=frames, seed=11)
    p5 = torch.from_numpy(synth.pack_float4(pos5, w5)).pin_memory()
    del pos5
    mdsf.structure_factor(p5[:4], box5, None, (512, 512, 512), device=dev)     # plan + first launches
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        sf5 = mdsf.structure_factor(p5, box5, None, (512, 512, 512), device=dev)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    dc = float(sf5[0, 0, 0].item())
    assert abs(dc - frames * float(np.sum(w5, dtype=np.float64)) ** 2) < 1e-5 * dc
    plan5 = mdsf.get_plan((512, 512, 512), box5, device=dev, max_atoms=1_000_000)
    note = (f"1M atoms, 25 nm cube, 6x6 columns, 512^3 grid, {frames} frames streamed from pinned host memory "
            f"(variant {plan5.tuning()['variant']}, batch {plan5.batch})")
    del sf5, p5, plan5
    clear_plans()
    torch.cuda.empty_cache()
    return frames / (ms / 1000.0), note


def run_stress_only(torch, dev, args):
    value, note = stress_512(torch, dev, steps=args.steps)
    print(json.dumps({"metric": "frames/s of the 512^3 stress grid (1M atoms, streamed from host)",
                      "value": value, "unit": "frames/s", "note": note}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 200 for the chain: ~0.6 s, long enough for clock samples; "
                         "5 for --impl reference; 3 for --batched-only)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=0)
    ap.add_argument("--variant", type=int, default=0)
    ap.add_argument("--tile-w", type=int, default=0)
    ap.add_argument("--no-overlap", action="store_true")
    ap.add_argument("--post-only", action="store_true",
                    help="only the post-processing rows (radial, (r, z) histograms, nearest node)")
    ap.add_argument("--zero-copy", action="store_true",
                    help="e2e: the kernels read the pinned host positions in place instead of staged copies")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--stream-chunk", type=int, default=0,
                    help="frames per host->device chunk of the e2e path (0: the API default, one batch)")
    ap.add_argument("--stress-only", action="store_true",
                    help="only the 512^3 stress grid (1M atoms, 40 frames from pinned host memory)")
    ap.add_argument("--batched-only", action="store_true",
                    help="only the 64 uneven batched systems (one graph, 2 warm-up + `--steps` replays)")
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
        return run_batched_only(torch, dev, args)
    if args.stress_only:
        return run_stress_only(torch, dev, args)
    if args.post_only:
        return run_post_only(torch, dev, args)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    pos, box, w = synth.columnar(n_atoms=N_ATOMS, box=BOX, frames=FRAMES, seed=2 + 7919 * rank)
    pos4_h = torch.from_numpy(synth.pack_float4(pos, w)).pin_memory()
    pos4 = pos4_h.to(dev)
    tuning = {}
    if args.batch:
        tuning["batch"] = args.batch
    if args.variant:
        tuning["variant"] = args.variant
    if args.tile_w:
        tuning["tile_w"] = args.tile_w
    if args.no_overlap:
        tuning["options"] = 1
    if not tuning:
        from mdsf import tune
        tuning = tune.lookup(DIMS) or {}   # else the plan's defaults (bucketed chain, 64 frames per batch)
    plan = mdsf.get_plan(DIMS, box, device=dev, max_atoms=N_ATOMS, **tuning)
    st = torch.cuda.current_stream(dev)
    sf = torch.zeros(plan.half_shape, dtype=torch.float64, device=dev)
    X, Y, Z = mdsf.plot_axes(plan.half_shape, box)
    Xd, Yd, Zd = (torch.from_numpy(a).to(dev) for a in (X, Y, Z))
    D = torch.empty((DIMS[0] - 2, DIMS[1] - 2, 2 * plan.nh - 3), dtype=torch.float64, device=dev)
    ew = [torch.empty(s, dtype=torch.float64, device=dev) for s in
          ((D.shape[0], D.shape[1]), (D.shape[0], D.shape[2]), (D.shape[1], D.shape[2]))]
    K = 2.0 * np.pi / WAVELENGTH

    def step_body():
        sf.zero_()
        sp = c_p(torch.cuda.current_stream(dev).cuda_stream)   # the capture stream inside graph capture
        call("msf_hist_sf_f32", plan.handle, _ptr(pos4), N_ATOMS, FRAMES, c_p(0), 0, _ptr(sf), sp)
        if world > 1:
            dist.all_reduce(sf)
        call("msf_sfplt", _ptr(sf), DIMS[0], DIMS[1], plan.nh, _ptr(D), sp)
        call("msf_ewald", _ptr(D), D.shape[0], D.shape[1], D.shape[2], _ptr(Xd), _ptr(Yd), _ptr(Zd), K,
             _ptr(ew[0]), _ptr(ew[1]), _ptr(ew[2]), sp)

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

    with Clocks(local) as clk:
        clk.mark_start()
        ms = timed(run, args.steps)
        clk.mark_end()
    clocks = clk.summary()
    ms_per_step = ms / args.steps
    value = FRAMES * world * args.steps / (ms / 1000.0)
    # correctness guard on the timed output: DC term = (sum of weights)^2 per frame
    dc = float(sf[0, 0, 0].item())
    dc_ref = FRAMES * world * float(np.sum(w, dtype=np.float64)) ** 2
    assert abs(dc - dc_ref) < 1e-5 * dc_ref, (dc, dc_ref)

    # ---- e2e: public API from pinned host buffers, D2H of sf in the timed region
    sf_h = torch.empty(plan.half_shape, dtype=torch.float64).pin_memory()

    d2h_stream = torch.cuda.Stream(dev)

    def e2e_step():
        out = mdsf.structure_factor(pos4_h, box, None, DIMS, device=dev, tuning=tuning,
                                    stream_chunk=args.stream_chunk or None, zero_copy=args.zero_copy)
        if world > 1:
            dist.all_reduce(out)
        # the read-back of this step's sf on its own stream, so that the next
        # step's kernels do not queue behind it (the timed region still ends
        # with a device-wide synchronize)
        done = torch.cuda.Event()
        done.record()
        with torch.cuda.stream(d2h_stream):
            d2h_stream.wait_event(done)
            sf_h.copy_(out, non_blocking=True)
            out.record_stream(d2h_stream)
    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    ms_e2e = timed(e2e_step, args.steps, join=(d2h_stream,))
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
    # compulsory bytes of each stage for one launch of `B` frames
    if plan.variant == 3:
        stage_bytes = {
            # positions read, bucket entries written, then read and written once more compacted
            1: lambda k: 16 * N_ATOMS * k + 8 * N_ATOMS * k + 16 * N_ATOMS * k,
            2: lambda k: 8 * N_ATOMS * k + 8 * Vh * k,              # bucket read, spectrum written
            4: lambda k: 8 * Vh * k + 16 * Vh,                      # spectrum read, sf read + written
        }
        stage_names = {1: "k_bucket_sort+scan+compact", 2: "k_plane_ct",
                       4: "k_xpower_tma" if plan.tma else "k_xpower_ct"}
    else:
        stage_bytes = {
            1: lambda k: 16 * N_ATOMS * k + 4 * V * k,             # positions read, grid written
            2: lambda k: 4 * V * k + 4 * V * k + 8 * Vh * k,        # grid read, grid zeroed, spectrum written
            4: lambda k: 8 * Vh * k + 16 * Vh,                      # spectrum read, sf read + written
        }
        stage_names = {1: "k_hist_deposit", 2: "k_plane" if plan.variant == 1 else "k_zrows+k_ycols",
                       4: "k_xpower"}
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

    extras = {}
    if not args.no_extras and rank == 0:
        extras = run_extras(mdsf, torch, dev, pos4, box, tuning, args)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_port_baseline(pos, box, w)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded columnar system (no dataset in the reference)",
            "config": {"workload": WORKLOAD, "frames_per_step": FRAMES, "n_atoms": N_ATOMS, "grid": list(DIMS),
                       "l2": "inputs larger than L2 (320 MB of float4 positions per step)",
                       "arithmetic": "int32 grid (FP32 binning exact vs FP64 edges), FP32 FFT, FP64 frame sum",
                       "tuning": plan.tuning(), "graph": world == 1, "parallelism": f"frames sharded x{world}"},
            "roofline": {"bound": "hbm", "kernel": stage_names[dom], "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": traffic, "traffic_note": traffic_note,
                         "peak_kind": peak_kind, "avg_launch_ms": avg_ms, "frames_per_launch": kfull,
                         "stage_ms_per_frame": {stage_names[s]: totals[s] / FRAMES for s in totals},
                         "chain_algorithmic_gbs": chain_gbs, "chain_frac": chain_gbs / peak},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "frames/s", "h2d_bytes_per_step": int(pos4_h.numel() * 4),
                    "d2h_bytes_per_step": int(sf_h.numel() * 8),
                    "h2d": ("kernels read the pinned host positions in place (mapped memory, NVLink-C2C)"
                            if args.zero_copy else "chunked copies from pinned host memory on a side stream")},
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clocks,
            "extras": extras,
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()
    return 0


def run_extras(mdsf, torch, dev, pos4, box, tuning, args):
    """Plain one-frame-per-launch path, the direct-sum gradient rate, the
    batched uneven systems and the 512^3 stress grid."""
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

    # direct sum: 20k atoms, 65,536 q, forward + adjoint, batch of 32 systems
    rng = np.random.default_rng(4)
    S_, N, M = 32, 20_000, 65_536
    r = torch.from_numpy(rng.uniform(0, 6.0, (S_, N, 3)).astype(np.float32)).to(dev).requires_grad_(True)
    f = torch.from_numpy(rng.choice(np.array([1, 6, 7, 8], np.float32), (S_, N))).to(dev)
    d = rng.standard_normal((M, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    q = torch.from_numpy((d * rng.uniform(5, 15, (M, 1))).astype(np.float32)).to(dev)
    target = torch.rand((S_, M), device=dev) * 100

    def grad_eval():
        S = mdsf.direct_sf(r, f, q)
        loss = torch.mean((torch.log1p(S) - torch.log1p(target)) ** 2)
        g, = torch.autograd.grad(loss, r)
        return g
    grad_eval()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    reps = 3
    for _ in range(reps):
        grad_eval()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    pairs = 2 * S_ * N * M
    out["grad_evals_per_s"] = S_ / (ms / 1000.0)
    out["grad_note"] = f"systems/s: forward+adjoint of {S_} systems x {N} atoms x {M} q per launch pair"
    out["direct_pairs_per_s"] = pairs / (ms / 1000.0)
    del r, f, q, target

    # batched uneven systems: 64 systems, log-uniform 5k-300k atoms, boxes 3-16 nm,
    # 2^a 3^b 5^c grids in 48-256, 20-200 frames, one CUDA graph over 8 streams
    from mdsf.batch import BatchedSystems, random_batch
    systems = random_batch(64, seed=5, device=dev)
    frames = sum(int(s["pos_w"].shape[0]) for s in systems)
    b = BatchedSystems(systems, n_streams=8, device=dev)
    b.run()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(2):
        b.run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 2
    out["batched_systems_frames_per_s"] = frames / (ms / 1000.0)
    variants = [b.tuning(i)["variant"] for i in range(64)]
    out["batched_systems_note"] = (f"64 systems, {frames} frames, one graph launch per run "
                                   f"({variants.count(3)} on the bucketed power-of-two chain, "
                                   f"{variants.count(4)} on the smooth mixed-radix chain)")
    del b, systems
    torch.cuda.empty_cache()

    # large stress grid: 1M atoms in a 25 nm cube (6 x 6 columns), 512^3, frames
    # streamed from pinned host memory through the public API (e2e)
    out["stress_512_frames_per_s"], out["stress_512_note"] = stress_512(torch, dev)
    out.update(radial_extra(torch, dev))
    out.update(rz_extra(torch, dev))
    out.update(nearest_extra(torch, dev))
    out.update(gro_ingest())
    return out


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
