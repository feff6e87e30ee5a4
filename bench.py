"""Benchmark of the torchmorph hot path on GB300.

Headline workload: exact 3-D Euclidean distance transform with feature
indices -- 4 bool volumes of 128^3, foreground iid Bernoulli(0.9) (seeds 0-2),
unit sampling, float32 distances + int32 indices.  Secondary workloads in
the same JSON line: flat 3x3 grey dilation (8 x 256^2 and an HBM-resident
8 x 4096^2), binary dilation, chessboard chamfer on the EDT volumes, and the
shared-cost batched Sinkhorn solve (256 pairs x 8192 points, eps 0.05 and
0.01, to an L1 marginal residual of 1e-6) on the tensor cores with its
float64 errors, next to the plain FP32 fused iterations.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm's CPU implementation (the
oracle restatement of it, all host threads) on the same workload; the
reference has no CPU path of its own for these operators.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "Gvoxel/s (EDT, grey dilation) and Sinkhorn solves/s at stated err; % roofline"
EDT_SHAPE = (4, 1, 128, 128, 128)
EDT_P = 0.9
EDT_BYTES_PER_VOXEL = 17  # 1 B bool in + 4 B float32 distance + 3 x 4 B int32 indices
L2_BYTES = 129 * 2**20


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), float(p.get("bf16_tflops", 1900.0)), "measured"
    return 6800.0, 1900.0, "fallback"


def edt_volumes(seed=0):
    rng = np.random.default_rng(seed)
    return rng.random(EDT_SHAPE) < EDT_P


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"tm_clocks_bench_{os.getpid()}.csv")
        self.gpu = gpu_index

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.fh, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax = float(parts[2])
                except ValueError:
                    continue
                for name, val in zip(names[1:], parts[5:9]):
                    if val.lower().startswith("active"):
                        reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def time_device(fn, sets, steps, warmup, stream):
    """Run fn(set) for warmup+steps iterations rotating over `sets`; return seconds of the timed steps."""
    import torch

    for i in range(warmup):
        fn(sets[i % len(sets)])
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for i in range(steps):
        fn(sets[i % len(sets)])
    end.record(stream)
    torch.cuda.synchronize()
    return start.elapsed_time(end) / 1e3


def graph_time(fn, sets, steps, warmup, stream):
    """Capture one CUDA graph per set holding fn(set) (one public-operator call), then
    time replays rotating over the sets: device time without the Python / launch
    overhead of eager calls.  Returns seconds per call."""
    import torch

    side = torch.cuda.Stream()
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        for st in sets:
            fn(st)
    stream.wait_stream(side)
    graphs = []
    for st in sets:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            fn(st)
        graphs.append(g)
    return time_device(lambda g: g.replay(), graphs, steps, warmup, stream) / steps


def bench_ours(args, rank, world):
    import torch

    import torchmorph_gb300 as tm
    from torchmorph_gb300 import _C

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)
    hbm_peak, _, peak_kind = peaks()
    nvox = int(np.prod(EDT_SHAPE))

    # ---- headline: EDT with indices, inputs resident in HBM
    nsets = 3  # 3 x (8 MB in + 134 MB out + 134 MB workspace) > 2 x L2
    vols = [edt_volumes(seed=1000 * rank + k) for k in range(nsets)]  # independent volumes
    host_in = torch.from_numpy(vols[0])
    sets = []
    for k in range(nsets):
        x = torch.from_numpy(vols[k]).to(dev)
        d = torch.empty(EDT_SHAPE, dtype=torch.float32, device=dev)
        i = torch.empty((3, *EDT_SHAPE), dtype=torch.int32, device=dev)
        sets.append((x, d, i))

    def edt_step(s):
        _C.edt(s[0], None, True, True, distances_out=s[1], indices_out=s[2])

    # correctness gate on the first set before timing
    edt_step(sets[0])
    torch.cuda.synchronize()

    # one CUDA graph per rotating set (each holds one public-operator call), so
    # the device time is not bounded by the Python / launch overhead per call
    side = torch.cuda.Stream(dev)
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        for s in sets:
            edt_step(s)
    stream.wait_stream(side)
    graphs = []
    for s in sets:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            edt_step(s)
        graphs.append(g)

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev.index) as clk:
        t_edt = time_device(lambda g: g.replay(), graphs, args.steps, args.warmup, stream)
    # the graph replays wrote the same results as the eager call
    ref = sets[0][2].clone()
    graphs[0].replay()
    torch.cuda.synchronize()
    assert torch.equal(ref, sets[0][2])
    if world > 1:
        t = torch.tensor([t_edt], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_edt = float(t.item())
    value = world * nvox * args.steps / t_edt / 1e9
    ms_step = t_edt / args.steps * 1e3
    achieved = EDT_BYTES_PER_VOXEL * nvox / (t_edt / args.steps) / 1e9

    # ---- e2e: public API, pinned host input -> device -> outputs back to pinned host.
    # Two streams with their own device and pinned buffers: step k + 1's input
    # copy and EDT run while step k's outputs are read back (the device-to-host
    # link, ~190 GB/s, bounds the step).
    pin_in = host_in.pin_memory()
    e2e_streams = [torch.cuda.Stream(dev), torch.cuda.Stream(dev)]
    e2e_bufs = []
    for _ in range(2):
        e2e_bufs.append((torch.empty(EDT_SHAPE, dtype=torch.bool, device=dev),
                         torch.empty(EDT_SHAPE, dtype=torch.float32, device=dev),
                         torch.empty((3, *EDT_SHAPE), dtype=torch.int32, device=dev),
                         torch.empty(EDT_SHAPE, dtype=torch.float32).pin_memory(),
                         torch.empty((3, *EDT_SHAPE), dtype=torch.int32).pin_memory()))

    def e2e_step(k):
        dev_in, dev_d, dev_i, pin_d, pin_i = e2e_bufs[k % 2]
        with torch.cuda.stream(e2e_streams[k % 2]):
            dev_in.copy_(pin_in, non_blocking=True)
            tm.euclidean_distance_transform(dev_in, return_distances=False, distances=dev_d, indices=dev_i)
            pin_d.copy_(dev_d, non_blocking=True)
            pin_i.copy_(dev_i, non_blocking=True)

    def e2e_run(nsteps):
        for st in e2e_streams:
            st.wait_stream(stream)
        for k in range(nsteps):
            e2e_step(k)
        for st in e2e_streams:
            stream.wait_stream(st)

    e2e_steps = max(3, args.steps // 2)
    e2e_run(max(args.warmup, 3))
    torch.cuda.synchronize()
    e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e_start.record(stream)
    e2e_run(e2e_steps)
    e_end.record(stream)
    torch.cuda.synchronize()
    t_e2e = e_start.elapsed_time(e_end) / 1e3
    e2e_value = world * nvox * e2e_steps / t_e2e / 1e9
    # the copy bound of the e2e step: the same outputs read back with plain pinned
    # device-to-host copies on the same two streams, no EDT
    def d2h_only(nsteps):
        for st in e2e_streams:
            st.wait_stream(stream)
        for k in range(nsteps):
            _, dev_d, dev_i, pin_d, pin_i = e2e_bufs[k % 2]
            with torch.cuda.stream(e2e_streams[k % 2]):
                pin_d.copy_(dev_d, non_blocking=True)
                pin_i.copy_(dev_i, non_blocking=True)
        for st in e2e_streams:
            stream.wait_stream(st)

    d2h_only(3)
    torch.cuda.synchronize()
    e_start.record(stream)
    d2h_only(e2e_steps)
    e_end.record(stream)
    torch.cuda.synchronize()
    t_d2h = e_start.elapsed_time(e_end) / 1e3
    d2h_gbps = nvox * 16 * e2e_steps / t_d2h / 1e9
    # the host copies must hold the same result as the device-resident runs
    for _, _, _, pin_d, pin_i in e2e_bufs:
        assert torch.equal(pin_i, sets[0][2].cpu()) and torch.equal(pin_d, sets[0][1].cpu())

    extra = {}
    if rank == 0 and not args.headline_only:
        extra = secondary(args, dev, stream, hbm_peak)

    result = {
        "metric": METRIC,
        "value": round(value, 4),
        "unit": "Gvoxel/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_step, 5),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32",
        "data": "synthetic: iid Bernoulli(0.9) foreground volumes, numpy seeds 1000 * rank + (0, 1, 2), one per rotating set",
        "config": edt_config(world),
        "e2e": {"value": round(e2e_value, 4), "unit": "Gvoxel/s",
                "h2d_bytes_per_step": int(nvox), "d2h_bytes_per_step": int(nvox * 16),
                "how": "public euclidean_distance_transform, pinned host input in and all outputs back every "
                       "step, two streams so that step k+1's copy-in and EDT overlap step k's read-back",
                "d2h_copy_GBps": round(d2h_gbps, 1),
                "copy_bound_Gvoxel_s": round(d2h_gbps / 16, 3),
                "frac_of_copy_bound": round(e2e_value / world / (d2h_gbps / 16), 4)},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak,
                     "unit": "GB/s", "frac": round(achieved / hbm_peak, 4),
                     "peak_kind": peak_kind,
                     "traffic": load_traffic("edt"),
                     "scope": "whole EDT op (background bitmap + shell search; the separable passes "
                              "launch and exit for items the search finished), 17 algorithmic B/voxel"},
        "gpu_launches": 4 * args.steps,
        "clocks": clk.summary(),
        "secondary": extra,
    }
    return result


def edt_config(world=1):
    """The headline workload's config, shared by both arms so that they name the same run."""
    return {
        "workload": "exact 3-D EDT with feature indices (scipy tie rule), 4 x 128^3 bool, "
                    "unit sampling; float32 distances + int32 indices",
        "batch": EDT_SHAPE[0], "volume": list(EDT_SHAPE[2:]), "foreground_p": EDT_P,
        "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
        "l2": "GPU arm: 3 rotating input/output/workspace sets (~1.3 GB) > L2; "
              "CPU arm: the whole workload per step (outputs 0.7 GB in float64/int64)",
    }


def load_traffic(kind):
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f).get(kind)


def grey_lines(args, dev, stream, hbm_peak):
    """Flat 3x3 grey dilation (reflect) of float32 U[0, 1): 8 x 256^2 (L2 resident) and
    8 x 4096^2 (HBM resident, two rotating inputs), 8 algorithmic B/voxel."""
    import torch

    from torchmorph_gb300 import _C

    g = torch.Generator(device="cpu").manual_seed(0)
    st3 = torch.zeros((3, 3), dtype=torch.float32)
    fp0 = torch.empty(0, dtype=torch.bool)

    def grey_line(shape, nsets):
        sets = []
        for _ in range(nsets):
            x = torch.rand(shape, generator=g).to(dev)
            sets.append(x)

        def step(x):
            _C.grey_dilation_cuda(x, st3, fp0, [0, 0], 1, 0.0)

        steps = max(args.steps, 10)
        t = time_device(step, sets, steps, args.warmup, stream)
        t_graph = graph_time(step, sets, steps, args.warmup, stream)
        nv = int(np.prod(shape))
        per = t / steps
        return {"Gvoxel/s": round(nv / per / 1e9, 3), "us_per_call": round(per * 1e6, 2),
                "achieved_GBps": round(8 * nv / per / 1e9, 1),
                "frac_of_hbm": round(8 * nv / per / 1e9 / hbm_peak, 4),
                "us_per_call_graph": round(t_graph * 1e6, 2),
                "frac_of_hbm_graph": round(8 * nv / t_graph / 1e9 / hbm_peak, 4)}

    out = {"grey_dilation_3x3_8x256x256": grey_line((8, 1, 256, 256), 8),
           "grey_dilation_3x3_8x4096x4096_hbm": grey_line((8, 1, 4096, 4096), 2)}

    # morphological gradient 3x3 on the HBM-resident shape: one pass (8 B/voxel) vs the
    # reference's composition of the two operators and a subtraction (28 B/voxel moved)
    import torchmorph_gb300 as tm

    xs = [torch.rand((8, 1, 4096, 4096), generator=g).to(dev) for _ in range(2)]
    steps = max(args.steps, 10)
    t1 = time_device(lambda x: tm.morphological_gradient(x, size=3), xs, steps, args.warmup, stream) / steps
    t2 = time_device(lambda x: _C.grey_dilation_cuda(x, st3, fp0, [0, 0], 1, 0.0)
                     - _C.grey_erosion_cuda(x, st3, fp0, [0, 0], 1, 0.0), xs, steps, args.warmup, stream) / steps
    nv = xs[0].numel()
    out["grey_gradient_3x3_8x4096x4096_one_pass"] = {
        "us_per_call": round(t1 * 1e6, 1), "Gvoxel/s": round(nv / t1 / 1e9, 3),
        "frac_of_hbm": round(8 * nv / t1 / 1e9 / hbm_peak, 4),
        "two_operators_us": round(t2 * 1e6, 1), "speedup_vs_two_operators": round(t2 / t1, 2)}
    # opening and white top-hat 3x3: one pass vs the reference's composition (two operator
    # launches, and a subtraction for the top-hat)
    for name, fn, comp in (
            ("opening", lambda x: tm.grey_opening(x, size=3),
             lambda x: _C.grey_dilation_cuda(_C.grey_erosion_cuda(x, st3, fp0, [0, 0], 1, 0.0), st3, fp0,
                                             [0, 0], 1, 0.0)),
            ("white_tophat", lambda x: tm.white_tophat(x, size=3),
             lambda x: x - _C.grey_dilation_cuda(_C.grey_erosion_cuda(x, st3, fp0, [0, 0], 1, 0.0), st3, fp0,
                                                 [0, 0], 1, 0.0))):
        t1 = time_device(fn, xs, steps, args.warmup, stream) / steps
        t2 = time_device(comp, xs, steps, args.warmup, stream) / steps
        out[f"grey_{name}_3x3_8x4096x4096_one_pass"] = {
            "us_per_call": round(t1 * 1e6, 1), "Gvoxel/s": round(nv / t1 / 1e9, 3),
            "frac_of_hbm": round(8 * nv / t1 / 1e9 / hbm_peak, 4),
            "composition_us": round(t2 * 1e6, 1), "speedup_vs_composition": round(t2 / t1, 2)}
    return out


def binary_lines(args, dev, stream, hbm_peak):
    """Binary dilation 3x3 box at 8 x 256^2 (L2 resident) and, HBM resident at 8 x 4096^2
    (bit-packed tiles), erosion with the default cross and the one-pass opening."""
    import torch

    import torchmorph_gb300 as tm
    from torchmorph_gb300 import _C

    out = {}
    g = torch.Generator(device="cpu").manual_seed(1)
    xb = (torch.rand((8, 1, 256, 256), generator=g) > 0.5).to(dev)
    box = torch.ones((3, 3), dtype=torch.bool)

    def bstep(x):
        _C.binary_dilation_cuda(x, box, [0, 0], False)

    steps = max(args.steps, 10)
    t = time_device(bstep, [xb], steps, args.warmup, stream)
    out["binary_dilation_3x3_8x256x256"] = {"Gvoxel/s": round(xb.numel() / (t / steps) / 1e9, 3),
                                            "us_per_call": round(t / steps * 1e6, 2)}
    # HBM-resident binary lines (bit-packed tiles): erosion with the default cross and the
    # one-pass opening, 8 x 4096^2 bool, two rotating inputs; 1 B in + 1 B out per voxel
    xbs = [(torch.rand((8, 1, 4096, 4096), generator=g) > 0.5).to(dev) for _ in range(2)]
    nbv = xbs[0].numel()
    for name, fn in (("binary_erosion_cross_8x4096x4096", lambda x: tm.binary_erosion(x)),
                     ("binary_opening_cross_8x4096x4096_one_pass", lambda x: tm.binary_opening(x))):
        tb = time_device(fn, xbs, steps, args.warmup, stream) / steps
        tg = graph_time(fn, xbs, steps, args.warmup, stream)  # device time without the host front end
        out[name] = {"us_per_call": round(tb * 1e6, 1), "us_per_call_graph": round(tg * 1e6, 1),
                     "Gvoxel/s": round(nbv / tg / 1e9, 3), "frac_of_hbm": round(2.0 * nbv / tg / 1e9 / hbm_peak, 4)}
    t2 = time_device(lambda x: tm.binary_dilation(tm.binary_erosion(x)), xbs, steps, args.warmup, stream) / steps
    out["binary_opening_cross_8x4096x4096_one_pass"]["composition_us"] = round(t2 * 1e6, 1)
    return out


def secondary(args, dev, stream, hbm_peak):
    """Grey/binary, chamfer, EDT shapes, ragged and Sinkhorn lines (rank 0 only)."""
    out = grey_lines(args, dev, stream, hbm_peak)
    out.update(binary_lines(args, dev, stream, hbm_peak))

    hbm = peaks()[0]
    out.update(cdt_lines(args, dev, stream))
    out.update(edt_shape_lines(args, dev, stream, hbm))
    out.update(ragged_lines(dev, stream, max(args.steps, 10), args.warmup))
    out.update(ragged_volume_lines(dev, stream, max(args.steps, 10), args.warmup))
    out.update(sinkhorn_lines(dev, stream, cpu_baseline=not args.no_cpu_baseline))
    out.update(pointcloud_lines(dev, stream, cpu_baseline=not args.no_cpu_baseline))
    return out


def cdt_lines(args, dev, stream):
    """Chamfer distances (distances only) on the EDT volumes: three independently seeded
    volumes rotating, preallocated outputs, 1 B in + 4 B out per voxel."""
    import torch

    from torchmorph_gb300 import _C

    out = {}
    hbm, _, kind = peaks()
    cvols = [(torch.from_numpy(edt_volumes(k)).to(dev), torch.empty(EDT_SHAPE, dtype=torch.float32, device=dev))
             for k in range(3)]
    for metric in ("chessboard", "taxicab", "chamfer345"):
        def cstep(s, metric=metric):
            _C.cdt(s[0], metric, True, False, distances_out=s[1])

        csteps = max(args.steps, 12)
        t_eager = time_device(cstep, cvols, csteps, max(args.warmup, 3), stream) / csteps
        t = graph_time(cstep, cvols, csteps, max(args.warmup, 3), stream)
        nv = cvols[0][0].numel()
        out[f"cdt_{metric}_4x128^3"] = {
            "Gvoxel/s": round(nv / t / 1e9, 3), "us_per_call": round(t * 1e6, 1),
            "us_per_eager_call": round(t_eager * 1e6, 1),
            "frac_of_hbm": round(5.0 * nv / t / 1e9 / hbm, 4), "peak_kind": kind,
            "volumes": "Bernoulli(0.9) foreground, seeds 0-2 rotating",
            "timing": "replays of one CUDA graph per rotating set (one call each)"}

    return out


def edt_shape_lines(args, dev, stream, hbm):
    """EDT with indices off the headline shape: rows of 200 voxels (2 x 96 x 160 x 200,
    Bernoulli(0.9): the general-width shell search) and a sparse background (4 x 128^3,
    Bernoulli(0.999): the separable passes), 17 algorithmic B/voxel."""
    import torch

    from torchmorph_gb300 import _C

    out = {}
    for name, shape, p in (("edt_2x96x160x200_p0.9", (2, 1, 96, 160, 200), 0.9),
                           ("edt_4x128^3_p0.999", EDT_SHAPE, 0.999)):
        sets = []
        for k in range(3):
            x = torch.from_numpy(np.random.default_rng(50 + k).random(shape) < p).to(dev)
            sets.append((x, torch.empty(shape, dtype=torch.float32, device=dev),
                         torch.empty((3, *shape), dtype=torch.int32, device=dev)))

        def step(s):
            _C.edt(s[0], None, True, True, distances_out=s[1], indices_out=s[2])

        steps = max(args.steps, 10)
        t = graph_time(step, sets, steps, max(args.warmup, 3), stream)
        nv = int(np.prod(shape))
        out[name] = {"Gvoxel/s": round(nv / t / 1e9, 3), "us_per_call": round(t * 1e6, 1),
                     "frac_of_hbm": round(17.0 * nv / t / 1e9 / hbm, 4),
                     "timing": "replays of one CUDA graph per rotating set (three seeded sets)"}
    return out


def ragged_images(seed=0, n=256):
    """256 2-D float32 images, H and W iid uniform integers in [32, 1024], values U[0, 1)."""
    rng = np.random.default_rng(seed)
    shapes = [(int(rng.integers(32, 1025)), int(rng.integers(32, 1025))) for _ in range(n)]
    return [rng.random(s, dtype=np.float32) for s in shapes]


def ragged_lines(dev, stream, steps, warmup):
    """Ragged batch: grey erosion size 5 and 15 plus binary opening of x > 0.5 (cross) on 256
    uneven images -- one persistent launch per operator, the sequence replayed as one CUDA
    graph -- against per-image launches of the drop-in operators."""
    import torch

    import torchmorph_gb300 as tm
    from torchmorph_gb300 import RaggedBatch, _C, ragged

    imgs = ragged_images()
    rb = RaggedBatch.from_images([torch.from_numpy(im).to(dev) for im in imgs])
    views = [v[None, None] for v in rb.images()]
    npx = rb.numel

    def pipeline(b):
        return (ragged.grey_erosion(b, size=5), ragged.grey_erosion(b, size=15),
                ragged.binary_opening(b.map(lambda x: x > 0.5)))

    def per_image(_):
        for v in views:
            tm.grey_erosion(v, size=5)
            tm.grey_erosion(v, size=15)
            tm.binary_opening(v > 0.5)

    # correctness gate: persistent results equal the per-image operators
    outs = pipeline(rb)
    for i in (0, 100, 255):
        assert torch.equal(outs[0][i], tm.grey_erosion(views[i], size=5)[0, 0])
        assert torch.equal(outs[1][i], tm.grey_erosion(views[i], size=15)[0, 0])
        assert torch.equal(outs[2][i], tm.binary_opening(views[i] > 0.5)[0, 0])
    graph, _ = ragged.capture(pipeline, rb)
    t_graph = time_device(lambda _: graph.replay(), [None], steps, warmup, stream) / steps
    t_eager = time_device(lambda _: pipeline(rb), [None], steps, warmup, stream) / steps
    t_img = time_device(per_image, [None], 3, 1, stream) / 3
    hbm, _, kind = peaks()
    algo = 18.0 * npx  # 4+4 (erosion 5) + 4+4 (erosion 15) + 1+1 (binary opening) bytes per pixel
    # opt-in backward of grey dilation (3x3, reflect) on an HBM-resident uniform batch
    x = torch.rand((8, 1, 2048, 2048), device=dev)
    st3 = torch.zeros((3, 3), dtype=torch.float32)
    fp0 = torch.empty(0, dtype=torch.bool)
    _, arg = _C.grey_dilation_arg(x, st3, fp0, [0, 0], 1, 0.0)
    g = torch.randn_like(x)
    t_fwd = time_device(lambda _: _C.grey_dilation_arg(x, st3, fp0, [0, 0], 1, 0.0), [None], steps,
                        warmup, stream) / steps
    t_bwd = time_device(lambda _: _C.grey_morphology_backward(g, arg, [3, 3], fp0, [0, 0], 1, True),
                        [None], steps, warmup, stream) / steps
    nb = x.numel()
    backward = {"grey_dilation_3x3_backward_8x2048x2048": {
        "forward_with_arg_us": round(t_fwd * 1e6, 1), "backward_us": round(t_bwd * 1e6, 1),
        "forward_with_arg_GBps": round(9.0 * nb / t_fwd / 1e9, 1),
        "forward_with_arg_frac_of_hbm": round(9.0 * nb / t_fwd / 1e9 / hbm, 4),
        "backward_GBps": round(9.0 * nb / t_bwd / 1e9, 1),
        "backward_frac_of_hbm": round(9.0 * nb / t_bwd / 1e9 / hbm, 4),
        "bytes_per_pixel": "forward 4 in + 4 out + 1 arg; backward 4 grad_out + 1 arg + 4 grad_in"}}
    return {**backward, "ragged_256_images_erosion5_15_binary_opening": {
        "pixels": npx, "ms_persistent_graph": round(t_graph * 1e3, 3),
        "ms_persistent_eager": round(t_eager * 1e3, 3), "ms_per_image_launches": round(t_img * 1e3, 3),
        "speedup_vs_per_image": round(t_img / t_graph, 2),
        "Gpixel/s": round(npx / t_graph / 1e9, 3),
        "roofline": {"bound": "hbm", "achieved": round(algo / t_graph / 1e9, 1), "peak": hbm,
                     "unit": "GB/s", "frac": round(algo / t_graph / 1e9 / hbm, 4), "peak_kind": kind,
                     "scope": "whole pipeline (the x > 0.5 threshold, a torch kernel, and one launch "
                              "per operator: erosion 5, erosion 15, the one-pass binary opening), 18 "
                              "algorithmic B/pixel"},
        "gpu_launches_per_step": 3}}


def ragged_volume_lines(dev, stream, steps, warmup):
    """Ragged 3-D batch: 64 volumes with D, H, W iid uniform in [16, 96], Bernoulli(0.9)
    foreground -- exact EDT with indices (one cooperative launch for all volumes) and
    grey erosion 3x3x3 of U[0, 1) values (one persistent launch), each replayed as a CUDA
    graph, against per-volume calls of the uniform operators."""
    import torch

    import torchmorph_gb300 as tm
    from torchmorph_gb300 import RaggedBatch, ragged

    rng = np.random.default_rng(0)
    shapes = [tuple(int(v) for v in rng.integers(16, 97, 3)) for _ in range(64)]
    fg = [rng.random(s) < 0.9 for s in shapes]
    vals = [rng.random(s, dtype=np.float32) for s in shapes]
    rb = RaggedBatch.from_images([torch.from_numpy(v).to(dev) for v in fg])
    rv = RaggedBatch.from_images([torch.from_numpy(v).to(dev) for v in vals])
    nvox = rb.numel
    views = [v[None, None] for v in rb.images()]
    vviews = [v[None, None] for v in rv.images()]
    # correctness gate against the per-volume operators
    d, _ = ragged.euclidean_distance_transform(rb, return_indices=True)
    e = ragged.grey_erosion(rv, size=3)
    for k in (0, 31, 63):
        dk, _ = tm.euclidean_distance_transform(views[k], return_indices=True)
        assert torch.equal(d[k], dk[0, 0])
        assert torch.equal(e[k], tm.grey_erosion(vviews[k], size=3)[0, 0])
    g_edt, _ = ragged.capture(lambda b: ragged.euclidean_distance_transform(b, return_indices=True), rb)
    g_ero, _ = ragged.capture(lambda b: ragged.grey_erosion(b, size=3), rv)
    t_edt = time_device(lambda _: g_edt.replay(), [None], steps, warmup, stream) / steps
    t_ero = time_device(lambda _: g_ero.replay(), [None], steps, warmup, stream) / steps
    t_edt_vol = time_device(lambda _: [tm.euclidean_distance_transform(v, return_indices=True) for v in views],
                            [None], 3, 1, stream) / 3
    t_ero_vol = time_device(lambda _: [tm.grey_erosion(v, size=3) for v in vviews], [None], 3, 1, stream) / 3
    hbm, _, kind = peaks()
    return {"ragged_64_volumes_edt_erosion3": {
        "voxels": nvox,
        "edt_ms_one_launch_graph": round(t_edt * 1e3, 3), "edt_ms_per_volume_calls": round(t_edt_vol * 1e3, 3),
        "edt_speedup_vs_per_volume": round(t_edt_vol / t_edt, 2),
        "edt_Gvoxel/s": round(nvox / t_edt / 1e9, 3),
        "edt_frac_of_hbm": round(17.0 * nvox / t_edt / 1e9 / hbm, 4),
        "erosion3_ms_one_launch_graph": round(t_ero * 1e3, 3),
        "erosion3_ms_per_volume_calls": round(t_ero_vol * 1e3, 3),
        "erosion3_speedup_vs_per_volume": round(t_ero_vol / t_ero, 2),
        "erosion3_frac_of_hbm": round(8.0 * nvox / t_ero / 1e9 / hbm, 4), "peak_kind": kind,
        "shapes": "D, H, W iid uniform integers in [16, 96], numpy seed 0"}}


def pointcloud_profile_case(dev):
    """Small point-cloud case for profiler captures: 64 problems, n and m log-uniform in
    [64, 512], the bench's mixture points, eps 0.05, 200 iterations without a stopping
    test, solved twice (the second solve is the captured one)."""
    import torch

    from torchmorph_gb300 import PointCloudSinkhorn, pack_clouds

    rng = np.random.default_rng(0)
    xs, ys = [], []
    for _ in range(64):
        n, m = (int(v) for v in np.exp(rng.uniform(np.log(64), np.log(512), 2)))
        means = rng.uniform(-1, 1, (4, 3))
        xs.append((means[rng.integers(0, 4, n)] + 0.2 * rng.standard_normal((n, 3))).astype(np.float32))
        ys.append((means[rng.integers(0, 4, m)] + 0.2 * rng.standard_normal((m, 3))).astype(np.float32))
    x, nx = pack_clouds([torch.from_numpy(v).to(dev) for v in xs])
    y, ny = pack_clouds([torch.from_numpy(v).to(dev) for v in ys])
    solver = PointCloudSinkhorn(epsilon=0.05, max_iter=200, threshold=0.0)
    for _ in range(2):
        solver.solve(x, y, nx, ny)
    torch.cuda.synchronize()
    return {"case": "pointcloud-profile", "problems": 64, "iterations": 200}


def pointcloud_problems(seed=0, count=512):
    """512 OT problems, n and m iid log-uniform integers in [64, 2048], points from a
    4-component Gaussian mixture in R^3 (means U[-1, 1]^3, sigma 0.2), uniform weights."""
    rng = np.random.default_rng(seed)
    lo, hi = np.log(64), np.log(2048)
    xs, ys = [], []
    for _ in range(count):
        n = int(np.clip(np.rint(np.exp(rng.uniform(lo, hi))), 64, 2048))
        m = int(np.clip(np.rint(np.exp(rng.uniform(lo, hi))), 64, 2048))
        means = rng.uniform(-1, 1, (4, 3))
        xs.append((means[rng.integers(0, 4, n)] + 0.2 * rng.standard_normal((n, 3))).astype(np.float32))
        ys.append((means[rng.integers(0, 4, m)] + 0.2 * rng.standard_normal((m, 3))).astype(np.float32))
    return xs, ys


def pointcloud_lines(dev, stream, cpu_baseline=True):
    """Ragged differentiable point-cloud Sinkhorn: 512 problems in one persistent launch,
    eps 0.05, to an L1 column-marginal error <= 1e-5; gradient w.r.t. the source points."""
    import torch

    import oracle
    from torchmorph_gb300 import PointCloudSinkhorn, pack_clouds

    xs, ys = pointcloud_problems()
    x, nx = pack_clouds([torch.from_numpy(v).to(dev) for v in xs])
    y, ny = pack_clouds([torch.from_numpy(v).to(dev) for v in ys])
    # 1e-4: with potentials of magnitude ~10 (mass moving between mixture components),
    # fp32 rounding of f, g alone perturbs the plan's marginals by ~1e-5
    eps, tol = 0.05, 1e-4
    solver = PointCloudSinkhorn(epsilon=eps, max_iter=5000, threshold=tol, check_every=10)
    pairs = sum(a * b for a, b in zip(nx, ny))
    # kernel efficiency with every problem active: 100 fixed iterations
    fixed = PointCloudSinkhorn(epsilon=eps, max_iter=100, threshold=0.0)
    fixed.solve(x, y, nx, ny)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    fixed.solve(x, y, nx, ny)
    e1.record(stream)
    torch.cuda.synchronize()
    t_fixed = e0.elapsed_time(e1) / 1e3 / 100
    ex2_peak = 16 * 152 * 2.07e9  # MUFU ex2 per clock per SM x SMs x max SM clock
    res = solver.solve(x, y, nx, ny)  # warm-up
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    res = solver.solve(x, y, nx, ny)
    e1.record(stream)
    torch.cuda.synchronize()
    t_solve = e0.elapsed_time(e1) / 1e3
    its = res["iterations"].cpu().numpy()
    # forward + backward through autograd (the solve, then the gradient kernel)
    xg = x.clone().requires_grad_(True)
    torch.cuda.synchronize()
    e0.record(stream)
    solver(xg, y, nx, ny).sum().backward()
    e1.record(stream)
    torch.cuda.synchronize()
    t_fb = e0.elapsed_time(e1) / 1e3
    # work: per problem and iteration 2 n m pair evaluations (one ex2 each)
    ex2 = float(sum(2.0 * a * b * int(k) for a, b, k in zip(nx, ny, its)))
    # float64 check on 6 problems: regularised cost and the returned plan's marginals
    f, g = res["f"].cpu().numpy().astype(np.float64), res["g"].cpu().numpy().astype(np.float64)
    ox, oy = np.cumsum([0] + nx), np.cumsum([0] + ny)
    rel, marg = 0.0, 0.0
    for p in range(0, 512, 512 // 6)[:6]:
        xp, yp = xs[p].astype(np.float64), ys[p].astype(np.float64)
        _, _, _, c64 = oracle.pointcloud_sinkhorn(xp, yp, eps, 100000, threshold=1e-12)
        rel = max(rel, abs(res["cost"][p].item() - c64) / abs(c64))
        C = ((xp[:, None] - yp[None]) ** 2).sum(-1)
        P = np.exp((f[ox[p]:ox[p + 1], None] + g[None, oy[p]:oy[p + 1]] - C) / eps) / (len(xp) * len(yp))
        marg = max(marg, np.abs(P.sum(0) - 1 / len(yp)).sum() + np.abs(P.sum(1) - 1 / len(xp)).sum())
    line = {"problems": 512, "pairs_per_half_iteration": pairs, "threshold": tol,
            "ms_solve": round(t_solve * 1e3, 3),
            "solves/s": round(512 / t_solve, 1), "ms_forward_backward": round(t_fb * 1e3, 3),
            "iterations_max": int(its.max()), "iterations_mean": round(float(its.mean()), 1),
            "iterations_p90": int(np.percentile(its, 90)), "problems_at_max_iter": int((its >= 5000).sum()),
            "ex2_per_s": float(f"{ex2 / t_solve:.4g}"),
            "ex2_frac_of_nominal": round(ex2 / t_solve / ex2_peak, 4),
            "us_per_iteration_all_active": round(t_fixed * 1e6, 1),
            "ex2_frac_of_nominal_all_active": round(2.0 * pairs / t_fixed / ex2_peak, 4),
            "rel_cost_error_vs_fp64": float(f"{rel:.3e}"),
            "marginal_l1_fp64_max": float(f"{marg:.3e}"), "fp64_problems_checked": 6,
            "launches_per_solve": 5}
    if cpu_baseline:
        cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
        t0 = time.perf_counter()
        k = 0
        for p in range(8):
            oracle.pointcloud_sinkhorn(xs[p], ys[p], eps, int(its[p]), threshold=0.0)
            k += 1
            if time.perf_counter() - t0 > 20:
                break
        per = (time.perf_counter() - t0) / k
        line["cpu_baseline"] = {"value": round(1.0 / per, 3), "unit": "solves/s", "cores": cores, "kind": "port",
                                "sample": f"{k} problems, float64 numpy log-domain oracle, same iteration "
                                          "counts as the GPU run"}
    return {"pointcloud_sinkhorn_512_ragged_eps0.05": line}


def sinkhorn_problem(dev, n=256, d=8192, seed=0):
    """Shared-cost Sinkhorn workload: x, y iid U[0,1]^3 (d points each), C = |x - y|^2
    scaled to max 1, n histogram pairs iid Dirichlet(1), float32."""
    import torch

    g = torch.Generator(device="cpu").manual_seed(seed)
    x = torch.rand((d, 3), generator=g, dtype=torch.float64)
    y = torch.rand((d, 3), generator=g, dtype=torch.float64)
    cost = torch.cdist(x, y).square()
    cost = (cost / cost.max()).float()
    rng = np.random.default_rng(seed)
    a = torch.tensor(rng.dirichlet(np.ones(d), n), dtype=torch.float32)
    b = torch.tensor(rng.dirichlet(np.ones(d), n), dtype=torch.float32)
    return a.to(dev), b.to(dev), cost.to(dev)


def fp64_sinkhorn_errors(a, b, cost, eps, log_u, log_v, dist, iterations, pairs=8):
    """Errors of a solve against float64 Sinkhorn (the reference's scaling iteration,
    optimal_transport.py:84-93, run in float64 on the device for `pairs` pairs and
    iterations + 2000 iterations): relative OT-cost error, and the float64 L1 row and
    column marginal errors of the returned plan."""
    import torch

    K = torch.exp(-cost.double() / eps)
    A, B = a[:pairs].double(), b[:pairs].double()
    u, v = torch.ones_like(A), torch.ones_like(B)
    for _ in range(iterations + 2000):
        u = A / (v @ K.T)
        v = B / (u @ K)
    ref = ((u @ (K * cost.double())) * v).sum(-1)
    U, V = torch.exp(log_u[:pairs].double()), torch.exp(log_v[:pairs].double())
    rows = (U * (V @ K.T) - A).abs().sum(-1)
    cols = (V * (U @ K) - B).abs().sum(-1)
    rel = ((dist[:pairs].double() - ref).abs() / ref).max().item()
    return {"rel_cost_error_vs_fp64": float(f"{rel:.3e}"),
            "marginal_l1_rows_fp64": float(f"{rows.max().item():.3e}"),
            "marginal_l1_cols_fp64": float(f"{cols.max().item():.3e}"),
            "fp64_pairs_checked": pairs}


def sinkhorn_cpu_baseline(a, b, cost, eps, iterations, pairs=2, sample_iters=6):
    """The float64 Sinkhorn oracle (scaling form, OpenMP over all host threads) on a
    sample of `pairs` pairs x `sample_iters` iterations, extrapolated to solves/s at the
    GPU run's iteration count."""
    import oracle

    oracle.build()
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    A = a[:pairs].double().cpu().numpy()
    B = b[:pairs].double().cpu().numpy()
    C = cost.double().cpu().numpy()
    oracle.sinkhorn(A, B, C, eps, 1, log_space=False, nthreads=cores)
    t0 = time.perf_counter()
    oracle.sinkhorn(A, B, C, eps, sample_iters, log_space=False, nthreads=cores)
    per_pair_iter = (time.perf_counter() - t0) / (pairs * sample_iters)
    return {"value": round(1.0 / (per_pair_iter * iterations), 3), "unit": "solves/s",
            "cores": cores, "kind": "port",
            "sample": f"{pairs} pairs x {sample_iters} float64 scaling iterations of the oracle, "
                      f"extrapolated to {iterations} iterations per solve"}


def sinkhorn_lines(dev, stream, cpu_baseline=True):
    """Shared-cost batched Sinkhorn, 256 pairs x 8192 points, eps 0.05 and 0.01, run to
    an L1 row-marginal residual <= 1e-6 on the tensor cores, against the plain FP32
    fused iterations on the same GPU."""
    import torch

    from torchmorph_gb300 import SinkhornSolver, _C

    a, b, cost = sinkhorn_problem(dev)
    n, d = a.shape
    out = {}
    for eps in (0.05, 0.01):
        # reuse_solves=False: the timed call solves again instead of returning the warm-up's result
        solver = SinkhornSolver(epsilon=eps, max_iter=20000, threshold=1e-6, tensor_cores=True,
                                reuse_solves=False)
        solver.solve(a, b, cost)  # warm-up
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        res = solver.solve(a, b, cost)
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        its = int(res["iterations"])
        log_u, log_v, dist, _, _ = _C.sinkhorn_tc_solve(a, b, cost, eps, its)
        line = {"solves/s": round(n / t, 1), "ms_per_solve_batch": round(t * 1e3, 3),
                "iterations": its, "us_per_iteration": round(t / its * 1e6, 1),
                "max_marginal_l1_reported": float(f"{res['marginal_error'].max().item():.3e}")}
        line.update(fp64_sinkhorn_errors(a, b, cost, eps, log_u, log_v, dist, its))
        if cpu_baseline:
            line["cpu_baseline"] = sinkhorn_cpu_baseline(a, b, cost, eps, its)
        out[f"sinkhorn_tc_256x8192_eps{eps}"] = line

    # pure iteration time (no setup / final cost): 60 minus 10 fixed iterations
    times = {}
    for k in (10, 60):
        _C.sinkhorn_tc_solve(a, b, cost, 0.05, k)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        _C.sinkhorn_tc_solve(a, b, cost, 0.05, k)
        e1.record(stream)
        torch.cuda.synchronize()
        times[k] = e0.elapsed_time(e1) / 1e3
    t_it = (times[60] - times[10]) / 50
    # per iteration: two products of (d x d) by (d x n), each as 3 bf16 MMA passes
    flops = 2 * 3 * 2.0 * d * d * n
    _, tc_peak, peak_kind = peaks()
    out["sinkhorn_tc_iteration_256x8192"] = {
        "us_per_iteration": round(t_it * 1e6, 1),
        "roofline": {"bound": "tensor", "achieved": round(flops / t_it / 1e12, 1),
                     "peak": tc_peak, "unit": "TFLOP/s", "frac": round(flops / t_it / 1e12 / tc_peak, 4),
                     "peak_kind": peak_kind,
                     "scope": "whole iteration (2 split-bf16 GEMMs of 8192x256x8192 with 3 MMA "
                              "passes each + 2 potential-split kernels); executed bf16 MMA flops"}}

    # the FP32 CUDA-core solver on the same GPU (tiled contractions, one persistent
    # launch per solve): per-iteration time from 13 minus 3 fixed iterations
    fp32 = {}
    for form, log_space in (("scaling", False), ("log", True)):
        t = {}
        for k in (3, 13):
            _C.sinkhorn_f32_solve(a, b, cost, 0.05, k, 0.0, log_space)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            _C.sinkhorn_f32_solve(a, b, cost, 0.05, k, 0.0, log_space)
            e1.record(stream)
            torch.cuda.synchronize()
            t[k] = e0.elapsed_time(e1) / 1e3
        fp32[form] = (t[13] - t[3]) / 10
    # scaling form: 2 d^2 n FMAs per half-step on the CUDA cores (2 flops each)
    fp32_flops = 2 * 2.0 * d * d * n
    out["sinkhorn_fp32_256x8192"] = {
        "ms_per_iteration_scaling": round(fp32["scaling"] * 1e3, 3),
        "ms_per_iteration_log": round(fp32["log"] * 1e3, 3),
        "scaling_TFLOPs_fp32": round(fp32_flops / fp32["scaling"] / 1e12, 1),
        "log_ex2_per_s": float(f"{2.0 * d * d * n / fp32['log']:.4g}"),
        "tensor_core_speedup_per_iteration_vs_scaling": round(fp32["scaling"] / t_it, 1),
        "tensor_core_speedup_per_iteration_vs_log": round(fp32["log"] / t_it, 1)}
    return out


def host_cores():
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()


def oracle_edt_rate(vols, warmup, steps, budget_s):
    """Oracle EDT (the reference algorithm restated in C: separable lower-envelope passes,
    OpenMP over every line of every volume) on the whole workload, all host threads.
    Returns (seconds per step, steps timed)."""
    import oracle

    oracle.build()
    cores = host_cores()
    for _ in range(warmup):
        oracle.edt(vols, nthreads=cores)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        oracle.edt(vols, nthreads=cores)
        times.append(time.perf_counter() - t0)
        if sum(times) > budget_s:
            break
    return sum(times) / len(times), len(times)


def _scipy_edt_volume(vol):
    from scipy import ndimage as ndi

    ndi.distance_transform_edt(vol, return_indices=True)
    return vol.size


def scipy_edt_rates(vols, budget_s=8.0):
    """scipy.ndimage.distance_transform_edt(return_indices=True) per volume: a loop on one
    thread, and a spawn-started process pool with one volume per worker."""
    import concurrent.futures as cf
    import multiprocessing as mp

    items = [np.ascontiguousarray(v[0]) for v in vols]
    nvox = sum(v.size for v in items)
    _scipy_edt_volume(items[0])  # import + warm-up
    t0, reps = time.perf_counter(), 0
    while True:
        for v in items:
            _scipy_edt_volume(v)
        reps += 1
        if time.perf_counter() - t0 > budget_s / 2 or reps >= 5:
            break
    one = nvox * reps / (time.perf_counter() - t0) / 1e9
    workers = min(len(items), host_cores())
    with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as pool:
        list(pool.map(_scipy_edt_volume, items))  # workers started and warmed outside the timing
        t0, reps = time.perf_counter(), 0
        while True:
            list(pool.map(_scipy_edt_volume, items))
            reps += 1
            if time.perf_counter() - t0 > budget_s / 2 or reps >= 10:
                break
        pooled = nvox * reps / (time.perf_counter() - t0) / 1e9
    return {"one_thread": {"value": round(one, 5), "unit": "Gvoxel/s", "cores": 1,
                           "sample": "the 4 volumes in a Python loop"},
            "process_pool": {"value": round(pooled, 5), "unit": "Gvoxel/s", "cores": workers,
                             "sample": f"the 4 volumes, one per worker of a {workers}-process pool"}}


def bench_reference(args):
    """The reference algorithm on the host CPU cores (oracle restatement, all threads)."""
    vols = edt_volumes(0)
    cores = host_cores()
    nvox = int(np.prod(EDT_SHAPE))
    per, nsteps = oracle_edt_rate(vols, args.warmup, args.steps, budget_s=60.0)
    value = nvox / per / 1e9
    return {
        "metric": METRIC, "impl": "reference", "value": round(value, 5), "unit": "Gvoxel/s",
        "n_gpus": args.gpus, "steps": nsteps, "warmup": args.warmup,
        "ms_per_step": round(per * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic: iid Bernoulli(0.9), numpy seed 0",
        "config": edt_config(args.gpus),
        "cpu_baseline": {"value": round(value, 5), "unit": "Gvoxel/s", "cores": cores, "kind": "port",
                         "sample": f"the full 4 x 128^3 workload, {nsteps} repetitions, OpenMP over "
                                   "the lines of every pass"},
        "e2e": {"value": round(value, 5), "unit": "Gvoxel/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def cpu_baseline_sample():
    """The reference arm's measurement, bounded: the oracle EDT on the whole 4 x 128^3
    workload with all host threads for ~10 s; scipy.ndimage beside it."""
    vols = edt_volumes(0)
    nvox = int(np.prod(EDT_SHAPE))
    per, reps = oracle_edt_rate(vols, 1, 100, budget_s=10.0)
    return {"value": round(nvox / per / 1e9, 5), "unit": "Gvoxel/s", "cores": host_cores(),
            "kind": "port", "sample": f"the full 4 x 128^3 workload, {reps} repetitions, oracle C port, "
                                      "OpenMP over the lines of every pass",
            "scipy": scipy_edt_rates(vols)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--headline-only", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--case", choices=["all", "grey", "binary", "cdt", "sinkhorn", "ragged", "ragged3d", "edt-shapes", "pointcloud",
                                       "pointcloud-profile"],
                    default="all",
                    help="only the shared-cost Sinkhorn, ragged-batch or point-cloud lines (one JSON object); "
                         "pointcloud-profile: the small fixed-iteration case used for ncu captures")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.case != "all" and args.impl == "ours":
        import torch

        dev = torch.device("cuda", 0)
        stream = torch.cuda.current_stream(dev)
        if args.case == "grey":
            print(json.dumps(grey_lines(args, dev, stream, peaks()[0])))
        elif args.case == "sinkhorn":
            print(json.dumps(sinkhorn_lines(dev, stream, cpu_baseline=not args.no_cpu_baseline)))
        elif args.case == "pointcloud":
            print(json.dumps(pointcloud_lines(dev, stream, cpu_baseline=not args.no_cpu_baseline)))
        elif args.case == "pointcloud-profile":
            print(json.dumps(pointcloud_profile_case(dev)))
        elif args.case == "ragged3d":
            print(json.dumps(ragged_volume_lines(dev, stream, max(args.steps, 10), args.warmup)))
        elif args.case == "binary":
            print(json.dumps(binary_lines(args, dev, stream, peaks()[0])))
        elif args.case == "cdt":
            print(json.dumps(cdt_lines(args, dev, stream)))
        elif args.case == "edt-shapes":
            print(json.dumps(edt_shape_lines(args, dev, stream, peaks()[0])))
        else:
            print(json.dumps(ragged_lines(dev, stream, max(args.steps, 10), args.warmup)))
        return

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(bench_reference(args)))
        return

    import torch

    if world > 1:
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        torch.distributed.init_process_group("nccl")
    result = bench_ours(args, rank, world)
    if rank == 0:
        result["cpu_baseline"] = None if args.no_cpu_baseline else cpu_baseline_sample()
        print(json.dumps(result))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
