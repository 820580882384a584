#!/usr/bin/env python
"""Benchmark of the GB300 upscaling backend (one JSON line on rank 0).

Workload (the headline metric's configuration): 1920x1080 RGB u8 frames
upscaled x2 to 3840x2160 by ACNetLegacy HDN0 through the full path (RGB->YUV
split, luma CNN, Catmull-Rom chroma resize, YUV->RGB merge); 8 distinct
frames per step, two alternating batches of 8 so each step's 50 MB of input
and 200 MB of output exceed the 129 MB L2.  Inputs are seeded synthetic
Voronoi-edge images (no public dataset is attached to this workload).

  value  output Mpx/s with inputs resident in HBM, CUDA events on the
         launching stream: the 8 frames of a step as one persistent launch
         (batch entry point) in the tensor-core forms; each frame's own
         launch (device-pointer entry point) is reported beside it
         ("per_frame_launch"), and the FP32 form runs frame by frame
  e2e    the same metric through the C ABI with pinned host buffers, H2D and
         D2H copies inside the timed region (several host threads share one
         processor, as the reference CLI does)

  batch  the batching workload: 64 RGB u8 images of uneven sizes (w in
         [256, 2048], h in [256, 1536]) x2 with ACNetLegacy HDN1, FP16 as one
         persistent launch per step (autotuned tile shape, CUDA-graph replay)
         against FP32 per-image launches

  video  the video workload: 8 frames of 1080p 10-bit YUV 4:2:0 u16 per step,
         x4 with ARNet-B8 (two x2 luma passes), FP16 tensor-core form vs FP32
  families  every network family of the reference on 1920x1080 u8 luma x2
         (device-resident, one launch sequence per frame): the tensor-core
         form where the family has one, and the plain FP32 form
  cli_default  the reference CLI's default model (ACNet<8> B8 HDN) on the
         headline's frames (8 RGB u8 1080p frames x2 per step, device
         resident): FP16 as one fused launch per step, FP32 frame by frame
  serve  the serving workload: Poisson arrivals (200 jobs/s) of mixed sizes,
         factors, models and formats through the serving loop; p50/p99
         latency and output Mpx/s, FP16 against FP32

--impl reference times the reference CPU path instead (the reference CPU
processor built from its sources where available, else the project's C
restatement of it) on the host cores, one frame per step.
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

METRIC = "Mpx/s out, 1080p→2160p ACNet: FP16-TC fused vs plain FP32; serve p50/p99 ms"
MODEL = "acnet-legacy-hdn0"
H, W, FACTOR = 1080, 1920, 2.0
OH, OW = 2160, 3840
FLOP_PER_OUT_PX = 2356.0  # ACNetLegacy x2: 9424 FLOP per input pixel
WORKLOAD = "1920x1080 RGB u8 -> 3840x2160 x2, ACNetLegacy HDN0, full split/CNN/chroma/merge path"
DATA = "synthetic: seeded 64-cell Voronoi-edge RGB u8 frames (blur 0.7, noise 2 LSB)"


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def make_frames(n, seed=0):
    from anime4kcpp_gb300 import synthetic
    base = [synthetic.rgb_u8(H, W, cells=64, seed=seed + i) for i in range(min(n, 4))]
    frames = []
    for i in range(n):
        b = base[i % len(base)]
        frames.append(np.ascontiguousarray(np.roll(b, shift=(37 * (i // len(base)), 53 * (i // len(base))), axis=(0, 1))))
    return frames


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


class ClockSampler:
    """SM clock, power and clock-event reasons sampled DURING the timed region.

    Reads them through NVML (the driver's libnvidia-ml, read-only queries)
    every 2 ms from a background thread, so even a region of a few tens of
    milliseconds gets samples; falls back to `nvidia-smi -lms 100` when the
    library cannot be loaded.  Nothing here changes a GPU setting."""

    # nvmlClocksEventReasons bits (nvml.h)
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}
    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, device, period_s=0.002):
        self.device = device
        self.period = period_s
        self.samples = []  # (sm_mhz, max_mhz, reasons bitmask)
        self.lines = []
        self.proc = None
        self.stop = threading.Event()
        self.thread = None
        self.source = None
        self.nvml = self._nvml()

    def _nvml(self):
        import ctypes
        try:
            lib = ctypes.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return None
            h = ctypes.c_void_p()
            # the CUDA device by its PCI address (NVML does not follow
            # CUDA_VISIBLE_DEVICES), else by index
            found = False
            try:
                import torch
                pr = torch.cuda.get_device_properties(self.device)
                bus = ("%08X:%02X:%02X.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)).encode()
                found = lib.nvmlDeviceGetHandleByPciBusId_v2(ctypes.c_char_p(bus), ctypes.byref(h)) == 0
            except Exception:
                found = False
            if not found and lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.device), ctypes.byref(h)) != 0:
                return None
            mx = ctypes.c_uint()
            if lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) != 0:
                return None
            self.max_mhz = float(mx.value)
            return lib, h
        except (OSError, AttributeError):
            return None

    def _poll(self):
        import ctypes
        lib, h = self.nvml
        clk, rs = ctypes.c_uint(), ctypes.c_ulonglong()
        get_reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        while not self.stop.is_set():
            if lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk)) == 0 and get_reasons(h, ctypes.byref(rs)) == 0:
                self.samples.append((float(clk.value), self.max_mhz, int(rs.value)))
            time.sleep(self.period)

    def __enter__(self):
        self.stop.clear()
        if self.nvml:
            self.source = "nvml every %.0f ms" % (self.period * 1e3)
            self.thread = threading.Thread(target=self._poll, daemon=True)
            self.thread.start()
            return self
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.source = "nvidia-smi every 100 ms"
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        self.stop.set()
        if self.thread:
            self.thread.join(timeout=2)
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        for clk, m, bits in self.samples:
            sm.append(clk)
            mx.append(m)
            for b, n in self.REASONS.items():
                if bits & b:
                    reasons.add(n)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm), "reasons": sorted(reasons),
                "source": self.source}


def reference_cpu_path():
    """The reference's CPU path as it runs on this host: the reference's own
    processor where it was compiled here (oracle/_ref), else the oracle's
    restatement of it in the operation order of the backend the reference
    selects on this host (aarch64: its NEON backend, as 4-lane vectors;
    x86-64: the same 4-lane order).  Returns (run(frame), kind, backend)."""
    import platform

    import oracle
    cores = os.cpu_count() or 1
    if oracle.ref_available():
        try:
            oracle.ref()
            name = oracle.ref().acref_name(MODEL.encode(), 0)
            return (lambda f: oracle.ref_process(f, FACTOR, MODEL, arch=0)), "reference", \
                (name.decode() if name else "reference CPU processor")
        except OSError:
            pass
    backend = "restated %s backend order (4-lane vectors), %s, %d threads" % (
        "NEON" if platform.machine() in ("aarch64", "arm64") else "NEON-order", platform.machine(), cores)
    return (lambda f: oracle.process(f, FACTOR, MODEL, threads=cores, order="neon")), "port", backend


def cpu_baseline(seconds=12.0):
    """The reference CPU path on this host's cores over a bounded sample of the
    workload: whole 1080p frames until ~`seconds` of work."""
    frame = make_frames(1, seed=100)[0]
    cores = os.cpu_count() or 1
    run, kind, backend = reference_cpu_path()
    use_ref = kind == "reference"

    def one():
        return run(frame)

    one()  # warm-up
    n, t0 = 0, time.perf_counter()
    while True:
        one()
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds or n >= 20:
            break
    return {"value": OW * OH * n / el / 1e6, "unit": "Mpx/s", "cores": cores,
            "kind": "reference" if use_ref else "port", "backend": backend,
            "sample": "%d full 1920x1080 RGB u8 frames x2 (%.1f s)" % (n, el)}


def run_reference(args, rank):
    if rank != 0:
        return None
    frame = make_frames(1, seed=100)[0]
    cores = os.cpu_count() or 1
    run, kind, backend = reference_cpu_path()
    use_ref = kind == "reference"

    def fn():
        return run(frame)
    for _ in range(args.warmup):
        fn()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        fn()
    el = time.perf_counter() - t0
    value = OW * OH * args.steps / el / 1e6
    kind = "reference" if use_ref else "port"
    return {
        "metric": METRIC, "value": value, "unit": "Mpx/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": DATA, "impl": "reference",
        "config": {"workload": WORKLOAD, "frames_per_step": 1, "note": "bounded sample: one frame per step on host cores"},
        "cpu_baseline": {"value": value, "unit": "Mpx/s", "cores": cores, "kind": kind, "backend": backend,
                         "sample": "%d steps of one 1920x1080 RGB u8 frame x2" % args.steps},
        "e2e": {"value": value, "unit": "Mpx/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def rank_barrier():
    """Barrier over the ranks of the process group (nothing on one rank)."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def max_over_ranks(x):
    """The largest x over the ranks (x itself on one rank).  The reduction
    tensor lives where the backend wants it: on the GPU for NCCL, on the host
    for gloo."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_mpx(px_per_rank, seconds, world):
    """Whole-job output Mpx/s of `world` replicas that each produced
    px_per_rank pixels, the slowest in `seconds` (weak scaling)."""
    return px_per_rank * world / seconds / 1e6


def time_device(ac, torch, proc, srcs, dsts, frames, steps, warmup, profile=False, clocks=None, batched=False):
    # A dedicated stream: the kernels and the timing events share it.
    stream = torch.cuda.Stream()
    handle = stream.cuda_stream
    nb = len(srcs) // frames

    def step(i):
        b = i % nb
        if batched:
            proc.process_batch_device(srcs[b * frames:(b + 1) * frames], dsts[b * frames:(b + 1) * frames], FACTOR,
                                      stream=handle, sync=False)
            return
        for j in range(frames):
            proc.process_device(srcs[b * frames + j], dsts[b * frames + j], FACTOR, stream=handle, sync=False)

    for i in range(warmup):
        step(i)
    torch.cuda.synchronize()
    if profile:
        proc.profile(True)
        proc.collect_profile()
    launches0 = ac.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx = clocks if clocks is not None else _Null()
    rank_barrier()  # every rank starts its timed steps together
    with ctx:
        e0.record(stream)
        for i in range(steps):
            step(i)
        e1.record(stream)
        torch.cuda.synchronize()
        rank_barrier()
        if clocks is not None:
            time.sleep(0.05)
    ms = e0.elapsed_time(e1)
    launches = ac.launch_count() - launches0
    prof = None
    if profile:
        prof = proc.collect_profile()
        proc.profile(False)
    if not proc.ok():
        raise RuntimeError(proc.error())
    return ms, launches, prof


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def time_e2e(ac, torch, proc, frames_host, outs_host, frames, steps, warmup, threads):
    """Host API: every call copies its frame in, runs, copies the result out.
    `threads` host threads (started before the clock) take the frames of all
    steps in order from a shared counter, as the reference CLI's thread pool
    takes images, so one step's copies overlap the next step's kernels; the
    timed region ends when every frame's result is in its host buffer."""
    import itertools

    def run(nsteps):
        total = nsteps * frames
        counter = itertools.count()
        errs = []
        go = threading.Event()

        def worker():
            go.wait()
            while True:
                k = next(counter)
                if k >= total:
                    return
                i, j = divmod(k, frames)
                idx = (i % 2) * frames + j
                proc.process(frames_host[idx], FACTOR, dst=outs_host[idx])
                if not proc.ok():
                    errs.append(proc.error())

        ts = [threading.Thread(target=worker) for _ in range(threads)]
        [t.start() for t in ts]
        rank_barrier()
        t0 = time.perf_counter()
        go.set()
        [t.join() for t in ts]
        el = time.perf_counter() - t0
        rank_barrier()
        if errs:
            raise RuntimeError(errs[0])
        return el

    run(warmup)
    return run(steps)


BATCH_MODEL = "acnet-legacy-hdn1"


def batch_images(n=64, seed=3):
    """n RGB u8 images with width uniform in [256, 2048] and height uniform in
    [256, 1536] (seeded), cut at seeded offsets from four 2048x1536 Voronoi-edge
    canvases (256 cells each)."""
    from anime4kcpp_gb300 import synthetic
    canvases = [synthetic.rgb_u8(1536, 2048, cells=256, seed=seed * 10 + i) for i in range(4)]
    rng = np.random.default_rng(seed)
    out = []
    for i, (h, w) in enumerate(synthetic.uneven_sizes(n, seed=seed)):
        c = canvases[i % 4]
        y0, x0 = int(rng.integers(0, 1536 - h + 1)), int(rng.integers(0, 2048 - w + 1))
        out.append(np.ascontiguousarray(c[y0:y0 + h, x0:x0 + w]))
    return out


def time_batch(ac, torch, args):
    """The batching workload: 64 uneven RGB u8 images x2 with ACNetLegacy HDN1.
    FP16: one persistent launch per step over all images (autotuned tile
    shape, replayed CUDA graph); FP32: one launch per image.  Output Mpx/s
    with inputs resident in HBM, CUDA events on the launching stream."""
    imgs = batch_images()
    srcs = [torch.from_numpy(x).cuda() for x in imgs]
    dsts = [torch.empty((2 * x.shape[0], 2 * x.shape[1], 3), dtype=torch.uint8, device="cuda") for x in imgs]
    out_px = sum(4 * x.shape[0] * x.shape[1] for x in imgs)
    stream = torch.cuda.Stream()
    res = {"workload": "64 RGB u8 images, w~U[256,2048], h~U[256,1536] (seed 3), x2 ACNetLegacy HDN1",
           "out_mpx_per_step": out_px / 1e6}
    for form, steps in (("fp16", max(3, args.batch_steps)), ("fp32", max(3, args.batch_steps // 4))):
        proc = ac.Processor("cuda", 0, BATCH_MODEL, precision=form)
        with torch.cuda.stream(stream):
            h = stream.cuda_stream

            def step():
                if form == "fp32":
                    for a, b in zip(srcs, dsts):
                        proc.process_device(a, b, 2.0, stream=h, sync=False)
                else:
                    proc.process_batch_device(srcs, dsts, 2.0, stream=h, sync=False)

            for _ in range(max(3, args.warmup)):
                step()
            torch.cuda.synchronize()
            l0, r0 = ac.launch_count(), ac.graph_replays()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                step()
            e1.record(stream)
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        if not proc.ok():
            raise RuntimeError(proc.error())
        res[form] = {"value": out_px * steps / (ms / 1e3) / 1e6, "unit": "Mpx/s", "ms_per_batch": ms / steps,
                     "steps": steps, "launches_per_batch": (ac.launch_count() - l0) / steps,
                     "graph_replays_per_batch": (ac.graph_replays() - r0) / steps}
        if form != "fp32":
            res[form]["plan"] = dict(proc.last_plan(), chosen_by="autotuner: every tile shape, and the network split "
                                                                  "in two launches, x {2, 1} CTAs per SM, timed once "
                                                                  "for this batch class")
        if not args.no_error_stats:
            res[form]["error"] = dict(error_vs_fp64(dsts[0].cpu().numpy(), imgs[0], BATCH_MODEL),
                                      sample="image 0 (%dx%d)" % (imgs[0].shape[1], imgs[0].shape[0]))
    res["fp16_over_fp32"] = res["fp16"]["value"] / res["fp32"]["value"]
    return res


def time_video(ac, torch, args):
    """The video workload: 120 frames of 1920x1080 10-bit YUV 4:2:0 in u16 (a
    seeded Voronoi-edge canvas translated 3 px per frame, noise 4 LSB), 8
    frames per call (15 calls per pass over the clip), x4 with ARNet-B8 as two
    chained x2 luma passes (Y shifted by 6 around the network, the reference
    CLI's recipe), chroma Catmull-Rom resized.  Output Mpx/s (luma frame
    pixels) with inputs resident in HBM; `args.video_steps` passes over the
    clip (FP32: half as many)."""
    from anime4kcpp_gb300 import synthetic
    nf, per_call = 120, 8
    canvas_y = synthetic.luma(1080, 1920 + 3 * nf, np.uint16, cells=256, seed=81, noise=4.0, bits=10)
    canvas_c = [synthetic.luma(540, 960 + 3 * nf // 2, np.uint16, cells=256, seed=82 + k, noise=4.0, bits=10) for k in range(2)]
    frames = []
    for f in range(nf):
        dx = 3 * f
        planes = (canvas_y[:, dx:dx + 1920], canvas_c[0][:, dx // 2:dx // 2 + 960], canvas_c[1][:, dx // 2:dx // 2 + 960])
        frames.append(tuple(torch.from_numpy(np.ascontiguousarray(p)).cuda() for p in planes))
    outs = [(torch.empty((4320, 7680), dtype=torch.uint16, device="cuda"),
             torch.empty((2160, 3840), dtype=torch.uint16, device="cuda"),
             torch.empty((2160, 3840), dtype=torch.uint16, device="cuda")) for _ in range(per_call)]
    calls = [frames[i:i + per_call] for i in range(0, nf, per_call)]
    res = {"workload": "120 frames 1920x1080 10-bit YUV420 u16 (canvas translated 3 px/frame), 8 frames per call, "
                       "x4 ARNet-B8 (two x2 luma passes, shift 6), chroma Catmull-Rom"}
    stream = torch.cuda.Stream()
    for form in ("fp16", "fp32"):
        proc = ac.Processor("cuda", 0, "arnet-b8", precision=form)
        steps = max(1, args.video_steps if form == "fp16" else args.video_steps // 2)
        with torch.cuda.stream(stream):
            h = stream.cuda_stream
            proc.process_yuv_device(calls[0], outs, 4.0, 6, stream=h, sync=True)
            l0 = ac.launch_count()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                for c in calls:
                    proc.process_yuv_device(c, outs, 4.0, 6, stream=h, sync=False)
            e1.record(stream)
            torch.cuda.synchronize()
        if not proc.ok():
            raise RuntimeError(proc.error())
        ms = e0.elapsed_time(e1) / steps
        res[form] = {"value": nf * 7680 * 4320 / (ms / 1e3) / 1e6, "unit": "Mpx/s", "ms_per_120_frames": ms,
                     "ms_per_frame": ms / nf, "passes": steps,
                     "launches_per_8_frames": (ac.launch_count() - l0) / (steps * len(calls))}
        if not args.no_error_stats:
            # the last call's first frame (frame 112), checked against the FP64 oracle
            res[form]["error"] = dict(video_error(outs[0][0].cpu().numpy(), calls[-1][0][0].cpu().numpy(), "arnet-b8"),
                                      frame=nf - per_call)
    res["fp16_over_fp32"] = res["fp16"]["value"] / res["fp32"]["value"]
    return res


FAMILIES = [("acnet-legacy-hdn0", True), ("acnet-f8b8-hdn", True), ("arnet-b8", True), ("artcnn-c4f16", True),
            ("artcnn-c4f32", True), ("fsrcnnx-f8", True), ("fsrcnnx-f16", True)]


def time_families(ac, torch, args):
    """Every network family on a 1920x1080 u8 luma plane x2 (Voronoi-edge
    content), device-resident, CUDA events on the launching stream: output
    Mpx/s of the FP16 tensor-core form (where the family has one) and of the
    plain FP32 form."""
    from anime4kcpp_gb300 import synthetic
    x = synthetic.luma(H, W, np.uint8, cells=64, seed=90)
    src = torch.from_numpy(x).cuda()
    dst = torch.empty((OH, OW), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    out = {"workload": "1920x1080 u8 luma -> 3840x2160 x2 per family, one frame per step"}
    for model, has_tc in FAMILIES:
        rec = {}
        for form in (("fp16", "fp32") if has_tc else ("fp32",)):
            p = ac.Processor("cuda", 0, model, precision=form)
            h = stream.cuda_stream
            for _ in range(2):
                p.process_device(src, dst, 2.0, stream=h, sync=False)
            torch.cuda.synchronize()
            steps = max(3, args.family_steps)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                p.process_device(src, dst, 2.0, stream=h, sync=False)
            e1.record(stream)
            torch.cuda.synchronize()
            if not p.ok():
                raise RuntimeError(p.error())
            ms = e0.elapsed_time(e1) / steps
            rec[form] = {"ms_per_frame": round(ms, 4), "value": OW * OH / (ms / 1e3) / 1e6, "unit": "Mpx/s"}
            if not args.no_error_stats:
                rec[form]["error"] = error_vs_fp64(dst.cpu().numpy(), x, model)
        if has_tc:
            rec["fp16_over_fp32"] = rec["fp16"]["value"] / rec["fp32"]["value"]
        out[model] = rec
    return out


CLI_MODEL = "acnet-f8b8-hdn"  # the reference CLI's default model


def time_cli_default(ac, torch, args):
    """ACNet<8> B8 HDN on 8 RGB u8 1920x1080 frames x2 per step, inputs
    resident in HBM, CUDA events on the launching stream.  FP16: the batch
    entry point, one persistent launch per step (split, CNN, chroma resample
    and merge fused); FP32: the per-layer FP32 pipeline frame by frame."""
    frames = make_frames(8, seed=200)
    srcs = [torch.from_numpy(f).cuda() for f in frames]
    dsts = [torch.empty((OH, OW, 3), dtype=torch.uint8, device="cuda") for _ in frames]
    stream = torch.cuda.Stream()
    h = stream.cuda_stream
    out = {"workload": "%s, 8 x 1920x1080 RGB u8 -> 3840x2160 per step" % CLI_MODEL}
    for form, steps in (("fp16", max(3, args.cli_steps)), ("fp32", max(3, args.cli_steps // 2))):
        p = ac.Processor("cuda", 0, CLI_MODEL, precision=form)

        def step():
            if form == "fp32":
                for a, b in zip(srcs, dsts):
                    p.process_device(a, b, 2.0, stream=h, sync=False)
            else:
                p.process_batch_device(srcs, dsts, 2.0, stream=h, sync=False)

        for _ in range(3):
            step()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        if not p.ok():
            raise RuntimeError(p.error())
        ms = e0.elapsed_time(e1) / steps
        out[form] = {"ms_per_step": round(ms, 4), "value": 8 * OW * OH / (ms / 1e3) / 1e6, "unit": "Mpx/s"}
        if not args.no_error_stats:
            out[form]["error"] = dict(error_vs_fp64(dsts[0].cpu().numpy(), frames[0], CLI_MODEL), sample="frame 0")
    out["fp16_over_fp32"] = out["fp16"]["value"] / out["fp32"]["value"]
    return out


SERVE_RES = [(480, 854), (720, 1280), (1080, 1920), (2160, 3840)]
SERVE_RES_W = [1, 2, 2, 1]
SERVE_MODELS = ["acnet-legacy-hdn0", "acnet-legacy-hdn1", "acnet-legacy-hdn2", "acnet-legacy-hdn3", "arnet-b8"]


_SERVE_BUFFERS = []


def serve_buffers(torch):
    """The serving workload's pinned host buffers: one input per size and
    format, and rings of output slots per (size, factor, format).  Allocated
    once per process, as a serving client allocates its staging memory at
    start-up (pinning and unpinning ~8.5 GB per run would also disturb the
    copies being measured)."""
    if _SERVE_BUFFERS:
        return _SERVE_BUFFERS[0]
    from anime4kcpp_gb300 import synthetic
    canvas = synthetic.rgb_u8(2160, 3840, cells=256, seed=70)
    luma = synthetic.luma(2160, 3840, np.uint16, cells=256, seed=71, noise=4.0, bits=10)
    chroma = [synthetic.luma(1080, 1920, np.uint16, cells=256, seed=72 + k, noise=4.0, bits=10) for k in range(2)]

    def pinned(a):
        return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()

    inputs = {}
    for ri, (h, w) in enumerate(SERVE_RES):
        inputs[(ri, "rgb")] = pinned(canvas[:h, :w])
        inputs[(ri, "yuv")] = (pinned(luma[:h, :w]), pinned(chroma[0][:h // 2, :w // 2]), pinned(chroma[1][:h // 2, :w // 2]))
    rings = {}
    for ri, (h, w) in enumerate(SERVE_RES):
        for f in (2, 4):
            n = 3 if (ri == 3 and f == 4) else 10
            rings[(ri, f, "rgb")] = [pinned(np.empty((f * h, f * w, 3), np.uint8)) for _ in range(n)]
            rings[(ri, f, "yuv")] = [(pinned(np.empty((f * h, f * w), np.uint16)),
                                      pinned(np.empty((f * h // 2, f * w // 2), np.uint16)),
                                      pinned(np.empty((f * h // 2, f * w // 2), np.uint16))) for _ in range(n)]
    _SERVE_BUFFERS.append((inputs, rings))
    return inputs, rings


def time_serve(ac, torch, args, forms=("fp16", "fp32")):
    """The serving workload: an open-loop Poisson stream of upscale jobs at
    `args.serve_rate` jobs/s for `args.serve_seconds` s through the serving
    loop (ac.Server, 80 GB HBM budget, `args.serve_workers` worker streams).  Sizes 854x480,
    1280x720, 1920x1080, 3840x2160 in ratio 1:2:2:1; factor 2 or 4 in ratio
    3:1; models ACNetLegacy HDN0-3 and ARNet B8 chosen uniformly; formats RGB
    u8 or 10-bit YUV 4:2:0 u16 (planar, shift 6) in ratio 4:1.  Latency =
    submit -> result in the caller's pinned host buffer.  Then the FP16 form
    at higher offered rates (`args.serve_load_rates`, `args.serve_load_seconds`
    each): where continuous batching engages."""
    import queue
    inputs, rings = serve_buffers(torch)
    free = {}
    for k, v in rings.items():
        free[k] = queue.Queue()
        for i in range(len(v)):
            free[k].put(i)

    def stream_of(rate, seconds, seed):
        rng = np.random.default_rng(seed)
        arrivals = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * seconds * 1.5) + 10))
        arrivals = arrivals[arrivals < seconds]
        picks = [(int(rng.choice(4, p=np.array(SERVE_RES_W) / 6.0)), 2 if rng.random() < 0.75 else 4,
                  SERVE_MODELS[int(rng.integers(0, 5))], "rgb" if rng.random() < 0.8 else "yuv") for _ in arrivals]
        return arrivals, picks

    def warm(srv):
        # every model, format, factor and size (processors, weights, work
        # buffers and pool blocks of every size class), largest first, as
        # many concurrent jobs of each kind as there are workers (each worker
        # thread keeps its own work buffers) as far as the output rings allow
        for ri in reversed(range(len(SERVE_RES))):
            for m in SERVE_MODELS:
                for fmt in ("rgb", "yuv"):
                    for f in (4, 2):
                        key = (ri, f, fmt)
                        held = [free[key].get_nowait() for _ in range(min(args.serve_workers, free[key].qsize()))]
                        try:
                            ts = [srv.submit(inputs[(ri, fmt)], rings[key][slot], m, float(f), 6 if fmt == "yuv" else 0)
                                  for slot in held]
                            for t in ts:
                                srv.wait(t, timeout=600.0)
                        finally:
                            for slot in held:
                                free[key].put(slot)

    def run(srv, arrivals, picks):
        done = queue.Queue()
        tickets = queue.Queue()
        stalls = [0]

        def collect():
            while True:
                item = tickets.get()
                if item is None:
                    return
                t, key, slot, meta = item
                r = srv.wait(t, timeout=600.0)
                free[key].put(slot)
                done.put((r, meta))

        collectors = [threading.Thread(target=collect, daemon=True) for _ in range(8)]
        [c.start() for c in collectors]
        st0 = srv.stats()
        t0 = time.perf_counter()
        for at, (ri, f, m, fmt) in zip(arrivals, picks):
            delay = t0 + at - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            key = (ri, f, fmt)
            try:
                slot = free[key].get_nowait()
            except queue.Empty:
                stalls[0] += 1
                slot = free[key].get()
            h, w = SERVE_RES[ri]
            t = srv.submit(inputs[(ri, fmt)], rings[key][slot], m, float(f), 6 if fmt == "yuv" else 0)
            tickets.put((t, key, slot, (ri, f, m, fmt, f * f * h * w)))
        for _ in collectors:
            tickets.put(None)
        [c.join() for c in collectors]
        wall = time.perf_counter() - t0
        st1 = srv.stats()
        res = [done.get() for _ in range(done.qsize())]

        def pct(vals, q):
            return float(np.percentile(vals, q)) if len(vals) else None

        lat = np.array([r["latency_ms"] for r, _ in res])
        ok = [r for r, _ in res if r["status"] == 0]
        r1080 = [r for r, m in res if m[0] == 2]
        lat1080 = np.array([r["latency_ms"] for r in r1080])
        lat1080x2 = np.array([r["latency_ms"] for r, m in res if m[0] == 2 and m[1] == 2 and m[3] == "rgb" and "acnet" in m[2]])
        by_class = {}
        for r, m in res:
            if m[0] == 2:
                by_class.setdefault((m[1], "arnet" if "arnet" in m[2] else "acnet", m[3]), []).append(r["device_ms"])
        return {
            "completed": len(ok), "failed": len(res) - len(ok), "jobs": len(res),
            "out_mpx_per_s": sum(m[4] for r, m in res if r["status"] == 0) / wall / 1e6,
            "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99),
            "p50_ms_1080p": pct(lat1080, 50), "p99_ms_1080p": pct(lat1080, 99),
            "p99_ms_1080p_acnet_x2_rgb": pct(lat1080x2, 99),
            # the 1080p p99 split: admission queue, waiting for a worker, on the device (copies included)
            "p99_ms_1080p_parts": {"admission": pct([r["queue_ms"] for r in r1080], 99),
                                   "worker_wait": pct([r["latency_ms"] - r["queue_ms"] - r["device_ms"] for r in r1080], 99),
                                   "device": pct([r["device_ms"] for r in r1080], 99)},
            # the device part on the worker's stream (CUDA events): input copies, processing, output
            # copies, and what the events do not cover (host work of the worker between them)
            "p99_ms_1080p_device_parts": {
                "h2d": pct([r["h2d_ms"] for r in r1080], 99), "compute": pct([r["compute_ms"] for r in r1080], 99),
                "d2h": pct([r["d2h_ms"] for r in r1080], 99),
                "outside_events": pct([r["device_ms"] - r["h2d_ms"] - r["compute_ms"] - r["d2h_ms"] for r in r1080], 99)},
            # 1080p classes (factor, family, format): jobs and p99 device ms
            "p99_device_ms_1080p_by_class": {
                "x%d/%s/%s" % (f, fam, fmt): {"jobs": len(v), "p99": pct(v, 99)}
                for (f, fam, fmt), v in sorted(by_class.items())},
            "mean_queue_ms": float(np.mean([r["queue_ms"] for r, _ in res])) if res else None,
            "batched_jobs": int(st1["batched_jobs"] - st0["batched_jobs"]), "batches": int(st1["batches"] - st0["batches"]),
            "mean_jobs_per_launch_when_batched": (st1["batched_jobs"] - st0["batched_jobs"]) /
            max(1, st1["batches"] - st0["batches"]),
            "device_allocs_during_run": int(st1["device_allocs"] - st0["device_allocs"]),
            "peak_admitted_gb": st1["peak_bytes"] / 1e9, "wall_s": wall, "generator_stalls": stalls[0]}

    out = {"workload": "Poisson %.0f jobs/s for %.0f s; 480p:720p:1080p:2160p = 1:2:2:1; x2:x4 = 3:1; "
                       "ACNetLegacy HDN0-3 / ARNet-B8 uniform; RGB u8 : 10-bit YUV420 u16 = 4:1; 80 GB budget, "
                       "%d worker streams" % (args.serve_rate, args.serve_seconds, args.serve_workers)}
    arrivals, picks = stream_of(args.serve_rate, args.serve_seconds, 7)
    out["jobs"] = len(arrivals)
    for form in forms:
        srv = ac.Server(0, form, hbm_budget_gb=80.0, workers=args.serve_workers)
        warm(srv)
        out[form] = run(srv, arrivals, picks)
        if form == "fp16" and args.serve_load_seconds > 0:
            loads = []
            for k, rate in enumerate(args.serve_load_rates):
                a, p = stream_of(rate, args.serve_load_seconds, 100 + k)
                rec = run(srv, a, p)
                loads.append(dict(rec, offered_jobs_per_s=rate, seconds=args.serve_load_seconds))
            out["fp16_load_points"] = loads
        srv.close()
    return out


def time_serve_saturation(ac, torch, args):
    """Continuous batching under saturation: 1920x1080 RGB u8 x2 ACNetLegacy
    HDN0 jobs (FP16) offered at `args.saturation_rate` jobs/s for 2 s through
    the serving loop; reports the served rate, latency and how many jobs
    shared launches."""
    import queue
    frame = torch.from_numpy(make_frames(1, seed=77)[0]).pin_memory().numpy()
    ring = [torch.empty((OH, OW, 3), dtype=torch.uint8).pin_memory().numpy() for _ in range(48)]
    free = queue.Queue()
    for i in range(len(ring)):
        free.put(i)
    srv = ac.Server(0, "fp16", hbm_budget_gb=80.0, workers=4)
    for _ in range(3):
        srv.wait(srv.submit(frame, ring[0], MODEL, 2.0))
    tickets, lats = queue.Queue(), []

    def collect():
        while True:
            item = tickets.get()
            if item is None:
                return
            r = srv.wait(item[0], timeout=600.0)
            free.put(item[1])
            lats.append((r["latency_ms"], r["batch"], r["status"]))

    cs = [threading.Thread(target=collect, daemon=True) for _ in range(8)]
    [c.start() for c in cs]
    n = int(args.saturation_rate * 2.0)
    t0 = time.perf_counter()
    for i in range(n):
        delay = t0 + i / args.saturation_rate - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        slot = free.get()
        tickets.put((srv.submit(frame, ring[slot], MODEL, 2.0), slot))
    for _ in cs:
        tickets.put(None)
    [c.join() for c in cs]
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    lat = np.array([x[0] for x in lats])
    return {"workload": "1920x1080 RGB u8 x2 HDN0 FP16 jobs offered at %.0f/s for 2 s (48 pinned output slots)"
                        % args.saturation_rate,
            "served_jobs_per_s": n / wall, "out_mpx_per_s": n * OW * OH / wall / 1e6,
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_batch": float(np.mean([x[1] for x in lats])), "batched_jobs": int(st["batched_jobs"]),
            "failed": int(sum(1 for x in lats if x[2] != 0))}


def error_vs_fp64(got, img, model):
    """Error statistics of one result against the FP64 oracle of the same
    path (the luma network in FP64, every other step at the reference's
    rounding points): max_abs, psnr_db, max_lsb, frac_within_1lsb.  Checker
    use of the oracle, outside every timed region."""
    import oracle
    exact, quant = oracle.pipeline_f64(img, model)
    st = oracle.error_stats(got, exact, quant)
    return {k: (round(v, 7) if isinstance(v, float) else v) for k, v in st.items()}


def video_error(got10, y10, model, shift=6):
    """Error of one x4 video frame's Y plane (10-bit content in u16) against
    the FP64 oracle at the reference CLI's rounding points: Y << shift, two
    FP64 x2 passes with the intermediate quantised to u16 (fromFloat), the
    result through fromFloat and >> shift.  In 10-bit LSB: max_lsb and
    frac_within_1lsb against that quantised output; psnr_db on the 10-bit
    grid (peak 1023) against it."""
    import oracle
    y16 = (y10.astype(np.uint32) << shift).astype(np.uint16)
    p1 = oracle.process_f64(y16, model)
    p2 = oracle.process_f64(oracle.from_float_np(p1, np.uint16), model)
    q10 = (oracle.from_float_np(p2, np.uint16) >> shift).astype(np.int64)
    d = got10.astype(np.int64) - q10
    mse = float(np.mean((d / 1023.0) ** 2))
    exact10 = np.clip(p2, 0.0, 1.0) * 65535.0 / (1 << shift)
    return {"max_abs": round(float(np.abs(got10 + 0.5 - exact10).max() / 1023.0), 7),
            "psnr_db": 99.0 if mse == 0 else round(10 * np.log10(1.0 / mse), 3),
            "max_lsb": int(np.abs(d).max()), "frac_within_1lsb": round(float((np.abs(d) <= 1).mean()), 7),
            "samples": int(d.size), "sample": "one frame's Y plane, 10-bit LSB; psnr against the quantised FP64 oracle"}


PREC_MODEL = "acnet-legacy-hdn3"


def time_precision(ac, torch, args):
    """The precision workload: one 3840x2160 RGB u8 frame (256 Voronoi cells)
    x2 to 7680x4320 with ACNetLegacy HDN3 in the FP16, BF16 and FP32 forms,
    and one 1920x1080 f32 luma plane (uniform [0, 1] cell values plus the
    outline structure) x2 with HDN3; each timed (inputs resident in HBM, one
    launch per frame, CUDA events on the launching stream) and checked
    against the FP64 oracle."""
    from anime4kcpp_gb300 import synthetic
    out = {"workload": "3840x2160 RGB u8 (256 cells) -> 7680x4320 and 1920x1080 f32 luma -> 3840x2160, "
                       "ACNetLegacy HDN3 x2, FP16 / BF16 / FP32"}
    stream = torch.cuda.Stream()
    h = stream.cuda_stream
    cases = [("rgb_4k_u8", synthetic.rgb_u8(2160, 3840, cells=256, seed=2160), (4320, 7680, 3), torch.uint8),
             ("luma_1080p_f32", synthetic.f32_luma_uniform(1080, 1920, seed=1081), (2160, 3840), torch.float32)]
    for name, img, oshape, odt in cases:
        src = torch.from_numpy(img).cuda()
        dst = torch.empty(oshape, dtype=odt, device="cuda")
        rec = {}
        for form in ("fp16", "bf16", "fp32"):
            p = ac.Processor("cuda", 0, PREC_MODEL, precision=form)
            for _ in range(2):
                p.process_device(src, dst, 2.0, stream=h, sync=False)
            torch.cuda.synchronize()
            steps = max(3, args.precision_steps)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                p.process_device(src, dst, 2.0, stream=h, sync=False)
            e1.record(stream)
            torch.cuda.synchronize()
            if not p.ok():
                raise RuntimeError(p.error())
            ms = e0.elapsed_time(e1) / steps
            rec[form] = {"ms_per_frame": round(ms, 4), "value": oshape[0] * oshape[1] / (ms / 1e3) / 1e6,
                         "unit": "Mpx/s", "error": error_vs_fp64(dst.cpu().numpy(), img, PREC_MODEL)}
        rec["fp16_over_fp32"] = rec["fp16"]["value"] / rec["fp32"]["value"]
        out[name] = rec
    return out


def run_gb300(args, rank, world, local_rank):
    import torch

    import anime4kcpp_gb300 as ac
    from anime4kcpp_gb300 import build
    build.build()
    torch.cuda.set_device(local_rank)
    frames = args.frames
    host = make_frames(2 * frames, seed=10 * rank)
    srcs = [torch.from_numpy(f).cuda() for f in host]
    dsts = [torch.empty((OH, OW, 3), dtype=torch.uint8, device="cuda") for _ in host]

    forms = {}
    headline = None
    for form in args.forms:
        proc = ac.Processor("cuda", local_rank, MODEL, precision=form)
        if not proc.ok():
            raise RuntimeError(proc.error())
        try:
            time_device(ac, torch, proc, srcs[:frames], dsts[:frames], frames, 1, 1)
        except RuntimeError as e:
            forms[form] = {"unavailable": str(e)}
            continue
        is_head = headline is None
        sampler = ClockSampler(local_rank) if is_head else None
        steps = args.steps if is_head else max(3, args.steps // 2)
        batched = form != "fp32" and not args.per_frame
        ms, launches, prof = time_device(ac, torch, proc, srcs, dsts, frames, steps, args.warmup, profile=True,
                                         clocks=sampler, batched=batched)
        out_px = OW * OH * frames * steps
        rec = {"value": out_px / (ms / 1e3) / 1e6, "ms_per_step": ms / steps, "launches": launches,
               "kernel_ms_per_launch": prof[0] / max(prof[1], 1), "kernel_launches": prof[1],
               "kernel_out_px": prof[2], "steps": steps, "launch": "one per step (8 frames)" if batched else "one per frame"}
        if batched:
            # the autotuner's plan for the 8-frame class: one kernel (fusion
            # depth 9) or the network split in two kernels (depth 5)
            rec["plan"] = proc.last_plan()
            rec["kernels_per_launch"] = 2 if rec["plan"].get("fusion_depth") == 5 else 1
            # the same frames, each in its own launch
            pms, plaunches, pprof = time_device(ac, torch, proc, srcs, dsts, frames, max(3, steps // 2), args.warmup,
                                                profile=True)
            psteps = max(3, steps // 2)
            rec["per_frame_launch"] = {"value": OW * OH * frames * psteps / (pms / 1e3) / 1e6, "ms_per_step": pms / psteps,
                                       "launches": plaunches, "kernel_ms_per_launch": pprof[0] / max(pprof[1], 1)}
        if not args.no_error_stats:
            torch.cuda.synchronize()
            rec["error"] = error_vs_fp64(dsts[0].cpu().numpy(), host[0], MODEL)
        forms[form] = rec
        if is_head:
            headline = (form, proc, rec, sampler)

    if headline is None:
        raise RuntimeError("no arithmetic form ran: %s" % forms)
    form, proc, rec, sampler = headline

    # max over ranks of the headline time
    if world > 1:
        rec["ms_per_step"] = max_over_ranks(rec["ms_per_step"])
        rec["value"] = replica_mpx(OW * OH * frames, rec["ms_per_step"] / 1e3, world)

    # end to end through the C ABI with pinned host buffers
    pin_src = [torch.from_numpy(f).pin_memory() for f in host]
    pin_dst = [torch.empty((OH, OW, 3), dtype=torch.uint8).pin_memory() for _ in host]
    # at least 40 steps (320 frames, ~60 ms): long enough that the host
    # threads' start and drain do not weigh on the figure
    e2e_steps = max(2 * args.steps, 40)
    el = time_e2e(ac, torch, proc, [p.numpy() for p in pin_src], [p.numpy() for p in pin_dst], frames, e2e_steps,
                  max(2, args.warmup), args.e2e_threads)
    e2e_value = replica_mpx(OW * OH * frames * e2e_steps, max_over_ranks(el), world)

    peaks = measured_peaks()
    kernel_s = rec["kernel_ms_per_launch"] / 1e3
    flops_per_launch = FLOP_PER_OUT_PX * rec["kernel_out_px"] / max(rec["kernel_launches"], 1)
    achieved = flops_per_launch / kernel_s / 1e12
    props = torch.cuda.get_device_properties(local_rank)
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    fp32_peak = 2.0 * 128 * props.multi_processor_count * sm_max * 1e6 / 1e12
    traffic = None
    tr_path = os.path.join(ROOT, "profiles", "traffic.json")
    split = rec.get("kernels_per_launch", 1) == 2
    if os.path.exists(tr_path):
        rec_t = json.load(open(tr_path)).get(form + ("_split" if split else ""))
        traffic = rec_t.get("bytes") if isinstance(rec_t, dict) else rec_t
    if form == "fp32":
        roofline = {"bound": "fp32-core", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                    "frac": achieved / fp32_peak, "traffic": traffic,
                    "peak_source": "computed 2 x 128 FP32 lanes x %d SMs x %.0f MHz (not in MEASURED_PEAKS)" % (props.multi_processor_count, sm_max)}
    else:
        # the kernel is timed alone over a short region (tens of ms): the
        # measured burst peak applies
        peak = float(peaks.get("bf16_tflops", 1900.0))
        roofline = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                    "traffic": traffic, "peak_source": "of measured (MEASURED_PEAKS.json bf16_tflops, burst)"
                    if "bf16_tflops" in peaks else "of fallback (1.9 PFLOP/s burst)",
                    "kernel": "the step's launch: head + tail kernels of the split network (fusion depth 5 + 4)"
                    if split else "the step's launch: the quad kernel, whole network (fusion depth 9)"}

    out = {
        "metric": METRIC, "value": rec["value"], "unit": "Mpx/s", "n_gpus": world, "steps": rec["steps"],
        "warmup": args.warmup, "ms_per_step": rec["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if form == "fp32" else ("f16" if form == "fp16" else "bf16"),
        "data": DATA,
        "config": {"workload": WORKLOAD, "frames_per_step": frames, "form": form, "launch": rec["launch"],
                   "value_is": ("the %d frames of a step as ONE persistent launch (batch entry point); one launch per "
                                "frame is value_per_frame_launch" % frames) if "per_frame_launch" in rec else
                               "one launch per frame",
                   "value_per_frame_launch": rec.get("per_frame_launch", {}).get("value"),
                   "l2": "inputs larger than L2: 2 alternating batches of 8 distinct frames (50 MB in, 200 MB out per step)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": e2e_value, "unit": "Mpx/s", "h2d_bytes_per_step": H * W * 3 * frames,
                "d2h_bytes_per_step": OH * OW * 3 * frames, "host_threads": args.e2e_threads, "steps": e2e_steps,
                "call": "ac_processor_process per frame (C ABI, pinned host buffers, copies in the timed region)"},
        "gpu_launches": rec["launches"],
        "roofline": roofline,
        "forms": {k: ({kk: round(vv, 4) if isinstance(vv, float) else vv for kk, vv in v.items()}) for k, v in forms.items()},
    }
    if "fp32" in forms and "value" in forms["fp32"]:
        for tc in ("fp16", "bf16"):
            if tc in forms and "value" in forms[tc]:
                out["%s_over_fp32" % tc] = forms[tc]["value"] / forms["fp32"]["value"]
    if "error" in rec:
        out["error"] = dict(rec["error"], oracle="FP64 network, reference rounding points (oracle.pipeline_f64)",
                            sample="frame 0 of the step, 1920x1080 RGB u8 x2")
    clocks = sampler.summary() if sampler else None
    out["clocks"] = clocks
    if rank == 0 and world == 1 and args.precision_steps > 0:
        out["precision"] = time_precision(ac, torch, args)
    if rank == 0 and world == 1 and not args.no_batch:
        out["batch"] = time_batch(ac, torch, args)
    if rank == 0 and world == 1 and args.video_steps > 0:
        out["video"] = time_video(ac, torch, args)
    if rank == 0 and world == 1 and args.family_steps > 0:
        out["families"] = time_families(ac, torch, args)
    if rank == 0 and world == 1 and args.cli_steps > 0:
        out["cli_default"] = time_cli_default(ac, torch, args)
    if rank == 0 and world == 1 and args.serve_seconds > 0:
        out["serve"] = time_serve(ac, torch, args)
        out["serve"]["saturation"] = time_serve_saturation(ac, torch, args)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--frames", type=int, default=8)
    ap.add_argument("--forms", default="fp16,fp32,bf16")
    ap.add_argument("--e2e-threads", type=int, default=8)
    ap.add_argument("--per-frame", action="store_true", help="time the tensor-core forms one launch per frame")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-image batching workload")
    ap.add_argument("--no-error-stats", action="store_true", help="skip the FP64-oracle error statistics")
    ap.add_argument("--precision-steps", type=int, default=5, help="frames per form of the precision workload (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=12)
    ap.add_argument("--video-steps", type=int, default=2, help="passes over the 120-frame clip of the video workload (0: skip)")
    ap.add_argument("--family-steps", type=int, default=10, help="frames per family and form in the families workload (0: skip)")
    ap.add_argument("--cli-steps", type=int, default=10, help="steps of the CLI-default-model workload (0: skip)")
    ap.add_argument("--serve-seconds", type=float, default=60.0, help="serving workload length per form (0: skip)")
    ap.add_argument("--serve-workers", type=int, default=8, help="worker streams of the serving loop")
    ap.add_argument("--serve-load-seconds", type=float, default=8.0, help="length of each higher-rate FP16 serving run (0: skip)")
    ap.add_argument("--serve-load-rates", default="400,600,1000", help="offered rates of the higher-rate FP16 serving runs, jobs/s")
    ap.add_argument("--serve-rate", type=float, default=200.0, help="serving workload arrival rate, jobs/s")
    ap.add_argument("--saturation-rate", type=float, default=4000.0, help="offered rate of the saturation run, jobs/s")
    args = ap.parse_args()
    args.forms = [f for f in args.forms.split(",") if f]
    args.serve_load_rates = [float(r) for r in args.serve_load_rates.split(",") if r]
    args.warmup = max(args.warmup, 3)

    rank, world, local_rank = env_int("RANK", 0), env_int("WORLD_SIZE", 1), env_int("LOCAL_RANK", 0)
    if args.impl == "reference":
        res = run_reference(args, rank)
        if res is not None:
            print(json.dumps(res), flush=True)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
        dist.barrier()
    res = run_gb300(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
