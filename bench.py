"""Benchmark of the isosurface-to-image path on GB300.

Workload (default): one 512^3 float64 field, sum of 64 seeded Fourier modes
with |k| in 1..16 and amplitude |k|^(-5/6), cut at +-0.5 std (two contour
objects), rendered at 1920 x 1080.  A step is one frame: classify, scan,
emit, smooth and rasterise both iso-surfaces into one image.

  value  cell-thresholds per second with the field resident in HBM (device
         entry point contour3d_gb300_render_device), CUDA events on the
         launching stream
  e2e    the same metric through the drop-in contour3d_execute with the field
         in host memory: the host->device copy of the field, the device->host
         copy of the image and the ppm write are inside the timed region

  roofline      the dominant stage's algorithmic bytes over its event time,
                against the measured HBM peak, with every stage's time
  cpu_baseline  the oracle on every host core on the whole workload, with
                the CPU model and a one-core point on a z-slab sample
  clocks        nvidia-smi SM clocks and throttle reasons during the timed
                region
  batched, served, large
                the batched form against the plain path on 64 uneven
                fields; the served form on a Poisson request stream; a
                1536^3 float32 field at 3840 x 2160

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

--impl reference times the CPU restatement of the reference (oracle/, run
with one thread per host core as emulated z-split ranks) on the whole
workload every step (about 4 s per step on 16 Grace cores); --cpu-table adds
the other workloads.  Under torchrun, every rank renders its own replica of
the workload (the path shards by z-slabs with one final reduction; each GPU
here renders a whole field).
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SHAPE = (512, 512, 512)
NMODES, KMIN, KMAX, POWER, SEED = 64, 1, 16, 5.0 / 6.0, 1
WIDTH, HEIGHT = 1920, 1080
CAM = (2.5, 2.0, 1.5)
CENTRE = (0.5, 0.5, 0.5)
COLORS = ((0, 255, 255), (255, 255, 0))
CPU_SAMPLE_SLICES_1 = 16  # z-nodes of the 512^2 x 512 field timed on one host core

# DRAM bytes (read + write) per unit processed, from one ncu --set full
# capture of each kernel on the 256^3 case of this workload; the full-size
# launch is scaled by its units
TRAFFIC_PER_UNIT = {
    "classify": (4.63, "cells"),     # k_classify_tma, both levels in one pass: 154.0 MB for 2 x 16.6 M cells
    "scan": (2.55, "cells"),         # k_scan (16-bit vertex offsets): 42.2 MB for 16.6 M cells
    "vertices": (32.5, "vertices"),  # k_vertices: 213.0 MB for 6.55 M vertices
    "emit": (41.5, "triangles"),     # k_emit: 544.3 MB for 13.1 M triangles
}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--shape", type=int, default=512,
                   help="nodes per axis (512 is the benchmark; smaller sizes are for profiler captures)")
    p.add_argument("--no-batched", action="store_true")
    p.add_argument("--no-served", action="store_true")
    p.add_argument("--no-large", action="store_true", help="skip the 1536^3 f32 field")
    p.add_argument("--workers", default="auto",
                   help="worker contexts of the batched and served forms (auto: tuned for the batched frames)")
    p.add_argument("--served-rates", default="50,100,200,400,max",
                   help="comma-separated request rates (req/s); max = submit without waiting")
    p.add_argument("--served-requests", type=int, default=500)
    p.add_argument("--no-tune", action="store_true",
                   help="keep the default launch shape (profiler captures: fewer launches before the timed ones)")
    p.add_argument("--cpu-table", action="store_true",
                   help="with --impl reference: also time the oracle on the other workloads")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        # the timed region starts once the sampler is running (its first line is out)
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 3.0 and os.path.getsize(self.path) == 0:
            time.sleep(0.005)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine type)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def cpu_baseline(field_sample: np.ndarray, std: float, cores: int):
    """The CPU oracle on a z-slab sample of the same field, one thread per core."""
    from contour3d_gb300 import _abi
    from oracle.lib import Oracle
    orc = Oracle()
    nz = field_sample.shape[0]
    g = _abi.unit_grid(SHAPE[2])
    scene = _abi.make_scene(CAM, CENTRE, WIDTH, HEIGHT)
    grids = (_abi.unit_grid(SHAPE[0]), _abi.unit_grid(SHAPE[1]), g[:nz])
    scene.contours = [_abi.Contour(field_sample, -0.5 * std, COLORS[0], grids=grids),
                      _abi.Contour(field_sample, 0.5 * std, COLORS[1], grids=grids)]
    t0 = time.perf_counter()
    orc.render(scene, nranks=cores)
    dt = time.perf_counter() - t0
    cells = 2 * (SHAPE[0] - 1) * (SHAPE[1] - 1) * (nz - 1)
    return cells / dt, dt, cells


def run_large(gpu, n=1536, frames=2):
    """The large single field: n^3 f32 (1536^3 = 14.5 GB), 256 Fourier modes
    |k| 1..48 with amplitude |k|^-11/6, four levels at +-0.5 and +-1 std,
    3840x2160, generated on the device; device-resident rendering.  The FP32
    field is widened exactly when read, so the result is the reference's FP64
    arithmetic on those values; what FP32 storage changes is the input, which
    fp32_input_vs_fp64 measures on a 256^3 crop of this field."""
    import torch
    from contour3d_gb300 import _abi, workloads
    f, std = workloads.modes_device(gpu, (n, n, n), nmodes=256, kmin=1, kmax=48, power=11.0 / 6.0, seed=4,
                                    dtype=torch.float32)
    W, H = 3840, 2160
    scene = _abi.make_scene(CAM, CENTRE, W, H)
    grids = [_abi.unit_grid(n)] * 3
    levels = [-std, -0.5 * std, 0.5 * std, std]
    fl = [(f.data_ptr(), 1, (n, n, n), grids, lv, c) for lv, c in zip(levels, workloads.PALETTE)]
    rgb = torch.empty(W * H * 3, dtype=torch.uint8, device="cuda")
    if gpu.render_device(scene, fl, rgb.data_ptr()) != 0:
        raise RuntimeError("large field: render failed")
    st = gpu.stats()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(frames):
        if gpu.render_device(scene, fl, rgb.data_ptr()) != 0:
            raise RuntimeError("large field: render failed")
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / frames
    cells = len(levels) * (n - 1) ** 3
    out = {"workload": f"{n}^3 f32 Fourier field (256 modes, |k| 1..48, |k|^-11/6), 4 levels (+-0.5, +-1 std), "
                       f"{W}x{H}", "ms_per_frame": ms, "cells_per_s": cells / (ms / 1e3),
           "triangles_per_frame": int(st.triangles), "triangles_per_s": st.triangles / (ms / 1e3),
           "slabs": int(st.slabs), "candidate_overflows": int(st.candidate_overflows),
           "library_device_gb": gpu.lib.contour3d_gb300_device_bytes() / 1e9, "field_gb": f.numel() * 4 / 1e9}
    del f
    torch.cuda.empty_cache()
    # the FP32 input against the FP64 one on a 256^3 crop of this field (its
    # centre, generated in both precisions from the same modes): vertex
    # displacement over every crossed edge, and the image at 3840x2160
    from contour3d_gb300 import fp32_error
    crop, off = 256, (n - 256) // 2
    fd = torch.empty((crop,) * 3, dtype=torch.float64, device="cuda")
    ff = torch.empty((crop,) * 3, dtype=torch.float32, device="cuda")
    for t, dt in ((fd, 0), (ff, 1)):
        gpu.fieldgen_modes_device(t.data_ptr(), dt, (crop,) * 3, 256, 1, 48, 11.0 / 6.0, 4, offset=(off,) * 3,
                                  glshape=(n, n, n))
    g2 = [_abi.unit_grid(n)[off:off + crop]] * 3
    imgs, tris = [], []
    for t, dt in ((fd, 0), (ff, 1)):
        o = torch.empty(W * H * 3, dtype=torch.uint8, device="cuda")
        if gpu.render_device(scene, [(t.data_ptr(), dt, (crop,) * 3, g2, lv, c)
                                     for lv, c in zip(levels, workloads.PALETTE)], o.data_ptr()) != 0:
            raise RuntimeError("fp32 comparison: render failed")
        torch.cuda.synchronize()
        imgs.append(o.cpu().numpy())
        tris.append(int(gpu.stats().triangles))
    out["fp32_input_vs_fp64"] = dict(
        {"field": f"{crop}^3 centre crop (offset {off}) of this field, generated in f64 and in f32",
         "image": f"{W}x{H}, the 4 levels", "triangles_f64": tris[0], "triangles_f32": tris[1],
         "f32_is_f64_rounded": bool(torch.equal(fd.float(), ff)),
         "vertices": fp32_error.vertex_error(fd, ff, levels, g2)},
        **fp32_error.image_difference(imgs[0], imgs[1]))
    del fd, ff
    return out


def run_batched(gpu, workers, nfields=64):
    """64 fields of uneven shape, each with its own levels and camera, 1024^2:
    the plain per-frame entry point one frame at a time, then the batched form
    (worker count from the autotuner unless given)."""
    import torch
    from contour3d_gb300 import _abi, autotune, workloads
    fields, frames, twins = workloads.batch_set(gpu, nfields=nfields, twins=True)
    outs = [torch.empty(f.width * f.height * 3, dtype=torch.uint8, device="cuda") for f in frames]
    packs = [workloads.frame_pack(gpu, fields[f.field], f, o) for f, o in zip(frames, outs)]
    per_frame = [len(f.levels) * (fields[f.field].shape[0] - 1) * (fields[f.field].shape[1] - 1) *
                 (fields[f.field].shape[2] - 1) for f in frames]
    cells = sum(per_frame)
    tuning = None
    if workers == "auto":
        tuning = autotune.tune_workers(gpu, packs, per_frame, [f.width * f.height for f in frames],
                                       torch.cuda.get_device_name())
        workers = tuning["workers"]
    workers = int(workers)
    sub = packs[:16]

    def sample():
        gpu.render_batch(sub, workers)
        torch.cuda.synchronize()

    shape_tuning = autotune.tune_launch_shape(gpu, sample, per_frame[:16], [f.width * f.height for f in frames[:16]],
                                              torch.cuda.get_device_name())
    # every frame once through each form first (worker contexts and the
    # library's own size their buffers from the frames they have seen), then
    # the median of three passes of each
    for p in packs:
        gpu.render_pack(p)
    gpu.render_batch(packs, workers)
    torch.cuda.synchronize()

    def timed(fn, reps=3):
        ts = []
        for _ in range(reps):
            for o in outs:
                o.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return sorted(ts)[reps // 2]

    def plain_pass():
        for p in packs:
            if gpu.render_pack(p) != 0:
                raise RuntimeError("plain frame failed")

    plain_s = timed(plain_pass)
    ref = [o.clone() for o in outs]
    batch_s = timed(lambda: gpu.render_batch(packs, workers))
    same = all(bool(torch.equal(a, b)) for a, b in zip(ref, outs))
    # the same batch with each frame classifying its own fields
    gpu.set_batch_classify(False)
    try:
        gpu.render_batch(packs, workers)
        own_s = timed(lambda: gpu.render_batch(packs, workers))
    finally:
        gpu.set_batch_classify(True)
    same = same and all(bool(torch.equal(a, b)) for a, b in zip(ref, outs))
    # the float32 half against the float64 fields they were rounded from: the
    # vertices of every crossed edge, and the frames rendered from both
    from contour3d_gb300 import fp32_error
    worst, rms2, edges, flips, px, maxd, rounded = 0.0, 0.0, 0, 0, 0, 0, True
    o64 = torch.empty(1024 * 1024 * 3, dtype=torch.uint8, device="cuda")
    for q, spec in enumerate(frames):
        if spec.field not in twins:
            continue
        f32, f64 = fields[spec.field], twins[spec.field]
        rounded = rounded and bool(torch.equal(f64.float(), f32))
        nz, ny, nx = f32.shape
        ve = fp32_error.vertex_error(f64, f32, spec.levels, [_abi.unit_grid(m) for m in (nx, ny, nz)])
        worst = max(worst, ve["max_in_node_spacings"])
        rms2 += ve["rms_in_node_spacings"] ** 2 * ve["edges_compared"]
        edges += ve["edges_compared"]
        flips += ve["edges_crossed_in_one_field_only"]
        if gpu.render_pack(workloads.frame_pack(gpu, f64, spec, o64)) != 0:
            raise RuntimeError("fp64 twin frame failed")
        torch.cuda.synchronize()
        d = fp32_error.image_difference(o64.cpu().numpy(), ref[q].cpu().numpy())
        px += d["pixels_differing"]
        maxd = max(maxd, d["max_channel_diff"])
    fp32 = {"frames": len(twins), "f32_is_f64_rounded": rounded, "edges_compared": edges,
            "edges_crossed_in_one_field_only": flips, "vertex_max_in_node_spacings": worst,
            "vertex_rms_in_node_spacings": (rms2 / edges) ** 0.5 if edges else 0.0,
            "pixels_differing": px, "pixels": len(twins) * 1024 * 1024, "max_channel_diff": maxd}
    return {"workload": f"{nfields} fields, dims 64..384, half f64 / half f32, 1-4 levels, own camera, 1024x1024",
            "frames": nfields, "cell_thresholds": int(cells), "workers": workers, "tuning": tuning,
            "launch_shape": shape_tuning,
            "plain": {"cells_per_s": cells / plain_s, "frames_per_s": nfields / plain_s, "s": plain_s},
            "batched": {"cells_per_s": cells / batch_s, "frames_per_s": nfields / batch_s, "s": batch_s,
                        "classification": "one persistent launch over every frame's (field, brick) items"},
            "batched_per_frame_classify": {"cells_per_s": cells / own_s, "frames_per_s": nfields / own_s,
                                           "s": own_s},
            "speedup": plain_s / batch_s, "images_identical": same, "fp32_input_vs_fp64": fp32}


def run_served(gpu, slots, rates, nreq, budget_gb=120.0, seed=99):
    """Request stream over resident fields (shapes {96^3, 192^3, 256x256x512,
    384^3, 768^3}, f32 and f64), 1-3 levels and a camera per request,
    1280x720; every 10 requests one field advances in place by a phase step
    omega dt (its readers finish first).  The plain path replays the same
    sequence one request at a time; the served path replays it as a Poisson
    stream at each rate ("max" submits without waiting).  Fields restart at
    time 0 before each replay, so every replay does the same work."""
    import torch
    from contour3d_gb300 import workloads
    rng = np.random.default_rng(seed)
    resident = []
    solver = torch.cuda.Stream()
    # the solver stand-in computes its fields in single precision (a double
    # field stores the widened sums): an update of the 768^3 double field
    # then costs milliseconds, not the ~0.2 s of a double-precision
    # evaluation on this GPU's FP64 rate, so the stream measures rendering
    for shp in workloads.SERVED_SHAPES:
        for dt in (torch.float32, torch.float64):
            f = torch.empty(shp, dtype=dt, device="cuda")
            std = gpu.fieldgen_modes_device_async(f.data_ptr(), 1 if dt == torch.float32 else 2, shp, 32, 1, 12,
                                                  5.0 / 6.0, len(resident) + 300, 0.0, solver.cuda_stream)
            resident.append({"t": f, "std": std, "time": 0.0, "seed": len(resident) + 300, "busy": []})
    solver.synchronize()
    resident_bytes = sum(r["t"].numel() * r["t"].element_size() for r in resident)
    out = {"workload": "Poisson stream, resident fields {96^3,192^3,256x256x512,384^3,768^3} x {f32,f64}, "
                       "1-3 levels, 1280x720, phase advance every 10 requests (single-precision solver stand-in)",
           "slots": slots, "budget_gb": budget_gb, "resident_gb": resident_bytes / 1e9, "rates": []}

    def advance(r, time_value):
        t = r["t"]
        r["time"] = time_value
        gpu.fieldgen_modes_device_async(t.data_ptr(), 2 if t.dtype == torch.float64 else 1, tuple(t.shape), 32, 1,
                                        12, 5.0 / 6.0, r["seed"], time_value, solver.cuda_stream)
        solver.synchronize()

    def restart():
        for r in resident:
            if r["time"] != 0.0:
                advance(r, 0.0)
            r["busy"] = []

    reqs = []
    for _ in range(nreq):
        fi = int(rng.integers(0, len(resident)))
        nlev = int(rng.integers(1, 4))
        lv = sorted(float(x) for x in rng.uniform(-0.8, 0.8, size=nlev) * resident[fi]["std"])
        reqs.append((fi, workloads.FrameSpec(0, lv, workloads.PALETTE[:nlev], workloads.random_camera(rng),
                                             1280, 720)))
    cells = 0
    for fi, spec in reqs:
        sh = resident[fi]["t"].shape
        cells += len(spec.levels) * (sh[0] - 1) * (sh[1] - 1) * (sh[2] - 1)
    out["cell_thresholds"] = cells
    outs = [torch.empty(1280 * 720 * 3, dtype=torch.uint8, device="cuda") for _ in range(nreq)]
    packs = [workloads.frame_pack(gpu, resident[fi]["t"], spec, outs[q]) for q, (fi, spec) in enumerate(reqs)]

    def updated(q):
        return resident[(q // 10) % len(resident)] if q and q % 10 == 0 else None

    # plain: the same sequence, one request at a time
    for p in packs[:3]:
        gpu.render_pack(p)
    restart()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for q, p in enumerate(packs):
        r = updated(q)
        if r is not None:
            advance(r, r["time"] + 0.01)
        gpu.render_pack(p)
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    out["plain"] = {"frames_per_s": nreq / plain_s, "cells_per_s": cells / plain_s}
    plain_img = [o.clone() for o in outs]
    for rate in rates:
        restart()
        for o in outs:
            o.zero_()
        torch.cuda.synchronize()
        gaps = rng.exponential(1.0 / rate, size=nreq) if rate else np.zeros(nreq)
        with gpu.server(slots, int(budget_gb * 1e9), resident_bytes) as sv:
            tickets, lat = [], []
            t_start = time.perf_counter()
            t_next = t_start
            for q, (fi, spec) in enumerate(reqs):
                t_next += gaps[q]
                while True:
                    d = t_next - time.perf_counter()
                    if d <= 0:
                        break
                    time.sleep(min(d, 0.002))
                r = updated(q)
                if r is not None:
                    for tk in r["busy"]:
                        lat.append(sv.wait(tk))
                        tickets.remove(tk)
                    r["busy"] = []
                    advance(r, r["time"] + 0.01)
                tk = sv.submit(packs[q])
                tickets.append(tk)
                resident[fi]["busy"].append(tk)
            for tk in tickets:
                lat.append(sv.wait(tk))
            wall = time.perf_counter() - t_start
            mem = sv.memory()
        torch.cuda.synchronize()
        same = all(torch.equal(a, b) for a, b in zip(outs, plain_img))
        ms = np.array([x.latency_ms for x in lat])
        out["rates"].append({"rate_req_s": rate if rate else "max", "requests": nreq,
                             "p50_ms": float(np.percentile(ms, 50)), "p99_ms": float(np.percentile(ms, 99)),
                             "frames_per_s": nreq / wall, "cells_per_s": cells / wall,
                             "p90_ms": float(np.percentile(ms, 90)),
                             "queue_p50_ms": float(np.percentile([x.queue_ms for x in lat], 50)),
                             "queue_p99_ms": float(np.percentile([x.queue_ms for x in lat], 99)),
                             "device_p50_ms": float(np.percentile([x.device_ms for x in lat], 50)),
                             "context_peak_gb": mem.peak_bytes / 1e9, "overcommits": int(mem.overcommits),
                             "idle_trims": int(mem.trims),
                             "images_identical_to_plain": bool(same)})
    return out


def cpu_scene_time(scene, cores, repeats=1):
    """Median seconds of the oracle rendering `scene` with `cores` threads."""
    from oracle.lib import Oracle
    orc = Oracle()
    ts = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        orc.render(scene, nranks=cores)
        ts.append(time.perf_counter() - t0)
    return float(np.median(ts))


def cpu_table(cores):
    """The oracle on the host cores for the other workloads: the 128^3 blob
    field (1 level, 1024^2), eight frames of the batched workload (float32
    fields widened, as the reference is double-only), and a 256^3 crop of
    the 1536^3 float32 field (4 levels, 3840x2160), each at every core and,
    for the small ones, at one core."""
    from contour3d_gb300 import _abi, fields, workloads
    from tests import cases
    rows = []
    s0 = cases.config0()
    c0 = 127 ** 3
    t_all, t_one = cpu_scene_time(s0, cores, 3), cpu_scene_time(s0, 1, 1)
    rows.append({"config": "128^3 f64 blobs, 1 level, 1024x1024", "cells": c0,
                 "cores": cores, "cells_per_s": c0 / t_all, "frames_per_s": 1.0 / t_all,
                 "one_core": {"cells_per_s": c0 / t_one, "frames_per_s": 1.0 / t_one}})
    flds, frames = workloads.batch_set(None, nfields=8, host=True)
    cells = t = 0.0
    for spec in frames:
        f = flds[spec.field].astype(np.float64)
        nz, ny, nx = f.shape
        grids = tuple(_abi.unit_grid(n) for n in (nx, ny, nz))
        sc = _abi.make_scene(spec.camera, CENTRE, spec.width, spec.height)
        sc.contours = [_abi.Contour(f, lv, c, grids=grids) for lv, c in zip(spec.levels, spec.colors)]
        t += cpu_scene_time(sc, cores)
        cells += len(spec.levels) * (nx - 1) * (ny - 1) * (nz - 1)
    rows.append({"config": "batched workload, first 8 of 64 frames (dims 64..384, 1-4 levels, 1024x1024)",
                 "cells": int(cells), "cores": cores, "cells_per_s": cells / t, "frames_per_s": 8 / t})
    n = 1536
    crop = 256
    off = (n - crop) // 2
    f32, std = fields.modes_threaded((crop, crop, crop), nmodes=256, kmin=1, kmax=48, power=11.0 / 6.0, seed=4,
                                     dtype=np.float32, offset=(off, off, off), glshape=(n, n, n))
    f = f32.astype(np.float64)
    g = tuple(_abi.unit_grid(n)[off:off + crop] for _ in range(3))
    sc = _abi.make_scene(CAM, CENTRE, 3840, 2160)
    sc.contours = [_abi.Contour(f, lv * std, c, grids=g) for lv, c in zip((-1.0, -0.5, 0.5, 1.0), workloads.PALETTE)]
    t4 = cpu_scene_time(sc, cores)
    c4 = 4 * (crop - 1) ** 3
    rows.append({"config": "256^3 centre crop of the 1536^3 f32 field (widened), 4 levels, 3840x2160",
                 "cells": c4, "cores": cores, "cells_per_s": c4 / t4, "frames_per_s": 1.0 / t4})
    return rows


def run_reference(args, rank, world):
    """CPU arm: the reference's algorithm restated in C (oracle/), every host
    core as an emulated z-split rank, on the full bench workload."""
    if rank != 0:
        return
    from contour3d_gb300 import fields
    cores = os.cpu_count() or 1
    field, std = fields.modes_threaded(SHAPE, NMODES, KMIN, KMAX, POWER, SEED)
    for _ in range(args.warmup):
        cpu_baseline(field, std, cores)
    times = []
    cells = 0
    for _ in range(args.steps):
        v, dt, cells = cpu_baseline(field, std, cores)
        times.append(dt)
    ms = 1000.0 * float(np.mean(times))
    value = cells / (ms / 1000.0)
    sample_desc = (f"the whole workload every step ({SHAPE[0]}^3 f64, two thresholds, 1920x1080), "
                   f"oracle/c3d_oracle.c with {cores} threads as emulated z-split ranks")
    out = {
        "metric": "cells_per_s", "value": value, "unit": "cell-thresholds/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Fourier field)",
        "impl": "reference",
        "config": {"workload": workload_name(), "sample": sample_desc},
        "cpu_baseline": {"value": value, "unit": "cell-thresholds/s", "cores": cores, "cpu_model": cpu_model(),
                         "kind": "port", "sample": sample_desc,
                         "mpi": "no MPI launcher on the GPU host: ranks are threads of one process"
                         if not shutil.which("mpirun") else "mpirun present; ranks are still threads"},
        "e2e": {"value": value, "unit": "cell-thresholds/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if args.cpu_table:
        out["cpu_table"] = cpu_table(cores)
    print(json.dumps(out))


def workload_name() -> str:
    return f"fourier-{SHAPE[0]}^3-f64-2thr-{WIDTH}x{HEIGHT}"


def main():
    global SHAPE
    args = parse()
    SHAPE = (args.shape,) * 3
    rank, world, local = dist_env()
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "gpu" else "gloo")
    if args.impl == "reference":
        run_reference(args, rank, world)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    torch.cuda.set_device(local)
    from contour3d_gb300 import _abi, lib
    gpu = lib.load()
    nz, ny, nx = SHAPE
    field = torch.empty(SHAPE, dtype=torch.float64, device="cuda")
    std = gpu.fieldgen_modes_device(field.data_ptr(), 0, SHAPE, NMODES, KMIN, KMAX, POWER, SEED)
    grids = [_abi.unit_grid(n) for n in (nx, ny, nz)]
    thresholds = (-0.5 * std, 0.5 * std)
    fdesc = [(field.data_ptr(), 0, (nx, ny, nz), grids, thr, col) for thr, col in zip(thresholds, COLORS)]
    scene = _abi.make_scene(CAM, CENTRE, WIDTH, HEIGHT)
    rgb = torch.empty(WIDTH * HEIGHT * 3, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    def step():
        rc = gpu.render_device(scene, fdesc, rgb.data_ptr(), stream.cuda_stream)
        if rc != 0:
            raise RuntimeError("render_device failed")

    for _ in range(max(3, args.warmup)):
        step()
    # the launch shape for this workload (cached per GPU and size class)
    from contour3d_gb300 import autotune

    def sample():
        step()
        step()
        torch.cuda.synchronize()

    shape_tuning = None
    if not args.no_tune:
        shape_tuning = autotune.tune_launch_shape(gpu, sample, [(nx - 1) * (ny - 1) * (nz - 1)], [WIDTH * HEIGHT],
                                                  torch.cuda.get_device_name())
        step()
    # untimed per-stage profile of one frame
    gpu.set_stage_timing(True)
    step()
    prof = gpu.stats()
    gpu.set_stage_timing(False)
    step()
    st = gpu.stats()
    launches_per_step = int(st.kernel_launches)

    sampler = ClockSampler(local)
    sampler.start()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / args.steps
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    cells_per_step = 2 * (nx - 1) * (ny - 1) * (nz - 1)
    value = world * cells_per_step / (ms / 1000.0)
    timed_graph = int(gpu.stats().graph)  # 2: the timed frames ran as the recorded CUDA graph

    # the same frame without the graph, and synchronised after every slab
    # pass (outside the timed region; CUDA events over 5 frames each)
    def frames_ms(n=5):
        step()
        step()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(n):
            step()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / n

    gpu.set_graphs(False)
    modes = {"graph_ms": ms, "timed_frames_graph": timed_graph, "unsynchronised_ms": frames_ms(),
             "launch_shape": shape_tuning}
    gpu.set_async(False)
    modes["synchronised_ms"] = frames_ms()
    gpu.set_async(True)
    gpu.set_graphs(True)

    # ---- roofline of the dominant stage (per-stage event times of one frame) ----
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    T = float(prof.triangles)
    V = float(prof.vertices)
    nodes = float(nx * ny * nz)
    cells = float((nx - 1) * (ny - 1) * (nz - 1))
    listed = float(prof.cover_triangles + prof.slivers)
    stage_ms = {"classify": prof.ms_classify, "scan": prof.ms_scan, "vertices": prof.ms_vertices,
                "emit": prof.ms_emit, "cover": prof.ms_cover, "exact": prof.ms_exact, "normals": prof.ms_normals,
                "shade": prof.ms_shade}
    # algorithmic bytes per frame (both objects): the bytes each stage must move
    # once -- inputs read once, outputs written once, cached re-reads not counted
    stage_bytes = {
        "classify": nodes * 8 + 2 * cells * 1,  # one pass over the field for both levels
        # cell codes 1 B; vertex offsets 2 B per cell (16-bit, relative to
        # the scan's 8192-cell segments), read by k_vertices once per 8 cells
        "scan": 2 * cells * (1 + 2) + T * 4,
        "vertices": 2 * cells * (1 + 2 / 8) + V * (2 * 8 + 16),
        "emit": T * 4 + 2 * cells * (1 + 2) + V * 16 + listed * 48 + float(prof.tiny) * 4,
        "cover": listed * 48 + float(prof.candidates) * 16,
        "exact": float(prof.candidates) * (16 + 4),  # each candidate and its pixel's depth floor read once
        "normals": WIDTH * HEIGHT * 16 * 2 + float(prof.winners) * (4 + 48 + 8),
        "shade": float(prof.shade_exact) * (4 + 48 + 8) + float(prof.normals) * (8 + 24),
    }
    dom = max(stage_ms, key=lambda k: stage_ms[k])
    achieved = stage_bytes[dom] / (stage_ms[dom] / 1000.0) / 1e9 if stage_ms[dom] > 0 else 0.0
    # DRAM bytes per unit of the dominant kernels, from the ncu captures in
    # profiles/ (256^3 case, scaled by the units processed)
    traffic = None
    if dom in TRAFFIC_PER_UNIT:
        per_unit, unit_name = TRAFFIC_PER_UNIT[dom]
        units = {"triangles": T, "cells": 2 * cells, "vertices": V}[unit_name]
        traffic = per_unit * units
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": traffic, "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"
                if "hbm_gbs" in peaks else "fallback 6800 GB/s (of fallback)",
                "stage_ms": stage_ms, "stage_gbs": {k: (stage_bytes[k] / (stage_ms[k] / 1000.0) / 1e9
                                                        if stage_ms[k] > 0 else None) for k in stage_ms},
                "triangles_per_frame": int(prof.triangles),
                "vertices_per_frame": int(prof.vertices),
                "candidates_per_frame": int(prof.candidates),
                "cover_triangles_per_frame": int(prof.cover_triangles),
                "tiny_per_frame": int(prof.tiny),
                "slivers_per_frame": int(prof.slivers),
                "exact_fragments_per_frame": int(prof.exact_fragments),
                "normals_per_frame": int(prof.normals)}

    # ---- end to end through the drop-in C entry point ----
    e2e = None
    if not args.no_e2e:
        host_t = field.cpu().pin_memory()  # the step's input in pinned host memory
        host_field = host_t.numpy()
        sc = _abi.make_scene(CAM, CENTRE, WIDTH, HEIGHT)
        sc.contours = [_abi.Contour(host_field, thr, col, grids=tuple(grids)) for thr, col in zip(thresholds, COLORS)]
        tmp = tempfile.mkdtemp()
        path = os.path.join(tmp, "frame.ppm")
        for _ in range(max(3, args.warmup)):  # the first calls allocate and page in
            if gpu.execute(sc, path) != 0:
                raise RuntimeError("contour3d_execute failed")
        steps2 = args.steps  # the same step count as the device-timed value
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps2):
            gpu.execute(sc, path)
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / steps2
        e2e = {"value": world * cells_per_step / dt, "unit": "cell-thresholds/s",
               "h2d_bytes_per_step": int(nodes * 8), "d2h_bytes_per_step": int(WIDTH * HEIGHT * 3),
               "ms_per_step": dt * 1000.0,
               "path": "contour3d_execute (field in pinned host memory, copied in every call; ppm written)"}
        os.unlink(path)
        os.rmdir(tmp)

    batched = served = large = None
    if rank == 0 and not args.no_large:
        large = run_large(gpu)
    if rank == 0 and not args.no_batched:
        batched = run_batched(gpu, args.workers)
    slots = batched["workers"] if batched else (6 if args.workers == "auto" else int(args.workers))
    if rank == 0 and not args.no_served:
        served = run_served(gpu, slots, [0.0 if x == "max" else float(x) for x in args.served_rates.split(",")],
                            args.served_requests)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        whole = field.cpu().numpy()
        cores = os.cpu_count() or 1
        v, dt, c = cpu_baseline(whole, std, cores)
        cpu = {"value": v, "unit": "cell-thresholds/s", "cores": cores, "cpu_model": cpu_model(), "kind": "port",
               "sample": f"the whole workload (512^3 f64, two thresholds, 1920x1080), "
                         f"oracle/c3d_oracle.c with {cores} threads ({dt:.2f} s)"}
        del whole
        # one core, on a thinner slab of the same field
        v1, dt1, _ = cpu_baseline(field[:CPU_SAMPLE_SLICES_1].cpu().numpy(), std, 1)
        cpu["sweep"] = [{"cores": 1, "value": v1, "sample": f"512x512x{CPU_SAMPLE_SLICES_1} z-slab ({dt1:.2f} s)"},
                        {"cores": cores, "value": v, "sample": f"whole 512^3 field ({dt:.2f} s)"}]

    if rank == 0:
        out = {
            "metric": "cells_per_s", "value": value, "unit": "cell-thresholds/s", "n_gpus": world,
            "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Fourier field)",
            "config": {"workload": workload_name(), "field": f"{nx}^3 f64, 64 modes |k| 1..16",
                       "thresholds": "+-0.5 std", "image": "1920x1080",
                       "l2": "inputs larger than L2 (1.07 GB field)", "parallelism": f"replicas x{world}"},
            "frames_per_s": 1000.0 / ms, "triangles_per_frame": int(st.triangles),
            "triangles_per_s": world * st.triangles / (ms / 1000.0),
            "gpu_launches": launches_per_step * args.steps,
            "roofline": roofline, "e2e": e2e, "cpu_baseline": cpu, "clocks": clocks, "frame_modes": modes,
            "batched": batched, "served": served, "large": large,
        }
        print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
