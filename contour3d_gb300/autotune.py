"""Autotuner: the batched form's worker count and the kernels' launch shape.

contour3d_gb300_render_batch overlaps frames by running them on several
worker contexts (streams and buffers of their own).  How many pay off depends
on the frames -- small fields leave the GPU idle between one frame's kernels,
large ones fill it alone -- and on the GPU.  tune_workers times a sample of the
caller's own frames at a few worker counts, keeps the fastest, and caches the
choice per (GPU, size class of the frames) in a JSON file, so the measurement
runs once per kind of batch.

tune_launch_shape does the same for the launch shape of the tunable kernels
(contour3d_gb300_set_launch_shape): node slices per classification brick,
and resident blocks per SM of the triangle pass's and the raster passes'
grids.  The shape does not change any result, only the time.

The cache lives at $CONTOUR3D_GB300_TUNE_CACHE, else
$XDG_CACHE_HOME/contour3d_gb300/tune.json (~/.cache when unset).  An unreadable
cache is ignored and rewritten.
"""
import json
import math
import os
import tempfile
import time
from typing import Callable, Dict, Optional, Sequence

CANDIDATES = (2, 4, 6, 8, 12)


def cache_path() -> str:
    env = os.environ.get("CONTOUR3D_GB300_TUNE_CACHE")
    if env:
        return env
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "contour3d_gb300", "tune.json")


def size_class(cells: Sequence[int], pixels: Sequence[int]) -> str:
    """A coarse key for a batch: log2 of the median cells and pixels per frame
    and the batch size rounded down to a power of two."""
    if not cells:
        return "empty"
    med = lambda v: sorted(v)[len(v) // 2]
    c = int(math.log2(max(1, med(cells))))
    p = int(math.log2(max(1, med(pixels))))
    n = 1 << int(math.log2(len(cells)))
    return f"c{c}-p{p}-n{n}"


def _load(path: str) -> Dict:
    try:
        with open(path) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def _store(path: str, data: Dict) -> None:
    d = os.path.dirname(path) or "."
    os.makedirs(d, exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=d, prefix=".tune-", suffix=".json")
    with os.fdopen(fd, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def tune(key: str, run: Callable[[int], float], candidates: Sequence[int] = CANDIDATES,
         path: Optional[str] = None) -> Dict:
    """The cached choice for `key`, or the fastest of `candidates` by run(w)
    (seconds for the sample at w workers), cached.  Returns
    {"workers": w, "seconds": {w: s, ...}, "cached": bool}."""
    path = path or cache_path()
    data = _load(path)
    hit = data.get(key)
    if isinstance(hit, dict) and isinstance(hit.get("workers"), int) and hit["workers"] > 0:
        return {"workers": hit["workers"], "seconds": hit.get("seconds", {}), "cached": True}
    seconds = {}
    for w in candidates:
        seconds[str(w)] = float(run(int(w)))
    best = min(seconds, key=lambda k: seconds[k])
    data[key] = {"workers": int(best), "seconds": seconds}
    try:
        _store(path, data)
    except OSError:
        pass  # a read-only cache only costs the next caller a measurement
    return {"workers": int(best), "seconds": seconds, "cached": False}


def tune_workers(gpu, packs, cells: Sequence[int], pixels: Sequence[int], device_name: str,
                 sample: int = 16, candidates: Sequence[int] = CANDIDATES, path: Optional[str] = None) -> Dict:
    """Worker count for render_batch on frames like `packs` (a warm-up batch,
    then one timed batch of `sample` frames per candidate)."""
    sub = list(packs[:sample])

    def run(w: int) -> float:
        import torch
        gpu.render_batch(sub, w)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        gpu.render_batch(sub, w)
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    key = f"{device_name}|{size_class(cells, pixels)}"
    return tune(key, run, candidates, path)


# (classification brick slices, triangle-pass blocks per SM, raster-pass blocks per SM)
SHAPES = ((32, 8, 8), (16, 8, 8), (64, 8, 8), (32, 6, 8), (32, 8, 6), (32, 4, 4))


def tune_shape(key: str, run: Callable[[tuple], float], candidates: Sequence[tuple] = SHAPES,
               path: Optional[str] = None) -> Dict:
    """The cached launch shape for `key`, or the fastest of `candidates` by
    run(shape) (seconds), cached.  Returns {"shape": [s, e, r], "seconds":
    {"s,e,r": t, ...}, "cached": bool}."""
    path = path or cache_path()
    data = _load(path)
    hit = data.get(key)
    if isinstance(hit, dict) and isinstance(hit.get("shape"), list) and len(hit["shape"]) == 3:
        return {"shape": [int(x) for x in hit["shape"]], "seconds": hit.get("seconds", {}), "cached": True}
    seconds = {}
    for c in candidates:
        seconds[",".join(str(int(x)) for x in c)] = float(run(tuple(int(x) for x in c)))
    best = min(seconds, key=lambda k: seconds[k])
    shape = [int(x) for x in best.split(",")]
    data[key] = {"shape": shape, "seconds": seconds}
    try:
        _store(path, data)
    except OSError:
        pass
    return {"shape": shape, "seconds": seconds, "cached": False}


def tune_launch_shape(gpu, run_sample: Callable[[], None], cells: Sequence[int], pixels: Sequence[int],
                      device_name: str, candidates: Sequence[tuple] = SHAPES, repeats: int = 3,
                      path: Optional[str] = None) -> Dict:
    """Launch shape for work like `run_sample` (renders a sample of the
    caller's frames and returns once they are done): each candidate is set,
    run once to warm up, then timed `repeats` times (best taken).  The chosen
    shape is left set."""

    def run(shape: tuple) -> float:
        gpu.set_launch_shape(*shape)
        run_sample()
        best = float("inf")
        for _ in range(repeats):
            t0 = time.perf_counter()
            run_sample()
            best = min(best, time.perf_counter() - t0)
        return best

    key = f"{device_name}|shape|{size_class(cells, pixels)}"
    r = tune_shape(key, run, candidates, path)
    gpu.set_launch_shape(*r["shape"])
    return r
