"""Autotuner for the batched launch: picks the screen-tile shape (width x
height), the threads per tile block and the number of records staged per
shared-memory pass of the persistent fused kernel by timing every candidate
on the caller's own batch (device time of the vertex, setup and fused
stages, CUDA-graph replay), then, for the best of those, the bounding-box
size up to which triangles are rasterised by the setup kernel instead of
being binned; and caches the winner in a JSON file keyed by GPU name and a
coarse class of the batch (scene count, triangle count and pixel count, each
bucketed by powers of two).

Every candidate produces the same pixels; only the work split changes."""
from __future__ import annotations

import json
import math
import os
from typing import Dict, List, Optional, Sequence, Tuple

from . import capi

# (tile width, tile height): square tiles plus wide ones, which shorten the
# per-row edge replay of triangles crossing several tiles.
SHAPES: List[Tuple[int, int]] = [(8, 8), (16, 16), (32, 16), (32, 32), (64, 16), (128, 8), (64, 32), (64, 64)]
CANDIDATES: List[Tuple[int, int, int, int]] = [(tw, th, t, ch) for tw, th in SHAPES for t in (64, 128, 256)
                                               for ch in (32, 64, 128)]


# bounding-box pixels up to which the setup kernel rasterises (0: bin all)
SMALL_MAX: List[int] = [0, 16, 64, 256]
DEFAULT_SMALL_MAX = 64


def apply(ctx: capi.Context, best: Dict) -> None:
    """Sets a tuning returned by tune() (or read from its cache)."""
    ctx.set_batch_tiling(best["tile_w"], best["tile_h"], best["threads"], best["chunk"])
    ctx.set_batch_small_max(best.get("small_max", DEFAULT_SMALL_MAX))


def cache_path() -> str:
    return os.environ.get("MR_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "minirender_gb300", "autotune.json"))


def gpu_name() -> str:
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:
        return "unknown-gpu"


def batch_class(n_scenes: int, n_tris: int, n_pixels: int) -> str:
    b = lambda x: int(math.log2(max(1, x)))  # noqa: E731
    return f"{gpu_name()}|scenes2^{b(n_scenes)}|tris2^{b(n_tris)}|px2^{b(n_pixels)}"


def _load(path: str) -> Dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _time_candidate(ctx: capi.Context, prepared, cand, repeats: int, small_max: int) -> float:
    scenes, ns, rs, nr = prepared
    ctx.set_batch_tiling(*cand)
    ctx.set_batch_small_max(small_max)
    ctx.render_batch(scenes, ns, rs, nr)   # captures this shape's graph
    ctx.batch_stats()
    best = float("inf")
    for _ in range(repeats):
        ctx.render_batch(scenes, ns, rs, nr)
        s = ctx.batch_stats()
        best = min(best, float(s.stage_ms[3]))  # whole batch, device time
    return best


def tune(ctx: capi.Context, prepared, key: str, candidates: Sequence[Tuple[int, int, int, int]] = CANDIDATES,
         repeats: int = 3, path: Optional[str] = None, force: bool = False) -> Dict:
    """Times `candidates` (tile_w, tile_h, threads, chunk) on the prepared
    batch, applies and caches the best.
    Returns {"tile_w", "tile_h", "threads", "chunk", "ms", "table"}."""
    path = path or cache_path()
    cache = _load(path)
    if not force and key in cache and "small_max" in cache[key]:
        best = cache[key]
        apply(ctx, best)
        return best
    ctx.set_batch_graphs(True)
    ctx.set_profiling(True)
    table = []
    try:
        for cand in candidates:
            try:
                ms = _time_candidate(ctx, prepared, cand, repeats, DEFAULT_SMALL_MAX)
            except capi.MRError:
                continue  # shape does not fit (shared memory / registers)
            table.append({"tile_w": cand[0], "tile_h": cand[1], "threads": cand[2], "chunk": cand[3],
                          "small_max": DEFAULT_SMALL_MAX, "ms": round(ms, 4)})
        if not table:
            raise RuntimeError("no batch tuning candidate could run")
        top = min(table, key=lambda r: r["ms"])
        cand = (top["tile_w"], top["tile_h"], top["threads"], top["chunk"])
        for sm in SMALL_MAX:
            if sm == DEFAULT_SMALL_MAX:
                continue
            ms = _time_candidate(ctx, prepared, cand, repeats, sm)
            table.append({"tile_w": cand[0], "tile_h": cand[1], "threads": cand[2], "chunk": cand[3],
                          "small_max": sm, "ms": round(ms, 4)})
    finally:
        ctx.set_profiling(False)
    best = dict(min(table, key=lambda r: r["ms"]))
    best["table"] = table
    apply(ctx, best)
    cache[key] = best
    try:  # written whole, then renamed: a concurrent reader never sees half a file
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = f"{path}.{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1)
        os.replace(tmp, path)
    except OSError:
        pass
    return best
