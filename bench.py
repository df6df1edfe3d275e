#!/usr/bin/env python3
"""Throughput of the GB300 rasterisation path.

Default workload: the single-large-mesh frame -- a displaced, textured
icosphere of 1,310,720 triangles at 1920x1080 with near-plane clipping
(minirender_gb300.workloads.config2).  One step = one complete frame through
mr_render (clear, setup/clip/small-triangle raster, binning, tile raster,
deferred resolve+shade to RGB8 and depth).

  value   frames/s with the mesh and texture resident in HBM, device time of
          K frames (CUDA events on the launching stream), L2 flushed between
          frames by writing a 256 MiB buffer.
  e2e     frames/s through the C ABI with host buffers: every step copies the
          mesh and texture from pinned host memory (mr_mesh_update,
          mr_texture_update), renders, and reads RGB8 + depth back.
  --impl reference
          the reference CPU algorithm (the oracle's C restatement; the
          reference's own build needs ASL, which is unavailable) on all host
          cores, one frame per thread per step.

Multi-GPU (torchrun): independent replicas, one per rank, no collective on
the data path; value = frames of all ranks / max over ranks of the time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "frames/s"
UNIT = "frames/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=None,
                   help="timed steps (default: enough for several clock samples under load -- "
                        "2000 frames for config1/config2, 200 for config3, 20 batches for config4; "
                        "10 for --impl reference, whose steps are CPU frames on every host thread)")
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="config2", choices=["config1", "config2", "config3", "config4", "config5"])
    p.add_argument("--rates", default="100,500,1000,2000,5000", help="request rates swept (config5)")
    p.add_argument("--requests", type=int, default=1500, help="requests per rate (config5)")
    p.add_argument("--serve-tuning", default="16,16,64,64,64",
                   help="tile_w,tile_h,threads,chunk,small_max of the render server's batches (config5)")
    p.add_argument("--serve-slots", type=int, default=3, help="render server batch slots (config5)")
    p.add_argument("--serve-max-batch", type=int, default=16, help="render server requests per batch (config5)")
    p.add_argument("--scenes", type=int, default=256, help="scenes per batch (config4)")
    p.add_argument("--tuning", default="",
                   help="tile,threads,chunk or tile_w,tile_h,threads,chunk[,small_max] for batches "
                        "(skips the autotuner)")
    p.add_argument("--views", type=int, default=8, help="camera views per batched launch (config1-3)")
    p.add_argument("--triangles", type=int, default=None,
                   help="config3 only: soup size (default 10,000,000; smaller soups for profiler captures)")
    p.add_argument("--size", default=None, help="config3 only: WxH frame (default 3840x2160)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true", help="skip the end-to-end legs (profiling runs)")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the batched (256-scene) and served (request stream) samples of the default line")
    p.add_argument("--e2e-contexts", type=int, default=3,
                   help="contexts taking alternate end-to-end steps (frames in flight)")
    return p.parse_args()


def make_workload(name, args=None):
    from minirender_gb300 import workloads as W
    if name == "config1":
        st, sc = W.config1()
        desc = "uv-sphere 64x32 (3,968 tris), 640x480, point light, RGB8+depth"
    elif name == "config3":
        n = getattr(args, "triangles", None) or 10_000_000
        w, h = (int(x) for x in (getattr(args, "size", None) or "3840x2160").split("x"))
        st, sc = W.config3(n_tris=n, width=w, height=h)
        desc = f"{n:,}-triangle soup (1-4 px^2, 5% exact duplicates), {w}x{h}, palette texture"
    else:
        st, sc = W.config2()
        desc = ("icosphere level 8 (1,310,720 tris) displaced by value noise, 1024^2 RGB8 "
                "texture, near-plane clipping, 1920x1080, RGB8+depth")
    return st, sc, desc


class Clocks:
    """nvidia-smi sampling thread for the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:  # no nvidia-smi on this machine
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return ws, rank, local


def max_over_ranks(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_counts(workload: str):
    """Per-kernel figures of one ncu capture of this workload (profiles/):
    {kernel: {"dram_bytes": read + write bytes per launch, "warp_inst":
    warp instructions per launch}}."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(p):
        return {}
    with open(p) as f:
        d = json.load(f).get(workload, {})
    return {k: v for k, v in d.items() if isinstance(v, dict)}


# Sample workloads of the default line's batched and served objects, and the
# fixed tunings they use (the autotuner's choice for the 256-scene batch on
# GB300; the render server's default for the request stream).
BATCH_SAMPLE_TUNING = {"tile_w": 64, "tile_h": 32, "threads": 256, "chunk": 64, "small_max": 64}
SERVE_SAMPLE = {"rate": 5000.0, "requests": 300, "slots": 3, "max_batch": 16, "tuning": (16, 16, 64, 64, 64),
                "repeats": 3}


def extras(local, stream):
    """The batched and served forms on short samples of their workloads, each
    next to the plain one-frame-per-call path on the same frames."""
    from minirender_gb300 import workloads as W
    out = {}
    items = W.config4(256)
    m = batch_measure(local, stream, items, steps=3, warmup=3, tuning=BATCH_SAMPLE_TUNING, profile=False)
    out["batched_config4"] = {
        "value": round(m["value"], 2), "unit": UNIT, "scenes": len(items), "batches_timed": 3,
        "ms_per_batch": round(m["total_s"] * 1e3 / 3, 4), "triangles_per_batch": m["T"],
        "pixels_per_batch": m["P"], "tuning": BATCH_SAMPLE_TUNING,
        "workload": "256 seeded scenes x 64 primitives, resolutions from {256^2, 512^2, 640x480, 1280x720}; "
                    "one mr_render_batch per step (CUDA graph replay), 3 steps back to back",
        "plain_one_frame_per_call": round(m["plain"], 2),
        "speedup_vs_plain": round(m["value"] / m["plain"], 3)}
    S = SERVE_SAMPLE
    rows, plain = serve_measure(local, [S["rate"]], S["requests"], S["slots"], S["max_batch"], S["tuning"],
                                repeats=S["repeats"])
    out["served_config5"] = {
        "unit": UNIT, "requests_per_stream": S["requests"], "streams_per_row": S["repeats"],
        "workload": "Poisson request stream of triangle soups (log-uniform 1k-2M triangles, 128x128.."
                    "3840x2160, 30 % re-renders of a resident mesh), 40 GB budget, RGB8 read back",
        "server": {"slots": S["slots"], "max_batch": S["max_batch"], "tuning": list(S["tuning"])},
        "at_rate": rows[0], "capacity": rows[1], "plain_at_rate": plain[0], "plain_capacity": plain[1],
        "served_vs_plain_at_rate": round(rows[0]["frames_per_s"] / plain[0]["frames_per_s"], 3),
        "served_vs_plain_capacity": round(rows[1]["frames_per_s"] / plain[1]["frames_per_s"], 3)}
    return out


_MESH_ARRAYS = ("vertices", "normals", "indices", "normalsI", "texcoords", "texcoordsI")


def _mesh_upload_bytes(m) -> int:
    """Bytes a mesh upload copies: index arrays given as the indices array
    itself are shared on the device, not copied again."""
    seen = {}
    for name in _MESH_ARRAYS:
        a = getattr(m, name)
        if a.size and name in ("texcoordsI",) and not m.texcoords.size:
            continue
        seen.setdefault((a.ctypes.data, a.nbytes), a.nbytes)
    return sum(seen.values())


def _pinned_copy(m):
    """The TriMesh's arrays copied into page-locked host memory, arrays that
    share memory (normalsI / texcoordsI given as the indices) still shared.
    Returns (mesh with the pinned arrays as attributes, tensors to keep)."""
    import copy
    import torch
    out = copy.copy(m)
    pinned, keep = {}, []
    for name in _MESH_ARRAYS:
        a = getattr(m, name)
        k = (a.ctypes.data, a.nbytes, a.dtype.str, a.shape)
        if k not in pinned:
            t = torch.empty(max(1, a.nbytes), dtype=torch.uint8).pin_memory()
            b = t[:a.nbytes].numpy().view(a.dtype).reshape(a.shape)
            b[...] = a
            keep.append(t)
            pinned[k] = b
        setattr(out, name, pinned[k])
    return out, keep


def scene_sizes(sc):
    from minirender_gb300 import scene as S
    flat = S.flatten(sc)
    V = sum(m.vertices.shape[0] for m in flat.meshes)
    T = sum(m.n_triangles for m in flat.meshes)
    mesh_bytes = sum(_mesh_upload_bytes(m) for m in flat.meshes)
    tex_bytes = sum(t.nbytes for t in flat.textures)
    return V, T, mesh_bytes, tex_bytes


def cpu_frames_per_s(st, sc, n_threads: int, frames: int):
    from oracle import oracle as O
    O.build(with_ref=False)
    secs = O.time_frames(st, sc, frames, n_threads)
    return frames / secs, secs


STAGES = ["clear+vertex", "setup", "large_raster", "-", "resolve"]
TUNING_KEYS = ("tile_w", "tile_h", "threads", "chunk", "small_max")
# kernels between the stage events of one plain frame ("-" is an empty
# interval kept so the stage list keeps its five slots)
KERNELS = {"clear+vertex": "k_clear+k_vertex", "setup": "k_setup", "large_raster": "k_raster_large",
           "-": "k_raster_large", "resolve": "k_resolve"}


def e2e_legs(args, ws, r, sc, st, flat, frame, rs, n, mesh_bytes, tex_bytes):
    """End-to-end frames/s through the C ABI with pinned host buffers: every
    step copies the mesh and texture up, renders, and reads RGB8 + depth back
    (mr_read_async).  `--e2e-contexts` contexts (default 3), each on its own
    stream, take turns and share one upload stream (mr_set_upload_stream), so
    one step's upload overlaps another's render and read-back; a context's
    next render first completes its previous frame's read.  The
    second figure keeps the mesh resident and only reads back."""
    from minirender_gb300.renderer import Renderer
    mesh = flat.meshes[0]
    pin = lambda a: torch_pin(np.ascontiguousarray(a))  # noqa: E731
    pm, _keep = _pinned_copy(mesh)
    ptex = [pin(t) for t in flat.textures]
    extra = []
    for _ in range(max(1, args.e2e_contexts) - 1):
        r2 = Renderer(0)
        r2.outputs = r.outputs
        r2.state = st
        r2.setScene(sc)
        extra.append((r2,) + tuple(r2.prepare()))
    lanes = []
    for rr, fr, rsx, nx in [(r, frame, rs, n)] + extra:
        lanes.append({"ctx": rr.ctx, "frame": fr, "rs": rsx, "n": nx, "mesh": rr._mesh_handle(mesh),
                      "tex": [rr._texture_handle(t) for t in flat.textures],
                      "rgb8": pin(np.empty((st.height, st.width, 3), np.uint8)),
                      "depth": pin(np.empty((st.height, st.width), np.float32))})
    h2d = mesh_bytes + tex_bytes
    d2h = lanes[0]["rgb8"].nbytes + lanes[0]["depth"].nbytes
    # one upload stream for all contexts: their updates cross the host link
    # one at a time, at its full rate, while the others render
    import torch
    up = torch.cuda.Stream()
    for L in lanes:
        L["ctx"].set_upload_stream(up.cuda_stream)

    def run(steps, upload):
        for k in range(steps):
            L = lanes[k % len(lanes)]
            c = L["ctx"]
            if upload:
                c.update_mesh(L["mesh"], pm.desc())
                for h, t in zip(L["tex"], ptex):
                    c.update_texture(h, t)
            c.render(L["frame"], L["rs"], L["n"], r.outputs)
            c.read_async(L["rgb8"], L["depth"])
        for L in lanes:
            L["ctx"].wait()

    try:
        run(4, True)
        barrier(ws)
        t0 = time.perf_counter()
        run(args.steps, True)
        e2e_s = max_over_ranks(time.perf_counter() - t0, ws)
        # resident variant: only the camera changes per frame
        run(4, False)
        t0 = time.perf_counter()
        run(args.steps, False)
        res_s = max_over_ranks(time.perf_counter() - t0, ws)
    finally:
        for L in lanes:
            L["ctx"].set_upload_stream(None)
        for x in extra:
            x[0].close()
    return args.steps * ws / e2e_s, args.steps * ws / res_s, h2d, d2h


def torch_pin(a: np.ndarray) -> np.ndarray:
    """A pinned host copy of `a` (page-locked through torch's host allocator)."""
    import torch
    return torch.from_numpy(a).pin_memory().numpy()


def scene_tris(sc) -> int:
    """Triangles submitted by one render() of the scene (every mesh node)."""
    from minirender_gb300 import scene as S
    flat = S.flatten(sc)
    return sum(flat.meshes[nd.mesh].n_triangles for nd in flat.nodes if nd.mesh >= 0)


def device_time_ms(stream, fn, flush=None):
    """Device time of fn() on `stream` between two CUDA events (L2 flushed first)."""
    import torch
    if flush is not None:
        flush.zero_()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1)


def batched_views(args, stream, flush, st, sc, views: int):
    """The same scene from `views` cameras in one batched launch (CUDA graph),
    tuned by the autotuner: frames/s and the tuning chosen."""
    from minirender_gb300 import autotune
    from minirender_gb300 import projection as pj
    from minirender_gb300.batch import BatchRenderer
    from minirender_gb300.frame import FrameState
    import copy
    items = []
    for k in range(views):
        s2 = copy.copy(st)
        s2.view = pj.mat_mul(st.view, pj.rotate_z(0.05 * k))
        items.append((s2, sc))
    br = BatchRenderer()
    br.ctx.set_stream(stream.cuda_stream)
    br.outputs = 3  # RGB8 | depth
    prep = br.prepare(items)
    tris = sum(scene_tris(it[1]) for it in items)
    px = sum(it[0].width * it[0].height for it in items)
    best = autotune.tune(br.ctx, prep, autotune.batch_class(len(items), tris, px))
    br.ctx.set_batch_graphs(True)
    for _ in range(max(3, args.warmup)):
        br.ctx.render_batch(*prep, br.outputs)
    br.ctx.batch_stats()
    tot = 0.0
    for _ in range(args.steps):
        tot += device_time_ms(stream, lambda: br.ctx.render_batch(*prep, br.outputs), flush)
    br.close()
    return views * args.steps / (tot / 1e3), best


def batch_measure(local, stream, items, steps, warmup, tuning=None, ws=1, profile=True):
    """`steps` batches of `items` (one mr_render_batch each, CUDA graph
    replay, K batches back to back between two CUDA events) and the same
    scenes through the plain path, one mr_render per scene.  tuning: a dict
    of TUNING_KEYS, or None for the autotuner."""
    import torch
    from minirender_gb300 import abi, autotune
    from minirender_gb300.batch import BatchRenderer
    from minirender_gb300.renderer import Renderer
    br = BatchRenderer(local)
    br.ctx.set_stream(stream.cuda_stream)
    br.outputs = abi.MR_OUT_RGB8 | abi.MR_OUT_DEPTH
    prep = br.prepare(items)
    T = sum(scene_tris(sc) for st, sc in items)
    P = sum(st.width * st.height for st, sc in items)
    if tuning is not None:
        best = dict(tuning, table=None)
        autotune.apply(br.ctx, best)
    else:
        best = autotune.tune(br.ctx, prep, autotune.batch_class(len(items), T, P))
    br.ctx.set_batch_graphs(True)
    for _ in range(max(3, warmup)):
        br.ctx.render_batch(*prep, br.outputs)
    br.ctx.batch_stats()
    stage = [None, None, None]
    if profile:
        br.ctx.set_profiling(True)
        br.ctx.set_batch_graphs(False)  # stage events need a launch outside the graph
        br.ctx.render_batch(*prep, br.outputs)
        s = br.ctx.batch_stats()
        stage = [round(float(x), 4) for x in s.stage_ms[:3]]
        br.ctx.set_profiling(False)
        br.ctx.set_batch_graphs(True)
        br.ctx.render_batch(*prep, br.outputs)
        br.ctx.batch_stats()
    clocks = Clocks(local)
    barrier(ws)
    torch.cuda.synchronize()
    clocks.start()
    # K batches back to back between two events: the host stages batch k+1
    # while the device renders batch k.  No L2 flush: every batch writes
    # 7 B of output per pixel (and 8 B of visibility words when the setup
    # rasterises small triangles), far more than L2 holds.
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        br.ctx.render_batch(*prep, br.outputs)
    e1.record(stream)
    e1.synchronize()
    clk = clocks.stop()
    total_s = max_over_ranks(e0.elapsed_time(e1) / 1e3, ws)
    value = len(items) * steps * ws / total_s
    # one batch at a time, waiting for each (host staging not overlapped)
    t0 = time.perf_counter()
    for _ in range(steps):
        br.ctx.render_batch(*prep, br.outputs)
        br.ctx.synchronize()
    wall = time.perf_counter() - t0
    # plain path: one mr_render per scene, same scenes
    r = Renderer(local)
    r.ctx.set_stream(stream.cuda_stream)
    r.outputs = abi.MR_OUT_RGB8 | abi.MR_OUT_DEPTH
    per = []
    for st, sc in items:
        r.state = st
        r.setScene(sc)
        per.append(r.prepare())
    for f, rs, n in per[:8]:
        r.ctx.render(f, rs, n, r.outputs)
    r.ctx.synchronize()
    # the same scenes one mr_render each, back to back between two events
    e0.record(stream)
    for _ in range(steps):
        for f, rs, n in per:
            r.ctx.render(f, rs, n, r.outputs)
    e1.record(stream)
    e1.synchronize()
    plain = len(items) * steps / (e0.elapsed_time(e1) / 1e3)
    t0 = time.perf_counter()
    for f, rs, n in per:
        r.ctx.render(f, rs, n, r.outputs)
    r.ctx.synchronize()
    plain_wall = len(items) / (time.perf_counter() - t0)
    r.close()
    br.close()
    return {"value": value, "total_s": total_s, "T": T, "P": P, "best": best, "stage": stage, "clocks": clk,
            "wall_value": len(items) * steps / wall, "plain": plain, "plain_wall": plain_wall}


def batch_arm(args, ws, rank, local):
    """Config 4: `--scenes` independent scenes (seeded primitive hierarchies,
    mixed resolutions) per step, rendered in one batched launch; compared with
    the plain one-frame-per-call path on the same scenes."""
    import torch
    from minirender_gb300 import autotune, build
    build.build()
    from minirender_gb300 import workloads as W
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    items = W.config4(args.scenes)
    tuning = None
    if args.tuning:
        tun = [int(x) for x in args.tuning.split(",")]
        if len(tun) == 3:
            tun = [tun[0]] + tun
        if len(tun) == 4:
            tun.append(autotune.DEFAULT_SMALL_MAX)
        tuning = dict(zip(TUNING_KEYS, tun))
    m = batch_measure(local, stream, items, args.steps, args.warmup, tuning, ws)
    best, P, T = m["best"], m["P"], m["T"]
    value = m["value"]
    return {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(m["total_s"] * 1e3 / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator)",
        "config": {"workload": f"{len(items)} scenes x 64 primitives (cube/sphere/cylinder, 8-64 segments), "
                               "random TRS hierarchy and materials, resolutions from "
                               "{256^2, 512^2, 640x480, 1280x720}, one batched launch per step",
                   "scenes": len(items), "triangles": T, "pixels": P,
                   "l2": f"not flushed: each batch writes {(7 + (8 if best['small_max'] > 0 else 0)) * P / 1e9:.2f} GB "
                         "of outputs and visibility words (> L2)",
                   "timing": "K batches back to back between two CUDA events (host staging overlapped)",
                   "tuning": {k: best[k] for k in TUNING_KEYS}},
        "mtri_per_s": round(value * T / len(items) / 1e6, 2),
        "wall_value_one_batch_at_a_time": round(m["wall_value"], 2),
        "plain_one_frame_per_call": {"value": round(m["plain"], 2), "wall_value": round(m["plain_wall"], 2),
                                     "unit": UNIT},
        "speedup_vs_plain": round(value / m["plain"], 3),
        "stage_ms": {"vertex": m["stage"][0], "setup": m["stage"][1], "fused_bin_raster_shade": m["stage"][2]},
        "autotune_table": best.get("table"),
        "gpu_launches": 3 * args.steps, "clocks": m["clocks"],
    }


def serve_measure(local, rates, n_requests, slots, max_batch, tuning, pool=None, plain_rates=None, repeats=1):
    """Poisson request streams (one per rate in `rates`, then one with every
    request queued at t = 0) through the render server, and the plain path
    (one mr_render + read per request) on the streams of `plain_rates`
    (default: the highest rate and the all-queued one).  With repeats > 1
    each stream runs that many times (the same requests, new mesh keys) and
    its row is the run with the median frames/s, all runs' rates listed."""
    import torch
    from minirender_gb300 import abi, capi
    from minirender_gb300 import workloads as W
    from minirender_gb300.server import RenderServer
    if pool is None:
        pool = W.config5_pool()
        # the asset store lives in page-locked host memory (uploads are DMA,
        # the same for the server and the plain path)
        for m in pool:
            _pin_mesh(m)
    ctx = capi.Context(local)
    tw, th, tthreads, tchunk, tsmall = tuning
    srv = RenderServer(ctx, budget_bytes=40 << 30, slots=slots, max_batch=max_batch, tile=tw,
                       tile_h=th, threads=tthreads, chunk=tchunk, small_max=tsmall)
    maxpx = 3840 * 2160
    ring = [torch.empty(maxpx * 3, dtype=torch.uint8).pin_memory().numpy() for _ in range(96)]
    ring_ticket = [None] * len(ring)

    def stream(reqs):
        tickets = []
        t0 = time.perf_counter()
        for i, q in enumerate(reqs):
            slot = i % len(ring)
            if ring_ticket[slot] is not None:
                srv.wait(ring_ticket[slot])
                ring_ticket[slot] = None
            delay = t0 + q["t"] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            st = q["state"]
            out = {"rgb8": ring[slot][: st.width * st.height * 3].reshape(st.height, st.width, 3)}
            t = srv.submit(st, pool[q["mesh"]], mesh_key=q["key"], texture_key=10_000_000 + q["mesh"],
                           outputs=abi.MR_OUT_RGB8, out=out)
            ring_ticket[slot] = t
            tickets.append(t)
        for k, t in enumerate(ring_ticket):
            if t is not None:
                srv.wait(t)
                ring_ticket[k] = None
        return time.perf_counter() - t0

    # warm-up: a paced stream, then a burst that forms the largest batches, so
    # every slot's buffers have grown and the memory pools are primed
    keys = iter(range(1, 1 << 40, 1 << 20))  # a fresh key range per stream
    stream(W.config5_requests(pool, 64, 1000.0, seed=1, key_base=next(keys)))
    stream(W.config5_requests(pool, 384, math.inf, seed=2, key_base=next(keys)))
    rows = []
    # capacity: every request queued at t = 0 (rate "inf")
    for rate in list(rates) + [math.inf]:
        runs = []
        for _ in range(repeats):
            reqs = W.config5_requests(pool, n_requests, rate, seed=_rate_seed(rate), key_base=next(keys))
            srv.reset_stats()
            wall = stream(reqs)
            s = srv.stats()
            runs.append({"rate_req_s": _rate_label(rate), "frames_per_s": round(s["completed"] / wall, 1),
                         "p50_ms": round(s["p50_us"] / 1e3, 3), "p99_ms": round(s["p99_us"] / 1e3, 3),
                         "max_ms": round(s["max_us"] / 1e3, 3), "mean_batch": round(s["mean_batch"], 2),
                         "requests": int(s["completed"])})
        rows.append(_median_run(runs))
    srv.close()
    ctx.close()
    plain_rates = plain_rates or (rates[-1], math.inf)
    plain_rows = [_median_run([plain_stream(n_requests, pool, ring, local, rate) for _ in range(repeats)])
                  for rate in plain_rates]
    return rows, plain_rows


def _median_run(runs):
    """The run with the median frames/s (the lower middle one for an even
    count), with every run's frames/s listed when there are several."""
    order = sorted(runs, key=lambda r: r["frames_per_s"])
    row = dict(order[(len(order) - 1) // 2])
    if len(runs) > 1:
        row["streams"] = len(runs)
        row["frames_per_s_each"] = [r["frames_per_s"] for r in runs]
    return row


def serve_arm(args, ws, rank, local):
    """Config 5: Poisson request streams at swept rates through the render
    server (continuous batching, resident meshes, 40 GB budget) and the same
    sequence through the plain one-frame-per-call path."""
    import torch
    from minirender_gb300 import build
    build.build()
    torch.cuda.set_device(local)
    tuning = tuple(int(x) for x in args.serve_tuning.split(","))
    rates = [float(x) for x in args.rates.split(",")]
    rows, plain_rows = serve_measure(local, rates, args.requests, args.serve_slots, args.serve_max_batch, tuning)
    served = rows[:-1]
    cap = rows[-1]
    best = max(served, key=lambda x: x["frames_per_s"])
    tw, th, tthreads, tchunk, tsmall = tuning
    return {
        "metric": METRIC, "value": best["frames_per_s"], "unit": UNIT, "n_gpus": ws,
        "steps": args.requests, "warmup": 64, "ms_per_step": round(1e3 / best["frames_per_s"], 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator)",
        "config": {"workload": "Poisson request stream; each request a triangle soup with log-uniform "
                               "1k-2M triangles at log-uniform 128x128..3840x2160, 30% re-render a "
                               "resident mesh with a new camera; 40 GB device budget; RGB8 read back",
                   "server": {"slots": args.serve_slots, "max_batch": args.serve_max_batch,
                              "tuning": {"tile_w": tw, "tile_h": th, "threads": tthreads, "chunk": tchunk,
                                         "small_max": tsmall}}},
        "rates": served, "capacity": cap,
        "plain_one_frame_per_call": plain_rows[0], "plain_capacity": plain_rows[1],
        "served_vs_plain_at_max_rate": round(served[-1]["frames_per_s"] / plain_rows[0]["frames_per_s"], 3),
        "served_vs_plain_capacity": round(cap["frames_per_s"] / plain_rows[1]["frames_per_s"], 3),
    }


def _pin_mesh(mesh) -> None:
    """Moves a TriMesh's arrays into page-locked host memory (in place)."""
    pm, keep = _pinned_copy(mesh)
    for name in _MESH_ARRAYS:
        setattr(mesh, name, getattr(pm, name))
    mesh._pinned = keep


def _rate_seed(rate: float) -> int:
    return int(rate) if math.isfinite(rate) else 99991


def _rate_label(rate: float):
    return rate if math.isfinite(rate) else "all queued at t=0"


def plain_stream(n_requests, pool, ring, local, rate):
    """The request sequence of `rate` through the plain path, one
    mr_render + synchronous read per request (arrival times honoured)."""
    from minirender_gb300 import abi
    from minirender_gb300 import workloads as W
    from minirender_gb300.renderer import Renderer
    reqs = W.config5_requests(pool, n_requests, rate, seed=_rate_seed(rate))
    r = Renderer(local)
    r.outputs = abi.MR_OUT_RGB8
    resident = {}
    tex_h = {}
    done_t = []
    t0 = time.perf_counter()
    for i, q in enumerate(reqs):
        now = time.perf_counter() - t0
        if now < q["t"]:
            time.sleep(q["t"] - now)
        mesh = pool[q["mesh"]]
        if q["key"] not in resident:
            resident[q["key"]] = r.ctx.upload_mesh(mesh.desc())
            if len(resident) > 64:
                old = next(iter(resident))
                r.ctx.free_mesh(resident.pop(old))
        if q["mesh"] not in tex_h:
            tex_h[q["mesh"]] = r.ctx.upload_texture(mesh.material.texture)
        rs = (abi.mr_renderable * 1)()
        rs[0].mesh = resident[q["key"]]
        rs[0].transform[:] = [float(x) for x in np.eye(4, dtype=np.float32).reshape(16)]
        m = mesh.material
        rs[0].material.diffuse[:] = [float(x) for x in m.diffuse]
        rs[0].material.specular[:] = [float(x) for x in m.specular]
        rs[0].material.emissive[:] = [float(x) for x in m.emissive]
        rs[0].material.shininess = float(m.shininess)
        rs[0].material.texture = tex_h[q["mesh"]]
        st = q["state"]
        r.ctx.render(st.to_c(), rs, 1, abi.MR_OUT_RGB8)
        out = ring[i % len(ring)][: st.width * st.height * 3]
        r.ctx.read_into(out, None)
        done_t.append(time.perf_counter() - t0)
    wall = time.perf_counter() - t0
    lat = np.array(done_t) - np.array([q["t"] for q in reqs])
    for h in resident.values():
        r.ctx.free_mesh(h)
    r.close()
    return {"rate_req_s": _rate_label(rate), "frames_per_s": round(len(reqs) / wall, 1),
            "p50_ms": round(float(np.percentile(lat, 50)) * 1e3, 3),
            "p99_ms": round(float(np.percentile(lat, 99)) * 1e3, 3)}


def gpu_arm(args, ws, rank, local):
    import torch
    from minirender_gb300 import abi, build
    build.build()
    from minirender_gb300.renderer import Renderer

    torch.cuda.set_device(local)
    st, sc, desc = make_workload(args.workload, args)
    V, T, mesh_bytes, tex_bytes = scene_sizes(sc)
    P = st.width * st.height
    r = Renderer(local)
    # A dedicated stream: the library and the timing events share it (the
    # legacy default stream's handle is 0, which the C ABI reads as "use the
    # context's own stream").
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    r.ctx.set_stream(stream.cuda_stream)
    r.outputs = abi.MR_OUT_RGB8 | abi.MR_OUT_DEPTH
    r.state = st
    r.setScene(sc)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    assert stream.cuda_stream != 0

    frame, rs, n = r.prepare()
    for _ in range(max(3, args.warmup)):
        r.ctx.render(frame, rs, n, r.outputs)
        r.ctx.stats()
    r.ctx.synchronize()
    # per-stage device times: a separate pass with events between the kernels
    r.ctx.set_profiling(True)
    stage_tot = np.zeros(len(STAGES))
    n_prof = min(args.steps, 10)
    for _ in range(n_prof):
        flush.zero_()
        r.ctx.render(frame, rs, n, r.outputs)
        s = r.ctx.stats()  # waits for the frame, reads per-stage event times
        stage_tot += np.array(s.stage_ms[:len(STAGES)], np.float64)
    stats = r.ctx.stats()
    r.ctx.set_profiling(False)
    clocks = Clocks(local)
    barrier(ws)
    torch.cuda.synchronize()
    clocks.start()
    step_ms = []
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r.ctx.render(frame, rs, n, r.outputs)
        e1.record(stream)
        r.ctx.stats()  # waits for the frame (and checks its status)
        step_ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier(ws)
    total_s = max_over_ranks(sum(step_ms) / 1e3, ws)
    value = args.steps * ws / total_s

    # ---- end to end through the C ABI, host buffers, copies inside the region
    from minirender_gb300 import scene as S
    flat = S.flatten(sc)
    e2e_value = res_value = None
    h2d = d2h = 0
    if not args.no_e2e:
        e2e_value, res_value, h2d, d2h = e2e_legs(args, ws, r, sc, st, flat, frame, rs, n,
                                                  mesh_bytes, tex_bytes)
    # ---- roofline of the dominant kernel
    stage_ms = stage_tot / n_prof
    dom = int(np.argmax(stage_ms))
    name = STAGES[dom]
    tex_px = P if flat.textures else 0
    n_big = int(stats.binned)
    # the library runs the per-vertex pass only when vertices are shared
    # (3T >= 2V); otherwise the setup reads and transforms corners itself
    vertex_pass = 3 * T >= 2 * V
    alg = {
        "clear+vertex": 8 * P + (12 * V + 24 * V + 16 * V if vertex_pass else 0),
        "setup": 12 * T + 12 * V + 64 * n_big,
        # row blocks (8 B each) and their records; the vis words it updates
        # are the clear's, resident in L2
        "large_raster": 8 * int(stats.bin_entries) + 64 * n_big,
        "-": 0,
        "resolve": 8 * P + 7 * P + 3 * tex_px,
    }
    peak, peak_kind = peaks()
    achieved = alg[name] / (stage_ms[dom] / 1e3) / 1e9
    counts = ncu_counts(args.workload).get(KERNELS[name], {})
    traffic = counts.get("dram_bytes")
    # instruction-issue ceiling: warp instructions of one launch (ncu) over
    # what the SMs' four schedulers can issue in the kernel's event time at
    # the median SM clock of the timed region
    n_sms = torch.cuda.get_device_properties(local).multi_processor_count
    mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz")
    issue_frac = None
    if counts.get("warp_inst") and mhz:
        issue_frac = counts["warp_inst"] / (n_sms * 4 * mhz * 1e6 * stage_ms[dom] / 1e3)
    frame_bytes = (32 * V if vertex_pass else 12 * V) + 36 * T + 16 * P + 7 * P + 3 * tex_px
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total_s * 1e3 / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator)",
        "config": {"workload": desc, "triangles": T, "vertices": V, "width": st.width,
                   "height": st.height, "l2": "flushed between frames (256 MiB write)",
                   "parallelism": "replicas" if ws > 1 else "single"},
        "mtri_per_s": round(value * T / 1e6, 2),
        "e2e": None if e2e_value is None else {
            "value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "contexts": max(1, args.e2e_contexts),
            "link_gbs": round((h2d + d2h) * e2e_value / ws / 1e9, 1)},
        "e2e_resident_mesh": None if res_value is None else {
            "value": round(res_value, 3), "unit": UNIT, "h2d_bytes_per_step": 0,
            "d2h_bytes_per_step": int(d2h)},
        "roofline": {"bound": "hbm", "kernel": KERNELS[name], "achieved": round(achieved, 2),
                     "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": peak_kind, "traffic": traffic,
                     "algorithmic_bytes": int(alg[name]), "kernel_ms": round(float(stage_ms[dom]), 5),
                     "issue_frac": None if issue_frac is None else round(issue_frac, 4),
                     "warp_inst": counts.get("warp_inst"), "sms": n_sms},
        "stage_ms": {k: round(float(v), 5) for k, v in zip(STAGES, stage_ms)},
        "frame_roofline": {"algorithmic_bytes": int(frame_bytes),
                           "achieved_gbs": round(frame_bytes / (total_s / args.steps * ws) / 1e9, 2),
                           "frac": round(frame_bytes / (total_s / args.steps * ws) / 1e9 / peak, 4)},
        "counters": {"clipped": int(stats.clipped), "rasterised": int(stats.rasterised),
                     "small_direct": int(stats.small_direct), "binned": int(stats.binned),
                     "bin_entries": int(stats.bin_entries)},
        # k_clear, [k_vertex], k_setup, k_raster_large, k_resolve per frame
        "gpu_launches": (5 if vertex_pass else 4) * args.steps,
        "clocks": clk,
    }
    if args.views > 0 and not args.no_e2e:
        bv, best = batched_views(args, stream, flush, st, sc, args.views)
        out["batched"] = {"value": round(bv, 3), "unit": UNIT, "views_per_launch": args.views,
                          "speedup_vs_plain": round(bv / value, 3),
                          "tuning": {k: best[k] for k in TUNING_KEYS}}
    if args.workload == "config2" and not args.no_extras:
        out.update(extras(local, stream))
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        n_threads = os.cpu_count() or 1
        frames = 2 * n_threads
        fps, secs = cpu_frames_per_s(st, sc, n_threads, frames)
        fps1, secs1 = cpu_frames_per_s(st, sc, 1, 1)
        out["cpu_baseline"] = {
            "value": round(fps, 4), "unit": UNIT, "cores": n_threads, "kind": "port",
            "sample": f"{frames} frames of the same workload, one renderer per thread on "
                      f"{n_threads} threads ({secs:.1f} s); single thread: {fps1:.4f} frames/s",
            "single_thread_value": round(fps1, 4)}
    r.close()
    return out


def reference_arm(args, ws, rank):
    if rank != 0:
        return None
    st, sc, desc = make_workload(args.workload, args)
    V, T, _, _ = scene_sizes(sc)
    n_threads = os.cpu_count() or 1
    for _ in range(max(0, args.warmup)):
        pass  # the C restatement has no warm-up state; keep the loop shape
    cpu_frames_per_s(st, sc, n_threads, n_threads)  # one untimed round (page-in)
    total = 0.0
    for _ in range(args.steps):
        _, secs = cpu_frames_per_s(st, sc, n_threads, n_threads)
        total += secs
    value = args.steps * n_threads / total
    return {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total * 1e3 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator)", "impl": "reference",
        "config": {"workload": desc, "triangles": T, "vertices": V, "width": st.width,
                   "height": st.height, "parallelism": "host threads"},
        "mtri_per_s": round(value * T / 1e6, 3),
        "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": n_threads, "kind": "port",
                         "sample": f"each step renders {n_threads} frames, one per host thread "
                                   "(the reference's own build needs ASL, which is not available)"},
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


DEFAULT_STEPS = {"config1": 2000, "config2": 2000, "config3": 200, "config4": 20, "config5": 1}


def main():
    args = parse()
    if args.steps is None:  # the reference arm's steps are whole CPU frames on every host thread
        args.steps = DEFAULT_STEPS[args.workload] if args.impl == "gb300" else 10
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        out = reference_arm(args, ws, rank)
    elif args.workload == "config4":
        out = batch_arm(args, ws, rank, local)
    elif args.workload == "config5":
        out = serve_arm(args, ws, rank, local)
    else:
        out = gpu_arm(args, ws, rank, local)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
