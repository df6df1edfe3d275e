"""Parity at the benchmark configurations' full sizes (device path vs the
oracle, bit-exact ids and depth, RGB8 within 1 LSB on >= 99.9 % of pixels):

* the heavy-overdraw soup: 10,000,000 triangles of 1-4 px^2 at 3840x2160,
  500,000 of them exact coplanar duplicates drawn after their originals,
  which must lose every depth tie (the reference's strict z < depth,
  src/Renderer.cpp:267) -- sub-triangle ids reach 2 x 10^7;
* the full 256-scene batch of primitive hierarchies through one
  mr_render_batch, every scene compared with the oracle's render of it alone;
* 32 serving requests drawn from the serving stream's own size
  distribution (triangle soups of 1k-2M triangles at 128x128 .. 3840x2160,
  30 % re-renders of a resident mesh), all submitted at once to the render
  server and each compared with the oracle's render of that request alone.

Per-case figures go to MR_PARITY_REPORT_DIR when it is set."""
import numpy as np
import pytest

from parity import assert_parity, compare, gpu_render, report
from minirender_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_config3_full_size(product_lib):
    """10 M-triangle soup at 3840x2160 with 5 % exact duplicates."""
    from minirender_gb300.renderer import Renderer
    st, sc = W.config3()
    mesh = sc.children[0]
    assert mesh.indices.size == 3 * 10_000_000 and (st.width, st.height) == (3840, 2160)
    r = Renderer(0)
    try:
        gpu, _ = gpu_render(st, sc, r)
        s = r.ctx.stats()
    finally:
        r.close()
    ref = O.render(st, sc)
    stats = compare(gpu, ref, "config3_full_10M_3840x2160")
    # duplicates (triangles 9.5M..10M) may never win: each ties its original,
    # which is drawn first
    ids = ref["ids"][ref["ids"] != 0xFFFFFFFF] >> 1
    stats["duplicate_winners"] = int((ids >= 9_500_000).sum())
    stats["max_id"] = int(gpu["ids"][gpu["ids"] != 0xFFFFFFFF].max())
    stats["rasterised"] = int(s.rasterised)
    report(stats, "fullsize")
    assert_parity(stats)
    assert stats["duplicate_winners"] == 0
    assert stats["covered"] > 7_000_000 and stats["max_id"] > 2 * 9_000_000


def test_config4_full_batch(product_lib):
    """All 256 scenes in one batched launch (graph replay on), each equal to
    the oracle's render of it alone."""
    from minirender_gb300.batch import BatchRenderer
    items = W.config4(256)
    b = BatchRenderer(0)
    try:
        b.render(items)
        got = [b.read(i) for i in range(len(items))]
    finally:
        b.close()
    rows = []
    for i, (st, sc) in enumerate(items):
        ref = O.render(st, sc)
        g = dict(got[i])
        g["image"] = ref["image"]  # the batch path outputs bytes, not floats
        rows.append(compare(g, ref, f"config4_full_scene{i}"))
    report(rows, "fullsize")
    for s in rows:
        assert_parity(s)
    assert sum(s["covered"] for s in rows) > 10_000_000


def test_config5_request_sample(product_lib):
    """32 requests of the serving stream at their real sizes (capped at the
    stream's own 2 M triangles), submitted together so they are batched with
    one another, each equal to the oracle's render of it alone."""
    from minirender_gb300 import abi, capi
    from minirender_gb300.scene import Scene
    from minirender_gb300.server import RenderServer
    pool = W.config5_pool()
    assert max(m.indices.size // 3 for m in pool) <= 2_000_000
    reqs = W.config5_requests(pool, 32, 5000.0, seed=11)
    ctx = capi.Context(0)
    srv = RenderServer(ctx, budget_bytes=40 << 30, slots=3, max_batch=16, tile=16, tile_h=16, threads=64,
                       chunk=64, small_max=64)
    outs, tickets = [], []
    try:
        for q in reqs:
            st = q["state"]
            out = {"rgb8": np.zeros((st.height, st.width, 3), np.uint8),
                   "depth": np.zeros((st.height, st.width), np.float32),
                   "ids": np.zeros((st.height, st.width), np.uint32)}
            tickets.append(srv.submit(st, pool[q["mesh"]], mesh_key=q["key"], texture_key=7000 + q["mesh"],
                                      outputs=abi.MR_OUT_RGB8 | abi.MR_OUT_DEPTH | abi.MR_OUT_TRI_ID, out=out))
            outs.append(out)
        sizes = [srv.wait(t).batch_size for t in tickets]
    finally:
        srv.close()
        ctx.close()
    assert max(sizes) > 1, "the sample was never batched"
    assert any(q["key"] == p["key"] for i, q in enumerate(reqs) for p in reqs[:i]), "no re-render in the sample"
    rows = []
    for i, q in enumerate(reqs):
        sc = Scene()
        sc.add(pool[q["mesh"]])
        ref = O.render(q["state"], sc)
        g = dict(outs[i])
        g["image"] = ref["image"]
        s = compare(g, ref, f"config5_req{i}_{q['state'].width}x{q['state'].height}")
        s["triangles"] = int(pool[q["mesh"]].indices.size // 3)
        s["batch_size"] = sizes[i]
        rows.append(s)
    report(rows, "fullsize")
    for s in rows:
        assert_parity(s)
