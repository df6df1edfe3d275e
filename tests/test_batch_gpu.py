"""Batched rendering (mr_render_batch): every scene of a batch equals the
oracle's render of that scene alone (bit-exact ids and depth, RGB8 within
1 LSB), with and without CUDA-graph replay, for every tuning."""
import numpy as np
import pytest

import edge_scenes as E
from parity import assert_parity, compare, report
from minirender_gb300 import projection as pj
from minirender_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

def _items():
    items = [W.config4_scene(s) for s in range(6)]
    items.append(W.config1())
    items.append(W.config2(level=6, width=480, height=270, tex_size=256))
    for name in ("near_clip", "ortho_negative_z", "ties", "big_triangles", "texture_wrap"):
        items.append(E.ALL[name]())
    return items


@pytest.fixture(scope="module")
def batch(product_lib):
    from minirender_gb300.batch import BatchRenderer
    b = BatchRenderer(0)
    yield b
    b.close()


@pytest.fixture(scope="module")
def refs():
    return [O.render(st, sc) for st, sc in _items()]


def _check_all(b, items, refs, tag):
    b.render(items)
    out = []
    for i, ref in enumerate(refs):
        got = b.read(i)
        got["image"] = ref["image"]  # the batch path outputs bytes, not floats
        stats = compare(got, ref, f"batch_{tag}_{i}")
        out.append(stats)
        assert_parity(stats)
    report(out, "batch")
    return out


@pytest.mark.parametrize("graphs", [False, True])
def test_batch_matches_oracle(batch, refs, graphs):
    batch.ctx.set_batch_graphs(graphs)
    batch.ctx.set_batch_tuning(16, 256, 64)
    _check_all(batch, _items(), refs, f"g{int(graphs)}")


def test_graph_replay_with_new_cameras(batch, refs):
    """A second batch of the same shape replays the captured graph; new
    cameras and lights must be picked up."""
    batch.ctx.set_batch_graphs(True)
    batch.ctx.set_batch_tuning(16, 256, 64)
    items = _items()
    _check_all(batch, items, refs, "first")
    moved = []
    for st, sc in items:
        st.view = pj.mat_mul(st.view, pj.rotate_z(0.3))
        st.light = np.array([0.5, -0.2, 1.0], np.float32)
        moved.append((st, sc))
    new_refs = [O.render(st, sc) for st, sc in moved]
    _check_all(batch, moved, new_refs, "replay")


@pytest.mark.parametrize("tw,th,threads,chunk", [(64, 16, 128, 128), (128, 8, 64, 32), (256, 4, 256, 64),
                                                  (4, 16, 64, 16), (64, 64, 256, 128)])
def test_batch_rectangular_tiles_same_result(batch, refs, tw, th, threads, chunk):
    batch.ctx.set_batch_graphs(True)
    batch.ctx.set_batch_tiling(tw, th, threads, chunk)
    try:
        _check_all(batch, _items(), refs, f"r{tw}x{th}_{threads}_{chunk}")
    finally:
        batch.ctx.set_batch_tuning(16, 256, 64)


@pytest.mark.parametrize("small_max", [0, 16, 4096])
def test_batch_small_max_same_result(batch, refs, small_max):
    """Triangles rasterised by the setup kernel (bbox <= small_max pixels)
    and triangles binned into the fused tile kernel give the same pixels."""
    batch.ctx.set_batch_graphs(True)
    batch.ctx.set_batch_tuning(16, 128, 64)
    batch.ctx.set_batch_small_max(small_max)
    try:
        _check_all(batch, _items(), refs, f"s{small_max}")
    finally:
        batch.ctx.set_batch_small_max(64)
        batch.ctx.set_batch_tuning(16, 256, 64)


def test_batch_tiling_rejects_bad_shapes(batch):
    from minirender_gb300 import capi
    for bad in [(48, 16, 64, 64), (512, 2, 64, 64), (8, 4, 64, 64), (64, 128, 64, 64), (128, 64, 64, 64),
                (16, 16, 96, 64)]:
        with pytest.raises(capi.MRError):
            batch.ctx.set_batch_tiling(*bad)
    for bad in (-1, 4097):
        with pytest.raises(capi.MRError):
            batch.ctx.set_batch_small_max(bad)


@pytest.mark.parametrize("tile,threads,chunk", [(8, 64, 16), (16, 128, 256), (32, 256, 32), (32, 128, 128)])
def test_batch_tuning_same_result(batch, refs, tile, threads, chunk):
    batch.ctx.set_batch_graphs(True)
    batch.ctx.set_batch_tuning(tile, threads, chunk)
    try:
        _check_all(batch, _items(), refs, f"t{tile}_{threads}_{chunk}")
    finally:
        batch.ctx.set_batch_tuning(16, 256, 64)


def test_batch_of_triangle_soups(batch):
    """Soups (no shared vertices: the kernels transform corners themselves,
    no per-vertex pass) with exact duplicate triangles, small and binned."""
    items = [W.config3(n_tris=20000, width=320, height=240, seed=70 + k) for k in range(3)]
    items.append(W.config3(n_tris=3000, width=640, height=360, seed=77))
    refs = [O.render(st, sc) for st, sc in items]
    batch.ctx.set_batch_graphs(True)
    try:
        for small_max in (64, 0):
            batch.ctx.set_batch_small_max(small_max)
            _check_all(batch, items, refs, f"soup{small_max}")
    finally:
        batch.ctx.set_batch_small_max(64)


def test_batch_of_random_scenes(batch):
    """48 seeded random scenes of uneven sizes and triangle counts in one
    batch (soups and indexed meshes, clipping, both projections, textures),
    with and without graph replay."""
    items = [E.random_scene(s) for s in range(48)]
    refs = [O.render(st, sc) for st, sc in items]
    for graphs in (False, True):
        batch.ctx.set_batch_graphs(graphs)
        _check_all(batch, items, refs, f"random_g{int(graphs)}")
    batch.ctx.set_batch_graphs(True)


def _switch_flags(k: int) -> int:
    """A cycle of renderable switch combinations (MR_RS_OWN_STATE with and
    without lighting, texturing and point light; 0 = the frame's)."""
    from minirender_gb300 import abi
    own, lit, tex, pt = abi.MR_RS_OWN_STATE, abi.MR_RS_LIGHTING, abi.MR_RS_TEXTURING, abi.MR_RS_POINT_LIGHT
    return (0, own | tex, own | lit, own | lit | tex | pt, own, own | lit | pt, own | tex | pt)[k % 7]


def test_batch_with_paint_switches(batch):
    """Renderables carrying their paint call's switches (MR_RS_OWN_STATE:
    lighting, texturing, light type) in a batch equal the oracle's render
    with the same flags, with and without graph replay."""
    items = [W.config4_scene(s) for s in range(3)]
    items.append(W.config2(level=5, width=320, height=200, tex_size=64))
    items.append(E.ALL["near_clip"]())
    items.append(E.ALL["texture_wrap"]())
    scenes, ns, rs, nr = batch.prepare(items)
    refs = []
    for s, (st, sc) in enumerate(items):
        first, n = scenes[s].first_renderable, scenes[s].n_renderables
        for i in range(n):
            rs[first + i].flags |= _switch_flags(first + i)
        refs.append(O.render(st, sc, flags=[_switch_flags(first + i) for i in range(n)]))
    for graphs in (False, True):
        batch.ctx.set_batch_graphs(graphs)
        batch.ctx.render_batch(scenes, ns, rs, nr, batch.outputs)
        out = []
        for i, ref in enumerate(refs):
            got = batch.read(i)
            got["image"] = ref["image"]
            stats = compare(got, ref, f"batch_switches_g{int(graphs)}_{i}")
            out.append(stats)
            assert_parity(stats)
        report(out, "batch")
    batch.ctx.set_batch_graphs(True)


def test_batch_with_empty_scenes(batch):
    """Scenes without renderables or with empty meshes come out as background
    (and do not disturb the other scenes of the batch)."""
    from minirender_gb300.scene import Scene, TriMesh
    st1, sc1 = W.config1(96, 64)
    empty = Scene()
    st_e = W.config1(80, 48)[0]
    hollow = Scene()
    hollow.add(TriMesh(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), np.zeros(0, np.int32)))
    items = [(st_e, empty), (st1, sc1), (st_e, hollow)]
    refs = [O.render(st, sc) for st, sc in items]
    batch.ctx.set_batch_graphs(False)
    _check_all(batch, items, refs, "empty")
    batch.ctx.set_batch_graphs(True)
