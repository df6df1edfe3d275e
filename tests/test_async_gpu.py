"""Asynchronous reads (mr_read_async + mr_wait): the same bytes as mr_read,
two contexts with frames in flight at once, and a frame whose large-triangle
row-block list overflowed (its remaining rows go through the spill list)
read asynchronously and synchronously."""
import numpy as np
import pytest

import edge_scenes as E
from parity import assert_parity, compare
from minirender_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _pinned(shape, dtype):
    import torch
    return torch.from_numpy(np.zeros(shape, dtype)).pin_memory().numpy()


def _targets(st):
    return (_pinned((st.height, st.width, 3), np.uint8), _pinned((st.height, st.width), np.float32),
            _pinned((st.height, st.width), np.uint32))


def _render_async(r, st, sc, bufs):
    r.state = st
    r.setScene(sc)
    frame, rs, n = r.prepare()
    r.ctx.render(frame, rs, n, r.outputs)
    r.ctx.read_async(*bufs)


def test_read_async_matches_read(product_lib):
    from minirender_gb300.renderer import Renderer
    st, sc = W.config2(level=6, width=640, height=360, tex_size=256)
    r = Renderer(0)
    try:
        r.state = st
        r.setScene(sc)
        r.render()
        want = r.ctx.read(rgb8=True, depth=True, tri_id=True)
        bufs = _targets(st)
        _render_async(r, st, sc, bufs)
        assert r.ctx.wait() == 0
        for k, b in zip(("rgb8", "depth", "ids"), bufs):
            assert np.array_equal(want[k].view(np.uint8), b.view(np.uint8)), k
    finally:
        r.close()


def test_two_contexts_in_flight(product_lib):
    """Frames alternate between two contexts (their own streams); each
    context's next render waits only for its own previous frame."""
    from minirender_gb300 import projection as pj
    from minirender_gb300.renderer import Renderer
    import copy
    st, sc = W.config2(level=6, width=480, height=270, tex_size=128)
    views = []
    for k in range(6):
        s2 = copy.copy(st)
        s2.view = pj.mat_mul(st.view, pj.rotate_z(0.3 * k))
        views.append(s2)
    want = []
    ref = Renderer(0)
    try:
        for s2 in views:
            ref.state = s2
            ref.setScene(sc)
            ref.render()
            want.append(ref.ctx.read(rgb8=True, depth=True, tri_id=True))
    finally:
        ref.close()
    rr = [Renderer(0), Renderer(0)]
    bufs = [[_targets(st) for _ in range(3)] for _ in range(2)]
    got = []
    try:
        for k, s2 in enumerate(views):
            r = rr[k % 2]
            if k >= 2:
                assert r.ctx.wait() == 0
                got.append([b.copy() for b in bufs[k % 2][(k // 2 - 1) % 3]])
            _render_async(r, s2, sc, bufs[k % 2][(k // 2) % 3])
        for k in (len(views) - 2, len(views) - 1):
            assert rr[k % 2].ctx.wait() == 0
            got.append([b.copy() for b in bufs[k % 2][(k // 2) % 3]])
    finally:
        for r in rr:
            r.close()
    for k, (w, g) in enumerate(zip(want, got)):
        for name, b in zip(("rgb8", "depth", "ids"), g):
            assert np.array_equal(w[name].view(np.uint8), b.view(np.uint8)), (k, name)


@pytest.mark.parametrize("mode", ["async", "sync"])
def test_row_block_overflow_spills(product_lib, mode):
    """A fresh context's row-block list is too small for this frame: the
    records whose blocks do not fit are rasterised from the spill list in the
    same launch, so the frame is complete without a re-run."""
    from minirender_gb300.renderer import Renderer
    st, sc = E.tall_layers()
    ref = O.render(st, sc)
    r = Renderer(0)
    try:
        if mode == "async":
            bufs = _targets(st)
            _render_async(r, st, sc, bufs)
            assert r.ctx.wait() == 0
            got = dict(zip(("rgb8", "depth", "ids"), bufs))
        else:
            r.state = st
            r.setScene(sc)
            r.render()
            got = r.ctx.read(rgb8=True, depth=True, tri_id=True)
        s = r.ctx.stats()
        assert s.bin_entries > (1 << 18)  # more row blocks than the first list holds
        assert np.array_equal(got["ids"], ref["ids"])
        assert np.array_equal(got["depth"].view(np.uint32), ref["depth"].view(np.uint32))
        d8 = np.abs(got["rgb8"].astype(np.int16) - ref["rgb8"].astype(np.int16)).max(-1)
        assert (d8 <= 1).mean() >= 0.999
    finally:
        r.close()


def test_shared_upload_stream_updates(product_lib):
    """Two contexts share one upload stream; every step updates the mesh
    (alternating between two vertex sets) before rendering it.  Each frame
    shows the vertices given for it: an update waits for the frames that
    read the old contents, and the frame waits for its update."""
    import copy
    import torch
    from minirender_gb300.renderer import Renderer
    from minirender_gb300.scene import TriMesh
    st, sc = W.config2(level=5, width=320, height=240, tex_size=64)
    m = sc.children[0]

    def pinned(a):
        return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()

    idx = pinned(m.indices)
    versions = []
    for scale in (1.0, 1.07):
        versions.append(TriMesh(pinned(m.vertices * np.float32(scale)), pinned(m.normals), idx, normalsI=idx,
                                texcoords=pinned(m.texcoords), texcoordsI=idx, material=m.material))
    want = []
    ref = Renderer(0)
    try:
        for v in versions:
            sc2 = copy.copy(sc)
            sc2.children = [v]
            ref.state = st
            ref.setScene(sc2)
            ref.render()
            want.append(ref.ctx.read(rgb8=True, depth=True, tri_id=True))
    finally:
        ref.close()
    assert not np.array_equal(want[0]["ids"], want[1]["ids"])
    up = torch.cuda.Stream()
    lanes = []
    for _ in range(2):
        r = Renderer(0)
        r.state = st
        r.setScene(sc)
        frame, rs, n = r.prepare()
        r.ctx.set_upload_stream(up.cuda_stream)
        lanes.append((r, frame, rs, n, r._mesh_handle(m)))
    steps = 8
    bufs = [_targets(st) for _ in range(steps)]
    try:
        for k in range(steps):
            r, frame, rs, n, h = lanes[k % 2]
            r.ctx.update_mesh(h, versions[(k // 2) % 2].desc())
            r.ctx.render(frame, rs, n, r.outputs)
            r.ctx.read_async(*bufs[k])
        for r, *_ in lanes:
            assert r.ctx.wait() == 0
    finally:
        for r, *_ in lanes:
            r.ctx.set_upload_stream(None)
            r.close()
    for k in range(steps):
        w = want[(k // 2) % 2]
        for name, b in zip(("rgb8", "depth", "ids"), bufs[k]):
            assert np.array_equal(w[name].view(np.uint8), b.view(np.uint8)), (k, name)
