"""mr_render_noalloc: the entry point for callers that cannot allocate device
memory (a host framework whose pool owns the device, or a real-time loop that
cannot pay for cudaMalloc/cudaFree).  It keeps its working memory in a fixed
device array inside the library, so this test checks that its output equals
the ordinary entry point's (mr_render through Renderer) and the oracle's on
two calls in a row -- the second call starts from the scratch the first one
left behind -- for an untextured and a textured scene, for large triangles
(records from the fixed store) and for more large triangles than the store
holds (the rest rasterised by the setup kernel); that a mesh with an
out-of-range index is reported and a good mesh right after it renders
correctly (no stale index-check bits); that an empty mesh with no outputs
succeeds; and that oversized requests are refused before any device work.

This file is named to be collected last; it passes on its own in a fresh
process as well as after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from parity import RGB8_FRAC_MIN
from minirender_gb300 import abi, capi
from oracle import oracle as O
from minirender_gb300 import scene as S
from minirender_gb300 import workloads as W
from minirender_gb300.renderer import Renderer

pytestmark = pytest.mark.gpu


def _scenes():
    yield "sphere_640x480", W.config1()
    yield "textured_icosphere_640x360", W.config2(level=6, width=640, height=360, tex_size=256)


def _existing(st, sc):
    r = Renderer(0)
    try:
        r.state = st
        r.setScene(sc)
        r.render()
        return {"rgb8": r.getImageRGB8().copy(), "depth": r.getDepth().copy(),
                "ids": r.getTriangleIds().copy()}
    finally:
        r.close()


def _device_mesh(mesh, indices=None):
    import torch
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    arrays = {k: getattr(mesh, k) for k in ("vertices", "normals", "texcoords", "indices", "normalsI",
                                            "texcoordsI")}
    if indices is not None:
        arrays["indices"] = indices
    keep = {k: dev(a) for k, a in arrays.items() if a.size}
    p = lambda k: keep[k].data_ptr() if k in keep else None  # noqa: E731
    desc = abi.mr_mesh_desc(p("vertices"), mesh.vertices.shape[0], p("normals"), mesh.normals.shape[0],
                            p("texcoords"), mesh.texcoords.shape[0], p("indices"), arrays["indices"].size,
                            p("normalsI"), mesh.normalsI.size, p("texcoordsI"), mesh.texcoordsI.size)
    return desc, keep


def _noalloc(st, sc, calls=2, indices=None, expect=abi.MR_OK):
    import torch
    flat = S.flatten(sc)
    rs, n = capi.collect_shapes(flat.nodes)
    assert n == 1
    mesh = flat.meshes[rs[0].mesh]
    desc, _keep = _device_mesh(mesh, indices)
    tex = flat.textures[0] if flat.textures else None
    tex_d = torch.from_numpy(np.ascontiguousarray(tex)).cuda() if tex is not None else None
    H, W_ = st.height, st.width
    rgb8 = torch.empty((H, W_, 3), dtype=torch.uint8, device="cuda")
    depth = torch.empty((H, W_), dtype=torch.float32, device="cuda")
    ids = torch.empty((H, W_), dtype=torch.int32, device="cuda")
    frame = st.to_c()
    xf = (C.c_float * 16)(*rs[0].transform)
    torch.cuda.synchronize()
    outs = []
    for _ in range(calls):
        rc = capi.lib().mr_render_noalloc(
            C.byref(frame), C.byref(desc), C.addressof(xf), C.byref(rs[0].material),
            tex_d.data_ptr() if tex_d is not None else None,
            tex.shape[0] if tex is not None else 0, tex.shape[1] if tex is not None else 0,
            int(tex is not None and tex.dtype == np.uint8),
            rgb8.data_ptr(), depth.data_ptr(), ids.data_ptr(), torch.cuda.current_stream().cuda_stream)
        assert rc == expect, capi.lib().mr_status_string(rc)
        outs.append({"rgb8": rgb8.cpu().numpy(), "depth": depth.cpu().numpy(),
                     "ids": ids.cpu().numpy().view(np.uint32)})
        rgb8.fill_(7)
        depth.fill_(-3.0)
        ids.fill_(5)
    return outs


def _same(got, want, what):
    assert np.array_equal(got["ids"], want["ids"]), f"{what}: visible ids differ"
    assert np.array_equal(got["depth"].view(np.uint32), want["depth"].view(np.uint32)), f"{what}: depth"
    d = np.abs(got["rgb8"].astype(np.int16) - want["rgb8"].astype(np.int16)).max(-1)
    assert (d <= 1).mean() >= RGB8_FRAC_MIN, f"{what}: rgb8"


@pytest.mark.parametrize("name,case", list(_scenes()), ids=[n for n, _ in _scenes()])
def test_noalloc_matches_existing_entry_point(product_lib, name, case):
    st, sc = case
    want = _existing(st, sc)
    ref = O.render(st, sc)
    for k, got in enumerate(_noalloc(st, sc)):
        _same(got, want, f"call {k} vs mr_render")
        _same(got, ref, f"call {k} vs the oracle")


def _strips(n, w, h, seed):
    """n thin horizontal triangles of 80-200 x 3 pixels (each bounding box
    above 64 pixels, so each one takes a large-triangle record), front-facing,
    at random depths, under an orthographic projection of one unit per pixel."""
    from minirender_gb300 import projection as pj
    from minirender_gb300.frame import FrameState
    rng = np.random.default_rng(seed)
    x0 = rng.uniform(-w / 2, w / 2 - 200, n)
    y0 = rng.uniform(-h / 2, h / 2 - 3, n)
    ln = rng.uniform(80, 200, n)
    z = -rng.uniform(2, 50, n)
    v = np.stack([np.stack([x0, y0, z], 1), np.stack([x0 + ln, y0 + 0.5, z], 1),
                  np.stack([x0, y0 + 2, z], 1)], 1).reshape(-1, 3).astype(np.float32)
    idx = np.arange(3 * n, dtype=np.int32)
    nrm = np.tile(np.array([[0.2, 0.3, 1]], np.float32), (3 * n, 1))
    sc = S.Scene()
    sc.add(S.TriMesh(v, nrm, idx, normalsI=idx, material=S.Material(diffuse=(0.3, 0.8, 0.5), shininess=12)))
    st = FrameState(width=w, height=h, projection=pj.projection_ortho(-w / 2, w / 2, -h / 2, h / 2, 1, 60),
                    light=np.array([0.3, 0.4, 1], np.float32))
    return st, sc


@pytest.mark.parametrize("case", ["big_triangles", "strips_past_the_record_store"])
def test_noalloc_large_triangles(product_lib, case):
    """Large sub-triangles take records from the fixed store and the
    row-parallel raster kernel; past the store's 32768 records the setup
    kernel rasterises them itself. Both equal the oracle and mr_render."""
    import edge_scenes as E
    st, sc = E.ALL["big_triangles"]() if case == "big_triangles" else _strips(40000, 1024, 768, 5)
    want = _existing(st, sc)
    ref = O.render(st, sc)
    assert (ref["ids"] != 0xFFFFFFFF).sum() > 10000
    for k, got in enumerate(_noalloc(st, sc)):
        _same(got, want, f"call {k} vs mr_render")
        _same(got, ref, f"call {k} vs the oracle")


def test_noalloc_bad_index_then_good_mesh(product_lib):
    """One out-of-range index (found by the index check, which reads only the
    caller's in-bounds index memory) gives MR_E_BAD_INDEX; the next call with
    a good mesh of the same triangle count returns MR_OK with the output of
    mr_render, so no stale index-check bit survives in the shared scratch."""
    st, sc = W.config1(160, 120)
    mesh = S.flatten(sc).meshes[0]
    bad = mesh.indices.copy()
    bad[7] = mesh.vertices.shape[0] + 11
    _noalloc(st, sc, calls=1, indices=bad, expect=abi.MR_E_BAD_INDEX)
    got = _noalloc(st, sc, calls=1)[0]
    _same(got, _existing(st, sc), "good mesh after a bad one")


def test_noalloc_empty_mesh_no_outputs(product_lib):
    """Zero triangles and no output buffers: nothing to draw, MR_OK."""
    import torch
    st, _ = W.config1(64, 48)
    frame = st.to_c()
    xf = (C.c_float * 16)(*np.eye(4, dtype=np.float32).reshape(16))
    rc = capi.lib().mr_render_noalloc(C.byref(frame), C.byref(abi.mr_mesh_desc()), C.addressof(xf),
                                      C.byref(abi.mr_material()), None, 0, 0, 0, None, None, None,
                                      torch.cuda.current_stream().cuda_stream)
    assert rc == abi.MR_OK, capi.lib().mr_status_string(rc)


def test_noalloc_rejects_oversized_requests(product_lib):
    """Sizes beyond the fixed scratch are refused before any device work (an
    empty mesh, so nothing could be dereferenced even if the check moved)."""
    st, _ = W.config1()
    mat = abi.mr_material()
    xf = (C.c_float * 16)(*np.eye(4, dtype=np.float32).reshape(16))
    for w, h in ((abi.MR_NOALLOC_MAX_SIDE + 1, 16), (2048, 2048)):
        st.width, st.height = w, h
        frame = st.to_c()
        rc = capi.lib().mr_render_noalloc(C.byref(frame), C.byref(abi.mr_mesh_desc()), C.addressof(xf),
                                          C.byref(mat), None, 0, 0, 0, None, None, None, None)
        assert rc == abi.MR_E_NOALLOC_LIMIT
    assert capi.lib().mr_status_string(abi.MR_E_NOALLOC_LIMIT).startswith(b"request exceeds")
