"""Device path vs the oracle on the benchmark configurations and edge cases
(bit-exact ids and depth, RGB8 within 1 LSB on >= 99.9% of pixels)."""
import numpy as np
import pytest

import edge_scenes as E
from parity import assert_parity, compare, gpu_render, report
from minirender_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu

@pytest.fixture(scope="module")
def renderer(product_lib):
    from minirender_gb300.renderer import Renderer
    r = Renderer(0)
    yield r
    r.close()


def _check(name, st, sc, renderer, **kw):
    ref = O.render(st, sc, normals=st.save_normals)
    gpu, _ = gpu_render(st, sc, renderer, **kw)
    stats = compare(gpu, ref, name)
    if st.save_normals:
        stats["normals_max_err"] = float(np.abs(gpu["normals"] - ref["normals"]).max())
    report(stats)
    assert_parity(stats)
    return stats


def test_config1(renderer):
    st, sc = W.config1()
    _check("config1", st, sc, renderer)


def test_config2_full(renderer):
    st, sc = W.config2()
    s = _check("config2", st, sc, renderer)
    assert s["covered"] > 500_000


def test_config3_scaled(renderer):
    st, sc = W.config3(n_tris=1_000_000, width=1920, height=1080)
    _check("config3_1M_1080p", st, sc, renderer)


@pytest.mark.parametrize("seed", range(48))
def test_random_scene(renderer, seed):
    """Seeded random scenes: soups (corner records) and indexed meshes
    (per-vertex pass), nested and instanced nodes, near-plane clipping,
    both projections, odd frame and texture sizes, every lighting switch."""
    st, sc = E.random_scene(seed)
    _check(f"random_{seed}", st, sc, renderer)


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_config4_scenes(renderer, seed):
    st, sc = W.config4_scene(seed)
    _check(f"config4_{seed}", st, sc, renderer)


@pytest.mark.parametrize("name", sorted(E.ALL))
def test_edge(renderer, name):
    st, sc = E.ALL[name]()
    _check(name, st, sc, renderer)


@pytest.mark.parametrize("tile,small", [(8, 0), (16, 4096), (32, 16), (16, 1)])
def test_tuning_variants_same_result(renderer, tile, small):
    """Tile size and the small-triangle limit change the work split, never
    the result."""
    st, sc = W.config2(level=6, width=640, height=360, tex_size=256)
    try:
        _check(f"tuning_{tile}_{small}", st, sc, renderer, tile=tile, small_max=small)
    finally:
        renderer.ctx.set_tuning(16, 64)


def test_deterministic(renderer):
    st, sc = W.config4_scene(7)
    a, _ = gpu_render(st, sc, renderer)
    b, _ = gpu_render(st, sc, renderer)
    for k in ("ids", "depth", "rgb8", "image"):
        assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), k


def test_shared_and_separate_index_arrays(renderer):
    """normalsI / texcoordsI passed as the indices array itself share its
    device copy; passed as equal but separate arrays they are copied: same
    pixels either way.  An update must keep the sharing of the upload."""
    from minirender_gb300 import capi
    from minirender_gb300.scene import Scene, TriMesh
    st, sc = W.config2(level=5, width=320, height=240, tex_size=64)
    m = sc.children[0]
    assert m.normalsI.ctypes.data == m.indices.ctypes.data == m.texcoordsI.ctypes.data
    sep = TriMesh(m.vertices, m.normals, m.indices, normalsI=m.indices.copy(), texcoords=m.texcoords,
                  texcoordsI=m.indices.copy(), material=m.material)
    sc2 = Scene()
    sc2.add(sep)
    a, _ = gpu_render(st, sc, renderer)
    b, _ = gpu_render(st, sc2, renderer)
    for k in ("ids", "depth", "rgb8"):
        assert np.array_equal(a[k].view(np.uint8), b[k].view(np.uint8)), k
    ctx = renderer.ctx
    h = ctx.upload_mesh(m.desc())
    try:
        with pytest.raises(capi.MRError):
            ctx.update_mesh(h, sep.desc())
        ctx.update_mesh(h, m.desc())
    finally:
        ctx.free_mesh(h)


@pytest.mark.parametrize("name", ["textured.obj", "plain.obj", "scene.x3d", "binary.stl", "ascii.stl"])
def test_loaded_models(renderer, tmp_path, name):
    """Models read by the library's loaders (OBJ with material library and
    texture, X3D with transforms and DEF/USE, binary and ASCII STL) render as
    the oracle renders the same scene."""
    import loader_files
    from minirender_gb300 import loaders
    from minirender_gb300 import projection as pj
    from minirender_gb300.frame import FrameState
    from minirender_gb300.scene import Scene
    loader_files.write_all(str(tmp_path))
    sc = Scene()
    sc.add(loaders.load_mesh(str(tmp_path / name)))
    st = FrameState(width=160, height=120,
                    projection=pj.projection_frustum(pj.deg2rad(50), np.float32(160) / np.float32(120), 0.5, 100),
                    view=pj.translate(0, 0, -6), light=np.array([0.3, 0.5, 1.0], np.float32),
                    ambient=sc.ambientLight)
    _check(f"loaded_{name}", st, sc, renderer)


def test_empty_frames(renderer):
    """A frame without renderables, and one whose only mesh is empty, render the
    background (depth 1e11, no triangle ids) as the reference does."""
    from minirender_gb300.scene import Scene, TriMesh
    st, _ = W.config1(64, 48)
    _check("empty_scene", st, Scene(), renderer)
    sc = Scene()
    sc.add(TriMesh(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), np.zeros(0, np.int32)))
    _check("empty_mesh", st, sc, renderer)


def _replay_paints(r, paints):
    """The paint records as Renderer calls: paintMesh (a mesh sharing the
    arrays but carrying the paint's material where they differ),
    setMaterial + paintTriangle per triangle of a triangle run, and setView
    for a ("view", m) item."""
    from minirender_gb300 import abi
    from minirender_gb300.scene import TriMesh, Vertex
    for p in paints:
        if isinstance(p, tuple):  # state calls between paints
            if p[0] == "view":
                r.setView(p[1])
            elif p[0] == "lighting":
                r.setLighting(p[1])
            elif p[0] == "texturing":
                r.setTexturing(p[1])
            elif p[0] == "light":
                r.setLight(p[1], p[2])
            elif p[0] == "background":
                r.setBackground(p[1])
            else:
                raise ValueError(p[0])
        elif p.flags & abi.MR_RS_MODELVIEW:
            r.setMaterial(p.material)
            m = p.mesh
            for t in range(m.indices.size // 3):
                v = [Vertex(m.vertices[3 * t + c], m.normals[3 * t + c], m.texcoords[3 * t + c]) for c in range(3)]
                r.paintTriangle(*v, world=not (p.flags & abi.MR_RS_NO_CLIP))
        else:
            mesh = p.mesh
            if mesh.material is not p.material:
                mesh = TriMesh(mesh.vertices, mesh.normals, mesh.indices, normalsI=mesh.normalsI,
                               texcoords=mesh.texcoords, texcoordsI=mesh.texcoordsI, material=p.material)
            r.paintMesh(mesh, p.transform)


@pytest.mark.parametrize("clear", [False, True])
def test_paint_mesh_and_triangles(renderer, clear):
    """Renderer.paintMesh / paintTriangle after render() (and after clear()):
    meshes, clipped and unclipped view-space triangles, exact ties -- the
    same pixels as the oracle's paint sequence (pinned to the reference's
    own paintMesh / paintTriangle)."""
    from minirender_gb300.scene import Scene
    st, paints = E.paint_sequence()
    renderer.state = st
    renderer.setScene(Scene())
    renderer.render()
    if clear:
        renderer.clear()
    _replay_paints(renderer, paints)
    gpu = {"image": renderer.getImage(), "depth": renderer.getDepth(), "ids": renderer.getTriangleIds(),
           "rgb8": renderer.getImageRGB8()}
    stats = compare(gpu, O.render_paints(st, paints), f"paints_clear{int(clear)}")
    report(stats)
    assert_parity(stats)
    assert stats["covered"] > 5000


@pytest.mark.parametrize("seed", range(32))
def test_random_paints(renderer, seed):
    """Seeded random paintMesh / paintTriangle sequences after render() and
    clear() (tests/edge_scenes.random_paints: new transforms and materials,
    RGB8 textures, clipped and unclipped view-space triangles, both
    projections), pinned to the reference's Renderer on the CPU: the mirror
    on GB300 equals the oracle."""
    import copy
    from minirender_gb300.scene import Scene
    st, paints = E.random_paints(seed)
    renderer.state = copy.deepcopy(st)
    empty = Scene()
    empty.ambientLight = st.ambient  # render() takes the scene's ambient, as the reference does
    renderer.setScene(empty)
    renderer.render()
    renderer.clear()
    _replay_paints(renderer, paints)
    gpu = {"image": renderer.getImage(), "depth": renderer.getDepth(), "ids": renderer.getTriangleIds(),
           "rgb8": renderer.getImageRGB8()}
    stats = compare(gpu, O.render_paints(st, paints), f"random_paints_{seed}")
    report(stats)
    assert_parity(stats)


def test_paint_after_view_change(renderer):
    """render() of a scene, paintMesh, setView, then more paintMesh and a
    paintTriangle run: the later meshes take the new view, the light stays
    where render() placed it (pinned to the reference's Renderer on the
    CPU)."""
    import copy
    st, calls, paints = E.view_change_paints(160, 120)
    _, sc = W.config1(160, 120)
    renderer.state = copy.deepcopy(st)  # setView below must not change the oracle's state
    renderer.setScene(sc)
    renderer.render()
    _replay_paints(renderer, calls)
    gpu = {"image": renderer.getImage(), "depth": renderer.getDepth(), "ids": renderer.getTriangleIds(),
           "rgb8": renderer.getImageRGB8()}
    stats = compare(gpu, O.render_paints(st, paints, base_scene=sc), "paints_view_change")
    report(stats)
    assert_parity(stats)
    assert stats["covered"] > 5000


def test_paint_after_state_changes(renderer):
    """setLighting / setTexturing / setLight / setBackground between paints
    after render(): each paint shades with the switches of its call, the
    light stays where render() placed it, the background is render()'s
    (pinned to the reference's Renderer on the CPU)."""
    import copy
    st, calls, paints = E.state_change_paints(160, 120)
    _, sc = W.config1(160, 120)
    renderer.state = copy.deepcopy(st)
    renderer.setScene(sc)
    renderer.render()
    _replay_paints(renderer, calls)
    gpu = {"image": renderer.getImage(), "depth": renderer.getDepth(), "ids": renderer.getTriangleIds(),
           "rgb8": renderer.getImageRGB8()}
    stats = compare(gpu, O.render_paints(st, paints, base_scene=sc), "paints_state_changes")
    report(stats)
    assert_parity(stats)
    assert stats["covered"] > 5000


def test_resident_meshes_follow_the_frame(renderer):
    """The mirror's caches hold the meshes and textures of the frame last
    drawn: switching scenes frees the old scene's meshes, and drawing it
    again re-sends them (the frames equal the oracle's each time)."""
    st_a, sc_a = E.random_scene(3)
    st_b, sc_b = W.config2(level=3, width=96, height=64, tex_size=16)
    from minirender_gb300 import scene as S
    for st, sc in ((st_a, sc_a), (st_b, sc_b), (st_a, sc_a)):
        renderer.state = st
        renderer.setScene(sc)
        renderer.render()
        flat = S.flatten(sc)
        assert set(renderer._meshes) == {S.geometry_key(m) for m in flat.meshes}
        assert len(renderer._textures) == len(flat.textures)
        gpu = {"image": renderer.getImage(), "depth": renderer.getDepth(), "ids": renderer.getTriangleIds(),
               "rgb8": renderer.getImageRGB8()}
        assert_parity(compare(gpu, O.render(st, sc), "resident_follow"))


def test_paint_over_rendered_scene(renderer):
    """render() of a scene, then paintTriangle runs over it: the scene's
    renderables come first in draw order."""
    st, sc = W.config1(160, 120)
    _, paints = E.paint_sequence(160, 120)
    tri_runs = [p for p in paints if p.flags]
    renderer.state = st
    renderer.setScene(sc)
    renderer.render()
    _replay_paints(renderer, tri_runs)
    gpu = {"image": renderer.getImage(), "depth": renderer.getDepth(), "ids": renderer.getTriangleIds(),
           "rgb8": renderer.getImageRGB8()}
    stats = compare(gpu, O.render_paints(st, tri_runs, base_scene=sc), "paints_over_scene")
    report(stats)
    assert_parity(stats)


def test_unknown_renderable_flags_rejected(renderer):
    from minirender_gb300 import capi
    from minirender_gb300.scene import Scene
    st, sc = W.config1(64, 48)
    renderer.state = st
    renderer.setScene(sc)
    frame, rs, n = renderer.prepare()
    from minirender_gb300 import abi
    rs[0].flags = abi.MR_RS_POINT_LIGHT << 1  # the first bit no flag uses
    with pytest.raises(capi.MRError):
        renderer.ctx.render(frame, rs, n, renderer.outputs)
    rs[0].flags = 0
    renderer.ctx.render(frame, rs, n, renderer.outputs)
    renderer.setScene(Scene())


def _range_cases():
    """getRangeImage cases: a perspective frame whose far plane (3.5) cuts
    through the visible sphere, so part of the covered pixels lie past
    `fardepth` and read as zero; an orthographic frame with depth below zero;
    and random scenes of both projections."""
    from minirender_gb300 import projection as pj
    st, sc = W.config1(160, 120)
    st.projection = pj.projection_frustum(pj.deg2rad(45), np.float32(160) / np.float32(120), 0.1, 3.5)
    yield "persp_far_cut", st, sc
    yield "ortho_negative_z", *E.ALL["ortho_negative_z"]()
    for seed in (1, 6, 11, 30):
        yield f"random_{seed}", *E.random_scene(seed)


@pytest.mark.parametrize("case", list(_range_cases()), ids=lambda c: c[0])
def test_range_image(renderer, case):
    """Renderer::getRangeImage (src/Renderer.cpp:388-415) on the device
    (mr_read_range_image) equals the oracle's bit for bit.  Another frame with
    a different projection and size is rendered on the same context first,
    so the range pass must read the last frame's projection, not a stale
    staged one."""
    name, st, sc = case
    other_st, other_sc = W.config2(level=4, width=200, height=150, tex_size=32)
    gpu_render(other_st, other_sc, renderer)
    gpu, r = gpu_render(st, sc, renderer)
    got = r.getRangeImage()
    ref = O.render(st, sc)
    assert np.array_equal(gpu["depth"].view(np.uint32), ref["depth"].view(np.uint32))
    want = O.range_image(st, ref["depth"])
    assert got.shape == want.shape
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), name
    if name == "persp_far_cut":
        covered = ref["ids"] != 0xFFFFFFFF
        zeroed = covered & np.all(want == 0, axis=-1)
        assert zeroed.sum() > 100 and (covered & ~zeroed).sum() > 100
