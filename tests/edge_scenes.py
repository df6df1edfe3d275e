"""Hand-built scenes for the edge cases of the reference rasteriser
(src/Renderer.cpp:121-309): exact depth ties, shared edges, the three
clipTriangle cases and its |dz| < 1e-6 branch, degenerate and off-screen
triangles, texture wrap-around, orthographic depth below zero, large
triangles spanning many tiles, lighting variants."""
import numpy as np

from minirender_gb300 import abi
from minirender_gb300 import projection as pj
from minirender_gb300.frame import FrameState
from minirender_gb300.scene import Material, Scene, SceneNode, TriMesh

f32 = np.float32


def _tri_mesh(verts, tris, normals=None, uvs=None, material=None):
    verts = np.asarray(verts, np.float32).reshape(-1, 3)
    tris = np.asarray(tris, np.int32).reshape(-1)
    if normals is None:
        normals = np.tile(np.array([[0, 0, 1]], np.float32), (verts.shape[0], 1))
    kw = {}
    if uvs is not None:
        kw = dict(texcoords=np.asarray(uvs, np.float32), texcoordsI=tris)
    return TriMesh(verts, normals, tris, normalsI=tris, material=material, **kw)


def _persp(w, h, near=0.5, far=100.0, fov=60):
    return pj.projection_frustum(pj.deg2rad(fov), f32(w) / f32(h), near, far)


def ties(w=96, h=64):
    """Two coplanar copies of a quad with different colours in one mesh and a
    third copy in a later renderable: the first drawn must win every tie."""
    v = [[-1, -1, -3], [1, -1, -3], [1, 1, -3], [-1, 1, -3]]
    quad = [0, 1, 2, 0, 2, 3]
    sc = Scene()
    m1 = _tri_mesh(v, quad + quad, material=Material(diffuse=(1, 0, 0)))
    m2 = _tri_mesh(v, quad, material=Material(diffuse=(0, 0, 1)))
    sc.add(m1)
    sc.add(m2)
    st = FrameState(width=w, height=h, projection=_persp(w, h), light=np.array([0, 0, 1], np.float32))
    return st, sc


def shared_edges(w=97, h=71):
    """A fan of thin triangles sharing edges and a vertex at a pixel centre."""
    n = 24
    ang = np.linspace(0, 2 * np.pi, n, endpoint=False)
    v = [[0, 0, -4]] + [[1.7 * np.cos(a), 1.7 * np.sin(a), -4] for a in ang]
    tris = []
    for i in range(n):
        tris += [0, 1 + i, 1 + (i + 1) % n]
    sc = Scene()
    sc.add(_tri_mesh(v, tris, material=Material(diffuse=(0.2, 0.9, 0.4), shininess=0)))
    st = FrameState(width=w, height=h, projection=_persp(w, h), light=np.array([0.3, 0.2, 1], np.float32))
    return st, sc


def near_clip(w=128, h=96):
    """Triangles crossing the near plane (z = -0.5) in all three
    configurations, in every vertex rotation, plus one whose crossing edge
    has |dz| < 1e-6 (clip() then uses k = 0.5)."""
    zn = -0.5
    tris_v = []
    for rot in range(3):
        for pattern in ([1, 1, 0], [1, 0, 1], [0, 1, 1], [1, 0, 0], [0, 1, 0], [0, 0, 1]):
            pts = []
            for c, inside in enumerate(pattern):
                ang = 2 * np.pi * c / 3 + rot * 0.7
                z = zn + 0.3 if inside else zn - 1.5 - 0.2 * c
                pts.append([0.8 * np.cos(ang) + 0.9 * (rot - 1), 0.8 * np.sin(ang), z])
            tris_v.append(pts)
    # |dz| < 1e-6 across the plane
    tris_v.append([[-0.2, -0.6, zn + 4e-7], [0.2, -0.6, zn - 4e-7], [0.0, -0.2, zn - 2.0]])
    verts = np.array(tris_v, np.float32).reshape(-1, 3)
    tris = np.arange(verts.shape[0], dtype=np.int32)
    # keep only front-facing windings so something is drawn; flip the others
    t = tris.reshape(-1, 3).copy()
    sc = Scene()
    both = np.concatenate([t, t[:, [0, 2, 1]]]).reshape(-1)
    uvs = np.random.default_rng(5).uniform(0, 1, (verts.shape[0], 2)).astype(np.float32)
    tex = np.random.default_rng(6).integers(0, 256, (16, 16, 3)).astype(np.uint8)
    nrm = np.random.default_rng(7).normal(size=(verts.shape[0], 3)).astype(np.float32)
    m = TriMesh(verts, nrm, both, normalsI=both, texcoords=uvs, texcoordsI=both,
                material=Material(texture=tex, shininess=20))
    sc.add(m)
    st = FrameState(width=w, height=h, projection=_persp(w, h, near=0.5, fov=90),
                    light=np.array([0.2, 0.5, 1], np.float32), light_is_point=True)
    return st, sc


def degenerate_offscreen(w=80, h=60):
    """Collinear (a == 0) and zero-area triangles, triangles entirely and
    partly off screen, one covering the whole screen."""
    v = [[0, 0, -3], [1, 1, -3], [2, 2, -3],            # collinear
         [0.5, 0.5, -3], [0.5, 0.5, -3], [0.6, 0.4, -3],  # repeated vertex
         [40, 40, -3], [41, 40, -3], [40, 41, -3],       # off screen
         [-2.5, -0.3, -2], [-0.9, -0.5, -2], [-2.0, 0.9, -2],  # partly off screen (left)
         [-30, -30, -9], [30, -30, -9], [0, 40, -9]]     # full screen, far
    tris = list(range(15))
    sc = Scene()
    sc.add(_tri_mesh(v, tris, material=Material(diffuse=(0.9, 0.8, 0.1), emissive=(0.05, 0, 0))))
    st = FrameState(width=w, height=h, projection=_persp(w, h),
                    background=np.array([0.1, 0.2, 0.3], np.float32))
    return st, sc


def texture_wrap(w=64, h=64):
    """UVs well outside [0,1]: fract() wraps the texel lookup; float texture."""
    v = [[-1, -1, -2.5], [1, -1, -2.5], [1, 1, -2.5], [-1, 1, -2.5]]
    uvs = [[0.25, 0.25], [3.75, 0.25], [3.75, 2.6], [0.25, 2.6]]
    tex = np.random.default_rng(11).uniform(0, 1, (7, 5, 3)).astype(np.float32)
    sc = Scene()
    sc.add(_tri_mesh(v, [0, 1, 2, 0, 2, 3], uvs=uvs, material=Material(texture=tex, shininess=0)))
    st = FrameState(width=w, height=h, projection=_persp(w, h))
    return st, sc


def ortho_negative_z(w=90, h=70):
    """Orthographic projection (P(3,3) = 1): depth is NDC z, part of it < 0,
    two interpenetrating triangles, lighting off (emissive only)."""
    v = [[-3, -2, -60], [3, -2, -90], [0, 3, -70],
         [-3, 2, -95], [3, 2, -55], [0, -3, -75]]
    sc = Scene()
    sc.add(_tri_mesh(v, [0, 1, 2], material=Material(emissive=(0.9, 0.1, 0.2))))
    sc.add(_tri_mesh(v, [3, 5, 4], material=Material(emissive=(0.1, 0.9, 0.2))))
    st = FrameState(width=w, height=h, projection=pj.projection_ortho(-4, 4, -3, 3, 50, 120),
                    lighting=False)
    return st, sc


def big_triangles(w=300, h=200):
    """Large overlapping triangles spanning many screen tiles (binned path),
    interleaved with tiny ones (direct path)."""
    rng = np.random.default_rng(21)
    verts, tris = [], []
    for k in range(12):
        c = rng.uniform(-1.5, 1.5, 2)
        r = rng.uniform(0.8, 3.0)
        z = -rng.uniform(2.5, 6.0)
        a0 = rng.uniform(0, 2 * np.pi)
        base = len(verts)
        for j in range(3):
            a = a0 - 2 * np.pi * j / 3
            verts.append([c[0] + r * np.cos(a), c[1] + r * np.sin(a), z + rng.uniform(-0.5, 0.5)])
        tris += [base, base + 2, base + 1]
        for _ in range(20):
            p = rng.uniform(-2, 2, 2)
            zz = -rng.uniform(2.5, 6.0)
            base = len(verts)
            s = 0.02
            verts += [[p[0], p[1], zz], [p[0], p[1] + s, zz], [p[0] + s, p[1], zz]]
            tris += [base, base + 2, base + 1]
    nrm = rng.normal(size=(len(verts), 3)).astype(np.float32)
    sc = Scene()
    sc.add(TriMesh(np.array(verts, np.float32), nrm, np.array(tris, np.int32),
                   material=Material(diffuse=(0.6, 0.6, 0.7), shininess=40)))
    st = FrameState(width=w, height=h, projection=_persp(w, h, near=1.0),
                    light=np.array([1, 2, 2], np.float32), light_is_point=True, save_normals=True)
    return st, sc


def tall_layers(w=8, h=16384, layers=800):
    """Hundreds of layered triangles covering a tall frame: their 32-row
    blocks outnumber the context's first row-block list, so most records are
    rasterised through the spill list."""
    rng = np.random.default_rng(4)
    verts, tris = [], []
    for k in range(layers):
        z = -rng.uniform(30.0, 60.0)
        base = len(verts)
        dx = rng.uniform(-0.5, 0.5)
        hw, top = rng.uniform(0.8, 3.0), rng.uniform(0.7, 6.0)
        # tilted along y, and edges crossing the strip, so the nearest layer
        # changes from row to row
        verts += [[-hw + dx, -3, z], [dx, top, z + rng.uniform(-25, 25)], [hw + dx, -3, z]]
        tris += [base, base + 2, base + 1]  # clockwise on screen: front-facing
    nrm = rng.normal(size=(len(verts), 3)).astype(np.float32)
    sc = Scene()
    sc.add(TriMesh(np.array(verts, np.float32), nrm, np.array(tris, np.int32),
                   material=Material(diffuse=(0.3, 0.7, 0.5), shininess=8)))
    st = FrameState(width=w, height=h, projection=pj.projection_ortho(-1, 1, -1, 1, 1.0, 100.0),
                    light=np.array([0.2, 0.4, 1], np.float32))
    return st, sc


ALL = {
    "ties": ties,
    "shared_edges": shared_edges,
    "near_clip": near_clip,
    "degenerate_offscreen": degenerate_offscreen,
    "texture_wrap": texture_wrap,
    "ortho_negative_z": ortho_negative_z,
    "big_triangles": big_triangles,
}


def paint_sequence(w=160, h=120):
    """render() then paintMesh / paintTriangle calls (src/Renderer.cpp:
    163-381): two meshes (one textured), a run of view-space triangles with
    near-plane clipping (one crossing the near plane, one wholly behind it),
    a run without clipping (world=false, one crossing), and the first mesh
    painted again at the same place (exact ties: the earlier paint wins).
    Returns (state, paints) as scene.Paint records."""
    from minirender_gb300 import workloads as W
    from minirender_gb300.scene import Paint, Vertex, append_triangle, triangle_paint
    rng = np.random.default_rng(17)
    _, s1 = W.config1(64, 48)
    sphere = s1.children[0]
    sphere.material = Material(diffuse=(0.8, 0.5, 0.3), shininess=32)
    tex = rng.integers(0, 256, (16, 16, 3)).astype(np.uint8)
    quad = _tri_mesh([[-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0]], [0, 1, 2, 0, 2, 3],
                     uvs=[[0, 0], [2, 0], [2, 2], [0, 2]], material=Material(diffuse=(1, 1, 1), texture=tex))
    st = FrameState(width=w, height=h, projection=_persp(w, h, near=0.5), view=pj.translate(0.2, -0.1, -4),
                    light=np.array([2, 3, 4], np.float32), light_is_point=True)
    t1 = pj.mat_mul(pj.translate(-0.6, 0, 0), pj.scale(0.8))
    t2 = pj.mat_mul(pj.translate(0.7, 0.2, -0.5), pj.rotate_y(0.6))
    paints = [Paint(sphere, t1, sphere.material), Paint(quad, t2, quad.material)]
    m3 = Material(diffuse=(0.2, 0.9, 0.4), specular=(0.5, 0.5, 0.5), shininess=8, texture=tex)
    # (vertex order clockwise on screen: front-facing)
    tri = [Vertex((-1.5, -1.0, -3.0), (0, 0, 1), (0.1, 0.1)), Vertex((0.3, -0.8, -3.5), (0, 0.3, 1), (0.5, 0.8)),
           Vertex((-0.5, 1.2, -2.5), (0.2, 0, 1), (0.9, 0.2))]
    p = triangle_paint(*tri, m3, True)
    append_triangle(p, Vertex((0.5, -0.5, -2.0), (0, 0, 1)), Vertex((1.5, -0.9, -2.2), (0, 0, 1)),
                    Vertex((1.2, 0.6, -0.3), (0, 0, 1)))  # crosses the near plane (z = -0.5)
    append_triangle(p, Vertex((0, 0, -0.2)), Vertex((0, 0.1, -0.1)), Vertex((0.1, 0, -0.3)))  # behind it
    paints.append(p)
    q = triangle_paint(Vertex((-1.2, 0.4, -2.8), (0, 0, 1), (0.3, 0.3)), Vertex((-0.9, -0.3, -3.1)),
                       Vertex((-0.2, 0.9, -2.9)), m3, False)
    # crosses the near plane, drawn unclipped
    append_triangle(q, Vertex((-0.3, -0.3, -1.2)), Vertex((0.1, -0.35, -1.0)), Vertex((-0.1, -0.1, -0.45)))
    paints.append(q)
    paints.append(Paint(sphere, t1, Material(diffuse=(0.1, 0.1, 0.9))))
    return st, paints


def view_change_paints(w=160, h=120):
    """paintMesh before and after setView, with a paintTriangle run between
    (src/Renderer.cpp:163-381: paintMesh takes the view current at the call,
    the light stays where render() placed it, view-space triangles ignore
    the view).  Returns (state, calls, paints): `calls` as the reference
    receives them (scene.Paint records and ("view", m) items), `paints` the
    same frame as one paint list -- the paints after the view change carry
    their modelview (view x transform, MR_RS_MODELVIEW)."""
    from minirender_gb300.scene import Paint
    st, seq = paint_sequence(w, h)
    sphere_paint, quad_paint, run = seq[0], seq[1], seq[2]
    v2 = pj.mat_mul(pj.translate(-0.4, 0.3, -4.5), pj.rotate_y(0.5))
    t3 = pj.mat_mul(pj.translate(0.9, -0.5, 0.3), pj.scale(0.5))
    last = Paint(sphere_paint.mesh, t3, Material(diffuse=(0.9, 0.2, 0.2), specular=(1, 1, 1), shininess=16))
    calls = [sphere_paint, ("view", v2), quad_paint, run, last]
    paints = [sphere_paint,
              Paint(quad_paint.mesh, pj.mat_mul(v2, quad_paint.transform), quad_paint.material, abi.MR_RS_MODELVIEW),
              run,
              Paint(last.mesh, pj.mat_mul(v2, last.transform), last.material, abi.MR_RS_MODELVIEW)]
    return st, calls, paints


def state_change_paints(w=160, h=120):
    """Paints between setLighting / setTexturing / setLight / setBackground
    calls (src/Renderer.cpp:163-381: paintTriangle reads the lighting,
    texturing and light-type switches at the call; the light's position is
    the one render() computed; the background is filled by clear()).
    Returns (state, calls, paints) as view_change_paints does: in `paints`
    a paint whose switches differ from the frame's carries MR_RS_OWN_STATE
    and its own switches."""
    from minirender_gb300.scene import Paint
    st, seq = paint_sequence(w, h)
    sphere_paint, quad_paint, run, again = seq[0], seq[1], seq[2], seq[4]
    t3 = pj.mat_mul(pj.translate(0.9, -0.5, 0.3), pj.scale(0.5))
    last = Paint(sphere_paint.mesh, t3, Material(diffuse=(0.9, 0.2, 0.2), specular=(1, 1, 1), shininess=16))
    own, lit, tex, point = abi.MR_RS_OWN_STATE, abi.MR_RS_LIGHTING, abi.MR_RS_TEXTURING, abi.MR_RS_POINT_LIGHT
    calls = [sphere_paint,
             ("lighting", False), quad_paint,                      # unlit, textured
             ("texturing", False), ("lighting", True), run,        # lit, untextured
             ("light", (-1.0, 2.0, 3.0), False), last,             # render()'s light used as a direction
             ("background", (0.5, 0.5, 0.5)),                      # after clear(): no effect
             ("texturing", True), ("light", (2.0, 3.0, 4.0), True), again]  # the frame's switches again
    paints = [sphere_paint,
              Paint(quad_paint.mesh, quad_paint.transform, quad_paint.material, own | tex | point),
              Paint(run.mesh, run.transform, run.material, run.flags | own | lit | point),
              Paint(last.mesh, last.transform, last.material, own | lit),
              again]
    return st, calls, paints


def random_scene(seed: int):
    """Seeded random scene for fuzzing the whole path: 1-4 meshes of 10-250
    triangles, each either a soup (every corner its own vertex) or indexed
    into a small shared vertex pool (3T >= 2V), with separate normal and
    texcoord index arrays; random windings (about half are culled), tiny,
    medium and screen-sized triangles, some crossing the near plane; meshes
    nested under transformed group nodes and under each other, one
    instanced twice; perspective or orthographic camera with a rotated and
    shifted view; materials with u8 or f32 textures of odd sizes and UVs up
    to 4, or none; directional or point light; lighting, texturing and the
    normals output switched at random; odd frame sizes."""
    rng = np.random.default_rng(9000 + seed)
    w = int(rng.integers(17, 180))
    h = int(rng.integers(13, 140))
    persp = rng.random() < 0.7
    if persp:
        near = float(rng.uniform(0.3, 1.5))
        proj = _persp(w, h, near=near, far=float(rng.uniform(30, 200)), fov=float(rng.uniform(35, 100)))
        zlo, zhi = -12.0, -0.1
    else:
        near = 0.5
        proj = pj.projection_ortho(-4, 4, -3, 3, near, 50.0)
        zlo, zhi = -45.0, -0.1

    def place(n):
        z = rng.uniform(zlo, zhi, n)
        spread = np.abs(z) * 0.7 if persp else np.full(n, 3.5)
        xy = rng.uniform(-1, 1, (n, 2)) * spread[:, None]
        return np.column_stack([xy, z])

    def make_mesh(n_tri):
        size_class = rng.choice(3, n_tri, p=[0.6, 0.3, 0.1])
        scale = np.array([0.02, 0.3, 3.0])[size_class]
        if rng.random() < 0.5:  # soup
            c = place(n_tri)
            verts = (c[:, None, :] + rng.normal(size=(n_tri, 3, 3)) * scale[:, None, None] *
                     np.array([1, 1, 0.6])).reshape(-1, 3)
            idx = np.arange(3 * n_tri, dtype=np.int32).reshape(-1, 3)
        else:  # indexed: 3T >= 2V
            n_v = max(3, int(1.5 * n_tri) // 2 + 1)
            verts = place(n_v)
            idx = np.empty((n_tri, 3), np.int32)
            for t in range(n_tri):
                a = int(rng.integers(n_v))
                # near neighbours in a sorted pool keep most triangles moderate
                nb = np.clip(a + rng.integers(-6, 7, 2), 0, n_v - 1)
                idx[t] = [a, nb[0], nb[1]]
            order = np.argsort(verts[:, 0] + 7 * verts[:, 1])
            verts = verts[order]
        if rng.random() < 0.1 and n_tri > 2:
            idx[1, 2] = idx[1, 0]  # a repeated corner: zero area
        n_n = int(rng.integers(1, 2 * n_tri + 2))
        normals = rng.normal(size=(n_n, 3)) * rng.uniform(0.2, 3.0)
        normals[np.abs(normals).sum(1) < 1e-3] = (0, 0, 1)
        nidx = rng.integers(0, n_n, (n_tri, 3)).astype(np.int32)
        kw = {}
        if rng.random() < 0.6:
            n_uv = int(rng.integers(1, 3 * n_tri + 1))
            kw = dict(texcoords=rng.uniform(0.01, 4.0, (n_uv, 2)).astype(np.float32),
                      texcoordsI=rng.integers(0, n_uv, 3 * n_tri).astype(np.int32))
        mat = None
        if rng.random() < 0.85:
            tex = None
            if rng.random() < 0.6:
                rows, cols = int(rng.integers(1, 40)), int(rng.integers(1, 40))
                if rng.random() < 0.5:
                    tex = rng.integers(0, 256, (rows, cols, 3)).astype(np.uint8)
                else:
                    tex = rng.uniform(0, 1, (rows, cols, 3)).astype(np.float32)
            shin = 0.0 if rng.random() < 0.2 else float(rng.uniform(1, 64))
            mat = Material(diffuse=rng.uniform(0, 1, 3), specular=rng.uniform(0, 1, 3),
                           emissive=rng.uniform(0, 0.3, 3) * (rng.random() < 0.3), shininess=shin, texture=tex)
        flip = rng.random(n_tri) < 0.5
        idx[flip] = idx[flip][:, [0, 2, 1]]
        nidx[flip] = nidx[flip][:, [0, 2, 1]]
        if "texcoordsI" in kw:
            ti = kw["texcoordsI"].reshape(-1, 3)
            ti[flip] = ti[flip][:, [0, 2, 1]]
        return TriMesh(np.asarray(verts, np.float32), np.asarray(normals, np.float32), idx.reshape(-1),
                       normalsI=nidx.reshape(-1), material=mat, **kw)

    def jitter():
        t = pj.mat_mul(pj.translate(*rng.uniform(-0.3, 0.3, 3)), pj.rotate_z(float(rng.uniform(-0.5, 0.5))))
        return pj.mat_mul(t, pj.scale(float(rng.uniform(0.8, 1.2))))

    sc = Scene()
    meshes = [make_mesh(int(rng.integers(10, 250))) for _ in range(int(rng.integers(1, 5)))]
    for k, m in enumerate(meshes):
        where = rng.integers(3)
        m.transform = jitter()
        if where == 0 or k == 0:
            sc.add(m)
        elif where == 1:
            g = SceneNode(jitter())
            sc.add(g)
            g.add(m)
        else:
            meshes[0].add(m)  # a mesh under a mesh: both transforms apply
    if len(meshes) > 1 and rng.random() < 0.5:  # the last mesh drawn again elsewhere
        g = SceneNode(jitter())
        sc.add(g)
        g.add(meshes[-1] if not meshes[-1].children else meshes[0])
    view = pj.mat_mul(pj.translate(*rng.uniform(-0.3, 0.3, 2), float(rng.uniform(-0.05, 0.05))),
                      pj.rotate_z(float(rng.uniform(-np.pi, np.pi))))
    point = rng.random() < 0.4
    light = (rng.uniform(-3, 3, 3) if point else rng.normal(size=3)).astype(np.float32)
    st = FrameState(width=w, height=h, projection=proj, view=view, light=light, light_is_point=point,
                    ambient=float(rng.uniform(0, 0.3)), background=rng.uniform(0, 1, 3).astype(np.float32),
                    lighting=rng.random() < 0.85, texturing=rng.random() < 0.8,
                    save_normals=rng.random() < 0.3)
    sc.ambientLight = np.float32(st.ambient)  # Renderer::render reads the scene's (src/Renderer.cpp:322)
    return st, sc


def random_paints(seed: int):
    """Seeded random paintMesh / paintTriangle sequence over a random scene's
    camera: meshes of that scene painted with new transforms and materials
    (textured or not), runs of view-space triangles with near-plane clipping
    (world = true) and without (world = false), some crossing the near plane
    or lying behind it, random windings.  Returns (state, paints)."""
    from minirender_gb300.scene import Paint, Vertex, append_triangle, triangle_paint
    st, sc = random_scene(seed)
    rng = np.random.default_rng(5000 + seed)
    meshes = []
    stack = [sc]
    while stack:
        n = stack.pop()
        if isinstance(n, TriMesh):
            meshes.append(n)
        stack.extend(n.children)
    P = np.asarray(st.projection, np.float32).reshape(4, 4)
    persp = P[3, 3] == 0
    zlo = -10.0 if persp else -40.0

    def material():
        tex = rng.integers(0, 256, (int(rng.integers(1, 20)), int(rng.integers(1, 20)), 3)).astype(np.uint8) \
            if rng.random() < 0.4 else None
        return Material(diffuse=rng.uniform(0, 1, 3), specular=rng.uniform(0, 1, 3),
                        emissive=rng.uniform(0, 0.2, 3), shininess=float(rng.uniform(0, 50)), texture=tex)

    def vertex():
        z = float(rng.uniform(zlo, 0.3))
        s = abs(z) * 0.6 if persp else 3.5
        return Vertex((rng.uniform(-s, s), rng.uniform(-s, s), z), rng.normal(size=3), rng.uniform(0, 3, 2))

    paints = []
    for _ in range(int(rng.integers(1, 7))):
        if meshes and rng.random() < 0.5:
            m = meshes[int(rng.integers(len(meshes)))]
            xf = pj.mat_mul(pj.translate(*rng.uniform(-0.5, 0.5, 3)), pj.rotate_z(float(rng.uniform(-1, 1))))
            paints.append(Paint(m, xf, material() if rng.random() < 0.7 else (m.material or Material())))
        else:
            p = triangle_paint(vertex(), vertex(), vertex(), material(), bool(rng.random() < 0.6))
            for _ in range(int(rng.integers(0, 12))):
                append_triangle(p, vertex(), vertex(), vertex())
            paints.append(p)
    return st, paints
