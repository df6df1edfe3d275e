"""ORACLE -- test infrastructure only: ctypes wrappers around

* ``_build/libmr_oracle.so``: the C restatement in mr_oracle.c, and
* ``_ref/libmr_ref.so``: the reference's own Renderer/Scene/primitives
  compiled against the ASL stand-in (present only where the reference
  sources were available at build time).

Only tests, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module; the product path never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

from minirender_gb300 import abi
from minirender_gb300 import scene as sc
from minirender_gb300.frame import FrameState

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libmr_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libmr_ref.so")
# the reference checkout the pin build reads in place (MR_REFERENCE_SRC overrides)
REF_SRC = os.environ.get("MR_REFERENCE_SRC", "/root/reference")

_lib = None
_ref = None


class _Tex(C.Structure):
    _fields_ = [("rgb", C.c_void_p), ("rows", C.c_int32), ("cols", C.c_int32)]


def build(with_ref: bool = True) -> None:
    """Compile the restatement (always) and the reference build (when the
    reference sources are present)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    if with_ref and os.path.isdir(os.path.join(REF_SRC, "src")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + REF_SRC], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(with_ref=False)
        L = C.CDLL(ORACLE_SO)
        L.mro_collect_shapes.restype = C.c_int
        L.mro_collect_shapes.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                         C.POINTER(C.c_int32)]
        L.mro_render.restype = C.c_int
        L.mro_render.argtypes = [C.POINTER(abi.mr_frame), C.c_void_p, C.c_int32, C.c_void_p,
                                 C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_void_p]
        L.mro_quantize_rgb8.argtypes = [C.c_void_p, C.c_int64, C.c_void_p]
        L.mro_decode_rgb8.argtypes = [C.c_void_p, C.c_int64, C.c_void_p]
        L.mro_range_image.argtypes = [C.POINTER(abi.mr_frame), C.c_void_p, C.c_void_p]
        for n in ("mro_mat4_mul",):
            getattr(L, n).argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.mro_mat4_inverse.argtypes = [C.c_void_p, C.c_void_p]
        L.mro_projection_frustum.argtypes = [C.c_float] * 4 + [C.c_void_p]
        L.mro_render_frames_mt.restype = C.c_double
        L.mro_render_frames_mt.argtypes = [C.POINTER(abi.mr_frame), C.c_void_p, C.c_int32,
                                           C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                           C.c_int32, C.c_int32]
        _lib = L
    return _lib


def ref_lib() -> Optional[C.CDLL]:
    """The reference build, or None where it cannot exist."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            if not os.path.isdir(os.path.join(REF_SRC, "src")):
                return None
            build(with_ref=True)
        L = C.CDLL(REF_SO)
        L.ref_render.restype = C.c_int
        L.ref_render.argtypes = [C.POINTER(abi.mr_frame), C.c_void_p, C.c_int32, C.c_void_p,
                                 C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_void_p]
        L.ref_primitive.restype = C.c_int
        L.ref_primitive.argtypes = [C.c_int, C.c_float, C.c_float, C.c_int, C.c_int, C.c_int,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p]
        L.ref_projection.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
        L.ref_mat4_mul.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_mat4_inverse.argtypes = [C.c_void_p, C.c_void_p]
        L.ref_model_load.restype = C.c_void_p
        L.ref_model_load.argtypes = [C.c_char_p]
        L.ref_model_counts.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_model_nodes.argtypes = [C.c_void_p, C.c_void_p]
        L.ref_model_mesh.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 7
        L.ref_model_texture.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_model_free.argtypes = [C.c_void_p]
        L.ref_ppm_load.restype = C.c_int
        L.ref_ppm_load.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_ppm_save.argtypes = [C.c_char_p, C.c_void_p, C.c_int32, C.c_int32]
        L.ref_stl_save.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p]
        L.ref_xyz_save.argtypes = [C.c_char_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p]
        L.ref_paint.restype = C.c_int
        L.ref_paint.argtypes = [C.POINTER(abi.mr_frame), C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_int,
                                C.c_int32] + [C.c_void_p] * 8
        _ref = L
    return _ref


def ref_load_mesh(path: str):
    """The reference's loadMesh(path), flattened: {"nodes": mr_node array in
    pre-order, "meshes": [dict of arrays], "textures": [(rows, cols, 3) float32]}
    or None when it returns NULL."""
    L = ref_lib()
    h = L.ref_model_load(path.encode())
    if not h:
        return None
    try:
        nn, nm, nt = C.c_int32(), C.c_int32(), C.c_int32()
        L.ref_model_counts(h, C.byref(nn), C.byref(nm), C.byref(nt))
        nodes = (abi.mr_node * max(1, nn.value))()
        L.ref_model_nodes(h, nodes)
        meshes = []
        for i in range(nm.value):
            cnt = np.zeros(6, np.int32)
            L.ref_model_mesh(h, i, _ptr(cnt), None, None, None, None, None, None)
            m = {"vertices": np.zeros((cnt[0], 3), np.float32), "normals": np.zeros((cnt[1], 3), np.float32),
                 "texcoords": np.zeros((cnt[2], 2), np.float32), "indices": np.zeros(cnt[3], np.int32),
                 "normalsI": np.zeros(cnt[4], np.int32), "texcoordsI": np.zeros(cnt[5], np.int32)}
            L.ref_model_mesh(h, i, _ptr(cnt), *[_ptr(m[k]) for k in ("vertices", "normals", "texcoords", "indices",
                                                                      "normalsI", "texcoordsI")])
            meshes.append(m)
        textures = []
        for i in range(nt.value):
            r, c = C.c_int32(), C.c_int32()
            L.ref_model_texture(h, i, C.byref(r), C.byref(c), None)
            t = np.zeros((r.value, c.value, 3), np.float32)
            L.ref_model_texture(h, i, C.byref(r), C.byref(c), _ptr(t))
            textures.append(t)
        return {"nodes": nodes[:nn.value], "meshes": meshes, "textures": textures}
    finally:
        L.ref_model_free(h)


def ref_load_ppm(path: str) -> np.ndarray:
    """The reference's loadPPM: (rows, cols, 3) float32 (empty if unreadable)."""
    L = ref_lib()
    r, c = C.c_int32(), C.c_int32()
    L.ref_ppm_load(path.encode(), C.byref(r), C.byref(c), None)
    out = np.zeros((r.value, c.value, 3), np.float32)
    if out.size:
        L.ref_ppm_load(path.encode(), C.byref(r), C.byref(c), _ptr(out))
    return out


def ref_save_ppm(path: str, rgb: np.ndarray) -> None:
    """The reference's savePPM of a float image (rows, cols, 3)."""
    a = np.ascontiguousarray(rgb, np.float32)
    ref_lib().ref_ppm_save(path.encode(), _ptr(a), a.shape[0], a.shape[1])


def ref_save_xyz(path: str, points: np.ndarray, transform=None) -> None:
    """The reference's saveXYZ of a (rows, cols, 3) float image."""
    a = np.ascontiguousarray(points, np.float32)
    xf = None if transform is None else np.ascontiguousarray(transform, np.float32)
    ref_lib().ref_xyz_save(path.encode(), _ptr(a), a.shape[0], a.shape[1], None if xf is None else _ptr(xf))


def ref_save_stl(path: str, desc, transform=None) -> None:
    """The reference's saveSTL of a mesh (mr_mesh_desc) under transform."""
    xf = None if transform is None else np.ascontiguousarray(transform, np.float32)
    ref_lib().ref_stl_save(path.encode(), C.byref(desc), None if xf is None else _ptr(xf))


def _ptr(a: np.ndarray):
    return a.ctypes.data


def decode_rgb8(tex: np.ndarray) -> np.ndarray:
    """loadPPM texel decode (src/io.cpp:407-410) via the C restatement."""
    tex = np.ascontiguousarray(tex, np.uint8)
    out = np.empty(tex.shape, np.float32)
    lib().mro_decode_rgb8(_ptr(tex), tex.size // 3, _ptr(out))
    return out


def quantize_rgb8(image: np.ndarray) -> np.ndarray:
    """savePPM conversion (src/io.cpp:358-362) via the C restatement."""
    image = np.ascontiguousarray(image, np.float32)
    out = np.empty(image.shape, np.uint8)
    lib().mro_quantize_rgb8(_ptr(image), image.size // 3, _ptr(out))
    return out


def _float_textures(textures):
    keep = []
    arr = (_Tex * max(1, len(textures)))()
    for i, t in enumerate(textures):
        f = decode_rgb8(t) if t.dtype == np.uint8 else np.ascontiguousarray(t, np.float32)
        keep.append(f)
        arr[i].rgb = _ptr(f)
        arr[i].rows = f.shape[0]
        arr[i].cols = f.shape[1]
    return arr, keep


def collect_shapes(flat: sc.Flat):
    n_nodes = len(flat.nodes)
    out = (abi.mr_renderable * max(1, n_nodes))()
    n = C.c_int32(0)
    rc = lib().mro_collect_shapes(C.addressof(flat.nodes), n_nodes, C.addressof(out), n_nodes,
                                  C.byref(n))
    if rc != 0:
        raise RuntimeError(f"mro_collect_shapes failed: {rc}")
    return out, n.value


def render(state: FrameState, scene: sc.SceneNode, normals: bool = False, flags=None) -> dict:
    """The C restatement: image (H,W,3) f32, depth (H,W) f32, ids (H,W) u32,
    rgb8 (H,W,3) u8 and optionally normals.  `flags` (one int per renderable
    in collectShapes order) are or-ed into the renderables' flags."""
    flat = sc.flatten(scene)
    rs, n = collect_shapes(flat)
    if flags is not None:
        for i in range(n):
            rs[i].flags |= int(flags[i])
    meshes = sc.mesh_descs(flat.meshes)
    tex, keep = _float_textures(flat.textures)
    f = state.to_c()
    H, W = state.height, state.width
    image = np.empty((H, W, 3), np.float32)
    depth = np.empty((H, W), np.float32)
    ids = np.empty((H, W), np.uint32)
    nrm = np.empty((H, W, 3), np.float32) if normals else None
    rc = lib().mro_render(C.byref(f), C.addressof(rs), n, C.addressof(meshes), len(flat.meshes),
                          C.addressof(tex), len(flat.textures), _ptr(image), _ptr(depth), _ptr(ids),
                          _ptr(nrm) if nrm is not None else None)
    if rc != 0:
        raise RuntimeError(f"mro_render failed: {rc}")
    out = {"image": image, "depth": depth, "ids": ids, "rgb8": quantize_rgb8(image)}
    if nrm is not None:
        out["normals"] = nrm
    return out


def render_paints(state: FrameState, paints, normals: bool = False, base_scene: sc.SceneNode = None) -> dict:
    """The C restatement of clear(), then render()'s renderables of
    `base_scene` (if given), then the paintMesh / paintTriangle calls
    `paints` (scene.Paint) in order, as the reference paints them one after
    the other (src/Renderer.cpp:163-381)."""
    meshes, mesh_ix, texs, tex_ix = [], {}, [], {}

    def mesh_index(m):
        if id(m) not in mesh_ix:
            mesh_ix[id(m)] = len(meshes)
            meshes.append(m)
        return mesh_ix[id(m)]

    def texture_index(t):
        if id(t) not in tex_ix:
            tex_ix[id(t)] = len(texs)
            texs.append(t)
        return tex_ix[id(t)]

    base = []
    if base_scene is not None:
        flat = sc.flatten(base_scene)
        rs0, n0 = collect_shapes(flat)
        for i in range(n0):
            r = abi.mr_renderable()
            C.memmove(C.addressof(r), C.addressof(rs0[i]), C.sizeof(r))
            r.mesh = mesh_index(flat.meshes[rs0[i].mesh])
            if r.material.texture >= 0:
                r.material.texture = texture_index(flat.textures[r.material.texture])
            base.append(r)
    prs = sc.paints_to_c(list(paints), mesh_index, texture_index)
    n = len(base) + len(paints)
    rs = (abi.mr_renderable * max(1, n))()
    for i, r in enumerate(base):
        rs[i] = r
    for j in range(len(paints)):
        rs[len(base) + j] = prs[j]
    descs = sc.mesh_descs(meshes)
    tex, keep = _float_textures(texs)
    f = state.to_c()
    H, W = state.height, state.width
    image = np.empty((H, W, 3), np.float32)
    depth = np.empty((H, W), np.float32)
    ids = np.empty((H, W), np.uint32)
    nrm = np.empty((H, W, 3), np.float32) if normals else None
    rc = lib().mro_render(C.byref(f), C.addressof(rs), n, C.addressof(descs), len(meshes), C.addressof(tex),
                          len(texs), _ptr(image), _ptr(depth), _ptr(ids), _ptr(nrm) if nrm is not None else None)
    if rc != 0:
        raise RuntimeError(f"mro_render failed: {rc}")
    out = {"image": image, "depth": depth, "ids": ids, "rgb8": quantize_rgb8(image)}
    if nrm is not None:
        out["normals"] = nrm
    return out


def range_image(state: FrameState, depth: np.ndarray) -> np.ndarray:
    f = state.to_c()
    depth = np.ascontiguousarray(depth, np.float32)
    out = np.empty(depth.shape + (3,), np.float32)
    lib().mro_range_image(C.byref(f), _ptr(depth), _ptr(out))
    return out


def time_frames(state: FrameState, scene: sc.SceneNode, n_frames: int, n_threads: int) -> float:
    """Seconds for n_frames independent renders on n_threads host threads."""
    flat = sc.flatten(scene)
    rs, n = collect_shapes(flat)
    meshes = sc.mesh_descs(flat.meshes)
    tex, keep = _float_textures(flat.textures)
    f = state.to_c()
    return lib().mro_render_frames_mt(C.byref(f), C.addressof(rs), n, C.addressof(meshes),
                                      len(flat.meshes), C.addressof(tex), len(flat.textures),
                                      n_frames, n_threads)


def ref_render(state: FrameState, scene: sc.SceneNode, normals: bool = False,
               range_xyz: bool = False) -> dict:
    """The reference Renderer itself (compiled from its sources)."""
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference build unavailable")
    flat = sc.flatten(scene)
    meshes = sc.mesh_descs(flat.meshes)
    tex, keep = _float_textures(flat.textures)
    f = state.to_c()
    H, W = state.height, state.width
    image = np.empty((H, W, 3), np.float32)
    depth = np.empty((H, W), np.float32)
    nrm = np.empty((H, W, 3), np.float32) if normals else None
    rng = np.empty((H, W, 3), np.float32) if range_xyz else None
    rc = L.ref_render(C.byref(f), C.addressof(flat.nodes), len(flat.nodes), C.addressof(meshes),
                      len(flat.meshes), C.addressof(tex), len(flat.textures), _ptr(image),
                      _ptr(depth), _ptr(nrm) if nrm is not None else None,
                      _ptr(rng) if rng is not None else None)
    if rc != 0:
        raise RuntimeError(f"ref_render failed: {rc}")
    out = {"image": image, "depth": depth, "rgb8": quantize_rgb8(image)}
    if nrm is not None:
        out["normals"] = nrm
    if rng is not None:
        out["range"] = rng
    return out


def ref_paint(state: FrameState, paints, clear: bool = False) -> dict:
    """The reference Renderer itself: render() of an empty scene (the state
    paintMesh uses), clear() if asked, then the paints in order -- paintMesh
    for a scene.Paint without MR_RS_MODELVIEW, setMaterial + paintTriangle
    per triangle of a paintTriangle run, and for the state items between
    them: setView(m) for ("view", m), setLighting(b) for ("lighting", b),
    setTexturing(b) for ("texturing", b), setLight(v, point) for
    ("light", v, point), setBackground(rgb) for ("background", rgb)."""
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference build unavailable")
    meshes, texs, tex_ix = [], [], {}
    kind, mesh, xf, tri, world, mats = [], [], [], [], [], []

    def texture_index(t):
        if id(t) not in tex_ix:
            tex_ix[id(t)] = len(texs)
            texs.append(t)
        return tex_ix[id(t)]

    for p in paints:
        if isinstance(p, tuple):
            m16 = np.zeros(16, np.float32)
            flag = 1
            if p[0] == "view":
                k, m16[:] = 2, np.asarray(p[1], np.float32).reshape(16)
            elif p[0] in ("lighting", "texturing"):
                k, flag = (3 if p[0] == "lighting" else 4), int(bool(p[1]))
            elif p[0] == "light":
                k, flag = 5, int(bool(p[2]))
                m16[:3] = np.asarray(p[1], np.float32).reshape(3)
            elif p[0] == "background":
                k, m16[:3] = 6, np.asarray(p[1], np.float32).reshape(3)
            else:
                raise ValueError(f"unknown state item {p[0]!r}")
            kind.append(k); mesh.append(-1); xf.append(m16.reshape(4, 4))
            mats.append(abi.mr_material()); world.append(flag); tri.append(np.zeros(24, np.float32))
            continue
        m = abi.mr_material()
        tex = p.material.texture
        sc._fill_material(m, p.material, texture_index(tex) if tex is not None else -1)
        if p.flags & abi.MR_RS_MODELVIEW:
            v, n, uv = p.mesh.vertices, p.mesh.normals, p.mesh.texcoords
            for t in range(p.mesh.indices.size // 3):
                kind.append(1); mesh.append(-1); xf.append(np.eye(4, dtype=np.float32)); mats.append(m)
                world.append(0 if p.flags & abi.MR_RS_NO_CLIP else 1)
                tri.append(np.concatenate([np.concatenate([v[3 * t + c], n[3 * t + c], uv[3 * t + c]])
                                           for c in range(3)]).astype(np.float32))
        else:
            kind.append(0); mesh.append(len(meshes)); meshes.append(p.mesh); xf.append(p.transform)
            mats.append(m); world.append(1); tri.append(np.zeros(24, np.float32))
    n = len(kind)
    descs = sc.mesh_descs(meshes)
    tex, keep = _float_textures(texs)
    mat_arr = (abi.mr_material * max(1, n))(*mats)
    kind_a = np.asarray(kind, np.int32); mesh_a = np.asarray(mesh, np.int32); world_a = np.asarray(world, np.int32)
    xf_a = np.ascontiguousarray(np.stack(xf) if n else np.zeros((1, 4, 4)), np.float32)
    tri_a = np.ascontiguousarray(np.stack(tri) if n else np.zeros((1, 24)), np.float32)
    f = state.to_c()
    H, W = state.height, state.width
    image = np.empty((H, W, 3), np.float32)
    depth = np.empty((H, W), np.float32)
    rc = L.ref_paint(C.byref(f), C.addressof(descs), len(meshes), C.addressof(tex), len(texs), int(clear), n,
                     _ptr(kind_a), _ptr(mesh_a), _ptr(xf_a), C.addressof(mat_arr), _ptr(tri_a), _ptr(world_a),
                     _ptr(image), _ptr(depth))
    if rc != 0:
        raise RuntimeError(f"ref_paint failed: {rc}")
    return {"image": image, "depth": depth, "rgb8": quantize_rgb8(image)}


def ref_primitive(kind: int, a: float, b: float = 0.0, seg: int = 0, hseg: int = 0,
                  caps: bool = True) -> dict:
    """Arrays from the reference's createCube(0)/createCylinder(1)/createSphere(2)."""
    L = ref_lib()
    counts = np.zeros(5, np.int32)
    L.ref_primitive(kind, a, b, seg, hseg, int(caps), _ptr(counts), None, None, None, None, None)
    v = np.empty((counts[0], 3), np.float32)
    n = np.empty((counts[1], 3), np.float32)
    t = np.empty((counts[2], 2), np.float32)
    i = np.empty(counts[3], np.int32)
    ni = np.empty(counts[4], np.int32)
    L.ref_primitive(kind, a, b, seg, hseg, int(caps), _ptr(counts), _ptr(v), _ptr(n), _ptr(t),
                    _ptr(i), _ptr(ni))
    return {"vertices": v, "normals": n, "texcoords": t, "indices": i, "normalsI": ni}


def ref_projection(kind: int, params) -> np.ndarray:
    p = np.asarray(params, np.float32)
    out = np.empty(16, np.float32)
    ref_lib().ref_projection(kind, _ptr(p), _ptr(out))
    return out.reshape(4, 4)


def ref_mat4_mul(a, b) -> np.ndarray:
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    out = np.empty(16, np.float32)
    ref_lib().ref_mat4_mul(_ptr(a), _ptr(b), _ptr(out))
    return out.reshape(4, 4)


def mat4_mul(a, b) -> np.ndarray:
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    out = np.empty(16, np.float32)
    lib().mro_mat4_mul(_ptr(a), _ptr(b), _ptr(out))
    return out.reshape(4, 4)


def mat4_inverse(a) -> np.ndarray:
    a = np.ascontiguousarray(a, np.float32)
    out = np.empty(16, np.float32)
    lib().mro_mat4_inverse(_ptr(a), _ptr(out))
    return out.reshape(4, 4)
