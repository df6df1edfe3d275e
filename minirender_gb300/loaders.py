"""Model and image files through the library's native loaders (host only):
``load_mesh`` (loadMesh, src/io.cpp:111-132: .stl, .obj + .mtl, .x3d),
``load_ppm`` / ``save_ppm`` (src/io.cpp:337-415) and ``save_stl``
(src/io.cpp:155-183), returning the Python scene model of ``scene.py``.

Textures stay RGB8 (the device decodes b/255.0f as loadPPM does)."""
from __future__ import annotations

import ctypes as C
from typing import List, Optional

import numpy as np

from . import abi, capi
from .scene import Material, SceneNode, TriMesh


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise capi.MRError(rc, f"{what}: {capi.lib().mr_status_string(rc).decode()}")


def _array(ptr, n: int, dtype, cols: int = 0) -> np.ndarray:
    if n == 0 or not ptr:
        return np.zeros((0, cols) if cols else (0,), dtype)
    a = np.ctypeslib.as_array(ptr, shape=(n * (cols or 1),)).copy().astype(dtype, copy=False)
    return a.reshape(-1, cols) if cols else a


def load_mesh(path: str) -> SceneNode:
    """The scene the reference's loadMesh builds for `path`."""
    L = capi.lib()
    h = C.c_void_p()
    _check(L.mr_model_load(path.encode(), C.byref(h)), f"mr_model_load({path})")
    try:
        nn, nm, nt = C.c_int32(), C.c_int32(), C.c_int32()
        _check(L.mr_model_counts(h, C.byref(nn), C.byref(nm), C.byref(nt)), "mr_model_counts")
        nodes = (abi.mr_node * max(1, nn.value))()
        _check(L.mr_model_nodes(h, nodes, nn.value), "mr_model_nodes")
        textures: List[np.ndarray] = []
        for i in range(nt.value):
            p, r, c = C.POINTER(C.c_uint8)(), C.c_int32(), C.c_int32()
            _check(L.mr_model_texture(h, i, C.byref(p), C.byref(r), C.byref(c)), "mr_model_texture")
            textures.append(_array(p, r.value * c.value * 3, np.uint8).reshape(r.value, c.value, 3))
        made: List[SceneNode] = []
        for i in range(nn.value):
            nd = nodes[i]
            xf = np.array(nd.transform[:], np.float32).reshape(4, 4)
            if nd.mesh >= 0:
                d = abi.mr_mesh_desc()
                _check(L.mr_model_mesh(h, nd.mesh, C.byref(d)), "mr_model_mesh")
                fp = C.POINTER(C.c_float)
                ip = C.POINTER(C.c_int32)
                node = TriMesh(_array(C.cast(d.vertices, fp), d.n_vertices, np.float32, 3),
                               _array(C.cast(d.normals, fp), d.n_normals, np.float32, 3),
                               _array(C.cast(d.indices, ip), d.n_indices, np.int32),
                               normalsI=_array(C.cast(d.normalsI, ip), d.n_normalsI, np.int32),
                               texcoords=_array(C.cast(d.texcoords, fp), d.n_texcoords, np.float32, 2),
                               texcoordsI=_array(C.cast(d.texcoordsI, ip), d.n_texcoordsI, np.int32),
                               transform=xf)
                if nd.has_material:
                    m = nd.material
                    node.material = Material(diffuse=m.diffuse[:], specular=m.specular[:], emissive=m.emissive[:],
                                             shininess=m.shininess, opacity=nd.opacity,
                                             texture=textures[m.texture] if m.texture >= 0 else None)
            else:
                node = SceneNode(xf)
            if nd.parent >= 0:
                made[nd.parent].add(node)
            made.append(node)
        return made[0]
    finally:
        L.mr_model_free(h)


def load_ppm(path: str) -> np.ndarray:
    """loadPPM's pixels as RGB8, (rows, cols, 3)."""
    L = capi.lib()
    r, c = C.c_int32(), C.c_int32()
    _check(L.mr_ppm_load(path.encode(), None, 0, C.byref(r), C.byref(c)), f"mr_ppm_load({path})")
    out = np.empty((r.value, c.value, 3), np.uint8)
    _check(L.mr_ppm_load(path.encode(), out.ctypes.data, out.nbytes, C.byref(r), C.byref(c)), "mr_ppm_load")
    return out


def save_ppm(path: str, rgb8: np.ndarray) -> None:
    """savePPM of an RGB8 image (rows, cols, 3)."""
    a = np.ascontiguousarray(rgb8, np.uint8)
    _check(capi.lib().mr_ppm_save(path.encode(), a.ctypes.data, a.shape[0], a.shape[1]), f"mr_ppm_save({path})")


def save_xyz(path: str, points: np.ndarray, transform: Optional[np.ndarray] = None) -> None:
    """saveXYZ: the points (rows, cols, 3) with z < -1e-5 (a range image's
    covered pixels) as "x y z" text lines, after `transform` (default the
    identity)."""
    a = np.ascontiguousarray(points, np.float32)
    if a.ndim != 3 or a.shape[2] != 3:
        raise ValueError("points must be (rows, cols, 3)")
    xf = None if transform is None else np.ascontiguousarray(transform, np.float32).reshape(4, 4)
    _check(capi.lib().mr_xyz_save(path.encode(), a.ctypes.data, a.shape[0], a.shape[1],
                                  None if xf is None else xf.ctypes.data), f"mr_xyz_save({path})")


def save_stl(path: str, mesh: TriMesh, transform: Optional[np.ndarray] = None) -> None:
    """saveSTL: binary STL of the mesh's triangles under `transform`
    (default: the mesh's own transform, as the reference uses)."""
    xf = np.ascontiguousarray(mesh.transform if transform is None else transform, np.float32)
    _check(capi.lib().mr_stl_save(path.encode(), C.byref(mesh.desc()), xf.ctypes.data), f"mr_stl_save({path})")
