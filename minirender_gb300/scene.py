"""Python mirror of minirender's scene model (include/minirender/Scene.h).

Same class and member names as the reference so calling code reads the same:
``Material`` (Scene.h:38-45, defaults src/Scene.cpp:65-71), ``SceneNode``
(Scene.h:55-63), ``TriMesh`` (Scene.h:73-87) and ``Scene`` (Scene.h:89-95).
Arrays are numpy: vertices/normals (N,3) float32, texcoords (N,2) float32,
indices/normalsI/texcoordsI (3T,) int32, textures (rows, cols, 3) uint8
(decoded as loadPPM does, src/io.cpp:407-410) or float32.

``flatten`` turns a scene into the pre-order ``mr_node`` array that
``mr_collect_shapes`` (the C restatement of Scene::collectShapes,
src/Scene.cpp:13-36) consumes, plus the list of distinct meshes and
textures it references.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional

import numpy as np

from . import abi


def identity() -> np.ndarray:
    return np.eye(4, dtype=np.float32)


class Material:
    """Material, include/minirender/Scene.h:38-45; defaults src/Scene.cpp:65-71."""

    def __init__(self, diffuse=(0.7, 0.7, 0.9), specular=(0.8, 0.8, 0.8), emissive=(0, 0, 0),
                 shininess=12.0, opacity=1.0, texture: Optional[np.ndarray] = None):
        self.diffuse = np.asarray(diffuse, np.float32)
        self.specular = np.asarray(specular, np.float32)
        self.emissive = np.asarray(emissive, np.float32)
        self.shininess = np.float32(shininess)
        self.opacity = np.float32(opacity)
        self.texture = texture  # (rows, cols, 3) uint8 or float32, or None


class SceneNode:
    """SceneNode, include/minirender/Scene.h:55-63."""

    def __init__(self, transform: Optional[np.ndarray] = None):
        self.visible = True
        self.transform = identity() if transform is None else np.asarray(transform, np.float32)
        self.children: List[SceneNode] = []

    def add(self, node: "SceneNode") -> "SceneNode":
        self.children.append(node)
        return node


class TriMesh(SceneNode):
    """TriMesh, include/minirender/Scene.h:73-87."""

    def __init__(self, vertices, normals, indices, normalsI=None, texcoords=None, texcoordsI=None,
                 material: Optional[Material] = None, transform=None):
        super().__init__(transform)
        self.vertices = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        self.normals = np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
        self.indices = np.ascontiguousarray(indices, np.int32).reshape(-1)
        self.normalsI = (self.indices if normalsI is None
                         else np.ascontiguousarray(normalsI, np.int32).reshape(-1))
        self.texcoords = (np.zeros((0, 2), np.float32) if texcoords is None
                          else np.ascontiguousarray(texcoords, np.float32).reshape(-1, 2))
        self.texcoordsI = (np.zeros(0, np.int32) if texcoordsI is None
                           else np.ascontiguousarray(texcoordsI, np.int32).reshape(-1))
        self.material = material
        self.version = 0  # bump after editing arrays in place so resident copies refresh

    @property
    def n_triangles(self) -> int:
        return self.indices.size // 3

    def desc(self) -> abi.mr_mesh_desc:
        """mr_mesh_desc pointing at this mesh's arrays (kept alive by self)."""
        def p(a):
            return a.ctypes.data if a.size else None
        return abi.mr_mesh_desc(p(self.vertices), self.vertices.shape[0],
                                p(self.normals), self.normals.shape[0],
                                p(self.texcoords), self.texcoords.shape[0],
                                p(self.indices), self.indices.size,
                                p(self.normalsI), self.normalsI.size,
                                p(self.texcoordsI), self.texcoordsI.size)


class Scene(SceneNode):
    """Scene, include/minirender/Scene.h:89-95 (ambientLight default 0.1)."""

    def __init__(self):
        super().__init__()
        self.ambientLight = np.float32(0.1)
        self.light = np.zeros(3, np.float32)


def _fill_material(dst: abi.mr_material, m: Material, tex_index: int) -> None:
    dst.diffuse[:] = [float(x) for x in m.diffuse]
    dst.specular[:] = [float(x) for x in m.specular]
    dst.emissive[:] = [float(x) for x in m.emissive]
    dst.shininess = float(m.shininess)
    dst.texture = tex_index


class Flat:
    """A scene flattened to the C-ABI's node form."""

    def __init__(self, nodes, meshes: List[TriMesh], textures: List[np.ndarray]):
        self.nodes = nodes
        self.meshes = meshes
        self.textures = textures


def flatten(scene: SceneNode) -> Flat:
    """Pre-order walk (parents before children, children in insertion order)."""
    order = []
    stack = [(scene, -1)]
    while stack:
        node, parent = stack.pop()
        idx = len(order)
        order.append((node, parent))
        for ch in reversed(node.children):
            stack.append((ch, idx))
    nodes = (abi.mr_node * len(order))()
    meshes: List[TriMesh] = []
    mesh_ix = {}
    textures: List[np.ndarray] = []
    tex_ix = {}
    for i, (node, parent) in enumerate(order):
        nd = nodes[i]
        nd.parent = parent
        nd.transform[:] = [float(x) for x in np.asarray(node.transform, np.float32).reshape(16)]
        nd.mesh = -1
        nd.has_material = 0
        nd.opacity = 1.0
        if isinstance(node, TriMesh):
            if id(node) not in mesh_ix:
                mesh_ix[id(node)] = len(meshes)
                meshes.append(node)
            nd.mesh = mesh_ix[id(node)]
            if node.material is not None:
                t = -1
                tex = node.material.texture
                if tex is not None and tex.shape[0] > 0:
                    if id(tex) not in tex_ix:
                        tex_ix[id(tex)] = len(textures)
                        textures.append(tex)
                    t = tex_ix[id(tex)]
                nd.has_material = 1
                nd.opacity = float(node.material.opacity)
                _fill_material(nd.material, node.material, t)
    return Flat(nodes, meshes, textures)


class Vertex:
    """Vertex, include/minirender/Scene.h:14-24: position, normal, uv (the
    arguments of Renderer::paintTriangle, in view space)."""

    def __init__(self, position, normal=(0, 0, 1), uv=(0, 0)):
        self.position = np.asarray(position, np.float32).reshape(3)
        self.normal = np.asarray(normal, np.float32).reshape(3)
        self.uv = np.asarray(uv, np.float32).reshape(2)


class Paint:
    """One paintMesh call (or a run of paintTriangle calls with one material
    and one clipping mode, gathered into a mesh): the mesh, its transform
    (the modelview itself when flags has MR_RS_MODELVIEW), the material and
    the mr_renderable flags."""

    def __init__(self, mesh: TriMesh, transform, material: Material, flags: int = 0):
        self.mesh = mesh
        self.transform = np.asarray(transform, np.float32).reshape(4, 4)
        self.material = material
        self.flags = int(flags)


def triangle_paint(a: Vertex, b: Vertex, c: Vertex, material: Material, world: bool) -> Paint:
    """paintTriangle(a, b, c, world) (src/Renderer.cpp:163-309) as a paint:
    a one-triangle mesh of view-space vertices, the identity as modelview."""
    v = [a, b, c]
    idx = np.arange(3, dtype=np.int32)
    mesh = TriMesh(np.stack([x.position for x in v]), np.stack([x.normal for x in v]), idx, normalsI=idx,
                   texcoords=np.stack([x.uv for x in v]), texcoordsI=idx, material=material)
    flags = abi.MR_RS_MODELVIEW | (0 if world else abi.MR_RS_NO_CLIP)
    return Paint(mesh, identity(), material, flags)


def append_triangle(p: Paint, a: Vertex, b: Vertex, c: Vertex) -> None:
    """Adds one more triangle (drawn after the others) to a paintTriangle run."""
    m = p.mesh
    n = m.vertices.shape[0]
    m.vertices = np.concatenate([m.vertices, np.stack([a.position, b.position, c.position])])
    m.normals = np.concatenate([m.normals, np.stack([a.normal, b.normal, c.normal])])
    m.texcoords = np.concatenate([m.texcoords, np.stack([a.uv, b.uv, c.uv])])
    m.indices = np.concatenate([m.indices, np.arange(n, n + 3, dtype=np.int32)])
    m.normalsI = m.indices
    m.texcoordsI = m.indices


def paints_to_c(paints: List[Paint], mesh_index, texture_index):
    """mr_renderable array for a paint list; mesh_index(mesh) and
    texture_index(texture) give the handles (or array indices)."""
    rs = (abi.mr_renderable * max(1, len(paints)))()
    for i, p in enumerate(paints):
        rs[i].mesh = mesh_index(p.mesh)
        rs[i].flags = p.flags
        rs[i].transform[:] = [float(x) for x in p.transform.reshape(16)]
        tex = p.material.texture
        _fill_material(rs[i].material, p.material, texture_index(tex) if tex is not None else -1)
    return rs


def geometry_key(mesh: TriMesh) -> tuple:
    """Identity of a mesh's arrays: TriMesh nodes that share their arrays share
    one resident copy on the device."""
    return (id(mesh.vertices), id(mesh.normals), id(mesh.texcoords), id(mesh.indices),
            id(mesh.normalsI), id(mesh.texcoordsI))


def mesh_descs(meshes: List[TriMesh]):
    arr = (abi.mr_mesh_desc * max(1, len(meshes)))()
    for i, m in enumerate(meshes):
        arr[i] = m.desc()
    return arr
