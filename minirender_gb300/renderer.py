"""``Renderer``: the reference's public Renderer interface
(include/minirender/Renderer.h:44-63) running on the GB300 path.

Same method names and argument meaning as minirender::Renderer.  ``render``
flattens the scene with Scene::collectShapes semantics, keeps meshes and
textures resident on the device (re-uploaded only when a mesh's ``version``
changes), and queues one frame through the C ABI; the getters read the
results back.

``paintMesh`` / ``paintTriangle`` draw into the current framebuffer as the
reference's do: after ``clear()`` (or ``render()``) the paints are recorded
and the next getter renders the scene's renderables and the paints, in call
order, as one frame -- the same pixels as painting them one after the other
(later fragments win only with a strictly smaller depth).  State follows the
reference call by call: ``paintMesh`` uses the view current at the call, and
every paint the lighting, texturing and light-type switches current at the
call; the light is placed as the last ``render()`` placed it (with its view,
light and light type; with no ``render()`` since ``clear()``, as the first
paint finds them); the background is the one of the last ``clear()`` /
``render()``.  Projection and the normals switch are the frame's: the state
when the frame is read.
"""
from __future__ import annotations

import copy

from typing import Dict, Optional

import numpy as np

from . import abi, capi
from . import scene as sc
from .frame import FrameState


class Renderer:
    def __init__(self, device: int = 0):
        self.ctx = capi.Context(device)
        self.state = FrameState()
        self.scene: Optional[sc.SceneNode] = None
        self._material = None
        self._meshes: Dict[tuple, tuple] = {}   # geometry key -> (handle, version, vertices)
        self._textures: Dict[int, tuple] = {}   # id(array) -> (handle, array)
        self._out: Optional[dict] = None
        self._rendered = False
        self._base = None                      # (renderables, count) of the last render()
        self._paints: list = []                # paintMesh / paintTriangle since then
        self._frame_state: Optional[FrameState] = None  # state that placed the frame's light
        self._clear_bg = None                  # background of the last clear() / render()
        self._used = (set(), set())            # mesh keys / texture ids the frame being built uses
        self._base_used = (set(), set())       # ... and those of the last render()
        self._dirty = False
        self.outputs = abi.MR_OUT_DEFAULT | abi.MR_OUT_RGB_F32

    # ---- setters, include/minirender/Renderer.h:45-55
    def setSize(self, w: int, h: int):
        self.state.width, self.state.height = int(w), int(h)
        self.clear()

    def aspect(self) -> float:
        return float(np.float32(self.state.width) / np.float32(self.state.height))

    def setScene(self, scene: sc.SceneNode):
        self.scene = scene

    def setProjection(self, m):
        self.state.projection = np.asarray(m, np.float32).reshape(4, 4)

    def setView(self, m):
        self.state.view = np.asarray(m, np.float32).reshape(4, 4)

    def setLight(self, v, point: bool = False):
        self.state.light = np.asarray(v, np.float32).reshape(3)
        self.state.light_is_point = bool(point)

    def setMaterial(self, material: sc.Material):
        # As in the reference, render() and paintMesh replace the current
        # material per mesh (src/Renderer.cpp:336); paintTriangle uses it.
        self._material = material

    def setLighting(self, on: bool):
        self.state.lighting = bool(on)

    def setTexturing(self, on: bool):
        self.state.texturing = bool(on)

    def setSaveNormals(self, on: bool):
        self.state.save_normals = bool(on)

    def setBackground(self, color):
        self.state.background = np.asarray(color, np.float32).reshape(3)

    def clear(self):
        """Renderer::clear (src/Renderer.cpp:113-119): background image,
        depth 1e11f."""
        self._out = None
        self._rendered = False
        self._base = None
        self._paints = []
        self._frame_state = None
        self._clear_bg = np.asarray(self.state.background, np.float32).copy()
        self._dirty = False

    def _frame(self) -> FrameState:
        """The state the frame's light was placed with: the last render()'s,
        or, with none since clear(), the first paint's."""
        if self._frame_state is None:
            self._frame_state = copy.deepcopy(self.state)
        return self._frame_state

    def _paint_flags(self) -> int:
        """MR_RS_OWN_STATE and the switches of this paint call when they
        differ from the frame's (src/Renderer.cpp:264-289 reads them per
        call)."""
        f, s = self._frame(), self.state
        cur = (bool(s.lighting), bool(s.texturing), bool(s.light_is_point))
        if cur == (bool(f.lighting), bool(f.texturing), bool(f.light_is_point)):
            return 0
        return (abi.MR_RS_OWN_STATE | (abi.MR_RS_LIGHTING if cur[0] else 0) |
                (abi.MR_RS_TEXTURING if cur[1] else 0) | (abi.MR_RS_POINT_LIGHT if cur[2] else 0))

    def paintMesh(self, mesh: sc.TriMesh, transform=None):
        """Renderer::paintMesh (src/Renderer.cpp:334-381): the mesh with the
        current view and `transform`, in the mesh's material (or the
        default), over what is already drawn."""
        mat = mesh.material if mesh.material is not None else sc.Material()
        self._material = mat
        xf = sc.identity() if transform is None else transform
        view = np.asarray(self.state.view, np.float32).reshape(4, 4)
        flags = self._paint_flags()
        if view.tobytes() == np.asarray(self._frame().view, np.float32).reshape(4, 4).tobytes():
            self._paints.append(sc.Paint(mesh, xf, mat, flags))
        else:
            # the view changed since the frame's light was placed: this
            # call's modelview, _view * transform (src/Renderer.cpp:337),
            # composed as the library composes it
            mv = capi.mat4_mul(view, np.asarray(xf, np.float32).reshape(4, 4))
            self._paints.append(sc.Paint(mesh, mv, mat, abi.MR_RS_MODELVIEW | flags))
        self._dirty = True

    def paintTriangle(self, a: sc.Vertex, b: sc.Vertex, c: sc.Vertex, world: bool = True):
        """Renderer::paintTriangle (src/Renderer.cpp:163-309): one triangle
        of view-space vertices in the current material; world=False skips the
        near-plane clipping."""
        mat = self._material if self._material is not None else sc.Material()
        flags = abi.MR_RS_MODELVIEW | (0 if world else abi.MR_RS_NO_CLIP) | self._paint_flags()
        last = self._paints[-1] if self._paints else None
        if last is not None and last.flags == flags and last.material is mat and getattr(last, "run", False):
            sc.append_triangle(last, a, b, c)
        else:
            p = sc.triangle_paint(a, b, c, mat, world)
            p.flags = flags  # with the switches of this call
            p.run = True
            self._paints.append(p)
        self._dirty = True

    # ---- frame
    def _mesh_handle(self, mesh: sc.TriMesh) -> int:
        key = sc.geometry_key(mesh)
        self._used[0].add(key)
        rec = self._meshes.get(key)
        if rec is not None and rec[2] is mesh.vertices:
            h, ver, _ = rec
            if ver != mesh.version:
                self.ctx.update_mesh(h, mesh.desc())
                self._meshes[key] = (h, mesh.version, mesh.vertices)
            return h
        h = self.ctx.upload_mesh(mesh.desc())
        self._meshes[key] = (h, mesh.version, mesh.vertices)
        return h

    def _texture_handle(self, tex: np.ndarray) -> int:
        self._used[1].add(id(tex))
        rec = self._textures.get(id(tex))
        if rec is not None and rec[1] is tex:
            return rec[0]
        h = self.ctx.upload_texture(tex)
        self._textures[id(tex)] = (h, tex)
        return h

    def prepare(self):
        """Flattens the scene (Scene::collectShapes), makes its meshes and
        textures resident and returns the (mr_frame, renderables, count)
        triple that mr_render takes."""
        if self.scene is None:
            raise RuntimeError("setScene() first")
        flat = sc.flatten(self.scene)
        rs, n = capi.collect_shapes(flat.nodes)
        mesh_h = [self._mesh_handle(m) for m in flat.meshes]
        tex_h = [self._texture_handle(t) for t in flat.textures]
        for i in range(n):
            rs[i].mesh = mesh_h[rs[i].mesh]
            if rs[i].material.texture >= 0:
                rs[i].material.texture = tex_h[rs[i].material.texture]
        self.state.ambient = getattr(self.scene, "ambientLight", np.float32(0.1))
        return self.state.to_c(), rs, n

    def _prune(self):
        """Frees the resident meshes and textures the frame just drawn does
        not use (the caches hold the meshes of the last frame only)."""
        meshes, textures = self._used
        for key in [k for k in self._meshes if k not in meshes]:
            self.ctx.free_mesh(self._meshes.pop(key)[0])
        for key in [k for k in self._textures if k not in textures]:
            self.ctx.free_texture(self._textures.pop(key)[0])

    def render(self):
        """Renderer::render (src/Renderer.cpp:311-332)."""
        self._used = (set(), set())
        frame, rs, n = self.prepare()
        self.ctx.render(frame, rs, n, self.outputs)
        self._base_used = (set(self._used[0]), set(self._used[1]))
        self._prune()
        self._out = None
        self._rendered = True
        self._base = (rs, n)
        self._paints = []
        self._frame_state = copy.deepcopy(self.state)
        self._clear_bg = np.asarray(self.state.background, np.float32).copy()
        self._dirty = False

    def _flush_paints(self):
        """Renders the last render()'s renderables and the paints since."""
        base_rs, base_n = self._base if self._base is not None else (None, 0)
        self._used = (set(self._base_used[0]), set(self._base_used[1])) if self._base is not None else (set(), set())
        prs = sc.paints_to_c(self._paints, self._mesh_handle, self._texture_handle)
        n = base_n + len(self._paints)
        rs = (abi.mr_renderable * max(1, n))()
        for i in range(base_n):
            rs[i] = base_rs[i]
        for j in range(len(self._paints)):
            rs[base_n + j] = prs[j]
        frame = self._frame_c()
        self.ctx.render(frame, rs, n, self.outputs)
        self._prune()
        self._rendered = True
        self._dirty = False
        self._out = None

    def _frame_c(self):
        """mr_frame of a flush: the light, its view and the default switches
        of the frame, the background of the last clear(), the rest current."""
        frame = self.state.to_c()
        f = self._frame()
        frame.view[:] = [float(x) for x in np.asarray(f.view, np.float32).reshape(16)]
        frame.light[:] = [float(x) for x in np.asarray(f.light, np.float32).reshape(3)]
        frame.light_is_point = int(bool(f.light_is_point))
        frame.lighting = int(bool(f.lighting))
        frame.texturing = int(bool(f.texturing))
        if self._clear_bg is not None:
            frame.background[:] = [float(x) for x in self._clear_bg]
        return frame

    def _read(self) -> dict:
        if self._dirty:
            self._flush_paints()
        if self._out is None:
            if not self._rendered:
                return self._cleared()
            self._out = self.ctx.read(rgb8=True, depth=True, rgb_f32=True, tri_id=True,
                                      normals=self.state.save_normals)
        return self._out

    def _cleared(self) -> dict:
        H, W = self.state.height, self.state.width
        img = np.empty((H, W, 3), np.float32)
        img[:] = np.asarray(self.state.background if self._clear_bg is None else self._clear_bg, np.float32)
        out = {"image": img, "depth": np.full((H, W), 1e11, np.float32),
               "ids": np.full((H, W), abi.MR_NO_TRIANGLE, np.uint32)}
        out["rgb8"] = np.clip(img * np.float32(255), 0, 255).astype(np.uint8)
        if self.state.save_normals:
            nrm = np.zeros((H, W, 3), np.float32)
            nrm[..., 2] = 1
            out["normals"] = nrm
        return out

    # ---- getters, include/minirender/Renderer.h:60-63
    def getDepth(self) -> np.ndarray:
        return self._read()["depth"]

    def getImage(self) -> np.ndarray:
        return self._read()["image"]

    def getImageRGB8(self) -> np.ndarray:
        """getImage() after savePPM's byte conversion (src/io.cpp:358-362)."""
        return self._read()["rgb8"]

    def getTriangleIds(self) -> np.ndarray:
        """Visible sub-triangle per pixel: 2*(global triangle)+clip part."""
        return self._read()["ids"]

    def getRangeImage(self) -> np.ndarray:
        self._read()
        return self.ctx.range_image()

    def getNormalsImage(self) -> np.ndarray:
        return self._read()["normals"]

    def stats(self) -> abi.mr_stats:
        return self.ctx.stats()

    def close(self):
        self.ctx.close()
