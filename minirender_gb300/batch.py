"""Many frames per call: ``BatchRenderer`` renders a list of (Renderer state,
scene) pairs -- each one what a separate ``Renderer.render()`` would draw --
through ``mr_render_batch``: one vertex pass, one setup pass and one
persistent fused bin-raster-shade kernel for all of them, optionally replayed
from a CUDA graph.  Meshes and textures stay resident across batches."""
from __future__ import annotations

import ctypes as C
from typing import List, Sequence, Tuple

import numpy as np

from . import abi, capi
from . import scene as sc
from .frame import FrameState


class BatchRenderer:
    def __init__(self, device: int = 0, ctx: capi.Context = None):
        self.ctx = ctx or capi.Context(device)
        self._meshes = {}
        self._textures = {}
        self.outputs = abi.MR_OUT_DEFAULT

    def _mesh_handle(self, mesh: sc.TriMesh) -> int:
        key = sc.geometry_key(mesh)
        rec = self._meshes.get(key)
        if rec is not None and rec[2] is mesh.vertices:
            if rec[1] != mesh.version:
                self.ctx.update_mesh(rec[0], mesh.desc())
                self._meshes[key] = (rec[0], mesh.version, mesh.vertices)
            return rec[0]
        h = self.ctx.upload_mesh(mesh.desc())
        self._meshes[key] = (h, mesh.version, mesh.vertices)
        return h

    def _texture_handle(self, tex: np.ndarray) -> int:
        rec = self._textures.get(id(tex))
        if rec is not None and rec[1] is tex:
            return rec[0]
        h = self.ctx.upload_texture(tex)
        self._textures[id(tex)] = (h, tex)
        return h

    def prepare(self, items: Sequence[Tuple[FrameState, sc.SceneNode]]):
        """Flattens every scene (Scene::collectShapes), makes meshes and
        textures resident, returns the (scenes, n, renderables, n_rs) arrays
        mr_render_batch takes."""
        per = []
        total = 0
        for st, scene in items:
            flat = sc.flatten(scene)
            rs, n = capi.collect_shapes(flat.nodes)
            mh = [self._mesh_handle(m) for m in flat.meshes]
            th = [self._texture_handle(t) for t in flat.textures]
            for i in range(n):
                rs[i].mesh = mh[rs[i].mesh]
                if rs[i].material.texture >= 0:
                    rs[i].material.texture = th[rs[i].material.texture]
            st.ambient = getattr(scene, "ambientLight", np.float32(0.1))
            per.append((st.to_c(), rs, n))
            total += n
        scenes = (abi.mr_batch_scene * len(per))()
        allrs = (abi.mr_renderable * max(1, total))()
        k = 0
        sz = C.sizeof(abi.mr_renderable)
        for i, (f, rs, n) in enumerate(per):
            scenes[i].frame = f
            scenes[i].first_renderable = k
            scenes[i].n_renderables = n
            if n:
                C.memmove(C.addressof(allrs) + k * sz, C.addressof(rs), n * sz)
            k += n
        return scenes, len(per), allrs, total

    def render(self, items: Sequence[Tuple[FrameState, sc.SceneNode]]):
        scenes, ns, rs, nr = self.prepare(items)
        self.ctx.render_batch(scenes, ns, rs, nr, self.outputs)
        return scenes, ns, rs, nr

    def read(self, scene: int) -> dict:
        return self.ctx.read_batch(scene)

    def close(self):
        self.ctx.close()
