"""``RenderServer``: Python handle on the library's render server
(mr_server_*): requests are queued, admitted against a device-memory budget
and rendered in batches by a native worker thread while earlier batches are
still running; meshes and textures stay resident between requests."""
from __future__ import annotations

import ctypes as C
from typing import Dict, Optional

import numpy as np

from . import abi, capi
from .frame import FrameState
from .scene import Material, TriMesh


class RenderServer:
    def __init__(self, ctx: capi.Context, budget_bytes: int = 40 << 30, slots: int = 2, max_batch: int = 32,
                 tile: int = 16, threads: int = 64, chunk: int = 64, tile_h: int = 0, small_max: int = -1):
        """tile x tile_h screen tiles (tile_h 0: square), threads per tile
        block and records per shared-memory pass of the fused batch kernel;
        small_max: bbox pixels up to which the setup kernel rasterises
        (negative: the library default)."""
        self.ctx = ctx
        o = abi.mr_server_opts(budget_bytes, slots, max_batch, tile, threads, chunk, tile_h, small_max)
        h = C.c_void_p()
        rc = capi.lib().mr_server_create(ctx.h, C.byref(o), C.byref(h))
        if rc != 0:
            raise capi.MRError(rc, "mr_server_create")
        self.h = h
        self._keep: Dict[int, tuple] = {}

    def submit(self, st: FrameState, mesh: TriMesh, mesh_key: int, transform=None,
               material: Optional[Material] = None, texture: Optional[np.ndarray] = None, texture_key: int = 0,
               outputs: int = abi.MR_OUT_DEFAULT, out: Optional[dict] = None) -> int:
        """Queues one frame of `mesh`; `out` may hold host arrays 'rgb8',
        'depth', 'ids' (page-locked for overlapped copies) to receive the result."""
        q = abi.mr_request()
        q.frame = st.to_c()
        q.mesh_key = mesh_key
        q.mesh = mesh.desc()
        xf = np.eye(4, dtype=np.float32) if transform is None else np.asarray(transform, np.float32)
        q.transform[:] = [float(x) for x in xf.reshape(16)]
        m = material or mesh.material or Material()
        q.material.diffuse[:] = [float(x) for x in m.diffuse]
        q.material.specular[:] = [float(x) for x in m.specular]
        q.material.emissive[:] = [float(x) for x in m.emissive]
        q.material.shininess = float(m.shininess)
        q.material.texture = -1
        tex = texture if texture is not None else (m.texture if m is not None else None)
        if tex is not None and texture_key:
            tex = np.asarray(tex)
            if tex.dtype != np.uint8 or tex.ndim != 3 or tex.shape[2] != 3:
                # requests carry RGB8 textures only; a cast would silently change float texels
                raise TypeError("render-server textures are (rows, cols, 3) uint8 RGB8 arrays")
            tex = np.ascontiguousarray(tex)
            q.texture_key = texture_key
            q.texture_rgb8 = tex.ctypes.data
            q.tex_rows, q.tex_cols = tex.shape[0], tex.shape[1]
        q.outputs = outputs
        out = out or {}
        for k, f in (("rgb8", "rgb8"), ("depth", "depth"), ("ids", "tri_id")):
            if k in out:
                setattr(q, f, out[k].ctypes.data)
        t = C.c_uint64()
        rc = capi.lib().mr_server_submit(self.h, C.byref(q), C.byref(t))
        if rc != 0:
            raise capi.MRError(rc, "mr_server_submit: " + capi.lib().mr_status_string(rc).decode())
        self._keep[t.value] = (q, mesh, tex, out)
        return t.value

    def wait(self, ticket: int, timeout_us: int = 60_000_000) -> abi.mr_request_info:
        info = abi.mr_request_info()
        rc = capi.lib().mr_server_wait(self.h, ticket, timeout_us, C.byref(info))
        if rc == abi.MR_E_NOT_READY:
            raise TimeoutError(f"request {ticket} not done")
        self._keep.pop(ticket, None)
        if rc != 0:
            raise capi.MRError(rc, "request failed")
        return info

    def stats(self) -> dict:
        s = abi.mr_server_stats()
        capi.lib().mr_server_get_stats(self.h, C.byref(s))
        return {k: getattr(s, k) for k, _ in abi.mr_server_stats._fields_}

    def reset_stats(self):
        capi.lib().mr_server_reset_stats(self.h)

    def close(self):
        if self.h:
            capi.lib().mr_server_destroy(self.h)
            self.h = None
