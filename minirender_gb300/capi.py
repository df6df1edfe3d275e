"""ctypes binding of include/minirender_gpu.h (libminirender_gpu.so).

There is no CPU fallback: if the library is missing or no CUDA device is
present, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import abi
from .build import LIB

_lib = None

_P = C.c_void_p
_I = C.c_int32
_F = C.c_float

_SIGS = {
    "mr_abi_version": ([], C.c_int),
    "mr_status_string": ([C.c_int], C.c_char_p),
    "mr_last_error": ([_P], C.c_char_p),
    "mr_create": ([C.c_int, C.POINTER(_P)], C.c_int),
    "mr_destroy": ([_P], C.c_int),
    "mr_set_stream": ([_P, _P], C.c_int),
    "mr_synchronize": ([_P], C.c_int),
    "mr_set_upload_stream": ([_P, _P], C.c_int),
    "mr_set_tuning": ([_P, C.c_int, C.c_int], C.c_int),
    "mr_set_profiling": ([_P, C.c_int], C.c_int),
    "mr_mesh_upload": ([_P, C.POINTER(abi.mr_mesh_desc), C.POINTER(_I)], C.c_int),
    "mr_mesh_update": ([_P, _I, C.POINTER(abi.mr_mesh_desc)], C.c_int),
    "mr_mesh_free": ([_P, _I], C.c_int),
    "mr_texture_upload_rgb8": ([_P, _P, _I, _I, C.POINTER(_I)], C.c_int),
    "mr_texture_upload_f32": ([_P, _P, _I, _I, C.POINTER(_I)], C.c_int),
    "mr_texture_update": ([_P, _I, _P], C.c_int),
    "mr_texture_free": ([_P, _I], C.c_int),
    "mr_render": ([_P, C.POINTER(abi.mr_frame), _P, _I, _I], C.c_int),
    "mr_read": ([_P, _P, _P, _P, _P, _P], C.c_int),
    "mr_read_async": ([_P, _P, _P, _P, _P, _P], C.c_int),
    "mr_wait": ([_P], C.c_int),
    "mr_get_outputs": ([_P, C.POINTER(abi.mr_outputs)], C.c_int),
    "mr_get_stats": ([_P, C.POINTER(abi.mr_stats)], C.c_int),
    "mr_read_range_image": ([_P, _P], C.c_int),
    "mr_render_noalloc": ([C.POINTER(abi.mr_frame), C.POINTER(abi.mr_mesh_desc), _P,
                           C.POINTER(abi.mr_material), _P, _I, _I, _I, _P, _P, _P, _P], C.c_int),
    "mr_set_batch_tuning": ([_P, C.c_int, C.c_int, C.c_int], C.c_int),
    "mr_set_batch_tiling": ([_P, C.c_int, C.c_int, C.c_int, C.c_int], C.c_int),
    "mr_set_batch_small_max": ([_P, C.c_int], C.c_int),
    "mr_model_load": ([C.c_char_p, _P], C.c_int),
    "mr_model_counts": ([_P, _P, _P, _P], C.c_int),
    "mr_model_nodes": ([_P, _P, C.c_int32], C.c_int),
    "mr_model_mesh": ([_P, C.c_int32, _P], C.c_int),
    "mr_model_texture": ([_P, C.c_int32, _P, _P, _P], C.c_int),
    "mr_model_free": ([_P], None),
    "mr_ppm_load": ([C.c_char_p, _P, C.c_int64, _P, _P], C.c_int),
    "mr_ppm_save": ([C.c_char_p, _P, C.c_int32, C.c_int32], C.c_int),
    "mr_stl_save": ([C.c_char_p, _P, _P], C.c_int),
    "mr_xyz_save": ([C.c_char_p, _P, C.c_int32, C.c_int32, _P], C.c_int),
    "mr_set_batch_graphs": ([_P, C.c_int], C.c_int),
    "mr_render_batch": ([_P, _P, _I, _P, _I, _I], C.c_int),
    "mr_read_batch": ([_P, _I, _P, _P, _P], C.c_int),
    "mr_get_batch_outputs": ([_P, _I, C.POINTER(abi.mr_outputs)], C.c_int),
    "mr_get_batch_stats": ([_P, C.POINTER(abi.mr_stats)], C.c_int),
    "mr_server_create": ([_P, C.POINTER(abi.mr_server_opts), C.POINTER(_P)], C.c_int),
    "mr_server_submit": ([_P, C.POINTER(abi.mr_request), C.POINTER(C.c_uint64)], C.c_int),
    "mr_server_wait": ([_P, C.c_uint64, C.c_int64, C.POINTER(abi.mr_request_info)], C.c_int),
    "mr_server_get_stats": ([_P, C.POINTER(abi.mr_server_stats)], C.c_int),
    "mr_server_reset_stats": ([_P], C.c_int),
    "mr_server_destroy": ([_P], C.c_int),
    "mr_collect_shapes": ([_P, _I, _P, _I, C.POINTER(_I)], C.c_int),
    "mr_mat4_mul": ([_P, _P, _P], None),
    "mr_mat4_inverse": ([_P, _P], None),
    "mr_projection_ortho": ([_F] * 6 + [_P], None),
    "mr_projection_perspective": ([_F] * 6 + [_P], None),
    "mr_projection_frustum": ([_F] * 4 + [_P], None),
    "mr_projection_frustum_h": ([_F] * 4 + [_P], None),
    "mr_projection_ortho_fov": ([_F] * 4 + [_P], None),
    "mr_projection_cv": ([_P, _F, _F, _F, _F, _P], None),
}


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError("libminirender_gpu.so is not built; run minirender_gb300.build.build()")
        L = C.CDLL(LIB)
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def declared_symbols():
    return list(_SIGS)


class MRError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{msg} (status {code})")
        self.code = code


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


class Context:
    """One mr_ctx: resident meshes/textures and frame buffers on one GPU."""

    def __init__(self, device: int = 0):
        h = _P()
        rc = lib().mr_create(device, C.byref(h))
        if rc != 0:
            raise MRError(rc, "mr_create: " + lib().mr_status_string(rc).decode())
        self.h = h
        self._frame_hw = None
        self._tex_layout = {}  # texture handle -> (dtype, shape) the library reads on update

    def _check(self, rc: int, what: str) -> int:
        if rc != 0:
            raise MRError(rc, f"{what}: {lib().mr_last_error(self.h).decode()}")
        return rc

    def close(self):
        if self.h:
            lib().mr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tuning(self, tile: int, small_max: int):
        self._check(lib().mr_set_tuning(self.h, tile, small_max), "mr_set_tuning")

    def set_profiling(self, on: bool):
        self._check(lib().mr_set_profiling(self.h, int(on)), "mr_set_profiling")

    def set_stream(self, stream_ptr: int):
        self._check(lib().mr_set_stream(self.h, stream_ptr), "mr_set_stream")

    def set_upload_stream(self, stream_ptr: Optional[int]):
        """Stream for mesh / texture updates (None: the context's own)."""
        self._check(lib().mr_set_upload_stream(self.h, stream_ptr), "mr_set_upload_stream")

    def synchronize(self):
        self._check(lib().mr_synchronize(self.h), "mr_synchronize")

    def upload_mesh(self, desc: abi.mr_mesh_desc) -> int:
        out = _I()
        self._check(lib().mr_mesh_upload(self.h, C.byref(desc), C.byref(out)), "mr_mesh_upload")
        return out.value

    def update_mesh(self, handle: int, desc: abi.mr_mesh_desc):
        self._check(lib().mr_mesh_update(self.h, handle, C.byref(desc)), "mr_mesh_update")

    def free_mesh(self, handle: int):
        self._check(lib().mr_mesh_free(self.h, handle), "mr_mesh_free")

    def upload_texture(self, tex: np.ndarray) -> int:
        out = _I()
        if tex.ndim != 3 or tex.shape[2] != 3:
            raise ValueError(f"textures are (rows, cols, 3) arrays, got shape {tex.shape}")
        if tex.dtype == np.uint8:
            t = np.ascontiguousarray(tex)
            rc = lib().mr_texture_upload_rgb8(self.h, _ptr(t), t.shape[0], t.shape[1], C.byref(out))
        else:
            t = np.ascontiguousarray(tex, np.float32)
            rc = lib().mr_texture_upload_f32(self.h, _ptr(t), t.shape[0], t.shape[1], C.byref(out))
        self._check(rc, "mr_texture_upload")
        self._tex_layout[out.value] = (t.dtype, t.shape)
        return out.value

    def update_texture(self, handle: int, tex: np.ndarray):
        """Re-sends a texture's texels; the library reads rows x cols x 3
        elements of the upload's type from the array, so it must match."""
        want = self._tex_layout.get(handle)
        if want is not None and (tex.dtype != want[0] or tex.shape != want[1] or not tex.flags.c_contiguous):
            raise ValueError(f"texture {handle} was uploaded as {want[1]} {want[0]}; "
                             f"got {tex.shape} {tex.dtype} (contiguous: {tex.flags.c_contiguous})")
        self._check(lib().mr_texture_update(self.h, handle, _ptr(tex)), "mr_texture_update")

    def free_texture(self, handle: int):
        self._check(lib().mr_texture_free(self.h, handle), "mr_texture_free")
        self._tex_layout.pop(handle, None)

    def render(self, frame: abi.mr_frame, renderables, n: int, outputs: int = abi.MR_OUT_DEFAULT):
        self._frame_hw = (frame.height, frame.width)
        self._outputs = outputs
        self._save_normals = bool(frame.save_normals)
        self._check(lib().mr_render(self.h, C.byref(frame), C.addressof(renderables) if n else None,
                                    n, outputs), "mr_render")

    def _hw(self):
        if self._frame_hw is None:
            raise RuntimeError("no frame has been rendered on this context")
        return self._frame_hw

    def read(self, rgb8=True, depth=True, rgb_f32=False, tri_id=True, normals=False,
             allow_bad_index: bool = False) -> dict:
        H, W = self._hw()
        out = {}
        if rgb8:
            out["rgb8"] = np.empty((H, W, 3), np.uint8)
        if depth:
            out["depth"] = np.empty((H, W), np.float32)
        if rgb_f32:
            out["image"] = np.empty((H, W, 3), np.float32)
        if tri_id:
            out["ids"] = np.empty((H, W), np.uint32)
        if normals:
            out["normals"] = np.empty((H, W, 3), np.float32)
        rc = lib().mr_read(self.h, _ptr(out.get("rgb8")), _ptr(out.get("depth")),
                           _ptr(out.get("image")), _ptr(out.get("ids")), _ptr(out.get("normals")))
        if rc == abi.MR_E_BAD_INDEX and allow_bad_index:
            out["bad_index"] = True
            return out
        self._check(rc, "mr_read")
        return out

    def read_into(self, rgb8: Optional[np.ndarray], depth: Optional[np.ndarray]) -> None:
        """D2H of RGB8 and depth into caller-owned (e.g. pinned) arrays."""
        self._check(lib().mr_read(self.h, _ptr(rgb8), _ptr(depth), None, None, None), "mr_read")

    def read_async(self, rgb8: Optional[np.ndarray], depth: Optional[np.ndarray],
                   tri_id: Optional[np.ndarray] = None) -> None:
        """Queues the D2H of RGB8, depth (and triangle ids) into caller-owned
        (pinned, for an asynchronous copy) arrays; wait() -- or the next
        read, render or stats call -- completes it."""
        if self._frame_hw is not None:  # the library writes a whole frame into each array
            H, W = self._frame_hw
            for a, dt, n, name in ((rgb8, np.uint8, 3 * H * W, "rgb8"), (depth, np.float32, H * W, "depth"),
                                   (tri_id, np.uint32, H * W, "tri_id")):
                if a is not None and (a.dtype != dt or a.size != n or not a.flags.c_contiguous):
                    raise ValueError(f"{name}: want {n} contiguous {np.dtype(dt)}, got {a.size} {a.dtype} "
                                     f"(contiguous: {a.flags.c_contiguous})")
        self._check(lib().mr_read_async(self.h, _ptr(rgb8), _ptr(depth), None, _ptr(tri_id), None),
                    "mr_read_async")

    def wait(self) -> int:
        """Completes the last frame and any queued reads; returns 0 or
        MR_E_BAD_INDEX (raises on other errors)."""
        rc = lib().mr_wait(self.h)
        if rc not in (0, abi.MR_E_BAD_INDEX):
            self._check(rc, "mr_wait")
        return rc

    def range_image(self) -> np.ndarray:
        H, W = self._hw()
        out = np.empty((H, W, 3), np.float32)
        self._check(lib().mr_read_range_image(self.h, _ptr(out)), "mr_read_range_image")
        return out

    def stats(self) -> abi.mr_stats:
        s = abi.mr_stats()
        rc = lib().mr_get_stats(self.h, C.byref(s))
        if rc not in (0, abi.MR_E_BAD_INDEX):
            self._check(rc, "mr_get_stats")
        return s

    # ---- batches
    def set_batch_tuning(self, tile: int, threads: int, chunk: int):
        self._check(lib().mr_set_batch_tuning(self.h, tile, threads, chunk), "mr_set_batch_tuning")

    def set_batch_tiling(self, tile_w: int, tile_h: int, threads: int, chunk: int):
        self._check(lib().mr_set_batch_tiling(self.h, tile_w, tile_h, threads, chunk), "mr_set_batch_tiling")

    def set_batch_small_max(self, small_max: int):
        self._check(lib().mr_set_batch_small_max(self.h, small_max), "mr_set_batch_small_max")

    def set_batch_graphs(self, on: bool):
        self._check(lib().mr_set_batch_graphs(self.h, int(on)), "mr_set_batch_graphs")

    def render_batch(self, scenes, n_scenes: int, renderables, n_rs: int,
                     outputs: int = abi.MR_OUT_DEFAULT):
        self._batch_hw = [(scenes[i].frame.height, scenes[i].frame.width) for i in range(n_scenes)]
        self._check(lib().mr_render_batch(self.h, C.addressof(scenes), n_scenes,
                                          C.addressof(renderables) if n_rs else None, n_rs, outputs),
                    "mr_render_batch")

    def read_batch(self, scene: int, rgb8=True, depth=True, tri_id=True) -> dict:
        H, W = self._batch_hw[scene]
        out = {}
        if rgb8:
            out["rgb8"] = np.empty((H, W, 3), np.uint8)
        if depth:
            out["depth"] = np.empty((H, W), np.float32)
        if tri_id:
            out["ids"] = np.empty((H, W), np.uint32)
        self._check(lib().mr_read_batch(self.h, scene, _ptr(out.get("rgb8")), _ptr(out.get("depth")),
                                        _ptr(out.get("ids"))), "mr_read_batch")
        return out

    def batch_stats(self) -> abi.mr_stats:
        s = abi.mr_stats()
        rc = lib().mr_get_batch_stats(self.h, C.byref(s))
        if rc not in (0, abi.MR_E_BAD_INDEX):
            self._check(rc, "mr_get_batch_stats")
        return s

    def outputs(self) -> abi.mr_outputs:
        o = abi.mr_outputs()
        self._check(lib().mr_get_outputs(self.h, C.byref(o)), "mr_get_outputs")
        return o


def collect_shapes(nodes) -> tuple:
    """Scene::collectShapes through the library's host helper."""
    n_nodes = len(nodes)
    out = (abi.mr_renderable * max(1, n_nodes))()
    n = _I(0)
    rc = lib().mr_collect_shapes(C.addressof(nodes), n_nodes, C.addressof(out), n_nodes, C.byref(n))
    if rc != 0:
        raise MRError(rc, "mr_collect_shapes")
    return out, n.value


def mat4_mul(a, b) -> np.ndarray:
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    out = np.empty(16, np.float32)
    lib().mr_mat4_mul(_ptr(a), _ptr(b), _ptr(out))
    return out.reshape(4, 4)


def mat4_inverse(a) -> np.ndarray:
    a = np.ascontiguousarray(a, np.float32)
    out = np.empty(16, np.float32)
    lib().mr_mat4_inverse(_ptr(a), _ptr(out))
    return out.reshape(4, 4)


def projection(kind: str, *args) -> np.ndarray:
    out = np.empty(16, np.float32)
    fn = {"ortho": lib().mr_projection_ortho, "perspective": lib().mr_projection_perspective,
          "frustum": lib().mr_projection_frustum, "frustum_h": lib().mr_projection_frustum_h,
          "ortho_fov": lib().mr_projection_ortho_fov}[kind]
    fn(*[float(a) for a in args], _ptr(out))
    return out.reshape(4, 4)
