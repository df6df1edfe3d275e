"""ctypes mirror of the structs in include/minirender_gpu.h.

The layouts here must match the C header field for field; a CPU test checks
the sizes against the compiled library's expectations.
"""
import ctypes as C

MR_OK = 0
MR_E_INVALID = -1
MR_E_CUDA = -2
MR_E_NOMEM = -3
MR_E_HANDLE = -4
MR_E_BAD_INDEX = -5
MR_E_BUDGET = -6
MR_E_TIMEOUT = -7
MR_E_NOT_READY = -8
MR_E_NO_DEVICE = -9
MR_E_NOALLOC_LIMIT = -10
MR_E_IO = -11
MR_NOALLOC_MAX_SIDE = 4096
MR_NOALLOC_MAX_PIXELS = 1 << 21
MR_NOALLOC_MAX_TRIANGLES = 1 << 22
MR_NO_TRIANGLE = 0xFFFFFFFF
MR_RS_MODELVIEW = 1  # mr_renderable.flags: transform is the modelview
MR_RS_NO_CLIP = 2    # mr_renderable.flags: no near-plane clipping
MR_RS_OWN_STATE = 4  # mr_renderable.flags: the three switches below replace the frame's
MR_RS_LIGHTING = 8
MR_RS_TEXTURING = 16
MR_RS_POINT_LIGHT = 32

MR_OUT_RGB8 = 1
MR_OUT_DEPTH = 2
MR_OUT_RGB_F32 = 4
MR_OUT_TRI_ID = 8
MR_OUT_DEFAULT = MR_OUT_RGB8 | MR_OUT_DEPTH | MR_OUT_TRI_ID

F3 = C.c_float * 3
F16 = C.c_float * 16


class mr_material(C.Structure):
    _fields_ = [("diffuse", F3), ("specular", F3), ("emissive", F3),
                ("shininess", C.c_float), ("texture", C.c_int32)]


class mr_mesh_desc(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("n_vertices", C.c_int32),
                ("normals", C.c_void_p), ("n_normals", C.c_int32),
                ("texcoords", C.c_void_p), ("n_texcoords", C.c_int32),
                ("indices", C.c_void_p), ("n_indices", C.c_int32),
                ("normalsI", C.c_void_p), ("n_normalsI", C.c_int32),
                ("texcoordsI", C.c_void_p), ("n_texcoordsI", C.c_int32)]


class mr_renderable(C.Structure):
    _fields_ = [("mesh", C.c_int32), ("flags", C.c_int32), ("transform", F16),
                ("material", mr_material)]


class mr_node(C.Structure):
    _fields_ = [("parent", C.c_int32), ("mesh", C.c_int32), ("transform", F16),
                ("has_material", C.c_int32), ("material", mr_material), ("opacity", C.c_float)]


class mr_frame(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32),
                ("projection", F16), ("view", F16),
                ("light", F3), ("light_is_point", C.c_int32),
                ("ambient", C.c_float), ("background", F3),
                ("lighting", C.c_int32), ("texturing", C.c_int32),
                ("save_normals", C.c_int32)]


class mr_outputs(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32),
                ("rgb8", C.c_void_p), ("depth", C.c_void_p), ("rgb_f32", C.c_void_p),
                ("tri_id", C.c_void_p), ("normals", C.c_void_p)]


class mr_stats(C.Structure):
    _fields_ = [("triangles", C.c_int64), ("clipped", C.c_int64), ("rasterised", C.c_int64),
                ("small_direct", C.c_int64), ("binned", C.c_int64), ("bin_entries", C.c_int64),
                ("error_flags", C.c_int64), ("stage_ms", C.c_float * 8), ("n_stages", C.c_int32)]


class mr_batch_scene(C.Structure):
    _fields_ = [("frame", mr_frame), ("first_renderable", C.c_int32), ("n_renderables", C.c_int32)]


class mr_server_opts(C.Structure):
    _fields_ = [("budget_bytes", C.c_uint64), ("slots", C.c_int32), ("max_batch", C.c_int32),
                ("tile", C.c_int32), ("threads", C.c_int32), ("chunk", C.c_int32), ("tile_h", C.c_int32),
                ("small_max", C.c_int32)]


class mr_request(C.Structure):
    _fields_ = [("frame", mr_frame), ("mesh_key", C.c_uint64), ("mesh", mr_mesh_desc), ("transform", F16),
                ("material", mr_material), ("texture_key", C.c_uint64), ("texture_rgb8", C.c_void_p),
                ("tex_rows", C.c_int32), ("tex_cols", C.c_int32), ("outputs", C.c_int32),
                ("rgb8", C.c_void_p), ("depth", C.c_void_p), ("tri_id", C.c_void_p)]


class mr_request_info(C.Structure):
    _fields_ = [("status", C.c_int32), ("batch_size", C.c_int32), ("queue_us", C.c_double),
                ("latency_us", C.c_double)]


class mr_server_stats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("rejected", C.c_int64),
                ("batches", C.c_int64), ("in_queue", C.c_int64), ("in_flight", C.c_int64),
                ("mean_batch", C.c_double), ("p50_us", C.c_double), ("p99_us", C.c_double),
                ("max_us", C.c_double), ("frames_per_s", C.c_double), ("resident_bytes", C.c_uint64),
                ("committed_bytes", C.c_uint64)]
