"""Host-side argument checks of the Python mirrors that run before any
device call: render-server requests (minirender_gb300/server.py) and the
context's texture and read targets (minirender_gb300/capi.py)."""
import numpy as np
import pytest

from minirender_gb300 import workloads as W
from minirender_gb300.server import RenderServer


@pytest.mark.parametrize("tex", [np.zeros((4, 4, 3), np.float32), np.zeros((4, 4), np.uint8),
                                 np.zeros((4, 4, 4), np.uint8)])
def test_non_rgb8_texture_is_refused(tex):
    srv = RenderServer.__new__(RenderServer)  # no device: the check precedes the C call
    st, sc = W.config1(32, 24)
    with pytest.raises(TypeError):
        srv.submit(st, sc.children[0], mesh_key=1, texture=tex, texture_key=2)


def test_context_texture_layout_checks():
    """Context.upload_texture / update_texture refuse arrays the library
    would read past (checked before any device call)."""
    from minirender_gb300 import capi
    ctx = capi.Context.__new__(capi.Context)  # no device
    ctx.h = None
    ctx._tex_layout = {7: (np.dtype(np.uint8), (4, 5, 3))}
    with pytest.raises(ValueError):
        ctx.upload_texture(np.zeros((4, 5), np.uint8))
    for bad in (np.zeros((4, 5, 3), np.float32), np.zeros((5, 4, 3), np.uint8),
                np.zeros((4, 10, 3), np.uint8)[:, ::2]):
        with pytest.raises(ValueError):
            ctx.update_texture(7, bad)


def test_read_async_target_checks():
    """read_async refuses targets smaller than the frame or of the wrong type."""
    from minirender_gb300 import capi
    ctx = capi.Context.__new__(capi.Context)  # no device
    ctx.h = None
    ctx._frame_hw = (6, 8)
    ok8, okd = np.zeros((6, 8, 3), np.uint8), np.zeros((6, 8), np.float32)
    for bad in ((np.zeros((6, 7, 3), np.uint8), okd), (ok8, np.zeros((6, 8), np.float64)),
                (ok8, okd, np.zeros((6, 8), np.int64)), (np.zeros((8, 6, 6), np.uint8)[:, :, ::2], okd)):
        with pytest.raises(ValueError):
            ctx.read_async(*bad)


def test_read_before_render_is_an_error():
    from minirender_gb300 import capi
    ctx = capi.Context.__new__(capi.Context)  # no device
    ctx.h = None
    ctx._frame_hw = None
    with pytest.raises(RuntimeError):
        ctx.read()
    with pytest.raises(RuntimeError):
        ctx.range_image()
