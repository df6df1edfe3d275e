"""Host-side request checks of the render server mirror
(minirender_gb300/server.py) that run before any device call."""
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
