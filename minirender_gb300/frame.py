"""Renderer state that one frame reads (src/Renderer.cpp:311-332), as a plain
record convertible to the C-ABI's ``mr_frame``."""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import abi


def _v(x, n):
    return np.asarray(x, np.float32).reshape(n)


@dataclass
class FrameState:
    width: int = 800                     # Renderer::setSize(800, 600), src/Renderer.cpp:87
    height: int = 600
    projection: np.ndarray = None        # default projectionOrtho(-40,40,-30,30,50,120), :88
    view: np.ndarray = field(default_factory=lambda: np.eye(4, dtype=np.float32))
    light: np.ndarray = None             # default Vec3(-0.15,0.6,1).normalized(), :89
    light_is_point: bool = False
    ambient: float = 0.1                 # Scene::ambientLight, src/Scene.cpp:75
    background: np.ndarray = field(default_factory=lambda: np.zeros(3, np.float32))
    lighting: bool = True
    texturing: bool = True
    save_normals: bool = False

    def to_c(self) -> abi.mr_frame:
        f = abi.mr_frame()
        f.width = int(self.width)
        f.height = int(self.height)
        proj = self.projection
        if proj is None:
            from .projection import projection_ortho
            proj = projection_ortho(-40, 40, -30, 30, 50, 120)
        f.projection[:] = [float(x) for x in _v(proj, 16)]
        f.view[:] = [float(x) for x in _v(self.view, 16)]
        light = self.light
        if light is None:
            l = np.array([-0.15, 0.6, 1.0], np.float32)
            ln = np.float32(math.sqrt(float(l[0] * l[0] + l[1] * l[1] + l[2] * l[2])))
            light = l / ln
        f.light[:] = [float(x) for x in _v(light, 3)]
        f.light_is_point = int(bool(self.light_is_point))
        f.ambient = float(np.float32(self.ambient))
        f.background[:] = [float(x) for x in _v(self.background, 3)]
        f.lighting = int(bool(self.lighting))
        f.texturing = int(bool(self.texturing))
        f.save_normals = int(bool(self.save_normals))
        return f
