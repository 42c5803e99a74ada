"""Headless point rendering: the reference's Renderer (include/renderer.h:43-63) without a
graphics API.

The reference uploads (x - 0.5) * 1.8 per particle as clip-space positions
(``setParticlePositions``) and draws them as 2-pixel points of colour (0.59, 0.54, 0.2) on
an 800 x 600 window cleared to grey 0.1 (``shaders/cube_vertex.glsl``,
``shaders/constant_fragment.glsl``), with no depth test and no blending.  Here:

* :meth:`Renderer.positions` is that vertex buffer (``mpm_render_positions``);
* :meth:`Renderer.render` rasterises the points on the GPU into an RGB8 image (rows top to
  bottom): the pixels whose centres fall inside a point's square, for points inside the clip
  volume, take the point colour (``mpm_render_points``);
* :func:`write_ppm` writes an image file.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

WIDTH, HEIGHT = 800, 600          # src/renderer.cpp window and viewport
POINT_SIZE = 2.0                  # gl_PointSize, shaders/cube_vertex.glsl
COLOR = (0.59, 0.54, 0.2)         # FragColor, shaders/constant_fragment.glsl
BACKGROUND = (0.1, 0.1, 0.1)      # glClearColor, include/renderer.h:45


def unorm8(c) -> tuple:
    """Float colour to 8-bit unsigned normalised (round to nearest)."""
    return tuple(int(np.floor(np.float32(v) * np.float32(255.0) + np.float32(0.5))) for v in c)


class Renderer:
    def __init__(self, width: int = WIDTH, height: int = HEIGHT, point_size: float = POINT_SIZE, color=COLOR,
                 background=BACKGROUND):
        self.width, self.height, self.point_size = int(width), int(height), float(point_size)
        self.color = unorm8(color)
        self.background = unorm8(background)

    def positions(self, sim) -> np.ndarray:
        out = np.empty((max(sim.n, 1), 3), np.float32)
        _lib.check(sim.L.mpm_render_positions(sim.ctx, out.ctypes.data_as(ctypes.c_void_p)), sim.ctx)
        return out[:sim.n]

    def render(self, sim) -> np.ndarray:
        img = np.empty((self.height, self.width, 3), np.uint8)
        fg = (ctypes.c_uint8 * 3)(*self.color)
        bg = (ctypes.c_uint8 * 3)(*self.background)
        _lib.check(sim.L.mpm_render_points(sim.ctx, self.width, self.height, self.point_size, fg, bg,
                                           img.ctypes.data_as(ctypes.c_void_p)), sim.ctx)
        return img


def write_ppm(path: str, img: np.ndarray) -> None:
    """Binary PPM (P6) of an (H, W, 3) uint8 image."""
    h, w, _ = img.shape
    with open(path, "wb") as f:
        f.write(f"P6 {w} {h} 255\n".encode())
        f.write(np.ascontiguousarray(img, np.uint8).tobytes())
