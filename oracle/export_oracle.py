"""CPU oracle of particle export and headless point rendering — TEST INFRASTRUCTURE ONLY
(the checker of the GPU packer and rasteriser; the product never imports it).

* :func:`bgeo_file` restates the file the reference's ParticleWriter produces through Partio
  (include/particle_writer.h:19-43: attributes id, position, velocity, radius = 0.1, in
  that order): Houdini classic binary geometry version 5 as Partio's writer lays it out —
  big-endian magic "Bgeo", 'V', version 5, point / primitive / group / attribute counts, one
  definition (name, size, type, zero defaults) per non-position attribute, then per point
  P = (x, y, z, 1) and the attributes in definition order, then the bytes 0x00 0xff.
  Partio is not vendored by the reference (its CMake file looks for an installed library,
  no version pinned) and is absent here; the layout is restated from its published writer.
  :func:`parse_bgeo` reads it back.
* :func:`render_points` restates the reference's OpenGL point drawing
  (include/renderer.h:43-63, shaders/cube_vertex.glsl: clip position (x - 0.5) * 1.8, w = 1;
  gl_PointSize 2; one constant colour, no depth test, no blending) as the GPU rasteriser
  defines it: a point inside the clip volume covers the pixels whose centres fall in the
  half-open square of side point_size around its window position.  float32 arithmetic,
  operation for operation.  No graphics stack exists here to pin it against.
"""
from __future__ import annotations

import gzip
import struct

import numpy as np

RECORD = np.dtype([("P", ">f4", 4), ("id", ">i4"), ("velocity", ">f4", 3), ("radius", ">f4")])
ATTRS = (("id", 1, 1), ("velocity", 3, 5), ("radius", 1, 0))  # name, size, type (0 float, 1 int, 5 vector)


def bgeo_header(n: int) -> bytes:
    h = struct.pack(">4scI", b"Bgeo", b"V", 5)
    # points, primitives, point groups, primitive groups, point / vertex / primitive / detail attributes
    h += struct.pack(">8I", n, 0, 0, 0, len(ATTRS), 0, 0, 0)
    for name, size, typ in ATTRS:
        h += struct.pack(">H", len(name)) + name.encode() + struct.pack(">HI", size, typ) + b"\0" * (4 * size)
    return h


def bgeo_records(x: np.ndarray, v: np.ndarray, radius: float = 0.1) -> bytes:
    n = len(x)
    r = np.zeros(n, RECORD)
    r["P"][:, :3] = np.asarray(x, np.float32)
    r["P"][:, 3] = 1.0
    r["id"] = np.arange(n, dtype=np.int32)
    r["velocity"] = np.asarray(v, np.float32)
    r["radius"] = np.float32(radius)
    return r.tobytes()


def bgeo_file(x: np.ndarray, v: np.ndarray, radius: float = 0.1) -> bytes:
    return bgeo_header(len(x)) + bgeo_records(x, v, radius) + b"\x00\xff"


def parse_bgeo(data: bytes) -> dict:
    if data[:2] == b"\x1f\x8b":
        data = gzip.decompress(data)
    magic, ver_c, ver = struct.unpack_from(">4scI", data, 0)
    assert magic == b"Bgeo" and ver_c == b"V" and ver == 5, (magic, ver_c, ver)
    counts = struct.unpack_from(">8I", data, 9)
    n, n_pt_attr = counts[0], counts[4]
    off = 9 + 32
    attrs = []
    for _ in range(n_pt_attr):
        (ln,) = struct.unpack_from(">H", data, off)
        name = data[off + 2:off + 2 + ln].decode()
        size, typ = struct.unpack_from(">HI", data, off + 2 + ln)
        off += 2 + ln + 6 + 4 * size
        attrs.append((name, size, typ))
    rec = np.frombuffer(data, RECORD, count=n, offset=off)
    tail = data[off + RECORD.itemsize * n:]
    return {"n": n, "counts": counts, "attrs": attrs, "records": rec, "tail": tail}


def positions(x: np.ndarray) -> np.ndarray:
    """(x - 0.5) * 1.8 in float32 (Renderer::setParticlePositions)."""
    x = np.asarray(x, np.float32)
    return (x - np.float32(0.5)) * np.float32(1.8)


def render_points(x: np.ndarray, W: int = 800, H: int = 600, size: float = 2.0, fg=(150, 138, 51),
                  bg=(26, 26, 26)) -> np.ndarray:
    f32 = np.float32
    img = np.empty((H, W, 3), np.uint8)
    img[:] = bg
    p = positions(x)
    inside = np.all(np.abs(p) <= f32(1.0), axis=1)
    p = p[inside]
    h = f32(0.5) * f32(size)
    xw = (p[:, 0] + f32(1.0)) * f32(0.5 * W)
    yw = (p[:, 1] + f32(1.0)) * f32(0.5 * H)
    i0 = np.maximum(0, np.ceil((xw - h) - f32(0.5)).astype(np.int64))
    i1 = np.minimum(W - 1, np.ceil((xw + h) - f32(0.5)).astype(np.int64) - 1)
    j0 = np.maximum(0, np.ceil((yw - h) - f32(0.5)).astype(np.int64))
    j1 = np.minimum(H - 1, np.ceil((yw + h) - f32(0.5)).astype(np.int64) - 1)
    mask = np.zeros((H, W), bool)
    span = int(np.ceil(size)) + 1
    for dj in range(span):
        for di in range(span):
            i, j = i0 + di, j0 + dj
            ok = (i <= i1) & (j <= j1)
            mask[H - 1 - j[ok], i[ok]] = True
    img[mask] = fg
    return img
