"""CPU tests of particle export and point rendering: the library's .bgeo header and file
writer against the oracle's restatement of Partio's layout (include/particle_writer.h:19-43),
the oracle's reader, and the oracle rasteriser on hand-checked points."""
import gzip

import numpy as np
import pytest


def _lib():
    from mpm_gb300 import build

    build.build()
    from mpm_gb300 import _lib as L

    return L


def test_header_matches_oracle():
    from mpm_gb300.particle_writer import bgeo_header

    from oracle import export_oracle as E

    _lib()
    for n in (0, 1, 123456789):
        assert bgeo_header(n) == E.bgeo_header(n)


def test_write_bgeo_file_matches_oracle(tmp_path):
    import ctypes

    from oracle import export_oracle as E

    L = _lib().lib()
    rng = np.random.default_rng(0)
    x, v = rng.random((1000, 3), dtype=np.float32), rng.normal(size=(1000, 3)).astype(np.float32)
    rec = np.frombuffer(E.bgeo_records(x, v), np.uint8).copy()
    p = tmp_path / "particles_0.bgeo"
    assert L.mpm_write_bgeo(str(p).encode(), rec.ctypes.data_as(ctypes.c_void_p), 1000) == 0
    data = p.read_bytes()
    assert data == E.bgeo_file(x, v)
    f = E.parse_bgeo(data)
    assert f["n"] == 1000 and [a[0] for a in f["attrs"]] == ["id", "velocity", "radius"]
    assert np.array_equal(f["records"]["P"][:, :3], x) and np.all(f["records"]["P"][:, 3] == 1)
    assert np.array_equal(f["records"]["id"], np.arange(1000)) and np.all(f["records"]["radius"] == np.float32(0.1))
    assert f["tail"] == b"\x00\xff"
    # the gzip form the reference writes reads back the same
    g = E.parse_bgeo(gzip.compress(data))
    assert np.array_equal(g["records"], f["records"])
    # unwritable path
    assert L.mpm_write_bgeo(str(tmp_path / "missing" / "x.bgeo").encode(), rec.ctypes.data_as(ctypes.c_void_p),
                            1000) == 7


def test_render_oracle_points():
    from mpm_gb300.renderer import BACKGROUND, COLOR, unorm8

    from oracle import export_oracle as E

    assert unorm8(COLOR) == (150, 138, 51) and unorm8(BACKGROUND) == (26, 26, 26)
    # x = 0.5 maps to clip 0 -> window (400, 300): pixels 399..400 x 299..300 (rows flipped)
    img = E.render_points(np.array([[0.5, 0.5, 0.5]], np.float32))
    lit = np.argwhere(np.all(img == (150, 138, 51), axis=2))
    assert sorted(map(tuple, lit)) == [(299, 399), (299, 400), (300, 399), (300, 400)]
    # outside the clip volume (x < 0.5 - 1 / 1.8): nothing drawn
    img = E.render_points(np.array([[-0.1, 0.5, 0.5], [0.5, 0.5, 1.2]], np.float32))
    assert np.all(img == 26)
    # the lower-left corner of the clip volume: one pixel left of the square survives
    img = E.render_points(np.array([[0.5 - 1 / 1.8 + 1e-6, 0.5 - 1 / 1.8 + 1e-6, 0.5]], np.float32))
    assert np.all(img[599, 0] == (150, 138, 51)) and (img == 150).sum() == 1
