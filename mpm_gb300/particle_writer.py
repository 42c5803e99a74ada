"""Particle export: the reference's ParticleWriter (include/particle_writer.h:19-43).

The reference writes every saved frame (src/main.cu:108-111) with Partio as
``particles_<frame>.bgeo``: per active particle its index ``id``, ``position``,
``velocity`` and ``radius`` 0.1, gzip-compressed.  Here the point records of that file are
packed on the GPU straight from the particle arrays and copied to pinned host memory on a
copy stream (``mpm_export_particles``), so the simulation keeps running while a frame is
copied and written:

* :class:`ParticleWriter` ``.writeParticles(path, sim)`` writes one frame synchronously.
* :class:`AsyncParticleWriter` ``.submit(path, sim)`` starts the export and returns at once;
  a background thread waits for the copy and writes the file while the caller advances the
  simulation.  Two slots alternate, so at most two frames are in flight.

Files are uncompressed unless ``compress=True`` (gzip, as the reference's
``Partio::write(path, data, true)``); readers of the format accept both.
"""
from __future__ import annotations

import ctypes
import gzip
import threading
from concurrent.futures import ThreadPoolExecutor

from . import _lib

RECORD_BYTES = 36
RADIUS = 0.1  # include/particle_writer.h:29


def bgeo_header(n: int) -> bytes:
    L = _lib.lib()
    size = L.mpm_bgeo_header(int(n), None, 0)
    buf = ctypes.create_string_buffer(size)
    L.mpm_bgeo_header(int(n), buf, size)
    return buf.raw


def _write(path: str, ptr: int, n: int, compress: bool):
    L = _lib.lib()
    if not compress:
        code = L.mpm_write_bgeo(str(path).encode(), ctypes.c_void_p(ptr), int(n))
        if code != 0:
            raise _lib.MpmError(code, f"cannot write {path}")
        return
    data = ctypes.string_at(ptr, RECORD_BYTES * n) if n else b""
    with gzip.open(path, "wb", compresslevel=1) as f:
        f.write(bgeo_header(n))
        f.write(data)
        f.write(b"\x00\xff")


def export_records(sim, slot: int = 0, radius: float = RADIUS):
    """Start the export of the active particles into slot; returns the particle count."""
    n = ctypes.c_int64()
    _lib.check(sim.L.mpm_export_particles(sim.ctx, int(slot), float(radius), ctypes.byref(n)), sim.ctx)
    return int(n.value)


def wait_records(sim, slot: int = 0):
    """(pointer, count) of slot's records in pinned host memory once copied."""
    ptr, n = ctypes.c_void_p(), ctypes.c_int64()
    _lib.check(sim.L.mpm_export_wait(sim.ctx, int(slot), ctypes.byref(ptr), ctypes.byref(n)), sim.ctx)
    return ptr.value or 0, int(n.value)


def records_bytes(sim, slot: int = 0) -> bytes:
    ptr, n = wait_records(sim, slot)
    return ctypes.string_at(ptr, RECORD_BYTES * n) if n else b""


class ParticleWriter:
    """ParticleWriter::writeParticles with the reference's attributes and file format."""

    def __init__(self, compress: bool = False, radius: float = RADIUS):
        self.compress = compress
        self.radius = radius

    def writeParticles(self, filepath: str, sim) -> int:
        export_records(sim, 0, self.radius)
        ptr, n = wait_records(sim, 0)
        _write(filepath, ptr, n, self.compress)
        return n


class AsyncParticleWriter:
    """Frames exported on the GPU and written by a background thread while the simulation
    advances.  ``close()`` (or leaving the ``with`` block) waits for every file."""

    def __init__(self, compress: bool = False, radius: float = RADIUS):
        self.compress = compress
        self.radius = radius
        self._pool = ThreadPoolExecutor(max_workers=1)
        self._pending = [None, None]
        self._slot = 0
        self._lock = threading.Lock()

    def submit(self, filepath: str, sim):
        slot = self._slot
        self._slot ^= 1
        if self._pending[slot] is not None:
            self._pending[slot].result()  # the slot's last frame is written before it is reused
        n = export_records(sim, slot, self.radius)

        def job():
            ptr, cnt = wait_records(sim, slot)
            _write(filepath, ptr, cnt, self.compress)
            return cnt

        self._pending[slot] = self._pool.submit(job)
        return n

    def close(self):
        for f in self._pending:
            if f is not None:
                f.result()
        self._pending = [None, None]
        self._pool.shutdown(wait=True)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
