"""CPU tests of the C ABI boundary: the library builds, loads, and exports every
entry point include/mpm_gb300.h declares (no compute calls without a GPU)."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")]


def declared_symbols():
    names = set()
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(mpm_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for required in ("mpm_create", "mpm_destroy", "mpm_set_materials", "mpm_upload_soa", "mpm_upload_aos",
                     "mpm_substep", "mpm_download_soa", "mpm_download_aos", "mpm_get_grid", "mpm_sync",
                     "mpm_last_error"):
        assert required in names


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="nvcc not available")
def test_library_exports_every_declared_symbol():
    from mpm_gb300 import build

    lib = build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing


def test_ctypes_signatures_cover_header():
    from mpm_gb300 import _lib

    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert set(declared_symbols()) <= bound, sorted(set(declared_symbols()) - bound)


def test_library_loads():
    from mpm_gb300 import _lib, build

    build.build()
    L = _lib.lib()
    for name, _, _ in _lib.SIGNATURES:
        assert hasattr(L, name)


def test_status_codes_match_header():
    from mpm_gb300 import _lib

    src = open(os.path.join(ROOT, "include", "mpm_gb300.h")).read()
    for code, name in _lib.STATUS_NAMES.items():
        m = re.search(rf"\b{name}\s*=\s*(\d+)", src)
        assert m and int(m.group(1)) == code, name


def test_struct_layouts_match_header():
    """The ctypes mirrors have the field order and sizes of the C structs."""
    import ctypes

    from mpm_gb300 import _lib

    assert ctypes.sizeof(_lib.MpmParams) == 32
    assert ctypes.sizeof(_lib.MpmMaterial) == 36
    src = open(os.path.join(ROOT, "include", "mpm_gb300.h")).read()
    body = re.search(r"typedef struct mpm_params \{(.*?)\} mpm_params;", src, re.S).group(1)
    fields = re.findall(r"\b(\w+);", re.sub(r"/\*.*?\*/", "", body, flags=re.S))
    assert fields == [f for f, _ in _lib.MpmParams._fields_]
    body = re.search(r"typedef struct mpm_material \{(.*?)\} mpm_material;", src, re.S).group(1)
    fields = re.findall(r"\b(\w+);", re.sub(r"/\*.*?\*/", "", body, flags=re.S))
    assert fields == [f for f, _ in _lib.MpmMaterial._fields_]


FACADE_PROGRAM = r"""
#include <cstdio>
#include "mpm_gb300.hpp"

int main(int argc, char** argv) {
  mpm_params p{};
  p.dt = 1e-4f; p.N = 32; p.gravity = -9.81f; p.sort_interval = 16;
  std::vector<mpm_material> mats(1);
  mats[0] = {MPM_MAT_SNOW, 1.0f / 200000, 400.f, 1.4e5f, 0.2f, 10.f, 0.975f, 1.0075f, 0.f};
  if (argc < 2) return 0;  // built and linked; running needs a GPU
  mpm_gb300::Simulation sim(p, mats);
  mpm_object o{};
  o.shape = MPM_SHAPE_SPHERE; o.size = 0.2f; o.position[0] = o.position[1] = o.position[2] = 0.4f;
  o.lifetime_end = 1e300;
  sim.addObject(o);
  for (int i = 0; i < 10; ++i) sim.advance();
  auto& ps = sim.syncDevice();
  std::printf("%zu %f\n", ps.size(), ps.empty() ? 0.f : ps[0].x[1]);
  // the frame outputs of the reference's main loop
  const std::string dir = argv[1];
  const size_t faces = mpm_gb300::MeshBuilder(64, 2).computeMesh(dir + "/mesh_00000.obj", sim);
  mpm_gb300::ParticleWriter().writeParticles(dir + "/particles_0.bgeo", sim);
  mpm_gb300::Renderer r;
  const auto& img = r.render(sim);
  r.writePPM(dir + "/frame.ppm");
  std::printf("%zu %zu\n", faces, img.size());
  return 0;
}
"""


def test_cpp_facade_compiles_and_links(tmp_path):
    """include/mpm_gb300.hpp (the Simulation facade) compiles against the C ABI and the
    program links against the built library (running it needs a GPU)."""
    import shutil
    import subprocess

    from mpm_gb300 import build

    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    lib = build.build()
    src = tmp_path / "facade.cpp"
    src.write_text(FACADE_PROGRAM)
    inc = os.path.join(ROOT, "include")
    exe = tmp_path / "facade"
    r = subprocess.run(["g++", "-std=c++17", "-I", inc, str(src), "-o", str(exe), lib,
                        "-Wl,-rpath," + os.path.dirname(lib)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert subprocess.run([str(exe)]).returncode == 0


def test_library_triangle_table_matches_oracle(oracle_lib):
    """The GPU mesher's compile-time triangle table (mpm_surface_table, no GPU needed) is
    the oracle's."""
    import ctypes

    import numpy as np

    from mpm_gb300 import _lib

    counts = np.empty(256, np.int32)
    slots = np.empty(256 * 30, np.int32)
    L = _lib.lib()
    assert L.mpm_surface_table(counts.ctypes.data_as(ctypes.c_void_p), slots.ctypes.data_as(ctypes.c_void_p)) == 0
    n, t = oracle_lib.surface_table()
    assert np.array_equal(counts, n) and np.array_equal(slots.reshape(256, 30), t)
