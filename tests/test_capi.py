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
