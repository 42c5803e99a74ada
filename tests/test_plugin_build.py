"""Material models compiled into a build of the library (include/mpm_gb300_policies.cuh):
the test translation unit tests/plugin_materials.cu builds into a library of its own, which
loads and reports its compiled-in kinds (no GPU needed); the library of the package knows
only the built-in kinds."""
import os

from mpm_gb300 import _lib, build

HERE = os.path.dirname(os.path.abspath(__file__))
PLUGIN = os.path.join(HERE, "plugin_materials.cu")


def test_plugin_build_registers_kinds(tmp_path):
    path = build.build_with_materials([PLUGIN], str(tmp_path / "libmpm_gb300_plugins.so"))
    L = _lib.load_library(path)
    assert [L.mpm_material_kind_available(k) for k in (0, 1, 2, 3)] == [1, 1, 1, 1]
    assert L.mpm_material_kind_available(16) == 1 and L.mpm_material_kind_available(17) == 1
    assert L.mpm_material_kind_available(18) == 0 and L.mpm_material_kind_available(4) == 0
    base = _lib.lib()
    assert base.mpm_material_kind_available(16) == 0 and base.mpm_material_kind_available(3) == 1
