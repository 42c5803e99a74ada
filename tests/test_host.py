"""CPU tests of the host-side logic: materials, scene generators, AoS records."""
import numpy as np

from mpm_gb300 import aos, materials, scenes


def test_material_constants_float32():
    m = materials.Material(materials.SNOW, 1.0 / 500000, 700.0, 1.4e5, 0.2, 10.0, 0.975, 1.0075)
    d = m.derived()
    E, nu = np.float32(1.4e5), np.float32(0.2)
    assert d["mu0"] == np.float32(E / (np.float32(2) * (np.float32(1) + nu)))
    assert d["lambda0"] == np.float32((E * nu) / ((np.float32(1) + nu) * (np.float32(1) - np.float32(2) * nu)))
    assert d["particle_mass"] == np.float32(np.float32(700.0) * np.float32(1.0 / 500000))


def test_toml_defaults_match_reference():
    """src/main.cu:35-43 defaults: density 700, E 1.4e5, Nu 0.2, hardening 10, clamps 0.975 / 1.0075."""
    m = materials.from_toml_table({"name": "snow"}, 500000)
    assert (m.density, m.E, m.nu, m.hardening, m.clamp_lo, m.clamp_hi) == (700.0, 1.4e5, 0.2, 10.0, 0.975, 1.0075)
    assert m.particle_volume == 1.0 / 500000


def test_scenes_deterministic():
    a = scenes.config_snow(n=5000, seed=3)
    b = scenes.config_snow(n=5000, seed=3)
    c = scenes.config_snow(n=5000, seed=4)
    assert np.array_equal(a["state"]["x"], b["state"]["x"])
    assert not np.array_equal(a["state"]["x"], c["state"]["x"])


def test_scene_shapes_and_regions():
    cfg = scenes.config_liquid(n=10000)
    x = cfg["state"]["x"]
    assert x.shape == (10000, 3) and x.dtype == np.float32
    assert np.all(x >= [0.1, 0.1, 0.1]) and np.all(x <= [0.5, 0.7, 0.9])
    cfg = scenes.config_snow(n=10000)
    x = cfg["state"]["x"].astype(np.float64)
    d1 = np.linalg.norm(x - [0.5, 0.3, 0.5], axis=1)
    d2 = np.linalg.norm(x - [0.5, 0.55, 0.5], axis=1)
    assert np.all((d1 <= 0.15 + 1e-6) | (d2 <= 0.1 + 1e-6))
    assert np.all(cfg["state"]["v"][:, 1] == -1.0)


def test_aos_record_layout_round_trip():
    cfg = scenes.mixed_scene(n=500, seed=1)
    st = cfg["state"]
    st["C"] = np.random.default_rng(0).standard_normal((500, 3, 3)).astype(np.float32)
    buf = aos.pack(st)
    assert buf.size == 500 * 104
    back = aos.unpack(buf)
    for k in ("x", "v", "C", "F", "Jp", "mat"):
        assert np.array_equal(back[k], st[k]), k
    # byte offsets of the reference record: material 0, x 4, v 16, F 28 (column-major), C 64, Jp 100
    rec = buf[:104]
    assert rec[0] == st["mat"][0]
    assert np.frombuffer(rec[4:16].tobytes(), np.float32).tolist() == st["x"][0].tolist()
    assert np.frombuffer(rec[28:40].tobytes(), np.float32).tolist() == st["F"][0][:, 0].tolist()
    assert np.frombuffer(rec[100:104].tobytes(), np.float32)[0] == st["Jp"][0]
