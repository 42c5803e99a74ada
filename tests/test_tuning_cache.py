"""The autotuner's JSON cache (mpm_gb300/csrc/tuning_cache.cpp), compiled for the host with
g++ and driven by a small program: store, replace, lookup by (device, build, class), and
files that are missing, foreign or damaged."""
import json
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "mpm_gb300", "csrc")

DRIVER = r'''
#include <cstdio>
#include <string>
#include "tuning_cache.h"
using namespace mpm;
int main(int argc, char** argv) {
  const std::string path = argv[1], cmd = argv[2];
  if (cmd == "store") {
    TuningEntry e;
    e.device = argv[3]; e.build = argv[4]; e.klass = argv[5];
    e.steps_per_warp = std::stoi(argv[6]); e.warps_per_cta = std::stoi(argv[7]); e.tile_box = std::stoi(argv[8]);
    e.sort_interval = std::stoi(argv[9]); e.us_per_substep = std::stod(argv[10]);
    return store_tuning(path, e) ? 0 : 3;
  }
  bool ok = true;
  auto entries = read_tuning_cache(path, &ok);
  TuningEntry e;
  if (!find_tuning(entries, argv[3], argv[4], argv[5], &e)) { std::printf("miss %d %zu\n", ok ? 1 : 0, entries.size()); return 0; }
  std::printf("hit %d %d %d %d %.3f\n", e.steps_per_warp, e.warps_per_cta, e.tile_box, e.sort_interval, e.us_per_substep);
  return 0;
}
'''


@pytest.fixture(scope="module")
def tool(tmp_path_factory):
    d = tmp_path_factory.mktemp("tuning")
    src = d / "driver.cpp"
    src.write_text(DRIVER)
    exe = d / "driver"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", CSRC, str(src), os.path.join(CSRC, "tuning_cache.cpp"), "-o",
                    str(exe)], check=True)
    return str(exe)


def run(tool, *args):
    r = subprocess.run([tool, *map(str, args)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return r.stdout.split()


def test_store_and_lookup(tool, tmp_path):
    path = tmp_path / "cache.json"
    assert run(tool, path, "find", "GB300", "b1", "liquid N=32")[0] == "miss"
    run(tool, path, "store", "GB300", "b1", "liquid N=32", 2, 12, 2, 16, 58.25)
    run(tool, path, "store", "GB300", "b1", "general N=64", 1, 6, 1, 16, 77.5)
    assert run(tool, path, "find", "GB300", "b1", "liquid N=32") == ["hit", "2", "12", "2", "16", "58.250"]
    assert run(tool, path, "find", "GB300", "b1", "general N=64") == ["hit", "1", "6", "1", "16", "77.500"]
    # another build or device measures again
    assert run(tool, path, "find", "GB300", "b2", "liquid N=32")[0] == "miss"
    assert run(tool, path, "find", "B200", "b1", "liquid N=32")[0] == "miss"
    # replacing keeps one entry per key; the file stays valid JSON
    run(tool, path, "store", "GB300", "b1", "liquid N=32", 4, 4, 1, 8, 55.0)
    assert run(tool, path, "find", "GB300", "b1", "liquid N=32") == ["hit", "4", "4", "1", "8", "55.000"]
    d = json.loads(path.read_text())
    assert d["format"] == "mpm_gb300 tuning cache 1" and len(d["entries"]) == 2


def test_quoted_keys_round_trip(tool, tmp_path):
    path = tmp_path / "cache.json"
    key = 'dev "x" \\ y'
    run(tool, path, "store", key, "b", "k", 2, 12, 1, 0, 1.0)
    assert run(tool, path, "find", key, "b", "k")[0] == "hit"
    assert json.loads(path.read_text())["entries"][0]["device"] == key


def test_foreign_and_damaged_files(tool, tmp_path):
    foreign = tmp_path / "foreign.json"
    foreign.write_text('{"something": "else"}')
    assert run(tool, foreign, "find", "a", "b", "c") == ["miss", "0", "0"]
    damaged = tmp_path / "damaged.json"
    run(tool, damaged, "store", "a", "b", "c", 2, 12, 1, 0, 1.0)
    text = damaged.read_text()
    damaged.write_text(text[: len(text) // 2])  # cut inside the entry
    assert run(tool, damaged, "find", "a", "b", "c")[0] == "miss"
    # an entry with a field of the wrong type is skipped, the others still read
    mixed = tmp_path / "mixed.json"
    mixed.write_text(json.dumps({"format": "mpm_gb300 tuning cache 1", "entries": [
        {"device": "a", "build": "b", "class": "c", "steps_per_warp": "two", "warps_per_cta": 12, "tile_box": 1,
         "sort_interval": 0, "us_per_substep": 1.0},
        {"device": "a", "build": "b", "class": "d", "steps_per_warp": 2, "warps_per_cta": 12, "tile_box": 1,
         "sort_interval": 0, "us_per_substep": 2.0}]}))
    assert run(tool, mixed, "find", "a", "b", "c")[0] == "miss"
    assert run(tool, mixed, "find", "a", "b", "d")[0] == "hit"
    # counts out of the int range or not integral, and non-finite times, skip the entry
    odd = tmp_path / "odd.json"
    odd.write_text('{"format": "mpm_gb300 tuning cache 1", "entries": ['
                   '{"device": "a", "build": "b", "class": "c", "steps_per_warp": 1e300, "warps_per_cta": 12, '
                   '"tile_box": 1, "sort_interval": 0, "us_per_substep": 1.0},'
                   '{"device": "a", "build": "b", "class": "d", "steps_per_warp": 2.5, "warps_per_cta": 12, '
                   '"tile_box": 1, "sort_interval": 0, "us_per_substep": 1.0},'
                   '{"device": "a", "build": "b", "class": "e", "steps_per_warp": 2, "warps_per_cta": 12, '
                   '"tile_box": 1, "sort_interval": 0, "us_per_substep": 1e999}]}')
    for k in "cde":
        assert run(tool, odd, "find", "a", "b", k)[0] == "miss"
    # a file that is not a cache is never overwritten by a store
    r = subprocess.run([tool, str(foreign), "store", "a", "b", "c", "2", "12", "1", "0", "1.0"], capture_output=True)
    assert r.returncode == 3
    assert foreign.read_text() == '{"something": "else"}'
    # a damaged cache of this format is ours: a store rewrites it with its readable entries
    run(tool, damaged, "store", "a", "b", "z", 2, 12, 1, 0, 1.0)
    assert run(tool, damaged, "find", "a", "b", "z")[0] == "hit"
