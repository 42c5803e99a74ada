// The autotuner's cache: launch shapes chosen per (device, build, workload class), kept in
// a small JSON file so a process reuses what an earlier one measured.
//
//   {"format": "mpm_gb300 tuning cache 1",
//    "entries": [
//      {"device": "...", "build": "...", "class": "...", "steps_per_warp": 2,
//       "warps_per_cta": 12, "tile_box": 1, "sort_interval": 16, "us_per_substep": 59.1},
//      ...]}
//
// Host code only (no CUDA); shared by the C ABI's mpm_autotune and the cache entry points.
#pragma once
#include <string>
#include <vector>

namespace mpm {

struct TuningEntry {
  std::string device, build, klass;
  int steps_per_warp = 2;
  int warps_per_cta = 12;
  int tile_box = 1;  // MPM_TILE_*
  int sort_interval = 0;
  double us_per_substep = 0.0;
};

// Entries of the cache file at `path` (empty when it is missing or holds none).  Entries
// with a missing or malformed field (a count that is not a 32-bit integer, a number that
// is not finite) are skipped; *ok (may be null) is false when the file
// exists but is not a cache file of this format.
std::vector<TuningEntry> read_tuning_cache(const std::string& path, bool* ok = nullptr);
// The entry with this device, build and class, if any.
bool find_tuning(const std::vector<TuningEntry>& entries, const std::string& device, const std::string& build,
                 const std::string& klass, TuningEntry* out);
// Writes the entries, replacing one with the same (device, build, class) as `e` or adding
// it; the file is written to a temporary name and renamed into place.  False on I/O error,
// and when `path` holds a file that is not a cache of this format (it is left unchanged).
bool store_tuning(const std::string& path, const TuningEntry& e);

}  // namespace mpm
