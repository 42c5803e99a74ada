// JSON cache of the autotuner (see tuning_cache.h).  A deliberately small reader: the
// file holds one flat object per entry, strings without escapes other than \" and \\,
// and numbers; anything else in an entry makes the reader skip that entry.
#include "tuning_cache.h"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>

namespace mpm {
namespace {

const char* kFormat = "mpm_gb300 tuning cache 1";

// Parses a JSON string starting at s[i] == '"'; advances i past it.
bool parse_string(const std::string& s, size_t& i, std::string& out) {
  if (i >= s.size() || s[i] != '"') return false;
  out.clear();
  for (++i; i < s.size(); ++i) {
    const char c = s[i];
    if (c == '"') {
      ++i;
      return true;
    }
    if (c == '\\') {
      if (++i >= s.size()) return false;
      out.push_back(s[i]);
    } else {
      out.push_back(c);
    }
  }
  return false;
}

void skip_ws(const std::string& s, size_t& i) {
  while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
}

// One flat object {"k": "v" | number, ...} starting at s[i] == '{'.
bool parse_object(const std::string& s, size_t& i, std::map<std::string, std::string>& kv) {
  if (i >= s.size() || s[i] != '{') return false;
  ++i;
  for (;;) {
    skip_ws(s, i);
    if (i < s.size() && s[i] == '}') {
      ++i;
      return true;
    }
    std::string key, val;
    if (!parse_string(s, i, key)) return false;
    skip_ws(s, i);
    if (i >= s.size() || s[i] != ':') return false;
    ++i;
    skip_ws(s, i);
    if (i < s.size() && s[i] == '"') {
      if (!parse_string(s, i, val)) return false;
      kv[key] = "s" + val;
    } else {
      const size_t b = i;
      while (i < s.size() && (std::isdigit((unsigned char)s[i]) || s[i] == '-' || s[i] == '+' || s[i] == '.' ||
                              s[i] == 'e' || s[i] == 'E'))
        ++i;
      if (i == b) return false;
      kv[key] = "n" + s.substr(b, i - b);
    }
    skip_ws(s, i);
    if (i < s.size() && s[i] == ',') ++i;
  }
}

bool get_str(const std::map<std::string, std::string>& kv, const char* k, std::string& out) {
  auto it = kv.find(k);
  if (it == kv.end() || it->second.empty() || it->second[0] != 's') return false;
  out = it->second.substr(1);
  return true;
}

bool get_num(const std::map<std::string, std::string>& kv, const char* k, double& out) {
  auto it = kv.find(k);
  if (it == kv.end() || it->second.empty() || it->second[0] != 'n') return false;
  char* end = nullptr;
  const std::string t = it->second.substr(1);
  out = std::strtod(t.c_str(), &end);
  return end && *end == '\0' && std::isfinite(out);
}

// A number field that is a 32-bit integer (anything else skips the entry).
bool get_int(const std::map<std::string, std::string>& kv, const char* k, int& out) {
  double v = 0.0;
  if (!get_num(kv, k, v) || v < -2147483648.0 || v > 2147483647.0 || v != std::floor(v)) return false;
  out = (int)v;
  return true;
}

// Whether `path` holds a file that is not a cache of this format (so it is not ours to
// replace).
bool foreign_file(const std::string& path) {
  std::ifstream f(path);
  if (!f) return false;
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string s = ss.str();
  bool blank = true;
  for (char c : s) blank = blank && std::isspace((unsigned char)c);
  return !blank && s.find(kFormat) == std::string::npos;
}

std::string quote(const std::string& s) {
  std::string o = "\"";
  for (char c : s) {
    if (c == '"' || c == '\\') o.push_back('\\');
    if ((unsigned char)c < 0x20) continue;
    o.push_back(c);
  }
  return o + "\"";
}

}  // namespace

std::vector<TuningEntry> read_tuning_cache(const std::string& path, bool* ok) {
  std::vector<TuningEntry> out;
  if (ok) *ok = true;
  std::ifstream f(path);
  if (!f) return out;
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string s = ss.str();
  if (s.find(kFormat) == std::string::npos) {
    if (ok) *ok = false;
    return out;
  }
  const size_t e = s.find("\"entries\"");
  if (e == std::string::npos) return out;
  size_t i = s.find('[', e);
  if (i == std::string::npos) return out;
  ++i;
  for (;;) {
    skip_ws(s, i);
    if (i >= s.size() || s[i] == ']') break;
    if (s[i] == ',') {
      ++i;
      continue;
    }
    std::map<std::string, std::string> kv;
    if (!parse_object(s, i, kv)) {
      if (ok) *ok = false;
      break;
    }
    TuningEntry t;
    if (get_str(kv, "device", t.device) && get_str(kv, "build", t.build) && get_str(kv, "class", t.klass) &&
        get_int(kv, "steps_per_warp", t.steps_per_warp) && get_int(kv, "warps_per_cta", t.warps_per_cta) &&
        get_int(kv, "tile_box", t.tile_box) && get_int(kv, "sort_interval", t.sort_interval) &&
        get_num(kv, "us_per_substep", t.us_per_substep))
      out.push_back(t);
  }
  return out;
}

bool find_tuning(const std::vector<TuningEntry>& entries, const std::string& device, const std::string& build,
                 const std::string& klass, TuningEntry* out) {
  for (const auto& e : entries)
    if (e.device == device && e.build == build && e.klass == klass) {
      if (out) *out = e;
      return true;
    }
  return false;
}

bool store_tuning(const std::string& path, const TuningEntry& e) {
  if (foreign_file(path)) return false;  // not a cache file: leave it alone
  bool ok = true;
  std::vector<TuningEntry> entries = read_tuning_cache(path, &ok);
  bool replaced = false;
  for (auto& x : entries)
    if (x.device == e.device && x.build == e.build && x.klass == e.klass) {
      x = e;
      replaced = true;
    }
  if (!replaced) entries.push_back(e);
  const std::string tmp = path + ".tmp";
  {
    std::ofstream f(tmp, std::ios::trunc);
    if (!f) return false;
    f << "{\"format\": " << quote(kFormat) << ",\n \"entries\": [";
    for (size_t k = 0; k < entries.size(); ++k) {
      const auto& x = entries[k];
      char us[64];
      std::snprintf(us, sizeof(us), "%.3f", x.us_per_substep);
      f << (k ? ",\n  " : "\n  ") << "{\"device\": " << quote(x.device) << ", \"build\": " << quote(x.build)
        << ", \"class\": " << quote(x.klass) << ", \"steps_per_warp\": " << x.steps_per_warp
        << ", \"warps_per_cta\": " << x.warps_per_cta << ", \"tile_box\": " << x.tile_box
        << ", \"sort_interval\": " << x.sort_interval << ", \"us_per_substep\": " << us << "}";
    }
    f << "\n ]}\n";
    if (!f) return false;
  }
  return std::rename(tmp.c_str(), path.c_str()) == 0;
}

}  // namespace mpm
