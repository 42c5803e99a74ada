/* CPU oracle of particle seeding — TEST INFRASTRUCTURE ONLY (the checker of the GPU
 * seeder; the product never links it).
 *
 * Restates, one candidate at a time, the reference's rejection sampler of
 * Simulation::addParticles (src/mpm.cu:346-394) with the object placement of
 * Simulation::loadMesh (src/mpm.cu:330-344: scale = size / longest bounding-box edge,
 * lowest corner at `position`) and the candidate count u32(density x bounding-box
 * volume) (src/mpm.cu:369-371).  The reference draws with rand() and tests meshes with
 * libigl's winding number (igl::winding_number); this restatement draws candidate i
 * from SplitMix64 (Steele, Lea, Flood, OOPSLA 2014) of seed + 3 i + axis and tests
 * meshes by the parity of +x ray crossings or, with inside_test = 1, by the generalized
 * winding number in double (libigl's solid_angle summed over the triangles, inside when
 * above 1/2), the rules the GPU seeder documents.
 *
 * The reference stores libigl's float winding number in an integer matrix and keeps a
 * candidate when that integer is 1 (src/mpm.cu:352, 383-385), so an interior point whose
 * float sum rounds to just below 1 is dropped: about half of them (a float32 sum over a
 * 1,280-triangle sphere puts 50 % of interior points below 1).  Neither the oracle nor the
 * GPU seeder reproduces that; both keep every point inside.
 * Every operation is an IEEE double (or float where the placement is float) with no
 * contraction (built with -ffp-contract=off), so GPU and oracle agree bit for bit.
 */
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <vector>

namespace {

uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

double uniform(uint64_t seed, uint64_t i, int axis) {
  return (double)(splitmix64(seed + 3ull * i + (uint64_t)axis) >> 11) * (1.0 / 9007199254740992.0);
}

double orient(double ay, double az, double by, double bz, double qy, double qz) {
  return (by - ay) * (qz - az) - (bz - az) * (qy - ay);
}

bool crosses(const float* a, const float* b, const float* c, double px, double py, double pz) {
  const double e0 = orient(b[1], b[2], c[1], c[2], py, pz);
  const double e1 = orient(c[1], c[2], a[1], a[2], py, pz);
  const double e2 = orient(a[1], a[2], b[1], b[2], py, pz);
  const bool pos = e0 > 0.0 && e1 > 0.0 && e2 > 0.0;
  const bool neg = e0 < 0.0 && e1 < 0.0 && e2 < 0.0;
  if (!pos && !neg) return false;
  const double s = (e0 + e1) + e2;
  const double xs = (e0 * (double)a[0] + e1 * (double)b[0]) + e2 * (double)c[0];
  return xs / s > px;
}

// A triangle's share of the winding number at p, as libigl's solid_angle computes it
// (include/igl/solid_angle.cpp of the reference's vendored libigl): atan2(det, |a||b||c| + (b.c)|a| + (c.a)|b| + (a.b)|c|) / (2 pi).
double winding_term(const float* A, const float* B, const float* C, const float p[3]) {
  double v[3][3];
  for (int d = 0; d < 3; ++d) {
    v[0][d] = (double)A[d] - (double)p[d];
    v[1][d] = (double)B[d] - (double)p[d];
    v[2][d] = (double)C[d] - (double)p[d];
  }
  const double la = std::sqrt(v[0][0] * v[0][0] + v[0][1] * v[0][1] + v[0][2] * v[0][2]);
  const double lb = std::sqrt(v[1][0] * v[1][0] + v[1][1] * v[1][1] + v[1][2] * v[1][2]);
  const double lc = std::sqrt(v[2][0] * v[2][0] + v[2][1] * v[2][1] + v[2][2] * v[2][2]);
  const double det = v[0][0] * v[1][1] * v[2][2] + v[1][0] * v[2][1] * v[0][2] + v[2][0] * v[0][1] * v[1][2] -
                     v[2][0] * v[1][1] * v[0][2] - v[1][0] * v[0][1] * v[2][2] - v[0][0] * v[2][1] * v[1][2];
  const double d0 = v[1][0] * v[2][0] + v[1][1] * v[2][1] + v[1][2] * v[2][2];
  const double d1 = v[2][0] * v[0][0] + v[2][1] * v[0][1] + v[2][2] * v[0][2];
  const double d2 = v[0][0] * v[1][0] + v[0][1] * v[1][1] + v[0][2] * v[1][2];
  return std::atan2(det, la * lb * lc + d0 * la + d1 * lb + d2 * lc) * 0.15915494309189535;
}

}  // namespace

extern "C" {

/* shape: 0 box (box_extent relative edges), 1 sphere, 2 mesh (vertices, triangles;
 * inside_test 0: ray parity, 1: winding number > 1/2).  Writes up to `capacity`
 * particles (3 floats each, candidate order) to x and returns the number kept, or -1 for
 * an invalid object. */
int64_t oracle_seed_object(int shape, float size, const float* position, const float* box_extent, uint64_t seed,
                           uint32_t density, const float* vertices, int64_t n_vertices, const int32_t* triangles,
                           int64_t n_triangles, int32_t inside_test, float* x, int64_t capacity) {
  double lo[3], range[3], center[3] = {0, 0, 0}, r2 = 0.0;
  std::vector<float> V;
  if (!(size > 0.f)) return -1;
  if (shape == 0) {
    float emax = 0.f;
    for (int c = 0; c < 3; ++c) emax = std::max(emax, box_extent[c]);
    if (!(emax > 0.f)) return -1;
    const float scale = size / emax;
    for (int c = 0; c < 3; ++c) {
      lo[c] = position[c];
      range[c] = (double)(box_extent[c] * scale);
    }
  } else if (shape == 1) {
    const double r = 0.5 * (double)size;
    for (int c = 0; c < 3; ++c) {
      lo[c] = position[c];
      range[c] = size;
      center[c] = lo[c] + r;
    }
    r2 = r * r;
  } else if (shape == 2) {
    if (n_vertices < 3 || n_triangles < 1) return -1;
    float vmin[3], vmax[3];
    for (int c = 0; c < 3; ++c) vmin[c] = vmax[c] = vertices[c];
    for (int64_t v = 0; v < n_vertices; ++v)
      for (int c = 0; c < 3; ++c) {
        vmin[c] = std::min(vmin[c], vertices[3 * v + c]);
        vmax[c] = std::max(vmax[c], vertices[3 * v + c]);
      }
    float length_max = 0.f;
    for (int c = 0; c < 3; ++c) length_max = std::max(length_max, vmax[c] - vmin[c]);
    if (!(length_max > 0.f)) return -1;
    const float scale = size / length_max;
    V.resize(3 * n_vertices);
    for (int64_t v = 0; v < n_vertices; ++v)
      for (int c = 0; c < 3; ++c) V[3 * v + c] = vertices[3 * v + c] * scale + (position[c] - scale * vmin[c]);
    float l[3], h[3];
    for (int c = 0; c < 3; ++c) l[c] = h[c] = V[c];
    for (int64_t v = 0; v < n_vertices; ++v)
      for (int c = 0; c < 3; ++c) {
        l[c] = std::min(l[c], V[3 * v + c]);
        h[c] = std::max(h[c], V[3 * v + c]);
      }
    for (int c = 0; c < 3; ++c) {
      lo[c] = l[c];
      range[c] = (double)h[c] - (double)l[c];
    }
  } else {
    return -1;
  }
  const double cand = (double)density * (range[0] * range[1] * range[2]);
  if (!(cand >= 0.0) || cand > 4294967295.0) return -1;
  const uint64_t candidates = (uint64_t)cand;
  int64_t kept = 0;
  for (uint64_t i = 0; i < candidates; ++i) {
    float p[3];
    for (int c = 0; c < 3; ++c) p[c] = (float)(lo[c] + uniform(seed, i, c) * range[c]);
    bool in = true;
    if (shape == 1) {
      const double dx = (double)p[0] - center[0], dy = (double)p[1] - center[1], dz = (double)p[2] - center[2];
      in = ((dx * dx + dy * dy) + dz * dz) < r2;
    } else if (shape == 2 && inside_test == 1) {
      double w = 0.0;
      for (int64_t t = 0; t < n_triangles; ++t)
        w += winding_term(&V[3 * triangles[3 * t]], &V[3 * triangles[3 * t + 1]], &V[3 * triangles[3 * t + 2]], p);
      in = w > 0.5;
    } else if (shape == 2) {
      int crossings = 0;
      for (int64_t t = 0; t < n_triangles; ++t)
        if (crosses(&V[3 * triangles[3 * t]], &V[3 * triangles[3 * t + 1]], &V[3 * triangles[3 * t + 2]], p[0], p[1],
                    p[2]))
          ++crossings;
      in = (crossings & 1) != 0;
    }
    if (!in) continue;
    if (kept < capacity)
      for (int c = 0; c < 3; ++c) x[3 * kept + c] = p[c];
    ++kept;
  }
  return kept;
}

}  // extern "C"
