/* CPU oracle of surface reconstruction — TEST INFRASTRUCTURE ONLY (the checker of the
 * GPU mesher; the product never links it).
 *
 * Distance field: a sequential restatement of fillVoxelGrid_distance
 * (include/mesh_builder.h:89-137) as MeshBuilder::computeMesh calls it
 * (include/mesh_builder.h:170-178): every node starts at the cutoff (radius + 1) voxel_dx
 * rounded to float; each particle lowers the nodes of the box
 * [int(x/dx - r), int(x/dx + r + 1)) (r = cutoff / dx, all in float) to
 * |x - (i, j, k) dx| computed in float, the squared norm summed as d0^2 + (d1^2 + d2^2)
 * (Eigen's unrolled reduction of a 3-vector).  The minimum does not depend on the
 * particle order, so the GPU's atomic scatter must match it bit for bit.
 *
 * Surface: MeshBuilder::computeMesh hands S = radius voxel_dx - field, on nodes at
 * (i, j, k) with i slowest (include/mesh_builder.h:181-194), to libigl's marching cubes
 * (the reference's vendored include/igl/copyleft/marching_cubes.cpp), then scales V by
 * voxel_dx.  The vertices are restated from that code: cubes are visited with k fastest,
 * a corner is inside when S > 0, and the crossed edges of each cube are visited in the
 * order of its edge slots 0..11 (corner pairs below, lower node index first); an edge
 * seen for the first time appends the vertex (1 - t) p0 + t p1, t = |S0| / (|S0| + |S1|),
 * computed in double.  The faces are this project's own triangulation of the same
 * crossings (libigl's triangle table is not restated): on each face of a cube, a segment
 * joins the edge where the face's corner cycle (counter-clockwise seen from outside)
 * enters the inside to the edge where it leaves it, and a face with two opposite inside
 * corners cuts each of them off; the segments of a cube close into loops, and each loop,
 * started at its lowest edge slot, is fanned from that edge.  Faces point outward.
 */
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <unordered_map>
#include <vector>

namespace {

// corner n of a cube at offset (di, dj, dk) from its lowest node
const int kCorner[8][3] = {{0, 0, 0}, {0, 0, 1}, {0, 1, 1}, {0, 1, 0}, {1, 0, 0}, {1, 0, 1}, {1, 1, 1}, {1, 1, 0}};
// edge slot -> its two corners, lower node index first
const int kEdge[12][2] = {{0, 1}, {1, 2}, {3, 2}, {0, 3}, {4, 5}, {5, 6}, {7, 6}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
// the six faces: corners counter-clockwise seen from outside the cube
const int kFace[6][4] = {{0, 1, 2, 3}, {4, 7, 6, 5}, {0, 4, 5, 1}, {3, 2, 6, 7}, {0, 3, 7, 4}, {1, 5, 6, 2}};

int edge_of(int a, int b) {
  for (int e = 0; e < 12; ++e)
    if ((kEdge[e][0] == a && kEdge[e][1] == b) || (kEdge[e][0] == b && kEdge[e][1] == a)) return e;
  return -1;
}

// The triangles (edge-slot triples) of a cube whose inside corners are the set bits of m.
std::vector<int> cube_triangles(unsigned m) {
  int next[12];
  for (int e = 0; e < 12; ++e) next[e] = -1;
  for (int f = 0; f < 6; ++f) {
    const int* q = kFace[f];
    bool in[4];
    int ntrans = 0;
    for (int r = 0; r < 4; ++r) in[r] = (m >> q[r]) & 1;
    for (int r = 0; r < 4; ++r) ntrans += in[r] != in[(r + 1) % 4];
    for (int r = 0; r < 4; ++r) {
      // corner r inside: the edge into it from r - 1 and the edge out of it to r + 1
      const int rp = (r + 3) % 4, rn = (r + 1) % 4;
      if (ntrans == 4) {
        if (in[r]) next[edge_of(q[rp], q[r])] = edge_of(q[r], q[rn]);
      } else if (ntrans == 2) {
        if (!in[r] && in[rn]) {
          // enters the inside on edge (r, r + 1); leaves it on the first edge after
          int s = rn;
          while (in[(s + 1) % 4]) s = (s + 1) % 4;
          next[edge_of(q[r], q[rn])] = edge_of(q[s], q[(s + 1) % 4]);
        }
      }
    }
  }
  std::vector<int> tris;
  bool seen[12] = {};
  for (int e0 = 0; e0 < 12; ++e0) {
    if (next[e0] < 0 || seen[e0]) continue;
    std::vector<int> loop;
    for (int e = e0; !seen[e]; e = next[e]) {
      seen[e] = true;
      loop.push_back(e);
    }
    for (size_t r = 1; r + 1 < loop.size(); ++r) {
      tris.push_back(loop[0]);
      tris.push_back(loop[r]);
      tris.push_back(loop[r + 1]);
    }
  }
  return tris;
}

}  // namespace

extern "C" {

/* x: n particles, 3 floats each.  field: G^3 floats, index (i G + j) G + k. */
void oracle_distance_field(const float* x, int64_t n, int32_t G, int32_t radius, double voxel_dx, float* field) {
  const float dx = (float)voxel_dx;
  const float cutoff = (float)((double)(uint32_t)(radius + 1) * voxel_dx);
  const int64_t cells = (int64_t)G * G * G;
  for (int64_t c = 0; c < cells; ++c) field[c] = cutoff;
  const float r = cutoff / dx;
  for (int64_t p = 0; p < n; ++p) {
    const float* xp = x + 3 * p;
    int lo[3], hi[3];
    for (int c = 0; c < 3; ++c) {
      const float g = xp[c] / dx;
      lo[c] = std::max(0, (int)(g - r));
      hi[c] = std::min((int)G, (int)(g + (float)((double)r + 1.0)));
    }
    for (int i = lo[0]; i < hi[0]; ++i) {
      const float d0 = xp[0] - (float)(uint32_t)i * dx;
      for (int j = lo[1]; j < hi[1]; ++j) {
        const float d1 = xp[1] - (float)(uint32_t)j * dx;
        for (int k = lo[2]; k < hi[2]; ++k) {
          const float d2 = xp[2] - (float)(uint32_t)k * dx;
          const float d = std::sqrt(d0 * d0 + (d1 * d1 + d2 * d2));
          float& f = field[((int64_t)i * G + j) * G + k];
          f = std::min(d, f);
        }
      }
    }
  }
}

/* Marching cubes of S = radius voxel_dx - field: vertices (nv x 3 doubles, world units)
 * and faces (nf x 3 vertex indices), copied up to the capacities; *nv and *nf receive
 * the counts. */
void oracle_surface_indexed(const float* field, int32_t G, int32_t radius, double voxel_dx, double* V, int64_t vcap,
                            int32_t* F, int64_t fcap, int64_t* nv, int64_t* nf) {
  std::vector<double> verts;
  std::vector<int32_t> faces;
  if (G >= 2) {
    const double iso = (double)(uint32_t)radius * voxel_dx;
    const int64_t GG = (int64_t)G * G;
    std::unordered_map<uint64_t, int32_t> edge_vertex;
    std::vector<std::vector<int>> table(256);
    for (unsigned m = 0; m < 256; ++m) table[m] = cube_triangles(m);
    for (int i = 0; i + 1 < G; ++i)
      for (int j = 0; j + 1 < G; ++j)
        for (int k = 0; k + 1 < G; ++k) {
          int64_t node[8];
          double S[8];
          unsigned m = 0;
          for (int n = 0; n < 8; ++n) {
            node[n] = (i + kCorner[n][0]) * GG + (int64_t)(j + kCorner[n][1]) * G + k + kCorner[n][2];
            S[n] = iso - (double)field[node[n]];
            m |= (unsigned)(S[n] > 0.0) << n;
          }
          if (m == 0 || m == 255) continue;
          int32_t id[12];
          for (int e = 0; e < 12; ++e) {
            const int a = kEdge[e][0], b = kEdge[e][1];
            if (((m >> a) & 1) == ((m >> b) & 1)) continue;
            const uint64_t key = (uint64_t)node[a] * (uint64_t)(GG * G) + (uint64_t)node[b];
            auto it = edge_vertex.find(key);
            if (it != edge_vertex.end()) {
              id[e] = it->second;
              continue;
            }
            const double s0 = std::fabs(S[a]), s1 = std::fabs(S[b]);
            const double t = s0 / (s0 + s1);
            const int p0[3] = {i + kCorner[a][0], j + kCorner[a][1], k + kCorner[a][2]};
            const int p1[3] = {i + kCorner[b][0], j + kCorner[b][1], k + kCorner[b][2]};
            id[e] = (int32_t)(verts.size() / 3);
            for (int c = 0; c < 3; ++c) {
              const double v = (1.0 - t) * (double)p0[c] + t * (double)p1[c];
              verts.push_back(v * voxel_dx);
            }
            edge_vertex.emplace(key, id[e]);
          }
          for (int e : table[m]) faces.push_back(id[e]);
        }
  }
  *nv = (int64_t)(verts.size() / 3);
  *nf = (int64_t)(faces.size() / 3);
  std::copy(verts.begin(), verts.begin() + 3 * std::min(*nv, vcap), V);
  std::copy(faces.begin(), faces.begin() + 3 * std::min(*nf, fcap), F);
}

/* The triangle table of the faces above: for each inside-corner mask m, n[m] triangles
 * as edge-slot triples in slots[m] (up to 10 triangles).  For tests of the GPU table. */
void oracle_surface_table(int32_t* n, int32_t* slots) {
  for (unsigned m = 0; m < 256; ++m) {
    const std::vector<int> t = cube_triangles(m);
    n[m] = (int32_t)(t.size() / 3);
    for (int r = 0; r < 30; ++r) slots[30 * m + r] = r < (int)t.size() ? t[r] : -1;
  }
}

}  // extern "C"
