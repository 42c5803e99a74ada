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
 * Surface: the reference hands S = radius voxel_dx - field (include/mesh_builder.h:188)
 * to libigl's marching cubes, which is not in this image.  The GPU extracts the same
 * zero level set by marching tetrahedra; this file restates that extraction: a corner is
 * inside when S > 0 in double (here tested directly, on the GPU through the equivalent
 * float threshold), each cell is split into the six tetrahedra around its main diagonal,
 * edge points are interpolated in float from the inside corner to the outside one,
 * triangles face outward by the tetrahedron's corner layout, and cells are visited in
 * (i, j, k) order.  IEEE float without contraction (built with -ffp-contract=off), so
 * the triangle lists agree bit for bit.
 */
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <vector>

namespace {

const int kTets[6][4] = {{0, 4, 6, 7}, {0, 4, 5, 7}, {0, 1, 5, 7}, {0, 1, 3, 7}, {0, 2, 3, 7}, {0, 2, 6, 7}};

int bit(int q, int c) { return (q >> (2 - c)) & 1; }

// edge point from the inside corner qi to the outside corner qo
void edge_point(const float f[8], int qi, int qo, int i, int j, int k, float iso, float vdx, float* p) {
  const float t = (iso - f[qi]) / (f[qo] - f[qi]);
  const int cell[3] = {i, j, k};
  for (int c = 0; c < 3; ++c) {
    const float a = (float)(cell[c] + bit(qi, c)), b = (float)(cell[c] + bit(qo, c));
    p[c] = (a + t * (b - a)) * vdx;
  }
}

int det3(int L, int A, int B, int C) {
  int u[3], v[3], w[3];
  for (int c = 0; c < 3; ++c) {
    u[c] = bit(A, c) - bit(L, c);
    v[c] = bit(B, c) - bit(L, c);
    w[c] = bit(C, c) - bit(L, c);
  }
  return u[0] * (v[1] * w[2] - v[2] * w[1]) - u[1] * (v[0] * w[2] - v[2] * w[0]) + u[2] * (v[0] * w[1] - v[1] * w[0]);
}

bool quad_flip(int a, int b, int c, int d) {
  int e1[3], e2[3], aw[3];
  for (int x = 0; x < 3; ++x) {
    e1[x] = bit(d, x) - bit(c, x);
    e2[x] = bit(b, x) + bit(d, x) - bit(a, x) - bit(c, x);
    aw[x] = bit(c, x) + bit(d, x) - bit(a, x) - bit(b, x);
  }
  const int n0 = e1[1] * e2[2] - e1[2] * e2[1], n1 = e1[2] * e2[0] - e1[0] * e2[2], n2 = e1[0] * e2[1] - e1[1] * e2[0];
  return n0 * aw[0] + n1 * aw[1] + n2 * aw[2] < 0;
}

void put_triangle(const float* p0, const float* p1, const float* p2, bool flip, std::vector<float>& out) {
  const float* q1 = flip ? p2 : p1;
  const float* q2 = flip ? p1 : p2;
  for (int c = 0; c < 3; ++c) out.push_back(p0[c]);
  for (int c = 0; c < 3; ++c) out.push_back(q1[c]);
  for (int c = 0; c < 3; ++c) out.push_back(q2[c]);
}

void tet_triangles(const float f[8], unsigned inside, int t, int i, int j, int k, float iso, float vdx,
                   std::vector<float>& out) {
  int q[4], in[4], n_in = 0;
  for (int r = 0; r < 4; ++r) {
    q[r] = kTets[t][r];
    in[r] = (inside >> q[r]) & 1;
    n_in += in[r];
  }
  if (n_in == 0 || n_in == 4) return;
  if (n_in == 1 || n_in == 3) {
    int lone = 0;
    for (int r = 0; r < 4; ++r)
      if (in[r] == (n_in == 1)) lone = r;
    int o[3], m = 0;
    for (int r = 0; r < 4; ++r)
      if (r != lone) o[m++] = q[r];
    float p[3][3];
    for (int e = 0; e < 3; ++e) {
      if (n_in == 1) edge_point(f, q[lone], o[e], i, j, k, iso, vdx, p[e]);
      else edge_point(f, o[e], q[lone], i, j, k, iso, vdx, p[e]);
    }
    const int det = det3(q[lone], o[0], o[1], o[2]);
    put_triangle(p[0], p[1], p[2], n_in == 1 ? det < 0 : det > 0, out);
    return;
  }
  int a = -1, b = -1, c = -1, d = -1;
  for (int r = 0; r < 4; ++r) {
    if (in[r]) (a < 0 ? a : b) = q[r];
    else (c < 0 ? c : d) = q[r];
  }
  float ac[3], ad[3], bd[3], bc[3];
  edge_point(f, a, c, i, j, k, iso, vdx, ac);
  edge_point(f, a, d, i, j, k, iso, vdx, ad);
  edge_point(f, b, d, i, j, k, iso, vdx, bd);
  edge_point(f, b, c, i, j, k, iso, vdx, bc);
  const bool flip = quad_flip(a, b, c, d);
  put_triangle(ac, ad, bd, flip, out);
  put_triangle(ac, bd, bc, flip, out);
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

/* Triangles of the level set radius voxel_dx - field = 0, 9 floats each, in cell order
 * (cell (i, j, k) at index (i (G-1) + j) (G-1) + k, then tetrahedra 0..5).  Writes up to
 * `capacity` triangles and returns the count. */
int64_t oracle_surface_mesh(const float* field, int32_t G, int32_t radius, double voxel_dx, float* tris,
                            int64_t capacity) {
  if (G < 2) return 0;
  // corner inside  <=>  S = radius voxel_dx - field > 0 in double  <=>  field < thr
  const double iso = (double)(uint32_t)radius * voxel_dx;
  const float iso_f = (float)iso;
  const float vdx = (float)voxel_dx;
  std::vector<float> out;
  for (int i = 0; i + 1 < G; ++i)
    for (int j = 0; j + 1 < G; ++j)
      for (int k = 0; k + 1 < G; ++k) {
        float f[8];
        unsigned inside = 0;
        for (int q = 0; q < 8; ++q) {
          f[q] = field[((int64_t)(i + (q >> 2)) * G + j + ((q >> 1) & 1)) * G + k + (q & 1)];
          inside |= (unsigned)((double)f[q] < iso) << q;
        }
        for (int t = 0; t < 6; ++t) tet_triangles(f, inside, t, i, j, k, iso_f, vdx, out);
      }
  const int64_t n = (int64_t)(out.size() / 9);
  std::copy(out.begin(), out.begin() + 9 * std::min(n, capacity), tris);
  return n;
}

}  // extern "C"
