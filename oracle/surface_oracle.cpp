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
 * zero level set by marching tetrahedra; this file restates that extraction (same split
 * of each cell into six tetrahedra around its main diagonal, same edge interpolation,
 * same orientation rule, same emission order) in IEEE double without contraction (built
 * with -ffp-contract=off), so the triangle lists agree bit for bit.
 */
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <vector>

namespace {

const int kTets[6][4] = {{0, 4, 6, 7}, {0, 4, 5, 7}, {0, 1, 5, 7}, {0, 1, 3, 7}, {0, 2, 3, 7}, {0, 2, 6, 7}};

void edge_point(const double v[8], int qa, int qb, int i, int j, int k, double vdx, double p[3]) {
  const double t = v[qa] / (v[qa] - v[qb]);
  const double a[3] = {(double)(i + (qa >> 2)), (double)(j + ((qa >> 1) & 1)), (double)(k + (qa & 1))};
  const double b[3] = {(double)(i + (qb >> 2)), (double)(j + ((qb >> 1) & 1)), (double)(k + (qb & 1))};
  for (int c = 0; c < 3; ++c) p[c] = (a[c] + t * (b[c] - a[c])) * vdx;
}

void put_triangle(const double p0[3], const double p1[3], const double p2[3], const double away[3],
                  std::vector<float>& out) {
  const double e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
  const double e2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
  const double nx = e1[1] * e2[2] - e1[2] * e2[1];
  const double ny = e1[2] * e2[0] - e1[0] * e2[2];
  const double nz = e1[0] * e2[1] - e1[1] * e2[0];
  const double dot = (nx * away[0] + ny * away[1]) + nz * away[2];
  const double* q1 = dot < 0.0 ? p2 : p1;
  const double* q2 = dot < 0.0 ? p1 : p2;
  for (int c = 0; c < 3; ++c) out.push_back((float)p0[c]);
  for (int c = 0; c < 3; ++c) out.push_back((float)q1[c]);
  for (int c = 0; c < 3; ++c) out.push_back((float)q2[c]);
}

void tet_triangles(const double v[8], int t, int i, int j, int k, double vdx, std::vector<float>& out) {
  int q[4], in[4], n_in = 0;
  for (int r = 0; r < 4; ++r) {
    q[r] = kTets[t][r];
    in[r] = v[q[r]] > 0.0;
    n_in += in[r];
  }
  if (n_in == 0 || n_in == 4) return;
  double cin[3] = {0, 0, 0}, cout[3] = {0, 0, 0};
  for (int r = 0; r < 4; ++r) {
    const double o[3] = {(double)(q[r] >> 2), (double)((q[r] >> 1) & 1), (double)(q[r] & 1)};
    for (int c = 0; c < 3; ++c) (in[r] ? cin : cout)[c] += o[c];
  }
  const double ni = n_in, no = 4 - n_in;
  const double away[3] = {cout[0] / no - cin[0] / ni, cout[1] / no - cin[1] / ni, cout[2] / no - cin[2] / ni};
  if (n_in == 1 || n_in == 3) {
    int lone = 0;
    for (int r = 0; r < 4; ++r)
      if (in[r] == (n_in == 1)) lone = r;
    double p[3][3];
    int m = 0;
    for (int r = 0; r < 4; ++r)
      if (r != lone) edge_point(v, q[lone], q[r], i, j, k, vdx, p[m++]);
    put_triangle(p[0], p[1], p[2], away, out);
    return;
  }
  int a = -1, b = -1, c = -1, d = -1;
  for (int r = 0; r < 4; ++r) {
    if (in[r]) (a < 0 ? a : b) = r;
    else (c < 0 ? c : d) = r;
  }
  double ac[3], ad[3], bd[3], bc[3];
  edge_point(v, q[a], q[c], i, j, k, vdx, ac);
  edge_point(v, q[a], q[d], i, j, k, vdx, ad);
  edge_point(v, q[b], q[d], i, j, k, vdx, bd);
  edge_point(v, q[b], q[c], i, j, k, vdx, bc);
  put_triangle(ac, ad, bd, away, out);
  put_triangle(ac, bd, bc, away, out);
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
  const double iso = (double)(uint32_t)radius * voxel_dx;
  std::vector<float> out;
  for (int i = 0; i + 1 < G; ++i)
    for (int j = 0; j + 1 < G; ++j)
      for (int k = 0; k + 1 < G; ++k) {
        double v[8];
        for (int q = 0; q < 8; ++q)
          v[q] = iso - (double)field[((int64_t)(i + (q >> 2)) * G + j + ((q >> 1) & 1)) * G + k + (q & 1)];
        for (int t = 0; t < 6; ++t) tet_triangles(v, t, i, j, k, voxel_dx, out);
      }
  const int64_t n = (int64_t)(out.size() / 9);
  std::copy(out.begin(), out.begin() + 9 * std::min(n, capacity), tris);
  return n;
}

}  // extern "C"
