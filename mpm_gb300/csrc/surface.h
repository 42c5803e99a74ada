// Surface reconstruction (surface.cu): the marching-tetrahedra step and the launchers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mpm {

// Distance field of the particles on a G^3 voxel grid of spacing voxel_dx with cutoff
// (radius + 1) voxels (MeshBuilder::computeMesh, include/mesh_builder.h:172-178).
cudaError_t launch_distance_field(const float* s, int64_t stride, int64_t n, int G, int radius, double voxel_dx,
                                  float* field, cudaStream_t st);
// Triangles (9 floats each: 3 vertices, cell order) of the level set
// radius * voxel_dx - field = 0; *tris_out is device memory owned by the caller.
cudaError_t extract_surface(const float* field, int G, int radius, double voxel_dx, cudaStream_t st, float** tris_out,
                            int64_t* n_out);

#ifdef __CUDACC__
// The six tetrahedra of a voxel cell around its diagonal from corner 0 to corner 7
// (Freudenthal's split: one per order of the three axis steps).  Corner q sits at
// offset (q >> 2, (q >> 1) & 1, q & 1).
__device__ __forceinline__ int tet_corner(int t, int v) {
  constexpr int kTets[6][4] = {{0, 4, 6, 7}, {0, 4, 5, 7}, {0, 1, 5, 7}, {0, 1, 3, 7}, {0, 2, 3, 7}, {0, 2, 6, 7}};
  return kTets[t][v];
}

// Point where the level set crosses edge (qa, qb) of the cell at (i, j, k), in world units.
__device__ __forceinline__ void edge_point(const double v[8], int qa, int qb, int i, int j, int k, double vdx,
                                           double p[3]) {
  const double t = __ddiv_rn(v[qa], __dsub_rn(v[qa], v[qb]));
  const double a[3] = {(double)(i + (qa >> 2)), (double)(j + ((qa >> 1) & 1)), (double)(k + (qa & 1))};
  const double b[3] = {(double)(i + (qb >> 2)), (double)(j + ((qb >> 1) & 1)), (double)(k + (qb & 1))};
#pragma unroll
  for (int c = 0; c < 3; ++c) p[c] = __dmul_rn(__dadd_rn(a[c], __dmul_rn(t, __dsub_rn(b[c], a[c]))), vdx);
}

// Writes triangle (p0, p1, p2), swapping p1 and p2 when its normal does not point along
// `away` (from the inside corners to the outside ones).
__device__ __forceinline__ void put_triangle(const double p0[3], const double p1[3], const double p2[3],
                                             const double away[3], float* out) {
  const double e1[3] = {__dsub_rn(p1[0], p0[0]), __dsub_rn(p1[1], p0[1]), __dsub_rn(p1[2], p0[2])};
  const double e2[3] = {__dsub_rn(p2[0], p0[0]), __dsub_rn(p2[1], p0[1]), __dsub_rn(p2[2], p0[2])};
  const double nx = __dsub_rn(__dmul_rn(e1[1], e2[2]), __dmul_rn(e1[2], e2[1]));
  const double ny = __dsub_rn(__dmul_rn(e1[2], e2[0]), __dmul_rn(e1[0], e2[2]));
  const double nz = __dsub_rn(__dmul_rn(e1[0], e2[1]), __dmul_rn(e1[1], e2[0]));
  const double dot = __dadd_rn(__dadd_rn(__dmul_rn(nx, away[0]), __dmul_rn(ny, away[1])), __dmul_rn(nz, away[2]));
  const double* q1 = dot < 0.0 ? p2 : p1;
  const double* q2 = dot < 0.0 ? p1 : p2;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    out[c] = (float)p0[c];
    out[3 + c] = (float)q1[c];
    out[6 + c] = (float)q2[c];
  }
}

// Triangles of tetrahedron t of the cell (values v of the level-set function S at its 8
// corners, inside where S > 0); writes them to out (9 floats each) unless out is null.
__device__ __forceinline__ int tet_triangles(const double v[8], int t, int i, int j, int k, double vdx, float* out) {
  int q[4], in[4], n_in = 0;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    q[r] = tet_corner(t, r);
    in[r] = v[q[r]] > 0.0;
    n_in += in[r];
  }
  if (n_in == 0 || n_in == 4) return 0;
  if (!out) return n_in == 2 ? 2 : 1;
  // direction from the inside corners' centroid to the outside ones' (grid units)
  double cin[3] = {0, 0, 0}, cout[3] = {0, 0, 0};
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const double o[3] = {(double)(q[r] >> 2), (double)((q[r] >> 1) & 1), (double)(q[r] & 1)};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (in[r]) cin[c] = __dadd_rn(cin[c], o[c]);
      else cout[c] = __dadd_rn(cout[c], o[c]);
    }
  }
  const double ni = (double)n_in, no = (double)(4 - n_in);
  const double away[3] = {__dsub_rn(__ddiv_rn(cout[0], no), __ddiv_rn(cin[0], ni)),
                          __dsub_rn(__ddiv_rn(cout[1], no), __ddiv_rn(cin[1], ni)),
                          __dsub_rn(__ddiv_rn(cout[2], no), __ddiv_rn(cin[2], ni))};
  if (n_in == 1 || n_in == 3) {
    // the corner on its own side and the three edges from it
    int lone = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r)
      if (in[r] == (n_in == 1)) lone = r;
    double p[3][3];
    int m = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r)
      if (r != lone) {
        edge_point(v, q[lone], q[r], i, j, k, vdx, p[m]);
        ++m;
      }
    put_triangle(p[0], p[1], p[2], away, out);
    return 1;
  }
  // two corners inside (a, b), two outside (c, d): the quad a-c, a-d, b-d, b-c
  int a = -1, b = -1, c = -1, d = -1;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    if (in[r]) {
      if (a < 0) a = r; else b = r;
    } else {
      if (c < 0) c = r; else d = r;
    }
  }
  double ac[3], ad[3], bd[3], bc[3];
  edge_point(v, q[a], q[c], i, j, k, vdx, ac);
  edge_point(v, q[a], q[d], i, j, k, vdx, ad);
  edge_point(v, q[b], q[d], i, j, k, vdx, bd);
  edge_point(v, q[b], q[c], i, j, k, vdx, bc);
  put_triangle(ac, ad, bd, away, out);
  put_triangle(ac, bd, bc, away, out + 9);
  return 2;
}
#endif

}  // namespace mpm
