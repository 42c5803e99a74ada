// Surface reconstruction (surface.cu): the marching-tetrahedra step and the launchers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mpm {

// Device buffers of the mesher, kept by the context between calls (grown, never shrunk).
struct SurfaceBuffers {
  float* field = nullptr;  // G^3 distance field
  int64_t field_cap = 0;
  int* counts = nullptr;   // triangles and surface cells per block of cells, then their exclusive scans
  int64_t counts_cap = 0;
  int2* cells = nullptr;   // per block of cells, its surface cells: packed (i, j, k), first triangle in the block
  int64_t cells_cap = 0;
  int* scan = nullptr;     // scan scratch
  int64_t scan_cap = 0;
  float* tris = nullptr;   // 9 floats per triangle
  int64_t tris_cap = 0;
  int* total = nullptr;    // pinned host words: the triangle and surface-cell counts
  bool raw = false;        // field holds squared distances (not yet min(cutoff, sqrt(.)))
  void release();
};

// Distance field of the particles into buf.field: a G^3 voxel grid of spacing voxel_dx
// with cutoff (radius + 1) voxels (MeshBuilder::computeMesh, include/mesh_builder.h:172-178).
// Without `finish` the buffer may be left holding the squared distances (buf.raw), which
// extract_surface reads directly.
cudaError_t launch_distance_field(const float* s, int64_t stride, int64_t n, int G, int radius, double voxel_dx,
                                  bool finish, SurfaceBuffers& buf, cudaStream_t st, int64_t* launches);
// Triangles (9 floats each: 3 vertices, cell order) of the level set
// radius * voxel_dx - field = 0 into buf.tris; synchronises the stream once (count).
cudaError_t extract_surface(int G, int radius, double voxel_dx, SurfaceBuffers& buf, cudaStream_t st,
                            int64_t* n_out, int64_t* launches);

#ifdef __CUDACC__
// The six tetrahedra of a voxel cell around its diagonal from corner 0 to corner 7
// (Freudenthal's split: one per order of the three axis steps).  Corner q sits at
// offset (q >> 2, (q >> 1) & 1, q & 1).
__device__ __forceinline__ int tet_corner(int t, int v) {
  constexpr int kTets[6][4] = {{0, 4, 6, 7}, {0, 4, 5, 7}, {0, 1, 5, 7}, {0, 1, 3, 7}, {0, 2, 3, 7}, {0, 2, 6, 7}};
  return kTets[t][v];
}

// Corner q of the cell sits at offset (q >> 2, (q >> 1) & 1, q & 1).
__device__ __forceinline__ int corner_bit(int q, int c) { return (q >> (2 - c)) & 1; }

// Point where the level set crosses the edge from inside corner qi to outside corner qo of
// the cell at (i, j, k), in world units.  Always interpolated from the inside corner, so
// a vertex shared by neighbouring tetrahedra and cells comes out bit-identical:
//   t = (iso - f_in) / (f_out - f_in),  p = (in + t (out - in)) dx   (float, no contraction)
__device__ __forceinline__ void edge_point(const float f[8], int qi, int qo, int i, int j, int k, float iso,
                                           float vdx, float* p) {
  const float t = __fdiv_rn(__fsub_rn(iso, f[qi]), __fsub_rn(f[qo], f[qi]));
  const int cell[3] = {i, j, k};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float a = (float)(cell[c] + corner_bit(qi, c)), b = (float)(cell[c] + corner_bit(qo, c));
    p[c] = __fmul_rn(__fadd_rn(a, __fmul_rn(t, __fsub_rn(b, a))), vdx);
  }
}

// det(A - L, B - L, C - L) of cell corners (integer offsets).
__device__ __forceinline__ int corner_det(int L, int A, int B, int C) {
  int u[3], v[3], w[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    u[c] = corner_bit(A, c) - corner_bit(L, c);
    v[c] = corner_bit(B, c) - corner_bit(L, c);
    w[c] = corner_bit(C, c) - corner_bit(L, c);
  }
  return u[0] * (v[1] * w[2] - v[2] * w[1]) - u[1] * (v[0] * w[2] - v[2] * w[0]) + u[2] * (v[0] * w[1] - v[1] * w[0]);
}

// Whether the quad (ac, ad, bd, bc) of a tetrahedron with a, b inside and c, d outside
// must be reversed to face outward: the normal of its triangle (ac, ad, bd) at the edge
// midpoints, (d - c) x (b + d - a - c), against the direction (c + d) - (a + b).
__device__ __forceinline__ bool quad_flip(int a, int b, int c, int d) {
  int e1[3], e2[3], aw[3];
#pragma unroll
  for (int x = 0; x < 3; ++x) {
    e1[x] = corner_bit(d, x) - corner_bit(c, x);
    e2[x] = corner_bit(b, x) + corner_bit(d, x) - corner_bit(a, x) - corner_bit(c, x);
    aw[x] = corner_bit(c, x) + corner_bit(d, x) - corner_bit(a, x) - corner_bit(b, x);
  }
  const int n0 = e1[1] * e2[2] - e1[2] * e2[1], n1 = e1[2] * e2[0] - e1[0] * e2[2], n2 = e1[0] * e2[1] - e1[1] * e2[0];
  return n0 * aw[0] + n1 * aw[1] + n2 * aw[2] < 0;
}

__device__ __forceinline__ void put_triangle(const float* p0, const float* p1, const float* p2, bool flip, float* out) {
  const float* q1 = flip ? p2 : p1;
  const float* q2 = flip ? p1 : p2;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    out[c] = p0[c];
    out[3 + c] = q1[c];
    out[6 + c] = q2[c];
  }
}

// Triangles of tetrahedron t of the cell (field values f at its 8 corners, corner q inside
// when bit q of `inside` is set), written to out (9 floats each), facing from the inside
// corners to the outside ones; returns their number.  Each triangle's orientation is fixed
// by the corners alone: the level set of the linear interpolant is a plane in the
// tetrahedron, so the sign of its normal against the tetrahedron's edges does not depend
// on where the plane cuts them.
__device__ __forceinline__ int tet_triangles(const float f[8], unsigned inside, int t, int i, int j, int k, float iso,
                                             float vdx, float* out) {
  int q[4], in[4], n_in = 0;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    q[r] = tet_corner(t, r);
    in[r] = (inside >> q[r]) & 1;
    n_in += in[r];
  }
  if (n_in == 0 || n_in == 4) return 0;
  if (n_in == 1 || n_in == 3) {
    // the corner alone on its side (L) and the others in tetrahedron order (A, B, C);
    // triangle (eLA, eLB, eLC) faces away from L when det(A - L, B - L, C - L) > 0
    const int want_in = n_in == 1;
    int lone = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r)
      if (in[r] == want_in) lone = r;
    int o[3], m = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r)
      if (r != lone) o[m++] = q[r];
    float p[3][3];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
      if (n_in == 1) edge_point(f, q[lone], o[e], i, j, k, iso, vdx, p[e]);
      else edge_point(f, o[e], q[lone], i, j, k, iso, vdx, p[e]);
    }
    const int det = corner_det(q[lone], o[0], o[1], o[2]);
    // outward: away from an inside L, towards an outside L
    const bool flip = n_in == 1 ? det < 0 : det > 0;
    put_triangle(p[0], p[1], p[2], flip, out);
    return 1;
  }
  // two corners inside (a, b), two outside (c, d): the quad a-c, a-d, b-d, b-c
  int a = -1, b = -1, c = -1, d = -1;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    if (in[r]) {
      if (a < 0) a = q[r]; else b = q[r];
    } else {
      if (c < 0) c = q[r]; else d = q[r];
    }
  }
  float ac[3], ad[3], bd[3], bc[3];
  edge_point(f, a, c, i, j, k, iso, vdx, ac);
  edge_point(f, a, d, i, j, k, iso, vdx, ad);
  edge_point(f, b, d, i, j, k, iso, vdx, bd);
  edge_point(f, b, c, i, j, k, iso, vdx, bc);
  const bool flip = quad_flip(a, b, c, d);
  put_triangle(ac, ad, bd, flip, out);
  put_triangle(ac, bd, bc, flip, out + 9);
  return 2;
}
#endif

}  // namespace mpm
