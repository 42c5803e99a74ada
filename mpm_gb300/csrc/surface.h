// Surface reconstruction (surface.cu): the distance field, marching cubes and the launchers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mpm {

// Device buffers of the mesher, kept by the context between calls (grown, never shrunk).
struct SurfaceBuffers {
  float* field = nullptr;  // G^3 distance field
  int64_t field_cap = 0;
  int* counts = nullptr;   // per block of cubes: triangles | new vertices | surface cubes, then their scan
  int64_t counts_cap = 0;
  int4* cells = nullptr;   // per block of cubes, its surface cubes: packed (i, j, k), first triangle and
                           // first vertex inside the block, inside-corner mask
  int64_t cells_cap = 0;
  int* scan = nullptr;     // scan scratch
  int64_t scan_cap = 0;
  double* verts = nullptr; // 3 doubles per vertex
  int64_t verts_cap = 0;
  int* faces = nullptr;    // 3 vertex indices per triangle
  int64_t faces_cap = 0;
  float* tris = nullptr;   // 9 floats per triangle (the triangle soup)
  int64_t tris_cap = 0;
  int* total = nullptr;    // pinned host words: triangle, vertex and surface-cube counts
  bool raw = false;        // field holds squared distances (not yet min(cutoff, sqrt(.)))
  void release();
};

// Distance field of the particles into buf.field: a G^3 voxel grid of spacing voxel_dx
// with cutoff (radius + 1) voxels (MeshBuilder::computeMesh, include/mesh_builder.h:172-178).
// Without `finish` the buffer may be left holding the squared distances (buf.raw), which
// extract_surface reads directly.
cudaError_t launch_distance_field(const float* s, int64_t stride, int64_t n, int G, int radius, double voxel_dx,
                                  bool finish, SurfaceBuffers& buf, cudaStream_t st, int64_t* launches);
// Marching cubes of the level set radius * voxel_dx - field = 0: vertices into buf.verts
// (in the order libigl's marching cubes creates them) and faces into buf.faces, plus the
// triangle soup into buf.tris when `soup`; synchronises the stream once (counts).
cudaError_t extract_surface(int G, int radius, double voxel_dx, SurfaceBuffers& buf, cudaStream_t st, bool soup,
                            int64_t* n_verts, int64_t* n_faces, int64_t* launches);
// The triangle table: counts[256] and slots[256 * 30] (edge slots, -1 past the count).
void surface_table(int32_t* counts, int32_t* slots);

// Device buffers of the Laplacian smoother (smooth.cu), kept by the context between calls
// (grown, never shrunk).
struct SmoothBuffers {
  double* C = nullptr;     // per face: the three cotangent entries and the double area
  int64_t C_cap = 0;
  double* vec = nullptr;   // per vertex: M, D = -L(i, i), 1 / S(i, i); then Y, r, p, q (3 each)
  int64_t vec_cap = 0;
  double* part = nullptr;  // per-block partial sums
  int64_t part_cap = 0;
  int* ints = nullptr;     // row offsets, fill counters, scan scratch, corners, row lengths, neighbours
  int64_t ints_cap = 0;
  double* w = nullptr;     // the entries L(i, j) of the rows' neighbours
  int64_t w_cap = 0;
  double* scal = nullptr;  // the solver's scalars
  int* flags = nullptr;    // check bits and the last-block ticket
  double* V = nullptr;     // staging of host vertices
  int64_t V_cap = 0;
  int* F = nullptr;        // staging of host faces
  int64_t F_cap = 0;
  double* host = nullptr;  // pinned words read back by the solver
  void release();
};

constexpr double kSmoothTolerance = 1e-12;  // relative residual per coordinate
constexpr int kSmoothMaxIterations = 20000;
constexpr int kSmoothCheckEvery = 16;       // iterations between residual read-backs

struct SmoothResult {
  int iterations = 0;
  double relative_residual = 0.0;  // largest over the coordinates
  bool converged = false;
  bool bad_index = false;  // a face index outside [0, n_vertices)
  bool bad_area = false;   // a face of zero area
};

// One implicit Laplacian smoothing step of the mesh (V: 3 doubles per vertex, F: 3 indices
// per face, both on the device), written over V, and the rescale to unit area
// (MeshBuilder::smoothMesh, include/mesh_builder.h:212-245).  V is left unchanged when the
// result reports a bad index, a degenerate face or no convergence.  Synchronises the stream.
cudaError_t smooth_mesh(double* V, const int* F, int64_t nv, int64_t nf, SmoothBuffers& sb, cudaStream_t st,
                        int64_t* launches, SmoothResult* res);

// Marching cubes in libigl's cube layout, on nodes (i, j, k) with k fastest as
// MeshBuilder::computeMesh lays them out (include/mesh_builder.h:181-193).  Corner n of a
// cube sits at offset kCorner[n] (di, dj, dk) from its lowest node; edge slot e joins
// corners kEdge[e][0] and kEdge[e][1], the lower node first.  The triangle table is this
// project's own: on each cube face (corners counter-clockwise seen from outside) a
// segment joins the edge where the corner cycle enters the inside (S > 0) to the edge
// where it leaves it, and a face with two opposite inside corners cuts each one off; the
// segments close into loops, and each loop (started at its lowest slot) is fanned from
// its first edge.  Neighbouring cubes see the same segments on their shared face, so the
// surface is closed; the triangles face outward (towards S < 0).
namespace mc {

constexpr int kCorner[8][3] = {{0, 0, 0}, {0, 0, 1}, {0, 1, 1}, {0, 1, 0}, {1, 0, 0}, {1, 0, 1}, {1, 1, 1}, {1, 1, 0}};
constexpr int kEdge[12][2] = {{0, 1}, {1, 2}, {3, 2}, {0, 3}, {4, 5}, {5, 6}, {7, 6}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
constexpr int kFace[6][4] = {{0, 1, 2, 3}, {4, 7, 6, 5}, {0, 4, 5, 1}, {3, 2, 6, 7}, {0, 3, 7, 4}, {1, 5, 6, 2}};

struct Table {
  uint8_t count[256];      // triangles of an inside-corner mask
  uint16_t crossed[256];   // its edge slots whose two corners differ
  int8_t slot[256][30];    // edge slots, 3 per triangle (at most 10)
};

constexpr int edge_of(int a, int b) {
  for (int e = 0; e < 12; ++e)
    if ((kEdge[e][0] == a && kEdge[e][1] == b) || (kEdge[e][0] == b && kEdge[e][1] == a)) return e;
  return -1;
}

// The edge slot along axis ax (0 i, 1 j, 2 k) whose lower corner sits at offset
// (o0, o1, o2); 15 when there is none.
constexpr int slot_along(int ax, int o0, int o1, int o2) {
  for (int e = 0; e < 12; ++e) {
    const int* a = kCorner[kEdge[e][0]];
    const int* b = kCorner[kEdge[e][1]];
    const int eax = a[0] != b[0] ? 0 : a[1] != b[1] ? 1 : 2;
    if (eax == ax && a[0] == o0 && a[1] == o1 && a[2] == o2) return e;
  }
  return 15;
}

constexpr Table make_table() {
  Table t{};
  for (int m = 0; m < 256; ++m) {
    int next[12] = {-1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1};
    unsigned crossed = 0;
    for (int e = 0; e < 12; ++e)
      if (((m >> kEdge[e][0]) ^ (m >> kEdge[e][1])) & 1) crossed |= 1u << e;
    for (int f = 0; f < 6; ++f) {
      bool in[4] = {false, false, false, false};
      for (int r = 0; r < 4; ++r) in[r] = (m >> kFace[f][r]) & 1;
      int enter[2] = {-1, -1}, leave = -1, ne = 0;
      for (int r = 0; r < 4; ++r) {
        const int rn = (r + 1) & 3;
        if (!in[r] && in[rn]) enter[ne++] = r;  // face edge r joins corners r and r + 1
        if (in[r] && !in[rn]) leave = r;
      }
      if (ne == 1) {
        next[edge_of(kFace[f][enter[0]], kFace[f][(enter[0] + 1) & 3])] =
            edge_of(kFace[f][leave], kFace[f][(leave + 1) & 3]);
      } else if (ne == 2) {  // opposite inside corners: each is cut off on its own
        for (int q = 0; q < 2; ++q) {
          const int r = enter[q];
          next[edge_of(kFace[f][r], kFace[f][(r + 1) & 3])] =
              edge_of(kFace[f][(r + 1) & 3], kFace[f][(r + 2) & 3]);
        }
      }
    }
    bool seen[12] = {false, false, false, false, false, false, false, false, false, false, false, false};
    int n = 0;
    for (int e0 = 0; e0 < 12; ++e0) {
      if (next[e0] < 0 || seen[e0]) continue;
      int loop[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
      int len = 0;
      for (int e = e0; !seen[e]; e = next[e]) {
        seen[e] = true;
        loop[len++] = e;
      }
      for (int r = 1; r + 1 < len; ++r, ++n) {
        t.slot[m][3 * n + 0] = (int8_t)loop[0];
        t.slot[m][3 * n + 1] = (int8_t)loop[r];
        t.slot[m][3 * n + 2] = (int8_t)loop[r + 1];
      }
    }
    for (int r = 3 * n; r < 30; ++r) t.slot[m][r] = -1;
    t.count[m] = (uint8_t)n;
    t.crossed[m] = (uint16_t)crossed;
  }
  return t;
}

}  // namespace mc

}  // namespace mpm
