// Surface reconstruction of the particles on the GPU.
//
// The reference meshes the particles on the host (MeshBuilder::computeMesh,
// include/mesh_builder.h:170-211): a voxel grid of side G (voxel_dx = N dx / G) holds, per
// node, the distance to the nearest particle within a cutoff of (radius + 1) voxels
// (fillVoxelGrid_distance, include/mesh_builder.h:89-137); the surface is the zero level
// of S = radius * voxel_dx - distance, extracted with libigl's marching cubes.  Here:
//   * the distance field is a particle scatter: one warp per particle walks the node box
//     the reference walks and lowers each node with an integer atomicMin on the float's
//     bits (distances are non-negative, so the orders agree); the float arithmetic is the
//     reference's, so the field matches its sequential loop bit for bit;
//   * the level set is extracted by marching tetrahedra: each voxel cell is split into the
//     six tetrahedra around its main diagonal (the same split in every cell, so the
//     surface has no cracks), each tetrahedron gives 0, 1 or 2 triangles with vertices
//     interpolated linearly on its edges, oriented from S > 0 to S < 0.  libigl is not
//     available; marching tetrahedra yields the same level set with a finer triangulation.
//     A count pass, an exclusive scan over blocks and a write pass emit the triangles in
//     cell order, so the mesh is deterministic.
#include <algorithm>
#include <cmath>

#include "mpm_internal.h"
#include "surface.h"

namespace mpm {

namespace {

constexpr int kSurfThreads = 256;

// One warp per particle: the node box [int(x/dx - r), int(x/dx + r + 1)) clamped to the
// grid, d = |x - x_node| in float (include/mesh_builder.h:112-133).
__global__ void distance_kernel(const float* __restrict__ s, int64_t st, int64_t n, float vdx, float rg, int G,
                                int* __restrict__ field) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t p = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); p < n; p += warps) {
    const float x0 = s[(kX + 0) * st + p], x1 = s[(kX + 1) * st + p], x2 = s[(kX + 2) * st + p];
    const float g0 = x0 / vdx, g1 = x1 / vdx, g2 = x2 / vdx;
    const int b0 = max(0, (int)(g0 - rg)), b1 = max(0, (int)(g1 - rg)), b2 = max(0, (int)(g2 - rg));
    const int e0 = min(G, (int)(g0 + (rg + 1.f))), e1 = min(G, (int)(g1 + (rg + 1.f))), e2 = min(G, (int)(g2 + (rg + 1.f)));
    const int n0 = e0 - b0, n1 = e1 - b1, n2 = e2 - b2;
    // a particle outside the grid (or NaN) has an empty box on some axis
    if (n0 <= 0 || n1 <= 0 || n2 <= 0) continue;
    const int vol = n0 * n1 * n2;
    for (int q = lane; q < vol; q += 32) {
      const int i = b0 + q / (n1 * n2), rem = q % (n1 * n2);
      const int j = b1 + rem / n2, k = b2 + rem % n2;
      const float d0 = __fsub_rn(x0, __fmul_rn((float)i, vdx));
      const float d1 = __fsub_rn(x1, __fmul_rn((float)j, vdx));
      const float d2 = __fsub_rn(x2, __fmul_rn((float)k, vdx));
      const float d = __fsqrt_rn(__fadd_rn(__fmul_rn(d0, d0), __fadd_rn(__fmul_rn(d1, d1), __fmul_rn(d2, d2))));
      atomicMin(field + ((int64_t)i * G + j) * G + k, __float_as_int(d));
    }
  }
}

__global__ void fill_kernel(int* field, int64_t cells, float value) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < cells; c += (int64_t)gridDim.x * blockDim.x)
    field[c] = __float_as_int(value);
}

__device__ __forceinline__ double level(const float* field, int G, int i, int j, int k, double iso) {
  return __dsub_rn(iso, (double)field[((int64_t)i * G + j) * G + k]);
}

// Triangles of one cell (up to 12): values of its 8 corners, then the 6 tetrahedra.
__device__ int cell_triangles(const float* field, int G, int64_t c, double iso, double vdx, float* out) {
  const int Gm = G - 1;
  const int i = (int)(c / ((int64_t)Gm * Gm)), j = (int)((c / Gm) % Gm), k = (int)(c % Gm);
  double v[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) v[q] = level(field, G, i + (q >> 2), j + ((q >> 1) & 1), k + (q & 1), iso);
  int cnt = 0;
#pragma unroll
  for (int t = 0; t < 6; ++t) cnt += tet_triangles(v, t, i, j, k, vdx, out ? out + 9 * cnt : nullptr);
  return cnt;
}

__global__ void __launch_bounds__(kSurfThreads) mc_count_kernel(const float* field, int G, double iso,
                                                                int* block_counts) {
  __shared__ int warp_sum[kSurfThreads / 32];
  const int64_t Gm = G - 1, cells = Gm * Gm * Gm;
  const int64_t c = (int64_t)blockIdx.x * kSurfThreads + threadIdx.x;
  int cnt = (c < cells) ? cell_triangles(field, G, c, iso, 0.0, nullptr) : 0;
#pragma unroll
  for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(kFull, cnt, o);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int tot = 0;
    for (int w = 0; w < kSurfThreads / 32; ++w) tot += warp_sum[w];
    block_counts[blockIdx.x] = tot;
  }
}

__global__ void __launch_bounds__(kSurfThreads) mc_write_kernel(const float* field, int G, double iso, double vdx,
                                                                const int* block_offsets, float* tris) {
  __shared__ int warp_sum[kSurfThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t Gm = G - 1, cells = Gm * Gm * Gm;
  const int64_t c = (int64_t)blockIdx.x * kSurfThreads + threadIdx.x;
  float local[9 * 12];
  const int cnt = (c < cells) ? cell_triangles(field, G, c, iso, vdx, local) : 0;
  int inc = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_sum[warp] = inc;
  __syncthreads();
  int wpre = 0;
  for (int w = 0; w < warp; ++w) wpre += warp_sum[w];
  const int64_t out = (int64_t)block_offsets[blockIdx.x] + wpre + inc - cnt;
  for (int q = 0; q < 9 * cnt; ++q) tris[9 * out + q] = local[q];
}

}  // namespace

cudaError_t launch_distance_field(const float* s, int64_t stride, int64_t n, int G, int radius, double voxel_dx,
                                  float* field, cudaStream_t st) {
  const int64_t cells = (int64_t)G * G * G;
  // fillVoxelGrid_distance takes dx and the cutoff as float (include/mesh_builder.h:89)
  const float vdx = (float)voxel_dx;
  const float cutoff = (float)((double)(radius + 1) * voxel_dx);
  fill_kernel<<<(int)std::min<int64_t>((cells + 255) / 256, 8192), 256, 0, st>>>((int*)field, cells, cutoff);
  if (n > 0) {
    const float rg = cutoff / vdx;
    const int blocks = (int)std::min<int64_t>((n + 7) / 8, 8192);
    distance_kernel<<<blocks, 256, 0, st>>>(s, stride, n, vdx, rg, G, (int*)field);
  }
  return cudaGetLastError();
}

cudaError_t extract_surface(const float* field, int G, int radius, double voxel_dx, cudaStream_t st, float** tris_out,
                            int64_t* n_out) {
  *tris_out = nullptr;
  *n_out = 0;
  if (G < 2) return cudaSuccess;
  const double vdx = voxel_dx;
  const double iso = (double)radius * vdx;  // S = radius * voxel_dx - distance (include/mesh_builder.h:188)
  const int64_t Gm = G - 1, cells = Gm * Gm * Gm;
  const int64_t nblocks = (cells + kSurfThreads - 1) / kSurfThreads;
  int* counts = nullptr;
  int* scratch = nullptr;
  cudaError_t e = cudaMalloc(&counts, sizeof(int) * (nblocks + 1));
  if (e == cudaSuccess) e = cudaMalloc(&scratch, sizeof(int) * scan_scratch_ints(nblocks + 1));
  if (e == cudaSuccess) e = cudaMemsetAsync(counts, 0, sizeof(int) * (nblocks + 1), st);
  if (e == cudaSuccess) {
    mc_count_kernel<<<(unsigned)nblocks, kSurfThreads, 0, st>>>(field, G, iso, counts);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = launch_exclusive_scan(counts, nblocks + 1, scratch, st, nullptr);
  int total = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&total, counts + nblocks, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  float* tris = nullptr;
  if (e == cudaSuccess && total > 0) {
    e = cudaMalloc(&tris, sizeof(float) * 9 * (size_t)total);
    if (e == cudaSuccess) {
      mc_write_kernel<<<(unsigned)nblocks, kSurfThreads, 0, st>>>(field, G, iso, vdx, counts, tris);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  cudaFree(counts);
  cudaFree(scratch);
  if (e != cudaSuccess) {
    cudaFree(tris);
    return e;
  }
  *tris_out = tris;
  *n_out = total;
  return cudaSuccess;
}

}  // namespace mpm
