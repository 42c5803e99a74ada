// Surface reconstruction of the particles on the GPU.
//
// The reference meshes the particles on the host (MeshBuilder::computeMesh,
// include/mesh_builder.h:170-211): a voxel grid of side G (voxel_dx = N dx / G) holds, per
// node, the distance to the nearest particle within a cutoff of (radius + 1) voxels
// (fillVoxelGrid_distance, include/mesh_builder.h:89-137); the surface is the zero level
// of S = radius * voxel_dx - distance, extracted with libigl's marching cubes.  Here:
//   * the distance field is a particle scatter of SQUARED distances: the square root is
//     monotone and correctly rounded, so sqrt(min s) = min sqrt(s) bit for bit and the
//     root is taken once per node afterwards (field = min(cutoff, sqrt(s_min))).  A CTA
//     takes 128 consecutive particles; when the union of their node boxes fits in shared
//     memory (the particles are cell-sorted, so it normally does) it scatters into a
//     shared tile with shared atomics and flushes each touched node with one global
//     atomicMin; otherwise each particle scatters straight to global memory.  Squared
//     distances are non-negative floats, so integer order on their bits is float order;
//     the float arithmetic per (particle, node) pair is the reference's, so the field
//     matches its sequential loop bit for bit;
//   * the level set is extracted by marching tetrahedra: each voxel cell is split into the
//     six tetrahedra around its main diagonal (the same split in every cell, so the
//     surface has no cracks), each tetrahedron gives 0, 1 or 2 triangles with vertices
//     interpolated linearly on its edges, oriented from S > 0 to S < 0.  libigl is not
//     available; marching tetrahedra yields the same level set with a finer triangulation.
//     Corners are classified as the reference's double S > 0 (one float compare against
//     the equivalent float threshold); edge points are interpolated in float (the
//     triangles are float anyway; the double path cost far more on this part, whose FP64
//     rate is a small fraction of its FP32 rate).  A count pass, an exclusive scan over
//     blocks and a write pass emit the triangles in cell order, so the mesh is
//     deterministic.
#include <algorithm>
#include <climits>
#include <cmath>

#include "mpm_internal.h"
#include "surface.h"

namespace mpm {

namespace {

constexpr int kSurfThreads = 256;
constexpr int kDistChunk = 128;     // particles per CTA and chunk
constexpr int kDistTile = 11264;    // shared-memory nodes of a chunk's tile (44 KB; all shared data stays under 48 KB)
constexpr unsigned kInfBits = 0x7f800000u;

struct NodeBox {
  int b[3], e[3];  // [b, e) per axis, clamped to the grid
};

// The node box [int(x/dx - r), int(x/dx + r + 1)) clamped to [0, G) (include/mesh_builder.h:112-121).
__device__ __forceinline__ NodeBox node_box(const float x[3], float vdx, float rg, int G) {
  NodeBox bx;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float g = x[c] / vdx;
    bx.b[c] = max(0, (int)(g - rg));
    bx.e[c] = min(G, (int)(g + (rg + 1.f)));
  }
  return bx;
}

// Squared distance from x to node (i, j, k) in the reference's float operations
// (x_node = i * dx, d = x - x_node, |d|^2 summed as d0^2 + (d1^2 + d2^2)).
__device__ __forceinline__ unsigned sq_dist_bits(const float x[3], int i, int j, int k, float vdx) {
  const float d0 = __fsub_rn(x[0], __fmul_rn((float)i, vdx));
  const float d1 = __fsub_rn(x[1], __fmul_rn((float)j, vdx));
  const float d2 = __fsub_rn(x[2], __fmul_rn((float)k, vdx));
  return __float_as_uint(__fadd_rn(__fmul_rn(d0, d0), __fadd_rn(__fmul_rn(d1, d1), __fmul_rn(d2, d2))));
}

// One warp walks the nodes of a particle's box, lane-strided in (i, j, k) order, and calls
// f(i, j, k) for each.  The position advances by 32 in mixed radix (no divisions in the loop).
template <class F>
__device__ __forceinline__ void walk_box(const NodeBox& bx, int lane, F&& f) {
  const int n0 = bx.e[0] - bx.b[0], n1 = bx.e[1] - bx.b[1], n2 = bx.e[2] - bx.b[2];
  if (n0 <= 0 || n1 <= 0 || n2 <= 0) return;  // outside the grid (or NaN)
  const int vol = n0 * n1 * n2;
  const int dk = 32 % n2, dj = (32 / n2) % n1, di = (32 / n2) / n1;
  int i = lane / (n1 * n2), j = (lane / n2) % n1, k = lane % n2;
  for (int q = lane; q < vol; q += 32) {
    f(bx.b[0] + i, bx.b[1] + j, bx.b[2] + k);
    k += dk;
    int carry = k >= n2;
    k -= carry ? n2 : 0;
    j += dj + carry;
    carry = j >= n1;
    j -= carry ? n1 : 0;
    i += di + carry;
  }
}

__global__ void fill_bits_kernel(unsigned* field, int64_t cells, unsigned value) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < cells; c += (int64_t)gridDim.x * blockDim.x)
    field[c] = value;
}

// Scatter of the squared distances of particles [p0, p0 + pc) of the chunk (positions in
// px) into dst, node (i, j, k) at ((i - B0) T1 + (j - B1)) T2 + (k - B2): a shared tile,
// or the global field with B = 0 and T1 = T2 = G.  Two particles per warp, one per half;
// lane kl of a half takes node column k = b2 + kl and holds the particle's squared axis
// terms for i = b0 + kl and j = b1 + kl, which the (i, j) loop broadcasts by shuffle.
// Needs every box to span at most 16 nodes per axis.  dump: 32 shared words, one per
// lane, that the shared-tile variant's idle lanes target instead of branching.
template <bool TILE>
__device__ __forceinline__ void scatter_half(unsigned* dst, int B0, int B1, int B2, int T1, int T2,
                                             const float (*px)[3], int p0, int pc, float vdx, float rg, int G,
                                             int warp, int lane, unsigned* dump) {
  const int h = lane & 16, kl = lane & 15;
  for (int q0 = 2 * warp; q0 < pc; q0 += 2 * (kSurfThreads / 32)) {
    const int q = q0 + (h >> 4);
    int n0 = 0, n1 = 0, n2 = 0;
    float D0 = 0.f, D1 = 0.f, D2 = 0.f;
    int base = 0;
    if (q < pc) {
      const float x[3] = {px[p0 + q][0], px[p0 + q][1], px[p0 + q][2]};
      const NodeBox bx = node_box(x, vdx, rg, G);
      n0 = bx.e[0] - bx.b[0];
      n1 = bx.e[1] - bx.b[1];
      n2 = bx.e[2] - bx.b[2];
      if (n0 <= 0 || n1 <= 0 || n2 <= 0) n0 = n1 = n2 = 0;  // outside the grid (or NaN)
      const float d0 = __fsub_rn(x[0], __fmul_rn((float)(bx.b[0] + kl), vdx));
      const float d1 = __fsub_rn(x[1], __fmul_rn((float)(bx.b[1] + kl), vdx));
      const float d2 = __fsub_rn(x[2], __fmul_rn((float)(bx.b[2] + kl), vdx));
      D0 = __fmul_rn(d0, d0);
      D1 = __fmul_rn(d1, d1);
      D2 = __fmul_rn(d2, d2);
      base = ((bx.b[0] - B0) * T1 + (bx.b[1] - B1)) * T2 + (bx.b[2] + kl - B2);
    }
    const int o0 = __shfl_xor_sync(kFull, n0, 16), o1 = __shfl_xor_sync(kFull, n1, 16);
    const int m0 = max(n0, o0), m1 = max(n1, o1);
    const bool live = kl < n2;
    const int plane = T1 * T2;
    if (TILE && n0 == o0 && n1 == o1) {
      // both halves walk the same (i, j) extents (the common case): the i terms sit in
      // registers and the unrolled i loop issues an atomic per node with no branch
      float D0r[16];
#pragma unroll
      for (int ii = 0; ii < 16; ++ii) D0r[ii] = __shfl_sync(kFull, D0, h | ii);
      const int step = live ? plane : 0;
      for (int jj = 0; jj < m1; ++jj) {
        const float e = __fadd_rn(__shfl_sync(kFull, D1, h | jj), D2);  // d1^2 + d2^2
        unsigned* a = live ? dst + base + jj * T2 : dump + lane;
#pragma unroll
        for (int ii = 0; ii < 16; ++ii) {
          if (ii >= m0) break;
          atomicMin(a, __float_as_uint(__fadd_rn(D0r[ii], e)));
          a += step;
        }
      }
      continue;
    }
    for (int jj = 0; jj < m1; ++jj) {
      const float e = __fadd_rn(__shfl_sync(kFull, D1, h | jj), D2);  // d1^2 + d2^2
      int idx = base + jj * T2;
      const bool row = live && jj < n1;
      for (int ii = 0; ii < m0; ++ii) {
        const float d0sq = __shfl_sync(kFull, D0, h | ii);
        if (row && ii < n0) atomicMin(&dst[idx], __float_as_uint(__fadd_rn(d0sq, e)));
        idx += plane;
      }
    }
  }
}

// The same scatter for boxes of any size: one particle per warp, nodes lane-strided.
__device__ __forceinline__ void scatter_walk(unsigned* dst, int B0, int B1, int B2, int T1, int T2,
                                             const float (*px)[3], int p0, int pc, float vdx, float rg, int G,
                                             int warp, int lane) {
  for (int q = warp; q < pc; q += kSurfThreads / 32) {
    const float x[3] = {px[p0 + q][0], px[p0 + q][1], px[p0 + q][2]};
    walk_box(node_box(x, vdx, rg, G), lane, [&](int i, int j, int k) {
      atomicMin(&dst[((i - B0) * T1 + (j - B1)) * T2 + (k - B2)], sq_dist_bits(x, i, j, k, vdx));
    });
  }
}

struct DistPass {
  int p0, pc;      // particles of the chunk
  int B[3], T[3];  // node box of their union
  int tiled;       // 1: through the shared tile, 0: straight to the field
};

// A CTA takes chunks of 128 consecutive particles.  The union of their node boxes is
// scattered through a shared tile when it fits; otherwise the chunk is split into halves
// and then 32-particle quarters, each through the tile when its own union fits and
// straight to the field when not.  half_boxes: every node box spans at most 16 nodes per
// axis.  The field indices fit in int (G <= 512).
__global__ void __launch_bounds__(kSurfThreads) distance_kernel(const float* __restrict__ s, int64_t st, int64_t n,
                                                                float vdx, float rg, int G, bool half_boxes,
                                                                unsigned* __restrict__ sq) {
  __shared__ unsigned tile[kDistTile];
  __shared__ float px[kDistChunk][3];
  __shared__ int red[kDistChunk / 32][6];
  __shared__ DistPass passes[kDistChunk / 32];
  __shared__ int npass;
  __shared__ unsigned dump[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t chunks = (n + kDistChunk - 1) / kDistChunk;
  for (int64_t ch = blockIdx.x; ch < chunks; ch += gridDim.x) {
    const int64_t base = ch * kDistChunk;
    const int cnt = (int)(n - base < kDistChunk ? n - base : kDistChunk);
    // the chunk's particles and the union of the node boxes of each 32 of them
    if (tid < kDistChunk) {
      int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {INT_MIN, INT_MIN, INT_MIN};
      if (tid < cnt) {
        float x[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) x[c] = px[tid][c] = s[(int64_t)(kX + c) * st + base + tid];
        const NodeBox bx = node_box(x, vdx, rg, G);
        if (bx.e[0] > bx.b[0] && bx.e[1] > bx.b[1] && bx.e[2] > bx.b[2]) {
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            lo[c] = bx.b[c];
            hi[c] = bx.e[c];
          }
        }
      }
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int o = 16; o; o >>= 1) {
          lo[c] = min(lo[c], __shfl_xor_sync(kFull, lo[c], o));
          hi[c] = max(hi[c], __shfl_xor_sync(kFull, hi[c], o));
        }
      if (lane == 0)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          red[warp][c] = lo[c];
          red[warp][3 + c] = hi[c];
        }
    }
    __syncthreads();
    if (tid == 0) {
      int np = 0;
      // union of the groups [wa, wb) of 32 particles; returns false when it is empty
      auto group = [&](int wa, int wb, DistPass& ps) {
        int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {INT_MIN, INT_MIN, INT_MIN};
        for (int w = wa; w < wb; ++w)
          for (int c = 0; c < 3; ++c) {
            lo[c] = min(lo[c], red[w][c]);
            hi[c] = max(hi[c], red[w][3 + c]);
          }
        ps.p0 = 32 * wa;
        ps.pc = min(cnt, 32 * wb) - ps.p0;
        for (int c = 0; c < 3; ++c) {
          ps.B[c] = lo[c];
          ps.T[c] = hi[c] - lo[c];
        }
        ps.tiled = (int64_t)ps.T[0] * ps.T[1] * ps.T[2] <= kDistTile;
        return ps.pc > 0 && ps.T[0] > 0 && ps.T[1] > 0 && ps.T[2] > 0;
      };
      DistPass ps;
      if (group(0, 4, ps) && ps.tiled) {
        passes[np++] = ps;
      } else {
        for (int hb = 0; hb < 4; hb += 2) {
          if (!group(hb, hb + 2, ps)) continue;
          if (ps.tiled) {
            passes[np++] = ps;
            continue;
          }
          for (int w = hb; w < hb + 2; ++w)
            if (group(w, w + 1, ps)) passes[np++] = ps;
        }
      }
      npass = np;
    }
    __syncthreads();
    const int np = npass;
    for (int k = 0; k < np; ++k) {
      const DistPass ps = passes[k];
      if (ps.tiled) {
        const int V = ps.T[0] * ps.T[1] * ps.T[2];
        for (int q = tid; q < V; q += kSurfThreads) tile[q] = kInfBits;
        __syncthreads();
        if (half_boxes)
          scatter_half<true>(tile, ps.B[0], ps.B[1], ps.B[2], ps.T[1], ps.T[2], px, ps.p0, ps.pc, vdx, rg, G, warp,
                             lane, dump);
        else
          scatter_walk(tile, ps.B[0], ps.B[1], ps.B[2], ps.T[1], ps.T[2], px, ps.p0, ps.pc, vdx, rg, G, warp, lane);
        __syncthreads();
        // flush: one (i, j) row per warp, lanes along k (coalesced reductions)
        const int rows = ps.T[0] * ps.T[1];
        for (int r = warp; r < rows; r += kSurfThreads / 32) {
          const int i = ps.B[0] + r / ps.T[1], j = ps.B[1] + r % ps.T[1];
          unsigned* out = sq + ((int64_t)i * G + j) * G + ps.B[2];
          for (int kk = lane; kk < ps.T[2]; kk += 32) {
            const unsigned v = tile[r * ps.T[2] + kk];
            if (v != kInfBits) atomicMin(out + kk, v);
          }
        }
        __syncthreads();  // the tile is reused by the next pass
      } else if (half_boxes) {
        scatter_half<false>(sq, 0, 0, 0, G, G, px, ps.p0, ps.pc, vdx, rg, G, warp, lane, dump);
      } else {
        scatter_walk(sq, 0, 0, 0, G, G, px, ps.p0, ps.pc, vdx, rg, G, warp, lane);
      }
    }
    __syncthreads();  // px, red and passes are reused by the next chunk
  }
}

// field = min(cutoff, sqrt(s_min)) in place (+inf where no particle reached: the cutoff).
__global__ void finish_distance_kernel(unsigned* field, int64_t cells, float cutoff) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < cells; c += (int64_t)gridDim.x * blockDim.x)
    field[c] = __float_as_uint(fminf(cutoff, __fsqrt_rn(__uint_as_float(field[c]))));
}

// Bit q of the mask: corner q of cell (i, j, k) is inside, i.e. its value is below thr
// (the field against the float threshold of S > 0, or the raw squared distance against
// the squared threshold).
__device__ __forceinline__ unsigned corner_mask(const float* field, int G, int i, int j, int k, float thr) {
  const float* f = field + ((int64_t)i * G + j) * G + k;
  const int64_t sj = G, si = (int64_t)G * G;
  unsigned m = 0;
  m |= (unsigned)(f[0] < thr) << 0;
  m |= (unsigned)(f[1] < thr) << 1;
  m |= (unsigned)(f[sj] < thr) << 2;
  m |= (unsigned)(f[sj + 1] < thr) << 3;
  m |= (unsigned)(f[si] < thr) << 4;
  m |= (unsigned)(f[si + 1] < thr) << 5;
  m |= (unsigned)(f[si + sj] < thr) << 6;
  m |= (unsigned)(f[si + sj + 1] < thr) << 7;
  return m;
}

// Triangles of a cell from its corner mask: per tetrahedron 1 when 1 or 3 corners are
// inside, 2 when 2 are.
__device__ __forceinline__ int mask_triangles(unsigned m) {
  int cnt = 0;
#pragma unroll
  for (int t = 0; t < 6; ++t) {
    const unsigned tm = (1u << tet_corner(t, 0)) | (1u << tet_corner(t, 1)) | (1u << tet_corner(t, 2)) |
                        (1u << tet_corner(t, 3));
    const int k = __popc(m & tm);
    cnt += (k == 2) ? 2 : (k == 1 || k == 3) ? 1 : 0;
  }
  return cnt;
}

// Cells are visited one (i, j) row at a time, `ksegs` blocks of kSurfThreads cells per
// row, so block order is cell order; false for the padding threads past the row's end.
__device__ __forceinline__ bool block_cell(int G, int ksegs, int& i, int& j, int& k) {
  const int Gm = G - 1;
  const int row = (int)(blockIdx.x / (unsigned)ksegs), seg = (int)blockIdx.x - row * ksegs;
  i = row / Gm;
  j = row - i * Gm;
  k = seg * kSurfThreads + (int)threadIdx.x;
  return k < Gm;
}

__global__ void __launch_bounds__(kSurfThreads) mc_count_kernel(const float* __restrict__ field, int G, int ksegs,
                                                                float thr, int* __restrict__ block_counts) {
  __shared__ int warp_sum[kSurfThreads / 32];
  int i, j, k, cnt = 0;
  if (block_cell(G, ksegs, i, j, k)) {
    const unsigned m = corner_mask(field, G, i, j, k, thr);
    if (m != 0 && m != 0xffu) cnt = mask_triangles(m);
  }
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

// RAW: the buffer holds the squared distances, the field value of a corner is
// min(cutoff, sqrt(s)) (what finish_distance_kernel stores).
template <bool RAW>
__global__ void __launch_bounds__(kSurfThreads) mc_write_kernel(const float* __restrict__ field, int G, int ksegs,
                                                                float thr, float cutoff, float iso, float vdx,
                                                                const int* __restrict__ block_offsets,
                                                                float* __restrict__ tris) {
  __shared__ int warp_sum[kSurfThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int i, j, k, cnt = 0;
  unsigned m = 0;
  if (block_cell(G, ksegs, i, j, k)) {
    m = corner_mask(field, G, i, j, k, thr);
    if (m != 0 && m != 0xffu) cnt = mask_triangles(m);
  }
  int inc = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_sum[warp] = inc;
  __syncthreads();
  if (cnt == 0) return;
  int wpre = 0;
  for (int w = 0; w < warp; ++w) wpre += warp_sum[w];
  float* out = tris + 9 * ((int64_t)block_offsets[blockIdx.x] + wpre + inc - cnt);
  float f[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const float v = field[((int64_t)(i + (q >> 2)) * G + j + ((q >> 1) & 1)) * G + k + (q & 1)];
    f[q] = RAW ? fminf(cutoff, __fsqrt_rn(v)) : v;
  }
#pragma unroll 1
  for (int t = 0; t < 6; ++t) out += 9 * tet_triangles(f, m, t, i, j, k, iso, vdx, out);
}

// The float threshold thr with  field < thr  <=>  iso - (double)field > 0.
float inside_threshold(double iso) {
  const float f = (float)iso;
  return (double)f < iso ? std::nextafter(f, INFINITY) : f;
}

// The least float s >= 0 with sqrt(s) >= thr (sqrt correctly rounded on host and device),
// so that  sqrt(s) < thr  <=>  s < sq_threshold(thr).
float sq_threshold(float thr) {
  if (!(thr > 0.f)) return 0.f;
  float s0 = thr * thr;
  while (s0 > 0.f && std::sqrt(std::nextafter(s0, 0.f)) >= thr) s0 = std::nextafter(s0, 0.f);
  while (std::sqrt(s0) < thr) s0 = std::nextafter(s0, INFINITY);
  return s0;
}

struct SurfaceConsts {
  float vdx, cutoff, thr;
  double iso;
};

// The reference's float dx and cutoff (fillVoxelGrid_distance takes them as float,
// include/mesh_builder.h:89) and the level S = radius voxel_dx - distance
// (include/mesh_builder.h:188).
SurfaceConsts surface_consts(int radius, double voxel_dx) {
  SurfaceConsts k;
  k.vdx = (float)voxel_dx;
  k.cutoff = (float)((double)(radius + 1) * voxel_dx);
  k.iso = (double)radius * voxel_dx;
  k.thr = inside_threshold(k.iso);
  return k;
}

template <class T>
cudaError_t reserve(T** p, int64_t* cap, int64_t need) {
  if (*cap >= need && *p) return cudaSuccess;
  cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  cudaError_t e = cudaMalloc(p, sizeof(T) * (size_t)need);
  if (e == cudaSuccess) *cap = need;
  return e;
}

}  // namespace

void SurfaceBuffers::release() {
  cudaFree(field);
  cudaFree(counts);
  cudaFree(scan);
  cudaFree(tris);
  cudaFreeHost(total);
  *this = SurfaceBuffers{};
}

cudaError_t launch_distance_field(const float* s, int64_t stride, int64_t n, int G, int radius, double voxel_dx,
                                  bool finish, SurfaceBuffers& buf, cudaStream_t st, int64_t* launches) {
  const int64_t cells = (int64_t)G * G * G;
  cudaError_t e = reserve(&buf.field, &buf.field_cap, cells);
  if (e != cudaSuccess) return e;
  const SurfaceConsts K = surface_consts(radius, voxel_dx);
  // raw squared distances classify like the field only while the cutoff is not inside
  buf.raw = !finish && K.cutoff >= K.thr;
  unsigned* sq = reinterpret_cast<unsigned*>(buf.field);
  const int fill_blocks = (int)std::min<int64_t>((cells + 255) / 256, 4096);
  fill_bits_kernel<<<fill_blocks, 256, 0, st>>>(sq, cells, kInfBits);
  if (n > 0) {
    const float rg = K.cutoff / K.vdx;
    const int64_t chunks = (n + kDistChunk - 1) / kDistChunk;
    // a box spans int(g + rg + 1) - int(g - rg) <= floor(2 rg + 1 + err) + 1 nodes per
    // axis, err (float rounding of the two ends) well below one node: at most 16 when
    // 2 rg + 3 <= 16
    const bool half_boxes = 2.0 * (double)rg + 3.0 <= 16.0;
    distance_kernel<<<(int)std::min<int64_t>(chunks, 152 * 32), kSurfThreads, 0, st>>>(s, stride, n, K.vdx, rg, G,
                                                                                      half_boxes, sq);
  }
  if (!buf.raw) finish_distance_kernel<<<fill_blocks, 256, 0, st>>>(sq, cells, K.cutoff);
  if (launches) *launches += 1 + (n > 0) + !buf.raw;
  return cudaGetLastError();
}

cudaError_t extract_surface(int G, int radius, double voxel_dx, SurfaceBuffers& buf, cudaStream_t st,
                            int64_t* n_out, int64_t* launches) {
  *n_out = 0;
  if (G < 2) return cudaSuccess;
  const SurfaceConsts K = surface_consts(radius, voxel_dx);
  const float thr = buf.raw ? sq_threshold(K.thr) : K.thr;
  const int Gm = G - 1;
  const int ksegs = (Gm + kSurfThreads - 1) / kSurfThreads;
  const int64_t nblocks = (int64_t)Gm * Gm * ksegs;
  cudaError_t e = reserve(&buf.counts, &buf.counts_cap, nblocks + 1);
  if (e == cudaSuccess) e = reserve(&buf.scan, &buf.scan_cap, scan_scratch_ints(nblocks + 1));
  if (e == cudaSuccess && !buf.total) e = cudaMallocHost(&buf.total, sizeof(int));
  if (e != cudaSuccess) return e;
  mc_count_kernel<<<(unsigned)nblocks, kSurfThreads, 0, st>>>(buf.field, G, ksegs, thr, buf.counts);
  e = cudaMemsetAsync(buf.counts + nblocks, 0, sizeof(int), st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = launch_exclusive_scan(buf.counts, nblocks + 1, buf.scan, st, launches);
  if (e == cudaSuccess) e = cudaMemcpyAsync(buf.total, buf.counts + nblocks, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  if (launches) *launches += 1;
  const int64_t total = *buf.total;
  if (total > 0) {
    e = reserve(&buf.tris, &buf.tris_cap, 9 * total);
    if (e != cudaSuccess) return e;
    const float iso = (float)K.iso;
    if (buf.raw)
      mc_write_kernel<true><<<(unsigned)nblocks, kSurfThreads, 0, st>>>(buf.field, G, ksegs, thr, K.cutoff, iso, K.vdx,
                                                                        buf.counts, buf.tris);
    else
      mc_write_kernel<false><<<(unsigned)nblocks, kSurfThreads, 0, st>>>(buf.field, G, ksegs, thr, K.cutoff, iso,
                                                                         K.vdx, buf.counts, buf.tris);
    e = cudaGetLastError();
    if (launches) *launches += 1;
  }
  *n_out = total;
  return e;
}

}  // namespace mpm
