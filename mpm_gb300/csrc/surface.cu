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
//     rate is a small fraction of its FP32 rate).  One sweep over the cells counts triangles
//     and surface cells per block and lists each block's surface cells in its slots;
//     exclusive scans over the blocks give their offsets; a dense emit pass (one thread per
//     surface cell, which finds its block by binary search) writes the triangles in cell
//     order, so the mesh is deterministic.
#include <algorithm>
#include <climits>
#include <cmath>
#include <utility>

#include "mpm_internal.h"
#include "surface.h"

namespace mpm {

namespace {

constexpr int kSurfThreads = 256;
constexpr int kDistThreads = 512;  // distance scatter: 16 warps share a chunk's tile
constexpr int kDistChunk = 128;     // particles per CTA and chunk
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

// Direct scatter of the squared distances of particles [p0, p0 + pc) of the chunk
// (positions in px) into the global field.  Two particles per warp, one per half; lane kl
// of a half takes node column k = b2 + kl and holds the particle's squared axis terms for
// i = b0 + kl and j = b1 + kl, which the (i, j) loop broadcasts by shuffle.  Needs every
// box to span at most 16 nodes per axis.
__device__ __forceinline__ void scatter_half_global(unsigned* sq, const float (*px)[3], int p0, int pc, float vdx,
                                                    float rg, int G, int warp, int lane) {
  const int h = lane & 16, kl = lane & 15;
  for (int q0 = 2 * warp; q0 < pc; q0 += 2 * (kDistThreads / 32)) {
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
      base = (bx.b[0] * G + bx.b[1]) * G + bx.b[2] + kl;
    }
    const int m0 = max(n0, __shfl_xor_sync(kFull, n0, 16)), m1 = max(n1, __shfl_xor_sync(kFull, n1, 16));
    const bool live = kl < n2;
    for (int jj = 0; jj < m1; ++jj) {
      const float e = __fadd_rn(__shfl_sync(kFull, D1, h | jj), D2);  // d1^2 + d2^2
      int idx = base + jj * G;
      const bool row = live && jj < n1;
      for (int ii = 0; ii < m0; ++ii) {
        const float d0sq = __shfl_sync(kFull, D0, h | ii);
        if (row && ii < n0) atomicMin(&sq[idx], __float_as_uint(__fadd_rn(d0sq, e)));
        idx += G * G;
      }
    }
  }
}

// Scatter of one particle's box into dst, node (i, j, k) at (i - B0) plane + (j - B1) row
// + (k - B2), boxes of any size: nodes lane-strided over the warp.
__device__ __forceinline__ void scatter_walk_one(unsigned* dst, int B0, int B1, int B2, int plane, int row,
                                                 const float x[3], const NodeBox& bx, float vdx, int lane) {
  walk_box(bx, lane, [&](int i, int j, int k) {
    atomicMin(&dst[(i - B0) * plane + (j - B1) * row + (k - B2)], sq_dist_bits(x, i, j, k, vdx));
  });
}

// The shared tile of a pass: up to kTileI x kTileJ x kTileK nodes, rows of kTileK words,
// planes of kTilePlane words.  kTilePlane = 16 (mod 32), so the two half-warps of the
// fixed-box scatter, one plane apart, use disjoint banks.  The fixed-box scatter's idle
// lanes reach up to one plane and 16 words past the pass's nodes (with +inf, a no-op), so
// the allocation has one plane and a row more.
constexpr int kTileI = 24, kTileJ = 32, kTileK = 32;
constexpr int kTilePlane = kTileJ * kTileK + 16;
constexpr int kTileWords = (kTileI + 1) * kTilePlane + kTileK;
constexpr size_t kTileBytes = sizeof(unsigned) * kTileWords;

// red.shared.min.u32 at byte offset OFF from a shared address.
template <int OFF>
__device__ __forceinline__ void red_min_shared(uint32_t addr, unsigned v) {
  asm volatile("red.shared.min.u32 [%0+%2], %1;" ::"r"(addr), "r"(v), "n"(OFF) : "memory");
}

template <int NB, int NM, int I>
__device__ __forceinline__ void fixed_node(uint32_t addr, const float (&Di)[NM], const float (&E)[NB]) {
  constexpr int m = I / NB, jj = I % NB;
  red_min_shared<4 * (2 * m * kTilePlane + jj * kTileK)>(addr, __float_as_uint(__fadd_rn(Di[m], E[jj])));
}

template <int NB, int NM, int... I>
__device__ __forceinline__ void fixed_nodes(uint32_t addr, const float (&Di)[NM], const float (&E)[NB],
                                            std::integer_sequence<int, I...>) {
  (fixed_node<NB, NM, I>(addr, Di, E), ...);
}

// Fixed-box scatter of one particle whose box spans NB x NB nodes in (i, j) and at most 16
// in k into the tile.  The warp's halves take the even and odd i planes, lane kl of a half
// node column k = b2 + kl; the squared axis terms sit in registers (+inf for a lane past
// the box's k extent and for the odd half's plane past an odd box), so every node is one
// add and one reduction at the lane's base address plus a compile-time offset, with no
// predicate.  s = d0^2 + (d1^2 + d2^2), the reference's order.
template <int NB>
__device__ __forceinline__ void scatter_fixed(uint32_t tile_addr, int B0, int B1, int B2, const float x[3],
                                              const int b[3], int n2, float vdx, int lane) {
  constexpr int NM = (NB + 1) / 2;
  const int h = lane >> 4, kl = lane & 15;
  const float d0 = __fsub_rn(x[0], __fmul_rn((float)(b[0] + kl), vdx));
  const float d1 = __fsub_rn(x[1], __fmul_rn((float)(b[1] + kl), vdx));
  const float d2 = __fsub_rn(x[2], __fmul_rn((float)(b[2] + kl), vdx));
  const float D0 = __fmul_rn(d0, d0), D1 = __fmul_rn(d1, d1);
  const float D2 = kl < n2 ? __fmul_rn(d2, d2) : __uint_as_float(kInfBits);
  float E[NB], Di[NM];
#pragma unroll
  for (int jj = 0; jj < NB; ++jj) E[jj] = __fadd_rn(__shfl_sync(kFull, D1, jj), D2);  // d1^2 + d2^2
#pragma unroll
  for (int m = 0; m < NM; ++m) {
    const float v = __shfl_sync(kFull, D0, min(2 * m + h, 15));
    Di[m] = (2 * m + h < NB) ? v : __uint_as_float(kInfBits);
  }
  const uint32_t addr = tile_addr + 4u * (uint32_t)((b[0] - B0 + h) * kTilePlane + (b[1] - B1) * kTileK + (b[2] - B2 + kl));
  fixed_nodes<NB, NM>(addr, Di, E, std::make_integer_sequence<int, NM * NB>{});
}

struct DistPass {
  int p0, pc;      // particles of the chunk
  int B[3], T[3];  // node box of their union
  int tiled;       // 1: through the shared tile, 0: straight to the field
};

// A CTA takes chunks of 128 consecutive particles.  The union of their node boxes is
// scattered through the shared tile (dynamic shared memory, kTileBytes) when it fits;
// otherwise the chunk is split into halves and then 32-particle quarters, each through
// the tile when its own union fits and straight to the field when not.  NB > 0: the
// (i, j) extent of an interior particle's box, scattered by the fixed-box path; other
// boxes take the generic walk.  half_boxes: every box spans at most 16 nodes per axis.
// The field indices fit in int (G <= 512).
template <int NB>
__global__ void __launch_bounds__(kDistThreads, 2) distance_kernel(const float* __restrict__ s, int64_t st, int64_t n,
                                                                   float vdx, float rg, int G, bool half_boxes,
                                                                   unsigned* __restrict__ sq) {
  extern __shared__ __align__(16) unsigned tile[];
  __shared__ float px[kDistChunk][3];
  __shared__ int pbox[kDistChunk][4];  // b0, b1, b2 and the extents packed 8 bits each (0: empty)
  __shared__ int red[kDistChunk / 32][6];
  __shared__ DistPass passes[kDistChunk / 32];
  __shared__ int npass;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t chunks = (n + kDistChunk - 1) / kDistChunk;
  // the whole tile starts at +inf; each pass's flush puts back +inf where it read, and a
  // pass changes no word outside the nodes it flushes, so the tile is all +inf again
  // before every pass
  for (int q = tid; q < kTileWords; q += kDistThreads) tile[q] = kInfBits;
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
        const bool any = bx.e[0] > bx.b[0] && bx.e[1] > bx.b[1] && bx.e[2] > bx.b[2];
        if (any) {
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            lo[c] = bx.b[c];
            hi[c] = bx.e[c];
          }
        }
        pbox[tid][0] = bx.b[0];
        pbox[tid][1] = bx.b[1];
        pbox[tid][2] = bx.b[2];
        pbox[tid][3] = any ? (bx.e[0] - bx.b[0]) | (bx.e[1] - bx.b[1]) << 8 | (bx.e[2] - bx.b[2]) << 16 : 0;
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
        ps.tiled = ps.T[0] <= kTileI && ps.T[1] <= kTileJ && ps.T[2] <= kTileK;
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
        const uint32_t tile_addr = (uint32_t)__cvta_generic_to_shared(tile);
        for (int q = warp; q < ps.pc; q += kDistThreads / 32) {
          const int p = ps.p0 + q;
          const int ext = pbox[p][3];
          if (ext == 0) continue;
          const float x[3] = {px[p][0], px[p][1], px[p][2]};
          const int b[3] = {pbox[p][0], pbox[p][1], pbox[p][2]};
          const int n0 = ext & 255, n1 = (ext >> 8) & 255, n2 = ext >> 16;
          if (NB > 0 && n0 == NB && n1 == NB && n2 <= 16) {
            scatter_fixed<(NB > 0 ? NB : 1)>(tile_addr, ps.B[0], ps.B[1], ps.B[2], x, b, n2, vdx, lane);
          } else {
            NodeBox bx;
            for (int c = 0; c < 3; ++c) bx.b[c] = b[c];
            bx.e[0] = b[0] + n0;
            bx.e[1] = b[1] + n1;
            bx.e[2] = b[2] + n2;
            scatter_walk_one(tile, ps.B[0], ps.B[1], ps.B[2], kTilePlane, kTileK, x, bx, vdx, lane);
          }
        }
        __syncthreads();
        // flush: one (i, j) row per warp, lanes along k (coalesced reductions), resetting
        // the tile to +inf
        int i = warp / ps.T[1], j = warp - i * ps.T[1];
        for (; i < ps.T[0];) {
          if (lane < ps.T[2]) {
            unsigned* w = tile + i * kTilePlane + j * kTileK + lane;
            const unsigned v = *w;
            if (v != kInfBits) {
              *w = kInfBits;
              atomicMin(sq + ((int64_t)(ps.B[0] + i) * G + ps.B[1] + j) * G + ps.B[2] + lane, v);
            }
          }
          j += kDistThreads / 32;
          while (j >= ps.T[1]) {
            j -= ps.T[1];
            ++i;
          }
        }
        __syncthreads();  // the tile is reused by the next pass
      } else if (half_boxes) {
        scatter_half_global(sq, px, ps.p0, ps.pc, vdx, rg, G, warp, lane);
      } else {
        for (int q = warp; q < ps.pc; q += kDistThreads / 32) {
          const float x[3] = {px[ps.p0 + q][0], px[ps.p0 + q][1], px[ps.p0 + q][2]};
          scatter_walk_one(sq, 0, 0, 0, G * G, G, x, node_box(x, vdx, rg, G), vdx, lane);
        }
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
// the squared threshold).  Indices fit in int (G <= 512).
__device__ __forceinline__ unsigned corner_mask(const float* field, int G, int i, int j, int k, float thr) {
  const float* f = field + (i * G + j) * G + k;
  const int sj = G, si = G * G;
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
  if (m == 0 || m == 0xffu) return 0;
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

// Cells are swept one (i, j) row at a time: grid (row segments of kSurfThreads cells, j, i),
// so the linear block index runs in cell order.  False for the padding past a row's end.
__device__ __forceinline__ bool block_cell(int G, int& i, int& j, int& k) {
  i = (int)blockIdx.z;
  j = (int)blockIdx.y;
  k = (int)blockIdx.x * kSurfThreads + (int)threadIdx.x;
  return k < G - 1;
}

__device__ __forceinline__ int64_t block_linear() {
  return ((int64_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
}

// The one sweep over the cells: per block, its triangle and surface-cell counts, and in the
// block's slots (kSurfThreads of them) its surface cells in cell order, each with its first
// triangle's offset inside the block.
__global__ void __launch_bounds__(kSurfThreads) mc_count_kernel(const float* __restrict__ field, int G, float thr,
                                                                int* __restrict__ block_tris,
                                                                int* __restrict__ block_cells,
                                                                int2* __restrict__ slots) {
  __shared__ int warp_tris[kSurfThreads / 32], warp_cells[kSurfThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int i, j, k, cnt = 0;
  if (block_cell(G, i, j, k)) cnt = mask_triangles(corner_mask(field, G, i, j, k, thr));
  const unsigned surf = __ballot_sync(kFull, cnt > 0);
  int inc = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) {
    warp_tris[warp] = inc;
    warp_cells[warp] = __popc(surf);
  }
  __syncthreads();
  const int64_t b = block_linear();
  if (threadIdx.x == 0) {
    int t = 0, c = 0;
    for (int w = 0; w < kSurfThreads / 32; ++w) {
      t += warp_tris[w];
      c += warp_cells[w];
    }
    block_tris[b] = t;
    block_cells[b] = c;
  }
  if (cnt == 0) return;
  int tpre = 0, cpre = 0;
  for (int w = 0; w < warp; ++w) {
    tpre += warp_tris[w];
    cpre += warp_cells[w];
  }
  const int rank = cpre + __popc(surf & ((1u << lane) - 1u));
  slots[b * kSurfThreads + rank] = make_int2((i << 20) | (j << 10) | k, tpre + inc - cnt);
}

// Triangles of the surface cells, one thread per cell.  RAW: the buffer holds the squared
// distances and a corner's field value is min(cutoff, sqrt(s)) (what
// finish_distance_kernel stores).
// Surface cell c (in cell order) is found in the slots of the block b whose exclusive scan
// of surface cells, cell_off[b], is the last one <= c; tri_off[b] is the block's first
// triangle.
template <bool RAW>
__global__ void __launch_bounds__(kSurfThreads) mc_emit_kernel(const float* __restrict__ field, int G, float thr,
                                                               float cutoff, float iso, float vdx,
                                                               const int* __restrict__ tri_off,
                                                               const int* __restrict__ cell_off, int64_t nblocks,
                                                               const int2* __restrict__ slots, int ncells,
                                                               float* __restrict__ tris) {
  const int c = blockIdx.x * kSurfThreads + threadIdx.x;
  if (c >= ncells) return;
  int64_t lo = 0, hi = nblocks - 1;  // cell_off[0] = 0 <= c < cell_off[nblocks] = ncells
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (cell_off[mid] <= c) lo = mid; else hi = mid - 1;
  }
  int2 e = slots[lo * kSurfThreads + (c - cell_off[lo])];
  e.y += tri_off[lo];
  const int i = e.x >> 20, j = (e.x >> 10) & 1023, k = e.x & 1023;
  float f[8];
  unsigned m = 0;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const float v = field[((i + (q >> 2)) * G + j + ((q >> 1) & 1)) * G + k + (q & 1)];
    m |= (unsigned)(v < thr) << q;
    f[q] = RAW ? fminf(cutoff, __fsqrt_rn(v)) : v;
  }
  float* out = tris + 9 * (int64_t)e.y;
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

template <int NB>
cudaError_t launch_distance_nb(int blocks, cudaStream_t st, const float* s, int64_t stride, int64_t n, float vdx,
                               float rg, int G, bool half_boxes, unsigned* sq) {
  // per function and device; cheap enough to set on every launch
  cudaError_t e =
      cudaFuncSetAttribute(distance_kernel<NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTileBytes);
  if (e != cudaSuccess) return e;
  distance_kernel<NB><<<blocks, kDistThreads, kTileBytes, st>>>(s, stride, n, vdx, rg, G, half_boxes, sq);
  return cudaGetLastError();
}

cudaError_t launch_distance(int nb, int blocks, cudaStream_t st, const float* s, int64_t stride, int64_t n, float vdx,
                            float rg, int G, bool half_boxes, unsigned* sq) {
  switch (nb) {
    case 3: return launch_distance_nb<3>(blocks, st, s, stride, n, vdx, rg, G, half_boxes, sq);
    case 5: return launch_distance_nb<5>(blocks, st, s, stride, n, vdx, rg, G, half_boxes, sq);
    case 7: return launch_distance_nb<7>(blocks, st, s, stride, n, vdx, rg, G, half_boxes, sq);
    case 9: return launch_distance_nb<9>(blocks, st, s, stride, n, vdx, rg, G, half_boxes, sq);
    case 11: return launch_distance_nb<11>(blocks, st, s, stride, n, vdx, rg, G, half_boxes, sq);
    case 13: return launch_distance_nb<13>(blocks, st, s, stride, n, vdx, rg, G, half_boxes, sq);
    case 15: return launch_distance_nb<15>(blocks, st, s, stride, n, vdx, rg, G, half_boxes, sq);
    default: return launch_distance_nb<0>(blocks, st, s, stride, n, vdx, rg, G, half_boxes, sq);
  }
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
  cudaFree(cells);
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
    // an interior box spans exactly 2 rg + 1 nodes when rg is a whole number
    const int nb = (rg == std::floor(rg) && 2.0 * (double)rg + 1.0 <= 15.0) ? 2 * (int)rg + 1 : 0;
    const int blocks = (int)std::min<int64_t>(chunks, 152 * 2 * 4);
    e = launch_distance(nb, blocks, st, s, stride, n, K.vdx, rg, G, half_boxes, sq);
    if (e != cudaSuccess) return e;
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
  const dim3 grid((unsigned)((Gm + kSurfThreads - 1) / kSurfThreads), (unsigned)Gm, (unsigned)Gm);
  const int64_t nblocks = (int64_t)grid.x * grid.y * grid.z;
  // counts: per-block triangles (nblocks + 1), then per-block surface cells (nblocks + 1)
  cudaError_t e = reserve(&buf.counts, &buf.counts_cap, 2 * (nblocks + 1));
  if (e == cudaSuccess) e = reserve(&buf.scan, &buf.scan_cap, scan_scratch_ints(nblocks + 1));
  if (e == cudaSuccess && !buf.total) e = cudaMallocHost(&buf.total, 2 * sizeof(int));
  if (e != cudaSuccess) return e;
  int* block_tris = buf.counts;
  int* block_cells = buf.counts + nblocks + 1;
  e = reserve(&buf.cells, &buf.cells_cap, nblocks * kSurfThreads);
  if (e != cudaSuccess) return e;
  mc_count_kernel<<<grid, kSurfThreads, 0, st>>>(buf.field, G, thr, block_tris, block_cells, buf.cells);
  e = cudaMemsetAsync(block_tris + nblocks, 0, sizeof(int), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(block_cells + nblocks, 0, sizeof(int), st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = launch_exclusive_scan(block_tris, nblocks + 1, buf.scan, st, launches);
  if (e == cudaSuccess) e = launch_exclusive_scan(block_cells, nblocks + 1, buf.scan, st, launches);
  if (e == cudaSuccess) e = cudaMemcpyAsync(buf.total, block_tris + nblocks, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(buf.total + 1, block_cells + nblocks, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  if (launches) *launches += 1;
  const int64_t total = buf.total[0];
  const int ncells = buf.total[1];
  if (total > 0) {
    e = reserve(&buf.tris, &buf.tris_cap, 9 * total);
    if (e != cudaSuccess) return e;
    const float iso = (float)K.iso;
    const unsigned eblocks = (unsigned)((ncells + kSurfThreads - 1) / kSurfThreads);
    if (buf.raw)
      mc_emit_kernel<true><<<eblocks, kSurfThreads, 0, st>>>(buf.field, G, thr, K.cutoff, iso, K.vdx, block_tris,
                                                             block_cells, nblocks, buf.cells, ncells, buf.tris);
    else
      mc_emit_kernel<false><<<eblocks, kSurfThreads, 0, st>>>(buf.field, G, thr, K.cutoff, iso, K.vdx, block_tris,
                                                              block_cells, nblocks, buf.cells, ncells, buf.tris);
    e = cudaGetLastError();
    if (launches) *launches += 1;
  }
  *n_out = total;
  return e;
}

}  // namespace mpm
