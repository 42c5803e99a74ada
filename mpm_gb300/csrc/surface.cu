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
//   * the level set is extracted by marching cubes in libigl's layout (the reference's
//     vendored include/igl/copyleft/marching_cubes.cpp, fed by
//     include/mesh_builder.h:181-194): cubes in node order with k fastest, a corner inside
//     when S > 0 (one float compare against the equivalent float threshold), and a vertex
//     created on each crossed edge the first time a cube sees it, at
//     (1 - t) p0 + t p1, t = |S0| / (|S0| + |S1|), in double, then scaled by voxel_dx.
//     So the vertex list is the reference's bit for bit and in its order: an edge is
//     first seen by its lowest cube, and a cube's new vertices follow its edge slots.  The
//     triangle table is this project's own (surface.h): it triangulates the same loops of
//     crossed edges per cube as libigl's table, with a fan inside each loop.
//     One sweep over the cubes counts triangles, new vertices and surface cubes per block
//     of cubes and lists each block's surface cubes in its slots; one scan over the three
//     counts gives the blocks' offsets; a dense emit pass (one thread per surface cube,
//     which finds its block by binary search) writes the vertices it creates, its faces
//     (a vertex created by an earlier cube is found through that cube's slot, again by
//     binary search) and, when asked, the triangle soup, so the mesh is deterministic.
#include <algorithm>
#include <climits>
#include <cmath>
#include <utility>

#include "mpm_internal.h"
#include "surface.h"

namespace mpm {

namespace {

constexpr int kSurfThreads = 128;
constexpr int kRowCubes = 2 * kSurfThreads;  // cubes per block of the count sweep: two per thread
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

// The triangle table in global memory: threads of a warp read different entries, which
// the read-only cache serves without the serialisation of divergent constant loads.
__device__ const mc::Table kMc = mc::make_table();

constexpr int kEmitThreads = 128;

// Compile-time facts of edge slot E: its corners, axis and lower-corner offsets.
template <int E>
struct Edge {
  static constexpr int a = mc::kEdge[E][0], b = mc::kEdge[E][1];
  static constexpr int o0 = mc::kCorner[a][0], o1 = mc::kCorner[a][1], o2 = mc::kCorner[a][2];
  static constexpr int ax = mc::kCorner[a][0] != mc::kCorner[b][0] ? 0 : mc::kCorner[a][1] != mc::kCorner[b][1] ? 1 : 2;
  // owned by a cube whose coordinate is 0 on each perpendicular axis where the edge
  // lies on the cube's lower side (bit p of `need_zero`)
  static constexpr int need_zero = (ax != 0 && o0 == 0 ? 1 : 0) | (ax != 1 && o1 == 0 ? 2 : 0) | (ax != 2 && o2 == 0 ? 4 : 0);
  static constexpr int slot_at(int s0, int s1, int s2) { return mc::slot_along(ax, o0 | s0, o1 | s1, o2 | s2); }
  // the owner's slot for the shifts (s0, s1, s2), 4 bits per combination s0 * 4 + s1 * 2 + s2
  static constexpr uint32_t owner_slots =
      (uint32_t)slot_at(0, 0, 0) | (uint32_t)slot_at(0, 0, 1) << 4 | (uint32_t)slot_at(0, 1, 0) << 8 |
      (uint32_t)slot_at(0, 1, 1) << 12 | (uint32_t)slot_at(1, 0, 0) << 16 | (uint32_t)slot_at(1, 0, 1) << 20 |
      (uint32_t)slot_at(1, 1, 0) << 24 | (uint32_t)slot_at(1, 1, 1) << 28;
};

// The edge slots whose vertex cube (i, j, k) creates: libigl visits the cubes in order and
// creates a vertex the first time an edge is seen, i.e. in the edge's lowest cube, which
// lowers each coordinate across the edge by one where it can.
template <int... E>
__device__ __forceinline__ unsigned owned_mask_impl(int zero, std::integer_sequence<int, E...>) {
  return ((((Edge<E>::need_zero & ~zero) == 0) ? 1u << E : 0u) | ...);
}
__device__ __forceinline__ unsigned owned_mask(int i, int j, int k) {
  const int zero = (i == 0 ? 1 : 0) | (j == 0 ? 2 : 0) | (k == 0 ? 4 : 0);
  return owned_mask_impl(zero, std::make_integer_sequence<int, 12>{});
}

// Cubes are swept one (i, j) row at a time: grid (row segments of kRowCubes cubes, j, i), so
// the linear block index runs in cube order (for G <= 513 a block holds a whole row).
__device__ __forceinline__ int64_t block_linear() {
  return ((int64_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
}

__device__ __forceinline__ int warp_inclusive(int v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(kFull, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// libigl's corner mask of a cube from its corners' inside bits on the four node rows
// (i, j), (i, j + 1), (i + 1, j), (i + 1, j + 1), at the cube's k (lo) and k + 1 (hi).
__device__ __forceinline__ unsigned mask_of(bool a00lo, bool a00hi, bool a01lo, bool a01hi, bool a10lo, bool a10hi,
                                            bool a11lo, bool a11hi) {
  return (unsigned)a00lo | (unsigned)a00hi << 1 | (unsigned)a01hi << 2 | (unsigned)a01lo << 3 | (unsigned)a10lo << 4 |
         (unsigned)a10hi << 5 | (unsigned)a11hi << 6 | (unsigned)a11lo << 7;
}

// The one sweep over the cubes, two neighbouring cubes (k, k + 1) per thread, which share
// the four corners at k + 1.  counts holds three runs of nblocks + 1 ints (triangles, new
// vertices, surface cubes per block, each run ending in a zero); the block's slots
// (kRowCubes of them) list its surface cubes in cube order with their first triangle and
// first vertex inside the block and their inside-corner mask.
__global__ void __launch_bounds__(kSurfThreads) mc_count_kernel(const float* __restrict__ field, int G, float thr,
                                                                int* __restrict__ counts, int64_t nblocks,
                                                                int4* __restrict__ slots) {
  __shared__ int warp_tris[kSurfThreads / 32], warp_verts[kSurfThreads / 32], warp_cells[kSurfThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = (int)blockIdx.z, j = (int)blockIdx.y;
  const int k = 2 * ((int)blockIdx.x * kSurfThreads + (int)threadIdx.x);
  const bool v0 = k < G - 1, v1 = k + 1 < G - 1;
  unsigned m0 = 0, m1 = 0;
  if (v0) {
    const float* f = field + (i * G + j) * G + k;
    const int sj = G, si = G * G;
    // k + 2 <= G - 1 whenever the second cube exists
    const bool a00 = f[0] < thr, a00h = f[1] < thr, a01 = f[sj] < thr, a01h = f[sj + 1] < thr;
    const bool a10 = f[si] < thr, a10h = f[si + 1] < thr, a11 = f[si + sj] < thr, a11h = f[si + sj + 1] < thr;
    m0 = mask_of(a00, a00h, a01, a01h, a10, a10h, a11, a11h);
    if (v1) {
      const bool b00 = f[2] < thr, b01 = f[sj + 2] < thr, b10 = f[si + 2] < thr, b11 = f[si + sj + 2] < thr;
      m1 = mask_of(a00h, b00, a01h, b01, a10h, b10, a11h, b11);
    }
  }
  const bool s0 = m0 != 0u && m0 != 0xffu, s1 = m1 != 0u && m1 != 0xffu;
  // almost every cube lies wholly inside or outside: a warp without a surface cube skips
  // the table and the scans
  const bool any = __ballot_sync(kFull, s0 || s1) != 0u;
  int nt0 = 0, nt1 = 0, nv0 = 0, nv1 = 0;
  int tinc = 0, vinc = 0, cinc = 0;
  if (any) {
    if (s0) {
      nt0 = __ldg(&kMc.count[m0]);
      nv0 = __popc(__ldg(&kMc.crossed[m0]) & owned_mask(i, j, k));
    }
    if (s1) {
      nt1 = __ldg(&kMc.count[m1]);
      nv1 = __popc(__ldg(&kMc.crossed[m1]) & owned_mask(i, j, k + 1));
    }
    tinc = warp_inclusive(nt0 + nt1, lane);
    vinc = warp_inclusive(nv0 + nv1, lane);
    cinc = warp_inclusive((int)s0 + (int)s1, lane);
  }
  if (lane == 31) {
    warp_tris[warp] = tinc;
    warp_verts[warp] = vinc;
    warp_cells[warp] = cinc;
  }
  __syncthreads();
  const int64_t b = block_linear();
  if (threadIdx.x == 0) {
    int t = 0, v = 0, c = 0;
    for (int w = 0; w < kSurfThreads / 32; ++w) {
      t += warp_tris[w];
      v += warp_verts[w];
      c += warp_cells[w];
    }
    counts[b] = t;
    counts[(nblocks + 1) + b] = v;
    counts[2 * (nblocks + 1) + b] = c;
    if (b == 0) counts[nblocks] = counts[2 * nblocks + 1] = counts[3 * nblocks + 2] = 0;
  }
  if (!s0 && !s1) return;
  int tpre = 0, vpre = 0, cpre = 0;
  for (int w = 0; w < warp; ++w) {
    tpre += warp_tris[w];
    vpre += warp_verts[w];
    cpre += warp_cells[w];
  }
  int rank = cpre + cinc - (int)s0 - (int)s1;
  const int t0 = tpre + tinc - nt0 - nt1, vv0 = vpre + vinc - nv0 - nv1;
  int4* out = slots + b * kRowCubes;
  if (s0) out[rank++] = make_int4((i << 20) | (j << 10) | k, t0, vv0, (int)m0);
  if (s1) out[rank] = make_int4((i << 20) | (j << 10) | (k + 1), t0 + nt0, vv0 + nv0, (int)m1);
}

// The three totals of the scanned counts into pinned host memory.
__global__ void mc_totals_kernel(const int* __restrict__ scan, int64_t nblocks, int* total) {
  total[0] = scan[nblocks];
  total[1] = scan[2 * nblocks + 1] - scan[nblocks + 1];
  total[2] = scan[3 * nblocks + 2] - scan[2 * nblocks + 2];
}

struct EmitArgs {
  const float* field;
  int G, gx;  // grid side, blocks per row of cubes
  float thr, cutoff;
  double iso, vdx;
  const int* scan;  // scanned counts (three runs of nblocks + 1)
  int64_t nblocks;
  const int4* slots;
  int ncells;
  double* verts;
  int* faces;
  float* tris;
};

// The vertex libigl creates on edge slot E of cube (i, j, k) (add_vertex: the point
// (1 - t) p0 + t p1 with t = |S0| / (|S0| + |S1|), p0 the lower node, in double; then
// scaled by voxel_dx as MeshBuilder::computeMesh does).
template <int E>
__device__ __forceinline__ void edge_position(const double S[8], int i, int j, int k, double vdx, double p[3]) {
  using D = Edge<E>;
  const double s0 = fabs(S[D::a]), s1 = fabs(S[D::b]);
  const double t = __ddiv_rn(s0, __dadd_rn(s0, s1));
  const double u = __dsub_rn(1.0, t);
  const int c[3] = {i + D::o0, j + D::o1, k + D::o2};
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const double a = (double)c[q], b = (double)(c[q] + (q == D::ax ? 1 : 0));
    p[q] = __dmul_rn(__dadd_rn(__dmul_rn(u, a), __dmul_rn(t, b)), vdx);
  }
}

// Index of the vertex on edge slot E of cube (i, j, k) when an earlier cube creates it: the
// owner cube is found in its block's slots by binary search (they are in cube order), and
// the vertex is the owner's first plus the owner's created edges before the owner's slot.
template <int E>
__device__ __forceinline__ int owner_vertex(const EmitArgs& a, int i, int j, int k) {
  using D = Edge<E>;
  const int s0 = (D::need_zero & 1) && i > 0, s1 = (D::need_zero & 2) && j > 0, s2 = (D::need_zero & 4) && k > 0;
  const int ci = i - s0, cj = j - s1, ck = k - s2;
  const int e2 = (int)((D::owner_slots >> (4 * (s0 * 4 + s1 * 2 + s2))) & 15u);
  const int64_t b = ((int64_t)ci * (a.G - 1) + cj) * a.gx + ck / kRowCubes;
  const int* cell_off = a.scan + 2 * (a.nblocks + 1);
  const int cnt = cell_off[b + 1] - cell_off[b];
  const int key = (ci << 20) | (cj << 10) | ck;
  const int* keys = reinterpret_cast<const int*>(a.slots + b * kRowCubes);
  int lo = 0, hi = cnt - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (keys[4 * mid] < key) lo = mid + 1; else hi = mid;
  }
  const int4 o = a.slots[b * kRowCubes + lo];
  const int* vert_off = a.scan + (a.nblocks + 1);
  const unsigned mine = __ldg(&kMc.crossed[o.w & 255]) & owned_mask(ci, cj, ck) & ((1u << e2) - 1u);
  return vert_off[b] - vert_off[0] + o.z + __popc(mine);
}

template <bool SOUP>
struct EmitScratch {
  int id[12][kEmitThreads];
  float pos[SOUP ? 36 : 1][kEmitThreads];
};

template <bool SOUP, int E>
__device__ __forceinline__ void emit_edge(const EmitArgs& a, const double S[8], int i, int j, int k, unsigned crossed,
                                          unsigned owned, int vbase, EmitScratch<SOUP>& sh, int tid) {
  if (!((crossed >> E) & 1u)) return;
  const bool own = (owned >> E) & 1u;
  int id;
  if (own) id = vbase + __popc(crossed & owned & ((1u << E) - 1u));
  else id = owner_vertex<E>(a, i, j, k);
  sh.id[E][tid] = id;
  if (own || SOUP) {
    double p[3];
    edge_position<E>(S, i, j, k, a.vdx, p);
    if (own)
#pragma unroll
      for (int q = 0; q < 3; ++q) a.verts[3 * (int64_t)id + q] = p[q];
    if (SOUP)
#pragma unroll
      for (int q = 0; q < 3; ++q) sh.pos[(3 * E + q) % (SOUP ? 36 : 1)][tid] = (float)p[q];
  }
}

template <bool SOUP, int... E>
__device__ __forceinline__ void emit_edges(const EmitArgs& a, const double S[8], int i, int j, int k, unsigned crossed,
                                           unsigned owned, int vbase, EmitScratch<SOUP>& sh, int tid,
                                           std::integer_sequence<int, E...>) {
  (emit_edge<SOUP, E>(a, S, i, j, k, crossed, owned, vbase, sh, tid), ...);
}

// Vertices, faces (and the triangle soup) of the surface cubes, one thread per cube.
// RAW: the buffer holds the squared distances and a corner's field value is
// min(cutoff, sqrt(s)) (what finish_distance_kernel stores).  Surface cube c (in cube
// order) is found in the slots of the block b whose scanned surface-cube count is the
// last one <= c.
template <bool RAW, bool SOUP>
__global__ void __launch_bounds__(kEmitThreads) mc_emit_kernel(const EmitArgs a) {
  __shared__ EmitScratch<SOUP> sh;
  const int tid = threadIdx.x;
  const int c = blockIdx.x * kEmitThreads + tid;
  if (c >= a.ncells) return;
  const int* tri_off = a.scan;
  const int* vert_off = a.scan + (a.nblocks + 1);
  const int* cell_off = a.scan + 2 * (a.nblocks + 1);
  const int c0 = cell_off[0];
  int64_t lo = 0, hi = a.nblocks - 1;  // cell_off[0] - c0 = 0 <= c < ncells
  while (lo < hi) {
    const int64_t mid = (lo + hi + 1) >> 1;
    if (cell_off[mid] - c0 <= c) lo = mid; else hi = mid - 1;
  }
  const int4 e = a.slots[lo * kRowCubes + (c - (cell_off[lo] - c0))];
  const int i = e.x >> 20, j = (e.x >> 10) & 1023, k = e.x & 1023;
  const int tbase = tri_off[lo] + e.y;
  const int vbase = vert_off[lo] - vert_off[0] + e.z;
  const unsigned m = (unsigned)e.w;
  const int G = a.G;
  double S[8];
#pragma unroll
  for (int n = 0; n < 8; ++n) {
    const int di = n >> 2, dj = (n >> 1) & 1, dk = ((n >> 1) ^ n) & 1;  // libigl's corner n
    const float v = a.field[((i + di) * G + j + dj) * G + k + dk];
    const float f = RAW ? fminf(a.cutoff, __fsqrt_rn(v)) : v;
    S[n] = __dsub_rn(a.iso, (double)f);
  }
  const unsigned crossed = __ldg(&kMc.crossed[m]);
  emit_edges<SOUP>(a, S, i, j, k, crossed, owned_mask(i, j, k), vbase, sh, tid, std::make_integer_sequence<int, 12>{});
  const int nt = __ldg(&kMc.count[m]);
  for (int t = 0; t < nt; ++t) {
    const int64_t f = (int64_t)(tbase + t);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const int sl = __ldg(&kMc.slot[m][3 * t + r]);
      a.faces[3 * f + r] = sh.id[sl][tid];
      if (SOUP)
#pragma unroll
        for (int q = 0; q < 3; ++q) a.tris[9 * f + 3 * r + q] = sh.pos[(3 * sl + q) % (SOUP ? 36 : 1)][tid];
    }
  }
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

void surface_table(int32_t* counts, int32_t* slots) {
  constexpr mc::Table t = mc::make_table();
  for (int m = 0; m < 256; ++m) {
    counts[m] = t.count[m];
    for (int r = 0; r < 30; ++r) slots[30 * m + r] = t.slot[m][r];
  }
}

void SurfaceBuffers::release() {
  cudaFree(field);
  cudaFree(cells);
  cudaFree(counts);
  cudaFree(scan);
  cudaFree(verts);
  cudaFree(faces);
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

cudaError_t extract_surface(int G, int radius, double voxel_dx, SurfaceBuffers& buf, cudaStream_t st, bool soup,
                            int64_t* n_verts, int64_t* n_faces, int64_t* launches) {
  *n_verts = *n_faces = 0;
  if (G < 2) return cudaSuccess;
  const SurfaceConsts K = surface_consts(radius, voxel_dx);
  const float thr = buf.raw ? sq_threshold(K.thr) : K.thr;
  const int Gm = G - 1;
  const dim3 grid((unsigned)((Gm + kRowCubes - 1) / kRowCubes), (unsigned)Gm, (unsigned)Gm);
  const int64_t nblocks = (int64_t)grid.x * grid.y * grid.z;
  // counts: per-block triangles, new vertices and surface cubes, nblocks + 1 each
  cudaError_t e = reserve(&buf.counts, &buf.counts_cap, 3 * (nblocks + 1));
  if (e == cudaSuccess) e = reserve(&buf.scan, &buf.scan_cap, scan_scratch_ints(3 * (nblocks + 1)));
  if (e == cudaSuccess && !buf.total) e = cudaMallocHost(&buf.total, 3 * sizeof(int));
  if (e == cudaSuccess) e = reserve(&buf.cells, &buf.cells_cap, nblocks * kRowCubes);
  if (e != cudaSuccess) return e;
  mc_count_kernel<<<grid, kSurfThreads, 0, st>>>(buf.field, G, thr, buf.counts, nblocks, buf.cells);
  e = cudaGetLastError();
  // one scan over the three runs: a run's offsets are its scanned values less its first
  if (e == cudaSuccess) e = launch_exclusive_scan(buf.counts, 3 * (nblocks + 1), buf.scan, st, launches);
  if (e == cudaSuccess) {
    mc_totals_kernel<<<1, 1, 0, st>>>(buf.counts, nblocks, buf.total);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  if (launches) *launches += 2;
  const int64_t nt = buf.total[0], nv = buf.total[1];
  const int ncells = buf.total[2];
  if (nt > 0) {
    e = reserve(&buf.verts, &buf.verts_cap, 3 * nv);
    if (e == cudaSuccess) e = reserve(&buf.faces, &buf.faces_cap, 3 * nt);
    if (e == cudaSuccess && soup) e = reserve(&buf.tris, &buf.tris_cap, 9 * nt);
    if (e != cudaSuccess) return e;
    EmitArgs a;
    a.field = buf.field;
    a.G = G;
    a.gx = (int)grid.x;
    a.thr = thr;
    a.cutoff = K.cutoff;
    a.iso = K.iso;
    a.vdx = voxel_dx;
    a.scan = buf.counts;
    a.nblocks = nblocks;
    a.slots = buf.cells;
    a.ncells = ncells;
    a.verts = buf.verts;
    a.faces = buf.faces;
    a.tris = soup ? buf.tris : nullptr;
    const unsigned eblocks = (unsigned)((ncells + kEmitThreads - 1) / kEmitThreads);
    if (buf.raw) {
      if (soup) mc_emit_kernel<true, true><<<eblocks, kEmitThreads, 0, st>>>(a);
      else mc_emit_kernel<true, false><<<eblocks, kEmitThreads, 0, st>>>(a);
    } else {
      if (soup) mc_emit_kernel<false, true><<<eblocks, kEmitThreads, 0, st>>>(a);
      else mc_emit_kernel<false, false><<<eblocks, kEmitThreads, 0, st>>>(a);
    }
    e = cudaGetLastError();
    if (launches) *launches += 1;
  }
  *n_verts = nt > 0 ? nv : 0;
  *n_faces = nt;
  return e;
}

}  // namespace mpm
