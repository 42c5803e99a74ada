// Warp-level building blocks shared by the substep and adjoint kernels.
#pragma once
#include "mpm_device.cuh"

namespace mpm {

constexpr int kRedStride = 33;     // float4 row stride of the per-warp transpose buffer
constexpr int kRedFloat4 = 27 * kRedStride;

__device__ __forceinline__ int pack_key(int b0, int b1, int b2) {
  return ((b0 + 4) << 20) | ((b1 + 4) << 10) | (b2 + 4);
}
__device__ __forceinline__ void unpack_key(int key, int& b0, int& b1, int& b2) {
  b0 = (key >> 20) - 4;
  b1 = ((key >> 10) & 1023) - 4;
  b2 = (key & 1023) - 4;
}

__device__ __forceinline__ void add_node(float4* grid, int N, int i, int j, int k, float4 val) {
  if ((unsigned)i < (unsigned)N && (unsigned)j < (unsigned)N && (unsigned)k < (unsigned)N)
    atomicAdd(grid + ((int64_t)i * N + j) * N + k, val);
}

__device__ __forceinline__ void f4add(float4& a, const float4 b) {
  a.x += b.x;
  a.y += b.y;
  a.z += b.z;
  a.w += b.w;
}

// p2g_node_contribution (include/TransferScheme.h:88-100) for all 27 nodes, written
// as column `lane` of the warp's transpose buffer: row n = node (a, b, c) holds
//   (w_n (m v + A dpos_n), w_n m).
__device__ __forceinline__ void p2g_write_column(float4* wbuf, int lane, const float w[3][3], const float d[3][3],
                                                 const float Aff[3][3], const float mv[3], float m) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float qa[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) qa[r] = fmaf(Aff[r][0], d[0][a], mv[r]);
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      float qab[3];
#pragma unroll
      for (int r = 0; r < 3; ++r) qab[r] = fmaf(Aff[r][1], d[1][b], qa[r]);
      const float wab = w[0][a] * w[1][b];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float wt = wab * w[2][c];
        float4 val;
        val.x = wt * fmaf(Aff[0][2], d[2][c], qab[0]);
        val.y = wt * fmaf(Aff[1][2], d[2][c], qab[1]);
        val.z = wt * fmaf(Aff[2][2], d[2][c], qab[2]);
        val.w = wt * m;
        wbuf[(a * 9 + b * 3 + c) * kRedStride + lane] = val;
      }
    }
  }
}

// Warp-collective scatter of 27 node values per lane (column `lane` of the warp's
// buffer, written by the caller; key = packed base cell, -1 for no contribution).
// Lane l < 27 walks the 32 columns in order, summing node l over each run of
// consecutive lanes that share a base cell (cell-sorted particles make a run per
// cell) and issuing one vector atomic per run; runs with key -1 are dropped.  The run
// boundaries are warp-uniform, so the walk does not diverge.
__device__ __forceinline__ void warp_scatter_runs(float4* wbuf, int lane, int key, float4* grid, int N) {
  const int prev = __shfl_up_sync(kFull, key, 1);
  const unsigned starts = __ballot_sync(kFull, lane == 0 || key != prev);
  __syncwarp();
  // walk the runs (warp-uniform loop); lane l < 27 sums node l over the run's columns
  const float4* row = wbuf + (lane < 27 ? lane : 0) * kRedStride;
  unsigned rs = starts;
#pragma unroll 1
  while (rs) {
    const int j0 = __ffs(rs) - 1;
    rs &= rs - 1u;
    const int j1 = rs ? __ffs(rs) - 1 : 32;
    const int run_key = __shfl_sync(kFull, key, j0);
    if (run_key >= 0 && lane < 27) {
      float4 s0 = make_float4(0.f, 0.f, 0.f, 0.f), s1 = s0, s2 = s0, s3 = s0;
      int j = j0;
#pragma unroll 1
      for (; j + 3 < j1; j += 4) {
        f4add(s0, row[j]);
        f4add(s1, row[j + 1]);
        f4add(s2, row[j + 2]);
        f4add(s3, row[j + 3]);
      }
#pragma unroll 1
      for (; j < j1; ++j) f4add(s0, row[j]);
      f4add(s0, s1);
      f4add(s2, s3);
      f4add(s0, s2);
      int b0, b1, b2;
      unpack_key(run_key, b0, b1, b2);
      add_node(grid, N, b0 + lane / 9, b1 + (lane / 3) % 3, b2 + lane % 3, s0);
    }
  }
  __syncwarp();
}

// weights_per_direction for all three dimensions plus the node offsets
// dpos = (base + a) dx - x (src/mpm.cu:50-60).
__device__ __forceinline__ void stencil(const float x[3], const GridConsts& K, int b[3], float w[3][3], float d[3][3]) {
#pragma unroll
  for (int dim = 0; dim < 3; ++dim) {
    QuadraticInterpolationKernel::weights_per_direction(x[dim], K.dx_inv, b[dim], w[dim]);
    d[dim][0] = fmaf((float)b[dim], K.dx, -x[dim]);
    d[dim][1] = d[dim][0] + K.dx;
    d[dim][2] = d[dim][1] + K.dx;
  }
}

// gridToParticle gather (src/mpm.cu:136-167 + g2p_node_contribution), factorised per
// dimension: v = sum w g, C = D sum w g dpos^T (D = 4/dx^2).  `node(a, b, c)`
// returns the grid velocity of node base + (a, b, c), zero outside the grid.
template <class NodeFn>
__device__ __forceinline__ void g2p_gather(NodeFn node, const GridConsts& K, const float w[3][3], const float d[3][3],
                                           float v[3], float C[3][3]) {
  float c0[3] = {0.f, 0.f, 0.f}, c1[3] = {0.f, 0.f, 0.f}, c2[3] = {0.f, 0.f, 0.f};
  v[0] = v[1] = v[2] = 0.f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float U[3] = {0.f, 0.f, 0.f}, Vv[3] = {0.f, 0.f, 0.f}, W[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int bb = 0; bb < 3; ++bb) {
      float S[3] = {0.f, 0.f, 0.f}, T[3] = {0.f, 0.f, 0.f};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float4 g = node(a, bb, c);
        const float wz = w[2][c], wzd = w[2][c] * d[2][c];
        S[0] = fmaf(wz, g.x, S[0]);
        S[1] = fmaf(wz, g.y, S[1]);
        S[2] = fmaf(wz, g.z, S[2]);
        T[0] = fmaf(wzd, g.x, T[0]);
        T[1] = fmaf(wzd, g.y, T[1]);
        T[2] = fmaf(wzd, g.z, T[2]);
      }
      const float wy = w[1][bb], wyd = w[1][bb] * d[1][bb];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        U[r] = fmaf(wy, S[r], U[r]);
        Vv[r] = fmaf(wyd, S[r], Vv[r]);
        W[r] = fmaf(wy, T[r], W[r]);
      }
    }
    const float wx = w[0][a], wxd = w[0][a] * d[0][a];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      v[r] = fmaf(wx, U[r], v[r]);
      c0[r] = fmaf(wxd, U[r], c0[r]);
      c1[r] = fmaf(wx, Vv[r], c1[r]);
      c2[r] = fmaf(wx, W[r], c2[r]);
    }
  }
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    C[r][0] = K.dinv * c0[r];
    C[r][1] = K.dinv * c1[r];
    C[r][2] = K.dinv * c2[r];
  }
}

struct G2POut {
  float v[3];
  float C[3][3];
};

// Gather straight from the P2G grid (grid op per node) for chunks whose tile does
// not fit in shared memory; out of line to keep the hot loop small.
static __device__ __noinline__ G2POut g2p_gather_global(const float4* grid_in, const GridConsts& K, float x0, float x1,
                                                 float x2) {
  const int N = K.N;
  const float x[3] = {x0, x1, x2};
  int b[3];
  float w[3][3], d[3][3];
  stencil(x, K, b, w, d);
  const int b0 = b[0], b1 = b[1], b2 = b[2];
  auto node = [&](int a, int bb, int c) -> float4 {
    const int i = b0 + a, j = b1 + bb, k = b2 + c;
    if ((unsigned)i >= (unsigned)N || (unsigned)j >= (unsigned)N || (unsigned)k >= (unsigned)N)
      return make_float4(0.f, 0.f, 0.f, 0.f);
    const float3 v = grid_node_velocity(__ldg(grid_in + ((int64_t)i * N + j) * N + k), i, j, k, K);
    return make_float4(v.x, v.y, v.z, 0.f);
  };
  G2POut o;
  g2p_gather(node, K, w, d, o.v, o.C);
  return o;
}


}  // namespace mpm
