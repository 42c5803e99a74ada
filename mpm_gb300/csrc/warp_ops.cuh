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

// Warp-collective scatter of 27 node values per lane (column `lane` of the warp's
// buffer, written by the caller; key = packed base cell, -1 for no contribution).
// Lane l < 27 walks the 32 columns in order, summing node l over each run of
// consecutive lanes that share a base cell (cell-sorted particles make a run per
// cell) and issuing one vector atomic per run; runs with key -1 are dropped.  The run
// boundaries are warp-uniform, so the walk does not diverge.
// `mass_scale` multiplies the summed .w (columns written with unit mass hold weights).
// SINGLE_RUN_PATH: a straight-line walk when the whole warp is one run.  It took the
// liquid substep from 61 to 59 us, but made the snow substep 8 us slower (its larger
// kernel), so only the liquid layout uses it.
template <bool SINGLE_RUN_PATH = false>
__device__ __forceinline__ void warp_scatter_runs(float4* wbuf, int lane, int key, float4* grid, int N,
                                                  float mass_scale = 1.f) {
  const int prev = __shfl_up_sync(kFull, key, 1);
  const unsigned starts = __ballot_sync(kFull, lane == 0 || key != prev);
  __syncwarp();
  // walk the runs (warp-uniform loop); lane l < 27 sums node l over the run's columns
  const float4* row = wbuf + (lane < 27 ? lane : 0) * kRedStride;
  if (SINGLE_RUN_PATH && starts == 1u) {
    // One run over the whole warp, the common case of dense scenes (a warp's 32
    // cell-sorted particles share a cell): the 32 columns in straight-line code, summed
    // in the order of the loop below (bit-identical).  Unrolled by two: the full unroll
    // spilled.
    if (key >= 0 && lane < 27) {
      float4 s0 = make_float4(0.f, 0.f, 0.f, 0.f), s1 = s0, s2 = s0, s3 = s0;
#pragma unroll 2
      for (int j = 0; j < 32; j += 4) {
        f4add(s0, row[j]);
        f4add(s1, row[j + 1]);
        f4add(s2, row[j + 2]);
        f4add(s3, row[j + 3]);
      }
      f4add(s0, s1);
      f4add(s2, s3);
      f4add(s0, s2);
      s0.w *= mass_scale;
      int b0, b1, b2;
      unpack_key(key, b0, b1, b2);
      add_node(grid, N, b0 + lane / 9, b1 + (lane / 3) % 3, b2 + lane % 3, s0);
    }
    __syncwarp();
    return;
  }
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
      s0.w *= mass_scale;
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

// Weights and base cells like stencil(), with the offsets f = x / dx - base instead of
// the node distances: the distance of node a is dpos = (a - f) dx.
__device__ __forceinline__ void stencil_f(const float x[3], const GridConsts& K, int b[3], float w[3][3], float f[3]) {
#pragma unroll
  for (int dim = 0; dim < 3; ++dim)
    QuadraticInterpolationKernel::weights_and_offset(x[dim], K.dx_inv, b[dim], w[dim], f[dim]);
}

// gridToParticle gather (src/mpm.cu:136-167 + g2p_node_contribution) with integer node
// offsets o in {0, 1, 2}^3: dpos = (o - f) dx, so
//   v = sum w g,   C = D sum w g dpos^T = D dx (sum w g o^T - v f^T)   (ddx = D dx),
// factorised per dimension; the o = 0 terms of the first moments vanish.
template <class NodeFn>
__device__ __forceinline__ void g2p_gather_f(NodeFn node, float ddx, const float w[3][3], const float f[3], float v[3],
                                             float C[3][3]) {
  float mx[3], my[3], mz[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float U[3], Vy[3], Wz[3];
#pragma unroll
    for (int bb = 0; bb < 3; ++bb) {
      const float4 g0 = node(a, bb, 0), g1 = node(a, bb, 1), g2 = node(a, bb, 2);
      const float w0 = w[2][0], w1 = w[2][1], w2 = w[2][2], w2x2 = 2.f * w[2][2];
      float S[3], T[3];
      S[0] = fmaf(w2, g2.x, fmaf(w1, g1.x, w0 * g0.x));
      S[1] = fmaf(w2, g2.y, fmaf(w1, g1.y, w0 * g0.y));
      S[2] = fmaf(w2, g2.z, fmaf(w1, g1.z, w0 * g0.z));
      T[0] = fmaf(w2x2, g2.x, w1 * g1.x);
      T[1] = fmaf(w2x2, g2.y, w1 * g1.y);
      T[2] = fmaf(w2x2, g2.z, w1 * g1.z);
      const float wy = w[1][bb];
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        U[r] = bb ? fmaf(wy, S[r], U[r]) : wy * S[r];
        Wz[r] = bb ? fmaf(wy, T[r], Wz[r]) : wy * T[r];
        if (bb == 1) Vy[r] = wy * S[r];
        if (bb == 2) Vy[r] = fmaf(2.f * wy, S[r], Vy[r]);
      }
    }
    const float wx = w[0][a];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      v[r] = a ? fmaf(wx, U[r], v[r]) : wx * U[r];
      my[r] = a ? fmaf(wx, Vy[r], my[r]) : wx * Vy[r];
      mz[r] = a ? fmaf(wx, Wz[r], mz[r]) : wx * Wz[r];
      if (a == 1) mx[r] = wx * U[r];
      if (a == 2) mx[r] = fmaf(2.f * wx, U[r], mx[r]);
    }
  }
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    C[r][0] = ddx * fmaf(-v[r], f[0], mx[r]);
    C[r][1] = ddx * fmaf(-v[r], f[1], my[r]);
    C[r][2] = ddx * fmaf(-v[r], f[2], mz[r]);
  }
}

// p2g_node_contribution (include/TransferScheme.h:88-100) for all 27 nodes with integer
// node offsets: node o = (a, b, c) receives w_o (m v + A dpos_o) = w_o (q0 + a E0 + b E1 + c E2)
// with E_k = dx A[:, k] (E[k][r]) and q0 = m v - sum_k E_k f_k.  Written as column `lane`
// of the warp's transpose buffer: row a*9 + b*3 + c holds (w_o (...), w_o m), or w_o in
// .w when UNIT_MASS (the walk scales the summed weight by the particles' common mass).
template <bool UNIT_MASS>
__device__ __forceinline__ void p2g_write_column_f(float4* wbuf, int lane, const float w[3][3], const float q0[3],
                                                   const float E[3][3], float m) {
  float qa[3] = {q0[0], q0[1], q0[2]};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (a) {
#pragma unroll
      for (int r = 0; r < 3; ++r) qa[r] += E[0][r];
    }
    float qab[3] = {qa[0], qa[1], qa[2]};
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      if (b) {
#pragma unroll
        for (int r = 0; r < 3; ++r) qab[r] += E[1][r];
      }
      const float wab = w[0][a] * w[1][b];
      float q[3] = {qab[0], qab[1], qab[2]};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (c) {
#pragma unroll
          for (int r = 0; r < 3; ++r) q[r] += E[2][r];
        }
        const float wt = wab * w[2][c];
        wbuf[(a * 9 + b * 3 + c) * kRedStride + lane] =
            make_float4(wt * q[0], wt * q[1], wt * q[2], UNIT_MASS ? wt : wt * m);
      }
    }
  }
}

struct G2POut {
  float v[3];
  float C[3][3];
};

}  // namespace mpm
