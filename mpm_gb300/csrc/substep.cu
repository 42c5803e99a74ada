// Fused MLS-MPM substep kernel for sm_103a.
//
// The reference runs four launches per substep (src/mpm.cu:323-329): cudaMemset of
// the grid, particleToGrid (27 x 4 float atomics per particle), gridOpKernel, and
// gridToParticle.  Here one launch does
//     G2P of substep n  (gather from the P2G grid of substep n, grid op applied on
//                        the fly while a block stages its grid tile in shared memory)
//   + constitutive update + advection, state written once
//   + P2G of substep n+1 (scatter of the new state)
//   + clearing of the grid buffer substep n-1 read,
// so particle state is read once and written once per substep and the three grid
// buffers rotate.  A P2G-only variant starts a run from uploaded state.
//
// Work decomposition: a CTA of 8 warps takes a contiguous chunk of cell-sorted
// particles; each warp walks its slice 32 particles at a time (lane = particle,
// coalesced SoA loads/stores).  P2G contributions are accumulated in registers
// (27 nodes x 4 values per lane) while the lane's particles stay in one cell; when a
// lane's cell changes, the warp flushes whole cell groups with a shuffle
// reduce-scatter (lane l ends with node l's total) and one vector atomic per node,
// or, when a warp's particles scatter over many cells, each lane adds its 27 nodes
// directly.  Dense scenes (100+ particles per cell) thus issue well under one
// global atomic per particle instead of the reference's 108.
#include <climits>

#include "mpm_internal.h"

namespace mpm {

constexpr int kMaxGroups = 3;  // cell groups reduced with shuffles per flush before falling back

__device__ __forceinline__ int pack_key(int b0, int b1, int b2) {
  return ((b0 + 4) << 20) | ((b1 + 4) << 10) | (b2 + 4);
}
__device__ __forceinline__ void unpack_key(int key, int& b0, int& b1, int& b2) {
  b0 = (key >> 20) - 4;
  b1 = ((key >> 10) & 1023) - 4;
  b2 = (key & 1023) - 4;
}

// p2g_node_contribution (include/TransferScheme.h:88-100) for all 27 nodes:
//   acc[n] += w_n (m v + A dpos_n), acc[n].w += w_n m
__device__ __forceinline__ void p2g_accumulate(float (&acc)[27][4], const float w[3][3], const float d[3][3],
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
        const int n = a * 9 + b * 3 + c;
#pragma unroll
        for (int r = 0; r < 3; ++r) acc[n][r] = fmaf(wt, fmaf(Aff[r][2], d[2][c], qab[r]), acc[n][r]);
        acc[n][3] = fmaf(wt, m, acc[n][3]);
      }
    }
  }
}

template <int H>
__device__ __forceinline__ void reduce_half(float (&r)[16][4], int lane) {
  const bool up = (lane & H) != 0;
#pragma unroll
  for (int j = 0; j < H; ++j)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const float lo = r[j][c], hi = r[j + H][c];
      const float send = up ? lo : hi;
      const float keep = up ? hi : lo;
      r[j][c] = keep + __shfl_xor_sync(kFull, send, H);
    }
}

__device__ __forceinline__ void add_node(float4* grid, int N, int i, int j, int k, float4 val) {
  if ((unsigned)i < (unsigned)N && (unsigned)j < (unsigned)N && (unsigned)k < (unsigned)N)
    atomicAdd(grid + ((int64_t)i * N + j) * N + k, val);
}

// Warp-collective: sum the accumulators of the lanes with in == true (one cell group,
// base cell `key`) and add the 27 node totals to the grid, one vector atomic per node.
__device__ __forceinline__ void flush_group(const float (&acc)[27][4], bool in, int key, int lane, float4* grid,
                                            int N) {
  float r[16][4];
  const bool up = (lane & 16) != 0;
#pragma unroll
  for (int j = 0; j < 16; ++j)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const float lo = acc[j][c];
      const float hi = (j + 16 < 27) ? acc[(j + 16 < 27) ? j + 16 : 0][c] : 0.f;
      float send = up ? lo : hi;
      float keep = up ? hi : lo;
      send = in ? send : 0.f;
      keep = in ? keep : 0.f;
      r[j][c] = keep + __shfl_xor_sync(kFull, send, 16);
    }
  reduce_half<8>(r, lane);
  reduce_half<4>(r, lane);
  reduce_half<2>(r, lane);
  reduce_half<1>(r, lane);
  if (lane < 27) {
    int b0, b1, b2;
    unpack_key(key, b0, b1, b2);
    add_node(grid, N, b0 + lane / 9, b1 + (lane / 3) % 3, b2 + lane % 3,
             make_float4(r[0][0], r[0][1], r[0][2], r[0][3]));
  }
}

// One lane adds its own 27 accumulators (sparse fallback).
__device__ __forceinline__ void flush_direct(const float (&acc)[27][4], int key, float4* grid, int N) {
  int b0, b1, b2;
  unpack_key(key, b0, b1, b2);
#pragma unroll
  for (int n = 0; n < 27; ++n)
    add_node(grid, N, b0 + n / 9, b1 + (n / 3) % 3, b2 + n % 3, make_float4(acc[n][0], acc[n][1], acc[n][2], acc[n][3]));
}

__device__ __forceinline__ void zero_acc(float (&acc)[27][4]) {
#pragma unroll
  for (int n = 0; n < 27; ++n)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[n][c] = 0.f;
}

// Warp-collective flush of every cell group whose `flag` is set in some member lane.
__device__ __forceinline__ void flush_groups(float (&acc)[27][4], int& acc_key, bool flag, int lane, float4* grid,
                                             int N) {
  const unsigned need = __ballot_sync(kFull, flag);
  const unsigned same = __match_any_sync(kFull, acc_key);
  const bool gflag = (same & need) != 0u && acc_key >= 0;
  const bool leader = gflag && lane == __ffs(same) - 1;
  unsigned leaders = __ballot_sync(kFull, leader);
  if (__popc(leaders) <= kMaxGroups) {
    while (leaders) {
      const int ll = __ffs(leaders) - 1;
      leaders &= leaders - 1u;
      const int K = __shfl_sync(kFull, acc_key, ll);
      const bool in = acc_key == K;
      flush_group(acc, in, K, lane, grid, N);
      if (in) {
        zero_acc(acc);
        acc_key = -1;
      }
    }
  } else if (gflag) {
    flush_direct(acc, acc_key, grid, N);
    zero_acc(acc);
    acc_key = -1;
  }
}

// Velocity of grid node (i,j,k) for G2P, either from the block's tile or straight
// from the P2G grid (grid op applied per fetch) when the tile did not fit.
struct NodeFetch {
  const float4* tile;
  const float4* grid_in;
  int t0, t1, t2, d1, d2;  // tile origin and extents (d0 implied)
  int vol;                 // nodes in the tile
  bool use_tile;
};

__device__ __forceinline__ float3 fetch_node(const NodeFetch& f, const SimConsts& K, int i, int j, int k) {
  if (f.use_tile) {
    const int idx = ((i - f.t0) * f.d1 + (j - f.t1)) * f.d2 + (k - f.t2);
    // every gathered node lies in the chunk's tile by construction; the check keeps a
    // node outside it (which would be a bug) on the global path instead of off the tile
    if ((unsigned)idx < (unsigned)f.vol && (unsigned)(k - f.t2) < (unsigned)f.d2 &&
        (unsigned)(j - f.t1) < (unsigned)f.d1) {
      const float4 g = f.tile[idx];
      return make_float3(g.x, g.y, g.z);
    }
  }
  const float4 g = __ldg(f.grid_in + ((int64_t)i * K.N + j) * K.N + k);
  return grid_node_velocity(g, i, j, k, K);
}

// gridToParticle gather (src/mpm.cu:136-167 + g2p_node_contribution), factorised per
// dimension: v = sum w g, C = D sum w g dpos^T (D = 4/dx^2), with nodes outside the
// grid skipped as the reference's clipped loop does.
__device__ __forceinline__ void g2p_gather(const NodeFetch& f, const SimConsts& K, const int b[3], const float w[3][3],
                                           const float d[3][3], float v[3], float C[3][3]) {
  const int N = K.N;
  const bool interior = b[0] >= 0 && b[0] + 2 < N && b[1] >= 0 && b[1] + 2 < N && b[2] >= 0 && b[2] + 2 < N;
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
        const int i = b[0] + a, j = b[1] + bb, k = b[2] + c;
        float3 g = make_float3(0.f, 0.f, 0.f);
        if (interior || ((unsigned)i < (unsigned)N && (unsigned)j < (unsigned)N && (unsigned)k < (unsigned)N))
          g = fetch_node(f, K, i, j, k);
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

// weights_per_direction for all three dimensions plus the node offsets
// dpos = (base + a) dx - x (src/mpm.cu:50-60).
__device__ __forceinline__ void stencil(const float x[3], const SimConsts& K, int b[3], float w[3][3], float d[3][3]) {
#pragma unroll
  for (int dim = 0; dim < 3; ++dim) {
    QuadraticInterpolationKernel::weights_per_direction(x[dim], K.dx_inv, b[dim], w[dim]);
#pragma unroll
    for (int a = 0; a < 3; ++a) d[dim][a] = (float)(b[dim] + a) * K.dx - x[dim];
  }
}

template <bool LIQ, bool G2P, bool P2G, bool GUARD>
__global__ void __launch_bounds__(kThreads, 1) step_kernel(const __grid_constant__ StepArgs A) {
  extern __shared__ float4 tile[];
  __shared__ int s_red[kWarps][6];
  __shared__ int s_box[7];

  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const SimConsts& K = A.K;
  const int N = K.N;
  float* __restrict__ s = A.s;
  const int64_t st = A.stride;
  const int64_t nchunks = (A.n + A.chunk - 1) / A.chunk;

  for (int64_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
    const int64_t p0 = ch * A.chunk;
    const int64_t p1 = min(p0 + (int64_t)A.chunk, A.n);
    NodeFetch nf;
    nf.tile = tile;
    nf.grid_in = A.grid_in;
    nf.use_tile = false;
    nf.t0 = nf.t1 = nf.t2 = 0;
    nf.d1 = nf.d2 = 1;
    nf.vol = 0;
    if (G2P) {
      // ---- bounding box of the chunk's base cells -> shared-memory velocity tile
      int lo0 = INT_MAX, lo1 = INT_MAX, lo2 = INT_MAX, hi0 = INT_MIN, hi1 = INT_MIN, hi2 = INT_MIN;
      for (int64_t p = p0 + tid; p < p1; p += kThreads) {
        if (GUARD && (int64_t)A.id[p] > A.guard_limit) continue;
        const float x0 = s[(kX + 0) * st + p], x1 = s[(kX + 1) * st + p], x2 = s[(kX + 2) * st + p];
        const int b0 = QuadraticInterpolationKernel::base_cell(x0, K.dx_inv);
        const int b1 = QuadraticInterpolationKernel::base_cell(x1, K.dx_inv);
        const int b2 = QuadraticInterpolationKernel::base_cell(x2, K.dx_inv);
        if (outside_domain(b0, b1, b2, N)) continue;
        lo0 = min(lo0, b0);
        lo1 = min(lo1, b1);
        lo2 = min(lo2, b2);
        hi0 = max(hi0, b0);
        hi1 = max(hi1, b1);
        hi2 = max(hi2, b2);
      }
      lo0 = __reduce_min_sync(kFull, lo0);
      lo1 = __reduce_min_sync(kFull, lo1);
      lo2 = __reduce_min_sync(kFull, lo2);
      hi0 = __reduce_max_sync(kFull, hi0);
      hi1 = __reduce_max_sync(kFull, hi1);
      hi2 = __reduce_max_sync(kFull, hi2);
      if (lane == 0) {
        s_red[warp][0] = lo0;
        s_red[warp][1] = lo1;
        s_red[warp][2] = lo2;
        s_red[warp][3] = hi0;
        s_red[warp][4] = hi1;
        s_red[warp][5] = hi2;
      }
      __syncthreads();
      if (tid == 0) {
        int l[3] = {INT_MAX, INT_MAX, INT_MAX}, h[3] = {INT_MIN, INT_MIN, INT_MIN};
        for (int w = 0; w < kWarps; ++w)
          for (int dd = 0; dd < 3; ++dd) {
            l[dd] = min(l[dd], s_red[w][dd]);
            h[dd] = max(h[dd], s_red[w][3 + dd]);
          }
        int64_t vol = 1;
        for (int dd = 0; dd < 3; ++dd) {
          l[dd] = max(l[dd], 0);
          h[dd] = (h[dd] == INT_MIN) ? -1 : min(h[dd] + 2, N - 1);
          const int ext = h[dd] >= l[dd] ? h[dd] - l[dd] + 1 : 0;
          s_box[dd] = l[dd];
          s_box[3 + dd] = ext;
          vol *= ext;
        }
        s_box[6] = (vol <= (int64_t)A.tile_cap) ? (int)vol : -1;
      }
      __syncthreads();
      const int vol = s_box[6];
      nf.t0 = s_box[0];
      nf.t1 = s_box[1];
      nf.t2 = s_box[2];
      nf.d1 = max(s_box[4], 1);
      nf.d2 = max(s_box[5], 1);
      nf.use_tile = vol >= 0;
      nf.vol = vol;
      if (nf.use_tile) {
        const int d12 = nf.d1 * nf.d2;
        for (int idx = tid; idx < vol; idx += kThreads) {
          const int i = nf.t0 + idx / d12;
          const int rem = idx - (idx / d12) * d12;
          const int j = nf.t1 + rem / nf.d2;
          const int k = nf.t2 + rem - (rem / nf.d2) * nf.d2;
          const float4 g = A.grid_in[((int64_t)i * N + j) * N + k];
          const float3 vv = grid_node_velocity(g, i, j, k, K);
          tile[idx] = make_float4(vv.x, vv.y, vv.z, 0.f);
        }
      }
      __syncthreads();
    }

    // ---- per-warp walk over the chunk slice, one particle per lane
    const int seg = A.chunk / kWarps;
    const int64_t wbeg = p0 + (int64_t)warp * seg;
    const int64_t wend = min(wbeg + seg, p1);
    float acc[27][4];
    int acc_key = -1;
    if (P2G) zero_acc(acc);

    for (int64_t pb = wbeg; pb < wend; pb += 32) {
      const int64_t p = pb + lane;
      const bool valid = p < wend;
      float x[3] = {0.f, 0.f, 0.f}, v[3] = {0.f, 0.f, 0.f}, Cm[3][3], F[3][3], Jp = 1.f;
      int mi = 0;
      bool frozen = !G2P;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          Cm[i][j] = 0.f;
          F[i][j] = (i == j) ? 1.f : 0.f;
        }
      if (valid) {
#pragma unroll
        for (int dd = 0; dd < 3; ++dd) x[dd] = s[(kX + dd) * st + p];
        Jp = s[kJp * st + p];
        if (!LIQ) {
#pragma unroll
          for (int i = 0; i < 9; ++i) F[i / 3][i % 3] = s[(kF + i) * st + p];
          if (A.mat) mi = A.mat[p];
        }
        if (GUARD && (int64_t)A.id[p] > A.guard_limit) frozen = true;
        if (frozen && P2G) {
#pragma unroll
          for (int dd = 0; dd < 3; ++dd) v[dd] = s[(kV + dd) * st + p];
#pragma unroll
          for (int i = 0; i < 9; ++i) Cm[i / 3][i % 3] = s[(kC + i) * st + p];
        }
      }
      const DevMaterial& M = K.mat[mi];

      // ---- G2P + constitutive update + advection (gridToParticle)
      bool have_uv = false;
      float Usv[3][3], Vsv[3][3];
      if (G2P && valid && !frozen) {
        int b[3];
        float w[3][3], d[3][3];
        stencil(x, K, b, w, d);
        if (!outside_domain(b[0], b[1], b[2], N)) {
          g2p_gather(nf, K, b, w, d, v, Cm);
          if (LIQ || M.kind == kLiquid) {
            // J <- J det(I + dt C), F = J^(1/3) I
            float G[3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
              for (int j = 0; j < 3; ++j) G[i][j] = (i == j ? 1.f : 0.f) + K.dt * Cm[i][j];
            Jp = Jp * det3(G);
            if (!LIQ) {
              const float cr = cbrtf(Jp);
#pragma unroll
              for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) F[i][j] = (i == j) ? cr : 0.f;
            }
          } else {
            // g2p_finish_particle: F <- (I + dt C) F   (include/TransferScheme.h:134-142)
            float Fn[3][3];
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
              for (int j = 0; j < 3; ++j)
                Fn[i][j] = F[i][j] + K.dt * (Cm[i][0] * F[0][j] + Cm[i][1] * F[1][j] + Cm[i][2] * F[2][j]);
            if (M.kind == kSnow) {
              // MMSnow::endOfStepMutation (include/MaterialModel.cuh:95-115)
              float sg[3];
              svd3(Fn, Usv, sg, Vsv);
#pragma unroll
              for (int i = 0; i < 3; ++i) sg[i] = clampf(sg[i], M.clamp_lo, M.clamp_hi);
              const float oldJ = det3(Fn);
#pragma unroll
              for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                  Fn[i][j] = Usv[i][0] * sg[0] * Vsv[j][0] + Usv[i][1] * sg[1] * Vsv[j][1] + Usv[i][2] * sg[2] * Vsv[j][2];
              const float Fdet = det3(Fn);
              Jp = clampf(Jp * oldJ / Fdet, 0.6f, 20.0f);
              have_uv = true;
            } else if (M.kind == kJelly) {
              // MMJelly::endOfStepMutation (include/MaterialModel.cuh:142-148)
              const float oldJ = det3_colwise(Fn);
              Jp = clampf(Jp * oldJ / det3_colwise(Fn), 0.6f, 20.0f);
            }
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
              for (int j = 0; j < 3; ++j) F[i][j] = Fn[i][j];
          }
#pragma unroll
          for (int dd = 0; dd < 3; ++dd) x[dd] = x[dd] + K.dt * v[dd];
          // ---- write back (particles[pi] = particle, src/mpm.cu:177)
#pragma unroll
          for (int dd = 0; dd < 3; ++dd) {
            s[(kX + dd) * st + p] = x[dd];
            s[(kV + dd) * st + p] = v[dd];
          }
#pragma unroll
          for (int i = 0; i < 9; ++i) s[(kC + i) * st + p] = Cm[i / 3][i % 3];
          if (!LIQ) {
#pragma unroll
            for (int i = 0; i < 9; ++i) s[(kF + i) * st + p] = F[i / 3][i % 3];
          }
          s[kJp * st + p] = Jp;
          if (A.check_finite && !isfinite(x[0] + x[1] + x[2] + v[0] + v[1] + v[2]))
            atomicOr(A.status, kStatusNonFinite);
        } else {
          frozen = true;  // completely outside: unchanged; P2G skips it too
        }
      }

      // ---- P2G of the next substep (particleToGrid)
      if (P2G) {
        int key = -1;
        float w[3][3], d[3][3], Aff[3][3], mv[3], m = 0.f;
        if (valid) {
          int b[3];
          stencil(x, K, b, w, d);
          if (!outside_domain(b[0], b[1], b[2], N)) {
            key = pack_key(b[0], b[1], b[2]);
            m = M.mass;
            float PF[3][3];
            if (LIQ || M.kind == kLiquid) {
              const float pr = M.bulk * (Jp - 1.f) * Jp;
#pragma unroll
              for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int j = 0; j < 3; ++j) PF[i][j] = (i == j) ? pr : 0.f;
            } else {
              float R[3][3];
              if (have_uv) {
                // F = U clamp(Sigma) V^T with clamp(Sigma) >= 0, so its polar rotation is U V^T
#pragma unroll
                for (int i = 0; i < 3; ++i)
#pragma unroll
                  for (int j = 0; j < 3; ++j)
                    R[i][j] = Usv[i][0] * Vsv[j][0] + Usv[i][1] * Vsv[j][1] + Usv[i][2] * Vsv[j][2];
              } else {
                float Sdummy[3][3];
                polar_decomposition(F, R, Sdummy);
              }
              compute_PF(M, F, R, Jp, PF);
            }
            // p2g_prepare_particle: affine = -D dt vol PF + m C (include/TransferScheme.h:78-85)
            const float sc = ((-K.dinv) * K.dt) * M.vol;
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
              for (int j = 0; j < 3; ++j) Aff[i][j] = fmaf(sc, PF[i][j], m * Cm[i][j]);
#pragma unroll
            for (int dd = 0; dd < 3; ++dd) mv[dd] = v[dd] * m;
          }
        }
        bool todo = key >= 0;
        if (todo && (acc_key < 0 || acc_key == key)) {
          acc_key = key;
          p2g_accumulate(acc, w, d, Aff, mv, m);
          todo = false;
        }
        if (__any_sync(kFull, todo)) {
          flush_groups(acc, acc_key, todo, lane, A.grid_out, N);
          if (todo) {
            acc_key = key;
            p2g_accumulate(acc, w, d, Aff, mv, m);
          }
        }
      }
    }
    if (P2G) flush_groups(acc, acc_key, acc_key >= 0, lane, A.grid_out, N);
    if (G2P) __syncthreads();  // the tile is rebuilt for the next chunk
  }

  // ---- clear the grid buffer the previous substep read (used by the launch after next)
  if (A.grid_zero) {
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int64_t i = (int64_t)blockIdx.x * kThreads + tid; i < A.grid_cells; i += (int64_t)gridDim.x * kThreads)
      A.grid_zero[i] = z;
  }
}

template <bool LIQ, bool G2P, bool P2G, bool GUARD>
static void* kernel_ptr() {
  return (void*)step_kernel<LIQ, G2P, P2G, GUARD>;
}

static void* select_kernel(StepKind kind, bool liquid, bool guard) {
#define MPM_SEL(L, G)                                                   \
  if (liquid == L && guard == G) {                                      \
    if (kind == kStepP2GOnly) return kernel_ptr<L, false, true, G>();   \
    if (kind == kStepFused) return kernel_ptr<L, true, true, G>();      \
    return kernel_ptr<L, true, false, G>();                             \
  }
  MPM_SEL(true, false)
  MPM_SEL(true, true)
  MPM_SEL(false, false)
  MPM_SEL(false, true)
#undef MPM_SEL
  return nullptr;
}

cudaError_t launch_step(const StepArgs& a, StepKind kind, bool liquid, bool guard, int grid_blocks, cudaStream_t st) {
  void* fn = select_kernel(kind, liquid, guard);
  const size_t smem = (kind == kStepP2GOnly) ? 0 : (size_t)a.tile_cap * sizeof(float4);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  StepArgs copy = a;
  void* args[] = {&copy};
  return cudaLaunchKernel(fn, dim3(grid_blocks), dim3(kThreads), args, smem, st);
}

int step_blocks_per_sm(StepKind kind, bool liquid, bool guard, size_t smem) {
  void* fn = select_kernel(kind, liquid, guard);
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 1;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kThreads, smem) != cudaSuccess || nb < 1) nb = 1;
  return nb;
}

}  // namespace mpm
