// Fused MLS-MPM substep kernel for sm_103a.
//
// The reference runs four launches per substep (src/mpm.cu:323-329): cudaMemset of
// the grid, particleToGrid (27 x 4 float atomics per particle), gridOpKernel, and
// gridToParticle.  Here one launch does
//     G2P of substep n  (gather from the P2G grid of substep n; the grid op is applied
//                        while a block stages its grid tile in shared memory)
//   + constitutive update + advection, state written once
//   + P2G of substep n+1 (scatter of the new state)
//   + clearing of the grid buffer substep n-1 read,
// so particle state is read once and written once per substep and the three grid
// buffers rotate.  A P2G-only variant starts a run from uploaded state.
//
// Work decomposition: warps are the scheduling unit.  Each warp of a 12-warp CTA
// takes a range of cell-sorted particles (steps_per_warp x 32) and walks it 32
// particles at a time (lane = particle, coalesced component-major loads/stores);
// further ranges are claimed from a global counter, so faster warps take more.
// G2P reads a per-warp shared-memory tile of grid velocities staged once for a
// window of steps whose base cells fit the tile.  P2G is a warp transpose-reduce:
// every lane writes its 27 node contributions as a column of a per-warp buffer, and
// lane l < 27 sums node l over each run of same-cell lanes and issues one vector
// atomic per run.  Dense scenes (100+ particles per cell) thus issue about one
// global atomic per node and step instead of the reference's 108 per particle.
//
// Code size matters: the hot loop holds one copy each of the gather, the column
// write and the run walk (the rare paths are out of line) so it stays resident in
// the instruction cache.
#include <climits>

#include "mpm_internal.h"
#include "warp_ops.cuh"

namespace mpm {

// One step's P2G scatter (particleToGrid's atomic loop, src/mpm.cu:47-73): each lane
// with a contribution writes its 27 node values as a column, then the warp reduces
// runs of same-cell lanes.
__device__ __forceinline__ void p2g_scatter_step(float4* wbuf, int lane, int key, const float w[3][3],
                                                 const float d[3][3], const float Aff[3][3], const float mv[3],
                                                 float m, float4* grid, int N) {
  if (__ballot_sync(kFull, key >= 0) == 0u) return;
  if (key >= 0) p2g_write_column(wbuf, lane, w, d, Aff, mv, m);
  warp_scatter_runs(wbuf, lane, key, grid, N);
}

// Per-warp grid tile: the nodes [lo, hi + 2]^3 around a box of base cells, with the
// grid op applied (grid velocity), zero outside the grid.  lo/hi are warp-uniform.
struct TileBox {
  int t0, t1, t2, d1, d2;
};

__device__ __forceinline__ bool box_fits(const int lo[3], const int hi[3], int cap) {
  int64_t vol = 1;
#pragma unroll
  for (int dd = 0; dd < 3; ++dd) vol *= (hi[dd] >= lo[dd]) ? (int64_t)(hi[dd] + 3 - lo[dd]) : 0;
  return vol <= cap;
}

__device__ __forceinline__ void warp_tile_build(float4* wtile, int lane, const int lo[3], const int hi[3],
                                                const float4* grid_in, const GridConsts& K, TileBox& tb) {
  int ext[3];
#pragma unroll
  for (int dd = 0; dd < 3; ++dd) ext[dd] = (hi[dd] >= lo[dd]) ? hi[dd] + 3 - lo[dd] : 0;
  const int vol = ext[0] * ext[1] * ext[2];
  const int N = K.N;
  tb.t0 = lo[0];
  tb.t1 = lo[1];
  tb.t2 = lo[2];
  tb.d1 = max(ext[1], 1);
  tb.d2 = max(ext[2], 1);
  const int d12 = tb.d1 * tb.d2;
  __syncwarp();  // every lane is done with the previous tile
  for (int idx = lane; idx < vol; idx += 32) {
    const int i = tb.t0 + idx / d12;
    const int rem = idx - (idx / d12) * d12;
    const int j = tb.t1 + rem / tb.d2;
    const int k = tb.t2 + rem - (rem / tb.d2) * tb.d2;
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    if ((unsigned)i < (unsigned)N && (unsigned)j < (unsigned)N && (unsigned)k < (unsigned)N) {
      const float3 vv = grid_node_velocity(grid_in[((int64_t)i * N + j) * N + k], i, j, k, K);
      out = make_float4(vv.x, vv.y, vv.z, 0.f);
    }
    wtile[idx] = out;
  }
  __syncwarp();
}

template <bool LIQ, bool G2P, bool P2G, bool GUARD, bool BATCH>
__global__ void __launch_bounds__(kStepThreads, 1) step_kernel(const __grid_constant__ StepArgs A) {
  extern __shared__ float4 smem[];
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  // per-warp regions: velocity tile (G2P), P2G transpose buffer
  float4* wtile = smem + warp * A.tile_cap;
  float4* wbuf = smem + (G2P ? kStepWarps * A.tile_cap : 0) + warp * kRedFloat4;
  GridConsts K = A.K.g;
  int N = K.N;
  const float4* gin = A.grid_in;
  float4* gout = A.grid_out;
  float* __restrict__ s = A.s;
  const int64_t st = A.stride;

  // Warps are the scheduling unit: each resident warp starts on one range of A.chunk
  // consecutive (cell-sorted) particles and claims further ranges from a global
  // counter while finishing the last step of its current one, so warps that run
  // faster take more ranges; no CTA barriers.
  if (blockIdx.x == 0 && tid == 0) *A.work_next = 0;
  if (BATCH) {
    // clear, per scene, the grid region the launch two substeps back accumulated (the
    // buffer this launch leaves for the next one to fill), then free its box slot
    for (int sc = blockIdx.x; sc < A.nscenes; sc += gridDim.x) {
      const int* bx = A.boxes + ((int64_t)sc * kBoxSlots + A.box_clear) * 6;
      const SceneDev& sd = A.scenes[sc];
      const int Ns = sd.g.N;
      const int l0 = max(bx[0], 0), l1 = max(bx[1], 0), l2 = max(bx[2], 0);
      const int h0 = min(bx[3] + 2, Ns - 1), h1 = min(bx[4] + 2, Ns - 1), h2 = min(bx[5] + 2, Ns - 1);
      if (h0 >= l0 && h1 >= l1 && h2 >= l2 && A.grid_zero) {
        const int e1 = h1 - l1 + 1, e2 = h2 - l2 + 1;
        const int64_t vol = (int64_t)(h0 - l0 + 1) * e1 * e2;
        float4* gz = A.grid_zero + sd.grid_offset;
        for (int64_t q = tid; q < vol; q += kStepThreads) {
          const int i = l0 + (int)(q / ((int64_t)e1 * e2));
          const int rem = (int)(q % ((int64_t)e1 * e2));
          gz[((int64_t)i * Ns + (l1 + rem / e2)) * Ns + (l2 + rem % e2)] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
      }
      if (tid < 6) A.boxes[((int64_t)sc * kBoxSlots + A.box_reset) * 6 + tid] = (tid < 3) ? INT_MAX : INT_MIN;
    }
  }
  const int64_t nranges = BATCH ? A.nranges : (A.n + A.chunk - 1) / A.chunk;
  const int64_t first_wave = (int64_t)gridDim.x * kStepWarps;
  int64_t r = (int64_t)blockIdx.x * kStepWarps + warp;
  while (r < nranges) {
    int claim = 0;
    int64_t wbeg, wend;
    int scene = 0;
    if (BATCH) {
      const int4 rg = A.ranges[r];
      scene = rg.x;
      wbeg = rg.y;
      wend = rg.z;
      const SceneDev& sd = A.scenes[scene];
      K = sd.g;
      N = K.N;
      gin = A.grid_in ? A.grid_in + sd.grid_offset : nullptr;
      gout = A.grid_out + sd.grid_offset;
    } else {
      wbeg = r * A.chunk;
      wend = min(wbeg + (int64_t)A.chunk, A.n);
    }
    int plo[3] = {INT_MAX, INT_MAX, INT_MAX}, phi[3] = {INT_MIN, INT_MIN, INT_MIN};  // P2G box (batch)
    TileBox tb{0, 0, 0, 1, 1};
    int64_t win_end = wbeg;  // end of the steps the current tile covers
    bool tile_ok = false;

    // ---- walk the range, one particle per lane; positions and Jp of the next step
    // are loaded one step ahead
    float nx0 = 0.f, nx1 = 0.f, nx2 = 0.f, nJ = 1.f;
    if (wbeg + lane < wend) {
      nx0 = s[(kX + 0) * st + wbeg + lane];
      nx1 = s[(kX + 1) * st + wbeg + lane];
      nx2 = s[(kX + 2) * st + wbeg + lane];
      nJ = s[kJp * st + wbeg + lane];
    }
    for (int64_t pb = wbeg; pb < wend; pb += 32) {
      if (G2P && pb >= win_end) {
        // grow a window of steps from pb while the union of their base-cell boxes fits
        // the warp's tile, then stage the tile once for the whole window
        int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {INT_MIN, INT_MIN, INT_MIN};
        int64_t we = pb;
        while (we < wend) {
          const int64_t q = we + lane;
          int slo[3] = {INT_MAX, INT_MAX, INT_MAX}, shi[3] = {INT_MIN, INT_MIN, INT_MIN};
          if (q < wend && !(GUARD && (int64_t)A.id[q] > A.guard_limit)) {
            int bb[3];
#pragma unroll
            for (int dd = 0; dd < 3; ++dd)
              bb[dd] = QuadraticInterpolationKernel::base_cell(s[(kX + dd) * st + q], K.dx_inv);
            if (!outside_domain(bb[0], bb[1], bb[2], N)) {
#pragma unroll
              for (int dd = 0; dd < 3; ++dd) slo[dd] = shi[dd] = bb[dd];
            }
          }
          int nlo[3], nhi[3];
#pragma unroll
          for (int dd = 0; dd < 3; ++dd) {
            nlo[dd] = min(lo[dd], __reduce_min_sync(kFull, slo[dd]));
            nhi[dd] = max(hi[dd], __reduce_max_sync(kFull, shi[dd]));
          }
          if (!box_fits(nlo, nhi, A.tile_cap)) break;
#pragma unroll
          for (int dd = 0; dd < 3; ++dd) {
            lo[dd] = nlo[dd];
            hi[dd] = nhi[dd];
          }
          we += 32;
        }
        tile_ok = we > pb;
        win_end = tile_ok ? we : pb + 32;  // a step that alone does not fit gathers from global
        if (tile_ok) warp_tile_build(wtile, lane, lo, hi, gin, K, tb);
      }
      const int64_t p = pb + lane;
      const bool valid = p < wend;
      if (pb + 32 >= wend && lane == 0) claim = atomicAdd(A.work, 1);
      float x[3] = {nx0, nx1, nx2}, v[3] = {0.f, 0.f, 0.f}, Cm[3][3], F[3][3], Jp = nJ;
      if (p + 32 < wend) {
        nx0 = s[(kX + 0) * st + p + 32];
        nx1 = s[(kX + 1) * st + p + 32];
        nx2 = s[(kX + 2) * st + p + 32];
        nJ = s[kJp * st + p + 32];
      }
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
      const DevMaterial& M = BATCH ? A.scenes[scene].m : A.K.mat[mi];
      // ---- G2P + constitutive update + advection (gridToParticle)
      bool have_uv = false;
      float Usv[3][3], Vsv[3][3];
      bool g2p_on = false;
      if (G2P && valid && !frozen) {
        int b[3];
        float w[3][3], d[3][3];
        stencil(x, K, b, w, d);
        g2p_on = !outside_domain(b[0], b[1], b[2], N);
        if (!g2p_on) {
          frozen = true;  // completely outside: unchanged; P2G skips it too
        } else if (tile_ok) {
          const int t0 = ((b[0] - tb.t0) * tb.d1 + (b[1] - tb.t1)) * tb.d2 + (b[2] - tb.t2);
          const int d12 = tb.d1 * tb.d2;
          auto node = [&](int a, int bb, int c) -> float4 { return wtile[t0 + a * d12 + bb * tb.d2 + c]; };
          g2p_gather(node, K, w, d, v, Cm);
        } else {
          // a step whose own box exceeds the tile (rare: a jump between brick rows)
          const G2POut o = g2p_gather_global(gin, K, x[0], x[1], x[2]);
#pragma unroll
          for (int r = 0; r < 3; ++r) {
            v[r] = o.v[r];
#pragma unroll
            for (int c = 0; c < 3; ++c) Cm[r][c] = o.C[r][c];
          }
        }
      }
      if (g2p_on) {
        {
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
            if (BATCH) {
#pragma unroll
              for (int dd = 0; dd < 3; ++dd) {
                plo[dd] = min(plo[dd], b[dd]);
                phi[dd] = max(phi[dd], b[dd]);
              }
            }
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
        p2g_scatter_step(wbuf, lane, key, w, d, Aff, mv, m, gout, N);
      }
    }
    if (BATCH && P2G) {
      // record the range's P2G box in its scene's slot (cleared two launches later)
      int* bx = A.boxes + ((int64_t)scene * kBoxSlots + A.box_record) * 6;
#pragma unroll
      for (int dd = 0; dd < 3; ++dd) {
        const int l = __reduce_min_sync(kFull, plo[dd]);
        const int h = __reduce_max_sync(kFull, phi[dd]);
        if (lane == 0 && h >= l) {
          atomicMin(bx + dd, l);
          atomicMax(bx + 3 + dd, h);
        }
      }
    }
    r = first_wave + __shfl_sync(kFull, claim, 0);
  }

  // ---- clear the grid buffer the previous substep read (used by the launch after next)
  if (!BATCH && A.grid_zero) {
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int64_t i = (int64_t)blockIdx.x * kStepThreads + tid; i < A.grid_cells;
         i += (int64_t)gridDim.x * kStepThreads)
      A.grid_zero[i] = z;
  }
}

template <bool LIQ, bool G2P, bool P2G, bool GUARD, bool BATCH>
static void* kernel_ptr() {
  return (void*)step_kernel<LIQ, G2P, P2G, GUARD, BATCH>;
}

static void* select_kernel(StepKind kind, bool liquid, bool guard, bool batch) {
  if (batch) {  // batches use the general layout, no guard
    if (kind == kStepP2GOnly) return kernel_ptr<false, false, true, false, true>();
    return kernel_ptr<false, true, true, false, true>();
  }
#define MPM_SEL(L, G)                                                        \
  if (liquid == L && guard == G) {                                           \
    if (kind == kStepP2GOnly) return kernel_ptr<L, false, true, G, false>(); \
    if (kind == kStepFused) return kernel_ptr<L, true, true, G, false>();    \
    return kernel_ptr<L, true, false, G, false>();                           \
  }
  MPM_SEL(true, false)
  MPM_SEL(true, true)
  MPM_SEL(false, false)
  MPM_SEL(false, true)
#undef MPM_SEL
  return nullptr;
}

size_t step_smem_bytes(StepKind kind, int tile_cap) {
  size_t b = 0;
  if (kind != kStepP2GOnly) b += (size_t)kStepWarps * tile_cap * sizeof(float4);
  if (kind != kStepG2POnly) b += (size_t)kStepWarps * kRedFloat4 * sizeof(float4);
  return b;
}

cudaError_t launch_step(const StepArgs& a, StepKind kind, bool liquid, bool guard, int grid_blocks, cudaStream_t st) {
  void* fn = select_kernel(kind, liquid, guard, a.nscenes > 0);
  const size_t smem = step_smem_bytes(kind, a.tile_cap);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  StepArgs copy = a;
  void* args[] = {&copy};
  return cudaLaunchKernel(fn, dim3(grid_blocks), dim3(kStepThreads), args, smem, st);
}

int step_blocks_per_sm(StepKind kind, bool liquid, bool guard, size_t smem, bool batch) {
  void* fn = select_kernel(kind, liquid, guard, batch);
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 1;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kStepThreads, smem) != cudaSuccess || nb < 1) nb = 1;
  return nb;
}

}  // namespace mpm
