// The single-scene fused substep kernel, as a template on the material policy.
//
// substep.cu instantiates it for the library's own materials (BuiltinMaterials); a
// translation unit that includes include/mpm_gb300_policies.cuh instantiates it for a
// material model of its own (the reference's compile-time MaterialModel alias,
// include/mpm.cuh:24-27).  See substep.cu for the design of the kernel.
#pragma once
#include <climits>

#include "mpm_internal.h"
#include "particle_ops.cuh"
#include "tma.cuh"

namespace mpm {

// One step's P2G scatter (particleToGrid's atomic loop, src/mpm.cu:47-73): each lane
// with a contribution writes its 27 node values as a column, then the warp reduces
// runs of same-cell lanes.
// UNIT_MASS: every particle of the warp has mass `run_mass` (a single-material table).
template <bool UNIT_MASS>
__device__ __forceinline__ void p2g_scatter_step(float4* wbuf, int lane, int key, const float w[3][3],
                                                 const float q0[3], const float E[3][3], float m, float run_mass,
                                                 float4* grid, int N) {
  if (__ballot_sync(kFull, key >= 0) == 0u) return;
  if (key >= 0) p2g_write_column_f<UNIT_MASS>(wbuf, lane, w, q0, E, m);
  warp_scatter_runs<UNIT_MASS>(wbuf, lane, key, grid, N, UNIT_MASS ? run_mass : 1.f);
}

// ===========================================================================
// Single scene
// ===========================================================================

// Velocity grid padding (nodes below / above the grid in each dimension) and the TMA
// tile boxes (X along the slowest grid index i, Z along the fastest index k).  A box of
// X x Y x Z nodes covers every step whose base cells span at most (X-2) x (Y-2) x (Z-2)
// cells.  Box 0 (4 x 4 x 6) covers one cell, or two neighbours along a row of a 4x4x4
// sort brick, including the wrap to the next row; box 1 (4 x 4 x 4) copies a third less
// for steps inside 2 x 2 x 2 cells; box 2 (4 x 6 x 6) also covers steps across a
// brick's rows, for sparser scenes.  The autotuner picks one per workload.
constexpr int kPadLo = 3, kPadHi = 2;
template <int TILE>
struct TileBox {
  static constexpr int X = 4, Y = (TILE == 2) ? 6 : 4, Z = (TILE == 1) ? 4 : 6;
  static constexpr int kNodes = X * Y * Z;
  static constexpr uint32_t kBytes = kNodes * sizeof(float4);
};
constexpr int tile_nodes(int tile) {
  return tile == 1 ? TileBox<1>::kNodes : (tile == 2 ? TileBox<2>::kNodes : TileBox<0>::kNodes);
}
enum TileState { kTileNone = 0, kTileSmem = 1, kTileGlobal = 2 };


// G2P gather straight from the velocity grid, for steps whose box exceeds the tile;
// out of line to keep the hot loop small.
static __device__ __noinline__ G2POut g2p_gather_vgrid(const float4* vgrid, GridConsts K, float x0, float x1,
                                                       float x2) {
  const float x[3] = {x0, x1, x2};
  int b[3];
  float w[3][3], f[3];
  stencil_f(x, K, b, w, f);
  const int P = K.N + kPadLo + kPadHi;
  const float4* vb = vgrid + ((int64_t)(b[0] + kPadLo) * P + (b[1] + kPadLo)) * P + (b[2] + kPadLo);
  auto node = [&](int a, int bb, int c) -> float4 { return __ldg(vb + ((int64_t)a * P + bb) * P + c); };
  G2POut o;
  g2p_gather_f(node, K.dinv * K.dx, w, f, o.v, o.C);
  return o;
}

// A load kept where it is written (volatile asm is not moved past the other volatile
// asm of the step, such as the mbarrier wait), so the next step's positions are
// requested at the top of the step and arrive while this step computes.
__device__ __forceinline__ float ld_pin(const float* p) {
  float v;
  asm volatile("ld.global.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}

// Positions, J and the G2P-guard state of one step's particle (lane).
template <bool GUARD>
__device__ __forceinline__ void load_step_head(const StepArgs& A, const float* s, int64_t st, int64_t p, bool valid,
                                               float x[3], float& J, bool& frz) {
  if (valid) {
    x[0] = ld_pin(s + (kX + 0) * st + p);
    x[1] = ld_pin(s + (kX + 1) * st + p);
    x[2] = ld_pin(s + (kX + 2) * st + p);
    J = ld_pin(s + kJp * st + p);
    if (GUARD) frz = (int64_t)A.id[p] > A.guard_limit;
  }
}

// Box of the base cells of a step's G2P particles (warp-collective).  When it fits the
// tile box, lane 0 starts the TMA copy of the tile into `tile`, completing on `bar`.
template <int TILE>
__device__ __forceinline__ int plan_tile(const float x[3], bool active, const GridConsts& K, int lane,
                                         const CUtensorMap* map, float4* tile, uint64_t* bar, int lo[3]) {
  using TB = TileBox<TILE>;
  int b[3], hi[3];
#pragma unroll
  for (int dd = 0; dd < 3; ++dd) b[dd] = QuadraticInterpolationKernel::base_cell(x[dd], K.dx_inv);
  active = active && !outside_domain(b[0], b[1], b[2], K.N);
#pragma unroll
  for (int dd = 0; dd < 3; ++dd) {
    lo[dd] = __reduce_min_sync(kFull, active ? b[dd] : INT_MAX);
    hi[dd] = __reduce_max_sync(kFull, active ? b[dd] : INT_MIN);
  }
  if (hi[0] < lo[0]) return kTileNone;
  if (hi[0] - lo[0] > TB::X - 3 || hi[1] - lo[1] > TB::Y - 3 || hi[2] - lo[2] > TB::Z - 3) return kTileGlobal;
  if (lane == 0) {
    // x coordinate in floats: 4 (lo + pad) is a multiple of 4 floats = 16 bytes
    mbar_arrive_expect_tx(bar, TB::kBytes);
    tma_load_3d(tile, map, 4 * (lo[2] + kPadLo), lo[1] + kPadLo, lo[0] + kPadLo, bar);
  }
  return kTileSmem;
}

__device__ __forceinline__ float4* align_smem128(float4* p) {
  const uint32_t a = smem_addr(p);
  return reinterpret_cast<float4*>(reinterpret_cast<char*>(p) + ((128u - (a & 127u)) & 127u));
}

// WARPS warps per CTA: 4, 6 or 12, so that 3, 2 or 1 CTAs (12 warps) are resident per SM
// at <= 168 registers; shared memory per warp is two TMA tiles (1.5 KB each for box 0)
// plus the 14.3 KB P2G transpose buffer, 17.3 KB (12 warps: 207 KB of the SM's 228 KB).
// TILE: the tile box (TileBox).  MAT: the material policy (particle_ops.cuh).
template <bool LIQ, bool G2P, bool P2G, bool GUARD, int WARPS, int TILE, class MAT = BuiltinMaterials>
__global__ void __launch_bounds__(WARPS * 32, WARPS >= kStepWarps ? 1 : kStepWarps / WARPS)
    scene_step_kernel(const __grid_constant__ StepArgs A) {
  using TB = TileBox<TILE>;
  constexpr int kTileNodes = TB::kNodes, kTileY = TB::Y, kTileZ = TB::Z;
  extern __shared__ float4 smem_dyn[];
  __shared__ int cta_next;  // next CTA-local range index to hand out
  float4* smem = align_smem128(smem_dyn);
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  // per-warp regions: two TMA tiles (G2P), the P2G transpose buffer, two mbarriers
  float4* tiles = smem + warp * (2 * kTileNodes);
  float4* wbuf = smem + (G2P ? WARPS * 2 * kTileNodes : 0) + warp * kRedFloat4;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + (G2P ? WARPS * 2 * kTileNodes : 0) +
                                               (P2G ? WARPS * kRedFloat4 : 0)) +
                   2 * warp;
  const GridConsts& K = A.K.g;  // read from the parameter space, not copied to registers
  const int N = K.N;
  const float ddx = K.dinv * K.dx;  // D dx of the node-offset gather
  float* __restrict__ s = A.s;
  // a G2P-only launch, or a fused launch of the general layout, may write the new state out
  // of place (the adjoint's recompute keeps every state of a segment)
  float* const s_w = ((!P2G || !LIQ) && A.s_out) ? A.s_out : s;
  const int64_t st = A.stride;
  const int64_t n = A.n, chunk = A.chunk;

  if (tid == 0) cta_next = WARPS;
  __syncthreads();
  if (G2P) {
    if (lane == 0) {
      mbar_init(bars, 1);
      mbar_init(bars + 1, 1);
      fence_barrier_init();
    }
    __syncwarp();
  }
  // Ranges of `chunk` particles: CTA c owns ranges c, c + G, c + 2G, ... (G = grid
  // size), interleaved through the sorted particles; its warps take them in turn from a
  // shared-memory counter, so the warps of a CTA balance each other without global
  // atomics.  Warp-uniform bookkeeping: the current range ends at `re`; `rn` is the next
  // range, claimed one range ahead so the step after a range's last is known early.
  const int64_t nranges = (n + chunk - 1) / chunk;
  const int G = (int)gridDim.x;
  const int64_t r0 = (int64_t)blockIdx.x + warp * G;
  if (r0 < nranges) {
    int claim = 0;
    if (lane == 0) claim = atomicAdd(&cta_next, 1);
    int64_t rn = (int64_t)blockIdx.x + __shfl_sync(kFull, claim, 0) * G;
    if (lane == 0) claim = atomicAdd(&cta_next, 1);
    int64_t pb = r0 * chunk;
    int64_t re = min(pb + chunk, n);
    float cx[3] = {0.f, 0.f, 0.f}, cJ = 1.f;
    bool cfz = false;
    load_step_head<GUARD>(A, s, st, pb + lane, pb + lane < re, cx, cJ, cfz);
    int tstate = kTileNone, tlo[3] = {0, 0, 0}, buf = 0;
    uint32_t parity = 0u;  // bit b: phase parity of bars[b]
    // the velocity pass (this launch's programmatic prerequisite) has completed past here
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (G2P) tstate = plan_tile<TILE>(cx, pb + lane < re && !cfz, K, lane, &A.vmap, tiles, bars, tlo);

    while (true) {
      const bool last = pb + 32 >= re;
      const bool more = !last || rn < nranges;
      const int64_t pn = last ? rn * chunk : pb + 32;
      const int64_t pe = last ? min(pn + chunk, n) : re;
      // the next step's positions, one step ahead
      float nx[3] = {0.f, 0.f, 0.f}, nJ = 1.f;
      bool nfz = false;
      const bool nvalid = more && pn + lane < pe;
      load_step_head<GUARD>(A, s, st, pn + lane, nvalid, nx, nJ, nfz);

      const int64_t p = pb + lane;
      const bool valid = p < re;
      float x[3] = {cx[0], cx[1], cx[2]}, v[3] = {0.f, 0.f, 0.f}, Cm[3][3], F[3][3], Jp = cJ;
      int mi = 0;
      bool frozen = !G2P || cfz;
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
          if (A.mat) {
            mi = A.mat[p];
            // an index past the table (caller-owned material arrays are not checked on
            // the host) is flagged and the particle takes material 0
            if (mi >= A.K.n_materials) {
              atomicOr(A.status, kStatusIndex);
              mi = 0;
            }
          }
        }
        if (frozen && P2G) {
#pragma unroll
          for (int dd = 0; dd < 3; ++dd) v[dd] = s[(kV + dd) * st + p];
#pragma unroll
          for (int i = 0; i < 9; ++i) Cm[i / 3][i % 3] = s[(kC + i) * st + p];
        }
      }
      const DevMaterial& M = A.K.mat[mi];
      PolarCache pc;
      pc.valid = false;
      bool g2p_on = false;
      // ---- G2P (gridToParticle, src/mpm.cu:109-167)
      if (G2P) {
        int b[3] = {0, 0, 0};
        float w[3][3], f[3];
        if (valid && !frozen) {
          stencil_f(x, K, b, w, f);
          g2p_on = !outside_domain(b[0], b[1], b[2], N);
          if (!g2p_on) frozen = true;  // completely outside: unchanged; P2G skips it too
        }
        if (tstate == kTileSmem) {
          if (!mbar_wait(bars + buf, (parity >> buf) & 1u) && lane == 0) atomicOr(A.status, kStatusTimeout);
          parity ^= 1u << buf;
          if (g2p_on) {
            const float4* t = tiles + buf * kTileNodes +
                              ((b[0] - tlo[0]) * kTileY + (b[1] - tlo[1])) * kTileZ + (b[2] - tlo[2]);
            auto node = [&](int a, int bb, int c) -> float4 { return t[(a * kTileY + bb) * kTileZ + c]; };
            g2p_gather_f(node, ddx, w, f, v, Cm);
          }
        } else if (tstate == kTileGlobal && g2p_on) {
          const G2POut o = g2p_gather_vgrid(A.vgrid, K, x[0], x[1], x[2]);
#pragma unroll
          for (int r = 0; r < 3; ++r) {
            v[r] = o.v[r];
#pragma unroll
            for (int c = 0; c < 3; ++c) Cm[r][c] = o.C[r][c];
          }
        }
        // The next step's tile goes to the other buffer, whose last reader was the
        // previous step (every lane has passed that step's P2G warp syncs).
        if (more)
          tstate = plan_tile<TILE>(nx, nvalid && !nfz, K, lane, &A.vmap, tiles + (buf ^ 1) * kTileNodes, bars + (buf ^ 1),
                             tlo);
      }
      if (g2p_on) {
        particle_update<LIQ, MAT>(M, K, x, v, Cm, F, Jp, pc);
        store_particle<LIQ>(s_w, st, p, x, v, Cm, F, Jp);
        if (A.check_finite && !isfinite(x[0] + x[1] + x[2] + v[0] + v[1] + v[2])) atomicOr(A.status, kStatusNonFinite);
      } else if (!LIQ && G2P && valid && s_w != s) {
        // out-of-place launch: a particle that G2P leaves alone keeps its state in the output
#pragma unroll 1
        for (int c = 0; c < kNumComps; ++c) s_w[c * st + p] = s[c * st + p];
      }
      // ---- P2G of the next substep (particleToGrid)
      if (P2G) {
        int key = -1;
        float w[3][3], f[3], E[3][3], q0[3], m = 0.f;
        if (valid) {
          int b[3];
          stencil_f(x, K, b, w, f);
          if (!outside_domain(b[0], b[1], b[2], N)) {
            key = pack_key(b[0], b[1], b[2]);
            if (!LIQ && A.rot) {
              // keep R for the adjoint; the stress below reuses it (R = R I^T)
              float R[3][3];
              polar_rotation(F, pc, R);
#pragma unroll
              for (int i = 0; i < 9; ++i) {
                A.rot[i * st + p] = R[i / 3][i % 3];
                pc.U[i / 3][i % 3] = R[i / 3][i % 3];
                pc.V[i / 3][i % 3] = (i / 3 == i % 3) ? 1.f : 0.f;
              }
              pc.valid = true;
            }
            p2g_prepare_f<LIQ, MAT>(M, K, F, Jp, Cm, v, pc, f, E, q0, m);
          }
        }
        p2g_scatter_step<LIQ>(wbuf, lane, key, w, q0, E, m, A.K.mat[0].mass, A.grid_out, N);
      }
      if (!more) break;
      if (last) {
        re = pe;
        rn = (int64_t)blockIdx.x + __shfl_sync(kFull, claim, 0) * G;
        if (lane == 0) claim = atomicAdd(&cta_next, 1);
      }
      pb = pn;
#pragma unroll
      for (int dd = 0; dd < 3; ++dd) cx[dd] = nx[dd];
      cJ = nJ;
      cfz = nfz;
      buf ^= 1;
    }
  }

  // ---- clear the grid buffer the previous substep read (used by the launch after next)
  if (A.grid_zero) {
    const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int64_t i = (int64_t)blockIdx.x * (WARPS * 32) + tid; i < A.grid_cells;
         i += (int64_t)gridDim.x * (WARPS * 32))
      A.grid_zero[i] = z;
  }
}


}  // namespace mpm
