// Device-side types and policy functions of the GB300 MLS-MPM substep.
//
// The reference binds its plug-in policies with compile-time aliases
// (include/mpm.cuh:24-27):
//   InterpolationKernel = QuadraticInterpolationKernel  (include/InterpolationKernel.cuh:53-74)
//   TransferScheme      = MLS_APIC_Scheme               (include/TransferScheme.h:56-143)
//   MaterialModel       = MMSnow                        (include/MaterialModel.cuh:67-116)
// The same policies exist here with the same method names, written for a
// register-resident, warp-cooperative kernel: weights are per-dimension arrays,
// matrices are float[3][3], and a material is a small POD selected per particle.
#pragma once
#include <stdint.h>

#include "svd3.cuh"

namespace mpm {

constexpr int kMaxMaterials = 16;
constexpr int kThreads = 256;  // CTA size of the auxiliary kernels (8 warps)
constexpr int kWarps = kThreads / 32;
constexpr int kStepThreads = 384;  // CTA size of the substep kernel (12 warps, <= 168 registers)
constexpr int kStepWarps = kStepThreads / 32;
// CTA of the P2G-only substep kernel (the first P2G of a run, the adjoint's recomputed P2G):
// it needs no G2P tiles and fits 128 registers, so 15 warps share an SM's shared memory
// (15 P2G transpose buffers, 209 KB) where the fused kernel's 168 registers allow 12.
constexpr int kP2GWarps = 15;
constexpr unsigned kFull = 0xffffffffu;

enum MatKind { kSnow = 0, kFixedCorotated = 1, kJelly = 2, kLiquid = 3 };
enum Boundary { kBoundaryRefFraction = 0, kBoundaryStickyCells = 1, kBoundarySeparateCells = 2 };

// Device status word bits.
enum StatusBits { kStatusNonFinite = 1, kStatusIndex = 2, kStatusTimeout = 4 };

// MaterialModel constants, derived in float exactly like the reference constructors
// (MaterialModelBase: mass = density * volume; MMFixedCorotated: mu0, lambda0).
struct DevMaterial {
  int kind;
  float vol, mass, mu0, lambda0, hardening, clamp_lo, clamp_hi, bulk;
};

// SimulationParameters (include/TransferScheme.h:6-29) plus the grid-op constants
// of one grid (one scene).
struct GridConsts {
  float dt, dx, dx_inv, dinv, dtg;  // dinv = D_inv_const diagonal = 4 dx_inv^2; dtg = dt * gravity
  int N;
  int boundary_mode, boundary_cells;
};

// Grid constants plus the material table.
struct SimConsts {
  GridConsts g;
  int n_materials;
  DevMaterial mat[kMaxMaterials];
};

// Particle state, component-major SoA: component k of particle p at s[k * stride + p].
// Components: x 0-2, v 3-5, C 6-14 (row-major), F 15-23 (row-major), Jp 24.
// The liquid-only layout touches x, v, C and J (component 24) only: 16 components.
enum Comp { kX = 0, kV = 3, kC = 6, kF = 15, kJp = 24, kNumComps = 25 };
constexpr int kLiquidComps = 16;

// ---------------------------------------------------------------------------
// InterpolationKernel: quadratic B-spline (include/InterpolationKernel.cuh:53-74)
// ---------------------------------------------------------------------------
struct QuadraticInterpolationKernel {
  static constexpr int size() { return 3; }
  static constexpr bool d_is_const() { return true; }
  // range_begin = int(x / dx - 0.5) (truncation, as Eigen's cast<int>), fx = x/dx - range_begin
  // x / dx is rounded on its own (__fmul_rn cannot be contracted into an FMA), so every
  // caller that derives a base cell from a position gets the same cell.
  __device__ __forceinline__ static float grid_coord(float x, float dx_inv) { return __fmul_rn(x, dx_inv); }
  __device__ __forceinline__ static int base_cell(float x, float dx_inv) {
    return (int)__fsub_rn(grid_coord(x, dx_inv), 0.5f);
  }
  __device__ __forceinline__ static void weights_per_direction(float x, float dx_inv, int& range_begin,
                                                               float w[3]) {
    const float xg = grid_coord(x, dx_inv);
    range_begin = (int)__fsub_rn(xg, 0.5f);
    const float fx = xg - (float)range_begin;
    const float a = 1.5f - fx, b = fx - 1.f, c = fx - 0.5f;
    w[0] = 0.5f * (a * a);
    w[1] = 0.75f - b * b;
    w[2] = 0.5f * (c * c);
  }
  // The same weights plus f = x / dx - range_begin, the particle's offset from its base
  // node in cells (in [0.5, 1.5)); node a of the stencil is at dpos = (a - f) dx.
  __device__ __forceinline__ static void weights_and_offset(float x, float dx_inv, int& range_begin, float w[3],
                                                            float& f) {
    const float xg = grid_coord(x, dx_inv);
    range_begin = (int)__fsub_rn(xg, 0.5f);
    const float fx = xg - (float)range_begin;
    const float a = 1.5f - fx, b = fx - 1.f, c = fx - 0.5f;
    w[0] = 0.5f * (a * a);
    w[1] = 0.75f - b * b;
    w[2] = 0.5f * (c * c);
    f = fx;
  }
  // D^-1 = 4 / dx^2 I for the quadratic kernel (computed on the host as (4 dx_inv) dx_inv)
};

// Completely outside the domain: src/mpm.cu:31-35, 130-134.
__device__ __forceinline__ bool outside_domain(int b0, int b1, int b2, int N) {
  return (b0 + 3 < 0) | (b0 >= N) | (b1 + 3 < 0) | (b1 >= N) | (b2 + 3 < 0) | (b2 >= N);
}

// ---------------------------------------------------------------------------
// Grid operation (gridOpKernel, src/mpm.cu:76-107) for one node, returning the
// velocity G2P reads (cell.head<3>()).  Nodes with mass <= 0 keep their raw value.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float3 grid_node_velocity(float4 g, int i, int j, int k, const GridConsts& K) {
  float3 v = make_float3(g.x, g.y, g.z);
  if (g.w > 0.f) {
    const float inv = 1.f / g.w;
    v.x = g.x * inv;
    v.y = g.y * inv;
    v.z = g.z * inv;
    v.y += K.dtg;
    bool sticky, floor_;
    const int N = K.N;
    if (K.boundary_mode == kBoundaryRefFraction) {
      const float b = 0.05f;
      const float fN = (float)N;
      const float x = (float)i / fN, y = (float)j / fN, z = (float)k / fN;
      sticky = x < b || x > 1.f - b || y > 1.f - b || z < b || z > 1.f - b;
      floor_ = y < b;
    } else if (K.boundary_mode == kBoundaryStickyCells) {
      const int bc = K.boundary_cells;
      sticky = i < bc || i >= N - bc || j < bc || j >= N - bc || k < bc || k >= N - bc;
      floor_ = false;
    } else {
      const int bc = K.boundary_cells;
      sticky = i < bc || i >= N - bc || j >= N - bc || k < bc || k >= N - bc;
      floor_ = j < bc;
    }
    if (sticky) v = make_float3(0.f, 0.f, 0.f);
    if (floor_) v.y = fmaxf(0.f, v.y);
  }
  return v;
}

__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fmaxf(fminf(v, hi), lo); }

// ---------------------------------------------------------------------------
// MaterialModel::computePF (include/MaterialModel.cuh:56-61, 85-93, 131-139):
//   P F^T = 2 mu (F - R) F^T + lambda (Jp - 1) Jp I, with mu, lambda scaled by
//   exp(h (1 - Jp)) for snow/jelly; the stress uses the stored Jp, not det F.
// R is the rotation of the polar decomposition of F, passed in by the caller
// (it may come from the SVD the plasticity step already computed).
// Liquid: P F^T = K (J - 1) J I.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void compute_PF(const DevMaterial& m, const float F[3][3], const float R[3][3],
                                           float Jp, float PF[3][3]) {
  float mu = m.mu0, lambda = m.lambda0;
  if (m.kind == kSnow || m.kind == kJelly) {
    const float e = (m.hardening == 0.f) ? 1.f : expf(m.hardening * (1.f - Jp));
    mu *= e;
    lambda *= e;
  }
  const float two_mu = 2.f * mu;
  const float lt = lambda * ((Jp - 1.f) * Jp);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float a0 = two_mu * (F[i][0] - R[i][0]);
      const float a1 = two_mu * (F[i][1] - R[i][1]);
      const float a2 = two_mu * (F[i][2] - R[i][2]);
      PF[i][j] = a0 * F[j][0] + a1 * F[j][1] + a2 * F[j][2] + (i == j ? lt : 0.f);
    }
}

}  // namespace mpm
