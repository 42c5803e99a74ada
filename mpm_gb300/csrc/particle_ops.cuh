// Per-particle pieces of the substep shared by the single-scene and batched kernels:
// the end of gridToParticle (F update, plasticity, advection), the state write-back,
// and p2g_prepare_particle (the affine momentum matrix).
#pragma once
#include "svd3.cuh"
#include "warp_ops.cuh"

namespace mpm {

// g2p_finish_particle + MaterialModel::endOfStepMutation + advection
// (include/TransferScheme.h:134-142, include/MaterialModel.cuh:95-115 and 142-148,
// src/mpm.cu:170-176).  The liquid keeps J <- J det(I + dt C) and F = J^(1/3) I.
// For snow the SVD of the updated F is returned in U, V (have_uv) so the next P2G
// takes the polar rotation of the clamped F as U V^T instead of a second SVD.
template <bool LIQ>
__device__ __forceinline__ void particle_update(const DevMaterial& M, const GridConsts& K, float x[3], const float v[3],
                                                const float Cm[3][3], float F[3][3], float& Jp, bool& have_uv,
                                                float Usv[3][3], float Vsv[3][3]) {
  if (LIQ || M.kind == kLiquid) {
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
    float Fn[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        Fn[i][j] = F[i][j] + K.dt * (Cm[i][0] * F[0][j] + Cm[i][1] * F[1][j] + Cm[i][2] * F[2][j]);
    if (M.kind == kSnow) {
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
}

// particles[pi] = particle (src/mpm.cu:177): one component-major write of the state.
template <bool LIQ>
__device__ __forceinline__ void store_particle(float* s, int64_t st, int64_t p, const float x[3], const float v[3],
                                               const float Cm[3][3], const float F[3][3], float Jp) {
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
}

// MaterialModel::computePF (include/MaterialModel.cuh:56-61, 85-93): P F^T of the
// particle.  For snow after plasticity the polar rotation of the clamped F is U V^T
// (have_uv): F = U clamp(Sigma) V^T with clamp(Sigma) >= 0.
template <bool LIQ>
__device__ __forceinline__ void material_PF(const DevMaterial& M, const float F[3][3], float Jp, bool have_uv,
                                            const float Usv[3][3], const float Vsv[3][3], float PF[3][3]) {
  if (LIQ || M.kind == kLiquid) {
    const float pr = M.bulk * (Jp - 1.f) * Jp;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) PF[i][j] = (i == j) ? pr : 0.f;
  } else {
    float R[3][3];
    if (have_uv) {
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
}

// p2g_prepare_particle (include/TransferScheme.h:64-86): affine = -D dt vol PF + m C,
// here in the node-offset form of p2g_write_column_f: E_k = dx affine[:, k] (dx folded
// into the affine's two scale factors) and q0 = m v - sum_k E_k f_k.
template <bool LIQ>
__device__ __forceinline__ void p2g_prepare_f(const DevMaterial& M, const GridConsts& K, const float F[3][3], float Jp,
                                              const float Cm[3][3], const float v[3], bool have_uv,
                                              const float Usv[3][3], const float Vsv[3][3], const float f[3],
                                              float E[3][3], float q0[3], float& m) {
  m = M.mass;
  float PF[3][3];
  material_PF<LIQ>(M, F, Jp, have_uv, Usv, Vsv, PF);
  const float scx = (((-K.dinv) * K.dt) * M.vol) * K.dx;
  const float mdx = m * K.dx;
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int r = 0; r < 3; ++r) E[k][r] = fmaf(scx, PF[r][k], mdx * Cm[r][k]);
#pragma unroll
  for (int r = 0; r < 3; ++r) q0[r] = fmaf(-E[2][r], f[2], fmaf(-E[1][r], f[1], fmaf(-E[0][r], f[0], m * v[r])));
}

}  // namespace mpm
