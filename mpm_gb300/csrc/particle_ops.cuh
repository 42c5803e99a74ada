// Per-particle pieces of the substep shared by the single-scene and batched kernels:
// the end of gridToParticle (F update, the material's end-of-step mutation, advection),
// the state write-back, and p2g_prepare_particle (the affine momentum matrix).
//
// The material enters as a policy class MAT with the reference's MaterialModel hooks
// (include/MaterialModel.cuh, bound by the alias MaterialModel in include/mpm.cuh:24-27):
//
//   struct MyMaterial {
//     // F holds (I + dt C) F of the G2P update on entry (g2p_finish_particle,
//     // include/TransferScheme.h:134-142); the hook applies the material's end-of-step
//     // mutation to F and Jp.  It may leave the polar rotation R = U V^T of the new F in
//     // pc (pc.valid = true), which computePF then reuses instead of a second SVD.
//     __device__ static void endOfStepMutation(const mpm::DevMaterial& m, const mpm::GridConsts& K,
//                                              const float C[3][3], float F[3][3], float& Jp,
//                                              mpm::PolarCache& pc);
//     // P F^T of the particle (MaterialModel::computePF).
//     __device__ static void computePF(const mpm::DevMaterial& m, const float F[3][3], float Jp,
//                                      const mpm::PolarCache& pc, float PF[3][3]);
//   };
//
// BuiltinMaterials is the policy of the material kinds the library ships (MMSnow,
// MMFixedCorotated, MMJelly, the weakly compressible liquid), dispatched on m.kind;
// include/mpm_gb300_policies.cuh compiles other policies into the kernel.
#pragma once
#include "svd3.cuh"
#include "warp_ops.cuh"

namespace mpm {

// The rotation of the polar decomposition of F, when the mutation already has it (F =
// U Sigma V^T with Sigma >= 0 gives R = U V^T).
struct PolarCache {
  bool valid;
  float U[3][3], V[3][3];
};

// R of a particle: U V^T from the cache, else the polar decomposition of F.
__device__ __forceinline__ void polar_rotation(const float F[3][3], const PolarCache& pc, float R[3][3]) {
  if (pc.valid) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        R[i][j] = pc.U[i][0] * pc.V[j][0] + pc.U[i][1] * pc.V[j][1] + pc.U[i][2] * pc.V[j][2];
  } else {
    float Sdummy[3][3];
    polar_decomposition(F, R, Sdummy);
  }
}

struct BuiltinMaterials {
  // MMSnow::endOfStepMutation (include/MaterialModel.cuh:95-115), MMJelly
  // (:141-148), nothing for MMFixedCorotated; the liquid keeps J <- J det(I + dt C) and
  // F = J^(1/3) I.  For snow the SVD of F gives U, V, so the next P2G takes the polar
  // rotation of the clamped F as U V^T.
  __device__ __forceinline__ static void endOfStepMutation(const DevMaterial& M, const GridConsts& K,
                                                           const float Cm[3][3], float F[3][3], float& Jp,
                                                           PolarCache& pc) {
    if (M.kind == kLiquid) {
      float G[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) G[i][j] = (i == j ? 1.f : 0.f) + K.dt * Cm[i][j];
      Jp = Jp * det3(G);
      const float cr = cbrtf(Jp);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) F[i][j] = (i == j) ? cr : 0.f;
    } else if (M.kind == kSnow) {
      float sg[3];
      svd3(F, pc.U, sg, pc.V);
#pragma unroll
      for (int i = 0; i < 3; ++i) sg[i] = clampf(sg[i], M.clamp_lo, M.clamp_hi);
      const float oldJ = det3(F);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j)
          F[i][j] = pc.U[i][0] * sg[0] * pc.V[j][0] + pc.U[i][1] * sg[1] * pc.V[j][1] + pc.U[i][2] * sg[2] * pc.V[j][2];
      const float Fdet = det3(F);
      Jp = clampf(Jp * oldJ / Fdet, 0.6f, 20.0f);
      pc.valid = true;
    } else if (M.kind == kJelly) {
      const float oldJ = det3_colwise(F);
      Jp = clampf(Jp * oldJ / det3_colwise(F), 0.6f, 20.0f);
    }
  }

  // MaterialModel::computePF (include/MaterialModel.cuh:56-61, 85-93, 131-139); liquid:
  // K (J - 1) J I.
  __device__ __forceinline__ static void computePF(const DevMaterial& M, const float F[3][3], float Jp,
                                                   const PolarCache& pc, float PF[3][3]) {
    if (M.kind == kLiquid) {
      const float pr = M.bulk * (Jp - 1.f) * Jp;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) PF[i][j] = (i == j) ? pr : 0.f;
    } else {
      float R[3][3];
      polar_rotation(F, pc, R);
      compute_PF(M, F, R, Jp, PF);
    }
  }
};

// g2p_finish_particle + MaterialModel::endOfStepMutation + advection
// (include/TransferScheme.h:134-142, src/mpm.cu:170-176).  LIQ: the single-liquid layout
// keeps only J <- J det(I + dt C) (no F).
template <bool LIQ, class MAT = BuiltinMaterials>
__device__ __forceinline__ void particle_update(const DevMaterial& M, const GridConsts& K, float x[3], const float v[3],
                                                const float Cm[3][3], float F[3][3], float& Jp, PolarCache& pc) {
  if (LIQ) {
    float G[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) G[i][j] = (i == j ? 1.f : 0.f) + K.dt * Cm[i][j];
    Jp = Jp * det3(G);
  } else {
    float Fn[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        Fn[i][j] = F[i][j] + K.dt * (Cm[i][0] * F[0][j] + Cm[i][1] * F[1][j] + Cm[i][2] * F[2][j]);
    MAT::endOfStepMutation(M, K, Cm, Fn, Jp, pc);
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

// MaterialModel::computePF of the particle; the single-liquid layout: K (J - 1) J I.
template <bool LIQ, class MAT = BuiltinMaterials>
__device__ __forceinline__ void material_PF(const DevMaterial& M, const float F[3][3], float Jp, const PolarCache& pc,
                                            float PF[3][3]) {
  if (LIQ) {
    const float pr = M.bulk * (Jp - 1.f) * Jp;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) PF[i][j] = (i == j) ? pr : 0.f;
  } else {
    MAT::computePF(M, F, Jp, pc, PF);
  }
}

// p2g_prepare_particle (include/TransferScheme.h:64-86): affine = -D dt vol PF + m C,
// here in the node-offset form of p2g_write_column_f: E_k = dx affine[:, k] (dx folded
// into the affine's two scale factors) and q0 = m v - sum_k E_k f_k.
template <bool LIQ, class MAT = BuiltinMaterials>
__device__ __forceinline__ void p2g_prepare_f(const DevMaterial& M, const GridConsts& K, const float F[3][3], float Jp,
                                              const float Cm[3][3], const float v[3], const PolarCache& pc,
                                              const float f[3], float E[3][3], float q0[3], float& m) {
  m = M.mass;
  float PF[3][3];
  material_PF<LIQ, MAT>(M, F, Jp, pc, PF);
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
