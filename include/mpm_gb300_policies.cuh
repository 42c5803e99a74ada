/*
 * mpm_gb300 — material models compiled into the substep kernel.
 *
 * The reference binds its material model at compile time: `using MaterialModel =
 * MMSnow<Particle>;` (include/mpm.cuh:25), where a MaterialModel provides computePF and
 * endOfStepMutation over a particle (include/MaterialModel.cuh).  Here a material model is
 * a policy class, a template parameter of the fused substep kernel, with the same two
 * hooks written for one particle held in registers:
 *
 *   struct MyMaterial {
 *     // P F^T of the particle (MaterialModel::computePF).  pc may hold the polar rotation
 *     // of F left by endOfStepMutation; mpm::polar_rotation(F, pc, R) returns it, or
 *     // computes it by an SVD when pc.valid is false.
 *     __device__ static void computePF(const mpm::DevMaterial& m, const float F[3][3], float Jp,
 *                                      const mpm::PolarCache& pc, float PF[3][3]);
 *     // MaterialModel::endOfStepMutation: F holds (I + dt C) F of the G2P update on entry
 *     // (g2p_finish_particle, include/TransferScheme.h:134-142); the hook updates F and Jp
 *     // in place, and may store U, V with R = U V^T in pc (pc.valid = true).
 *     __device__ static void endOfStepMutation(const mpm::DevMaterial& m, const mpm::GridConsts& K,
 *                                              const float C[3][3], float F[3][3], float& Jp,
 *                                              mpm::PolarCache& pc);
 *   };
 *
 * The material's constants come from its mpm_material row, derived as the reference's
 * constructors do (mpm::DevMaterial: vol, mass, mu0, lambda0, hardening, clamp_lo,
 * clamp_hi, bulk), and the grid constants from mpm::GridConsts (dt, dx, ...).  Helpers the
 * built-in models use are available: mpm::svd3, mpm::det3, mpm::det3_colwise,
 * mpm::polar_rotation, mpm::compute_PF, mpm::clampf.
 *
 * In one .cu file of a build of the library (mpm_gb300.build.build_with_materials compiles
 * such files into a library of their own):
 *
 *   #include "mpm_gb300_policies.cuh"
 *   struct MyMaterial { ... };
 *   MPM_GB300_REGISTER_MATERIAL(MyMaterial, 16)
 *
 * instantiates the substep kernels for MyMaterial and registers them under material kind 16
 * (MPM_MAT_USER_BASE .. MPM_MAT_USER_END - 1) when the library is loaded.  A context whose
 * material table uses kind 16 (mpm_set_materials; every row of that table of kind 16) runs
 * them.  Such a context uses the default launch shape (12 warps per CTA, tile box 4x4x6) and
 * the general particle layout; batches, the no-allocation substep, the differentiable
 * substeps and the G2P guard take the built-in kinds only.
 *
 * The interpolation kernel stays the reference's QuadraticInterpolationKernel, the only one
 * it defines (InterpolationKernelBase<3, true>, include/InterpolationKernel.cuh:55): the
 * transfers' layouts (the 27-node P2G transpose, the G2P tile boxes) are built on its
 * three-node support.
 *
 * Compile with the library's flags and the include paths of include/ and mpm_gb300/csrc/.
 */
#ifndef MPM_GB300_POLICIES_CUH
#define MPM_GB300_POLICIES_CUH

#include "mpm_gb300.h"
#include "substep_kernel.cuh"

#define MPM_GB300_REGISTER_MATERIAL(Policy, KIND)                                                         \
  static_assert((KIND) >= MPM_MAT_USER_BASE && (KIND) < MPM_MAT_USER_END,                               \
                "material kinds of compiled-in models are MPM_MAT_USER_BASE .. MPM_MAT_USER_END - 1"); \
  namespace {                                                                                           \
  struct mpm_gb300_register_##Policy {                                                                  \
    mpm_gb300_register_##Policy() {                                                                     \
      mpm::register_material_kernels(                                                                   \
          (KIND), mpm::MaterialKernels{                                                                 \
                      (void*)mpm::scene_step_kernel<false, true, true, false, mpm::kStepWarps, 0, Policy>,  \
                      (void*)mpm::scene_step_kernel<false, false, true, false, mpm::kStepWarps, 0, Policy>, \
                      (void*)mpm::scene_step_kernel<false, true, false, false, mpm::kStepWarps, 0, Policy>}); \
    }                                                                                                   \
  } mpm_gb300_register_instance_##Policy;                                                               \
  }

#endif /* MPM_GB300_POLICIES_CUH */
