// Material models compiled into a build of the library through the public policy header
// (include/mpm_gb300_policies.cuh) alone, for tests/test_gpu_plugin.py and
// tests/test_plugin_build.py.
//
//   kind 16, PluginJelly: the reference's MMJelly (include/MaterialModel.cuh:119-150):
//     P F^T = 2 mu (F - R) F^T + lambda (Jp - 1) Jp I with mu, lambda scaled by
//     exp(h (1 - Jp)), and its end-of-step Jp update (both determinants taken of the same
//     F, so Jp only clamps to [0.6, 20]);
//   kind 17, PluginStiffJelly: the same with twice the shear modulus, so its results equal
//     those of MMJelly with mu0 doubled and differ from PluginJelly's.
#include "mpm_gb300_policies.cuh"

template <int MU_SCALE>
struct JellyModel {
  __device__ static void computePF(const mpm::DevMaterial& m, const float F[3][3], float Jp, const mpm::PolarCache& pc,
                                   float PF[3][3]) {
    const float e = (m.hardening == 0.f) ? 1.f : expf(m.hardening * (1.f - Jp));
    const float mu = (MU_SCALE * m.mu0) * e, lambda = m.lambda0 * e;
    float R[3][3];
    mpm::polar_rotation(F, pc, R);
    const float lt = lambda * ((Jp - 1.f) * Jp);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        float acc = (i == j) ? lt : 0.f;
        for (int k = 0; k < 3; ++k) acc += 2.f * mu * (F[i][k] - R[i][k]) * F[j][k];
        PF[i][j] = acc;
      }
  }
  __device__ static void endOfStepMutation(const mpm::DevMaterial& m, const mpm::GridConsts& K, const float C[3][3],
                                           float F[3][3], float& Jp, mpm::PolarCache& pc) {
    const float oldJ = mpm::det3_colwise(F);
    Jp = mpm::clampf(Jp * oldJ / mpm::det3_colwise(F), 0.6f, 20.0f);
  }
};

using PluginJelly = JellyModel<1>;
using PluginStiffJelly = JellyModel<2>;

MPM_GB300_REGISTER_MATERIAL(PluginJelly, 16)
MPM_GB300_REGISTER_MATERIAL(PluginStiffJelly, 17)
