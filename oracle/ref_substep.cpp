/* Test infrastructure: the reference's own substep policies, compiled for the host.
 *
 * The reference's policy headers (include/types.h, InterpolationKernel.cuh,
 * TransferScheme.h, MaterialModel.cuh) and src/linalg.cu + include/svd3_cuda.h are
 * compiled unmodified from the reference checkout, against the project-written Eigen
 * subset and CUDA stand-ins in oracle/ref_shim/.  src/mpm.cu itself cannot be compiled
 * (it needs Boost, libigl and GLFW), so the three kernels' loops are restated here as a
 * serial host loop that calls the policies exactly as the kernels do:
 *   particleToGrid  src/mpm.cu:14-74
 *   gridOpKernel    src/mpm.cu:76-107
 *   gridToParticle  src/mpm.cu:109-178
 * with the bindings of include/mpm.cuh:24-27 (MaterialModel = MMSnow).  The only
 * departure: node writes outside the grid are skipped (the reference's P2G upper clip,
 * src/mpm.cu:42-44, would write past the grid; the golden scenes never reach it).
 * Built into oracle/_ref by oracle/build.py; used by tests/golden/ref_substep_vectors.py. */
#include <stdint.h>

#include <vector>

#include <cuda.h>

#include "types.h"
// src/linalg.cu first: its device functions are declared by include/linalg.h only
// under nvcc, and MaterialModel.cuh names them in its templates.
#include "linalg.cu"
#include "InterpolationKernel.cuh"
#include "TransferScheme.h"
#include "MaterialModel.cuh"

using Particle = MLS_APIC_Particle;
using MaterialModel = MMSnow<Particle>;
using InterpolationKernel = QuadraticInterpolationKernel;
using TransferScheme = MLS_APIC_Scheme<InterpolationKernel>;

namespace {

const real kGravity = -9.81;  // src/mpm.cu:6
const int kGridVectorSize = 4;

void particle_to_grid(std::vector<Particle>& particles, std::vector<Vec4>& grid, const std::vector<MaterialModel>& mats,
                      const SimulationParameters& par, const InterpolationKernel& kernel) {
  const int N = (int)par.N;
  for (size_t pi = 0; pi < particles.size(); ++pi) {
    Particle particle = particles[pi];
    MaterialModel material_model = mats[particle.material_type];
    TransferScheme scheme;
    scheme.p2g_prepare_particle(particle, par, kernel, material_model);
    Veci rb = scheme.get_range_begin();
    bool outside = false;
    for (int d = 0; d < 3; ++d)
      if (rb(d) + int(kernel.size()) < 0 || rb(d) >= N) outside = true;
    if (outside) continue;
    Vec dist;
    const int ib = std::max(0, -rb(0)), jb = std::max(0, -rb(1)), kb = std::max(0, -rb(2));
    const int ie = std::min((int)kernel.size(), N + rb(0)), je = std::min((int)kernel.size(), N + rb(1)),
              ke = std::min((int)kernel.size(), N + rb(2));
    for (int i = ib; i < ie; ++i) {
      const int ig = rb[0] + i;
      dist[0] = ig * par.dx - particle.x[0];
      for (int j = jb; j < je; ++j) {
        const int jg = rb[1] + j;
        dist[1] = jg * par.dx - particle.x[1];
        for (int k = kb; k < ke; ++k) {
          const int kg = rb[2] + k;
          dist[2] = kg * par.dx - particle.x[2];
          Vec4 contribution;
          scheme.p2g_node_contribution(particle, dist, material_model.particleMass, i, j, k, contribution);
          if (ig >= N || jg >= N || kg >= N) continue;
          Vec4& cell = grid[(size_t)N * N * ig + (size_t)N * jg + kg];
          for (int c = 0; c < kGridVectorSize; ++c) cell[c] += contribution[c];
        }
      }
    }
  }
}

void grid_op(std::vector<Vec4>& grid, int N, float dt) {
  for (int xi = 0; xi < N; ++xi)
    for (int yi = 0; yi < N; ++yi)
      for (int zi = 0; zi < N; ++zi) {
        Vec4& cell = grid[(size_t)N * (N * xi + yi) + zi];
        if (!(cell[3] > 0.0)) continue;
        for (int w = 0; w < kGridVectorSize; ++w) cell[w] /= cell[3];
        cell[1] += dt * kGravity;
        const real boundary = 0.05;
        const real x = real(xi) / N, y = real(yi) / N, z = real(zi) / N;
        if (x < boundary || x > 1 - boundary || y > 1 - boundary || z < boundary || z > 1 - boundary) {
          cell[0] = 0.0;
          cell[1] = 0.0;
          cell[2] = 0.0;
        }
        if (y < boundary) cell[1] = std::max(real(0.0), cell[1]);
      }
}

void grid_to_particle(std::vector<Particle>& particles, const std::vector<Vec4>& grid,
                      const std::vector<MaterialModel>& mats, const SimulationParameters& par,
                      const InterpolationKernel& kernel) {
  const int N = (int)par.N;
  for (size_t pi = 0; pi < particles.size(); ++pi) {
    if ((int64_t)pi > (int64_t)N * N * N) continue;  // src/mpm.cu:114
    Particle particle = particles[pi];
    const MaterialModel& material_model = mats[particle.material_type];
    TransferScheme scheme;
    scheme.g2p_prepare_particle(particle, par, kernel);
    Veci rb = scheme.get_range_begin();
    bool outside = false;
    for (int d = 0; d < 3; ++d)
      if (rb(d) + int(kernel.size()) < 0 || rb(d) >= N) outside = true;
    if (outside) continue;
    Vec dist;
    const int ib = std::max(0, -rb(0)), jb = std::max(0, -rb(1)), kb = std::max(0, -rb(2));
    const int ie = std::min((int)kernel.size(), N - rb(0)), je = std::min((int)kernel.size(), N - rb(1)),
              ke = std::min((int)kernel.size(), N - rb(2));
    for (int i = ib; i < ie; ++i) {
      const int ig = rb(0) + i;
      dist[0] = ig * par.dx - particle.x(0);
      for (int j = jb; j < je; ++j) {
        const int jg = rb(1) + j;
        dist[1] = jg * par.dx - particle.x(1);
        for (int k = kb; k < ke; ++k) {
          const int kg = rb(2) + k;
          dist[2] = kg * par.dx - particle.x(2);
          const Vec4& cell = grid[(size_t)N * N * ig + (size_t)N * jg + kg];
          scheme.g2p_node_contribution(particle, dist, cell, i, j, k);
        }
      }
    }
    scheme.g2p_finish_particle(particle, par);
    material_model.endOfStepMutation(particle);
    particle.x += par.dt * particle.v;
    particles[pi] = particle;
  }
}

}  // namespace

/* materials: per material 7 floats (volume, density, E, Nu, hardening, lo, hi), the
 * MMSnow constructor arguments.  State in row-major SoA (x[3n], v[3n], C[9n], F[9n],
 * Jp[n], mat[n]), advanced in place.  grid_out (optional): N^3 x 4 after the last P2G. */
extern "C" int ref_substep(int64_t n, float* x, float* v, float* C, float* F, float* Jp, const uint8_t* mat,
                           const float* materials, int nmat, float dt, int N, int nsteps, float* grid_out) {
  std::vector<MaterialModel> mats;
  for (int i = 0; i < nmat; ++i) {
    const float* m = materials + 7 * i;
    mats.push_back(MaterialModel(m[0], m[1], m[2], m[3], m[4], m[5], m[6]));
  }
  SimulationParameters par(dt, (u32)N);
  InterpolationKernel kernel;
  std::vector<Particle> ps(n);
  for (int64_t p = 0; p < n; ++p) {
    Vec xp, vp;
    for (int d = 0; d < 3; ++d) {
      xp(d) = x[3 * p + d];
      vp(d) = v[3 * p + d];
    }
    ps[p] = Particle(mat[p], xp, vp);
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        ps[p].F(r, c) = F[9 * p + 3 * r + c];
        ps[p].C(r, c) = C[9 * p + 3 * r + c];
      }
    ps[p].Jp = Jp[p];
  }
  std::vector<Vec4> grid((size_t)N * N * N);
  for (int s = 0; s < nsteps; ++s) {
    for (auto& g : grid) g = Vec4::Zero();  // Simulation::resetGrid
    particle_to_grid(ps, grid, mats, par, kernel);
    if (grid_out && s == nsteps - 1)
      for (size_t c = 0; c < grid.size(); ++c)
        for (int q = 0; q < 4; ++q) grid_out[4 * c + q] = grid[c][q];
    grid_op(grid, N, dt);
    grid_to_particle(ps, grid, mats, par, kernel);
  }
  for (int64_t p = 0; p < n; ++p) {
    for (int d = 0; d < 3; ++d) {
      x[3 * p + d] = ps[p].x(d);
      v[3 * p + d] = ps[p].v(d);
    }
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        F[9 * p + 3 * r + c] = ps[p].F(r, c);
        C[9 * p + 3 * r + c] = ps[p].C(r, c);
      }
    Jp[p] = ps[p].Jp;
  }
  return 0;
}
