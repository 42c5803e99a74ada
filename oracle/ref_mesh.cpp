/* Test infrastructure: the reference's own distance field, compiled for the host.
 *
 * include/mesh_builder.h is compiled unmodified from the reference checkout, with its
 * CLIOptions from include/options.h (and the vendored cxxopts.h), against the
 * project-written stand-ins in oracle/ref_shim/ (the Eigen subset, boost::multi_array,
 * declaration-only libigl).  ref_distance_field calls the header's
 * fillVoxelGrid_distance (include/mesh_builder.h:89-138) with the arguments
 * MeshBuilder::computeMesh passes (include/mesh_builder.h:167-174):
 *   voxel_dx = params.N * params.dx / double(VoxelGridSide)
 *   distance_cutoff = (flags.mesh_particle_radius + 1) * voxel_dx
 * Built without OpenMP, so the header's parallel particle loop (whose unsynchronised
 * minimum is a data race when it runs threaded) runs sequentially.
 * Built into oracle/_ref by oracle/build.py; used by tests/golden/ref_mesh_vectors.py. */
#include <stdint.h>

#include <vector>

#include "options.h"
#include "mesh_builder.h"

namespace {

struct Point {
  Vec x;
};

}  // namespace

extern "C" {

/* voxel_dx of a MeshBuilder of side G for the grid of SimulationParameters(dt, N). */
double ref_voxel_dx(uint32_t N, uint32_t G) {
  SimulationParameters params(1e-4f, N);
  return params.N * params.dx / double(G);
}

/* x: n particles, 3 floats each; field: G^3 floats, index (i G + j) G + k. */
int ref_distance_field(const float* x, int64_t n, uint32_t G, uint32_t radius, double voxel_dx, float* field) {
  std::vector<Point> particles((size_t)n);
  for (int64_t p = 0; p < n; ++p)
    for (int c = 0; c < 3; ++c) particles[p].x(c) = x[3 * p + c];
  boost::multi_array<float, 3> sdf(boost::extents[G][G][G]);
  const u32 mesh_particle_radius = radius;
  fillVoxelGrid_distance(particles, voxel_dx, (mesh_particle_radius + 1) * voxel_dx, sdf);
  const float* d = sdf.data();
  for (int64_t c = 0; c < (int64_t)G * G * G; ++c) field[c] = d[c];
  return 0;
}

}  // extern "C"
