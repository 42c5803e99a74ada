/* Test infrastructure: the reference's own surface reconstruction, compiled for the host.
 *
 * include/mesh_builder.h is compiled unmodified from the reference checkout, with its
 * CLIOptions from include/options.h (and the vendored cxxopts.h) and libigl's marching
 * cubes from the reference's vendored include/igl/copyleft/, against the project-written
 * stand-ins in oracle/ref_shim/ (the Eigen subset with dynamic matrices,
 * boost::multi_array, aborting placeholders for the smoothing and decimation calls, and
 * an in-memory writeOBJ).
 *
 * ref_compute_mesh runs MeshBuilder::computeMesh (include/mesh_builder.h:165-211) itself,
 * with the default flags but the grid side and particle radius (no smoothing, no
 * decimation), and returns the V and F it hands to igl::writeOBJ.
 * ref_distance_field calls the header's
 * fillVoxelGrid_distance (include/mesh_builder.h:89-138) with the arguments
 * MeshBuilder::computeMesh passes (include/mesh_builder.h:167-174):
 *   voxel_dx = params.N * params.dx / double(VoxelGridSide)
 *   distance_cutoff = (flags.mesh_particle_radius + 1) * voxel_dx
 * Built without OpenMP, so the header's parallel particle loop (whose unsynchronised
 * minimum is a data race when it runs threaded) runs sequentially.
 * Built into oracle/_ref by oracle/build.py; used by tests/golden/ref_mesh_vectors.py. */
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

#include "options.h"
#include "mesh_builder.h"

namespace {

struct Point {
  Vec x;
};

}  // namespace

extern "C" {

/* MeshBuilder(params(dt, N), flags, G).computeMesh on n particles; V (nv x 3 doubles)
 * and F (nf x 3 ints, 0-based) as passed to writeOBJ, copied up to the capacities.
 * Returns 0. */
int ref_compute_mesh(const float* x, int64_t n, uint32_t N, uint32_t G, uint32_t radius, double* V, int64_t vcap,
                     int32_t* F, int64_t fcap, int64_t* nv, int64_t* nf) {
  std::vector<Point> particles((size_t)n);
  for (int64_t p = 0; p < n; ++p)
    for (int c = 0; c < 3; ++c) particles[p].x(c) = x[3 * p + c];
  std::string rs = std::to_string(radius), gs = std::to_string(G), ns = std::to_string(N);
  const char* argv[] = {"mpm", "-N", ns.c_str(), "--mesh-grid", gs.c_str(), "--mesh-particle-radius", rs.c_str()};
  CLIOptions flags(7, const_cast<char**>(argv));
  SimulationParameters params(flags.dt, flags.N);
  MeshBuilder builder(params, flags, flags.mesh_grid);
  builder.computeMesh("mesh.obj", particles);
  const igl::WrittenMesh& m = igl::written_mesh();
  *nv = (int64_t)(m.V.size() / 3);
  *nf = (int64_t)(m.F.size() / 3);
  for (int64_t i = 0; i < 3 * std::min(*nv, vcap); ++i) V[i] = m.V[i];
  for (int64_t i = 0; i < 3 * std::min(*nf, fcap); ++i) F[i] = m.F[i];
  return 0;
}

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
