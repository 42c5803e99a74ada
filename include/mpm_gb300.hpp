/* C++ facade of the mpm_gb300 C ABI with the method names of the reference's host class
 * Simulation (include/mpm.cuh:44-106), so a caller of the reference keeps its code shape:
 *
 *   mpm_gb300::Simulation sim(params, materials);        // Simulation(flags, kernel, models)
 *   sim.addObject(object);                               // Simulation::addObject
 *   sim.initCuda(particles);                             // or upload the reference's AoS records
 *   for (...) sim.advance();                             // Simulation::advance
 *   auto& ps = sim.syncDevice();                         // Simulation::syncDevice + particle list
 *
 * and the frame-output classes of the reference's main loop (src/main.cu:72-111), which here
 * read the particles on the GPU instead of a host particle list:
 *
 *   mpm_gb300::MeshBuilder(250, 5).computeMesh("mesh_00000.obj", sim);   // include/mesh_builder.h
 *   mpm_gb300::ParticleWriter().writeParticles("particles_0.bgeo", sim);  // include/particle_writer.h
 *   mpm_gb300::Renderer r; r.render(sim); r.writePPM("frame.ppm");       // include/renderer.h
 *
 * Header only; link against libmpm_gb300.so.  Errors throw mpm_gb300::Error with the
 * library's message (the reference exits or does not check).  Particle records are the
 * reference's 104-byte MLS_APIC_Particle layout (u8 material, 3 pad bytes, x, v, F, C
 * column-major, Jp), which mpm_upload_aos / mpm_download_aos read and write.
 */
#pragma once

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "mpm_gb300.h"

namespace mpm_gb300 {

class Error : public std::runtime_error {
 public:
  Error(mpm_status code, const std::string& what) : std::runtime_error(what), code_(code) {}
  mpm_status code() const { return code_; }

 private:
  mpm_status code_;
};

/* One particle in the reference's layout (include/TransferScheme.h:46-54 with Eigen's
 * column-major 3x3 matrices). */
struct Particle {
  uint8_t material_type;
  uint8_t pad[3];
  float x[3];
  float v[3];
  float F[9];  // column-major
  float C[9];  // column-major
  float Jp;
};
static_assert(sizeof(Particle) == 104, "reference particle record is 104 bytes");

class Simulation {
 public:
  Simulation(const mpm_params& params, const std::vector<mpm_material>& materials) {
    check(mpm_create(&params, &ctx_), "mpm_create");
    check(mpm_set_materials(ctx_, materials.data(), (int32_t)materials.size()), "mpm_set_materials");
  }
  ~Simulation() {
    if (ctx_) mpm_destroy(ctx_);
  }
  Simulation(const Simulation&) = delete;
  Simulation& operator=(const Simulation&) = delete;

  /* Simulation::addObject: seed the object on the GPU; returns its particle count. */
  int64_t addObject(const mpm_object& object) {
    int64_t n = 0;
    check(mpm_add_object(ctx_, &object, &n), "mpm_add_object");
    return n;
  }

  /* Simulation::initCuda / particlesToDevice: upload the reference's particle records. */
  void initCuda(const std::vector<Particle>& particles) {
    check(mpm_upload_aos(ctx_, particles.data(), (int64_t)particles.size()), "mpm_upload_aos");
  }

  /* Simulation::advance: one substep (asynchronous). */
  void advance(int32_t substeps = 1) { check(mpm_substep(ctx_, substeps), "mpm_substep"); }

  /* Simulation::syncDevice + getActiveParticleList: blocking readback of all particles. */
  std::vector<Particle>& syncDevice() {
    check(mpm_sync(ctx_), "mpm_sync");
    particles_.resize((size_t)getFullParticleCount());
    if (!particles_.empty()) check(mpm_download_aos(ctx_, particles_.data()), "mpm_download_aos");
    return particles_;
  }

  int64_t getFullParticleCount() const { return mpm_particle_count(ctx_); }
  double t() const { return mpm_time(ctx_); }
  mpm_ctx* handle() const { return ctx_; }

 private:
  void check(mpm_status st, const char* call) const {
    if (st == MPM_OK) return;
    char msg[512] = {0};
    if (ctx_) mpm_last_error(ctx_, msg, sizeof(msg));
    throw Error(st, std::string(call) + " failed (status " + std::to_string((int)st) + "): " + msg);
  }

  mpm_ctx* ctx_ = nullptr;
  std::vector<Particle> particles_;
};

/* MeshBuilder(params, flags, grid_size) / computeMesh (include/mesh_builder.h:19-34,
 * 165-211): the surface of the simulation's particles on a grid_side^3 voxel grid with the
 * given particle radius (in voxels), written as an OBJ file: libigl's marching-cubes
 * vertex list (bit for bit, in its order) and outward faces over the same edge loops.
 * laplacian_smooth (the reference's --laplacian_smooth) smooths the vertices as
 * MeshBuilder::smoothMesh does (mpm_surface_smooth). */
class MeshBuilder {
 public:
  explicit MeshBuilder(int32_t grid_side = 250, int32_t particle_radius = 5, bool laplacian_smooth = false)
      : grid_side_(grid_side), radius_(particle_radius), smooth_(laplacian_smooth) {}

  /* The triangle soup, 9 floats per triangle (the faces of mesh(), in order). */
  std::vector<float> triangles(Simulation& sim) const {
    int64_t n = 0;
    std::vector<float> t(9 * 65536);
    status(sim, mpm_surface_mesh(sim.handle(), grid_side_, radius_, t.data(), 65536, &n));
    if (n > 65536) {
      t.resize(9 * (size_t)n);
      status(sim, mpm_surface_mesh(sim.handle(), grid_side_, radius_, t.data(), n, &n));
    }
    t.resize(9 * (size_t)n);
    return t;
  }

  /* The indexed mesh: 3 doubles per vertex, 3 zero-based vertex indices per face. */
  void mesh(Simulation& sim, std::vector<double>& V, std::vector<int32_t>& F) const {
    int64_t nv = 0, nf = 0;
    V.resize(3 * 65536);
    F.resize(3 * 65536);
    status(sim, mpm_surface_mesh_indexed(sim.handle(), grid_side_, radius_, V.data(), 65536, F.data(), 65536, &nv,
                                         &nf));
    if (nv > 65536 || nf > 65536) {
      V.resize(3 * (size_t)nv);
      F.resize(3 * (size_t)nf);
      status(sim, mpm_surface_mesh_indexed(sim.handle(), grid_side_, radius_, V.data(), nv, F.data(), nf, &nv, &nf));
    }
    V.resize(3 * (size_t)nv);
    F.resize(3 * (size_t)nf);
    /* --laplacian_smooth: MeshBuilder::smoothMesh (include/mesh_builder.h:212-245) */
    if (smooth_ && nf > 0) status(sim, mpm_surface_smooth(sim.handle(), V.data(), nv, F.data(), nf, nullptr));
  }

  /* Writes the OBJ file (igl::writeOBJ's v / f lines); returns the number of faces. */
  size_t computeMesh(const std::string& filename, Simulation& sim) const {
    std::vector<double> V;
    std::vector<int32_t> F;
    mesh(sim, V, F);
    FILE* out = std::fopen(filename.c_str(), "w");
    if (!out) throw Error(MPM_ERR_IO, "cannot write " + filename);
    for (size_t v = 0; v < V.size() / 3; ++v) std::fprintf(out, "v %.17g %.17g %.17g\n", V[3 * v], V[3 * v + 1], V[3 * v + 2]);
    for (size_t q = 0; q < F.size() / 3; ++q) std::fprintf(out, "f %d %d %d\n", F[3 * q] + 1, F[3 * q + 1] + 1, F[3 * q + 2] + 1);
    if (std::fclose(out) != 0) throw Error(MPM_ERR_IO, "cannot write " + filename);
    return F.size() / 3;
  }

 private:
  static void status(Simulation& sim, mpm_status st) {
    if (st == MPM_OK) return;
    char msg[512] = {0};
    mpm_last_error(sim.handle(), msg, sizeof(msg));
    throw Error(st, std::string("surface: ") + msg);
  }
  int32_t grid_side_, radius_;
  bool smooth_;
};

/* ParticleWriter::writeParticles (include/particle_writer.h:19-43): the active particles
 * as a .bgeo file with the reference's attributes (id, position, velocity, radius 0.1),
 * packed on the GPU. */
class ParticleWriter {
 public:
  void writeParticles(const std::string& filepath, Simulation& sim, float radius = 0.1f) const {
    int64_t n = 0;
    const void* rec = nullptr;
    check(sim, mpm_export_particles(sim.handle(), 0, radius, &n));
    check(sim, mpm_export_wait(sim.handle(), 0, &rec, &n));
    const mpm_status st = mpm_write_bgeo(filepath.c_str(), rec, n);
    if (st != MPM_OK) throw Error(st, "cannot write " + filepath);
  }

 private:
  static void check(Simulation& sim, mpm_status st) {
    if (st == MPM_OK) return;
    char msg[512] = {0};
    mpm_last_error(sim.handle(), msg, sizeof(msg));
    throw Error(st, std::string("export: ") + msg);
  }
};

/* Renderer::render (include/renderer.h:43-63) without a window: the particles as 2-pixel
 * points of the reference's colour on its 800 x 600 frame, into an RGB8 image (rows top to
 * bottom) that writePPM saves. */
class Renderer {
 public:
  Renderer(int32_t width = 800, int32_t height = 600) : w_(width), h_(height), rgb_(3 * (size_t)width * height) {}

  const std::vector<uint8_t>& render(Simulation& sim) {
    const uint8_t color[3] = {150, 138, 51}, background[3] = {26, 26, 26};  // 0.59 0.54 0.2 / 0.1 as unorm8
    const mpm_status st = mpm_render_points(sim.handle(), w_, h_, 2.0f, color, background, rgb_.data());
    if (st != MPM_OK) {
      char msg[512] = {0};
      mpm_last_error(sim.handle(), msg, sizeof(msg));
      throw Error(st, std::string("render: ") + msg);
    }
    return rgb_;
  }

  void writePPM(const std::string& filename) const {
    FILE* out = std::fopen(filename.c_str(), "wb");
    if (!out) throw Error(MPM_ERR_IO, "cannot write " + filename);
    std::fprintf(out, "P6 %d %d 255\n", w_, h_);
    const bool ok = std::fwrite(rgb_.data(), 1, rgb_.size(), out) == rgb_.size();
    if (std::fclose(out) != 0 || !ok) throw Error(MPM_ERR_IO, "cannot write " + filename);
  }

 private:
  int32_t w_, h_;
  std::vector<uint8_t> rgb_;
};

}  // namespace mpm_gb300
