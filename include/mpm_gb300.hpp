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
#include <unordered_map>
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
 * 170-211): the surface of the simulation's particles on a grid_side^3 voxel grid with the
 * given particle radius (in voxels), written as an OBJ file.  Vertices shared by triangles
 * are welded (they are bit-identical); triangles collapsed where the surface passes through
 * a voxel node are dropped. */
class MeshBuilder {
 public:
  explicit MeshBuilder(int32_t grid_side = 250, int32_t particle_radius = 5)
      : grid_side_(grid_side), radius_(particle_radius) {}

  /* The triangle soup, 9 floats per triangle (cell order). */
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

  /* Writes the OBJ file; returns the number of faces. */
  size_t computeMesh(const std::string& filename, Simulation& sim) const {
    const std::vector<float> t = triangles(sim);
    struct Key {
      uint32_t b[3];
      bool operator==(const Key& o) const { return b[0] == o.b[0] && b[1] == o.b[1] && b[2] == o.b[2]; }
    };
    struct Hash {
      size_t operator()(const Key& k) const {
        return ((size_t)k.b[0] * 73856093u) ^ ((size_t)k.b[1] * 19349663u) ^ ((size_t)k.b[2] * 83492791u);
      }
    };
    std::unordered_map<Key, uint32_t, Hash> index;
    std::vector<float> verts;
    std::vector<uint32_t> faces;
    for (size_t q = 0; q < t.size() / 9; ++q) {
      uint32_t f[3];
      for (int c = 0; c < 3; ++c) {
        Key k;
        std::memcpy(k.b, &t[9 * q + 3 * c], 12);
        auto it = index.find(k);
        if (it == index.end()) {
          it = index.emplace(k, (uint32_t)(verts.size() / 3)).first;
          verts.insert(verts.end(), &t[9 * q + 3 * c], &t[9 * q + 3 * c] + 3);
        }
        f[c] = it->second;
      }
      if (f[0] != f[1] && f[1] != f[2] && f[0] != f[2]) faces.insert(faces.end(), f, f + 3);
    }
    FILE* out = std::fopen(filename.c_str(), "w");
    if (!out) throw Error(MPM_ERR_IO, "cannot write " + filename);
    for (size_t v = 0; v < verts.size() / 3; ++v)
      std::fprintf(out, "v %.9g %.9g %.9g\n", verts[3 * v], verts[3 * v + 1], verts[3 * v + 2]);
    for (size_t q = 0; q < faces.size() / 3; ++q)
      std::fprintf(out, "f %u %u %u\n", faces[3 * q] + 1, faces[3 * q + 1] + 1, faces[3 * q + 2] + 1);
    if (std::fclose(out) != 0) throw Error(MPM_ERR_IO, "cannot write " + filename);
    return faces.size() / 3;
  }

 private:
  static void status(Simulation& sim, mpm_status st) {
    if (st == MPM_OK) return;
    char msg[512] = {0};
    mpm_last_error(sim.handle(), msg, sizeof(msg));
    throw Error(st, std::string("surface: ") + msg);
  }
  int32_t grid_side_, radius_;
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
