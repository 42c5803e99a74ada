/* C++ facade of the mpm_gb300 C ABI with the method names of the reference's host class
 * Simulation (include/mpm.cuh:44-106), so a caller of the reference keeps its code shape:
 *
 *   mpm_gb300::Simulation sim(params, materials);        // Simulation(flags, kernel, models)
 *   sim.addObject(object);                               // Simulation::addObject
 *   sim.initCuda(particles);                             // or upload the reference's AoS records
 *   for (...) sim.advance();                             // Simulation::advance
 *   auto& ps = sim.syncDevice();                         // Simulation::syncDevice + particle list
 *
 * Header only; link against libmpm_gb300.so.  Errors throw mpm_gb300::Error with the
 * library's message (the reference exits or does not check).  Particle records are the
 * reference's 104-byte MLS_APIC_Particle layout (u8 material, 3 pad bytes, x, v, F, C
 * column-major, Jp), which mpm_upload_aos / mpm_download_aos read and write.
 */
#pragma once

#include <cstdint>
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

}  // namespace mpm_gb300
