// Shared definitions of the GPU particle seeder (seeding.cu) and its host-side setup.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "mpm_gb300.h"

namespace mpm {

enum SeedKind { kSeedBox = 0, kSeedSphere = 1, kSeedMesh = 2 };

// One object to seed: candidates are uniform in [lo, lo + range); a sphere keeps those
// with squared distance to `center` below r2; a mesh (scaled vertices, triangles and a
// (y, z) bin table of the triangles) keeps those with an odd number of +x ray crossings.
struct SeedShape {
  int kind;
  uint64_t seed;
  uint64_t candidates;
  double lo[3], range[3];
  double center[3], r2;
  const float* verts;
  const int* tris;
  const int* bin_start;  // bins_y * bins_z + 1 offsets into bin_tris
  const int* bin_tris;
  int bins_y, bins_z;
  double bin_y0, bin_z0, bin_inv_dy, bin_inv_dz;
  int winding;  // mesh: 1 = generalized winding number > 1/2 instead of ray parity
  int n_tris;
};

// SplitMix64 (Steele, Lea, Flood, OOPSLA 2014): a bijective 64-bit mix of a counter.
__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Coordinate `axis` of candidate i as a double in [0, 1) with 53 random bits.
__host__ __device__ __forceinline__ double seed_uniform(uint64_t seed, uint64_t i, int axis) {
  return (double)(splitmix64(seed + 3ull * i + (uint64_t)axis) >> 11) * (1.0 / 9007199254740992.0);
}

#ifdef __CUDACC__
// Sign of the edge function (by - ay)(qz - az) - (bz - az)(qy - ay) of float inputs when a
// float evaluation decides it, 0 when it does not.  Each subtraction, product and the final
// difference rounds by at most u = 2^-24 relative, so the float result is within
// 4u (|t1| + |t2|) of the exact value; outside 4e-7 (|t1| + |t2|) the exact value has the
// float result's sign and is far above the double evaluation's error, so the double edge
// function has that sign too.  (Infinities and NaN compare false: undecided.)
__device__ __forceinline__ int orient_sign_f(float ay, float az, float by, float bz, float qy, float qz) {
  const float t1 = __fmul_rn(__fsub_rn(by, ay), __fsub_rn(qz, az));
  const float t2 = __fmul_rn(__fsub_rn(bz, az), __fsub_rn(qy, ay));
  const float o = __fsub_rn(t1, t2);
  const float bound = 4.0e-7f * (fabsf(t1) + fabsf(t2));
  return o > bound ? 1 : (o < -bound ? -1 : 0);
}

// Does the +x ray from (px, py, pz) cross triangle abc?  Its (y, z) projection must
// contain (py, pz) strictly (all three edge functions of one sign; points on an edge are
// a measure-zero set), and the plane's x above (py, pz) must exceed px.  The decision is
// the double evaluation's; a float pre-test (orient_sign_f) rejects, with the same answer,
// the triangles whose edge functions have decided, differing signs, which is nearly all of
// them (FP64 runs at a small fraction of the FP32 rate on this part).
__device__ __forceinline__ bool ray_crosses(const float* a, const float* b, const float* c, float qx, float qy,
                                            float qz) {
  {
    const int s0 = orient_sign_f(b[1], b[2], c[1], c[2], qy, qz);
    const int s1 = orient_sign_f(c[1], c[2], a[1], a[2], qy, qz);
    if (s0 * s1 < 0) return false;
    const int s2 = orient_sign_f(a[1], a[2], b[1], b[2], qy, qz);
    if (s0 * s2 < 0 || s1 * s2 < 0) return false;
  }
  const double px = qx, py = qy, pz = qz;
  auto orient = [](double ay, double az, double by, double bz, double qy, double qz) {
    return __dsub_rn(__dmul_rn(__dsub_rn(by, ay), __dsub_rn(qz, az)), __dmul_rn(__dsub_rn(bz, az), __dsub_rn(qy, ay)));
  };
  const double e0 = orient(b[1], b[2], c[1], c[2], py, pz);
  const double e1 = orient(c[1], c[2], a[1], a[2], py, pz);
  const double e2 = orient(a[1], a[2], b[1], b[2], py, pz);
  const bool pos = e0 > 0.0 && e1 > 0.0 && e2 > 0.0;
  const bool neg = e0 < 0.0 && e1 < 0.0 && e2 < 0.0;
  if (!pos && !neg) return false;
  const double s = __dadd_rn(__dadd_rn(e0, e1), e2);
  const double xs = __dadd_rn(__dadd_rn(__dmul_rn(e0, (double)a[0]), __dmul_rn(e1, (double)b[0])),
                              __dmul_rn(e2, (double)c[0]));
  return __ddiv_rn(xs, s) > px;
}
#endif

// Seeds one shape on the GPU; *x_out (device, 3 floats per particle, candidate order,
// owned by the caller, cudaFree) and *n_out receive the kept particles.
cudaError_t seed_shape_gpu(const SeedShape& sh, cudaStream_t st, float** x_out, int64_t* n_out);

// A SeedShape with the device copies of a mesh it points to.
struct SeedShapeOwner {
  SeedShape sh{};
  float* d_verts = nullptr;
  int* d_tris = nullptr;
  int* d_bin_start = nullptr;
  int* d_bin_tris = nullptr;
  void release();
  ~SeedShapeOwner() { release(); }
};

// The shape of an object at `density` candidates per unit volume (validates the object).
mpm_status build_seed_shape(const mpm_object& o, uint32_t density, SeedShapeOwner& out);

}  // namespace mpm
