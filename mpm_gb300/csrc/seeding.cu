// Particle seeding of scene objects on the GPU.
//
// The reference seeds an object on the host (Simulation::addParticles,
// src/mpm.cu:346-394): candidates = u32(density x bounding-box volume) points uniform in
// the bounding box of the scaled mesh (Simulation::loadMesh, src/mpm.cu:330-344), each
// kept when libigl's winding number says it is inside.  Here the same rejection sampler
// runs as two GPU passes over the candidates (count, exclusive scan over blocks, write),
// so the kept particles come out in candidate order; the count pass keeps one bit per
// candidate, and the write pass regenerates only the kept candidates.  Candidate i's coordinates come from
// SplitMix64 (Steele, Lea and Flood, "Fast splittable pseudorandom number generators",
// OOPSLA 2014) of seed + 3 i + axis, so seeding is reproducible on any device and on the
// host.  Inside tests: boxes keep every candidate, spheres compare the squared distance
// to the centre, closed triangle meshes count ray crossings along +x (odd = inside) with
// triangles binned by their (y, z) bounding boxes.  All arithmetic is IEEE double with
// explicit rounding intrinsics, so the host restatement in the oracle agrees bit for bit.
#include <algorithm>
#include <cmath>
#include <vector>

#include "mpm_internal.h"
#include "seeding.h"

namespace mpm {

namespace {

constexpr int kSeedThreads = 256;
constexpr int kSeedPerThread = 8;
constexpr int64_t kSeedPerBlock = (int64_t)kSeedThreads * kSeedPerThread;

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

__device__ __forceinline__ void candidate(const SeedShape& sh, uint64_t i, float p[3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double u = seed_uniform(sh.seed, i, c);
    p[c] = (float)dadd(sh.lo[c], dmul(u, sh.range[c]));
  }
}

__device__ bool inside_mesh(const SeedShape& sh, const float p[3]) {
  const double py = p[1], pz = p[2];
  // the point's bin, clamped like the triangles' bin ranges
  const int by = min(max((int)floor(dmul(dsub(py, sh.bin_y0), sh.bin_inv_dy)), 0), sh.bins_y - 1);
  const int bz = min(max((int)floor(dmul(dsub(pz, sh.bin_z0), sh.bin_inv_dz)), 0), sh.bins_z - 1);
  const int bin = by * sh.bins_z + bz;
  int crossings = 0;
  for (int q = sh.bin_start[bin]; q < sh.bin_start[bin + 1]; ++q) {
    const int t = sh.bin_tris[q];
    const float* a = sh.verts + 3 * sh.tris[3 * t + 0];
    const float* b = sh.verts + 3 * sh.tris[3 * t + 1];
    const float* c = sh.verts + 3 * sh.tris[3 * t + 2];
    if (ray_crosses(a, b, c, p[0], p[1], p[2])) ++crossings;
  }
  return (crossings & 1) != 0;
}

// The generalized winding number of the mesh at p (Jacobson, Kavan, Sorkine-Hornung,
// "Robust inside-outside segmentation using generalized winding numbers", SIGGRAPH 2013):
// the sum over triangles of their signed solid angles over 4 pi, each
// atan2(det, |a||b||c| + (b.c)|a| + (c.a)|b| + (a.b)|c|) / (2 pi) with a, b, c the corners
// relative to p, in the order of libigl's solid_angle (include/igl/solid_angle.cpp of the
// reference's vendored libigl), the reference's inside test.  FP64.
__device__ double winding_number_d(const SeedShape& sh, const float p[3]) {
  const double inv2pi = 0.15915494309189535;
  double w = 0.0;
  for (int t = 0; t < sh.n_tris; ++t) {
    const float* A = sh.verts + 3 * sh.tris[3 * t + 0];
    const float* B = sh.verts + 3 * sh.tris[3 * t + 1];
    const float* C = sh.verts + 3 * sh.tris[3 * t + 2];
    double v[3][3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      v[0][d] = (double)A[d] - (double)p[d];
      v[1][d] = (double)B[d] - (double)p[d];
      v[2][d] = (double)C[d] - (double)p[d];
    }
    const double la = sqrt(v[0][0] * v[0][0] + v[0][1] * v[0][1] + v[0][2] * v[0][2]);
    const double lb = sqrt(v[1][0] * v[1][0] + v[1][1] * v[1][1] + v[1][2] * v[1][2]);
    const double lc = sqrt(v[2][0] * v[2][0] + v[2][1] * v[2][1] + v[2][2] * v[2][2]);
    const double det = v[0][0] * v[1][1] * v[2][2] + v[1][0] * v[2][1] * v[0][2] + v[2][0] * v[0][1] * v[1][2] -
                       v[2][0] * v[1][1] * v[0][2] - v[1][0] * v[0][1] * v[2][2] - v[0][0] * v[2][1] * v[1][2];
    const double d0 = v[1][0] * v[2][0] + v[1][1] * v[2][1] + v[1][2] * v[2][2];
    const double d1 = v[2][0] * v[0][0] + v[2][1] * v[0][1] + v[2][2] * v[0][2];
    const double d2 = v[0][0] * v[1][0] + v[0][1] * v[1][1] + v[0][2] * v[1][2];
    w += atan2(det, la * lb * lc + d0 * la + d1 * lb + d2 * lc) * inv2pi;
  }
  return w;
}

// Inside test by the winding number: w > 1/2.  The sum is first taken in FP32 with a
// bound on its rounding error (per triangle: the float corner vectors, determinant and
// denominator are within 24 u |a||b||c| of exact, u = 2^-24, which moves atan2 by at most
// (|den| e + |det| e) / (det^2 + den^2); plus atan2f's and the summation's own error).  A
// point whose FP32 sum is farther from 1/2 than twice the bound is decided by it; the rest
// (points at the surface, or in the mouth of an open mesh's hole) take the FP64 sum, so the
// decision is the FP64 one.
__device__ bool inside_winding(const SeedShape& sh, const float p[3]) {
  const float u = 5.9604645e-8f;
  float w = 0.f, bound = 0.f;
  for (int t = 0; t < sh.n_tris; ++t) {
    const float* A = sh.verts + 3 * sh.tris[3 * t + 0];
    const float* B = sh.verts + 3 * sh.tris[3 * t + 1];
    const float* C = sh.verts + 3 * sh.tris[3 * t + 2];
    float v[3][3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      v[0][d] = A[d] - p[d];
      v[1][d] = B[d] - p[d];
      v[2][d] = C[d] - p[d];
    }
    const float la = sqrtf(v[0][0] * v[0][0] + v[0][1] * v[0][1] + v[0][2] * v[0][2]);
    const float lb = sqrtf(v[1][0] * v[1][0] + v[1][1] * v[1][1] + v[1][2] * v[1][2]);
    const float lc = sqrtf(v[2][0] * v[2][0] + v[2][1] * v[2][1] + v[2][2] * v[2][2]);
    const float det = v[0][0] * v[1][1] * v[2][2] + v[1][0] * v[2][1] * v[0][2] + v[2][0] * v[0][1] * v[1][2] -
                      v[2][0] * v[1][1] * v[0][2] - v[1][0] * v[0][1] * v[2][2] - v[0][0] * v[2][1] * v[1][2];
    const float d0 = v[1][0] * v[2][0] + v[1][1] * v[2][1] + v[1][2] * v[2][2];
    const float d1 = v[2][0] * v[0][0] + v[2][1] * v[0][1] + v[2][2] * v[0][2];
    const float d2 = v[0][0] * v[1][0] + v[0][1] * v[1][1] + v[0][2] * v[1][2];
    const float lll = la * lb * lc;
    const float den = lll + d0 * la + d1 * lb + d2 * lc;
    w += atan2f(det, den) * 0.15915494f;
    const float e = 24.f * u * lll;
    const float r2 = det * det + den * den;
    // atan2f: within a few ulps of its result (at most pi; 8 ulps allowed); the sum rounds
    // once per term
    bound += ((fabsf(den) + fabsf(det)) * e / r2 + 8.f * u * 3.1415927f) * 0.15915494f + u * fabsf(w);
  }
  if (fabsf(w - 0.5f) > 2.f * bound + 1e-6f) return w > 0.5f;  // also false for NaN bounds: FP64
  return winding_number_d(sh, p) > 0.5;
}

__device__ __forceinline__ bool inside(const SeedShape& sh, const float p[3]) {
  if (sh.kind == kSeedBox) return true;
  if (sh.kind == kSeedSphere) {
    const double dx = dsub((double)p[0], sh.center[0]);
    const double dy = dsub((double)p[1], sh.center[1]);
    const double dz = dsub((double)p[2], sh.center[2]);
    return dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz)) < sh.r2;
  }
  return sh.winding ? inside_winding(sh, p) : inside_mesh(sh, p);
}

// Pass 1: kept candidates per block, and per thread the mask of its kept candidates (the
// write pass reads it instead of testing again; the mesh test dominates seeding).
__global__ void __launch_bounds__(kSeedThreads) seed_count_kernel(SeedShape sh, int* block_counts,
                                                                  uint8_t* masks) {
  __shared__ int warp_sum[kSeedThreads / 32];
  const uint64_t base = (uint64_t)blockIdx.x * kSeedPerBlock + (uint64_t)threadIdx.x * kSeedPerThread;
  unsigned mask = 0;
  for (int j = 0; j < kSeedPerThread; ++j) {
    const uint64_t i = base + j;
    if (i >= sh.candidates) break;
    float p[3];
    candidate(sh, i, p);
    if (inside(sh, p)) mask |= 1u << j;
  }
  masks[(uint64_t)blockIdx.x * kSeedThreads + threadIdx.x] = (uint8_t)mask;
  int kept = __popc(mask);
#pragma unroll
  for (int o = 16; o; o >>= 1) kept += __shfl_xor_sync(kFull, kept, o);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = kept;
  __syncthreads();
  if (threadIdx.x == 0) {
    int tot = 0;
    for (int w = 0; w < kSeedThreads / 32; ++w) tot += warp_sum[w];
    block_counts[blockIdx.x] = tot;
  }
}

// Pass 2: write kept candidates in candidate order (block offsets from the scan).
__global__ void __launch_bounds__(kSeedThreads) seed_write_kernel(SeedShape sh, const int* block_offsets,
                                                                  const uint8_t* masks, float* x) {
  __shared__ int warp_sum[kSeedThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t base = (uint64_t)blockIdx.x * kSeedPerBlock + (uint64_t)threadIdx.x * kSeedPerThread;
  const unsigned mask = masks[(uint64_t)blockIdx.x * kSeedThreads + threadIdx.x];
  const int kept = __popc(mask);
  int inc = kept;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_sum[warp] = inc;
  __syncthreads();
  int wpre = 0;
  for (int w = 0; w < warp; ++w) wpre += warp_sum[w];
  int64_t out = (int64_t)block_offsets[blockIdx.x] + wpre + inc - kept;
  for (int j = 0; j < kSeedPerThread; ++j) {
    if (!(mask & (1u << j))) continue;
    float p[3];
    candidate(sh, base + j, p);
    x[3 * out + 0] = p[0];
    x[3 * out + 1] = p[1];
    x[3 * out + 2] = p[2];
    ++out;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side: the shape of an mpm_object, scaled and placed as Simulation::loadMesh does
// (src/mpm.cu:330-344: scale = size / longest bounding-box edge, lowest corner at
// `position`), and the candidate count of Simulation::addParticles (src/mpm.cu:369-371).
// ---------------------------------------------------------------------------

void SeedShapeOwner::release() {
  cudaFree(d_verts);
  cudaFree(d_tris);
  cudaFree(d_bin_start);
  cudaFree(d_bin_tris);
  d_verts = nullptr;
  d_tris = nullptr;
  d_bin_start = nullptr;
  d_bin_tris = nullptr;
}

mpm_status build_seed_shape(const mpm_object& o, uint32_t density, SeedShapeOwner& out) {
  out.release();
  SeedShape& sh = out.sh;
  sh = SeedShape{};
  sh.seed = o.seed;
  if (!(o.size > 0.f) || !std::isfinite(o.size)) return MPM_ERR_INVALID;
  if (o.inside_test != MPM_INSIDE_RAY_PARITY && o.inside_test != MPM_INSIDE_WINDING) return MPM_ERR_INVALID;
  for (int c = 0; c < 3; ++c)
    if (!std::isfinite(o.position[c])) return MPM_ERR_INVALID;
  if (o.shape == MPM_SHAPE_BOX) {
    float emax = 0.f;
    for (int c = 0; c < 3; ++c) {
      if (!(o.box_extent[c] > 0.f)) return MPM_ERR_INVALID;
      emax = std::max(emax, o.box_extent[c]);
    }
    const float scale = o.size / emax;
    sh.kind = kSeedBox;
    for (int c = 0; c < 3; ++c) {
      sh.lo[c] = o.position[c];
      sh.range[c] = (double)(o.box_extent[c] * scale);
    }
  } else if (o.shape == MPM_SHAPE_SPHERE) {
    sh.kind = kSeedSphere;
    const double r = 0.5 * (double)o.size;
    for (int c = 0; c < 3; ++c) {
      sh.lo[c] = o.position[c];
      sh.range[c] = o.size;
      sh.center[c] = sh.lo[c] + r;
    }
    sh.r2 = r * r;
  } else if (o.shape == MPM_SHAPE_MESH) {
    if (!o.vertices || !o.triangles || o.n_vertices < 3 || o.n_triangles < 1 || o.n_triangles > (1 << 26))
      return MPM_ERR_INVALID;
    for (int64_t t = 0; t < 3 * o.n_triangles; ++t)
      if (o.triangles[t] < 0 || o.triangles[t] >= o.n_vertices) return MPM_ERR_INVALID;
    float vmin[3], vmax[3];
    for (int c = 0; c < 3; ++c) vmin[c] = vmax[c] = o.vertices[c];
    for (int64_t v = 0; v < o.n_vertices; ++v)
      for (int c = 0; c < 3; ++c) {
        const float x = o.vertices[3 * v + c];
        if (!std::isfinite(x)) return MPM_ERR_INVALID;
        vmin[c] = std::min(vmin[c], x);
        vmax[c] = std::max(vmax[c], x);
      }
    float length_max = 0.f;
    for (int c = 0; c < 3; ++c) length_max = std::max(length_max, vmax[c] - vmin[c]);
    if (!(length_max > 0.f)) return MPM_ERR_INVALID;
    const float scale = o.size / length_max;
    std::vector<float> V(3 * o.n_vertices);
    for (int64_t v = 0; v < o.n_vertices; ++v)
      for (int c = 0; c < 3; ++c) V[3 * v + c] = o.vertices[3 * v + c] * scale + (o.position[c] - scale * vmin[c]);
    float lo[3], hi[3];
    for (int c = 0; c < 3; ++c) lo[c] = hi[c] = V[c];
    for (int64_t v = 0; v < o.n_vertices; ++v)
      for (int c = 0; c < 3; ++c) {
        lo[c] = std::min(lo[c], V[3 * v + c]);
        hi[c] = std::max(hi[c], V[3 * v + c]);
      }
    sh.kind = kSeedMesh;
    sh.winding = o.inside_test == MPM_INSIDE_WINDING ? 1 : 0;
    sh.n_tris = (int)o.n_triangles;
    for (int c = 0; c < 3; ++c) {
      sh.lo[c] = lo[c];
      sh.range[c] = (double)hi[c] - (double)lo[c];
    }
    // (y, z) bins of the triangles' projected bounding boxes
    const int nb = (int)std::min<int64_t>(256, std::max<int64_t>(1, (int64_t)std::sqrt((double)o.n_triangles)));
    sh.bins_y = sh.bins_z = nb;
    sh.bin_y0 = sh.lo[1];
    sh.bin_z0 = sh.lo[2];
    sh.bin_inv_dy = sh.range[1] > 0.0 ? nb / sh.range[1] : 0.0;
    sh.bin_inv_dz = sh.range[2] > 0.0 ? nb / sh.range[2] : 0.0;
    auto bin_of = [&](double v, double v0, double inv) {
      const int b = (int)std::floor((v - v0) * inv);
      return std::min(std::max(b, 0), nb - 1);
    };
    std::vector<std::vector<int>> bins((size_t)nb * nb);
    for (int64_t t = 0; t < o.n_triangles; ++t) {
      double ylo = 1e300, yhi = -1e300, zlo = 1e300, zhi = -1e300;
      for (int k = 0; k < 3; ++k) {
        const float* p = &V[3 * o.triangles[3 * t + k]];
        ylo = std::min(ylo, (double)p[1]);
        yhi = std::max(yhi, (double)p[1]);
        zlo = std::min(zlo, (double)p[2]);
        zhi = std::max(zhi, (double)p[2]);
      }
      const int y0 = bin_of(ylo, sh.bin_y0, sh.bin_inv_dy), y1 = bin_of(yhi, sh.bin_y0, sh.bin_inv_dy);
      const int z0 = bin_of(zlo, sh.bin_z0, sh.bin_inv_dz), z1 = bin_of(zhi, sh.bin_z0, sh.bin_inv_dz);
      for (int by = y0; by <= y1; ++by)
        for (int bz = z0; bz <= z1; ++bz) bins[(size_t)by * nb + bz].push_back((int)t);
    }
    std::vector<int> start(bins.size() + 1, 0), flat;
    for (size_t b = 0; b < bins.size(); ++b) {
      start[b + 1] = start[b] + (int)bins[b].size();
      flat.insert(flat.end(), bins[b].begin(), bins[b].end());
    }
    std::vector<int> tris(o.triangles, o.triangles + 3 * o.n_triangles);
    if (cudaMalloc(&out.d_verts, sizeof(float) * V.size()) || cudaMalloc(&out.d_tris, sizeof(int) * tris.size()) ||
        cudaMalloc(&out.d_bin_start, sizeof(int) * start.size()) ||
        cudaMalloc(&out.d_bin_tris, sizeof(int) * std::max<size_t>(flat.size(), 1)) ||
        cudaMemcpy(out.d_verts, V.data(), sizeof(float) * V.size(), cudaMemcpyHostToDevice) ||
        cudaMemcpy(out.d_tris, tris.data(), sizeof(int) * tris.size(), cudaMemcpyHostToDevice) ||
        cudaMemcpy(out.d_bin_start, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice) ||
        (!flat.empty() && cudaMemcpy(out.d_bin_tris, flat.data(), sizeof(int) * flat.size(), cudaMemcpyHostToDevice))) {
      out.release();
      return MPM_ERR_CUDA;
    }
    sh.verts = out.d_verts;
    sh.tris = out.d_tris;
    sh.bin_start = out.d_bin_start;
    sh.bin_tris = out.d_bin_tris;
  } else {
    return MPM_ERR_INVALID;
  }
  // u32 particle_count_target = particle_density * volume_bounding_box (truncation)
  const double vol = sh.range[0] * sh.range[1] * sh.range[2];
  const double cand = (double)density * vol;
  if (!(cand >= 0.0) || cand > 4294967295.0) {
    out.release();
    return MPM_ERR_UNSUPPORTED;
  }
  sh.candidates = (uint64_t)cand;
  return MPM_OK;
}

cudaError_t seed_shape_gpu(const SeedShape& sh, cudaStream_t st, float** x_out, int64_t* n_out) {
  *x_out = nullptr;
  *n_out = 0;
  if (sh.candidates == 0) return cudaSuccess;
  const int64_t nblocks = (int64_t)((sh.candidates + kSeedPerBlock - 1) / kSeedPerBlock);
  if (nblocks > (int64_t)INT32_MAX) return cudaErrorInvalidValue;
  int* counts = nullptr;
  int* scratch = nullptr;
  uint8_t* masks = nullptr;
  cudaError_t e = cudaMalloc(&counts, sizeof(int) * (nblocks + 1));
  if (e == cudaSuccess) e = cudaMalloc(&scratch, sizeof(int) * scan_scratch_ints(nblocks + 1));
  if (e == cudaSuccess) e = cudaMalloc(&masks, (size_t)nblocks * kSeedThreads);
  if (e == cudaSuccess) e = cudaMemsetAsync(counts, 0, sizeof(int) * (nblocks + 1), st);
  if (e == cudaSuccess) {
    seed_count_kernel<<<(unsigned)nblocks, kSeedThreads, 0, st>>>(sh, counts, masks);
    e = cudaGetLastError();
  }
  // exclusive scan over nblocks + 1 entries: the last one is the total
  if (e == cudaSuccess) e = launch_exclusive_scan(counts, nblocks + 1, scratch, st, nullptr);
  int total = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&total, counts + nblocks, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  float* x = nullptr;
  if (e == cudaSuccess && total > 0) {
    e = cudaMalloc(&x, sizeof(float) * 3 * (size_t)total);
    if (e == cudaSuccess) {
      seed_write_kernel<<<(unsigned)nblocks, kSeedThreads, 0, st>>>(sh, counts, masks, x);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  cudaFree(counts);
  cudaFree(scratch);
  cudaFree(masks);
  if (e != cudaSuccess) {
    cudaFree(x);
    return e;
  }
  *x_out = x;
  *n_out = total;
  return cudaSuccess;
}

}  // namespace mpm
