// Particle export and headless point rendering, straight from the device SoA.
//
// Export: the reference writes each saved frame with Partio
// (ParticleWriter::writeParticles, include/particle_writer.h:19-43): per active particle an
// int "id" (its index in the active list), the vector "position", the vector "velocity" and
// the float "radius" 0.1, through Partio::write(path, data, true) to a .bgeo file.  Partio
// (wdas/partio; found by the reference's CMake file, not vendored, no pinned version) writes
// Houdini's classic binary geometry, version 5: a big-endian header, one definition per
// non-position attribute, then per point its homogeneous position (x, y, z, 1) followed by
// the attributes in definition order, then two terminator bytes.  bgeo_pack_kernel writes
// those point records (36 bytes: P, id, velocity, radius) already byte-swapped, in
// active-list order (gathering through the inverse of the id array), so the host only adds
// the header and the terminator.
//
// Render: the reference draws the particles with OpenGL (Renderer::render,
// include/renderer.h:43-63; shaders/cube_vertex.glsl, shaders/constant_fragment.glsl): the
// vertex position (x - 0.5) * 1.8 is the clip-space position with w = 1, every point is a
// 2 x 2 pixel square of one constant colour, there is no depth test and no blending, on an
// 800 x 600 frame cleared to grey 0.1.  There is no graphics stack here: project_kernel
// produces the vertex buffer the reference uploads (setParticlePositions), and
// splat_kernel rasterises the points into a coverage mask that colour_kernel turns into an
// RGB8 image (rows top to bottom).
#include <algorithm>

#include "export.h"
#include "mpm_internal.h"

namespace mpm {

namespace {

constexpr int kExportThreads = 256;

__device__ __forceinline__ uint32_t be32(uint32_t v) { return __byte_perm(v, 0, 0x0123); }

// Thread r writes record r (the particle at device slot inv[r]): the block's records are
// staged in shared memory and stored as 16-byte chunks (a block's 256 records, 9216 bytes,
// start 16-byte aligned).
__global__ void __launch_bounds__(kExportThreads) bgeo_pack_kernel(const float* __restrict__ s, int64_t st,
                                                                   const uint32_t* __restrict__ inv, int64_t n,
                                                                   float radius, uint32_t* __restrict__ out) {
  __shared__ __align__(16) uint32_t rec[kExportThreads * 9];
  const int64_t r0 = (int64_t)blockIdx.x * kExportThreads;
  const int64_t r = r0 + threadIdx.x;
  if (r < n) {
    const int64_t p = inv ? inv[r] : r;
    uint32_t* w = rec + 9 * threadIdx.x;
    w[0] = be32(__float_as_uint(s[(kX + 0) * st + p]));
    w[1] = be32(__float_as_uint(s[(kX + 1) * st + p]));
    w[2] = be32(__float_as_uint(s[(kX + 2) * st + p]));
    w[3] = be32(__float_as_uint(1.f));
    w[4] = be32((uint32_t)r);
    w[5] = be32(__float_as_uint(s[(kV + 0) * st + p]));
    w[6] = be32(__float_as_uint(s[(kV + 1) * st + p]));
    w[7] = be32(__float_as_uint(s[(kV + 2) * st + p]));
    w[8] = be32(__float_as_uint(radius));
  }
  __syncthreads();
  const int64_t cnt = n - r0 < kExportThreads ? n - r0 : kExportThreads;
  const int words = (int)(9 * cnt);
  uint4* dst = reinterpret_cast<uint4*>(out + 9 * r0);
  const uint4* src = reinterpret_cast<const uint4*>(rec);
  for (int q = threadIdx.x; q < words / 4; q += kExportThreads) dst[q] = src[q];
  for (int q = (words / 4) * 4 + threadIdx.x; q < words; q += kExportThreads) out[9 * r0 + q] = rec[q];
}

// (x - 0.5) * 1.8 per coordinate (Renderer::setParticlePositions), active-list order.
__device__ __forceinline__ float clip_coord(float x) { return __fmul_rn(__fsub_rn(x, 0.5f), 1.8f); }

__global__ void project_kernel(const float* __restrict__ s, int64_t st, const uint32_t* __restrict__ inv, int64_t n,
                               float* __restrict__ out) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int64_t p = inv ? inv[r] : r;
#pragma unroll
  for (int c = 0; c < 3; ++c) out[3 * r + c] = clip_coord(s[(kX + c) * st + p]);
}

__global__ void clear_mask_kernel(uint8_t* mask, int64_t pixels) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < pixels; q += (int64_t)gridDim.x * blockDim.x)
    mask[q] = 0;
}

// A point whose clip position lies inside the clip volume covers the pixels whose centres
// fall in the square [xw - size/2, xw + size/2) x [yw - size/2, yw + size/2), window
// coordinates xw = (xd + 1) W / 2, yw = (yd + 1) H / 2 (origin bottom left).
__global__ void splat_kernel(const float* __restrict__ s, int64_t st, int64_t n, int W, int H, float size,
                             uint8_t* __restrict__ mask) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const float xd = clip_coord(s[(kX + 0) * st + p]);
  const float yd = clip_coord(s[(kX + 1) * st + p]);
  const float zd = clip_coord(s[(kX + 2) * st + p]);
  if (!(fabsf(xd) <= 1.f && fabsf(yd) <= 1.f && fabsf(zd) <= 1.f)) return;  // clipped (or NaN)
  const float xw = __fmul_rn(__fadd_rn(xd, 1.f), 0.5f * (float)W);
  const float yw = __fmul_rn(__fadd_rn(yd, 1.f), 0.5f * (float)H);
  const float h = 0.5f * size;
  // pixel i is covered when i + 0.5 is in [xw - h, xw + h)
  const int i0 = max(0, (int)ceilf(__fsub_rn(__fsub_rn(xw, h), 0.5f)));
  const int i1 = min(W - 1, (int)ceilf(__fsub_rn(__fadd_rn(xw, h), 0.5f)) - 1);
  const int j0 = max(0, (int)ceilf(__fsub_rn(__fsub_rn(yw, h), 0.5f)));
  const int j1 = min(H - 1, (int)ceilf(__fsub_rn(__fadd_rn(yw, h), 0.5f)) - 1);
  for (int j = j0; j <= j1; ++j)
    for (int i = i0; i <= i1; ++i) mask[(int64_t)(H - 1 - j) * W + i] = 1;
}

__global__ void colour_kernel(const uint8_t* __restrict__ mask, int64_t pixels, uchar3 fg, uchar3 bg,
                              uint8_t* __restrict__ rgb) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < pixels; q += (int64_t)gridDim.x * blockDim.x) {
    const uchar3 c = mask[q] ? fg : bg;
    rgb[3 * q + 0] = c.x;
    rgb[3 * q + 1] = c.y;
    rgb[3 * q + 2] = c.z;
  }
}

int blocks_for(int64_t n) { return (int)std::max<int64_t>(1, (n + kExportThreads - 1) / kExportThreads); }

}  // namespace

cudaError_t launch_bgeo_pack(const float* s, int64_t stride, const uint32_t* inv, int64_t n, float radius,
                             void* records, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  bgeo_pack_kernel<<<blocks_for(n), kExportThreads, 0, st>>>(s, stride, inv, n, radius, (uint32_t*)records);
  return cudaGetLastError();
}

cudaError_t launch_project(const float* s, int64_t stride, const uint32_t* inv, int64_t n, float* out,
                           cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  project_kernel<<<blocks_for(n), kExportThreads, 0, st>>>(s, stride, inv, n, out);
  return cudaGetLastError();
}

cudaError_t launch_render_points(const float* s, int64_t stride, int64_t n, int W, int H, float point_size,
                                 const uint8_t fg[3], const uint8_t bg[3], uint8_t* mask, uint8_t* rgb,
                                 cudaStream_t st) {
  const int64_t pixels = (int64_t)W * H;
  const int pblocks = (int)std::min<int64_t>(blocks_for(pixels), 4096);
  clear_mask_kernel<<<pblocks, kExportThreads, 0, st>>>(mask, pixels);
  if (n > 0) splat_kernel<<<blocks_for(n), kExportThreads, 0, st>>>(s, stride, n, W, H, point_size, mask);
  colour_kernel<<<pblocks, kExportThreads, 0, st>>>(mask, pixels, make_uchar3(fg[0], fg[1], fg[2]),
                                                   make_uchar3(bg[0], bg[1], bg[2]), rgb);
  return cudaGetLastError();
}

// Houdini classic binary geometry, version 5, as Partio's writer lays it out: magic "Bgeo",
// 'V', version, the point / primitive / group / attribute counts, then per attribute its
// name (16-bit length and bytes), its size (16-bit), its type (0 float, 1 int, 5 vector)
// and that many zero defaults; every integer big-endian.
int64_t bgeo_header(int64_t n, uint8_t* out, int64_t capacity) {
  uint8_t buf[256];
  int64_t k = 0;
  auto put32 = [&](uint32_t v) {
    buf[k++] = (uint8_t)(v >> 24);
    buf[k++] = (uint8_t)(v >> 16);
    buf[k++] = (uint8_t)(v >> 8);
    buf[k++] = (uint8_t)v;
  };
  auto put16 = [&](uint16_t v) {
    buf[k++] = (uint8_t)(v >> 8);
    buf[k++] = (uint8_t)v;
  };
  put32(('B' << 24) | ('g' << 16) | ('e' << 8) | 'o');
  buf[k++] = 'V';
  put32(5);                 // version
  put32((uint32_t)n);       // points
  put32(0);                 // primitives
  put32(0);                 // point groups
  put32(0);                 // primitive groups
  put32(3);                 // point attributes (id, velocity, radius; the position is P)
  put32(0);                 // vertex attributes
  put32(0);                 // primitive attributes
  put32(0);                 // detail attributes
  struct Attr {
    const char* name;
    uint16_t size;
    uint32_t type;
  };
  const Attr attrs[3] = {{"id", 1, 1}, {"velocity", 3, 5}, {"radius", 1, 0}};
  for (const Attr& a : attrs) {
    uint16_t len = 0;
    while (a.name[len]) ++len;
    put16(len);
    for (uint16_t c = 0; c < len; ++c) buf[k++] = (uint8_t)a.name[c];
    put16(a.size);
    put32(a.type);
    for (int c = 0; c < a.size; ++c) put32(0);
  }
  if (out && capacity >= k)
    for (int64_t c = 0; c < k; ++c) out[c] = buf[c];
  return k;
}

}  // namespace mpm
