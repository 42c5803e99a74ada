// Particle export and headless point rendering (export.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mpm {

constexpr int kBgeoRecordBytes = 36;  // P (x y z 1), id, velocity, radius: 9 big-endian words
constexpr uint8_t kBgeoTerminator[2] = {0x00, 0xff};

// BGEO point records of the n particles in active-list order: record r holds the particle
// at device slot inv[r] (r when inv is null).
cudaError_t launch_bgeo_pack(const float* s, int64_t stride, const uint32_t* inv, int64_t n, float radius,
                             void* records, cudaStream_t st);
// The BGEO header for n points into out (when capacity allows); returns its size in bytes.
int64_t bgeo_header(int64_t n, uint8_t* out, int64_t capacity);
// Clip-space positions (x - 0.5) * 1.8, 3 floats per particle in active-list order (inv as
// for launch_bgeo_pack).
cudaError_t launch_project(const float* s, int64_t stride, const uint32_t* inv, int64_t n, float* out,
                           cudaStream_t st);
// RGB8 image (W x H, rows top to bottom) of the particles as point_size squares of colour fg
// on bg; mask holds W * H bytes of scratch.
cudaError_t launch_render_points(const float* s, int64_t stride, int64_t n, int W, int H, float point_size,
                                 const uint8_t fg[3], const uint8_t bg[3], uint8_t* mask, uint8_t* rgb,
                                 cudaStream_t st);

}  // namespace mpm
