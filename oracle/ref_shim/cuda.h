/* Host stand-in for <cuda.h> used when compiling the reference's own
 * include/svd3_cuda.h and policy headers with g++ (oracle/_ref, test
 * infrastructure).  It defines the CUDA qualifiers as no-ops and the three
 * rounding intrinsics the SVD uses from their documented semantics:
 *   __fadd_rn / __fsub_rn : IEEE single add/sub, round to nearest even
 *                           (plain float arithmetic with -ffp-contract=off);
 *   __frsqrt_rn           : 1/sqrt(x) rounded to nearest (computed in double,
 *                           then rounded to float).
 * No NVIDIA implementation is reproduced. */
#ifndef MPM_REF_SHIM_CUDA_H
#define MPM_REF_SHIM_CUDA_H
#include <math.h>
#ifndef __device__
#define __device__
#endif
#ifndef __host__
#define __host__
#endif
#ifndef __global__
#define __global__
#endif
#ifndef __forceinline__
#define __forceinline__ inline
#endif
static inline float __fadd_rn(float a, float b) { return a + b; }
static inline float __fsub_rn(float a, float b) { return a - b; }
static inline float __frsqrt_rn(float x) { return (float)(1.0 / sqrt((double)x)); }
#ifdef __cplusplus
static inline float max(float a, float b) { return fmaxf(a, b); }
static inline float min(float a, float b) { return fminf(a, b); }
#endif
#endif
