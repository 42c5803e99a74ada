/* Host stand-in for <cuda_runtime.h> when the reference's headers are compiled with
 * g++ for the golden vectors (oracle/_ref, test infrastructure). */
#ifndef MPM_REF_SHIM_CUDA_RUNTIME_H
#define MPM_REF_SHIM_CUDA_RUNTIME_H
#include <cstdio>
#include <cstdlib>
#include "cuda.h"
typedef int cudaError_t;
enum { cudaSuccess = 0 };
static inline const char* cudaGetErrorString(cudaError_t) { return ""; }
#endif
