/* Test infrastructure: the reference's own 3x3 SVD (include/svd3_cuda.h of
 * kekeblom/mpm, a transcription of McAdams et al. TR1690) compiled for the host
 * from the reference checkout through oracle/ref_shim/cuda.h, exported for the
 * oracle tests.  Built into oracle/_ref by oracle/build.py; never shipped. */
#include <stdint.h>
#include <cuda.h>
#include "svd3_cuda.h"

extern "C" void ref_svd(int64_t n, const float* A, float* U, float* s, float* V) {
  for (int64_t i = 0; i < n; ++i) {
    const float* a = A + 9 * i;
    float* u = U + 9 * i;
    float* v = V + 9 * i;
    float* q = s + 3 * i;
    svd(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8],
        u[0], u[1], u[2], u[3], u[4], u[5], u[6], u[7], u[8],
        q[0], q[1], q[2],
        v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8]);
  }
}
