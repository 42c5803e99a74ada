// 3x3 singular value decomposition for one thread, FP32, register resident.
//
// Method: McAdams, Selle, Tamstorf, Teran, Sifakis, "Computing the Singular Value
// Decomposition of 3x3 matrices with minimal branching and elementary floating point
// operations", UW-Madison TR1690 (2011) — the method the reference uses
// (include/svd3_cuda.h:5-9).  This is an independent implementation:
//   1. S = A^T A;
//   2. four cyclic Jacobi sweeps over the planes (1,2), (2,3), (3,1) with the
//      approximate Givens half-angle (ratio test against gamma = 3 + 2 sqrt 2, fixed
//      pi/8 otherwise), rotations accumulated as a quaternion;
//   3. V from the normalised quaternion, B = A V, columns sorted by decreasing norm
//      (each swap negates one column so V stays a rotation);
//   4. QR of B with three sign-robust Givens rotations -> U and the singular values.
// Output: A ~= U diag(s) V^T, U and V proper rotations, s[0] >= s[1] >= |s[2]|,
// s[2] carrying the sign of det A.
#pragma once

namespace mpm {

struct Mat3 {
  float m[9];  // row-major
  __device__ __forceinline__ float& operator()(int r, int c) { return m[3 * r + c]; }
  __device__ __forceinline__ float operator()(int r, int c) const { return m[3 * r + c]; }
};

// Hardware reciprocal square root refined by one Newton step in residual form:
// y1 = y + (y / 2) e with e = 1 - x y^2 evaluated by an FMA, so the correction is carried
// in a small number at full relative precision.  The product form y (1.5 - x y^2 / 2)
// rounds its factor near 1.0, where the float grid is coarse; that left a systematic
// error in the quaternion and Givens normalisations, so U and V came out slightly
// non-orthonormal in one direction.  Through det(U clamp(S) V^T) it drifted snow's Jp by
// 3e-7 per substep (1.7e-4 over 500 substeps against the FP64 oracle) and biased F - R
// in the elastic stress (2.3e-3 in dL/dE over 256 substeps).  With the residual form the
// drift is the FP32 oracle's (1.6e-5 over 500 substeps) at the same speed.
__device__ __forceinline__ float rsqrt_nr(float x) {
  const float y = rsqrtf(x);
  const float e = fmaf(-(x * y), y, 1.0f);
  return fmaf(0.5f * y, e, y);
}

__device__ __forceinline__ void jacobi_half_angle(float app, float apq, float aqq, float& ch, float& sh) {
  const float gamma = 5.828427124746190f;  // 3 + 2 sqrt(2)
  sh = 0.5f * apq;
  ch = app - aqq;
  const bool tiny = sh * sh < 1e-20f;
  sh = tiny ? 0.f : sh;
  ch = tiny ? 1.f : ch;
  const float sh2 = sh * sh, ch2 = ch * ch;
  const float w = rsqrt_nr(sh2 + ch2);
  const bool fixed = ch2 <= gamma * sh2;
  ch = fixed ? 0.92387953251128674f : ch * w;
  sh = fixed ? 0.38268343236508978f : sh * w;
}

// Symmetric S <- G^T S G, G = [[c,-s],[s,c]] in plane (p,q), r the remaining index.
template <int P, int Q, int R>
__device__ __forceinline__ void jacobi_conjugate(float S[3][3], float c, float s) {
  const float spp = S[P][P], sqq = S[Q][Q], spq = S[P][Q], spr = S[P][R], sqr = S[Q][R];
  const float cc = c * c, ss = s * s, cs = c * s;
  S[P][P] = cc * spp + 2.f * cs * spq + ss * sqq;
  S[Q][Q] = ss * spp - 2.f * cs * spq + cc * sqq;
  const float npq = (cc - ss) * spq - cs * (spp - sqq);
  S[P][Q] = npq;
  S[Q][P] = npq;
  const float npr = c * spr + s * sqr;
  const float nqr = c * sqr - s * spr;
  S[P][R] = npr;
  S[R][P] = npr;
  S[Q][R] = nqr;
  S[R][Q] = nqr;
}

// q <- q * (ch, sh e_axis)
template <int AXIS>
__device__ __forceinline__ void quat_rotate(float q[4], float ch, float sh) {
  const float w = q[0], x = q[1], y = q[2], z = q[3];
  if (AXIS == 2) {
    q[0] = ch * w - sh * z;
    q[1] = ch * x + sh * y;
    q[2] = ch * y - sh * x;
    q[3] = ch * z + sh * w;
  } else if (AXIS == 0) {
    q[0] = ch * w - sh * x;
    q[1] = ch * x + sh * w;
    q[2] = ch * y + sh * z;
    q[3] = ch * z - sh * y;
  } else {
    q[0] = ch * w - sh * y;
    q[1] = ch * x - sh * z;
    q[2] = ch * y + sh * w;
    q[3] = ch * z + sh * x;
  }
}

template <int P, int Q, int R, int AXIS>
__device__ __forceinline__ void jacobi_step(float S[3][3], float q[4]) {
  float ch, sh;
  jacobi_half_angle(S[P][P], S[P][Q], S[Q][Q], ch, sh);
  const float c = ch * ch - sh * sh;
  const float s = 2.f * ch * sh;
  jacobi_conjugate<P, Q, R>(S, c, s);
  quat_rotate<AXIS>(q, ch, sh);
}

__device__ __forceinline__ void qr_half_angle(float a1, float a2, float& ch, float& sh) {
  const float eps = 1e-12f;
  sh = (a2 * a2 >= eps) ? a2 : 0.f;
  float c0 = fmaxf(fabsf(a1), eps);
  const float r2 = c0 * c0 + sh * sh;
  const float rho = r2 * rsqrt_nr(r2);
  c0 = c0 + rho;
  const bool neg = a1 < 0.f;
  ch = neg ? sh : c0;
  sh = neg ? c0 : sh;
  const float w = rsqrt_nr(ch * ch + sh * sh);
  ch *= w;
  sh *= w;
}

// Rows p, q of B rotated by G^T; columns p, q of U rotated by G.
template <int P, int Q>
__device__ __forceinline__ void qr_step(float B[3][3], float U[3][3]) {
  float ch, sh;
  qr_half_angle(B[P][P], B[Q][P], ch, sh);
  const float c = ch * ch - sh * sh;
  const float s = 2.f * ch * sh;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float bp = B[P][k], bq = B[Q][k];
    B[P][k] = c * bp + s * bq;
    B[Q][k] = c * bq - s * bp;
    const float up = U[k][P], uq = U[k][Q];
    U[k][P] = c * up + s * uq;
    U[k][Q] = c * uq - s * up;
  }
}

template <int A, int B, int NEG>
__device__ __forceinline__ void cond_swap_cols(bool swap, float M[3][3], float V[3][3]) {
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    float ma = M[r][A], mb = M[r][B], va = V[r][A], vb = V[r][B];
    float na = swap ? mb : ma, nb = swap ? ma : mb;
    float wa = swap ? vb : va, wb = swap ? va : vb;
    M[r][A] = na;
    M[r][B] = nb;
    V[r][A] = wa;
    V[r][B] = wb;
    if (swap) {
      M[r][NEG] = -M[r][NEG];
      V[r][NEG] = -V[r][NEG];
    }
  }
}

__device__ __forceinline__ void svd3(const float A[3][3], float U[3][3], float s[3], float V[3][3]) {
  float S[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) S[i][j] = A[0][i] * A[0][j] + A[1][i] * A[1][j] + A[2][i] * A[2][j];
  float q[4] = {1.f, 0.f, 0.f, 0.f};
#pragma unroll
  for (int sweep = 0; sweep < 4; ++sweep) {
    jacobi_step<0, 1, 2, 2>(S, q);
    jacobi_step<1, 2, 0, 0>(S, q);
    jacobi_step<2, 0, 1, 1>(S, q);
  }
  const float qn = rsqrt_nr(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  const float w = q[0] * qn, x = q[1] * qn, y = q[2] * qn, z = q[3] * qn;
  const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, xz = x * z, yz = y * z;
  const float wx = w * x, wy = w * y, wz = w * z;
  V[0][0] = 1.f - 2.f * (yy + zz);
  V[0][1] = 2.f * (xy - wz);
  V[0][2] = 2.f * (xz + wy);
  V[1][0] = 2.f * (xy + wz);
  V[1][1] = 1.f - 2.f * (xx + zz);
  V[1][2] = 2.f * (yz - wx);
  V[2][0] = 2.f * (xz - wy);
  V[2][1] = 2.f * (yz + wx);
  V[2][2] = 1.f - 2.f * (xx + yy);

  float B[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) B[i][j] = A[i][0] * V[0][j] + A[i][1] * V[1][j] + A[i][2] * V[2][j];

  float r1 = B[0][0] * B[0][0] + B[1][0] * B[1][0] + B[2][0] * B[2][0];
  float r2 = B[0][1] * B[0][1] + B[1][1] * B[1][1] + B[2][1] * B[2][1];
  float r3 = B[0][2] * B[0][2] + B[1][2] * B[1][2] + B[2][2] * B[2][2];
  bool sw = r1 < r2;
  cond_swap_cols<0, 1, 1>(sw, B, V);
  {
    float t = sw ? r2 : r1;
    r2 = sw ? r1 : r2;
    r1 = t;
  }
  sw = r1 < r3;
  cond_swap_cols<0, 2, 0>(sw, B, V);
  {
    float t = sw ? r3 : r1;
    r3 = sw ? r1 : r3;
    r1 = t;
  }
  sw = r2 < r3;
  cond_swap_cols<1, 2, 2>(sw, B, V);

#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) U[i][j] = (i == j) ? 1.f : 0.f;
  qr_step<0, 1>(B, U);
  qr_step<0, 2>(B, U);
  qr_step<1, 2>(B, U);
  s[0] = B[0][0];
  s[1] = B[1][1];
  s[2] = B[2][2];
}

// src/linalg.cu:48-53 (first-row cofactor expansion)
__device__ __forceinline__ float det3(const float M[3][3]) {
  const float sub1 = M[1][0] * M[2][1] - M[1][1] * M[2][0];
  const float sub2 = M[1][0] * M[2][2] - M[1][2] * M[2][0];
  const float sub3 = M[1][1] * M[2][2] - M[1][2] * M[2][1];
  return M[0][0] * sub3 - M[0][1] * sub2 + M[0][2] * sub1;
}

// Eigen's 3x3 determinant (column-wise cofactor expansion), used by MMJelly.
__device__ __forceinline__ float det3_colwise(const float m[3][3]) {
  return m[0][0] * (m[1][1] * m[2][2] - m[2][1] * m[1][2]) - m[1][0] * (m[0][1] * m[2][2] - m[2][1] * m[0][2]) +
         m[2][0] * (m[0][1] * m[1][2] - m[1][1] * m[0][2]);
}

// linalg::polar_decomposition_device (src/linalg.cu:18-33): R = U V^T, S = V Sigma V^T.
__device__ __forceinline__ void polar_decomposition(const float A[3][3], float R[3][3], float S[3][3]) {
  float U[3][3], V[3][3], s[3];
  svd3(A, U, s, V);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      R[i][j] = U[i][0] * V[j][0] + U[i][1] * V[j][1] + U[i][2] * V[j][2];
      S[i][j] = V[i][0] * s[0] * V[j][0] + V[i][1] * s[1] * V[j][1] + V[i][2] * s[2] * V[j][2];
    }
}

}  // namespace mpm
