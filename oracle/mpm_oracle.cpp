/*
 * CPU oracle for the MLS-MPM substep — TEST INFRASTRUCTURE ONLY (see mpm_oracle.h).
 *
 * A restatement of the reference substep, templated on the arithmetic type:
 *   - Simulation::advance        src/mpm.cu:323-329  (reset grid, P2G, grid op, G2P)
 *   - particleToGrid             src/mpm.cu:14-74
 *   - gridOpKernel               src/mpm.cu:76-107
 *   - gridToParticle             src/mpm.cu:109-178
 *   - MLS_APIC_Scheme hooks      include/TransferScheme.h:56-143
 *   - QuadraticInterpolationKernel::weights_per_direction / D_inv_const
 *                                include/InterpolationKernel.cuh:53-74
 *   - MMFixedCorotated / MMSnow / MMJelly
 *                                include/MaterialModel.cuh:40-150
 *   - polar / svd / determinant  src/linalg.cu:18-53
 *   - 3x3 SVD                    McAdams, Selle, Tamstorf, Teran, Sifakis, "Computing the
 *                                SVD of 3x3 matrices with minimal branching and elementary
 *                                floating point operations", UW-Madison TR1690 (2011), the
 *                                method cited by include/svd3_cuda.h:5-9.
 *
 * Deliberate deviations from the reference (documented, not reproducible safely):
 *   - Q2: the reference clips the P2G stencil at the upper faces with N + range_begin
 *     (src/mpm.cu:42-44) and so writes outside the grid; the oracle clips with N - base
 *     on both transfers (as G2P does at src/mpm.cu:140-142).
 *   - Q1 out-of-range threads: with g2p_guard on, particles 0..N^3 run G2P
 *     (src/mpm.cu:114); threads past the particle count are not emulated.
 */
#include "mpm_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <typename T>
struct Mat3 {
  T m[9];
  T& operator()(int r, int c) { return m[3 * r + c]; }
  const T& operator()(int r, int c) const { return m[3 * r + c]; }
  static Mat3 zero() {
    Mat3 a;
    for (int i = 0; i < 9; ++i) a.m[i] = T(0);
    return a;
  }
  static Mat3 identity() {
    Mat3 a = zero();
    a(0, 0) = a(1, 1) = a(2, 2) = T(1);
    return a;
  }
};

template <typename T>
Mat3<T> matmul(const Mat3<T>& a, const Mat3<T>& b) {
  Mat3<T> r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r(i, j) = a(i, 0) * b(0, j) + a(i, 1) * b(1, j) + a(i, 2) * b(2, j);
  return r;
}

template <typename T>
Mat3<T> transpose(const Mat3<T>& a) {
  Mat3<T> r;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) r(i, j) = a(j, i);
  return r;
}

/* src/linalg.cu:48-53 (cofactor expansion along the first row). */
template <typename T>
T det3(const Mat3<T>& M) {
  T sub1 = M(1, 0) * M(2, 1) - M(1, 1) * M(2, 0);
  T sub2 = M(1, 0) * M(2, 2) - M(1, 2) * M(2, 0);
  T sub3 = M(1, 1) * M(2, 2) - M(1, 2) * M(2, 1);
  return M(0, 0) * sub3 - M(0, 1) * sub2 + M(0, 2) * sub1;
}

/* Eigen's fixed-size 3x3 determinant (column-wise cofactor expansion), used by
 * MMJelly::endOfStepMutation (include/MaterialModel.cuh:142-148). */
template <typename T>
T det3_eigen(const Mat3<T>& m) {
  return m(0, 0) * (m(1, 1) * m(2, 2) - m(2, 1) * m(1, 2)) -
         m(1, 0) * (m(0, 1) * m(2, 2) - m(2, 1) * m(0, 2)) +
         m(2, 0) * (m(0, 1) * m(1, 2) - m(1, 1) * m(0, 2));
}

inline float rsqrt_rn(float x) { return (float)(1.0 / std::sqrt((double)x)); }
inline double rsqrt_rn(double x) { return 1.0 / std::sqrt(x); }

/* ---------------------------------------------------------------------------
 * 3x3 SVD.  A = U diag(s) V^T with U, V proper rotations, s sorted by
 * decreasing magnitude, s[2] carrying the sign of det(A).
 *
 * Method (McAdams et al. TR1690):
 *   1. S = A^T A.
 *   2. Jacobi eigen-analysis of S with cyclic sweeps over the planes (1,2),
 *      (2,3), (3,1); each rotation is kept as a half-angle quaternion factor and
 *      the accumulated quaternion gives V.  In float the rotation angle is the
 *      paper's approximate Givens angle (ratio test against gamma = 3+2*sqrt(2),
 *      fixed pi/8 half-angle otherwise) and 4 sweeps are run; in double the
 *      exact Jacobi angle is used until the off-diagonal vanishes.
 *   3. B = A V; columns sorted by decreasing norm (a swap negates one column so
 *      that V stays a rotation).
 *   4. QR of B by three Givens rotations (planes (1,2), (1,3), (2,3)), with the
 *      paper's sign-robust half-angle construction; U is their product and s is
 *      the diagonal of the triangular factor.
 * ------------------------------------------------------------------------- */
template <typename T>
struct Quat {
  T w, x, y, z;
};

template <typename T>
void jacobi_angle(T app, T apq, T aqq, bool exact, T& ch, T& sh) {
  if (exact) {
    if (apq == T(0)) {
      ch = T(1);
      sh = T(0);
      return;
    }
    // inner rotation |theta| <= pi/4 (cyclic Jacobi converges only with these)
    const T d = app - aqq;
    T theta = (d == T(0)) ? T(0.78539816339744831) * (apq > T(0) ? T(1) : T(-1))
                          : T(0.5) * std::atan(T(2) * apq / d);
    ch = std::cos(theta * T(0.5));
    sh = std::sin(theta * T(0.5));
    return;
  }
  const T gamma = T(5.828427124746190);  // 3 + 2 sqrt(2)
  const T tiny = T(1e-20);
  sh = T(0.5) * apq;
  ch = app - aqq;
  if (sh * sh < tiny) {
    sh = T(0);
    ch = T(1);
  }
  T sh2 = sh * sh, ch2 = ch * ch;
  T w = rsqrt_rn(sh2 + ch2);
  if (ch2 <= gamma * sh2) {
    ch = T(0.92387953251128674);  // cos(pi/8)
    sh = T(0.38268343236508978);  // sin(pi/8)
  } else {
    ch *= w;
    sh *= w;
  }
}

/* S <- G^T S G for the rotation [[c,-s],[s,c]] in plane (p,q); r is the third index. */
template <typename T>
void conjugate(Mat3<T>& S, int p, int q, int r, T c, T s) {
  T spp = S(p, p), sqq = S(q, q), spq = S(p, q), spr = S(p, r), sqr = S(q, r);
  T npp = c * c * spp + T(2) * c * s * spq + s * s * sqq;
  T nqq = s * s * spp - T(2) * c * s * spq + c * c * sqq;
  T npq = (c * c - s * s) * spq - c * s * (spp - sqq);
  T npr = c * spr + s * sqr;
  T nqr = c * sqr - s * spr;
  S(p, p) = npp;
  S(q, q) = nqq;
  S(p, q) = S(q, p) = npq;
  S(p, r) = S(r, p) = npr;
  S(q, r) = S(r, q) = nqr;
}

/* q <- q * (ch, sh * e_axis); axis 0 = x (plane (2,3)), 1 = y (plane (3,1)), 2 = z (plane (1,2)). */
template <typename T>
void quat_mul_axis(Quat<T>& q, int axis, T ch, T sh) {
  Quat<T> o = q;
  if (axis == 2) {
    q.w = ch * o.w - sh * o.z;
    q.x = ch * o.x + sh * o.y;
    q.y = ch * o.y - sh * o.x;
    q.z = ch * o.z + sh * o.w;
  } else if (axis == 0) {
    q.w = ch * o.w - sh * o.x;
    q.x = ch * o.x + sh * o.w;
    q.y = ch * o.y + sh * o.z;
    q.z = ch * o.z - sh * o.y;
  } else {
    q.w = ch * o.w - sh * o.y;
    q.x = ch * o.x - sh * o.z;
    q.y = ch * o.y + sh * o.w;
    q.z = ch * o.z + sh * o.x;
  }
}

template <typename T>
void qr_givens(T a1, T a2, bool exact, T& ch, T& sh) {
  const T eps = exact ? T(1e-100) : T(1e-12);
  sh = (a2 * a2 >= eps) ? a2 : T(0);
  ch = std::max(T(std::fabs(a1)), eps);
  T rho = std::sqrt(ch * ch + sh * sh);
  ch = ch + rho;
  if (a1 < T(0)) std::swap(ch, sh);
  T w = rsqrt_rn(ch * ch + sh * sh);
  ch *= w;
  sh *= w;
}

template <typename T>
void svd3(const Mat3<T>& A, Mat3<T>& U, T s[3], Mat3<T>& V, bool exact) {
  Mat3<T> S = matmul(transpose(A), A);
  Quat<T> q{T(1), T(0), T(0), T(0)};
  const int planes[3][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}};
  const int axes[3] = {2, 0, 1};
  int sweeps = exact ? 40 : 4;
  for (int sw = 0; sw < sweeps; ++sw) {
    for (int k = 0; k < 3; ++k) {
      int p = planes[k][0], qq = planes[k][1], r = planes[k][2];
      T ch, sh;
      jacobi_angle(S(p, p), S(p, qq), S(qq, qq), exact, ch, sh);
      T c = ch * ch - sh * sh;
      T sn = T(2) * ch * sh;
      conjugate(S, p, qq, r, c, sn);
      quat_mul_axis(q, axes[k], ch, sh);
    }
    if (exact) {
      T off = std::fabs(S(0, 1)) + std::fabs(S(1, 2)) + std::fabs(S(0, 2));
      T diag = std::fabs(S(0, 0)) + std::fabs(S(1, 1)) + std::fabs(S(2, 2));
      if (off <= T(1e-300) || off <= diag * T(1e-18)) break;
    }
  }
  T qn = rsqrt_rn(q.w * q.w + q.x * q.x + q.y * q.y + q.z * q.z);
  q.w *= qn;
  q.x *= qn;
  q.y *= qn;
  q.z *= qn;
  T xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
  T xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
  T wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
  V(0, 0) = T(1) - T(2) * (yy + zz);
  V(0, 1) = T(2) * (xy - wz);
  V(0, 2) = T(2) * (xz + wy);
  V(1, 0) = T(2) * (xy + wz);
  V(1, 1) = T(1) - T(2) * (xx + zz);
  V(1, 2) = T(2) * (yz - wx);
  V(2, 0) = T(2) * (xz - wy);
  V(2, 1) = T(2) * (yz + wx);
  V(2, 2) = T(1) - T(2) * (xx + yy);

  Mat3<T> B = matmul(A, V);
  auto colnorm = [&](int c) { return B(0, c) * B(0, c) + B(1, c) * B(1, c) + B(2, c) * B(2, c); };
  auto swapcols = [&](int a, int b, int neg) {
    for (int r = 0; r < 3; ++r) {
      std::swap(B(r, a), B(r, b));
      std::swap(V(r, a), V(r, b));
      B(r, neg) = -B(r, neg);
      V(r, neg) = -V(r, neg);
    }
  };
  T r1 = colnorm(0), r2 = colnorm(1), r3 = colnorm(2);
  if (r1 < r2) {
    swapcols(0, 1, 1);
    std::swap(r1, r2);
  }
  if (r1 < r3) {
    swapcols(0, 2, 0);
    std::swap(r1, r3);
  }
  if (r2 < r3) {
    swapcols(1, 2, 2);
    std::swap(r2, r3);
  }

  U = Mat3<T>::identity();
  const int qrp[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  for (int k = 0; k < 3; ++k) {
    int p = qrp[k][0], qq = qrp[k][1];
    T ch, sh;
    qr_givens(B(p, p), B(qq, p), exact, ch, sh);
    T c = ch * ch - sh * sh;
    T sn = T(2) * ch * sh;
    for (int col = 0; col < 3; ++col) {
      T bp = B(p, col), bq = B(qq, col);
      B(p, col) = c * bp + sn * bq;
      B(qq, col) = c * bq - sn * bp;
    }
    for (int row = 0; row < 3; ++row) {
      T up = U(row, p), uq = U(row, qq);
      U(row, p) = c * up + sn * uq;
      U(row, qq) = c * uq - sn * up;
    }
  }
  s[0] = B(0, 0);
  s[1] = B(1, 1);
  s[2] = B(2, 2);
}

/* src/linalg.cu:18-33: R = U V^T, S = V Sigma V^T. */
template <typename T>
void polar(const Mat3<T>& A, Mat3<T>& R, Mat3<T>& S, bool exact) {
  Mat3<T> U, V;
  T s[3];
  svd3(A, U, s, V, exact);
  Mat3<T> Vt = transpose(V);
  R = matmul(U, Vt);
  Mat3<T> VS;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) VS(r, c) = V(r, c) * s[c];
  S = matmul(VS, Vt);
}

template <typename T>
struct Real;
template <>
struct Real<float> {
  static constexpr bool exact = false;
};
template <>
struct Real<double> {
  static constexpr bool exact = true;
};

template <typename T>
T clampv(T v, T lo, T hi) {
  return std::fmax(std::fmin(v, hi), lo);
}

/* MaterialModel::computePF, include/MaterialModel.cuh:56-61 (fixed corotated),
 * :85-93 (snow), :131-139 (jelly); liquid: K (J-1) J I (weakly compressible,
 * the lambda-term form with mu = 0). Stress uses the stored Jp, not det F. */
template <typename T>
Mat3<T> compute_PF(const oracle_material& mm, const Mat3<T>& F, T Jp) {
  Mat3<T> PF;
  if (mm.kind == ORACLE_MAT_LIQUID) {
    PF = Mat3<T>::zero();
    T p = T(mm.bulk) * (Jp - T(1)) * Jp;
    PF(0, 0) = PF(1, 1) = PF(2, 2) = p;
    return PF;
  }
  Mat3<T> R, S;
  polar(F, R, S, Real<T>::exact);
  T mu, lambda;
  if (mm.kind == ORACLE_MAT_FIXED_COROTATED) {
    mu = T(mm.mu0);
    lambda = T(mm.lambda0);
  } else {
    /* real e = std::exp(hardening * (1.0 - Jp)) is evaluated in double. */
    T e = T(std::exp((double)mm.hardening * (1.0 - (double)Jp)));
    mu = T(mm.mu0) * e;
    lambda = T(mm.lambda0) * e;
  }
  T two_mu = T(2.0 * (double)mu);
  Mat3<T> FmR;
  for (int i = 0; i < 9; ++i) FmR.m[i] = two_mu * (F.m[i] - R.m[i]);
  PF = matmul(FmR, transpose(F));
  T lt = T((double)lambda * (((double)Jp - 1.0) * (double)Jp));
  PF(0, 0) += lt;
  PF(1, 1) += lt;
  PF(2, 2) += lt;
  return PF;
}

template <typename T>
struct Params {
  T dt, dx, dx_inv, dinv, gravity;
  int N;
};

template <typename T>
Params<T> make_params(const oracle_config* cfg) {
  Params<T> p;
  p.N = cfg->N;
  p.dt = T(cfg->dt);
  p.gravity = T(cfg->gravity);
  if (std::is_same<T, float>::value) {
    /* SimulationParameters (include/TransferScheme.h:22-28): dx = 1.0/N (double,
     * stored as float), dx_inv = 1.0/dx. D_inv_const = I * 4.0 * dx_inv * dx_inv. */
    float dx = (float)(1.0 / (double)cfg->N);
    float dxi = (float)(1.0 / (double)dx);
    p.dx = T(dx);
    p.dx_inv = T(dxi);
    p.dinv = T((4.0f * dxi) * dxi);
  } else {
    p.dx = T(1.0 / (double)cfg->N);
    p.dx_inv = T(cfg->N);
    p.dinv = T(4) * p.dx_inv * p.dx_inv;
  }
  return p;
}

/* QuadraticInterpolationKernel::weights_per_direction (InterpolationKernel.cuh:57-69). */
template <typename T>
void weights(const T x[3], T dx_inv, int base[3], T w[3][3]) {
  for (int d = 0; d < 3; ++d) {
    T xg = x[d] * dx_inv;
    base[d] = (int)(xg - T(0.5));
    T fx = xg - (T)base[d];
    w[d][0] = T(0.5) * (T(1.5) - fx) * (T(1.5) - fx);
    w[d][1] = T(0.75) - (fx - T(1)) * (fx - T(1));
    w[d][2] = T(0.5) * (fx - T(0.5)) * (fx - T(0.5));
  }
}

inline bool outside(const int base[3], int N) {
  for (int d = 0; d < 3; ++d)
    if (base[d] + 3 < 0 || base[d] >= N) return true;
  return false;
}

template <typename T>
void load_mat(const T* a, int64_t p, Mat3<T>& M) {
  for (int i = 0; i < 9; ++i) M.m[i] = a[9 * p + i];
}
template <typename T>
void store_mat(T* a, int64_t p, const Mat3<T>& M) {
  for (int i = 0; i < 9; ++i) a[9 * p + i] = M.m[i];
}

int resolve_threads(int n) {
#ifdef _OPENMP
  return n > 0 ? n : omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

/* particleToGrid (src/mpm.cu:14-74) with p2g_prepare_particle / p2g_node_contribution
 * (include/TransferScheme.h:66-100). Threads accumulate into private grids. */
template <typename T>
void p2g(const oracle_config* cfg, const Params<T>& P, int64_t n, const T* x, const T* v, const T* C,
         const T* F, const T* Jp, const uint8_t* mat, std::vector<T>& grid, int nthreads) {
  const int N = P.N;
  const size_t cells = (size_t)N * N * N;
  std::fill(grid.begin(), grid.end(), T(0));
  std::vector<std::vector<T>> priv(nthreads > 1 ? nthreads : 0);
#pragma omp parallel num_threads(nthreads)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    T* g = grid.data();
    if (nthreads > 1) {
      priv[tid].assign(cells * 4, T(0));
      g = priv[tid].data();
    }
#pragma omp for schedule(static)
    for (int64_t p = 0; p < n; ++p) {
      const oracle_material& mm = cfg->materials[mat ? mat[p] : 0];
      T xp[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]};
      int base[3];
      T w[3][3];
      weights(xp, P.dx_inv, base, w);
      Mat3<T> Fm, Cm;
      load_mat(F, p, Fm);
      load_mat(C, p, Cm);
      Mat3<T> PF = compute_PF(mm, Fm, Jp[p]);
      T s = ((-P.dinv) * P.dt) * T(mm.particle_volume);
      T mass = T(mm.particle_mass);
      Mat3<T> A;
      for (int i = 0; i < 9; ++i) A.m[i] = s * PF.m[i] + mass * Cm.m[i];
      if (outside(base, N)) continue;
      int lo[3], hi[3];
      for (int d = 0; d < 3; ++d) {
        lo[d] = std::max(0, -base[d]);
        hi[d] = std::min(3, N - base[d]);
      }
      T vm[3] = {v[3 * p] * mass, v[3 * p + 1] * mass, v[3 * p + 2] * mass};
      for (int i = lo[0]; i < hi[0]; ++i) {
        int ig = base[0] + i;
        T d0 = T(ig) * P.dx - xp[0];
        for (int j = lo[1]; j < hi[1]; ++j) {
          int jg = base[1] + j;
          T d1 = T(jg) * P.dx - xp[1];
          for (int k = lo[2]; k < hi[2]; ++k) {
            int kg = base[2] + k;
            T d2 = T(kg) * P.dx - xp[2];
            T wt = w[0][i] * w[1][j] * w[2][k];
            T ad0 = A(0, 0) * d0 + A(0, 1) * d1 + A(0, 2) * d2;
            T ad1 = A(1, 0) * d0 + A(1, 1) * d1 + A(1, 2) * d2;
            T ad2 = A(2, 0) * d0 + A(2, 1) * d1 + A(2, 2) * d2;
            T* cell = g + 4 * ((size_t)N * N * ig + (size_t)N * jg + kg);
            cell[0] += wt * (vm[0] + ad0);
            cell[1] += wt * (vm[1] + ad1);
            cell[2] += wt * (vm[2] + ad2);
            cell[3] += wt * mass;
          }
        }
      }
    }
  }
  if (nthreads > 1) {
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int64_t c = 0; c < (int64_t)(cells * 4); ++c) {
      T acc = T(0);
      for (int t = 0; t < nthreads; ++t) acc += priv[t][c];
      grid[c] = acc;
    }
  }
}

/* gridOpKernel (src/mpm.cu:76-107): divide all four components by the mass
 * (the mass slot becomes 1), gravity on y, walls. */
template <typename T>
void grid_op(const oracle_config* cfg, const Params<T>& P, std::vector<T>& grid, int nthreads) {
  const int N = P.N;
  const int bc = cfg->boundary_cells;
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j)
      for (int k = 0; k < N; ++k) {
        T* cell = grid.data() + 4 * ((size_t)N * (N * i + j) + k);
        if (!(cell[3] > T(0))) continue;
        T m = cell[3];
        cell[0] /= m;
        cell[1] /= m;
        cell[2] /= m;
        cell[3] /= m;
        cell[1] += P.dt * P.gravity;
        bool sticky = false, floor = false;
        if (cfg->boundary_mode == ORACLE_BOUNDARY_REF_FRACTION) {
          const T b = T(0.05);
          T xx = T(i) / T(N), yy = T(j) / T(N), zz = T(k) / T(N);
          sticky = xx < b || xx > T(1) - b || yy > T(1) - b || zz < b || zz > T(1) - b;
          floor = yy < b;
        } else if (cfg->boundary_mode == ORACLE_BOUNDARY_STICKY_CELLS) {
          sticky = i < bc || i >= N - bc || j < bc || j >= N - bc || k < bc || k >= N - bc;
        } else {
          sticky = i < bc || i >= N - bc || j >= N - bc || k < bc || k >= N - bc;
          floor = j < bc;
        }
        if (sticky) cell[0] = cell[1] = cell[2] = T(0);
        if (floor) cell[1] = std::fmax(T(0), cell[1]);
      }
}

/* gridToParticle (src/mpm.cu:109-178) with g2p_* hooks (TransferScheme.h:102-142)
 * and endOfStepMutation (MaterialModel.cuh:95-115, :142-148). */
template <typename T>
void g2p(const oracle_config* cfg, const Params<T>& P, int64_t n, T* x, T* v, T* C, T* F, T* Jp,
         const uint8_t* mat, const std::vector<T>& grid, int nthreads) {
  const int N = P.N;
  int64_t limit = n;
  if (cfg->g2p_guard) {
    int64_t n3 = (int64_t)N * N * N;
    limit = std::min<int64_t>(n, n3 + 1);
  }
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (int64_t p = 0; p < limit; ++p) {
    const oracle_material& mm = cfg->materials[mat ? mat[p] : 0];
    T xp[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]};
    int base[3];
    T w[3][3];
    weights(xp, P.dx_inv, base, w);
    if (outside(base, N)) continue;
    int lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::max(0, -base[d]);
      hi[d] = std::min(3, N - base[d]);
    }
    T vn[3] = {T(0), T(0), T(0)};
    Mat3<T> Cn = Mat3<T>::zero();
    for (int i = lo[0]; i < hi[0]; ++i) {
      int ig = base[0] + i;
      T d0 = T(ig) * P.dx - xp[0];
      for (int j = lo[1]; j < hi[1]; ++j) {
        int jg = base[1] + j;
        T d1 = T(jg) * P.dx - xp[1];
        for (int k = lo[2]; k < hi[2]; ++k) {
          int kg = base[2] + k;
          T d2 = T(kg) * P.dx - xp[2];
          const T* cell = grid.data() + 4 * ((size_t)N * N * ig + (size_t)N * jg + kg);
          T wt = w[0][i] * w[1][j] * w[2][k];
          T wv[3] = {wt * cell[0], wt * cell[1], wt * cell[2]};
          vn[0] += wv[0];
          vn[1] += wv[1];
          vn[2] += wv[2];
          T dd[3] = {d0 * P.dinv, d1 * P.dinv, d2 * P.dinv};
          for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) Cn(r, c) += wv[r] * dd[c];
        }
      }
    }
    Mat3<T> Fm;
    load_mat(F, p, Fm);
    T J = Jp[p];
    if (mm.kind == ORACLE_MAT_LIQUID) {
      Mat3<T> G = Mat3<T>::identity();
      for (int i = 0; i < 9; ++i) G.m[i] += P.dt * Cn.m[i];
      J = J * det3(G);
      T cr = std::cbrt(J);
      Fm = Mat3<T>::zero();
      Fm(0, 0) = Fm(1, 1) = Fm(2, 2) = cr;
    } else {
      Mat3<T> G = Mat3<T>::identity();
      for (int i = 0; i < 9; ++i) G.m[i] += P.dt * Cn.m[i];
      Fm = matmul(G, Fm);
      if (mm.kind == ORACLE_MAT_SNOW) {
        Mat3<T> U, V;
        T s[3];
        svd3(Fm, U, s, V, Real<T>::exact);
        for (int d = 0; d < 3; ++d) s[d] = clampv(s[d], T(mm.clamp_lo), T(mm.clamp_hi));
        T oldJ = det3(Fm);
        Mat3<T> US;
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) US(r, c) = U(r, c) * s[c];
        Fm = matmul(US, transpose(V));
        T Fdet = det3(Fm);
        J = clampv(J * oldJ / Fdet, T(0.6), T(20.0));
      } else if (mm.kind == ORACLE_MAT_JELLY) {
        T oldJ = det3_eigen(Fm);
        J = clampv(J * oldJ / det3_eigen(Fm), T(0.6), T(20.0));
      }
    }
    store_mat(F, p, Fm);
    Jp[p] = J;
    store_mat(C, p, Cn);
    for (int d = 0; d < 3; ++d) {
      v[3 * p + d] = vn[d];
      x[3 * p + d] = xp[d] + P.dt * vn[d];
    }
  }
}

template <typename T>
int substep(const oracle_config* cfg, int64_t n, T* x, T* v, T* C, T* F, T* Jp, const uint8_t* mat,
            int nsteps, T* grid_p2g, T* grid_op_out) {
  if (!cfg || cfg->N <= 0 || cfg->N > 1024 || n < 0 || nsteps < 0) return 1;
  if (cfg->n_materials <= 0 || cfg->n_materials > ORACLE_MAX_MATERIALS) return 2;
  if (mat)
    for (int64_t p = 0; p < n; ++p)
      if (mat[p] >= cfg->n_materials) return 3;
  Params<T> P = make_params<T>(cfg);
  int nt = resolve_threads(cfg->nthreads);
  size_t cells = (size_t)P.N * P.N * P.N;
  std::vector<T> grid(cells * 4);
  for (int s = 0; s < nsteps; ++s) {
    p2g(cfg, P, n, x, v, C, F, Jp, mat, grid, nt);
    if (grid_p2g && s == nsteps - 1) std::memcpy(grid_p2g, grid.data(), sizeof(T) * cells * 4);
    grid_op(cfg, P, grid, nt);
    if (grid_op_out && s == nsteps - 1) std::memcpy(grid_op_out, grid.data(), sizeof(T) * cells * 4);
    g2p(cfg, P, n, x, v, C, F, Jp, mat, grid, nt);
  }
  return 0;
}

template <typename T>
void svd_batch(int64_t n, const T* A, T* U, T* s, T* V) {
  for (int64_t i = 0; i < n; ++i) {
    Mat3<T> a, u, vv;
    load_mat(A, i, a);
    svd3(a, u, s + 3 * i, vv, Real<T>::exact);
    store_mat(U, i, u);
    store_mat(V, i, vv);
  }
}

template <typename T>
void polar_batch(int64_t n, const T* A, T* R, T* S) {
  for (int64_t i = 0; i < n; ++i) {
    Mat3<T> a, r, ss;
    load_mat(A, i, a);
    polar(a, r, ss, Real<T>::exact);
    store_mat(R, i, r);
    store_mat(S, i, ss);
  }
}

}  // namespace

extern "C" {

int oracle_substep_f64(const oracle_config* cfg, int64_t n, double* x, double* v, double* C, double* F,
                       double* Jp, const uint8_t* mat, int nsteps, double* grid_p2g, double* grid_op) {
  return substep<double>(cfg, n, x, v, C, F, Jp, mat, nsteps, grid_p2g, grid_op);
}

int oracle_substep_f32(const oracle_config* cfg, int64_t n, float* x, float* v, float* C, float* F,
                       float* Jp, const uint8_t* mat, int nsteps, float* grid_p2g, float* grid_op) {
  return substep<float>(cfg, n, x, v, C, F, Jp, mat, nsteps, grid_p2g, grid_op);
}

void oracle_svd_f32(int64_t n, const float* A, float* U, float* s, float* V) { svd_batch<float>(n, A, U, s, V); }
void oracle_svd_f64(int64_t n, const double* A, double* U, double* s, double* V) {
  svd_batch<double>(n, A, U, s, V);
}
void oracle_polar_f32(int64_t n, const float* A, float* R, float* S) { polar_batch<float>(n, A, R, S); }
void oracle_polar_f64(int64_t n, const double* A, double* R, double* S) { polar_batch<double>(n, A, R, S); }

float oracle_det_f32(const float* M) {
  Mat3<float> m;
  for (int i = 0; i < 9; ++i) m.m[i] = M[i];
  return det3(m);
}

double oracle_time_f32(const oracle_config* cfg, int64_t n, float* x, float* v, float* C, float* F, float* Jp,
                       const uint8_t* mat, int nsteps) {
  auto t0 = std::chrono::steady_clock::now();
  int rc = substep<float>(cfg, n, x, v, C, F, Jp, mat, nsteps, nullptr, nullptr);
  auto t1 = std::chrono::steady_clock::now();
  if (rc) return -1.0;
  return std::chrono::duration<double>(t1 - t0).count();
}

int oracle_max_threads(void) { return resolve_threads(0); }

}  // extern "C"
