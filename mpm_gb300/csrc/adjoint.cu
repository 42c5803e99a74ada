// Differentiable substep: checkpointed forward and hand-written adjoint kernels.
//
// The reference has no gradients.  This file differentiates the substep of
// src/mpm.cu:14-178 for two materials:
//   MMFixedCorotated (include/MaterialModel.cuh:40-62): P F^T = 2 mu (F - R) F^T +
//     lambda (Jp - 1) Jp I, no plasticity;
//   MMSnow (include/MaterialModel.cuh:67-116): the same stress with mu, lambda scaled by
//     e = exp(h (1 - Jp)) (computePF, :85-93), and the plasticity of endOfStepMutation
//     (:95-115): F^ = (I + dt C') F = U S V^T, F' = U clamp(S, lo, hi) V^T,
//     Jp' = clamp(Jp det F^ / det F', 0.6, 20).
// One substep n maps state_n = (x, v, C, F, Jp) to state_{n+1}; its adjoint runs three
// kernels:
//   adj_g2p    per particle: back through advection, the plasticity (the SVD and clamp
//              adjoint below, and the Jp update), the F update and the G2P gather;
//              gathers the grid velocity and SCATTERS the grid-velocity adjoint (the
//              G2P adjoint is a cell-sorted scatter, reduced per warp like P2G);
//   adj_gridop per node: back through the grid operation (division by the mass,
//              gravity, walls) to adjoints of the P2G momentum and mass; also clears
//              the grid-velocity adjoint and computes the grid velocities of the
//              previous substep for its adj_g2p;
//   adj_p2g    per particle: GATHERS the momentum/mass adjoints (the P2G adjoint is a
//              gather) and goes back through the affine term, the stress (with the
//              polar decomposition's adjoint and the hardening factor's dependence on
//              Jp) and the weights; accumulates dL/dmu0 and dL/dlambda0.
// The P2G part of substep n and the G2P part of substep n - 1 touch one particle's
// adjoint only, so adj_step runs them as one pass per particle (the adjoint of state_n
// stays in registers); per substep the backward launches adj_gridop and adj_step, with
// adj_g2p and adj_p2g alone at the two ends of a segment.
// The forward run stores the state every `checkpoint_every` substeps; the backward
// pass recomputes each segment forward (keeping every state, P2G grid and the polar
// rotation each P2G used, so the P2G adjoint needs no SVD) and then runs the adjoint
// substeps in reverse.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "mpm_internal.h"
#include "warp_ops.cuh"

namespace mpm {

struct AdjArgs {
  const float* s;      // state_n, component-major (stride)
  const float* s1;     // state_{n+1}
  float* a;            // adjoint state: in = adjoint of state_{n+1}, out = of state_n
  int64_t stride, n;
  const float4* grid;  // P2G grid of substep n: (m v, m)
  const float4* vgrid; // grid velocity of substep n (grid op applied)
  float4* gvel;        // grid-velocity adjoint, scattered by adj_g2p
  const float4* gmom;  // (m v, m) adjoints, written by adj_gridop, gathered by adj_p2g
  const float* rot;    // polar rotation R of each particle's F in state_n, kept by the
                       // recompute's P2G (9 components, the state's stride)
  double* pgrad;       // [dL/dmu, dL/dlambda]
  GridConsts K;
  DevMaterial M;
};

// Launch shapes, one particle per thread. adj_g2p: 4-warp blocks, three per SM (12 warps,
// 14 KB of shared memory per warp); at one 8-warp block per SM (its shared memory and 136
// registers) the backward of 100k particles took 3.5 % longer (snow). adj_p2g: 4-warp
// blocks, four per SM (16 warps at 127 registers); capping it at 96 or 80 registers for 20
// or 21 warps per SM spilled and ran slower.
constexpr int kAdjG2PWarps = 4, kAdjG2PBlocksPerSM = 3;
constexpr int kAdjP2GWarps = 4, kAdjP2GBlocksPerSM = 4;

// d w_a / d f for the quadratic B-spline (include/InterpolationKernel.cuh:64-66)
__device__ __forceinline__ void weight_derivs(float x, float dx_inv, float dw[3]) {
  const float xg = QuadraticInterpolationKernel::grid_coord(x, dx_inv);
  const int b = (int)__fsub_rn(xg, 0.5f);
  const float f = xg - (float)b;
  dw[0] = -(1.5f - f) * dx_inv;
  dw[1] = -2.f * (f - 1.f) * dx_inv;
  dw[2] = (f - 0.5f) * dx_inv;
}

__device__ __forceinline__ float ld(const float* s, int64_t st, int comp, int64_t p) { return s[comp * st + p]; }

// Grid velocities of the last substep of a segment for the adjoint kernels; also clears
// the grid-velocity adjoint that adj_g2p accumulates into.  (adj_gridop does both for the
// other substeps.)
__global__ void adj_velocity_kernel(const float4* grid, float4* vgrid, float4* gadj, GridConsts K) {
  const int N = K.N;
  const int64_t cells = (int64_t)N * N * N;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < cells; c += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(c / ((int64_t)N * N)), j = (int)((c / N) % N), k = (int)(c % N);
    const float3 v = grid_node_velocity(grid[c], i, j, k, K);
    vgrid[c] = make_float4(v.x, v.y, v.z, 0.f);
    gadj[c] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// Adjoint of the snow plasticity at F^ (MMSnow::endOfStepMutation,
// include/MaterialModel.cuh:95-115).  With F^ = U S V^T (U, V rotations, S = diag(s)) and
// g = clamp(., lo, hi) applied to each singular value, F' = U g(S) V^T is an isotropic
// function of F^.  In the SVD frame, B = U^T dF^ V maps to U^T dF' V = M(B):
//   M_ii = g'(s_i) B_ii;
//   for i != j, with sym = (B_ij + B_ji) / 2 and skw = (B_ij - B_ji) / 2,
//   M_ij = a_ij sym + b_ij skw, M_ji = a_ij sym - b_ij skw,
//   a_ij = (g_i - g_j) / (s_i - s_j)  (1 when both are inside the band, 0 when both are
//          clamped to the same bound, the mean of g' when s_i = s_j),
//   b_ij = (g_i + g_j) / (s_i + s_j).
// M is symmetric in the Frobenius inner product, so the adjoint is F^bar = U M(U^T F'bar V) V^T.
// The Jp update Jp' = Jp r, r = det F^ / det F' = prod s_i / prod g_i (U, V rotations), has,
// when Jp' is not clamped to [0.6, 20], dJp'/dJp = r and dJp'/dF^ = Jp' U diag(1/s_i - g'_i/g_i) V^T.
// Returns the F^ adjoint in Fhb (from F'bar = Fb and Jp'bar = jb) and r; *unclamped tells
// whether Jp' was inside [0.6, 20].
__device__ __forceinline__ void snow_plasticity_adjoint(const float Fh[3][3], float Jp, float lo, float hi,
                                                        const float Fb[3][3], float jb, float Fhb[3][3], float& r,
                                                        bool& unclamped) {
  float U[3][3], V[3][3], s[3];
  svd3(Fh, U, s, V);
  float g[3], gp[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    g[i] = clampf(s[i], lo, hi);
    gp[i] = (s[i] > lo && s[i] < hi) ? 1.f : 0.f;
  }
  r = (s[0] / g[0]) * (s[1] / g[1]) * (s[2] / g[2]);
  const float jn = Jp * r;
  unclamped = jn > 0.6f && jn < 20.f;
  // B = U^T Fb V
  float T[3][3], B[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) T[i][j] = Fb[i][0] * V[0][j] + Fb[i][1] * V[1][j] + Fb[i][2] * V[2][j];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) B[i][j] = U[0][i] * T[0][j] + U[1][i] * T[1][j] + U[2][i] * T[2][j];
  float Mm[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    Mm[i][i] = gp[i] * B[i][i];
    if (unclamped) Mm[i][i] += jb * jn * (1.f / s[i] - gp[i] / g[i]);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i + 1; j < 3; ++j) {
      float a;
      if (gp[i] != 0.f && gp[j] != 0.f) {
        a = 1.f;
      } else if (gp[i] == 0.f && gp[j] == 0.f && g[i] == g[j]) {
        a = 0.f;
      } else {
        const float d = s[i] - s[j];
        a = (fabsf(d) > 1e-12f) ? (g[i] - g[j]) / d : 0.5f * (gp[i] + gp[j]);
      }
      const float den = s[i] + s[j];
      const float b = (fabsf(den) > 1e-12f) ? (g[i] + g[j]) / den : 0.f;
      const float sym = 0.5f * (B[i][j] + B[j][i]), skw = 0.5f * (B[i][j] - B[j][i]);
      Mm[i][j] = a * sym + b * skw;
      Mm[j][i] = a * sym - b * skw;
    }
  // Fhb = U Mm V^T
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) T[i][j] = Mm[i][0] * V[j][0] + Mm[i][1] * V[j][1] + Mm[i][2] * V[j][2];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) Fhb[i][j] = U[i][0] * T[0][j] + U[i][1] * T[1][j] + U[i][2] * T[2][j];
}

// Back through x' = x + dt v', the snow plasticity (above), F^ = (I + dt C') F and the G2P
// gather (src/mpm.cu:136-176) for particle p of substep n (A.s = state_n, A.s1 = state_{n+1}).
// In: the adjoint of the particle's state_{n+1} (ax, av, aC, aF, jb).  Returns false, with
// nothing written, when the particle is outside the domain at state_n (frozen: its adjoint
// passes through).  Else out: the adjoint of state_n's x, F and Jp through this part of the
// substep (gx, Fa, jo; v and C of state_n get theirs from the P2G adjoint alone), the
// velocity adjoints of its 27 nodes in wbuf (lane's column) and its cell key.
__device__ __forceinline__ bool g2p_adjoint(const AdjArgs& A, int64_t p, int lane, float4* wbuf, const float ax[3],
                                            const float av[3], const float aC[3][3], const float aF_in[3][3], float jb,
                                            float gx[3], float Fa[3][3], float& jo, int& key) {
  const GridConsts& K = A.K;
  const int N = K.N;
  const int64_t st = A.stride;
  float x[3], w[3][3], d[3][3];
  int b[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) x[q] = ld(A.s, st, kX + q, p);
  stencil(x, K, b, w, d);
  if (outside_domain(b[0], b[1], b[2], N)) return false;
  key = pack_key(b[0], b[1], b[2]);
  float F[3][3], C1[3][3], aF[3][3];
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    F[q / 3][q % 3] = ld(A.s, st, kF + q, p);
    C1[q / 3][q % 3] = ld(A.s1, st, kC + q, p);
    aF[q / 3][q % 3] = aF_in[q / 3][q % 3];
  }
  jo = jb;
  if (A.M.kind == kSnow) {
    // aF holds the adjoint of F' = U clamp(S) V^T: take it back to F^ = (I + dt C') F,
    // and the Jp' adjoint back to Jp
    float Fh[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        Fh[r][c] = F[r][c] + K.dt * (C1[r][0] * F[0][c] + C1[r][1] * F[1][c] + C1[r][2] * F[2][c]);
    const float Jp = ld(A.s, st, kJp, p);
    float Fhb[3][3], ratio;
    bool unclamped;
    snow_plasticity_adjoint(Fh, Jp, A.M.clamp_lo, A.M.clamp_hi, aF, jb, Fhb, ratio, unclamped);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int c = 0; c < 3; ++c) aF[r][c] = Fhb[r][c];
    jo = unclamped ? jb * ratio : 0.f;
  }
  // v' total adjoint, C' total adjoint
  float vt[3], Ct[3][3];
#pragma unroll
  for (int q = 0; q < 3; ++q) vt[q] = av[q] + K.dt * ax[q];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c)
      Ct[r][c] = aC[r][c] + K.dt * (aF[r][0] * F[c][0] + aF[r][1] * F[c][1] + aF[r][2] * F[c][2]);
  // F adjoint: (I + dt C')^T F'adj
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c)
      Fa[r][c] = aF[r][c] + K.dt * (C1[0][r] * aF[0][c] + C1[1][r] * aF[1][c] + C1[2][r] * aF[2][c]);
  // gather grid velocity; x adjoint through the weights and dpos; node velocity adjoints
  float dwd[3][3];
#pragma unroll
  for (int q = 0; q < 3; ++q) weight_derivs(x[q], K.dx_inv, dwd[q]);
#pragma unroll
  for (int q = 0; q < 3; ++q) gx[q] = ax[q];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int bb = 0; bb < 3; ++bb)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int i = b[0] + a, j = b[1] + bb, k = b[2] + c;
        float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
        if ((unsigned)i < (unsigned)N && (unsigned)j < (unsigned)N && (unsigned)k < (unsigned)N)
          g = __ldg(A.vgrid + ((int64_t)i * N + j) * N + k);
        const float wt = w[0][a] * w[1][bb] * w[2][c];
        const float dd[3] = {d[0][a], d[1][bb], d[2][c]};
        const float vi[3] = {g.x, g.y, g.z};
        float Cd[3], CTv[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          Cd[r] = Ct[r][0] * dd[0] + Ct[r][1] * dd[1] + Ct[r][2] * dd[2];
          CTv[r] = Ct[0][r] * vi[0] + Ct[1][r] * vi[1] + Ct[2][r] * vi[2];
        }
        // w-adjoint = v'adj . v_i + D v_i . (C'adj d)
        const float wbar = vt[0] * vi[0] + vt[1] * vi[1] + vt[2] * vi[2] +
                           K.dinv * (vi[0] * Cd[0] + vi[1] * Cd[1] + vi[2] * Cd[2]);
        const float gw[3] = {dwd[0][a] * w[1][bb] * w[2][c], w[0][a] * dwd[1][bb] * w[2][c],
                             w[0][a] * w[1][bb] * dwd[2][c]};
#pragma unroll
        for (int r = 0; r < 3; ++r) gx[r] += wbar * gw[r] - K.dinv * wt * CTv[r];
        // velocity adjoint of node i
        wbuf[(a * 9 + bb * 3 + c) * kRedStride + lane] =
            make_float4(wt * (vt[0] + K.dinv * Cd[0]), wt * (vt[1] + K.dinv * Cd[1]), wt * (vt[2] + K.dinv * Cd[2]), 0.f);
      }
  return true;
}

__device__ __forceinline__ void load_adjoint(const AdjArgs& A, int64_t p, float ax[3], float av[3], float aC[3][3],
                                             float aF[3][3], float& aJp) {
  const int64_t st = A.stride;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    ax[q] = ld(A.a, st, kX + q, p);
    av[q] = ld(A.a, st, kV + q, p);
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    aC[q / 3][q % 3] = ld(A.a, st, kC + q, p);
    aF[q / 3][q % 3] = ld(A.a, st, kF + q, p);
  }
  aJp = ld(A.a, st, kJp, p);
}

__device__ __forceinline__ void store_adjoint(const AdjArgs& A, int64_t p, const float ax[3], const float av[3],
                                              const float aC[3][3], const float aF[3][3], float aJp) {
  const int64_t st = A.stride;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    A.a[(kX + q) * st + p] = ax[q];
    A.a[(kV + q) * st + p] = av[q];
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    A.a[(kC + q) * st + p] = aC[q / 3][q % 3];
    A.a[(kF + q) * st + p] = aF[q / 3][q % 3];
  }
  A.a[kJp * st + p] = aJp;
}

// The G2P part of substep n alone (the last substep of a segment): A.a holds the adjoint
// of state_{n+1}; x, F and Jp of it are replaced by their G2P-part adjoints of state_n.
__global__ void __launch_bounds__(kAdjG2PWarps * 32, kAdjG2PBlocksPerSM) adj_g2p_kernel(const AdjArgs A) {
  extern __shared__ float4 smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float4* wbuf = smem + warp * kRedFloat4;
  const int64_t st = A.stride;
  const int64_t nsteps = (A.n + 31) / 32;
  for (int64_t ws = (int64_t)blockIdx.x * kAdjG2PWarps + warp; ws < nsteps; ws += (int64_t)gridDim.x * kAdjG2PWarps) {
    const int64_t p = ws * 32 + lane;
    int key = -1;
    if (p < A.n) {
      float ax[3], av[3], aC[3][3], aF[3][3], aJp, gx[3], Fa[3][3], jo;
      load_adjoint(A, p, ax, av, aC, aF, aJp);
      if (g2p_adjoint(A, p, lane, wbuf, ax, av, aC, aF, aJp, gx, Fa, jo, key)) {
#pragma unroll
        for (int q = 0; q < 3; ++q) A.a[(kX + q) * st + p] = gx[q];
#pragma unroll
        for (int q = 0; q < 9; ++q) A.a[(kF + q) * st + p] = Fa[q / 3][q % 3];
        A.a[kJp * st + p] = jo;
      }
    }
    if (__ballot_sync(kFull, key >= 0)) warp_scatter_runs(wbuf, lane, key, A.gvel, A.K.N);
  }
}

// Back through gridOpKernel (src/mpm.cu:76-107): the velocity adjoint gvel -> (m v, m)
// adjoints in gmom.  In the same pass, per node: gvel is cleared for the adj_g2p of the
// previous substep, and when prev_grid (that substep's P2G grid) is given, its grid
// velocity goes to vgrid (adj_g2p of this substep has finished reading it).
__global__ void adj_gridop_kernel(const float4* __restrict__ grid, float4* __restrict__ gvel,
                                  float4* __restrict__ gmom, const float4* __restrict__ prev_grid,
                                  float4* __restrict__ vgrid, GridConsts K) {
  const int N = K.N;
  const int cells = N * N * N;  // N <= 1000
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < cells; c += gridDim.x * blockDim.x) {
    const float4 g = grid[c];
    float4 ga = gvel[c];
    const float4 pg = prev_grid ? prev_grid[c] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int i = c / (N * N), rem = c - i * (N * N);
    const int j = rem / N, k = rem - j * N;
    gvel[c] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (prev_grid) {
      const float3 v = grid_node_velocity(pg, i, j, k, K);
      vgrid[c] = make_float4(v.x, v.y, v.z, 0.f);
    }
    if (g.w > 0.f) {
      bool sticky, floor_;
      if (K.boundary_mode == kBoundaryRefFraction) {
        const float bnd = 0.05f, fN = (float)N;
        const float x = (float)i / fN, y = (float)j / fN, z = (float)k / fN;
        sticky = x < bnd || x > 1.f - bnd || y > 1.f - bnd || z < bnd || z > 1.f - bnd;
        floor_ = y < bnd;
      } else if (K.boundary_mode == kBoundaryStickyCells) {
        const int bc = K.boundary_cells;
        sticky = i < bc || i >= N - bc || j < bc || j >= N - bc || k < bc || k >= N - bc;
        floor_ = false;
      } else {
        const int bc = K.boundary_cells;
        sticky = i < bc || i >= N - bc || j >= N - bc || k < bc || k >= N - bc;
        floor_ = j < bc;
      }
      const float inv = 1.f / g.w;
      if (sticky) ga = make_float4(0.f, 0.f, 0.f, 0.f);
      if (floor_ && !(g.y * inv + K.dtg > 0.f)) ga.y = 0.f;
      // v = m v / m (+ gravity): d/d(mv) = 1/m, d/dm = -(m v)/m^2
      const float mb = -(ga.x * g.x + ga.y * g.y + ga.z * g.z) * inv * inv;
      gmom[c] = make_float4(ga.x * inv, ga.y * inv, ga.z * inv, mb);
    } else {
      gmom[c] = make_float4(ga.x, ga.y, ga.z, 0.f);  // raw value passed through (v = m v)
    }
  }
}

__device__ __forceinline__ void cross_mat(const float y[3], float Y[3][3]) {
  Y[0][0] = 0.f;
  Y[0][1] = -y[2];
  Y[0][2] = y[1];
  Y[1][0] = y[2];
  Y[1][1] = 0.f;
  Y[1][2] = -y[0];
  Y[2][0] = -y[1];
  Y[2][1] = y[0];
  Y[2][2] = 0.f;
}

// Back through the P2G scatter (src/mpm.cu:14-74, TransferScheme.h:66-100) and
// MMFixedCorotated::computePF, with the polar decomposition's adjoint:
//   F = R S, dR = R [w]x with (tr(S) I - S) w = axial(R^T dF - dF^T R), so for a
//   rotation adjoint Rbar: Fbar = R [y]x, y = (tr(S) I - S)^-1 k, k = axial part of R^T Rbar.
// One particle p of substep n (A.s = state_n).  In: ax, aF, aJp hold the G2P-part adjoints
// of state_n's x, F and Jp.  Returns false, with nothing changed, when the particle is
// outside the domain at state_n.  Else out: the full adjoint of state_n in (ax, av, aC, aF,
// aJp); dL/dmu0 and dL/dlambda0 accumulate into mubar and lambar.
__device__ __forceinline__ bool p2g_adjoint(const AdjArgs& A, int64_t p, float ax[3], float av[3], float aC[3][3],
                                            float aF[3][3], float& aJp, double& mubar, double& lambar) {
  const GridConsts& K = A.K;
  const DevMaterial& M = A.M;
  const int N = K.N;
  const int64_t st = A.stride;
  float x[3], v[3], C[3][3], F[3][3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    x[q] = ld(A.s, st, kX + q, p);
    v[q] = ld(A.s, st, kV + q, p);
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    C[q / 3][q % 3] = ld(A.s, st, kC + q, p);
    F[q / 3][q % 3] = ld(A.s, st, kF + q, p);
  }
  const float Jp = ld(A.s, st, kJp, p);
  int b[3];
  float w[3][3], d[3][3];
  stencil(x, K, b, w, d);
  if (outside_domain(b[0], b[1], b[2], N)) return false;  // frozen: adjoint passes through
  float R[3][3];  // the rotation the forward's P2G used
#pragma unroll
  for (int q = 0; q < 9; ++q) R[q / 3][q % 3] = A.rot[q * st + p];
  float PF[3][3];
  compute_PF(M, F, R, Jp, PF);
  const float m = M.mass;
  const float sc = ((-K.dinv) * K.dt) * M.vol;
  float Aff[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) Aff[r][c] = sc * PF[r][c] + m * C[r][c];
  float dwd[3][3];
#pragma unroll
  for (int q = 0; q < 3; ++q) weight_derivs(x[q], K.dx_inv, dwd[q]);
  float vb[3] = {0.f, 0.f, 0.f}, Ab[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
  float xb[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int bb = 0; bb < 3; ++bb)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int i = b[0] + a, j = b[1] + bb, k = b[2] + c;
        if ((unsigned)i >= (unsigned)N || (unsigned)j >= (unsigned)N || (unsigned)k >= (unsigned)N) continue;
        const float4 g = __ldg(A.gmom + ((int64_t)i * N + j) * N + k);
        const float gm[3] = {g.x, g.y, g.z};
        const float wt = w[0][a] * w[1][bb] * w[2][c];
        const float dd[3] = {d[0][a], d[1][bb], d[2][c]};
        float contrib[3], ATg[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          contrib[r] = m * v[r] + Aff[r][0] * dd[0] + Aff[r][1] * dd[1] + Aff[r][2] * dd[2];
          ATg[r] = Aff[0][r] * gm[0] + Aff[1][r] * gm[1] + Aff[2][r] * gm[2];
          vb[r] += wt * m * gm[r];
        }
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int cc = 0; cc < 3; ++cc) Ab[r][cc] += wt * gm[r] * dd[cc];
        const float wbar = gm[0] * contrib[0] + gm[1] * contrib[1] + gm[2] * contrib[2] + g.w * m;
        const float gw[3] = {dwd[0][a] * w[1][bb] * w[2][c], w[0][a] * dwd[1][bb] * w[2][c],
                             w[0][a] * w[1][bb] * dwd[2][c]};
#pragma unroll
        for (int r = 0; r < 3; ++r) xb[r] += wbar * gw[r] - wt * ATg[r];
      }
  // affine = sc PF + m C
  float PFb[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) PFb[r][c] = sc * Ab[r][c];
  // PF = e (2 mu0 G + lambda0 (Jp - 1) Jp I), G = (F - R) F^T, e = exp(h (1 - Jp)) for snow
  // and jelly with h != 0 (compute_PF), else 1
  const bool hardens = (M.kind == kSnow || M.kind == kJelly) && M.hardening != 0.f;
  const float e = hardens ? expf(M.hardening * (1.f - Jp)) : 1.f;
  const float mu = M.mu0 * e;
  float G[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c)
      G[r][c] = (F[r][0] - R[r][0]) * F[c][0] + (F[r][1] - R[r][1]) * F[c][1] + (F[r][2] - R[r][2]) * F[c][2];
  float pg = 0.f;  // <PFb, G>
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) pg += PFb[r][c] * G[r][c];
  const float trb = PFb[0][0] + PFb[1][1] + PFb[2][2];
  // dL/dmu0 = e <PFb, 2 G>, dL/dlambda0 = e tr(PFb) (Jp - 1) Jp
  mubar += (double)(2.f * e * pg);
  lambar += (double)(e * trb * ((Jp - 1.f) * Jp));
  // dL/dJp: de/dJp = -h e on both terms, and d((Jp - 1) Jp)/dJp = 2 Jp - 1
  const float jbar = (hardens ? -M.hardening * e * (2.f * M.mu0 * pg + M.lambda0 * ((Jp - 1.f) * Jp) * trb) : 0.f) +
                     M.lambda0 * e * (2.f * Jp - 1.f) * trb;
  // F adjoint of G(F) = (F - R) F^T with Gbar = 2 mu PFb
  float Gb[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) Gb[r][c] = 2.f * mu * PFb[r][c];
  float Fb[3][3], Rb[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float gf = 0.f, gtf = 0.f, gtr = 0.f;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        gf += Gb[r][q] * F[q][c];
        gtf += Gb[q][r] * F[q][c];
        gtr += Gb[q][r] * R[q][c];
      }
      Fb[r][c] = gf + gtf - gtr;
      Rb[r][c] = -gf;
    }
  // polar adjoint
  float Kr[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) Kr[r][c] = R[0][r] * Rb[0][c] + R[1][r] * Rb[1][c] + R[2][r] * Rb[2][c];
  const float kv[3] = {Kr[2][1] - Kr[1][2], Kr[0][2] - Kr[2][0], Kr[1][0] - Kr[0][1]};
  float Sp[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) Sp[r][c] = R[0][r] * F[0][c] + R[1][r] * F[1][c] + R[2][r] * F[2][c];
  const float tr = Sp[0][0] + Sp[1][1] + Sp[2][2];
  float T[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) T[r][c] = (r == c ? tr : 0.f) - 0.5f * (Sp[r][c] + Sp[c][r]);
  // y = T^-1 k by the adjugate
  const float det = det3(T);
  float y[3] = {0.f, 0.f, 0.f};
  if (fabsf(det) > 1e-30f) {
    float adj[3][3];
    adj[0][0] = T[1][1] * T[2][2] - T[1][2] * T[2][1];
    adj[0][1] = T[0][2] * T[2][1] - T[0][1] * T[2][2];
    adj[0][2] = T[0][1] * T[1][2] - T[0][2] * T[1][1];
    adj[1][0] = T[1][2] * T[2][0] - T[1][0] * T[2][2];
    adj[1][1] = T[0][0] * T[2][2] - T[0][2] * T[2][0];
    adj[1][2] = T[0][2] * T[1][0] - T[0][0] * T[1][2];
    adj[2][0] = T[1][0] * T[2][1] - T[1][1] * T[2][0];
    adj[2][1] = T[0][1] * T[2][0] - T[0][0] * T[2][1];
    adj[2][2] = T[0][0] * T[1][1] - T[0][1] * T[1][0];
    const float id = 1.f / det;
#pragma unroll
    for (int r = 0; r < 3; ++r) y[r] = id * (adj[r][0] * kv[0] + adj[r][1] * kv[1] + adj[r][2] * kv[2]);
  }
  float Y[3][3];
  cross_mat(y, Y);
#pragma unroll
  for (int r = 0; r < 3; ++r)
#pragma unroll
    for (int c = 0; c < 3; ++c) Fb[r][c] += R[r][0] * Y[0][c] + R[r][1] * Y[1][c] + R[r][2] * Y[2][c];
  // the adjoint of state_n (x and F add to the G2P parts)
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    ax[q] += xb[q];
    av[q] = vb[q];
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    aC[q / 3][q % 3] = m * Ab[q / 3][q % 3];
    aF[q / 3][q % 3] += Fb[q / 3][q % 3];
  }
  aJp += jbar;
  return true;
}

// Block reduction of the parameter gradients into A.pgrad (every thread of the block calls it).
template <int WARPS>
__device__ __forceinline__ void reduce_pgrad(const AdjArgs& A, double mubar, double lambar) {
  __shared__ double red[2][WARPS];
  for (int o = 16; o; o >>= 1) {
    mubar += __shfl_xor_sync(kFull, mubar, o);
    lambar += __shfl_xor_sync(kFull, lambar, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    red[0][warp] = mubar;
    red[1][warp] = lambar;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a0 = 0.0, a1 = 0.0;
    for (int q = 0; q < WARPS; ++q) {
      a0 += red[0][q];
      a1 += red[1][q];
    }
    atomicAdd(A.pgrad, a0);
    atomicAdd(A.pgrad + 1, a1);
  }
}

// The P2G part of substep n alone (the first substep of a segment): A.a holds the G2P-part
// adjoints of state_n's x, F and Jp; it ends with the full adjoint of state_n.
__global__ void __launch_bounds__(kAdjP2GWarps * 32, kAdjP2GBlocksPerSM) adj_p2g_kernel(const AdjArgs A) {
  double mubar = 0.0, lambar = 0.0;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < A.n; p += (int64_t)gridDim.x * blockDim.x) {
    float ax[3], av[3], aC[3][3], aF[3][3], aJp;
    load_adjoint(A, p, ax, av, aC, aF, aJp);
    if (p2g_adjoint(A, p, ax, av, aC, aF, aJp, mubar, lambar)) store_adjoint(A, p, ax, av, aC, aF, aJp);
  }
  reduce_pgrad<kAdjP2GWarps>(A, mubar, lambar);
}

// P2G part of substep n (An) and G2P part of substep n - 1 (Ap, the substep before) in one
// pass per particle: the adjoint of the particle's state_n stays in registers between them.
// A.a holds the G2P-part adjoints of state_n's x, F and Jp on entry and those of
// state_{n-1} on exit (the whole adjoint where the particle is outside the domain).
__global__ void __launch_bounds__(kAdjG2PWarps * 32, kAdjG2PBlocksPerSM) adj_step_kernel(const AdjArgs An,
                                                                                         const AdjArgs Ap) {
  extern __shared__ float4 smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float4* wbuf = smem + warp * kRedFloat4;
  const int64_t st = An.stride;
  const int64_t nsteps = (An.n + 31) / 32;
  double mubar = 0.0, lambar = 0.0;
  for (int64_t ws = (int64_t)blockIdx.x * kAdjG2PWarps + warp; ws < nsteps; ws += (int64_t)gridDim.x * kAdjG2PWarps) {
    const int64_t p = ws * 32 + lane;
    int key = -1;
    if (p < An.n) {
      float ax[3], av[3], aC[3][3], aF[3][3], aJp;
#pragma unroll
      for (int q = 0; q < 3; ++q) ax[q] = ld(An.a, st, kX + q, p);
#pragma unroll
      for (int q = 0; q < 9; ++q) aF[q / 3][q % 3] = ld(An.a, st, kF + q, p);
      aJp = ld(An.a, st, kJp, p);
      if (!p2g_adjoint(An, p, ax, av, aC, aF, aJp, mubar, lambar)) {
        // outside at state_n: the stored adjoint passes through whole
#pragma unroll
        for (int q = 0; q < 3; ++q) av[q] = ld(An.a, st, kV + q, p);
#pragma unroll
        for (int q = 0; q < 9; ++q) aC[q / 3][q % 3] = ld(An.a, st, kC + q, p);
      }
      float gx[3], Fa[3][3], jo;
      if (g2p_adjoint(Ap, p, lane, wbuf, ax, av, aC, aF, aJp, gx, Fa, jo, key)) {
#pragma unroll
        for (int q = 0; q < 3; ++q) An.a[(kX + q) * st + p] = gx[q];
#pragma unroll
        for (int q = 0; q < 9; ++q) An.a[(kF + q) * st + p] = Fa[q / 3][q % 3];
        An.a[kJp * st + p] = jo;
      } else {
        store_adjoint(An, p, ax, av, aC, aF, aJp);  // outside at state_{n-1}
      }
    }
    if (__ballot_sync(kFull, key >= 0)) warp_scatter_runs(wbuf, lane, key, Ap.gvel, Ap.K.N);
  }
  reduce_pgrad<kAdjG2PWarps>(An, mubar, lambar);
}

}  // namespace mpm

using namespace mpm;

struct mpm_diff {
  mpm_params params{};
  mpm_material material{};
  SimConsts K{};
  int64_t n = 0, stride = 0;
  int ckpt_every = 16, max_steps = 0, nsteps = 0;
  int num_sms = 1;
  cudaStream_t stream = nullptr;
  float* ckpt = nullptr;       // (max_steps / ckpt_every + 1) states
  float* seg = nullptr;        // (ckpt_every + 1) states
  float4* seg_grid = nullptr;  // ckpt_every P2G grids
  float* seg_rot = nullptr;     // ckpt_every x 9 components: the polar rotation of each P2G
  float4* grid3 = nullptr;     // 3 rotating grids for the forward run
  float4* vgrid = nullptr;      // grid velocities of the adjoint kernels
  float4* step_vgrid = nullptr; // padded velocity grid of the forward substep kernels
  VelocityGrid vel;
  float4* gadj = nullptr;       // grid-velocity adjoint
  float4* gmom = nullptr;       // grid (m v, m) adjoints
  float* adj = nullptr;
  double* pgrad = nullptr;
  float* stage = nullptr;
  uint32_t* id = nullptr;   // slot q holds particle id[q] (the cell order of the initial state)
  uint32_t* inv = nullptr;  // particle p sits in slot inv[p]
  // cell sort of the initial positions (keys, counts, scan block sums, a check flag)
  uint32_t* keys = nullptr;
  int* counts = nullptr;
  int* block_sums = nullptr;
  int* bad = nullptr;
  int64_t sort_keys = 0;
  int* status = nullptr;
  int64_t cells = 0;
  // a full segment of the backward (recompute and adjoint substeps) as a CUDA graph: every
  // full segment launches the same kernels on the same buffers; dropped when the material
  // changes (its constants are kernel parameters)
  cudaGraphExec_t seg_graph = nullptr;
  std::string last_error;
};

namespace {

size_t state_floats(const mpm_diff* d) { return (size_t)kNumComps * d->stride; }

mpm_status dlaunch(mpm_diff* d, StepKind kind, float* state, const float4* gin, float4* gout,
                   float4* gzero = nullptr, float* state_out = nullptr, float* rot = nullptr) {
  StepArgs a{};
  a.s = state;
  a.s_out = state_out;
  a.rot = rot;
  a.stride = d->stride;
  a.mat = nullptr;
  a.id = d->id;
  a.n = d->n;
  a.grid_in = gin;
  a.grid_out = gout;
  a.grid_zero = gzero;
  a.grid_cells = d->cells;
  set_vgrid(a, d->vel);
  a.status = d->status;
  a.K = d->K;
  int chunk = 0, blocks = 0;
  step_launch_shape(d->num_sms, d->n, false, false, kind, 2, chunk, blocks);
  a.chunk = chunk;
  if (launch_step(a, kind, false, false, blocks, d->stream, nullptr, StepTuning{kStepWarps, 0}, &d->vel) != cudaSuccess)
    return MPM_ERR_CUDA;
  return MPM_OK;
}

// Recomputes a segment of len substeps from the state in states[0], keeping every state
// (states + j * sf) and every P2G grid (grids + j * cells, the first one cleared
// beforehand): P2G of the first state, then fused launches (G2P of substep j into state
// j + 1, out of place, and P2G of j + 1, clearing the grid after), then the last G2P.
// Each P2G also keeps the polar rotation of its F in rots + j * 9 * stride.
mpm_status recompute_segment(mpm_diff* d, float* states, float4* grids, float* rots, int len) {
  const size_t sf = state_floats(d);
  auto state = [&](int j) { return states + sf * j; };
  auto grid = [&](int j) { return j < len ? grids + d->cells * j : nullptr; };
  auto rot = [&](int j) { return rots + (size_t)9 * d->stride * j; };
  mpm_status st = dlaunch(d, kStepP2GOnly, state(0), nullptr, grid(0), grid(1), nullptr, rot(0));
  for (int j = 0; j + 1 < len && st == MPM_OK; ++j)
    st = dlaunch(d, kStepFused, state(j), grid(j), grid(j + 1), grid(j + 2), state(j + 1), rot(j + 1));
  if (st != MPM_OK) return st;
  return dlaunch(d, kStepG2POnly, state(len - 1), grid(len - 1), nullptr, nullptr, state(len));
}

// One warp per 32 particles, blocks of `warps` warps, at most 8 rounds of the resident blocks
// (the kernels loop over the rest).
int adj_blocks(const mpm_diff* d, int warps, int per_sm) {
  const int64_t need = ((d->n + 31) / 32 + warps - 1) / warps;
  return (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)d->num_sms * per_sm * 8));
}

}  // namespace

extern "C" {

mpm_status mpm_diff_create(const mpm_params* params, const mpm_material* material, int64_t n, int32_t max_steps,
                           int32_t checkpoint_every, mpm_diff** out) {
  if (!params || !material || !out || n <= 0 || max_steps <= 0 || checkpoint_every <= 0) return MPM_ERR_INVALID;
  if (material->kind != MPM_MAT_FIXED_COROTATED && material->kind != MPM_MAT_SNOW) return MPM_ERR_UNSUPPORTED;
  if (params->N < 4 || params->N > 1000 || !(params->dt > 0.f) || params->g2p_guard) return MPM_ERR_INVALID;
  *out = nullptr;
  mpm_diff* d = new mpm_diff();
  d->params = *params;
  d->material = *material;
  make_sim_consts(*params, material, 1, d->K);
  d->n = n;
  d->stride = (n + 63) / 64 * 64;
  d->ckpt_every = checkpoint_every;
  d->max_steps = max_steps;
  d->cells = (int64_t)params->N * params->N * params->N;
  int dev = 0;
  const size_t sf = state_floats(d) * sizeof(float);
  const int nck = max_steps / checkpoint_every + 2;
  if (cudaGetDevice(&dev) || cudaDeviceGetAttribute(&d->num_sms, cudaDevAttrMultiProcessorCount, dev) ||
      cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking) || cudaMalloc(&d->ckpt, sf * nck) ||
      cudaMalloc(&d->seg, sf * (checkpoint_every + 1)) ||
      cudaMalloc(&d->seg_grid, sizeof(float4) * d->cells * checkpoint_every) ||
      cudaMalloc(&d->seg_rot, sizeof(float) * 9 * d->stride * checkpoint_every) ||
      cudaMalloc(&d->grid3, sizeof(float4) * d->cells * 3) || cudaMalloc(&d->vgrid, sizeof(float4) * d->cells) ||
      cudaMalloc(&d->gadj, sizeof(float4) * d->cells) || cudaMalloc(&d->gmom, sizeof(float4) * d->cells) ||
      cudaMalloc(&d->adj, sf) ||
      cudaMalloc(&d->pgrad, 2 * sizeof(double)) || cudaMalloc(&d->stage, sf) ||
      cudaMalloc(&d->id, sizeof(uint32_t) * d->stride) || cudaMalloc(&d->inv, sizeof(uint32_t) * d->stride) ||
      cudaMalloc(&d->keys, sizeof(uint32_t) * d->stride) || cudaMalloc(&d->bad, sizeof(int)) ||
      cudaMalloc(&d->status, sizeof(int)) ||
      cudaMemset(d->status, 0, sizeof(int)) || cudaMemset(d->ckpt, 0, sf * nck) || cudaMemset(d->seg, 0, sf) ||
      cudaMemset(d->adj, 0, sf) ||
      cudaMalloc(&d->step_vgrid, sizeof(float4) * vgrid_nodes((int)params->N))) {
    mpm_diff_destroy(d);
    return MPM_ERR_NOMEM;
  }
  {
    const int64_t nb = (params->N + 3) / 4;
    d->sort_keys = nb * nb * nb * 64;
    const int64_t per = 256 * 8;  // counts per block of the blocked scan
    if (cudaMalloc(&d->counts, sizeof(int) * d->sort_keys) ||
        cudaMalloc(&d->block_sums, sizeof(int) * std::max<int64_t>((d->sort_keys + per - 1) / per, 1))) {
      mpm_diff_destroy(d);
      return MPM_ERR_NOMEM;
    }
  }
  if (vgrid_bind(d->vel, d->step_vgrid, (int)params->N) != cudaSuccess) {
    mpm_diff_destroy(d);
    return MPM_ERR_CUDA;
  }
  if (launch_iota(d->id, n, d->stream) != cudaSuccess) {
    mpm_diff_destroy(d);
    return MPM_ERR_CUDA;
  }
  *out = d;
  return MPM_OK;
}

mpm_status mpm_diff_destroy(mpm_diff* d) {
  if (!d) return MPM_ERR_INVALID;
  if (d->stream) cudaStreamSynchronize(d->stream);
  if (d->seg_graph) cudaGraphExecDestroy(d->seg_graph);
  for (void* p : {(void*)d->ckpt, (void*)d->seg, (void*)d->seg_grid, (void*)d->seg_rot, (void*)d->grid3, (void*)d->vgrid,
                  (void*)d->step_vgrid, (void*)d->gadj, (void*)d->gmom, (void*)d->adj, (void*)d->pgrad, (void*)d->stage, (void*)d->id,
                  (void*)d->inv, (void*)d->keys, (void*)d->counts, (void*)d->block_sums, (void*)d->bad,
                  (void*)d->status})
    cudaFree(p);
  if (d->stream) cudaStreamDestroy(d->stream);
  delete d;
  return MPM_OK;
}

mpm_status mpm_diff_set_material(mpm_diff* d, const mpm_material* material) {
  if (!d || !material) return MPM_ERR_INVALID;
  if (material->kind != MPM_MAT_FIXED_COROTATED && material->kind != MPM_MAT_SNOW) return MPM_ERR_UNSUPPORTED;
  if (material->kind != d->material.kind) return MPM_ERR_INVALID;  // the recompute needs the same model
  d->material = *material;
  make_sim_consts(d->params, material, 1, d->K);
  if (d->seg_graph) {
    cudaStreamSynchronize(d->stream);
    cudaGraphExecDestroy(d->seg_graph);
    d->seg_graph = nullptr;
  }
  return MPM_OK;
}

// Forward run of nsteps substeps from the host state (interleaved x[3n], v[3n], C[9n],
// F[9n], Jp[n]); keeps a checkpoint every checkpoint_every substeps.  The final state
// goes to the host arrays given (any may be NULL).
mpm_status mpm_diff_forward(mpm_diff* d, const float* x0, const float* v0, const float* C0, const float* F0,
                            const float* Jp0, int32_t nsteps, float* x_out, float* v_out) {
  if (!d || !x0 || nsteps <= 0 || nsteps > d->max_steps) return MPM_ERR_INVALID;
  const int64_t n = d->n;
  float* xs = d->stage;
  float* vs = xs + 3 * n;
  float* Cs = vs + 3 * n;
  float* Fs = Cs + 9 * n;
  float* Js = Fs + 9 * n;
  cudaStream_t s = d->stream;
  if (cudaMemcpyAsync(xs, x0, 12 * n, cudaMemcpyHostToDevice, s) ||
      (v0 && cudaMemcpyAsync(vs, v0, 12 * n, cudaMemcpyHostToDevice, s)) ||
      (C0 && cudaMemcpyAsync(Cs, C0, 36 * n, cudaMemcpyHostToDevice, s)) ||
      (F0 && cudaMemcpyAsync(Fs, F0, 36 * n, cudaMemcpyHostToDevice, s)) ||
      (Jp0 && cudaMemcpyAsync(Js, Jp0, 4 * n, cudaMemcpyHostToDevice, s)))
    return MPM_ERR_CUDA;
  // The particles run in the cell order of their initial positions (as a context's periodic
  // sort keeps them): P2G then merges a warp's contributions per cell and the gathers stay
  // local.  id / inv map between that order and the caller's; over one run the particles
  // move a fraction of a cell, so the order is kept to its end.
  SortArgs so{};
  so.n = n;
  so.keys = d->keys;
  so.perm = d->id;
  so.counts = d->counts;
  so.block_sums = d->block_sums;
  so.cells = d->sort_keys;
  so.N = (int)d->params.N;
  so.dx_inv = d->K.g.dx_inv;
  if (launch_presort(xs, nullptr, so, d->inv, d->bad, d->num_sms, s, nullptr) != cudaSuccess) return MPM_ERR_CUDA;
  const HostArrays staged{xs, v0 ? vs : nullptr, C0 ? Cs : nullptr, F0 ? Fs : nullptr, Jp0 ? Js : nullptr};
  if (launch_deinterleave_arrays(staged, d->ckpt, d->stride, n, d->bad, s, d->inv) != cudaSuccess)
    return MPM_ERR_CUDA;
  // work copy of the state; fused launches with three rotating grids, checkpoints copied out
  const size_t sb = state_floats(d) * sizeof(float);
  float* work = d->seg;
  if (cudaMemcpyAsync(work, d->ckpt, sb, cudaMemcpyDeviceToDevice, s)) return MPM_ERR_CUDA;
  if (cudaMemsetAsync(d->grid3, 0, sizeof(float4) * d->cells * 3, s)) return MPM_ERR_CUDA;
  float4* g[3] = {d->grid3, d->grid3 + d->cells, d->grid3 + 2 * d->cells};
  int cur = 0;
  mpm_status st = dlaunch(d, kStepP2GOnly, work, nullptr, g[1]);
  if (st != MPM_OK) return st;
  cur = 1;
  for (int32_t i = 0; i < nsteps; ++i) {
    // fused: G2P of substep i from g[cur], P2G of i+1 into g[cur+1], clear g[cur+2]
    StepArgs a{};
    a.s = work;
    a.stride = d->stride;
    a.id = d->id;
    a.n = n;
    a.grid_in = g[cur];
    a.grid_out = g[(cur + 1) % 3];
    a.grid_zero = g[(cur + 2) % 3];
    a.grid_cells = d->cells;
    set_vgrid(a, d->vel);
    a.status = d->status;
    a.K = d->K;
    int chunk = 0, blocks = 0;
    step_launch_shape(d->num_sms, n, false, false, kStepFused, 2, chunk, blocks);
    a.chunk = chunk;
    if (launch_step(a, kStepFused, false, false, blocks, s, nullptr, StepTuning{kStepWarps, 0}, &d->vel) != cudaSuccess)
      return MPM_ERR_CUDA;
    cur = (cur + 1) % 3;
    if ((i + 1) % d->ckpt_every == 0 && i + 1 < nsteps)
      if (cudaMemcpyAsync(d->ckpt + state_floats(d) * ((i + 1) / d->ckpt_every), work, sb, cudaMemcpyDeviceToDevice,
                          s))
        return MPM_ERR_CUDA;
  }
  d->nsteps = nsteps;
  if (x_out || v_out) {
    // back to the caller's order
    if (launch_interleave(work, d->stride, d->inv, n, d->stage, 0, kFieldX | kFieldV, s) != cudaSuccess)
      return MPM_ERR_CUDA;
    if (x_out && cudaMemcpyAsync(x_out, d->stage, 12 * n, cudaMemcpyDeviceToHost, s)) return MPM_ERR_CUDA;
    if (v_out && cudaMemcpyAsync(v_out, d->stage + 3 * n, 12 * n, cudaMemcpyDeviceToHost, s)) return MPM_ERR_CUDA;
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) return MPM_ERR_CUDA;
  return MPM_OK;
}

// Backward pass of the last forward run.  Inputs: dL/dx and dL/dv of the final state
// (host, interleaved; either may be NULL for zero).  Outputs (host, any may be NULL):
// dL/d of the initial x, v, C, F and dL/dmu0, dL/dlambda0 of the material.
mpm_status mpm_diff_backward(mpm_diff* d, const float* gx_final, const float* gv_final, float* gx0, float* gv0,
                             float* gC0, float* gF0, double* gmu_glambda) {
  if (!d || d->nsteps <= 0) return MPM_ERR_INVALID;
  const int64_t n = d->n;
  cudaStream_t s = d->stream;
  const size_t sf = state_floats(d);
  const size_t sb = sf * sizeof(float);
  float* xs = d->stage;
  float* vs = xs + 3 * n;
  if (cudaMemsetAsync(d->stage, 0, sb, s) || cudaMemsetAsync(d->pgrad, 0, 2 * sizeof(double), s) ||
      (gx_final && cudaMemcpyAsync(xs, gx_final, 12 * n, cudaMemcpyHostToDevice, s)) ||
      (gv_final && cudaMemcpyAsync(vs, gv_final, 12 * n, cudaMemcpyHostToDevice, s)))
    return MPM_ERR_CUDA;
  // adjoint state = (gx, gv, 0, 0, 0) in the run's cell order; the stage holds interleaved
  // x, v, C, F, Jp slots (all read, so no component takes a rest value)
  {
    float* Cz = vs + 3 * n;
    float* Fz = Cz + 9 * n;
    const HostArrays g{xs, vs, Cz, Fz, Fz + 9 * n};
    if (launch_deinterleave_arrays(g, d->adj, d->stride, n, d->bad, s, d->inv) != cudaSuccess) return MPM_ERR_CUDA;
  }
  const int nseg = (d->nsteps + d->ckpt_every - 1) / d->ckpt_every;
  AdjArgs A{};
  A.stride = d->stride;
  A.n = n;
  A.a = d->adj;
  A.gvel = d->gadj;
  A.gmom = d->gmom;
  A.vgrid = d->vgrid;
  A.pgrad = d->pgrad;
  A.K = d->K.g;
  A.M = d->K.mat[0];
  const int g2p_blocks = adj_blocks(d, kAdjG2PWarps, kAdjG2PBlocksPerSM);
  const int p2g_blocks = adj_blocks(d, kAdjP2GWarps, kAdjP2GBlocksPerSM);
  const size_t smem = (size_t)kAdjG2PWarps * kRedFloat4 * sizeof(float4);
  if (cudaFuncSetAttribute(adj_g2p_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) ||
      cudaFuncSetAttribute(adj_g2p_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100) ||
      cudaFuncSetAttribute(adj_step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) ||
      cudaFuncSetAttribute(adj_step_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100))
    return MPM_ERR_CUDA;
  const int gblocks = (int)std::min<int64_t>((d->cells + 255) / 256, 4096);
  // one segment after its checkpoint is in d->seg: recompute it, keeping every state and P2G
  // grid, then the adjoint substeps in reverse
  auto segment = [&](int len) -> mpm_status {
    if (cudaMemsetAsync(d->seg_grid, 0, sizeof(float4) * d->cells, s)) return MPM_ERR_CUDA;
    mpm_status st = recompute_segment(d, d->seg, d->seg_grid, d->seg_rot, len);
    if (st != MPM_OK) return st;
    auto args = [&](int j) {
      AdjArgs a = A;
      a.s = d->seg + sf * j;
      a.s1 = d->seg + sf * (j + 1);
      a.grid = d->seg_grid + d->cells * j;
      a.rot = d->seg_rot + (size_t)9 * d->stride * j;
      return a;
    };
    // the G2P part of the last substep, then per substep the grid-op adjoint and the fused
    // P2G part of substep j with the G2P part of j - 1; the P2G part of substep 0 alone
    const AdjArgs last = args(len - 1);
    adj_velocity_kernel<<<gblocks, 256, 0, s>>>(last.grid, d->vgrid, d->gadj, A.K);
    adj_g2p_kernel<<<g2p_blocks, kAdjG2PWarps * 32, smem, s>>>(last);
    for (int j = len - 1; j >= 0; --j) {
      const AdjArgs An = args(j);
      adj_gridop_kernel<<<gblocks, 256, 0, s>>>(An.grid, d->gadj, d->gmom, j > 0 ? An.grid - d->cells : nullptr,
                                                d->vgrid, A.K);
      if (j > 0)
        adj_step_kernel<<<g2p_blocks, kAdjG2PWarps * 32, smem, s>>>(An, args(j - 1));
      else
        adj_p2g_kernel<<<p2g_blocks, kAdjP2GWarps * 32, 0, s>>>(An);
      if (cudaGetLastError() != cudaSuccess) return MPM_ERR_CUDA;
    }
    return MPM_OK;
  };
  bool warmed = d->seg_graph != nullptr;  // the first full segment runs eagerly (kernel set-up)
  for (int sgi = nseg - 1; sgi >= 0; --sgi) {
    const int s0 = sgi * d->ckpt_every;
    const int len = std::min(d->ckpt_every, d->nsteps - s0);
    if (cudaMemcpyAsync(d->seg, d->ckpt + sf * sgi, sb, cudaMemcpyDeviceToDevice, s)) return MPM_ERR_CUDA;
    if (len < d->ckpt_every || !warmed) {
      const mpm_status st = segment(len);
      if (st != MPM_OK) return st;
      warmed = warmed || len == d->ckpt_every;
      continue;
    }
    if (!d->seg_graph) {
      cudaGraph_t g = nullptr;
      if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) return MPM_ERR_CUDA;
      const mpm_status st = segment(len);
      const cudaError_t e = cudaStreamEndCapture(s, &g);
      if (st != MPM_OK || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return st != MPM_OK ? st : MPM_ERR_CUDA;
      }
      const cudaError_t ei = cudaGraphInstantiate(&d->seg_graph, g, 0);
      cudaGraphDestroy(g);
      if (ei != cudaSuccess) {
        d->seg_graph = nullptr;
        return MPM_ERR_CUDA;
      }
    }
    if (cudaGraphLaunch(d->seg_graph, s)) return MPM_ERR_CUDA;
  }
  // out: adjoint of the initial state, host interleaved, in the caller's order
  if (launch_interleave(d->adj, d->stride, d->inv, n, d->stage, 0, kFieldAll, s) != cudaSuccess) return MPM_ERR_CUDA;
  float* Cs = vs + 3 * n;
  float* Fs = Cs + 9 * n;
  if ((gx0 && cudaMemcpyAsync(gx0, xs, 12 * n, cudaMemcpyDeviceToHost, s)) ||
      (gv0 && cudaMemcpyAsync(gv0, vs, 12 * n, cudaMemcpyDeviceToHost, s)) ||
      (gC0 && cudaMemcpyAsync(gC0, Cs, 36 * n, cudaMemcpyDeviceToHost, s)) ||
      (gF0 && cudaMemcpyAsync(gF0, Fs, 36 * n, cudaMemcpyDeviceToHost, s)) ||
      (gmu_glambda && cudaMemcpyAsync(gmu_glambda, d->pgrad, 2 * sizeof(double), cudaMemcpyDeviceToHost, s)))
    return MPM_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return MPM_ERR_CUDA;
  return MPM_OK;
}

}  // extern "C"
