/*
 * CPU oracle for the MLS-MPM substep — TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain C++ restatement of the reference substep (kekeblom/mpm) used
 * as the checker for the CUDA path. Only tests/, __graft_entry__.smoke() and
 * bench.py's cpu_baseline / --impl reference legs may load it. The product
 * (mpm_gb300/) never links or calls anything in oracle/.
 *
 * Parity pinning: the 3x3 SVD / polar / determinant leaf is pinned by the
 * matrices and tolerances of the reference's own tests (tests/test_linalg.cu)
 * and by the reference's own svd3_cuda.h compiled on the host (oracle/_ref).
 * The substep itself has no golden vectors in the reference; the restated loop
 * structure is pinned against the reference's own policy headers compiled with
 * a project-written Eigen subset (oracle/ref_substep.cpp, oracle/_ref).
 *
 * Layout: SoA-in-AoS per particle, row-major 3x3 matrices:
 *   x[3n], v[3n], C[9n] (C[9p + 3r + c]), F[9n], Jp[n], mat[n] (u8 material index).
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORACLE_MAX_MATERIALS = 16 };

/* Material kinds (shared numbering with the product's C-ABI). */
enum {
  ORACLE_MAT_SNOW = 0,            /* MMSnow (include/MaterialModel.cuh:67-116) */
  ORACLE_MAT_FIXED_COROTATED = 1, /* MMFixedCorotated (include/MaterialModel.cuh:40-62) */
  ORACLE_MAT_JELLY = 2,           /* MMJelly (include/MaterialModel.cuh:119-150) */
  ORACLE_MAT_LIQUID = 3           /* weakly compressible liquid (not in the reference) */
};

/* Boundary rules for the grid operation. */
enum {
  ORACLE_BOUNDARY_REF_FRACTION = 0, /* src/mpm.cu:92-105: idx/N < 0.05 etc. */
  ORACLE_BOUNDARY_STICKY_CELLS = 1, /* all six walls sticky within `boundary_cells` */
  ORACLE_BOUNDARY_SEPARATE_CELLS = 2 /* reference structure, cell-count thickness */
};

typedef struct {
  int kind;
  float particle_volume; /* MaterialModelBase::particleVolume */
  float particle_mass;   /* density * volume, computed in float */
  float mu0, lambda0;    /* Lame parameters, computed in float */
  float hardening;
  float clamp_lo, clamp_hi;
  float bulk;            /* liquid bulk modulus */
} oracle_material;

typedef struct {
  float dt;
  int N;
  float gravity;
  int boundary_mode;
  int boundary_cells;
  int g2p_guard;   /* 1: reproduce src/mpm.cu:114 (only particles 0..N^3 run G2P) */
  int nthreads;    /* OpenMP threads (<=0: all) */
  int n_materials;
  oracle_material materials[ORACLE_MAX_MATERIALS];
} oracle_config;

/* Runs `nsteps` substeps in place. If grid_p2g / grid_op are non-null they
 * receive the last substep's grid after P2G and after the grid operation
 * (N^3 x 4, index N*(N*i+j)+k, components (m*v, m) / post-op values).
 * Returns 0 on success. */
int oracle_substep_f64(const oracle_config* cfg, int64_t n, double* x, double* v, double* C,
                       double* F, double* Jp, const uint8_t* mat, int nsteps,
                       double* grid_p2g, double* grid_op);
int oracle_substep_f32(const oracle_config* cfg, int64_t n, float* x, float* v, float* C,
                       float* F, float* Jp, const uint8_t* mat, int nsteps,
                       float* grid_p2g, float* grid_op);

/* 3x3 SVD: McAdams et al. (UW-Madison TR1690, 2011) in float (4 Jacobi sweeps),
 * exact cyclic Jacobi to convergence in double. A, U, V row-major (9 per matrix),
 * s = 3 singular values (s[2] carries the sign of det A). */
void oracle_svd_f32(int64_t n, const float* A, float* U, float* s, float* V);
void oracle_svd_f64(int64_t n, const double* A, double* U, double* s, double* V);
void oracle_polar_f32(int64_t n, const float* A, float* R, float* S);
void oracle_polar_f64(int64_t n, const double* A, double* R, double* S);
float oracle_det_f32(const float* M);

/* Time `nsteps` FP32 substeps on `nthreads` threads; returns seconds. */
double oracle_time_f32(const oracle_config* cfg, int64_t n, float* x, float* v, float* C,
                       float* F, float* Jp, const uint8_t* mat, int nsteps);

int oracle_max_threads(void);

#ifdef __cplusplus
}
#endif
