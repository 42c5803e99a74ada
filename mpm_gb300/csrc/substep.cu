// Fused MLS-MPM substep kernels for sm_103a.
//
// The reference runs four launches per substep (src/mpm.cu:323-329): cudaMemset of
// the grid, particleToGrid (27 x 4 float atomics per particle), gridOpKernel, and
// gridToParticle.  Here a substep is
//   a velocity pass: the grid operation applied once per node of the P2G grid of
//                    substep n, written to a zero-padded velocity grid, and
//   one fused launch: G2P of substep n from the velocity grid
//                     + constitutive update + advection, state written once
//                     + P2G of substep n+1 (scatter of the new state)
//                     + clearing of the grid buffer substep n-1 read,
// so particle state is read once and written once per substep and the three P2G
// grid buffers rotate.  A P2G-only variant starts a run from uploaded state.
//
// Work decomposition: warps are the scheduling unit.  Each warp of a 12-warp CTA
// takes a range of cell-sorted particles (steps_per_warp x 32) and walks it 32
// particles at a time (lane = particle, coalesced component-major loads/stores).  A
// CTA owns every G-th range (G = grid size); its warps take them in turn from a
// shared-memory counter, so faster warps take more without global atomics (one
// global counter serialised 15k claims per launch at a single L2 slice).
//
// G2P reads a per-step tile of the velocity grid in shared memory: a fixed box of
// 4 x 4 x 6 nodes that one TMA copy (cp.async.bulk.tensor, completion on an mbarrier)
// loads.  The copy for step k+1 is issued during step k, from positions loaded one
// step ahead, into the other of two buffers, so its latency hides behind the
// update and P2G of step k.  The box covers every step whose base cells span at most
// 2 x 2 x 4 cells (one cell in dense scenes, or two neighbours in the bricked sort
// order); other steps gather straight from the velocity grid.
//
// P2G is a warp transpose-reduce: every lane writes its 27 node contributions as a
// column of a per-warp buffer, and lane l < 27 sums node l over each run of same-cell
// lanes and issues one vector atomic per run.  Dense scenes (100+ particles per cell)
// thus issue about one global atomic per node and step instead of the reference's 108
// per particle.
//
// Batches of scenes (batch.cu) use batch_step_kernel below: per-range scene constants,
// a velocity pass over each scene's recorded P2G box, sparse grid clearing.
#include <cudaTypedefs.h>

#include <algorithm>
#include <climits>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "substep_kernel.cuh"

namespace mpm {

// ===========================================================================
// Single scene
// ===========================================================================

// gridOpKernel (src/mpm.cu:76-107) for every node, into the padded velocity grid;
// padding nodes get zeros.
// The substep kernel is launched as its programmatic dependent: it may start (claim
// ranges, load its first positions) while this pass runs, and waits for the pass
// with griddepcontrol.wait before it reads the velocity grid.
// One thread per padded node, in the padded grid's order (consecutive threads take
// consecutive k), so every warp is full: a block per padded row left most of each block's
// threads idle (69 of 128 at N = 64).  Padded grids stay below 2^31 nodes (N <= 1000).
__global__ void grid_velocity_kernel(const float4* __restrict__ grid, float4* __restrict__ vgrid, GridConsts K) {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  const int N = K.N, P = N + kPadLo + kPadHi;
  const int q = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (q >= P * P * P) return;
  const int pi = q / (P * P), rem = q - pi * (P * P);
  const int pj = rem / P, pk = rem - pj * P;
  const int i = pi - kPadLo, j = pj - kPadLo, k = pk - kPadLo;
  float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
  if ((unsigned)i < (unsigned)N && (unsigned)j < (unsigned)N && (unsigned)k < (unsigned)N) {
    const float3 v = grid_node_velocity(grid[(i * N + j) * N + k], i, j, k, K);
    out = make_float4(v.x, v.y, v.z, 0.f);
  }
  vgrid[q] = out;
}

// ===========================================================================
// Batch of scenes
// ===========================================================================

// Velocity pass of a batch (blockIdx.y = scene): the grid op over the nodes of the
// scene's last recorded P2G box, [lo, hi + 2] in each dimension (the stencils of the
// particles whose P2G recorded it), zero where the node is outside the grid.
__global__ void batch_velocity_kernel(const float4* __restrict__ grid, float4* __restrict__ vgrid,
                                      const SceneDev* __restrict__ scenes, const int* __restrict__ boxes, int slot) {
  const int sc = blockIdx.y;
  const SceneDev& sd = scenes[sc];
  const int N = sd.g.N, P = N + kPadLo + kPadHi;
  const int* bx = boxes + ((int64_t)sc * kBoxSlots + slot) * 6;
  const int l0 = max(bx[0], -kPadLo), l1 = max(bx[1], -kPadLo), l2 = max(bx[2], -kPadLo);
  const int h0 = min(bx[3] + 2, N + kPadHi - 1), h1 = min(bx[4] + 2, N + kPadHi - 1),
            h2 = min(bx[5] + 2, N + kPadHi - 1);
  if (h0 < l0 || h1 < l1 || h2 < l2) return;
  const int e1 = h1 - l1 + 1, e2 = h2 - l2 + 1;
  const int64_t e12 = (int64_t)e1 * e2, vol = (int64_t)(h0 - l0 + 1) * e12;
  const float4* g = grid + sd.grid_offset;
  float4* vg = vgrid + sd.vgrid_offset;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < vol; q += (int64_t)gridDim.x * blockDim.x) {
    const int di = (int)(q / e12);
    const int rem = (int)(q - (int64_t)di * e12);
    const int i = l0 + di, j = l1 + rem / e2, k = l2 + rem % e2;
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    if ((unsigned)i < (unsigned)N && (unsigned)j < (unsigned)N && (unsigned)k < (unsigned)N) {
      const float3 v = grid_node_velocity(g[((int64_t)i * N + j) * N + k], i, j, k, sd.g);
      out = make_float4(v.x, v.y, v.z, 0.f);
    }
    vg[((int64_t)(i + kPadLo) * P + (j + kPadLo)) * P + (k + kPadLo)] = out;
  }
}

// G2P gather from a padded velocity grid through L1 (`base`: the node of the
// particle's base cell), for the batch kernel; out of line to keep its loop small.
static __device__ __noinline__ G2POut g2p_gather_padded(const float4* base, int P, float ddx, float dx_inv, float x0,
                                                        float x1, float x2) {
  const float x[3] = {x0, x1, x2};
  float w[3][3], f[3];
  int b[3];
#pragma unroll
  for (int dim = 0; dim < 3; ++dim)
    QuadraticInterpolationKernel::weights_and_offset(x[dim], dx_inv, b[dim], w[dim], f[dim]);
  auto node = [&](int a, int bb, int c) -> float4 { return __ldg(base + ((int64_t)a * P + bb) * P + c); };
  G2POut o;
  g2p_gather_f(node, ddx, w, f, o.v, o.C);
  return o;
}

// Batched substep: ranges of the range table never cross a scene, so a warp loads its
// scene's constants once per range.  G2P gathers the scene's velocity grid (written by
// batch_velocity_kernel) through L1; each scene's P2G box is recorded so the grid it
// accumulated is cleared sparsely two launches later and the next velocity pass covers it.
template <bool G2P, bool P2G>
__global__ void __launch_bounds__(kStepThreads, 1) batch_step_kernel(const __grid_constant__ StepArgs A) {
  extern __shared__ float4 smem[];
  __shared__ int cta_next;  // next CTA-local range index (ranges c, c + G, ... of CTA c)
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  float4* wbuf = smem + warp * kRedFloat4;
  float* __restrict__ s = A.s;
  const int64_t st = A.stride;

  if (tid == 0) cta_next = kStepWarps;
  // clear, per scene, the grid region the launch two substeps back accumulated (the
  // buffer this launch leaves for the next one to fill), then free its box slot
  for (int sc = blockIdx.x; sc < A.nscenes; sc += gridDim.x) {
    const int* bx = A.boxes + ((int64_t)sc * kBoxSlots + A.box_clear) * 6;
    const SceneDev& sd = A.scenes[sc];
    const int Ns = sd.g.N;
    const int l0 = max(bx[0], 0), l1 = max(bx[1], 0), l2 = max(bx[2], 0);
    const int h0 = min(bx[3] + 2, Ns - 1), h1 = min(bx[4] + 2, Ns - 1), h2 = min(bx[5] + 2, Ns - 1);
    if (h0 >= l0 && h1 >= l1 && h2 >= l2 && A.grid_zero) {
      const int e1 = h1 - l1 + 1, e2 = h2 - l2 + 1;
      const int64_t vol = (int64_t)(h0 - l0 + 1) * e1 * e2;
      float4* gz = A.grid_zero + sd.grid_offset;
      for (int64_t q = tid; q < vol; q += kStepThreads) {
        const int i = l0 + (int)(q / ((int64_t)e1 * e2));
        const int rem = (int)(q % ((int64_t)e1 * e2));
        gz[((int64_t)i * Ns + (l1 + rem / e2)) * Ns + (l2 + rem % e2)] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    if (tid < 6) A.boxes[((int64_t)sc * kBoxSlots + A.box_reset) * 6 + tid] = (tid < 3) ? INT_MAX : INT_MIN;
  }
  __syncthreads();
  const int64_t nranges = A.nranges;
  const int G = (int)gridDim.x;
  int64_t r = (int64_t)blockIdx.x + warp * G;
  while (r < nranges) {
    int claim = 0;
    const int4 rg = A.ranges[r];
    const int scene = rg.x;
    const int64_t wbeg = rg.y, wend = rg.z;
    const SceneDev& sd = A.scenes[scene];
    const GridConsts K = sd.g;
    const int N = K.N;
    const DevMaterial& M = sd.m;
    float4* gout = A.grid_out + sd.grid_offset;
    const float4* vg = A.vgrid + sd.vgrid_offset;
    const int P = N + kPadLo + kPadHi;
    const float ddx = K.dinv * K.dx;
    int plo[3] = {INT_MAX, INT_MAX, INT_MAX}, phi[3] = {INT_MIN, INT_MIN, INT_MIN};

    float nx0 = 0.f, nx1 = 0.f, nx2 = 0.f, nJ = 1.f;
    if (wbeg + lane < wend) {
      nx0 = s[(kX + 0) * st + wbeg + lane];
      nx1 = s[(kX + 1) * st + wbeg + lane];
      nx2 = s[(kX + 2) * st + wbeg + lane];
      nJ = s[kJp * st + wbeg + lane];
    }
    for (int64_t pb = wbeg; pb < wend; pb += 32) {
      const int64_t p = pb + lane;
      const bool valid = p < wend;
      if (pb + 32 >= wend && lane == 0) claim = atomicAdd(&cta_next, 1);
      float x[3] = {nx0, nx1, nx2}, v[3] = {0.f, 0.f, 0.f}, Cm[3][3], F[3][3], Jp = nJ;
      if (p + 32 < wend) {
        nx0 = s[(kX + 0) * st + p + 32];
        nx1 = s[(kX + 1) * st + p + 32];
        nx2 = s[(kX + 2) * st + p + 32];
        nJ = s[kJp * st + p + 32];
      }
      bool frozen = !G2P;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          Cm[i][j] = 0.f;
          F[i][j] = (i == j) ? 1.f : 0.f;
        }
      if (valid) {
#pragma unroll
        for (int i = 0; i < 9; ++i) F[i / 3][i % 3] = s[(kF + i) * st + p];
        if (frozen && P2G) {
#pragma unroll
          for (int dd = 0; dd < 3; ++dd) v[dd] = s[(kV + dd) * st + p];
#pragma unroll
          for (int i = 0; i < 9; ++i) Cm[i / 3][i % 3] = s[(kC + i) * st + p];
        }
      }
      PolarCache pc;
      pc.valid = false;
      bool g2p_on = false;
      if (G2P && valid && !frozen) {
        int b[3];
#pragma unroll
        for (int dd = 0; dd < 3; ++dd) b[dd] = QuadraticInterpolationKernel::base_cell(x[dd], K.dx_inv);
        g2p_on = !outside_domain(b[0], b[1], b[2], N);
        if (!g2p_on) {
          frozen = true;
        } else {
          const G2POut o = g2p_gather_padded(
              vg + ((int64_t)(b[0] + kPadLo) * P + (b[1] + kPadLo)) * P + (b[2] + kPadLo), P, ddx, K.dx_inv, x[0], x[1],
              x[2]);
#pragma unroll
          for (int r2 = 0; r2 < 3; ++r2) {
            v[r2] = o.v[r2];
#pragma unroll
            for (int c = 0; c < 3; ++c) Cm[r2][c] = o.C[r2][c];
          }
        }
      }
      if (g2p_on) {
        particle_update<false>(M, K, x, v, Cm, F, Jp, pc);
        store_particle<false>(s, st, p, x, v, Cm, F, Jp);
        if (A.check_finite && !isfinite(x[0] + x[1] + x[2] + v[0] + v[1] + v[2])) atomicOr(A.status, kStatusNonFinite);
      }
      if (P2G) {
        int key = -1;
        float w[3][3], f[3], E[3][3], q0[3], m = 0.f;
        if (valid) {
          int b[3];
          stencil_f(x, K, b, w, f);
          if (!outside_domain(b[0], b[1], b[2], N)) {
            key = pack_key(b[0], b[1], b[2]);
#pragma unroll
            for (int dd = 0; dd < 3; ++dd) {
              plo[dd] = min(plo[dd], b[dd]);
              phi[dd] = max(phi[dd], b[dd]);
            }
            p2g_prepare_f<false>(M, K, F, Jp, Cm, v, pc, f, E, q0, m);
          }
        }
        // every particle of a scene has the scene's mass: unit-mass columns, each run's
        // summed weight scaled by it (the single-run walk made this larger kernel slower)
        if (__ballot_sync(kFull, key >= 0) != 0u) {
          if (key >= 0) p2g_write_column_f<true>(wbuf, lane, w, q0, E, m);
          warp_scatter_runs<false>(wbuf, lane, key, gout, N, M.mass);
        }
      }
    }
    if (P2G) {
      // record the range's P2G box in its scene's slot (cleared two launches later)
      int* bx = A.boxes + ((int64_t)scene * kBoxSlots + A.box_record) * 6;
#pragma unroll
      for (int dd = 0; dd < 3; ++dd) {
        const int l = __reduce_min_sync(kFull, plo[dd]);
        const int h = __reduce_max_sync(kFull, phi[dd]);
        if (lane == 0 && h >= l) {
          atomicMin(bx + dd, l);
          atomicMax(bx + 3 + dd, h);
        }
      }
    }
    r = (int64_t)blockIdx.x + (int64_t)__shfl_sync(kFull, claim, 0) * G;
  }
}

// ===========================================================================
// Host side
// ===========================================================================

int64_t vgrid_nodes(int N) {
  const int64_t P = (int64_t)N + kPadLo + kPadHi;
  return P * P * P;
}

namespace {

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

}  // namespace

cudaError_t vgrid_bind(VelocityGrid& v, float4* ptr, int N) {
  if (!ptr || N < 1 || (reinterpret_cast<uintptr_t>(ptr) & 15u)) return cudaErrorInvalidValue;
  PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
  if (!encode) return cudaErrorNotSupported;
  // the grid as float32 [P][P][4 P]: one node is 4 consecutive floats
  const cuuint64_t P = (cuuint64_t)N + kPadLo + kPadHi;
  const cuuint64_t dims[3] = {4 * P, P, P};
  const cuuint64_t strides[2] = {16 * P, 16 * P * P};  // bytes, dimensions 1 and 2
  const cuuint32_t estr[3] = {1, 1, 1};
  const cuuint32_t boxes[kTileShapes][3] = {{4 * TileBox<0>::Z, TileBox<0>::Y, TileBox<0>::X},
                                            {4 * TileBox<1>::Z, TileBox<1>::Y, TileBox<1>::X},
                                            {4 * TileBox<2>::Z, TileBox<2>::Y, TileBox<2>::X}};
  for (int t = 0; t < kTileShapes; ++t) {
    const CUresult r = encode(&v.map[t], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, ptr, dims, strides, boxes[t], estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return cudaErrorInvalidValue;
  }
  v.ptr = ptr;
  v.N = N;
  return cudaSuccess;
}

void set_vgrid(StepArgs& a, const VelocityGrid& v, int tile) {
  a.vgrid = v.ptr;
  a.vmap = v.map[(tile >= 0 && tile < kTileShapes) ? tile : 0];
}

cudaError_t launch_batch_velocity(const float4* grid, float4* vgrid, const SceneDev* scenes, int nscenes,
                                  const int* boxes, int slot, cudaStream_t st) {
  if (nscenes <= 0) return cudaSuccess;
  batch_velocity_kernel<<<dim3(16, nscenes), kThreads, 0, st>>>(grid, vgrid, scenes, boxes, slot);
  return cudaGetLastError();
}

// Self-check of the bounded-wait path: one warp waits on an mbarrier that nothing
// arrives on, gives up after `polls` polls and reports kStatusTimeout, as the substep
// kernel does when a tile copy never completes.
__global__ void wait_timeout_probe(int* status, int polls) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_barrier_init();
  }
  __syncwarp();
  if (!mbar_wait(&bar, 0u, polls) && threadIdx.x == 0) atomicOr(status, kStatusTimeout);
}

cudaError_t launch_wait_timeout_probe(int* status, int polls, cudaStream_t st) {
  wait_timeout_probe<<<1, 32, 0, st>>>(status, polls);
  return cudaGetLastError();
}

// Kernels of material policies compiled in by include/mpm_gb300_policies.cuh, by kind.
namespace {
std::mutex& registry_mutex() {
  static std::mutex mu;
  return mu;
}
std::map<int, MaterialKernels>& registry() {
  static std::map<int, MaterialKernels> r;
  return r;
}
}  // namespace

bool register_material_kernels(int kind, const MaterialKernels& k) {
  if (kind < kUserKindBase || kind >= kUserKindEnd || !k.fused || !k.p2g_only || !k.g2p_only) return false;
  std::lock_guard<std::mutex> lock(registry_mutex());
  return registry().emplace(kind, k).second;
}

bool find_material_kernels(int kind, MaterialKernels* out) {
  std::lock_guard<std::mutex> lock(registry_mutex());
  auto it = registry().find(kind);
  if (it == registry().end()) return false;
  if (out) *out = it->second;
  return true;
}

template <bool LIQ, bool G2P, bool P2G, bool GUARD, int WARPS, int TILE = 0>
static void* scene_kernel() {
  return (void*)scene_step_kernel<LIQ, G2P, P2G, GUARD, WARPS, TILE>;
}

StepTuning step_tuning(StepKind kind, bool guard, bool batch, StepTuning want) {
  // The fused substep of the plain layouts comes in every CTA size with tile box 0, and
  // with boxes 1 and 2 at 12 warps; the P2G-only launch of the plain layouts uses
  // kP2GWarps; the G2P-only launch, the G2P-guard variants and batches use 12 warps and
  // box 0.
  StepTuning t{kStepWarps, 0};
  if (!batch && !guard && kind == kStepP2GOnly) return StepTuning{kP2GWarps, 0};
  if (batch || guard || kind != kStepFused) return t;
  if (want.tile == 1 || want.tile == 2) {
    t.tile = want.tile;
    return t;
  }
  if (want.warps == 4 || want.warps == 6) t.warps = want.warps;
  return t;
}

static void* select_kernel(StepKind kind, bool liquid, bool guard, bool batch, StepTuning want) {
  if (batch) {  // batches use the general layout, no guard
    if (kind == kStepP2GOnly) return (void*)batch_step_kernel<false, true>;
    return (void*)batch_step_kernel<true, true>;
  }
  const StepTuning t = step_tuning(kind, guard, batch, want);
  if (kind == kStepFused && !guard) {
    if (t.warps == 4) return liquid ? scene_kernel<true, true, true, false, 4>() : scene_kernel<false, true, true, false, 4>();
    if (t.warps == 6) return liquid ? scene_kernel<true, true, true, false, 6>() : scene_kernel<false, true, true, false, 6>();
    if (t.tile == 1)
      return liquid ? scene_kernel<true, true, true, false, kStepWarps, 1>()
                    : scene_kernel<false, true, true, false, kStepWarps, 1>();
    if (t.tile == 2)
      return liquid ? scene_kernel<true, true, true, false, kStepWarps, 2>()
                    : scene_kernel<false, true, true, false, kStepWarps, 2>();
  }
#define MPM_SEL(L, G)                                                                \
  if (liquid == L && guard == G) {                                                   \
    if (kind == kStepP2GOnly) return scene_kernel<L, false, true, G, G ? kStepWarps : kP2GWarps>(); \
    if (kind == kStepFused) return scene_kernel<L, true, true, G, kStepWarps>();     \
    return scene_kernel<L, true, false, G, kStepWarps>();                            \
  }
  MPM_SEL(true, false)
  MPM_SEL(true, true)
  MPM_SEL(false, false)
  MPM_SEL(false, true)
#undef MPM_SEL
  return nullptr;
}

size_t step_smem_bytes(StepKind kind, bool batch, StepTuning want) {
  size_t b = 0;
  if (batch) return (kind != kStepG2POnly) ? (size_t)kStepWarps * kRedFloat4 * sizeof(float4) : 16;
  const StepTuning t = step_tuning(kind, false, batch, want);
  if (kind != kStepP2GOnly) b += (size_t)t.warps * 2 * (tile_nodes(t.tile) * sizeof(float4) + sizeof(uint64_t));
  if (kind != kStepG2POnly) b += (size_t)t.warps * kRedFloat4 * sizeof(float4);
  return b + 128;  // alignment of the TMA tiles
}

// The kernel's dynamic shared memory limit, set once per kernel, size and device.
cudaError_t prepare_step_kernel(void* fn, size_t smem) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  static std::mutex mu;
  static std::vector<std::tuple<void*, size_t, int>> done;
  std::lock_guard<std::mutex> lock(mu);
  for (const auto& d : done)
    if (std::get<0>(d) == fn && std::get<1>(d) == smem && std::get<2>(d) == dev) return cudaSuccess;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) done.emplace_back(fn, smem, dev);
  return e;
}

cudaError_t launch_step(const StepArgs& a, StepKind kind, bool liquid, bool guard, int grid_blocks, cudaStream_t st,
                        int64_t* launches, StepTuning want, const VelocityGrid* vel) {
  const bool batch = a.nscenes > 0;
  // a single-scene G2P launch reads its tiles with the tensor map of the kernel's box:
  // the map is taken here, from the velocity grid, for the box the launch uses
  if (!batch && kind != kStepP2GOnly && !vel) return cudaErrorInvalidValue;
  void* fn = select_kernel(kind, liquid, guard, batch, want);
  StepTuning t = step_tuning(kind, guard, batch, want);
  const int mkind = a.K.n_materials > 0 ? a.K.mat[0].kind : 0;
  if (!batch && mkind >= kUserKindBase) {
    // a material compiled in through include/mpm_gb300_policies.cuh: its own kernels, in
    // the default launch shape, general layout, no G2P guard
    MaterialKernels mk{};
    if (guard || liquid || !find_material_kernels(mkind, &mk)) return cudaErrorInvalidValue;
    fn = (kind == kStepFused) ? mk.fused : (kind == kStepP2GOnly ? mk.p2g_only : mk.g2p_only);
    t = StepTuning{kStepWarps, 0};
  }
  const int warps = t.warps;
  const size_t smem = step_smem_bytes(kind, batch, t);
  cudaError_t e = prepare_step_kernel(fn, smem);
  if (e != cudaSuccess) return e;
  if (!batch && kind != kStepP2GOnly) {
    if (!vel->ptr || !a.grid_in) return cudaErrorInvalidValue;
    const int P = a.K.g.N + kPadLo + kPadHi;
    const int64_t nodes = (int64_t)P * P * P;
    grid_velocity_kernel<<<(unsigned)((nodes + 255) / 256), 256, 0, st>>>(a.grid_in, vel->ptr, a.K.g);
    if (launches) *launches += 1;
  }
  StepArgs copy = a;
  if (!batch && kind != kStepP2GOnly) set_vgrid(copy, *vel, t.tile);
  void* args[] = {&copy};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid_blocks);
  cfg.blockDim = dim3(batch ? kStepThreads : warps * 32);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  // programmatic dependent launch after the velocity pass (see grid_velocity_kernel)
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = (!batch && kind != kStepP2GOnly) ? 1 : 0;
  e = cudaLaunchKernelExC(&cfg, fn, args);
  if (launches) *launches += 1;
  return e;
}

int step_blocks_per_sm(StepKind kind, bool liquid, bool guard, size_t smem, bool batch, StepTuning want) {
  void* fn = select_kernel(kind, liquid, guard, batch, want);
  const int warps = step_tuning(kind, guard, batch, want).warps;
  if (prepare_step_kernel(fn, smem) != cudaSuccess) return 1;
  // the answer depends on the kernel, its shared memory and the device only: ask once
  int dev = 0;
  cudaGetDevice(&dev);
  static std::mutex mu;
  static std::vector<std::tuple<void*, size_t, int, int>> known;
  std::lock_guard<std::mutex> lock(mu);
  for (const auto& k : known)
    if (std::get<0>(k) == fn && std::get<1>(k) == smem && std::get<2>(k) == dev) return std::get<3>(k);
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, batch ? kStepThreads : warps * 32, smem) != cudaSuccess ||
      nb < 1)
    nb = 1;
  known.emplace_back(fn, smem, dev, nb);
  return nb;
}

}  // namespace mpm
