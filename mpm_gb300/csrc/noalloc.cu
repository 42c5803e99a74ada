// A substep entry point that allocates nothing.
//
// Some callers cannot call cudaMalloc: plugins loaded into a host application that
// owns all device memory through its own pool, and embedded or real-time callers that
// forbid allocation after start-up (an allocation can block, fail or fragment memory at
// a time they do not choose).  mpm_substep_noalloc serves them: the caller passes the
// particle state in its own device memory, and the only scratch the substep needs (three
// rotating P2G grids, the padded velocity grid and the device status word) lives in the
// file-scope array below, which every GPU that loads this library holds until the
// process exits.  mpm_noalloc_status reads and clears that status word.
#include <mutex>

#include "mpm_internal.h"

namespace {

constexpr int kNoAllocMaxN = 32;  // largest grid the static scratch holds
constexpr int64_t kNoAllocCells = (int64_t)kNoAllocMaxN * kNoAllocMaxN * kNoAllocMaxN;
// the velocity grid is padded to (N + 5)^3 nodes
constexpr int64_t kNoAllocVelNodes = (int64_t)(kNoAllocMaxN + 5) * (kNoAllocMaxN + 5) * (kNoAllocMaxN + 5);
// three grids of kNoAllocCells float4 nodes, the velocity grid, then one float4 whose
// first word is the device status word (kStatus* bits, set by the kernels, kept until
// mpm_noalloc_status clears it):
// (3 x 32768 + 50653 + 1) x 16 B = 2.27 MiB
constexpr int64_t kScratchFloat4 = 3 * kNoAllocCells + kNoAllocVelNodes + 1;

static __device__ __align__(256) float4 g_noalloc_scratch[kScratchFloat4];

// Device address of g_noalloc_scratch per device.  In host code the symbol's name is
// only a host-side stand-in, so the address comes from cudaGetSymbolAddress, taken
// once per device with that device current.
constexpr int kMaxDevices = 64;
float4* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

mpm_status scratch_for_current_device(float4** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return MPM_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return MPM_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_addr[dev]) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return MPM_ERR_CUDA;
    g_scratch_addr[dev] = static_cast<float4*>(ptr);
  }
  *out = g_scratch_addr[dev];
  return MPM_OK;
}

int* status_word(float4* scratch) { return reinterpret_cast<int*>(scratch + 3 * kNoAllocCells + kNoAllocVelNodes); }

}  // namespace

using namespace mpm;

extern "C" mpm_status mpm_substep_noalloc(const mpm_params* params, const mpm_material* materials,
                                          int32_t n_materials, float* state, int64_t stride, const uint8_t* mat,
                                          int64_t n, int32_t nsteps, void* stream) {
  if (!params || !materials || n_materials <= 0 || n_materials > MPM_MAX_MATERIALS) return MPM_ERR_INVALID;
  if (params->N < 4 || params->N > (uint32_t)kNoAllocMaxN) return MPM_ERR_UNSUPPORTED;  // beyond the scratch
  if (!(params->dt > 0.f) || params->boundary_mode < 0 || params->boundary_mode > 2) return MPM_ERR_INVALID;
  if (params->boundary_cells < 0 || (uint32_t)params->boundary_cells * 2 > params->N) return MPM_ERR_INVALID;
  if (params->g2p_guard) return MPM_ERR_UNSUPPORTED;  // needs the original particle indices
  if (n < 0 || nsteps < 0 || (n > 0 && (!state || stride < n))) return MPM_ERR_INVALID;
  for (int i = 0; i < n_materials; ++i)
    if (materials[i].kind < 0 || materials[i].kind > MPM_MAT_LIQUID || !(materials[i].particle_volume > 0.f) ||
        !(materials[i].density > 0.f))
      return MPM_ERR_INVALID;
  if (n == 0 || nsteps == 0) return MPM_OK;

  float4* scratch = nullptr;
  mpm_status st = scratch_for_current_device(&scratch);
  if (st != MPM_OK) return st;
  int dev = 0, num_sms = 1;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return MPM_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  const int64_t cells = (int64_t)params->N * params->N * params->N;
  float4* grid[3] = {scratch, scratch + kNoAllocCells, scratch + 2 * kNoAllocCells};
  VelocityGrid vel;
  if (vgrid_bind(vel, scratch + 3 * kNoAllocCells, (int)params->N) != cudaSuccess) return MPM_ERR_CUDA;
  int* status = status_word(scratch);
  // the array keeps the previous call's contents: clear the first P2G target (the other
  // grids are cleared by the launches before they are written); the status word is kept,
  // so a fault of an earlier call stays visible until mpm_noalloc_status reads it
  if (cudaMemsetAsync(grid[1], 0, sizeof(float4) * cells, s) != cudaSuccess) return MPM_ERR_CUDA;

  StepArgs a{};
  a.s = state;
  a.stride = stride;
  a.mat = mat;
  a.id = nullptr;
  a.n = n;
  a.grid_cells = cells;
  set_vgrid(a, vel);
  a.guard_limit = 0;
  a.check_finite = params->check_finite ? 1 : 0;
  a.status = status;
  make_sim_consts(*params, materials, n_materials, a.K);
  const bool liquid = n_materials == 1 && materials[0].kind == MPM_MAT_LIQUID;

  int cur = 0;
  for (int32_t i = -1; i < nsteps; ++i) {
    const StepKind kind = (i < 0) ? kStepP2GOnly : kStepFused;
    int chunk = 0, blocks = 0;
    step_launch_shape(num_sms, n, liquid, false, kind, 2, chunk, blocks);
    a.chunk = chunk;
    a.grid_in = (kind == kStepP2GOnly) ? nullptr : grid[cur];
    a.grid_out = grid[(cur + 1) % 3];
    a.grid_zero = grid[(cur + 2) % 3];
    if (launch_step(a, kind, liquid, false, blocks, s, nullptr, StepTuning{kStepWarps, 0}, &vel) != cudaSuccess)
      return MPM_ERR_CUDA;
    cur = (cur + 1) % 3;
  }
  return MPM_OK;
}

extern "C" mpm_status mpm_noalloc_status(void* stream) {
  float4* scratch = nullptr;
  mpm_status st = scratch_for_current_device(&scratch);
  if (st != MPM_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int* status = status_word(scratch);
  int bits = 0;
  // the copy is ordered after the substeps enqueued on `stream`; the host waits for it
  if (cudaMemcpyAsync(&bits, status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return MPM_ERR_CUDA;
  if (bits != 0) {
    if (cudaMemsetAsync(status, 0, sizeof(int), s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
      return MPM_ERR_CUDA;
  }
  if (bits & kStatusTimeout) return MPM_ERR_TIMEOUT;
  if (bits & (kStatusNonFinite | kStatusIndex)) return MPM_ERR_STATE;
  return MPM_OK;
}

extern "C" mpm_status mpm_noalloc_check_wait_timeout(int32_t polls, void* stream) {
  if (polls < 1 || polls > (1 << 20)) return MPM_ERR_INVALID;
  float4* scratch = nullptr;
  mpm_status st = scratch_for_current_device(&scratch);
  if (st != MPM_OK) return st;
  if (launch_wait_timeout_probe(status_word(scratch), polls, static_cast<cudaStream_t>(stream)) != cudaSuccess)
    return MPM_ERR_CUDA;
  return MPM_OK;
}
