// C ABI of the GB300 MLS-MPM substep: context, buffers, launch sequencing.
//
// Replaces the reference's host class Simulation (include/mpm.cuh:44-106,
// src/mpm.cu:180-329).  Grid buffers rotate through three slots so that a substep
// is one fused launch (see substep.cu); particles are component-major SoA sorted by
// cell every `sort_interval` substeps.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "mpm_gb300.h"
#include "mpm_internal.h"
#include "seeding.h"
#include "surface.h"
#include "export.h"
#include "tuning_cache.h"

using namespace mpm;

// A scene object: its seeded particle positions (device) and, while active, the id range
// its particles hold in the context.
struct ObjectRec {
  mpm_object desc{};  // host mesh pointers are not kept
  float* d_x = nullptr;
  int64_t count = 0;
  bool active = false;
  uint32_t id0 = 0;
};

struct mpm_ctx {
  mpm_params params{};
  SimConsts K{};
  int n_materials = 0;
  mpm_material mats[MPM_MAX_MATERIALS]{};
  bool liquid_layout = false;

  int device = 0;
  int num_sms = 1;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;

  // particles
  int64_t n = 0, stride = 0, capacity = 0;
  float* sA = nullptr;
  float* sB = nullptr;
  uint8_t* matA = nullptr;
  uint8_t* matB = nullptr;
  uint32_t* idA = nullptr;
  uint32_t* idB = nullptr;
  uint32_t* keys = nullptr;
  bool have_mat = false;

  // grid: three rotating P2G buffers and the padded velocity grid G2P reads
  float4* grid[3] = {nullptr, nullptr, nullptr};
  float4* vgrid_mem = nullptr;
  VelocityGrid vel;
  int64_t cells = 0;
  int64_t sort_keys = 0;  // key space of the bricked cell sort (>= cells)
  int cur = 0;            // slot holding the P2G grid of the next substep (when pending)
  // Calls that are followed by an upload (copies every substep) would throw away the P2G
  // the fused step prefetches for the next substep: once that is seen, such calls end with
  // a G2P-only step, until a call follows one of them without an upload in between.
  bool tail_g2p = false;
  bool ended_g2p = false;  // the last call ended with a G2P-only step
  int prev = -1;          // slot the last completed substep's G2P read
  bool pending = false;

  // sort scratch
  int* counts = nullptr;
  int* block_sums = nullptr;

  // staging
  float* stage = nullptr;
  size_t stage_bytes = 0;
  int* status = nullptr;
  int* work = nullptr;  // [2]: upload position check, [3]: cell-order position check
  // the two position checks of an upload in cell order, in mapped pinned memory: the
  // kernels write them and the host reads them after its synchronisation (no copy)
  int* host_flags = nullptr;
  int* host_flags_dev = nullptr;
  bool unsorted = true;  // particle order unrelated to cells (upload, append): the next sort gathers
  // the inverse of the id permutation while the ids are unchanged: the one a cell-ordered
  // upload leaves in the sort scratch, or the last one computed into the spare id copy;
  // null when it has to be computed (inverse_ids)
  const uint32_t* inv = nullptr;

  int64_t substeps = 0;
  int64_t since_sort = 0;
  int64_t launches = 0;
  int steps_per_warp = 2;
  StepTuning tuning{kStepWarps, 0};  // launch shape of the fused substep kernel
  std::string last_error;

  double t = 0.0;  // simulated time (Simulation::t)
  std::vector<ObjectRec> objects;
  SurfaceBuffers surf;
  SmoothBuffers smooth;
  struct ExportSlot {
    void* dev = nullptr;   // packed records on the device
    void* host = nullptr;  // pinned copy
    int64_t cap = 0;       // records both hold
    int64_t n = 0;
    cudaEvent_t packed = nullptr, copied = nullptr;
    bool pending = false;
  } exports[2];
  cudaStream_t copy_stream = nullptr;
  float* positions = nullptr;  // clip-space positions of the renderer
  int64_t positions_cap = 0;
  uint8_t* image = nullptr;  // mask (W H) then RGB (3 W H)
  int64_t image_cap = 0;
};

namespace {

mpm_status fail(mpm_ctx* c, mpm_status code, const std::string& msg) {
  if (c) c->last_error = msg;
  return code;
}

#define MPM_CUDA(ctx, call)                                                                          \
  do {                                                                                               \
    cudaError_t _e = (call);                                                                         \
    if (_e != cudaSuccess)                                                                           \
      return fail((ctx), _e == cudaErrorMemoryAllocation ? MPM_ERR_NOMEM : MPM_ERR_CUDA,             \
                  std::string(#call) + ": " + cudaGetErrorString(_e));                               \
  } while (0)

bool valid_params(const mpm_params* p, std::string& why) {
  if (!p) {
    why = "params is NULL";
    return false;
  }
  if (p->N < 4 || p->N > 1000) {
    why = "N must be in [4, 1000]";
    return false;
  }
  if (!(p->dt > 0.f) || !std::isfinite(p->dt)) {
    why = "dt must be positive and finite";
    return false;
  }
  if (p->boundary_mode < 0 || p->boundary_mode > 2) {
    why = "unknown boundary_mode";
    return false;
  }
  if (p->boundary_cells < 0 || (uint32_t)p->boundary_cells * 2 > p->N) {
    why = "boundary_cells out of range";
    return false;
  }
  if (p->sort_interval < 0) {
    why = "sort_interval must be >= 0";
    return false;
  }
  return true;
}

void derive_consts(mpm_ctx* c) { mpm::make_sim_consts(c->params, c->mats, c->n_materials, c->K); }

// The compact liquid layout (x, v, C, J) is used when the table is a single liquid.
bool all_liquid(const mpm_ctx* c) { return c->n_materials == 1 && c->mats[0].kind == MPM_MAT_LIQUID; }

// Whether [p, p + bytes) lies in one pinned host allocation the device can address; *dev
// receives the device view of p.  Pageable or unknown memory goes through copies instead.
bool device_view(const void* p, size_t bytes, const void** dev) {
  if (!p || bytes == 0) return false;
  cudaPointerAttributes a{}, b{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  const char* last = (const char*)p + bytes - 1;
  if (cudaPointerGetAttributes(&b, last) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type != cudaMemoryTypeHost || b.type != cudaMemoryTypeHost || !a.devicePointer || !b.devicePointer)
    return false;
  if ((const char*)b.devicePointer - (const char*)a.devicePointer != (ptrdiff_t)(bytes - 1)) return false;
  *dev = a.devicePointer;
  return true;
}

mpm_status ensure_stage(mpm_ctx* c, size_t bytes) {
  if (c->stage_bytes >= bytes) return MPM_OK;
  if (c->stage) cudaFree(c->stage);
  c->stage = nullptr;
  c->stage_bytes = 0;
  MPM_CUDA(c, cudaMalloc(&c->stage, bytes));
  c->stage_bytes = bytes;
  return MPM_OK;
}

void free_particles(mpm_ctx* c) {
  cudaFree(c->sA);
  cudaFree(c->sB);
  cudaFree(c->matA);
  cudaFree(c->matB);
  cudaFree(c->idA);
  cudaFree(c->idB);
  cudaFree(c->keys);
  c->sA = c->sB = nullptr;
  c->matA = c->matB = nullptr;
  c->idA = c->idB = nullptr;
  c->keys = nullptr;
  c->capacity = 0;
}

mpm_status ensure_particles(mpm_ctx* c, int64_t n) {
  if (n <= c->capacity && c->sA) return MPM_OK;
  c->inv = nullptr;
  free_particles(c);
  const int64_t cap = std::max<int64_t>(64, (n + 63) / 64 * 64);
  const size_t fbytes = sizeof(float) * (size_t)kNumComps * cap;
  MPM_CUDA(c, cudaMalloc(&c->sA, fbytes));
  MPM_CUDA(c, cudaMalloc(&c->sB, fbytes));
  MPM_CUDA(c, cudaMalloc(&c->matA, cap));
  MPM_CUDA(c, cudaMalloc(&c->matB, cap));
  MPM_CUDA(c, cudaMalloc(&c->idA, sizeof(uint32_t) * cap));
  MPM_CUDA(c, cudaMalloc(&c->idB, sizeof(uint32_t) * cap));
  MPM_CUDA(c, cudaMalloc(&c->keys, sizeof(uint32_t) * 2 * cap));  // sort keys, then the sort's permutation
  c->capacity = cap;
  c->stride = cap;
  return MPM_OK;
}

// Grows the particle arrays to hold `need` particles, keeping the current ones.
mpm_status grow_particles(mpm_ctx* c, int64_t need) {
  if (need <= c->capacity && c->sA) return MPM_OK;
  if (!c->sA || c->n == 0) return ensure_particles(c, need);
  const int64_t cap = std::max<int64_t>((need + 63) / 64 * 64, 2 * c->capacity);
  const size_t fbytes = sizeof(float) * (size_t)kNumComps * cap;
  float *sA = nullptr, *sB = nullptr;
  uint8_t *mA = nullptr, *mB = nullptr;
  uint32_t *iA = nullptr, *iB = nullptr, *keys = nullptr;
  auto undo = [&]() {
    for (void* p : {(void*)sA, (void*)sB, (void*)mA, (void*)mB, (void*)iA, (void*)iB, (void*)keys}) cudaFree(p);
    return fail(c, MPM_ERR_NOMEM, "cannot grow the particle arrays");
  };
  if (cudaMalloc(&sA, fbytes) || cudaMalloc(&sB, fbytes) || cudaMalloc(&mA, cap) || cudaMalloc(&mB, cap) ||
      cudaMalloc(&iA, sizeof(uint32_t) * cap) || cudaMalloc(&iB, sizeof(uint32_t) * cap) ||
      cudaMalloc(&keys, sizeof(uint32_t) * 2 * cap))
    return undo();
  for (int k = 0; k < kNumComps; ++k)
    MPM_CUDA(c, cudaMemcpyAsync(sA + (size_t)k * cap, c->sA + (size_t)k * c->stride, sizeof(float) * c->n,
                                cudaMemcpyDeviceToDevice, c->stream));
  MPM_CUDA(c, cudaMemcpyAsync(mA, c->matA, c->n, cudaMemcpyDeviceToDevice, c->stream));
  MPM_CUDA(c, cudaMemcpyAsync(iA, c->idA, sizeof(uint32_t) * c->n, cudaMemcpyDeviceToDevice, c->stream));
  MPM_CUDA(c, cudaStreamSynchronize(c->stream));
  c->inv = nullptr;
  free_particles(c);
  c->sA = sA;
  c->sB = sB;
  c->matA = mA;
  c->matB = mB;
  c->idA = iA;
  c->idB = iB;
  c->keys = keys;
  c->capacity = c->stride = cap;
  return MPM_OK;
}

void free_objects(mpm_ctx* c) {
  for (auto& o : c->objects) cudaFree(o.d_x);
  c->objects.clear();
}

// The particle set changed: the next substep re-sorts and restarts with a P2G launch.
void particles_changed(mpm_ctx* c) {
  c->inv = nullptr;
  c->pending = false;
  c->since_sort = c->params.sort_interval;
}

mpm_status activate_object(mpm_ctx* c, ObjectRec& o) {
  const int64_t k = o.count;
  if (k > 0) {
    if (c->n + k > (int64_t)0xffffffffLL) return fail(c, MPM_ERR_INVALID, "too many particles");
    mpm_status st = grow_particles(c, c->n + k);
    if (st != MPM_OK) return st;
    const uint8_t mi = (uint8_t)o.desc.material;
    if (!c->liquid_layout && mi != 0 && !c->have_mat) {
      if (c->n > 0) MPM_CUDA(c, cudaMemsetAsync(c->matA, 0, c->n, c->stream));
      c->have_mat = true;
    }
    MPM_CUDA(c, launch_append_object(c->sA, c->stride, c->n, k, o.d_x, o.desc.velocity, c->liquid_layout,
                                     c->have_mat ? c->matA : nullptr, mi, c->idA, (uint32_t)c->n, c->stream));
    c->launches += 1;
    o.id0 = (uint32_t)c->n;
    c->n += k;
    c->unsorted = true;  // the new particles sit at the end in seeding order
    particles_changed(c);
  }
  o.active = true;
  return MPM_OK;
}

mpm_status retire_object(mpm_ctx* c, ObjectRec& o) {
  const int64_t k = o.count;
  if (k > 0) {
    const int64_t n = c->n;
    int* flags = nullptr;
    int* scratch = nullptr;
    if (cudaMalloc(&flags, sizeof(int) * (n + 1)) || cudaMalloc(&scratch, sizeof(int) * scan_scratch_ints(n + 1))) {
      cudaFree(flags);
      return fail(c, MPM_ERR_NOMEM, "cannot allocate the compaction scratch");
    }
    const uint32_t lo = o.id0, hi = o.id0 + (uint32_t)k;
    cudaError_t e = launch_remove_ids(c->sA, c->sB, c->stride, n, c->idA, c->idB, c->have_mat ? c->matA : nullptr,
                                      c->matB, lo, hi, c->liquid_layout, flags, scratch, c->stream, &c->launches);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(flags);
    cudaFree(scratch);
    if (e != cudaSuccess) return fail(c, MPM_ERR_CUDA, std::string("object removal: ") + cudaGetErrorString(e));
    std::swap(c->sA, c->sB);
    std::swap(c->matA, c->matB);
    std::swap(c->idA, c->idB);
    c->n = n - k;
    for (auto& other : c->objects)
      if (other.active && other.id0 > lo) other.id0 -= (uint32_t)k;
    particles_changed(c);
  }
  o.active = false;
  return MPM_OK;
}

// SimObject::isActive (include/mpm.cuh:36-38) at the current time, for every object.
mpm_status update_objects(mpm_ctx* c) {
  for (auto& o : c->objects) {
    const bool want = c->t >= o.desc.lifetime_begin && c->t < o.desc.lifetime_end;
    mpm_status st = MPM_OK;
    if (want && !o.active) st = activate_object(c, o);
    if (!want && o.active) st = retire_object(c, o);
    if (st != MPM_OK) return st;
  }
  return MPM_OK;
}

StepArgs make_step_args(mpm_ctx* c) {
  StepArgs a{};
  a.s = c->sA;
  a.stride = c->stride;
  a.mat = c->have_mat ? c->matA : nullptr;
  a.id = c->idA;
  a.n = c->n;
  a.grid_cells = c->cells;
  set_vgrid(a, c->vel);
  a.guard_limit = (int64_t)c->params.N * c->params.N * c->params.N;
  a.check_finite = c->params.check_finite;
  a.status = c->status;
  a.K = c->K;
  return a;
}

// A compiled-in material (include/mpm_gb300_policies.cuh) runs its kernels in the default
// launch shape; the steps per warp still apply.
bool compiled_in_material(const mpm_ctx* c) { return c->n_materials > 0 && c->mats[0].kind >= MPM_MAT_USER_BASE; }

StepTuning ctx_tuning(const mpm_ctx* c) { return compiled_in_material(c) ? StepTuning{kStepWarps, 0} : c->tuning; }

void launch_shape(mpm_ctx* c, StepKind kind, bool guard, int& chunk, int& blocks) {
  mpm::step_launch_shape(c->num_sms, c->n, c->liquid_layout, guard, kind, c->steps_per_warp, chunk, blocks,
                         ctx_tuning(c));
}

mpm_status run_step(mpm_ctx* c, StepKind kind) {
  StepArgs a = make_step_args(c);
  const bool guard = c->params.g2p_guard != 0;
  if (guard && compiled_in_material(c))
    return fail(c, MPM_ERR_UNSUPPORTED, "the G2P guard is not available with a compiled-in material");
  int chunk, blocks;
  launch_shape(c, kind, guard, chunk, blocks);
  a.chunk = chunk;
  const int r = c->cur;
  a.grid_in = (kind == kStepP2GOnly) ? nullptr : c->grid[r];
  a.grid_out = c->grid[(r + 1) % 3];
  a.grid_zero = c->grid[(r + 2) % 3];
  MPM_CUDA(c, launch_step(a, kind, c->liquid_layout, guard, blocks, c->stream, &c->launches, ctx_tuning(c), &c->vel));
  if (kind != kStepP2GOnly) c->prev = r;
  c->cur = (r + 1) % 3;
  c->pending = kind != kStepG2POnly;
  return MPM_OK;
}

// g2p_next: the launch after this sort is a G2P launch over the sorted particles (the
// P2G of its substep is already on the grid), so the sort may move only what that
// launch reads back (SortArgs::partial).
mpm_status run_sort(mpm_ctx* c, bool g2p_next) {
  if (c->n == 0) return MPM_OK;
  SortArgs s{};
  s.sA = c->sA;
  s.sB = c->sB;
  s.stride = c->stride;
  s.n = c->n;
  s.matA = c->have_mat ? c->matA : nullptr;
  s.matB = c->matB;
  s.idA = c->idA;
  s.idB = c->idB;
  s.keys = c->keys;
  // particles in arbitrary order (just uploaded or appended) sort faster by gathering
  s.perm = c->unsorted ? c->keys + c->capacity : nullptr;
  s.counts = c->counts;
  s.block_sums = c->block_sums;
  s.cells = c->sort_keys;
  s.N = (int)c->params.N;
  s.dx_inv = c->K.g.dx_inv;
  // liquid layout: x, v, C, J (16 components); general: all 25
  s.ncomp = c->liquid_layout ? kLiquidComps : kNumComps;
  // guarded particles skip G2P and scatter their stored v and C, so they keep the full move
  s.partial = g2p_next && !c->unsorted && c->params.g2p_guard == 0 && c->sort_keys <= (int64_t)kKeyOutside;
  c->inv = nullptr;
  MPM_CUDA(c, launch_sort(s, c->num_sms, c->stream, &c->launches));
  std::swap(c->sA, c->sB);
  std::swap(c->matA, c->matB);
  std::swap(c->idA, c->idB);
  c->since_sort = 0;
  c->unsorted = false;
  return MPM_OK;
}

mpm_status check_ready(mpm_ctx* c) {
  if (!c) return MPM_ERR_INVALID;
  if (c->n_materials == 0) return fail(c, MPM_ERR_INVALID, "no materials set (mpm_set_materials)");
  return MPM_OK;
}

// The inverse of the id permutation (the slot of each particle in upload order): the
// cached one while the ids are unchanged, else computed into the spare id copy.
cudaError_t inverse_ids(mpm_ctx* c, const uint32_t** inv) {
  if (!c->inv) {
    const cudaError_t e = launch_inverse(c->idA, c->n, c->idB, c->stream);
    if (e != cudaSuccess) return e;
    c->launches += c->n > 0;
    c->inv = c->idB;
  }
  *inv = c->inv;
  return cudaSuccess;
}

}  // namespace

namespace mpm {

// SimulationParameters (include/TransferScheme.h:6-29) and the material constants,
// derived in float exactly as the reference constructors do.
void make_grid_consts(const mpm_params& p, GridConsts& K) {
  K.N = (int)p.N;
  K.dt = p.dt;
  // dx = 1.0/N (double, stored as float), dx_inv = 1.0/dx; D_inv_const = I * 4.0 * dx_inv * dx_inv
  const float dx = (float)(1.0 / (double)p.N);
  const float dxi = (float)(1.0 / (double)dx);
  K.dx = dx;
  K.dx_inv = dxi;
  K.dinv = (4.0f * dxi) * dxi;
  K.dtg = p.dt * p.gravity;
  K.boundary_mode = p.boundary_mode;
  K.boundary_cells = p.boundary_cells;
}

void make_sim_consts(const mpm_params& p, const mpm_material* mats, int n_materials, SimConsts& K) {
  make_grid_consts(p, K.g);
  K.n_materials = n_materials;
  for (int i = 0; i < n_materials; ++i) make_dev_material(mats[i], K.mat[i]);
}

void make_dev_material(const mpm_material& m, DevMaterial& d) {
  {
    d.kind = m.kind;
    d.vol = m.particle_volume;
    d.mass = m.density * m.particle_volume;                       // MaterialModelBase
    d.mu0 = m.E / (2.f * (1.f + m.nu));                            // MMFixedCorotated
    d.lambda0 = m.E * m.nu / ((1.f + m.nu) * (1.f - 2.f * m.nu));
    d.hardening = m.hardening;
    d.clamp_lo = m.clamp_lo;
    d.clamp_hi = m.clamp_hi;
    d.bulk = m.bulk;
  }
}

// Ranges of steps_per_warp steps (32 particles each), halved while a resident warp
// would get fewer than 6 ranges: the kernel deals ranges out dynamically, and with
// fewer, coarser ranges the warps finish unevenly (a 500k-particle snow substep ran 6%
// faster with 1-step than with 2-step ranges).
void step_launch_shape(int num_sms, int64_t n, bool liquid, bool guard, StepKind kind, int steps_per_warp,
                       int& chunk, int& blocks, StepTuning want) {
  const StepTuning t = step_tuning(kind, guard, false, want);
  const int warps = t.warps;
  const size_t smem = step_smem_bytes(kind, false, t);
  const int bps = step_blocks_per_sm(kind, liquid, guard, smem, false, t);
  const int64_t resident_warps = (int64_t)num_sms * bps * warps;
  int64_t steps = steps_per_warp;
  while (steps > 1 && n < resident_warps * 32 * steps * 6) steps /= 2;
  chunk = (int)(steps * 32);
  const int64_t nranges = (n + chunk - 1) / chunk;
  blocks = (int)std::max<int64_t>(1, std::min<int64_t>((nranges + warps - 1) / warps, (int64_t)num_sms * bps));
}

}  // namespace mpm

extern "C" {

mpm_status mpm_create(const mpm_params* params, mpm_ctx** out) {
  if (!out) return MPM_ERR_INVALID;
  *out = nullptr;
  std::string why;
  if (!valid_params(params, why)) return MPM_ERR_INVALID;
  mpm_ctx* c = new mpm_ctx();
  c->params = *params;
  derive_consts(c);
  auto bail = [&](mpm_status s) {
    mpm_destroy(c);
    return s;
  };
  if (cudaGetDevice(&c->device) != cudaSuccess) return bail(MPM_ERR_CUDA);
  if (cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess)
    return bail(MPM_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) return bail(MPM_ERR_CUDA);
  c->stream = c->own_stream;
  c->cells = (int64_t)params->N * params->N * params->N;
  for (int i = 0; i < 3; ++i) {
    if (cudaMalloc(&c->grid[i], sizeof(float4) * c->cells) != cudaSuccess) return bail(MPM_ERR_NOMEM);
    if (cudaMemsetAsync(c->grid[i], 0, sizeof(float4) * c->cells, c->stream) != cudaSuccess)
      return bail(MPM_ERR_CUDA);
  }
  if (cudaMalloc(&c->vgrid_mem, sizeof(float4) * vgrid_nodes((int)params->N)) != cudaSuccess)
    return bail(MPM_ERR_NOMEM);
  if (vgrid_bind(c->vel, c->vgrid_mem, (int)params->N) != cudaSuccess) return bail(MPM_ERR_CUDA);
  const int per = kThreads * 8;
  const int64_t nbr = (params->N + 3) / 4;
  c->sort_keys = nbr * nbr * nbr * 64;
  const int64_t nb = (c->sort_keys + per - 1) / per;
  if (cudaMalloc(&c->counts, sizeof(int) * c->sort_keys) != cudaSuccess) return bail(MPM_ERR_NOMEM);
  if (cudaMalloc(&c->block_sums, sizeof(int) * std::max<int64_t>(nb, 1)) != cudaSuccess) return bail(MPM_ERR_NOMEM);
  if (cudaMalloc(&c->status, sizeof(int)) != cudaSuccess) return bail(MPM_ERR_NOMEM);
  if (cudaMalloc(&c->work, 4 * sizeof(int)) != cudaSuccess) return bail(MPM_ERR_NOMEM);
  if (cudaMemsetAsync(c->work, 0, 4 * sizeof(int), c->stream) != cudaSuccess) return bail(MPM_ERR_CUDA);
  if (cudaHostAlloc(&c->host_flags, 4 * sizeof(int), cudaHostAllocMapped) != cudaSuccess) return bail(MPM_ERR_NOMEM);
  if (cudaHostGetDevicePointer(&c->host_flags_dev, c->host_flags, 0) != cudaSuccess) return bail(MPM_ERR_CUDA);

  if (cudaMemsetAsync(c->status, 0, sizeof(int), c->stream) != cudaSuccess) return bail(MPM_ERR_CUDA);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) return bail(MPM_ERR_CUDA);
  *out = c;
  return MPM_OK;
}

mpm_status mpm_destroy(mpm_ctx* c) {
  if (!c) return MPM_ERR_INVALID;
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_objects(c);
  free_particles(c);
  for (auto& g : c->grid) cudaFree(g);
  cudaFree(c->vgrid_mem);
  c->surf.release();
  c->smooth.release();
  if (c->copy_stream) {
    cudaStreamSynchronize(c->copy_stream);
    cudaStreamDestroy(c->copy_stream);
  }
  for (auto& x : c->exports) {
    cudaFree(x.dev);
    cudaFreeHost(x.host);
    if (x.packed) cudaEventDestroy(x.packed);
    if (x.copied) cudaEventDestroy(x.copied);
  }
  cudaFree(c->positions);
  cudaFree(c->image);
  cudaFree(c->counts);
  cudaFree(c->block_sums);
  cudaFree(c->stage);
  cudaFree(c->status);
  cudaFree(c->work);
  cudaFreeHost(c->host_flags);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
  return MPM_OK;
}

mpm_status mpm_set_stream(mpm_ctx* c, void* stream) {
  if (!c) return MPM_ERR_INVALID;
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return MPM_OK;
}

mpm_status mpm_set_params(mpm_ctx* c, const mpm_params* p) {
  if (!c) return MPM_ERR_INVALID;
  std::string why;
  if (!valid_params(p, why)) return fail(c, MPM_ERR_INVALID, why);
  if (p->N != c->params.N) return fail(c, MPM_ERR_INVALID, "N cannot change on a live context");
  c->params = *p;
  derive_consts(c);
  c->pending = false;  // the prefetched P2G used the old dt
  return MPM_OK;
}

mpm_status mpm_set_materials(mpm_ctx* c, const mpm_material* m, int32_t count) {
  if (!c) return MPM_ERR_INVALID;
  if (!m || count <= 0 || count > MPM_MAX_MATERIALS) return fail(c, MPM_ERR_INVALID, "material count out of range");
  const bool user = m[0].kind >= MPM_MAT_USER_BASE;
  for (int i = 0; i < count; ++i) {
    const bool known = (m[i].kind >= 0 && m[i].kind <= MPM_MAT_LIQUID) || find_material_kernels(m[i].kind, nullptr);
    if (!known) return fail(c, MPM_ERR_INVALID, "unknown material kind (not built in and not compiled in)");
    if (user && m[i].kind != m[0].kind)
      return fail(c, MPM_ERR_INVALID, "a table with a compiled-in material kind holds that kind only");
    if (!user && m[i].kind >= MPM_MAT_USER_BASE)
      return fail(c, MPM_ERR_INVALID, "a table with a compiled-in material kind holds that kind only");
    if (!(m[i].particle_volume > 0.f) || !(m[i].density > 0.f))
      return fail(c, MPM_ERR_INVALID, "particle_volume and density must be positive");
  }
  const bool was_liquid = c->liquid_layout;
  for (int i = 0; i < count; ++i) c->mats[i] = m[i];
  c->n_materials = count;
  const bool liq = all_liquid(c);
  if (c->n > 0 && liq != was_liquid)
    return fail(c, MPM_ERR_INVALID, "material table change would switch the particle layout; set materials before upload");
  c->liquid_layout = liq;
  derive_consts(c);
  c->pending = false;
  return MPM_OK;
}

mpm_status mpm_upload_soa(mpm_ctx* c, int64_t n, const float* x, const float* v, const float* C, const float* F,
                          const float* Jp, const uint8_t* mat) {
  mpm_status st = check_ready(c);
  if (st != MPM_OK) return st;
  if (n < 0 || (n > 0 && !x)) return fail(c, MPM_ERR_INVALID, "x is required");
  if (n > (int64_t)0xffffffffLL) return fail(c, MPM_ERR_INVALID, "too many particles");
  if (mat)
    for (int64_t p = 0; p < n; ++p)
      if (mat[p] >= c->n_materials) return fail(c, MPM_ERR_INVALID, "material index out of range");
  // The positions are checked on the GPU (a host loop over them cost more than the
  // copies) and the context changes only once they pass.  Arrays in pinned host memory are
  // read by the conversion kernel itself over the host link; others go through the staging
  // buffer with copies.  When the particle arrays keep their size, the conversion writes
  // the spare copy, which replaces the current one after the check.
  const bool grow = n > c->capacity || !c->sA;
  // a per-particle material array keeps the upload order (its bytes are copied as given),
  // so only uploads without one are put in cell order on the way in
  bool mixed = !c->liquid_layout && c->n_materials > 1;
  if (mat)
    for (int64_t p = 0; p < n && !mixed; ++p) mixed = mat[p] != 0;
  const bool presort = n > 0 && !grow && !mixed;
  // the same particle count again: each particle goes to the slot its id holds, keeping the
  // device order and the ids
  const bool in_place = presort && n == c->n;
  if (!in_place) c->inv = nullptr;  // the paths below write the spare id copy or the sort scratch
  bool presorted = false, kept_order = false, in_place_done = false;
  HostArrays arr{};
  bool direct = false;
  if (n > 0 && !grow) {
    const void *dx = nullptr, *dv = nullptr, *dC = nullptr, *dF = nullptr, *dJ = nullptr;
    direct = device_view(x, 12 * n, &dx) && (!v || device_view(v, 12 * n, &dv)) &&
             (!C || device_view(C, 36 * n, &dC)) && (!F || device_view(F, 36 * n, &dF)) &&
             (!Jp || device_view(Jp, 4 * n, &dJ));
    if (direct) arr = HostArrays{(const float*)dx, (const float*)dv, (const float*)dC, (const float*)dF, (const float*)dJ};
  }
  if (n > 0 && !direct) {
    st = ensure_stage(c, 25 * sizeof(float) * (size_t)n);
    if (st != MPM_OK) return st;
    float* xs = c->stage;
    float* vs = xs + 3 * n;
    float* Cs = vs + 3 * n;
    float* Fs = Cs + 9 * n;
    float* Js = Fs + 9 * n;
    MPM_CUDA(c, cudaStreamSynchronize(c->stream));  // the stage may still feed an earlier call
    MPM_CUDA(c, cudaMemcpyAsync(xs, x, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, c->stream));
    if (v) MPM_CUDA(c, cudaMemcpyAsync(vs, v, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, c->stream));
    if (C) MPM_CUDA(c, cudaMemcpyAsync(Cs, C, sizeof(float) * 9 * n, cudaMemcpyHostToDevice, c->stream));
    if (F) MPM_CUDA(c, cudaMemcpyAsync(Fs, F, sizeof(float) * 9 * n, cudaMemcpyHostToDevice, c->stream));
    if (Jp) MPM_CUDA(c, cudaMemcpyAsync(Js, Jp, sizeof(float) * n, cudaMemcpyHostToDevice, c->stream));
    arr = HostArrays{xs, v ? vs : nullptr, C ? Cs : nullptr, F ? Fs : nullptr, Jp ? Js : nullptr};
  }
  if (n > 0) {
    int bad = 0;
    if (grow) {
      // check the staged positions before the old arrays are released
      MPM_CUDA(c, launch_check_finite(arr.x, 3 * n, c->work + 2, c->stream));
      MPM_CUDA(c, cudaMemcpyAsync(&bad, c->work + 2, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      MPM_CUDA(c, cudaStreamSynchronize(c->stream));
      c->launches += 1;
      if (bad) return fail(c, MPM_ERR_INVALID, "non-finite particle position");
      st = ensure_particles(c, n);
      if (st != MPM_OK) return st;
      MPM_CUDA(c, launch_deinterleave_arrays(arr, c->sA, c->stride, n, c->work + 2, c->stream));
    } else if (in_place) {
      // The particles keep the device order (cell order as of the last sort) and their ids:
      // particle p goes to slot inv[p], read over the host link in one pass.  A count of the
      // slots whose cell key falls below their predecessor's tells whether the new positions
      // still follow that order; when they do not (a different scene of the same size), the
      // next substep sorts first.
      if (direct) MPM_CUDA(c, cudaStreamSynchronize(c->stream));  // earlier work may read the spare copy
      const uint32_t* inv = nullptr;
      MPM_CUDA(c, inverse_ids(c, &inv));
      volatile int* flags = c->host_flags;  // no kernel still writes them: synchronised above
      flags[0] = 0;
      flags[2] = 0;
      MPM_CUDA(c, launch_deinterleave_arrays(arr, c->sB, c->stride, n, c->host_flags_dev, c->stream, inv, true));
      MPM_CUDA(c, launch_order_check(c->sB, c->stride, n, c->K.g.dx_inv, (int)c->params.N, c->work,
                                     c->host_flags_dev + 2, c->stream));
      MPM_CUDA(c, cudaStreamSynchronize(c->stream));  // also: the caller may reuse the host arrays on return
      if (flags[0]) return fail(c, MPM_ERR_INVALID, "non-finite particle position");
      std::swap(c->sA, c->sB);
      c->launches += 1;
      // more than one slot in 8 out of cell order: sort before the next substep
      kept_order = (int64_t)flags[2] * 8 <= n;
      in_place_done = true;
    } else if (presort) {
      if (direct) MPM_CUDA(c, cudaStreamSynchronize(c->stream));  // earlier work may read the stage
      // Cell order from the positions first, then each particle goes straight to its slot:
      // the sort the first substep would run (a gather of every array) is not needed.
      // Host positions are copied to the stage on the way, so the host link carries them once.
      float* xcopy = nullptr;
      if (direct) {
        st = ensure_stage(c, 3 * sizeof(float) * (size_t)n);
        if (st != MPM_OK) return st;
        xcopy = c->stage;
      }
      SortArgs so{};
      so.n = n;
      so.keys = c->keys;
      // slot q holds particle perm[q]: the new id array, written into the spare id copy
      so.perm = c->idB;
      uint32_t* dest = c->keys + c->capacity;  // particle p goes to slot dest[p]
      so.counts = c->counts;
      so.block_sums = c->block_sums;
      so.cells = c->sort_keys;
      so.N = (int)c->params.N;
      so.dx_inv = c->K.g.dx_inv;
      // the check flags are read once, at the end: until then only the spare particle and id
      // copies, the stage and sort scratch have been written, so a rejected upload leaves the
      // context as it was.
      // No kernel still writes the flags: both paths synchronised the stream above.
      volatile int* flags = c->host_flags;
      flags[0] = 0;
      flags[1] = 0;
      MPM_CUDA(c, launch_presort(arr.x, xcopy, so, dest, c->host_flags_dev + 1, c->num_sms, c->stream, &c->launches,
                                 true));
      HostArrays sorted_arr = arr;
      if (xcopy) sorted_arr.x = xcopy;
      MPM_CUDA(c, launch_deinterleave_arrays(sorted_arr, c->sB, c->stride, n, c->host_flags_dev, c->stream, dest, true));
      MPM_CUDA(c, cudaStreamSynchronize(c->stream));  // also: the caller may reuse the host arrays on return
      if (flags[0] || flags[1]) return fail(c, MPM_ERR_INVALID, "non-finite particle position");
      std::swap(c->sA, c->sB);
      std::swap(c->idA, c->idB);
      c->inv = dest;
      presorted = true;
    } else {
      if (direct) MPM_CUDA(c, cudaStreamSynchronize(c->stream));  // earlier work may read the spare copy
      MPM_CUDA(c, launch_deinterleave_arrays(arr, c->sB, c->stride, n, c->work + 2, c->stream));
      MPM_CUDA(c, cudaMemcpyAsync(&bad, c->work + 2, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      MPM_CUDA(c, cudaStreamSynchronize(c->stream));
      if (bad) return fail(c, MPM_ERR_INVALID, "non-finite particle position");
      std::swap(c->sA, c->sB);
    }
    c->launches += 1;
  }
  if (n == 0) {
    st = ensure_particles(c, 0);
    if (st != MPM_OK) return st;
  }
  c->n = n;
  // a prefetched P2G is thrown away here: end later calls with a G2P-only step
  if (c->pending || c->ended_g2p) c->tail_g2p = true;
  c->ended_g2p = false;
  c->pending = false;
  c->prev = -1;
  c->substeps = 0;
  // a cell-ordered upload starts the sort interval afresh; one that kept the order keeps
  // its schedule; otherwise sort before the first substep
  if (!kept_order) c->since_sort = presorted ? 0 : c->params.sort_interval;
  c->unsorted = !presorted && !kept_order;
  c->t = 0.0;
  free_objects(c);
  if (n == 0) return MPM_OK;
  if (!presorted && !in_place_done) {
    MPM_CUDA(c, launch_iota(c->idA, n, c->stream));
    c->launches += 1;
  }
  c->have_mat = !c->liquid_layout && c->n_materials > 1;
  if (c->have_mat) {
    if (mat) {
      MPM_CUDA(c, cudaMemcpyAsync(c->matA, mat, n, cudaMemcpyHostToDevice, c->stream));
    } else {
      MPM_CUDA(c, cudaMemsetAsync(c->matA, 0, n, c->stream));
    }
  } else if (mat) {
    for (int64_t p = 0; p < n; ++p)
      if (mat[p] != 0) {
        c->have_mat = true;
        break;
      }
    if (c->have_mat) MPM_CUDA(c, cudaMemcpyAsync(c->matA, mat, n, cudaMemcpyHostToDevice, c->stream));
  }
  // Host buffers may be reused by the caller as soon as we return.
  MPM_CUDA(c, cudaStreamSynchronize(c->stream));
  return MPM_OK;
}

mpm_status mpm_upload_aos(mpm_ctx* c, const void* particles, int64_t n) {
  mpm_status st = check_ready(c);
  if (st != MPM_OK) return st;
  if (n < 0 || (n > 0 && !particles)) return fail(c, MPM_ERR_INVALID, "particles is NULL");
  std::vector<float> x(3 * n), v(3 * n), C(9 * n), F(9 * n), J(n);
  std::vector<uint8_t> mat(n);
  const uint8_t* b = (const uint8_t*)particles;
  for (int64_t p = 0; p < n; ++p) {
    const uint8_t* r = b + 104 * p;
    float f[25];
    std::memcpy(f, r + 4, sizeof(f));
    mat[p] = r[0];
    for (int d = 0; d < 3; ++d) {
      x[3 * p + d] = f[d];
      v[3 * p + d] = f[3 + d];
    }
    // Eigen matrices are column-major: element (row, col) at col * 3 + row
    for (int rr = 0; rr < 3; ++rr)
      for (int cc = 0; cc < 3; ++cc) {
        F[9 * p + 3 * rr + cc] = f[6 + cc * 3 + rr];
        C[9 * p + 3 * rr + cc] = f[15 + cc * 3 + rr];
      }
    J[p] = f[24];
  }
  return mpm_upload_soa(c, n, x.data(), v.data(), C.data(), F.data(), J.data(), mat.data());
}

mpm_status mpm_substep(mpm_ctx* c, int32_t nsteps) {
  mpm_status st = check_ready(c);
  if (st != MPM_OK) return st;
  if (nsteps < 0) return fail(c, MPM_ERR_INVALID, "nsteps must be >= 0");
  // the last call ended without the prefetched P2G and the state was not replaced since:
  // that P2G is needed after all, so calls end with the fused step again
  if (nsteps > 0 && c->ended_g2p) c->tail_g2p = false;
  if (nsteps > 0) c->ended_g2p = false;
  for (int32_t i = 0; i < nsteps; ++i) {
    if (!c->objects.empty()) {
      st = update_objects(c);
      if (st != MPM_OK) return st;
    }
    if (c->n > 0) {
      if (c->params.sort_interval > 0 && c->since_sort >= c->params.sort_interval) {
        st = run_sort(c, c->pending);
        if (st != MPM_OK) return st;
      }
      if (!c->pending) {
        st = run_step(c, kStepP2GOnly);
        if (st != MPM_OK) return st;
      }
      const bool g2p_only = c->tail_g2p && i == nsteps - 1 && c->objects.empty();
      st = run_step(c, g2p_only ? kStepG2POnly : kStepFused);
      if (st != MPM_OK) return st;
      c->ended_g2p = g2p_only;
    }
    c->substeps += 1;
    c->since_sort += 1;
    c->t += c->params.dt;  // Simulation::advance, src/mpm.cu:328
  }
  return MPM_OK;
}

mpm_status mpm_add_object(mpm_ctx* c, const mpm_object* obj, int64_t* n_particles) {
  mpm_status st = check_ready(c);
  if (st != MPM_OK) return st;
  if (!obj) return fail(c, MPM_ERR_INVALID, "object is NULL");
  if (obj->material < 0 || obj->material >= c->n_materials)
    return fail(c, MPM_ERR_INVALID, "object material index out of range");
  if (!(obj->lifetime_end > obj->lifetime_begin)) return fail(c, MPM_ERR_INVALID, "empty object lifetime");
  // density = u32(1.0 / particleVolume) (Simulation::addObject, src/mpm.cu:247)
  const double dens = 1.0 / (double)c->mats[obj->material].particle_volume;
  if (!(dens >= 1.0) || dens > 4294967295.0) return fail(c, MPM_ERR_INVALID, "particle volume out of range");
  SeedShapeOwner shape;
  st = build_seed_shape(*obj, (uint32_t)dens, shape);
  if (st != MPM_OK) return fail(c, st, "invalid object shape");
  ObjectRec rec;
  rec.desc = *obj;
  rec.desc.vertices = nullptr;
  rec.desc.triangles = nullptr;
  MPM_CUDA(c, cudaStreamSynchronize(c->stream));
  MPM_CUDA(c, seed_shape_gpu(shape.sh, c->stream, &rec.d_x, &rec.count));
  c->launches += 5;
  c->objects.push_back(rec);
  if (n_particles) *n_particles = rec.count;
  if (c->t >= obj->lifetime_begin && c->t < obj->lifetime_end) return activate_object(c, c->objects.back());
  return MPM_OK;
}

double mpm_time(const mpm_ctx* c) { return c ? c->t : 0.0; }

int32_t mpm_object_count(const mpm_ctx* c) { return c ? (int32_t)c->objects.size() : -1; }

mpm_status mpm_seed_object(const mpm_object* obj, uint32_t density, float* x, int64_t capacity, int64_t* n) {
  if (!obj || !n || capacity < 0 || (capacity > 0 && !x)) return MPM_ERR_INVALID;
  SeedShapeOwner shape;
  mpm_status st = build_seed_shape(*obj, density, shape);
  if (st != MPM_OK) return st;
  float* d_x = nullptr;
  int64_t count = 0;
  if (seed_shape_gpu(shape.sh, nullptr, &d_x, &count) != cudaSuccess) return MPM_ERR_CUDA;
  const int64_t copy = std::min(count, capacity);
  cudaError_t e = copy > 0 ? cudaMemcpy(x, d_x, sizeof(float) * 3 * copy, cudaMemcpyDeviceToHost) : cudaSuccess;
  cudaFree(d_x);
  if (e != cudaSuccess) return MPM_ERR_CUDA;
  *n = count;
  return MPM_OK;
}

mpm_status mpm_sync(mpm_ctx* c) {
  if (!c) return MPM_ERR_INVALID;
  MPM_CUDA(c, cudaStreamSynchronize(c->stream));
  int flag = 0;
  MPM_CUDA(c, cudaMemcpy(&flag, c->status, sizeof(int), cudaMemcpyDeviceToHost));
  if (flag) {
    MPM_CUDA(c, cudaMemset(c->status, 0, sizeof(int)));
    if (flag & kStatusTimeout) return fail(c, MPM_ERR_TIMEOUT, "device wait timed out");
    if (flag & kStatusNonFinite) return fail(c, MPM_ERR_STATE, "non-finite particle state");
    return fail(c, MPM_ERR_STATE, "device index check failed");
  }
  return MPM_OK;
}

mpm_status mpm_download_soa(mpm_ctx* c, float* x, float* v, float* C, float* F, float* Jp, uint8_t* mat) {
  if (!c) return MPM_ERR_INVALID;
  const int64_t n = c->n;
  if (n == 0) return MPM_OK;
  // the particles sit in cell order: gather them in upload order through the inverse of
  // the id array
  const uint32_t* inv = nullptr;
  MPM_CUDA(c, inverse_ids(c, &inv));
  {
    // pinned host arrays are written by the conversion kernel itself over the host link
    const void *dx = nullptr, *dv = nullptr, *dC = nullptr, *dF = nullptr, *dJ = nullptr;
    const bool direct = (x || v || C || F || Jp) && (!x || device_view(x, 12 * n, &dx)) &&
                        (!v || device_view(v, 12 * n, &dv)) && (!C || device_view(C, 36 * n, &dC)) &&
                        (!F || device_view(F, 36 * n, &dF)) && (!Jp || device_view(Jp, 4 * n, &dJ));
    if (direct) {
      const OutArrays o{(float*)dx, (float*)dv, (float*)dC, (float*)dF, (float*)dJ};
      MPM_CUDA(c, launch_interleave_arrays(c->sA, c->stride, inv, n, o, c->liquid_layout, c->stream));
      c->launches += 1;
      x = v = C = F = Jp = nullptr;  // written
    }
  }
  mpm_status st = ensure_stage(c, 25 * sizeof(float) * (size_t)n + (size_t)n);
  if (st != MPM_OK) return st;
  const unsigned fields = (x ? kFieldX : 0) | (v ? kFieldV : 0) | (C ? kFieldC : 0) | (F ? kFieldF : 0) |
                          (Jp ? kFieldJ : 0);
  MPM_CUDA(c, launch_interleave(c->sA, c->stride, inv, n, c->stage, c->liquid_layout, fields, c->stream));
  c->launches += fields != 0;
  float* xs = c->stage;
  float* vs = xs + 3 * n;
  float* Cs = vs + 3 * n;
  float* Fs = Cs + 9 * n;
  float* Js = Fs + 9 * n;
  if (x) MPM_CUDA(c, cudaMemcpyAsync(x, xs, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
  if (v) MPM_CUDA(c, cudaMemcpyAsync(v, vs, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
  if (C) MPM_CUDA(c, cudaMemcpyAsync(C, Cs, sizeof(float) * 9 * n, cudaMemcpyDeviceToHost, c->stream));
  if (F) MPM_CUDA(c, cudaMemcpyAsync(F, Fs, sizeof(float) * 9 * n, cudaMemcpyDeviceToHost, c->stream));
  if (Jp) MPM_CUDA(c, cudaMemcpyAsync(Jp, Js, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream));
  if (mat) {
    if (c->have_mat) {
      uint8_t* ms = (uint8_t*)(Js + n);
      MPM_CUDA(c, launch_scatter_u8(c->matA, c->idA, n, ms, c->stream));
      c->launches += 1;
      MPM_CUDA(c, cudaMemcpyAsync(mat, ms, n, cudaMemcpyDeviceToHost, c->stream));
    } else {
      std::memset(mat, 0, n);
    }
  }
  MPM_CUDA(c, cudaStreamSynchronize(c->stream));
  return MPM_OK;
}

mpm_status mpm_download_aos(mpm_ctx* c, void* particles) {
  if (!c) return MPM_ERR_INVALID;
  const int64_t n = c->n;
  if (n > 0 && !particles) return fail(c, MPM_ERR_INVALID, "particles is NULL");
  std::vector<float> x(3 * n), v(3 * n), C(9 * n), F(9 * n), J(n);
  std::vector<uint8_t> mat(n);
  mpm_status st = mpm_download_soa(c, x.data(), v.data(), C.data(), F.data(), J.data(), mat.data());
  if (st != MPM_OK) return st;
  uint8_t* b = (uint8_t*)particles;
  for (int64_t p = 0; p < n; ++p) {
    uint8_t* r = b + 104 * p;
    float f[25];
    for (int d = 0; d < 3; ++d) {
      f[d] = x[3 * p + d];
      f[3 + d] = v[3 * p + d];
    }
    for (int rr = 0; rr < 3; ++rr)
      for (int cc = 0; cc < 3; ++cc) {
        f[6 + cc * 3 + rr] = F[9 * p + 3 * rr + cc];
        f[15 + cc * 3 + rr] = C[9 * p + 3 * rr + cc];
      }
    f[24] = J[p];
    std::memset(r, 0, 4);
    r[0] = mat[p];
    std::memcpy(r + 4, f, sizeof(f));
  }
  return MPM_OK;
}

mpm_status mpm_get_grid(mpm_ctx* c, int32_t which, float* out) {
  if (!c || !out) return MPM_ERR_INVALID;
  if (which != 0 && which != 1) return fail(c, MPM_ERR_INVALID, "which must be 0 (post-P2G) or 1 (post-op)");
  if (c->prev < 0) return fail(c, MPM_ERR_INVALID, "no completed substep since the last upload");
  const size_t bytes = sizeof(float4) * c->cells;
  if (which == 0) {
    MPM_CUDA(c, cudaMemcpyAsync(out, c->grid[c->prev], bytes, cudaMemcpyDeviceToHost, c->stream));
  } else {
    mpm_status st = ensure_stage(c, bytes);
    if (st != MPM_OK) return st;
    MPM_CUDA(c, launch_grid_op(c->grid[c->prev], (float4*)c->stage, c->K.g, c->stream));
    c->launches += 1;
    MPM_CUDA(c, cudaMemcpyAsync(out, c->stage, bytes, cudaMemcpyDeviceToHost, c->stream));
  }
  MPM_CUDA(c, cudaStreamSynchronize(c->stream));
  return MPM_OK;
}

namespace {

// voxel_dx = N dx / grid_side in the reference's types (include/mesh_builder.h:172).
double voxel_dx_of(const mpm_ctx* c, int G) { return (double)((float)c->params.N * c->K.g.dx) / (double)G; }

mpm_status surface_field(mpm_ctx* c, int32_t G, int32_t radius, bool finish) {
  // G <= 512 keeps the mesher's counts (at most 5 triangles, 3 vertices and one surface
  // cube per cube of the (G-1)^3) within int32
  if (G < 2 || G > 512 || radius < 0 || radius > 64) return fail(c, MPM_ERR_INVALID, "grid_side or radius out of range");
  cudaError_t e = launch_distance_field(c->sA, c->stride, c->n, G, radius, voxel_dx_of(c, G), finish, c->surf,
                                        c->stream, &c->launches);
  if (e != cudaSuccess) return fail(c, MPM_ERR_CUDA, std::string("distance field: ") + cudaGetErrorString(e));
  return MPM_OK;
}

}  // namespace

mpm_status mpm_surface_distance(mpm_ctx* c, int32_t G, int32_t radius, float* out) {
  if (!c || !out) return MPM_ERR_INVALID;
  mpm_status st = surface_field(c, G, radius, true);
  if (st != MPM_OK) return st;
  cudaError_t e =
      cudaMemcpyAsync(out, c->surf.field, sizeof(float) * (size_t)G * G * G, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail(c, MPM_ERR_CUDA, cudaGetErrorString(e));
  return MPM_OK;
}

mpm_status mpm_surface_mesh(mpm_ctx* c, int32_t G, int32_t radius, float* tris, int64_t capacity, int64_t* n_tris) {
  if (!c || !n_tris || capacity < 0 || (capacity > 0 && !tris)) return MPM_ERR_INVALID;
  mpm_status st = surface_field(c, G, radius, false);
  if (st != MPM_OK) return st;
  int64_t nv = 0, n = 0;
  cudaError_t e = extract_surface(G, radius, voxel_dx_of(c, G), c->surf, c->stream, true, &nv, &n, &c->launches);
  const int64_t copy = std::min(n, capacity);
  if (e == cudaSuccess && copy > 0)
    e = cudaMemcpyAsync(tris, c->surf.tris, sizeof(float) * 9 * (size_t)copy, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail(c, MPM_ERR_CUDA, std::string("surface: ") + cudaGetErrorString(e));
  *n_tris = n;
  return MPM_OK;
}

mpm_status mpm_surface_mesh_indexed(mpm_ctx* c, int32_t G, int32_t radius, double* vertices, int64_t vertex_capacity,
                                    int32_t* faces, int64_t face_capacity, int64_t* n_vertices, int64_t* n_faces) {
  if (!c || !n_vertices || !n_faces || vertex_capacity < 0 || face_capacity < 0 ||
      (vertex_capacity > 0 && !vertices) || (face_capacity > 0 && !faces))
    return MPM_ERR_INVALID;
  mpm_status st = surface_field(c, G, radius, false);
  if (st != MPM_OK) return st;
  int64_t nv = 0, nf = 0;
  cudaError_t e = extract_surface(G, radius, voxel_dx_of(c, G), c->surf, c->stream, false, &nv, &nf, &c->launches);
  const int64_t vcopy = std::min(nv, vertex_capacity), fcopy = std::min(nf, face_capacity);
  if (e == cudaSuccess && vcopy > 0)
    e = cudaMemcpyAsync(vertices, c->surf.verts, sizeof(double) * 3 * (size_t)vcopy, cudaMemcpyDeviceToHost,
                        c->stream);
  if (e == cudaSuccess && fcopy > 0)
    e = cudaMemcpyAsync(faces, c->surf.faces, sizeof(int32_t) * 3 * (size_t)fcopy, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail(c, MPM_ERR_CUDA, std::string("surface: ") + cudaGetErrorString(e));
  *n_vertices = nv;
  *n_faces = nf;
  return MPM_OK;
}

mpm_status mpm_surface_table(int32_t* counts, int32_t* slots) {
  if (!counts || !slots) return MPM_ERR_INVALID;
  surface_table(counts, slots);
  return MPM_OK;
}

mpm_status mpm_surface_distance_device(mpm_ctx* c, int32_t G, int32_t radius, const float** field) {
  if (!c || !field) return MPM_ERR_INVALID;
  mpm_status st = surface_field(c, G, radius, true);
  if (st != MPM_OK) return st;
  *field = c->surf.field;
  return MPM_OK;
}

mpm_status mpm_surface_mesh_device(mpm_ctx* c, int32_t G, int32_t radius, const float** tris, int64_t* n_tris) {
  if (!c || !tris || !n_tris) return MPM_ERR_INVALID;
  mpm_status st = surface_field(c, G, radius, false);
  if (st != MPM_OK) return st;
  int64_t nv = 0, n = 0;
  cudaError_t e = extract_surface(G, radius, voxel_dx_of(c, G), c->surf, c->stream, true, &nv, &n, &c->launches);
  if (e != cudaSuccess) return fail(c, MPM_ERR_CUDA, std::string("surface: ") + cudaGetErrorString(e));
  *tris = c->surf.tris;
  *n_tris = n;
  return MPM_OK;
}

mpm_status mpm_surface_mesh_indexed_device(mpm_ctx* c, int32_t G, int32_t radius, const double** vertices,
                                           const int32_t** faces, int64_t* n_vertices, int64_t* n_faces) {
  if (!c || !vertices || !faces || !n_vertices || !n_faces) return MPM_ERR_INVALID;
  mpm_status st = surface_field(c, G, radius, false);
  if (st != MPM_OK) return st;
  int64_t nv = 0, nf = 0;
  cudaError_t e = extract_surface(G, radius, voxel_dx_of(c, G), c->surf, c->stream, false, &nv, &nf, &c->launches);
  if (e != cudaSuccess) return fail(c, MPM_ERR_CUDA, std::string("surface: ") + cudaGetErrorString(e));
  *vertices = c->surf.verts;
  *faces = c->surf.faces;
  *n_vertices = nv;
  *n_faces = nf;
  return MPM_OK;
}

namespace {

// smooth_mesh on device arrays and its outcome as a status.
mpm_status smooth_device(mpm_ctx* c, double* V, int64_t nv, const int32_t* F, int64_t nf, int32_t* iterations) {
  if (nv > 0 && nf == 0) return fail(c, MPM_ERR_INVALID, "smooth: vertices without faces (the system is singular)");
  if (nv == 0 && nf > 0) return fail(c, MPM_ERR_INVALID, "smooth: a face index is outside [0, n_vertices)");
  SmoothResult r;
  cudaError_t e = smooth_mesh(V, F, nv, nf, c->smooth, c->stream, &c->launches, &r);
  if (e != cudaSuccess)
    return fail(c, e == cudaErrorMemoryAllocation ? MPM_ERR_NOMEM : MPM_ERR_CUDA,
                std::string("smooth: ") + cudaGetErrorString(e));
  if (iterations) *iterations = r.iterations;
  if (r.bad_index) return fail(c, MPM_ERR_INVALID, "smooth: a face index is outside [0, n_vertices)");
  if (r.bad_area) return fail(c, MPM_ERR_INVALID, "smooth: a face has zero area (its cotangent weights are not finite)");
  if (!r.converged)
    return fail(c, MPM_ERR_STATE, "smooth: conjugate gradients did not converge (relative residual " +
                                      std::to_string(r.relative_residual) + " after " +
                                      std::to_string(r.iterations) + " iterations)");
  MPM_CUDA(c, cudaStreamSynchronize(c->stream));
  return MPM_OK;
}

}  // namespace

mpm_status mpm_surface_smooth(mpm_ctx* c, double* vertices, int64_t nv, const int32_t* faces, int64_t nf,
                              int32_t* iterations) {
  if (!c || nv < 0 || nf < 0 || (nv > 0 && !vertices) || (nf > 0 && !faces) || nv > INT32_MAX ||
      nf > INT32_MAX / 3)
    return MPM_ERR_INVALID;
  SmoothBuffers& sb = c->smooth;
  auto grow = [](auto*& p, int64_t& cap, int64_t need) {
    if (p && cap >= need) return cudaSuccess;
    cudaFree(p);
    p = nullptr;
    cap = 0;
    const cudaError_t e = cudaMalloc(&p, sizeof(*p) * (size_t)std::max<int64_t>(need, 1));
    if (e == cudaSuccess) cap = need;
    return e;
  };
  MPM_CUDA(c, grow(sb.V, sb.V_cap, 3 * nv));
  MPM_CUDA(c, grow(sb.F, sb.F_cap, 3 * nf));
  if (nv > 0)
    MPM_CUDA(c, cudaMemcpyAsync(sb.V, vertices, sizeof(double) * 3 * (size_t)nv, cudaMemcpyHostToDevice, c->stream));
  if (nf > 0)
    MPM_CUDA(c, cudaMemcpyAsync(sb.F, faces, sizeof(int32_t) * 3 * (size_t)nf, cudaMemcpyHostToDevice, c->stream));
  const mpm_status st = smooth_device(c, sb.V, nv, sb.F, nf, iterations);
  if (st != MPM_OK) return st;
  if (nv > 0)
    MPM_CUDA(c, cudaMemcpyAsync(vertices, sb.V, sizeof(double) * 3 * (size_t)nv, cudaMemcpyDeviceToHost, c->stream));
  MPM_CUDA(c, cudaStreamSynchronize(c->stream));
  return MPM_OK;
}

mpm_status mpm_surface_smooth_device(mpm_ctx* c, double* vertices, int64_t nv, const int32_t* faces, int64_t nf,
                                     int32_t* iterations) {
  if (!c || nv < 0 || nf < 0 || (nv > 0 && !vertices) || (nf > 0 && !faces) || nv > INT32_MAX ||
      nf > INT32_MAX / 3)
    return MPM_ERR_INVALID;
  return smooth_device(c, vertices, nv, faces, nf, iterations);
}

mpm_status mpm_export_particles(mpm_ctx* c, int32_t slot, float radius, int64_t* n) {
  if (!c || !n || slot < 0 || slot > 1) return MPM_ERR_INVALID;
  auto& x = c->exports[slot];
  if (!c->copy_stream) MPM_CUDA(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
  if (!x.packed) {
    MPM_CUDA(c, cudaEventCreateWithFlags(&x.packed, cudaEventDisableTiming));
    MPM_CUDA(c, cudaEventCreateWithFlags(&x.copied, cudaEventDisableTiming));
  }
  const int64_t cnt = c->n;
  if (x.pending) {
    if (cnt > x.cap) {
      MPM_CUDA(c, cudaEventSynchronize(x.copied));  // the buffers are about to be replaced
    } else {
      MPM_CUDA(c, cudaStreamWaitEvent(c->stream, x.copied, 0));  // the device buffer is still being read
    }
  }
  if (cnt > x.cap) {
    cudaFree(x.dev);
    cudaFreeHost(x.host);
    x.dev = x.host = nullptr;
    x.cap = 0;
    const size_t bytes = (size_t)kBgeoRecordBytes * (size_t)cnt;
    if (cudaMalloc(&x.dev, bytes) != cudaSuccess) return fail(c, MPM_ERR_NOMEM, "export: device buffer");
    if (cudaMallocHost(&x.host, bytes) != cudaSuccess) return fail(c, MPM_ERR_NOMEM, "export: pinned buffer");
    x.cap = cnt;
  }
  const uint32_t* inv = nullptr;
  MPM_CUDA(c, inverse_ids(c, &inv));
  MPM_CUDA(c, launch_bgeo_pack(c->sA, c->stride, inv, cnt, radius, x.dev, c->stream));
  MPM_CUDA(c, cudaEventRecord(x.packed, c->stream));
  MPM_CUDA(c, cudaStreamWaitEvent(c->copy_stream, x.packed, 0));
  if (cnt > 0)
    MPM_CUDA(c, cudaMemcpyAsync(x.host, x.dev, (size_t)kBgeoRecordBytes * (size_t)cnt, cudaMemcpyDeviceToHost,
                                c->copy_stream));
  MPM_CUDA(c, cudaEventRecord(x.copied, c->copy_stream));
  c->launches += cnt > 0;
  x.n = cnt;
  x.pending = true;
  *n = cnt;
  return MPM_OK;
}

mpm_status mpm_export_wait(mpm_ctx* c, int32_t slot, const void** records, int64_t* n) {
  if (!c || !records || !n || slot < 0 || slot > 1) return MPM_ERR_INVALID;
  auto& x = c->exports[slot];
  if (!x.pending) return fail(c, MPM_ERR_INVALID, "export_wait: nothing exported into this slot");
  MPM_CUDA(c, cudaEventSynchronize(x.copied));
  *records = x.host;
  *n = x.n;
  return MPM_OK;
}

int64_t mpm_bgeo_header(int64_t n, uint8_t* out, int64_t capacity) { return bgeo_header(n, out, capacity); }

mpm_status mpm_write_bgeo(const char* path, const void* records, int64_t n) {
  if (!path || n < 0 || (n > 0 && !records)) return MPM_ERR_INVALID;
  uint8_t head[256];
  const int64_t hn = bgeo_header(n, head, sizeof(head));
  FILE* f = std::fopen(path, "wb");
  if (!f) return MPM_ERR_IO;
  bool ok = std::fwrite(head, 1, (size_t)hn, f) == (size_t)hn;
  if (ok && n > 0)
    ok = std::fwrite(records, 1, (size_t)kBgeoRecordBytes * (size_t)n, f) == (size_t)kBgeoRecordBytes * (size_t)n;
  if (ok) ok = std::fwrite(kBgeoTerminator, 1, 2, f) == 2;
  ok = (std::fclose(f) == 0) && ok;
  return ok ? MPM_OK : MPM_ERR_IO;
}

mpm_status mpm_render_positions_device(mpm_ctx* c, const float** positions) {
  if (!c || !positions) return MPM_ERR_INVALID;
  if (c->n > c->positions_cap) {
    cudaFree(c->positions);
    c->positions = nullptr;
    c->positions_cap = 0;
    if (cudaMalloc(&c->positions, sizeof(float) * 3 * (size_t)c->n) != cudaSuccess)
      return fail(c, MPM_ERR_NOMEM, "render: positions");
    c->positions_cap = c->n;
  }
  const uint32_t* inv = nullptr;
  MPM_CUDA(c, inverse_ids(c, &inv));
  MPM_CUDA(c, launch_project(c->sA, c->stride, inv, c->n, c->positions, c->stream));
  c->launches += c->n > 0;
  *positions = c->positions;
  return MPM_OK;
}

mpm_status mpm_render_positions(mpm_ctx* c, float* out) {
  if (!c || (!out && c->n > 0)) return MPM_ERR_INVALID;
  const float* d = nullptr;
  mpm_status st = mpm_render_positions_device(c, &d);
  if (st != MPM_OK) return st;
  if (c->n > 0)
    MPM_CUDA(c, cudaMemcpyAsync(out, d, sizeof(float) * 3 * (size_t)c->n, cudaMemcpyDeviceToHost, c->stream));
  MPM_CUDA(c, cudaStreamSynchronize(c->stream));
  return MPM_OK;
}

mpm_status mpm_render_points(mpm_ctx* c, int32_t W, int32_t H, float point_size, const uint8_t color[3],
                             const uint8_t background[3], uint8_t* rgb) {
  if (!c || !rgb || !color || !background || W <= 0 || H <= 0 || W > 16384 || H > 16384 || !(point_size > 0.f) ||
      !(point_size <= 64.f))
    return fail(c, MPM_ERR_INVALID, "render: bad image size, point size or buffer");
  const int64_t pixels = (int64_t)W * H;
  if (4 * pixels > c->image_cap) {
    cudaFree(c->image);
    c->image = nullptr;
    c->image_cap = 0;
    if (cudaMalloc(&c->image, (size_t)(4 * pixels)) != cudaSuccess) return fail(c, MPM_ERR_NOMEM, "render: image");
    c->image_cap = 4 * pixels;
  }
  MPM_CUDA(c, launch_render_points(c->sA, c->stride, c->n, W, H, point_size, color, background, c->image,
                                   c->image + pixels, c->stream));
  c->launches += 2 + (c->n > 0);
  MPM_CUDA(c, cudaMemcpyAsync(rgb, c->image + pixels, (size_t)(3 * pixels), cudaMemcpyDeviceToHost, c->stream));
  MPM_CUDA(c, cudaStreamSynchronize(c->stream));
  return MPM_OK;
}

mpm_status mpm_check_wait_timeout(mpm_ctx* c, int32_t polls) {
  if (!c || polls < 1 || polls > (1 << 20)) return MPM_ERR_INVALID;
  MPM_CUDA(c, launch_wait_timeout_probe(c->status, polls, c->stream));
  c->launches += 1;
  return mpm_sync(c);
}

mpm_status mpm_sort(mpm_ctx* c) {
  if (!c) return MPM_ERR_INVALID;
  return run_sort(c, false);
}

mpm_status mpm_substep_many(mpm_ctx* const* ctxs, int32_t count, int32_t nsteps) {
  if (!ctxs || count < 0 || nsteps < 0) return MPM_ERR_INVALID;
  for (int32_t i = 0; i < count; ++i)
    if (!ctxs[i]) return MPM_ERR_INVALID;
  for (int32_t s = 0; s < nsteps; ++s)
    for (int32_t i = 0; i < count; ++i) {
      const mpm_status st = mpm_substep(ctxs[i], 1);
      if (st != MPM_OK) return st;
    }
  return MPM_OK;
}

int64_t mpm_particle_count(const mpm_ctx* c) { return c ? c->n : -1; }
int64_t mpm_substep_count(const mpm_ctx* c) { return c ? c->substeps : -1; }
int64_t mpm_launch_count(const mpm_ctx* c) { return c ? c->launches : -1; }

mpm_status mpm_last_error(const mpm_ctx* c, char* buf, size_t len) {
  if (!c || !buf || len == 0) return MPM_ERR_INVALID;
  std::snprintf(buf, len, "%s", c->last_error.c_str());
  return MPM_OK;
}

mpm_status mpm_set_tuning(mpm_ctx* c, int32_t steps_per_warp, int32_t warps_per_cta, int32_t tile_box) {
  if (!c) return MPM_ERR_INVALID;
  if (steps_per_warp < 0 || steps_per_warp > 256) return fail(c, MPM_ERR_INVALID, "steps_per_warp out of range");
  if (warps_per_cta != 0 && warps_per_cta != 4 && warps_per_cta != 6 && warps_per_cta != 12)
    return fail(c, MPM_ERR_INVALID, "warps_per_cta must be 4, 6 or 12 (0 keeps the current value)");
  if (tile_box < 0 || tile_box > MPM_TILE_4x6x6)
    return fail(c, MPM_ERR_INVALID, "tile_box must be one of MPM_TILE_* (0 keeps the default box)");
  StepTuning t = c->tuning;
  if (warps_per_cta) t.warps = warps_per_cta;
  if (tile_box) t.tile = tile_box - 1;
  if (t.tile != 0 && t.warps != kStepWarps)
    return fail(c, MPM_ERR_INVALID, "the 4x4x4 and 4x6x6 tile boxes run with 12 warps per CTA");
  if (steps_per_warp) c->steps_per_warp = steps_per_warp;
  c->tuning = t;
  return MPM_OK;
}

// ---------------------------------------------------------------------------
// Autotuner.  The reference launches a fixed 64-thread block per 64 particles
// (src/mpm.cu:217-222); here the fused kernel's launch shape is searched per workload
// class on a clone of the caller's scene, so the caller's state is not touched.
// ---------------------------------------------------------------------------
}  // extern "C"

namespace {

struct TuneCandidate {
  int spw, warps, tile_box, sort;  // tile_box: MPM_TILE_*
};

std::string device_key(int dev) {
  cudaDeviceProp p{};
  if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) return "unknown device";
  char b[320];
  std::snprintf(b, sizeof(b), "%s (%d SMs, cc %d.%d)", p.name, p.multiProcessorCount, p.major, p.minor);
  return b;
}

// Changes with every build of this file, so a rebuilt library measures again.
const char* build_key() { return "mpm_gb300 " __DATE__ " " __TIME__; }

// Workload class: particle layout, grid size, particle count to the nearest power of two,
// and the material kinds present.
std::string class_key(const mpm_ctx* c) {
  unsigned kinds = 0;
  for (int i = 0; i < c->n_materials; ++i) kinds |= 1u << c->mats[i].kind;
  const int lg = c->n > 0 ? (int)std::lround(std::log2((double)c->n)) : 0;
  char b[160];
  std::snprintf(b, sizeof(b), "%s N=%u n~2^%d kinds=0x%x", c->liquid_layout ? "liquid" : "general", c->params.N, lg,
                kinds);
  return b;
}

// A context with the caller's parameters, materials and particle arrays (copied on the
// device), for timing launch shapes.
mpm_status tuning_clone(mpm_ctx* c, mpm_ctx** out) {
  mpm_ctx* t = nullptr;
  mpm_status st = mpm_create(&c->params, &t);
  if (st != MPM_OK) return st;
  st = mpm_set_materials(t, c->mats, c->n_materials);
  if (st == MPM_OK) st = ensure_particles(t, c->n);
  if (st != MPM_OK) {
    mpm_destroy(t);
    return st;
  }
  *out = t;
  return MPM_OK;
}

// Resets the clone to the caller's current particles.
mpm_status tuning_restore(mpm_ctx* c, mpm_ctx* t) {
  MPM_CUDA(c, cudaMemcpy2DAsync(t->sA, sizeof(float) * t->stride, c->sA, sizeof(float) * c->stride,
                                sizeof(float) * c->n, kNumComps, cudaMemcpyDeviceToDevice, t->stream));
  if (c->have_mat) MPM_CUDA(c, cudaMemcpyAsync(t->matA, c->matA, c->n, cudaMemcpyDeviceToDevice, t->stream));
  MPM_CUDA(c, cudaMemcpyAsync(t->idA, c->idA, sizeof(uint32_t) * c->n, cudaMemcpyDeviceToDevice, t->stream));
  t->n = c->n;
  t->inv = nullptr;
  t->have_mat = c->have_mat;
  t->unsorted = c->unsorted;
  t->pending = false;
  t->tail_g2p = t->ended_g2p = false;
  t->prev = -1;
  t->substeps = 0;
  t->t = 0.0;
  return MPM_OK;
}

// Mean device time of one substep (microseconds) with candidate k: `warm` substeps (the
// run's first P2G and, with sorting, a sort), then `steps` timed substeps.
mpm_status time_candidate(mpm_ctx* c, mpm_ctx* t, const TuneCandidate& k, int warm, int steps, cudaEvent_t e0,
                          cudaEvent_t e1, double* us) {
  mpm_status st = tuning_restore(c, t);
  if (st != MPM_OK) return st;
  t->steps_per_warp = k.spw;
  t->tuning = StepTuning{k.warps, k.tile_box - 1};
  t->params.sort_interval = k.sort;
  t->since_sort = k.sort;  // sort first, as after an upload
  st = mpm_substep(t, warm);
  if (st != MPM_OK) return fail(c, st, "tuning: " + t->last_error);
  MPM_CUDA(c, cudaEventRecord(e0, t->stream));
  st = mpm_substep(t, steps);
  if (st != MPM_OK) return fail(c, st, "tuning: " + t->last_error);
  MPM_CUDA(c, cudaEventRecord(e1, t->stream));
  st = mpm_sync(t);
  if (st != MPM_OK) return fail(c, st, "tuning: " + t->last_error);
  float ms = 0.f;
  MPM_CUDA(c, cudaEventElapsedTime(&ms, e0, e1));
  *us = 1e3 * (double)ms / steps;
  return MPM_OK;
}

void apply_tuning(mpm_ctx* c, const TuneCandidate& k, bool with_sort) {
  c->steps_per_warp = k.spw;
  c->tuning = StepTuning{k.warps, k.tile_box - 1};
  if (with_sort) c->params.sort_interval = k.sort;
}

}  // namespace

extern "C" {

mpm_status mpm_autotune(mpm_ctx* c, const char* cache_path, int32_t flags, int32_t budget_substeps,
                        mpm_tuning* out) {
  mpm_status st = check_ready(c);
  if (st != MPM_OK) return st;
  if (c->n <= 0) return fail(c, MPM_ERR_INVALID, "autotune needs uploaded particles");
  if (budget_substeps < 0 || budget_substeps > 4096) return fail(c, MPM_ERR_INVALID, "budget_substeps out of range");
  if (flags & ~(MPM_TUNE_SORT_INTERVAL | MPM_TUNE_IGNORE_CACHE)) return fail(c, MPM_ERR_INVALID, "unknown flags");
  const bool with_sort = (flags & MPM_TUNE_SORT_INTERVAL) != 0;
  const std::string dkey = device_key(c->device), bkey = build_key();
  const std::string ckey = class_key(c) + (with_sort ? " +sort" : "");
  TuneCandidate best{c->steps_per_warp, c->tuning.warps, c->tuning.tile + 1, c->params.sort_interval};
  mpm_tuning res{};
  if (cache_path && !(flags & MPM_TUNE_IGNORE_CACHE)) {
    TuningEntry e;
    if (find_tuning(read_tuning_cache(cache_path), dkey, bkey, ckey, &e) && e.steps_per_warp >= 1 &&
        e.steps_per_warp <= 256 && (e.warps_per_cta == 4 || e.warps_per_cta == 6 || e.warps_per_cta == 12) &&
        e.tile_box >= MPM_TILE_4x4x6 && e.tile_box <= MPM_TILE_4x6x6 && e.sort_interval >= 0 &&
        (e.tile_box == MPM_TILE_4x4x6 || e.warps_per_cta == kStepWarps)) {
      best = TuneCandidate{e.steps_per_warp, e.warps_per_cta, e.tile_box, with_sort ? e.sort_interval : best.sort};
      apply_tuning(c, best, with_sort);
      res = mpm_tuning{best.spw, best.warps, best.tile_box, c->params.sort_interval, e.us_per_substep, 1, 0};
      if (out) *out = res;
      return MPM_OK;
    }
  }
  MPM_CUDA(c, cudaStreamSynchronize(c->stream));  // the clone copies the current particles
  mpm_ctx* t = nullptr;
  st = tuning_clone(c, &t);
  if (st != MPM_OK) return fail(c, st, "tuning: cannot create the trial context");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    mpm_destroy(t);
    return fail(c, MPM_ERR_CUDA, "tuning: cannot create events");
  }
  const int steps = budget_substeps > 0 ? budget_substeps : 48;
  const int warm = 4;
  int timed = 0;
  double best_us = 0.0;
  auto run = [&](TuneCandidate k, int n_steps, double* us) -> mpm_status {
    ++timed;
    return time_candidate(c, t, k, warm, n_steps, e0, e1, us);
  };
  // Coordinate descent from the current shape: steps per warp, CTA size, tile box and,
  // when asked for, the sort interval; a knob moves only for a gain above 1 %, so timing
  // noise does not flip it.
  st = run(best, steps, &best_us);
  auto consider = [&](TuneCandidate k, int n_steps, double base_us, TuneCandidate& cur, double& cur_us) {
    double us = 0.0;
    if (st != MPM_OK) return;
    st = run(k, n_steps, &us);
    if (st == MPM_OK && us < 0.99 * cur_us && us < 0.99 * base_us) {
      cur = k;
      cur_us = us;
    }
  };
  for (int spw : {1, 2, 4, 8})
    if (spw != best.spw) {
      TuneCandidate k = best;
      k.spw = spw;
      TuneCandidate cur = best;
      double cur_us = best_us;
      consider(k, steps, best_us, cur, cur_us);
      best = cur;
      best_us = cur_us;
    }
  for (int warps : {4, 6, 12})
    if (warps != best.warps) {
      TuneCandidate k = best;
      k.warps = warps;
      k.tile_box = MPM_TILE_4x4x6;
      TuneCandidate cur = best;
      double cur_us = best_us;
      consider(k, steps, best_us, cur, cur_us);
      best = cur;
      best_us = cur_us;
    }
  for (int box : {MPM_TILE_4x4x6, MPM_TILE_4x4x4, MPM_TILE_4x6x6})
    if (box != best.tile_box) {
      TuneCandidate k = best;
      k.tile_box = box;
      if (box != MPM_TILE_4x4x6) k.warps = kStepWarps;
      TuneCandidate cur = best;
      double cur_us = best_us;
      consider(k, steps, best_us, cur, cur_us);
      best = cur;
      best_us = cur_us;
    }
  if (with_sort && st == MPM_OK) {
    // a sort interval is timed over at least two of its periods; the current shape is
    // re-timed over the same length so the comparison is even
    for (int si : {4, 8, 16, 32, 64})
      if (si != best.sort) {
        const int n_steps = std::max(steps, 2 * std::max(si, best.sort));
        double base_us = 0.0;
        if (st == MPM_OK) st = run(best, n_steps, &base_us);
        TuneCandidate k = best;
        k.sort = si;
        TuneCandidate cur = best;
        double cur_us = base_us;
        consider(k, n_steps, base_us, cur, cur_us);
        if (st == MPM_OK && cur.sort != best.sort) {
          best = cur;
          best_us = cur_us;
        }
      }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  mpm_destroy(t);
  if (st != MPM_OK) return st;
  apply_tuning(c, best, with_sort);
  res = mpm_tuning{best.spw, best.warps, best.tile_box, c->params.sort_interval, best_us, 0, timed};
  if (cache_path) {
    TuningEntry e;
    e.device = dkey;
    e.build = bkey;
    e.klass = ckey;
    e.steps_per_warp = best.spw;
    e.warps_per_cta = best.warps;
    e.tile_box = best.tile_box;
    e.sort_interval = c->params.sort_interval;
    e.us_per_substep = best_us;
    if (!store_tuning(cache_path, e)) {
      if (out) *out = res;
      return fail(c, MPM_ERR_IO, std::string("tuning: cannot write the cache file ") + cache_path);
    }
  }
  if (out) *out = res;
  return MPM_OK;
}

int32_t mpm_material_kind_available(int32_t kind) {
  if (kind >= 0 && kind <= MPM_MAT_LIQUID) return 1;
  return find_material_kernels(kind, nullptr) ? 1 : 0;
}

mpm_status mpm_get_tuning(const mpm_ctx* c, mpm_tuning* out) {
  if (!c || !out) return MPM_ERR_INVALID;
  *out = mpm_tuning{c->steps_per_warp, c->tuning.warps, c->tuning.tile + 1, c->params.sort_interval, 0.0, 0, 0};
  return MPM_OK;
}

}  // extern "C"
