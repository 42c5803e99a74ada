// Batched scenes: many independent MLS-MPM scenes (own N, dt, material, particle
// count) advanced together, one launch per substep for the whole batch.
//
// The reference simulates one scene per Simulation (include/mpm.cuh:44-106); a batch is
// the GB300 form of running many of them: all particles sit in one component-major
// SoA (scene after scene, each scene cell-sorted inside its segment), all grids in one
// pool, and the fused substep kernel walks a table of particle ranges that never cross
// a scene boundary.  Grids are cleared sparsely (the box each scene's P2G touched),
// not as dense N^3 blocks.  A run of substeps can be captured once as a CUDA graph and
// replayed.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <set>
#include <string>
#include <vector>

#include "mpm_internal.h"
#include "tuning_cache.h"

using namespace mpm;

struct mpm_batch {
  int nscenes = 0;
  std::vector<mpm_scene> scenes;
  std::vector<int64_t> start;  // nscenes + 1
  SimConsts K{};
  int sort_interval = 16;
  // 8 steps per range: consecutive steps of a warp gather nearby nodes, which L1 then
  // holds; longer ranges balance worse (the 256-scene workload: 8.35e9 particle-substeps/s
  // against 8.31e9 with 4 steps, 8.16e9 with 2, 7.79e9 with 1, 8.09e9 with 16, 7.42e9 with 32)
  int steps_per_warp = 8;
  int blocks_p2g = 1, blocks_fused = 1;  // launch grids, fixed at creation (outside any capture)

  int device = 0, num_sms = 1;
  cudaStream_t stream = nullptr, own_stream = nullptr;

  int64_t n = 0, stride = 0;
  float* sA = nullptr;
  float* sB = nullptr;
  uint8_t* matA = nullptr;
  uint8_t* matB = nullptr;
  uint32_t* idA = nullptr;
  uint32_t* idB = nullptr;
  uint32_t* keys = nullptr;

  int64_t cells = 0;  // total grid nodes of all scenes
  float4* grid[3] = {nullptr, nullptr, nullptr};
  float4* vgrid = nullptr;  // padded velocity grids of all scenes
  int64_t vcells = 0;
  SceneDev* d_scenes = nullptr;
  int64_t* d_start = nullptr;
  uint32_t* d_key_base = nullptr;
  int64_t key_space = 0;
  int* counts = nullptr;
  int* block_sums = nullptr;
  int4* d_ranges = nullptr;
  int nranges = 0;
  int* boxes = nullptr;
  int* status = nullptr;
  float* stage = nullptr;

  int cur = 0;
  bool pending = false;
  int64_t launch_index = 0;  // fused/P2G launches since upload (selects the box slots)
  int64_t since_sort = 0;
  int64_t launches = 0;
  struct Graph {
    cudaGraphExec_t exec;
    int64_t launches;  // kernels one replay runs
    int sorts;         // cell sorts one replay runs (each swaps the particle buffers)
    int since_sort;    // substeps after the replay's last sort
  };
  std::map<std::pair<int, int>, Graph> graphs;  // (nsteps, launch_index % 6) -> graph
  std::string last_error;
};

namespace {

mpm_status bfail(mpm_batch* b, mpm_status code, const std::string& msg) {
  if (b) b->last_error = msg;
  return code;
}

#define BCUDA(b, call)                                                                          \
  do {                                                                                          \
    cudaError_t _e = (call);                                                                    \
    if (_e != cudaSuccess)                                                                      \
      return bfail((b), _e == cudaErrorMemoryAllocation ? MPM_ERR_NOMEM : MPM_ERR_CUDA,         \
                   std::string(#call) + ": " + cudaGetErrorString(_e));                         \
  } while (0)

void free_graphs(mpm_batch* b) {
  for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second.exec);
  b->graphs.clear();
}

// The range table for the batch's steps_per_warp (ranges of 32 * steps_per_warp
// particles that never cross a scene) and the launch grids sized by its length.  The
// caller makes sure no launch still reads the old table.
mpm_status build_ranges(mpm_batch* b) {
  std::vector<int4> ranges;
  const int64_t chunk = 32 * (int64_t)b->steps_per_warp;
  for (int i = 0; i < b->nscenes; ++i)
    for (int64_t p = 0; p < b->scenes[i].count; p += chunk)
      ranges.push_back(make_int4(i, (int)(b->start[i] + p), (int)(b->start[i] + std::min(p + chunk, b->scenes[i].count)),
                                 0));
  cudaFree(b->d_ranges);
  b->d_ranges = nullptr;
  b->nranges = 0;
  BCUDA(b, cudaMalloc(&b->d_ranges, sizeof(int4) * std::max<size_t>(ranges.size(), 1)));
  if (!ranges.empty())
    BCUDA(b, cudaMemcpy(b->d_ranges, ranges.data(), sizeof(int4) * ranges.size(), cudaMemcpyHostToDevice));
  b->nranges = (int)ranges.size();
  for (int k = 0; k < 2; ++k) {
    const StepKind kind = k ? kStepFused : kStepP2GOnly;
    const int bps = step_blocks_per_sm(kind, false, false, step_smem_bytes(kind, true), true);
    const int blocks = std::max(1, std::min((b->nranges + kStepWarps - 1) / kStepWarps, b->num_sms * bps));
    (k ? b->blocks_fused : b->blocks_p2g) = blocks;
  }
  return MPM_OK;
}

mpm_status launch(mpm_batch* b, StepKind kind) {
  StepArgs a{};
  a.s = b->sA;
  a.stride = b->stride;
  a.mat = nullptr;  // the material comes from the scene table
  a.id = b->idA;
  a.n = b->n;
  a.status = b->status;
  a.K = b->K;
  a.nscenes = b->nscenes;
  a.ranges = b->d_ranges;
  a.nranges = b->nranges;
  a.scenes = b->d_scenes;
  a.boxes = b->boxes;
  const int64_t L = b->launch_index;
  a.box_record = (int)(L % kBoxSlots);
  a.box_clear = (int)((L + kBoxSlots - 2) % kBoxSlots);
  a.box_reset = (int)((L + 1) % kBoxSlots);
  const int r = b->cur;
  a.grid_in = (kind == kStepP2GOnly) ? nullptr : b->grid[r];
  a.vgrid = b->vgrid;
  if (kind != kStepP2GOnly) {
    // velocity pass over the boxes the previous launch's P2G recorded
    BCUDA(b, launch_batch_velocity(b->grid[r], b->vgrid, b->d_scenes, b->nscenes, b->boxes,
                                   (int)((L + kBoxSlots - 1) % kBoxSlots), b->stream));
    b->launches += 1;
  }
  a.grid_out = b->grid[(r + 1) % 3];
  a.grid_zero = b->grid[(r + 2) % 3];
  a.chunk = 32 * b->steps_per_warp;
  const int blocks = (kind == kStepP2GOnly) ? b->blocks_p2g : b->blocks_fused;
  BCUDA(b, launch_step(a, kind, false, false, blocks, b->stream, &b->launches));
  b->cur = (r + 1) % 3;
  b->launch_index += 1;
  b->pending = true;
  return MPM_OK;
}

// g2p_next: as run_sort in capi.cu (the launch after the sort is a fused launch)
mpm_status sort(mpm_batch* b, bool g2p_next) {
  SortArgs s{};
  s.sA = b->sA;
  s.sB = b->sB;
  s.stride = b->stride;
  s.n = b->n;
  s.matA = nullptr;  // per-scene materials: nothing per particle to move
  s.matB = b->matB;
  s.idA = b->idA;
  s.idB = b->idB;
  s.keys = b->keys;
  s.counts = b->counts;
  s.block_sums = b->block_sums;
  s.cells = b->key_space;
  s.ncomp = kNumComps;
  s.nscenes = b->nscenes;
  s.scene_start = b->d_start;
  s.scene_key_base = b->d_key_base;
  s.scenes = b->d_scenes;
  s.partial = g2p_next && b->key_space <= (int64_t)kKeyOutside;
  BCUDA(b, launch_sort(s, b->num_sms, b->stream, &b->launches));
  std::swap(b->sA, b->sB);
  std::swap(b->matA, b->matB);
  std::swap(b->idA, b->idB);
  b->since_sort = 0;
  return MPM_OK;
}

// Zero P2G grids and empty box slots, as after an upload (synchronises: the box table
// is copied from the host).
mpm_status fresh_grids(mpm_batch* b) {
  for (auto& g : b->grid) BCUDA(b, cudaMemsetAsync(g, 0, sizeof(float4) * b->cells, b->stream));
  std::vector<int> boxes(6 * kBoxSlots * b->nscenes);
  for (size_t i = 0; i < boxes.size(); ++i) boxes[i] = (i % 6 < 3) ? INT_MAX : INT_MIN;
  BCUDA(b, cudaMemcpyAsync(b->boxes, boxes.data(), sizeof(int) * boxes.size(), cudaMemcpyHostToDevice, b->stream));
  BCUDA(b, cudaStreamSynchronize(b->stream));
  return MPM_OK;
}

mpm_status advance(mpm_batch* b, int32_t nsteps) {
  for (int32_t i = 0; i < nsteps; ++i) {
    if (b->sort_interval > 0 && b->since_sort >= b->sort_interval) {
      mpm_status st = sort(b, b->pending);
      if (st != MPM_OK) return st;
    }
    if (!b->pending) {
      mpm_status st = launch(b, kStepP2GOnly);
      if (st != MPM_OK) return st;
    }
    mpm_status st = launch(b, kStepFused);
    if (st != MPM_OK) return st;
    b->since_sort += 1;
  }
  return MPM_OK;
}

}  // namespace

extern "C" {

mpm_status mpm_batch_create(const mpm_scene* scenes, int32_t nscenes, int32_t sort_interval, mpm_batch** out) {
  if (!out || !scenes || nscenes <= 0 || sort_interval < 0) return MPM_ERR_INVALID;
  *out = nullptr;
  for (int i = 0; i < nscenes; ++i) {
    const mpm_params& p = scenes[i].params;
    if (p.N < 4 || p.N > 1000 || !(p.dt > 0.f) || p.boundary_mode < 0 || p.boundary_mode > 2 ||
        p.boundary_cells < 0 || (uint32_t)p.boundary_cells * 2 > p.N || scenes[i].count < 0)
      return MPM_ERR_INVALID;
    if (p.g2p_guard) return MPM_ERR_UNSUPPORTED;
    const mpm_material& m = scenes[i].material;
    if (m.kind < 0 || m.kind > MPM_MAT_LIQUID || !(m.particle_volume > 0.f) || !(m.density > 0.f))
      return MPM_ERR_INVALID;
  }

  mpm_batch* b = new mpm_batch();
  auto bail = [&](mpm_status s) {
    mpm_batch_destroy(b);
    return s;
  };
  b->nscenes = nscenes;
  b->scenes.assign(scenes, scenes + nscenes);
  make_sim_consts(scenes[0].params, &scenes[0].material, 1, b->K);
  b->sort_interval = sort_interval;
  if (cudaGetDevice(&b->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, b->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(MPM_ERR_CUDA);
  b->stream = b->own_stream;

  // particle segments, grid pool, sort key bases, range table
  b->start.resize(nscenes + 1);
  std::vector<SceneDev> sd(nscenes);
  std::vector<uint32_t> key_base(nscenes);
  int64_t off = 0, cells = 0, keys = 0, vcells = 0;
  for (int i = 0; i < nscenes; ++i) {
    b->start[i] = off;
    make_grid_consts(scenes[i].params, sd[i].g);
    make_dev_material(scenes[i].material, sd[i].m);
    sd[i].grid_offset = cells;
    sd[i].vgrid_offset = vcells;
    const int64_t N = scenes[i].params.N;
    cells += N * N * N;
    vcells += vgrid_nodes((int)N);
    const int64_t nb = (N + 3) / 4;
    key_base[i] = (uint32_t)keys;
    keys += nb * nb * nb * 64;
    off += scenes[i].count;
  }
  b->start[nscenes] = off;
  if (off > (int64_t)INT_MAX || keys > (int64_t)UINT32_MAX) return bail(MPM_ERR_UNSUPPORTED);
  b->n = off;
  b->stride = std::max<int64_t>(64, (off + 63) / 64 * 64);
  b->cells = cells;
  b->vcells = vcells;
  b->key_space = keys;
  if (build_ranges(b) != MPM_OK) return bail(MPM_ERR_NOMEM);

  const size_t fb = sizeof(float) * (size_t)kNumComps * b->stride;
  if (cudaMalloc(&b->sA, fb) || cudaMalloc(&b->sB, fb) || cudaMalloc(&b->matA, b->stride) ||
      cudaMalloc(&b->matB, b->stride) || cudaMalloc(&b->idA, 4 * b->stride) || cudaMalloc(&b->idB, 4 * b->stride) ||
      cudaMalloc(&b->keys, 4 * b->stride) || cudaMalloc(&b->stage, fb))
    return bail(MPM_ERR_NOMEM);
  for (auto& g : b->grid) {
    if (cudaMalloc(&g, sizeof(float4) * std::max<int64_t>(cells, 1))) return bail(MPM_ERR_NOMEM);
    if (cudaMemsetAsync(g, 0, sizeof(float4) * cells, b->stream)) return bail(MPM_ERR_CUDA);
  }
  if (cudaMalloc(&b->vgrid, sizeof(float4) * std::max<int64_t>(vcells, 1))) return bail(MPM_ERR_NOMEM);
  if (cudaMemsetAsync(b->vgrid, 0, sizeof(float4) * vcells, b->stream)) return bail(MPM_ERR_CUDA);
  const int64_t nbs = (keys + kThreads * 8 - 1) / (kThreads * 8);
  if (cudaMalloc(&b->counts, 4 * keys) || cudaMalloc(&b->block_sums, 4 * std::max<int64_t>(nbs, 1)) ||
      cudaMalloc(&b->d_scenes, sizeof(SceneDev) * nscenes) || cudaMalloc(&b->d_start, 8 * (nscenes + 1)) ||
      cudaMalloc(&b->d_key_base, 4 * nscenes) || cudaMalloc(&b->boxes, sizeof(int) * 6 * kBoxSlots * nscenes) ||
      cudaMalloc(&b->status, sizeof(int)))
    return bail(MPM_ERR_NOMEM);
  std::vector<int> boxes(6 * kBoxSlots * nscenes);
  for (size_t i = 0; i < boxes.size(); ++i) boxes[i] = (i % 6 < 3) ? INT_MAX : INT_MIN;
  if (cudaMemcpy(b->d_scenes, sd.data(), sizeof(SceneDev) * nscenes, cudaMemcpyHostToDevice) ||
      cudaMemcpy(b->d_start, b->start.data(), 8 * (nscenes + 1), cudaMemcpyHostToDevice) ||
      cudaMemcpy(b->d_key_base, key_base.data(), 4 * nscenes, cudaMemcpyHostToDevice) ||
      cudaMemcpy(b->boxes, boxes.data(), sizeof(int) * boxes.size(), cudaMemcpyHostToDevice) ||
      cudaMemset(b->status, 0, sizeof(int)) ||
      cudaStreamSynchronize(b->stream))
    return bail(MPM_ERR_CUDA);
  *out = b;
  return MPM_OK;
}

mpm_status mpm_batch_destroy(mpm_batch* b) {
  if (!b) return MPM_ERR_INVALID;
  if (b->stream) cudaStreamSynchronize(b->stream);
  free_graphs(b);
  for (void* p : {(void*)b->sA, (void*)b->sB, (void*)b->matA, (void*)b->matB, (void*)b->idA, (void*)b->idB,
                  (void*)b->keys, (void*)b->stage, (void*)b->grid[0], (void*)b->grid[1], (void*)b->grid[2], (void*)b->vgrid,
                  (void*)b->counts, (void*)b->block_sums, (void*)b->d_scenes, (void*)b->d_start, (void*)b->d_key_base,
                  (void*)b->d_ranges, (void*)b->boxes, (void*)b->status})
    cudaFree(p);
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  delete b;
  return MPM_OK;
}

mpm_status mpm_batch_set_stream(mpm_batch* b, void* stream) {
  if (!b) return MPM_ERR_INVALID;
  if (!stream) return bfail(b, MPM_ERR_INVALID, "a batch needs a non-default stream (graph capture)");
  b->stream = (cudaStream_t)stream;
  free_graphs(b);
  return MPM_OK;
}

mpm_status mpm_batch_upload_soa(mpm_batch* b, const float* x, const float* v, const float* C, const float* F,
                                const float* Jp) {
  if (!b) return MPM_ERR_INVALID;
  const int64_t n = b->n;
  if (n > 0 && !x) return bfail(b, MPM_ERR_INVALID, "x is required");
  for (int64_t i = 0; i < 3 * n; ++i)
    if (!std::isfinite(x[i])) return bfail(b, MPM_ERR_INVALID, "non-finite particle position");
  b->pending = false;
  b->launch_index = 0;
  b->since_sort = b->sort_interval;
  if (n == 0) return MPM_OK;
  float* xs = b->stage;
  float* vs = xs + 3 * n;
  float* Cs = vs + 3 * n;
  float* Fs = Cs + 9 * n;
  float* Js = Fs + 9 * n;
  BCUDA(b, cudaMemcpyAsync(xs, x, 12 * n, cudaMemcpyHostToDevice, b->stream));
  if (v) BCUDA(b, cudaMemcpyAsync(vs, v, 12 * n, cudaMemcpyHostToDevice, b->stream));
  if (C) BCUDA(b, cudaMemcpyAsync(Cs, C, 36 * n, cudaMemcpyHostToDevice, b->stream));
  if (F) BCUDA(b, cudaMemcpyAsync(Fs, F, 36 * n, cudaMemcpyHostToDevice, b->stream));
  if (Jp) BCUDA(b, cudaMemcpyAsync(Js, Jp, 4 * n, cudaMemcpyHostToDevice, b->stream));
  BCUDA(b, launch_deinterleave(b->stage, b->sA, b->stride, n, v != nullptr, C != nullptr, F != nullptr,
                               Jp != nullptr, b->stream));
  BCUDA(b, launch_iota(b->idA, n, b->stream));
  b->launches += 2;
  const mpm_status st = fresh_grids(b);
  if (st != MPM_OK) return st;
  BCUDA(b, cudaStreamSynchronize(b->stream));
  return MPM_OK;
}

mpm_status mpm_batch_substep(mpm_batch* b, int32_t nsteps) {
  if (!b || nsteps < 0) return MPM_ERR_INVALID;
  if (b->n == 0) return MPM_OK;
  return advance(b, nsteps);
}

mpm_status mpm_batch_substep_graph(mpm_batch* b, int32_t nsteps) {
  if (!b || nsteps < 0) return MPM_ERR_INVALID;
  if (b->n == 0 || nsteps == 0) return MPM_OK;
  if (!b->pending) {  // the first P2G of a run stays outside the graph
    mpm_status st = launch(b, kStepP2GOnly);
    if (st != MPM_OK) return st;
  }
  // A captured run is nsteps fused launches with a cell sort (when sorting is on) before the
  // first and then every sort_interval substeps: a 256-scene workload ran 8.28e9
  // particle-substeps/s with one sort per 50-substep replay and 8.55e9 with one per 16.
  // The graph bakes in the particle-buffer roles and the grid and box-slot
  // indices (launch index mod 6), so one graph is kept per (nsteps, phase, buffer role).
  const bool sorting = b->sort_interval > 0;
  const int role = (b->sA < b->sB) ? 0 : 1;
  const int key_phase = (int)(b->launch_index % 6) * 2 + role;
  const std::pair<int, int> key(nsteps, key_phase);
  auto it = b->graphs.find(key);
  if (it == b->graphs.end()) {
    const int cur = b->cur;
    const int64_t li = b->launch_index, ss = b->since_sort, lc = b->launches;
    float* sA = b->sA;
    float* sB = b->sB;
    uint8_t* mA = b->matA;
    uint8_t* mB = b->matB;
    uint32_t* iA = b->idA;
    uint32_t* iB = b->idB;
    BCUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    mpm_status st = MPM_OK;
    int sorts = 0, since = 0;
    for (int32_t i = 0; i < nsteps && st == MPM_OK; ++i) {
      if (sorting && i % b->sort_interval == 0) {
        st = sort(b, true);  // a fused launch follows (the run's first P2G ran before the capture)
        ++sorts;
        since = 0;
      }
      if (st == MPM_OK) st = launch(b, kStepFused);
      ++since;
    }
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    const int64_t captured = b->launches - lc;
    // capturing recorded the work without running it: restore the host-side state
    b->cur = cur;
    b->launch_index = li;
    b->since_sort = ss;
    b->launches = lc;
    b->sA = sA;
    b->sB = sB;
    b->matA = mA;
    b->matB = mB;
    b->idA = iA;
    b->idB = iB;
    if (st != MPM_OK) {
      if (g) cudaGraphDestroy(g);
      return st;
    }
    if (e != cudaSuccess) return bfail(b, MPM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    cudaGraphExec_t ge = nullptr;
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bfail(b, MPM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    it = b->graphs.emplace(key, mpm_batch::Graph{ge, captured, sorts, since}).first;
  }
  BCUDA(b, cudaGraphLaunch(it->second.exec, b->stream));
  b->launches += it->second.launches;
  // advance the host-side state exactly as the recorded work does
  if (it->second.sorts % 2) {
    std::swap(b->sA, b->sB);
    std::swap(b->matA, b->matB);
    std::swap(b->idA, b->idB);
  }
  b->cur = (int)((b->cur + nsteps) % 3);
  b->launch_index += nsteps;
  b->since_sort = it->second.since_sort;
  return MPM_OK;
}

mpm_status mpm_batch_sync(mpm_batch* b) {
  if (!b) return MPM_ERR_INVALID;
  BCUDA(b, cudaStreamSynchronize(b->stream));
  int flag = 0;
  BCUDA(b, cudaMemcpy(&flag, b->status, sizeof(int), cudaMemcpyDeviceToHost));
  if (flag) {
    BCUDA(b, cudaMemset(b->status, 0, sizeof(int)));
    return bfail(b, MPM_ERR_STATE, "non-finite particle state");
  }
  return MPM_OK;
}

mpm_status mpm_batch_download_soa(mpm_batch* b, float* x, float* v, float* C, float* F, float* Jp) {
  if (!b) return MPM_ERR_INVALID;
  const int64_t n = b->n;
  if (n == 0) return MPM_OK;
  const unsigned fields = (x ? kFieldX : 0) | (v ? kFieldV : 0) | (C ? kFieldC : 0) | (F ? kFieldF : 0) |
                          (Jp ? kFieldJ : 0);
  uint32_t* inv = b->keys;  // free outside the sort
  BCUDA(b, launch_inverse(b->idA, n, inv, b->stream));
  BCUDA(b, launch_interleave(b->sA, b->stride, inv, n, b->stage, 0, fields, b->stream));
  b->launches += 2;
  float* xs = b->stage;
  float* vs = xs + 3 * n;
  float* Cs = vs + 3 * n;
  float* Fs = Cs + 9 * n;
  float* Js = Fs + 9 * n;
  if (x) BCUDA(b, cudaMemcpyAsync(x, xs, 12 * n, cudaMemcpyDeviceToHost, b->stream));
  if (v) BCUDA(b, cudaMemcpyAsync(v, vs, 12 * n, cudaMemcpyDeviceToHost, b->stream));
  if (C) BCUDA(b, cudaMemcpyAsync(C, Cs, 36 * n, cudaMemcpyDeviceToHost, b->stream));
  if (F) BCUDA(b, cudaMemcpyAsync(F, Fs, 36 * n, cudaMemcpyDeviceToHost, b->stream));
  if (Jp) BCUDA(b, cudaMemcpyAsync(Jp, Js, 4 * n, cudaMemcpyDeviceToHost, b->stream));
  BCUDA(b, cudaStreamSynchronize(b->stream));
  return MPM_OK;
}

int64_t mpm_batch_particle_count(const mpm_batch* b) { return b ? b->n : -1; }
int64_t mpm_batch_launch_count(const mpm_batch* b) { return b ? b->launches : -1; }

mpm_status mpm_batch_last_error(const mpm_batch* b, char* buf, size_t len) {
  if (!b || !buf || len == 0) return MPM_ERR_INVALID;
  std::snprintf(buf, len, "%s", b->last_error.c_str());
  return MPM_OK;
}

mpm_status mpm_batch_set_steps_per_warp(mpm_batch* b, int32_t steps_per_warp) {
  if (!b) return MPM_ERR_INVALID;
  if (steps_per_warp < 1 || steps_per_warp > 256) return bfail(b, MPM_ERR_INVALID, "steps_per_warp must be 1..256");
  if (steps_per_warp == b->steps_per_warp) return MPM_OK;
  BCUDA(b, cudaStreamSynchronize(b->stream));  // launches in flight read the old range table
  free_graphs(b);
  b->steps_per_warp = steps_per_warp;
  return build_ranges(b);
}

mpm_status mpm_batch_set_sort_interval(mpm_batch* b, int32_t sort_interval) {
  if (!b) return MPM_ERR_INVALID;
  if (sort_interval < 0) return bfail(b, MPM_ERR_INVALID, "sort_interval must be >= 0");
  if (sort_interval == b->sort_interval) return MPM_OK;
  BCUDA(b, cudaStreamSynchronize(b->stream));  // captured graphs bake the old schedule in
  free_graphs(b);
  b->sort_interval = sort_interval;
  b->since_sort = std::min<int64_t>(b->since_sort, sort_interval);
  return MPM_OK;
}

mpm_status mpm_batch_get_tuning(const mpm_batch* b, mpm_tuning* out) {
  if (!b || !out) return MPM_ERR_INVALID;
  *out = mpm_tuning{b->steps_per_warp, kStepWarps, 0, b->sort_interval, 0.0, 0, 0};
  return MPM_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Autotuner of a batch: the range size of the batched kernel (steps per warp), timed as
// replayed graphs on a copy of the batch, cached like the single-scene shapes.
// ---------------------------------------------------------------------------
namespace {

std::string batch_device_key(int dev) {
  cudaDeviceProp p{};
  if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) return "unknown device";
  char b[320];
  std::snprintf(b, sizeof(b), "%s (%d SMs, cc %d.%d)", p.name, p.multiProcessorCount, p.major, p.minor);
  return b;
}

// Changes with every build of this file, so a rebuilt library measures again.
const char* batch_build_key() { return "mpm_gb300 batch " __DATE__ " " __TIME__; }

// Workload class of a batch: scene count, particle count to the nearest power of two, the
// grid sides and the material kinds present.
std::string batch_class_key(const mpm_batch* b) {
  std::set<unsigned> sides;
  unsigned kinds = 0;
  for (const auto& sc : b->scenes) {
    sides.insert(sc.params.N);
    kinds |= 1u << sc.material.kind;
  }
  std::string ns;
  for (unsigned n : sides) ns += (ns.empty() ? "" : ",") + std::to_string(n);
  const int lg = b->n > 0 ? (int)std::lround(std::log2((double)b->n)) : 0;
  char buf[96];
  std::snprintf(buf, sizeof(buf), "batch scenes=%d n~2^%d kinds=0x%x N=", b->nscenes, lg, kinds);
  return buf + ns;
}

// The trial batch t gets b's particles (same scenes, so the same layout) and fresh grids.
mpm_status restore_from(mpm_batch* t, const mpm_batch* b) {
  BCUDA(t, cudaMemcpyAsync(t->sA, b->sA, sizeof(float) * (size_t)kNumComps * (size_t)b->stride,
                           cudaMemcpyDeviceToDevice, t->stream));
  BCUDA(t, cudaMemcpyAsync(t->idA, b->idA, sizeof(uint32_t) * (size_t)b->n, cudaMemcpyDeviceToDevice, t->stream));
  t->pending = false;
  t->launch_index = 0;
  t->since_sort = t->sort_interval;
  return fresh_grids(t);
}

}  // namespace

extern "C" {

mpm_status mpm_batch_autotune(mpm_batch* b, const char* cache_path, int32_t flags, int32_t budget_substeps,
                              mpm_tuning* out) {
  if (!b) return MPM_ERR_INVALID;
  if (b->n <= 0) return bfail(b, MPM_ERR_INVALID, "autotune needs uploaded particles");
  if (budget_substeps < 0 || budget_substeps > 4096) return bfail(b, MPM_ERR_INVALID, "budget_substeps out of range");
  if (flags & ~(MPM_TUNE_IGNORE_CACHE | MPM_TUNE_SORT_INTERVAL)) return bfail(b, MPM_ERR_INVALID, "unknown flags");
  const bool with_sort = (flags & MPM_TUNE_SORT_INTERVAL) != 0;
  const std::string dkey = batch_device_key(b->device), bkey = batch_build_key();
  const std::string ckey = batch_class_key(b) + (with_sort ? " +sort" : "");
  if (cache_path && !(flags & MPM_TUNE_IGNORE_CACHE)) {
    TuningEntry e;
    if (find_tuning(read_tuning_cache(cache_path), dkey, bkey, ckey, &e) && e.steps_per_warp >= 1 &&
        e.steps_per_warp <= 256 && e.sort_interval >= 0) {
      mpm_status st = mpm_batch_set_steps_per_warp(b, e.steps_per_warp);
      if (st == MPM_OK && with_sort) st = mpm_batch_set_sort_interval(b, e.sort_interval);
      if (st != MPM_OK) return st;
      if (out) *out = mpm_tuning{b->steps_per_warp, kStepWarps, 0, b->sort_interval, e.us_per_substep, 1, 0};
      return MPM_OK;
    }
  }
  BCUDA(b, cudaStreamSynchronize(b->stream));  // the trial batch copies the current particles
  mpm_batch* t = nullptr;
  mpm_status st = mpm_batch_create(b->scenes.data(), b->nscenes, b->sort_interval, &t);
  if (st != MPM_OK) return bfail(b, st, "tuning: cannot create the trial batch");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    if (e0) cudaEventDestroy(e0);
    mpm_batch_destroy(t);
    return bfail(b, MPM_ERR_CUDA, "tuning: cannot create events");
  }
  // replays of a multiple of 6 substeps keep the box-slot phase, so a graph is captured
  // once per buffer role: two replays capture both, the next two are timed
  const int steps = std::max(6, ((budget_substeps > 0 ? budget_substeps : 24) + 5) / 6 * 6);
  int timed = 0;
  auto time_spw = [&](int spw, double* us, int sort_interval = -1, int n_steps = 0) -> mpm_status {
    ++timed;
    const int len = n_steps > 0 ? n_steps : steps;
    mpm_status s2 = mpm_batch_set_steps_per_warp(t, spw);
    if (s2 == MPM_OK && sort_interval >= 0) s2 = mpm_batch_set_sort_interval(t, sort_interval);
    if (s2 == MPM_OK) s2 = restore_from(t, b);
    for (int r = 0; r < 2 && s2 == MPM_OK; ++r) s2 = mpm_batch_substep_graph(t, len);
    if (s2 != MPM_OK) return s2;
    if (cudaEventRecord(e0, t->stream) != cudaSuccess) return MPM_ERR_CUDA;
    for (int r = 0; r < 2 && s2 == MPM_OK; ++r) s2 = mpm_batch_substep_graph(t, len);
    if (s2 != MPM_OK) return s2;
    if (cudaEventRecord(e1, t->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) return MPM_ERR_CUDA;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) return MPM_ERR_CUDA;
    *us = 1e3 * (double)ms / (2.0 * len);
    return mpm_batch_sync(t);
  };
  int best = b->steps_per_warp;
  double best_us = 0.0;
  st = time_spw(best, &best_us);
  const double base_us = best_us;
  for (int spw : {1, 2, 4, 8, 16}) {
    if (st != MPM_OK) break;
    if (spw == b->steps_per_warp) continue;
    double us = 0.0;
    st = time_spw(spw, &us);
    // a knob moves only for a gain above 1 %, so timing noise does not flip it
    if (st == MPM_OK && us < 0.99 * best_us && us < 0.99 * base_us) {
      best = spw;
      best_us = us;
    }
  }
  int best_sort = b->sort_interval;
  if (with_sort && st == MPM_OK) {
    // sort intervals over replays of 48 substeps (a multiple of each), against the current
    // interval re-timed over the same length
    double base = 0.0;
    st = time_spw(best, &base, b->sort_interval, 48);
    double cur = base;
    for (int si : {8, 12, 16, 24}) {
      if (st != MPM_OK) break;
      if (si == b->sort_interval) continue;
      double us = 0.0;
      st = time_spw(best, &us, si, 48);
      if (st == MPM_OK && us < 0.99 * cur && us < 0.99 * base) {
        best_sort = si;
        cur = us;
      }
    }
    if (st == MPM_OK && best_sort != b->sort_interval) best_us = cur;
  }
  std::string why = st != MPM_OK ? t->last_error : std::string();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  mpm_batch_destroy(t);
  if (st != MPM_OK) return bfail(b, st, "tuning: " + why);
  st = mpm_batch_set_steps_per_warp(b, best);
  if (st == MPM_OK) st = mpm_batch_set_sort_interval(b, best_sort);
  if (st != MPM_OK) return st;
  const mpm_tuning res{best, kStepWarps, 0, b->sort_interval, best_us, 0, timed};
  if (out) *out = res;
  if (cache_path) {
    TuningEntry e;
    e.device = dkey;
    e.build = bkey;
    e.klass = ckey;
    e.steps_per_warp = best;
    e.warps_per_cta = kStepWarps;
    e.tile_box = MPM_TILE_4x4x6;  // unused by a batch (no G2P tile); a valid value for the file
    e.sort_interval = b->sort_interval;
    e.us_per_substep = best_us;
    if (!store_tuning(cache_path, e))
      return bfail(b, MPM_ERR_IO, std::string("tuning: cannot write the cache file ") + cache_path);
  }
  return MPM_OK;
}

}  // extern "C"
