// Internal host/device interface between the C ABI (capi.cu) and the kernels.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "mpm_device.cuh"

namespace mpm {

// One scene of a batch: its grid constants and where its grid starts in the pooled
// grid buffers.
struct SceneDev {
  GridConsts g;
  DevMaterial m;  // every particle of a scene has the scene's material
  int64_t grid_offset;   // of the scene's grid in the pooled P2G grids
  int64_t vgrid_offset;  // of the scene's padded velocity grid ((N + 5)^3 nodes) in the pool
};

constexpr int kBoxSlots = 6;  // per-scene P2G box slots (record / clear / reset rotate)

// Arguments of the fused substep kernel.  One launch = G2P of substep n (from
// grid_in, the P2G grid of substep n) + P2G of substep n+1 (into grid_out) +
// clearing grid_zero (the grid substep n-1 read), so the three grid buffers rotate.
struct StepArgs {
  float* s;               // component-major particle state
  float* s_out;           // G2P-only launches: where the updated state goes (null: in place)
  float* rot;             // null, or where P2G writes each particle's polar rotation R of F
                          // (9 components at the state's stride; particles inside the domain)
  int64_t stride;         // component stride (elements)
  const uint8_t* mat;     // material index per particle (general layout), may be null
  const uint32_t* id;     // original particle index (for the G2P guard)
  int64_t n;
  const float4* grid_in;  // P2G grid to apply (m v, m); null for a P2G-only launch
  float4* grid_out;       // P2G accumulation target (already zero)
  float4* grid_zero;      // buffer to clear for the launch after next
  int64_t grid_cells;
  int chunk;              // particles per range (multiple of 32); ranges go to warps dynamically
  int64_t guard_limit;    // G2P only for id <= guard_limit when the guard is on
  int check_finite;
  int* status;
  // batch mode (nscenes > 0): ranges never straddle scenes; grids are cleared sparsely
  int nscenes;
  const int4* ranges;     // (scene, begin, end, 0)
  int nranges;
  const SceneDev* scenes;
  int* boxes;             // [scene][kBoxSlots][6]: lo xyz, hi xyz of P2G base cells
  int box_record, box_clear, box_reset;
  // single-scene G2P: the padded velocity grid the launch's first kernel writes from
  // grid_in, and its TMA tensor map
  float4* vgrid;
  CUtensorMap vmap;
  SimConsts K;
};

// Velocity grid of a single-scene substep: the grid operation applied to a P2G grid,
// padded by 3 nodes below and 2 above in each dimension ((N + 5)^3 float4 nodes, zero
// in the padding), so the G2P stencil of every particle that is not completely
// outside the domain reads inside it; plus the TMA tensor maps of its tiles, one per
// tile box.
constexpr int kTileShapes = 3;
struct VelocityGrid {
  CUtensorMap map[kTileShapes];
  float4* ptr = nullptr;
  int N = 0;
};
int64_t vgrid_nodes(int N);
// Describes caller-owned memory of vgrid_nodes(N) float4 (16-byte aligned) as a velocity grid.
cudaError_t vgrid_bind(VelocityGrid& v, float4* ptr, int N);
// Points a launch's arguments at a velocity grid and the tensor map of tile box `tile`.
void set_vgrid(StepArgs& a, const VelocityGrid& v, int tile = 0);

// Launch shape knobs of the fused single-scene substep: warps per CTA (4, 6 or 12) and
// the G2P tile box (0: 4x4x6, 1: 4x4x4, 2: 4x6x6; boxes 1 and 2 with 12 warps).
struct StepTuning {
  int warps;
  int tile;
};
// One warp waiting `polls` times on an mbarrier nothing arrives on; sets kStatusTimeout.
cudaError_t launch_wait_timeout_probe(int* status, int polls, cudaStream_t st);
// Velocity pass of a batch: for every scene, the grid op over the nodes of the P2G box
// recorded in box slot `slot` (plus the stencil's 2 nodes), into the padded velocity grids.
cudaError_t launch_batch_velocity(const float4* grid, float4* vgrid, const SceneDev* scenes, int nscenes,
                                  const int* boxes, int slot, cudaStream_t st);

enum StepKind { kStepP2GOnly = 0, kStepFused = 1, kStepG2POnly = 2 };

// Material kinds of policies compiled in through include/mpm_gb300_policies.cuh
// (MPM_MAT_USER_BASE ... in the C ABI) and their kernels: the fused substep, the
// P2G-only launch that starts a run and the G2P-only launch that may end one.
constexpr int kUserKindBase = 16, kUserKindEnd = 64;
struct MaterialKernels {
  void* fused;
  void* p2g_only;
  void* g2p_only;
};
// Registers the kernels of material kind `kind` (once per kind; false if the kind is out
// of range or taken).
bool register_material_kernels(int kind, const MaterialKernels& k);
// The kernels of a registered kind.
bool find_material_kernels(int kind, MaterialKernels* out);

// Launches one substep (a.nscenes > 0: a batch). liquid = liquid-only layout.  A
// single-scene launch with G2P is two kernels: the velocity pass (grid_in -> a.vgrid)
// and the substep kernel.  *launches (may be null) counts the kernels.
// want: launch shape asked for (StepTuning; launches other than the single-scene fused
// substep use 12 warps and box 0).  vel: the velocity grid, required by single-scene
// launches with G2P (the launch reads it through the tensor map of its box).
cudaError_t launch_step(const StepArgs& a, StepKind kind, bool liquid, bool guard, int grid_blocks,
                        cudaStream_t st, int64_t* launches = nullptr, StepTuning want = StepTuning{kStepWarps, 0},
                        const VelocityGrid* vel = nullptr);
// The launch shape a launch of this kind uses when `want` is asked for.
StepTuning step_tuning(StepKind kind, bool guard, bool batch, StepTuning want);
// Dynamic shared memory of a variant: G2P tiles + per-warp P2G reduction buffers.
size_t step_smem_bytes(StepKind kind, bool batch, StepTuning want = StepTuning{kStepWarps, 0});
// Max resident CTAs per SM for the variant at the given dynamic shared memory.
int step_blocks_per_sm(StepKind kind, bool liquid, bool guard, size_t smem, bool batch = false,
                       StepTuning want = StepTuning{kStepWarps, 0});

}  // namespace mpm

#include "mpm_gb300.h"

namespace mpm {

// Device constants from the C ABI parameters and material table.
void make_grid_consts(const mpm_params& p, GridConsts& K);
void make_dev_material(const mpm_material& m, DevMaterial& d);
void make_sim_consts(const mpm_params& p, const mpm_material* mats, int n_materials, SimConsts& K);
// Range size (chunk, particles) and grid size of a substep launch.
void step_launch_shape(int num_sms, int64_t n, bool liquid, bool guard, StepKind kind, int steps_per_warp,
                       int& chunk, int& blocks, StepTuning want = StepTuning{kStepWarps, 0});

// Cell sort (counting sort by the linear index of the base cell).
struct SortArgs {
  const float* sA;
  float* sB;
  int64_t stride;
  int64_t n;
  const uint8_t* matA;
  uint8_t* matB;
  const uint32_t* idA;
  uint32_t* idB;
  uint32_t* keys;
  uint32_t* perm;  // n words, or null: with it the sort ranks, then gathers (for unsorted input)
  uint32_t* inv;   // with perm, optional: the inverse permutation (particle p -> its slot)
  int* counts;   // one per sort key
  int* block_sums;
  int64_t cells;  // sort key space (bricked cell index range)
  int N;
  float dx_inv;
  int ncomp;            // kLiquidComps (x, v, C, J) or kNumComps (all)
  // nonzero: the next launch runs G2P on the sorted particles (its P2G grid is already
  // built), so particles inside the domain move only x, J (and F); a scatter sort only,
  // key space at most kKeyOutside
  int partial;
  // batch mode (nscenes > 0): keys are scene_key_base[scene] + the bricked key in the scene's grid
  int nscenes;
  const int64_t* scene_start;      // nscenes + 1 particle offsets
  const uint32_t* scene_key_base;  // nscenes
  const SceneDev* scenes;
};
// Bit of a stored sort key that flags a particle completely outside the domain (partial sorts).
constexpr uint32_t kKeyOutside = 0x80000000u;
cudaError_t launch_sort(const SortArgs& a, int num_sms, cudaStream_t st, int64_t* launches);

// Host-interleaved <-> component-major conversion.
cudaError_t launch_deinterleave(const float* stage, float* s, int64_t stride, int64_t n, int has_v,
                                int has_C, int has_F, int has_Jp, cudaStream_t st);
// Per-particle host-layout arrays (x, v: 3 floats; C, F: 9 row-major; J: 1), any of them
// null, in memory the device can read (device memory or mapped pinned host memory).
struct HostArrays {
  const float *x, *v, *C, *F, *J;
};
struct OutArrays {
  float *x, *v, *C, *F, *J;
};
// Arrays -> component-major particle arrays in one pass (missing fields take their rest
// values); *bad = 1 when a position is not finite (*bad is zeroed first on the stream
// unless bad_zeroed: a flag the caller cleared, e.g. in mapped host memory).
cudaError_t launch_deinterleave_arrays(HostArrays a, float* s, int64_t stride, int64_t n, int* bad, cudaStream_t st,
                                       const uint32_t* dest = nullptr, bool bad_zeroed = false);
// Cell order of positions before they are uploaded (x: x, y, z per particle, host-visible
// or device memory): keys and counts of a (keys, counts, block_sums, cells, N, dx_inv, n),
// the permutation into a.perm (slot q holds particle perm[q]) and its inverse into dest
// (particle p goes to slot dest[p]); a copy of the positions into xcopy when not null;
// *bad = 1 when a position is not finite (zeroed first unless bad_zeroed, as above).
cudaError_t launch_presort(const float* x, float* xcopy, const SortArgs& a, uint32_t* dest, int* bad, int num_sms,
                           cudaStream_t st, int64_t* launches, bool bad_zeroed = false);
// Number of slots q of the component-major arrays whose cell key (the sort's bricked key)
// is below slot q - 1's, written to *out (host-visible) by the kernel; counters: two ints
// of device memory, zero between calls.
cudaError_t launch_order_check(const float* s, int64_t stride, int64_t n, float dx_inv, int N, int* counters, int* out,
                               cudaStream_t st);
// Component-major particle arrays -> the non-null arrays in upload order (inv as from
// launch_inverse, null for the identity).
cudaError_t launch_interleave_arrays(const float* s, int64_t stride, const uint32_t* inv, int64_t n, OutArrays o,
                                     int liquid_layout, cudaStream_t st);
// Fields of launch_interleave.
constexpr unsigned kFieldX = 1, kFieldV = 2, kFieldC = 4, kFieldF = 8, kFieldJ = 16, kFieldAll = 31;
// inv[id[p]] = p: the device slot of each particle in upload order.
cudaError_t launch_inverse(const uint32_t* id, int64_t n, uint32_t* inv, cudaStream_t st);
// Staging arrays (x, v, C, F, Jp blocks) in upload order from the particle arrays, inv as
// from launch_inverse (null: device order is upload order), only the requested fields.
cudaError_t launch_interleave(const float* s, int64_t stride, const uint32_t* inv, int64_t n, float* stage,
                              int liquid_layout, unsigned fields, cudaStream_t st);
cudaError_t launch_iota(uint32_t* id, int64_t n, cudaStream_t st);
// *flag = 1 when any of the m floats is not finite (0 otherwise).
cudaError_t launch_check_finite(const float* x, int64_t m, int* flag, cudaStream_t st);
cudaError_t launch_scatter_u8(const uint8_t* src, const uint32_t* id, int64_t n, uint8_t* dst, cudaStream_t st);
// Scene objects: append k seeded particles (positions xs, 3 floats each) at index n0 with
// velocity v, C = 0, F = I, Jp = 1, material mat_index and ids id0.., and remove the
// particles with ids in [lo, hi) into the other SoA copy (ids above hi shift down;
// flags holds n + 1 ints, scratch scan_scratch_ints(n + 1)).
cudaError_t launch_append_object(float* s, int64_t st, int64_t n0, int64_t k, const float* xs, const float v[3],
                                 bool liquid, uint8_t* mat, uint8_t mat_index, uint32_t* id, uint32_t id0,
                                 cudaStream_t stream);
cudaError_t launch_remove_ids(const float* sA, float* sB, int64_t st, int64_t n, const uint32_t* idA, uint32_t* idB,
                              const uint8_t* matA, uint8_t* matB, uint32_t lo, uint32_t hi, bool liquid, int* flags,
                              int* scratch, cudaStream_t stream, int64_t* launches);
// In-place exclusive scan of m ints (three kernels); scratch holds scan_scratch_ints(m) ints.
int64_t scan_scratch_ints(int64_t m);
cudaError_t launch_exclusive_scan(int* data, int64_t m, int* scratch, cudaStream_t st, int64_t* launches);
// Post-op grid with the reference's mass slot (src/mpm.cu:86-88).
cudaError_t launch_grid_op(const float4* in, float4* out, GridConsts K, cudaStream_t st);

}  // namespace mpm
