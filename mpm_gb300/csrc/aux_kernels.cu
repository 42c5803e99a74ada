// Auxiliary kernels: periodic cell sort, host-layout conversion, grid-op readback.
#include "mpm_internal.h"

namespace mpm {

// ---------------------------------------------------------------------------
// Cell sort: counting sort of particles by a bricked key of their base cell:
// bricks of 4x4x4 cells in row-major order, cells row-major inside a brick.  Any
// run of consecutive sorted particles then covers a compact box of cells in all
// three dimensions, which keeps the substep kernel's per-chunk grid tile small.
// histogram (warp-aggregated atomics) -> exclusive scan -> scatter.  Order inside
// a cell is not stable; the substep does not depend on it.
// ---------------------------------------------------------------------------
// *outside (when given): the particle lies completely outside the domain, by the test
// and the base cells the substep uses (so the two always agree).
__device__ __forceinline__ uint32_t cell_key_of(const float x[3], float dx_inv, int N, bool* outside = nullptr) {
  int b[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) b[d] = QuadraticInterpolationKernel::base_cell(x[d], dx_inv);
  if (outside) *outside = outside_domain(b[0], b[1], b[2], N);
#pragma unroll
  for (int d = 0; d < 3; ++d) b[d] = min(max(b[d], 0), N - 1);
  const uint32_t nb = (uint32_t)(N + 3) >> 2;
  const uint32_t brick = ((uint32_t)(b[0] >> 2) * nb + (uint32_t)(b[1] >> 2)) * nb + (uint32_t)(b[2] >> 2);
  return brick * 64u + (uint32_t)(((b[0] & 3) << 4) | ((b[1] & 3) << 2) | (b[2] & 3));
}

__device__ __forceinline__ uint32_t cell_key(const float* s, int64_t st, int64_t p, float dx_inv, int N,
                                             bool* outside = nullptr) {
  const float x[3] = {s[(kX + 0) * st + p], s[(kX + 1) * st + p], s[(kX + 2) * st + p]};
  return cell_key_of(x, dx_inv, N, outside);
}

// Scene of particle p in a batch (binary search over the scene offsets).
__device__ __forceinline__ int scene_of(const int64_t* start, int nscenes, int64_t p) {
  int lo = 0, hi = nscenes - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= p) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// The counter of a stored key: partial sorts (key spaces of at most 2^31) flag keys in bit
// 31; other sorts use every bit (batches may have key spaces up to 2^32).
__device__ __forceinline__ uint32_t key_slot(const SortArgs& a, uint32_t key) {
  return a.partial ? (key & ~kKeyOutside) : key;
}

// The stored sort key of particle p: its bricked cell key, with kKeyOutside set in a
// partial sort when the particle lies completely outside the domain.
__device__ __forceinline__ uint32_t sort_key(const SortArgs& a, int64_t p) {
  bool outside = false;
  uint32_t key;
  if (a.nscenes > 0) {
    const int sc = scene_of(a.scene_start, a.nscenes, p);
    const GridConsts& g = a.scenes[sc].g;
    key = a.scene_key_base[sc] + cell_key(a.sA, a.stride, p, g.dx_inv, g.N, &outside);
  } else {
    key = cell_key(a.sA, a.stride, p, a.dx_inv, a.N, &outside);
  }
  return (a.partial && outside) ? (key | kKeyOutside) : key;
}

__global__ void sort_histogram(SortArgs a) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < a.n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = base + threadIdx.x;
    const bool valid = p < a.n;
    uint32_t key = valid ? sort_key(a, p) : 0xffffffffu;
    if (valid) a.keys[p] = key;
    const unsigned same = __match_any_sync(kFull, key);
    if (valid && lane == __ffs(same) - 1) atomicAdd(a.counts + key_slot(a, key), __popc(same));
  }
}

constexpr int kScanItems = 8;  // per thread; a block scans kThreads * kScanItems counts

// In-place exclusive scan of counts[] in blocks; block totals to block_sums[].
__global__ void scan_blocks(int* counts, int64_t m, int* block_sums) {
  __shared__ int warp_tot[kWarps];
  const int64_t off = (int64_t)blockIdx.x * kThreads * kScanItems + (int64_t)threadIdx.x * kScanItems;
  int v[kScanItems];
  int sum = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = (off + i < m) ? counts[off + i] : 0;
    sum += v[i];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int inc = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_tot[warp] = inc;
  __syncthreads();
  int wpre = 0, tot = 0;
  for (int w = 0; w < kWarps; ++w) {
    if (w < warp) wpre += warp_tot[w];
    tot += warp_tot[w];
  }
  int run = wpre + inc - sum;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (off + i < m) counts[off + i] = run;
    run += v[i];
  }
  if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

// Exclusive scan of the block totals by one CTA (loops over tiles of 256).
__global__ void scan_block_sums(int* block_sums, int nb) {
  __shared__ int warp_tot[kWarps];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int base = 0; base < nb; base += kThreads) {
    const int i = base + threadIdx.x;
    const int v = i < nb ? block_sums[i] : 0;
    int inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(kFull, inc, o);
      if (lane >= o) inc += t;
    }
    if (lane == 31) warp_tot[warp] = inc;
    __syncthreads();
    int wpre = 0, tot = 0;
    for (int w = 0; w < kWarps; ++w) {
      if (w < warp) wpre += warp_tot[w];
      tot += warp_tot[w];
    }
    if (i < nb) block_sums[i] = carry + wpre + inc - v;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
}

__global__ void scan_add(int* counts, int64_t m, const int* block_sums) {
  const int64_t off = (int64_t)blockIdx.x * kThreads * kScanItems;
  const int add = block_sums[blockIdx.x];
  for (int i = threadIdx.x; i < kThreads * kScanItems; i += kThreads)
    if (off + i < m) counts[off + i] += add;
}

// Component k of the layout's c-th moved component: the liquid layout moves x, v, C
// (components 0-14) and J (component 24); the general layout moves all 25.
template <bool LIQ>
__device__ __forceinline__ int moved_comp(int c) {
  return LIQ ? (c < kLiquidComps - 1 ? c : kJp) : c;
}

// Component k of the c-th component the substep reads back from memory when the
// particle's G2P runs: x and J (liquid layout); x, F and Jp (general layout).  v and C
// are G2P outputs, rewritten before they are read again.
template <bool LIQ>
__device__ __forceinline__ int carried_comp(int c) {
  return c < 3 ? kX + c : ((LIQ || c == 12) ? kJp : kF + (c - 3));
}

template <bool LIQ, bool PARTIAL>
__device__ __forceinline__ void move_particle(const float* __restrict__ sA, float* __restrict__ sB, int64_t st,
                                              int64_t p, int64_t q) {
  constexpr int NC = PARTIAL ? (LIQ ? 4 : 13) : (LIQ ? kLiquidComps : kNumComps);
  float vals[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) vals[c] = __ldg(sA + (PARTIAL ? carried_comp<LIQ>(c) : moved_comp<LIQ>(c)) * st + p);
#pragma unroll
  for (int c = 0; c < NC; ++c) sB[(PARTIAL ? carried_comp<LIQ>(c) : moved_comp<LIQ>(c)) * st + q] = vals[c];
}

// Scatter every particle to its sorted slot.  All components of a particle are
// loaded before any is stored, so a thread keeps 16 or 25 loads in flight.
// PARTIAL: the launch after the sort runs G2P on every particle inside the domain
// (the P2G of the next substep is already on the grid), which rewrites v and C
// without reading them, so those particles move only their carried components; a
// particle flagged outside the domain keeps its whole state through the substep and
// moves all of it.
template <bool LIQ, bool PARTIAL>
__global__ void sort_scatter(SortArgs a) {
  const int lane = threadIdx.x & 31;
  const float* __restrict__ sA = a.sA;
  float* __restrict__ sB = a.sB;
  const int64_t st = a.stride;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < a.n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = base + threadIdx.x;
    const bool valid = p < a.n;
    const uint32_t key = valid ? a.keys[p] : 0xffffffffu;
    const unsigned same = __match_any_sync(kFull, key);
    const int leader = __ffs(same) - 1;
    int start = 0;
    if (valid && lane == leader) start = atomicAdd(a.counts + key_slot(a, key), __popc(same));
    start = __shfl_sync(kFull, start, leader);
    if (!valid) continue;
    const int64_t q = (int64_t)start + __popc(same & ((1u << lane) - 1u));
    if (PARTIAL && !(key & kKeyOutside))
      move_particle<LIQ, true>(sA, sB, st, p, q);
    else
      move_particle<LIQ, false>(sA, sB, st, p, q);
    if (a.matA) a.matB[q] = a.matA[p];
    a.idB[q] = a.idA[p];
  }
}

// The sort for particles in arbitrary order (after an upload): scattering them would write
// every component to a random slot, so sort_rank only writes the permutation (slot q holds
// particle perm[q]) and sort_gather fills each slot with coalesced writes.
__global__ void sort_rank(SortArgs a) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < a.n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = base + threadIdx.x;
    const bool valid = p < a.n;
    const uint32_t key = valid ? a.keys[p] : 0xffffffffu;
    const unsigned same = __match_any_sync(kFull, key);
    const int leader = __ffs(same) - 1;
    int start = 0;
    if (valid && lane == leader) start = atomicAdd(a.counts + key_slot(a, key), __popc(same));
    start = __shfl_sync(kFull, start, leader);
    if (valid) {
      const int64_t q = (int64_t)start + __popc(same & ((1u << lane) - 1u));
      a.perm[q] = (uint32_t)p;
      if (a.inv) a.inv[p] = (uint32_t)q;  // coalesced: p is this thread's particle
    }
  }
}

template <bool LIQ>
__global__ void sort_gather(SortArgs a) {
  constexpr int NC = LIQ ? kLiquidComps : kNumComps;
  const float* __restrict__ sA = a.sA;
  float* __restrict__ sB = a.sB;
  const int64_t st = a.stride;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < a.n; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = a.perm[q];
    float vals[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) vals[c] = __ldg(sA + moved_comp<LIQ>(c) * st + p);
#pragma unroll
    for (int c = 0; c < NC; ++c) sB[moved_comp<LIQ>(c) * st + q] = vals[c];
    if (a.matA) a.matB[q] = a.matA[p];
    a.idB[q] = a.idA[p];
  }
}

// Exclusive scan of a small key space (a multiple of 4 counts) by one CTA: each of
// kScanThreads threads scans kScanRun consecutive counts in registers (int4 loads),
// then the CTA scans the threads' totals; tiles of kScanThreads x kScanRun counts
// carry their total into the next.  One launch instead of the three of the blocked
// scan, used up to one tile (kSmallScan keys, N <= 32): beyond that the single SM's
// bandwidth makes it slower than the blocked scan.
constexpr int kScanThreads = 1024;
constexpr int kScanRun = 32;
constexpr int64_t kSmallScan = (int64_t)kScanThreads * kScanRun;  // one tile: one SM's bandwidth suffices

__global__ void __launch_bounds__(kScanThreads) scan_small(int* counts, int64_t m) {
  __shared__ int warp_tot[kScanThreads / 32];
  __shared__ int carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  for (int64_t tile = 0; tile < m; tile += (int64_t)kScanThreads * kScanRun) {
    const int64_t off = tile + (int64_t)threadIdx.x * kScanRun;
    int4 v[kScanRun / 4];
    int sum = 0;
#pragma unroll
    for (int i = 0; i < kScanRun / 4; ++i) {
      v[i] = (off + 4 * i < m) ? reinterpret_cast<const int4*>(counts + off)[i] : make_int4(0, 0, 0, 0);
      sum += v[i].x + v[i].y + v[i].z + v[i].w;
    }
    int inc = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(kFull, inc, o);
      if (lane >= o) inc += t;
    }
    __syncthreads();  // warp_tot and carry of the previous tile are consumed
    if (lane == 31) warp_tot[warp] = inc;
    __syncthreads();
    int wpre = 0;
    if (lane < kScanThreads / 32) wpre = warp_tot[lane];
    int wscan = wpre;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(kFull, wscan, o);
      if (lane >= o) wscan += t;
    }
    const int before_warp = __shfl_sync(kFull, wscan - wpre, warp);  // exclusive prefix of this warp
    const int tile_total = __shfl_sync(kFull, wscan, kScanThreads / 32 - 1);
    int run = carry + before_warp + inc - sum;
#pragma unroll
    for (int i = 0; i < kScanRun / 4; ++i) {
      int4 o;
      o.x = run;
      run += v[i].x;
      o.y = run;
      run += v[i].y;
      o.z = run;
      run += v[i].z;
      o.w = run;
      run += v[i].w;
      if (off + 4 * i < m) reinterpret_cast<int4*>(counts + off)[i] = o;
    }
    __syncthreads();
    if (threadIdx.x == 0) carry += tile_total;
  }
}

// Exclusive scan of the cell counts; returns the number of launches.
int scan_cell_counts(const SortArgs& a, cudaStream_t st) {
  if (a.cells <= kSmallScan && a.cells % 4 == 0) {
    scan_small<<<1, kScanThreads, 0, st>>>(a.counts, a.cells);
    return 1;
  }
  const int per = kThreads * kScanItems;
  const int nb = (int)((a.cells + per - 1) / per);
  scan_blocks<<<nb, kThreads, 0, st>>>(a.counts, a.cells, a.block_sums);
  scan_block_sums<<<1, kThreads, 0, st>>>(a.block_sums, nb);
  scan_add<<<nb, kThreads, 0, st>>>(a.counts, a.cells, a.block_sums);
  return 3;
}

// Cell keys and their histogram of positions given as x, y, z per particle (host-visible
// or device memory), with a copy of the positions to xcopy (when not null) and *bad = 1
// for a position that is not finite.
__global__ void presort_keys_kernel(const float* __restrict__ x, float* __restrict__ xcopy, SortArgs a, int* bad) {
  const int lane = threadIdx.x & 31;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < a.n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = base + threadIdx.x;
    const bool valid = p < a.n;
    uint32_t key = 0xffffffffu;
    if (valid) {
      const float xp[3] = {x[3 * p], x[3 * p + 1], x[3 * p + 2]};
      if (!isfinite(xp[0]) || !isfinite(xp[1]) || !isfinite(xp[2])) *bad = 1;
      if (xcopy) {
        xcopy[3 * p] = xp[0];
        xcopy[3 * p + 1] = xp[1];
        xcopy[3 * p + 2] = xp[2];
      }
      key = cell_key_of(xp, a.dx_inv, a.N);
      a.keys[p] = key;
    }
    const unsigned same = __match_any_sync(kFull, key);
    if (valid && lane == __ffs(same) - 1) atomicAdd(a.counts + key, __popc(same));
  }
}

cudaError_t launch_sort(const SortArgs& a, int num_sms, cudaStream_t st, int64_t* launches) {
  if (a.n == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(a.counts, 0, sizeof(int) * a.cells, st);
  if (e != cudaSuccess) return e;
  int blocks = (int)std::min<int64_t>((a.n + kThreads - 1) / kThreads, (int64_t)num_sms * 8);
  sort_histogram<<<blocks, kThreads, 0, st>>>(a);
  int n_launch = 2 + scan_cell_counts(a, st);
  if (a.perm) {
    sort_rank<<<blocks, kThreads, 0, st>>>(a);
    if (a.ncomp == kLiquidComps)
      sort_gather<true><<<blocks, kThreads, 0, st>>>(a);
    else
      sort_gather<false><<<blocks, kThreads, 0, st>>>(a);
    n_launch += 1;
  } else if (a.ncomp == kLiquidComps) {
    if (a.partial)
      sort_scatter<true, true><<<blocks, kThreads, 0, st>>>(a);
    else
      sort_scatter<true, false><<<blocks, kThreads, 0, st>>>(a);
  } else if (a.partial) {
    sort_scatter<false, true><<<blocks, kThreads, 0, st>>>(a);
  } else {
    sort_scatter<false, false><<<blocks, kThreads, 0, st>>>(a);
  }
  if (launches) *launches += n_launch;
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Host layout (per-particle interleaved x[3n] v[3n] C[9n] F[9n] Jp[n], staged
// contiguously in that order) <-> component-major device layout.
// ---------------------------------------------------------------------------
__global__ void deinterleave_kernel(const float* stage, float* s, int64_t st, int64_t n, int has_v, int has_C,
                                    int has_F, int has_Jp) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const float* xs = stage;
    const float* vs = xs + 3 * n;
    const float* Cs = vs + 3 * n;
    const float* Fs = Cs + 9 * n;
    const float* Js = Fs + 9 * n;
    for (int d = 0; d < 3; ++d) {
      s[(kX + d) * st + p] = xs[3 * p + d];
      s[(kV + d) * st + p] = has_v ? vs[3 * p + d] : 0.f;
    }
    for (int i = 0; i < 9; ++i) {
      s[(kC + i) * st + p] = has_C ? Cs[9 * p + i] : 0.f;
      s[(kF + i) * st + p] = has_F ? Fs[9 * p + i] : ((i % 4 == 0) ? 1.f : 0.f);
    }
    s[kJp * st + p] = has_Jp ? Js[p] : 1.f;
  }
}

__global__ void inverse_kernel(const uint32_t* __restrict__ id, int64_t n, uint32_t* __restrict__ inv) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
    inv[id[p]] = (uint32_t)p;
}

// Staging arrays in upload order: thread r gathers particle inv[r] (scattered reads) and
// writes its own entries of the requested fields (coalesced writes).
__global__ void interleave_kernel(const float* __restrict__ s, int64_t st, const uint32_t* __restrict__ inv, int64_t n,
                                  float* __restrict__ stage, int liquid_layout, unsigned fields) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = inv ? inv[r] : r;
    float* xs = stage;
    float* vs = xs + 3 * n;
    float* Cs = vs + 3 * n;
    float* Fs = Cs + 9 * n;
    float* Js = Fs + 9 * n;
    if (fields & kFieldX)
      for (int d = 0; d < 3; ++d) xs[3 * r + d] = s[(kX + d) * st + p];
    if (fields & kFieldV)
      for (int d = 0; d < 3; ++d) vs[3 * r + d] = s[(kV + d) * st + p];
    if (fields & kFieldC)
      for (int i = 0; i < 9; ++i) Cs[9 * r + i] = s[(kC + i) * st + p];
    if (fields & (kFieldF | kFieldJ)) {
      const float J = s[kJp * st + p];
      if (fields & kFieldJ) Js[r] = J;
      if (fields & kFieldF) {
        const float cr = liquid_layout ? cbrtf(J) : 0.f;
        for (int i = 0; i < 9; ++i)
          Fs[9 * r + i] = liquid_layout ? ((i % 4 == 0) ? cr : 0.f) : s[(kF + i) * st + p];
      }
    }
  }
}

__global__ void iota_kernel(uint32_t* id, int64_t n) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
    id[p] = (uint32_t)p;
}

__global__ void scatter_u8_kernel(const uint8_t* src, const uint32_t* id, int64_t n, uint8_t* dst) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x)
    dst[id[p]] = src[p];
}

static int grid_for(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 4096)); }

cudaError_t launch_deinterleave(const float* stage, float* s, int64_t stride, int64_t n, int has_v, int has_C,
                                int has_F, int has_Jp, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  deinterleave_kernel<<<grid_for(n), 256, 0, st>>>(stage, s, stride, n, has_v, has_C, has_F, has_Jp);
  return cudaGetLastError();
}

namespace {

// The block's part of a host array (w floats per particle) through shared memory: 16-byte
// loads or stores of the contiguous range when it is 16-byte aligned, plain ones otherwise.
template <int W>
__device__ __forceinline__ void load_rows(const float* __restrict__ src, int64_t r0, int cnt, float* tile) {
  const float* base = src + W * r0;
  const int words = W * cnt;
  if ((reinterpret_cast<uintptr_t>(base) & 15) == 0) {
    const float4* b4 = reinterpret_cast<const float4*>(base);
    for (int q = threadIdx.x; q < words / 4; q += blockDim.x) reinterpret_cast<float4*>(tile)[q] = b4[q];
    for (int q = (words / 4) * 4 + threadIdx.x; q < words; q += blockDim.x) tile[q] = base[q];
  } else {
    for (int q = threadIdx.x; q < words; q += blockDim.x) tile[q] = base[q];
  }
}

template <int W>
__device__ __forceinline__ void store_rows(float* __restrict__ dst, int64_t r0, int cnt, const float* tile) {
  float* base = dst + W * r0;
  const int words = W * cnt;
  if ((reinterpret_cast<uintptr_t>(base) & 15) == 0) {
    float4* b4 = reinterpret_cast<float4*>(base);
    for (int q = threadIdx.x; q < words / 4; q += blockDim.x) b4[q] = reinterpret_cast<const float4*>(tile)[q];
    for (int q = (words / 4) * 4 + threadIdx.x; q < words; q += blockDim.x) base[q] = tile[q];
  } else {
    for (int q = threadIdx.x; q < words; q += blockDim.x) base[q] = tile[q];
  }
}

constexpr int kRowsPerBlock = 256;

// Host-interleaved arrays (device-visible host memory, or device memory) -> component-major
// particle arrays; *bad = 1 when a position is not finite.  One block per 256 particles,
// each array moved through shared memory in contiguous 16-byte pieces.
__global__ void __launch_bounds__(kRowsPerBlock) deinterleave_arrays_kernel(HostArrays a, float* __restrict__ s,
                                                                            int64_t st, int64_t n,
                                                                            const uint32_t* __restrict__ dest, int* bad) {
  __shared__ __align__(16) float tile[9 * kRowsPerBlock];
  const int64_t r0 = (int64_t)blockIdx.x * kRowsPerBlock;
  const int cnt = (int)(n - r0 < kRowsPerBlock ? n - r0 : kRowsPerBlock);
  const int t = threadIdx.x;
  const int64_t p = r0 + t;
  // row p's device slot: its own, or its place in cell order (dest, from launch_presort)
  const int64_t q = t < cnt ? (dest ? (int64_t)dest[p] : p) : 0;
  auto field = [&](const float* src, int W, int comp0, auto def) {
    if (src) {
      if (W == 1) load_rows<1>(src, r0, cnt, tile);
      else if (W == 3) load_rows<3>(src, r0, cnt, tile);
      else load_rows<9>(src, r0, cnt, tile);
    }
    __syncthreads();
    if (t < cnt)
      for (int d = 0; d < W; ++d) {
        const float v = src ? tile[W * t + d] : def(d);
        if (comp0 == kX && !isfinite(v)) *bad = 1;
        s[(int64_t)(comp0 + d) * st + q] = v;
      }
    __syncthreads();
  };
  field(a.x, 3, kX, [](int) { return 0.f; });
  field(a.v, 3, kV, [](int) { return 0.f; });
  field(a.C, 9, kC, [](int) { return 0.f; });
  field(a.F, 9, kF, [](int d) { return (d % 4 == 0) ? 1.f : 0.f; });
  field(a.J, 1, kJp, [](int) { return 1.f; });
}

// Component-major particle arrays -> host arrays in upload order (record r from device slot
// inv[r]), written through shared memory in contiguous 16-byte pieces.
__global__ void __launch_bounds__(kRowsPerBlock) interleave_arrays_kernel(const float* __restrict__ s, int64_t st,
                                                                          const uint32_t* __restrict__ inv, int64_t n,
                                                                          OutArrays o, int liquid_layout) {
  __shared__ __align__(16) float tile[9 * kRowsPerBlock];
  const int64_t r0 = (int64_t)blockIdx.x * kRowsPerBlock;
  const int cnt = (int)(n - r0 < kRowsPerBlock ? n - r0 : kRowsPerBlock);
  const int t = threadIdx.x;
  const int64_t p = t < cnt ? (inv ? (int64_t)inv[r0 + t] : r0 + t) : 0;
  auto field = [&](float* dst, int W, auto value) {
    if (!dst) return;
    if (t < cnt)
      for (int d = 0; d < W; ++d) tile[W * t + d] = value(d);
    __syncthreads();
    if (W == 1) store_rows<1>(dst, r0, cnt, tile);
    else if (W == 3) store_rows<3>(dst, r0, cnt, tile);
    else store_rows<9>(dst, r0, cnt, tile);
    __syncthreads();
  };
  field(o.x, 3, [&](int d) { return s[(int64_t)(kX + d) * st + p]; });
  field(o.v, 3, [&](int d) { return s[(int64_t)(kV + d) * st + p]; });
  field(o.C, 9, [&](int d) { return s[(int64_t)(kC + d) * st + p]; });
  field(o.F, 9, [&](int d) {
    if (!liquid_layout) return s[(int64_t)(kF + d) * st + p];
    return (d % 4 == 0) ? cbrtf(s[(int64_t)kJp * st + p]) : 0.f;
  });
  field(o.J, 1, [&](int) { return s[(int64_t)kJp * st + p]; });
}

}  // namespace

cudaError_t launch_deinterleave_arrays(HostArrays a, float* s, int64_t stride, int64_t n, int* bad, cudaStream_t st,
                                       const uint32_t* dest, bool bad_zeroed) {
  cudaError_t e = bad_zeroed ? cudaSuccess : cudaMemsetAsync(bad, 0, sizeof(int), st);
  if (e != cudaSuccess || n == 0) return e;
  deinterleave_arrays_kernel<<<(unsigned)((n + kRowsPerBlock - 1) / kRowsPerBlock), kRowsPerBlock, 0, st>>>(
      a, s, stride, n, dest, bad);
  return cudaGetLastError();
}

cudaError_t launch_interleave_arrays(const float* s, int64_t stride, const uint32_t* inv, int64_t n, OutArrays o,
                                     int liquid_layout, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  interleave_arrays_kernel<<<(unsigned)((n + kRowsPerBlock - 1) / kRowsPerBlock), kRowsPerBlock, 0, st>>>(
      s, stride, inv, n, o, liquid_layout);
  return cudaGetLastError();
}

cudaError_t launch_inverse(const uint32_t* id, int64_t n, uint32_t* inv, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  inverse_kernel<<<grid_for(n), 256, 0, st>>>(id, n, inv);
  return cudaGetLastError();
}

// Cell-order check of an upload that kept the particle order: counts the slots whose cell
// key is below the previous slot's.  The block that finishes last writes the count to *out
// (host-visible memory) and resets the two device counters (count, ticket) for the next call.
__global__ void order_check_kernel(const float* __restrict__ s, int64_t st, int64_t n, float dx_inv, int N,
                                   int* counters, int* out) {
  __shared__ int block_count;
  if (threadIdx.x == 0) block_count = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  int mine = 0;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = base + threadIdx.x;
    const bool valid = q < n;
    const uint32_t key = valid ? cell_key(s, st, q, dx_inv, N) : 0u;
    uint32_t prev = __shfl_up_sync(kFull, key, 1);
    if (lane == 0 && valid && q > 0) prev = cell_key(s, st, q - 1, dx_inv, N);
    mine += __popc(__ballot_sync(kFull, valid && q > 0 && key < prev));
  }
  if (lane == 0 && mine) atomicAdd(&block_count, mine);
  __syncthreads();
  if (threadIdx.x == 0) {
    if (block_count) atomicAdd(counters, block_count);
    __threadfence();
    if (atomicAdd(counters + 1, 1) == (int)gridDim.x - 1) {
      *out = atomicExch(counters, 0);
      counters[1] = 0;
    }
  }
}

cudaError_t launch_order_check(const float* s, int64_t stride, int64_t n, float dx_inv, int N, int* counters, int* out,
                               cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  order_check_kernel<<<grid_for(n), 256, 0, st>>>(s, stride, n, dx_inv, N, counters, out);
  return cudaGetLastError();
}

cudaError_t launch_presort(const float* x, float* xcopy, const SortArgs& a, uint32_t* dest, int* bad, int num_sms,
                           cudaStream_t st, int64_t* launches, bool bad_zeroed) {
  if (a.n == 0) return cudaSuccess;
  cudaError_t e = bad_zeroed ? cudaSuccess : cudaMemsetAsync(bad, 0, sizeof(int), st);
  if (e == cudaSuccess) e = cudaMemsetAsync(a.counts, 0, sizeof(int) * a.cells, st);
  if (e != cudaSuccess) return e;
  const int blocks = (int)std::min<int64_t>((a.n + kThreads - 1) / kThreads, (int64_t)num_sms * 8);
  presort_keys_kernel<<<blocks, kThreads, 0, st>>>(x, xcopy, a, bad);
  int n_launch = 2 + scan_cell_counts(a, st);
  SortArgs r = a;
  r.inv = dest;  // the ranking writes the inverse too
  sort_rank<<<blocks, kThreads, 0, st>>>(r);
  if (launches) *launches += n_launch;
  return cudaGetLastError();
}

cudaError_t launch_interleave(const float* s, int64_t stride, const uint32_t* inv, int64_t n, float* stage,
                              int liquid_layout, unsigned fields, cudaStream_t st) {
  if (n == 0 || fields == 0) return cudaSuccess;
  interleave_kernel<<<grid_for(n), 256, 0, st>>>(s, stride, inv, n, stage, liquid_layout, fields);
  return cudaGetLastError();
}

namespace {
__global__ void check_finite_kernel(const float* __restrict__ x, int64_t m, int* flag) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
    if (!isfinite(x[i])) *flag = 1;  // every writer stores the same value
}
}  // namespace

cudaError_t launch_check_finite(const float* x, int64_t m, int* flag, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int), st);
  if (e != cudaSuccess || m == 0) return e;
  check_finite_kernel<<<(int)std::min<int64_t>(grid_for(m), 2048), 256, 0, st>>>(x, m, flag);
  return cudaGetLastError();
}

cudaError_t launch_iota(uint32_t* id, int64_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  iota_kernel<<<grid_for(n), 256, 0, st>>>(id, n);
  return cudaGetLastError();
}

cudaError_t launch_scatter_u8(const uint8_t* src, const uint32_t* id, int64_t n, uint8_t* dst, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  scatter_u8_kernel<<<grid_for(n), 256, 0, st>>>(src, id, n, dst);
  return cudaGetLastError();
}

// gridOpKernel (src/mpm.cu:76-107) over the whole grid, for readback: nodes with
// mass > 0 get the operated velocity and mass slot 1 (the reference divides all four
// components by the mass); others keep their raw value.
__global__ void grid_op_kernel(const float4* in, float4* out, GridConsts K) {
  const int N = K.N;
  const int64_t cells = (int64_t)N * N * N;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < cells; c += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(c / ((int64_t)N * N));
    const int j = (int)((c / N) % N);
    const int k = (int)(c % N);
    const float4 g = in[c];
    const float3 v = grid_node_velocity(g, i, j, k, K);
    out[c] = make_float4(v.x, v.y, v.z, g.w > 0.f ? g.w / g.w : g.w);
  }
}

// ---------------------------------------------------------------------------
// Scene objects joining or leaving a context: appending seeded particles and removing
// the particles of a retired object (an id range) by compaction.
// ---------------------------------------------------------------------------
__global__ void append_object_kernel(float* s, int64_t st, int64_t n0, int64_t k, const float* xs, float vx, float vy,
                                     float vz, int liquid, uint8_t* mat, uint8_t mat_index, uint32_t* id,
                                     uint32_t id0) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < k; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = n0 + p;
#pragma unroll
    for (int d = 0; d < 3; ++d) s[(kX + d) * st + q] = xs[3 * p + d];
    s[(kV + 0) * st + q] = vx;
    s[(kV + 1) * st + q] = vy;
    s[(kV + 2) * st + q] = vz;
#pragma unroll
    for (int i = 0; i < 9; ++i) s[(kC + i) * st + q] = 0.f;
    if (!liquid) {
#pragma unroll
      for (int i = 0; i < 9; ++i) s[(kF + i) * st + q] = (i % 4 == 0) ? 1.f : 0.f;
    }
    s[kJp * st + q] = 1.f;
    if (mat) mat[q] = mat_index;
    id[q] = id0 + (uint32_t)p;
  }
}

__global__ void keep_flags_kernel(const uint32_t* id, int64_t n, uint32_t lo, uint32_t hi, int* flags) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p <= n; p += (int64_t)gridDim.x * blockDim.x)
    flags[p] = (p < n && (id[p] < lo || id[p] >= hi)) ? 1 : 0;
}

template <bool LIQ>
__global__ void compact_kernel(const float* __restrict__ sA, float* __restrict__ sB, int64_t st, int64_t n,
                               const int* __restrict__ pos, const uint32_t* idA, uint32_t* idB, const uint8_t* matA,
                               uint8_t* matB, uint32_t lo, uint32_t hi) {
  constexpr int NC = LIQ ? kLiquidComps : kNumComps;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t i = idA[p];
    if (i >= lo && i < hi) continue;
    const int64_t q = pos[p];
#pragma unroll
    for (int c = 0; c < NC; ++c) sB[moved_comp<LIQ>(c) * st + q] = sA[moved_comp<LIQ>(c) * st + p];
    idB[q] = i >= hi ? i - (hi - lo) : i;
    if (matA) matB[q] = matA[p];
  }
}

cudaError_t launch_append_object(float* s, int64_t st, int64_t n0, int64_t k, const float* xs, const float v[3],
                                 bool liquid, uint8_t* mat, uint8_t mat_index, uint32_t* id, uint32_t id0,
                                 cudaStream_t stream) {
  if (k <= 0) return cudaSuccess;
  const int blocks = (int)std::min<int64_t>((k + kThreads - 1) / kThreads, 4096);
  append_object_kernel<<<blocks, kThreads, 0, stream>>>(s, st, n0, k, xs, v[0], v[1], v[2], liquid ? 1 : 0, mat,
                                                          mat_index, id, id0);
  return cudaGetLastError();
}

cudaError_t launch_remove_ids(const float* sA, float* sB, int64_t st, int64_t n, const uint32_t* idA, uint32_t* idB,
                              const uint8_t* matA, uint8_t* matB, uint32_t lo, uint32_t hi, bool liquid, int* flags,
                              int* scratch, cudaStream_t stream, int64_t* launches) {
  const int blocks = (int)std::min<int64_t>((n + kThreads) / kThreads, 4096);
  keep_flags_kernel<<<blocks, kThreads, 0, stream>>>(idA, n, lo, hi, flags);
  cudaError_t e = launch_exclusive_scan(flags, n + 1, scratch, stream, launches);
  if (e != cudaSuccess) return e;
  if (liquid)
    compact_kernel<true><<<blocks, kThreads, 0, stream>>>(sA, sB, st, n, flags, idA, idB, matA, matB, lo, hi);
  else
    compact_kernel<false><<<blocks, kThreads, 0, stream>>>(sA, sB, st, n, flags, idA, idB, matA, matB, lo, hi);
  if (launches) *launches += 2;
  return cudaGetLastError();
}

int64_t scan_scratch_ints(int64_t m) { return (m + kThreads * kScanItems - 1) / (kThreads * kScanItems) + 1; }

cudaError_t launch_exclusive_scan(int* data, int64_t m, int* scratch, cudaStream_t st, int64_t* launches) {
  if (m <= 0) return cudaSuccess;
  const int per = kThreads * kScanItems;
  const int nb = (int)((m + per - 1) / per);
  scan_blocks<<<nb, kThreads, 0, st>>>(data, m, scratch);
  scan_block_sums<<<1, kThreads, 0, st>>>(scratch, nb);
  scan_add<<<nb, kThreads, 0, st>>>(data, m, scratch);
  if (launches) *launches += 3;
  return cudaGetLastError();
}

cudaError_t launch_grid_op(const float4* in, float4* out, GridConsts K, cudaStream_t st) {
  const int64_t cells = (int64_t)K.N * K.N * K.N;
  grid_op_kernel<<<grid_for(cells), 256, 0, st>>>(in, out, K);
  return cudaGetLastError();
}

}  // namespace mpm
