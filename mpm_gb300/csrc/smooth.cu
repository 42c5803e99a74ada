// Laplacian smoothing of a triangle mesh on the GPU (MeshBuilder::smoothMesh,
// include/mesh_builder.h:212-245, applied by computeMesh when --laplacian_smooth is set).
//
// The reference makes one implicit smoothing step with libigl and rescales to unit area:
//   L = cotmatrix(V, F), M = massmatrix(V, F, BARYCENTRIC),
//   U = (M - 0.001 L)^-1 M V,   U /= sqrt(0.5 sum doublearea(U, F)),
// and factors S = M - 0.001 L by a sparse Cholesky (SimplicialLLT).  Here, in double as
// there:
//   - one thread per face forms libigl's cotangent entries from the squared edge lengths and
//     Kahan's form of Heron's area with the lengths sorted in decreasing order
//     (cotmatrix_entries, doublearea of edge lengths with NaN replaced by 0):
//     C(f, e) = (l2_a + l2_b - l2_e) / dblA / 4 for the edge e opposite corner e;
//   - the faces' corners are grouped by vertex (a count, a scan and a fill, each row then
//     sorted by corner); each corner gives its vertex two neighbours with the entries of the
//     edges to them, and a row's entries to the same neighbour are summed (in corner
//     order), so that row i holds L's off-diagonal entries L(i, j) as libigl's triplets sum
//     them (cotmatrix).  Row i also gives the lumped mass M(i) = sum of dblA / 6 over its
//     corners (massmatrix_intrinsic, BARYCENTRIC) and D(i) = -L(i, i), the sum of its entries;
//   - the solve is written for the displacement Y = U - V: S Y = M V - S V = 0.001 L V, whose
//     right side is formed once as 0.001 sum C (V_j - V_i).  Y is small next to V, so the
//     products S p = M p - 0.001 (sum L(i, j) p_j - D(i) p_i) round no worse than the
//     difference form at one fused multiply-add per neighbour and coordinate.  The three
//     coordinates are solved together by conjugate gradients preconditioned by the diagonal
//     of S, to a relative residual |M V - S U| <= 1e-12 |M V| per coordinate.  -L is the
//     stiffness matrix of linear elements and so positive semidefinite whatever the
//     triangles' shapes; S is then positive definite on the vertices that faces use (the
//     reference's LLT needs the same).  A vertex no face uses has a zero row and keeps its
//     position (scaled like the rest);
//   - an iteration is three kernels over the vertices: q = S p, then the update of Y and r,
//     then the new direction.  The block that finishes a kernel last (a ticket counter, no
//     waiting) sums the blocks' partial sums in block order and leaves the step length
//     alpha = r.z / p.q or the factor beta = r'.z' / r.z for the next kernel; a batch of
//     iterations between two residual read-backs runs as one CUDA graph;
//   - the area is libigl's 3-D doublearea of U = V + Y (the double areas projected on the
//     planes (x, y), (y, z), (z, x), summed in squares).
// GB300 runs double precision at a small fraction of its single-precision rate, so the
// kernels spend their double operations sparingly: one fused multiply-add per entry, a
// precomputed inverse diagonal, and warp sums that halve the values they carry at the first
// exchange.  Every sum runs in a fixed order, so a call's result is reproducible bit for bit
// (rows of more than 64 corners are left unsorted).  It agrees with a direct solve of the
// same system to the solver's tolerance times the condition number.
#include <algorithm>
#include <cmath>

#include "mpm_internal.h"
#include "surface.h"

namespace mpm {

namespace {

constexpr int kSmoothThreads = 256;
constexpr int kSmoothWarps = kSmoothThreads / 32;
constexpr int kSortedRow = 64;  // rows up to this many corners are sorted and merged

// Scalars, in SmoothBuffers::scal: per coordinate alpha, beta, r.z, r.r, b.b, then the area.
enum : int { kAlpha = 0, kBeta = 3, kRz = 6, kRr = 9, kBb = 12, kArea = 15, kScalars = 16 };
// SmoothBuffers::flags: [0] the check bits, [1] the last-block ticket.
enum : int { kBadArea = 1, kBadIndex = 2 };

// Sums K values over the block into tot (every thread receives the totals).  A warp first
// exchanges half of its values across the half-warps (K even), then sums the rest by
// butterfly; warp 0 sums the warps' results.  The order depends only on the block size.
template <int K>
__device__ __forceinline__ void block_allreduce(const double (&v)[K], double (&tot)[K]) {
  static_assert(K % 2 == 0, "an even number of values");
  constexpr int H = K / 2;
  __shared__ double red[K][kSmoothWarps];
  __shared__ double out[K];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool upper = (lane & 16) != 0;
  double h[H];
#pragma unroll
  for (int j = 0; j < H; ++j) {
    const double keep = upper ? v[H + j] : v[j];
    const double give = upper ? v[j] : v[H + j];
    h[j] = keep + __shfl_xor_sync(0xffffffffu, give, 16);
  }
#pragma unroll
  for (int o = 8; o; o >>= 1)
#pragma unroll
    for (int j = 0; j < H; ++j) h[j] += __shfl_xor_sync(0xffffffffu, h[j], o);
  __syncthreads();  // red and out may still be read by a previous call
  if (lane == 0)
#pragma unroll
    for (int j = 0; j < H; ++j) red[j][warp] = h[j];
  if (lane == 16)
#pragma unroll
    for (int j = 0; j < H; ++j) red[H + j][warp] = h[j];
  __syncthreads();
  if (threadIdx.x < K) {
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < kSmoothWarps; ++q) s += red[threadIdx.x][q];
    out[threadIdx.x] = s;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) tot[k] = out[k];
}

// Writes the block's sums of v to part[blockIdx.x * K ...]; in the block that finishes last
// (of nblk), returns true with the totals over all blocks, summed in block order, in tot.
template <int K>
__device__ __forceinline__ bool block_sum_last(const double (&v)[K], double* part, int nblk, int* ticket,
                                               double (&tot)[K]) {
  __shared__ int last;
  double b[K];
  block_allreduce<K>(v, b);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) part[blockIdx.x * K + k] = b[k];
    __threadfence();
    last = atomicAdd(ticket, 1) == nblk - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double s[K];
#pragma unroll
  for (int k = 0; k < K; ++k) s[k] = 0.0;
  for (int q = threadIdx.x; q < nblk; q += kSmoothThreads)
#pragma unroll
    for (int k = 0; k < K; ++k) s[k] += __ldcg(part + q * K + k);
  block_allreduce<K>(s, tot);
  if (threadIdx.x == 0) *ticket = 0;
  return true;
}

// Per face: checks the indices, forms the cotangent entries and the double area
// (C[4 f ..] = C0, C1, C2, dblA) and counts each vertex's corners.
__global__ void smooth_faces_kernel(const double* __restrict__ V, const int* __restrict__ F, int64_t nf,
                                    int64_t nv, double* __restrict__ C, int* __restrict__ count, int* flags) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int v[3] = {F[3 * f], F[3 * f + 1], F[3 * f + 2]};
  if (v[0] < 0 || v[0] >= nv || v[1] < 0 || v[1] >= nv || v[2] < 0 || v[2] >= nv) {
    atomicOr(flags, kBadIndex);
    return;
  }
  // squared edge lengths, edge e opposite corner e: (1,2), (2,0), (0,1)
  const int ea[3] = {1, 2, 0}, eb[3] = {2, 0, 1};
  double l2[3];
#pragma unroll
  for (int e = 0; e < 3; ++e) {
    const double* a = V + 3 * (int64_t)v[ea[e]];
    const double* b = V + 3 * (int64_t)v[eb[e]];
    const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    l2[e] = dx * dx + dy * dy + dz * dz;
  }
  double a = sqrt(l2[0]), b = sqrt(l2[1]), c = sqrt(l2[2]), t;
  if (a < b) { t = a; a = b; b = t; }
  if (b < c) { t = b; b = c; c = t; }
  if (a < b) { t = a; a = b; b = t; }
  const double arg = (a + (b + c)) * (c - (a - b)) * (c + (a - b)) * (a + (b - c));
  double dblA = 2.0 * 0.25 * sqrt(arg);
  if (dblA != dblA) dblA = 0.0;
  if (!(dblA > 0.0)) atomicOr(flags, kBadArea);  // the reference's entries are not finite here
  C[4 * f + 0] = (l2[1] + l2[2] - l2[0]) / dblA / 4.0;
  C[4 * f + 1] = (l2[2] + l2[0] - l2[1]) / dblA / 4.0;
  C[4 * f + 2] = (l2[0] + l2[1] - l2[2]) / dblA / 4.0;
  C[4 * f + 3] = dblA;
#pragma unroll
  for (int k = 0; k < 3; ++k) atomicAdd(count + v[k], 1);
}

// Each corner 3 f + k into its vertex's row (in any order; sorted afterwards).
__global__ void smooth_fill_kernel(const int* __restrict__ F, int64_t nf, const int* __restrict__ rowptr,
                                   int* __restrict__ fill, int* __restrict__ corner) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int v = F[3 * f + k];
    const int slot = atomicAdd(fill + v, 1);
    corner[rowptr[v] + slot] = (int)(3 * f + k);
  }
}

// Per vertex: sorts its corners, expands each into two (neighbour, entry) pairs at
// 2 rowptr[i] .., sorts those by neighbour (stably) and sums the entries of a neighbour;
// leaves the row's length, M(i), D(i) and 1 / S(i, i).
__global__ void smooth_expand_kernel(const int* __restrict__ F, const double* __restrict__ C, int64_t nv,
                                     const int* __restrict__ rowptr, int* __restrict__ corner,
                                     int* __restrict__ nbr, double* __restrict__ w, int* __restrict__ len,
                                     double* __restrict__ M, double* __restrict__ D, double* __restrict__ inv) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += (int64_t)gridDim.x * blockDim.x) {
    const int lo = rowptr[i], hi = rowptr[i + 1];
    const bool sorted = hi - lo <= kSortedRow;
    if (sorted)
      for (int a = lo + 1; a < hi; ++a) {  // insertion sort of the corners
        const int key = corner[a];
        int b = a - 1;
        while (b >= lo && corner[b] > key) {
          corner[b + 1] = corner[b];
          --b;
        }
        corner[b + 1] = key;
      }
    double m = 0.0, d = 0.0;
    const int64_t base = 2 * (int64_t)lo;  // 2 pairs per corner: up to 6 x (faces) entries
    for (int e = lo; e < hi; ++e) {
      const int id = corner[e];
      const int f = id / 3, k = id - 3 * f;
      const int k1 = k == 2 ? 0 : k + 1, k2 = k == 0 ? 2 : k - 1;
      // the edge to corner k1 is opposite corner k2, the edge to corner k2 opposite k1
      const double w1 = C[4 * (int64_t)f + k2], w2 = C[4 * (int64_t)f + k1];
      const int64_t o = base + 2 * (int64_t)(e - lo);
      nbr[o] = F[3 * (int64_t)f + k1];
      w[o] = w1;
      nbr[o + 1] = F[3 * (int64_t)f + k2];
      w[o + 1] = w2;
      m += C[4 * (int64_t)f + 3] / 6.0;
      d += w1 + w2;
    }
    int n = 2 * (hi - lo);
    if (sorted && n > 1) {
      for (int64_t a = base + 1; a < base + n; ++a) {  // stable insertion sort by neighbour
        const int kn = nbr[a];
        const double kw = w[a];
        int64_t b = a - 1;
        while (b >= base && nbr[b] > kn) {
          nbr[b + 1] = nbr[b];
          w[b + 1] = w[b];
          --b;
        }
        nbr[b + 1] = kn;
        w[b + 1] = kw;
      }
      int u = 1;
      for (int64_t a = base + 1; a < base + n; ++a) {
        if (nbr[a] == nbr[base + u - 1]) {
          w[base + u - 1] += w[a];
        } else {
          nbr[base + u] = nbr[a];
          w[base + u] = w[a];
          ++u;
        }
      }
      n = u;
    }
    len[i] = n;
    M[i] = m;
    D[i] = d;
    const double diag = m + 0.001 * d;
    inv[i] = diag > 0.0 ? 1.0 / diag : 0.0;
  }
}

struct Solver {
  const int* rowptr;
  const int* len;
  const int* nbr;
  const double* w;
  const double* M;
  const double* D;
  const double* inv;
  double* y;
  double* r;
  double* p;
  double* q;
  double* part;
  double* scal;
  int* ticket;
  int64_t nv;
  int nblk;
};

// b = M V, Y = 0, r = 0.001 L V (difference form), p = r / S(i, i); totals of r.z, b.b, r.r.
__global__ void smooth_init_kernel(Solver s, const double* __restrict__ V) {
  double acc[10] = {};  // r.z, b.b, r.r (3 each), padding
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < s.nv; i += (int64_t)gridDim.x * blockDim.x) {
    const double vi[3] = {V[3 * i], V[3 * i + 1], V[3 * i + 2]};
    double lv[3] = {0.0, 0.0, 0.0};
    const int64_t o = 2 * (int64_t)s.rowptr[i];
    const int n = s.len[i];
    for (int64_t e = o; e < o + n; ++e) {
      const int j = s.nbr[e];
      const double we = s.w[e];
#pragma unroll
      for (int k = 0; k < 3; ++k) lv[k] += we * (V[3 * (int64_t)j + k] - vi[k]);
    }
    const double m = s.M[i], inv = s.inv[i];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double b = m * vi[k];
      const double rv = 0.001 * lv[k];
      const double z = inv * rv;
      s.y[3 * i + k] = 0.0;
      s.r[3 * i + k] = rv;
      s.p[3 * i + k] = z;
      acc[k] += rv * z;
      acc[3 + k] += b * b;
      acc[6 + k] += rv * rv;
    }
  }
  double tot[10];
  if (block_sum_last<10>(acc, s.part, s.nblk, s.ticket, tot) && threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      s.scal[kRz + k] = tot[k];
      s.scal[kBb + k] = tot[3 + k];
      s.scal[kRr + k] = tot[6 + k];
    }
}

// q = S p = M p - 0.001 (sum L(i, j) p_j - D(i) p_i); alpha = r.z / p.q.
__global__ void smooth_apply_kernel(Solver s) {
  double acc[4] = {};  // p.q (3), padding
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < s.nv; i += (int64_t)gridDim.x * blockDim.x) {
    const double pi[3] = {s.p[3 * i], s.p[3 * i + 1], s.p[3 * i + 2]};
    const double d = s.D[i], m = s.M[i];
    double lp[3] = {-d * pi[0], -d * pi[1], -d * pi[2]};
    const int64_t o = 2 * (int64_t)s.rowptr[i];
    const int n = s.len[i];
    for (int64_t e = o; e < o + n; ++e) {
      const int j = s.nbr[e];
      const double we = s.w[e];
#pragma unroll
      for (int k = 0; k < 3; ++k) lp[k] = fma(we, s.p[3 * (int64_t)j + k], lp[k]);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double qv = fma(m, pi[k], -0.001 * lp[k]);
      s.q[3 * i + k] = qv;
      acc[k] = fma(pi[k], qv, acc[k]);
    }
  }
  double tot[4];
  if (block_sum_last<4>(acc, s.part, s.nblk, s.ticket, tot) && threadIdx.x < 3) {
    const int k = threadIdx.x;
    s.scal[kAlpha + k] = tot[k] != 0.0 ? s.scal[kRz + k] / tot[k] : 0.0;
  }
}

// Y += alpha p, r -= alpha q; beta = r'.z' / r.z, and r'.r' for the host.
__global__ void smooth_update_kernel(Solver s) {
  const double alpha[3] = {s.scal[kAlpha], s.scal[kAlpha + 1], s.scal[kAlpha + 2]};
  double acc[6] = {};  // r'.z' (3), r'.r' (3)
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < s.nv; i += (int64_t)gridDim.x * blockDim.x) {
    const double inv = s.inv[i];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const double pv = s.p[3 * i + k];
      s.y[3 * i + k] = fma(alpha[k], pv, s.y[3 * i + k]);
      const double rv = fma(-alpha[k], s.q[3 * i + k], s.r[3 * i + k]);
      s.r[3 * i + k] = rv;
      acc[k] = fma(rv * inv, rv, acc[k]);
      acc[3 + k] = fma(rv, rv, acc[3 + k]);
    }
  }
  double tot[6];
  if (block_sum_last<6>(acc, s.part, s.nblk, s.ticket, tot) && threadIdx.x < 3) {
    const int k = threadIdx.x;
    const double rz = s.scal[kRz + k];
    s.scal[kBeta + k] = rz != 0.0 ? tot[k] / rz : 0.0;
    s.scal[kRz + k] = tot[k];
    s.scal[kRr + k] = tot[3 + k];
  }
}

// p = r / S(i, i) + beta p.
__global__ void smooth_direction_kernel(Solver s) {
  const double beta[3] = {s.scal[kBeta], s.scal[kBeta + 1], s.scal[kBeta + 2]};
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < s.nv; i += (int64_t)gridDim.x * blockDim.x) {
    const double inv = s.inv[i];
#pragma unroll
    for (int k = 0; k < 3; ++k) s.p[3 * i + k] = fma(beta[k], s.p[3 * i + k], inv * s.r[3 * i + k]);
  }
}

// libigl's 3-D double areas of the faces of V + Y, summed.
__global__ void smooth_area_kernel(Solver s, const double* __restrict__ V, const int* __restrict__ F, int64_t nf) {
  double acc[2] = {0.0, 0.0};
  for (int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += (int64_t)gridDim.x * blockDim.x) {
    double P[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int64_t v = F[3 * f + c];
#pragma unroll
      for (int k = 0; k < 3; ++k) P[c][k] = V[3 * v + k] + s.y[3 * v + k];
    }
    double a = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int x = d, y = d == 2 ? 0 : d + 1;
      const double rx = P[0][x] - P[2][x], sx = P[1][x] - P[2][x], ry = P[0][y] - P[2][y], sy = P[1][y] - P[2][y];
      const double pd = rx * sy - ry * sx;
      a += pd * pd;
    }
    acc[0] += sqrt(a);
  }
  double tot[2];
  if (block_sum_last<2>(acc, s.part, s.nblk, s.ticket, tot) && threadIdx.x == 0) s.scal[kArea] = tot[0];
}

// V = (V + Y) / sqrt(area), area = half the summed double areas.
__global__ void smooth_scale_kernel(Solver s, double* __restrict__ V) {
  const double scale = sqrt(0.5 * s.scal[kArea]);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < 3 * s.nv; i += (int64_t)gridDim.x * blockDim.x)
    V[i] = (V[i] + s.y[i]) / scale;
}

template <class T>
cudaError_t ensure(T*& p, int64_t& cap, int64_t need) {
  if (p && cap >= need) return cudaSuccess;
  cudaFree(p);
  p = nullptr;
  cap = 0;
  const cudaError_t e = cudaMalloc(&p, sizeof(T) * (size_t)std::max<int64_t>(need, 1));
  if (e == cudaSuccess) cap = need;
  return e;
}

int blocks_for(int64_t n) { return (int)std::max<int64_t>((n + kSmoothThreads - 1) / kSmoothThreads, 1); }

// One batch of kSmoothCheckEvery iterations.
void enqueue_batch(const Solver& s, cudaStream_t st) {
  for (int it = 0; it < kSmoothCheckEvery; ++it) {
    smooth_apply_kernel<<<s.nblk, kSmoothThreads, 0, st>>>(s);
    smooth_update_kernel<<<s.nblk, kSmoothThreads, 0, st>>>(s);
    smooth_direction_kernel<<<s.nblk, kSmoothThreads, 0, st>>>(s);
  }
}

// Whether work can be captured from this stream into a graph: not the legacy or per-thread
// default stream, and not a stream that is itself being captured.
bool capturable(cudaStream_t st) {
  if (st == 0 || st == cudaStreamLegacy || st == cudaStreamPerThread) return false;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  return cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone;
}

}  // namespace

void SmoothBuffers::release() {
  cudaFree(C);
  cudaFree(vec);
  cudaFree(part);
  cudaFree(scal);
  cudaFree(flags);
  cudaFree(ints);
  cudaFree(w);
  cudaFree(V);
  cudaFree(F);
  cudaFreeHost(host);
  *this = SmoothBuffers{};
}

cudaError_t smooth_mesh(double* V, const int* F, int64_t nv, int64_t nf, SmoothBuffers& sb, cudaStream_t st,
                        int64_t* launches, SmoothResult* res) {
  *res = SmoothResult{};
  if (nv <= 0) {
    res->converged = true;
    return cudaSuccess;
  }
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  // vertex kernels: at most 4 blocks per SM, looping over the vertices, so that the last
  // block sums few partials
  const int nblk = std::min(blocks_for(nv), 4 * std::max(sms, 1));
  const int fb = blocks_for(nf);
  const int64_t nc = 3 * nf;  // corners
  const int64_t scan_n = nv + 1;
  const int64_t n_scratch = scan_scratch_ints(scan_n);
  // ints: row offsets and fill counters (nv + 1 each), scan scratch, corners, row lengths,
  // neighbours (2 per corner)
  const int64_t n_ints = 2 * scan_n + n_scratch + nc + nv + 2 * nc;
  if ((e = ensure(sb.C, sb.C_cap, 4 * std::max<int64_t>(nf, 1))) != cudaSuccess) return e;
  if ((e = ensure(sb.vec, sb.vec_cap, 15 * nv)) != cudaSuccess) return e;  // M, D, 1/S(i,i); Y, r, p, q
  if ((e = ensure(sb.part, sb.part_cap, 10 * (int64_t)nblk)) != cudaSuccess) return e;
  if ((e = ensure(sb.ints, sb.ints_cap, n_ints)) != cudaSuccess) return e;
  if ((e = ensure(sb.w, sb.w_cap, std::max<int64_t>(2 * nc, 1))) != cudaSuccess) return e;
  if (!sb.scal && (e = cudaMalloc(&sb.scal, kScalars * sizeof(double))) != cudaSuccess) return e;
  if (!sb.flags && (e = cudaMalloc(&sb.flags, 2 * sizeof(int))) != cudaSuccess) return e;
  if (!sb.host && (e = cudaMallocHost(&sb.host, 8 * sizeof(double))) != cudaSuccess) return e;
  int* rowptr = sb.ints;  // nv + 1: counts, then their exclusive scan
  int* fill = rowptr + scan_n;
  int* scratch = fill + scan_n;
  int* corner = scratch + n_scratch;
  int* len = corner + nc;
  int* nbr = len + nv;
  Solver s;
  s.rowptr = rowptr;
  s.len = len;
  s.nbr = nbr;
  s.w = sb.w;
  double* M = sb.vec;
  double* D = M + nv;
  double* inv = D + nv;
  s.M = M;
  s.D = D;
  s.inv = inv;
  s.y = inv + nv;
  s.r = s.y + 3 * nv;
  s.p = s.r + 3 * nv;
  s.q = s.p + 3 * nv;
  s.part = sb.part;
  s.scal = sb.scal;
  s.ticket = sb.flags + 1;
  s.nv = nv;
  s.nblk = nblk;
  int64_t n_launch = 0;
  double* host = sb.host;  // [0..3) b.b, [3..6) r.r, [6] the check bits
  int* flags_host = reinterpret_cast<int*>(host + 6);

  // entries, checks and the corners per vertex
  if ((e = cudaMemsetAsync(rowptr, 0, sizeof(int) * 2 * scan_n, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(sb.flags, 0, 2 * sizeof(int), st)) != cudaSuccess) return e;
  if (nf > 0) {
    smooth_faces_kernel<<<fb, kSmoothThreads, 0, st>>>(V, F, nf, nv, sb.C, rowptr, sb.flags);
    ++n_launch;
  }
  if ((e = cudaMemcpyAsync(flags_host, sb.flags, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  res->bad_index = (*flags_host & kBadIndex) != 0;
  res->bad_area = (*flags_host & kBadArea) != 0;
  if (res->bad_index || res->bad_area) {
    if (launches) *launches += n_launch;
    return cudaSuccess;
  }
  // rows, their merged entries, M, D and 1 / S(i, i); the initial residual
  if ((e = launch_exclusive_scan(rowptr, scan_n, scratch, st, &n_launch)) != cudaSuccess) return e;
  if (nf > 0) {
    smooth_fill_kernel<<<fb, kSmoothThreads, 0, st>>>(F, nf, rowptr, fill, corner);
    ++n_launch;
  }
  smooth_expand_kernel<<<nblk, kSmoothThreads, 0, st>>>(F, sb.C, nv, rowptr, corner, nbr, sb.w, len, M, D, inv);
  smooth_init_kernel<<<nblk, kSmoothThreads, 0, st>>>(s, V);
  n_launch += 2;
  if ((e = cudaMemcpyAsync(host, sb.scal + kBb, 3 * sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return e;
  if ((e = cudaMemcpyAsync(host + 3, sb.scal + kRr, 3 * sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return e;
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  const double bb[3] = {host[0], host[1], host[2]};
  // the largest relative residual over the coordinates (NaN propagates)
  auto relres = [&](const double* rr) {
    double worst = 0.0;
    for (int k = 0; k < 3; ++k) {
      const double v = bb[k] > 0.0 ? std::sqrt(rr[k] / bb[k]) : (rr[k] > 0.0 ? INFINITY : 0.0);
      if (v != v) return v;
      worst = std::max(worst, v);
    }
    return worst;
  };
  double rel = relres(host + 3);

  // batches of iterations, as one graph where the stream allows it
  cudaGraphExec_t exec = nullptr;
  int it = 0;
  while (!(rel <= kSmoothTolerance) && it < kSmoothMaxIterations && rel == rel) {
    if (!exec && capturable(st)) {
      cudaGraph_t graph = nullptr;
      if ((e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
      enqueue_batch(s, st);
      const cudaError_t ce = cudaStreamEndCapture(st, &graph);
      if (ce == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
      if (graph) cudaGraphDestroy(graph);
      if (ce != cudaSuccess) return ce;
      if (e != cudaSuccess) return e;
    }
    if (exec) {
      e = cudaGraphLaunch(exec, st);
    } else {
      enqueue_batch(s, st);
      e = cudaGetLastError();
    }
    n_launch += 3 * kSmoothCheckEvery;
    it += kSmoothCheckEvery;
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(host + 3, sb.scal + kRr, 3 * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
      if (exec) cudaGraphExecDestroy(exec);
      return e;
    }
    rel = relres(host + 3);
  }
  if (exec) cudaGraphExecDestroy(exec);
  res->iterations = it;
  res->relative_residual = rel;
  res->converged = rel <= kSmoothTolerance;
  if (res->converged) {
    smooth_area_kernel<<<nblk, kSmoothThreads, 0, st>>>(s, V, F, nf);
    smooth_scale_kernel<<<nblk, kSmoothThreads, 0, st>>>(s, V);
    n_launch += 2;
  }
  if (launches) *launches += n_launch;
  return cudaGetLastError();
}

}  // namespace mpm
