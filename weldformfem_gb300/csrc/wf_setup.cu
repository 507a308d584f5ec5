// Device-side setup for wf_init: the connectivity tables the step kernels
// read (SoA element nodes, node -> element lists as CSR slots) and the
// initial state fills, built on the GPU from the caller's AoS arrays after one
// upload each, instead of on host threads.
//
// Node -> element lists (setNodElem, Domain_d.C:1508-1611): the entries of
// node n are the slots e * npe + a with elnod[e][a] == n, in ascending slot
// order (element-ascending, as the reference's serial build leaves them).
// Built as count -> exclusive scan -> placement -> per-list sort: placement
// claims positions with atomics, so its order within a list is arbitrary, and
// the sort of each list restores the one deterministic order. Every step of
// it is integer work, so the tables equal the host build bit for bit.
#include "wf_internal.cuh"

namespace wf {
namespace {

constexpr int kThreads = 256;
constexpr int kScanItems = 16;                        // per thread
constexpr int kScanTile = kThreads * kScanItems;      // per block

inline unsigned grid_for(int64_t n, int threads = kThreads) {
  const int64_t g = (n + threads - 1) / threads;
  return (unsigned)std::min<int64_t>(std::max<int64_t>(g, 1), 1 << 20);
}

#define GRID_STRIDE(i, n) \
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); \
       i += (int64_t)gridDim.x * blockDim.x)

__global__ void k_count(const int32_t *el, int64_t ent, int32_t *cnt) {
  GRID_STRIDE(i, ent) atomicAdd(&cnt[el[i]], 1);
}

// Block-wide exclusive scan of one value per thread; returns the prefix and
// the block total.
__device__ __forceinline__ int32_t block_scan(int32_t v, int32_t &total) {
  __shared__ int32_t warp[kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp[w] = x;
  __syncthreads();
  if (w == 0) {
    int32_t s = lane < kThreads / 32 ? warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < kThreads / 32) warp[lane] = s;
  }
  __syncthreads();
  const int32_t before = (w > 0 ? warp[w - 1] : 0) + x - v;
  total = warp[kThreads / 32 - 1];
  __syncthreads();
  return before;
}

// (1) per tile of kScanTile counts: their sum
__global__ void __launch_bounds__(kThreads) k_tile_sums(const int32_t *cnt, int64_t n,
                                                        int32_t *tsum) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  int32_t s = 0;
  for (int j = 0; j < kScanItems; j++) {
    const int64_t i = base + (int64_t)j * kThreads + threadIdx.x;
    if (i < n) s += cnt[i];
  }
  int32_t total;
  block_scan(s, total);
  if (threadIdx.x == 0) tsum[blockIdx.x] = total;
}

// (2) exclusive scan of the tile sums in place, one block
__global__ void __launch_bounds__(kThreads) k_scan_tile_sums(int32_t *tsum, int64_t nt) {
  int32_t carry = 0;
  for (int64_t b = 0; b < nt; b += kThreads) {
    const int64_t i = b + threadIdx.x;
    const int32_t v = i < nt ? tsum[i] : 0;
    int32_t total;
    const int32_t p = block_scan(v, total);
    if (i < nt) tsum[i] = carry + p;
    carry += total;
  }
}

// (3) offsets: each thread scans kScanItems consecutive counts of its tile;
// off[n] = entries of the nodes before n, off[nn] = all entries.
__global__ void __launch_bounds__(kThreads) k_tile_offsets(const int32_t *cnt, int64_t n,
                                                           const int32_t *tsum, int32_t *off) {
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int32_t v[kScanItems];
  int32_t s = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    v[j] = base + j < n ? cnt[base + j] : 0;
    s += v[j];
  }
  int32_t total;
  int32_t run = tsum[blockIdx.x] + block_scan(s, total);
#pragma unroll
  for (int j = 0; j < kScanItems; j++) {
    if (base + j < n) off[base + j] = run;
    run += v[j];
    if (base + j == n - 1) off[n] = run;
  }
}

__global__ void k_place(const int32_t *el, int64_t ent, const int32_t *off, int32_t *fill,
                        int32_t *slot) {
  GRID_STRIDE(i, ent) {
    const int32_t n = el[i];
    slot[off[n] + atomicAdd(&fill[n], 1)] = (int32_t)i;
  }
}

// Insertion sort of each node's list (a few to a few dozen entries).
__global__ void k_sort_lists(const int32_t *off, int64_t nn, int32_t *slot) {
  GRID_STRIDE(n, nn) {
    const int32_t b = off[n], c = off[n + 1] - b;
    int32_t *s = slot + b;
    for (int32_t i = 1; i < c; i++) {
      const int32_t v = s[i];
      int32_t j = i - 1;
      while (j >= 0 && s[j] > v) {
        s[j + 1] = s[j];
        j--;
      }
      s[j + 1] = v;
    }
  }
}

// elnod[e][a] (AoS) -> soa[a * ne + e]
__global__ void k_elnod_soa(const int32_t *el, int64_t ne, int npe, int32_t *soa) {
  GRID_STRIDE(j, ne * npe) {
    const int64_t a = j / ne, e = j - a * ne;
    soa[j] = el[e * npe + a];
  }
}

// x[n][k] (AoS, nn nodes) -> out[k * np + n], zero in the padding n >= nn
__global__ void k_coords_soa(const double *x, int64_t nn, int64_t np, double *out) {
  GRID_STRIDE(j, 3 * np) {
    const int64_t k = j / np, n = j - k * np;
    out[j] = n < nn ? x[3 * n + k] : 0.0;
  }
}

// SoA [3][np] -> AoS [nn][3]
__global__ void k_coords_aos(const double *soa, int64_t nn, int64_t np, double *out) {
  GRID_STRIDE(j, 3 * nn) {
    const int64_t n = j / 3, k = j - 3 * n;
    out[j] = soa[k * np + n];
  }
}

__global__ void k_fill(double *p, double v, int64_t n) {
  GRID_STRIDE(i, n) p[i] = v;
}

__global__ void k_initial_yield(const MatDev *mats, const int32_t *emat, int64_t ne, double *sy) {
  GRID_STRIDE(e, ne) sy[e] = mats[emat ? emat[e] : 0].sy0;
}

// v = 0 except the z components of nodes with a z velocity BC (the preamble
// zeroes v inside its per-dimension BC loop, so only the last dimension's
// values survive into the first step)
__global__ void k_initial_velocity(const uint32_t *bc, const double *bcval, int64_t nn,
                                   int64_t np, double *v) {
  GRID_STRIDE(j, 3 * np) {
    const int64_t k = j / np, n = j - k * np;
    double val = 0.0;
    if (k == 2 && n < nn) {
      const uint32_t code = bc[n];
      if ((code >> 2) & 1u) val = bcval[3 * (code >> 3) + 2];
    }
    v[j] = val;
  }
}

}  // namespace

int64_t connectivity_scratch_ints(int64_t nn) {
  return 2 * nn + (nn + kScanTile - 1) / kScanTile + 1;
}

cudaError_t build_connectivity(const int32_t *el_aos, int64_t ne, int npe, int64_t nn,
                               int32_t *el_soa, int32_t *off, int32_t *slot, int32_t *scratch,
                               cudaStream_t st) {
  const int64_t ent = ne * npe, ntiles = (nn + kScanTile - 1) / kScanTile;
  int32_t *cnt = scratch, *fill = scratch + nn, *tsum = scratch + 2 * nn;
  cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(int32_t) * 2 * nn, st);
  if (e != cudaSuccess) return e;
  k_count<<<grid_for(ent), kThreads, 0, st>>>(el_aos, ent, cnt);
  k_tile_sums<<<(unsigned)ntiles, kThreads, 0, st>>>(cnt, nn, tsum);
  k_scan_tile_sums<<<1, kThreads, 0, st>>>(tsum, ntiles);
  k_tile_offsets<<<(unsigned)ntiles, kThreads, 0, st>>>(cnt, nn, tsum, off);
  k_place<<<grid_for(ent), kThreads, 0, st>>>(el_aos, ent, off, fill, slot);
  k_sort_lists<<<grid_for(nn), kThreads, 0, st>>>(off, nn, slot);
  k_elnod_soa<<<grid_for(ent), kThreads, 0, st>>>(el_aos, ne, npe, el_soa);
  return cudaGetLastError();
}

void coords_soa(const double *x_aos, int64_t nn, int64_t np, double *out, cudaStream_t st) {
  k_coords_soa<<<grid_for(3 * np), kThreads, 0, st>>>(x_aos, nn, np, out);
}

void coords_aos(const double *soa, int64_t nn, int64_t np, double *out, cudaStream_t st) {
  k_coords_aos<<<grid_for(3 * nn), kThreads, 0, st>>>(soa, nn, np, out);
}

void fill_values(double *p, double v, int64_t n, cudaStream_t st) {
  k_fill<<<grid_for(n), kThreads, 0, st>>>(p, v, n);
}

void initial_yield(const StepParams &P, double *sy, cudaStream_t st) {
  k_initial_yield<<<grid_for(P.ne), kThreads, 0, st>>>(P.mats, P.emat, P.ne, sy);
}

void initial_velocity(const StepParams &P, double *v, cudaStream_t st) {
  k_initial_velocity<<<grid_for(3 * P.np), kThreads, 0, st>>>(P.bc, P.bcval, P.nn, P.np, v);
}

}  // namespace wf
