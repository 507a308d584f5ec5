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
#include <cmath>
#include <cstdint>

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

// ---- element tiles ------------------------------------------------------------

// Bin of each element: its centroid's cube of side 1 / inv_h from (x0, y0, z0).
__global__ void k_tile_bin(const int32_t *el, const double *x, int64_t np, int64_t ne, int npe,
                           double x0, double y0, double z0, double inv_h, int nbx, int nby,
                           int nbz, int32_t *key) {
  GRID_STRIDE(e, ne) {
    double c[3] = {0.0, 0.0, 0.0};
    for (int a = 0; a < npe; a++) {
      const int32_t n = el[a * ne + e];
      for (int k = 0; k < 3; k++) c[k] += x[k * np + n];
    }
    const double o[3] = {x0, y0, z0};
    const int nb[3] = {nbx, nby, nbz};
    int ib[3];
    for (int k = 0; k < 3; k++) {
      const double f = floor((c[k] / npe - o[k]) * inv_h);
      ib[k] = f < 0.0 ? 0 : (f >= (double)nb[k] ? nb[k] - 1 : (int)f);
    }
    key[e] = (ib[2] * nby + ib[1]) * nbx + ib[0];
  }
}

// In-place ascending bitonic sort of buf[0, p2) (p2 a power of two) by the
// block's threads.
template <int THREADS>
__device__ __forceinline__ void block_bitonic(int32_t *buf, int p2) {
  for (int k = 2; k <= p2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < p2; i += THREADS) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const int32_t a = buf[i], b = buf[ixj];
          const bool up = (i & k) == 0;
          if ((a > b) == up) {
            buf[i] = b;
            buf[ixj] = a;
          }
        }
      }
      __syncthreads();
    }
  }
}

// Sorts each bin's element list ascending (bins of at most kTileBinMax).
__global__ void __launch_bounds__(512) k_bin_sort(const int32_t *boff, int32_t *sorted) {
  __shared__ int32_t buf[kTileBinMax];
  const int32_t lo = boff[blockIdx.x], c = boff[blockIdx.x + 1] - lo;
  if (c <= 1) return;
  int p2 = 1;
  while (p2 < c) p2 <<= 1;
  for (int i = threadIdx.x; i < p2; i += 512) buf[i] = i < c ? sorted[lo + i] : INT32_MAX;
  __syncthreads();
  block_bitonic<512>(buf, p2);
  for (int i = threadIdx.x; i < c; i += 512) sorted[lo + i] = buf[i];
}

// Exclusive scan of one value per thread over a block of 512 threads.
__device__ __forceinline__ int32_t block_scan512(int32_t v, int32_t &total) {
  __shared__ int32_t warp[16];
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
    int32_t s = lane < 16 ? warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 16; o <<= 1) {
      const int32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < 16) warp[lane] = s;
  }
  __syncthreads();
  const int32_t before = (w > 0 ? warp[w - 1] : 0) + x - v;
  total = warp[15];
  __syncthreads();
  return before;
}

// One block per tile: the tile's distinct nodes (sorted), which of them are
// interior (all their elements in the tile), and each element corner's
// tile-local node index. err bit 0: a tile holds more than kTileNodes nodes;
// bit 1: two elements of a tile hold one node at the same corner.
__global__ void __launch_bounds__(512) k_tile_nodes(const int32_t *el, int64_t ne,
                                                    const int32_t *eoff, const int32_t *elems,
                                                    const int32_t *off, int32_t *nodes,
                                                    int32_t *ncount, uint16_t *lel,
                                                    int32_t *iflag, int32_t *err,
                                                    unsigned long long *islots) {
  __shared__ int32_t ids[8 * kTileElems];
  __shared__ int32_t uniq[kTileNodes];
  __shared__ int32_t start[kTileNodes + 1];
  __shared__ uint32_t used[8][kTileNodes / 32];
  const int t = blockIdx.x, tid = threadIdx.x;
  const int32_t e0 = eoff[t], c = eoff[t + 1] - e0;
  for (int i = tid; i < 8 * kTileElems; i += 512) {
    const int j = i >> 3, a = i & 7;
    ids[i] = j < c ? el[a * ne + elems[e0 + j]] : INT32_MAX;
  }
  for (int i = tid; i < 8 * (kTileNodes / 32); i += 512) (&used[0][0])[i] = 0u;
  __syncthreads();
  block_bitonic<512>(ids, 8 * kTileElems);
  // distinct values: thread tid looks at entries [8 tid, 8 tid + 8)
  int32_t u = 0;
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const int i = 8 * tid + q;
    u += (ids[i] != INT32_MAX && (i == 0 || ids[i] != ids[i - 1])) ? 1 : 0;
  }
  int32_t total = 0;
  int32_t pos = block_scan512(u, total);
  if (total > kTileNodes) {
    if (tid == 0) atomicOr(err, 1);
    return;   // block-uniform
  }
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const int i = 8 * tid + q;
    if (ids[i] != INT32_MAX && (i == 0 || ids[i] != ids[i - 1])) {
      uniq[pos] = ids[i];
      start[pos] = i;
      pos++;
    }
  }
  if (tid == 0) start[total] = 8 * c;
  __syncthreads();
  for (int q = tid; q < total; q += 512) {
    const int32_t id = uniq[q];
    const int32_t m = start[q + 1] - start[q];
    const bool interior = m == off[id + 1] - off[id];
    nodes[(int64_t)t * kTileNodes + q] = interior ? id : (int32_t)((uint32_t)id | 0x80000000u);
    if (interior) {
      iflag[id] = 1;
      atomicAdd(islots, (unsigned long long)m);
    }
  }
  if (tid == 0) ncount[t] = total;
  if (tid < c) {
    const int32_t e = elems[e0 + tid];
#pragma unroll
    for (int a = 0; a < 8; a++) {
      const int32_t id = el[a * ne + e];
      int lo = 0, hi = total - 1;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (uniq[mid] < id) lo = mid + 1;
        else hi = mid;
      }
      lel[a * ne + e0 + tid] = (uint16_t)lo;
      const uint32_t bit = 1u << (lo & 31);
      if (atomicOr(&used[a][lo >> 5], bit) & bit) atomicOr(err, 2);
    }
  }
}

// 1 for a node interior to no tile, 0 otherwise (in place).
__global__ void k_shared_flags(int32_t *f, int64_t nn) {
  GRID_STRIDE(n, nn) f[n] = f[n] ? 0 : 1;
}

__global__ void k_shared_scatter(const int32_t *f, const int32_t *soff, int64_t nn,
                                 int32_t *shared) {
  GRID_STRIDE(n, nn) if (f[n]) shared[soff[n]] = (int32_t)n;
}

// Flags elements whose corners differ from the AddBoxLength numbering.
__global__ void k_box_check(const int32_t *el, int64_t ne, int nx, int ny, int32_t *err) {
  GRID_STRIDE(e, ne) {
    const int64_t i = e % nx, j = (e / nx) % ny, k = e / ((int64_t)nx * ny);
    const int64_t px = nx + 1, pxy = (int64_t)(nx + 1) * (ny + 1);
    const int64_t n0 = i + px * j + pxy * k;
    const int64_t c[8] = {n0, n0 + 1, n0 + 1 + px, n0 + px,
                          n0 + pxy, n0 + 1 + pxy, n0 + 1 + px + pxy, n0 + px + pxy};
    bool ok = true;
    for (int a = 0; a < 8; a++) ok &= el[a * ne + e] == c[a];
    if (!ok) atomicOr(err, 1);
  }
}

}  // namespace

namespace {
__global__ void k_check_range(const int32_t *el, int64_t n, int64_t nn, int32_t *bad) {
  bool b = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t v = el[i];
    b |= (v < 0) | ((int64_t)v >= nn);
  }
  if (__any_sync(0xffffffffu, b) && (threadIdx.x & 31) == 0) atomicOr(bad, 1);
}
}  // namespace

namespace {
__global__ void k_scatter_u32(uint32_t *dst, const int32_t *idx, const uint32_t *val, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[idx[i]] = val[i];
}
__global__ void k_or_u8(uint8_t *dst, const int32_t *idx, uint8_t bit, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[idx[i]] |= bit;   // the lists hold each node once
}
}  // namespace

void scatter_u32(uint32_t *dst, const int32_t *idx, const uint32_t *val, int64_t n,
                 cudaStream_t st) {
  if (n > 0) k_scatter_u32<<<grid_for(n), kThreads, 0, st>>>(dst, idx, val, n);
}

void or_flags(uint8_t *dst, const int32_t *idx, uint8_t bit, int64_t n, cudaStream_t st) {
  if (n > 0) k_or_u8<<<grid_for(n), kThreads, 0, st>>>(dst, idx, bit, n);
}

cudaError_t check_connectivity(const int32_t *el, int64_t n, int64_t nn, int32_t *flag,
                               cudaStream_t st, int *bad) {
  *bad = 1;
  int32_t h = 1;
  cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int32_t), st);
  if (e != cudaSuccess) return e;
  const int64_t grid = std::min<int64_t>((n + kThreads - 1) / kThreads, 152 * 16);
  k_check_range<<<(unsigned)std::max<int64_t>(grid, 1), kThreads, 0, st>>>(el, n, nn, flag);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(&h, flag, sizeof(int32_t), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return e;
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
  *bad = h;
  return cudaSuccess;
}

cudaError_t check_box(const int32_t *el_soa, int64_t ne, int64_t nn, int nx, int ny, int nz,
                      cudaStream_t st, int *is_box) {
  *is_box = 0;
  if (nx <= 0 || ny <= 0 || nz <= 0 || (int64_t)nx * ny * nz != ne ||
      (int64_t)(nx + 1) * (ny + 1) * (nz + 1) != nn)
    return cudaSuccess;
  int32_t *err = nullptr;
  cudaError_t e = cudaMalloc(&err, sizeof(int32_t));
  if (e != cudaSuccess) return e;
  int32_t herr = 1;
  if ((e = cudaMemsetAsync(err, 0, sizeof(int32_t), st)) == cudaSuccess) {
    k_box_check<<<grid_for(ne), kThreads, 0, st>>>(el_soa, ne, nx, ny, err);
    if ((e = cudaMemcpyAsync(&herr, err, sizeof(int32_t), cudaMemcpyDeviceToHost, st)) ==
        cudaSuccess)
      e = cudaStreamSynchronize(st);
  }
  cudaFree(err);
  if (e == cudaSuccess && herr == 0) *is_box = 1;
  return e;
}

cudaError_t build_tiles(const int32_t *el_soa, const double *x_soa, int64_t np, int64_t ne,
                        int64_t nn, const int32_t *off, const double bbox[6], int shared_threads,
                        DeviceAlloc keep, void *keep_ctx, cudaStream_t st, TileParams &T,
                        std::string &why) {
  why.clear();
  T = TileParams{};
  if (ne <= 0 || nn <= 0) {
    why = "empty mesh";
    return cudaSuccess;
  }
  // cubes of about 8 element sizes, the element size from the bounding box
  double ext[3], vol = 1.0;
  for (int k = 0; k < 3; k++) {
    ext[k] = bbox[3 + k] - bbox[k];
    vol *= ext[k];
  }
  if (!(vol > 0.0) || !std::isfinite(vol)) {
    why = "degenerate bounding box";
    return cudaSuccess;
  }
  const double hb = 8.0 * std::cbrt(vol / (double)ne);
  int nb[3];
  double nbins_d = 1.0;
  for (int k = 0; k < 3; k++) {
    nb[k] = std::max(1, (int)std::ceil(ext[k] / hb));
    nbins_d *= nb[k];
  }
  if (nbins_d > (double)(1 << 24)) {
    why = "too many bins";
    return cudaSuccess;
  }
  const int64_t nbins = (int64_t)nbins_d;
  // temporaries: bin keys, bin counts and fills, scan scratch, flags
  const int64_t nscan = (nn + kScanTile - 1) / kScanTile;
  const size_t n_tmp =
      (size_t)ne + 2 * (size_t)nbins + 2 * (size_t)nn + 1 + (size_t)nscan + 1 + 3;
  int32_t *tmp = nullptr;
  cudaError_t e = cudaMalloc(&tmp, sizeof(int32_t) * n_tmp);
  if (e != cudaSuccess) return e;
  int32_t *key = tmp, *cnt = key + ne, *fill = cnt + nbins, *flag = fill + nbins;
  int32_t *soff = flag + nn, *tsum = soff + nn + 1, *err = tsum + nscan;
  // interior-node list entries (8-byte aligned slot after err)
  unsigned long long *islots = reinterpret_cast<unsigned long long *>(
      reinterpret_cast<uintptr_t>(err + 2) & ~uintptr_t(7));
  auto done = [&](cudaError_t r) {
    cudaStreamSynchronize(st);
    cudaFree(tmp);
    return r;
  };
  if ((e = cudaMemsetAsync(cnt, 0, sizeof(int32_t) * 2 * nbins, st)) != cudaSuccess) return done(e);
  if ((e = cudaMemsetAsync(flag, 0, sizeof(int32_t) * nn, st)) != cudaSuccess) return done(e);
  if ((e = cudaMemsetAsync(err, 0, sizeof(int32_t) * 4, st)) != cudaSuccess) return done(e);
  k_tile_bin<<<grid_for(ne), kThreads, 0, st>>>(el_soa, x_soa, np, ne, 8, bbox[0], bbox[1],
                                                bbox[2], 1.0 / hb, nb[0], nb[1], nb[2], key);
  k_count<<<grid_for(ne), kThreads, 0, st>>>(key, ne, cnt);
  // bin offsets and tile boundaries on the host (one small copy)
  std::vector<int32_t> hc(nbins);
  if ((e = cudaMemcpyAsync(hc.data(), cnt, sizeof(int32_t) * nbins, cudaMemcpyDeviceToHost,
                           st)) != cudaSuccess)
    return done(e);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return done(e);
  std::vector<int32_t> boff(nbins + 1), eoff;
  eoff.reserve(ne / kTileElems + nbins + 1);
  int32_t run = 0;
  for (int64_t b = 0; b < nbins; b++) {
    boff[b] = run;
    if (hc[b] > kTileBinMax) {
      why = "a bin holds more than 4096 elements";
      return done(cudaSuccess);
    }
    for (int32_t i = 0; i < hc[b]; i += kTileElems) eoff.push_back(run + i);
    run += hc[b];
  }
  boff[nbins] = run;
  eoff.push_back(run);
  const int32_t ntiles = (int32_t)eoff.size() - 1;
  // device tables kept with the domain
  int32_t *d_boff = nullptr, *d_eoff = nullptr, *elems = nullptr, *nodes = nullptr;
  int32_t *ncount = nullptr;
  uint16_t *lel = nullptr;
  auto kp = [&](void **p, size_t bytes) { return keep(keep_ctx, p, bytes); };
  if ((e = kp((void **)&d_eoff, sizeof(int32_t) * (ntiles + 1))) != cudaSuccess ||
      (e = kp((void **)&elems, sizeof(int32_t) * ne)) != cudaSuccess ||
      (e = kp((void **)&lel, sizeof(uint16_t) * 8 * ne)) != cudaSuccess ||
      (e = kp((void **)&ncount, sizeof(int32_t) * ntiles)) != cudaSuccess ||
      (e = kp((void **)&nodes, sizeof(int32_t) * (size_t)ntiles * kTileNodes)) != cudaSuccess)
    return done(e);
  // the bin offsets live in the (now unused) fill array's place after placement
  if ((e = cudaMalloc(&d_boff, sizeof(int32_t) * (nbins + 1))) != cudaSuccess) return done(e);
  auto done2 = [&](cudaError_t r) {
    cudaStreamSynchronize(st);
    cudaFree(d_boff);
    return done(r);
  };
  if ((e = cudaMemcpyAsync(d_boff, boff.data(), sizeof(int32_t) * (nbins + 1),
                           cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(d_eoff, eoff.data(), sizeof(int32_t) * (ntiles + 1),
                           cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return done2(e);
  k_place<<<grid_for(ne), kThreads, 0, st>>>(key, ne, d_boff, fill, elems);
  k_bin_sort<<<(unsigned)nbins, 512, 0, st>>>(d_boff, elems);
  k_tile_nodes<<<(unsigned)ntiles, 512, 0, st>>>(el_soa, ne, d_eoff, elems, off, nodes, ncount,
                                                 lel, flag, err, islots);
  int32_t herr = 0;
  unsigned long long hislots = 0;
  std::vector<int32_t> hnc(ntiles);
  if ((e = cudaMemcpyAsync(&herr, err, sizeof(int32_t), cudaMemcpyDeviceToHost, st)) !=
          cudaSuccess ||
      (e = cudaMemcpyAsync(&hislots, islots, sizeof(hislots), cudaMemcpyDeviceToHost, st)) !=
          cudaSuccess ||
      (e = cudaMemcpyAsync(hnc.data(), ncount, sizeof(int32_t) * ntiles, cudaMemcpyDeviceToHost,
                           st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return done2(e);
  if (herr & 1) {
    why = "a tile holds more than 1024 nodes";
    return done2(cudaSuccess);
  }
  if (herr & 2) {
    why = "two elements of a tile hold one node at the same corner";
    return done2(cudaSuccess);
  }
  // the shared nodes, ascending: flags -> offsets -> scatter
  k_shared_flags<<<grid_for(nn), kThreads, 0, st>>>(flag, nn);
  k_tile_sums<<<(unsigned)nscan, kThreads, 0, st>>>(flag, nn, tsum);
  k_scan_tile_sums<<<1, kThreads, 0, st>>>(tsum, nscan);
  k_tile_offsets<<<(unsigned)nscan, kThreads, 0, st>>>(flag, nn, tsum, soff);
  int32_t nshared = 0;
  if ((e = cudaMemcpyAsync(&nshared, soff + nn, sizeof(int32_t), cudaMemcpyDeviceToHost, st)) !=
          cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return done2(e);
  int32_t *shared = nullptr;
  double *partials = nullptr;
  const int64_t sgrid = std::max<int64_t>(1, (nshared + shared_threads - 1) / shared_threads);
  if ((e = kp((void **)&shared, sizeof(int32_t) * std::max(nshared, 1))) != cudaSuccess ||
      (e = kp((void **)&partials, sizeof(double) * (ntiles + sgrid))) != cudaSuccess)
    return done2(e);
  k_shared_scatter<<<grid_for(nn), kThreads, 0, st>>>(flag, soff, nn, shared);
  if ((e = cudaGetLastError()) != cudaSuccess) return done2(e);
  T.ntiles = ntiles;
  T.nshared = nshared;
  T.eoff = d_eoff;
  T.elems = elems;
  T.lel = lel;
  T.ncount = ncount;
  T.nodes = nodes;
  T.shared = shared;
  T.partials = partials;
  T.tile_nodes = 0;
  for (int32_t c : hnc) T.tile_nodes += c;
  T.shared_slots = 8 * ne - (int64_t)hislots;
  return done2(cudaSuccess);
}

int64_t connectivity_scratch_ints(int64_t nn) {
  return 2 * nn + (nn + kScanTile - 1) / kScanTile + 1;
}

cudaError_t build_connectivity(const int32_t *el_aos, int64_t ne, int npe, int64_t nn,
                               int32_t *el_soa, int32_t *off, int32_t *slot, int32_t *scratch,
                               cudaStream_t st) {
  const int64_t ent = ne * npe;
  if (el_soa) k_elnod_soa<<<grid_for(ent), kThreads, 0, st>>>(el_aos, ne, npe, el_soa);
  if (!off) return cudaGetLastError();
  const int64_t ntiles = (nn + kScanTile - 1) / kScanTile;
  int32_t *cnt = scratch, *fill = scratch + nn, *tsum = scratch + 2 * nn;
  cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(int32_t) * 2 * nn, st);
  if (e != cudaSuccess) return e;
  k_count<<<grid_for(ent), kThreads, 0, st>>>(el_aos, ent, cnt);
  k_tile_sums<<<(unsigned)ntiles, kThreads, 0, st>>>(cnt, nn, tsum);
  k_scan_tile_sums<<<1, kThreads, 0, st>>>(tsum, ntiles);
  k_tile_offsets<<<(unsigned)ntiles, kThreads, 0, st>>>(cnt, nn, tsum, off);
  k_place<<<grid_for(ent), kThreads, 0, st>>>(el_aos, ent, off, fill, slot);
  k_sort_lists<<<grid_for(nn), kThreads, 0, st>>>(off, nn, slot);
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
