// Device reductions: minimum element edge length (CFL time-step rule).
#include <algorithm>
#include <cstring>

#include "wf_internal.cuh"

namespace wf {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ double edge_len(const double *x, int64_t np, int32_t a, int32_t b) {
  const double dx = x[b] - x[a], dy = x[np + b] - x[np + a], dz = x[2 * np + b] - x[2 * np + a];
  return sqrt(dx * dx + dy * dy + dz * dz);
}

// Shortest element edge (hexahedron: 12 edges, tetrahedron: 6), reduced with
// an order-free min so the result does not depend on the launch shape. The
// value is positive, so its bit pattern orders like an unsigned integer.
__global__ void k_min_edge(const int32_t *elnod, const double *x, int64_t np, int64_t ne,
                           int npe, unsigned long long *out) {
  __shared__ double sh[kThreads / 32];
  double best = 1.0e300;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ne;
       e += (int64_t)gridDim.x * blockDim.x) {
    int32_t n[8];
    for (int a = 0; a < npe; a++) n[a] = elnod[a * ne + e];
    if (npe == 8) {
      const int E[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                            {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
      for (int k = 0; k < 12; k++) best = fmin(best, edge_len(x, np, n[E[k][0]], n[E[k][1]]));
    } else {
      const int E[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
      for (int k = 0; k < 6; k++) best = fmin(best, edge_len(x, np, n[E[k][0]], n[E[k][1]]));
    }
  }
  for (int o = 16; o > 0; o >>= 1) best = fmin(best, __shfl_down_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = best;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < kThreads / 32; i++) best = fmin(best, sh[i]);
    atomicMin(out, (unsigned long long)__double_as_longlong(best));
  }
}

__global__ void k_set(unsigned long long *p, unsigned long long v) { *p = v; }

// One block per specimen: sum of its reaction nodes' contributions in list
// order (each thread a fixed strided subset, then a fixed tree).
__global__ void k_spec_reaction(StepParams P) {
  __shared__ double sh[4];
  const int s = blockIdx.x;
  const int32_t b = P.rl_off[s], e = P.rl_off[s + 1];
  double t = 0.0;
  for (int32_t i = b + threadIdx.x; i < e; i += blockDim.x) t += P.rnode[P.rlist[i]];
  for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += sh[w];
    const long long step = P.st->step - 1;  // advanced by this step's node kernel
    if (step >= 0 && step < P.hist_cap) P.hist_spec[step * P.nspec + s] = tot;
  }
}

}  // namespace

void spec_reaction(const StepParams &P, cudaStream_t st) {
  k_spec_reaction<<<P.nspec, 128, 0, st>>>(P);
}

void min_edge_length(const int32_t *elnod, const double *x, int64_t np, int64_t ne, int npe,
                     double *out_dev, cudaStream_t st) {
  unsigned long long *o = reinterpret_cast<unsigned long long *>(out_dev);
  const double big = 1.0e300;
  unsigned long long bits;
  std::memcpy(&bits, &big, sizeof(bits));
  k_set<<<1, 1, 0, st>>>(o, bits);
  int grid = (int)std::min<int64_t>((ne + kThreads - 1) / kThreads, 152 * 8);
  k_min_edge<<<grid, kThreads, 0, st>>>(elnod, x, np, ne, npe, o);
}

}  // namespace wf
