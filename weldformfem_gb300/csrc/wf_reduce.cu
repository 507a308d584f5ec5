// Device reductions: minimum element edge length (CFL time-step rule),
// per-specimen reaction sums and the energy history.
#include <algorithm>
#include <cstring>

#include "wf_internal.cuh"

namespace wf {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ double edge_len2(const double *x, int64_t np, int64_t a, int64_t b) {
  const double dx = x[b] - x[a], dy = x[np + b] - x[np + a], dz = x[2 * np + b] - x[2 * np + a];
  return dx * dx + dy * dy + dz * dz;
}
__device__ __forceinline__ double edge_len(const double *x, int64_t np, int32_t a, int32_t b) {
  return sqrt(edge_len2(x, np, a, b));
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

// Box meshes: every element edge joins a node to its +x, +y or +z neighbour,
// so the shortest edge is the shortest of those grid edges, each taken once
// (a quarter of the element edges). The squared lengths are the element
// kernel's (a reversed edge negates the differences exactly), and sqrt is
// correctly rounded and monotone, so the minimum of the squares' root is the
// element kernel's minimum bit for bit.
__global__ void k_min_edge_box(const double *x, int64_t np, int32_t bx, int32_t by, int32_t bz,
                               unsigned long long *out) {
  __shared__ double sh[kThreads / 32];
  const int64_t nx1 = bx + 1, nxy = nx1 * (by + 1), nn = nxy * (bz + 1);
  double best2 = 1.0e300;
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < nn;
       n += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = n / nxy, r = n - k * nxy, j = r / nx1, i = r - j * nx1;
    if (i < bx) best2 = fmin(best2, edge_len2(x, np, n, n + 1));
    if (j < by) best2 = fmin(best2, edge_len2(x, np, n, n + nx1));
    if (k < bz) best2 = fmin(best2, edge_len2(x, np, n, n + nxy));
  }
  double best = sqrt(best2);
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

// Fixed-order block sum of doubles (shuffle tree per warp, warps in index
// order); valid in thread 0. Callers separate two calls with __syncthreads.
__device__ __forceinline__ double block_sum(double v, double *sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
  return t;
}

// Domain_d::computeEnergies (Mechanical.C:2145-2185) at the end of the step
// (Solver_explicit.C:1029-1031): Ekin = sum_n m_n |v_n|^2 / 2 and
// dEint = dt * sum_e (sigma_e . str_rate_e) vol_e over the six stored Voigt
// components, Eint += dEint. Block partials, then the last block to finish
// sums them in block order: deterministic.
template <class Item>
__device__ __forceinline__ void energy_reduce(const StepParams &P, Item item) {
  __shared__ double sh[kThreads / 32];
  __shared__ bool am_last;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double k = 0.0, w = 0.0;
  item(i, k, w);
  const double kb = block_sum(k, sh);
  __syncthreads();
  const double wb = block_sum(w, sh);
  if (threadIdx.x == 0) {
    P.epart[2 * blockIdx.x] = kb;
    P.epart[2 * blockIdx.x + 1] = wb;
    __threadfence();
    am_last = atomicAdd(&P.st->energy_blocks, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (am_last) {
    __threadfence();
    double tk = 0.0, tw = 0.0;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
      tk += ((volatile double *)P.epart)[2 * b];
      tw += ((volatile double *)P.epart)[2 * b + 1];
    }
    const double K = block_sum(tk, sh);
    __syncthreads();
    const double Wt = block_sum(tw, sh);
    if (threadIdx.x == 0) {
      const long long s = P.st->step - 1;  // advanced by this step's node kernel
      const double eint = P.st->eint + Wt * P.dt;
      P.st->eint = eint;
      if (s >= 0 && s < P.hist_cap) {
        P.ekin_hist[s] = K;
        P.eint_hist[s] = eint;
      }
      P.st->energy_blocks = 0u;
    }
  }
}

__global__ void __launch_bounds__(kThreads) k_energy_fp64(StepParams P, Fp64State S) {
  energy_reduce(P, [&](int64_t i, double &k, double &w) {
    if (i < P.nn) {
      const double vx = S.v[i], vy = S.v[P.np + i], vz = S.v[2 * P.np + i];
      k = 0.5 * S.mass[i] * (vx * vx + vy * vy + vz * vz);
    }
    if (i < P.ne) {
      const int64_t ne = P.ne;
      double sdot = 0.0;
      for (int c = 0; c < 6; c++) sdot += S.sig[c * ne + i] * S.sr[c * ne + i];
      w = sdot * S.vol[i];
    }
  });
}

__global__ void __launch_bounds__(kThreads) k_energy_mixed(StepParams P, MixState M) {
  energy_reduce(P, [&](int64_t i, double &k, double &w) {
    if (i < P.nn) {
      const double vx = M.v[i], vy = M.v[P.np + i], vz = M.v[2 * P.np + i];
      k = 0.5 * (double)M.mass[i] * (vx * vx + vy * vy + vz * vz);
    }
    if (i < P.ne) w = (double)M.edot[i];
  });
}

}  // namespace

int energy_grid(const StepParams &P) {
  return (int)((std::max(P.nn, P.ne) + kThreads - 1) / kThreads);
}

void energy_fp64(const StepParams &P, const Fp64State &S, cudaStream_t st) {
  k_energy_fp64<<<energy_grid(P), kThreads, 0, st>>>(P, S);
}

void energy_mixed(const StepParams &P, const MixState &M, cudaStream_t st) {
  k_energy_mixed<<<energy_grid(P), kThreads, 0, st>>>(P, M);
}

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

void min_edge_length_box(const double *x, int64_t np, int32_t bx, int32_t by, int32_t bz,
                         double *out_dev, cudaStream_t st) {
  unsigned long long *o = reinterpret_cast<unsigned long long *>(out_dev);
  const double big = 1.0e300;
  unsigned long long bits;
  std::memcpy(&bits, &big, sizeof(bits));
  k_set<<<1, 1, 0, st>>>(o, bits);
  const int64_t nn = (int64_t)(bx + 1) * (by + 1) * (bz + 1);
  int grid = (int)std::min<int64_t>((nn + kThreads - 1) / kThreads, 152 * 8);
  k_min_edge_box<<<grid, kThreads, 0, st>>>(x, np, bx, by, bz, o);
}

}  // namespace wf
