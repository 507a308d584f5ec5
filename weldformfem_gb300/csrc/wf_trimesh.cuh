// Motion of the rigid triangle-mesh bodies, shared by both precisions.
#pragma once

#include "wf_internal.cuh"

namespace wf {

// End of the loop body (Solver_explicit.C:980-1004), run by one block once
// every node of the step has been updated: the die velocity ramps as
// sqrt(Time / (0.01 end_t)) over the first 1 % of the end time, the mesh moves
// by v dt, and normals and plane coefficients are recomputed (far node 2).
// F32 also refreshes the FP32 copies the mixed-precision contact reads: node
// positions relative to P.tri_ref, normals, and plane coefficients relative
// to P.tri_ref.
template <bool F32>
__device__ void tri_move(const StepParams &P, double time) {
  const double rf = 1.0e-2;
  double f = 1.0;
  if (time < rf * P.end_t) f = pow(time / (rf * P.end_t), 0.5);
  for (int32_t i = threadIdx.x; i < 3 * P.tri_nn; i += blockDim.x) {
    const double vk = f * P.tri_v[i];
    P.tri_x[i] = P.tri_x[i] + vk * P.dt;
    if constexpr (F32) P.tri_xf[i] = (float)(P.tri_x[i] - P.tri_ref[i % 3]);
  }
  __syncthreads();
  for (int32_t e = threadIdx.x; e < P.tri_ne; e += blockDim.x) {
    const double *p0 = &P.tri_x[3 * P.tri_el[3 * e]];
    const double *p1 = &P.tri_x[3 * P.tri_el[3 * e + 1]];
    const double *p2 = &P.tri_x[3 * P.tri_el[3 * e + 2]];
    const double u[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    const double w0[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
    const double w[3] = {u[1] * w0[2] - u[2] * w0[1], u[2] * w0[0] - u[0] * w0[2],
                         u[0] * w0[1] - u[1] * w0[0]};
    const double len = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    const double inv = 1.0 / len;
    const double nn0 = w[0] * inv, nn1 = w[1] * inv, nn2 = w[2] * inv;
    P.tri_nrm[3 * e] = nn0;
    P.tri_nrm[3 * e + 1] = nn1;
    P.tri_nrm[3 * e + 2] = nn2;
    P.tri_pp[e] = p2[0] * nn0 + p2[1] * nn1 + p2[2] * nn2;
    if constexpr (F32) {
      P.tri_nf[3 * e] = (float)nn0;
      P.tri_nf[3 * e + 1] = (float)nn1;
      P.tri_nf[3 * e + 2] = (float)nn2;
      P.tri_ppf[e] = (float)((p2[0] - P.tri_ref[0]) * nn0 + (p2[1] - P.tri_ref[1]) * nn1 +
                             (p2[2] - P.tri_ref[2]) * nn2);
    }
  }
}

}  // namespace wf
