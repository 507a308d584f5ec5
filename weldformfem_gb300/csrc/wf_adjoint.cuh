// Internal declarations of the reverse (adjoint) pass of the FP64 step.
#pragma once

#include "wf_internal.cuh"

namespace wf {

// Device buffers of the reverse pass. Stash arrays hold the start-of-step
// state of every step of the segment being reversed (slot = step - first
// step of the segment); the adjoint state is the derivative of the loss with
// respect to the state at the start of the step being reversed.
struct AdjArgs {
  // stash of the current segment
  double *sx, *sv, *spa;    // [seg][3][np] position, corrected velocity, prev accel
  double *sjr, *smass;      // [seg][np]    volume ratio and lumped mass of the step
  double *sfi;              // [seg][3][np] assembled internal force of the step
  double *stau;             // [seg][6][ne] Jaumann stress
  double *spls;             // [seg][ne]    equivalent plastic strain
  // adjoint state
  double *X, *V, *PA;       // [3][np]
  double *T;                // [6][ne]
  double *EP;               // [ne]
  // per-step scratch
  double *fib, *vpb;        // [3][np] adjoint of internal force / predicted velocity
  double *mb, *sb;          // [np]    adjoint of lumped mass / nodal volume sum
  double *inv_s0, *dmds;    // [np]    1 / s0 and d(mass)/d(volume sum)
  double *cx, *cv, *cgeo;   // [npe][3][ne] per element-node contributions
  double *cj, *volb;        // [ne]
  double *gth;              // [3][ne] per-element dL/d(E, sigma_y0, H), summed over steps
  // inputs
  const double *seed;       // [nsteps] dL/dR of each recorded step
  const double *s0;         // [np] sum of the initial element volumes at the node
  const double *rho;        // [ne] element density (constant during the run)
};

void adj_node_constants(const StepParams &P, const AdjArgs &A, cudaStream_t st);
void adj_stash_state(const StepParams &P, const Fp64State &S, const AdjArgs &A, int slot,
                     cudaStream_t st);
void adj_stash_step(const StepParams &P, const Fp64State &S, const AdjArgs &A, int slot,
                    cudaStream_t st);
// One reverse step: node, element, gather and volume kernels.
void adj_reverse_step(const StepParams &P, const AdjArgs &A, int slot, long long seed_index,
                      int have_geo, bool fp32, cudaStream_t st);

}  // namespace wf
