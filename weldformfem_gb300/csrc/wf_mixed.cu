// Mixed-precision step kernels: FP32 element and node arithmetic, positions
// as compensated float pairs, reaction sums in FP64.
//
// Same four phases and the same formulas as the FP64 kernels (wf_fp64.cu),
// including the reference's Jaumann-term tensor product, with these changes:
//  * element geometry uses coordinates relative to the element's first node,
//    formed from (hi, lo) float pairs, so no FP64 instruction is issued;
//  * for hexahedra, the Jacobian, the velocity gradient, the hourglass modes
//    and the nodal forces go through a Walsh transform of the nodal values
//    (the same quantities as the reference's per-node loops, in 24 additions
//    per component instead of a loop over nodes and derivatives);
//  * the element force written for assembly is f_elem - f_hourglass;
//  * the lumped mass is voln * (mean density of the node's elements), the
//    same quantity as the reference's sum of rho_e * voln / count;
//  * with default options the pressure is -K (J_avg - 1) (pressure
//    algorithm 0 with zero stabilisation, as the reference defaults);
//  * displacements are x - x0 (exported in FP64), total strain is not kept.
#include <map>
#include <mutex>
#include <utility>

#include "wf_internal.cuh"
#include "wf_trimesh.cuh"

namespace wf {
namespace {

constexpr int kElemThreads = 128;
constexpr int kNodeThreads = 256;
// Resident blocks per SM the node kernel is compiled for (registers per
// thread = 65536 / (256 * this)); a build-time tunable.
#ifndef WF_NODE_MIN_BLOCKS
#define WF_NODE_MIN_BLOCKS 6
#endif

// (hi, lo) pair helpers ------------------------------------------------------
__device__ __forceinline__ float2 split_d(double v) {
  const float hi = (float)v;
  return make_float2(hi, (float)(v - (double)hi));
}
// Height of the rigid plane z0 + vz t (FP64) as a (hi, lo) pair.
__device__ __forceinline__ float2 die_height(const StepParams &P, double time) {
  return split_d(P.c_z0 + P.c_vz * time);
}

// (hi, lo) + b with TwoSum and renormalisation (Knuth / Dekker).
__device__ __forceinline__ float2 pair_add(float2 a, float b) {
  const float s = __fadd_rn(a.x, b);
  const float bb = __fsub_rn(s, a.x);
  const float err = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  const float t = __fadd_rn(err, a.y);
  const float hi = __fadd_rn(s, t);
  const float lo = __fsub_rn(t, __fsub_rn(hi, s));
  return make_float2(hi, lo);
}
// a - b for nearby points: hi parts subtract exactly when within a factor 2.
__device__ __forceinline__ float pair_rel(float2 a, float2 b) {
  return __fadd_rn(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y));
}

// Loads of data that other threads write during the run: through the
// read-only path (__ldg) in the per-phase kernels, where it is constant for
// the launch, and through L2 (__ldcg) in the persistent cluster kernel, whose
// phases share one launch.
template <bool CG, typename T>
__device__ __forceinline__ T ldx(const T *p) {
  if constexpr (CG)
    return __ldcg(p);
  else
    return __ldg(p);
}

// Box meshes (P.box): the corners of element e in the AddBoxLength numbering.
__device__ __forceinline__ void box_corners(const StepParams &P, int64_t e, int32_t (&nid)[8]) {
  const uint32_t ue = (uint32_t)e;
  const uint32_t k = fdiv(ue, P.fd_exy);
  const uint32_t r = ue - k * P.fd_exy.d;
  const uint32_t j = fdiv(r, P.fd_ex);
  const uint32_t i = r - j * P.fd_ex.d;
  const int32_t px = (int32_t)P.fd_nx.d, pxy = (int32_t)P.fd_nxy.d;
  const int32_t n0 = (int32_t)i + px * (int32_t)j + pxy * (int32_t)k;
  nid[0] = n0;
  nid[1] = n0 + 1;
  nid[2] = n0 + 1 + px;
  nid[3] = n0 + px;
  nid[4] = n0 + pxy;
  nid[5] = n0 + 1 + pxy;
  nid[6] = n0 + 1 + px + pxy;
  nid[7] = n0 + px + pxy;
}

template <int NPE>
__device__ __forceinline__ float weightf() {
  return NPE == 8 ? 8.0f : 1.0f / 6.0f;
}

template <int NPE, bool CG, bool BOX = false>
__device__ __forceinline__ void rel_coords(const StepParams &P, const MixState &M, int64_t e,
                                           float (&r)[NPE][3], int32_t (&nid)[NPE]) {
  if constexpr (BOX && NPE == 8) {
    box_corners(P, e, nid);
  } else {
#pragma unroll
    for (int a = 0; a < NPE; a++) nid[a] = __ldg(&P.elnod[a * P.ne + e]);
  }
  float2 o[3];
#pragma unroll
  for (int k = 0; k < 3; k++) o[k] = ldx<CG>(&M.xh[k * P.np + nid[0]]);
#pragma unroll
  for (int k = 0; k < 3; k++) r[0][k] = 0.0f;
#pragma unroll
  for (int a = 1; a < NPE; a++)
#pragma unroll
    for (int k = 0; k < 3; k++) r[a][k] = pair_rel(ldx<CG>(&M.xh[k * P.np + nid[a]]), o[k]);
}

template <int NPE>
__device__ __forceinline__ void jacobian_f(const float (&x2)[NPE][3], float J[3][3]) {
  if constexpr (NPE == 8) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      J[0][k] = 0.125f * (-x2[0][k] + x2[1][k] + x2[2][k] - x2[3][k] - x2[4][k] + x2[5][k] +
                          x2[6][k] - x2[7][k]);
      J[1][k] = 0.125f * (-x2[0][k] - x2[1][k] + x2[2][k] + x2[3][k] - x2[4][k] - x2[5][k] +
                          x2[6][k] + x2[7][k]);
      J[2][k] = 0.125f * (-x2[0][k] - x2[1][k] - x2[2][k] - x2[3][k] + x2[4][k] + x2[5][k] +
                          x2[6][k] + x2[7][k]);
    }
  } else {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      J[0][k] = x2[1][k] - x2[0][k];
      J[1][k] = x2[2][k] - x2[0][k];
      J[2][k] = x2[3][k] - x2[0][k];
    }
  }
}

__device__ __forceinline__ float det3f(const float J[3][3]) {
  return J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
         J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
}

template <int NPE>
__device__ __forceinline__ void shape_derivs_f(const float J[3][3], float dH[3][NPE]) {
  float inv[3][3];
  inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]);
  inv[1][0] = -(J[1][0] * J[2][2] - J[1][2] * J[2][0]);
  inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  inv[0][1] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]);
  inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]);
  inv[2][1] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]);
  inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]);
  inv[1][2] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]);
  inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]);
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float a0 = inv[k][0], a1 = inv[k][1], a2 = inv[k][2];
    if constexpr (NPE == 8) {
      dH[k][0] = 0.125f * (-a0 - a1 - a2);
      dH[k][1] = 0.125f * (a0 - a1 - a2);
      dH[k][2] = 0.125f * (a0 + a1 - a2);
      dH[k][3] = 0.125f * (-a0 + a1 - a2);
      dH[k][4] = 0.125f * (-a0 - a1 + a2);
      dH[k][5] = 0.125f * (a0 - a1 + a2);
      dH[k][6] = 0.125f * (a0 + a1 + a2);
      dH[k][7] = 0.125f * (-a0 + a1 + a2);
    } else {
      dH[k][0] = -a0 - a1 - a2;
      dH[k][1] = a0;
      dH[k][2] = a1;
      dH[k][3] = a2;
    }
  }
}

// ---------------------------------------------------------------------------
template <int NPE, bool CG, bool BOX = false>
__device__ __forceinline__ void geometry_one(const StepParams &P, const MixState &M, float *vol,
                                             int64_t e) {
  float r[NPE][3];
  int32_t nid[NPE];
  rel_coords<NPE, CG, BOX>(P, M, e, r, nid);
  float J[3][3];
  jacobian_f<NPE>(r, J);
  vol[e] = det3f(J) * weightf<NPE>();
}

// Launch shapes are chosen at run time by the autotuner (wf_api.cu): block
// size BS and a grid-stride loop (several elements per thread).
// Two elements per iteration when the grid strides (a persistent grid or
// several items per thread): both elements' coordinate gathers are issued
// before either's arithmetic, so twice the loads are in flight.
template <int NPE, int BS, bool BOX>
__global__ void __launch_bounds__(BS) k_mix_geometry(StepParams P, MixState M, float *vol) {
  const int64_t stride = (int64_t)gridDim.x * BS;
  int64_t e = (int64_t)blockIdx.x * BS + threadIdx.x;
  for (; e + stride < P.ne; e += 2 * stride) {
    float r0[NPE][3], r1[NPE][3];
    int32_t n0[NPE], n1[NPE];
    rel_coords<NPE, false, BOX>(P, M, e, r0, n0);
    rel_coords<NPE, false, BOX>(P, M, e + stride, r1, n1);
    float J0[3][3], J1[3][3];
    jacobian_f<NPE>(r0, J0);
    jacobian_f<NPE>(r1, J1);
    vol[e] = det3f(J0) * weightf<NPE>();
    vol[e + stride] = det3f(J1) * weightf<NPE>();
  }
  if (e < P.ne) geometry_one<NPE, false, BOX>(P, M, vol, e);
}

// Rigid triangle-mesh contact of one external node in FP32 (the FP64 step's
// CalcContactForces restatement, Contact.C:31-334): coordinates relative to
// P.tri_ref; the first triangle, in order, that the node penetrates with its
// projection inside gives the penalty normal force
// pf * min(E A / l, 0.2 m / dt^2) * d, 20 % critical damping and Coulomb
// friction from the accumulated slip. A node out of contact keeps its last
// contact force. The node's reaction share (normal-force magnitude, rigid
// body 0 only) goes to M.cfn.
template <bool CG>
__device__ __forceinline__ void tri_contact_mixed(const StepParams &P, const MixState &M,
                                                  int64_t n, float mass) {
  const int64_t np = P.np;
  float x[3], v[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float2 h = M.xh[k * np + n];
    x[k] = (float)(((double)h.x + (double)h.y) - P.tri_ref[k]);
    v[k] = M.vp[k * np + n];
  }
  float cfn = 0.f;
  for (int32_t j = 0; j < P.tri_ne; j++) {
    const float n0 = ldx<CG>(&P.tri_nf[3 * j]), n1 = ldx<CG>(&P.tri_nf[3 * j + 1]),
                n2 = ldx<CG>(&P.tri_nf[3 * j + 2]);
    const float dd = (n0 * x[0] + n1 * x[1] + n2 * x[2]) - ldx<CG>(&P.tri_ppf[j]);
    if (!(dd < 0.f)) continue;
    const float Q[3] = {x[0] - n0 * dd, x[1] - n1 * dd, x[2] - n2 * dd};
    bool inside = true;
    for (int l = 0; l < 3 && inside; l++) {
      const int nx = l + 1 > 2 ? 0 : l + 1;
      const int32_t ia = 3 * __ldg(&P.tri_el[3 * j + l]), ib = 3 * __ldg(&P.tri_el[3 * j + nx]);
      const float a0 = ldx<CG>(&P.tri_xf[ia]), a1 = ldx<CG>(&P.tri_xf[ia + 1]),
                  a2 = ldx<CG>(&P.tri_xf[ia + 2]);
      const float e1[3] = {ldx<CG>(&P.tri_xf[ib]) - a0, ldx<CG>(&P.tri_xf[ib + 1]) - a1,
                           ldx<CG>(&P.tri_xf[ib + 2]) - a2};
      const float e2[3] = {Q[0] - a0, Q[1] - a1, Q[2] - a2};
      const float crit = (e1[1] * e2[2] - e1[2] * e2[1]) * n0 +
                         (e1[2] * e2[0] - e1[0] * e2[2]) * n1 +
                         (e1[0] * e2[1] - e1[1] * e2[0]) * n2;
      if (crit < 0.f) inside = false;
    }
    if (!inside) continue;
    const float dt = P.f_dt;
    const float v_reln = v[0] * n0 + v[1] * n1 + v[2] * n2;
    const float kgeo = (float)(P.tri_E0 * P.node_area[n] / P.nodlen[n]);
    const float kmass = 0.2f * mass / (dt * dt);
    const float k = (kmass < kgeo) ? kmass : kgeo;
    const float ccrit = 2.0f * mass * sqrtf(k / mass);
    const float sc = -((float)P.tri_pf * k * dd + 0.2f * ccrit * v_reln);
    float cf[3] = {n0 * sc, n1 * sc, n2 * sc};
    const float cfn_j = sqrtf(cf[0] * cf[0] + cf[1] * cf[1] + cf[2] * cf[2]);
    // friction from the accumulated tangential slip
    const float vt[3] = {v[0] - n0 * v_reln, v[1] - n1 * v_reln, v[2] - n2 * v_reln};
    float ut[3];
#pragma unroll
    for (int q = 0; q < 3; q++) ut[q] = M.ut[q * np + n] + vt[q] * dt;
    const float ft[3] = {-k * ut[0], -k * ut[1], -k * ut[2]};
    const float ft_mag = sqrtf(ft[0] * ft[0] + ft[1] * ft[1] + ft[2] * ft[2]);
    const float fn_norm = fabsf(cf[0] * n0 + cf[1] * n1 + cf[2] * n2);
    float F[3] = {ft[0], ft[1], ft[2]};
    if (!(ft_mag <= (float)P.tri_mu_s * fn_norm)) {
      // sliding: dynamic friction along -v_t (none when v_t vanishes)
      const float vtn = sqrtf(vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2]);
      const float md = vtn > 0.f ? -((float)P.tri_mu_d * fn_norm) / vtn : 0.f;
#pragma unroll
      for (int q = 0; q < 3; q++) {
        F[q] = vt[q] * md;
        ut[q] = 0.f;
      }
    }
#pragma unroll
    for (int q = 0; q < 3; q++) {
      M.ut[q * np + n] = ut[q];
      M.cf[q * np + n] = cf[q] + F[q];
    }
    if (__ldg(&P.tri_mid[j]) == 0) cfn = cfn_j;
    // heat from the die (Contact.C:309), kept after the contact ends
    if (P.thermal)
      M.qc[n] = (float)(P.tri_hc * P.node_area[n]) * ((float)P.tri_Tdie - M.T[n].x);
    break;
  }
  M.cfn[n] = cfn;
}

// Nodal volumes -> J ratio and lumped mass; for contact candidates also the
// rigid-plane contact force (it needs only x, the predicted velocity and the
// step's mass, all final here, so it is computed before the element phase).
// Nodal phase of one node, in two parts: nodal_gather sums the volumes of the
// node's elements in list order (and loads its constants), nodal_rest forms
// the J ratio, the lumped mass and, for contact candidates, the contact force.
// zd: the rigid plane's height at the step's time as a (hi, lo) float pair,
// formed once per thread by the caller (die_height), so that the gap of a
// contact node takes no FP64 instruction.
template <int NPE, bool CG, bool BOX = false>
__device__ __forceinline__ void nodal_gather(const StepParams &P, const MixState &M,
                                             const float *vol, int64_t n, float &s, float2 &nc) {
  s = 0.0f;
  if constexpr (BOX && NPE == 8) {
    // the node's elements in list order, computed from its indices
    int32_t el[8], cor[8];
    box_node_list(P, n, el, cor);
    nc = __ldg(&M.nc[n]);
    float g[8];
#pragma unroll
    for (int j = 0; j < 8; j++) g[j] = (el[j] >= 0) ? ldx<CG>(&vol[el[j]]) : 0.0f;
#pragma unroll
    for (int j = 0; j < 8; j++)
      if (el[j] >= 0) s += g[j];
  } else {
    const int32_t b = __ldg(&P.off[n]), c = __ldg(&P.off[n + 1]) - b;
    nc = __ldg(&M.nc[n]);   // issued before the gather, used after it
    for (int32_t k0 = 0; k0 < c; k0 += 8) {
      int32_t sl[8];
#pragma unroll
      for (int j = 0; j < 8; j++) sl[j] = (k0 + j < c) ? __ldg(&P.slot[b + k0 + j]) : -1;
      float g[8];
#pragma unroll
      for (int j = 0; j < 8; j++) g[j] = (sl[j] >= 0) ? ldx<CG>(&vol[sl[j] / NPE]) : 0.0f;
#pragma unroll
      for (int j = 0; j < 8; j++) s += g[j];
    }
  }
}

// The rest of a node's nodal phase from its volume sum s and constants nc:
// J ratio, lumped mass, contact force.
template <int NPE, bool CG>
__device__ __forceinline__ void nodal_rest(const StepParams &P, const MixState &M, int64_t n,
                                           float s, float2 nc, float2 zd) {
  M.jr[n] = s * nc.x;
  float mass;
  if (P.mass_mode == 0) {
    mass = (s * (1.0f / NPE)) * nc.y;
    M.mass[n] = mass;
  } else {
    mass = M.mass[n];
  }
  if (P.tri_on) {
    if (P.nflag[n] & NF_CONTACT) tri_contact_mixed<CG>(P, M, n, mass);
  } else if (P.contact && (P.nflag[n] & NF_CONTACT)) {
    // rigid plane, outward normal (0, 0, -1), at z0 + vz * Time
    // (Domain_d::CalcContactForces, Contact.C:58-323, one plane)
    const int64_t np = P.np;
    const float2 xz = M.xh[2 * np + n];
    const float vp0 = M.vp[n], vp1 = M.vp[np + n], vp2 = M.vp[2 * np + n];
    // hi parts subtract exactly near contact (within a factor 2)
    const float gap = __fadd_rn(__fsub_rn(zd.x, xz.x), __fsub_rn(zd.y, xz.y));
    float cf0 = 0.f, cf1 = 0.f, cf2 = 0.f;
    if (gap < 0.f) {
      const float kmass = 0.2f * mass / (P.f_dt * P.f_dt);
      const float k = (kmass < P.f_c_k) ? kmass : P.f_c_k;
      const float ccrit = 2.0f * mass * sqrtf(k / mass);
      cf2 = k * gap + 0.2f * ccrit * (-vp2);
      float ut0 = M.ut[n] + vp0 * P.f_dt;
      float ut1 = M.ut[np + n] + vp1 * P.f_dt;
      float ftx = -k * ut0, fty = -k * ut1;
      const float ft_max = P.f_c_mu * fabsf(cf2);
      if (!(sqrtf(ftx * ftx + fty * fty) <= ft_max)) {
        const float vt = sqrtf(vp0 * vp0 + vp1 * vp1);
        if (vt > 0.f) {
          ftx = -ft_max * vp0 / vt;
          fty = -ft_max * vp1 / vt;
        } else {
          ftx = fty = 0.f;
        }
        ut0 = ut1 = 0.f;
      }
      M.ut[n] = ut0;
      M.ut[np + n] = ut1;
      cf0 = ftx;
      cf1 = fty;
    }
    M.cf[n] = cf0;
    M.cf[np + n] = cf1;
    M.cf[2 * np + n] = cf2;
  }
}

template <int NPE, bool CG, bool BOX = false>
__device__ __forceinline__ void nodal_one(const StepParams &P, const MixState &M,
                                          const float *vol, int64_t n, float2 zd) {
  float s;
  float2 nc;
  nodal_gather<NPE, CG, BOX>(P, M, vol, n, s, nc);
  nodal_rest<NPE, CG>(P, M, n, s, nc, zd);
}

// Two nodes per iteration when the grid strides: both nodes' volume gathers
// are in flight before either's rest.
template <int NPE, int BS, bool BOX>
__global__ void __launch_bounds__(BS) k_mix_nodal(StepParams P, MixState M, const float *vol) {
  // the die height once per block: FP64 runs at 1/64 of the FP32 rate, and
  // formed by every thread it kept the FP64 pipe two-thirds busy
  __shared__ float2 s_zd;
  if (threadIdx.x == 0) s_zd = P.contact ? die_height(P, P.st->time) : make_float2(0.f, 0.f);
  __syncthreads();
  const float2 zd = s_zd;
  const int64_t stride = (int64_t)gridDim.x * BS;
  int64_t n = (int64_t)blockIdx.x * BS + threadIdx.x;
  for (; n + stride < P.nn; n += 2 * stride) {
    float s0, s1;
    float2 c0, c1;
    nodal_gather<NPE, false, BOX>(P, M, vol, n, s0, c0);
    nodal_gather<NPE, false, BOX>(P, M, vol, n + stride, s1, c1);
    nodal_rest<NPE, false>(P, M, n, s0, c0, zd);
    nodal_rest<NPE, false>(P, M, n + stride, s1, c1, zd);
  }
  if (n < P.nn) nodal_one<NPE, false, BOX>(P, M, vol, n, zd);
}

// Jaumann rate + radial return, shared by both element types. The
// reference's tensor3 product (Tensor3.C:290-303) written out for a
// symmetric tau and the spin W (antisymmetric, zero diagonal): only the six
// stored components are formed, terms that multiply a zero of W are dropped.
// In: strain rate sr (xx yy zz xy yz xz), spin (w01, w12, w02), pressure p.
// Writes the new tau and eps_p; returns sigma = tau - p I in sg.
// LAW = 0: linear hardening only (the common case, fewer registers); LAW = 1:
// every material model.
// Element state (tau [6][ne], eps_p [ne]) in HBM, read and written in place
// (the mixed state's arrays, addressed from the kernel parameters).
struct StateInPlace {
  __device__ __forceinline__ void load(const StepParams &P, const MixState &M, int64_t e,
                                       float &t0, float &t1, float &t2, float &t3, float &t4,
                                       float &t5, float &p) const {
    const int64_t ne = P.ne;
    t0 = M.tau[e]; t1 = M.tau[ne + e]; t2 = M.tau[2 * ne + e];
    t3 = M.tau[3 * ne + e]; t4 = M.tau[4 * ne + e]; t5 = M.tau[5 * ne + e];
    p = M.pls[e];
  }
  __device__ __forceinline__ void store(const StepParams &P, const MixState &M, int64_t e,
                                        float t0, float t1, float t2, float t3, float t4,
                                        float t5, float p) const {
    const int64_t ne = P.ne;
    M.pls[e] = p;
    M.tau[e] = t0; M.tau[ne + e] = t1; M.tau[2 * ne + e] = t2;
    M.tau[3 * ne + e] = t3; M.tau[4 * ne + e] = t4; M.tau[5 * ne + e] = t5;
  }
  __device__ __forceinline__ bool owns() const { return true; }
};

// IO: where the element's tau and eps_p come from and go to (StateInPlace:
// HBM, read and written in place; StateSwept: loaded ahead by the column
// sweep, written to the other buffer of a pair, or not at all for a halo
// element).
// GMT law in FP32 (CalcGMTYieldStress and CalcGMTTangentModulus,
// Material.cuh:417-478) from its temperature-reduced constants
// A = C1 exp(C2 T), n = n1 T + n2, I = I1 T + I2, q = m1 T + m2: reduced on the
// host at the material's uniform temperature, or here from the element's
// temperature under thermal coupling. With e and r clamped to their ranges,
// sigma_y = A e^n exp(I / e) r^q and Et = A r^q e^(n - 2) (e n - I) exp(I / e).
// Returns (sigma_y at rate r, Et at rate rt). Not inlined: the law's
// temporaries stay out of the register budget of the element kernels.
struct GmtF {
  float A, n, I, q;
};
template <bool TH>
__device__ __forceinline__ GmtF gmt_consts(const MatF &m, float T) {
  if constexpr (TH) {
    T = clamp_range(T, m.g_Tmin, m.g_Tmax);
    return GmtF{m.g_C1 * expf(m.g_C2 * T), m.g_n1 * T + m.g_n2, m.g_I1 * T + m.g_I2,
                m.g_m1 * T + m.g_m2};
  } else {
    return GmtF{m.g_A, m.g_n, m.g_I, m.g_q};
  }
}
__device__ __noinline__ float2 gmt_law_f(GmtF g, float emin, float emax, float rmin, float rmax,
                                         float e, float r, float rt) {
  e = clamp_range(e, emin, emax);
  r = clamp_range(r, rmin, rmax);
  rt = clamp_range(rt, rmin, rmax);
  const float ex = expf(g.I / e);
  const float sy = g.A * powf(e, g.n) * ex * powf(r, g.q);
  const float et = g.A * powf(rt, g.q) * powf(e, g.n - 2.0f) * (e * g.n - g.I) * ex;
  return make_float2(sy, et);
}

template <int LAW, bool TH, class IO>
__device__ __forceinline__ void stress_update(const StepParams &P, const MixState &M, int64_t e,
                                              const IO &io,
                                              const MatF &m, const float (&sr)[6], float w01,
                                              float w12, float w02, float p, float jTh,
                                              float (&sg)[6], float &sdot, float &qpl) {
  const float dt = P.espec ? P.specf[P.espec[e]].dt : P.f_dt;
  float t0, t1, t2, t3, t4, t5, pls;
  io.load(P, M, e, t0, t1, t2, t3, t4, t5, pls);
  {
    // tau W^T                      W tau
    const float srt0 = t3 * w01 + t5 * w02, rs0 = w01 * t3 + w02 * t5;    // xx
    const float srt1 = t3 * w01 - t4 * w12, rs1 = w12 * t4 - w01 * t3;    // yy
    const float srt2 = t5 * w02 + t4 * w12, rs2 = -(w02 * t5 + w12 * t4); // zz
    const float srt3 = t0 * w01 - t5 * w12, rs3 = w01 * t1 + w02 * t4;    // xy
    const float srt4 = t3 * w02 + t1 * w12, rs4 = w12 * t2 - w01 * t5;    // yz
    const float srt5 = t0 * w02 + t3 * w12, rs5 = w01 * t4 + w02 * t2;    // xz
    const float c = (1.0f / 3.0f) * (sr[0] + sr[1] + sr[2]);
    const float g2 = 2.0f * m.G;
    t0 += ((sr[0] - c) * g2 + srt0 + rs0) * dt;
    t1 += ((sr[1] - c) * g2 + srt1 + rs1) * dt;
    t2 += ((sr[2] - c) * g2 + srt2 + rs2) * dt;
    t3 += (sr[3] * g2 + srt3 + rs3) * dt;
    t4 += (sr[4] * g2 + srt4 + rs4) * dt;
    t5 += (sr[5] * g2 + srt5 + rs5) * dt;
  }
  // deviatoric trial stress of sigma_trial = tau - p I
  const float c2 = (1.0f / 3.0f) * ((t0 - p) + (t1 - p) + (t2 - p));
  const float d0s = (t0 - p) - c2, d1s = (t1 - p) - c2, d2s = (t2 - p) - c2;
  const float J2 = 0.5f * (d0s * d0s + 2.0f * t3 * t3 + 2.0f * t5 * t5 + d1s * d1s +
                           2.0f * t4 * t4 + d2s * d2s);
  const float sig_trial = sqrtf(3.0f * J2);
  float sy;
  float eff = 0.f;
  float dep = 0.f;
  float et_gmt = 0.f;
  if (LAW == 0) {
    sy = m.sy0 + m.H * pls;
  } else if (m.model == WF_MAT_JOHNSON_COOK || m.model == WF_MAT_GMT) {
    eff = sqrtf(0.5f * ((sr[0] - sr[1]) * (sr[0] - sr[1]) + (sr[1] - sr[2]) * (sr[1] - sr[2]) +
                        (sr[2] - sr[0]) * (sr[2] - sr[0])) +
                3.0f * (sr[3] * sr[3] + sr[4] * sr[4] + sr[5] * sr[5]));
    if (m.model == WF_MAT_JOHNSON_COOK) {
      const float srate = (eff == 0.f) ? 1.e-5f : eff;
      sy = (m.sy0 + m.jc_B * powf(pls, m.jc_n)) * (1.0f + m.jc_C * logf(srate / m.jc_eps0)) *
           jTh;
    } else {
      const float2 yt = gmt_law_f(gmt_consts<TH>(m, jTh), m.g_emin, m.g_emax, m.g_rmin,
                                  m.g_rmax, pls, eff, (P.f_max_edot < eff) ? P.f_max_edot : eff);
      sy = yt.x;
      et_gmt = yt.y;
    }
  } else if (m.model == WF_MAT_HOLLOMON) {
    sy = (pls + m.eps0 > m.eps1) ? m.hol_K * powf(pls + m.eps0, m.hol_m) : m.sy0;
  } else {
    sy = m.sy0 + m.H * pls;
  }
  if (sy < sig_trial) {
    float H;
    if (LAW == 0) {
      H = m.H;
    } else if (m.model == WF_MAT_JOHNSON_COOK) {
      const float er = (P.f_max_edot < eff) ? P.f_max_edot : eff;
      H = (pls > 0.f) ? m.jc_n * m.jc_B * powf(pls, m.jc_n - 1.f) *
                            (1.0f + m.jc_C * logf(er / m.jc_eps0)) * jTh
                      : m.E * 0.1f;
    } else if (m.model == WF_MAT_GMT) {
      H = et_gmt;
    } else {
      H = (m.model == WF_MAT_HOLLOMON)
              ? ((pls + m.eps0 > m.eps1)
                     ? m.hol_K * m.hol_m * powf(pls + m.eps0, m.hol_m - 1.0f)
                     : 0.f)
              : m.H;
    }
    const float dgamma = (sig_trial - sy) / (3.0f * m.G + H);
    const float factor = 1.0f - (3.0f * m.G * dgamma) / sig_trial;
    t0 = d0s * factor; t1 = d1s * factor; t2 = d2s * factor;
    t3 *= factor; t4 *= factor; t5 *= factor;
    pls += dgamma;
    dep = dgamma;
  }
  io.store(P, M, e, t0, t1, t2, t3, t4, t5, pls);
  sg[0] = t0 - p; sg[1] = t1 - p; sg[2] = t2 - p;
  sg[3] = t3; sg[4] = t4; sg[5] = t5;
  // plastic heat m_plheatfraction sigma : (d eps_p / dt) (Mechanical.C:1783-1810)
  if (TH && dep > 0.f) {
    const float f = dep / sy;
    const float ixx = f * (sg[0] - 0.5f * (sg[1] + sg[2]));
    const float iyy = f * (sg[1] - 0.5f * (sg[0] + sg[2]));
    const float izz = f * (sg[2] - 0.5f * (sg[0] + sg[1]));
    const float ixy = 1.5f * f * sg[3], iyz = 1.5f * f * sg[4], ixz = 1.5f * f * sg[5];
    qpl = P.f_plheat * (sg[0] * ixx + 2.0f * sg[3] * ixy + 2.0f * sg[5] * ixz + sg[1] * iyy +
                        2.0f * sg[4] * iyz + sg[2] * izz) / dt;
  }
  // sigma . str_rate over the six stored components (energy history)
  if (P.energy_on)
    sdot = sg[0] * sr[0] + sg[1] * sr[1] + sg[2] * sr[2] + sg[3] * sr[3] + sg[4] * sr[4] +
           sg[5] * sr[5];
}

// Walsh transform over the corners of the hexahedron. Node a of the
// AddBoxLength numbering sits at (xi, eta, zeta) = signs of
// (-,-,-) (+,-,-) (+,+,-) (-,+,-) (-,-,+) (+,-,+) (+,+,+) (-,+,+).
// o = sums of v weighted by {1, xi, eta, zeta, eta zeta, xi zeta, xi eta,
// xi eta zeta}: the first four are the trilinear shape functions' derivative
// directions at the centre, the last four the Flanagan-Belytschko hourglass
// base vectors Gamma_0..3 (test_1el_3D.cpp:166-169). 24 additions.
__device__ __forceinline__ void walsh8(const float (&v)[8], float (&o)[8]) {
  const float a0 = v[1] + v[0], b0 = v[1] - v[0];  // along xi at (eta-, zeta-)
  const float a1 = v[2] + v[3], b1 = v[2] - v[3];  // (eta+, zeta-)
  const float a2 = v[5] + v[4], b2 = v[5] - v[4];  // (eta-, zeta+)
  const float a3 = v[6] + v[7], b3 = v[6] - v[7];  // (eta+, zeta+)
  const float c0 = a1 + a0, d0 = a1 - a0, e0 = b1 + b0, f0 = b1 - b0;  // along eta, zeta-
  const float c1 = a3 + a2, d1 = a3 - a2, e1 = b3 + b2, f1 = b3 - b2;  // zeta+
  o[0] = c1 + c0;
  o[3] = c1 - c0;
  o[2] = d1 + d0;
  o[4] = d1 - d0;
  o[1] = e1 + e0;
  o[5] = e1 - e0;
  o[6] = f1 + f0;
  o[7] = f1 - f0;
}

// Transpose of walsh8 with no constant term: the node values of
// sum_b o[b] phi_b for b = 1..7.
__device__ __forceinline__ void walsh8_synth(const float (&o)[8], float (&v)[8]) {
  const float c1 = o[3], c0 = -o[3];
  const float d1 = o[2] + o[4], d0 = o[2] - o[4];
  const float e1 = o[1] + o[5], e0 = o[1] - o[5];
  const float f1 = o[6] + o[7], f0 = o[6] - o[7];
  const float a1 = c0 + d0, a0 = c0 - d0, b1 = e0 + f0, b0 = e0 - f0;
  const float a3 = c1 + d1, a2 = c1 - d1, b3 = e1 + f1, b2 = e1 - f1;
  v[1] = a0 + b0; v[0] = a0 - b0;
  v[2] = a1 + b1; v[3] = a1 - b1;
  v[5] = a2 + b2; v[4] = a2 - b2;
  v[6] = a3 + b3; v[7] = a3 - b3;
}

// Thermal coupling, element side (the FP64 step's restatement of
// calcThermalExpansion and ThermalCalcs in FP32). Before the stress update:
// the strain rate's diagonal loses exp_T times the mean of the previous step's
// element-node rates read at the element's node ids, and a Johnson-Cook
// element's temperature factor uses the mean of its node temperatures.
template <int NPE, bool CG>
__device__ __forceinline__ void thermal_pre(const StepParams &P, const MixState &M,
                                            const MatF &m, const int32_t (&nid)[NPE],
                                            long long step, float (&sr)[6], float &jTh) {
  const float *prev = M.dte + ((step + 1) & 1) * P.ne * NPE;
  float g = 0.f, ts = 0.f;
#pragma unroll
  for (int a = 0; a < NPE; a++) {
    g += ldx<CG>(&prev[nid[a]]);
    ts += ldx<CG>(&M.T[nid[a]]).x;
  }
  const float c = m.exp_T * (g * (1.0f / NPE));
  sr[0] -= c;
  sr[1] -= c;
  sr[2] -= c;
  if (m.model == WF_MAT_JOHNSON_COOK)
    jTh = 1.0f - powf((ts * (1.0f / NPE) - m.jc_Tt) / (m.jc_Tm - m.jc_Tt), m.jc_m);
  else if (m.model == WF_MAT_GMT)
    jTh = ts * (1.0f / NPE);
}

// After the forces: the element-node temperature rates -(K T)_a / m_a plus the
// plastic heat 0.9 q vol / n / (m_a cp_T), written to the step's buffer.
// KT holds (K T)_a / kf; qvol = q vol.
template <int NPE, bool CG>
__device__ __forceinline__ void thermal_rates(const StepParams &P, const MixState &M,
                                              const MatF &m, int64_t e,
                                              const int32_t (&nid)[NPE], long long step,
                                              const float (&KT)[NPE], float kf, float qvol) {
  float *cur = M.dte + (step & 1) * P.ne * NPE + e * NPE;
  const float ppn = 0.9f * qvol * (1.0f / NPE);
#pragma unroll
  for (int a = 0; a < NPE; a++) {
    const float mi = ldx<CG>(&M.mass[nid[a]]);
    cur[a] = -(kf * KT[a]) / mi + ppn / (mi * m.cp_T);
  }
}

// Where an element's node values come from. GlobalNodes: the node arrays in
// HBM through the element's connectivity (per-phase kernels, cluster run);
// TileNodes (below): a tile's node arrays staged in shared memory through
// tile-local indices. Both return the same values, so an element computes
// the same forces bit for bit from either.
// CGX: positions and predicted velocities through L2 as well (the cluster
// run); the dataflow step reads them through L1 (no tile of its launch writes
// them before every read of them is done) and only the J ratios through L2.
template <bool CG, bool BOX = false, bool CGX = CG>
struct GlobalNodes {
  const float2 *xh;
  const float *vp, *jr;
  int64_t np;
  int32_t nid[8];
  __device__ __forceinline__ GlobalNodes(const StepParams &P, const MixState &M, int64_t e)
      : xh(M.xh), vp(M.vp), jr(M.jr), np(P.np) {
    if constexpr (BOX) {
      box_corners(P, e, nid);
    } else {
#pragma unroll
      for (int a = 0; a < 8; a++) nid[a] = __ldg(&P.elnod[a * P.ne + e]);
    }
  }
  __device__ __forceinline__ float2 x(int a, int k) const { return ldx<CGX>(&xh[k * np + nid[a]]); }
  __device__ __forceinline__ float v(int a, int k) const { return ldx<CGX>(&vp[k * np + nid[a]]); }
  __device__ __forceinline__ float j(int a) const { return ldx<CG>(&jr[nid[a]]); }
};

// Artificial viscosity (calcArtificialViscosity, Mechanical.C:1948-1977) of
// one element: q = av0 c |eps_v| l + av1 (eps_v l)^2, capped at 1e9, with
// c = sqrt(K / rho), l = vol^(1/3) and eps_v the trace of the strain rate,
// added to the normal stresses with the sign opposite to eps_v. Returns the
// signed term qs (0 when |eps_v| <= 1e-12); it adds qs eps_v to the stress
// power.
__device__ __forceinline__ float artificial_viscosity(const StepParams &P, const MatF &m,
                                                      float eps_v, float vol, float (&sg)[6]) {
  if (!(fabsf(eps_v) > 1e-12f)) return 0.f;
  const float c = sqrtf(m.K / m.rho);
  const float l = cbrtf(vol);
  const float el = eps_v * l;
  float q = P.f_av0 * c * fabsf(eps_v) * l + P.f_av1 * (el * el);
  q = (1e9f < q) ? 1e9f : q;
  const float qs = (eps_v > 0.f) ? -q : q;
  sg[0] += qs;
  sg[1] += qs;
  sg[2] += qs;
  return qs;
}

// Element forces to HBM, SoA by (local node, component): fe[(a * 3 + k) * ne + e].
struct ForcesToHbm {
  float *fe;
  int64_t ne, e;
  __device__ __forceinline__ void put(int a, int k, float f) { fe[(a * 3 + k) * ne + e] = f; }
};

// Hexahedron: with dN_a/dx = (1/8) adj(J)^T-row . s(a) / detJ at the centre,
// the velocity gradient is adj(J) G / (8 detJ) with G the Walsh sums of the
// nodal velocities, and the nodal forces are the synthesis of
// T = adj(J)^T sigma (w / 8 = 1) plus the hourglass coefficients ch h_j.
// Same quantities as the reference's per-node loops, fewer operations.
// EARLY_JR: gather the nodes' volume ratios with the positions, so that their
// loads are in flight during the Jacobian arithmetic (the cluster run, one
// element per thread, gathers them later: early it spills there).
template <int LAW, bool EARLY_JR, bool TH, class Nodes, class Out, class IO>
__device__ __forceinline__ void element_hex_core(const StepParams &P, const MixState &M,
                                                 int64_t e, const Nodes &nd, float *stash,
                                                 int stride, long long step, Out &out,
                                                 const IO &io) {
  float A[3][3], detJ;
  float J_avg = 0.f;
  {
    // coordinates relative to node 0, from the (hi, lo) pairs
    float r[8][3];
    float2 o[3];
#pragma unroll
    for (int k = 0; k < 3; k++) o[k] = nd.x(0, k);
#pragma unroll
    for (int k = 0; k < 3; k++) r[0][k] = 0.0f;
#pragma unroll
    for (int a = 1; a < 8; a++)
#pragma unroll
      for (int k = 0; k < 3; k++) r[a][k] = pair_rel(nd.x(a, k), o[k]);
    if constexpr (EARLY_JR) {
#pragma unroll
      for (int a = 0; a < 8; a++) J_avg += nd.j(a);
    }
    float J[3][3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      float v[8], o8[8];
#pragma unroll
      for (int a = 0; a < 8; a++) v[a] = r[a][k];
      walsh8(v, o8);
      J[0][k] = 0.125f * o8[1];
      J[1][k] = 0.125f * o8[2];
      J[2][k] = 0.125f * o8[3];
    }
    A[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]);
    A[1][0] = -(J[1][0] * J[2][2] - J[1][2] * J[2][0]);
    A[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    A[0][1] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]);
    A[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]);
    A[2][1] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]);
    A[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]);
    A[1][2] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]);
    A[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]);
    detJ = J[0][0] * A[0][0] + J[0][1] * A[1][0] + J[0][2] * A[2][0];
  }
  const float vol = detJ * 8.0f;
  const MatF &m = P.matf[P.emat ? __ldg(&P.emat[e]) : 0];
  // velocity Walsh sums: G[m][k] (derivative directions), hm[k][j] (hourglass)
  float G[3][3], hm[3][4];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float v[8], o[8];
#pragma unroll
    for (int a = 0; a < 8; a++) v[a] = nd.v(a, k);
    walsh8(v, o);
    G[0][k] = o[1];
    G[1][k] = o[2];
    G[2][k] = o[3];
#pragma unroll
    for (int j = 0; j < 4; j++) hm[k][j] = o[4 + j];
  }
  // hourglass forces' coefficients ch h_j, kept in shared memory (one column
  // per thread) across the stress update to free registers
  {
    const float ch = P.hg_on ? P.f_hg_coef * powf(vol, 0.6666666f) * m.rho * 0.25f * m.cs0 : 0.f;
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
      for (int j = 0; j < 4; j++) stash[(k * 4 + j) * stride] = ch * hm[k][j];
  }
  if constexpr (!EARLY_JR) {
#pragma unroll
    for (int a = 0; a < 8; a++) J_avg += nd.j(a);
  }
  // velocity gradient L[i][k] = d v_k / d x_i
  const float fl = 0.125f / detJ;
  float L[3][3];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int k = 0; k < 3; k++) L[i][k] = fl * (A[i][0] * G[0][k] + A[i][1] * G[1][k] + A[i][2] * G[2][k]);
  float sr[6] = {L[0][0], L[1][1], L[2][2], 0.5f * (L[1][0] + L[0][1]),
                 0.5f * (L[2][1] + L[1][2]), 0.5f * (L[2][0] + L[0][2])};
  const float w01 = 0.5f * (L[1][0] - L[0][1]);
  const float w12 = 0.5f * (L[2][1] - L[1][2]);
  const float w02 = 0.5f * (L[2][0] - L[0][2]);
  float jTh = m.jc_Th;
  if constexpr (TH) thermal_pre<8, !EARLY_JR>(P, M, m, nd.nid, step, sr, jTh);
  float J_bar = J_avg * 0.125f;
  if (J_bar < 0.0f) J_bar = 0.2f;
  const float p = -m.K * (J_bar - 1.0f);
  float sg[6], sdot = 0.f, qpl = 0.f;
  const float eps_v = sr[0] + sr[1] + sr[2];
  stress_update<LAW, TH>(P, M, e, io, m, sr, w01, w12, w02, p, jTh, sg, sdot, qpl);
  if (P.av_on) sdot += artificial_viscosity(P, m, eps_v, vol, sg) * eps_v;
  if (P.energy_on && io.owns()) M.edot[e] = sdot * vol;
  // sigma as a symmetric 3x3: S[i][k]
  const float S[3][3] = {{sg[0], sg[3], sg[5]}, {sg[3], sg[1], sg[4]}, {sg[5], sg[4], sg[2]}};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float o[8], f[8];
    o[0] = 0.f;
#pragma unroll
    for (int mm = 0; mm < 3; mm++) o[1 + mm] = A[0][mm] * S[0][k] + A[1][mm] * S[1][k] + A[2][mm] * S[2][k];
#pragma unroll
    for (int j = 0; j < 4; j++) o[4 + j] = stash[(k * 4 + j) * stride];
    walsh8_synth(o, f);
#pragma unroll
    for (int a = 0; a < 8; a++) out.put(a, k, f[a]);
  }
  if constexpr (TH) {
    // conduction in the same Walsh form: grad T detJ = A (Walsh sums of T) / 8,
    // (K T)_a = k_T / detJ * synthesis of A^T grad T detJ (w = 8 cancels 1/8)
    constexpr bool CG = !EARLY_JR;
    float tv[8], oT[8], KT[8];
#pragma unroll
    for (int a = 0; a < 8; a++) tv[a] = ldx<CG>(&M.T[nd.nid[a]]).x;
    walsh8(tv, oT);
    float BT[3];
#pragma unroll
    for (int d = 0; d < 3; d++)
      BT[d] = 0.125f * (A[d][0] * oT[1] + A[d][1] * oT[2] + A[d][2] * oT[3]);
    float o[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int mm = 0; mm < 3; mm++) o[1 + mm] = A[0][mm] * BT[0] + A[1][mm] * BT[1] + A[2][mm] * BT[2];
    walsh8_synth(o, KT);
    thermal_rates<8, CG>(P, M, m, e, nd.nid, step, KT, m.k_T / detJ, qpl * vol);
  }
}

// Per-phase kernels and the cluster run: node values from HBM, forces to HBM.
template <int LAW, bool CG, bool TH, bool BOX = false>
__device__ __forceinline__ void element_hex(const StepParams &P, const MixState &M, int64_t e,
                                            float *stash, int stride, long long step) {
  const GlobalNodes<CG, BOX> nd(P, M, e);
  ForcesToHbm out{M.fe, P.ne, e};
  element_hex_core<LAW, !CG, TH>(P, M, e, nd, stash, stride, step, out,
                                 StateInPlace{});
}

// Tetrahedron: per-node shape derivatives (Domain_d.C:1866-1887).
template <int LAW, bool CG, bool TH>
__device__ __forceinline__ void element_tet(const StepParams &P, const MixState &M, int64_t e,
                                            long long step) {
  const int64_t ne = P.ne;
  int32_t nid[4];
  float dH[3][4];
  float detJ;
  float vpn[4][3], jrn[4];
  {
    float r[4][3];
    rel_coords<4, CG>(P, M, e, r, nid);
    // the nodes' predicted velocities and volume ratios, gathered before the
    // Jacobian arithmetic so that their loads are in flight during it
#pragma unroll
    for (int a = 0; a < 4; a++) {
      vpn[a][0] = ldx<CG>(&M.vp[nid[a]]);
      vpn[a][1] = ldx<CG>(&M.vp[P.np + nid[a]]);
      vpn[a][2] = ldx<CG>(&M.vp[2 * P.np + nid[a]]);
      jrn[a] = ldx<CG>(&M.jr[nid[a]]);
    }
    float J[3][3];
    jacobian_f<4>(r, J);
    shape_derivs_f<4>(J, dH);
    detJ = det3f(J);
  }
  const MatF &m = P.matf[P.emat ? __ldg(&P.emat[e]) : 0];
  float s00 = 0.f, s11 = 0.f, s22 = 0.f, s01 = 0.f, s12 = 0.f, s02 = 0.f;
  float w01 = 0.f, w12 = 0.f, w02 = 0.f;
  float J_avg = 0.f;
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const float v0 = vpn[a][0], v1 = vpn[a][1], v2 = vpn[a][2];
    const float d0 = dH[0][a], d1 = dH[1][a], d2 = dH[2][a];
    s00 += d0 * v0;
    s11 += d1 * v1;
    s22 += d2 * v2;
    s01 += d1 * v0 + d0 * v1;
    w01 += d1 * v0 - d0 * v1;
    s12 += d2 * v1 + d1 * v2;
    s02 += d2 * v0 + d0 * v2;
    w12 += d2 * v1 - d1 * v2;
    w02 += d2 * v0 - d0 * v2;
    J_avg += jrn[a];
  }
  const float f = 1.0f / detJ;
  const float fh = 0.5f * f;
  float sr[6] = {s00 * f, s11 * f, s22 * f, s01 * fh, s12 * fh, s02 * fh};
  w01 *= fh; w12 *= fh; w02 *= fh;
  float jTh = m.jc_Th;
  if constexpr (TH) thermal_pre<4, CG>(P, M, m, nid, step, sr, jTh);
  J_avg *= 0.25f;
  float J_bar = J_avg;
  if (J_bar < 0.0f) J_bar = 0.2f;
  const float p = -m.K * (J_bar - 1.0f);
  float sg[6], sdot = 0.f, qpl = 0.f;
  stress_update<LAW, TH>(P, M, e, StateInPlace{}, m, sr, w01, w12, w02, p, jTh, sg, sdot,
                         qpl);
  const float w = weightf<4>();
  if (P.av_on) sdot += artificial_viscosity(P, m, sr[0] + sr[1] + sr[2], detJ * w, sg) *
                       (sr[0] + sr[1] + sr[2]);
  if (P.energy_on) M.edot[e] = sdot * (detJ * w);
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const float d0 = dH[0][a], d1 = dH[1][a], d2 = dH[2][a];
    M.fe[(a * 3) * ne + e] = (d0 * sg[0] + d1 * sg[3] + d2 * sg[5]) * w;
    M.fe[(a * 3 + 1) * ne + e] = (d1 * sg[1] + d0 * sg[3] + d2 * sg[4]) * w;
    M.fe[(a * 3 + 2) * ne + e] = (d2 * sg[2] + d1 * sg[4] + d0 * sg[5]) * w;
  }
  if constexpr (TH) {
    // conduction K_ij = (sum_d dN_i detJ dN_j detJ) k_T / detJ w against the
    // temperatures relative to node 0's (K's rows sum to zero): no FP32
    // cancellation between the absolute temperatures
    float Te[4], KT[4];
    const float T0n = ldx<CG>(&M.T[nid[0]]).x;
    Te[0] = 0.f;
#pragma unroll
    for (int a = 1; a < 4; a++) Te[a] = ldx<CG>(&M.T[nid[a]]).x - T0n;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      float t = 0.f;
#pragma unroll
      for (int k = 0; k < 4; k++)
        t += (dH[0][i] * dH[0][k] + dH[1][i] * dH[1][k] + dH[2][i] * dH[2][k]) * Te[k];
      KT[i] = t;
    }
    thermal_rates<4, CG>(P, M, m, e, nid, step, KT, m.k_T / detJ * w, qpl * (detJ * w));
  }
}

template <int NPE, int LAW, bool CG, bool TH, bool BOX = false>
__device__ __forceinline__ void element_one(const StepParams &P, const MixState &M, int64_t e,
                                            float *stash, int stride, long long step) {
  if constexpr (NPE == 8)
    element_hex<LAW, CG, TH, BOX>(P, M, e, stash, stride, step);
  else
    element_tet<LAW, CG, TH>(P, M, e, step);
}

// Resident threads per SM the element kernel is compiled for (1024: at most
// 64 registers per thread), a build-time constant.
#ifndef WF_ELEM_THREADS_PER_SM
#define WF_ELEM_THREADS_PER_SM 1024
#endif
constexpr int elem_min_blocks(int bs) { return WF_ELEM_THREADS_PER_SM / bs; }

template <int NPE, int BS, int LAW, bool TH, bool BOX>
__global__ void __launch_bounds__(BS, elem_min_blocks(BS)) k_mix_elements(StepParams P,
                                                                          MixState M) {
  __shared__ float stash[NPE == 8 ? 12 * BS : 1];
  const long long step = TH ? P.st->step : 0;
  for (int64_t e = (int64_t)blockIdx.x * BS + threadIdx.x; e < P.ne; e += (int64_t)gridDim.x * BS)
    element_one<NPE, LAW, false, TH, BOX>(P, M, e, &stash[threadIdx.x], BS, step);
}

// ---------------------------------------------------------------------------
// Block sum in a fixed order (shuffle tree per warp, warps in index order);
// warps with no nonzero value skip their FP64 shuffles. Valid in thread 0.
__device__ __forceinline__ double block_sum_sparse(float vf, double *sh) {
  const unsigned any = __ballot_sync(0xffffffffu, vf != 0.0f);
  double v = 0.0;
  if (any) {
    v = (double)vf;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += sh[i];
  return t;
}

// Fixed-order block sum of doubles (all warps reduce). Valid in thread 0.
__device__ __forceinline__ double block_sum_dense(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += sh[i];
  return t;
}

// Update of one node from its assembled internal force fi (the element forces
// summed in list order): non-finite check, accelerations, velocity BCs,
// Chung-Hulbert corrector and the next predictor. x and vp are the node's
// position pair and predicted velocity (read by the caller from HBM or from
// a staged copy); the new ones go to xo and vpo (the arrays they were read
// from, or the other buffers of the column sweep's pairs). Returns the node's
// reaction contribution.
// A node's own state read by its update (loaded ahead of the gather by the
// column sweep, where the gather does not wait for HBM).
struct NodeIn {
  float vold[3], pa[3];
  float mass;
  uint32_t code;
  uint8_t fl;
};
template <bool CG = false>
__device__ __forceinline__ NodeIn node_in(const StepParams &P, const MixState &M, int64_t n) {
  NodeIn in;
  const int64_t np = P.np;
  in.fl = P.nflag[n];
  in.mass = CG ? __ldcg(&M.mass[n]) : M.mass[n];   // written by the nodal phase
#pragma unroll
  for (int k = 0; k < 3; k++) {
    in.vold[k] = M.v[k * np + n];
    in.pa[k] = M.pa[k * np + n];
  }
  in.code = P.bc[n];
  return in;
}

template <int NPE, bool CG>
__device__ __forceinline__ float node_finish(const StepParams &P, const MixState &M, int64_t n,
                                             long long step, float fi0, float fi1, float fi2,
                                             float2 (&x)[3], const float (&vp)[3], float2 *xo,
                                             float *vpo, const NodeIn &in) {
  float r = 0.0f;
  const int64_t np = P.np;
  const int64_t ne = P.ne;
  float fi[3] = {fi0, fi1, fi2};
#pragma unroll
  for (int k = 0; k < 3; k++)
    if (!isfinite(fi[k])) {
      fi[k] = 0.f;
      atomicOr(&P.st->status, 1u);
      atomicMin(&P.st->first_bad_node, (long long)n);
    }
  const uint8_t fl = in.fl;
  const float mass = in.mass;
  const float inv_m = 1.0f / mass;
  float vold[3], pa[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    vold[k] = in.vold[k];
    pa[k] = in.pa[k];
  }
  float cf[3] = {0.f, 0.f, 0.f};
  if (P.contact && (fl & NF_CONTACT)) {
    cf[0] = ldx<CG>(&M.cf[n]);
    cf[1] = ldx<CG>(&M.cf[np + n]);
    cf[2] = ldx<CG>(&M.cf[2 * np + n]);
    r = P.tri_on ? ldx<CG>(&M.cfn[n]) : fabsf(cf[2]);
  }
  if (!P.contact && (fl & NF_REACTION)) {
    if (P.rnode)
      P.rnode[n] = fi[P.react_dim];  // summed per specimen by the reaction kernel
    else
      r = fi[P.react_dim];
  }
  float c_dt = P.f_dt, c_cu_pred = P.f_cu_pred, c_cu_corr = P.f_cu_corr;
  float c_cv_corr = P.f_cv_corr, c_cv_pred = P.f_cv_pred;
  if (P.nspec_of) {
    const SpecF sf = P.specf[P.nspec_of[n]];
    c_dt = sf.dt; c_cu_pred = sf.cu_pred; c_cu_corr = sf.cu_corr;
    c_cv_corr = sf.cv_corr; c_cv_pred = sf.cv_pred;
  }
  const uint32_t code = in.code;
  const float *bvf = &P.bcvalf[3 * (code >> 3)];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const bool fixed = (code >> k) & 1u;
    float a = (cf[k] - fi[k]) * inv_m;
    if (fixed) a = 0.f;
    a = P.f_fcorr * (a - P.f_alpha * pa[k]);
    float v = vp[k] + c_cv_corr * a;
    const float bv = fixed ? __ldg(&bvf[k]) : 0.f;
    if (fixed) v = bv;
    const float udt = c_dt * (vold[k] + c_cu_pred * pa[k]) + c_cu_corr * a;
    x[k] = pair_add(x[k], udt);
    float vnext = v + c_cv_pred * a;
    if (fixed) vnext = bv;
    xo[k * np + n] = x[k];
    M.v[k * np + n] = v;
    M.pa[k * np + n] = a;
    vpo[k * np + n] = vnext;
  }
  if (P.thermal) {
    // ThermalCalcs node part: the step's element-node rates in list order and
    // the die heat over m cp of material 0
    const float *cur = M.dte + (step & 1) * ne * NPE;
    float sT = 0.f;
    const int32_t b = __ldg(&P.off[n]), c = __ldg(&P.off[n + 1]) - b;
    for (int32_t k = 0; k < c; k++) sT += ldx<CG>(&cur[__ldg(&P.slot[b + k])]);
    M.T[n] = pair_add(M.T[n], (sT + M.qc[n] / (mass * P.f_cp0)) * c_dt);
  }
  return r;
}

// Node update of one node: gather of the element forces in list order, then
// node_finish. Returns the node's reaction contribution.
template <int NPE, bool CG, bool BOX = false>
__device__ __forceinline__ float node_one(const StepParams &P, const MixState &M, int64_t n,
                                          long long step) {
  const int64_t ne = P.ne;
  float fi0 = 0.f, fi1 = 0.f, fi2 = 0.f;
  if constexpr (BOX && NPE == 8) {
    // the node's elements in list order, from its indices; all loads issued
    // before the sum, which adds the existing entries in list order
    int32_t el[8], cor[8];
    box_node_list(P, n, el, cor);
    float g0[8], g1[8], g2[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      g0[j] = g1[j] = g2[j] = 0.f;
      if (el[j] >= 0) {
        const int64_t base = (int64_t)cor[j] * 3 * ne + el[j];
        g0[j] = ldx<CG>(&M.fe[base]);
        g1[j] = ldx<CG>(&M.fe[base + ne]);
        g2[j] = ldx<CG>(&M.fe[base + 2 * ne]);
      }
    }
#pragma unroll
    for (int j = 0; j < 8; j++)
      if (el[j] >= 0) {
        fi0 += g0[j];
        fi1 += g1[j];
        fi2 += g2[j];
      }
    const int64_t np = P.np;
    float2 x[3];
    float vp[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      x[k] = M.xh[k * np + n];
      vp[k] = M.vp[k * np + n];
    }
    return node_finish<NPE, CG>(P, M, n, step, fi0, fi1, fi2, x, vp, M.xh, M.vp,
                                node_in<CG>(P, M, n));
  }
  const int32_t b = __ldg(&P.off[n]), c = __ldg(&P.off[n + 1]) - b;
  // gather over the node's element list in list order, eight entries at a
  // time so that the slot and force loads of a chunk are all in flight
  for (int32_t k0 = 0; k0 < c; k0 += 8) {
    int32_t sl[8];
#pragma unroll
    for (int j = 0; j < 8; j++) sl[j] = (k0 + j < c) ? __ldg(&P.slot[b + k0 + j]) : -1;
    float g0[8], g1[8], g2[8];
#pragma unroll
    for (int j = 0; j < 8; j++) {
      g0[j] = g1[j] = g2[j] = 0.f;
      if (sl[j] >= 0) {
        const int64_t base = (int64_t)(sl[j] % NPE) * 3 * ne + sl[j] / NPE;
        g0[j] = ldx<CG>(&M.fe[base]);
        g1[j] = ldx<CG>(&M.fe[base + ne]);
        g2[j] = ldx<CG>(&M.fe[base + 2 * ne]);
      }
    }
#pragma unroll
    for (int j = 0; j < 8; j++) {
      fi0 += g0[j];
      fi1 += g1[j];
      fi2 += g2[j];
    }
  }
  const int64_t np = P.np;
  float2 x[3];
  float vp[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    x[k] = M.xh[k * np + n];
    vp[k] = M.vp[k * np + n];
  }
  return node_finish<NPE, CG>(P, M, n, step, fi0, fi1, fi2, x, vp, M.xh, M.vp,
                              node_in<CG>(P, M, n));
}

template <int NPE, bool BOX>
__global__ void __launch_bounds__(kNodeThreads, WF_NODE_MIN_BLOCKS) k_mix_nodes(StepParams P,
                                                                             MixState M) {
  __shared__ double sh[kNodeThreads / 32];
  __shared__ bool am_last;
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const float r = (n < P.nn) ? node_one<NPE, false, BOX>(P, M, n, P.st->step) : 0.0f;
  // reaction: only warps holding a contribution reduce (FP64, fixed order);
  // the last block to finish sums all block partials with the whole block.
  const double bs = block_sum_sparse(r, sh);
  if (threadIdx.x == 0) {
    P.partials[blockIdx.x] = bs;
    __threadfence();
    const unsigned prev = atomicAdd(&P.st->done_blocks, 1u);
    am_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (am_last) {
    __threadfence();
    const double time = P.st->time;
    double t = 0.0;
    for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x)
      t += ((volatile double *)P.partials)[i];
    const double tot = block_sum_dense(t, sh);
    if (threadIdx.x == 0) {
      const long long s = P.st->step;
      if (s < P.hist_cap) P.hist[s] = tot;
      P.st->step = s + 1;
      P.st->time = time + P.dt;
      P.st->done_blocks = 0u;
    }
    if (P.tri_on) tri_move<true>(P, time);
  }
}

// ---------------------------------------------------------------------------
// Tiled step for hexahedra: element phase and assembly of a tile in one block.
//
// One block per tile (TileParams, built at init), one thread per element. The
// tile's node positions, predicted velocities and volume ratios are staged in
// shared memory once; each element computes its forces from the staged copy
// (the per-phase element arithmetic, so the same forces bit for bit) and
// keeps them in registers. The block then sums them into per-node
// accumulators in shared memory in eight passes, one per corner, in the
// corner order 6, 7, 5, 4, 2, 3, 1, 0: for the AddBoxLength numbering that is
// the element-ascending order of every node's list, so an interior node's
// force is the per-phase gather's sum bit for bit (two elements of a tile
// never hold one node at the same corner: checked at init). Interior nodes
// (all their elements in the tile) are then updated by the block; a corner
// force whose node is shared goes to HBM for the shared-node kernel, which
// gathers it in list order. The element-force round trip through HBM is left
// only for shared nodes.

// A tile's staged node values through tile-local indices.
struct TileNodes {
  const float2 *sx;
  const float *svp, *sjr;
  int32_t loc[8];
  __device__ __forceinline__ float2 x(int a, int k) const { return sx[k * kTileNodes + loc[a]]; }
  __device__ __forceinline__ float v(int a, int k) const { return svp[k * kTileNodes + loc[a]]; }
  __device__ __forceinline__ float j(int a) const { return sjr[loc[a]]; }
};

// Element forces kept in registers (all indices compile-time after unrolling).
struct ForcesToRegs {
  float (&f)[8][3];
  __device__ __forceinline__ void put(int a, int k, float v) { f[a][k] = v; }
};

// Dynamic shared memory of the tile kernel: staged positions (hi, lo),
// predicted velocities, volume ratios, force accumulators, node ids, and the
// hourglass stash of each thread.
constexpr size_t kTileSmem = sizeof(float2) * 3 * kTileNodes + sizeof(float) * 3 * kTileNodes +
                             sizeof(float) * kTileNodes + sizeof(float) * 3 * kTileNodes +
                             sizeof(int32_t) * kTileNodes + sizeof(float) * 12 * kTileElems;

template <int LAW>
__global__ void __launch_bounds__(kTileElems, 2) k_mix_tile(StepParams P, MixState M,
                                                            TileParams T) {
  extern __shared__ __align__(16) unsigned char smem[];
  float2 *sx = reinterpret_cast<float2 *>(smem);
  float *svp = reinterpret_cast<float *>(sx + 3 * kTileNodes);
  float *sjr = svp + 3 * kTileNodes;
  float *acc = sjr + kTileNodes;
  int32_t *sid = reinterpret_cast<int32_t *>(acc + 3 * kTileNodes);
  float *stash = reinterpret_cast<float *>(sid + kTileNodes);
  __shared__ double sh[kTileElems / 32];
  const int t = blockIdx.x, tid = threadIdx.x;
  const int64_t np = P.np, ne = P.ne;
  const int nt = __ldg(&T.ncount[t]);
  const int32_t *tn = T.nodes + (int64_t)t * kTileNodes;
  const long long step = P.st->step;
  for (int i = tid; i < nt; i += kTileElems) {
    const int32_t id = __ldg(&tn[i]);
    const int64_t n = id & 0x7fffffff;
    sid[i] = id;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      sx[k * kTileNodes + i] = __ldg(&M.xh[k * np + n]);
      svp[k * kTileNodes + i] = __ldg(&M.vp[k * np + n]);
      acc[k * kTileNodes + i] = 0.0f;
    }
    sjr[i] = __ldg(&M.jr[n]);
  }
  __syncthreads();
  const int32_t e0 = __ldg(&T.eoff[t]);
  const bool act = tid < __ldg(&T.eoff[t + 1]) - e0;
  float f[8][3];
  TileNodes nd{sx, svp, sjr, {0, 0, 0, 0, 0, 0, 0, 0}};
  if (act) {
    const int64_t pos = e0 + tid;
    const int64_t e = __ldg(&T.elems[pos]);
#pragma unroll
    for (int a = 0; a < 8; a++) nd.loc[a] = __ldg(&T.lel[a * ne + pos]);
    ForcesToRegs out{f};
    element_hex_core<LAW, true, false>(P, M, e, nd, &stash[tid], kTileElems, step, out,
                                       StateInPlace{});
    // corner forces of shared nodes: to HBM, for the shared-node gather
#pragma unroll
    for (int a = 0; a < 8; a++)
      if (sid[nd.loc[a]] < 0) {
#pragma unroll
        for (int k = 0; k < 3; k++) M.fe[(a * 3 + k) * ne + e] = f[a][k];
      }
  }
  // corner passes: no two elements of the tile write one accumulator in a pass
  constexpr int kOrder[8] = {6, 7, 5, 4, 2, 3, 1, 0};
#pragma unroll
  for (int q = 0; q < 8; q++) {
    __syncthreads();
    if (act) {
      const int a = kOrder[q];
      const int l = nd.loc[a];
#pragma unroll
      for (int k = 0; k < 3; k++) acc[k * kTileNodes + l] += f[a][k];
    }
  }
  __syncthreads();
  // interior nodes: the node update with the tile's sums
  double r = 0.0;
  for (int i = tid; i < nt; i += kTileElems) {
    const int32_t id = sid[i];
    if (id >= 0) {
      float2 x[3];
      float vp[3];
#pragma unroll
      for (int k = 0; k < 3; k++) {
        x[k] = sx[k * kTileNodes + i];
        vp[k] = svp[k * kTileNodes + i];
      }
      r += (double)node_finish<8, false>(P, M, id, step, acc[i], acc[kTileNodes + i],
                                         acc[2 * kTileNodes + i], x, vp, M.xh, M.vp,
                                         node_in(P, M, id));
    }
  }
  const double bsum = block_sum_dense(r, sh);
  if (tid == 0) T.partials[t] = bsum;
}

// The shared nodes: list-order gather from HBM and node update; the last
// block adds the reaction partials of the tiles and of its own blocks in a
// fixed order and advances the step state.
template <bool BOX>
__global__ void __launch_bounds__(kNodeThreads, WF_NODE_MIN_BLOCKS) k_mix_shared(StepParams P,
                                                                              MixState M,
                                                                              TileParams T) {
  __shared__ double sh[kNodeThreads / 32];
  __shared__ bool am_last;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const float r =
      (i < T.nshared) ? node_one<8, false, BOX>(P, M, __ldg(&T.shared[i]), P.st->step) : 0.0f;
  const double bs = block_sum_sparse(r, sh);
  if (threadIdx.x == 0) {
    T.partials[T.ntiles + blockIdx.x] = bs;
    __threadfence();
    const unsigned prev = atomicAdd(&P.st->done_blocks, 1u);
    am_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (am_last) {
    __threadfence();
    const double time = P.st->time;
    double t = 0.0;
    const int64_t np_all = (int64_t)T.ntiles + gridDim.x;
    for (int64_t j = threadIdx.x; j < np_all; j += blockDim.x)
      t += ((volatile double *)T.partials)[j];
    const double tot = block_sum_dense(t, sh);
    if (threadIdx.x == 0) {
      const long long s = P.st->step;
      if (s < P.hist_cap) P.hist[s] = tot;
      P.st->step = s + 1;
      P.st->time = time + P.dt;
      P.st->done_blocks = 0u;
    }
  }
}

// ---------------------------------------------------------------------------
// Column sweep for box meshes (hexahedra in the AddBoxLength numbering): the
// element and node phases of a step in one kernel, the element forces kept in
// shared memory.
//
// The node grid (nx+1) x (ny+1) is cut into columns of at most 31 x CY nodes,
// one block each; a block sweeps its column's node planes k = 0..nz. It holds
// the elements that touch its nodes (its own and a one-element ring on the -x
// and -y sides, at most 32 x (CY+1) per layer, one thread each) and computes
// the ring elements again rather than exchanging forces with the neighbour
// column, so every node gathers all its element forces inside its block.
//   * Node planes are staged in shared memory (cp.async, three slots, issued
//     a layer ahead): positions (hi, lo), predicted velocities, J ratios.
//   * Each element of layer k computes its forces from the staged planes k
//     and k+1 with the per-phase element arithmetic (so bit for bit the same
//     forces) into a shared-memory buffer; an element owned by the block (its
//     corner 0 is one of the block's nodes) writes its tau and eps_p, a ring
//     element writes nothing.
//   * Each node of plane k adds the forces of its elements in list order: the
//     four of layer k-1 (corners 6, 7, 5, 4), summed in the previous layer and
//     carried in registers, then the four of layer k (corners 2, 3, 1, 0) --
//     the per-phase gather's order, so bit for bit its sum -- and is updated
//     (node_finish); it starts the sum of plane k+1 from layer k.
// Two barriers per layer separate the element and node phases; a thread's
// next element state and its node's next own state are loaded a phase ahead.
// Every array a block reads for its ring (positions, predicted velocities,
// tau, eps_p) is one of a pair: the step reads one buffer and writes the
// other, so no block sees another's update of the same step. The reaction is
// summed per thread over its planes (FP64), per block, and over blocks in
// block order by the last block, which advances the step state; its order
// differs from the node kernel's.
constexpr int kSwEX = 32;            // elements per row of a column layer (one warp)
constexpr int kSwNX = kSwEX + 1;     // staged nodes per row
template <int CY>
struct SweepShape {
  static constexpr int threads = kSwEX * (CY + 1);
  static constexpr int plane = kSwNX * (CY + 2);   // staged nodes per plane
  // per staged plane: positions [3][plane] float2, predicted velocities
  // [3][plane], J ratios [plane]
  static constexpr size_t slot_bytes = (size_t)plane * (3 * 8 + 3 * 4 + 4);
  // three staged planes, the element forces [24][threads], the hourglass
  // stash
  static constexpr size_t smem = 3 * slot_bytes + sizeof(float) * 36 * threads;
};

__device__ __forceinline__ void cp_async4(void *dst, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// An element's corners in the staged planes: corner a at staged index
// b + {0, 1, kSwNX + 1, kSwNX}[a & 3] of the lower (a < 4) or upper plane.
template <int PL>
struct SweepNodes {
  const float2 *x0, *x1;
  const float *v0, *v1, *j0, *j1;
  int b;
  static __device__ __forceinline__ int off(int a) {
    return (a & 3) == 0 ? 0 : (a & 3) == 1 ? 1 : (a & 3) == 2 ? kSwNX + 1 : kSwNX;
  }
  __device__ __forceinline__ float2 x(int a, int k) const {
    return (a < 4 ? x0 : x1)[k * PL + b + off(a)];
  }
  __device__ __forceinline__ float v(int a, int k) const {
    return (a < 4 ? v0 : v1)[k * PL + b + off(a)];
  }
  __device__ __forceinline__ float j(int a) const { return (a < 4 ? j0 : j1)[b + off(a)]; }
};

// Element forces into shared memory, [corner * 3 + component][thread].
template <int NT>
struct ForcesToSmem {
  float *sf;
  int t;
  __device__ __forceinline__ void put(int a, int k, float f) { sf[(a * 3 + k) * NT + t] = f; }
};

// tau and eps_p loaded a layer ahead (t[0..5] tau, t[6] eps_p); written to
// the other buffers of the pairs by the owning block (tau_o non-null), not by
// a ring.
__device__ __forceinline__ void load_elem_state(const MixState &M, int64_t ne, int64_t e,
                                                float (&t)[7]) {
#pragma unroll
  for (int c = 0; c < 6; c++) t[c] = M.tau[c * ne + e];
  t[6] = M.pls[e];
}
struct StateSwept {
  float t[6], p;
  float *tau_o, *pls_o;
  int64_t ne, e;
  __device__ __forceinline__ StateSwept(const float (&in)[7], int64_t ne_, int64_t e_, bool own,
                                        float *to, float *po)
      : p(in[6]), tau_o(own ? to : nullptr), pls_o(po), ne(ne_), e(e_) {
#pragma unroll
    for (int c = 0; c < 6; c++) t[c] = in[c];
  }
  __device__ __forceinline__ void load(const StepParams &, const MixState &, int64_t, float &t0,
                                       float &t1, float &t2, float &t3, float &t4, float &t5,
                                       float &pp) const {
    t0 = t[0]; t1 = t[1]; t2 = t[2]; t3 = t[3]; t4 = t[4]; t5 = t[5];
    pp = p;
  }
  __device__ __forceinline__ void store(const StepParams &, const MixState &, int64_t, float t0,
                                        float t1, float t2, float t3, float t4, float t5,
                                        float pp) const {
    if (tau_o) {
      pls_o[e] = pp;
      tau_o[e] = t0; tau_o[ne + e] = t1; tau_o[2 * ne + e] = t2;
      tau_o[3 * ne + e] = t3; tau_o[4 * ne + e] = t4; tau_o[5 * ne + e] = t5;
    }
  }
  __device__ __forceinline__ bool owns() const { return tau_o != nullptr; }
};

template <int LAW, int CY>
__global__ void __launch_bounds__(SweepShape<CY>::threads, 2) k_mix_sweep(StepParams P,
                                                                         MixState M,
                                                                         SweepParams W) {
  using S = SweepShape<CY>;
  constexpr int NT = S::threads, PL = S::plane;
  extern __shared__ __align__(16) unsigned char smem[];
  float *sf = reinterpret_cast<float *>(smem + 3 * S::slot_bytes);
  float *stash = sf + 24 * NT;
  __shared__ double sh[NT / 32];
  __shared__ bool am_last;
  const int t = threadIdx.x, lx = t & 31, ly = t >> 5;
  const int bx = P.bx, by = P.by, bz = P.bz;
  const int nx1 = bx + 1, ny1 = by + 1;
  const int cx = (int)(blockIdx.x % (unsigned)W.ncx), cy = (int)(blockIdx.x / (unsigned)W.ncx);
  const int i0 = (int)((int64_t)cx * nx1 / W.ncx), i1 = (int)((int64_t)(cx + 1) * nx1 / W.ncx);
  const int j0 = (int)((int64_t)cy * ny1 / W.ncy), j1 = (int)((int64_t)(cy + 1) * ny1 / W.ncy);
  // the column's elements: [ea, ea + nex) x [fa, fa + ney) in each layer;
  // its staged nodes: (nex + 1) x (ney + 1) from (ea, fa)
  const int ea = max(i0 - 1, 0), fa = max(j0 - 1, 0);
  const int nex = min(i1, bx) - ea, ney = min(j1, by) - fa;
  const int snx = nex + 1, sn = snx * (ney + 1);
  const int64_t np = P.np, ne = P.ne;
  const int64_t pxy = (int64_t)nx1 * ny1, exy = (int64_t)bx * by;
  // element role: element (ea + lx, fa + ly) of each layer
  const bool e_act = lx < nex && ly < ney;
  const bool e_own = e_act && ea + lx >= i0 && fa + ly >= j0;
  const int64_t e_col = (int64_t)(ea + lx) + (int64_t)bx * (fa + ly);
  // node role: node (i0 + lx, j0 + ly) of each plane, and the column-local
  // indices of its elements (-1,-1), (0,-1), (-1,0), (0,0) in a layer (-1: none)
  const bool n_act = lx < i1 - i0 && ly < j1 - j0;
  const int gi = i0 + lx, gj = j0 + ly;
  int q[4];
#pragma unroll
  for (int dj = 0; dj < 2; dj++)
#pragma unroll
    for (int di = 0; di < 2; di++) {
      const int ei = gi - 1 + di, ej = gj - 1 + dj;
      q[dj * 2 + di] =
          (ei >= 0 && ei < bx && ej >= 0 && ej < by) ? (ei - ea) + kSwEX * (ej - fa) : -1;
    }
  const int ns = (gi - ea) + kSwNX * (gj - fa);
  const int64_t n_col = (int64_t)gi + (int64_t)nx1 * gj;

  auto slot_x = [&](int pz) {
    return reinterpret_cast<float2 *>(smem + (pz % 3) * S::slot_bytes);
  };
  // plane pz into its slot, by the threads first, first + stride, ...
  auto stage = [&](int pz, int first, int stride) {
    float2 *sx = slot_x(pz);
    float *sv = reinterpret_cast<float *>(sx + 3 * PL);
    float *sj = sv + 3 * PL;
    for (int idx = first; idx < sn; idx += stride) {
      const int si = idx % snx, sy = idx / snx;
      const int64_t n = (int64_t)(ea + si) + (int64_t)nx1 * (fa + sy) + pxy * pz;
      const int o = si + kSwNX * sy;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        cp_async8(&sx[k * PL + o], &M.xh[k * np + n]);
        cp_async4(&sv[k * PL + o], &M.vp[k * np + n]);
      }
      cp_async4(&sj[o], &M.jr[n]);
    }
  };
  // plane pz by one warp, row by row (no division per node)
  auto stage_rows = [&](int pz) {
    float2 *sx = slot_x(pz);
    float *sv = reinterpret_cast<float *>(sx + 3 * PL);
    float *sj = sv + 3 * PL;
    for (int sy = 0; sy <= ney; sy++) {
      const int64_t row = (int64_t)ea + (int64_t)nx1 * (fa + sy) + pxy * pz;
      for (int si = lx; si < snx; si += 32) {
        const int64_t n = row + si;
        const int o = si + kSwNX * sy;
#pragma unroll
        for (int k = 0; k < 3; k++) {
          cp_async8(&sx[k * PL + o], &M.xh[k * np + n]);
          cp_async4(&sv[k * PL + o], &M.vp[k * np + n]);
        }
        cp_async4(&sj[o], &M.jr[n]);
      }
    }
  };
  // the node's own staged position and predicted velocity of plane pz
  auto own_node = [&](int pz, float2 (&x)[3], float (&vp)[3]) {
    const float2 *sx = slot_x(pz);
    const float *sv = reinterpret_cast<const float *>(sx + 3 * PL);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      x[k] = sx[k * PL + ns];
      vp[k] = sv[k * PL + ns];
    }
  };

  stage(0, t, NT);
  stage(1, t, NT);
  cp_async_commit();
  const long long step = P.st->step;
  float pf0 = 0.f, pf1 = 0.f, pf2 = 0.f;   // plane k's sum over layer k-1
  double racc = 0.0;
  // the element state of the thread's element in the next layer, and the
  // node's own state of the next plane: loaded one phase ahead of their use
  float tn[7];
  if (e_act) load_elem_state(M, ne, e_col, tn);
  NodeIn nin;
  if (n_act) nin = node_in(P, M, n_col);
  for (int k = 0; k < bz; k++) {
    cp_async_wait_all();
    __syncthreads();   // planes k, k+1 staged; the previous layer's reads done
    if (e_act) {
      const int64_t e = e_col + exy * k;
      const StateSwept io(tn, ne, e, e_own, W.tau_o, W.pls_o);
      const float2 *x0 = slot_x(k), *x1 = slot_x(k + 1);
      const float *v0 = reinterpret_cast<const float *>(x0 + 3 * PL);
      const float *v1 = reinterpret_cast<const float *>(x1 + 3 * PL);
      const SweepNodes<PL> nd{x0, x1, v0, v1, v0 + 3 * PL, v1 + 3 * PL, lx + kSwNX * ly};
      ForcesToSmem<NT> out{sf, t};
      element_hex_core<LAW, true, false>(P, M, e, nd, &stash[t], NT, step, out, io);
      if (k + 1 < bz) load_elem_state(M, ne, e + exy, tn);
    }
    __syncthreads();
    // the last row of warps holds no nodes: it stages plane k + 2 while the
    // others update plane k (its slot held plane k - 1, read in the layer
    // before)
    if (ly == CY) {
      if (k + 2 <= bz) stage_rows(k + 2);
      cp_async_commit();
    }
    if (n_act) {
      constexpr int cb[4] = {2, 3, 1, 0}, ct[4] = {6, 7, 5, 4};
      float f0 = pf0, f1 = pf1, f2 = pf2;
      float u0 = 0.f, u1 = 0.f, u2 = 0.f;
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (q[j] >= 0) {
          f0 += sf[(cb[j] * 3) * NT + q[j]];
          f1 += sf[(cb[j] * 3 + 1) * NT + q[j]];
          f2 += sf[(cb[j] * 3 + 2) * NT + q[j]];
          u0 += sf[(ct[j] * 3) * NT + q[j]];
          u1 += sf[(ct[j] * 3 + 1) * NT + q[j]];
          u2 += sf[(ct[j] * 3 + 2) * NT + q[j]];
        }
      float2 x[3];
      float vp[3];
      own_node(k, x, vp);
      const NodeIn cur = nin;
      nin = node_in(P, M, n_col + pxy * (k + 1));   // plane k+1 <= nz exists
      racc += (double)node_finish<8, false>(P, M, n_col + pxy * k, step, f0, f1, f2, x, vp,
                                            W.xh_o, W.vp_o, cur);
      pf0 = u0;
      pf1 = u1;
      pf2 = u2;
    }
  }
  // the top plane: layer nz-1's forces only (staged by the last layer's wait)
  if (n_act) {
    float2 x[3];
    float vp[3];
    own_node(bz, x, vp);
    racc += (double)node_finish<8, false>(P, M, n_col + pxy * bz, step, pf0, pf1, pf2, x, vp,
                                          W.xh_o, W.vp_o, nin);
  }
  const double bs = block_sum_dense(racc, sh);
  if (t == 0) {
    W.partials[blockIdx.x] = bs;
    __threadfence();
    const unsigned prev = atomicAdd(&P.st->done_blocks, 1u);
    am_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (am_last) {
    __threadfence();
    const double time = P.st->time;
    double tt = 0.0;
    for (unsigned i = t; i < gridDim.x; i += NT) tt += ((volatile double *)W.partials)[i];
    const double tot = block_sum_dense(tt, sh);
    if (t == 0) {
      const long long s = P.st->step;
      if (s < P.hist_cap) P.hist[s] = tot;
      P.st->step = s + 1;
      P.st->time = time + P.dt;
      P.st->done_blocks = 0u;
    }
  }
}

// ---------------------------------------------------------------------------
// Dataflow step for box meshes: the four phases of a step in one persistent
// launch, run as a wavefront through the element layers.
//
// The step's work is cut into tiles (FlowParams.tile elements or nodes of one
// layer or plane); the items are the phases of a layer: geometry G(l) and
// element phase E(l) of element layer l, nodal phase N1(p) and node update
// N2(p) of node plane p. Each block takes tiles by ticket (one atomic counter)
// in the order of the item table, built on the host in wavefront order: stage
// s holds G(s), N1(s-1), E(s-3), N2(s-lag). A tile waits until the items it
// reads are done:
//   N1(p) <- G(p-1), G(p)      (the volumes around the plane)
//   E(l)  <- N1(l), N1(l+1)    (the J ratios, masses, contact forces)
//   N2(p) <- E(p-1), E(p)      (the element forces of the plane's elements)
// Every tile an item depends on has a smaller ticket, so it was taken by a
// running block that waits only on smaller tickets in turn: the launch cannot
// deadlock however many blocks are resident. The node update of plane p writes
// its positions and predicted velocities only after every phase that reads
// them (G(p-1), G(p), N1(p), E(p-1), E(p)) is done: they are all in its
// dependency chain. Data written in the launch is read through L2 (__ldcg);
// a producer fences before its tile is counted, and a consumer's block waits
// on the counters with an acquire load in one thread and a barrier. The
// element forces of a layer are read while they are still in L2, a stage or
// two after they were written. Each element and node runs the per-phase
// arithmetic, so the state is bitwise the per-phase step's; the reaction is
// summed per node tile, and over tiles in a fixed order by a one-block kernel
// after the launch, which advances the step state.
//
// The waits are bounded (kFlowSpin polls): a wait that runs out sets bit 1 of
// the step status, which wf_sync reports, and the tile goes on.
constexpr int kFlowThreads = 256;
constexpr int kFlowSpin = 1 << 18;

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// a[i] without a runtime index into a kernel parameter (which would copy the
// array to local memory)
__device__ __forceinline__ int pick4(const int32_t (&a)[4], int i) {
  return i == 0 ? a[0] : (i == 1 ? a[1] : (i == 2 ? a[2] : a[3]));
}

__device__ __forceinline__ void red_release(unsigned *p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

template <int LAW>
__global__ void __launch_bounds__(kFlowThreads, 1024 / kFlowThreads) k_mix_flow(StepParams P,
                                                                               MixState M,
                                                                               float *vol,
                                                                               FlowParams F) {
  extern __shared__ int s_first[];   // [nstages + 1] the stage table
  __shared__ float stash[12 * kFlowThreads];
  __shared__ double sh[kFlowThreads / 32];
  __shared__ int s_tk[1];
  const int tid = threadIdx.x;
  // the next step's counters (no block of this launch reads them)
  if (blockIdx.x == 0)
    for (int i = tid; i < F.ncnt; i += kFlowThreads) F.cnt_next[i] = 0u;
  for (int i = tid; i <= F.nstages; i += kFlowThreads) s_first[i] = __ldg(&F.stage_first[i]);
  const int bz = P.bz;
  const int64_t exy = (int64_t)P.bx * P.by;
  const int64_t pxy = (int64_t)(P.bx + 1) * (P.by + 1);
  // the tile of ticket tk: its stage (binary search in the table), then the
  // stage's items in kind order
  auto decode = [&](int tk, int &kind, int &l, int &tile) {
    int lo = 0, hi = F.nstages - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (s_first[mid] <= tk) lo = mid;
      else hi = mid - 1;
    }
    int rem = tk - s_first[lo];
    kind = 0;
    l = 0;
#pragma unroll
    for (int q = 0; q < kFlowKinds; q++) {
      const int lq = lo - F.off[q], lmax = (q == 0 || q == 2) ? bz - 1 : bz;
      if (lq < 0 || lq > lmax) continue;
      if (rem < F.ntiles[q]) {
        kind = q;
        l = lq;
        break;
      }
      rem -= F.ntiles[q];
    }
    tile = rem;
  };
  __syncthreads();   // the stage table
  for (;;) {
    if (tid == 0) {
      const int tk = (int)atomicAdd(&F.cnt[0], 1u);
      s_tk[0] = tk;
      if (tk < F.total) {
        int kind, l, tile;
        decode(tk, kind, l, tile);
        // the items this tile reads (kind dk, layers d0..d1), each complete
        int dk = -1, d0 = 0, d1 = 0;
        if (kind == 1) { dk = 0; d0 = l - 1; d1 = l; }
        if (kind == 2) { dk = 1; d0 = l; d1 = l + 1; }
        if (kind == 3) { dk = 2; d0 = l - 1; d1 = l; }
        if (dk >= 0) {
          const unsigned need = (unsigned)pick4(F.ntiles, dk);
          const int lmax = (dk == 1) ? bz : bz - 1;
          for (int dl = d0; dl <= d1; dl++) {
            if (dl < 0 || dl > lmax) continue;
            const unsigned *c = F.cnt + 1 + dk * F.bz1 + dl;
            int spins = 0;
            while (ld_acquire(c) < need) {
              if (++spins > kFlowSpin) {
                atomicOr(&P.st->status, 2u);
                break;
              }
              __nanosleep(64);
            }
          }
        }
      }
    }
    __syncthreads();
    const int tk = s_tk[0];
    if (tk >= F.total) break;
    int kind, l, tile;
    decode(tk, kind, l, tile);
    const int T = pick4(F.tsize, kind);
    if (kind == 0 || kind == 2) {
      const int64_t e0 = exy * l + (int64_t)tile * T;
      const int64_t e1 = min(e0 + T, exy * (l + 1));
      if (kind == 0) {
        // positions: not written before this read (L1 is safe)
        for (int64_t e = e0 + tid; e < e1; e += kFlowThreads)
          geometry_one<8, false, true>(P, M, vol, e);
      } else {
        const long long step = 0;   // thermal coupling is not run here
        for (int64_t e = e0 + tid; e < e1; e += kFlowThreads) {
          const GlobalNodes<true, true, false> nd(P, M, e);
          ForcesToHbm out{M.fe, P.ne, e};
          element_hex_core<LAW, true, false>(P, M, e, nd, &stash[tid], kFlowThreads, step, out,
                                             StateInPlace{});
        }
      }
    } else {
      const int64_t n0 = pxy * l + (int64_t)tile * T;
      const int64_t n1 = min(n0 + T, pxy * (l + 1));
      if (kind == 1) {
        const float2 zd = die_height(P, P.st->time);   // the step's time (set by the finish)
        for (int64_t n = n0 + tid; n < n1; n += kFlowThreads)
          nodal_one<8, true, true>(P, M, vol, n, zd);
      } else {
        double r = 0.0;
        for (int64_t n = n0 + tid; n < n1; n += kFlowThreads)
          r += (double)node_one<8, true, true>(P, M, n, 0);
        const double bs = block_sum_dense(r, sh);
        if (tid == 0) F.partials[(int64_t)l * F.ntiles[3] + tile] = bs;
      }
    }
    // the tile's writes, then its count: a release by one thread after the
    // barrier (which orders the block's writes before it), by another warp
    // than the one that takes the next ticket
    __syncthreads();
    if (tid == 32) red_release(&F.cnt[1 + kind * F.bz1 + l], 1u);
  }
}

// After the dataflow launch: the reaction over the node tiles in (plane,
// tile) order, and the step state.
__global__ void __launch_bounds__(kFlowThreads) k_mix_flow_finish(StepParams P, FlowParams F) {
  __shared__ double sh[kFlowThreads / 32];
  const int64_t np_t = (int64_t)F.bz1 * F.ntiles[3];
  double t = 0.0;
  for (int64_t i = threadIdx.x; i < np_t; i += kFlowThreads) t += F.partials[i];
  const double tot = block_sum_dense(t, sh);
  if (threadIdx.x == 0) {
    const long long s = P.st->step;
    if (s < P.hist_cap) P.hist[s] = tot;
    P.st->step = s + 1;
    P.st->time = P.st->time + P.dt;
  }
}

// ---------------------------------------------------------------------------
// Small meshes: a whole run of steps in one launch of one thread-block
// cluster. The four phases of a step are separated by cluster barriers
// (release / acquire at cluster scope). Each block owns fixed element and
// node ranges, so per-element and per-node state is read back by the thread
// that wrote it, and what other blocks wrote (positions, predicted
// velocities, volumes, volume ratios, element forces) is loaded through L2.
// Each element and node is updated with the same arithmetic as in the
// per-phase kernels; the reaction is summed per thread and per block (FP64)
// into a [steps][blocks] staging array whose rows block 0 adds in block order
// at the end of the launch, so its summation order differs from the
// per-phase node kernel's.
__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
  asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
}

template <int NPE, int BS, int LAW, bool TH>
__global__ void __launch_bounds__(BS) k_mix_cluster_run(StepParams P, MixState M, float *vol,
                                                        double *part, int64_t nsteps) {
  __shared__ float stash[NPE == 8 ? 12 * BS : 1];
  __shared__ double sh[BS / 32];
  __shared__ float2 s_zd;
  const int64_t nb = gridDim.x, b = blockIdx.x;
  const int t = threadIdx.x;
  const int64_t e0 = P.ne * b / nb, e1 = P.ne * (b + 1) / nb;
  const int64_t n0 = P.nn * b / nb, n1 = P.nn * (b + 1) / nb;
  double time = __ldcg(&P.st->time);
  const long long step0 = __ldcg(&P.st->step);
  for (int64_t it = 0; it < nsteps; it++) {
    // the die height once per block (FP64), read after the barrier
    if (t == 0) s_zd = P.contact ? die_height(P, time) : make_float2(0.f, 0.f);
    for (int64_t e = e0 + t; e < e1; e += BS) geometry_one<NPE, true>(P, M, vol, e);
    cluster_barrier();
    {
      const float2 zd = s_zd;
      for (int64_t n = n0 + t; n < n1; n += BS) nodal_one<NPE, true>(P, M, vol, n, zd);
    }
    cluster_barrier();
    for (int64_t e = e0 + t; e < e1; e += BS)
      element_one<NPE, LAW, true, TH>(P, M, e, &stash[t], BS, step0 + it);
    cluster_barrier();
    double r = 0.0;
    for (int64_t n = n0 + t; n < n1; n += BS)
      r += (double)node_one<NPE, true>(P, M, n, step0 + it);
    const double bsum = block_sum_dense(r, sh);
    if (t == 0) part[it * nb + b] = bsum;   // step it, block b
    cluster_barrier();
    if (b == 0 && P.tri_on) tri_move<true>(P, time);
    time = time + P.dt;
  }
  // reaction history: block partials of each step added in block order
  if (b == 0) {
    for (int64_t it = t; it < nsteps; it += BS) {
      double tot = 0.0;
      for (int64_t i = 0; i < nb; i++) tot += __ldcg(&part[it * nb + i]);
      if (step0 + it < P.hist_cap) P.hist[step0 + it] = tot;
    }
    if (t == 0) {
      P.st->step = step0 + nsteps;
      P.st->time = time;
    }
  }
}

__global__ void k_mix_predict(StepParams P, MixState M) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= P.nn) return;
  const uint32_t code = P.bc[n];
  for (int k = 0; k < 3; k++) {
    const float cv = P.nspec_of ? P.specf[P.nspec_of[n]].cv_pred : P.f_cv_pred;
    float v = M.v[k * P.np + n] + cv * M.pa[k * P.np + n];
    if ((code >> k) & 1u) v = P.bcvalf[3 * (code >> 3) + k];
    M.vp[k * P.np + n] = v;
  }
}

// Copies the FP64 initial state (after the preamble) into the mixed arrays.
// The mixed state of the nodes from the FP64 preamble values: positions as
// compensated pairs, initial positions, velocities.
__global__ void k_mix_init_nodes(StepParams P, MixState M, Fp64State S) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= P.nn) return;
  const int64_t np = P.np;
  for (int k = 0; k < 3; k++) {
    const double x = S.x[k * np + n];
    M.xh[k * np + n] = split_d(x);
    M.x0[k * np + n] = x;
    M.v[k * np + n] = (float)S.v[k * np + n];
    M.pa[k * np + n] = 0.f;
  }
}

// The nodes' constant part of the nodal phase from the initial element
// volumes (FP32, from the mixed geometry kernel): s0 = the sum of the node's
// element volumes in list order (CalcNodalVol, Mechanical.C:1555-1572),
// nc = (1 / s0, the mean initial density of its elements), and the initial
// lumped mass, J ratio and the FP64 copies read back by the host.
template <int NPE>
__global__ void k_mix_init_nodal(StepParams P, MixState M, Fp64State S, const float *vol,
                                 const double *rho0) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= P.nn) return;
  float s = 0.0f;
  double rs = 0.0;
  int32_t c = 0;
  if (NPE == 8 && P.box) {
    int32_t el[8], cor[8];
    box_node_list(P, n, el, cor);
#pragma unroll
    for (int j = 0; j < 8; j++)
      if (el[j] >= 0) {
        s += vol[el[j]];
        rs += rho0[el[j]];
        c++;
      }
  } else {
    const int32_t b = P.off[n];
    c = P.off[n + 1] - b;
    for (int32_t k = 0; k < c; k++) {
      const int32_t e = P.slot[b + k] / NPE;
      s += vol[e];
      rs += rho0[e];
    }
  }
  const float2 nc = make_float2(1.0f / s, (float)(rs / c));
  M.nc[n] = nc;
  const float mass = (s * (1.0f / NPE)) * nc.y;
  M.mass[n] = mass;
  M.jr[n] = s * nc.x;
  S.s0[n] = s;
  S.voln[n] = (double)s / NPE;
  S.mass[n] = mass;
}

// The elements' FP64 copies: volume, initial volume, detJ, density.
template <int NPE>
__global__ void k_mix_init_elems(StepParams P, Fp64State S, const float *vol,
                                 const double *rho0) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= P.ne) return;
  const double v = vol[e];
  S.vol[e] = v;
  S.vol0[e] = v;
  S.detJ[e] = v / (NPE == 8 ? 8.0 : 1.0 / 6.0);
  S.rho[e] = rho0[e];
}

// Writes the mixed state into the FP64 arrays read back by the host.
template <int NPE>
__global__ void k_mix_export_nodes(StepParams P, MixState M, Fp64State S) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= P.nn) return;
  const int64_t np = P.np;
  for (int k = 0; k < 3; k++) {
    const float2 h = M.xh[k * np + n];
    const double x = (double)h.x + (double)h.y;
    S.x[k * np + n] = x;
    S.u[k * np + n] = x - M.x0[k * np + n];
    S.v[k * np + n] = M.v[k * np + n];
    S.pa[k * np + n] = M.pa[k * np + n];
    S.cf[k * np + n] = M.cf[k * np + n];
  }
  S.mass[n] = M.mass[n];
  S.jr[n] = M.jr[n];
  if (P.thermal) S.T[n] = (double)M.T[n].x + (double)M.T[n].y;
}

// Displacement (u = x - x0) or position of the mixed state straight into an
// AoS [nn][3] buffer, as k_mix_export_nodes forms them.
__global__ void k_mix_node_aos(StepParams P, MixState M, int displacement, double *out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * P.nn) return;
  const int64_t n = i / 3, k = i - 3 * n, np = P.np;
  const float2 h = M.xh[k * np + n];
  const double x = (double)h.x + (double)h.y;
  out[i] = displacement ? x - M.x0[k * np + n] : x;
}

template <int NPE>
__global__ void k_mix_export_elems(StepParams P, MixState M, Fp64State S, const float *vol) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= P.ne) return;
  const int64_t ne = P.ne;
  const MatF m = P.matf[P.emat ? P.emat[e] : 0];
  float J_avg = 0.f;
  for (int a = 0; a < NPE; a++) J_avg += M.jr[P.elnod[a * ne + e]];
  J_avg *= (1.0f / NPE);
  const float p = -m.K * ((J_avg < 0.f ? 0.2f : J_avg) - 1.0f);
  S.p[e] = p;
  S.vol[e] = vol[e];
  const float pls = M.pls[e];
  S.pls[e] = pls;
  // exported yield stress; for Johnson-Cook and GMT its value at unit rate
  // factor (edot = eps0_dot, resp. edot = 1 clamped to the GMT range) and the
  // material's uniform temperature
  S.sy[e] = (m.model == WF_MAT_HOLLOMON)
                ? ((pls + m.eps0 > m.eps1) ? m.hol_K * powf(pls + m.eps0, m.hol_m) : m.sy0)
            : (m.model == WF_MAT_JOHNSON_COOK) ? (m.sy0 + m.jc_B * powf(pls, m.jc_n)) * m.jc_Th
            : (m.model == WF_MAT_GMT)          ? gmt_law_f(gmt_consts<false>(m, 0.f), m.g_emin, m.g_emax,
                                                         m.g_rmin, m.g_rmax, pls, 1.0f, 1.0f).x
                                               : m.sy0 + m.H * pls;
  for (int c = 0; c < 6; c++) {
    const double t = M.tau[c * ne + e];
    S.tau[c * ne + e] = t;
    S.sig[c * ne + e] = (c < 3) ? t - (double)p : t;
  }
}

inline unsigned grid_for(int64_t n, int threads) {
  return (unsigned)((n + threads - 1) / threads);
}

}  // namespace

int mix_node_grid(int64_t nn) { return (int)grid_for(nn, kNodeThreads); }

void mix_init(const StepParams &P, const MixState &M, const Fp64State &S, float *vol,
              const double *rho0, cudaStream_t st) {
  k_mix_init_nodes<<<grid_for(P.nn, kNodeThreads), kNodeThreads, 0, st>>>(P, M, S);
  mix_geometry(P, M, vol, st, LaunchCfg{});
  if (P.npe == 8) {
    k_mix_init_nodal<8><<<grid_for(P.nn, kNodeThreads), kNodeThreads, 0, st>>>(P, M, S, vol, rho0);
    k_mix_init_elems<8><<<grid_for(P.ne, kElemThreads), kElemThreads, 0, st>>>(P, S, vol, rho0);
  } else {
    k_mix_init_nodal<4><<<grid_for(P.nn, kNodeThreads), kNodeThreads, 0, st>>>(P, M, S, vol, rho0);
    k_mix_init_elems<4><<<grid_for(P.ne, kElemThreads), kElemThreads, 0, st>>>(P, S, vol, rho0);
  }
}

namespace {

// Grid of a tunable launch: ceil(n / (bs * ept)) blocks, or with ept = 0 a
// persistent grid of (SMs x resident blocks per SM) that strides over the
// whole range. Occupancy and SM count are looked up once per instantiation.
template <typename Kernel>
unsigned tuned_grid(Kernel kernel, int bs, int ept, int64_t n) {
  const unsigned full = grid_for(n, bs);
  if (ept > 0) return grid_for(n, bs * ept);
  static std::mutex mu;
  static std::map<std::pair<const void *, int>, unsigned> cache;  // (kernel, device)
  int dev = 0;
  cudaGetDevice(&dev);
  unsigned g;
  {
    std::lock_guard<std::mutex> lock(mu);
    auto key = std::make_pair((const void *)kernel, dev);
    auto it = cache.find(key);
    if (it == cache.end()) {
      int sms = 0, per_sm = 0;
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, bs, 0);
      it = cache.emplace(key, (unsigned)(sms * (per_sm < 1 ? 1 : per_sm))).first;
    }
    g = it->second;
  }
  return g < full ? g : full;
}

template <int NPE, bool BOX>
void launch_geometry_box(const StepParams &P, const MixState &M, float *vol, cudaStream_t st,
                         LaunchCfg c) {
  switch (c.bs) {
    case 64: {
      const unsigned g = tuned_grid(k_mix_geometry<NPE, 64, BOX>, 64, c.ept, P.ne);
      k_mix_geometry<NPE, 64, BOX><<<g, 64, 0, st>>>(P, M, vol);
      break;
    }
    case 256: {
      const unsigned g = tuned_grid(k_mix_geometry<NPE, 256, BOX>, 256, c.ept, P.ne);
      k_mix_geometry<NPE, 256, BOX><<<g, 256, 0, st>>>(P, M, vol);
      break;
    }
    default: {
      const unsigned g = tuned_grid(k_mix_geometry<NPE, 128, BOX>, 128, c.ept, P.ne);
      k_mix_geometry<NPE, 128, BOX><<<g, 128, 0, st>>>(P, M, vol);
      break;
    }
  }
}

template <int NPE>
void launch_geometry(const StepParams &P, const MixState &M, float *vol, cudaStream_t st,
                     LaunchCfg c) {
  if (NPE == 8 && P.box) launch_geometry_box<NPE, true>(P, M, vol, st, c);
  else launch_geometry_box<NPE, false>(P, M, vol, st, c);
}

template <int NPE, bool BOX>
void launch_nodal_box(const StepParams &P, const MixState &M, const float *vol, cudaStream_t st,
                      LaunchCfg c) {
  switch (c.bs) {
    case 64: {
      const unsigned g = tuned_grid(k_mix_nodal<NPE, 64, BOX>, 64, c.ept, P.nn);
      k_mix_nodal<NPE, 64, BOX><<<g, 64, 0, st>>>(P, M, vol);
      break;
    }
    case 128: {
      const unsigned g = tuned_grid(k_mix_nodal<NPE, 128, BOX>, 128, c.ept, P.nn);
      k_mix_nodal<NPE, 128, BOX><<<g, 128, 0, st>>>(P, M, vol);
      break;
    }
    default: {
      const unsigned g = tuned_grid(k_mix_nodal<NPE, 256, BOX>, 256, c.ept, P.nn);
      k_mix_nodal<NPE, 256, BOX><<<g, 256, 0, st>>>(P, M, vol);
      break;
    }
  }
}

template <int NPE>
void launch_nodal(const StepParams &P, const MixState &M, const float *vol, cudaStream_t st,
                  LaunchCfg c) {
  if (NPE == 8 && P.box) launch_nodal_box<NPE, true>(P, M, vol, st, c);
  else launch_nodal_box<NPE, false>(P, M, vol, st, c);
}

template <int NPE, int LAW, bool TH, bool BOX>
void launch_elements_box(const StepParams &P, const MixState &M, cudaStream_t st, LaunchCfg c) {
  switch (c.bs) {
    case 64: {
      const unsigned g = tuned_grid(k_mix_elements<NPE, 64, LAW, TH, BOX>, 64, c.ept, P.ne);
      k_mix_elements<NPE, 64, LAW, TH, BOX><<<g, 64, 0, st>>>(P, M);
      break;
    }
    case 256: {
      const unsigned g = tuned_grid(k_mix_elements<NPE, 256, LAW, TH, BOX>, 256, c.ept, P.ne);
      k_mix_elements<NPE, 256, LAW, TH, BOX><<<g, 256, 0, st>>>(P, M);
      break;
    }
    default: {
      const unsigned g = tuned_grid(k_mix_elements<NPE, 128, LAW, TH, BOX>, 128, c.ept, P.ne);
      k_mix_elements<NPE, 128, LAW, TH, BOX><<<g, 128, 0, st>>>(P, M);
      break;
    }
  }
}

// Box variants are built for hexahedra without thermal coupling (the thermal
// element kernels keep the loaded connectivity).
template <int NPE, int LAW, bool TH>
void launch_elements_law(const StepParams &P, const MixState &M, cudaStream_t st, LaunchCfg c) {
  if constexpr (NPE == 8 && !TH) {
    if (P.box) {
      launch_elements_box<NPE, LAW, TH, true>(P, M, st, c);
      return;
    }
  }
  launch_elements_box<NPE, LAW, TH, false>(P, M, st, c);
}

template <int NPE>
void launch_elements(const StepParams &P, const MixState &M, cudaStream_t st, LaunchCfg c) {
  if (P.thermal) {
    if (P.mat_general)
      launch_elements_law<NPE, 1, true>(P, M, st, c);
    else
      launch_elements_law<NPE, 0, true>(P, M, st, c);
  } else if (P.mat_general) {
    launch_elements_law<NPE, 1, false>(P, M, st, c);
  } else {
    launch_elements_law<NPE, 0, false>(P, M, st, c);
  }
}

template <int NPE, int BS, int LAW>
cudaError_t cluster_launch(const StepParams &P, const MixState &M, float *vol, double *part,
                           int64_t nsteps, int blocks, cudaStream_t st, bool query, int *fits) {
  auto kern = P.thermal ? k_mix_cluster_run<NPE, BS, LAW, true>
                        : k_mix_cluster_run<NPE, BS, LAW, false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)blocks;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3((unsigned)blocks);
  cfg.blockDim = dim3(BS);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (query) {
    int n = 0;
    e = cudaOccupancyMaxActiveClusters(&n, kern, &cfg);
    *fits = (e == cudaSuccess) ? n : 0;
    return e;
  }
  return cudaLaunchKernelEx(&cfg, kern, P, M, vol, part, nsteps);
}

template <int NPE, int LAW>
cudaError_t cluster_dispatch_bs(const StepParams &P, const MixState &M, float *vol, double *part,
                                int64_t nsteps, int blocks, int bs, cudaStream_t st, bool query,
                                int *fits) {
  switch (bs) {
    case 64:
      return cluster_launch<NPE, 64, LAW>(P, M, vol, part, nsteps, blocks, st, query, fits);
    case 128:
      return cluster_launch<NPE, 128, LAW>(P, M, vol, part, nsteps, blocks, st, query, fits);
    default:
      return cluster_launch<NPE, 256, LAW>(P, M, vol, part, nsteps, blocks, st, query, fits);
  }
}

cudaError_t cluster_dispatch(const StepParams &P, const MixState &M, float *vol, double *part,
                             int64_t nsteps, int blocks, int bs, cudaStream_t st, bool query,
                             int *fits) {
  if (P.npe == 8)
    return P.mat_general
               ? cluster_dispatch_bs<8, 1>(P, M, vol, part, nsteps, blocks, bs, st, query, fits)
               : cluster_dispatch_bs<8, 0>(P, M, vol, part, nsteps, blocks, bs, st, query, fits);
  return P.mat_general
             ? cluster_dispatch_bs<4, 1>(P, M, vol, part, nsteps, blocks, bs, st, query, fits)
             : cluster_dispatch_bs<4, 0>(P, M, vol, part, nsteps, blocks, bs, st, query, fits);
}

}  // namespace

void mix_geometry(const StepParams &P, const MixState &M, float *vol, cudaStream_t st,
                  LaunchCfg c) {
  if (P.npe == 8) launch_geometry<8>(P, M, vol, st, c);
  else launch_geometry<4>(P, M, vol, st, c);
}

void mix_nodal(const StepParams &P, const MixState &M, const float *vol, cudaStream_t st,
               LaunchCfg c) {
  if (P.npe == 8) launch_nodal<8>(P, M, vol, st, c);
  else launch_nodal<4>(P, M, vol, st, c);
}

void mix_elements(const StepParams &P, const MixState &M, const float *, cudaStream_t st,
                  LaunchCfg c) {
  if (P.npe == 8) launch_elements<8>(P, M, st, c);
  else launch_elements<4>(P, M, st, c);
}

void mix_nodes(const StepParams &P, const MixState &M, cudaStream_t st, int node_grid) {
  if (P.npe == 8 && P.box)
    k_mix_nodes<8, true><<<node_grid, kNodeThreads, 0, st>>>(P, M);
  else if (P.npe == 8)
    k_mix_nodes<8, false><<<node_grid, kNodeThreads, 0, st>>>(P, M);
  else
    k_mix_nodes<4, false><<<node_grid, kNodeThreads, 0, st>>>(P, M);
}

static_assert(kSharedThreads == kNodeThreads, "the shared-node kernel runs node-kernel blocks");
int mix_shared_grid(const TileParams &T) {
  return std::max(1, (int)grid_for(T.nshared, kNodeThreads));
}

void mix_tile(const StepParams &P, const MixState &M, const TileParams &T, cudaStream_t st) {
  auto kern = P.mat_general ? k_mix_tile<1> : k_mix_tile<0>;
  static std::mutex mu;
  static std::map<std::pair<const void *, int>, bool> set;   // (kernel, device)
  int dev = 0;
  cudaGetDevice(&dev);
  {
    std::lock_guard<std::mutex> lock(mu);
    bool &done = set[std::make_pair((const void *)kern, dev)];
    if (!done) {
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTileSmem);
      done = true;
    }
  }
  kern<<<(unsigned)T.ntiles, kTileElems, kTileSmem, st>>>(P, M, T);
}

void mix_shared(const StepParams &P, const MixState &M, const TileParams &T, cudaStream_t st) {
  if (P.box)
    k_mix_shared<true><<<(unsigned)mix_shared_grid(T), kNodeThreads, 0, st>>>(P, M, T);
  else
    k_mix_shared<false><<<(unsigned)mix_shared_grid(T), kNodeThreads, 0, st>>>(P, M, T);
}

namespace {
using SweepKernel = void (*)(StepParams, MixState, SweepParams);
template <int CY>
SweepKernel sweep_kernel_cy(const StepParams &P) {
  return P.mat_general ? k_mix_sweep<1, CY> : k_mix_sweep<0, CY>;
}
// The kernel, its block size and shared memory for W.cy (set up once per
// kernel and device: the dynamic shared memory above the default 48 KB).
SweepKernel sweep_kernel(const StepParams &P, const SweepParams &W, int *threads, size_t *smem) {
  SweepKernel k;
  if (W.cy == 4) {
    k = sweep_kernel_cy<4>(P);
    *threads = SweepShape<4>::threads;
    *smem = SweepShape<4>::smem;
  } else {
    k = sweep_kernel_cy<8>(P);
    *threads = SweepShape<8>::threads;
    *smem = SweepShape<8>::smem;
  }
  static std::mutex mu;
  static std::map<std::pair<const void *, int>, bool> set;   // (kernel, device)
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  bool &done = set[std::make_pair((const void *)k, dev)];
  if (!done) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem);
    done = true;
  }
  return k;
}
}  // namespace

int sweep_columns(const StepParams &P, SweepParams &W) {
  if (W.cy != 4) W.cy = 8;
  W.ncx = (P.bx + 1 + (kSwEX - 1) - 1) / (kSwEX - 1);
  W.ncy = (P.by + 1 + W.cy - 1) / W.cy;
  return W.ncx * W.ncy;
}

bool sweep_fits(const StepParams &P, const SweepParams &W) {
  int threads = 0;
  size_t smem = 0;
  const SweepKernel k = sweep_kernel(P, W, &threads, &smem);
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k, threads, smem) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return blocks >= 1;
}

void mix_sweep(const StepParams &P, const MixState &M, const SweepParams &W, cudaStream_t st) {
  int threads = 0;
  size_t smem = 0;
  const SweepKernel k = sweep_kernel(P, W, &threads, &smem);
  k<<<(unsigned)(W.ncx * W.ncy), threads, smem, st>>>(P, M, W);
}

int flow_grid(const StepParams &P) {
  auto kern = P.mat_general ? k_mix_flow<1> : k_mix_flow<0>;
  // the stage table's shared memory at the largest mesh the step takes
  const size_t smem = sizeof(int) * (kFlowMaxLayers + 20);
  static std::mutex mu;
  static std::map<std::pair<const void *, int>, bool> set;   // (kernel, device)
  int dev = 0;
  cudaGetDevice(&dev);
  {
    std::lock_guard<std::mutex> lock(mu);
    bool &done = set[std::make_pair((const void *)kern, dev)];
    if (!done) {
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      done = true;
    }
  }
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, kFlowThreads, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return per * P.sms;
}

void flow_stages(const StepParams &P, int tile, int lag, bool split, std::vector<int> &first,
                 FlowParams &F) {
  const int64_t exy = (int64_t)P.bx * P.by, pxy = (int64_t)(P.bx + 1) * (P.by + 1);
  const int bz = P.bz;
  // the light phases (geometry, nodal) in tiles four times larger
  F.tsize[0] = F.tsize[1] = 4 * tile;
  F.tsize[2] = F.tsize[3] = tile;
  const int64_t per[kFlowKinds] = {exy, pxy, exy, pxy};
  for (int q = 0; q < kFlowKinds; q++)
    F.ntiles[q] = (int)((per[q] + F.tsize[q] - 1) / F.tsize[q]);
  F.split = split ? 1 : 0;
  if (split) {
    // geometry and nodal phases done before the launch: element tiles wait on
    // nothing (their items need zero tiles of the nodal phase), node-update
    // tiles lag them by `lag` layers
    F.ntiles[0] = F.ntiles[1] = 0;
    F.off[0] = F.off[1] = F.off[2] = 0;
    F.off[3] = lag;
  } else {
    // stage offsets 0, lag/3, 2 lag/3, lag: each phase a third of the lag
    // behind the one it reads
    F.off[0] = 0;
    F.off[1] = std::max(1, lag / 3);
    F.off[2] = std::max(F.off[1] + 1, 2 * lag / 3);
    F.off[3] = std::max(F.off[2] + 1, lag);
  }
  F.nstages = bz + F.off[3] + 1;
  first.assign(F.nstages + 1, 0);
  int t = 0;
  for (int s = 0; s < F.nstages; s++) {
    first[s] = t;
    for (int q = 0; q < kFlowKinds; q++) {
      const int l = s - F.off[q], lmax = (q == 0 || q == 2) ? bz - 1 : bz;
      if (l >= 0 && l <= lmax) t += F.ntiles[q];
    }
  }
  first[F.nstages] = t;
  F.total = t;
  F.bz1 = bz + 1;
  F.ncnt = 1 + kFlowKinds * F.bz1;
}

void mix_flow(const StepParams &P, const MixState &M, float *vol, const FlowParams &F,
              cudaStream_t st) {
  auto kern = P.mat_general ? k_mix_flow<1> : k_mix_flow<0>;
  kern<<<(unsigned)F.grid, kFlowThreads, sizeof(int) * (F.nstages + 1), st>>>(P, M, vol, F);
  k_mix_flow_finish<<<1, kFlowThreads, 0, st>>>(P, F);
}

int mix_cluster_fits(const StepParams &P, const MixState &M, float *vol, int blocks, int bs) {
  int fits = 0;
  if (cluster_dispatch(P, M, vol, nullptr, 0, blocks, bs, nullptr, true, &fits) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return fits;
}

cudaError_t mix_cluster_run(const StepParams &P, const MixState &M, float *vol, double *part,
                            int64_t nsteps, int blocks, int bs, cudaStream_t st) {
  return cluster_dispatch(P, M, vol, part, nsteps, blocks, bs, st, false, nullptr);
}

void mix_predict(const StepParams &P, const MixState &M, cudaStream_t st) {
  k_mix_predict<<<grid_for(P.nn, kNodeThreads), kNodeThreads, 0, st>>>(P, M);
}

void mix_node_aos(const StepParams &P, const MixState &M, bool displacement, double *out,
                  cudaStream_t st) {
  k_mix_node_aos<<<grid_for(3 * P.nn, kNodeThreads), kNodeThreads, 0, st>>>(P, M, displacement ? 1 : 0,
                                                                             out);
}

void mix_export(const StepParams &P, const MixState &M, const Fp64State &S, const float *vol,
                cudaStream_t st) {
  if (P.npe == 8) {
    k_mix_export_nodes<8><<<grid_for(P.nn, kNodeThreads), kNodeThreads, 0, st>>>(P, M, S);
    k_mix_export_elems<8><<<grid_for(P.ne, kElemThreads), kElemThreads, 0, st>>>(P, M, S, vol);
  } else {
    k_mix_export_nodes<4><<<grid_for(P.nn, kNodeThreads), kNodeThreads, 0, st>>>(P, M, S);
    k_mix_export_elems<4><<<grid_for(P.ne, kElemThreads), kElemThreads, 0, st>>>(P, M, S, vol);
  }
}

}  // namespace wf
