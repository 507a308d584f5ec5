// FP64 step kernels: the reference's arithmetic, operation for operation.
//
// This translation unit is compiled with --fmad=false so that every
// expression rounds exactly as the reference CPU code does with FMA
// contraction off (the reference build passes --fmad=false to nvcc,
// src/common/CMakeLists.txt:16). One step is four launches:
//   geometry  (element): J, detJ, volume             -> vol
//   nodal     (node)   : volume sums, lumped mass, J ratio
//   elements  (element): dN, D/W, pressure, Jaumann + radial return,
//                        B^T sigma, hourglass        -> element forces
//   nodes     (node)   : deterministic gather of element forces over the
//                        node->element lists, contact, acceleration, BCs,
//                        Chung-Hulbert corrector, position update and the
//                        next step's predictor; reaction sum (last block).
#include "wf_internal.cuh"
#include "wf_trimesh.cuh"

namespace wf {
namespace {

constexpr int kElemThreads = 128;
constexpr int kNodeThreads = 256;

// Flanagan-Belytschko hourglass base vectors of the 8-node hexahedron
// (test_1el_3D.cpp:166-169), as compile-time signs.
__device__ __forceinline__ constexpr int hg_sig(int j, int a) {
  constexpr signed char t[4][8] = {{1, 1, -1, -1, -1, -1, 1, 1},
                                   {1, -1, -1, 1, -1, 1, 1, -1},
                                   {1, -1, 1, -1, 1, -1, 1, -1},
                                   {-1, 1, -1, 1, 1, -1, 1, -1}};
  return t[j][a];
}

__device__ __forceinline__ double det3(const double J[3][3]) {
  // Matrix::calcDet (include/common/Matrix.h:593-620)
  return J[0][0] * J[1][1] * J[2][2] - J[0][0] * J[1][2] * J[2][1] -
         J[0][1] * J[1][0] * J[2][2] + J[0][1] * J[1][2] * J[2][0] +
         J[0][2] * J[1][0] * J[2][1] - J[0][2] * J[1][1] * J[2][0];
}

// Jacobian of the element from its node coordinates
// (Domain_d.C:1822-1830 hexahedron, :1866-1870 tetrahedron).
template <int NPE>
__device__ __forceinline__ void jacobian(const double (&x2)[NPE][3], double J[3][3]) {
  if constexpr (NPE == 8) {
#pragma unroll
    for (int k = 0; k < 3; k++) {
      J[0][k] = 0.125 * (-x2[0][k] + x2[1][k] + x2[2][k] - x2[3][k] - x2[4][k] + x2[5][k] +
                         x2[6][k] - x2[7][k]);
      J[1][k] = 0.125 * (-x2[0][k] - x2[1][k] + x2[2][k] + x2[3][k] - x2[4][k] - x2[5][k] +
                         x2[6][k] + x2[7][k]);
      J[2][k] = 0.125 * (-x2[0][k] - x2[1][k] - x2[2][k] - x2[3][k] + x2[4][k] + x2[5][k] +
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

// dN/dx * detJ from the adjugate of J (AdjMat, Matrix.h:694-727;
// Domain_d.C:1842-1851 hexahedron, :1881-1887 tetrahedron).
template <int NPE>
__device__ __forceinline__ void shape_derivs(const double J[3][3], double dH[3][NPE]) {
  double inv[3][3];
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
    const double a0 = inv[k][0], a1 = inv[k][1], a2 = inv[k][2];
    if constexpr (NPE == 8) {
      dH[k][0] = 0.125 * (-a0 - a1 - a2);
      dH[k][1] = 0.125 * (a0 - a1 - a2);
      dH[k][2] = 0.125 * (a0 + a1 - a2);
      dH[k][3] = 0.125 * (-a0 + a1 - a2);
      dH[k][4] = 0.125 * (-a0 - a1 + a2);
      dH[k][5] = 0.125 * (a0 - a1 + a2);
      dH[k][6] = 0.125 * (a0 + a1 + a2);
      dH[k][7] = 0.125 * (-a0 + a1 + a2);
    } else {
      dH[k][0] = -a0 - a1 - a2;
      dH[k][1] = a0;
      dH[k][2] = a1;
      dH[k][3] = a2;
    }
  }
}

template <int NPE>
__device__ __forceinline__ double weight() {
  return NPE == 8 ? 8.0 : 1.0 / 6.0;
}

template <int NPE>
__device__ __forceinline__ void gather_x(const StepParams &P, const double *x, int64_t e,
                                         double (&x2)[NPE][3], int32_t (&nid)[NPE]) {
#pragma unroll
  for (int a = 0; a < NPE; a++) nid[a] = __ldg(&P.elnod[a * P.ne + e]);
#pragma unroll
  for (int a = 0; a < NPE; a++) {
    x2[a][0] = __ldg(&x[nid[a]]);
    x2[a][1] = __ldg(&x[P.np + nid[a]]);
    x2[a][2] = __ldg(&x[2 * P.np + nid[a]]);
  }
}

// ---------------------------------------------------------------------------
// geometry: vol = 0.0 + detJ * w * 1.0 (Mechanical.C:264-293)
template <int NPE>
__global__ void __launch_bounds__(kElemThreads) k_fp64_geometry(StepParams P, Fp64State S,
                                                           int store_detj) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= P.ne) return;
  double x2[NPE][3];
  int32_t nid[NPE];
  gather_x<NPE>(P, S.x, e, x2, nid);
  double J[3][3];
  jacobian<NPE>(x2, J);
  double detJ = det3(J);
  double v = 0.0;
  v += detJ * weight<NPE>() * 1.0;
  S.vol[e] = v;
  if (store_detj) S.detJ[e] = detJ;
}

// ---------------------------------------------------------------------------
// nodal: CalcNodalVol (Mechanical.C:1555-1572), CalcNodalMassFromVol
// (:1576-1601) and the nodal volume ratio of calcElemPressure (:694-705).
// init_mode 1 also forms the constant sum of initial volumes.
// BOX: the node's elements computed from its indices (box meshes of a mixed
// domain, whose preamble runs this kernel), in the lists' order.
template <int NPE, bool BOX>
__global__ void __launch_bounds__(kNodeThreads) k_fp64_nodal(StepParams P, Fp64State S,
                                                        int init_mode) {
  int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= P.nn) return;
  int32_t b = 0, c = 0;
  int32_t bel[8];
  if constexpr (BOX) {
    int32_t el[8], cor[8];
    box_node_list(P, n, el, cor);
#pragma unroll
    for (int j = 0; j < 8; j++)
      if (el[j] >= 0) bel[c++] = el[j];
  } else {
    b = __ldg(&P.off[n]);
    c = __ldg(&P.off[n + 1]) - b;
  }
  auto elem = [&](int32_t k) -> int32_t {
    if constexpr (BOX)
      return bel[k];
    else
      return __ldg(&P.slot[b + k]) / NPE;
  };
  double s = 0.0, s0 = 0.0;
  for (int32_t k = 0; k < c; k++) {
    int32_t e = elem(k);
    s += __ldg(&S.vol[e]);
    if (init_mode) s0 += __ldg(&S.vol0[e]);
  }
  if (init_mode) S.s0[n] = s0;
  else s0 = S.s0[n];
  double voln = s;
  voln /= NPE;
  S.voln[n] = voln;
  if (P.mass_mode == 0 || init_mode) {
    double mass = 0.0;
    const double f = 1.0;
    for (int32_t k = 0; k < c; k++) {
      int32_t e = elem(k);
      mass += f * __ldg(&S.rho[e]) * voln / c;
    }
    S.mass[n] = mass;
  }
  S.jr[n] = s / s0;
}

// GMT law (CalcGMTYieldStress and CalcGMTTangentModulus, Material.cuh:417-478)
// in FP64: strain e, strain rate r and temperature T clamped to the
// material's ranges, then the reference's products in its order; mp points to
// the material in global memory. Not inlined: the law's temporaries stay out
// of the element kernel's register budget.
static __device__ __noinline__ double gmt_sy(double e, double r, double T, const MatDev *mp) {
  const MatDev &m = *mp;
  e = clamp_range(e, m.g_emin, m.g_emax);
  r = clamp_range(r, m.g_rmin, m.g_rmax);
  T = clamp_range(T, m.g_Tmin, m.g_Tmax);
  return m.g_C1 * exp(m.g_C2 * T) * pow(e, m.g_n1 * T + m.g_n2) * exp((m.g_I1 * T + m.g_I2) / e) *
         pow(r, m.g_m1 * T + m.g_m2);
}
static __device__ __noinline__ double gmt_et(double e, double r, double T, const MatDev *mp) {
  const MatDev &m = *mp;
  e = clamp_range(e, m.g_emin, m.g_emax);
  r = clamp_range(r, m.g_rmin, m.g_rmax);
  T = clamp_range(T, m.g_Tmin, m.g_Tmax);
  return m.g_C1 * exp(m.g_C2 * T) * pow(r, m.g_m1 * T + m.g_m2) * pow(e, T * m.g_n1 + m.g_n2 - 2.0) *
         (-m.g_I1 * T - m.g_I2 + e * (m.g_n1 * T + m.g_n2)) * exp((m.g_I1 * T + m.g_I2) / e);
}

__device__ __forceinline__ double hollomon_sy(double strain, const MatDev &m) {
  if (strain + m.eps0 > m.eps1) return m.hol_K * pow(strain + m.eps0, m.hol_m);
  return m.sy0;
}
__device__ __forceinline__ double hollomon_et(double strain, const MatDev &m) {
  if (strain + m.eps0 > m.eps1) return m.hol_K * m.hol_m * pow(strain + m.eps0, (m.hol_m - 1.0));
  return 0.;
}

// ---------------------------------------------------------------------------
// elements: calcElemJAndDerivatives, calcElemStrainRates (Mechanical.C:41-126),
// calcElemPressure (:691-819) or calcElemPressureANP (:1220-1250),
// CalcStressStrain (:1664-1839), calcArtificialViscosity (:1948-1977),
// calcElemForces (:375-481) and the 3-D viscous hourglass forces.
// TH: thermal coupling (a separate instantiation keeps the common case's
// register allocation).
template <int NPE, bool TH>
__global__ void __launch_bounds__(kElemThreads) k_fp64_elements(StepParams P, Fp64State S) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= P.ne) return;
  const int64_t ne = P.ne;
  int32_t nid[NPE];
  double dH[3][NPE];
  double detJ;
  {
    double x2[NPE][3];
    gather_x<NPE>(P, S.x, e, x2, nid);
    double J[3][3];
    jacobian<NPE>(x2, J);
    shape_derivs<NPE>(J, dH);
    detJ = det3(J);
  }
  double vol = 0.0;
  vol += detJ * weight<NPE>() * 1.0;
  const int32_t mat_id = P.emat ? __ldg(&P.emat[e]) : 0;
  const MatDev m = P.mats[mat_id];

  // strain rate and spin (str_rate / rot_rate, upper triangle)
  double s00 = 0.0, s11 = 0.0, s22 = 0.0, s01 = 0.0, s12 = 0.0, s02 = 0.0;
  double w01 = 0.0, w12 = 0.0, w02 = 0.0;
  double hm[3][4];
#pragma unroll
  for (int k = 0; k < 3; k++)
#pragma unroll
    for (int j = 0; j < 4; j++) hm[k][j] = 0.0;
  double div_v = 0.0;
  const double f = 1.0 / detJ;
#pragma unroll
  for (int a = 0; a < NPE; a++) {
    const double v0 = __ldg(&S.vp[nid[a]]);
    const double v1 = __ldg(&S.vp[P.np + nid[a]]);
    const double v2 = __ldg(&S.vp[2 * P.np + nid[a]]);
    const double d0 = dH[0][a], d1 = dH[1][a], d2 = dH[2][a];
    s00 = s00 + d0 * f * v0;
    s11 = s11 + d1 * f * v1;
    s22 = s22 + d2 * f * v2;
    s01 = s01 + f * (d1 * v0 + d0 * v1);
    w01 = w01 + f * (d1 * v0 - d0 * v1);
    s12 = s12 + f * (d2 * v1 + d1 * v2);
    s02 = s02 + f * (d2 * v0 + d0 * v2);
    w12 = w12 + f * (d2 * v1 - d1 * v2);
    w02 = w02 + f * (d2 * v0 - d0 * v2);
    if (P.stab_on) div_v += d0 * v0 + d1 * v1 + d2 * v2;
    if constexpr (NPE == 8) {
      if (P.hg_on) {
#pragma unroll
        for (int j = 0; j < 4; j++) {
          // v * Gamma with Gamma = +-1 is exact: add or subtract
          if (hg_sig(j, a) > 0) {
            hm[0][j] += v0; hm[1][j] += v1; hm[2][j] += v2;
          } else {
            hm[0][j] -= v0; hm[1][j] -= v1; hm[2][j] -= v2;
          }
        }
      }
    }
  }
  s01 = s01 * 0.5; s02 = s02 * 0.5; s12 = s12 * 0.5;
  w01 = w01 * 0.5; w02 = w02 * 0.5; w12 = w12 * 0.5;
  const long long step = TH ? P.st->step : 0;
  if constexpr (TH) {
    // calcThermalExpansion (Thermal.C:163-178): the previous step's
    // element-node temperature rates read at the element's node ids, as the
    // reference indexes them
    const double *prev = S.dte + ((step + 1) & 1) * ne * NPE;
    double g = 0.0;
#pragma unroll
    for (int a = 0; a < NPE; a++) g += 1.0 / NPE * prev[nid[a]];
    const double c = m.exp_T * g;
    s00 = s00 - c;
    s11 = s11 - c;
    s22 = s22 - c;
  }

  // pressure
  double p;
  if (P.press_alg == 1) {
    p = S.p[e];
    for (int a = 0; a < NPE; a++) p += P.k0 * (1.0 - __ldg(&S.jr[nid[a]]));
    p *= 0.25 * NPE;
  } else {
    const double K = m.K;
    const double J_local = vol / __ldg(&S.vol0[e]);
    double J_avg = 0.0;
#pragma unroll
    for (int a = 0; a < NPE; a++) J_avg += __ldg(&S.jr[nid[a]]);
    J_avg /= NPE;
    if (!P.stab_on) {
      // All stabilisation parameters zero: J_bar = 0 * J_local + 1 * J_avg
      // = J_avg and the 0 * log(J_bar) term adds only a signed zero.
      double J_bar = J_avg;
      if (J_bar < 0.0) J_bar = 0.2;
      p = -K * (J_bar - 1.0);
    } else {
      const double *st = P.stab;
      const double rho_e = S.rho[e];
      const double h = pow(vol, 1.0 / 3.0);
      bool is_contact = false;
      if (P.contact) {
        for (int a = 0; a < NPE; a++) {
          double c0 = S.cf[nid[a]], c1 = S.cf[P.np + nid[a]], c2 = S.cf[2 * P.np + nid[a]];
          if (c0 * c0 + c1 * c1 + c2 * c2 > 0) { is_contact = true; break; }
        }
      }
      double alpha = is_contact ? st[1] : st[0];
      double J_bar = alpha * J_local + (1 - alpha) * J_avg;
      if (J_bar < st[9]) J_bar = 0.2;
      double p_physical = -K * (st[6] * log(J_bar) + (1.0 - st[6]) * (J_bar - 1.0));
      double c = sqrt(K / rho_e);
      double tau = h / (2.0 * c);
      double p_pspg = 0.0;
      double p_hg = (is_contact ? st[3] : st[2]) * K * fabs(J_local - J_avg);
      double p_q = 0.0;
      if (div_v < 0.0) {
        double t1 = st[7] * tau * div_v * K, t2 = st[8] * K;
        p_pspg = (t2 < t1) ? t2 : t1;
        double q1 = st[4] * rho_e * h * c * (-div_v);
        double delta_J = 1.0 - J_local;
        double q2 = st[5] * K * delta_J;
        p_q = is_contact ? 0.5 * (q1 + q2) : ((q1 < q2) ? q2 : q1);
      }
      p = p_physical + p_pspg + p_hg + p_q;
    }
  }

  // Jaumann rate + radial return (CalcStressStrain). The tensor3 algebra of
  // the reference (Tensor3.C) written out on the six stored components: the
  // addends that multiply an exact zero of the spin or of the identity's
  // off-diagonal are dropped, which leaves every value unchanged (only the
  // sign of an exact zero could differ) and saves FP64 instructions.
  const double dt = P.espec ? P.spec_dt[P.espec[e]] : P.dt;
  double t0 = S.tau[e], t1 = S.tau[ne + e], t2 = S.tau[2 * ne + e];
  double t3 = S.tau[3 * ne + e], t4 = S.tau[4 * ne + e], t5 = S.tau[5 * ne + e];
  {
    // SRT = tau * Trans(W), RS = W * tau with the product of Tensor3.C:290-303
    const double srt0 = t3 * w01 + t5 * w02;    // xx
    const double srt1 = t3 * w01 - t4 * w12;    // yy
    const double srt2 = t5 * w02 + t4 * w12;    // zz
    const double srt3 = t0 * w01 - t5 * w12;    // xy
    const double srt4 = t3 * w02 + t1 * w12;    // yz
    const double srt5 = t0 * w02 + t3 * w12;    // xz
    const double rs0 = w01 * t3 + w02 * t5;
    const double rs1 = w12 * t4 - w01 * t3;
    const double rs2 = -(w02 * t5 + w12 * t4);
    const double rs3 = w01 * t1 + w02 * t4;
    const double rs4 = w12 * t2 - w01 * t5;
    const double rs5 = w01 * t4 + w02 * t2;
    const double c = 1.0 / 3.0 * (s00 + s11 + s22);
    const double g2 = 2.0 * m.G;
    t0 = t0 + (((s00 - c) * g2 + srt0) + rs0) * dt;
    t1 = t1 + (((s11 - c) * g2 + srt1) + rs1) * dt;
    t2 = t2 + (((s22 - c) * g2 + srt2) + rs2) * dt;
    t3 = t3 + ((s01 * g2 + srt3) + rs3) * dt;
    t4 = t4 + ((s12 * g2 + srt4) + rs4) * dt;
    t5 = t5 + ((s02 * g2 + srt5) + rs5) * dt;
  }
  // sigma_trial = -p I + tau; s_trial = sigma_trial - tr/3 I
  const double st0 = t0 - p, st1 = t1 - p, st2 = t2 - p;
  const double c2 = (1.0 / 3.0) * (st0 + st1 + st2);
  const double d0s = st0 - c2, d1s = st1 - c2, d2s = st2 - c2;
  const double J2 = 0.5 * (d0s * d0s + 2.0 * t3 * t3 + 2.0 * t5 * t5 + d1s * d1s +
                           2.0 * t4 * t4 + d2s * d2s);
  const double sig_trial = sqrt(3.0 * J2);
  double pls = S.pls[e];
  double sy;
  double eff = 0.0;
  double jTh = m.jc_Th;
  double temp = m.g_T;  // GMT element temperature
  if (m.model == WF_MAT_JOHNSON_COOK || m.model == WF_MAT_GMT) {
    // effective strain rate (Mechanical.C:1701-1705)
    eff = sqrt(0.5 * ((s00 - s11) * (s00 - s11) + (s11 - s22) * (s11 - s22) +
                      (s22 - s00) * (s22 - s00)) +
               3.0 * (s01 * s01 + s12 * s12 + s02 * s02));
    if constexpr (TH) {
      // element temperature: mean of its node temperatures (the reference
      // reads T[e], a node array indexed by element)
      double ts = 0.0;
#pragma unroll
      for (int a = 0; a < NPE; a++) ts += S.T[nid[a]];
      temp = ts / NPE;
      if (m.model == WF_MAT_JOHNSON_COOK) jTh = 1.0 - pow((temp - m.jc_Tt) / (m.jc_Tm - m.jc_Tt), m.jc_m);
    }
    if (m.model == WF_MAT_JOHNSON_COOK) {
      // CalcJohnsonCookYieldStress (Material.cuh:377-392)
      const double sr = (eff == 0.0) ? 1.e-5 : eff;
      sy = (m.sy0 + m.jc_B * pow(pls, m.jc_n)) * (1.0 + m.jc_C * log(sr / m.jc_eps0)) * jTh;
    } else {
      sy = gmt_sy(pls, eff, temp, P.mats + mat_id);
    }
  } else if (m.model == WF_MAT_HOLLOMON) {
    sy = hollomon_sy(pls, m);
  } else {
    sy = m.sy0 + m.H * pls;
  }
  double dep = 0.0;
  if (sy < sig_trial) {
    double H;
    if (m.model == WF_MAT_JOHNSON_COOK) {
      // CalcJohnsonCookTangentModulus (Material.cuh:397-410) at min(edot, m_max_edot)
      const double er = (P.max_edot < eff) ? P.max_edot : eff;
      H = (pls > 0.) ? m.jc_n * m.jc_B * pow(pls, m.jc_n - 1.) *
                           (1.0 + m.jc_C * log(er / m.jc_eps0)) * jTh
                     : m.E * 0.1;
    } else if (m.model == WF_MAT_GMT) {
      H = gmt_et(pls, (P.max_edot < eff) ? P.max_edot : eff, temp, P.mats + mat_id);
    } else {
      H = (m.model == WF_MAT_HOLLOMON) ? hollomon_et(pls, m) : m.H;
    }
    const double G = m.G;
    const double dgamma = (sig_trial - sy) / (3.0 * G + H);
    const double factor = 1.0 - (3.0 * G * dgamma) / sig_trial;
    t0 = d0s * factor; t1 = d1s * factor; t2 = d2s * factor;
    t3 = t3 * factor; t4 = t4 * factor; t5 = t5 * factor;
    pls += dgamma;
    dep = dgamma;
  }
  double SG[6] = {t0 - p, t1 - p, t2 - p, t3, t4, t5};
  // plastic heat (Mechanical.C:1783-1810): m_plheatfraction sigma : (d eps_p / dt), the
  // plastic strain increment along the returned stress, shear terms doubled
  double q_pl = 0.0;
  if (TH && dep > 0.0) {
    const double f = dep / sy;
    const double idt = 1. / dt;
    const double ixx = f * (SG[0] - 0.5 * (SG[1] + SG[2]));
    const double iyy = f * (SG[1] - 0.5 * (SG[0] + SG[2]));
    const double izz = f * (SG[2] - 0.5 * (SG[0] + SG[1]));
    const double ixy = 1.5 * f * (SG[3]), ixz = 1.5 * f * (SG[5]), iyz = 1.5 * f * (SG[4]);
    q_pl = P.plheat_frac * (SG[0] * (ixx * idt) + 2.0 * SG[3] * (ixy * idt) +
                            2.0 * SG[5] * (ixz * idt) + SG[1] * (iyy * idt) +
                            2.0 * SG[4] * (iyz * idt) + SG[2] * (izz * idt));
  }
  // total strain: eps = eps + dt * D
  {
    double e0 = S.eps[e], e1 = S.eps[ne + e], e2 = S.eps[2 * ne + e];
    double e3 = S.eps[3 * ne + e], e4 = S.eps[4 * ne + e], e5 = S.eps[5 * ne + e];
    S.eps[e] = e0 + s00 * dt;
    S.eps[ne + e] = e1 + s11 * dt;
    S.eps[2 * ne + e] = e2 + s22 * dt;
    S.eps[3 * ne + e] = e3 + s01 * dt;
    S.eps[4 * ne + e] = e4 + s12 * dt;
    S.eps[5 * ne + e] = e5 + s02 * dt;
  }
  // artificial viscosity (serial in the reference; per element here)
  if (P.av_on) {
    const double c = sqrt(m.K / S.rho[e]);
    const double eps_v = (s00 + s11 + s22);
    if (fabs(eps_v) > 1e-12) {
      const double l = pow(vol, 1.0 / 3.0);
      double q = P.av[0] * c * fabs(eps_v) * l + P.av[1] * pow(eps_v * l, 2);
      q = (1e9 < q) ? 1e9 : q;
      const double qs = (eps_v > 0) ? -q : q;
      SG[0] += qs;
      SG[1] += qs;
      SG[2] += qs;
    }
  }
  S.p[e] = p;
  S.pls[e] = pls;
  S.sy[e] = sy;
  const double sg0 = SG[0], sg1 = SG[1], sg2 = SG[2], sg3 = SG[3], sg4 = SG[4], sg5 = SG[5];
  S.sig[e] = sg0; S.sig[ne + e] = sg1; S.sig[2 * ne + e] = sg2;
  S.sig[3 * ne + e] = sg3; S.sig[4 * ne + e] = sg4; S.sig[5 * ne + e] = sg5;
  S.tau[e] = t0; S.tau[ne + e] = t1; S.tau[2 * ne + e] = t2;
  S.tau[3 * ne + e] = t3; S.tau[4 * ne + e] = t4; S.tau[5 * ne + e] = t5;
  S.sr[e] = s00; S.sr[ne + e] = s11; S.sr[2 * ne + e] = s22;
  S.sr[3 * ne + e] = s01; S.sr[4 * ne + e] = s12; S.sr[5 * ne + e] = s02;
  S.rr[e] = 0.0; S.rr[ne + e] = 0.0; S.rr[2 * ne + e] = 0.0;
  S.rr[3 * ne + e] = w01; S.rr[4 * ne + e] = w12; S.rr[5 * ne + e] = w02;

  // element forces f = w * B^T sigma (3-D branch of calcElemForces)
  double *fe = &S.fe[e * NPE * 3];
  const double w = weight<NPE>();
#pragma unroll
  for (int a = 0; a < NPE; a++) {
    const double d0 = dH[0][a], d1 = dH[1][a], d2 = dH[2][a];
    // 0.0 + d * sigma * 1.0 of the reference is d * sigma (exact)
    double f0 = d0 * sg0, f1 = d1 * sg1, f2 = d2 * sg2;
    f0 += d1 * sg3 + d2 * sg5;
    f1 += d0 * sg3 + d2 * sg4;
    f2 += d1 * sg4 + d0 * sg5;
    fe[3 * a] = f0 * w;
    fe[3 * a + 1] = f1 * w;
    fe[3 * a + 2] = f2 * w;
  }
  if constexpr (NPE == 8) {
    if (P.hg_on) {
      const double ch = P.hg_coef * pow(vol, 0.6666666) * S.rho[e] * 0.25 * m.cs0;
      double chm[3][4];
#pragma unroll
      for (int k = 0; k < 3; k++)
#pragma unroll
        for (int j = 0; j < 4; j++) chm[k][j] = ch * hm[k][j];
      double *fh = &S.fhg[e * 24];
#pragma unroll
      for (int i = 0; i < 8; i++) {
#pragma unroll
        for (int k = 0; k < 3; k++) {
          // acc -= ch * h * Gamma with Gamma = +-1: exact sign flips
          double acc = 0.0;
#pragma unroll
          for (int j = 0; j < 4; j++) {
            if (hg_sig(j, i) > 0) acc -= chm[k][j];
            else acc += chm[k][j];
          }
          fh[3 * i + k] = acc;
        }
      }
    }
  }
  if constexpr (TH) {
    // Domain_d::ThermalCalcs (Thermal.C:27-106), element part: conduction
    // K_ij = (sum_d dN_i detJ dN_j detJ) k_T / detJ w against the node
    // temperatures, and the plastic heat 0.9 q vol split evenly over the nodes
    double Te[NPE];
#pragma unroll
    for (int a = 0; a < NPE; a++) Te[a] = S.T[nid[a]];
    const double heat = 0.9 * q_pl;
    const double elem_pow = heat * vol;
    const double pow_per_node = elem_pow / NPE;
    double *cur = S.dte + (step & 1) * ne * NPE + e * NPE;
    const double wt = weight<NPE>();
    for (int i = 0; i < NPE; i++) {
      double dT = 0.0;
      for (int k = 0; k < NPE; k++) {
        double kk = 0.0;
#pragma unroll
        for (int dd = 0; dd < 3; dd++) kk += dH[dd][i] * dH[dd][k];
        dT += kk * m.k_T / detJ * wt * Te[k];
      }
      const double mi = S.mass[nid[i]];
      const double m_inv = 1.0 / mi;
      double r = -m_inv * dT;
      r += pow_per_node / (mi * m.cp_T);
      cur[i] = r;
    }
  }
}

// ---------------------------------------------------------------------------
// deterministic block sum (fixed shuffle tree, warps combined in order)
__device__ __forceinline__ double block_sum(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += sh[i];
  }
  return t;
}

// Rigid triangle-mesh contact of one external node (Domain_d::CalcContactForces,
// Contact.C:31-334): the first triangle, in order, that the node penetrates
// (d < 0 with its projection inside the triangle) gives the penalty normal
// force pf * min(E A / l, 0.2 m / dt^2) * d plus damping, then Coulomb
// friction from the accumulated tangential slip (static cap, else dynamic
// force along -v_t, slip reset). A node out of contact keeps its last contact
// force, as in the reference. Returns the normal-force magnitude when the
// triangle belongs to rigid body 0, the only body the reaction sums
// (Contact.C:229, :326-329), else 0.
__device__ __forceinline__ double tri_contact(const StepParams &P, const Fp64State &S, int64_t n,
                                              const double (&x)[3], const double (&v)[3],
                                              double m, double (&cf)[3]) {
  const int64_t np = P.np;
  cf[0] = S.cf[n];
  cf[1] = S.cf[np + n];
  cf[2] = S.cf[2 * np + n];
  double cfn = 0.0;
  for (int32_t j = 0; j < P.tri_ne; j++) {
    const double n0 = P.tri_nrm[3 * j], n1 = P.tri_nrm[3 * j + 1], n2 = P.tri_nrm[3 * j + 2];
    const double dd = (n0 * x[0] + n1 * x[1] + n2 * x[2]) - P.tri_pp[j];
    if (!(dd < 0)) continue;
    const double Q[3] = {x[0] - n0 * dd, x[1] - n1 * dd, x[2] - n2 * dd};
    bool inside = true;
    for (int l = 0; l < 3 && inside; l++) {
      const int nx = l + 1 > 2 ? 0 : l + 1;
      const double *a = &P.tri_x[3 * P.tri_el[3 * j + l]];
      const double *b = &P.tri_x[3 * P.tri_el[3 * j + nx]];
      const double e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
      const double e2[3] = {Q[0] - a[0], Q[1] - a[1], Q[2] - a[2]};
      const double c0 = e1[1] * e2[2] - e1[2] * e2[1];
      const double c1 = e1[2] * e2[0] - e1[0] * e2[2];
      const double c2 = e1[0] * e2[1] - e1[1] * e2[0];
      const double crit = c0 * n0 + c1 * n1 + c2 * n2;
      if (crit < 0.0) inside = false;
    }
    if (!inside) continue;
    const double dt = P.dt;
    const double v_reln = v[0] * n0 + v[1] * n1 + v[2] * n2;
    const double kgeo = P.tri_E0 * P.node_area[n] / P.nodlen[n];
    const double kmass = 0.2 * m / (dt * dt);
    const double k = (kmass < kgeo) ? kmass : kgeo;
    const double omega = sqrt(k / m);
    const double ccrit = 2.0 * m * omega;
    const double F_damp = 0.2 * ccrit * v_reln;
    const double F_normal = P.tri_pf * k * dd;
    const double sc = -(F_normal + F_damp);
    cf[0] = n0 * sc;
    cf[1] = n1 * sc;
    cf[2] = n2 * sc;
    cfn = sqrt(cf[0] * cf[0] + cf[1] * cf[1] + cf[2] * cf[2]);
    // friction
    const double vn = v[0] * n0 + v[1] * n1 + v[2] * n2;
    const double vt[3] = {v[0] - n0 * vn, v[1] - n1 * vn, v[2] - n2 * vn};
    double ut[3] = {S.ut[n], S.ut[np + n], S.ut[2 * np + n]};
    const double du[3] = {vt[0] * dt, vt[1] * dt, vt[2] * dt};
    const double ua[3] = {ut[0] + du[0], ut[1] + du[1], ut[2] + du[2]};
    ut[0] += du[0];
    ut[1] += du[1];
    ut[2] += du[2];
    const double mk = -k;
    const double ft[3] = {ua[0] * mk, ua[1] * mk, ua[2] * mk};
    const double ft_mag = sqrt(ft[0] * ft[0] + ft[1] * ft[1] + ft[2] * ft[2]);
    const double cn = cf[0] * n0 + cf[1] * n1 + cf[2] * n2;
    const double Fn[3] = {n0 * cn, n1 * cn, n2 * cn};
    const double fn_norm = sqrt(Fn[0] * Fn[0] + Fn[1] * Fn[1] + Fn[2] * Fn[2]);
    double F[3];
    if (ft_mag <= P.tri_mu_s * fn_norm) {
      F[0] = ft[0];
      F[1] = ft[1];
      F[2] = ft[2];
    } else {
      const double md = -(P.tri_mu_d * fn_norm);
      const double vnorm = sqrt(vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2]);
      const double inv = 1.0 / vnorm;
      F[0] = (vt[0] * md) * inv;
      F[1] = (vt[1] * md) * inv;
      F[2] = (vt[2] * md) * inv;
      ut[0] = ut[1] = ut[2] = 0.0;
    }
    S.ut[n] = ut[0];
    S.ut[np + n] = ut[1];
    S.ut[2 * np + n] = ut[2];
    cf[0] += F[0];
    cf[1] += F[1];
    cf[2] += F[2];
    if (P.tri_mid[j] != 0) cfn = 0.0;
    // heat from the die (Contact.C:309), kept after the contact ends
    if (P.thermal) S.qc[n] = P.tri_hc * P.node_area[n] * (P.tri_Tdie - S.T[n]);
    break;
  }
  S.cf[n] = cf[0];
  S.cf[np + n] = cf[1];
  S.cf[2 * np + n] = cf[2];
  return cfn;
}

// nodes: assemblyForces (Matrices.C:42-87) as a gather over the node's
// element list, the non-finite clamp (Solver_explicit.C:777-785), plane
// contact (Contact.C:58-323), calcAccel (Mechanical.C:321-341), ImposeBCA,
// UpdateCorrectionAccVel (Domain_d.C:981-997), ImposeBCV,
// UpdateCorrectionPos (:1005-1025) and the next step's UpdatePrediction
// (:961-974) + ImposeBCV, which this kernel hands to the next step as vp.
template <int NPE>
__global__ void __launch_bounds__(kNodeThreads) k_fp64_nodes(StepParams P, Fp64State S) {
  __shared__ double sh[kNodeThreads / 32];
  __shared__ bool am_last;
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const double time = P.st->time;
  double r = 0.0;
  if (n < P.nn) {
    const int64_t np = P.np;
    const int32_t b = __ldg(&P.off[n]), c = __ldg(&P.off[n + 1]) - b;
    double fi[3] = {0.0, 0.0, 0.0};
    for (int32_t k = 0; k < c; k++) {
      const int64_t base = (int64_t)__ldg(&P.slot[b + k]) * 3;
      fi[0] += __ldg(&S.fe[base]);
      fi[1] += __ldg(&S.fe[base + 1]);
      fi[2] += __ldg(&S.fe[base + 2]);
    }
    if (P.hg_on) {
      for (int32_t k = 0; k < c; k++) {
        const int64_t base = (int64_t)__ldg(&P.slot[b + k]) * 3;
        fi[0] -= __ldg(&S.fhg[base]);
        fi[1] -= __ldg(&S.fhg[base + 1]);
        fi[2] -= __ldg(&S.fhg[base + 2]);
      }
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
      if (!isfinite(fi[k])) {
        fi[k] = 0.0;
        atomicOr(&P.st->status, 1u);
        atomicMin(&P.st->first_bad_node, (long long)n);
      }
      S.fi[k * np + n] = fi[k];
    }
    const uint8_t fl = P.nflag[n];
    const double mass = S.mass[n];
    double x[3], vold[3], vp[3], pa[3], u[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      x[k] = S.x[k * np + n];
      vold[k] = S.v[k * np + n];
      vp[k] = S.vp[k * np + n];
      pa[k] = S.pa[k * np + n];
      u[k] = S.u[k * np + n];
    }
    double cf[3] = {0.0, 0.0, 0.0};
    if (P.tri_on) {
      if (fl & NF_CONTACT) r = tri_contact(P, S, n, x, vp, mass, cf);
    } else if (P.contact && (fl & NF_CONTACT)) {
      // rigid plane, outward normal (0, 0, -1), at z0 + vz * Time
      const double zd = P.c_z0 + P.c_vz * time;
      const double gap = zd - x[2];
      if (gap < 0) {
        // kcont = min(k_geometric, 0.2 m / dt^2) (Contact.C:190-193)
        const double kmass = 0.2 * mass / (P.dt * P.dt);
        const double k = (kmass < P.c_k) ? kmass : P.c_k;
        const double v_reln = vp[2] * -1.0;
        const double omega = sqrt(k / mass);
        const double ccrit = 2.0 * mass * omega;
        const double F_damp = 0.2 * ccrit * v_reln;
        const double F_normal = k * gap;
        const double cfz = -(F_normal + F_damp) * -1.0;
        cf[2] = cfz;
        r = fabs(cfz);
        double ut0 = S.ut[n] + vp[0] * P.dt;
        double ut1 = S.ut[np + n] + vp[1] * P.dt;
        double ftx = -k * ut0, fty = -k * ut1;
        const double ft_mag = sqrt(ftx * ftx + fty * fty);
        const double ft_max = P.c_mu * fabs(cfz);
        if (!(ft_mag <= ft_max)) {
          const double vt = sqrt(vp[0] * vp[0] + vp[1] * vp[1]);
          if (vt > 0.0) {
            ftx = -ft_max * vp[0] / vt;
            fty = -ft_max * vp[1] / vt;
          } else {
            ftx = fty = 0.0;
          }
          ut0 = ut1 = 0.0;
        }
        S.ut[n] = ut0;
        S.ut[np + n] = ut1;
        cf[0] += ftx;
        cf[1] += fty;
      }
      S.cf[n] = cf[0];
      S.cf[np + n] = cf[1];
      S.cf[2 * np + n] = cf[2];
    }
    if (!P.contact && (fl & NF_REACTION)) {
      if (P.rnode)
        P.rnode[n] = fi[P.react_dim];  // summed per specimen by the reaction kernel
      else
        r = fi[P.react_dim];
    }
    const uint32_t code = P.bc[n];
    const double *bv = &P.bcval[3 * (code >> 3)];
    const double dt = P.nspec_of ? P.spec_dt[P.nspec_of[n]] : P.dt;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      double a = (0.0 - fi[k]) / mass;
      if (P.contact) a += cf[k] / mass;
      if (code & (1u << k)) a = 0.0;
      a = P.fcorr * (a - P.alpha * pa[k]);
      double v = vp[k] + P.gamma * dt * a;
      if (code & (1u << k)) v = bv[k];
      double udt = dt * (vold[k] + (0.5 - P.beta) * dt * pa[k]);
      udt += P.beta * dt * dt * a;
      x[k] += udt;
      u[k] += udt;
      double vnext = v + (1.0 - P.gamma) * dt * a;
      if (code & (1u << k)) vnext = bv[k];
      S.x[k * np + n] = x[k];
      S.u[k * np + n] = u[k];
      S.v[k * np + n] = v;
      S.pa[k * np + n] = a;
      S.vp[k * np + n] = vnext;
    }
    if (P.thermal) {
      // ThermalCalcs node part (Thermal.C:108-126): element-node rates of the
      // step gathered in list order, plus the die heat over m cp of material 0
      const double *cur = S.dte + (P.st->step & 1) * P.ne * NPE;
      double sT = 0.0;
      for (int32_t k = 0; k < c; k++) sT += cur[__ldg(&P.slot[b + k])];
      S.T[n] = S.T[n] + (sT + S.qc[n] * 1.0 / (mass * P.cp0)) * P.dt;
    }
  }
  // reaction: block partial, then the last block to finish sums all partials
  // (each thread a fixed strided subset, then a fixed tree): deterministic.
  const double bs = block_sum(r, sh);
  if (threadIdx.x == 0) {
    P.partials[blockIdx.x] = bs;
    __threadfence();
    const unsigned prev = atomicAdd(&P.st->done_blocks, 1u);
    am_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (am_last) {
    __threadfence();
    double t = 0.0;
    for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x)
      t += ((volatile double *)P.partials)[i];
    const double tot = block_sum(t, sh);
    if (threadIdx.x == 0) {
      const long long s = P.st->step;
      if (s < P.hist_cap) P.hist[s] = tot;
      P.st->step = s + 1;
      P.st->time = time + P.dt;
      P.st->done_blocks = 0u;
    }
    if (P.tri_on) tri_move<false>(P, time);
  }
}

// predictor for the first step of a run: vp = v + (1 - gamma) dt prev_a, BCs
__global__ void k_fp64_predict(StepParams P, Fp64State S) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= P.nn) return;
  const uint32_t code = P.bc[n];
  const double *bv = &P.bcval[3 * (code >> 3)];
  for (int k = 0; k < 3; k++) {
    const double dt = P.nspec_of ? P.spec_dt[P.nspec_of[n]] : P.dt;
    double v = S.v[k * P.np + n] + (1.0 - P.gamma) * dt * S.pa[k * P.np + n];
    if (code & (1u << k)) v = bv[k];
    S.vp[k * P.np + n] = v;
  }
}

// calcElemDensity (Mechanical.C:295-319): rho = rho_0 * vol_0 / vol
__global__ void k_fp64_density(StepParams P, Fp64State S, const double *rho0) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= P.ne) return;
  S.rho[e] = rho0[e] * S.vol0[e] / S.vol[e];
}

inline unsigned grid_for(int64_t n, int threads) {
  return (unsigned)((n + threads - 1) / threads);
}

}  // namespace

// Block size of the FP64 per-element and per-node kernels. GB300's FP64 rate
// per SM is low, so a small mesh is spread over more SMs with smaller blocks
// (down to one warp) until there are two blocks per SM; large meshes keep
// max_threads.
static int spread(int64_t n, int max_threads, int sms) {
  int t = max_threads;
  while (t > 32 && grid_for(n, t) < 2 * (int64_t)sms) t /= 2;
  return t;
}

int fp64_node_grid(int64_t nn, int sms) {
  return (int)grid_for(nn, spread(nn, kNodeThreads, sms));
}

void fp64_geometry(const StepParams &P, const Fp64State &S, cudaStream_t st, bool store_detj) {
  const int t = spread(P.ne, kElemThreads, P.sms);
  if (P.npe == 8)
    k_fp64_geometry<8><<<grid_for(P.ne, t), t, 0, st>>>(P, S, store_detj);
  else
    k_fp64_geometry<4><<<grid_for(P.ne, t), t, 0, st>>>(P, S, store_detj);
}

void fp64_nodal(const StepParams &P, const Fp64State &S, cudaStream_t st, int init_mode) {
  const int t = spread(P.nn, kNodeThreads, P.sms);
  if (P.npe == 8 && P.box)
    k_fp64_nodal<8, true><<<grid_for(P.nn, t), t, 0, st>>>(P, S, init_mode);
  else if (P.npe == 8)
    k_fp64_nodal<8, false><<<grid_for(P.nn, t), t, 0, st>>>(P, S, init_mode);
  else
    k_fp64_nodal<4, false><<<grid_for(P.nn, t), t, 0, st>>>(P, S, init_mode);
}

void fp64_elements(const StepParams &P, const Fp64State &S, cudaStream_t st) {
  const int t = spread(P.ne, kElemThreads, P.sms);
  const unsigned g = (unsigned)grid_for(P.ne, t);
  if (P.npe == 8)
    if (P.thermal)
      k_fp64_elements<8, true><<<g, t, 0, st>>>(P, S);
    else
      k_fp64_elements<8, false><<<g, t, 0, st>>>(P, S);
  else
    if (P.thermal)
      k_fp64_elements<4, true><<<g, t, 0, st>>>(P, S);
    else
      k_fp64_elements<4, false><<<g, t, 0, st>>>(P, S);
}

void fp64_nodes(const StepParams &P, const Fp64State &S, cudaStream_t st, int node_grid) {
  // node_grid = fp64_node_grid(P.nn, P.sms): blocks of the spread size
  const int t = spread(P.nn, kNodeThreads, P.sms);
  if (P.npe == 8)
    k_fp64_nodes<8><<<node_grid, t, 0, st>>>(P, S);
  else
    k_fp64_nodes<4><<<node_grid, t, 0, st>>>(P, S);
}

void fp64_predict(const StepParams &P, const Fp64State &S, cudaStream_t st) {
  k_fp64_predict<<<grid_for(P.nn, kNodeThreads), kNodeThreads, 0, st>>>(P, S);
}

void fp64_density(const StepParams &P, const Fp64State &S, const double *rho0, cudaStream_t st) {
  k_fp64_density<<<grid_for(P.ne, kElemThreads), kElemThreads, 0, st>>>(P, S, rho0);
}

}  // namespace wf
