// Reverse mode (adjoint) of the FP64 explicit step.
//
// The forward step is the map (x, v, a_prev, tau, eps_p) -> next state plus the
// reaction R (sum of the assembled internal force over the reaction nodes).
// For a loss L(R_0 .. R_{N-1}) the caller supplies dL/dR_n; the reverse pass
// returns dL/d(E, sigma_y0, H) of every material. One reverse step is four
// kernels, mirroring the forward phases in reverse order:
//   k_adj_nodes    (node)   : Chung-Hulbert corrector/position update, BCs,
//                             acceleration a = -f/m, reaction seed
//                             -> adjoints of f_int, mass, v_pred, x, v, a_prev
//   k_adj_elements (element): recomputes the element phase from the stored
//                             start-of-step state and back-propagates element
//                             forces, hourglass forces, sigma = tau - p I, the
//                             J2 return map (consistent plastic-branch
//                             derivative), pressure -K (J_avg - 1), the
//                             reference's Jaumann terms, D/W, dN/dx and J
//                             -> per element-node contributions
//   k_adj_gather   (node)   : gathers those contributions over the node's
//                             element list (deterministic, no atomics), the
//                             predictor v_pred = v + (1-gamma) dt a_prev, and
//                             the adjoint of the nodal volume sum
//   k_adj_volume   (element): volume -> detJ -> J -> x contributions, gathered
//                             by the next reverse step's node kernel.
// Material gradients accumulate per element and are summed per material on
// the host in element order. The element kernel is templated on the scalar
// type of its arithmetic (FP64, or FP32 for the reduced-precision adjoint).
#include <vector>

#include "wf_adjoint.cuh"

namespace wf {
namespace {

constexpr int kThreads = 128;

__device__ __forceinline__ constexpr int hg_sign(int j, int a) {
  constexpr signed char t[4][8] = {{1, 1, -1, -1, -1, -1, 1, 1},
                                   {1, -1, -1, 1, -1, 1, 1, -1},
                                   {1, -1, 1, -1, 1, -1, 1, -1},
                                   {-1, 1, -1, 1, 1, -1, 1, -1}};
  return t[j][a];
}

// d J[m][k] / d x[a][k] (hexahedron: 0.125 * sign; tetrahedron: one-hot).
template <int NPE>
__device__ __forceinline__ double tj(int m, int a) {
  if constexpr (NPE == 8) {
    constexpr signed char s[3][8] = {{-1, 1, 1, -1, -1, 1, 1, -1},
                                     {-1, -1, 1, 1, -1, -1, 1, 1},
                                     {-1, -1, -1, -1, 1, 1, 1, 1}};
    return 0.125 * s[m][a];
  } else {
    return (a == m + 1) ? 1.0 : (a == 0 ? -1.0 : 0.0);
  }
}

template <typename T, int NPE>
struct ElemGeom {
  T J[3][3], A[3][3], dH[3][NPE], detJ;
};

template <typename T, int NPE>
__device__ __forceinline__ void geom_forward(const T (&x)[NPE][3], ElemGeom<T, NPE> &g) {
  for (int m = 0; m < 3; m++)
    for (int k = 0; k < 3; k++) {
      T s = 0;
      for (int a = 0; a < NPE; a++) s += (T)tj<NPE>(m, a) * x[a][k];
      g.J[m][k] = s;
    }
  const auto &J = g.J;
  // A = adj(J): A[k][m] = cofactor[m][k]
  g.A[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]);
  g.A[1][0] = -(J[1][0] * J[2][2] - J[1][2] * J[2][0]);
  g.A[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  g.A[0][1] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]);
  g.A[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]);
  g.A[2][1] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]);
  g.A[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]);
  g.A[1][2] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]);
  g.A[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]);
  for (int k = 0; k < 3; k++)
    for (int a = 0; a < NPE; a++) {
      T s = 0;
      for (int m = 0; m < 3; m++) s += g.A[k][m] * (T)tj<NPE>(m, a);
      g.dH[k][a] = s;
    }
  g.detJ = J[0][0] * g.A[0][0] + J[0][1] * g.A[1][0] + J[0][2] * g.A[2][0];
}

// Adds to Jb the adjoint of J given the adjoint Ab of A = adj(J).
template <typename T>
__device__ __forceinline__ void adj_reverse(const T J[3][3], const T Ab[3][3], T Jb[3][3]) {
  // A00 = J11 J22 - J12 J21
  Jb[1][1] += Ab[0][0] * J[2][2]; Jb[2][2] += Ab[0][0] * J[1][1];
  Jb[1][2] -= Ab[0][0] * J[2][1]; Jb[2][1] -= Ab[0][0] * J[1][2];
  // A10 = -(J10 J22 - J12 J20)
  Jb[1][0] -= Ab[1][0] * J[2][2]; Jb[2][2] -= Ab[1][0] * J[1][0];
  Jb[1][2] += Ab[1][0] * J[2][0]; Jb[2][0] += Ab[1][0] * J[1][2];
  // A20 = J10 J21 - J11 J20
  Jb[1][0] += Ab[2][0] * J[2][1]; Jb[2][1] += Ab[2][0] * J[1][0];
  Jb[1][1] -= Ab[2][0] * J[2][0]; Jb[2][0] -= Ab[2][0] * J[1][1];
  // A01 = -(J01 J22 - J02 J21)
  Jb[0][1] -= Ab[0][1] * J[2][2]; Jb[2][2] -= Ab[0][1] * J[0][1];
  Jb[0][2] += Ab[0][1] * J[2][1]; Jb[2][1] += Ab[0][1] * J[0][2];
  // A11 = J00 J22 - J02 J20
  Jb[0][0] += Ab[1][1] * J[2][2]; Jb[2][2] += Ab[1][1] * J[0][0];
  Jb[0][2] -= Ab[1][1] * J[2][0]; Jb[2][0] -= Ab[1][1] * J[0][2];
  // A21 = -(J00 J21 - J01 J20)
  Jb[0][0] -= Ab[2][1] * J[2][1]; Jb[2][1] -= Ab[2][1] * J[0][0];
  Jb[0][1] += Ab[2][1] * J[2][0]; Jb[2][0] += Ab[2][1] * J[0][1];
  // A02 = J01 J12 - J02 J11
  Jb[0][1] += Ab[0][2] * J[1][2]; Jb[1][2] += Ab[0][2] * J[0][1];
  Jb[0][2] -= Ab[0][2] * J[1][1]; Jb[1][1] -= Ab[0][2] * J[0][2];
  // A12 = -(J00 J12 - J02 J10)
  Jb[0][0] -= Ab[1][2] * J[1][2]; Jb[1][2] -= Ab[1][2] * J[0][0];
  Jb[0][2] += Ab[1][2] * J[1][0]; Jb[1][0] += Ab[1][2] * J[0][2];
  // A22 = J00 J11 - J01 J10
  Jb[0][0] += Ab[2][2] * J[1][1]; Jb[1][1] += Ab[2][2] * J[0][0];
  Jb[0][1] -= Ab[2][2] * J[1][0]; Jb[1][0] -= Ab[2][2] * J[0][1];
}

// ---------------------------------------------------------------------------
// Reverse of the node phase of step s.
__global__ void k_adj_nodes(StepParams P, AdjArgs A, int s, long long gstep, int have_geo) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= P.nn) return;
  const int64_t np = P.np, ne = P.ne;
  const int npe = P.npe;
  double xb[3];
  for (int k = 0; k < 3; k++) xb[k] = A.X[k * np + n];
  if (have_geo) {
    // geometry contributions of the step after this one, in list order
    const int32_t b = P.off[n], c = P.off[n + 1] - b;
    for (int32_t q = 0; q < c; q++) {
      const int32_t sl = P.slot[b + q];
      const int64_t e = sl / npe, loc = sl % npe;
      for (int k = 0; k < 3; k++) xb[k] += A.cgeo[(loc * 3 + k) * ne + e];
    }
  }
  const double dt = P.dt;
  const double m = A.smass[(int64_t)s * np + n];
  const double inv_m = 1.0 / m;
  const uint32_t code = P.bc[n];
  double mb = 0.0;
  for (int k = 0; k < 3; k++) {
    const bool fixed = (code >> k) & 1u;
    const double vbn = A.V[k * np + n], pabn = A.PA[k * np + n];
    const double fi = A.sfi[((int64_t)s * 3 + k) * np + n];
    const double abar = pabn + (fixed ? 0.0 : P.gamma * dt * vbn) + P.beta * dt * dt * xb[k];
    const double araw = fixed ? 0.0 : P.fcorr * abar;
    double fib = -araw * inv_m;
    mb += araw * fi * (inv_m * inv_m);
    if ((P.nflag[n] & NF_REACTION) && k == P.react_dim) fib += A.seed[gstep];
    A.fib[k * np + n] = fib;
    A.vpb[k * np + n] = fixed ? 0.0 : vbn;
    A.X[k * np + n] = xb[k];
    A.V[k * np + n] = dt * xb[k];
    A.PA[k * np + n] = -P.alpha * P.fcorr * abar + dt * (0.5 - P.beta) * dt * xb[k];
  }
  A.mb[n] = mb;
}

// Reverse of the element phase of step s (recomputed from the stored state).
template <typename T, int NPE>
__global__ void __launch_bounds__(kThreads) k_adj_elements(StepParams P, AdjArgs A, int s) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= P.ne) return;
  const int64_t np = P.np, ne = P.ne;
  const double *sx = A.sx + (int64_t)s * 3 * np, *sv = A.sv + (int64_t)s * 3 * np;
  const double *spa = A.spa + (int64_t)s * 3 * np, *sjr = A.sjr + (int64_t)s * np;
  const double *stau = A.stau + (int64_t)s * 6 * ne, *spls = A.spls + (int64_t)s * ne;
  const double dt_d = P.dt;
  const T dt = (T)dt_d;
  int32_t nid[NPE];
  T x[NPE][3], vp[NPE][3];
  for (int a = 0; a < NPE; a++) {
    nid[a] = P.elnod[a * ne + e];
    const uint32_t code = P.bc[nid[a]];
    for (int k = 0; k < 3; k++) {
      x[a][k] = (T)sx[k * np + nid[a]];
      double v = sv[k * np + nid[a]] + (1.0 - P.gamma) * dt_d * spa[k * np + nid[a]];
      if ((code >> k) & 1u) v = P.bcval[3 * (code >> 3) + k];
      vp[a][k] = (T)v;
    }
  }
  const MatDev m = P.mats[P.emat ? P.emat[e] : 0];
  const T K = (T)m.K, G = (T)m.G, H = (T)m.H, sy0 = (T)m.sy0;
  ElemGeom<T, NPE> g;
  geom_forward<T, NPE>(x, g);
  const T w = (NPE == 8) ? (T)8.0 : (T)(1.0 / 6.0);
  const T vol = g.detJ * w;
  const T f = (T)1 / g.detJ;
  // strain rate and spin
  T gr[3][NPE];
  for (int k = 0; k < 3; k++)
    for (int a = 0; a < NPE; a++) gr[k][a] = g.dH[k][a] * f;
  T D[6] = {0, 0, 0, 0, 0, 0}, W3[3] = {0, 0, 0};  // D: xx yy zz xy yz xz; W: xy yz xz
  for (int a = 0; a < NPE; a++) {
    D[0] += gr[0][a] * vp[a][0];
    D[1] += gr[1][a] * vp[a][1];
    D[2] += gr[2][a] * vp[a][2];
    D[3] += (T)0.5 * (gr[1][a] * vp[a][0] + gr[0][a] * vp[a][1]);
    D[4] += (T)0.5 * (gr[2][a] * vp[a][1] + gr[1][a] * vp[a][2]);
    D[5] += (T)0.5 * (gr[2][a] * vp[a][0] + gr[0][a] * vp[a][2]);
    W3[0] += (T)0.5 * (gr[1][a] * vp[a][0] - gr[0][a] * vp[a][1]);
    W3[1] += (T)0.5 * (gr[2][a] * vp[a][1] - gr[1][a] * vp[a][2]);
    W3[2] += (T)0.5 * (gr[2][a] * vp[a][0] - gr[0][a] * vp[a][2]);
  }
  const T w01 = W3[0], w12 = W3[1], w02 = W3[2];
  T Javg = 0;
  for (int a = 0; a < NPE; a++) Javg += (T)sjr[nid[a]];
  Javg /= (T)NPE;
  const T p = -K * (Javg - (T)1);
  T t[6];
  for (int c = 0; c < 6; c++) t[c] = (T)stau[c * ne + e];
  const T epl = (T)spls[e];
  // Jaumann terms of the reference's product: Q = SRT + RS per stored component
  T Q[6];
  Q[0] = (T)2 * (t[3] * w01 + t[5] * w02);
  Q[1] = 0;
  Q[2] = 0;
  Q[3] = w01 * (t[0] + t[1]) - t[5] * w12 + w02 * t[4];
  Q[4] = t[3] * w02 + w12 * (t[1] + t[2]) - w01 * t[5];
  Q[5] = w02 * (t[0] + t[2]) + t[3] * w12 + w01 * t[4];
  const T c3 = (D[0] + D[1] + D[2]) / (T)3;
  T Dd[6] = {D[0] - c3, D[1] - c3, D[2] - c3, D[3], D[4], D[5]};
  T ts[6];
  for (int c = 0; c < 6; c++) ts[c] = t[c] + dt * ((T)2 * G * Dd[c] + Q[c]);
  // deviatoric trial stress (the pressure cancels in the deviator)
  const T tr3 = (ts[0] + ts[1] + ts[2]) / (T)3;
  T sdev[6] = {ts[0] - tr3, ts[1] - tr3, ts[2] - tr3, ts[3], ts[4], ts[5]};
  const T J2 = (T)0.5 * (sdev[0] * sdev[0] + sdev[1] * sdev[1] + sdev[2] * sdev[2] +
                         (T)2 * (sdev[3] * sdev[3] + sdev[4] * sdev[4] + sdev[5] * sdev[5]));
  const T seq = sqrt((T)3 * J2);
  const T sy = sy0 + H * epl;
  const bool plastic = sy < seq;
  T tn[6], dgam = 0, fac = 1;
  if (plastic) {
    dgam = (seq - sy) / ((T)3 * G + H);
    fac = (T)1 - (T)3 * G * dgam / seq;
    for (int c = 0; c < 6; c++) tn[c] = sdev[c] * fac;
  } else {
    for (int c = 0; c < 6; c++) tn[c] = ts[c];
  }
  T sig[6] = {tn[0] - p, tn[1] - p, tn[2] - p, tn[3], tn[4], tn[5]};
  // hourglass modes and coefficient
  T hm[3][4];
  T ch = 0;
  const bool hg = (NPE == 8) && P.hg_on;
  if (hg) {
    for (int k = 0; k < 3; k++)
      for (int j = 0; j < 4; j++) {
        T sacc = 0;
        for (int a = 0; a < NPE; a++) sacc += (T)hg_sign(j, a % 8) * vp[a][k];
        hm[k][j] = sacc;
      }
    ch = (T)P.hg_coef * pow(vol, (T)0.6666666) * (T)A.rho[e] * (T)0.25 * (T)m.cs0;
  }

  // ---- reverse ------------------------------------------------------------
  T fb[NPE][3];
  for (int a = 0; a < NPE; a++)
    for (int k = 0; k < 3; k++) fb[a][k] = (T)A.fib[k * np + nid[a]];
  T dHb[3][NPE];
  for (int k = 0; k < 3; k++)
    for (int a = 0; a < NPE; a++) dHb[k][a] = 0;
  T sigb[6] = {0, 0, 0, 0, 0, 0};
  for (int a = 0; a < NPE; a++) {
    const T d0 = g.dH[0][a], d1 = g.dH[1][a], d2 = g.dH[2][a];
    const T f0 = fb[a][0] * w, f1 = fb[a][1] * w, f2 = fb[a][2] * w;
    sigb[0] += f0 * d0;
    sigb[1] += f1 * d1;
    sigb[2] += f2 * d2;
    sigb[3] += f0 * d1 + f1 * d0;
    sigb[4] += f1 * d2 + f2 * d1;
    sigb[5] += f0 * d2 + f2 * d0;
    dHb[0][a] += f0 * sig[0] + f1 * sig[3] + f2 * sig[5];
    dHb[1][a] += f0 * sig[3] + f1 * sig[1] + f2 * sig[4];
    dHb[2][a] += f0 * sig[5] + f1 * sig[4] + f2 * sig[2];
  }
  T vpb[NPE][3];
  for (int a = 0; a < NPE; a++)
    for (int k = 0; k < 3; k++) vpb[a][k] = 0;
  T volb = 0, Kb = 0, Gb = 0, Hb = 0, sy0b = 0;
  if (hg) {
    // f_hg[a][k] = -ch sum_j hm[k][j] Gamma_j[a], assembled with a minus sign:
    // adjoint of f_hg is -fb
    T chb = 0;
    for (int k = 0; k < 3; k++)
      for (int j = 0; j < 4; j++) {
        T hb = 0;
        for (int a = 0; a < NPE; a++) hb += (T)hg_sign(j, a % 8) * fb[a][k];
        // d f_hg / d hm = -ch Gamma; fhg_bar = -fb  =>  hm_bar = ch * hb
        chb += hb * hm[k][j];
        const T hmb = ch * hb;
        for (int a = 0; a < NPE; a++) vpb[a][k] += hmb * (T)hg_sign(j, a % 8);
      }
    // f_hg_bar . (-sum hm Gamma) with f_hg_bar = -fb gives + sum fb Gamma hm
    volb += chb * ch * (T)0.6666666 / vol;
    Kb += chb * ch * (T)0.5 / K;  // cs0 = sqrt(K / rho)
  }
  // sigma = tau_new - p I
  T tnb[6];
  for (int c = 0; c < 6; c++) tnb[c] = sigb[c] + (T)A.T[c * ne + e];
  T pb = -(sigb[0] + sigb[1] + sigb[2]);
  T eplb = (T)A.EP[e];
  // return map
  T tsb[6];
  if (plastic) {
    T facb = 0;
    T sdb[6];
    for (int c = 0; c < 6; c++) {
      facb += tnb[c] * sdev[c];
      sdb[c] = tnb[c] * fac;
    }
    const T den = (T)3 * G + H;
    const T dgb = eplb + facb * (-(T)3 * G / seq);
    const T seqb = facb * ((T)3 * G * dgam / (seq * seq)) + dgb / den;
    const T syb = -dgb / den;
    Gb += facb * (-(T)3 * dgam / seq) + dgb * (-(T)3 * (seq - sy) / (den * den));
    Hb += dgb * (-(seq - sy) / (den * den)) + syb * epl;
    sy0b += syb;
    eplb = eplb + syb * H;  // eps_p_new = eps_p + dgamma; sigma_y = sy0 + H eps_p
    // seq = sqrt(3 J2): d seq / d s_c = 3 / (2 seq) * (s_c, or 2 s_c off-diagonal)
    const T q = (T)1.5 / seq * seqb;
    for (int c = 0; c < 3; c++) sdb[c] += q * sdev[c];
    for (int c = 3; c < 6; c++) sdb[c] += q * (T)2 * sdev[c];
    const T mean = (sdb[0] + sdb[1] + sdb[2]) / (T)3;
    for (int c = 0; c < 3; c++) tsb[c] = sdb[c] - mean;
    for (int c = 3; c < 6; c++) tsb[c] = sdb[c];
  } else {
    for (int c = 0; c < 6; c++) tsb[c] = tnb[c];
  }
  // pressure p = -K (J_avg - 1)
  const T Javgb = -K * pb;
  Kb += -(Javg - (T)1) * pb;
  // Jaumann update ts = t + dt (2 G Dd + Q(t, W))
  T tb[6];
  for (int c = 0; c < 6; c++) tb[c] = tsb[c];
  T Qb[6];
  for (int c = 0; c < 6; c++) Qb[c] = dt * tsb[c];
  T Ddb[6];
  for (int c = 0; c < 6; c++) {
    Ddb[c] = dt * (T)2 * G * tsb[c];
    Gb += dt * (T)2 * Dd[c] * tsb[c];
  }
  T w01b = 0, w12b = 0, w02b = 0;
  // Q0 = 2 (t3 w01 + t5 w02)
  tb[3] += Qb[0] * (T)2 * w01; tb[5] += Qb[0] * (T)2 * w02;
  w01b += Qb[0] * (T)2 * t[3]; w02b += Qb[0] * (T)2 * t[5];
  // Q3 = w01 (t0 + t1) - t5 w12 + w02 t4
  tb[0] += Qb[3] * w01; tb[1] += Qb[3] * w01; tb[5] -= Qb[3] * w12; tb[4] += Qb[3] * w02;
  w01b += Qb[3] * (t[0] + t[1]); w12b -= Qb[3] * t[5]; w02b += Qb[3] * t[4];
  // Q4 = t3 w02 + w12 (t1 + t2) - w01 t5
  tb[3] += Qb[4] * w02; tb[1] += Qb[4] * w12; tb[2] += Qb[4] * w12; tb[5] -= Qb[4] * w01;
  w02b += Qb[4] * t[3]; w12b += Qb[4] * (t[1] + t[2]); w01b -= Qb[4] * t[5];
  // Q5 = w02 (t0 + t2) + t3 w12 + w01 t4
  tb[0] += Qb[5] * w02; tb[2] += Qb[5] * w02; tb[3] += Qb[5] * w12; tb[4] += Qb[5] * w01;
  w02b += Qb[5] * (t[0] + t[2]); w12b += Qb[5] * t[3]; w01b += Qb[5] * t[4];
  // deviator of D
  T Db[6];
  {
    const T mean = (Ddb[0] + Ddb[1] + Ddb[2]) / (T)3;
    for (int c = 0; c < 3; c++) Db[c] = Ddb[c] - mean;
    for (int c = 3; c < 6; c++) Db[c] = Ddb[c];
  }
  // D, W from gr and vp
  T grb[3][NPE];
  for (int k = 0; k < 3; k++)
    for (int a = 0; a < NPE; a++) grb[k][a] = 0;
  {
    const T h01p = (T)0.5 * (Db[3] + w01b), h01m = (T)0.5 * (Db[3] - w01b);
    const T h12p = (T)0.5 * (Db[4] + w12b), h12m = (T)0.5 * (Db[4] - w12b);
    const T h02p = (T)0.5 * (Db[5] + w02b), h02m = (T)0.5 * (Db[5] - w02b);
    for (int a = 0; a < NPE; a++) {
      grb[0][a] += Db[0] * vp[a][0];
      vpb[a][0] += Db[0] * gr[0][a];
      grb[1][a] += Db[1] * vp[a][1];
      vpb[a][1] += Db[1] * gr[1][a];
      grb[2][a] += Db[2] * vp[a][2];
      vpb[a][2] += Db[2] * gr[2][a];
      grb[1][a] += h01p * vp[a][0];
      vpb[a][0] += h01p * gr[1][a];
      grb[0][a] += h01m * vp[a][1];
      vpb[a][1] += h01m * gr[0][a];
      grb[2][a] += h12p * vp[a][1];
      vpb[a][1] += h12p * gr[2][a];
      grb[1][a] += h12m * vp[a][2];
      vpb[a][2] += h12m * gr[1][a];
      grb[2][a] += h02p * vp[a][0];
      vpb[a][0] += h02p * gr[2][a];
      grb[0][a] += h02m * vp[a][2];
      vpb[a][2] += h02m * gr[0][a];
    }
  }
  // gr = dH f, f = 1 / detJ
  T fbar = 0;
  for (int k = 0; k < 3; k++)
    for (int a = 0; a < NPE; a++) {
      dHb[k][a] += grb[k][a] * f;
      fbar += grb[k][a] * g.dH[k][a];
    }
  T detJb = -fbar * f * f;
  // dH = A T
  T Ab[3][3];
  for (int k = 0; k < 3; k++)
    for (int mm = 0; mm < 3; mm++) {
      T sacc = 0;
      for (int a = 0; a < NPE; a++) sacc += dHb[k][a] * (T)tj<NPE>(mm, a);
      Ab[k][mm] = sacc;
    }
  T Jb[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  adj_reverse<T>(g.J, Ab, Jb);
  // detJ (strain-rate path; the volume path is handled by k_adj_volume)
  for (int mm = 0; mm < 3; mm++)
    for (int k = 0; k < 3; k++) Jb[mm][k] += detJb * g.A[k][mm];
  // outputs
  for (int a = 0; a < NPE; a++)
    for (int k = 0; k < 3; k++) {
      T xb = 0;
      for (int mm = 0; mm < 3; mm++) xb += Jb[mm][k] * (T)tj<NPE>(mm, a);
      A.cx[(a * 3 + k) * ne + e] = (double)xb;
      A.cv[(a * 3 + k) * ne + e] = (double)vpb[a][k];
    }
  A.cj[e] = (double)(Javgb / (T)NPE);
  A.volb[e] = (double)volb;
  for (int c = 0; c < 6; c++) A.T[c * ne + e] = (double)tb[c];
  A.EP[e] = (double)eplb;
  // material gradients: K = E / (3 (1 - 2 nu)), G = E / (2 (1 + nu))
  const double Eb = (double)Kb * (m.K / m.E) + (double)Gb * (m.G / m.E);
  A.gth[e] += Eb;
  A.gth[ne + e] += (double)sy0b;
  A.gth[2 * ne + e] += (double)Hb;
}

// Walsh transform over the hexahedron's corners and its transpose (node a at
// the signs of (xi, eta, zeta) of the AddBoxLength numbering): o = sums of v
// weighted by {1, xi, eta, zeta, eta zeta, xi zeta, xi eta, xi eta zeta};
// the synthesis returns the node values of sum_b o[b] phi_b for b = 1..7.
template <typename T>
__device__ __forceinline__ void walsh8t(const T (&v)[8], T (&o)[8]) {
  const T a0 = v[1] + v[0], b0 = v[1] - v[0], a1 = v[2] + v[3], b1 = v[2] - v[3];
  const T a2 = v[5] + v[4], b2 = v[5] - v[4], a3 = v[6] + v[7], b3 = v[6] - v[7];
  const T c0 = a1 + a0, d0 = a1 - a0, e0 = b1 + b0, f0 = b1 - b0;
  const T c1 = a3 + a2, d1 = a3 - a2, e1 = b3 + b2, f1 = b3 - b2;
  o[0] = c1 + c0; o[3] = c1 - c0; o[2] = d1 + d0; o[4] = d1 - d0;
  o[1] = e1 + e0; o[5] = e1 - e0; o[6] = f1 + f0; o[7] = f1 - f0;
}
template <typename T>
__device__ __forceinline__ void walsh8t_synth(const T (&o)[8], T (&v)[8]) {
  const T c1 = o[3], c0 = -o[3];
  const T d1 = o[2] + o[4], d0 = o[2] - o[4], e1 = o[1] + o[5], e0 = o[1] - o[5];
  const T f1 = o[6] + o[7], f0 = o[6] - o[7];
  const T a1 = c0 + d0, a0 = c0 - d0, b1 = e0 + f0, b0 = e0 - f0;
  const T a3 = c1 + d1, a2 = c1 - d1, b3 = e1 + f1, b2 = e1 - f1;
  v[1] = a0 + b0; v[0] = a0 - b0; v[2] = a1 + b1; v[3] = a1 - b1;
  v[5] = a2 + b2; v[4] = a2 - b2; v[6] = a3 + b3; v[7] = a3 - b3;
}

// Reverse of the element phase of step s for hexahedra, in the Walsh form:
// J = W(x)/8, the velocity gradient adj(J) W(v) / (8 detJ), the forces the
// synthesis of adj(J)^T sigma and of the hourglass terms ch h_j (the same
// quantities as the per-node formulation of the forward kernel). Outputs as
// k_adj_elements. Coordinates enter relative to the element's first node.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_adj_hex(StepParams P, AdjArgs A, int s) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= P.ne) return;
  const int64_t np = P.np, ne = P.ne;
  const double *sx = A.sx + (int64_t)s * 3 * np, *sv = A.sv + (int64_t)s * 3 * np;
  const double *spa = A.spa + (int64_t)s * 3 * np, *sjr = A.sjr + (int64_t)s * np;
  const double *stau = A.stau + (int64_t)s * 6 * ne, *spls = A.spls + (int64_t)s * ne;
  const double dt_d = P.dt;
  const T dt = (T)dt_d;
  int32_t nid[8];
  for (int a = 0; a < 8; a++) nid[a] = P.elnod[a * ne + e];
  // Jacobian from relative coordinates
  T J[3][3];
  for (int k = 0; k < 3; k++) {
    const double x0 = sx[k * np + nid[0]];
    T v[8], o[8];
    for (int a = 0; a < 8; a++) v[a] = (T)(sx[k * np + nid[a]] - x0);
    walsh8t(v, o);
    for (int mm = 0; mm < 3; mm++) J[mm][k] = (T)0.125 * o[1 + mm];
  }
  T Am[3][3];  // adj(J): Am[k][m] = cofactor[m][k]
  Am[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]);
  Am[1][0] = -(J[1][0] * J[2][2] - J[1][2] * J[2][0]);
  Am[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
  Am[0][1] = -(J[0][1] * J[2][2] - J[0][2] * J[2][1]);
  Am[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]);
  Am[2][1] = -(J[0][0] * J[2][1] - J[0][1] * J[2][0]);
  Am[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]);
  Am[1][2] = -(J[0][0] * J[1][2] - J[0][2] * J[1][0]);
  Am[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]);
  const T detJ = J[0][0] * Am[0][0] + J[0][1] * Am[1][0] + J[0][2] * Am[2][0];
  const T vol = detJ * (T)8;
  // predicted velocities: Walsh sums G (derivative directions) and hm (hourglass)
  T G[3][3], hm[3][4];
  for (int k = 0; k < 3; k++) {
    T v[8], o[8];
    for (int a = 0; a < 8; a++) {
      const uint32_t code = P.bc[nid[a]];
      double vv = sv[k * np + nid[a]] + (1.0 - P.gamma) * dt_d * spa[k * np + nid[a]];
      if ((code >> k) & 1u) vv = P.bcval[3 * (code >> 3) + k];
      v[a] = (T)vv;
    }
    walsh8t(v, o);
    for (int mm = 0; mm < 3; mm++) G[mm][k] = o[1 + mm];
    for (int j = 0; j < 4; j++) hm[k][j] = o[4 + j];
  }
  const MatDev m = P.mats[P.emat ? P.emat[e] : 0];
  const T K = (T)m.K, Gm = (T)m.G, H = (T)m.H, sy0 = (T)m.sy0;
  const T fl = (T)0.125 / detJ;
  T L[3][3];
  for (int i = 0; i < 3; i++)
    for (int k = 0; k < 3; k++)
      L[i][k] = fl * (Am[i][0] * G[0][k] + Am[i][1] * G[1][k] + Am[i][2] * G[2][k]);
  const T D[6] = {L[0][0], L[1][1], L[2][2], (T)0.5 * (L[1][0] + L[0][1]),
                  (T)0.5 * (L[2][1] + L[1][2]), (T)0.5 * (L[2][0] + L[0][2])};
  const T w01 = (T)0.5 * (L[1][0] - L[0][1]);
  const T w12 = (T)0.5 * (L[2][1] - L[1][2]);
  const T w02 = (T)0.5 * (L[2][0] - L[0][2]);
  T Javg = 0;
  for (int a = 0; a < 8; a++) Javg += (T)sjr[nid[a]];
  Javg /= (T)8;
  const T p = -K * (Javg - (T)1);
  T t[6];
  for (int c = 0; c < 6; c++) t[c] = (T)stau[c * ne + e];
  const T epl = (T)spls[e];
  T Q[6];
  Q[0] = (T)2 * (t[3] * w01 + t[5] * w02);
  Q[1] = 0;
  Q[2] = 0;
  Q[3] = w01 * (t[0] + t[1]) - t[5] * w12 + w02 * t[4];
  Q[4] = t[3] * w02 + w12 * (t[1] + t[2]) - w01 * t[5];
  Q[5] = w02 * (t[0] + t[2]) + t[3] * w12 + w01 * t[4];
  const T c3 = (D[0] + D[1] + D[2]) / (T)3;
  const T Dd[6] = {D[0] - c3, D[1] - c3, D[2] - c3, D[3], D[4], D[5]};
  T ts[6];
  for (int c = 0; c < 6; c++) ts[c] = t[c] + dt * ((T)2 * Gm * Dd[c] + Q[c]);
  const T tr3 = (ts[0] + ts[1] + ts[2]) / (T)3;
  const T sdev[6] = {ts[0] - tr3, ts[1] - tr3, ts[2] - tr3, ts[3], ts[4], ts[5]};
  const T J2 = (T)0.5 * (sdev[0] * sdev[0] + sdev[1] * sdev[1] + sdev[2] * sdev[2] +
                         (T)2 * (sdev[3] * sdev[3] + sdev[4] * sdev[4] + sdev[5] * sdev[5]));
  const T seq = sqrt((T)3 * J2);
  const T sy = sy0 + H * epl;
  const bool plastic = sy < seq;
  T tn[6], dgam = 0, fac = 1;
  if (plastic) {
    dgam = (seq - sy) / ((T)3 * Gm + H);
    fac = (T)1 - (T)3 * Gm * dgam / seq;
    for (int c = 0; c < 6; c++) tn[c] = sdev[c] * fac;
  } else {
    for (int c = 0; c < 6; c++) tn[c] = ts[c];
  }
  const T S[3][3] = {{tn[0] - p, tn[3], tn[5]}, {tn[3], tn[1] - p, tn[4]}, {tn[5], tn[4], tn[2] - p}};
  const T ch = P.hg_on ? (T)P.hg_coef * pow(vol, (T)0.6666666) * (T)A.rho[e] * (T)0.25 * (T)m.cs0
                       : (T)0;

  // ---- reverse ------------------------------------------------------------
  // forces: f = synth(T, ch hm) with T = adj(J)^T S; the transpose is W(fb)
  T Tb[3][3], hmb[3][4];
  T chb = 0;
  for (int k = 0; k < 3; k++) {
    T v[8], o[8];
    for (int a = 0; a < 8; a++) v[a] = (T)A.fib[k * np + nid[a]];
    walsh8t(v, o);
    for (int mm = 0; mm < 3; mm++) Tb[mm][k] = o[1 + mm];
    for (int j = 0; j < 4; j++) {
      chb += o[4 + j] * hm[k][j];
      hmb[k][j] = ch * o[4 + j];
    }
  }
  T Ab[3][3];
  T Sb[3][3];
  for (int i = 0; i < 3; i++)
    for (int mm = 0; mm < 3; mm++) {
      T acc = 0;
      for (int k = 0; k < 3; k++) acc += S[i][k] * Tb[mm][k];
      Ab[i][mm] = acc;
    }
  for (int i = 0; i < 3; i++)
    for (int k = 0; k < 3; k++)
      Sb[i][k] = Am[i][0] * Tb[0][k] + Am[i][1] * Tb[1][k] + Am[i][2] * Tb[2][k];
  T sigb[6] = {Sb[0][0], Sb[1][1], Sb[2][2], Sb[0][1] + Sb[1][0], Sb[1][2] + Sb[2][1],
               Sb[0][2] + Sb[2][0]};
  T volb = 0, Kb = 0, Gb = 0, Hb = 0, sy0b = 0;
  if (P.hg_on) {
    volb += chb * ch * (T)0.6666666 / vol;
    Kb += chb * ch * (T)0.5 / K;  // cs0 = sqrt(K / rho)
  }
  // sigma = tau_new - p I
  T tnb[6];
  for (int c = 0; c < 6; c++) tnb[c] = sigb[c] + (T)A.T[c * ne + e];
  const T pb = -(sigb[0] + sigb[1] + sigb[2]);
  T eplb = (T)A.EP[e];
  T tsb[6];
  if (plastic) {
    T facb = 0;
    T sdb[6];
    for (int c = 0; c < 6; c++) {
      facb += tnb[c] * sdev[c];
      sdb[c] = tnb[c] * fac;
    }
    const T den = (T)3 * Gm + H;
    const T dgb = eplb + facb * (-(T)3 * Gm / seq);
    const T seqb = facb * ((T)3 * Gm * dgam / (seq * seq)) + dgb / den;
    const T syb = -dgb / den;
    Gb += facb * (-(T)3 * dgam / seq) + dgb * (-(T)3 * (seq - sy) / (den * den));
    Hb += dgb * (-(seq - sy) / (den * den)) + syb * epl;
    sy0b += syb;
    eplb = eplb + syb * H;
    const T q = (T)1.5 / seq * seqb;
    for (int c = 0; c < 3; c++) sdb[c] += q * sdev[c];
    for (int c = 3; c < 6; c++) sdb[c] += q * (T)2 * sdev[c];
    const T mean = (sdb[0] + sdb[1] + sdb[2]) / (T)3;
    for (int c = 0; c < 3; c++) tsb[c] = sdb[c] - mean;
    for (int c = 3; c < 6; c++) tsb[c] = sdb[c];
  } else {
    for (int c = 0; c < 6; c++) tsb[c] = tnb[c];
  }
  const T Javgb = -K * pb;
  Kb += -(Javg - (T)1) * pb;
  T tb[6], Qb[6], Ddb[6];
  for (int c = 0; c < 6; c++) {
    tb[c] = tsb[c];
    Qb[c] = dt * tsb[c];
    Ddb[c] = dt * (T)2 * Gm * tsb[c];
    Gb += dt * (T)2 * Dd[c] * tsb[c];
  }
  T w01b = 0, w12b = 0, w02b = 0;
  tb[3] += Qb[0] * (T)2 * w01; tb[5] += Qb[0] * (T)2 * w02;
  w01b += Qb[0] * (T)2 * t[3]; w02b += Qb[0] * (T)2 * t[5];
  tb[0] += Qb[3] * w01; tb[1] += Qb[3] * w01; tb[5] -= Qb[3] * w12; tb[4] += Qb[3] * w02;
  w01b += Qb[3] * (t[0] + t[1]); w12b -= Qb[3] * t[5]; w02b += Qb[3] * t[4];
  tb[3] += Qb[4] * w02; tb[1] += Qb[4] * w12; tb[2] += Qb[4] * w12; tb[5] -= Qb[4] * w01;
  w02b += Qb[4] * t[3]; w12b += Qb[4] * (t[1] + t[2]); w01b -= Qb[4] * t[5];
  tb[0] += Qb[5] * w02; tb[2] += Qb[5] * w02; tb[3] += Qb[5] * w12; tb[4] += Qb[5] * w01;
  w02b += Qb[5] * (t[0] + t[2]); w12b += Qb[5] * t[3]; w01b += Qb[5] * t[4];
  T Db[6];
  {
    const T mean = (Ddb[0] + Ddb[1] + Ddb[2]) / (T)3;
    for (int c = 0; c < 3; c++) Db[c] = Ddb[c] - mean;
    for (int c = 3; c < 6; c++) Db[c] = Ddb[c];
  }
  // D, W from the velocity gradient L
  T Lb[3][3] = {{Db[0], 0, 0}, {0, Db[1], 0}, {0, 0, Db[2]}};
  Lb[1][0] += (T)0.5 * (Db[3] + w01b);
  Lb[0][1] += (T)0.5 * (Db[3] - w01b);
  Lb[2][1] += (T)0.5 * (Db[4] + w12b);
  Lb[1][2] += (T)0.5 * (Db[4] - w12b);
  Lb[2][0] += (T)0.5 * (Db[5] + w02b);
  Lb[0][2] += (T)0.5 * (Db[5] - w02b);
  // L = fl adj(J) G
  T flb = 0;
  for (int i = 0; i < 3; i++)
    for (int k = 0; k < 3; k++) flb += Lb[i][k] * L[i][k];
  flb /= fl;
  T Gbar[3][3];
  for (int mm = 0; mm < 3; mm++)
    for (int k = 0; k < 3; k++)
      Gbar[mm][k] = fl * (Am[0][mm] * Lb[0][k] + Am[1][mm] * Lb[1][k] + Am[2][mm] * Lb[2][k]);
  for (int i = 0; i < 3; i++)
    for (int mm = 0; mm < 3; mm++)
      Ab[i][mm] += fl * (Lb[i][0] * G[mm][0] + Lb[i][1] * G[mm][1] + Lb[i][2] * G[mm][2]);
  const T detJb = -flb * fl / detJ;
  // predicted velocities: the transpose of the Walsh analysis
  for (int k = 0; k < 3; k++) {
    T o[8], v[8];
    o[0] = 0;
    for (int mm = 0; mm < 3; mm++) o[1 + mm] = Gbar[mm][k];
    for (int j = 0; j < 4; j++) o[4 + j] = hmb[k][j];
    walsh8t_synth(o, v);
    for (int a = 0; a < 8; a++) A.cv[(a * 3 + k) * ne + e] = (double)v[a];
  }
  // adj(J) and detJ back to J, then to the coordinates
  T Jb[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
  adj_reverse<T>(J, Ab, Jb);
  for (int mm = 0; mm < 3; mm++)
    for (int k = 0; k < 3; k++) Jb[mm][k] += detJb * Am[k][mm];
  for (int k = 0; k < 3; k++) {
    T o[8], v[8];
    o[0] = 0;
    for (int mm = 0; mm < 3; mm++) o[1 + mm] = (T)0.125 * Jb[mm][k];
    for (int j = 4; j < 8; j++) o[j] = 0;
    walsh8t_synth(o, v);
    for (int a = 0; a < 8; a++) A.cx[(a * 3 + k) * ne + e] = (double)v[a];
  }
  A.cj[e] = (double)(Javgb / (T)8);
  A.volb[e] = (double)volb;
  for (int c = 0; c < 6; c++) A.T[c * ne + e] = (double)tb[c];
  A.EP[e] = (double)eplb;
  const double Eb = (double)Kb * (m.K / m.E) + (double)Gb * (m.G / m.E);
  A.gth[e] += Eb;
  A.gth[ne + e] += (double)sy0b;
  A.gth[2 * ne + e] += (double)Hb;
}

// Node gather of the element contributions; predictor and nodal-volume reverse.
__global__ void k_adj_gather(StepParams P, AdjArgs A) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= P.nn) return;
  const int64_t np = P.np, ne = P.ne;
  const int npe = P.npe;
  const int32_t b = P.off[n], c = P.off[n + 1] - b;
  double vpb[3] = {A.vpb[n], A.vpb[np + n], A.vpb[2 * np + n]};
  double xb[3] = {0, 0, 0};
  double jrb = 0.0;
  for (int32_t q = 0; q < c; q++) {
    const int32_t sl = P.slot[b + q];
    const int64_t e = sl / npe, loc = sl % npe;
    for (int k = 0; k < 3; k++) {
      vpb[k] += A.cv[(loc * 3 + k) * ne + e];
      xb[k] += A.cx[(loc * 3 + k) * ne + e];
    }
    jrb += A.cj[e];
  }
  const uint32_t code = P.bc[n];
  const double dt = P.dt;
  for (int k = 0; k < 3; k++) {
    A.X[k * np + n] += xb[k];
    if (!((code >> k) & 1u)) {
      A.V[k * np + n] += vpb[k];
      A.PA[k * np + n] += (1.0 - P.gamma) * dt * vpb[k];
    }
  }
  // jr = s / s0; mass = sum_e rho_e (s / npe) / c, recomputed each step
  double sb = jrb * A.inv_s0[n];
  if (P.mass_mode == 0) sb += A.mb[n] * A.dmds[n];
  A.sb[n] = sb;
}

// Volume adjoint (hourglass part + nodal sums) through detJ and J to x.
template <int NPE>
__global__ void k_adj_volume(StepParams P, AdjArgs A, int s) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= P.ne) return;
  const int64_t np = P.np, ne = P.ne;
  const double *sx = A.sx + (int64_t)s * 3 * np;
  double x[NPE][3];
  double volb = A.volb[e];
  for (int a = 0; a < NPE; a++) {
    const int32_t n = P.elnod[a * ne + e];
    volb += A.sb[n];
    for (int k = 0; k < 3; k++) x[a][k] = sx[k * np + n];
  }
  const double w = (NPE == 8) ? 8.0 : 1.0 / 6.0;
  const double detJb = w * volb;
  if constexpr (NPE == 8) {
    // d detJ / d J = cofactors; J = W(x) / 8 relative to node 0, x-bar its transpose
    double J[3][3];
    for (int k = 0; k < 3; k++) {
      double v[8], o[8];
      for (int a = 0; a < 8; a++) v[a] = x[a][k] - x[0][k];
      walsh8t(v, o);
      for (int mm = 0; mm < 3; mm++) J[mm][k] = 0.125 * o[1 + mm];
    }
    double C[3][3];  // cofactors C[m][k] = d detJ / d J[m][k]
    C[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    C[0][1] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    C[0][2] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    C[1][0] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
    C[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
    C[1][2] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
    C[2][0] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    C[2][1] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
    C[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    for (int k = 0; k < 3; k++) {
      double o[8], v[8];
      o[0] = 0.0;
      for (int mm = 0; mm < 3; mm++) o[1 + mm] = 0.125 * detJb * C[mm][k];
      for (int j = 4; j < 8; j++) o[j] = 0.0;
      walsh8t_synth(o, v);
      for (int a = 0; a < 8; a++) A.cgeo[(a * 3 + k) * ne + e] = v[a];
    }
  } else {
    ElemGeom<double, NPE> g;
    geom_forward<double, NPE>(x, g);
    for (int a = 0; a < NPE; a++)
      for (int k = 0; k < 3; k++) {
        double xb = 0;
        for (int mm = 0; mm < 3; mm++) xb += detJb * g.A[k][mm] * tj<NPE>(mm, a);
        A.cgeo[(a * 3 + k) * ne + e] = xb;
      }
  }
}

// Copies the start-of-step state into the stash slot s.
__global__ void k_adj_stash(StepParams P, Fp64State S, AdjArgs A, int s) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t np = P.np, ne = P.ne;
  if (i < 3 * np) {
    A.sx[(int64_t)s * 3 * np + i] = S.x[i];
    A.sv[(int64_t)s * 3 * np + i] = S.v[i];
    A.spa[(int64_t)s * 3 * np + i] = S.pa[i];
  }
  if (i < 6 * ne) A.stau[(int64_t)s * 6 * ne + i] = S.tau[i];
  if (i < ne) A.spls[(int64_t)s * ne + i] = S.pls[i];
}

// Copies the nodal quantities of step s (after its nodal and node phases).
__global__ void k_adj_stash_step(StepParams P, Fp64State S, AdjArgs A, int s) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t np = P.np;
  if (i < np) {
    A.sjr[(int64_t)s * np + i] = S.jr[i];
    A.smass[(int64_t)s * np + i] = S.mass[i];
  }
  if (i < 3 * np) A.sfi[(int64_t)s * 3 * np + i] = S.fi[i];
}

// Per-node constants of the reverse: 1 / s0 and d(mass)/d(sum of element
// volumes) = sum_e rho_e / (count npe) (CalcNodalMassFromVol, Mechanical.C:1576-1601).
__global__ void k_adj_node_constants(StepParams P, AdjArgs A) {
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= P.nn) return;
  const int32_t b = P.off[n], c = P.off[n + 1] - b;
  double rho_sum = 0.0;
  for (int32_t q = 0; q < c; q++) rho_sum += A.rho[P.slot[b + q] / P.npe];
  A.inv_s0[n] = 1.0 / A.s0[n];
  A.dmds[n] = rho_sum / ((double)c * P.npe);
}

inline unsigned grid_for(int64_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

}  // namespace

void adj_node_constants(const StepParams &P, const AdjArgs &A, cudaStream_t st) {
  k_adj_node_constants<<<grid_for(P.nn), kThreads, 0, st>>>(P, A);
}

void adj_stash_state(const StepParams &P, const Fp64State &S, const AdjArgs &A, int s,
                     cudaStream_t st) {
  const int64_t n = std::max<int64_t>(3 * P.np, 6 * P.ne);
  k_adj_stash<<<grid_for(n), kThreads, 0, st>>>(P, S, A, s);
}

void adj_stash_step(const StepParams &P, const Fp64State &S, const AdjArgs &A, int s,
                    cudaStream_t st) {
  k_adj_stash_step<<<grid_for(3 * P.np), kThreads, 0, st>>>(P, S, A, s);
}

void adj_reverse_step(const StepParams &P, const AdjArgs &A, int s, long long gstep, int have_geo,
                      bool fp32, cudaStream_t st) {
  k_adj_nodes<<<grid_for(P.nn), kThreads, 0, st>>>(P, A, s, gstep, have_geo);
  if (P.npe == 8) {
    if (fp32)
      k_adj_hex<float><<<grid_for(P.ne), kThreads, 0, st>>>(P, A, s);
    else
      k_adj_hex<double><<<grid_for(P.ne), kThreads, 0, st>>>(P, A, s);
  } else {
    if (fp32)
      k_adj_elements<float, 4><<<grid_for(P.ne), kThreads, 0, st>>>(P, A, s);
    else
      k_adj_elements<double, 4><<<grid_for(P.ne), kThreads, 0, st>>>(P, A, s);
  }
  k_adj_gather<<<grid_for(P.nn), kThreads, 0, st>>>(P, A);
  if (P.npe == 8)
    k_adj_volume<8><<<grid_for(P.ne), kThreads, 0, st>>>(P, A, s);
  else
    k_adj_volume<4><<<grid_for(P.ne), kThreads, 0, st>>>(P, A, s);
}

}  // namespace wf
