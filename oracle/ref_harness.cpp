// Test oracle harness around the reference WeldFormFEM CPU code.
//
// TEST INFRASTRUCTURE ONLY. This file is compiled together with the
// reference's own translation units (src/common/{Domain_d,Mechanical,
// Matrices,Contact,Mesh,VTKWriter,Thermal}.C and src/explicit/Solver_explicit.C,
// read in place from the reference checkout) into oracle/_ref/libwfref.so by
// oracle/build_ref.sh. Nothing in the product links or loads it; tests and the
// golden-fixture generator call it through ctypes.
//
// Pattern: a subclass of MetFEM::Domain_d with protected access, as the
// reference's own test harness does (src/common/test_1el_3D.cpp:67).
//
// Two modes:
//  * verbatim  (O1): wfr_solve_verbatim() calls Domain_d::SolveChungHulbert()
//    unchanged (src/explicit/Solver_explicit.C:101-1271).
//  * stepwise  (O2): wfr_init()/wfr_step() call the same Domain_d members in
//    the order of the reference loop (Solver_explicit.C:346-1167). Three
//    pieces that the reference C++ path lacks are restated here, each one
//    switchable:
//      - linear isotropic hardening in the radial return (the reference's
//        BILINEAR model never updates sigma_y and reads an uninitialised Et,
//        src/common/Mechanical.C:1723-1770); restated from
//        Mechanical.C:1664-1839 with sigma_y = sy0 + H*eps_p and Et = H;
//      - 3-D viscous hourglass forces for 1-point hexahedra (the reference's
//        calcElemHourglassForces is a no-op in 3-D, Mechanical.C:1939-1942);
//        restated from src/common/test_1el_3D.cpp:159-199 with the current
//        element volume and density;
//    and the step records the top reaction force (sum of the internal force
//    over a node set, after assemblyForces).
//  A rigid triangle mesh (TriMesh_d) can be attached; the stepwise loop then
//  calls the reference's own CalcContactForces (Contact.C:31-334), records
//  its reaction (react_force[0].z) and ramps, moves and re-planes the mesh at
//  the end of the step as SolveChungHulbert does (Solver_explicit.C:980-1004).
//  With all switches off, O2 reproduces O1 bit for bit (checked by tests).
#include "Domain_d.h"
#include "Material.cuh"
#include "Mesh.h"
#include "VTKWriter.h"
// NastranReader::read is an inline member defined in this source file, so it
// is compiled here, where the harness constructs a reader.
#include "NastranReader.cpp"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

using namespace MetFEM;

namespace {

struct PlaneContact {
  bool on = false;
  double z0 = 0.0;      // plane height at t = 0
  double vz = 0.0;      // plane velocity (negative: moving down)
  double kpen = 0.0;    // penalty stiffness [N/m per node area unit], see below
  double mu = 0.0;      // Coulomb friction coefficient
};

class RefDomain : public Domain_d {
 public:
  // restated-piece switches
  int linear_hardening = 0;
  double hg_coef = 0.0;
  std::vector<double> mat_H;               // per material hardening modulus
  std::vector<Material_> mats;             // material table (index = id)
  std::vector<int> elem_mat;               // per element material id
  std::vector<int> reaction_nodes;
  int reaction_dim = 2;
  std::vector<double> reaction_hist;
  std::vector<double> ekin_hist, eint_hist;  // computeEnergies after every step
  double eint_acc = 0.0;
  TriMesh_d *tm = nullptr;                  // rigid triangle mesh (contact)
  double temp = 0.0;                        // uniform temperature T[]
  bool thermal_on = false;
  std::vector<double3> v_orig;              // its velocity before the ramp

  // A TriMesh_d filled from arrays: one mesh with the given id, uniform
  // velocity (node_v and m_v); normals, centroids and plane coefficients as
  // the reference computes them.
  static TriMesh_d *mesh_from_arrays(int nn, const double *xyz, int ne, const int *tri,
                                     const double *vel, int id) {
    TriMesh_d *m = new TriMesh_d();
    m->dimension = 3;
    m->nodecount = nn;
    m->elemcount = ne;
    m->mesh_count = 1;
    malloc_t(m->node, double3, nn);
    malloc_t(m->node_v, double3, nn);
    malloc_t(m->elnode, int, 3 * ne);
    malloc_t(m->centroid, double3, ne);
    malloc_t(m->normal, double3, ne);
    malloc_t(m->pplane, double, ne);
    malloc_t(m->nfar, int, ne);
    malloc_t(m->ele_mesh_id, int, ne);
    malloc_t(m->react_force, double3, 1);
    malloc_t(m->react_p_force, double, 1);
    malloc_t(m->mu_sta, double, 1);
    malloc_t(m->mu_dyn, double, 1);
    for (int n = 0; n < nn; n++) {
      m->node[n] = make_double3(xyz[3 * n], xyz[3 * n + 1], xyz[3 * n + 2]);
      m->node_v[n] = make_double3(vel[0], vel[1], vel[2]);
    }
    for (int e = 0; e < ne; e++) {
      for (int k = 0; k < 3; k++) m->elnode[3 * e + k] = tri[3 * e + k];
      m->ele_mesh_id[e] = id;
    }
    m->m_v = make_double3(vel[0], vel[1], vel[2]);
    m->react_force[0] = make_double3(0., 0., 0.);
    m->heat_cond = 0.0;
    m->T_const = 20.;  // main.C:714
    m->CalcCentroids();
    m->CalcNormals();
    m->CalcSpheres();
    return m;
  }
  void set_trimesh(int nn, const double *xyz, int ne, const int *tri, const double *vel,
                   double mu_s, double mu_d, double pf) {
    tm = mesh_from_arrays(nn, xyz, ne, tri, vel, 0);
    tm->mu_sta[0] = mu_s;
    tm->mu_dyn[0] = mu_d;
    setContactPF(pf);
  }
  // The driver's second rigid body (main.C:756-830): SetMeshVel, addMeshData
  // (whose body is TriMesh_d::AddMesh, called here on the mesh that init
  // attaches with setTriMesh), then CalcSpheres over the whole mesh.
  void add_trimesh(int nn, const double *xyz, int ne, const int *tri, const double *vel) {
    TriMesh_d *m = mesh_from_arrays(nn, xyz, ne, tri, vel, tm->mesh_count);
    tm->AddMesh(*m);
    tm->CalcSpheres();
  }
  long step_count = 0;

  void zero_uninitialised() {
    // Arrays that SetDimension allocates with malloc and the reference never
    // initialises before reading them (Domain_d.C:457-621).
    const int n3 = m_node_count * m_dim;
    const int e6 = m_elem_count * 6;
    const int ea = m_elem_count * m_nodxelem * m_dim;
    for (int i = 0; i < n3; i++) {
      prev_a[i] = 0.0; a[i] = 0.0; v[i] = 0.0; u[i] = 0.0; u_dt[i] = 0.0;
      m_fi[i] = 0.0; m_fe[i] = 0.0; contforce[i] = 0.0;
    }
    for (int i = 0; i < e6; i++) {
      m_sigma[i] = 0.0; m_tau[i] = 0.0; m_eps[i] = 0.0;
      m_str_rate[i] = 0.0; m_rot_rate[i] = 0.0; m_strain_pl_incr[i] = 0.0;
    }
    for (int i = 0; i < ea; i++) { m_f_elem[i] = 0.0; m_f_elem_hg[i] = 0.0; }
    for (int e = 0; e < m_elem_count; e++) { p[e] = 0.0; pl_strain[e] = 0.0; }
    m_artifvisc[0] = 0.0;
    m_artifvisc[1] = 0.0;
    // thermal arrays, also read before they are first written
    for (int i = 0; i < m_elem_count * m_nodxelem; i++) m_dTedt[i] = 0.0;
    for (int e = 0; e < m_elem_count * m_gp_count; e++) m_q_plheat[e] = 0.0;
    for (int n = 0; n < m_node_count; n++) q_cont_conv[n] = 0.0;
  }

  // Preamble of SolveChungHulbert (Solver_explicit.C:120-268), CPU branch.
  void init_stepwise() {
    AssignMatAddress();
    apply_elem_materials();
    InitValues();
    for (int d = 0; d < m_dim; d++) {
      for (int n = 0; n < m_node_count * m_dim; n++) v[n] = a[n] = u[n] = 0.0;
      ImposeBCV(d);
    }
    double rho_b = 0.818200;
    m_alpha = (2.0 * rho_b - 1.0) / (1.0 + rho_b);
    m_beta = (5.0 - 3.0 * rho_b) / ((1.0 + rho_b) * (1.0 + rho_b) * (2.0 - rho_b));
    m_gamma = 1.5 - m_alpha;
    calcElemJAndDerivatives();
    CalcElemInitialVol();
    CalcElemVol();
    calcElemDensity();
    CalcNodalVol();
    CalcNodalMassFromVol();
    for (int n = 0; n < m_node_count; n++)
      for (int d = 0; d < m_dim; d++) ut_prev[m_dim * n + d] = 0.0;
    for (int n = 0; n < m_node_count; n++) T[n] = temp;
    if (thermal_on) setThermalOn();  // main.C:435-441 (setTemp is the loop above)
    if (tm) {
      // what main.C does before the solve (main.C:647-650, :862-873)
      setTriMesh(tm);
      setContactOn();
      SearchExtNodes();
      calcMinEdgeLength();
      v_orig.assign(tm->node_v, tm->node_v + tm->nodecount);
    }
    Time = 0.0;
    step_count = 0;
  }

  void apply_elem_materials() {
    if (elem_mat.empty() || mats.empty()) return;
    for (int e = 0; e < m_elem_count; e++) mat[e] = &mats[elem_mat[e]];
  }

  // CalcStressStrain with linear isotropic hardening, restated from
  // Mechanical.C:1664-1839 (same tensor algebra, same operation order).
  void stress_linear_hardening(double dt_) {
    for (int e = 0; e < m_elem_count; e++) {
      tensor3 RotationRateT, SRT, RS, RotRate, StrRate, ShearStress, Sigma,
          Strain_pl_incr, Strain;
      Strain_pl_incr = nullTensor3();
      int offset_s = e;
      int offset_t = offset_s * 6;
      ShearStress = FromFlatSym(m_tau, offset_t);
      StrRate = FromFlatSym(m_str_rate, offset_t);
      RotRate = FromFlatAntiSym(m_rot_rate, offset_t);
      Strain = FromFlatSym(m_eps, offset_t);
      SRT = ShearStress * Trans(RotRate);
      RS = RotRate * ShearStress;
      ShearStress = ShearStress +
                    dt_ * (2.0 * mat[e]->Elastic().G() *
                               (StrRate - 1.0 / 3.0 * Trace(StrRate) * Identity()) +
                           SRT + RS);
      tensor3 Sigma_trial = -p[offset_s] * Identity() + ShearStress;
      tensor3 s_trial = Sigma_trial - (1.0 / 3.0) * Trace(Sigma_trial) * Identity();
      double J2 = 0.5 * (s_trial.xx * s_trial.xx + 2.0 * s_trial.xy * s_trial.xy +
                         2.0 * s_trial.xz * s_trial.xz + s_trial.yy * s_trial.yy +
                         2.0 * s_trial.yz * s_trial.yz + s_trial.zz * s_trial.zz);
      double sig_trial = sqrt(3.0 * J2);
      int mid = elem_mat.empty() ? 0 : elem_mat[e];
      double H = mat_H.empty() ? 0.0 : mat_H[mid];
      sigma_y[e] = mat[e]->sy0 + H * pl_strain[e];
      double dep = 0.0;
      if (sigma_y[e] < sig_trial) {
        double G = mat[e]->Elastic().G();
        double dgamma = (sig_trial - sigma_y[e]) / (3.0 * G + H);
        double factor = 1.0 - (3.0 * G * dgamma) / sig_trial;
        ShearStress = s_trial * factor;
        pl_strain[e] += dgamma;
        dep = dgamma;
      }
      Sigma = -p[offset_s] * Identity() + ShearStress;
      if (m_thermal) m_q_plheat[e] = 0.0;
      if (dep > 0.0) {
        double f = dep / sigma_y[e];
        Strain_pl_incr.xx = f * (Sigma.xx - 0.5 * (Sigma.yy + Sigma.zz));
        Strain_pl_incr.yy = f * (Sigma.yy - 0.5 * (Sigma.xx + Sigma.zz));
        Strain_pl_incr.zz = f * (Sigma.zz - 0.5 * (Sigma.xx + Sigma.yy));
        Strain_pl_incr.xy = Strain_pl_incr.yx = 1.5 * f * (Sigma.xy);
        Strain_pl_incr.xz = Strain_pl_incr.zx = 1.5 * f * (Sigma.xz);
        Strain_pl_incr.yz = Strain_pl_incr.zy = 1.5 * f * (Sigma.yz);
        if (m_thermal) {  // Mechanical.C:1797-1810
          tensor3 depdt = 1. / dt_ * Strain_pl_incr;
          m_q_plheat[e] = m_plheatfraction *
                          (Sigma.xx * depdt.xx + 2.0 * Sigma.xy * depdt.yx +
                           2.0 * Sigma.xz * depdt.zx + Sigma.yy * depdt.yy +
                           2.0 * Sigma.yz * depdt.yz + Sigma.zz * depdt.zz);
        }
      }
      Strain = Strain + dt_ * StrRate;
      ToFlatSymPtr(Sigma, m_sigma, offset_t);
      ToFlatSymPtr(ShearStress, m_tau, offset_t);
      ToFlatSymPtr(Strain, m_eps, offset_t);
      ToFlatSymPtr(Strain_pl_incr, m_strain_pl_incr, offset_t);
    }
  }

  // 3-D viscous hourglass control for 1-point hexahedra, restated from
  // test_1el_3D.cpp:159-199 (calc_hg_forces), with the current element volume
  // and density (the Fortran prototype f90_ver/src/Mechanical.f90:299 also
  // uses the current volume).
  void hourglass_3d() {
    static const double Sig[4][8] = {{1., 1., -1., -1., -1., -1., 1., 1.},
                                     {1., -1., -1., 1., -1., 1., 1., -1.},
                                     {1., -1., 1., -1., 1., -1., 1., -1.},
                                     {-1., 1., -1., 1., 1., -1., 1., -1.}};
    for (int e = 0; e < m_elem_count; e++) {
      double *fhg = &m_f_elem_hg[e * 8 * 3];
      double hmod[3][4] = {{0.0}};
      for (int i = 0; i < 8; i++)
        for (int d = 0; d < 3; d++) fhg[3 * i + d] = 0.0;
      for (int j = 0; j < 4; j++)
        for (int i = 0; i < 8; i++)
          for (int d = 0; d < 3; d++) hmod[d][j] += getVElem(e, i, d) * Sig[j][i];
      double ch = hg_coef * pow(vol[e], 0.6666666) * rho[e] * 0.25 * mat[e]->cs0;
      for (int j = 0; j < 4; j++)
        for (int i = 0; i < 8; i++)
          for (int d = 0; d < 3; d++) fhg[3 * i + d] -= ch * hmod[d][j] * Sig[j][i];
    }
  }

  // One iteration of the reference loop body, CPU branch, default options
  // (Solver_explicit.C:346-1167).
  void step() {
    UpdatePrediction();
    for (int d = 0; d < m_dim; d++) ImposeBCV(d);
    calcElemJAndDerivatives();
    CalcElemVol();
    CalcNodalVol();
    CalcNodalMassFromVol();
    calcElemStrainRates();
    if (m_thermal) calcThermalExpansion();  // Solver_explicit.C:719-720
    if (m_press_algorithm == 0)
      calcElemPressure();
    else if (m_press_algorithm == 1)
      calcElemPressureANP();
    calcNodalPressureFromElemental();
    if (linear_hardening)
      stress_linear_hardening(dt);
    else
      CalcStressStrain(dt);
    calcArtificialViscosity();
    calcElemForces();
    calcElemHourglassForces();
    if (hg_coef != 0.0 && m_dim == 3 && m_nodxelem == 8) hourglass_3d();
    if (tm) CalcContactForces();
    assemblyForces();
    for (int i = 0; i < m_node_count * m_dim; ++i)
      if (!std::isfinite(m_fi[i])) m_fi[i] = 0.0;
    double r = 0.0;
    if (tm)
      r = tm->react_force[0].z;
    else
      for (size_t k = 0; k < reaction_nodes.size(); k++)
        r += m_fi[m_dim * reaction_nodes[k] + reaction_dim];
    reaction_hist.push_back(r);
    calcAccel();
    ImposeBCAAllDim();
    UpdateCorrectionAccVel();
    ImposeBCVAllDim();
    UpdateCorrectionPos();
    if (tm) {
      const double RAMP_FRACTION = 1.0e-2;  // Solver_explicit.C:309, :980-991
      double f = 1.0;
      if (Time < RAMP_FRACTION * end_t) f = pow(Time / (RAMP_FRACTION * end_t), 0.5);
      for (int n = 0; n < tm->nodecount; n++) tm->node_v[n] = f * v_orig[n];
      tm->Move(dt);
      tm->CalcCentroids();
      tm->CalcNormals();
      tm->UpdatePlaneCoeff();
    }
    if (m_thermal) ThermalCalcs();  // Solver_explicit.C:1008-1011
    // end of the loop body (Solver_explicit.C:1029-1031)
    double ekin = 0.0, deint = 0.0, devisc = 0.0;
    computeEnergies(dt, ekin, deint, devisc);
    eint_acc += deint;
    ekin_hist.push_back(ekin);
    eint_hist.push_back(eint_acc);
    Time += dt;
    step_count++;
  }

  double *node_arr(int which) {
    switch (which) {
      case 0: return x;
      case 1: return v;
      case 2: return a;
      case 3: return u;
      case 4: return prev_a;
      case 5: return m_fi;
      case 6: return u_dt;
      default: return nullptr;
    }
  }
  double *node_scalar(int which) {
    switch (which) {
      case 0: return m_mdiag;
      case 1: return m_voln;
      case 2: return p_node;
      case 3: return T;
      default: return nullptr;
    }
  }
  double *elem_scalar(int which) {
    switch (which) {
      case 0: return vol;
      case 1: return vol_0;
      case 2: return m_detJ;
      case 3: return p;
      case 4: return pl_strain;
      case 5: return sigma_y;
      case 6: return rho;
      default: return nullptr;
    }
  }
  double *elem_tensor(int which) {
    switch (which) {
      case 0: return m_sigma;
      case 1: return m_tau;
      case 2: return m_eps;
      case 3: return m_str_rate;
      case 4: return m_rot_rate;
      default: return nullptr;
    }
  }
  int dim() const { return m_dim; }
  int npe() const { return m_nodxelem; }
  int nn() const { return m_node_count; }
  int get_surface(unsigned char *ext, double *area, double *nodlen) const {
    if (!tm) return 0;
    for (int i = 0; i < m_node_count; i++) {
      ext[i] = ext_nodes[i] ? 1 : 0;
      area[i] = node_area[i];
      double l = 0.0;
      for (int e = 0; e < m_nodel_count[i]; e++)
        l += m_elem_length[m_nodel[m_nodel_offset[i] + e]];
      nodlen[i] = l / m_nodel_count[i];
    }
    return m_node_count;
  }
  void get_contforce(double *out) const {
    std::memcpy(out, contforce, sizeof(double) * m_node_count * m_dim);
  }
  int ne() const { return m_elem_count; }
  void get_derivs(double *out) {
    // [E][3][npe]
    for (int e = 0; e < m_elem_count; e++)
      for (int d = 0; d < 3; d++)
        for (int j = 0; j < m_nodxelem; j++)
          out[(e * 3 + d) * m_nodxelem + j] = getDerivative(e, 0, d, j);
  }
  void get_elem_forces(double *f, double *fhg) {
    int n = m_elem_count * m_nodxelem * m_dim;
    std::memcpy(f, m_f_elem, sizeof(double) * n);
    std::memcpy(fhg, m_f_elem_hg, sizeof(double) * n);
  }
  void get_conn(int *elnod, int *nodel, int *nodel_loc, int *off, int *cnt) {
    for (int i = 0; i < m_elem_count * m_nodxelem; i++) elnod[i] = (int)m_elnod[i];
    int tot = 0;
    for (int n = 0; n < m_node_count; n++) {
      off[n] = m_nodel_offset[n];
      cnt[n] = m_nodel_count[n];
      tot += m_nodel_count[n];
    }
    for (int i = 0; i < tot; i++) {
      nodel[i] = m_nodel[i];
      nodel_loc[i] = m_nodel_loc[i];
    }
  }
  void set_conn_from_elnod(int *elnod) { setNodElem(elnod); }
  void set_time(double t) { Time = t; }
  double time() const { return Time; }
  double get_dt() const { return dt; }
  void set_press_alg(int alg) { m_press_algorithm = alg; }
  void set_stab(const double *s) {
    m_stab.alpha_free = s[0]; m_stab.alpha_contact = s[1];
    m_stab.hg_coeff_free = s[2]; m_stab.hg_coeff_contact = s[3];
    m_stab.av_coeff_div = s[4]; m_stab.av_coeff_bulk = s[5];
    m_stab.log_factor = s[6]; m_stab.pspg_scale = s[7];
    m_stab.p_pspg_bulkfac = s[8]; m_stab.J_min = s[9];
  }
  void set_artif_visc(double al, double be) { m_artifvisc[0] = al; m_artifvisc[1] = be; }
  void quiet_output() { setdtOut(1.0e30); }
};

}  // namespace

extern "C" {

void *wfr_create(void) { return new RefDomain(); }
void wfr_destroy(void *h) { delete static_cast<RefDomain *>(h); }

// AddBoxLength(V = origin, L, r, red_int = true, tritetra) (Domain_d.C:1136)
void wfr_add_box(void *h, double ox, double oy, double oz, double Lx, double Ly,
                 double Lz, double r, int tritetra) {
  RefDomain *d = static_cast<RefDomain *>(h);
  d->AddBoxLength(make_double3(ox, oy, oz), make_double3(Lx, Ly, Lz), r, true,
                  tritetra != 0);
  d->zero_uninitialised();
}

// Builds a domain from explicit nodes and connectivity through the same path
// CreateFromLSDyna uses (SetDimension + setNodElem, Domain_d.C:1647-1699).
void wfr_set_mesh(void *h, int nn, int ne, int npe, const double *xyz,
                  const int *elnod) {
  RefDomain *d = static_cast<RefDomain *>(h);
  LS_Dyna::lsdynaReader rd;
  rd.m_node.resize(nn);
  for (int n = 0; n < nn; n++)
    for (int k = 0; k < 3; k++) rd.m_node[n].m_x[k] = xyz[3 * n + k];
  rd.m_elem.resize(ne);
  rd.m_elem_count = ne;
  for (int e = 0; e < ne; e++) {
    rd.m_elem[e].node.resize(npe);
    for (int a = 0; a < npe; a++) rd.m_elem[e].node[a] = elnod[e * npe + a];
  }
  d->m_timeint_type = TimeInt::EXPLICIT;
  d->CreateFromLSDyna(rd);
  d->zero_uninitialised();
}

int wfr_dim(void *h) { return static_cast<RefDomain *>(h)->dim(); }
int wfr_npe(void *h) { return static_cast<RefDomain *>(h)->npe(); }
int wfr_node_count(void *h) { return static_cast<RefDomain *>(h)->nn(); }
int wfr_elem_count(void *h) { return static_cast<RefDomain *>(h)->ne(); }

void wfr_get_conn(void *h, int *elnod, int *nodel, int *nodel_loc, int *off, int *cnt) {
  static_cast<RefDomain *>(h)->get_conn(elnod, nodel, nodel_loc, off, cnt);
}

void wfr_set_node(void *h, int n, double x, double y, double z) {
  static_cast<RefDomain *>(h)->setNode(n, x, y, z);
}

// Material table. model: 0 BILINEAR (linear hardening restated when
// wfr_set_linear_hardening(1)), 1 HOLLOMON (reference law, Material.cuh:353).
void wfr_set_materials(void *h, int nmat, const double *E, const double *nu,
                       const double *rho, const double *sy0, const double *H,
                       const int *model, const double *hol_K, const double *hol_m) {
  RefDomain *d = static_cast<RefDomain *>(h);
  d->mats.clear();
  d->mat_H.clear();
  for (int i = 0; i < nmat; i++) {
    Elastic_ el(E[i], nu[i]);
    Material_ m(el);
    m.cs0 = sqrt(m.Elastic().BulkMod() / rho[i]);
    m.Material_model = model[i];
    m.sy0 = sy0[i];
    m.Ep = 0.0;
    if (model[i] == HOLLOMON) m.InitHollomon(el, sy0[i], hol_K[i], hol_m[i]);
    d->mats.push_back(m);
    d->mat_H.push_back(H[i]);
  }
  d->setDensity(rho[0]);
  d->AssignMaterial(&d->mats[0]);
}

// Material_::Init_JohnsonCook (Material.cuh:105-114) on material `mat`; the
// reference's CalcStressStrain reads the temperature T[e], set uniform here.
void wfr_set_johnson_cook(void *h, int mat, double B, double n, double C, double eps0, double m,
                          double Tm, double Tt, double T) {
  RefDomain *d = static_cast<RefDomain *>(h);
  Material_ &M = d->mats[mat];
  Elastic_ el = M.Elastic();
  M.Init_JohnsonCook(el, M.sy0, B, n, C, eps0, m, Tm, Tt);
  d->temp = T;
  // AssignMaterial copies material 0 into the domain (Domain_d.C:903-907)
  if (mat == 0) d->AssignMaterial(&d->mats[0]);
}

// The GMT law on material `mat`: the reference's CalcStressStrain reads the
// constants from the Material_ fields (Material.cuh:63-78), which the GMT
// class constructor leaves unset (its own members of the same names hide
// them), so they are set here directly; c = {n1, n2, C1, C2, m1, m2, I1, I2},
// range = {e_min, e_max, er_min, er_max, T_min, T_max}; T the uniform T[].
void wfr_set_gmt(void *h, int mat, const double *c, const double *range, double T) {
  RefDomain *d = static_cast<RefDomain *>(h);
  Material_ &M = d->mats[mat];
  M.Material_model = _GMT_;
  M.n1 = c[0]; M.n2 = c[1]; M.C1 = c[2]; M.C2 = c[3];
  M.m1 = c[4]; M.m2 = c[5]; M.I1 = c[6]; M.I2 = c[7];
  M.e_min = range[0]; M.e_max = range[1];
  M.er_min = range[2]; M.er_max = range[3];
  M.T_min = range[4]; M.T_max = range[5];
  d->temp = T;
  if (mat == 0) d->AssignMaterial(&d->mats[0]);
}

// Thermal coupling as the JSON driver sets it (main.C:424-441): every node at T0.
void wfr_set_thermal(void *h, int on, double T0) {
  RefDomain *d = static_cast<RefDomain *>(h);
  d->thermal_on = on != 0;
  d->temp = T0;
}
// Material thermal constants (main.C:575-577) on material `mat`, re-assigned
// because AssignMaterial copies material 0.
void wfr_set_material_thermal(void *h, int mat, double k_T, double cp_T, double exp_T) {
  RefDomain *d = static_cast<RefDomain *>(h);
  d->mats[mat].k_T = k_T;
  d->mats[mat].cp_T = cp_T;
  d->mats[mat].exp_T = exp_T;
  if (mat == 0) d->AssignMaterial(&d->mats[0]);
}
// Die heat transfer (main.C:714-719): TriMesh_d heat_cond and T_const.
void wfr_set_contact_heat(void *h, double heat_cond, double T_die) {
  RefDomain *d = static_cast<RefDomain *>(h);
  if (d->tm) {
    d->tm->heat_cond = heat_cond;
    d->tm->T_const = T_die;
  }
}

void wfr_set_elem_materials(void *h, const int *ids) {
  RefDomain *d = static_cast<RefDomain *>(h);
  d->elem_mat.assign(ids, ids + d->ne());
}

void wfr_set_linear_hardening(void *h, int on) {
  static_cast<RefDomain *>(h)->linear_hardening = on;
}
void wfr_set_hourglass(void *h, double coef) { static_cast<RefDomain *>(h)->hg_coef = coef; }
void wfr_set_press_algorithm(void *h, int alg) { static_cast<RefDomain *>(h)->set_press_alg(alg); }
void wfr_set_stab(void *h, const double *s10) { static_cast<RefDomain *>(h)->set_stab(s10); }
void wfr_set_artif_visc(void *h, double al, double be) {
  static_cast<RefDomain *>(h)->set_artif_visc(al, be);
}
// Domain_d::m_plheatfraction and m_max_edot, as the JSON driver sets them
// from plHeatFrac and maxStrRate (main.C:218, 228).
void wfr_set_plastic_heat_fraction(void *h, double f) {
  static_cast<RefDomain *>(h)->m_plheatfraction = f;
}
void wfr_set_max_strain_rate(void *h, double r) { static_cast<RefDomain *>(h)->m_max_edot = r; }

void wfr_add_bc_vel_node(void *h, int node, int dim, double val) {
  static_cast<RefDomain *>(h)->AddBCVelNode(node, dim, val);
}
void wfr_allocate_bcs(void *h) { static_cast<RefDomain *>(h)->AllocateBCs(); }

void wfr_set_reaction_nodes(void *h, int n, const int *nodes, int dim) {
  RefDomain *d = static_cast<RefDomain *>(h);
  d->reaction_nodes.assign(nodes, nodes + n);
  d->reaction_dim = dim;
}

void wfr_set_dt(void *h, double dt) { static_cast<RefDomain *>(h)->SetDT(dt); }
void wfr_set_end_time(void *h, double t) { static_cast<RefDomain *>(h)->SetEndTime(t); }
void wfr_set_nproc(void *h, int n) { static_cast<RefDomain *>(h)->setNproc(n); }

void wfr_init(void *h) { static_cast<RefDomain *>(h)->init_stepwise(); }
void wfr_step(void *h, int nsteps) {
  RefDomain *d = static_cast<RefDomain *>(h);
  for (int s = 0; s < nsteps; s++) d->step();
}
double wfr_time(void *h) { return static_cast<RefDomain *>(h)->time(); }

// O1: the unmodified reference loop. Runs until end time; writes its own
// side files (Contact_Forces.csv, out.vtk, ...) into the current directory.
void wfr_solve_verbatim(void *h) {
  RefDomain *d = static_cast<RefDomain *>(h);
  d->quiet_output();
  d->SolveChungHulbert();
}

int wfr_get_node_vec(void *h, int which, double *out) {
  RefDomain *d = static_cast<RefDomain *>(h);
  double *p = d->node_arr(which);
  if (!p) return -1;
  std::memcpy(out, p, sizeof(double) * d->nn() * d->dim());
  return 0;
}
int wfr_get_node_scalar(void *h, int which, double *out) {
  RefDomain *d = static_cast<RefDomain *>(h);
  double *p = d->node_scalar(which);
  if (!p) return -1;
  std::memcpy(out, p, sizeof(double) * d->nn());
  return 0;
}
int wfr_get_elem_scalar(void *h, int which, double *out) {
  RefDomain *d = static_cast<RefDomain *>(h);
  double *p = d->elem_scalar(which);
  if (!p) return -1;
  std::memcpy(out, p, sizeof(double) * d->ne());
  return 0;
}
int wfr_get_elem_tensor(void *h, int which, double *out) {
  RefDomain *d = static_cast<RefDomain *>(h);
  double *p = d->elem_tensor(which);
  if (!p) return -1;
  std::memcpy(out, p, sizeof(double) * d->ne() * 6);
  return 0;
}
void wfr_get_derivs(void *h, double *out) { static_cast<RefDomain *>(h)->get_derivs(out); }
void wfr_get_elem_forces(void *h, double *f, double *fhg) {
  static_cast<RefDomain *>(h)->get_elem_forces(f, fhg);
}
int wfr_get_reaction(void *h, double *out, int maxn) {
  RefDomain *d = static_cast<RefDomain *>(h);
  int n = (int)d->reaction_hist.size();
  if (n > maxn) n = maxn;
  for (int i = 0; i < n; i++) out[i] = d->reaction_hist[i];
  return (int)d->reaction_hist.size();
}

void wfr_set_trimesh(void *h, int nn, const double *xyz, int ne, const int *tri,
                     const double *vel, double mu_s, double mu_d, double pf) {
  static_cast<RefDomain *>(h)->set_trimesh(nn, xyz, ne, tri, vel, mu_s, mu_d, pf);
}
void wfr_add_trimesh(void *h, int nn, const double *xyz, int ne, const int *tri,
                     const double *vel) {
  static_cast<RefDomain *>(h)->add_trimesh(nn, xyz, ne, tri, vel);
}
// The reference's Nastran die: NastranReader(path) and
// TriMesh_d(reader, flipnormals, orientNormals, orient_pt) (Mesh.C:560-760).
// Writes up to cap nodes and triangles; returns the node count, *ntri the
// triangle count.
int wfr_nastran_trimesh(const char *path, int flip, int orient, const double *pt, double *xyz,
                        int cap_nodes, int *tri, int cap_tris, int *ntri) {
  NastranReader reader(path);
  const double3 op = make_double3(pt[0], pt[1], pt[2]);
  TriMesh_d m(reader, flip != 0, orient != 0, op);
  for (int n = 0; n < m.nodecount && n < cap_nodes; n++) {
    xyz[3 * n] = m.node[n].x;
    xyz[3 * n + 1] = m.node[n].y;
    xyz[3 * n + 2] = m.node[n].z;
  }
  for (int e = 0; e < m.elemcount && e < cap_tris; e++)
    for (int k = 0; k < 3; k++) tri[3 * e + k] = m.elnode[3 * e + k];
  *ntri = m.elemcount;
  return m.nodecount;
}
int wfr_get_trimesh_nodes(void *h, double *out, int cap) {
  RefDomain *d = static_cast<RefDomain *>(h);
  if (!d->tm) return 0;
  for (int n = 0; n < d->tm->nodecount && n < cap; n++) {
    out[3 * n] = d->tm->node[n].x;
    out[3 * n + 1] = d->tm->node[n].y;
    out[3 * n + 2] = d->tm->node[n].z;
  }
  return d->tm->nodecount;
}
// External-node flags, nodal areas and mean element lengths of the surface
// search (SearchExtNodes, calcMinEdgeLength) after init.
int wfr_get_surface(void *h, unsigned char *ext, double *area, double *nodlen) {
  return static_cast<RefDomain *>(h)->get_surface(ext, area, nodlen);
}
int wfr_get_contforce(void *h, double *out) {
  static_cast<RefDomain *>(h)->get_contforce(out);
  return 0;
}

int wfr_get_energies(void *h, double *ekin, double *eint, int maxn) {
  RefDomain *d = static_cast<RefDomain *>(h);
  int n = (int)d->ekin_hist.size();
  if (n > maxn) n = maxn;
  for (int i = 0; i < n; i++) {
    ekin[i] = d->ekin_hist[i];
    eint[i] = d->eint_hist[i];
  }
  return (int)d->ekin_hist.size();
}

// The reference's own legacy VTK writer on the current state
// (VTKWriter::VTKWriter + writeFile, VTKWriter.C:238-672).
void wfr_write_vtk(void *h, const char *path) {
  RefDomain *d = static_cast<RefDomain *>(h);
  VTKWriter w(d, path);
  w.writeFile();
}

}  // extern "C"
