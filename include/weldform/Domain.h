// Header-only C++ facade over the C ABI (include/wf.h) with the member names
// of the reference's MetFEM::Domain_d (include/common/Domain_d.h:231-1044),
// Material_ and Elastic_ (include/common/Material.cuh:15-156), so drivers
// written against the reference (src/common/main_1_elem_3d.C,
// src/explicit/main.C) port by changing the namespace.
//
// Differences from the reference object: errors throw std::runtime_error
// instead of printing; node readback (getDispVec, ...) reads a host copy
// refreshed after every solve or run.
#pragma once

#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "wf.h"

namespace weldform {

struct double3 {
  double x, y, z;
};
inline double3 make_double3(double x, double y, double z) { return double3{x, y, z}; }
using vector_t = double3;

// Elastic_ (Material.cuh:15-34)
class Elastic_ {
 public:
  Elastic_() : E_m(0), nu_m(0) {}
  Elastic_(double e, double nu) : E_m(e), nu_m(nu) {}
  double E() const { return E_m; }
  double Poisson() const { return nu_m; }
  double BulkMod() const { return E_m / (3.0 * (1.0 - 2.0 * nu_m)); }
  double G() const { return E_m / (2.0 * (1.0 + nu_m)); }

 private:
  double E_m, nu_m;
};

// model numbers of Material.cuh:9-12 (GMT_MODEL is the reference's _GMT_)
enum { BILINEAR = 0, HOLLOMON = 1, JOHNSON_COOK = 2, GMT_MODEL = 3 };

// Material_ (Material.cuh:36-156): the fields the explicit step reads.
class Material_ {
 public:
  Material_() = default;
  explicit Material_(const Elastic_ &el) : elastic_m(el) {}
  const Elastic_ &Elastic() const { return elastic_m; }
  void InitHollomon(const Elastic_ &el, double sy0_, double k_, double m_) {
    elastic_m = el;
    Material_model = HOLLOMON;
    sy0 = sy0_;
    K = k_;
    m = m_;
  }
  // Material_::Init_JohnsonCook (Material.cuh:105-114); T is the uniform
  // element temperature the yield function reads without thermal coupling
  // (with it, each element takes the mean of its node temperatures)
  void Init_JohnsonCook(const Elastic_ &el, double a, double b, double n_, double c,
                        double eps_0_, double m_, double T_m_, double T_t_, double T_ = 0.0) {
    elastic_m = el;
    Material_model = JOHNSON_COOK;
    sy0 = a;
    B = b;
    n = n_;
    C = c;
    eps_0 = eps_0_;
    m = m_;
    T_m = T_m_;
    T_t = T_t_;
    T = T_;
  }
  int Material_model = BILINEAR;
  double sy0 = 1.0e10;  // as the reference constructor
  double B = 0.0, n = 1.0, C = 0.0, eps_0 = 1.0, T_m = 1.0e10, T_t = 0.0, T = 0.0;
  double Ep = 0.0;      // hardening modulus of the bilinear law
  double K = 1.0, m = 1.0;
  double cs0 = 0.0;     // informational; the library uses sqrt(K_bulk / rho)
  double k_T = 0.0, cp_T = 0.0, exp_T = 0.0;  // thermal (Material.cuh:81-83)
  // GMT constants and ranges (Material.cuh:63-78)
  double C1 = 0.0, C2 = 0.0, m1 = 0.0, m2 = 0.0, n1 = 0.0, n2 = 0.0, I1 = 0.0, I2 = 0.0;
  double e_min = 0.0, e_max = 1.0e10, er_min = 0.0, er_max = 1.0e10, T_min = 0.0, T_max = 1.0e10;

 private:
  Elastic_ elastic_m;
};

// GMT (Material.cuh:255-290) with the constructor's argument order. The
// constants go to the Material_ fields the law reads; T (inherited) is the
// temperature without thermal coupling. e_min must be > 0 (wf_set_gmt).
class GMT : public Material_ {
 public:
  GMT(const Elastic_ &el, double n1_, double n2_, double C1_, double C2_, double m1_, double m2_,
      double I1_, double I2_, double e_min_ = 0.0, double e_max_ = 1.0e10, double er_min_ = 0.0,
      double er_max_ = 1.0e10, double T_min_ = 0.0, double T_max_ = 1.0e10)
      : Material_(el) {
    Material_model = GMT_MODEL;
    n1 = n1_; n2 = n2_; C1 = C1_; C2 = C2_; m1 = m1_; m2 = m2_; I1 = I1_; I2 = I2_;
    e_min = e_min_; e_max = e_max_; er_min = er_min_; er_max = er_max_;
    T_min = T_min_; T_max = T_max_;
  }
};

class Domain_d {
 public:
  explicit Domain_d(int precision = WF_FP64, int device = 0) {
    check(wf_domain_create_on_device(&d_, device), "Domain_d");
    check(wf_set_precision(d_, precision), "precision");
  }
  ~Domain_d() {
    if (d_) wf_domain_destroy(d_);
  }
  Domain_d(const Domain_d &) = delete;
  Domain_d &operator=(const Domain_d &) = delete;

  // mesh (Domain_d.h:440-441, 495, 687)
  void AddBoxLength(const vector_t &V, const vector_t &L, const double &r,
                    const bool &red_int = true, const bool &tritetra = false) {
    const double v[3] = {V.x, V.y, V.z}, l[3] = {L.x, L.y, L.z};
    check(wf_add_box_length(d_, v, l, r, red_int ? 1 : 0, tritetra ? 1 : 0), "AddBoxLength");
  }
  void setNodElem(int64_t nn, int64_t ne, int npe, const double *xyz, const int32_t *elnod) {
    check(wf_set_mesh(d_, nn, ne, npe, xyz, elnod), "setNodElem");
  }
  void setNode(const int &i, const double &x, const double &y, const double &z) {
    check(wf_set_node(d_, i, x, y, z), "setNode");
  }
  int getNodeCount() const { return (int)sizes().nn; }
  int getElemCount() const { return (int)sizes().ne; }

  // material (Domain_d.h:554, 583)
  void setDensity(const double &r) {
    rho_ = r;
    check(wf_set_density(d_, r), "setDensity");
  }
  void AssignMaterial(Material_ *m) { AssignMaterials(std::vector<Material_ *>{m}); }
  void AssignMaterials(const std::vector<Material_ *> &ms) {
    std::vector<wf_material> t(ms.size());
    for (size_t i = 0; i < ms.size(); i++) {
      const Material_ &m = *ms[i];
      t[i] = wf_material{m.Material_model, m.Elastic().E(), m.Elastic().Poisson(), rho_,
                         m.sy0, m.Ep, m.K, m.m};
    }
    check(wf_set_materials(d_, (int32_t)t.size(), t.data()), "AssignMaterial");
    for (size_t i = 0; i < ms.size(); i++) {
      const Material_ &m = *ms[i];
      if (m.Material_model == JOHNSON_COOK)
        check(wf_set_johnson_cook(d_, (int32_t)i, m.B, m.n, m.C, m.eps_0, m.m, m.T_m, m.T_t, m.T),
              "Init_JohnsonCook");
      if (m.Material_model == GMT_MODEL) {
        const double c[8] = {m.n1, m.n2, m.C1, m.C2, m.m1, m.m2, m.I1, m.I2};
        const double r[6] = {m.e_min, m.e_max, m.er_min, m.er_max, m.T_min, m.T_max};
        check(wf_set_gmt(d_, (int32_t)i, c, r, m.T), "GMT");
      }
      if (m.cp_T > 0.0)
        check(wf_set_material_thermal(d_, (int32_t)i, m.k_T, m.cp_T, m.exp_T), "thermal");
    }
  }
  // thermal coupling (Domain_d.h:676-684): setThermalOn, setTemp(T0)
  void setThermalOn() {
    thermal_ = true;
    check(wf_set_thermal(d_, 1, T0_), "setThermalOn");
  }
  void setTemp(const double &val) {
    T0_ = val;
    check(wf_set_thermal(d_, thermal_ ? 1 : 0, T0_), "setTemp");
  }
  // TriMesh_d heat_cond and T_const of the rigid bodies
  void setContactHeat(double heat_cond, double T_die) {
    check(wf_set_contact_heat(d_, heat_cond, T_die), "contact heat");
  }
  void setElemMaterials(const std::vector<int32_t> &ids) {
    check(wf_set_elem_materials(d_, ids.data()), "setElemMaterials");
  }

  // BCs (Domain_d.h:518, 536-537)
  void AddBCVelNode(const int &node, const int &dim, const double &val) {
    check(wf_add_bc_vel_node(d_, node, dim, val), "AddBCVelNode");
  }
  int AddBCVelZone(const vector_t &start, const vector_t &end, const vector_t &vel) {
    const double s[3] = {start.x, start.y, start.z}, e[3] = {end.x, end.y, end.z},
                 v[3] = {vel.x, vel.y, vel.z};
    int64_t c = 0;
    check(wf_add_bc_vel_zone(d_, s, e, v, &c), "AddBCVelZone");
    return (int)c;
  }
  void AllocateBCs() { check(wf_allocate_bcs(d_), "AllocateBCs"); }

  // time and options (Domain_d.h:634-636, 671-672, 770)
  void SetDT(const double &dt) { check(wf_set_dt(d_, dt), "SetDT"); }
  void SetEndTime(const double &t) { check(wf_set_end_time(d_, t), "SetEndTime"); }
  void setHourglass(double coef) { check(wf_set_hourglass(d_, coef), "setHourglass"); }
  void setPressAlgorithm(int alg) { check(wf_set_press_algorithm(d_, alg), "m_press_algorithm"); }
  void setArtifVisc(double a, double b) { check(wf_set_artif_visc(d_, a, b), "m_artifvisc"); }
  // m_plheatfraction and m_max_edot (Domain_d.h:783, 824)
  void setPlasticHeatFraction(double f) {
    check(wf_set_plastic_heat_fraction(d_, f), "m_plheatfraction");
  }
  void setMaxStrainRate(double r) { check(wf_set_max_strain_rate(d_, r), "m_max_edot"); }
  void setContactPlane(double z0, double vz, double kpen, double mu,
                       const std::vector<int32_t> &cand) {
    check(wf_set_contact_plane(d_, z0, vz, kpen, mu, (int64_t)cand.size(), cand.data()),
          "setContactPlane");
  }
  // setTriMesh + setContactOn + setContactPF (Domain_d.h:464, :642, :771) for
  // one rigid triangle mesh with a uniform velocity
  void setTriMesh(const std::vector<double> &xyz, const std::vector<int32_t> &tri,
                  const vector_t &vel, double mu_static = 0.0, double mu_dynamic = 0.0,
                  double penalty_factor = 0.1) {
    const double v[3] = {vel.x, vel.y, vel.z};
    check(wf_set_contact_trimesh(d_, (int64_t)xyz.size() / 3, xyz.data(),
                                 (int64_t)tri.size() / 3, tri.data(), v, mu_static, mu_dynamic,
                                 penalty_factor),
          "setTriMesh");
  }
  // addMeshData (Domain_d.C:2780, TriMesh_d::AddMesh): another rigid body with
  // its own uniform velocity; only body 0 (setTriMesh) feeds the reaction
  void addMeshData(const std::vector<double> &xyz, const std::vector<int32_t> &tri,
                   const vector_t &vel) {
    const double v[3] = {vel.x, vel.y, vel.z};
    check(wf_add_contact_trimesh(d_, (int64_t)xyz.size() / 3, xyz.data(),
                                 (int64_t)tri.size() / 3, tri.data(), v),
          "addMeshData");
  }
  // TriMesh_d(NastranReader(path), flipnormals, orientNormals, orient_pt)
  // (Mesh.C:560-760): die nodes and triangles from a Nastran file
  static void ReadNastranMesh(const std::string &path, bool flipnormals, bool orientNormals,
                              const vector_t &orient_pt, std::vector<double> &xyz,
                              std::vector<int32_t> &tri) {
    const double p[3] = {orient_pt.x, orient_pt.y, orient_pt.z};
    const double *pp = orientNormals ? p : nullptr;
    int64_t nn = 0, nt = 0;
    char err[512] = {0};
    wf_status s = wf_read_nastran(path.c_str(), flipnormals, pp, nullptr, 0, nullptr, 0, &nn,
                                  &nt, err, sizeof(err));
    if (s == WF_OK) {
      xyz.resize(3 * nn);
      tri.resize(3 * nt);
      s = wf_read_nastran(path.c_str(), flipnormals, pp, xyz.data(), nn, tri.data(), nt, &nn,
                          &nt, err, sizeof(err));
    }
    if (s != WF_OK) throw std::runtime_error(path + ": " + err);
  }
  // CreateFromLSDyna (Domain_d.C:1647-1699) from a keyword file
  void CreateFromLSDyna(const std::string &path) {
    check(wf_load_lsdyna(d_, path.c_str()), "CreateFromLSDyna");
  }
  // The JSON driver's setup (src/explicit/main.C:125-1005): mesh, material,
  // BCs, options, dt and end time from a deck
  wf_deck_info LoadDeck(const std::string &path) {
    wf_deck_info info{};
    char err[512] = {0};
    const wf_status s = wf_load_deck(d_, path.c_str(), &info, err, sizeof(err));
    if (s != WF_OK) throw std::runtime_error(path + ": " + err);
    return info;
  }
  void setEnergyHistory(bool on) { check(wf_set_energy_history(d_, on ? 1 : 0), "energies"); }
  void WriteVTK(const std::string &path) {
    check(wf_write_vtk(d_, path.c_str()), "VTKWriter");
  }
  void setReactionNodes(const std::vector<int32_t> &nodes, int dim = 2) {
    check(wf_set_reaction_nodes(d_, (int64_t)nodes.size(), nodes.data(), dim), "reaction");
  }
  // Shortest element edge of the current mesh (after the mesh is uploaded).
  double getMinLength() {
    ensure_init();
    double h = 0.0;
    check(wf_min_edge_length(d_, &h), "getMinLength");
    return h;
  }

  // run (Domain_d.h:633)
  void SolveChungHulbert() {
    ensure_init();
    int64_t n = 0;
    check(wf_solve(d_, &n), "SolveChungHulbert");
    refresh();
  }
  void Run(int64_t nsteps) {
    ensure_init();
    check(wf_run(d_, nsteps), "run");
    refresh();
  }

  // readback (Domain_d.h:476-489)
  vector_t getDispVec(const int &n) const { return at(u_, n); }
  vector_t getVelVec(const int &n) const { return at(v_, n); }
  vector_t getPosVec3(const int &n) const { return at(x_, n); }
  vector_t getIntForceVec(const int &n) const { return at(fi_, n); }
  double getPlStrain(const int &e) const { return pl_.at(e); }
  std::vector<double> getReactionHistory() {
    int64_t n = 0;
    check(wf_get_reaction_history(d_, nullptr, 0, &n), "reaction");
    std::vector<double> r(n);
    check(wf_get_reaction_history(d_, r.data(), n, &n), "reaction");
    return r;
  }
  wf_domain *handle() { return d_; }

 private:
  struct Sizes {
    int64_t nn, ne, tot;
    int32_t npe;
  };
  Sizes sizes() const {
    Sizes s{};
    check(wf_get_sizes(d_, &s.nn, &s.ne, &s.npe, &s.tot), "sizes");
    return s;
  }
  void check(wf_status s, const char *what) const {
    if (s != WF_OK)
      throw std::runtime_error(std::string(what) + ": " + wf_status_string(s) + ": " +
                               wf_last_error(d_));
  }
  void ensure_init() {
    if (!initialized_) {
      check(wf_init(d_), "init");
      initialized_ = true;
    }
  }
  void refresh() {
    const Sizes s = sizes();
    x_.resize(3 * s.nn);
    u_.resize(3 * s.nn);
    v_.resize(3 * s.nn);
    fi_.resize(3 * s.nn);
    pl_.resize(s.ne);
    check(wf_get_node_field(d_, WF_NODE_X, x_.data()), "x");
    check(wf_get_node_field(d_, WF_NODE_U, u_.data()), "u");
    check(wf_get_node_field(d_, WF_NODE_V, v_.data()), "v");
    check(wf_get_node_field(d_, WF_NODE_FI, fi_.data()), "fi");
    check(wf_get_elem_scalar(d_, WF_ELEM_PL_STRAIN, pl_.data()), "pl_strain");
  }
  static vector_t at(const std::vector<double> &a, int n) {
    return make_double3(a.at(3 * n), a.at(3 * n + 1), a.at(3 * n + 2));
  }

  wf_domain *d_ = nullptr;
  bool initialized_ = false;
  double rho_ = 0.0;
  bool thermal_ = false;
  double T0_ = 20.0;
  std::vector<double> x_, u_, v_, fi_, pl_;
};

}  // namespace weldform
