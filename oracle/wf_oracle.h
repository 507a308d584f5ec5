/* CPU restatement of the WeldFormFEM explicit updated-Lagrangian step.
 *
 * TEST INFRASTRUCTURE ONLY. This is the oracle the CUDA path is checked
 * against, and the "port" CPU baseline that bench.py times. Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it; the
 * product library never links or calls it.
 *
 * Every routine restates one reference routine (file:line in its comment)
 * with the same operation order, so that with -ffp-contract=off it agrees bit
 * for bit with the reference compiled from its own sources (oracle/_ref).
 * The API mirrors the product's C ABI (include/wf.h) with a wfo_ prefix.
 */
#ifndef WF_ORACLE_H
#define WF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct wfo_domain wfo_domain;

/* Material_ / Elastic_ (include/common/Material.cuh:15-156). */
typedef struct {
  int model;      /* 0 = bilinear (linear isotropic hardening), 1 = Hollomon, 2 = Johnson-Cook */
  double E, nu, rho;
  double sy0;     /* initial yield stress */
  double H;       /* hardening modulus d(sigma_y)/d(eps_p), model 0 */
  double hol_K, hol_m; /* Hollomon sigma_y = K (eps_p + eps0)^m, model 1 */
} wfo_material;

wfo_domain *wfo_create(void);
void wfo_destroy(wfo_domain *d);
void wfo_set_threads(wfo_domain *d, int nthreads);

/* Domain_d::AddBoxLength(V, L, r, red_int=true, tritetra) (Domain_d.C:1136). */
int wfo_add_box_length(wfo_domain *d, const double V[3], const double L[3], double r,
                       int tritetra);
/* SetDimension + setNodElem, as Domain_d::CreateFromLSDyna (Domain_d.C:1647). */
int wfo_set_mesh(wfo_domain *d, int64_t nn, int64_t ne, int npe, const double *xyz,
                 const int32_t *elnod);
int wfo_set_nodes(wfo_domain *d, const double *xyz);
void wfo_sizes(const wfo_domain *d, int64_t *nn, int64_t *ne, int *npe, int64_t *nodel_tot);
void wfo_get_connectivity(const wfo_domain *d, int32_t *elnod, int32_t *nodel,
                          int32_t *nodel_loc, int32_t *offset, int32_t *count);

int wfo_set_materials(wfo_domain *d, int nmat, const wfo_material *m);
int wfo_set_elem_materials(wfo_domain *d, const int32_t *ids);
/* Johnson-Cook constants of material `mat` (model 2) and its temperature. */
int wfo_set_johnson_cook(wfo_domain *d, int mat, double B, double n, double C, double eps0,
                         double m, double Tm, double Tt, double T);
/* GMT law: c = {n1, n2, C1, C2, m1, m2, I1, I2}, range = {e_min, e_max,
 * er_min, er_max, T_min, T_max}, T the uniform element temperature. */
int wfo_set_gmt(wfo_domain *d, int mat, const double *c, const double *range, double T);
/* Thermal coupling (Domain_d::setThermalOn / setTemp): every node at T0 at init. */
void wfo_set_thermal(wfo_domain *d, int on, double T0);
/* Conductivity, heat capacity and expansion coefficient of material `mat`. */
int wfo_set_material_thermal(wfo_domain *d, int mat, double k_T, double cp_T, double exp_T);
/* Die heat transfer coefficient and temperature (TriMesh_d heat_cond, T_const). */
void wfo_set_contact_heat(wfo_domain *d, double heat_cond, double T_die);
int wfo_add_bc_vel_node(wfo_domain *d, int64_t node, int dim, double val);
int wfo_allocate_bcs(wfo_domain *d);
int wfo_set_reaction_nodes(wfo_domain *d, int64_t n, const int32_t *nodes, int dim);

void wfo_set_dt(wfo_domain *d, double dt);
void wfo_set_end_time(wfo_domain *d, double t);
void wfo_set_hourglass(wfo_domain *d, double coef);
void wfo_set_press_algorithm(wfo_domain *d, int alg);
void wfo_set_stab(wfo_domain *d, const double s[10]);
void wfo_set_artif_visc(wfo_domain *d, double alpha, double beta);
/* m_plheatfraction and m_max_edot (defaults 0.9 and 1e6). */
void wfo_set_plastic_heat_fraction(wfo_domain *d, double f);
void wfo_set_max_strain_rate(wfo_domain *d, double r);
/* 0: lumped mass recomputed every step from the current volume, as the
 * reference loop does (Solver_explicit.C:605-607); 1: mass fixed at its
 * initial value, as the reference's one-element test driver does
 * (src/common/test_1el_3D.cpp:269-270). */
void wfo_set_mass_mode(wfo_domain *d, int mode);
/* Rigid flat die z = z0 + vz t, penalty + Coulomb (Contact.C:58-323). */
void wfo_set_contact_plane(wfo_domain *d, double z0, double vz, double kpen, double mu,
                           const int32_t *cand_nodes, int64_t ncand);

int wfo_init(wfo_domain *d);
int wfo_run(wfo_domain *d, int64_t nsteps);
/* Steps until Time >= end_t, as `while (Time < end_t)` (Solver_explicit.C:346). */
int64_t wfo_solve(wfo_domain *d);
double wfo_time(const wfo_domain *d);

/* Readback. Node vectors: 0 x, 1 v, 2 a, 3 u, 4 prev_a, 5 fi, 6 u_dt, 7 contforce.
 * Node scalars: 0 mass, 1 voln, 2 p_node. Element scalars: 0 vol, 1 vol0, 2 detJ,
 * 3 p, 4 pl_strain, 5 sigma_y, 6 rho. Element tensors (Voigt xx,yy,zz,xy,yz,xz):
 * 0 sigma, 1 tau, 2 eps, 3 str_rate, 4 rot_rate. */
int wfo_get_node_vec(const wfo_domain *d, int which, double *out);
int wfo_get_node_scalar(wfo_domain *d, int which, double *out);
int wfo_get_elem_scalar(const wfo_domain *d, int which, double *out);
int wfo_get_elem_tensor(const wfo_domain *d, int which, double *out);
/* dN/dx * detJ as [E][3][npe]. */
void wfo_get_derivs(const wfo_domain *d, double *out);
void wfo_get_elem_forces(const wfo_domain *d, double *f, double *fhg);
int64_t wfo_get_reaction(const wfo_domain *d, double *out, int64_t cap);
/* Rigid triangle-mesh contact (Domain_d::CalcContactForces, Contact.C:31-334):
 * mesh nodes xyz[3 nnodes], triangles tri[3 ntri], uniform velocity vel,
 * static/dynamic friction, penalty factor (m_contPF). */
void wfo_set_contact_trimesh(wfo_domain *d, int64_t nnodes, const double *xyz, int64_t ntri,
                             const int32_t *tri, const double vel[3], double mu_static,
                             double mu_dynamic, double penalty_factor);
/* Appends rigid body 1, 2, ... (TriMesh_d::AddMesh); only contacts with body 0
 * feed the reaction. Returns -1 without a first body. */
int wfo_add_contact_trimesh(wfo_domain *d, int64_t nnodes, const double *xyz, int64_t ntri,
                            const int32_t *tri, const double vel[3]);
int64_t wfo_get_trimesh_nodes(const wfo_domain *d, double *out, int64_t cap_nodes);
int64_t wfo_get_surface(const wfo_domain *d, uint8_t *ext, double *node_area, double *nodlen);
/* Kinetic energy and accumulated internal energy after each step
 * (Domain_d::computeEnergies, Mechanical.C:2145-2185; Solver_explicit.C:1029-1031). */
int64_t wfo_get_energies(const wfo_domain *d, double *ekin, double *eint, int64_t cap);
/* The loop body in two halves (up to the element and contact forces; from
 * assemblyForces on) and the halo data a slab decomposition exchanges:
 * element forces of [e0, e1) (f_elem then f_hg) and node state of [n0, n1)
 * (x, v, a, prev_a, u). */
void wfo_step_begin(wfo_domain *d);
void wfo_step_end(wfo_domain *d);
int wfo_get_elem_forces_range(const wfo_domain *d, int64_t e0, int64_t e1, double *out);
int wfo_set_elem_forces_range(wfo_domain *d, int64_t e0, int64_t e1, const double *in);
int wfo_get_node_state_range(const wfo_domain *d, int64_t n0, int64_t n1, double *out);
int wfo_set_node_state_range(wfo_domain *d, int64_t n0, int64_t n1, const double *in);

#ifdef __cplusplus
}
#endif
#endif
