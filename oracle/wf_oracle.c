/* CPU restatement of the WeldFormFEM explicit updated-Lagrangian step.
 *
 * TEST INFRASTRUCTURE ONLY (see wf_oracle.h). Built with -ffp-contract=off so
 * that every expression is evaluated exactly as written; each function names
 * the reference routine it restates. Element and node loops are OpenMP
 * parallel; every per-item result is computed by one thread in the reference
 * order, so results do not depend on the thread count.
 */
#include "wf_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  int model;
  double E, nu, rho, sy0, H, hol_K, hol_m;
  double K, G, cs0;          /* Elastic_ (Material.cuh:24-27) */
  double eps0, eps1;         /* Hollomon (Material.cuh:90-104) */
  /* Johnson-Cook (Material_::Init_JohnsonCook, Material.cuh:105-114) and the
   * element temperature it reads (uniform here) */
  double jc_B, jc_n, jc_C, jc_eps0, jc_m, jc_Tm, jc_Tt, jc_T;
  /* GMT (Material_ C1, C2, n1, n2, m1, m2, I1, I2 and the e, er, T ranges,
   * Material.cuh:63-78) and its (uniform) element temperature */
  double g_C1, g_C2, g_n1, g_n2, g_m1, g_m2, g_I1, g_I2;
  double g_emin, g_emax, g_rmin, g_rmax, g_Tmin, g_Tmax, g_T;
  /* thermal constants (Material_ k_T, cp_T, exp_T, Material.cuh:81-83) */
  double k_T, cp_T, exp_T;
} mat_t;

struct wfo_domain {
  int dim, npe, nthreads;
  int64_t nn, ne, nodel_tot;
  double *x, *v, *a, *u, *u_dt, *prev_a, *fi, *fe, *contforce, *ut_prev;
  double *mass, *voln, *p_node, *voln_sum, *voln0_sum, *mass0;
  int32_t *elnod, *nodel, *nodel_loc, *nodel_off, *nodel_cnt;
  double *detJ, *dH, *vol, *vol0, *rho, *rho0, *p, *pl_strain, *sigma_y;
  double *sigma, *tau, *eps, *str_rate, *rot_rate, *pl_incr;
  double *f_elem, *f_hg;
  int nmat;
  mat_t *mats;
  int32_t *elem_mat;
  /* velocity BCs: host staging lists (AddBCVelNode) */
  int64_t bc_count[3], bc_cap[3];
  int64_t *bc_nod[3];
  double *bc_val[3];
  double dt, end_t, time;
  double alpha, beta, gamma;
  double hg_coef;
  int press_alg, mass_mode;
  double stab[10];
  double artif[2];
  double plheat_frac, max_edot;  /* m_plheatfraction, m_max_edot (Domain_d.h:783, 824) */
  int32_t *react_nodes;
  int64_t n_react;
  int react_dim;
  double *react_hist;
  double *ekin_hist, *eint_hist;   /* computeEnergies after every step */
  double eint;
  int64_t hist_len, hist_cap;
  /* rigid plane contact */
  int contact;
  double c_z0, c_vz, c_kpen, c_mu;
  uint8_t *cand;
  double *cfn;
  /* rigid triangle mesh (TriMesh_d, Mesh.h:69-171) and the part's external
   * surface (SearchExtNodes / CalcExtFaceAreas, Domain_d.C:110-290) */
  int tri_on;
  int64_t tri_nn, tri_ne;
  double *tri_x, *tri_vorig, *tri_nrm, *tri_pp;
  int32_t *tri_el, *tri_mid; /* tri_mid: rigid-body index of each triangle */
  int32_t tri_meshes;
  double tri_mu_s, tri_mu_d, tri_pf;
  uint8_t *ext;
  double *node_area, *nodlen, *elem_len;
  /* thermal coupling (Thermal.C): nodal temperature, plastic heat per element,
   * element-node temperature rates, contact heat per node */
  int thermal;
  double T0;
  double *T, *q_plheat, *dTedt, *q_cont;
  double heat_cond, T_die;
  int64_t step_count;
};

#define OMP_FOR _Pragma("omp parallel for schedule(static)")

static void *xcalloc(size_t n, size_t s) { return calloc(n ? n : 1, s); }

static mat_t *mat_of(const wfo_domain *d, int64_t e) {
  return &d->mats[d->elem_mat ? d->elem_mat[e] : 0];
}

wfo_domain *wfo_create(void) {
  wfo_domain *d = (wfo_domain *)calloc(1, sizeof(wfo_domain));
  d->dim = 3;
  d->react_dim = 2;
  d->c_mu = 0.0;
  d->nthreads = 0;
  d->T_die = 20.0;  /* TriMesh_d T_const as the driver sets it (main.C:714) */
  d->plheat_frac = 0.9;   /* Domain_d constructor (Domain_d.h:271) */
  d->max_edot = 1.0e6;    /* Domain_d.h:824 */
  return d;
}

static void free_mesh(wfo_domain *d) {
  void **ptrs[] = {(void **)&d->x, (void **)&d->v, (void **)&d->a, (void **)&d->u,
                   (void **)&d->u_dt, (void **)&d->prev_a, (void **)&d->fi,
                   (void **)&d->fe, (void **)&d->contforce, (void **)&d->ut_prev,
                   (void **)&d->mass, (void **)&d->voln, (void **)&d->p_node,
                   (void **)&d->voln_sum, (void **)&d->voln0_sum, (void **)&d->mass0,
                   (void **)&d->elnod, (void **)&d->nodel, (void **)&d->nodel_loc,
                   (void **)&d->nodel_off, (void **)&d->nodel_cnt, (void **)&d->detJ,
                   (void **)&d->dH, (void **)&d->vol, (void **)&d->vol0, (void **)&d->rho,
                   (void **)&d->rho0, (void **)&d->p, (void **)&d->pl_strain,
                   (void **)&d->sigma_y, (void **)&d->sigma, (void **)&d->tau,
                   (void **)&d->eps, (void **)&d->str_rate, (void **)&d->rot_rate,
                   (void **)&d->pl_incr, (void **)&d->f_elem, (void **)&d->f_hg,
                   (void **)&d->elem_mat, (void **)&d->cand, (void **)&d->cfn,
                   (void **)&d->ext, (void **)&d->node_area, (void **)&d->nodlen,
                   (void **)&d->elem_len, (void **)&d->T, (void **)&d->q_plheat,
                   (void **)&d->dTedt, (void **)&d->q_cont};
  for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++) {
    free(*ptrs[i]);
    *ptrs[i] = NULL;
  }
}

static void free_trimesh(wfo_domain *d) {
  free(d->tri_x);
  free(d->tri_vorig);
  free(d->tri_nrm);
  free(d->tri_pp);
  free(d->tri_el);
  free(d->tri_mid);
  d->tri_x = d->tri_vorig = d->tri_nrm = d->tri_pp = NULL;
  d->tri_el = d->tri_mid = NULL;
  d->tri_on = 0;
  d->tri_meshes = 0;
}

void wfo_destroy(wfo_domain *d) {
  if (!d) return;
  free_mesh(d);
  free_trimesh(d);
  for (int k = 0; k < 3; k++) {
    free(d->bc_nod[k]);
    free(d->bc_val[k]);
  }
  free(d->mats);
  free(d->react_nodes);
  free(d->react_hist);
  free(d->ekin_hist);
  free(d->eint_hist);
  free(d);
}

void wfo_set_threads(wfo_domain *d, int n) {
  d->nthreads = n;
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#endif
}

/* SetDimension (Domain_d.C:457-621): allocation; every array starts at zero
 * (the reference leaves several uninitialised; the harness zeroes them). */
static int alloc_mesh(wfo_domain *d, int64_t nn, int64_t ne, int npe) {
  free_mesh(d);
  d->nn = nn;
  d->ne = ne;
  d->npe = npe;
  size_t n3 = (size_t)nn * 3, e6 = (size_t)ne * 6, ea = (size_t)ne * npe;
  d->x = xcalloc(n3, 8); d->v = xcalloc(n3, 8); d->a = xcalloc(n3, 8);
  d->u = xcalloc(n3, 8); d->u_dt = xcalloc(n3, 8); d->prev_a = xcalloc(n3, 8);
  d->fi = xcalloc(n3, 8); d->fe = xcalloc(n3, 8); d->contforce = xcalloc(n3, 8);
  d->ut_prev = xcalloc(n3, 8);
  d->mass = xcalloc(nn, 8); d->voln = xcalloc(nn, 8); d->p_node = xcalloc(nn, 8);
  d->voln_sum = xcalloc(nn, 8); d->voln0_sum = xcalloc(nn, 8); d->mass0 = xcalloc(nn, 8);
  d->elnod = xcalloc(ea, 4);
  d->nodel_off = xcalloc(nn, 4); d->nodel_cnt = xcalloc(nn, 4);
  d->detJ = xcalloc(ne, 8); d->dH = xcalloc(ea * 3, 8);
  d->vol = xcalloc(ne, 8); d->vol0 = xcalloc(ne, 8); d->rho = xcalloc(ne, 8);
  d->rho0 = xcalloc(ne, 8); d->p = xcalloc(ne, 8); d->pl_strain = xcalloc(ne, 8);
  d->sigma_y = xcalloc(ne, 8);
  d->sigma = xcalloc(e6, 8); d->tau = xcalloc(e6, 8); d->eps = xcalloc(e6, 8);
  d->str_rate = xcalloc(e6, 8); d->rot_rate = xcalloc(e6, 8); d->pl_incr = xcalloc(e6, 8);
  d->f_elem = xcalloc(ea * 3, 8); d->f_hg = xcalloc(ea * 3, 8);
  d->cand = xcalloc(nn, 1); d->cfn = xcalloc(nn, 8);
  d->T = xcalloc(nn, 8); d->q_plheat = xcalloc(ne, 8); d->dTedt = xcalloc(ea, 8);
  d->q_cont = xcalloc(nn, 8);
  return 0;
}

/* Node -> element lists, element-ascending per node: the counting pass and
 * fill pass of Domain_d::setNodElem (Domain_d.C:1508-1611) and of the tail of
 * AddBoxLength (Domain_d.C:1436-1481). */
static int build_nodel(wfo_domain *d) {
  int64_t nn = d->nn, ne = d->ne;
  int npe = d->npe;
  for (int64_t n = 0; n < nn; n++) d->nodel_cnt[n] = 0;
  for (int64_t i = 0; i < ne * npe; i++) {
    int32_t n = d->elnod[i];
    if (n < 0 || n >= nn) return -1;
    d->nodel_cnt[n]++;
  }
  int64_t tot = 0;
  for (int64_t n = 0; n < nn; n++) {
    d->nodel_off[n] = (int32_t)tot;
    tot += d->nodel_cnt[n];
  }
  d->nodel_tot = tot;
  free(d->nodel);
  free(d->nodel_loc);
  d->nodel = xcalloc(tot, 4);
  d->nodel_loc = xcalloc(tot, 4);
  for (int64_t n = 0; n < nn; n++) d->nodel_cnt[n] = 0;
  for (int64_t e = 0; e < ne; e++)
    for (int a = 0; a < npe; a++) {
      int32_t n = d->elnod[e * npe + a];
      int64_t k = d->nodel_off[n] + d->nodel_cnt[n];
      d->nodel[k] = (int32_t)e;
      d->nodel_loc[k] = a;
      d->nodel_cnt[n]++;
    }
  return 0;
}

/* Domain_d::AddBoxLength (Domain_d.C:1136-1504), 3-D branch, 1-point
 * integration. Coordinates are accumulated by repeated addition of 2r as
 * the reference does (Domain_d.C:1215-1235); hexahedra are numbered x-fastest
 * (:1313-1346); tritetra splits each cell into six tetrahedra (:1383-1391). */
int wfo_add_box_length(wfo_domain *d, const double V[3], const double L[3], double r,
                       int tritetra) {
  int nel[3];
  nel[0] = (int)(L[0] / (2.0 * r));
  nel[1] = (int)(L[1] / (2.0 * r));
  nel[2] = (int)(L[2] / (2.0 * r));
  if (!(L[2] > 0.0) || nel[0] <= 0 || nel[1] <= 0 || nel[2] <= 0) return -1;
  int64_t nc = (int64_t)(nel[0] + 1) * (nel[1] + 1) * (nel[2] + 1);
  int64_t ne = (int64_t)nel[0] * nel[1] * nel[2] * (tritetra ? 6 : 1);
  int npe = tritetra ? 4 : 8;
  alloc_mesh(d, nc, ne, npe);
  int64_t p = 0;
  double Xz = V[2];
  for (int k = 0; k < nel[2] + 1; k++) {
    double Xy = V[1];
    for (int j = 0; j < nel[1] + 1; j++) {
      double Xx = V[0];
      for (int i = 0; i < nel[0] + 1; i++) {
        d->x[3 * p] = Xx;
        d->x[3 * p + 1] = Xy;
        d->x[3 * p + 2] = Xz;
        p++;
        Xx = Xx + 2.0 * r;
      }
      Xy = Xy + 2.0 * r;
    }
    Xz = Xz + 2 * r;
  }
  int64_t ei = 0;
  int64_t nnodz = (int64_t)(nel[0] + 1) * (nel[1] + 1);
  for (int ez = 0; ez < nel[2]; ez++)
    for (int ey = 0; ey < nel[1]; ey++)
      for (int ex = 0; ex < nel[0]; ex++) {
        int64_t nb1 = nnodz * ez + (int64_t)(nel[0] + 1) * ey + ex;
        int64_t nb2 = nnodz * ez + (int64_t)(nel[0] + 1) * (ey + 1) + ex;
        int32_t h[8] = {(int32_t)nb1,           (int32_t)(nb1 + 1),
                        (int32_t)(nb2 + 1),     (int32_t)nb2,
                        (int32_t)(nb1 + nnodz), (int32_t)(nb1 + nnodz + 1),
                        (int32_t)(nb2 + nnodz + 1), (int32_t)(nb2 + nnodz)};
        if (!tritetra) {
          for (int a = 0; a < 8; a++) d->elnod[ei + a] = h[a];
          ei += 8;
        } else {
          static const int T[6][4] = {{0, 1, 3, 5}, {1, 2, 3, 5}, {0, 5, 3, 4},
                                      {4, 5, 3, 7}, {5, 6, 3, 7}, {5, 2, 3, 6}};
          for (int t = 0; t < 6; t++) {
            for (int a = 0; a < 4; a++) d->elnod[ei + a] = h[T[t][a]];
            ei += 4;
          }
        }
      }
  return build_nodel(d);
}

int wfo_set_mesh(wfo_domain *d, int64_t nn, int64_t ne, int npe, const double *xyz,
                 const int32_t *elnod) {
  if (nn <= 0 || ne <= 0 || (npe != 4 && npe != 8)) return -1;
  alloc_mesh(d, nn, ne, npe);
  memcpy(d->x, xyz, sizeof(double) * 3 * nn);
  memcpy(d->elnod, elnod, sizeof(int32_t) * ne * npe);
  return build_nodel(d);
}

int wfo_set_nodes(wfo_domain *d, const double *xyz) {
  memcpy(d->x, xyz, sizeof(double) * 3 * d->nn);
  return 0;
}

void wfo_sizes(const wfo_domain *d, int64_t *nn, int64_t *ne, int *npe, int64_t *tot) {
  if (nn) *nn = d->nn;
  if (ne) *ne = d->ne;
  if (npe) *npe = d->npe;
  if (tot) *tot = d->nodel_tot;
}

void wfo_get_connectivity(const wfo_domain *d, int32_t *elnod, int32_t *nodel,
                          int32_t *nodel_loc, int32_t *offset, int32_t *count) {
  if (elnod) memcpy(elnod, d->elnod, sizeof(int32_t) * d->ne * d->npe);
  if (nodel) memcpy(nodel, d->nodel, sizeof(int32_t) * d->nodel_tot);
  if (nodel_loc) memcpy(nodel_loc, d->nodel_loc, sizeof(int32_t) * d->nodel_tot);
  if (offset) memcpy(offset, d->nodel_off, sizeof(int32_t) * d->nn);
  if (count) memcpy(count, d->nodel_cnt, sizeof(int32_t) * d->nn);
}

/* Elastic_(E, nu) (Material.cuh:24-27), Material_::InitHollomon (:90-104),
 * cs0 = sqrt(K / rho) as every reference driver sets it (main.C:507). */
int wfo_set_materials(wfo_domain *d, int nmat, const wfo_material *m) {
  if (nmat <= 0) return -1;
  free(d->mats);
  d->mats = (mat_t *)calloc(nmat, sizeof(mat_t));
  d->nmat = nmat;
  for (int i = 0; i < nmat; i++) {
    mat_t *t = &d->mats[i];
    t->model = m[i].model;
    t->E = m[i].E; t->nu = m[i].nu; t->rho = m[i].rho;
    t->sy0 = m[i].sy0; t->H = m[i].H; t->hol_K = m[i].hol_K; t->hol_m = m[i].hol_m;
    t->K = t->E / (3.0 * (1.0 - 2.0 * t->nu));
    t->G = t->E / (2.0 * (1.0 + t->nu));
    t->cs0 = sqrt(t->K / t->rho);
    if (t->model == 1) {
      t->eps0 = t->sy0 / t->E;
      t->eps1 = pow(t->sy0 / t->hol_K, 1. / t->hol_m);
    }
  }
  /* Domain_d::setDensity (Domain_d.C:952): rho_0 of every element. */
  for (int64_t e = 0; e < d->ne; e++) d->rho0[e] = d->mats[0].rho;
  return 0;
}

int wfo_set_johnson_cook(wfo_domain *d, int mat, double B, double n, double C, double eps0,
                         double m, double Tm, double Tt, double T) {
  if (mat < 0 || mat >= d->nmat) return -1;
  mat_t *t = &d->mats[mat];
  t->jc_B = B;
  t->jc_n = n;
  t->jc_C = C;
  t->jc_eps0 = eps0;
  t->jc_m = m;
  t->jc_Tm = Tm;
  t->jc_Tt = Tt;
  t->jc_T = T;
  return 0;
}

/* GMT(el, n1, n2, C1, C2, m1, m2, I1, I2, e_min, e_max, er_min, er_max, T_min,
 * T_max) (Material.cuh:271-290) with the constants reaching the Material_
 * fields that CalcGMTYieldStress reads; c = {n1, n2, C1, C2, m1, m2, I1, I2},
 * range = {e_min, e_max, er_min, er_max, T_min, T_max}. */
int wfo_set_gmt(wfo_domain *d, int mat, const double *c, const double *range, double T) {
  if (mat < 0 || mat >= d->nmat || !c || !range) return -1;
  mat_t *t = &d->mats[mat];
  t->g_n1 = c[0]; t->g_n2 = c[1]; t->g_C1 = c[2]; t->g_C2 = c[3];
  t->g_m1 = c[4]; t->g_m2 = c[5]; t->g_I1 = c[6]; t->g_I2 = c[7];
  t->g_emin = range[0]; t->g_emax = range[1];
  t->g_rmin = range[2]; t->g_rmax = range[3];
  t->g_Tmin = range[4]; t->g_Tmax = range[5];
  t->g_T = T;
  return 0;
}

int wfo_set_elem_materials(wfo_domain *d, const int32_t *ids) {
  free(d->elem_mat);
  d->elem_mat = xcalloc(d->ne, 4);
  for (int64_t e = 0; e < d->ne; e++) {
    if (ids[e] < 0 || ids[e] >= d->nmat) return -1;
    d->elem_mat[e] = ids[e];
  }
  return 0;
}

/* Domain_d::AddBCVelNode (Domain_d.C:1057-1061). */
int wfo_add_bc_vel_node(wfo_domain *d, int64_t node, int dim, double val) {
  if (dim < 0 || dim > 2 || node < 0 || node >= d->nn) return -1;
  if (d->bc_count[dim] == d->bc_cap[dim]) {
    int64_t cap = d->bc_cap[dim] ? 2 * d->bc_cap[dim] : 64;
    d->bc_nod[dim] = realloc(d->bc_nod[dim], sizeof(int64_t) * cap);
    d->bc_val[dim] = realloc(d->bc_val[dim], sizeof(double) * cap);
    d->bc_cap[dim] = cap;
  }
  d->bc_nod[dim][d->bc_count[dim]] = node;
  d->bc_val[dim][d->bc_count[dim]] = val;
  d->bc_count[dim]++;
  return 0;
}

int wfo_allocate_bcs(wfo_domain *d) { (void)d; return 0; }

int wfo_set_reaction_nodes(wfo_domain *d, int64_t n, const int32_t *nodes, int dim) {
  free(d->react_nodes);
  d->react_nodes = xcalloc(n, 4);
  memcpy(d->react_nodes, nodes, sizeof(int32_t) * n);
  d->n_react = n;
  d->react_dim = dim;
  return 0;
}

void wfo_set_dt(wfo_domain *d, double dt) { d->dt = dt; }
void wfo_set_end_time(wfo_domain *d, double t) { d->end_t = t; }
void wfo_set_hourglass(wfo_domain *d, double c) { d->hg_coef = c; }
void wfo_set_press_algorithm(wfo_domain *d, int alg) { d->press_alg = alg; }
void wfo_set_stab(wfo_domain *d, const double s[10]) { memcpy(d->stab, s, sizeof(d->stab)); }
void wfo_set_artif_visc(wfo_domain *d, double al, double be) { d->artif[0] = al; d->artif[1] = be; }
void wfo_set_plastic_heat_fraction(wfo_domain *d, double f) { d->plheat_frac = f; }
void wfo_set_max_strain_rate(wfo_domain *d, double r) { d->max_edot = r; }
void wfo_set_mass_mode(wfo_domain *d, int mode) { d->mass_mode = mode; }

/* Triangle-mesh normals (TriMesh_d::CalcNormals, Mesh.h:236-262) and plane
 * coefficients with the far node nfar = 2 (CalcSpheres / UpdatePlaneCoeff,
 * Mesh.h:275-284, :300-320). */
static void tri_normals_planes(wfo_domain *d) {
  for (int64_t e = 0; e < d->tri_ne; e++) {
    const double *p0 = &d->tri_x[3 * d->tri_el[3 * e]];
    const double *p1 = &d->tri_x[3 * d->tri_el[3 * e + 1]];
    const double *p2 = &d->tri_x[3 * d->tri_el[3 * e + 2]];
    const double u[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    const double v[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
    const double w[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2],
                         u[0] * v[1] - u[1] * v[0]};
    const double len = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    const double inv = 1.0 / len;
    double *n = &d->tri_nrm[3 * e];
    n[0] = w[0] * inv;
    n[1] = w[1] * inv;
    n[2] = w[2] * inv;
    d->tri_pp[e] = p2[0] * n[0] + p2[1] * n[1] + p2[2] * n[2];
  }
}

void wfo_set_contact_trimesh(wfo_domain *d, int64_t nnodes, const double *xyz, int64_t ntri,
                             const int32_t *tri, const double vel[3], double mu_static,
                             double mu_dynamic, double penalty_factor) {
  free_trimesh(d);
  d->tri_on = 1;
  d->contact = 1;
  d->tri_nn = nnodes;
  d->tri_ne = ntri;
  d->tri_x = xcalloc(3 * nnodes, 8);
  d->tri_vorig = xcalloc(3 * nnodes, 8);
  d->tri_nrm = xcalloc(3 * ntri, 8);
  d->tri_pp = xcalloc(ntri, 8);
  d->tri_el = xcalloc(3 * ntri, 4);
  d->tri_mid = xcalloc(ntri, 4);
  d->tri_meshes = 1;
  memcpy(d->tri_x, xyz, sizeof(double) * 3 * nnodes);
  memcpy(d->tri_el, tri, sizeof(int32_t) * 3 * ntri);
  for (int64_t n = 0; n < nnodes; n++)
    for (int k = 0; k < 3; k++) d->tri_vorig[3 * n + k] = vel[k];
  d->tri_mu_s = mu_static;
  d->tri_mu_d = mu_dynamic;
  d->tri_pf = penalty_factor;
  tri_normals_planes(d);
}

/* TriMesh_d::AddMesh (Mesh.C:445-545): the body's nodes and triangles are
 * appended, triangle node indices offset by the node count so far; its nodes
 * take its velocity, its triangles the next mesh index. */
int wfo_add_contact_trimesh(wfo_domain *d, int64_t nnodes, const double *xyz, int64_t ntri,
                            const int32_t *tri, const double vel[3]) {
  if (!d->tri_on) return -1;
  const int64_t nn0 = d->tri_nn, ne0 = d->tri_ne;
  const int64_t nn = nn0 + nnodes, ne = ne0 + ntri;
  d->tri_x = realloc(d->tri_x, sizeof(double) * 3 * nn);
  d->tri_vorig = realloc(d->tri_vorig, sizeof(double) * 3 * nn);
  d->tri_nrm = realloc(d->tri_nrm, sizeof(double) * 3 * ne);
  d->tri_pp = realloc(d->tri_pp, sizeof(double) * ne);
  d->tri_el = realloc(d->tri_el, sizeof(int32_t) * 3 * ne);
  d->tri_mid = realloc(d->tri_mid, sizeof(int32_t) * ne);
  if (!d->tri_x || !d->tri_vorig || !d->tri_nrm || !d->tri_pp || !d->tri_el || !d->tri_mid) {
    fprintf(stderr, "wf_oracle: out of memory\n");
    abort();
  }
  memcpy(&d->tri_x[3 * nn0], xyz, sizeof(double) * 3 * nnodes);
  for (int64_t n = 0; n < nnodes; n++)
    for (int k = 0; k < 3; k++) d->tri_vorig[3 * (nn0 + n) + k] = vel[k];
  for (int64_t i = 0; i < 3 * ntri; i++) d->tri_el[3 * ne0 + i] = (int32_t)(tri[i] + nn0);
  for (int64_t e = 0; e < ntri; e++) d->tri_mid[ne0 + e] = d->tri_meshes;
  d->tri_meshes++;
  d->tri_nn = nn;
  d->tri_ne = ne;
  tri_normals_planes(d);
  return 0;
}

int64_t wfo_get_trimesh_nodes(const wfo_domain *d, double *out, int64_t cap) {
  const int64_t n = d->tri_nn < cap ? d->tri_nn : cap;
  if (out && d->tri_on && n > 0) memcpy(out, d->tri_x, sizeof(double) * 3 * n);
  return d->tri_on ? d->tri_nn : 0;
}

int64_t wfo_get_surface(const wfo_domain *d, uint8_t *ext, double *node_area, double *nodlen) {
  if (!d->ext) return 0;
  if (ext) memcpy(ext, d->ext, d->nn);
  if (node_area) memcpy(node_area, d->node_area, sizeof(double) * d->nn);
  if (nodlen) memcpy(nodlen, d->nodlen, sizeof(double) * d->nn);
  return d->nn;
}

void wfo_set_contact_plane(wfo_domain *d, double z0, double vz, double kpen, double mu,
                           const int32_t *cand, int64_t ncand) {
  d->contact = 1;
  d->c_z0 = z0;
  d->c_vz = vz;
  d->c_kpen = kpen;
  d->c_mu = mu;
  memset(d->cand, 0, d->nn);
  for (int64_t i = 0; i < ncand; i++) d->cand[cand[i]] = 1;
}

/* ---------------------------------------------------------------------- */
/* Step phases                                                             */
/* ---------------------------------------------------------------------- */

/* Domain_d::ImposeBCV / ImposeBCA (Domain_d.C:1109-1134): serial, list order
 * (a later entry for the same dof wins). */
static void impose_bcv(wfo_domain *d, int dim) {
  for (int64_t i = 0; i < d->bc_count[dim]; i++)
    d->v[3 * d->bc_nod[dim][i] + dim] = d->bc_val[dim][i];
}
static void impose_bca(wfo_domain *d, int dim) {
  for (int64_t i = 0; i < d->bc_count[dim]; i++) d->a[3 * d->bc_nod[dim][i] + dim] = 0.0;
}

/* Domain_d::UpdatePrediction (Domain_d.C:961-974). */
static void update_prediction(wfo_domain *d) {
  const double dt = d->dt, b = d->beta, g = d->gamma;
  int64_t n3 = d->nn * 3;
  OMP_FOR
  for (int64_t ig = 0; ig < n3; ig++) {
    d->u_dt[ig] = dt * (d->v[ig] + (0.5 - b) * dt * d->prev_a[ig]);
    d->v[ig] += (1.0 - g) * dt * d->prev_a[ig];
  }
}

/* Matrix::calcDet for 3x3 (include/common/Matrix.h:593-620). */
static double det3(const double J[3][3]) {
  return J[0][0] * J[1][1] * J[2][2] - J[0][0] * J[1][2] * J[2][1] -
         J[0][1] * J[1][0] * J[2][2] + J[0][1] * J[1][2] * J[2][0] +
         J[0][2] * J[1][0] * J[2][1] - J[0][2] * J[1][1] * J[2][0];
}

/* AdjMat: transposed cofactor matrix (include/common/Matrix.h:694-727). */
static void adj3(const double A[3][3], double R[3][3]) {
  double C[3][3];
  C[0][0] = (A[1][1] * A[2][2] - A[1][2] * A[2][1]);
  C[0][1] = -(A[1][0] * A[2][2] - A[1][2] * A[2][0]);
  C[0][2] = (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
  C[1][0] = -(A[0][1] * A[2][2] - A[0][2] * A[2][1]);
  C[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]);
  C[1][2] = -(A[0][0] * A[2][1] - A[0][1] * A[2][0]);
  C[2][0] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]);
  C[2][1] = -(A[0][0] * A[1][2] - A[0][2] * A[1][0]);
  C[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) R[i][j] = C[j][i];
}

/* Domain_d::calcElemJAndDerivatives, 1-point branches (Domain_d.C:1701-2044):
 * hexahedron (:1822-1851) and tetrahedron (:1866-1887); detJ (:1894). */
static void calc_jacobian_derivs(wfo_domain *d) {
  const int npe = d->npe;
  OMP_FOR
  for (int64_t e = 0; e < d->ne; e++) {
    double x2[8][3], J[3][3], inv[3][3];
    for (int i = 0; i < npe; i++) {
      int64_t n = d->elnod[e * npe + i];
      x2[i][0] = d->x[3 * n];
      x2[i][1] = d->x[3 * n + 1];
      x2[i][2] = d->x[3 * n + 2];
    }
    double *dH = &d->dH[e * 3 * npe];
    if (npe == 8) {
      for (int k = 0; k < 3; k++) {
        J[0][k] = 0.125 * (-x2[0][k] + x2[1][k] + x2[2][k] - x2[3][k] - x2[4][k] +
                           x2[5][k] + x2[6][k] - x2[7][k]);
        J[1][k] = 0.125 * (-x2[0][k] - x2[1][k] + x2[2][k] + x2[3][k] - x2[4][k] -
                           x2[5][k] + x2[6][k] + x2[7][k]);
        J[2][k] = 0.125 * (-x2[0][k] - x2[1][k] - x2[2][k] - x2[3][k] + x2[4][k] +
                           x2[5][k] + x2[6][k] + x2[7][k]);
      }
      adj3(J, inv);
      for (int k = 0; k < 3; k++) {
        double a0 = inv[k][0], a1 = inv[k][1], a2 = inv[k][2];
        double *r = &dH[k * 8];
        r[0] = 0.125 * (-a0 - a1 - a2);
        r[1] = 0.125 * (a0 - a1 - a2);
        r[2] = 0.125 * (a0 + a1 - a2);
        r[3] = 0.125 * (-a0 + a1 - a2);
        r[4] = 0.125 * (-a0 - a1 + a2);
        r[5] = 0.125 * (a0 - a1 + a2);
        r[6] = 0.125 * (a0 + a1 + a2);
        r[7] = 0.125 * (-a0 + a1 + a2);
      }
    } else {
      for (int k = 0; k < 3; k++) {
        J[0][k] = x2[1][k] - x2[0][k];
        J[1][k] = x2[2][k] - x2[0][k];
        J[2][k] = x2[3][k] - x2[0][k];
      }
      adj3(J, inv);
      for (int k = 0; k < 3; k++) {
        double *r = &dH[k * 4];
        r[0] = -inv[k][0] - inv[k][1] - inv[k][2];
        r[1] = inv[k][0];
        r[2] = inv[k][1];
        r[3] = inv[k][2];
      }
    }
    d->detJ[e] = det3(J);
  }
}

/* Domain_d::CalcElemVol (Mechanical.C:264-293): vol = detJ * w, w = 8 (hex),
 * 1/6 (tet). */
static void calc_elem_vol(wfo_domain *d) {
  const double w = (d->npe == 8) ? 8.0 : 1.0 / 6.0;
  const double f = 1.0;
  OMP_FOR
  for (int64_t e = 0; e < d->ne; e++) {
    double v = 0.0;
    v += d->detJ[e] * w * f;
    d->vol[e] = v;
  }
}

/* Domain_d::CalcNodalVol (Mechanical.C:1555-1572). */
static void calc_nodal_vol(wfo_domain *d) {
  OMP_FOR
  for (int64_t n = 0; n < d->nn; n++) {
    double s = 0.0;
    for (int32_t k = 0; k < d->nodel_cnt[n]; k++) s += d->vol[d->nodel[d->nodel_off[n] + k]];
    s /= d->npe;
    d->voln[n] = s;
  }
}

/* Domain_d::CalcNodalMassFromVol (Mechanical.C:1576-1601). */
static void calc_nodal_mass(wfo_domain *d) {
  OMP_FOR
  for (int64_t n = 0; n < d->nn; n++) {
    double mass = 0.0, f = 1.0;
    for (int32_t k = 0; k < d->nodel_cnt[n]; k++) {
      int64_t e = d->nodel[d->nodel_off[n] + k];
      mass += f * d->rho[e] * d->voln[n] / d->nodel_cnt[n];
    }
    d->mass[n] = mass;
  }
}

/* Domain_d::calcElemStrainRates (Mechanical.C:41-126), 3-D. Stored Voigt
 * [xx, yy, zz, xy, yz, xz]; the spin keeps its upper triangle. */
static void calc_strain_rates(wfo_domain *d) {
  const int npe = d->npe;
  OMP_FOR
  for (int64_t e = 0; e < d->ne; e++) {
    double s[3][3] = {{0}}, w[3][3] = {{0}};
    double f = 1.0 / d->detJ[e];
    const double *dH = &d->dH[e * 3 * npe];
    for (int n = 0; n < npe; n++) {
      int64_t g = d->elnod[e * npe + n];
      const double *vn = &d->v[3 * g];
      double d0 = dH[n], d1 = dH[npe + n], d2 = dH[2 * npe + n];
      s[0][0] = s[0][0] + d0 * f * vn[0];
      s[1][1] = s[1][1] + d1 * f * vn[1];
      s[2][2] = s[2][2] + d2 * f * vn[2];
      s[0][1] = s[0][1] + f * (d1 * vn[0] + d0 * vn[1]);
      w[0][1] = w[0][1] + f * (d1 * vn[0] - d0 * vn[1]);
      s[1][2] = s[1][2] + f * (d2 * vn[1] + d1 * vn[2]);
      s[0][2] = s[0][2] + f * (d2 * vn[0] + d0 * vn[2]);
      w[1][2] = w[1][2] + f * (d2 * vn[1] - d1 * vn[2]);
      w[0][2] = w[0][2] + f * (d2 * vn[0] - d0 * vn[2]);
    }
    s[0][1] = s[0][1] * 0.5; s[0][2] = s[0][2] * 0.5; s[1][2] = s[1][2] * 0.5;
    w[0][1] = w[0][1] * 0.5; w[0][2] = w[0][2] * 0.5; w[1][2] = w[1][2] * 0.5;
    double *sr = &d->str_rate[6 * e], *rr = &d->rot_rate[6 * e];
    sr[0] = s[0][0]; sr[1] = s[1][1]; sr[2] = s[2][2];
    sr[3] = s[0][1]; sr[4] = s[1][2]; sr[5] = s[0][2];
    rr[0] = 0.0; rr[1] = 0.0; rr[2] = 0.0;
    rr[3] = w[0][1]; rr[4] = w[1][2]; rr[5] = w[0][2];
  }
}

/* Domain_d::calcElemPressure (Mechanical.C:691-819), pressure algorithm 0:
 * J_avg = mean over the element's nodes of (sum of current volumes) /
 * (sum of initial volumes) over each node's elements; J_bar blends it with
 * the element J; the stabilisation terms are all zero by default. */
static void calc_pressure_alg0(wfo_domain *d) {
  const int npe = d->npe;
  const double *st = d->stab;
  OMP_FOR
  for (int64_t n = 0; n < d->nn; n++) {
    double s0 = 0.0, s = 0.0;
    for (int32_t k = 0; k < d->nodel_cnt[n]; k++) {
      int64_t e = d->nodel[d->nodel_off[n] + k];
      s0 += d->vol0[e];
      s += d->vol[e];
    }
    d->voln0_sum[n] = s0;
    d->voln_sum[n] = s;
  }
  OMP_FOR
  for (int64_t e = 0; e < d->ne; e++) {
    const mat_t *m = mat_of(d, e);
    double K = m->K;
    double rho_e = d->rho[e];
    double vol0 = d->vol0[e], vol1 = d->vol[e];
    double J_local = vol1 / vol0;
    double h = pow(vol1, 1.0 / 3.0);
    int is_contact = 0;
    if (d->contact) {
      for (int a = 0; a < npe; a++) {
        int64_t nid = d->elnod[e * npe + a];
        const double *cf = &d->contforce[3 * nid];
        if (cf[0] * cf[0] + cf[1] * cf[1] + cf[2] * cf[2] > 0) { is_contact = 1; break; }
      }
    }
    double J_avg = 0.0;
    for (int a = 0; a < npe; a++) {
      int64_t nid = d->elnod[e * npe + a];
      J_avg += d->voln_sum[nid] / d->voln0_sum[nid];
    }
    J_avg /= npe;
    double alpha = is_contact ? st[1] : st[0];
    double J_bar = alpha * J_local + (1 - alpha) * J_avg;
    if (J_bar < st[9]) J_bar = 0.2;
    double p_physical = -K * (st[6] * log(J_bar) + (1.0 - st[6]) * (J_bar - 1.0));
    double c = sqrt(K / rho_e);
    double tau = h / (2.0 * c);
    double div_v = 0.0;
    const double *dH = &d->dH[e * 3 * npe];
    for (int a = 0; a < npe; a++) {
      int64_t nid = d->elnod[e * npe + a];
      const double *va = &d->v[3 * nid];
      div_v += dH[a] * va[0] + dH[npe + a] * va[1] + dH[2 * npe + a] * va[2];
    }
    double p_pspg = 0.0;
    double p_hg = (is_contact ? st[3] : st[2]) * K * fabs(J_local - J_avg);
    double p_q = 0.0;
    if (div_v < 0.0) {
      double t1 = st[7] * tau * div_v * K, t2 = st[8] * K;
      p_pspg = (t2 < t1) ? t2 : t1;
      double q1 = st[4] * rho_e * h * c * (-div_v);
      double delta_J = 1.0 - J_local;
      double q2 = st[5] * K * delta_J;
      if (is_contact)
        p_q = 0.5 * (q1 + q2);
      else
        p_q = (q1 < q2) ? q2 : q1;
    }
    d->p[e] = p_physical + p_pspg + p_hg + p_q;
  }
}

/* Domain_d::calcElemPressureANP (Mechanical.C:1220-1250), pressure
 * algorithm 1. As in the reference, p[e] is not reset before accumulating. */
static void calc_pressure_anp(wfo_domain *d) {
  const int npe = d->npe;
  double k = d->mats[0].K;
  OMP_FOR
  for (int64_t n = 0; n < d->nn; n++) {
    double s0 = 0.0, s = 0.0;
    for (int32_t q = 0; q < d->nodel_cnt[n]; q++) {
      int64_t e = d->nodel[d->nodel_off[n] + q];
      s0 += d->vol0[e];
      s += d->vol[e];
    }
    double pn = k * (1.0 - s / s0);
    d->voln_sum[n] = pn; /* scratch: nodal pressure */
    d->p_node[n] = pn;
  }
  OMP_FOR
  for (int64_t e = 0; e < d->ne; e++) {
    for (int a = 0; a < npe; a++) d->p[e] += d->voln_sum[d->elnod[e * npe + a]];
    d->p[e] *= 0.25 * npe;
  }
}

/* Domain_d::calcNodalPressureFromElemental (Mechanical.C:1187-1213): serial
 * volume-weighted scatter; feeds only the nodal pressure output. */
static void calc_nodal_pressure(wfo_domain *d) {
  const int npe = d->npe;
  double *acc = (double *)calloc(d->nn, sizeof(double));
  for (int64_t n = 0; n < d->nn; n++) d->p_node[n] = 0.0;
  for (int64_t e = 0; e < d->ne; e++)
    for (int a = 0; a < npe; a++) {
      int64_t nid = d->elnod[e * npe + a];
      d->p_node[nid] += d->p[e] * d->vol[e];
      acc[nid] += d->vol[e];
    }
  for (int64_t n = 0; n < d->nn; n++)
    if (acc[n] > 0.0) d->p_node[n] /= acc[n];
  free(acc);
}

/* tensor3 as 9 doubles in row order xx xy xz / yx yy yz / zx zy zz. */
enum { XX, XY, XZ, YX, YY, YZ, ZX, ZY, ZZ };

/* operator*(tensor3, tensor3) exactly as written in include/common/Tensor3.C:290-303
 * (its off-diagonal entries pair a's rows with b's rows). */
static void t3_mul(const double *a, const double *b, double *r) {
  r[XX] = a[XX] * b[XX] + a[XY] * b[YX] + a[XZ] * b[ZX];
  r[XY] = a[XX] * b[YX] + a[XY] * b[YY] + a[XZ] * b[YZ];
  r[XZ] = a[XX] * b[ZX] + a[XY] * b[ZY] + a[XZ] * b[ZZ];
  r[YX] = a[YX] * b[XX] + a[YY] * b[YX] + a[YZ] * b[ZX];
  r[YY] = a[YX] * b[YX] + a[YY] * b[YY] + a[YZ] * b[YZ];
  r[YZ] = a[YX] * b[ZX] + a[YY] * b[ZY] + a[YZ] * b[ZZ];
  r[ZX] = a[ZX] * b[XX] + a[ZY] * b[YX] + a[ZZ] * b[ZX];
  r[ZY] = a[ZX] * b[YX] + a[ZY] * b[YY] + a[ZZ] * b[YZ];
  r[ZZ] = a[ZX] * b[ZX] + a[ZY] * b[ZY] + a[ZZ] * b[ZZ];
}
static void t3_from_sym(const double *f, double *t) {
  t[XX] = f[0]; t[YY] = f[1]; t[ZZ] = f[2];
  t[XY] = t[YX] = f[3]; t[YZ] = t[ZY] = f[4]; t[XZ] = t[ZX] = f[5];
}
static void t3_from_antisym(const double *f, double *t) {
  t[XX] = f[0]; t[YY] = f[1]; t[ZZ] = f[2];
  t[XY] = f[3]; t[YZ] = f[4]; t[XZ] = f[5];
  t[YX] = -f[3]; t[ZY] = -f[4]; t[ZX] = -f[5];
}
static void t3_trans(const double *m, double *r) {
  r[XX] = m[XX]; r[YY] = m[YY]; r[ZZ] = m[ZZ];
  r[XY] = m[YX]; r[XZ] = m[ZX]; r[YX] = m[XY];
  r[YZ] = m[ZY]; r[ZX] = m[XZ]; r[ZY] = m[YZ];
}
static void t3_to_sym(const double *t, double *f) {
  f[0] = t[XX]; f[1] = t[YY]; f[2] = t[ZZ]; f[3] = t[XY]; f[4] = t[YZ]; f[5] = t[XZ];
}
static double t3_trace(const double *t) { return (t[XX] + t[YY] + t[ZZ]); }
/* s * Identity() (operator*(double, tensor3) with Identity(), Tensor3.C:343). */
static void t3_scaled_identity(double s, double *r) {
  for (int i = 0; i < 9; i++) r[i] = ((i == XX || i == YY || i == ZZ) ? 1. : 0.) * s;
}

/* CalcHollomonYieldStress / CalcHollomonTangentModulus (Material.cuh:353-395). */
/* CalcJohnsonCookYieldStress (Material.cuh:377-392). */
static double jc_sy(double strain, double strain_rate, const mat_t *m, double temp) {
  double T_h = (temp - m->jc_Tt) / (m->jc_Tm - m->jc_Tt);
  double sr = strain_rate;
  if (strain_rate == 0.0) sr = 1.e-5;
  return (m->sy0 + m->jc_B * pow(strain, m->jc_n)) * (1.0 + m->jc_C * log(sr / m->jc_eps0)) *
         (1.0 - pow(T_h, m->jc_m));
}

/* CalcJohnsonCookTangentModulus (Material.cuh:397-410). */
static double jc_et(double plstrain, double strain_rate, const mat_t *m, double temp) {
  double T_h = (temp - m->jc_Tt) / (m->jc_Tm - m->jc_Tt);
  double Et = 0.;
  if (plstrain > 0.)
    Et = m->jc_n * m->jc_B * pow(plstrain, m->jc_n - 1.) *
         (1.0 + m->jc_C * log(strain_rate / m->jc_eps0)) * (1.0 - pow(T_h, m->jc_m));
  else
    Et = m->E * 0.1;
  return Et;
}

/* CalcGMTYieldStress (Material.cuh:417-452): strain, rate and temperature
 * clamped to their ranges. */
static double gmt_sy(double strain, double strain_rate, double temp, const mat_t *m) {
  double e = strain, er = strain_rate, T = temp;
  if (e < m->g_emin) e = m->g_emin;
  else if (e > m->g_emax) e = m->g_emax;
  if (er < m->g_rmin) er = m->g_rmin;
  else if (er > m->g_rmax) er = m->g_rmax;
  if (T < m->g_Tmin) T = m->g_Tmin;
  else if (T > m->g_Tmax) T = m->g_Tmax;
  return m->g_C1 * exp(m->g_C2 * T) * pow(e, m->g_n1 * T + m->g_n2) *
         exp((m->g_I1 * T + m->g_I2) / e) * pow(er, m->g_m1 * T + m->g_m2);
}

/* CalcGMTTangentModulus (Material.cuh:454-478): d sigma_y / d e. */
static double gmt_et(double plstrain, double strain_rate, double temp, const mat_t *m) {
  double e = plstrain, er = strain_rate, T = temp;
  if (plstrain < m->g_emin) e = m->g_emin;
  else if (plstrain > m->g_emax) e = m->g_emax;
  if (strain_rate < m->g_rmin) er = m->g_rmin;
  else if (strain_rate > m->g_rmax) er = m->g_rmax;
  if (temp < m->g_Tmin) T = m->g_Tmin;
  else if (temp > m->g_Tmax) T = m->g_Tmax;
  return m->g_C1 * exp(m->g_C2 * T) * pow(er, m->g_m1 * T + m->g_m2) *
         pow(e, T * m->g_n1 + m->g_n2 - 2.0) *
         (-m->g_I1 * T - m->g_I2 + e * (m->g_n1 * T + m->g_n2)) *
         exp((m->g_I1 * T + m->g_I2) / e);
}

static double hollomon_sy(double strain, const mat_t *m) {
  if (strain + m->eps0 > m->eps1) return m->hol_K * pow(strain + m->eps0, m->hol_m);
  return m->sy0;
}
static double hollomon_et(double strain, const mat_t *m) {
  if (strain + m->eps0 > m->eps1)
    return m->hol_K * m->hol_m * pow(strain + m->eps0, (m->hol_m - 1.0));
  return 0.;
}

/* Domain_d::CalcStressStrain (Mechanical.C:1664-1839): Jaumann-rate update of
 * the deviatoric stress and J2 radial return. Linear isotropic hardening
 * (model 0) uses sigma_y = sy0 + H eps_p and Et = H in the same return map;
 * Hollomon (model 1) is the reference law. */
static void calc_stress_strain(wfo_domain *d) {
  const double dt = d->dt;
  OMP_FOR
  for (int64_t e = 0; e < d->ne; e++) {
    const mat_t *m = mat_of(d, e);
    double SS[9], SR[9], RR[9], RT[9], SRT[9], RS[9], EPS[9], I[9], A[9];
    t3_from_sym(&d->tau[6 * e], SS);
    t3_from_sym(&d->str_rate[6 * e], SR);
    t3_from_antisym(&d->rot_rate[6 * e], RR);
    t3_from_sym(&d->eps[6 * e], EPS);
    t3_trans(RR, RT);
    t3_mul(SS, RT, SRT);
    t3_mul(RR, SS, RS);
    double c = 1.0 / 3.0 * t3_trace(SR);
    t3_scaled_identity(c, I);
    double g2 = 2.0 * m->G;
    for (int i = 0; i < 9; i++) {
      A[i] = (SR[i] - I[i]) * g2;
      A[i] = A[i] + SRT[i];
      A[i] = A[i] + RS[i];
      SS[i] = SS[i] + A[i] * dt;
    }
    double P[9], ST[9], S[9];
    t3_scaled_identity(-d->p[e], P);
    for (int i = 0; i < 9; i++) ST[i] = P[i] + SS[i];
    double c2 = (1.0 / 3.0) * t3_trace(ST);
    t3_scaled_identity(c2, I);
    for (int i = 0; i < 9; i++) S[i] = ST[i] - I[i];
    double J2 = 0.5 * (S[XX] * S[XX] + 2.0 * S[XY] * S[XY] + 2.0 * S[XZ] * S[XZ] +
                       S[YY] * S[YY] + 2.0 * S[YZ] * S[YZ] + S[ZZ] * S[ZZ]);
    double sig_trial = sqrt(3.0 * J2);
    double H;
    /* effective strain rate (Mechanical.C:1701-1705) */
    double eff = sqrt(0.5 * ((SR[XX] - SR[YY]) * (SR[XX] - SR[YY]) +
                             (SR[YY] - SR[ZZ]) * (SR[YY] - SR[ZZ]) +
                             (SR[ZZ] - SR[XX]) * (SR[ZZ] - SR[XX])) +
                      3.0 * (SR[XY] * SR[XY] + SR[YZ] * SR[YZ] + SR[XZ] * SR[XZ]));
    /* Johnson-Cook and GMT temperature: the material's (uniform)
     * temperature, or with thermal coupling the mean of the element's node
     * temperatures (the reference reads T[e], a node array indexed by
     * element) */
    double temp = (m->model == 3) ? m->g_T : m->jc_T;
    if (d->thermal && (m->model == 2 || m->model == 3)) {
      double ts = 0.0;
      for (int a = 0; a < d->npe; a++) ts += d->T[d->elnod[e * d->npe + a]];
      temp = ts / d->npe;
    }
    if (m->model == 2) {
      d->sigma_y[e] = jc_sy(d->pl_strain[e], eff, m, temp);
    } else if (m->model == 3) {
      d->sigma_y[e] = gmt_sy(d->pl_strain[e], eff, temp, m);
    } else if (m->model == 1) {
      d->sigma_y[e] = hollomon_sy(d->pl_strain[e], m);
    } else {
      d->sigma_y[e] = m->sy0 + m->H * d->pl_strain[e];
    }
    eff = (d->max_edot < eff) ? d->max_edot : eff;  /* min(eff, m_max_edot) */
    double dep = 0.0;
    if (d->sigma_y[e] < sig_trial) {
      if (m->model == 2)
        H = jc_et(d->pl_strain[e], eff, m, temp);
      else if (m->model == 3)
        H = gmt_et(d->pl_strain[e], eff, temp, m);
      else
        H = (m->model == 1) ? hollomon_et(d->pl_strain[e], m) : m->H;
      double G = m->G;
      double dgamma = (sig_trial - d->sigma_y[e]) / (3.0 * G + H);
      double factor = 1.0 - (3.0 * G * dgamma) / sig_trial;
      for (int i = 0; i < 9; i++) SS[i] = S[i] * factor;
      d->pl_strain[e] += dgamma;
      dep = dgamma;
    }
    double SG[9];
    for (int i = 0; i < 9; i++) SG[i] = P[i] + SS[i];
    double *pi = &d->pl_incr[6 * e];
    if (dep > 0.0) {
      double f = dep / d->sigma_y[e];
      pi[0] = f * (SG[XX] - 0.5 * (SG[YY] + SG[ZZ]));
      pi[1] = f * (SG[YY] - 0.5 * (SG[XX] + SG[ZZ]));
      pi[2] = f * (SG[ZZ] - 0.5 * (SG[XX] + SG[YY]));
      pi[3] = 1.5 * f * (SG[XY]);
      pi[4] = 1.5 * f * (SG[YZ]);
      pi[5] = 1.5 * f * (SG[XZ]);
    } else {
      for (int i = 0; i < 6; i++) pi[i] = 0.0;
    }
    /* plastic heat (Mechanical.C:1783-1810): 0.9 sigma : (incr / dt) with the
     * shear terms doubled */
    if (d->thermal) {
      d->q_plheat[e] = 0.0;
      if (dep > 0.0) {
        const double idt = 1. / dt;
        const double dxx = pi[0] * idt, dyy = pi[1] * idt, dzz = pi[2] * idt;
        const double dxy = pi[3] * idt, dyz = pi[4] * idt, dxz = pi[5] * idt;
        d->q_plheat[e] = d->plheat_frac * (SG[XX] * dxx + 2.0 * SG[XY] * dxy + 2.0 * SG[XZ] * dxz +
                                SG[YY] * dyy + 2.0 * SG[YZ] * dyz + SG[ZZ] * dzz);
      }
    }
    for (int i = 0; i < 9; i++) EPS[i] = EPS[i] + SR[i] * dt;
    t3_to_sym(SG, &d->sigma[6 * e]);
    t3_to_sym(SS, &d->tau[6 * e]);
    t3_to_sym(EPS, &d->eps[6 * e]);
  }
}

/* Domain_d::calcArtificialViscosity (Mechanical.C:1948-1977), serial. */
static void calc_artificial_viscosity(wfo_domain *d) {
  double alpha = d->artif[0], beta = d->artif[1];
  double q_max = 1e9;
  for (int64_t e = 0; e < d->ne; e++) {
    const mat_t *m = mat_of(d, e);
    double c = sqrt(m->K / d->rho[e]);
    const double *sr = &d->str_rate[6 * e];
    double eps_v = (sr[0] + sr[1] + sr[2]);
    if (fabs(eps_v) > 1e-12) {
      double l = pow(d->vol[e], 1.0 / 3.0);
      double q = alpha * c * fabs(eps_v) * l + beta * pow(eps_v * l, 2);
      q = (q_max < q) ? q_max : q;
      double q_signed = (eps_v > 0) ? -q : q;
      d->sigma[6 * e + 0] += q_signed;
      d->sigma[6 * e + 1] += q_signed;
      d->sigma[6 * e + 2] += q_signed;
    }
  }
}

/* Domain_d::calcElemForces (Mechanical.C:375-481), 3-D: f = w * B^T sigma. */
static void calc_elem_forces(wfo_domain *d) {
  const int npe = d->npe;
  const double w = (npe == 8) ? 8.0 : 1.0 / 6.0;
  OMP_FOR
  for (int64_t e = 0; e < d->ne; e++) {
    const double *dH = &d->dH[e * 3 * npe];
    const double *s = &d->sigma[6 * e];
    double *f = &d->f_elem[e * npe * 3];
    double fc = 1.0;
    for (int n = 0; n < npe; n++) {
      double d0 = dH[n], d1 = dH[npe + n], d2 = dH[2 * npe + n];
      f[3 * n + 0] = 0.0;
      f[3 * n + 1] = 0.0;
      f[3 * n + 2] = 0.0;
      f[3 * n + 0] += d0 * s[0] * fc;
      f[3 * n + 1] += d1 * s[1] * fc;
      f[3 * n + 2] += d2 * s[2] * fc;
      f[3 * n + 0] += d1 * s[3] + d2 * s[5];
      f[3 * n + 1] += d0 * s[3] + d2 * s[4];
      f[3 * n + 2] += d1 * s[4] + d0 * s[5];
    }
    for (int i = 0; i < npe * 3; i++) f[i] *= w;
  }
}

/* 3-D viscous hourglass control of 1-point hexahedra (Flanagan-Belytschko
 * base vectors), restated from src/common/test_1el_3D.cpp:159-199 with the
 * current element volume and density: f_hg = -c_h sum_j (v . Gamma_j) Gamma_j,
 * c_h = coef * V^0.6666666 * rho * 0.25 * cs0. */
static const double HG_SIG[4][8] = {{1., 1., -1., -1., -1., -1., 1., 1.},
                                    {1., -1., -1., 1., -1., 1., 1., -1.},
                                    {1., -1., 1., -1., 1., -1., 1., -1.},
                                    {-1., 1., -1., 1., 1., -1., 1., -1.}};
static void calc_hourglass(wfo_domain *d) {
  if (d->hg_coef == 0.0 || d->npe != 8) return;
  OMP_FOR
  for (int64_t e = 0; e < d->ne; e++) {
    const mat_t *m = mat_of(d, e);
    double *fhg = &d->f_hg[e * 24];
    double hmod[3][4] = {{0.0}};
    double vel[8][3];
    for (int i = 0; i < 8; i++) {
      int64_t g = d->elnod[e * 8 + i];
      vel[i][0] = d->v[3 * g]; vel[i][1] = d->v[3 * g + 1]; vel[i][2] = d->v[3 * g + 2];
      fhg[3 * i] = fhg[3 * i + 1] = fhg[3 * i + 2] = 0.0;
    }
    for (int j = 0; j < 4; j++)
      for (int i = 0; i < 8; i++)
        for (int k = 0; k < 3; k++) hmod[k][j] += vel[i][k] * HG_SIG[j][i];
    double ch = d->hg_coef * pow(d->vol[e], 0.6666666) * d->rho[e] * 0.25 * m->cs0;
    for (int j = 0; j < 4; j++)
      for (int i = 0; i < 8; i++)
        for (int k = 0; k < 3; k++) fhg[3 * i + k] -= ch * hmod[k][j] * HG_SIG[j][i];
  }
}

/* Penalty + Coulomb contact of candidate nodes against a rigid flat die with
 * outward normal (0, 0, -1) at z = z0 + vz * Time, restated from
 * Domain_d::CalcContactForces (Contact.C:58-323) for one infinite plane:
 * normal force -(k d + 0.2 c_crit v_n) n with c_crit = 2 m sqrt(k / m),
 * tangential trial force -k * (accumulated slip), capped at mu |F_n| in the
 * sliding direction (slip reset when sliding). The stiffness is the given
 * penalty k in place of E A / l, still capped at 0.2 m / dt^2; forces of candidate
 * nodes out of contact are cleared (the reference keeps stale values). The
 * per-node normal-force magnitude feeds the contact reaction (Contact.C:326). */
static void calc_contact(wfo_domain *d) {
  const double dt = d->dt;
  const double zd = d->c_z0 + d->c_vz * d->time;
  const double nz = -1.0;
  const double kpen = d->c_kpen;
  OMP_FOR
  for (int64_t i = 0; i < d->nn; i++) {
    d->cfn[i] = 0.0;
    if (!d->cand[i]) continue;
    double *cf = &d->contforce[3 * i];
    double gap = zd - d->x[3 * i + 2];
    if (!(gap < 0)) {
      cf[0] = cf[1] = cf[2] = 0.0;
      continue;
    }
    double m = d->mass[i];
    const double *vi = &d->v[3 * i];
    double v_reln = vi[2] * nz;
    /* kcont = min(k_geometric, 0.2 m / dt^2) (Contact.C:190-193), with the
     * given penalty as the geometric stiffness */
    double kmass = 0.2 * m / (dt * dt);
    double k = (kmass < kpen) ? kmass : kpen;
    double omega = sqrt(k / m);
    double ccrit = 2.0 * m * omega;
    double F_damp = 0.2 * ccrit * v_reln;
    double F_normal = k * gap;
    double cfz = -(F_normal + F_damp) * nz;
    cf[0] = 0.0;
    cf[1] = 0.0;
    cf[2] = cfz;
    d->cfn[i] = fabs(cfz);
    /* tangential part: v_tan = v - (v . n) n = (vx, vy, 0) */
    double vtx = vi[0], vty = vi[1];
    double *ut = &d->ut_prev[3 * i];
    ut[0] += vtx * dt;
    ut[1] += vty * dt;
    double ftx = -k * ut[0], fty = -k * ut[1];
    double ft_mag = sqrt(ftx * ftx + fty * fty);
    double fn_mag = fabs(cfz);
    double ft_max = d->c_mu * fn_mag;
    if (!(ft_mag <= ft_max)) {
      double vt = sqrt(vtx * vtx + vty * vty);
      if (vt > 0.0) {
        ftx = -ft_max * vtx / vt;
        fty = -ft_max * vty / vt;
      } else {
        ftx = fty = 0.0;
      }
      ut[0] = ut[1] = ut[2] = 0.0;
    }
    cf[0] += ftx;
    cf[1] += fty;
  }
}

/* Domain_d::assemblyForces (Matrices.C:42-87): per node, sum of element
 * forces over its elements in list order, minus the hourglass forces. */
static void assembly_forces(wfo_domain *d) {
  const int npe = d->npe;
  OMP_FOR
  for (int64_t n = 0; n < d->nn; n++) {
    double f0 = 0.0, f1 = 0.0, f2 = 0.0;
    int32_t off = d->nodel_off[n], cnt = d->nodel_cnt[n];
    for (int32_t k = 0; k < cnt; k++) {
      int64_t base = ((int64_t)d->nodel[off + k] * npe + d->nodel_loc[off + k]) * 3;
      f0 += d->f_elem[base]; f1 += d->f_elem[base + 1]; f2 += d->f_elem[base + 2];
    }
    for (int32_t k = 0; k < cnt; k++) {
      int64_t base = ((int64_t)d->nodel[off + k] * npe + d->nodel_loc[off + k]) * 3;
      f0 -= d->f_hg[base]; f1 -= d->f_hg[base + 1]; f2 -= d->f_hg[base + 2];
    }
    /* non-finite clamp of Solver_explicit.C:777-785 */
    d->fi[3 * n] = isfinite(f0) ? f0 : 0.0;
    d->fi[3 * n + 1] = isfinite(f1) ? f1 : 0.0;
    d->fi[3 * n + 2] = isfinite(f2) ? f2 : 0.0;
  }
}

/* Domain_d::calcAccel (Mechanical.C:321-341). */
static void calc_accel(wfo_domain *d) {
  OMP_FOR
  for (int64_t n = 0; n < d->nn; n++) {
    for (int k = 0; k < 3; k++)
      d->a[3 * n + k] = (d->fe[3 * n + k] - d->fi[3 * n + k]) / d->mass[n];
    if (d->contact)
      for (int k = 0; k < 3; k++) d->a[3 * n + k] += d->contforce[3 * n + k] / d->mass[n];
  }
}

/* Domain_d::UpdateCorrectionAccVel (Domain_d.C:981-997). */
static void update_correction_acc_vel(wfo_domain *d) {
  double f = 1.0 / (1.0 - d->alpha);
  const double al = d->alpha, g = d->gamma, dt = d->dt;
  int64_t n3 = d->nn * 3;
  OMP_FOR
  for (int64_t ig = 0; ig < n3; ig++) {
    d->a[ig] = f * (d->a[ig] - al * d->prev_a[ig]);
    d->v[ig] += g * dt * d->a[ig];
  }
}

/* Domain_d::UpdateCorrectionPos (Domain_d.C:1005-1025). */
static void update_correction_pos(wfo_domain *d) {
  const double b = d->beta, dt = d->dt;
  int64_t n3 = d->nn * 3;
  OMP_FOR
  for (int64_t ig = 0; ig < n3; ig++) {
    d->u_dt[ig] += b * dt * dt * d->a[ig];
    d->x[ig] += d->u_dt[ig];
    d->prev_a[ig] = d->a[ig];
    d->u[ig] += d->u_dt[ig];
  }
}

/* ---- triangle-mesh contact ------------------------------------------------ */
/* Face tables of the reference (Domain_d.h:184-193). */
static const int TET_FACES[4][3] = {{0, 1, 2}, {0, 1, 3}, {1, 2, 3}, {0, 2, 3}};
static const int HEX_FACES[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4},
                                    {2, 3, 7, 6}, {0, 3, 7, 4}, {1, 2, 6, 5}};

typedef struct {
  int32_t k[4];
  int32_t count;
  int32_t used;
} face_slot;

static uint64_t face_hash(const int32_t *k) {
  uint64_t h = 1469598103934665603ull;
  for (int i = 0; i < 4; i++) {
    h ^= (uint64_t)(uint32_t)k[i];
    h *= 1099511628211ull;
  }
  return h;
}

static void sort_key(const int32_t *in, int n, int32_t *k) {
  for (int i = 0; i < 4; i++) k[i] = i < n ? in[i] : -1;
  for (int i = 1; i < n; i++)
    for (int j = i; j > 0 && k[j - 1] > k[j]; j--) {
      int32_t t = k[j];
      k[j] = k[j - 1];
      k[j - 1] = t;
    }
}

static face_slot *face_find(face_slot *tab, uint64_t mask, const int32_t *k) {
  uint64_t i = face_hash(k) & mask;
  for (;;) {
    face_slot *s = &tab[i];
    if (!s->used || (s->k[0] == k[0] && s->k[1] == k[1] && s->k[2] == k[2] && s->k[3] == k[3]))
      return s;
    i = (i + 1) & mask;
  }
}

static double tri_area(const double *p0, const double *p1, const double *p2) {
  const double v1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
  const double v2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
  const double c[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2],
                       v1[0] * v2[1] - v1[1] * v2[0]};
  return 0.5 * sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
}

/* External nodes and nodal areas (SearchExtNodes + CalcExtFaceAreas): a face
 * used by one element is external; its area goes in equal shares to its nodes,
 * faces taken in element order and local face order. Tetrahedra use the
 * reference's triangular face table; hexahedra the quadrilateral table
 * (hexa_faces), each quadrilateral's area as the triangles (0,1,2) + (0,2,3).
 * Element lengths: the 3-D branch of calcMinEdgeLength (Domain_d.C:2236-2262),
 * the smallest height of the tetrahedron of the element's first four nodes;
 * nodlen = mean over the node's elements (Contact.C:145-152). */
static void tri_setup_surface(wfo_domain *d) {
  const int npe = d->npe, nf = npe == 8 ? 6 : 4, fn = npe == 8 ? 4 : 3;
  const int64_t nfaces = d->ne * nf;
  uint64_t cap = 1;
  while (cap < 2 * (uint64_t)nfaces + 2) cap <<= 1;
  face_slot *tab = calloc(cap, sizeof(face_slot));
  int32_t key[4], fnodes[4];
  for (int64_t e = 0; e < d->ne; e++)
    for (int f = 0; f < nf; f++) {
      for (int q = 0; q < fn; q++)
        fnodes[q] = d->elnod[e * npe + (npe == 8 ? HEX_FACES[f][q] : TET_FACES[f][q])];
      sort_key(fnodes, fn, key);
      face_slot *s = face_find(tab, cap - 1, key);
      if (!s->used) {
        s->used = 1;
        memcpy(s->k, key, sizeof(key));
      }
      s->count++;
    }
  free(d->ext);
  free(d->node_area);
  free(d->nodlen);
  free(d->elem_len);
  d->ext = xcalloc(d->nn, 1);
  d->node_area = xcalloc(d->nn, 8);
  d->nodlen = xcalloc(d->nn, 8);
  d->elem_len = xcalloc(d->ne, 8);
  for (int64_t e = 0; e < d->ne; e++)
    for (int f = 0; f < nf; f++) {
      for (int q = 0; q < fn; q++)
        fnodes[q] = d->elnod[e * npe + (npe == 8 ? HEX_FACES[f][q] : TET_FACES[f][q])];
      sort_key(fnodes, fn, key);
      if (face_find(tab, cap - 1, key)->count != 1) continue;
      const double *p0 = &d->x[3 * fnodes[0]], *p1 = &d->x[3 * fnodes[1]], *p2 = &d->x[3 * fnodes[2]];
      double share;
      if (fn == 3) {
        share = tri_area(p0, p1, p2) / 3.0;
      } else {
        const double *p3 = &d->x[3 * fnodes[3]];
        share = (tri_area(p0, p1, p2) + tri_area(p0, p2, p3)) / 4.0;
      }
      for (int q = 0; q < fn; q++) {
        d->ext[fnodes[q]] = 1;
        d->node_area[fnodes[q]] += share;
      }
    }
  free(tab);
  for (int64_t e = 0; e < d->ne; e++) {
    const int32_t *n = &d->elnod[e * npe];
    const double *A = &d->x[3 * n[0]], *B = &d->x[3 * n[1]], *C = &d->x[3 * n[2]],
                 *D = &d->x[3 * n[3]];
    const double *faces[4][3] = {{B, C, D}, {A, C, D}, {A, B, D}, {A, B, C}};
    double hmin = 1.0e6;
    for (int i = 0; i < 4; i++) {
      const double *f0 = faces[i][0], *f1 = faces[i][1], *f2 = faces[i][2];
      const double x1[3] = {f1[0] - f0[0], f1[1] - f0[1], f1[2] - f0[2]};
      const double x2[3] = {f2[0] - f0[0], f2[1] - f0[1], f2[2] - f0[2]};
      double nn[3] = {x1[1] * x2[2] - x1[2] * x2[1], x1[2] * x2[0] - x1[0] * x2[2],
                      x1[0] * x2[1] - x1[1] * x2[0]};
      const double area = sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
      if (area < 1e-12) continue;
      const double inv = 1.0 / area;
      nn[0] *= inv;
      nn[1] *= inv;
      nn[2] *= inv;
      const double *P = &d->x[3 * n[i]];
      const double vec[3] = {P[0] - f0[0], P[1] - f0[1], P[2] - f0[2]};
      const double h = fabs(vec[0] * nn[0] + vec[1] * nn[1] + vec[2] * nn[2]);
      if (h < hmin) hmin = h;
    }
    d->elem_len[e] = hmin;
  }
  for (int64_t i = 0; i < d->nn; i++) {
    double l = 0.0;
    const int32_t b = d->nodel_off[i], c = d->nodel_cnt[i];
    for (int32_t k = 0; k < c; k++) l += d->elem_len[d->nodel[b + k]];
    d->nodlen[i] = l / c;
  }
}

/* Domain_d::CalcContactForces (Contact.C:31-334) against the rigid triangle
 * mesh: for each external node, the first triangle (in order) it penetrates
 * (d < 0, projection inside the triangle) gives a penalty normal force with
 * stiffness min(E A / l, 0.2 m / dt^2) times the penalty factor, a damping
 * force, and Coulomb friction from the accumulated tangential slip (static
 * cap, then dynamic force along -v_t). As in the reference, a node that leaves
 * contact keeps its last contact force. The reaction is the sum of normal-force
 * magnitudes of the nodes in contact with rigid body 0. */
static void calc_contact_trimesh(wfo_domain *d) {
  const double dt = d->dt;
  const double E0 = d->mats[0].E;
  for (int64_t i = 0; i < d->nn; i++) {
    d->cfn[i] = 0.0;
    if (!d->ext[i]) continue;
    const double *x = &d->x[3 * i];
    const double *v = &d->v[3 * i];
    for (int64_t j = 0; j < d->tri_ne; j++) {
      const double *nr = &d->tri_nrm[3 * j];
      const double dd = (nr[0] * x[0] + nr[1] * x[1] + nr[2] * x[2]) - d->tri_pp[j];
      if (!(dd < 0)) continue;
      const double Q[3] = {x[0] - nr[0] * dd, x[1] - nr[1] * dd, x[2] - nr[2] * dd};
      int inside = 1;
      for (int l = 0; l < 3 && inside; l++) {
        const int nx = l + 1 > 2 ? 0 : l + 1;
        const double *a = &d->tri_x[3 * d->tri_el[3 * j + l]];
        const double *b = &d->tri_x[3 * d->tri_el[3 * j + nx]];
        const double e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
        const double e2[3] = {Q[0] - a[0], Q[1] - a[1], Q[2] - a[2]};
        const double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                             e1[0] * e2[1] - e1[1] * e2[0]};
        const double crit = c[0] * nr[0] + c[1] * nr[1] + c[2] * nr[2];
        if (crit < 0.0) inside = 0;
      }
      if (!inside) continue;
      const double m = d->mass[i];
      const double v_reln = v[0] * nr[0] + v[1] * nr[1] + v[2] * nr[2];
      const double kgeo = E0 * d->node_area[i] / d->nodlen[i];
      const double kmass = 0.2 * m / (dt * dt);
      const double k = (kmass < kgeo) ? kmass : kgeo;  /* std::min(kgeo, kmass) */
      const double omega = sqrt(k / m);
      const double ccrit = 2.0 * m * omega;
      const double F_damp = 0.2 * ccrit * v_reln;
      const double F_normal = d->tri_pf * k * dd;
      const double s = -(F_normal + F_damp);
      double *cf = &d->contforce[3 * i];
      cf[0] = nr[0] * s;
      cf[1] = nr[1] * s;
      cf[2] = nr[2] * s;
      /* only contacts with rigid body 0 feed the reaction (Contact.C:326-329) */
      if (d->tri_mid[j] == 0) d->cfn[i] = sqrt(cf[0] * cf[0] + cf[1] * cf[1] + cf[2] * cf[2]);
      /* friction */
      const double vn = v[0] * nr[0] + v[1] * nr[1] + v[2] * nr[2];
      const double vt[3] = {v[0] - nr[0] * vn, v[1] - nr[1] * vn, v[2] - nr[2] * vn};
      double *ut = &d->ut_prev[3 * i];
      const double du[3] = {vt[0] * dt, vt[1] * dt, vt[2] * dt};
      const double ua[3] = {ut[0] + du[0], ut[1] + du[1], ut[2] + du[2]};
      ut[0] += du[0];
      ut[1] += du[1];
      ut[2] += du[2];
      const double mk = -k;
      const double ft[3] = {ua[0] * mk, ua[1] * mk, ua[2] * mk};
      const double ft_mag = sqrt(ft[0] * ft[0] + ft[1] * ft[1] + ft[2] * ft[2]);
      const double cn = cf[0] * nr[0] + cf[1] * nr[1] + cf[2] * nr[2];
      const double Fn[3] = {nr[0] * cn, nr[1] * cn, nr[2] * cn};
      const double fn_norm = sqrt(Fn[0] * Fn[0] + Fn[1] * Fn[1] + Fn[2] * Fn[2]);
      double F[3];
      if (ft_mag <= d->tri_mu_s * fn_norm) {
        F[0] = ft[0];
        F[1] = ft[1];
        F[2] = ft[2];
      } else {
        const double md = -(d->tri_mu_d * fn_norm);
        const double vnorm = sqrt(vt[0] * vt[0] + vt[1] * vt[1] + vt[2] * vt[2]);
        const double inv = 1.0 / vnorm;
        F[0] = (vt[0] * md) * inv;
        F[1] = (vt[1] * md) * inv;
        F[2] = (vt[2] * md) * inv;
        ut[0] = ut[1] = ut[2] = 0.0;
      }
      cf[0] += F[0];
      cf[1] += F[1];
      cf[2] += F[2];
      /* heat from the die (Contact.C:309); kept after contact ends */
      d->q_cont[i] = d->heat_cond * d->node_area[i] * (d->T_die - d->T[i]);
      break;
    }
  }
}

/* End of the loop body (Solver_explicit.C:980-1004): the die velocity ramps
 * as sqrt(Time / (0.01 end_t)) over the first 1 % of the end time, the mesh
 * moves by v dt and its normals and planes are recomputed. */
static void tri_move(wfo_domain *d) {
  const double rf = 1.0e-2;
  double f = 1.0;
  if (d->time < rf * d->end_t) f = pow(d->time / (rf * d->end_t), 0.5);
  for (int64_t n = 0; n < d->tri_nn; n++)
    for (int k = 0; k < 3; k++) {
      const double vk = f * d->tri_vorig[3 * n + k];
      d->tri_x[3 * n + k] = d->tri_x[3 * n + k] + vk * d->dt;
    }
  tri_normals_planes(d);
}

/* Domain_d::calcThermalExpansion (Thermal.C:163-178): the strain rate's
 * diagonal loses exp_T * mean of m_dTedt at the element's node ids. As in the
 * reference, the element-node array of the previous step's temperature rates
 * is indexed by node id. */
static void calc_thermal_expansion(wfo_domain *d) {
  const int npe = d->npe;
  OMP_FOR
  for (int64_t e = 0; e < d->ne; e++) {
    const mat_t *m = mat_of(d, e);
    double g = 0.0;
    for (int i = 0; i < npe; i++) g += 1.0 / npe * d->dTedt[d->elnod[e * npe + i]];
    const double c = m->exp_T * g;
    double *sr = &d->str_rate[6 * e];
    sr[0] = sr[0] - c;
    sr[1] = sr[1] - c;
    sr[2] = sr[2] - c;
  }
}

/* Domain_d::ThermalCalcs (Thermal.C:27-126): per element the conduction
 * matrix K_ij = (sum_d dN_i detJ dN_j detJ) k_T / detJ w times the element's
 * node temperatures, and the plastic heat 0.9 q vol split evenly over the
 * nodes: dT_e,i = -(1 / m_i) (K T)_i + (q_e vol / n) / (m_i cp_T). Then per
 * node, in node-to-element list order, T += (sum dT_e,i + q_cont / (m cp_T of
 * material 0)) dt. */
static void thermal_calcs(wfo_domain *d) {
  const int npe = d->npe;
  const double w = (npe == 8) ? 8.0 : 1.0 / 6.0;
  OMP_FOR
  for (int64_t e = 0; e < d->ne; e++) {
    const mat_t *m = mat_of(d, e);
    const double *dH = &d->dH[e * 3 * npe];
    const int32_t *en = &d->elnod[e * npe];
    double Kt[8][8], Te[8];
    for (int i = 0; i < npe; i++)
      for (int j = 0; j < npe; j++) {
        double k = 0.0;
        for (int dd = 0; dd < 3; dd++) k += dH[dd * npe + i] * dH[dd * npe + j];
        Kt[i][j] = k * m->k_T / d->detJ[e] * w;
      }
    for (int i = 0; i < npe; i++) Te[i] = d->T[en[i]];
    const double heat = 0.9 * d->q_plheat[e];
    const double elem_pow = heat * d->vol[e];
    const double pow_per_node = elem_pow / npe;
    for (int i = 0; i < npe; i++) {
      double dT = 0.0;
      for (int k = 0; k < npe; k++) dT += Kt[i][k] * Te[k];
      const double m_inv = 1.0 / d->mass[en[i]];
      double r = -m_inv * dT;
      r += pow_per_node / (d->mass[en[i]] * m->cp_T);
      d->dTedt[e * npe + i] = r;
    }
  }
  const double cp0 = d->mats[0].cp_T;
  OMP_FOR
  for (int64_t n = 0; n < d->nn; n++) {
    double s = 0.0;
    for (int32_t k = 0; k < d->nodel_cnt[n]; k++) {
      const int64_t i = d->nodel_off[n] + k;
      s += d->dTedt[(int64_t)d->nodel[i] * npe + d->nodel_loc[i]];
    }
    d->T[n] += (s + d->q_cont[n] * 1.0 / (d->mass[n] * cp0)) * d->dt;
  }
}

void wfo_set_thermal(wfo_domain *d, int on, double T0) {
  d->thermal = on;
  d->T0 = T0;
}

int wfo_set_material_thermal(wfo_domain *d, int mat, double k_T, double cp_T, double exp_T) {
  if (mat < 0 || mat >= d->nmat) return -1;
  d->mats[mat].k_T = k_T;
  d->mats[mat].cp_T = cp_T;
  d->mats[mat].exp_T = exp_T;
  return 0;
}

void wfo_set_contact_heat(wfo_domain *d, double heat_cond, double T_die) {
  d->heat_cond = heat_cond;
  d->T_die = T_die;
}

/* Preamble of Domain_d::SolveChungHulbert (Solver_explicit.C:120-268). */
int wfo_init(wfo_domain *d) {
  if (!d->mats || !d->nn) return -1;
  for (int64_t e = 0; e < d->ne; e++) {
    d->pl_strain[e] = 0.0;
    d->sigma_y[e] = mat_of(d, e)->sy0;
  }
  for (int k = 0; k < 3; k++) {
    for (int64_t n = 0; n < d->nn * 3; n++) d->v[n] = d->a[n] = d->u[n] = 0.0;
    impose_bcv(d, k);
  }
  double rho_b = 0.818200;
  d->alpha = (2.0 * rho_b - 1.0) / (1.0 + rho_b);
  d->beta = (5.0 - 3.0 * rho_b) / ((1.0 + rho_b) * (1.0 + rho_b) * (2.0 - rho_b));
  d->gamma = 1.5 - d->alpha;
  calc_jacobian_derivs(d);
  calc_elem_vol(d);
  for (int64_t e = 0; e < d->ne; e++) d->vol0[e] = d->vol[e];
  calc_elem_vol(d);
  /* Domain_d::calcElemDensity (Mechanical.C:295-319) */
  for (int64_t e = 0; e < d->ne; e++) d->rho[e] = d->rho0[e] * d->vol0[e] / d->vol[e];
  calc_nodal_vol(d);
  calc_nodal_mass(d);
  memcpy(d->mass0, d->mass, sizeof(double) * d->nn);
  memset(d->ut_prev, 0, sizeof(double) * 3 * d->nn);
  /* setTemp (Domain_d.h:678-684) and zero thermal rates */
  if (d->thermal) {
    for (int64_t n = 0; n < d->nn; n++) d->T[n] = d->T0;
    memset(d->q_plheat, 0, sizeof(double) * d->ne);
    memset(d->dTedt, 0, sizeof(double) * d->ne * d->npe);
    memset(d->q_cont, 0, sizeof(double) * d->nn);
  }
  d->time = 0.0;
  d->step_count = 0;
  d->hist_len = 0;
  d->eint = 0.0;
  if (d->tri_on) tri_setup_surface(d);
  return 0;
}

static void record_reaction(wfo_domain *d, double r) {
  if (d->hist_len == d->hist_cap) {
    d->hist_cap = d->hist_cap ? 2 * d->hist_cap : 1024;
    d->react_hist = realloc(d->react_hist, sizeof(double) * d->hist_cap);
    d->ekin_hist = realloc(d->ekin_hist, sizeof(double) * d->hist_cap);
    d->eint_hist = realloc(d->eint_hist, sizeof(double) * d->hist_cap);
  }
  d->react_hist[d->hist_len++] = r;
}

/* Domain_d::computeEnergies (Mechanical.C:2145-2185): kinetic energy of the
 * end-of-step velocity with the step's lumped mass, and the internal energy
 * increment dt * sum_e (sigma . str_rate) vol_e over the six stored Voigt
 * components (shear terms counted once, as the reference does). Serial sums in
 * node and element order. */
static void compute_energies(const wfo_domain *d, double *ekin, double *deint) {
  double k = 0.0;
  for (int64_t n = 0; n < d->nn; n++) {
    const double vx = d->v[3 * n], vy = d->v[3 * n + 1], vz = d->v[3 * n + 2];
    k += 0.5 * d->mass[n] * (vx * vx + vy * vy + vz * vz);
  }
  double ed = 0.0;
  for (int64_t e = 0; e < d->ne; e++) {
    const double *s = &d->sigma[6 * e], *r = &d->str_rate[6 * e];
    const double sdot = s[0] * r[0] + s[1] * r[1] + s[2] * r[2] + s[3] * r[3] + s[4] * r[4] + s[5] * r[5];
    ed += sdot * d->vol[e];
  }
  *ekin = k;
  *deint = ed * d->dt;
}

/* One iteration of the loop body of SolveChungHulbert, CPU branch with default
 * options (Solver_explicit.C:346-1167), in two halves: step_begin runs up to
 * the element and contact forces, step_end from assemblyForces on (the split
 * a slab decomposition exchanges its halo element forces at). */
static void one_step(wfo_domain *d);
static void step_begin(wfo_domain *d);
static void step_end(wfo_domain *d);

static void one_step(wfo_domain *d) {
  step_begin(d);
  step_end(d);
}

static void step_begin(wfo_domain *d) {
  update_prediction(d);
  for (int k = 0; k < 3; k++) impose_bcv(d, k);
  calc_jacobian_derivs(d);
  calc_elem_vol(d);
  if (d->mass_mode == 0) {
    calc_nodal_vol(d);
    calc_nodal_mass(d);
  }
  calc_strain_rates(d);
  if (d->thermal) calc_thermal_expansion(d);
  if (d->press_alg == 1)
    calc_pressure_anp(d);
  else
    calc_pressure_alg0(d);
  calc_nodal_pressure(d);
  calc_stress_strain(d);
  calc_artificial_viscosity(d);
  calc_elem_forces(d);
  calc_hourglass(d);
  if (d->tri_on)
    calc_contact_trimesh(d);
  else if (d->contact)
    calc_contact(d);
}

static void step_end(wfo_domain *d) {
  assembly_forces(d);
  double r = 0.0;
  if (d->contact) {
    for (int64_t i = 0; i < d->nn; i++) r += d->cfn[i];
  } else {
    for (int64_t k = 0; k < d->n_react; k++) r += d->fi[3 * d->react_nodes[k] + d->react_dim];
  }
  record_reaction(d, r);
  calc_accel(d);
  for (int k = 0; k < 3; k++) impose_bca(d, k);
  update_correction_acc_vel(d);
  for (int k = 0; k < 3; k++) impose_bcv(d, k);
  update_correction_pos(d);
  if (d->tri_on) tri_move(d);
  if (d->thermal) thermal_calcs(d);
  {
    double ekin, deint;
    compute_energies(d, &ekin, &deint);
    d->eint += deint;
    d->ekin_hist[d->hist_len - 1] = ekin;
    d->eint_hist[d->hist_len - 1] = d->eint;
  }
  d->time += d->dt;
  d->step_count++;
}

void wfo_step_begin(wfo_domain *d) { step_begin(d); }
void wfo_step_end(wfo_domain *d) { step_end(d); }

/* Element forces of elements [e0, e1): f_elem then f_hg, npe x 3 each. */
int wfo_get_elem_forces_range(const wfo_domain *d, int64_t e0, int64_t e1, double *out) {
  if (e0 < 0 || e1 > d->ne || e0 > e1) return -1;
  const size_t k = (size_t)(e1 - e0) * d->npe * 3;
  memcpy(out, d->f_elem + e0 * d->npe * 3, sizeof(double) * k);
  memcpy(out + k, d->f_hg + e0 * d->npe * 3, sizeof(double) * k);
  return 0;
}
int wfo_set_elem_forces_range(wfo_domain *d, int64_t e0, int64_t e1, const double *in) {
  if (e0 < 0 || e1 > d->ne || e0 > e1) return -1;
  const size_t k = (size_t)(e1 - e0) * d->npe * 3;
  memcpy(d->f_elem + e0 * d->npe * 3, in, sizeof(double) * k);
  memcpy(d->f_hg + e0 * d->npe * 3, in + k, sizeof(double) * k);
  return 0;
}

/* Node state of nodes [n0, n1): x, v, a, prev_a, u (3 each per node, field
 * after field). */
int wfo_get_node_state_range(const wfo_domain *d, int64_t n0, int64_t n1, double *out) {
  if (n0 < 0 || n1 > d->nn || n0 > n1) return -1;
  const size_t k = (size_t)(n1 - n0) * 3;
  const double *src[5] = {d->x, d->v, d->a, d->prev_a, d->u};
  for (int f = 0; f < 5; f++) memcpy(out + f * k, src[f] + 3 * n0, sizeof(double) * k);
  return 0;
}
int wfo_set_node_state_range(wfo_domain *d, int64_t n0, int64_t n1, const double *in) {
  if (n0 < 0 || n1 > d->nn || n0 > n1) return -1;
  const size_t k = (size_t)(n1 - n0) * 3;
  double *dst[5] = {d->x, d->v, d->a, d->prev_a, d->u};
  for (int f = 0; f < 5; f++) memcpy(dst[f] + 3 * n0, in + f * k, sizeof(double) * k);
  return 0;
}

int wfo_run(wfo_domain *d, int64_t nsteps) {
  for (int64_t s = 0; s < nsteps; s++) one_step(d);
  return 0;
}

int64_t wfo_solve(wfo_domain *d) {
  int64_t n = 0;
  while (d->time < d->end_t) {
    one_step(d);
    n++;
  }
  return n;
}

double wfo_time(const wfo_domain *d) { return d->time; }

int wfo_get_node_vec(const wfo_domain *d, int which, double *out) {
  const double *src[] = {d->x, d->v, d->a, d->u, d->prev_a, d->fi, d->u_dt, d->contforce};
  if (which < 0 || which > 7) return -1;
  memcpy(out, src[which], sizeof(double) * 3 * d->nn);
  return 0;
}

int wfo_get_node_scalar(wfo_domain *d, int which, double *out) {
  const double *src[] = {d->mass, d->voln, d->p_node, d->T};
  if (which < 0 || which > 3) return -1;
  memcpy(out, src[which], sizeof(double) * d->nn);
  return 0;
}

int wfo_get_elem_scalar(const wfo_domain *d, int which, double *out) {
  const double *src[] = {d->vol, d->vol0, d->detJ, d->p, d->pl_strain, d->sigma_y, d->rho};
  if (which < 0 || which > 6) return -1;
  memcpy(out, src[which], sizeof(double) * d->ne);
  return 0;
}

int wfo_get_elem_tensor(const wfo_domain *d, int which, double *out) {
  const double *src[] = {d->sigma, d->tau, d->eps, d->str_rate, d->rot_rate};
  if (which < 0 || which > 4) return -1;
  memcpy(out, src[which], sizeof(double) * 6 * d->ne);
  return 0;
}

void wfo_get_derivs(const wfo_domain *d, double *out) {
  memcpy(out, d->dH, sizeof(double) * 3 * d->npe * d->ne);
}

void wfo_get_elem_forces(const wfo_domain *d, double *f, double *fhg) {
  memcpy(f, d->f_elem, sizeof(double) * 3 * d->npe * d->ne);
  memcpy(fhg, d->f_hg, sizeof(double) * 3 * d->npe * d->ne);
}

int64_t wfo_get_reaction(const wfo_domain *d, double *out, int64_t cap) {
  int64_t n = d->hist_len < cap ? d->hist_len : cap;
  if (out && n > 0) memcpy(out, d->react_hist, sizeof(double) * n);
  return d->hist_len;
}

int64_t wfo_get_energies(const wfo_domain *d, double *ekin, double *eint, int64_t cap) {
  int64_t n = d->hist_len < cap ? d->hist_len : cap;
  if (ekin && n > 0) memcpy(ekin, d->ekin_hist, sizeof(double) * n);
  if (eint && n > 0) memcpy(eint, d->eint_hist, sizeof(double) * n);
  return d->hist_len;
}
