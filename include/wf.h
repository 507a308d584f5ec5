/* weldform-gb300: C ABI of the GB300 explicit updated-Lagrangian step.
 *
 * Drop-in for the solve loop of the reference's MetFEM::Domain_d
 * (include/common/Domain_d.h:231-1044, loop in src/explicit/Solver_explicit.C:
 * 101-1271). Each entry point names the reference member it replaces.
 *
 * Conventions
 *  - Every function returns wf_status; none exits or prints. wf_last_error()
 *    gives a one-line message for the last failing call on a domain.
 *  - Host pointers are borrowed for the duration of the call only. Device
 *    memory is owned by the library; one CUDA stream per domain. A domain
 *    handle is not thread-safe.
 *  - Node vectors are interleaved x[3n+d] and element tensors are Voigt
 *    [xx, yy, zz, xy, yz, xz], as the reference's arrays (Domain_d.h:841-1043).
 *  - Precision: WF_FP64 computes every quantity in FP64 with the reference's
 *    operation order; WF_MIXED computes element arithmetic in FP32 and keeps
 *    FP64 for nodal positions, displacements, the time step and reaction sums.
 */
#ifndef WF_H
#define WF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define WF_API __attribute__((visibility("default")))
#else
#define WF_API
#endif

typedef enum {
  WF_OK = 0,
  WF_ERR_ARG = 1,         /* invalid argument (null, out of range, wrong size) */
  WF_ERR_STATE = 2,       /* call out of order (e.g. run before init) */
  WF_ERR_CUDA = 3,        /* CUDA runtime error (no device, launch failure) */
  WF_ERR_NOMEM = 4,       /* host or device allocation failed */
  WF_ERR_UNSUPPORTED = 5, /* option not supported in the selected mode */
  WF_ERR_NONFINITE = 6,   /* non-finite state detected by the device checks */
  WF_ERR_TIMEOUT = 7      /* a bounded device wait ran out */
} wf_status;

typedef enum { WF_FP64 = 0, WF_MIXED = 1 } wf_precision;

typedef enum {
  WF_MAT_BILINEAR = 0, WF_MAT_HOLLOMON = 1, WF_MAT_JOHNSON_COOK = 2, WF_MAT_GMT = 3
} wf_material_model;

/* Material_ + Elastic_ (include/common/Material.cuh:15-156). BILINEAR is
 * linear isotropic hardening sigma_y = sy0 + H eps_p. HOLLOMON is the
 * reference law sigma_y = K (eps_p + sy0/E)^m past the plateau
 * (Material.cuh:353-395). cs0 = sqrt(K_bulk / rho) as the reference drivers
 * set it (src/explicit/main.C:507). */
typedef struct {
  int32_t model;
  double E, nu, rho;
  double sy0, H;
  double hol_K, hol_m;
} wf_material;

/* StabilizationParams (Domain_d.h:139-152), used by pressure algorithm 0;
 * all zero by default as in the reference constructor (Domain_d.h:292-303). */
typedef struct {
  double alpha_free, alpha_contact, hg_coeff_free, hg_coeff_contact;
  double av_coeff_div, av_coeff_bulk, log_factor, pspg_scale, p_pspg_bulkfac, J_min;
} wf_stab;

/* Node vector fields for wf_get_node_field. */
enum {
  WF_NODE_X = 0, WF_NODE_V = 1, WF_NODE_A = 2, WF_NODE_U = 3, WF_NODE_PREV_A = 4,
  WF_NODE_FI = 5, WF_NODE_CONTFORCE = 7
};
/* Node scalar fields. */
enum { WF_NODE_MASS = 0, WF_NODE_VOLN = 1, WF_NODE_PRESSURE = 2, WF_NODE_TEMP = 3 };
/* Element scalar fields. */
enum {
  WF_ELEM_VOL = 0, WF_ELEM_VOL0 = 1, WF_ELEM_DETJ = 2, WF_ELEM_P = 3,
  WF_ELEM_PL_STRAIN = 4, WF_ELEM_SIGMA_Y = 5, WF_ELEM_RHO = 6
};
/* Element tensor fields (Voigt, 6 per element). */
enum { WF_ELEM_SIGMA = 0, WF_ELEM_TAU = 1, WF_ELEM_EPS = 2, WF_ELEM_STR_RATE = 3, WF_ELEM_ROT_RATE = 4 };

typedef struct wf_domain wf_domain;

/* Domain_d::Domain_d (Domain_d.h:245). Selects device 0 unless
 * wf_domain_create_on_device is used. */
WF_API wf_status wf_domain_create(wf_domain **out);
WF_API wf_status wf_domain_create_on_device(wf_domain **out, int device);
/* Domain_d::Free (Domain_d.C:786-900). */
WF_API wf_status wf_domain_destroy(wf_domain *d);
WF_API const char *wf_last_error(const wf_domain *d);
WF_API const char *wf_status_string(wf_status s);
WF_API int32_t wf_abi_version(void);

/* ---- mesh ---------------------------------------------------------------- */
/* Domain_d::AddBoxLength(V, L, r, red_int, tritetra) (Domain_d.C:1136-1504):
 * structured box of hexahedra (tritetra = 0) or six tetrahedra per cell,
 * same node and element numbering, node->element lists element-ascending.
 * Only 3-D, one-point integration (red_int != 0) is supported. */
WF_API wf_status wf_add_box_length(wf_domain *d, const double V[3], const double L[3], double r,
                                   int32_t red_int, int32_t tritetra);
/* Domain_d::CreateFromLSDyna / setNodElem (Domain_d.C:1508-1699): explicit
 * nodes (xyz[3*nn]) and connectivity (elnod[ne*npe], npe = 8 or 4). */
WF_API wf_status wf_set_mesh(wf_domain *d, int64_t nn, int64_t ne, int32_t npe, const double *xyz,
                             const int32_t *elnod);
/* Domain_d::setNode (Domain_d.C:2473) for one node, and for all nodes. */
WF_API wf_status wf_set_node(wf_domain *d, int64_t n, double x, double y, double z);
WF_API wf_status wf_set_nodes(wf_domain *d, const double *xyz);
/* getNodeCount / getElemCount (Domain_d.h:561-563). */
WF_API wf_status wf_get_sizes(const wf_domain *d, int64_t *nn, int64_t *ne, int32_t *npe,
                              int64_t *nodel_total);
/* m_elnod, m_nodel, m_nodel_loc, m_nodel_offset, m_nodel_count (Domain_d.h:961-965).
 * The lists are element-ascending per node; before wf_init they are built on
 * the host on first request, after it read back from the device tables the
 * step uses. Any output pointer may be NULL. */
WF_API wf_status wf_get_connectivity(const wf_domain *d, int32_t *elnod, int32_t *nodel,
                                     int32_t *nodel_loc, int32_t *offset, int32_t *count);

/* ---- material ------------------------------------------------------------ */
/* Domain_d::setDensity (Domain_d.C:952). */
WF_API wf_status wf_set_density(wf_domain *d, double rho);
/* Domain_d::AssignMaterial (Domain_d.C:903): material table; entry 0 is the
 * default of every element. Sets the density of every element to mats[0].rho. */
WF_API wf_status wf_set_materials(wf_domain *d, int32_t nmat, const wf_material *mats);
/* Material_::Init_JohnsonCook (Material.cuh:105-114) for a material of model
 * WF_MAT_JOHNSON_COOK: sigma_y = (sy0 + B eps_p^n) (1 + C ln(edot / eps0_dot))
 * (1 - T_h^m), T_h = (T - T_transition) / (T_melt - T_transition), and the
 * tangent modulus n B eps_p^(n-1) (1 + C ln(edot' / eps0_dot)) (1 - T_h^m)
 * (E / 10 at eps_p = 0) of the radial return (CalcJohnsonCookYieldStress,
 * CalcJohnsonCookTangentModulus, Material.cuh:377-410; CalcStressStrain,
 * Mechanical.C:1701-1770). edot is the element's effective strain rate
 * sqrt(((Dxx-Dyy)^2 + (Dyy-Dzz)^2 + (Dzz-Dxx)^2) / 2 + 3 (Dxy^2 + Dyz^2 + Dxz^2))
 * (1e-5 where it is exactly 0) and edot' = min(edot, cap), cap from
 * wf_set_max_strain_rate (default 1e6). T is the
 * (uniform) temperature of the material's elements; with thermal coupling
 * (wf_set_thermal) each element takes the mean of its node temperatures
 * instead. Call after wf_set_materials and before wf_init. */
WF_API wf_status wf_set_johnson_cook(wf_domain *d, int32_t mat, double B, double n, double C,
                                     double eps0_dot, double m, double T_melt,
                                     double T_transition, double T);
/* The GMT law (class GMT, Material.cuh:255-290; CalcGMTYieldStress and
 * CalcGMTTangentModulus, Material.cuh:417-478) for a material of model
 * WF_MAT_GMT. With e = eps_p, r = edot and T each clamped to its range,
 *   sigma_y = C1 exp(C2 T) e^(n1 T + n2) exp((I1 T + I2) / e) r^(m1 T + m2),
 *   Et = C1 exp(C2 T) r^(m1 T + m2) e^(n1 T + n2 - 2)
 *        (e (n1 T + n2) - I1 T - I2) exp((I1 T + I2) / e),
 * sigma_y at the element's effective strain rate edot (as for Johnson-Cook,
 * without its 1e-5 floor) and Et at min(edot, cap) (CalcStressStrain,
 * Mechanical.C:1727-1749). c = {n1, n2, C1, C2, m1, m2, I1, I2}, the order of
 * the input deck's "const" (main.C:548-551). range = {e_min, e_max, er_min,
 * er_max, T_min, T_max} (the class defaults are {0, 1e10, 0, 1e10, 0, 1e10});
 * e_min must be > 0, since at e = 0 both functions are 0 * inf.
 * T is the temperature as for wf_set_johnson_cook. (The reference's GMT
 * constructor stores the eight constants in members of the derived class that
 * hide Material_'s, which the two functions read, so a reference deck's GMT
 * material runs with Material_'s uninitialised values; here the constants
 * reach the law.) Call after wf_set_materials and before wf_init. */
WF_API wf_status wf_set_gmt(wf_domain *d, int32_t mat, const double c[8], const double range[6],
                            double T);
/* Domain_d::m_plheatfraction (Domain_d.h:783, default 0.9; deck key
 * Configuration.plHeatFrac): the fraction of the plastic work rate that
 * CalcStressStrain turns into the element's heat source (Mechanical.C:1804);
 * thermal coupling only. In [0, 1], before wf_init. */
WF_API wf_status wf_set_plastic_heat_fraction(wf_domain *d, double f);
/* Domain_d::m_max_edot (Domain_d.h:824, default 1e6; deck key
 * Configuration.maxStrRate): the effective strain rate at which the
 * Johnson-Cook and GMT tangent moduli are evaluated is capped there
 * (Mechanical.C:1737). > 0, before wf_init. */
WF_API wf_status wf_set_max_strain_rate(wf_domain *d, double r);
/* Per-element material index (the reference's mat[e] pointers). */
WF_API wf_status wf_set_elem_materials(wf_domain *d, const int32_t *ids);

/* ---- boundary conditions -------------------------------------------------- */
/* Domain_d::AddBCVelNode (Domain_d.C:1057). */
WF_API wf_status wf_add_bc_vel_node(wf_domain *d, int64_t node, int32_t dim, double val);
/* AddBCVelNode for n entries at once, in order (node[i], dim[i], val[i]). */
WF_API wf_status wf_add_bc_vel_nodes(wf_domain *d, int64_t n, const int64_t *node,
                                     const int32_t *dim, const double *val);
/* Domain_d::AddBCVelZone (Domain_d.C:432-452); *count = nodes inside. */
WF_API wf_status wf_add_bc_vel_zone(wf_domain *d, const double start[3], const double end[3],
                                    const double vel[3], int64_t *count);
/* Domain_d::AllocateBCs (Domain_d.C:1063). */
WF_API wf_status wf_allocate_bcs(wf_domain *d);

/* ---- options ---------------------------------------------------------------- */
WF_API wf_status wf_set_dt(wf_domain *d, double dt);         /* SetDT (Domain_d.h:635) */
WF_API wf_status wf_set_end_time(wf_domain *d, double t);    /* SetEndTime (Domain_d.h:636) */
/* WF_FP64 (default) or WF_MIXED. The mixed path takes every option of the
 * step but non-default stabilisation parameters and pressure algorithm 1
 * (WF_ERR_UNSUPPORTED at wf_init: algorithm 1 adds k0 (1 - J ratio) to each
 * element's pressure every step, and an FP32 J ratio near 1 resolves the
 * volume change only to about 6e-8). Its exported sigma leaves out the
 * artificial viscosity term (the strain rate is not kept). */
WF_API wf_status wf_set_precision(wf_domain *d, int32_t precision);
/* Viscous hourglass coefficient of 1-point hexahedra (0 = off): the 3-D form
 * of the reference's test driver (src/common/test_1el_3D.cpp:159-199). */
WF_API wf_status wf_set_hourglass(wf_domain *d, double coef);
/* m_press_algorithm (Domain_d.h:672): 0 = nodal-averaged J (default), 1 = ANP. */
WF_API wf_status wf_set_press_algorithm(wf_domain *d, int32_t alg);
WF_API wf_status wf_set_stab(wf_domain *d, const wf_stab *s);          /* m_stab */
WF_API wf_status wf_set_artif_visc(wf_domain *d, double alpha, double beta); /* m_artifvisc */
/* 0: lumped mass recomputed each step from the current volume (reference
 * loop, Solver_explicit.C:605-607); 1: mass kept at its initial value. */
WF_API wf_status wf_set_mass_mode(wf_domain *d, int32_t mode);
/* Energy history (before wf_init; off by default): after every step the
 * kinetic energy sum_n m_n |v_n|^2 / 2 and the internal energy accumulated
 * as Eint += dt * sum_e (sigma_e . str_rate_e) vol_e over the six stored
 * Voigt components (Domain_d::computeEnergies, Mechanical.C:2145-2185, called
 * at Solver_explicit.C:1029-1031). Adds one reduction launch per step. */
WF_API wf_status wf_set_energy_history(wf_domain *d, int32_t on);
/* *n = steps recorded; copies min(cap, *n) values into each non-null array. */
WF_API wf_status wf_get_energy_history(wf_domain *d, double *ekin, double *eint, int64_t cap,
                                       int64_t *n);
/* Reaction history: per step, sum over `nodes` of the assembled internal
 * force component `dim` (recorded after assembly). */
WF_API wf_status wf_set_reaction_nodes(wf_domain *d, int64_t n, const int32_t *nodes, int32_t dim);
/* Rigid flat die with outward normal -z at z = z0 + vz*t, acting on the
 * candidate nodes (Domain_d::CalcContactForces, Contact.C:31-334, for one
 * plane): normal stiffness min(kpen, 0.2 m / dt^2) as the reference caps it,
 * Coulomb coefficient mu. With contact on, the reaction history records the
 * sum of normal contact forces. */
WF_API wf_status wf_set_contact_plane(wf_domain *d, double z0, double vz, double kpen, double mu,
                                      int64_t ncand, const int32_t *cand_nodes);

/* Thermal coupling (Domain_d::setThermalOn / setTemp,
 * ThermalCalcs, Thermal.C:27-126; calcThermalExpansion, :163-178): every node
 * starts at T0; each element adds to its nodes' temperature rates the
 * conduction term -(1/m_i) (K T)_i with K_ij = (sum_d dN_i detJ dN_j detJ)
 * k_T / detJ w, and the plastic heat 0.9 q vol / n / (m_i cp_T), where
 * q = 0.9 sigma : (d eps_p / dt) is formed in the radial return
 * (Mechanical.C:1783-1810; the reference applies the 0.9 plastic-work fraction
 * twice); nodes in contact with a rigid body receive heat_cond * A *
 * (T_die - T), kept after the contact ends (Contact.C:309); then
 * T += (sum of rates + die heat / (m cp_T of material 0)) dt. The strain
 * rate's diagonal loses exp_T times the mean of the previous step's
 * element-node rates read at the element's node ids, as the reference indexes
 * them. A Johnson-Cook element takes the mean of its node temperatures (the
 * reference reads T[e], a node array indexed by element). Readback:
 * wf_get_node_scalar(WF_NODE_TEMP). Before wf_init; one domain (no
 * specimens, no adjoint). The mixed-precision step evaluates the same terms
 * in FP32 with the temperature kept as a compensated float pair. */
WF_API wf_status wf_set_thermal(wf_domain *d, int32_t on, double T0);
/* Conductivity k_T, heat capacity cp_T (> 0) and expansion coefficient of
 * material `mat` (Material_ k_T, cp_T, exp_T; deck keys thermalCond,
 * thermalHeatCap, thermalExp). */
WF_API wf_status wf_set_material_thermal(wf_domain *d, int32_t mat, double k_T, double cp_T,
                                         double exp_T);
/* Heat transfer coefficient and temperature of the rigid bodies (TriMesh_d
 * heat_cond, T_const; deck Contact keys heatCondCoeff, dieTemp; defaults 0 and
 * 20). */
WF_API wf_status wf_set_contact_heat(wf_domain *d, double heat_cond, double T_die);

/* Rigid triangle-mesh die (Domain_d::setTriMesh / setContactOn / setContactPF,
 * Domain_d.h:464, :642, :771; CalcContactForces, Contact.C:31-334): mesh nodes
 * xyz[3 nnodes], triangles tri[3 ntri] (normal (n1-n0)x(n2-n0) pointing toward
 * the part), uniform velocity vel[3], static and dynamic Coulomb coefficients
 * and the penalty factor (reference default 0.1). The part's external surface
 * is found at wf_init (faces used by one element; tetrahedra with the
 * reference's triangle table, hexahedra with its quadrilateral table) and each
 * external node contacts the first triangle it penetrates: normal force
 * pf * min(E A / l, 0.2 m / dt^2) * depth plus damping, then Coulomb friction
 * from the accumulated slip. As in the reference, a node keeps its last contact
 * force after it leaves contact, the die velocity ramps as
 * sqrt(t / (0.01 end time)) over the first 1 % of the end time, and the
 * reaction history records the sum of normal-force magnitudes. This mesh is
 * rigid body 0; wf_add_contact_trimesh appends more. Both precisions: the
 * mixed step evaluates the contact in FP32 with coordinates relative to the
 * centre of the part's bounding box, the die kept in FP64. */
WF_API wf_status wf_set_contact_trimesh(wf_domain *d, int64_t nnodes, const double *xyz,
                                        int64_t ntri, const int32_t *tri, const double vel[3],
                                        double mu_static, double mu_dynamic,
                                        double penalty_factor);
/* Appends another rigid body to the contact mesh (TriMesh_d::AddMesh,
 * Mesh.C:445-545; Domain_d::addMeshData, Domain_d.C:2780): its nodes xyz[3 nnodes]
 * and triangles tri[3 ntri] (indices into this body's own nodes) with uniform
 * velocity vel[3]. Bodies take the indices 1, 2, ... in the order added; a
 * node contacts the first triangle it penetrates over all bodies in that
 * order, friction and penalty factor are those of wf_set_contact_trimesh, and
 * the reaction history sums only the contacts with body 0 (Contact.C:326-329).
 * Called after wf_set_contact_trimesh and before wf_init. */
WF_API wf_status wf_add_contact_trimesh(wf_domain *d, int64_t nnodes, const double *xyz,
                                        int64_t ntri, const int32_t *tri, const double vel[3]);
/* Current die node positions (3 per node, all bodies in order): *n = node
 * count, copies min(cap, *n). */
WF_API wf_status wf_get_trimesh_nodes(wf_domain *d, double *out, int64_t cap, int64_t *n);

/* ---- batched ensemble --------------------------------------------------------- */
/* Declares the mesh a batch of nspec independent specimens (no counterpart in
 * the reference, which runs one domain per process): specimen s owns elements
 * [elem_off[s], elem_off[s+1]) and nodes [node_off[s], node_off[s+1]) and no
 * element may reference another specimen's node. Each specimen advances with
 * its own time step dt[s] (wf_set_dt is then not needed) and records its own
 * reaction history over the reaction nodes it owns. All specimens step
 * together in the same four launches. Not combinable with contact. */
WF_API wf_status wf_set_specimens(wf_domain *d, int32_t nspec, const int64_t *elem_off,
                                  const int64_t *node_off, const double *dt);
/* Reaction history of one specimen: *n = steps recorded, copies min(cap, *n). */
WF_API wf_status wf_get_specimen_reaction(wf_domain *d, int32_t spec, double *out, int64_t cap,
                                          int64_t *n);

/* ---- run ---------------------------------------------------------------------- */
/* Preamble of SolveChungHulbert (Solver_explicit.C:120-268): uploads the
 * mesh, imposes initial BCs, computes initial geometry, volumes and masses.
 * The time step may be set before or after (wf_min_edge_length works once
 * the mesh is on the device); it must be set before wf_run. */
WF_API wf_status wf_init(wf_domain *d);
/* nsteps iterations of the loop body (Solver_explicit.C:346-1167). The
 * per-phase kernels of the steps are replayed from CUDA graphs: graphs of 32
 * steps, then one graph of the remaining steps (a single remaining step is
 * launched directly). A graph is captured and instantiated the first time a
 * run needs it and kept until a launch parameter changes (time step, end
 * time, launch shapes, history growth). */
WF_API wf_status wf_run(wf_domain *d, int64_t nsteps);
/* No counterpart in the reference. Captures and instantiates now the graphs
 * a following wf_run(d, nsteps) replays (and grows the histories it fills),
 * so that the run itself does no capture. Runs nothing. */
WF_API wf_status wf_prepare_run(wf_domain *d, int64_t nsteps);
/* No counterpart in the reference. One step in two halves, for a slab
 * decomposition of one mesh over several domains (weldformfem_gb300/slabs.py):
 * wf_step_begin queues the predictor, geometry, nodal and element phases
 * (the loop body up to the element forces, Solver_explicit.C:346-760),
 * wf_step_end the assembly and node update (assemblyForces onwards). Between
 * them wf_get_halo_forces / wf_set_halo_forces read and overwrite the element
 * and hourglass forces of elements [e0, e1) (2 x (e1 - e0) x npe x 3 doubles:
 * forces, then hourglass forces, per element and local node); after
 * wf_step_end, wf_get_halo_nodes / wf_set_halo_nodes read and overwrite the
 * node state a step starts from for nodes [n0, n1): positions, velocities,
 * previous accelerations and displacements (12 x (n1 - n0) doubles: field,
 * then component, then node). Host buffers; the calls wait for the domain's
 * stream. In mixed precision the halves run the per-phase kernels (whatever
 * the step mode of wf_run); the forces are the FP32 element-minus-hourglass
 * forces widened to doubles (npe x 3 rows of (e1 - e0) values, then as many
 * zeros), and the node state is 18 x (n1 - n0) doubles: position hi and lo
 * parts, velocity, previous acceleration, predicted velocity and contact slip,
 * each exact. Not with specimens, thermal coupling, triangle-mesh contact or
 * the energy history (WF_ERR_UNSUPPORTED). */
WF_API wf_status wf_step_begin(wf_domain *d);
WF_API wf_status wf_step_end(wf_domain *d);
WF_API wf_status wf_get_halo_forces(wf_domain *d, int64_t e0, int64_t e1, double *out);
WF_API wf_status wf_set_halo_forces(wf_domain *d, int64_t e0, int64_t e1, const double *in);
/* Values per node of wf_get_halo_nodes / wf_set_halo_nodes: 12 (FP64) or 18
 * (mixed); the buffers hold that many times (n1 - n0) doubles. */
WF_API wf_status wf_get_halo_node_width(const wf_domain *d, int32_t *values_per_node);
WF_API wf_status wf_get_halo_nodes(wf_domain *d, int64_t n0, int64_t n1, double *out);
WF_API wf_status wf_set_halo_nodes(wf_domain *d, int64_t n0, int64_t n1, const double *in);
/* Domain_d::SolveChungHulbert: steps while Time < end time; *nsteps = count. */
WF_API wf_status wf_solve(wf_domain *d, int64_t *nsteps);
WF_API wf_status wf_get_time(const wf_domain *d, double *t, int64_t *step);
/* Waits for the domain's stream and reports any device-side error status.
 * As the reference loop does (Solver_explicit.C:777-785), a non-finite
 * assembled internal force is cleared to zero and the run goes on; the node
 * kernels also raise a flag, which the first wf_sync (or wf_solve) after the
 * wf_run that raised it reports as WF_ERR_NONFINITE, with the smallest
 * offending node id in wf_last_error(). The flag is then cleared, so a
 * later wf_sync reports only new occurrences. Readbacks do not check it. */
WF_API wf_status wf_sync(wf_domain *d);
/* Minimum element edge length of the current mesh (device reduction). */
WF_API wf_status wf_min_edge_length(wf_domain *d, double *hmin);
/* Per-phase timing. While on, wf_run launches the four kernels of each step
 * directly (no graph) with CUDA events around each, on the domain's stream.
 * wf_get_phase_times returns the accumulated milliseconds of the geometry,
 * nodal, element and node phases (ms[4]) and the steps timed; reset != 0
 * clears the accumulators after reading. */
WF_API wf_status wf_set_phase_timing(wf_domain *d, int32_t on);
WF_API wf_status wf_get_phase_times(wf_domain *d, double ms[4], int64_t *steps, int32_t reset);
/* Launch-shape autotuning of the mixed-precision geometry, nodal and element
 * kernels (on by default): at wf_init the library times each kernel on the
 * domain's own data for block sizes {64, 128, 256} x {1, 2} items per
 * thread or a persistent grid of (SMs x resident blocks) (items_per_thread
 * reported as 0), all grid-stride, timed in interleaved rounds, and keeps the
 * fastest; the kernels' results do not
 * depend on the shape, and the state the element kernel advances is restored
 * after the trials. The choice is kept for the life of the process, keyed by
 * the device, the element type, the mesh sizes and the kernel variant
 * (material law, contact, thermal coupling, energy history, specimens): a
 * later domain with the same key takes it without timing again.
 * wf_get_launch_config reports the choice for phase 0 (geometry), 1 (nodal)
 * or 2 (element). */
WF_API wf_status wf_set_autotune(wf_domain *d, int32_t on);
WF_API wf_status wf_get_launch_config(const wf_domain *d, int32_t phase, int32_t *block,
                                      int32_t *items_per_thread, double *ms);
/* Sets a launch shape by hand (block 64, 128 or 256; items_per_thread >= 1, or
 * 0 for a persistent grid); with autotuning off before wf_init, or any time
 * after it (the choice replaces the tuned one). */
WF_API wf_status wf_set_launch_config(wf_domain *d, int32_t phase, int32_t block,
                                      int32_t items_per_thread);
/* Step scheduling of the mixed-precision path. Mode 1: each step is the four
 * phase kernels (geometry, nodal, element, node), replayed as a CUDA graph.
 * Mode 2: a whole wf_run is one launch of one thread-block cluster (up to 16
 * blocks, sized at wf_init for meshes of at most 65536 elements) whose blocks
 * own fixed element and node ranges and meet at cluster barriers between the
 * phases: same per-element and per-node arithmetic, so the state is bitwise
 * that of mode 1; the reaction sum runs in another order. Not with specimens,
 * the energy history or phase timing. Mode 3 (hexahedra): the element and
 * node phases become a tiled kernel and a shared-node kernel. At wf_init the
 * elements are binned by centroid into cubes of about 8 element sizes and cut
 * into tiles of at most 512 elements; one block per tile stages the tile's
 * nodes in shared memory, computes its elements' forces (same arithmetic as
 * mode 1), sums them per node in shared memory and updates the nodes all of
 * whose elements are in the tile; the other ("shared") nodes gather their
 * forces from HBM in list order, as in mode 1. On meshes numbered like
 * AddBoxLength's, every node's force is summed in mode 1's order, so the
 * state is bitwise that of mode 1; the reaction sum runs in another order.
 * Not with specimens, thermal coupling, the energy history or triangle-mesh
 * contact; the tiles are built by wf_init when mode 3 is set before it, and
 * wf_get_tiles tells whether the mesh was tiled. Mode 4 (box meshes of
 * hexahedra, see wf_set_box_indexing): the element and node phases become one
 * column sweep. The node grid is cut into columns of at most 31 x 8 nodes
 * (x, y; or 31 x 4, wf_set_sweep_rows), one block each, which sweeps its
 * column's element layers upwards with the element forces in shared memory:
 * it computes the elements around its nodes (those of the neighbouring
 * columns' ring included, again), and each node adds its eight element forces
 * in list order, so the state is bitwise that of mode 1; the reaction sum
 * runs in another order. Positions, predicted velocities, tau and eps_p are
 * held twice (read one copy, write the other). Not with specimens, thermal
 * coupling or triangle-mesh contact; wf_get_sweep tells whether the mesh is
 * swept. Mode 5 (the same meshes): after the geometry and nodal kernels, one
 * persistent launch runs the element and node phases as a wavefront through
 * the element layers. The work is cut into tiles of 512 elements or nodes of
 * one layer or plane (wf_set_flow_tiles); blocks take tiles in a fixed ticket
 * order (the elements of layer s, then the node update of plane s-lag) and a
 * node tile waits, with a bounded wait, for the element tiles it reads, so
 * the element forces are read back from L2 shortly after they are written.
 * Each element and node runs mode 1's arithmetic: the state is bitwise that
 * of mode 1; the reaction sum runs in another order. A wait that runs out (a
 * bug, never
 * expected) makes the next wf_sync return WF_ERR_TIMEOUT. On GB300 mode 5 is
 * slower than modes 4 and 1 (the blocks' waits and ticket traffic cost more
 * than the L2 reuse saves) and is only run when asked for. Mode 0 (default)
 * picks mode 2 for meshes of at most 3000 elements, else mode 4 where the mesh
 * is swept and its columns fill the GPU (at least 95 % of two per SM: a
 * column is a sequence of layers), else mode 1. wf_get_step_mode reports the mode the next wf_run uses and,
 * for mode 2, the cluster's blocks and block size, for mode 3 the tiles and
 * threads per tile, for mode 4 the columns and threads per column, for mode 5
 * the blocks and threads per block (0 otherwise). */
WF_API wf_status wf_set_step_mode(wf_domain *d, int32_t mode);
/* No counterpart in the reference. Node rows per column of the column sweep
 * (4 or 8, default 8), before wf_init. wf_get_sweep: the columns along x and
 * y and the rows per column, or zeros and, in why (NUL-terminated, at most
 * why_cap bytes), the reason the mesh is not swept. Any output may be NULL. */
WF_API wf_status wf_set_sweep_rows(wf_domain *d, int32_t rows);
/* No counterpart in the reference. Dataflow step (mode 5): items per tile (a
 * multiple of 256, 256 to 8192; default 512) and the layers the node update
 * lags the elements (1 to 16; default 4), before wf_init. wf_get_flow: tiles
 * per step and blocks per launch, or zeros and, in why, the reason the mesh
 * has no dataflow step. Any output may be NULL. */
WF_API wf_status wf_set_flow_tiles(wf_domain *d, int32_t tile, int32_t lag);
WF_API wf_status wf_get_flow(const wf_domain *d, int32_t *tiles, int32_t *grid, char *why,
                             int64_t why_cap);
WF_API wf_status wf_get_sweep(const wf_domain *d, int32_t *columns_x, int32_t *columns_y,
                              int32_t *rows, char *why, int64_t why_cap);
/* No counterpart in the reference. Box meshes: when the connectivity is the
 * AddBoxLength numbering of nx x ny x nz hexahedra (checked element by element
 * at wf_init, however the mesh was uploaded), the mixed-precision kernels
 * compute each element's corners and each node's element list (in list
 * order, with the node's corner in each element) from the indices instead of
 * reading the connectivity and list arrays: the same values in the same
 * order, so the same results bit for bit, with 128 bytes less HBM traffic per
 * element and step. On by default; wf_set_box_indexing(d, 0) before wf_init
 * keeps reading the arrays. wf_get_box gives nx, ny, nz, or zeros when the
 * domain does not use it. */
WF_API wf_status wf_set_box_indexing(wf_domain *d, int32_t on);
WF_API wf_status wf_get_box(const wf_domain *d, int32_t dims[3]);
/* No counterpart in the reference. The tiles built at wf_init for step mode
 * 3: their number, the number of shared nodes, the sum over tiles of their
 * distinct nodes and the node-list entries of the shared nodes (the counts
 * the tiled kernels' memory traffic follows), or zeros and, in why (a
 * NUL-terminated string of at most why_cap bytes), the reason the mesh was
 * not tiled. Any output may be NULL. */
WF_API wf_status wf_get_tiles(const wf_domain *d, int32_t *ntiles, int32_t *nshared,
                              int64_t *tile_nodes, int64_t *shared_slots, char *why,
                              int64_t why_cap);
WF_API wf_status wf_get_step_mode(const wf_domain *d, int32_t *mode, int32_t *blocks,
                                  int32_t *block_size);
/* Number of kernels this domain has launched since wf_init (graph nodes
 * included). */
WF_API wf_status wf_get_launch_count(const wf_domain *d, int64_t *n);
/* Number of step graphs this domain has replayed since wf_init. */
WF_API wf_status wf_get_graph_launches(const wf_domain *d, int64_t *n);
/* The domain's CUDA stream (a cudaStream_t), for callers that order their
 * own work or CUDA events after the domain's kernels. */
WF_API wf_status wf_get_stream(const wf_domain *d, void **stream);
/* Bytes copied host->device and device->host by this domain so far. */
WF_API wf_status wf_get_transfer_bytes(const wf_domain *d, int64_t *h2d, int64_t *d2h);

/* ---- allocation-free entry point ------------------------------------------------ */
/* No counterpart in the reference. For callers that cannot allocate device
 * memory (code inside another framework's memory pool, loops that must not
 * risk the synchronisation cudaMalloc/cudaFree can cause, hosts with a device
 * budget fixed up front): each element's volume (determinant of its Jacobian
 * times the integration weight: 8 at the centre of a hexahedron, 1/6 for a
 * tetrahedron), then each node's volume (the sum of its elements' volumes in
 * list order, divided by the nodes per element), computed without any
 * allocation. The caller
 * passes device pointers: xyz[3*nn] interleaved coordinates, elnod[ne*npe]
 * (npe 8 or 4), the node->element lists as wf_get_connectivity returns them
 * (nodel_offset[nn], nodel_count[nn], nodel[total]) and voln[nn] for the
 * result (sum of the node's element volumes divided by npe); work is queued
 * on `stream` (a cudaStream_t, 0 for the default stream) and the call
 * returns without waiting.
 * The element volumes go to a static device array of WF_NOALLOC_MAX_ELEMS
 * doubles (8 MiB) that every GPU which loads the library holds until exit;
 * ne above that returns WF_ERR_UNSUPPORTED. The array is shared by all calls
 * and keeps the last call's contents; calls that overlap on the GPU race.
 * The first call on a device looks up the array's device address (again
 * after the device's context has been replaced, e.g. by cudaDeviceReset);
 * make that first call before any stream capture. A launch error of the call
 * returns WF_ERR_CUDA and is cleared; a CUDA error already pending on the
 * calling thread is left pending and not reported here. */
#define WF_NOALLOC_MAX_ELEMS 1048576
WF_API wf_status wf_nodal_volumes_noalloc(const double *xyz, const int32_t *elnod, int64_t nn,
                                          int64_t ne, int32_t npe, const int32_t *nodel_offset,
                                          const int32_t *nodel_count, const int32_t *nodel,
                                          double *voln, void *stream);

/* ---- adjoint ---------------------------------------------------------------------- */
/* No counterpart in the reference, which computes no derivatives. Reverse mode
 * of the FP64 step for material identification: for a loss L(R_0 .. R_{N-1})
 * of the reaction history over N steps, the gradient with respect to E,
 * sigma_y0 and H of every material.
 * wf_adjoint_forward runs nsteps steps from the current state, as wf_run
 * does, and keeps an in-memory checkpoint of the state (x, v, prev_a, u, tau,
 * eps, eps_p) every `every` steps (0: about sqrt(nsteps); -1: keep every
 * step's inputs instead, no checkpoints and no recompute in the reverse pass,
 * when the device has room: nsteps (14 nn + 7 ne) doubles). Supported: FP64
 * precision, bilinear materials, pressure algorithm 0 with default
 * stabilisation, no artificial viscosity, no contact, no specimens.
 * wf_adjoint_backward takes dL_dR[nsteps] (host) and writes
 * grad[3 * nmat] = (dL/dE, dL/dsigma_y0, dL/dH) of each material in turn. It
 * recomputes each segment from its checkpoint, reverses it step by step
 * (node update, internal-force gather, element stress update with the
 * consistent derivative of the radial return, hourglass forces, nodal volumes
 * and masses), and leaves the domain in the state at the end of the forward
 * run, so it may be called again with another dL_dR. reverse_fp32 != 0 runs
 * the element reverse arithmetic in FP32 (the recomputed forward stays FP64).
 * The domain must not step between the two calls. */
WF_API wf_status wf_adjoint_forward(wf_domain *d, int64_t nsteps, int64_t every);
WF_API wf_status wf_adjoint_backward(wf_domain *d, const double *dL_dR, int32_t reverse_fp32,
                                     double *grad);

/* ---- input files and output ------------------------------------------------------- */
/* JSON deck of the reference's explicit driver (src/explicit/main.C:125-1005),
 * read on the host into a deck object that wf_deck_apply replays on a domain.
 * Read: Configuration (simTime, outTime, cflFactor, pressAlgorithm, plHeatFrac,
 * maxStrRate, artifViscCoeffs, xSymm/ySymm/zSymm, symtol), Stabilization, Materials[0]
 * (Bilinear: const[0] = tangent modulus Et, H = E Et / (E - Et); Hollomon:
 * const = [K, n]; JohnsonCook: A = yieldStress0, const = [B, n, C, eps0_dot]
 * with m = 1, T_melt = 1e10, T_transition = 0 as the non-thermal driver sets
 * them, temperature 0; GMT: const = [n1, n2, C1, C2, m1, m2, I1, I2] with
 * e_range, er_range, T_range, see wf_set_gmt; NortonHoff is rejected, since no
 * function of the reference's step reads its constants: CalcStressStrain keeps
 * the initial yield stress and, once the element yields, reads an unset
 * tangent modulus), DomainBlocks[0] (File: an LS-DYNA .k mesh, path relative to
 * the deck; Box: a 3-D box of elemLength cells, elemType TriTet for
 * tetrahedra) and BoundaryConditions (one velocity zone per condition, from
 * its start/end box or, when it has none, from the DomainZones entry of its
 * zoneId), then the symmetry-plane BCs, in the reference's order. The time
 * step is cflFactor * (shortest segment between the first four nodes of each
 * element) / sqrt(K / rho), the reference's calcMinEdgeLength in 3-D.
 * RigidBodies[0] and RigidBodies[1] (the reference driver reads no further
 * entries) become rigid triangle meshes, body 0 through
 * wf_set_contact_trimesh and body 1 through wf_add_contact_trimesh: type
 * Plane is TriMesh_d::AxisPlaneMesh on axis z from start/dim with partSide
 * cells per side and flipnormals; type File is a Nastran mesh (fileName,
 * relative to the deck; see wf_read_nastran) with flipnormals, orientNormals
 * (default true) and orientPoint (default the mean of the part's nodes). Each
 * body moves with the velocity of the boundary condition whose zoneId is the
 * body's; the Contact block gives fricCoeffStatic, fricCoeffDynamic and
 * penaltyFactor; as in the reference driver, a contact deck applies no
 * velocity zones to the part (symmetry planes only). Configuration.thermal
 * turns on the thermal coupling (wf_set_thermal) with the keys listed in
 * wf_deck_info; a JohnsonCook material then takes m, T_melt, T_transition
 * from const[4..6]. Axisymmetric/plane-strain, Perzyna and Line (2-D) rigid
 * bodies return WF_ERR_UNSUPPORTED. Configuration.hourglass3D (not a reference key,
 * default 0 as the reference's 3-D no-op) sets the viscous hourglass
 * coefficient. Errors are written into err (err_len bytes, may be null). */
typedef struct wf_deck wf_deck;
typedef struct {
  int64_t nn, ne;        /* mesh */
  int32_t npe;
  int32_t press_alg;
  int64_t n_bc;          /* AddBCVelNode calls: zone BCs (3 per node) then symmetry */
  int64_t zone_nodes;    /* nodes inside the velocity zones, summed over zones */
  int32_t n_zones;
  int32_t has_stab;
  double dt, end_time, out_time, cfl, min_length, sound_speed, hourglass;
  double artif_visc[2];
  wf_stab stab;
  wf_material material;
  /* rigid body 0 (RigidBodies[0]): its mesh sizes and velocity */
  int32_t contact;
  int32_t die_nodes, die_tris;
  double die_vel[3];
  double mu_static, mu_dynamic, penalty_factor;
  /* Johnson-Cook material: B, n, C, eps0_dot, m, T_melt, T_transition, T */
  double johnson_cook[8];
  int32_t rigid_bodies;  /* number of rigid bodies read (0, 1 or 2) */
  /* thermal coupling: Configuration.thermal, InitialConditions Temp (default
   * 20), Materials[0] thermalCond / thermalHeatCap / thermalExp, Contact
   * heatCondCoeff / dieTemp (default 20) */
  int32_t thermal;
  double T0, thermal_k, thermal_cp, thermal_exp, heat_cond, die_temp;
  /* GMT material: const n1, n2, C1, C2, m1, m2, I1, I2 and e_range, er_range,
   * T_range (main.C:548-552) */
  double gmt[8], gmt_range[6];
  /* Configuration plHeatFrac (default 0.9) and maxStrRate (default 1e6) */
  double plheat_frac, max_edot;
} wf_deck_info;
WF_API wf_status wf_deck_read(const char *path, wf_deck **out, char *err, int64_t err_len);
WF_API wf_status wf_deck_free(wf_deck *k);
WF_API wf_status wf_deck_get_info(const wf_deck *k, wf_deck_info *info);
/* xyz[3 nn] interleaved, elnod[ne npe]; either may be null. */
WF_API wf_status wf_deck_get_mesh(const wf_deck *k, double *xyz, int32_t *elnod);
/* Rigid body 0 of a contact deck: xyz[3 die_nodes], tri[3 die_tris]; either may be null. */
WF_API wf_status wf_deck_get_die(const wf_deck *k, double *xyz, int32_t *tri);
/* Rigid body `body` (0 .. rigid_bodies-1): sizes, velocity, xyz[3 nnodes] and
 * tri[3 ntris] (indices into the body's own nodes); any output may be null. */
WF_API wf_status wf_deck_get_body(const wf_deck *k, int32_t body, int64_t *nnodes, int64_t *ntris,
                                  double vel[3], double *xyz, int32_t *tri);
/* Nastran bulk-data die mesh (NastranReader::read, NastranReader.cpp:34-180, and
 * TriMesh_d(NastranReader&, ...), Mesh.C:560-760): GRID cards give the nodes
 * (fixed 8-column fields: id in columns 8-15, x y z from column 24; a D
 * exponent reads as E and a field without an exponent letter takes one before
 * its first sign after the first column, "1.5-3" = 1.5E-3), CTRIA cards the
 * triangles (node ids from column 24), each kind read as consecutive lines
 * from its first card. flip_normals swaps every triangle's first two nodes;
 * with orient_pt non-null, a triangle whose normal points away from the
 * interior point C + 2 (C - P) (C the mean node, P = orient_pt) is turned too,
 * so normals face P. Writes min(cap, count) nodes and triangles (either buffer
 * may be null) and the counts. CBEAM/CBAR line meshes return
 * WF_ERR_UNSUPPORTED. */
WF_API wf_status wf_read_nastran(const char *path, int32_t flip_normals, const double *orient_pt,
                                 double *xyz, int64_t cap_nodes, int32_t *tri, int64_t cap_tris,
                                 int64_t *nnodes, int64_t *ntris, char *err, int64_t err_len);
/* The n_bc AddBCVelNode calls in order; any array may be null. */
WF_API wf_status wf_deck_get_bcs(const wf_deck *k, int64_t *node, int32_t *dim, double *val);
/* Mesh, material, BCs (then AllocateBCs), options, dt and end time onto d. */
WF_API wf_status wf_deck_apply(const wf_deck *k, wf_domain *d);
/* wf_deck_read + wf_deck_apply; info may be null. */
WF_API wf_status wf_load_deck(wf_domain *d, const char *path, wf_deck_info *info, char *err,
                              int64_t err_len);
/* Domain_d::CreateFromLSDyna (Domain_d.C:1647-1699): *NODE and *ELEMENT_SOLID
 * cards (fixed columns or comma-separated), nodes numbered in card order,
 * elements with n5..n8 equal to n4 read as tetrahedra. */
WF_API wf_status wf_load_lsdyna(wf_domain *d, const char *path);
/* VTKWriter (VTKWriter.C:238-672): legacy ASCII VTK file of the current
 * state in the reference writer's layout. Points: the part's nodes, then the
 * rigid triangle meshes' nodes; cells: the part's elements, then the
 * triangles. Point data Position, DISP, Acceleration, Velocity, Part_ID,
 * Temp (thermal coupling), ContForce, nod_mass, stress (von Mises of the
 * node-averaged stress), ext_nodes, nod_area, nod_p, SIGMAT (node-averaged
 * stress), EPSR (node-averaged strain rate, FP64 step only); cell data
 * ele_area (written as 0), pressure, pl_strain, DDEVT (strain rate, FP64
 * step only), J, Vol, Rho, Vol_0, sigy. Values with 9 significant digits
 * (coordinates 17). Waits for the domain's stream. */
WF_API wf_status wf_write_vtk(wf_domain *d, const char *path);
/* No counterpart in the reference, whose loop stops to write each output
 * (Solver_explicit.C:1036-1156). Asynchronous output: wf_snapshot queues on
 * the domain's stream a device copy of the fields wf_write_vtk writes, then
 * on a second stream a copy of them into pinned host memory, and returns at
 * once with the slot (0 or 1) that holds them; the steps queued after it run
 * while the copy proceeds. wf_write_snapshot_vtk(d, slot, path) waits for
 * that slot's copy (not for later steps), writes the file exactly as
 * wf_write_vtk would have written it at the snapshot's step (byte for byte),
 * and frees the slot. Two slots: a third wf_snapshot before one of them is
 * written returns WF_ERR_STATE. */
WF_API wf_status wf_snapshot(wf_domain *d, int32_t *slot);
WF_API wf_status wf_write_snapshot_vtk(wf_domain *d, int32_t slot, const char *path);

/* ---- readback (host buffers) -------------------------------------------------- */
WF_API wf_status wf_get_node_field(wf_domain *d, int32_t field, double *out);   /* 3*nn */
WF_API wf_status wf_get_node_scalar(wf_domain *d, int32_t field, double *out);  /* nn */
WF_API wf_status wf_get_elem_scalar(wf_domain *d, int32_t field, double *out);  /* ne */
WF_API wf_status wf_get_elem_tensor(wf_domain *d, int32_t field, double *out);  /* 6*ne */
/* getDispVec / getVelVec over all nodes (Domain_d.h:476-489). */
WF_API wf_status wf_get_disp(wf_domain *d, double *out);
WF_API wf_status wf_get_vel(wf_domain *d, double *out);
WF_API wf_status wf_get_pl_strain(wf_domain *d, double *out);
/* Reaction history since wf_init: *n = steps recorded; copies min(cap, *n). */
WF_API wf_status wf_get_reaction_history(wf_domain *d, double *out, int64_t cap, int64_t *n);
/* Overwrites the nodal state (x, v, prev_a, u; any may be null) from host. */
WF_API wf_status wf_set_node_state(wf_domain *d, const double *x, const double *v,
                                   const double *prev_a, const double *u);

#ifdef __cplusplus
}
#endif
#endif /* WF_H */
