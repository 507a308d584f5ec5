// Internal declarations of the GB300 explicit-step library (not installed).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

#include "wf.h"

namespace wf {

// Per-material constants on the device (Elastic_ / Material_, Material.cuh).
struct MatDev {
  double K, G, sy0, H, cs0, hol_K, hol_m, eps0, eps1, E;
  double jc_B, jc_n, jc_C, jc_eps0, jc_Th;  // Johnson-Cook; jc_Th = 1 - T_h^m (host-computed)
  double jc_m, jc_Tm, jc_Tt;                 // its temperature terms (thermal coupling)
  double k_T, cp_T, exp_T;                   // conductivity, heat capacity, expansion
  // GMT constants, the clamping ranges of strain, strain rate and temperature,
  // and the element temperature without thermal coupling
  double g_C1, g_C2, g_n1, g_n2, g_m1, g_m2, g_I1, g_I2;
  double g_emin, g_emax, g_rmin, g_rmax, g_Tmin, g_Tmax, g_T;
  int32_t model;
  int32_t pad;
};

// FP32 material constants of the mixed kernels.
struct MatF {
  // jc_Th: 1 - T_h^m of Johnson-Cook, or the GMT temperature (uniform; the
  // thermal step takes both from the element's node temperatures instead)
  float K, G, sy0, H, cs0, rho, hol_K, hol_m, eps0, eps1;
  float jc_B, jc_n, jc_C, jc_eps0, jc_Th, E;
  float jc_m, jc_Tm, jc_Tt, k_T, cp_T, exp_T;
  // GMT: the constants (thermal step), the ranges, and A = C1 exp(C2 T),
  // n = n1 T + n2, I = I1 T + I2, q = m1 T + m2 at the uniform temperature
  float g_C1, g_C2, g_n1, g_n2, g_m1, g_m2, g_I1, g_I2;
  float g_emin, g_emax, g_rmin, g_rmax, g_Tmin, g_Tmax;
  float g_A, g_n, g_I, g_q;
  int32_t model;
  int32_t pad;
};

// FP32 time-step constants of one specimen of a batched ensemble.
struct SpecF {
  float dt, cu_pred, cu_corr, cv_corr, cv_pred, pad0, pad1, pad2;
};

// Division of 32-bit unsigned values by a divisor fixed at init without a
// divide instruction (Granlund and Montgomery's round-up method):
// q = (t + ((n - t) >> 1)) >> (s - 1) with t = umulhi(m, n), s = ceil(log2 d),
// m = floor(2^32 (2^s - d) / d) + 1; exact for every 32-bit n.
struct FastDiv {
  uint32_t d, m;
  int32_t s;
};
inline FastDiv make_fastdiv(uint32_t d) {
  FastDiv f{d, 0u, 0};
  if (d <= 1) return f;
  int s = 0;
  while ((1ull << s) < d) s++;
  f.m = (uint32_t)((((unsigned long long)1 << 32) * ((1ull << s) - d)) / d + 1);
  f.s = s;
  return f;
}
#ifdef __CUDACC__
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv &f) {
  if (f.d == 1) return n;
  const uint32_t t = __umulhi(f.m, n);
  return (t + ((n - t) >> 1)) >> (f.s - 1);
}

// clamp of the GMT law's strain, strain rate and temperature to their ranges
__device__ __forceinline__ double clamp_range(double v, double lo, double hi) {
  return (v < lo) ? lo : (v > hi) ? hi : v;
}
__device__ __forceinline__ float clamp_range(float v, float lo, float hi) {
  return (v < lo) ? lo : (v > hi) ? hi : v;
}
#endif

// Device-resident scalars advanced by the node kernel of every step.
struct StepState {
  double time;        // Time of the reference loop (start of the current step)
  long long step;     // steps completed since wf_init
  unsigned int done_blocks;  // last-block-done counter of the node kernel
  unsigned int status;       // bit 0: a non-finite internal force was cleared
  long long first_bad_node;  // smallest node id whose force was cleared (LLONG_MAX: none)
  double eint;               // accumulated internal energy (energy history)
  unsigned int energy_blocks;  // last-block-done counter of the energy kernel
  unsigned int pad;
};

// Node flags (uint8 per node).
enum : uint8_t { NF_REACTION = 1, NF_CONTACT = 2 };

// Kernel parameters shared by both precisions. Node arrays are SoA with
// component stride np (padded node count); element arrays are SoA with
// component stride ne unless noted.
struct StepParams {
  int64_t nn, ne, np;
  int32_t npe;
  int32_t mass_mode;
  int32_t press_alg;
  int32_t react_dim;
  int32_t contact;
  int32_t stab_on;
  int32_t av_on;
  int32_t hg_on;
  double hg_coef;
  double stab[10];
  double av[2];
  double plheat_frac;     // plastic work fraction turned into heat (m_plheatfraction)
  double max_edot;        // strain-rate cap of the rate-dependent tangents (m_max_edot)
  // Chung-Hulbert constants (Solver_explicit.C:193-197), host-computed
  double alpha, beta, gamma, fcorr;  // fcorr = 1 / (1 - alpha)
  double dt;
  // contact plane
  double c_z0, c_vz, c_k, c_mu;
  // mesh
  const int32_t *elnod;   // [npe][ne]
  const int32_t *off;     // [nn + 1]
  const int32_t *slot;    // [total]: e * npe + local node
  const uint32_t *bc;     // [nn]: bits 0..2 constrained dofs, bits 3.. value set
  const double *bcval;    // [nsets][3]
  const float *bcvalf;    // [nsets][3] the same values rounded to FP32 (mixed kernels)
  const uint8_t *nflag;   // [nn]
  const MatDev *mats;
  const int32_t *emat;    // [ne] or null
  int32_t mat_general;    // 1 when a material is not bilinear (mixed kernels' general law)
  double k0;              // bulk modulus of material 0 (pressure algorithm 1)
  // FP32 constants of the mixed kernels (host-rounded once)
  float f_dt, f_alpha, f_fcorr;
  float f_cu_pred;        // (0.5 - beta) * dt
  float f_cu_corr;        // beta * dt * dt
  float f_cv_corr;        // gamma * dt
  float f_cv_pred;        // (1 - gamma) * dt
  float f_hg_coef, f_c_k, f_c_mu;
  float f_av0, f_av1;               // artificial viscosity coefficients (mixed)
  float f_plheat, f_max_edot;       // plheat_frac, max_edot (mixed)
  const struct MatF *matf;
  // batched ensemble (all null / zero for a single domain)
  int32_t nspec;
  const uint16_t *espec;  // [ne] specimen of each element
  const uint16_t *nspec_of;  // [nn] specimen of each node
  const double *spec_dt;  // [nspec]
  const SpecF *specf;     // [nspec]
  double *rnode;          // [nn] reaction contribution of each reaction node
  const int32_t *rlist;   // reaction nodes grouped by specimen
  const int32_t *rl_off;  // [nspec + 1]
  double *hist_spec;      // [hist_cap][nspec]
  // reduction scratch
  double *partials;       // [grid of the node kernel]
  double *hist;           // [hist_cap]
  int64_t hist_cap;
  // rigid triangle-mesh contact (bodies concatenated; velocity per die node)
  int32_t tri_on;
  int32_t tri_nn, tri_ne;
  double *tri_x;            // [3 tri_nn] node positions, moved every step
  const double *tri_v;      // [3 tri_nn] velocity before the start-up ramp
  double *tri_nrm;          // [3 tri_ne] unit normals
  double *tri_pp;           // [tri_ne] plane coefficients
  const int32_t *tri_el;    // [3 tri_ne]
  const int32_t *tri_mid;   // [tri_ne] rigid-body index; body 0 feeds the reaction
  const double *node_area;  // [nn] external-surface area share of each node
  const double *nodlen;     // [nn] mean element length at each node
  double tri_mu_s, tri_mu_d, tri_pf, tri_E0, end_t;
  // FP32 copies for the mixed-precision contact, relative to tri_ref
  float *tri_xf;            // [3 tri_nn]
  float *tri_nf;            // [3 tri_ne]
  float *tri_ppf;           // [tri_ne] n . (p2 - tri_ref)
  double tri_ref[3];
  int32_t sms;              // multiprocessors of the device (launch shapes)
  float f_cp0;              // FP32 heat capacity of material 0 (mixed thermal)
  // thermal coupling (Domain_d::ThermalCalcs), FP64 step
  int32_t thermal;
  double cp0;               // heat capacity of material 0 (die heat term)
  double tri_hc, tri_Tdie;  // die heat transfer coefficient and temperature
  // energy history (Domain_d::computeEnergies after every step), when on
  int32_t energy_on;
  double *epart;          // [2 * grid of the energy kernel]
  double *ekin_hist, *eint_hist;  // [hist_cap]
  StepState *st;
  // box mesh of bx x by x bz hexahedra in the AddBoxLength numbering (box = 1,
  // checked at init): the mixed per-phase kernels compute element corners and
  // node lists from the indices instead of loading elnod / off / slot
  int32_t box, bx, by, bz;
  FastDiv fd_ex, fd_exy;  // bx, bx by: element index -> (i, j, k)
  FastDiv fd_nx, fd_nxy;  // bx + 1, (bx + 1)(by + 1): node index -> (i, j, k)
};

// FP64 state (all doubles).
struct Fp64State {
  double *x, *v, *vp, *pa, *u, *fi, *cf, *ut;   // [3][np]
  double *mass, *voln, *jr, *s0;                 // [np]
  double *vol, *vol0, *rho, *p, *pls, *sy, *detJ;  // [ne]
  double *tau, *sig, *eps, *sr, *rr;             // [6][ne]
  double *fe, *fhg;                              // [ne][npe][3]
  // thermal coupling: nodal temperature, die heat per node (kept after the
  // contact ends), and the element-node temperature rates of the step in two
  // buffers [2][ne][npe] chosen by step parity (the thermal expansion of a
  // step reads the previous step's)
  double *T, *qc, *dte;
};

// Mixed state. Positions are compensated float pairs (hi + lo, ~48-bit
// significand) so neither the element nor the node kernels issue FP64
// instructions; displacements are x - x0, formed in FP64 on export.
// Everything else is FP32.
struct MixState {
  float2 *xh;                     // [3][np] (hi, lo)
  float *v, *vp, *pa;             // [3][np]
  float *cf, *ut;                 // [3][np], [3][np] contact force / slip
  float *cfn;                     // [np] reaction share of the step (triangle-mesh contact)
  float *mass, *jr;               // [np]
  float2 *nc;                     // [np] (1 / sum of initial volumes, mean density)
  float *pls;                     // [ne]
  float *tau;                     // [6][ne]
  float *fe;                      // [ne][npe][3] element force minus hourglass force
  double *x0;                     // [3][np] initial positions (export only)
  float *edot;                    // [ne] sigma . str_rate * vol (energy history only)
  // thermal coupling: temperature as a compensated pair, die heat per node,
  // element-node temperature rates [2][ne][npe] chosen by step parity
  float2 *T;
  float *qc, *dte;
};

// Element tiles of the fused element + assembly step (mixed hexahedra). The
// elements are binned by centroid into cubes of about 8 element sizes; each
// bin is split into tiles of at most kTileElems elements in ascending element
// order. A tile's nodes are staged in shared memory; a node is "interior" to
// a tile when every element that holds it is in that tile, "shared" when it
// is interior to no tile.
constexpr int kTileElems = 512;    // elements per tile, one thread each
constexpr int kTileNodes = 1024;   // distinct nodes per tile at most
constexpr int kTileBinMax = 4096;  // elements per bin at most
constexpr int kSharedThreads = 256;  // block size of the shared-node kernel
struct TileParams {
  int32_t ntiles;
  int32_t nshared;
  const int32_t *eoff;     // [ntiles + 1] tile boundaries in elems
  const int32_t *elems;    // [ne] element ids, tile by tile, ascending within a tile
  const uint16_t *lel;     // [8][ne] tile-local node index of corner a of elems[i]
  const int32_t *ncount;   // [ntiles] distinct nodes of each tile
  const int32_t *nodes;    // [ntiles][kTileNodes] node ids ascending; bit 31: shared
  const int32_t *shared;   // [nshared] the shared nodes, ascending
  double *partials;        // [ntiles + blocks of the shared-node kernel] reaction partials
  int64_t tile_nodes;      // sum of ncount (host-side statistic)
  int64_t shared_slots;    // node-list entries of the shared nodes (host-side statistic)
};

// Column sweep of box meshes (mix_sweep): the node grid cut into ncx x ncy
// columns, one block each. The arrays a block reads for its neighbours'
// elements come in pairs: a step reads MixState's buffer (xh, vp, tau, pls)
// and writes the other one, given here; the host swaps the two after each
// step.
struct SweepParams {
  int32_t ncx = 0, ncy = 0;
  int32_t cy = 0;                 // node rows per column (the kernel variant)
  float2 *xh_o = nullptr;         // [3][np]
  float *vp_o = nullptr;          // [3][np]
  float *tau_o = nullptr;         // [6][ne]
  float *pls_o = nullptr;         // [ne]
  double *partials = nullptr;     // [ncx * ncy] reaction per column
};

// Dataflow step of box meshes (mix_flow): one persistent launch per step. Its
// work is cut into tiles of elements or nodes of one layer or plane; items
// (kind, layer) are the four phases of one layer: 0 geometry of element layer
// l, 1 nodal phase of node plane l, 2 element phase of layer l, 3 node update
// of plane l. Stage s holds the items G(s), N1(s - off[1]), E(s - off[2]),
// N2(s - off[3]) that exist, in that order; blocks take tiles in ticket order
// (stages in order, the tiles of an item consecutively) and wait for the
// items a tile reads through per-item done counters. Two counter sets
// alternate between steps: a launch counts in cnt and zeroes cnt_next.
constexpr int kFlowKinds = 4;
constexpr int kFlowMaxLayers = 4096;   // element layers the stage table holds at most
struct FlowParams {
  const int *stage_first = nullptr;  // [nstages + 1] first ticket of each stage
  int32_t nstages = 0;
  int32_t off[kFlowKinds] = {0, 1, 3, 4};   // stage offset of each kind
  int32_t tsize[kFlowKinds] = {0, 0, 0, 0};   // elements or nodes per tile
  int32_t ntiles[kFlowKinds] = {0, 0, 0, 0};  // tiles per item
  int32_t total = 0;              // tickets (tiles) per step
  int32_t bz1 = 0;                // layers + 1: counter stride per kind
  int32_t grid = 0;               // blocks of the launch
  int32_t ncnt = 0;               // counters per set: 1 + kFlowKinds * bz1
  unsigned *cnt = nullptr;        // [0] next ticket, [1 + kind * bz1 + l] tiles done of an item
  unsigned *cnt_next = nullptr;   // the next step's set
  double *partials = nullptr;     // [bz1 * ntiles[3]] reaction per node-update tile
  int32_t split = 0;              // 1: the geometry and nodal phases run as their own
                                  // kernels before the launch (no G, N1 tiles)
};

// Host-side view of one state for the legacy VTK writer (write_vtk_text,
// wf_deck.cpp). Node vectors are AoS [nn][3]; element tensors hold 6 values
// per element (Voigt xx yy zz xy yz xz), AoS [ne][6] or SoA [6][ne]. Null
// optional arrays are written as zeros (or left out: T, sr).
struct VtkView {
  int64_t nn = 0, ne = 0;
  int32_t npe = 0;
  const double *x = nullptr, *u = nullptr, *v = nullptr, *a = nullptr, *cf = nullptr;
  const double *mass = nullptr, *T = nullptr;         // T: thermal coupling only
  const double *p = nullptr, *pl = nullptr, *vol = nullptr, *vol0 = nullptr;
  const double *rho = nullptr, *sy = nullptr;
  const double *sig = nullptr, *sr = nullptr;         // sr: FP64 step only
  bool sig_soa = false, sr_soa = false;
  const int32_t *elnod = nullptr;                     // [ne][npe]
  const uint8_t *ext = nullptr;                       // external-surface flags (contact)
  const double *area = nullptr;                       // external-surface area shares
  int64_t tri_nn = 0, tri_ne = 0;                     // rigid triangle meshes (contact)
  const double *tri_x = nullptr;                      // [tri_nn][3]
  const int32_t *tri_el = nullptr;                    // [tri_ne][3]
  double T_die = 0.0;
};
// Writes the view as the reference's legacy VTK writer lays it out
// (VTKWriter.C:238-664: same blocks, names and order); false on an I/O error.
bool write_vtk_text(const char *path, const VtkView &v);

// Records `msg` as the domain's last error and returns s (wf_api.cu).
wf_status domain_fail(wf_domain *d, wf_status s, const std::string &msg);

// Structured box mesh of Domain_d::AddBoxLength (host; wf_api.cu).
bool box_mesh(const double V[3], const double L[3], double r, bool tritetra,
              std::vector<double> &x, std::vector<int32_t> &elnod, std::string &err);

// ---- FP64 launchers (wf_fp64.cu) ------------------------------------------
void fp64_geometry(const StepParams &P, const Fp64State &S, cudaStream_t st, bool store_detj);
void fp64_nodal(const StepParams &P, const Fp64State &S, cudaStream_t st, int init_mode);
void fp64_elements(const StepParams &P, const Fp64State &S, cudaStream_t st);
void fp64_nodes(const StepParams &P, const Fp64State &S, cudaStream_t st, int node_grid);
void fp64_predict(const StepParams &P, const Fp64State &S, cudaStream_t st);
void fp64_density(const StepParams &P, const Fp64State &S, const double *rho0, cudaStream_t st);
int fp64_node_grid(int64_t nn, int sms);

// Launch shape of a tunable kernel: block size and items per thread
// (grid-stride loop; grid = ceil(n / (bs * ept))).
struct LaunchCfg {
  int bs = 128;
  int ept = 1;
};

// ---- Mixed launchers (wf_mixed.cu) ----------------------------------------
// The mixed state from the preamble's positions and velocities: initial
// element volumes (mixed geometry kernel, into vol), node constants, masses
// and the FP64 copies of the initial volumes, masses and densities.
void mix_init(const StepParams &P, const MixState &M, const Fp64State &S, float *vol,
              const double *rho0, cudaStream_t st);
void mix_geometry(const StepParams &P, const MixState &M, float *vol, cudaStream_t st,
                  LaunchCfg c);
void mix_nodal(const StepParams &P, const MixState &M, const float *vol, cudaStream_t st,
               LaunchCfg c);
void mix_elements(const StepParams &P, const MixState &M, const float *vol, cudaStream_t st,
                  LaunchCfg c);
void mix_nodes(const StepParams &P, const MixState &M, cudaStream_t st, int node_grid);
void mix_predict(const StepParams &P, const MixState &M, cudaStream_t st);
// Tiled step of hexahedra (replaces mix_elements + mix_nodes): the element
// phase and interior-node assembly and update per tile, then the shared nodes.
void mix_tile(const StepParams &P, const MixState &M, const TileParams &T, cudaStream_t st);
void mix_shared(const StepParams &P, const MixState &M, const TileParams &T, cudaStream_t st);
int mix_shared_grid(const TileParams &T);
// Column sweep of a box mesh (replaces mix_elements + mix_nodes): reads M's
// positions, predicted velocities, tau and eps_p and writes W's. The column
// shape: sweep_columns fills W.ncx, W.ncy, W.cy for the box and returns the
// number of blocks; sweep_fits tells whether the kernel can launch here.
int sweep_columns(const StepParams &P, SweepParams &W);
bool sweep_fits(const StepParams &P, const SweepParams &W);
void mix_sweep(const StepParams &P, const MixState &M, const SweepParams &W, cudaStream_t st);
// Dataflow step of a box mesh (replaces the four phase kernels): flow_stages
// builds the stage table on the host and fills F's sizes, mix_flow launches
// one step. flow_grid: the persistent grid (0: the
// kernel cannot launch here).
int flow_grid(const StepParams &P);
void flow_stages(const StepParams &P, int tile, int lag, bool split, std::vector<int> &first,
                 FlowParams &F);
void mix_flow(const StepParams &P, const MixState &M, float *vol, const FlowParams &F,
              cudaStream_t st);
// Whole runs of steps in one launch of one cluster of `blocks` blocks of `bs`
// threads (64, 128 or 256), for small meshes; mix_cluster_fits returns how
// many such clusters can be resident (0: the shape cannot launch).
int mix_cluster_fits(const StepParams &P, const MixState &M, float *vol, int blocks, int bs);
// part: [nsteps][blocks] staging for the reaction's block partials.
cudaError_t mix_cluster_run(const StepParams &P, const MixState &M, float *vol, double *part,
                            int64_t nsteps, int blocks, int bs, cudaStream_t st);
// The mixed state's displacements (or positions) as AoS [nn][3] doubles, as
// the export forms them, without exporting the other fields.
void mix_node_aos(const StepParams &P, const MixState &M, bool displacement, double *out,
                  cudaStream_t st);
void mix_export(const StepParams &P, const MixState &M, const Fp64State &S, const float *vol,
                cudaStream_t st);
int mix_node_grid(int64_t nn);

// ---- reductions (wf_reduce.cu) ---------------------------------------------
// Per-specimen reaction sums of the step just completed (batched ensemble).
void spec_reaction(const StepParams &P, cudaStream_t st);
// Kinetic energy and internal-energy increment of the step just completed,
// appended to the energy history (fixed-order reduction).
int energy_grid(const StepParams &P);
void energy_fp64(const StepParams &P, const Fp64State &S, cudaStream_t st);
void energy_mixed(const StepParams &P, const MixState &M, cudaStream_t st);
// Minimum element edge length over the mesh (exact: min is order-free).
void min_edge_length(const int32_t *elnod, const double *x, int64_t np, int64_t ne, int npe,
                     double *out_dev, cudaStream_t st);
// Box meshes (AddBoxLength numbering, nx x ny x nz elements): the same
// minimum over the grid edges, each edge once.
void min_edge_length_box(const double *x, int64_t np, int32_t bx, int32_t by, int32_t bz,
                         double *out_dev, cudaStream_t st);

#ifdef __CUDACC__
// ---- box meshes (AddBoxLength numbering, P.box) -----------------------------------
// The elements around node n in list order (ascending, the node lists'
// order) and n's corner in each; el[q] = -1 where the box has none. q = dk * 4
// + dj * 2 + di for the element (i - 1 + di, j - 1 + dj, k - 1 + dk); the
// corner at (1 - di, 1 - dj, 1 - dk) of the element is 4 z + (x ^ 3 y).
__device__ __forceinline__ void box_node_list(const StepParams &P, int64_t n, int32_t (&el)[8],
                                              int32_t (&cor)[8]) {
  const uint32_t un = (uint32_t)n;
  const int32_t k = (int32_t)fdiv(un, P.fd_nxy);
  const uint32_t r = un - (uint32_t)k * P.fd_nxy.d;
  const int32_t j = (int32_t)fdiv(r, P.fd_nx);
  const int32_t i = (int32_t)(r - (uint32_t)j * P.fd_nx.d);
#pragma unroll
  for (int dk = 0; dk < 2; dk++)
#pragma unroll
    for (int dj = 0; dj < 2; dj++)
#pragma unroll
      for (int di = 0; di < 2; di++) {
        const int32_t ii = i - 1 + di, jj = j - 1 + dj, kk = k - 1 + dk;
        const bool ok = ii >= 0 && ii < P.bx && jj >= 0 && jj < P.by && kk >= 0 && kk < P.bz;
        const int q = dk * 4 + dj * 2 + di;
        el[q] = ok ? ii + P.bx * (jj + P.by * kk) : -1;
        cor[q] = 4 * (1 - dk) + ((1 - di) ^ (3 * (1 - dj)));
      }
}
#endif

// ---- device setup (wf_setup.cu) ------------------------------------------------
// Node -> element lists from the AoS connectivity on the device: SoA element
// nodes, CSR offsets [nn + 1] and slots e * npe + a, ascending within each
// node's list (the host build's order). scratch holds
// connectivity_scratch_ints(nn) ints. With off null only the SoA element nodes
// are built (box meshes whose kernels compute the lists), with el_soa null
// only the lists.
int64_t connectivity_scratch_ints(int64_t nn);
// dst[idx[i]] = val[i] and dst[idx[i]] |= bit for i < n (distinct indices).
void scatter_u32(uint32_t *dst, const int32_t *idx, const uint32_t *val, int64_t n,
                 cudaStream_t st);
void or_flags(uint8_t *dst, const int32_t *idx, uint8_t bit, int64_t n, cudaStream_t st);
// Whether every entry of el[0, n) names a node in [0, nn) (*bad = 0), on the
// device; flag: one device int of scratch. Synchronises st.
cudaError_t check_connectivity(const int32_t *el, int64_t n, int64_t nn, int32_t *flag,
                               cudaStream_t st, int *bad);
cudaError_t build_connectivity(const int32_t *el_aos, int64_t ne, int npe, int64_t nn,
                               int32_t *el_soa, int32_t *off, int32_t *slot, int32_t *scratch,
                               cudaStream_t st);
// Element tiles (TileParams) of a hexahedral mesh from the SoA connectivity,
// the SoA FP64 coordinates and the node-list offsets, built on the device.
// bbox = {min x, min y, min z, max x, max y, max z}. Device arrays that stay
// with the domain come from `keep` (freed with it); temporaries are freed
// before returning. Returns cudaSuccess and sets `why` (non-empty) when the
// mesh does not tile (a bin or tile over its limits, or two elements of a
// tile holding one node at the same corner).
using DeviceAlloc = cudaError_t (*)(void *ctx, void **p, size_t bytes);
cudaError_t build_tiles(const int32_t *el_soa, const double *x_soa, int64_t np, int64_t ne,
                        int64_t nn, const int32_t *off, const double bbox[6], int shared_threads,
                        DeviceAlloc keep, void *keep_ctx, cudaStream_t st, TileParams &T,
                        std::string &why);

// Whether the SoA connectivity is the AddBoxLength numbering of nx x ny x nz
// hexahedra (*is_box = 1): a device check of every element.
cudaError_t check_box(const int32_t *el_soa, int64_t ne, int64_t nn, int nx, int ny, int nz,
                      cudaStream_t st, int *is_box);

// AoS [nn][3] -> SoA [3][np], zero padded
void coords_soa(const double *x_aos, int64_t nn, int64_t np, double *out, cudaStream_t st);
// SoA [3][np] -> AoS [nn][3]
void coords_aos(const double *soa, int64_t nn, int64_t np, double *out, cudaStream_t st);
void fill_values(double *p, double v, int64_t n, cudaStream_t st);
// sigma_y = sy0 of each element's material
void initial_yield(const StepParams &P, double *sy, cudaStream_t st);
// v after the preamble's BC loop: zero but the z velocity BCs
void initial_velocity(const StepParams &P, double *v, cudaStream_t st);

}  // namespace wf
