// Host side of the C ABI (include/wf.h): domain lifecycle, mesh and
// node->element lists, BC tables, device buffers, the step loop (captured in
// CUDA graphs) and readback.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cfloat>
#include <cstdarg>
#include <cstddef>
#include <climits>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <atomic>
#include <tuple>
#include <utility>
#include <vector>

#include "wf_adjoint.cuh"
#include "wf_internal.cuh"


namespace wf {

// Structured box of Domain_d::AddBoxLength (Domain_d.C:1136-1504): nel =
// floor(L / 2r) cells per axis, nodes x-fastest with coordinates formed by
// repeated addition of 2r (:1215-1235), hexahedra in the same order
// (:1316-1345) or six tetrahedra per cell (:1383-1388).
bool box_mesh(const double V[3], const double L[3], double r, bool tritetra,
              std::vector<double> &x, std::vector<int32_t> &elnod, std::string &err) {
  int nel[3];
  for (int k = 0; k < 3; k++) nel[k] = (int)(L[k] / (2.0 * r));
  if (nel[0] <= 0 || nel[1] <= 0 || nel[2] <= 0) {
    err = "box smaller than one element";
    return false;
  }
  const int npe = tritetra ? 4 : 8;
  const int64_t nn = (int64_t)(nel[0] + 1) * (nel[1] + 1) * (nel[2] + 1);
  const int64_t ne = (int64_t)nel[0] * nel[1] * nel[2] * (tritetra ? 6 : 1);
  if (ne * npe >= (int64_t)INT32_MAX) {
    err = "mesh too large";
    return false;
  }
  x.assign(3 * nn, 0.0);
  int64_t p = 0;
  double Xz = V[2];
  for (int k = 0; k <= nel[2]; k++) {
    double Xy = V[1];
    for (int j = 0; j <= nel[1]; j++) {
      double Xx = V[0];
      for (int i = 0; i <= nel[0]; i++) {
        x[3 * p] = Xx;
        x[3 * p + 1] = Xy;
        x[3 * p + 2] = Xz;
        p++;
        Xx = Xx + 2.0 * r;
      }
      Xy = Xy + 2.0 * r;
    }
    Xz = Xz + 2 * r;
  }
  elnod.assign(ne * npe, 0);
  static const int T[6][4] = {{0, 1, 3, 5}, {1, 2, 3, 5}, {0, 5, 3, 4},
                              {4, 5, 3, 7}, {5, 6, 3, 7}, {5, 2, 3, 6}};
  const int64_t nnodz = (int64_t)(nel[0] + 1) * (nel[1] + 1);
  int64_t ei = 0;
  for (int ez = 0; ez < nel[2]; ez++)
    for (int ey = 0; ey < nel[1]; ey++)
      for (int ex = 0; ex < nel[0]; ex++) {
        const int64_t nb1 = nnodz * ez + (int64_t)(nel[0] + 1) * ey + ex;
        const int64_t nb2 = nnodz * ez + (int64_t)(nel[0] + 1) * (ey + 1) + ex;
        const int32_t h[8] = {(int32_t)nb1, (int32_t)(nb1 + 1), (int32_t)(nb2 + 1),
                              (int32_t)nb2, (int32_t)(nb1 + nnodz), (int32_t)(nb1 + nnodz + 1),
                              (int32_t)(nb2 + nnodz + 1), (int32_t)(nb2 + nnodz)};
        if (!tritetra) {
          for (int a = 0; a < 8; a++) elnod[ei + a] = h[a];
          ei += 8;
        } else {
          for (int t = 0; t < 6; t++) {
            for (int a = 0; a < 4; a++) elnod[ei + a] = h[T[t][a]];
            ei += 4;
          }
        }
      }
  return true;
}

// Allocator whose resize() leaves trivial elements uninitialised: the large
// host copies of the mesh are overwritten right after they are sized.
template <typename T>
struct NoInitAlloc : std::allocator<T> {
  template <typename U>
  struct rebind {
    using other = NoInitAlloc<U>;
  };
  NoInitAlloc() = default;
  template <typename U>
  NoInitAlloc(const NoInitAlloc<U> &) {}
  template <typename U>
  void construct(U *p) noexcept {
    ::new (static_cast<void *>(p)) U;
  }
  template <typename U, typename... Args>
  void construct(U *p, Args &&...args) {
    ::new (static_cast<void *>(p)) U(std::forward<Args>(args)...);
  }
};
template <typename T>
using hvec = std::vector<T, NoInitAlloc<T>>;

}  // namespace wf

using namespace wf;

struct wf_domain {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  // host mesh
  int32_t npe = 0;
  int64_t nn = 0, ne = 0, np = 0;
  // the mesh as set, on the device ([nn][3] coordinates, [ne][npe]
  // connectivity, from the library's pool): uploaded by wf_set_mesh and
  // wf_add_box_length; x and elnod mirror it on the host once a host caller
  // needs them (mesh_host)
  double *mesh_x = nullptr;
  int32_t *mesh_el = nullptr;
  int32_t *mesh_flag = nullptr;   // scratch of the connectivity check
  bool mesh_host = false;
  hvec<double> x;                 // interleaved [3 nn]
  hvec<int32_t> elnod;            // [ne npe]
  // node -> element lists on the host, built when a host caller needs them
  // (wf_get_connectivity, the part's surface search); wf_init builds the
  // device copy itself
  std::vector<int32_t> nodel, nodel_loc, nodel_off, nodel_cnt;
  // materials
  std::vector<wf_material> mats;
  double plheat_frac = 0.9;        // m_plheatfraction (Domain_d.h:271)
  double max_edot = 1.0e6;         // m_max_edot (Domain_d.h:824)
  std::vector<std::array<double, 8>> jc;  // Johnson-Cook B, n, C, eps0_dot, m, T_melt, T_t, T
  // GMT n1, n2, C1, C2, m1, m2, I1, I2, e_min, e_max, er_min, er_max, T_min, T_max, T
  std::vector<std::array<double, 15>> gmt;
  std::vector<std::array<double, 3>> mat_thermal;  // k_T, cp_T, exp_T per material
  bool thermal = false;
  double T0 = 20.0;
  double tri_hc = 0.0, tri_Tdie = 20.0;             // die heat transfer
  std::vector<int32_t> emat;
  double rho_all = 0.0;
  bool rho_set = false;
  // BCs (AddBCVelNode staging)
  std::vector<int64_t> bc_nod[3];
  std::vector<double> bc_val[3];
  bool bcs_allocated = false;
  // options
  double dt = 0.0, end_t = 0.0;
  int precision = WF_FP64;
  double hg = 0.0;
  int press_alg = 0, mass_mode = 0;
  bool energy = false;
  wf_stab stab{};
  double av[2] = {0.0, 0.0};
  std::vector<int32_t> react_nodes;
  int react_dim = 2;
  bool contact = false;
  double c_z0 = 0, c_vz = 0, c_k = 0, c_mu = 0;
  std::vector<int32_t> cand;
  // rigid triangle-mesh contact
  bool tri = false;
  std::vector<double> tri_x;
  std::vector<int32_t> tri_el;
  std::vector<double> tri_v;      // [3 per node] velocity before the start-up ramp
  std::vector<int32_t> tri_mid;   // [per triangle] rigid-body (mesh) index
  int32_t tri_meshes = 0;
  double tri_mu_s = 0.0, tri_mu_d = 0.0, tri_pf = 0.1;
  // device
  bool initialized = false;
  std::vector<void *> allocs;
  void *init_stage = nullptr;     // AoS uploads and scratch of wf_init, freed at its end
  double *readback = nullptr;     // [3 nn] AoS staging of node-field readbacks
  StepParams P{};
  Fp64State S{};
  MixState M{};
  float *mvol = nullptr;          // mixed: element volume scratch
  double *rho0_dev = nullptr;
  int node_grid = 0;
  int64_t hist_cap = 0;
  int64_t host_step = 0;          // steps launched since init
  double host_time = 0.0;         // Time accumulated on the host (mirror)
  bool mix_valid_fp64 = false;    // FP64 export of the mixed state is current
  // step graphs keyed by their number of steps (times 2, plus the sweep's
  // buffer parity at their start): kGraphSteps for long runs and one per
  // remainder length wf_run has met (built on first use, or ahead of time by
  // wf_prepare_run)
  std::map<int64_t, cudaGraphExec_t> graphs;
  // per-phase timing
  bool phase_timing = false;
  std::vector<cudaEvent_t> ev_pool;   // 5 events per timed step
  size_t ev_used = 0;
  double phase_ms[4] = {0, 0, 0, 0};
  int64_t phase_steps = 0;
  int64_t launches = 0;
  int64_t graph_launches = 0;     // step graphs replayed since wf_init
  int64_t h2d_bytes = 0, d2h_bytes = 0;
  // asynchronous output: two snapshot slots, each a device copy of the state
  // fields and a pinned host copy filled on the output stream
  struct Snapshot {
    double *dev = nullptr, *host = nullptr;
    size_t count = 0;
    cudaEvent_t ready = nullptr, done = nullptr;
    int state = 0;                // 0 free, 1 queued or copied, not yet written
  } snap[2];
  cudaStream_t out_stream = nullptr;
  int snap_next = 0;
  std::vector<uint8_t> surf_ext;  // external-surface flags and areas (contact), for the VTK
  std::vector<double> surf_area;
  // pinned copy of the device step state, queued after every wf_run and
  // read by the next wf_sync (the non-finite force check)
  StepState *st_host = nullptr;
  bool st_pending = false;
  // launch shapes of the tunable mixed kernels (geometry, nodal, elements)
  bool autotune = true;
  bool tune_cached = false;       // the last init took its shapes from the process cache
  LaunchCfg cfg[3] = {LaunchCfg{128, 1}, LaunchCfg{256, 1}, LaunchCfg{128, 1}};
  double cfg_ms[3] = {0, 0, 0};
  // step scheduling (mixed): 0 automatic, 1 per-phase kernels, 2 one cluster
  // launch per run, 3 tiled element + assembly kernels, 4 column sweep; the
  // cluster shape is found at init for small meshes, the tiles are built at
  // init for meshes of hexahedra that the tiled kernels cover, the sweep's
  // buffers for box meshes
  int32_t step_mode = 0;
  bool tiled = false;             // tiles built (TileParams T valid)
  bool use_box = true;            // box meshes: connectivity computed in the mixed kernels
  bool half_open = false;         // wf_step_begin called, wf_step_end not yet
  TileParams T{};
  std::string tile_why;           // why the mesh was not tiled
  // column sweep (step mode 4, box meshes): the pairs of buffers of the
  // arrays it reads for neighbouring columns; pair[parity] is the current one
  // (in M), pair[parity ^ 1] the one the next sweep writes (in W)
  bool sweep = false;             // set up at init (W valid)
  int32_t sweep_rows = 8;         // node rows per column (4 or 8), chosen before init
  SweepParams W{};
  std::string sweep_why;          // why the mesh has no column sweep
  int parity = 0;
  float2 *xh_pair[2] = {nullptr, nullptr};
  float *vp_pair[2] = {nullptr, nullptr}, *tau_pair[2] = {nullptr, nullptr};
  float *pls_pair[2] = {nullptr, nullptr};
  // dataflow step (step mode 5, box meshes): its item table and two counter
  // sets, flow_cnt[flow_par] counted by the next step
  bool flow = false;
  FlowParams F{};
  std::string flow_why;
  unsigned *flow_cnt[2] = {nullptr, nullptr};
  int flow_par = 0;
  int32_t flow_tile = 512, flow_lag = 4;
  int cl_blocks = 0, cl_bs = 0;
  double *cl_part = nullptr;      // [kClusterChunk][cl_blocks] reaction partials
  double *edge_min = nullptr;     // the shortest edge (wf_min_edge_length's device result)
  // batched ensemble
  int32_t nspec = 0;
  std::vector<int64_t> spec_eoff, spec_noff;
  std::vector<double> spec_dt;
  // adjoint recording: checkpoints of the forward run and reverse-pass buffers
  std::vector<void *> adj_allocs;
  int64_t adj_steps = 0, adj_every = 0, adj_first = 0;
  bool adj_store_all = false;     // every step stashed in the forward, no recompute
  int64_t adj_nck = 0;
  double *ck_node = nullptr;      // [nck][4][3 np]: x, v, prev_a, u
  double *ck_elem = nullptr;      // [nck][13][ne]: tau, eps, eps_p
  StepState *ck_st = nullptr;     // [nck]
  AdjArgs A{};
  double *adj_seed = nullptr;     // [adj_steps]
  bool adj_buffers = false;
};

namespace {

// Destroys the domain's step graphs (they hold launch parameters by value).
void drop_graphs(wf_domain *d) {
  for (auto &g : d->graphs) cudaGraphExecDestroy(g.second);
  d->graphs.clear();
}

wf_status fail(wf_domain *d, wf_status s, const char *fmt, ...) {
  if (d) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    d->err = buf;
  }
  return s;
}

#define CUDA_TRY(call)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(d, e_ == cudaErrorMemoryAllocation ? WF_ERR_NOMEM : WF_ERR_CUDA,       \
                  "%s: %s", #call, cudaGetErrorString(e_));                              \
  } while (0)

// Device allocation freed with the domain, left uninitialised (the caller
// writes every element).
// Device memory of the domains comes from one stream-ordered pool per device
// that keeps what domains give back (release threshold: all of it): a domain
// set up after another of its size takes memory that is already mapped
// instead of mapping new pages. Allocations and frees are ordered on the
// domain's stream.
cudaError_t device_pool(int dev, cudaMemPool_t *out) {
  static std::mutex mu;
  static std::map<int, cudaMemPool_t> pools;
  std::lock_guard<std::mutex> lock(mu);
  auto it = pools.find(dev);
  if (it != pools.end()) {
    *out = it->second;
    return cudaSuccess;
  }
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaMemPool_t pool = nullptr;
  cudaError_t e = cudaMemPoolCreate(&pool, &props);
  if (e != cudaSuccess) return e;
  uint64_t keep = UINT64_MAX;
  e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  if (e != cudaSuccess) return e;
  pools[dev] = pool;
  *out = pool;
  return cudaSuccess;
}

cudaError_t pool_alloc(wf_domain *d, void **q, size_t bytes) {
  cudaMemPool_t pool = nullptr;
  cudaError_t e = device_pool(d->device, &pool);
  if (e != cudaSuccess) return e;
  return cudaMallocFromPoolAsync(q, std::max<size_t>(bytes, 1), pool, d->stream);
}

// The device copy of the mesh and its host mirror (defined with the mesh
// entry points).
void free_mesh_dev(wf_domain *d);
wf_status host_mesh(const wf_domain *cd);

template <typename T>
cudaError_t dalloc_raw(wf_domain *d, T **p, size_t count) {
  void *q = nullptr;
  cudaError_t e = pool_alloc(d, &q, std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess) return e;
  d->allocs.push_back(q);
  *p = static_cast<T *>(q);
  return cudaSuccess;
}

template <typename T>
cudaError_t dalloc(wf_domain *d, T **p, size_t count) {
  void *q = nullptr;
  cudaError_t e = pool_alloc(d, &q, std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess) return e;
  d->allocs.push_back(q);
  *p = static_cast<T *>(q);
  return cudaMemsetAsync(q, 0, std::max<size_t>(count, 1) * sizeof(T), d->stream);
}

void free_adjoint(wf_domain *d) {
  for (void *p : d->adj_allocs) cudaFree(p);
  d->adj_allocs.clear();
  d->adj_steps = d->adj_every = d->adj_nck = 0;
  d->adj_store_all = false;
  d->ck_node = d->ck_elem = nullptr;
  d->ck_st = nullptr;
  d->A = AdjArgs{};
  d->adj_seed = nullptr;
  d->adj_buffers = false;
}

void free_device(wf_domain *d) {
  free_adjoint(d);
  drop_graphs(d);
  // nothing of the domain's may still run when its memory goes back
  if (d->stream) cudaStreamSynchronize(d->stream);
  if (d->out_stream) cudaStreamSynchronize(d->out_stream);
  for (void *p : d->allocs) cudaFreeAsync(p, d->stream);
  d->allocs.clear();
  if (d->st_host) cudaFreeHost(d->st_host);
  d->st_host = nullptr;
  d->st_pending = false;
  for (auto &sn : d->snap) {
    if (sn.dev) cudaFree(sn.dev);
    if (sn.host) cudaFreeHost(sn.host);
    if (sn.ready) cudaEventDestroy(sn.ready);
    if (sn.done) cudaEventDestroy(sn.done);
    sn = wf_domain::Snapshot{};
  }
  d->snap_next = 0;
  d->surf_ext.clear();
  d->surf_area.clear();
  if (d->init_stage) cudaFreeAsync(d->init_stage, d->stream);
  d->init_stage = nullptr;
  for (cudaEvent_t ev : d->ev_pool) cudaEventDestroy(ev);
  d->ev_pool.clear();
  d->ev_used = 0;
  d->S = Fp64State{};
  d->M = MixState{};
  d->readback = nullptr;
  d->mvol = nullptr;
  d->tiled = false;
  d->T = TileParams{};
  d->edge_min = nullptr;
  d->sweep = d->flow = false;
  d->W = SweepParams{};
  d->F = FlowParams{};
  for (int k = 0; k < 2; k++) {
    d->xh_pair[k] = nullptr;
    d->vp_pair[k] = d->tau_pair[k] = d->pls_pair[k] = nullptr;
    d->flow_cnt[k] = nullptr;
  }
  d->initialized = false;
}

// Host threads for the setup loops over large meshes: f(begin, end) on
// contiguous chunks of [0, n); small ranges run inline.
template <typename F>
void host_parallel(int64_t n, F f) {
  constexpr int64_t kMinChunk = int64_t(1) << 20;
  int64_t T = (int64_t)std::min(32u, std::max(1u, std::thread::hardware_concurrency()));
  T = std::min<int64_t>(T, (n + kMinChunk - 1) / kMinChunk);
  if (T <= 1) {
    f((int64_t)0, n);
    return;
  }
  std::vector<std::thread> th;
  for (int64_t t = 0; t < T; t++) th.emplace_back(f, n * t / T, n * (t + 1) / T);
  for (std::thread &x : th) x.join();
}

// Node -> element lists, element-ascending per node (setNodElem,
// Domain_d.C:1508-1611; tail of AddBoxLength, :1436-1481), built by host
// threads over contiguous element chunks: (1) each chunk counts its entries
// per node (8-bit counters, one array per chunk); (2) per node, the chunks'
// counts become their starting ranks (chunk order = element order) and the
// totals give the offsets; (3) each chunk places its entries in element order
// from those ranks. Every list comes out element-ascending, exactly as one
// thread would build it; a node with 255 or more entries in one chunk falls
// back to the single-threaded build.
void build_nodel_serial(wf_domain *d) {
  const int64_t nn = d->nn, ent = d->ne * d->npe;
  const int32_t *el = d->elnod.data();
  d->nodel_cnt.assign(nn, 0);
  for (int64_t i = 0; i < ent; i++) d->nodel_cnt[el[i]]++;
  d->nodel_off.assign(nn + 1, 0);
  int64_t tot = 0;
  for (int64_t n = 0; n < nn; n++) {
    d->nodel_off[n] = (int32_t)tot;
    tot += d->nodel_cnt[n];
  }
  d->nodel_off[nn] = (int32_t)tot;
  d->nodel.assign(tot, 0);
  d->nodel_loc.assign(tot, 0);
  std::vector<int32_t> fill(nn, 0);
  for (int64_t i = 0; i < ent; i++) {
    const int32_t n = el[i];
    const int64_t k = d->nodel_off[n] + fill[n]++;
    d->nodel[k] = (int32_t)(i / d->npe);
    d->nodel_loc[k] = (int32_t)(i % d->npe);
  }
}

void build_nodel(wf_domain *d) {
  const int64_t nn = d->nn, ne = d->ne, ent = ne * d->npe;
  const int npe = d->npe;
  const int32_t *el = d->elnod.data();
  const int64_t T = std::min<int64_t>(
      std::min(32u, std::max(1u, std::thread::hardware_concurrency())),
      std::max<int64_t>(1, ent / (int64_t(1) << 20)));
  if (T <= 1) {
    build_nodel_serial(d);
    return;
  }
  std::vector<std::vector<uint8_t>> rank(T);
  std::atomic<bool> overflow{false};
  auto chunk = [&](int64_t t, int64_t &e0, int64_t &e1) {
    e0 = ne * t / T;
    e1 = ne * (t + 1) / T;
  };
  {  // (1) per-chunk counts
    std::vector<std::thread> th;
    for (int64_t t = 0; t < T; t++)
      th.emplace_back([&, t]() {
        rank[t].assign(nn, 0);
        uint8_t *c = rank[t].data();
        int64_t e0, e1;
        chunk(t, e0, e1);
        for (int64_t i = e0 * npe; i < e1 * npe; i++)
          if (++c[el[i]] == 255) overflow = true;
      });
    for (std::thread &x : th) x.join();
  }
  if (overflow) {
    build_nodel_serial(d);
    return;
  }
  // (2) per node: totals, and each chunk's starting rank within the node's list
  d->nodel_cnt.assign(nn, 0);
  int32_t *cnt = d->nodel_cnt.data();
  host_parallel(nn, [&](int64_t n0, int64_t n1) {
    for (int64_t n = n0; n < n1; n++) {
      int32_t r = 0;
      for (int64_t t = 0; t < T; t++) {
        const uint8_t c = rank[t][n];
        rank[t][n] = (uint8_t)r;
        r += c;
      }
      cnt[n] = r;
    }
  });
  bool big = false;
  for (int64_t n = 0; n < nn && !big; n++) big = cnt[n] > 255;
  if (big) {
    build_nodel_serial(d);
    return;
  }
  d->nodel_off.assign(nn + 1, 0);
  int64_t tot = 0;
  for (int64_t n = 0; n < nn; n++) {
    d->nodel_off[n] = (int32_t)tot;
    tot += cnt[n];
  }
  d->nodel_off[nn] = (int32_t)tot;
  d->nodel.assign(tot, 0);
  d->nodel_loc.assign(tot, 0);
  const int32_t *off = d->nodel_off.data();
  int32_t *lst = d->nodel.data(), *loc = d->nodel_loc.data();
  {  // (3) placement in element order from each chunk's ranks
    std::vector<std::thread> th;
    for (int64_t t = 0; t < T; t++)
      th.emplace_back([&, t]() {
        uint8_t *r = rank[t].data();
        int64_t e0, e1;
        chunk(t, e0, e1);
        for (int64_t i = e0 * npe; i < e1 * npe; i++) {
          const int32_t n = el[i];
          const int64_t k = off[n] + r[n]++;
          lst[k] = (int32_t)(i / npe);
          loc[k] = (int32_t)(i % npe);
        }
      });
    for (std::thread &x : th) x.join();
  }
}

// The device tables of an initialised domain read back as host lists.
bool download_lists(wf_domain *d) {
  const int64_t nn = d->nn, ent = d->ne * d->npe;
  std::vector<int32_t> off(nn + 1), slot(ent);
  if (cudaSetDevice(d->device) != cudaSuccess ||
      cudaMemcpyAsync(off.data(), d->P.off, sizeof(int32_t) * (nn + 1), cudaMemcpyDeviceToHost,
                      d->stream) != cudaSuccess ||
      cudaMemcpyAsync(slot.data(), d->P.slot, sizeof(int32_t) * ent, cudaMemcpyDeviceToHost,
                      d->stream) != cudaSuccess ||
      cudaStreamSynchronize(d->stream) != cudaSuccess)
    return false;
  d->nodel.resize(ent);
  d->nodel_loc.resize(ent);
  d->nodel_cnt.resize(nn);
  host_parallel(ent, [&](int64_t k0, int64_t k1) {
    for (int64_t k = k0; k < k1; k++) {
      d->nodel[k] = slot[k] / d->npe;
      d->nodel_loc[k] = slot[k] % d->npe;
    }
  });
  for (int64_t n = 0; n < nn; n++) d->nodel_cnt[n] = off[n + 1] - off[n];
  d->nodel_off = std::move(off);
  return true;
}

// The host lists, built on first use after the mesh was set: from the
// device tables once wf_init has built them, else by host threads. False
// when the device tables could not be read back.
bool ensure_host_lists(const wf_domain *cd) {
  wf_domain *d = const_cast<wf_domain *>(cd);
  if (d->nodel_off.size() == (size_t)d->nn + 1) return true;
  if (d->initialized && d->P.slot) return download_lists(d);
  if (host_mesh(d) != WF_OK) return false;
  build_nodel(d);
  return true;
}

// Triangle normals and plane coefficients (TriMesh_d::CalcNormals,
// UpdatePlaneCoeff with far node 2; Mesh.h:236-284).
void tri_normals_planes(const std::vector<double> &x, const std::vector<int32_t> &el,
                        std::vector<double> &nrm, std::vector<double> &pp) {
  const size_t ne = el.size() / 3;
  nrm.assign(3 * ne, 0.0);
  pp.assign(ne, 0.0);
  for (size_t e = 0; e < ne; e++) {
    const double *p0 = &x[3 * el[3 * e]], *p1 = &x[3 * el[3 * e + 1]], *p2 = &x[3 * el[3 * e + 2]];
    const double u[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
    const double v[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
    const double w[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2],
                         u[0] * v[1] - u[1] * v[0]};
    const double len = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    const double inv = 1.0 / len;
    double *n = &nrm[3 * e];
    n[0] = w[0] * inv;
    n[1] = w[1] * inv;
    n[2] = w[2] * inv;
    pp[e] = p2[0] * n[0] + p2[1] * n[1] + p2[2] * n[2];
  }
}

double tri_area(const double *p0, const double *p1, const double *p2) {
  const double v1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
  const double v2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
  const double c[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2],
                       v1[0] * v2[1] - v1[1] * v2[0]};
  return 0.5 * std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
}

// External surface of the part (SearchExtNodes + CalcExtFaceAreas,
// Domain_d.C:110-290): faces used by one element are external, their area goes
// in equal shares to their nodes (faces in element order and local order;
// tetrahedra with the reference's triangle table, hexahedra with its
// quadrilateral table, a quadrilateral's area as triangles (0,1,2) + (0,2,3)).
// Element length: the smallest height of the tetrahedron of the element's
// first four nodes (calcMinEdgeLength, Domain_d.C:2236-2262); nodlen is its
// mean over the node's elements (Contact.C:145-152).
void part_surface(const wf_domain *d, std::vector<uint8_t> &ext, std::vector<double> &area,
                  std::vector<double> &nodlen) {
  static const int TF[4][3] = {{0, 1, 2}, {0, 1, 3}, {1, 2, 3}, {0, 2, 3}};
  static const int HF[6][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}, {0, 1, 5, 4},
                               {2, 3, 7, 6}, {0, 3, 7, 4}, {1, 2, 6, 5}};
  const int npe = d->npe, nf = npe == 8 ? 6 : 4, fn = npe == 8 ? 4 : 3;
  std::map<std::array<int32_t, 4>, int> count;
  auto face = [&](int64_t e, int f, int32_t *fnodes) {
    std::array<int32_t, 4> k{-1, -1, -1, -1};
    for (int q = 0; q < fn; q++) {
      fnodes[q] = d->elnod[e * npe + (npe == 8 ? HF[f][q] : TF[f][q])];
      k[q] = fnodes[q];
    }
    std::sort(k.begin(), k.begin() + fn);
    return k;
  };
  int32_t fnodes[4];
  for (int64_t e = 0; e < d->ne; e++)
    for (int f = 0; f < nf; f++) count[face(e, f, fnodes)]++;
  ext.assign(d->nn, 0);
  area.assign(d->nn, 0.0);
  nodlen.assign(d->nn, 0.0);
  const double *X = d->x.data();
  for (int64_t e = 0; e < d->ne; e++)
    for (int f = 0; f < nf; f++) {
      if (count[face(e, f, fnodes)] != 1) continue;
      const double *p0 = &X[3 * fnodes[0]], *p1 = &X[3 * fnodes[1]], *p2 = &X[3 * fnodes[2]];
      double share;
      if (fn == 3) {
        share = tri_area(p0, p1, p2) / 3.0;
      } else {
        const double *p3 = &X[3 * fnodes[3]];
        share = (tri_area(p0, p1, p2) + tri_area(p0, p2, p3)) / 4.0;
      }
      for (int q = 0; q < fn; q++) {
        ext[fnodes[q]] = 1;
        area[fnodes[q]] += share;
      }
    }
  std::vector<double> elen(d->ne);
  for (int64_t e = 0; e < d->ne; e++) {
    const int32_t *n = &d->elnod[e * npe];
    const double *A = &X[3 * n[0]], *B = &X[3 * n[1]], *C = &X[3 * n[2]], *D = &X[3 * n[3]];
    const double *faces[4][3] = {{B, C, D}, {A, C, D}, {A, B, D}, {A, B, C}};
    double hmin = 1.0e6;
    for (int i = 0; i < 4; i++) {
      const double *f0 = faces[i][0], *f1 = faces[i][1], *f2 = faces[i][2];
      const double x1[3] = {f1[0] - f0[0], f1[1] - f0[1], f1[2] - f0[2]};
      const double x2[3] = {f2[0] - f0[0], f2[1] - f0[1], f2[2] - f0[2]};
      double nn[3] = {x1[1] * x2[2] - x1[2] * x2[1], x1[2] * x2[0] - x1[0] * x2[2],
                      x1[0] * x2[1] - x1[1] * x2[0]};
      const double ar = std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
      if (ar < 1e-12) continue;
      const double inv = 1.0 / ar;
      nn[0] *= inv;
      nn[1] *= inv;
      nn[2] *= inv;
      const double *P = &X[3 * n[i]];
      const double vec[3] = {P[0] - f0[0], P[1] - f0[1], P[2] - f0[2]};
      const double h = std::fabs(vec[0] * nn[0] + vec[1] * nn[1] + vec[2] * nn[2]);
      if (h < hmin) hmin = h;
    }
    elen[e] = hmin;
  }
  for (int64_t i = 0; i < d->nn; i++) {
    double l = 0.0;
    const int32_t b = d->nodel_off[i], c = d->nodel_cnt[i];
    for (int32_t k = 0; k < c; k++) l += elen[d->nodel[b + k]];
    nodlen[i] = l / c;
  }
}

void reset_mesh(wf_domain *d) {
  free_device(d);
  free_mesh_dev(d);
  d->x = hvec<double>();
  d->elnod = hvec<int32_t>();
  d->mesh_host = false;
  for (int k = 0; k < 3; k++) {
    d->bc_nod[k].clear();
    d->bc_val[k].clear();
  }
  d->emat.clear();
  d->react_nodes.clear();
  d->cand.clear();
  d->contact = false;
  d->tri = false;
  d->tri_x.clear();
  d->tri_el.clear();
  d->tri_v.clear();
  d->tri_mid.clear();
  d->tri_meshes = 0;
  d->bcs_allocated = false;
  d->nspec = 0;
  d->spec_eoff.clear();
  d->spec_noff.clear();
  d->spec_dt.clear();
  d->nodel.clear();
  d->nodel_loc.clear();
  d->nodel_off.clear();
  d->nodel_cnt.clear();
}

wf_status need_mesh(wf_domain *d) {
  if (!d) return WF_ERR_ARG;
  if (d->nn <= 0) return fail(d, WF_ERR_STATE, "no mesh defined");
  return WF_OK;
}

// Frees the device copy of the mesh.
void free_mesh_dev(wf_domain *d) {
  if (d->stream) cudaStreamSynchronize(d->stream);
  if (d->mesh_x) cudaFreeAsync(d->mesh_x, d->stream);
  if (d->mesh_el) cudaFreeAsync(d->mesh_el, d->stream);
  if (d->mesh_flag) cudaFreeAsync(d->mesh_flag, d->stream);
  d->mesh_x = nullptr;
  d->mesh_el = nullptr;
  d->mesh_flag = nullptr;
}

// Uploads the mesh (nn, ne, npe set) into its device copy and checks there
// that every connectivity entry names a node in [0, nn). Returns once the
// copies are done: the caller's arrays can go.
wf_status mesh_upload(wf_domain *d, const double *xyz, const int32_t *el) {
  CUDA_TRY(cudaSetDevice(d->device));
  free_mesh_dev(d);
  const size_t xb = sizeof(double) * 3 * d->nn, eb = sizeof(int32_t) * d->ne * d->npe;
  CUDA_TRY(pool_alloc(d, reinterpret_cast<void **>(&d->mesh_x), xb));
  CUDA_TRY(pool_alloc(d, reinterpret_cast<void **>(&d->mesh_el), eb));
  CUDA_TRY(pool_alloc(d, reinterpret_cast<void **>(&d->mesh_flag), sizeof(int32_t)));
  CUDA_TRY(cudaMemcpyAsync(d->mesh_x, xyz, xb, cudaMemcpyHostToDevice, d->stream));
  CUDA_TRY(cudaMemcpyAsync(d->mesh_el, el, eb, cudaMemcpyHostToDevice, d->stream));
  d->h2d_bytes += (int64_t)(xb + eb);
  int bad = 1;
  CUDA_TRY(check_connectivity(d->mesh_el, d->ne * d->npe, d->nn, d->mesh_flag, d->stream, &bad));
  if (bad) return fail(d, WF_ERR_ARG, "connectivity references a node outside [0, nn)");
  return WF_OK;
}

// The host mirror of the mesh, downloaded from the device copy on first use.
wf_status host_mesh(const wf_domain *cd) {
  wf_domain *d = const_cast<wf_domain *>(cd);
  if (d->mesh_host || d->nn <= 0) return WF_OK;
  CUDA_TRY(cudaSetDevice(d->device));
  d->x.resize(3 * d->nn);
  d->elnod.resize(d->ne * d->npe);
  CUDA_TRY(cudaMemcpyAsync(d->x.data(), d->mesh_x, sizeof(double) * 3 * d->nn,
                           cudaMemcpyDeviceToHost, d->stream));
  CUDA_TRY(cudaMemcpyAsync(d->elnod.data(), d->mesh_el, sizeof(int32_t) * d->ne * d->npe,
                           cudaMemcpyDeviceToHost, d->stream));
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  d->mesh_host = true;
  return WF_OK;
}

}  // namespace

wf_status wf::domain_fail(wf_domain *d, wf_status s, const std::string &msg) {
  return fail(d, s, "%s", msg.c_str());
}

// Definitions of the functions declared extern "C" in wf.h (C linkage is
// inherited from those declarations).

WF_API int32_t wf_abi_version(void) { return 1; }

WF_API const char *wf_status_string(wf_status s) {
  switch (s) {
    case WF_OK: return "ok";
    case WF_ERR_ARG: return "invalid argument";
    case WF_ERR_STATE: return "call out of order";
    case WF_ERR_CUDA: return "CUDA error";
    case WF_ERR_NOMEM: return "out of memory";
    case WF_ERR_UNSUPPORTED: return "unsupported option";
    case WF_ERR_NONFINITE: return "non-finite state";
    case WF_ERR_TIMEOUT: return "device wait timed out";
  }
  return "unknown status";
}

WF_API const char *wf_last_error(const wf_domain *d) { return d ? d->err.c_str() : "null domain"; }

WF_API wf_status wf_domain_create_on_device(wf_domain **out, int device) {
  if (!out) return WF_ERR_ARG;
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count <= device || device < 0) return WF_ERR_CUDA;
  wf_domain *d = new (std::nothrow) wf_domain();
  if (!d) return WF_ERR_NOMEM;
  d->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete d;
    return WF_ERR_CUDA;
  }
  *out = d;
  return WF_OK;
}

WF_API wf_status wf_domain_create(wf_domain **out) { return wf_domain_create_on_device(out, 0); }

WF_API wf_status wf_domain_destroy(wf_domain *d) {
  if (!d) return WF_ERR_ARG;
  cudaSetDevice(d->device);
  if (d->stream) cudaStreamSynchronize(d->stream);
  if (d->out_stream) cudaStreamSynchronize(d->out_stream);
  free_device(d);
  free_mesh_dev(d);
  if (d->stream) cudaStreamDestroy(d->stream);
  if (d->out_stream) cudaStreamDestroy(d->out_stream);
  delete d;
  return WF_OK;
}

// ---- mesh -----------------------------------------------------------------
WF_API wf_status wf_add_box_length(wf_domain *d, const double V[3], const double L[3], double r,
                                   int32_t red_int, int32_t tritetra) {
  if (!d || !V || !L) return WF_ERR_ARG;
  if (!red_int) return fail(d, WF_ERR_UNSUPPORTED, "only one-point (reduced) integration");
  if (!(L[2] > 0.0)) return fail(d, WF_ERR_UNSUPPORTED, "only 3-D boxes (L.z > 0)");
  if (!(r > 0.0)) return fail(d, WF_ERR_ARG, "r must be positive");
  reset_mesh(d);
  std::string err;
  std::vector<double> bx;
  std::vector<int32_t> be;
  if (!wf::box_mesh(V, L, r, tritetra != 0, bx, be, err)) {
    d->nn = d->ne = 0;
    return fail(d, WF_ERR_ARG, "%s", err.c_str());
  }
  d->x.assign(bx.begin(), bx.end());
  d->elnod.assign(be.begin(), be.end());
  d->mesh_host = true;
  d->npe = tritetra ? 4 : 8;
  d->nn = (int64_t)(d->x.size() / 3);
  d->ne = (int64_t)(d->elnod.size() / d->npe);
  const wf_status s = mesh_upload(d, d->x.data(), d->elnod.data());
  if (s) {
    d->nn = d->ne = 0;
    return s;
  }
  return WF_OK;
}

WF_API wf_status wf_set_mesh(wf_domain *d, int64_t nn, int64_t ne, int32_t npe, const double *xyz,
                             const int32_t *elnod) {
  if (!d || !xyz || !elnod || nn <= 0 || ne <= 0) return WF_ERR_ARG;
  if (npe != 4 && npe != 8)
    return fail(d, WF_ERR_UNSUPPORTED, "npe must be 8 (hexahedra) or 4 (tetrahedra)");
  if (ne * npe >= (int64_t)INT32_MAX || nn >= (int64_t)INT32_MAX)
    return fail(d, WF_ERR_ARG, "mesh too large");
  reset_mesh(d);
  d->npe = npe;
  d->nn = nn;
  d->ne = ne;
  // straight to the device copy (no host copy: the host mirror is made when
  // a host caller needs it); the range check runs there
  const wf_status s = mesh_upload(d, xyz, elnod);
  if (s) {
    d->nn = d->ne = 0;
    free_mesh_dev(d);
    return s;
  }
  return WF_OK;
}

WF_API wf_status wf_set_node(wf_domain *d, int64_t n, double x, double y, double z) {
  wf_status s = need_mesh(d);
  if (s) return s;
  if (n < 0 || n >= d->nn) return fail(d, WF_ERR_ARG, "node %lld out of range", (long long)n);
  if (d->initialized) return fail(d, WF_ERR_STATE, "setNode after init");
  const double v[3] = {x, y, z};
  if (d->mesh_host) std::memcpy(&d->x[3 * n], v, sizeof(v));
  CUDA_TRY(cudaSetDevice(d->device));
  CUDA_TRY(cudaMemcpyAsync(d->mesh_x + 3 * n, v, sizeof(v), cudaMemcpyHostToDevice, d->stream));
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  return WF_OK;
}

WF_API wf_status wf_set_nodes(wf_domain *d, const double *xyz) {
  wf_status s = need_mesh(d);
  if (s) return s;
  if (!xyz) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "setNode after init");
  if (d->mesh_host) std::memcpy(d->x.data(), xyz, sizeof(double) * 3 * d->nn);
  CUDA_TRY(cudaSetDevice(d->device));
  CUDA_TRY(cudaMemcpyAsync(d->mesh_x, xyz, sizeof(double) * 3 * d->nn, cudaMemcpyHostToDevice,
                           d->stream));
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  d->h2d_bytes += (int64_t)(sizeof(double) * 3 * d->nn);
  return WF_OK;
}

WF_API wf_status wf_get_sizes(const wf_domain *d, int64_t *nn, int64_t *ne, int32_t *npe,
                              int64_t *tot) {
  if (!d) return WF_ERR_ARG;
  if (nn) *nn = d->nn;
  if (ne) *ne = d->ne;
  if (npe) *npe = d->npe;
  if (tot) *tot = d->ne * d->npe;   // every entry is on one node's list
  return WF_OK;
}

WF_API wf_status wf_get_connectivity(const wf_domain *d, int32_t *elnod, int32_t *nodel,
                                     int32_t *nodel_loc, int32_t *offset, int32_t *count) {
  if (!d) return WF_ERR_ARG;
  if ((nodel || nodel_loc || offset || count) && !ensure_host_lists(d))
    return fail(const_cast<wf_domain *>(d), WF_ERR_CUDA, "reading back the node lists failed");
  if (elnod) {
    const wf_status hs = host_mesh(d);
    if (hs) return hs;
    std::copy(d->elnod.begin(), d->elnod.end(), elnod);
  }
  if (nodel) std::copy(d->nodel.begin(), d->nodel.end(), nodel);
  if (nodel_loc) std::copy(d->nodel_loc.begin(), d->nodel_loc.end(), nodel_loc);
  if (offset) std::copy(d->nodel_off.begin(), d->nodel_off.begin() + d->nn, offset);
  if (count) std::copy(d->nodel_cnt.begin(), d->nodel_cnt.end(), count);
  return WF_OK;
}

// ---- material -------------------------------------------------------------
WF_API wf_status wf_set_density(wf_domain *d, double rho) {
  if (!d || !(rho > 0.0)) return WF_ERR_ARG;
  d->rho_all = rho;
  d->rho_set = true;
  return WF_OK;
}

WF_API wf_status wf_set_materials(wf_domain *d, int32_t nmat, const wf_material *mats) {
  if (!d || nmat <= 0 || !mats) return WF_ERR_ARG;
  for (int i = 0; i < nmat; i++) {
    const wf_material &m = mats[i];
    if (!(m.E > 0) || !(m.rho > 0) || !(m.nu > -1.0 && m.nu < 0.5))
      return fail(d, WF_ERR_ARG, "material %d: need E > 0, rho > 0, -1 < nu < 0.5", i);
    if (m.model != WF_MAT_BILINEAR && m.model != WF_MAT_HOLLOMON &&
        m.model != WF_MAT_JOHNSON_COOK && m.model != WF_MAT_GMT)
      return fail(d, WF_ERR_UNSUPPORTED, "material %d: model %d", i, m.model);
    if (m.model == WF_MAT_HOLLOMON && !(m.hol_K > 0 && m.hol_m > 0))
      return fail(d, WF_ERR_ARG, "material %d: Hollomon needs K > 0, m > 0", i);
  }
  d->mats.assign(mats, mats + nmat);
  d->jc.assign(nmat, std::array<double, 8>{0, 0, 0, 0, 0, 0, 0, 0});
  d->gmt.assign(nmat, std::array<double, 15>{});
  d->mat_thermal.assign(nmat, std::array<double, 3>{0, 0, 0});
  d->rho_all = mats[0].rho;
  d->rho_set = true;
  return WF_OK;
}

WF_API wf_status wf_set_johnson_cook(wf_domain *d, int32_t mat, double B, double n, double C,
                                     double eps0_dot, double m, double T_melt,
                                     double T_transition, double T) {
  if (!d) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "materials are set before init");
  if (mat < 0 || mat >= (int32_t)d->mats.size())
    return fail(d, WF_ERR_ARG, "material %d out of range", mat);
  if (d->mats[mat].model != WF_MAT_JOHNSON_COOK)
    return fail(d, WF_ERR_STATE, "material %d is not of model WF_MAT_JOHNSON_COOK", mat);
  if (!(eps0_dot > 0) || !(T_melt != T_transition))
    return fail(d, WF_ERR_ARG, "Johnson-Cook needs eps0_dot > 0 and T_melt != T_transition");
  d->jc[mat] = {B, n, C, eps0_dot, m, T_melt, T_transition, T};
  return WF_OK;
}

WF_API wf_status wf_set_plastic_heat_fraction(wf_domain *d, double f) {
  if (!d) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "the plastic heat fraction is set before init");
  if (!(f >= 0.0 && f <= 1.0)) return fail(d, WF_ERR_ARG, "plastic heat fraction %g not in [0, 1]", f);
  d->plheat_frac = f;
  return WF_OK;
}

WF_API wf_status wf_set_max_strain_rate(wf_domain *d, double r) {
  if (!d) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "the strain-rate cap is set before init");
  if (!(r > 0.0)) return fail(d, WF_ERR_ARG, "strain-rate cap %g <= 0", r);
  d->max_edot = r;
  return WF_OK;
}

WF_API wf_status wf_set_gmt(wf_domain *d, int32_t mat, const double c[8], const double range[6],
                            double T) {
  if (!d) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "materials are set before init");
  if (mat < 0 || mat >= (int32_t)d->mats.size())
    return fail(d, WF_ERR_ARG, "material %d out of range", mat);
  if (d->mats[mat].model != WF_MAT_GMT)
    return fail(d, WF_ERR_STATE, "material %d is not of model WF_MAT_GMT", mat);
  if (!c || !range) return fail(d, WF_ERR_ARG, "GMT needs its constants and ranges");
  for (int q = 0; q < 8; q++)
    if (!std::isfinite(c[q])) return fail(d, WF_ERR_ARG, "GMT constant %d is not finite", q);
  for (int q = 0; q < 6; q += 2)
    if (!(range[q] <= range[q + 1])) return fail(d, WF_ERR_ARG, "GMT range %d: need min <= max", q / 2);
  if (!(range[0] > 0))
    return fail(d, WF_ERR_ARG, "GMT needs e_min > 0 (at e = 0 the law is 0 * inf)");
  std::array<double, 15> &g = d->gmt[mat];
  for (int q = 0; q < 8; q++) g[q] = c[q];
  for (int q = 0; q < 6; q++) g[8 + q] = range[q];
  g[14] = T;
  return WF_OK;
}

// ---- thermal coupling (Thermal.C) ---------------------------------------------------
WF_API wf_status wf_set_thermal(wf_domain *d, int32_t on, double T0) {
  if (!d) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "thermal coupling is set before init");
  d->thermal = on != 0;
  d->T0 = T0;
  return WF_OK;
}

WF_API wf_status wf_set_material_thermal(wf_domain *d, int32_t mat, double k_T, double cp_T,
                                         double exp_T) {
  if (!d) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "materials are set before init");
  if (mat < 0 || mat >= (int32_t)d->mats.size())
    return fail(d, WF_ERR_ARG, "material %d out of range", mat);
  if (!(k_T >= 0) || !(cp_T > 0)) return fail(d, WF_ERR_ARG, "need k_T >= 0 and cp_T > 0");
  d->mat_thermal[mat] = {k_T, cp_T, exp_T};
  return WF_OK;
}

WF_API wf_status wf_set_contact_heat(wf_domain *d, double heat_cond, double T_die) {
  if (!d) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "contact heat is set before init");
  d->tri_hc = heat_cond;
  d->tri_Tdie = T_die;
  return WF_OK;
}

WF_API wf_status wf_set_elem_materials(wf_domain *d, const int32_t *ids) {
  wf_status s = need_mesh(d);
  if (s) return s;
  if (!ids) return WF_ERR_ARG;
  for (int64_t e = 0; e < d->ne; e++)
    if (ids[e] < 0 || ids[e] >= (int32_t)d->mats.size())
      return fail(d, WF_ERR_ARG, "element %lld: material id %d out of range", (long long)e, ids[e]);
  d->emat.assign(ids, ids + d->ne);
  return WF_OK;
}

// ---- BCs --------------------------------------------------------------------
WF_API wf_status wf_add_bc_vel_node(wf_domain *d, int64_t node, int32_t dim, double val) {
  wf_status s = need_mesh(d);
  if (s) return s;
  if (dim < 0 || dim > 2) return fail(d, WF_ERR_ARG, "dim must be 0, 1 or 2");
  if (node < 0 || node >= d->nn) return fail(d, WF_ERR_ARG, "node %lld out of range", (long long)node);
  d->bc_nod[dim].push_back(node);
  d->bc_val[dim].push_back(val);
  d->bcs_allocated = false;
  return WF_OK;
}

WF_API wf_status wf_add_bc_vel_nodes(wf_domain *d, int64_t n, const int64_t *node,
                                     const int32_t *dim, const double *val) {
  wf_status s = need_mesh(d);
  if (s) return s;
  if (n < 0 || (n > 0 && (!node || !dim || !val))) return WF_ERR_ARG;
  for (int64_t i = 0; i < n; i++)
    if (dim[i] < 0 || dim[i] > 2 || node[i] < 0 || node[i] >= d->nn)
      return fail(d, WF_ERR_ARG, "entry %lld: node %lld dim %d out of range", (long long)i,
                  (long long)node[i], dim[i]);
  for (int64_t i = 0; i < n; i++) {
    d->bc_nod[dim[i]].push_back(node[i]);
    d->bc_val[dim[i]].push_back(val[i]);
  }
  d->bcs_allocated = false;
  return WF_OK;
}

WF_API wf_status wf_add_bc_vel_zone(wf_domain *d, const double start[3], const double end[3],
                                    const double vel[3], int64_t *count) {
  wf_status s = need_mesh(d);
  if (s) return s;
  if (!start || !end || !vel) return WF_ERR_ARG;
  s = host_mesh(d);
  if (s) return s;
  int64_t c = 0;
  for (int64_t a = 0; a < d->nn; a++) {
    bool in = true;
    for (int k = 0; k < 3; k++)
      if (d->x[3 * a + k] < start[k] || d->x[3 * a + k] > end[k]) in = false;
    if (in) {
      for (int k = 0; k < 3; k++) {
        d->bc_nod[k].push_back(a);
        d->bc_val[k].push_back(vel[k]);
      }
      c++;
    }
  }
  if (count) *count = c;
  d->bcs_allocated = false;
  return WF_OK;
}

WF_API wf_status wf_allocate_bcs(wf_domain *d) {
  wf_status s = need_mesh(d);
  if (s) return s;
  d->bcs_allocated = true;
  return WF_OK;
}

// ---- options ------------------------------------------------------------------
WF_API wf_status wf_set_dt(wf_domain *d, double dt) {
  if (!d || !(dt > 0.0) || !std::isfinite(dt)) return WF_ERR_ARG;
  d->dt = dt;
  drop_graphs(d);
  return WF_OK;
}

WF_API wf_status wf_set_end_time(wf_domain *d, double t) {
  if (!d) return WF_ERR_ARG;
  d->end_t = t;
  if (d->initialized && d->P.end_t != t) {
    // the die ramp of triangle-mesh contact reads the end time
    d->P.end_t = t;
    drop_graphs(d);
  }
  return WF_OK;
}

WF_API wf_status wf_set_precision(wf_domain *d, int32_t prec) {
  if (!d || (prec != WF_FP64 && prec != WF_MIXED)) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "precision must be set before init");
  d->precision = prec;
  return WF_OK;
}

WF_API wf_status wf_set_hourglass(wf_domain *d, double coef) {
  if (!d || !(coef >= 0.0)) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "options must be set before init");
  d->hg = coef;
  return WF_OK;
}

WF_API wf_status wf_set_press_algorithm(wf_domain *d, int32_t alg) {
  if (!d || (alg != 0 && alg != 1)) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "options must be set before init");
  d->press_alg = alg;
  return WF_OK;
}

WF_API wf_status wf_set_stab(wf_domain *d, const wf_stab *st) {
  if (!d || !st) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "options must be set before init");
  d->stab = *st;
  return WF_OK;
}

WF_API wf_status wf_set_artif_visc(wf_domain *d, double alpha, double beta) {
  if (!d) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "options must be set before init");
  d->av[0] = alpha;
  d->av[1] = beta;
  return WF_OK;
}

WF_API wf_status wf_set_mass_mode(wf_domain *d, int32_t mode) {
  if (!d || (mode != 0 && mode != 1)) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "options must be set before init");
  d->mass_mode = mode;
  return WF_OK;
}

WF_API wf_status wf_set_energy_history(wf_domain *d, int32_t on) {
  if (!d) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "the energy history is chosen before init");
  d->energy = on != 0;
  return WF_OK;
}

WF_API wf_status wf_set_reaction_nodes(wf_domain *d, int64_t n, const int32_t *nodes, int32_t dim) {
  wf_status s = need_mesh(d);
  if (s) return s;
  if ((n > 0 && !nodes) || dim < 0 || dim > 2) return WF_ERR_ARG;
  for (int64_t i = 0; i < n; i++)
    if (nodes[i] < 0 || nodes[i] >= d->nn) return fail(d, WF_ERR_ARG, "reaction node out of range");
  if (d->initialized) return fail(d, WF_ERR_STATE, "options must be set before init");
  d->react_nodes.assign(nodes, nodes + n);
  d->react_dim = dim;
  return WF_OK;
}

WF_API wf_status wf_set_contact_plane(wf_domain *d, double z0, double vz, double kpen, double mu,
                                      int64_t ncand, const int32_t *cand) {
  wf_status s = need_mesh(d);
  if (s) return s;
  if ((ncand > 0 && !cand) || !(kpen > 0) || !(mu >= 0)) return WF_ERR_ARG;
  for (int64_t i = 0; i < ncand; i++)
    if (cand[i] < 0 || cand[i] >= d->nn) return fail(d, WF_ERR_ARG, "contact node out of range");
  if (d->initialized) return fail(d, WF_ERR_STATE, "options must be set before init");
  d->contact = true;
  d->c_z0 = z0;
  d->c_vz = vz;
  d->c_k = kpen;
  d->c_mu = mu;
  d->cand.assign(cand, cand + ncand);
  return WF_OK;
}

// ---- batched ensemble ------------------------------------------------------------
WF_API wf_status wf_set_contact_trimesh(wf_domain *d, int64_t nnodes, const double *xyz,
                                        int64_t ntri, const int32_t *tri, const double vel[3],
                                        double mu_static, double mu_dynamic,
                                        double penalty_factor) {
  wf_status s = need_mesh(d);
  if (s) return s;
  if (!xyz || !tri || !vel || nnodes < 3 || ntri < 1) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "the contact mesh is set before init");
  for (int64_t i = 0; i < 3 * ntri; i++)
    if (tri[i] < 0 || tri[i] >= nnodes)
      return fail(d, WF_ERR_ARG, "triangle %lld references node %d", (long long)(i / 3), tri[i]);
  d->tri = true;
  d->tri_x.assign(xyz, xyz + 3 * nnodes);
  d->tri_el.assign(tri, tri + 3 * ntri);
  d->tri_v.resize(3 * nnodes);
  for (int64_t i = 0; i < 3 * nnodes; i++) d->tri_v[i] = vel[i % 3];
  d->tri_mid.assign(ntri, 0);
  d->tri_meshes = 1;
  d->tri_mu_s = mu_static;
  d->tri_mu_d = mu_dynamic;
  d->tri_pf = penalty_factor;
  d->contact = true;
  return WF_OK;
}

// TriMesh_d::AddMesh (Mesh.C:445-545): the new body's nodes and triangles are
// appended (triangle node indices offset by the current node count), its nodes
// take its velocity and its triangles its mesh index.
WF_API wf_status wf_add_contact_trimesh(wf_domain *d, int64_t nnodes, const double *xyz,
                                        int64_t ntri, const int32_t *tri, const double vel[3]) {
  wf_status s = need_mesh(d);
  if (s) return s;
  if (!xyz || !tri || !vel || nnodes < 3 || ntri < 1) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "the contact mesh is set before init");
  if (!d->tri) return fail(d, WF_ERR_STATE, "wf_set_contact_trimesh sets the first rigid body");
  const int64_t base = (int64_t)d->tri_x.size() / 3;
  if (base + nnodes > INT32_MAX || (int64_t)d->tri_mid.size() + ntri > INT32_MAX)
    return fail(d, WF_ERR_ARG, "contact mesh too large");
  for (int64_t i = 0; i < 3 * ntri; i++)
    if (tri[i] < 0 || tri[i] >= nnodes)
      return fail(d, WF_ERR_ARG, "triangle %lld references node %d", (long long)(i / 3), tri[i]);
  d->tri_x.insert(d->tri_x.end(), xyz, xyz + 3 * nnodes);
  for (int64_t i = 0; i < 3 * ntri; i++) d->tri_el.push_back((int32_t)(tri[i] + base));
  for (int64_t i = 0; i < 3 * nnodes; i++) d->tri_v.push_back(vel[i % 3]);
  d->tri_mid.insert(d->tri_mid.end(), ntri, d->tri_meshes);
  d->tri_meshes++;
  return WF_OK;
}

WF_API wf_status wf_get_trimesh_nodes(wf_domain *d, double *out, int64_t cap, int64_t *n) {
  if (!d || !n) return WF_ERR_ARG;
  if (!d->initialized || !d->P.tri_on) return fail(d, WF_ERR_STATE, "no contact mesh on the device");
  CUDA_TRY(cudaSetDevice(d->device));
  *n = d->P.tri_nn;
  const int64_t m = std::min<int64_t>(cap, d->P.tri_nn);
  if (out && m > 0) {
    CUDA_TRY(cudaMemcpyAsync(out, d->P.tri_x, sizeof(double) * 3 * m, cudaMemcpyDeviceToHost,
                             d->stream));
    CUDA_TRY(cudaStreamSynchronize(d->stream));
  }
  return WF_OK;
}

WF_API wf_status wf_set_specimens(wf_domain *d, int32_t nspec, const int64_t *elem_off,
                                  const int64_t *node_off, const double *dt) {
  wf_status s = need_mesh(d);
  if (s) return s;
  if (nspec <= 0 || nspec > 65535 || !elem_off || !node_off || !dt)
    return fail(d, WF_ERR_ARG, "need 1..65535 specimens and their offsets and time steps");
  if (d->initialized) return fail(d, WF_ERR_STATE, "specimens must be set before init");
  if (elem_off[0] != 0 || node_off[0] != 0 || elem_off[nspec] != d->ne || node_off[nspec] != d->nn)
    return fail(d, WF_ERR_ARG, "specimen offsets must start at 0 and end at the mesh sizes");
  s = host_mesh(d);
  if (s) return s;
  for (int32_t k = 0; k < nspec; k++) {
    if (elem_off[k + 1] <= elem_off[k] || node_off[k + 1] <= node_off[k])
      return fail(d, WF_ERR_ARG, "specimen %d is empty or offsets decrease", k);
    if (!(dt[k] > 0.0) || !std::isfinite(dt[k]))
      return fail(d, WF_ERR_ARG, "specimen %d: time step must be positive", k);
    for (int64_t e = elem_off[k]; e < elem_off[k + 1]; e++)
      for (int a = 0; a < d->npe; a++) {
        const int32_t n = d->elnod[e * d->npe + a];
        if (n < node_off[k] || n >= node_off[k + 1])
          return fail(d, WF_ERR_ARG, "element %lld references a node of another specimen",
                      (long long)e);
      }
  }
  d->nspec = nspec;
  d->spec_eoff.assign(elem_off, elem_off + nspec + 1);
  d->spec_noff.assign(node_off, node_off + nspec + 1);
  d->spec_dt.assign(dt, dt + nspec);
  return WF_OK;
}

WF_API wf_status wf_get_specimen_reaction(wf_domain *d, int32_t spec, double *out, int64_t cap,
                                          int64_t *n) {
  if (!d) return WF_ERR_ARG;
  if (!d->initialized) return fail(d, WF_ERR_STATE, "wf_init not called");
  if (spec < 0 || spec >= d->nspec) return fail(d, WF_ERR_ARG, "specimen %d out of range", spec);
  CUDA_TRY(cudaSetDevice(d->device));
  const int64_t have = d->host_step;
  if (n) *n = have;
  const int64_t m = std::min(cap, have);
  if (out && m > 0) {
    std::vector<double> all((size_t)m * d->nspec);
    d->d2h_bytes += (int64_t)(sizeof(double) * all.size());
    CUDA_TRY(cudaMemcpyAsync(all.data(), d->P.hist_spec, sizeof(double) * all.size(),
                             cudaMemcpyDeviceToHost, d->stream));
    CUDA_TRY(cudaStreamSynchronize(d->stream));
    for (int64_t i = 0; i < m; i++) out[i] = all[(size_t)i * d->nspec + spec];
  }
  return WF_OK;
}

// ---- init -------------------------------------------------------------------------
namespace {

template <typename T, typename A>
cudaError_t upload(wf_domain *d, T **dst, const std::vector<T, A> &src) {
  cudaError_t e = dalloc(d, dst, src.size());
  if (e != cudaSuccess) return e;
  if (src.empty()) return cudaSuccess;
  d->h2d_bytes += (int64_t)(src.size() * sizeof(T));
  return cudaMemcpyAsync(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice,
                         d->stream);
}

// Per-node BC code: bits 0..2 = constrained dofs, bits 3.. = index of the
// node's value triple; for repeated entries the later one wins, as the serial
// BC loops of the reference (Domain_d.C:1109-1134) leave it.
void bc_tables(wf_domain *d, std::vector<int32_t> &bnode, std::vector<uint32_t> &bcode,
               std::vector<double> &vals) {
  // the records in call order; for a node and dimension the last one wins
  struct Rec {
    int64_t n;
    int k;
    double v;
  };
  std::vector<Rec> r;
  bool sorted = true;   // each dimension's list ascending (the usual case): a merge suffices
  for (int k = 0; k < 3; k++) {
    const auto &nk = d->bc_nod[k];
    for (size_t i = 1; i < nk.size() && sorted; i++) sorted = nk[i - 1] <= nk[i];
  }
  if (sorted) {
    // three-way merge by (node, dimension); within a dimension the list
    // order is kept, so a repeated node's later value stays later
    size_t at[3] = {0, 0, 0};
    r.reserve(d->bc_nod[0].size() + d->bc_nod[1].size() + d->bc_nod[2].size());
    for (;;) {
      int kb = -1;
      for (int k = 0; k < 3; k++)
        if (at[k] < d->bc_nod[k].size() &&
            (kb < 0 || d->bc_nod[k][at[k]] < d->bc_nod[kb][at[kb]]))
          kb = k;
      if (kb < 0) break;
      r.push_back({d->bc_nod[kb][at[kb]], kb, d->bc_val[kb][at[kb]]});
      at[kb]++;
    }
  } else {
    for (int k = 0; k < 3; k++)
      for (size_t i = 0; i < d->bc_nod[k].size(); i++)
        r.push_back({d->bc_nod[k][i], k, d->bc_val[k][i]});
    std::stable_sort(r.begin(), r.end(), [](const Rec &a, const Rec &b) {
      return a.n < b.n || (a.n == b.n && a.k < b.k);
    });
  }
  // keyed on the values' bit patterns: every value keeps its own set, NaN
  // included (double comparisons would merge a NaN into another set); sets
  // numbered in ascending node order
  auto bits = [](double v) {
    uint64_t u;
    std::memcpy(&u, &v, sizeof u);
    return u;
  };
  std::map<std::tuple<uint64_t, uint64_t, uint64_t>, uint32_t> sets;
  vals.assign(3, 0.0);
  sets[std::make_tuple(bits(0.0), bits(0.0), bits(0.0))] = 0;
  bnode.clear();
  bcode.clear();
  bnode.reserve(r.size());
  bcode.reserve(r.size());
  // neighbouring BC nodes mostly share their values: the last set found is
  // checked before the map
  auto last_key = std::make_tuple(bits(0.0), bits(0.0), bits(0.0));
  uint32_t last_id = 0;
  for (size_t i = 0; i < r.size();) {
    const int64_t n = r[i].n;
    double v3[3] = {0.0, 0.0, 0.0};
    uint32_t mask = 0;
    for (; i < r.size() && r[i].n == n; i++) {
      v3[r[i].k] = r[i].v;
      mask |= 1u << r[i].k;
    }
    const auto key = std::make_tuple(bits(v3[0]), bits(v3[1]), bits(v3[2]));
    uint32_t id;
    if (key == last_key) {
      id = last_id;
    } else {
      auto it = sets.find(key);
      if (it == sets.end()) {
        id = (uint32_t)(vals.size() / 3);
        sets[key] = id;
        vals.insert(vals.end(), v3, v3 + 3);
      } else {
        id = it->second;
      }
      last_key = key;
      last_id = id;
    }
    bnode.push_back((int32_t)n);
    bcode.push_back((id << 3) | mask);
  }
}

}  // namespace

namespace {

// Bounding box of the host coordinates {min x, y, z, max x, y, z}.
void host_bbox(const wf_domain *d, double bb[6]) {
  const int64_t nn = d->nn;
  const double *x = d->x.data();
  std::mutex mu;
  for (int k = 0; k < 3; k++) {
    bb[k] = INFINITY;
    bb[3 + k] = -INFINITY;
  }
  host_parallel(nn, [&](int64_t i0, int64_t i1) {
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t n = i0; n < i1; n++)
      for (int k = 0; k < 3; k++) {
        lo[k] = std::min(lo[k], x[3 * n + k]);
        hi[k] = std::max(hi[k], x[3 * n + k]);
      }
    std::lock_guard<std::mutex> lock(mu);
    for (int k = 0; k < 3; k++) {
      bb[k] = std::min(bb[k], lo[k]);
      bb[3 + k] = std::max(bb[3 + k], hi[k]);
    }
  });
}

// Element counts per axis if the host connectivity starts like an
// AddBoxLength box (the device check then confirms every element); else zeros.
void box_dims(const wf_domain *d, int *nx, int *ny, int *nz) {
  *nx = *ny = *nz = 0;
  if (d->npe != 8 || d->ne <= 0) return;
  int32_t first[8];
  const int32_t *e0 = first;
  if (d->mesh_host) {
    e0 = d->elnod.data();
  } else if (cudaMemcpy(first, d->mesh_el, sizeof(first), cudaMemcpyDeviceToHost) !=
             cudaSuccess) {
    cudaGetLastError();
    return;
  }
  const int64_t px = (int64_t)e0[3] - e0[0];
  if (e0[0] != 0 || px < 2 || e0[4] % px != 0) return;
  const int64_t py = e0[4] / px;
  if (py < 2) return;
  const int64_t exy = (px - 1) * (py - 1);
  if (d->ne % exy != 0) return;
  const int64_t ez = d->ne / exy;
  if (px * py * (ez + 1) != d->nn || ez >= INT32_MAX) return;
  *nx = (int)(px - 1);
  *ny = (int)(py - 1);
  *nz = (int)ez;
}

// Device allocation kept with the domain (build_tiles' tables).
cudaError_t keep_alloc(void *ctx, void **p, size_t bytes) {
  return dalloc_raw(static_cast<wf_domain *>(ctx), reinterpret_cast<char **>(p), bytes);
}

// Times each candidate launch shape of the three tunable mixed kernels on the
// domain's data and keeps the fastest. The element kernel advances the
// deviatoric stress and plastic strain, the nodal kernel the contact slip:
// both are saved before the trials and restored after.
// Launch shapes chosen by the autotuner, kept for the life of the process and
// keyed by everything the tuned kernels' speed depends on (device, element
// type, mesh sizes, material-law and coupling variants): a later domain of
// the same mesh shape takes them instead of timing the candidates again.
struct TuneKey {
  int device;
  int32_t npe, mat_general, thermal, contact, tri_on, energy_on, specimens, tiled;
  int64_t ne, nn;
  bool operator<(const TuneKey &o) const {
    return std::tie(device, npe, mat_general, thermal, contact, tri_on, energy_on, specimens,
                    tiled, ne, nn) < std::tie(o.device, o.npe, o.mat_general, o.thermal,
                                              o.contact, o.tri_on, o.energy_on, o.specimens,
                                              o.tiled, o.ne, o.nn);
  }
};
struct TuneResult {
  LaunchCfg cfg[3];
  double ms[3];
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneResult> g_tune_cache;

bool tiled_mode(const wf_domain *d);
bool sweep_mode(const wf_domain *d);
// Whether the steps run the per-phase element kernel (the tiled step and the
// column sweep do not: it is not tuned for them).
bool flow_mode(const wf_domain *d);
bool runs_element_kernel(const wf_domain *d) {
  return !tiled_mode(d) && !sweep_mode(d) && !flow_mode(d);
}

TuneKey tune_key(const wf_domain *d) {
  const StepParams &P = d->P;
  return TuneKey{d->device, P.npe, P.mat_general, P.thermal, P.contact, P.tri_on, P.energy_on,
                 P.nspec ? 1 : 0, runs_element_kernel(d) ? 0 : 1, d->ne, d->nn};
}

wf_status autotune_launches(wf_domain *d) {
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune_cache.find(tune_key(d));
    if (it != g_tune_cache.end()) {
      for (int k = 0; k < 3; k++) {
        d->cfg[k] = it->second.cfg[k];
        d->cfg_ms[k] = it->second.ms[k];
      }
      d->tune_cached = true;
      return WF_OK;
    }
  }
  d->tune_cached = false;
  const StepParams &P = d->P;
  MixState &M = d->M;
  const int64_t ne = d->ne, np = d->np;
  // the state the trials advance, saved in a device scratch buffer
  const size_t n_tau = 6 * ne, n_pls = ne, n_ut = 3 * np, n_cf = 3 * np;
  float *save = nullptr;
  CUDA_TRY(pool_alloc(d, reinterpret_cast<void **>(&save), 4 * (n_tau + n_pls + n_ut + n_cf)));
  float *s_tau = save, *s_pls = s_tau + n_tau, *s_ut = s_pls + n_pls, *s_cf = s_ut + n_ut;
  CUDA_TRY(cudaMemcpyAsync(s_tau, M.tau, 4 * n_tau, cudaMemcpyDeviceToDevice, d->stream));
  CUDA_TRY(cudaMemcpyAsync(s_pls, M.pls, 4 * n_pls, cudaMemcpyDeviceToDevice, d->stream));
  CUDA_TRY(cudaMemcpyAsync(s_ut, M.ut, 4 * n_ut, cudaMemcpyDeviceToDevice, d->stream));
  CUDA_TRY(cudaMemcpyAsync(s_cf, M.cf, 4 * n_cf, cudaMemcpyDeviceToDevice, d->stream));
  cudaEvent_t a, b;
  CUDA_TRY(cudaEventCreate(&a));
  CUDA_TRY(cudaEventCreate(&b));
  // items per thread 1, 2, or 0: a persistent grid (SMs x resident blocks).
  // The candidates are timed in interleaved rounds so that a drift of the
  // clocks while the GPU warms up does not favour the ones timed last; the
  // second round times only those within kKeep of the first round's best.
  // Each timing covers two launches, or one on meshes of a million elements
  // and more (a launch there lasts tens of microseconds or more, well above
  // the events' resolution).
  const int sizes[3] = {64, 128, 256}, epts[3] = {1, 2, 0};
  constexpr int kRounds = 2;
  const int reps = ne >= (int64_t(1) << 20) ? 1 : 2;
  constexpr double kKeep = 1.25;
  // the per-phase element kernel is not run by tiled or swept steps: not
  // tuned then
  const int nphase = runs_element_kernel(d) ? 3 : 2;
  for (int phase = 0; phase < nphase; phase++) {
    std::vector<LaunchCfg> cands;
    for (int bs : sizes)
      for (int ept : epts) cands.push_back(LaunchCfg{bs, ept});
    std::vector<double> total(cands.size(), 0.0);
    std::vector<int> timed(cands.size(), 0);
    std::vector<bool> alive(cands.size(), true);
    for (int round = 0; round < kRounds; round++) {
      if (round == 1) {
        // all candidates have one timing after the first round
        const double best0 = *std::min_element(total.begin(), total.end());
        for (size_t i = 0; i < cands.size(); i++) alive[i] = total[i] <= kKeep * best0;
      }
      for (size_t i = 0; i < cands.size(); i++) {
        if (!alive[i]) continue;
        const LaunchCfg c = cands[i];
        auto launch = [&]() {
          if (phase == 0) mix_geometry(P, M, d->mvol, d->stream, c);
          else if (phase == 1) mix_nodal(P, M, d->mvol, d->stream, c);
          else mix_elements(P, M, d->mvol, d->stream, c);
        };
        if (round == 0) launch();  // warm-up
        cudaEventRecord(a, d->stream);
        for (int r = 0; r < reps; r++) launch();
        cudaEventRecord(b, d->stream);
        CUDA_TRY(cudaEventSynchronize(b));
        CUDA_TRY(cudaGetLastError());
        float ms = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&ms, a, b));
        total[i] += ms;
        timed[i] += reps;
      }
    }
    size_t best = 0;
    while (!alive[best]) best++;
    for (size_t i = best + 1; i < cands.size(); i++)
      if (alive[i] && total[i] < total[best]) best = i;
    d->cfg[phase] = cands[best];
    d->cfg_ms[phase] = total[best] / timed[best];
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  CUDA_TRY(cudaMemcpyAsync(M.tau, s_tau, 4 * n_tau, cudaMemcpyDeviceToDevice, d->stream));
  CUDA_TRY(cudaMemcpyAsync(M.pls, s_pls, 4 * n_pls, cudaMemcpyDeviceToDevice, d->stream));
  CUDA_TRY(cudaMemcpyAsync(M.ut, s_ut, 4 * n_ut, cudaMemcpyDeviceToDevice, d->stream));
  CUDA_TRY(cudaMemcpyAsync(M.cf, s_cf, 4 * n_cf, cudaMemcpyDeviceToDevice, d->stream));
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  CUDA_TRY(cudaFreeAsync(save, d->stream));
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    TuneResult r;
    for (int k = 0; k < 3; k++) {
      r.cfg[k] = d->cfg[k];
      r.ms[k] = d->cfg_ms[k];
    }
    g_tune_cache[tune_key(d)] = r;
  }
  return WF_OK;
}

}  // namespace

WF_API wf_status wf_set_autotune(wf_domain *d, int32_t on) {
  if (!d) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "autotuning is chosen before init");
  d->autotune = on != 0;
  return WF_OK;
}

WF_API wf_status wf_set_launch_config(wf_domain *d, int32_t phase, int32_t block,
                                      int32_t items_per_thread) {
  if (!d || phase < 0 || phase > 2) return WF_ERR_ARG;
  if (block != 64 && block != 128 && block != 256)
    return fail(d, WF_ERR_ARG, "block size must be 64, 128 or 256");
  if (items_per_thread < 0) return fail(d, WF_ERR_ARG, "items per thread must be >= 0");
  d->cfg[phase] = LaunchCfg{block, items_per_thread};
  d->cfg_ms[phase] = 0.0;
  drop_graphs(d);
  return WF_OK;
}

// Meshes up to kClusterMaxElems elements get a cluster shape at init (the
// cluster run can then be chosen by hand); up to kClusterAutoElems the
// automatic mode uses it.
constexpr int64_t kClusterMaxElems = 65536;
constexpr int64_t kClusterAutoElems = 3000;
constexpr int64_t kClusterChunk = 4096;   // steps per cluster launch

namespace {
// Whether the next wf_run of d runs as one cluster launch.
bool cluster_mode(const wf_domain *d) {
  if (d->precision != WF_MIXED || d->nspec || d->P.energy_on || d->phase_timing || !d->cl_blocks)
    return false;
  return d->step_mode == 2 || (d->step_mode == 0 && d->ne <= kClusterAutoElems);
}
// Whether the automatic mode picks the tiled kernels for tiled meshes.
constexpr bool kTiledAuto = false;
// Whether the steps of d run as tiled element + assembly kernels.
bool tiled_mode(const wf_domain *d) {
  if (d->precision != WF_MIXED || !d->tiled) return false;
  return d->step_mode == 3 || (kTiledAuto && d->step_mode == 0 && !cluster_mode(d));
}
// Whether the automatic mode picks the column sweep for box meshes: when its
// columns fill the GPU (the kernel holds two blocks per SM; each column is a
// sequence of layers, so fewer columns leave SMs idle and the per-phase
// kernels are faster: a 32^3 box has 10 columns).
constexpr bool kSweepAuto = true;
bool sweep_fills_gpu(const wf_domain *d) {
  return 20 * (int64_t)d->W.ncx * d->W.ncy >= 19 * 2 * (int64_t)d->P.sms;
}
// Whether the steps of d run as the column sweep.
bool flow_mode(const wf_domain *d);
bool sweep_mode(const wf_domain *d) {
  if (d->precision != WF_MIXED || !d->sweep) return false;
  return d->step_mode == 4 || (kSweepAuto && d->step_mode == 0 && !cluster_mode(d) &&
                               !flow_mode(d) && sweep_fills_gpu(d));
}
// Whether the automatic mode picks the dataflow step for box meshes (before
// the column sweep): not, the sweep is faster on GB300.
constexpr bool kFlowAuto = false;
// Whether the dataflow step leaves the geometry and nodal phases to their own
// kernels (its launch then pipelines element and node-update tiles only).
constexpr bool kFlowSplit = true;
// Whether the steps of d run as the dataflow step.
bool flow_mode(const wf_domain *d) {
  if (d->precision != WF_MIXED || !d->flow) return false;
  return d->step_mode == 5 || (kFlowAuto && d->step_mode == 0 && !cluster_mode(d));
}
// Makes buffer p of each pair the current one (in M) and the other the one
// the next sweep writes (in W).
void set_parity(wf_domain *d, int p) {
  d->parity = p;
  d->M.xh = d->xh_pair[p];
  d->M.vp = d->vp_pair[p];
  d->M.tau = d->tau_pair[p];
  d->M.pls = d->pls_pair[p];
  d->W.xh_o = d->xh_pair[p ^ 1];
  d->W.vp_o = d->vp_pair[p ^ 1];
  d->W.tau_o = d->tau_pair[p ^ 1];
  d->W.pls_o = d->pls_pair[p ^ 1];
}
}  // namespace

WF_API wf_status wf_set_step_mode(wf_domain *d, int32_t mode) {
  if (!d || mode < 0 || mode > 5) return WF_ERR_ARG;
  if (mode != d->step_mode) drop_graphs(d);   // the graphs hold the other kernels
  d->step_mode = mode;
  return WF_OK;
}

WF_API wf_status wf_get_step_mode(const wf_domain *d, int32_t *mode, int32_t *blocks,
                                  int32_t *block_size) {
  if (!d) return WF_ERR_ARG;
  const bool c = d->initialized && cluster_mode(d);
  const bool t = d->initialized && !c && tiled_mode(d);
  const bool f = d->initialized && !c && !t && flow_mode(d);
  const bool w = d->initialized && !c && !t && !f && sweep_mode(d);
  if (mode) *mode = c ? 2 : (t ? 3 : (f ? 5 : (w ? 4 : 1)));
  if (blocks)
    *blocks = c ? d->cl_blocks
                : (t ? d->T.ntiles : (f ? d->F.grid : (w ? d->W.ncx * d->W.ncy : 0)));
  if (block_size)
    *block_size =
        c ? d->cl_bs : (t ? kTileElems : (f ? 256 : (w ? 32 * (d->W.cy + 1) : 0)));
  return WF_OK;
}

WF_API wf_status wf_set_flow_tiles(wf_domain *d, int32_t tile, int32_t lag) {
  if (!d) return WF_ERR_ARG;
  if (tile < 256 || tile > 8192 || (tile & 255))
    return fail(d, WF_ERR_ARG, "dataflow tiles hold a multiple of 256 items, 256 to 8192");
  if (lag < 1 || lag > 16) return fail(d, WF_ERR_ARG, "the node-update lag is 1 to 16 stages");
  if (d->initialized) return fail(d, WF_ERR_STATE, "the dataflow tiles are chosen before init");
  d->flow_tile = tile;
  d->flow_lag = lag;
  return WF_OK;
}

WF_API wf_status wf_get_flow(const wf_domain *d, int32_t *tiles, int32_t *grid, char *why,
                             int64_t why_cap) {
  if (!d) return WF_ERR_ARG;
  const bool on = d->initialized && d->flow;
  if (tiles) *tiles = on ? d->F.total : 0;
  if (grid) *grid = on ? d->F.grid : 0;
  if (why && why_cap > 0) {
    const std::string &w = d->initialized ? d->flow_why : std::string("wf_init not called");
    const size_t n = std::min<size_t>(w.size(), (size_t)why_cap - 1);
    std::memcpy(why, w.data(), n);
    why[n] = 0;
  }
  return WF_OK;
}

WF_API wf_status wf_set_sweep_rows(wf_domain *d, int32_t rows) {
  if (!d) return WF_ERR_ARG;
  if (rows != 4 && rows != 8) return fail(d, WF_ERR_ARG, "sweep columns have 4 or 8 node rows");
  if (d->initialized) return fail(d, WF_ERR_STATE, "the sweep's columns are chosen before init");
  d->sweep_rows = rows;
  return WF_OK;
}

WF_API wf_status wf_get_sweep(const wf_domain *d, int32_t *columns_x, int32_t *columns_y,
                              int32_t *rows, char *why, int64_t why_cap) {
  if (!d) return WF_ERR_ARG;
  const bool on = d->initialized && d->sweep;
  if (columns_x) *columns_x = on ? d->W.ncx : 0;
  if (columns_y) *columns_y = on ? d->W.ncy : 0;
  if (rows) *rows = on ? d->W.cy : 0;
  if (why && why_cap > 0) {
    const std::string &w = d->initialized ? d->sweep_why : std::string("wf_init not called");
    const size_t n = std::min<size_t>(w.size(), (size_t)why_cap - 1);
    std::memcpy(why, w.data(), n);
    why[n] = 0;
  }
  return WF_OK;
}

WF_API wf_status wf_set_box_indexing(wf_domain *d, int32_t on) {
  if (!d) return WF_ERR_ARG;
  if (d->initialized) return fail(d, WF_ERR_STATE, "box indexing is chosen before init");
  d->use_box = on != 0;
  return WF_OK;
}

WF_API wf_status wf_get_box(const wf_domain *d, int32_t dims[3]) {
  if (!d || !dims) return WF_ERR_ARG;
  const bool on = d->initialized && d->P.box;
  dims[0] = on ? d->P.bx : 0;
  dims[1] = on ? d->P.by : 0;
  dims[2] = on ? d->P.bz : 0;
  return WF_OK;
}

WF_API wf_status wf_get_tiles(const wf_domain *d, int32_t *ntiles, int32_t *nshared,
                              int64_t *tile_nodes, int64_t *shared_slots, char *why,
                              int64_t why_cap) {
  if (!d) return WF_ERR_ARG;
  if (!d->initialized) return fail(const_cast<wf_domain *>(d), WF_ERR_STATE, "wf_init not called");
  if (ntiles) *ntiles = d->tiled ? d->T.ntiles : 0;
  if (nshared) *nshared = d->tiled ? d->T.nshared : 0;
  if (tile_nodes) *tile_nodes = d->tiled ? d->T.tile_nodes : 0;
  if (shared_slots) *shared_slots = d->tiled ? d->T.shared_slots : 0;
  if (why && why_cap > 0) {
    const std::string &w = d->tiled ? std::string() : d->tile_why;
    const size_t n = std::min<size_t>(w.size(), (size_t)why_cap - 1);
    std::memcpy(why, w.data(), n);
    why[n] = '\0';
  }
  return WF_OK;
}

WF_API wf_status wf_get_launch_config(const wf_domain *d, int32_t phase, int32_t *block,
                                      int32_t *items_per_thread, double *ms) {
  if (!d || phase < 0 || phase > 2) return WF_ERR_ARG;
  if (block) *block = d->cfg[phase].bs;
  if (items_per_thread) *items_per_thread = d->cfg[phase].ept;
  if (ms) *ms = d->cfg_ms[phase];
  return WF_OK;
}

WF_API wf_status wf_init(wf_domain *d) {
  wf_status s = need_mesh(d);
  if (s) return s;
  if (d->mats.empty()) return fail(d, WF_ERR_STATE, "no material assigned (AssignMaterial)");
  if (d->precision == WF_MIXED) {
    // pressure algorithm 1 adds k0 (1 - J ratio) to each element's pressure
    // every step; an FP32 J ratio near 1 resolves the volume change only to
    // about 6e-8, and the sum carries that error on (12 % in the
    // displacements of the 12-step tetrahedral case against FP64)
    if (d->press_alg != 0)
      return fail(d, WF_ERR_UNSUPPORTED, "mixed precision supports pressure algorithm 0 only");
    const double *sp = &d->stab.alpha_free;
    for (int i = 0; i < 10; i++)
      if (sp[i] != 0.0)
        return fail(d, WF_ERR_UNSUPPORTED, "mixed precision supports default stabilisation only");
  }
  if (d->nspec && d->contact)
    return fail(d, WF_ERR_UNSUPPORTED, "contact is not supported in a batched ensemble");
  if (d->nspec && d->energy)
    return fail(d, WF_ERR_UNSUPPORTED, "the energy history is not kept for a batched ensemble");
  if (d->thermal && d->nspec)
    return fail(d, WF_ERR_UNSUPPORTED, "thermal coupling is not kept for a batched ensemble");
  if (d->thermal)
    for (size_t i = 0; i < d->mats.size(); i++)
      if (!(d->mat_thermal[i][1] > 0))
        return fail(d, WF_ERR_STATE, "material %zu: wf_set_material_thermal not called", i);
  CUDA_TRY(cudaSetDevice(d->device));
  free_device(d);
  const int64_t nn = d->nn, ne = d->ne;
  const int64_t np = (nn + 31) / 32 * 32;
  d->np = np;
  StepParams &P = d->P;
  P = StepParams{};
  {
    int sms = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d->device));
    P.sms = sms;
  }
  P.nn = nn;
  P.ne = ne;
  P.np = np;
  P.npe = d->npe;
  P.mass_mode = d->mass_mode;
  P.press_alg = d->press_alg;
  P.react_dim = d->react_dim;
  P.contact = d->contact ? 1 : 0;
  const double *sp = &d->stab.alpha_free;
  for (int i = 0; i < 10; i++) {
    P.stab[i] = sp[i];
    if (sp[i] != 0.0) P.stab_on = 1;
  }
  P.av[0] = d->av[0];
  P.av[1] = d->av[1];
  P.plheat_frac = d->plheat_frac;
  P.max_edot = d->max_edot;
  P.f_plheat = (float)d->plheat_frac;
  P.f_max_edot = (float)std::min(d->max_edot, (double)FLT_MAX);
  P.av_on = (d->av[0] != 0.0 || d->av[1] != 0.0) ? 1 : 0;
  P.hg_on = (d->hg != 0.0 && d->npe == 8) ? 1 : 0;
  P.hg_coef = d->hg;
  const double rho_b = 0.818200;  // Solver_explicit.C:193-197
  P.alpha = (2.0 * rho_b - 1.0) / (1.0 + rho_b);
  P.beta = (5.0 - 3.0 * rho_b) / ((1.0 + rho_b) * (1.0 + rho_b) * (2.0 - rho_b));
  P.gamma = 1.5 - P.alpha;
  P.fcorr = 1.0 / (1.0 - P.alpha);
  P.dt = d->dt;
  P.c_z0 = d->c_z0;
  P.c_vz = d->c_vz;
  P.c_k = d->c_k;
  P.c_mu = d->c_mu;

  // connectivity (SoA elnod) and node lists (slots e*npe + local), built on
  // the device from the mesh's device copy (wf_set_mesh)
  const int64_t ent = ne * d->npe;
  int32_t *el = nullptr;
  CUDA_TRY(dalloc_raw(d, &el, ent));
  P.elnod = el;
  const double *x_aos = d->mesh_x;
  CUDA_TRY(build_connectivity(d->mesh_el, ne, d->npe, nn, el, nullptr, nullptr, nullptr,
                              d->stream));
  // a box mesh (AddBoxLength numbering, however it was uploaded; mixed
  // precision): the mixed kernels compute corners and node lists instead of
  // loading them
  if (d->precision == WF_MIXED) {
    int bnx = 0, bny = 0, bnz = 0, is_box = 0;
    box_dims(d, &bnx, &bny, &bnz);
    if (d->npe == 8 && !d->nspec && d->use_box && bnx > 0)
      CUDA_TRY(check_box(P.elnod, ne, nn, bnx, bny, bnz, d->stream, &is_box));
    P.box = is_box;
    if (is_box) {
      P.bx = bnx;
      P.by = bny;
      P.bz = bnz;
      P.fd_ex = make_fastdiv((uint32_t)bnx);
      P.fd_exy = make_fastdiv((uint32_t)bnx * (uint32_t)bny);
      P.fd_nx = make_fastdiv((uint32_t)bnx + 1u);
      P.fd_nxy = make_fastdiv(((uint32_t)bnx + 1u) * ((uint32_t)bny + 1u));
    }
  }
  // the node lists, unless no kernel of the domain can read them: a mixed box
  // mesh without thermal coupling or triangle-mesh contact, too large for the
  // cluster run, and no tiled steps (host lists are then built from the host
  // mirror if a host caller asks)
  const bool lists = !(P.box && !d->thermal && !d->tri && d->step_mode != 3 &&
                       ne > kClusterMaxElems);
  if (lists) {
    int32_t *off = nullptr, *sl = nullptr;
    CUDA_TRY(dalloc_raw(d, &off, nn + 1));
    CUDA_TRY(dalloc_raw(d, &sl, ent));
    P.off = off;
    P.slot = sl;
    void *stage = nullptr;
    CUDA_TRY(pool_alloc(d, &stage, sizeof(int32_t) * connectivity_scratch_ints(nn)));
    d->init_stage = stage;
    CUDA_TRY(build_connectivity(d->mesh_el, ne, d->npe, nn, nullptr, off, sl,
                                static_cast<int32_t *>(stage), d->stream));
  }
  // BC codes per node (value set << 3 | fixed dimensions), zero but at the
  // BC nodes: scattered on the device from the BC nodes' records
  std::vector<int32_t> bnode;
  std::vector<uint32_t> bcode;
  std::vector<double> vals;
  bc_tables(d, bnode, bcode, vals);
  uint32_t *bc = nullptr;
  double *bcv = nullptr;
  CUDA_TRY(dalloc(d, &bc, nn));
  {
    int32_t *bn = nullptr;
    uint32_t *bv = nullptr;
    CUDA_TRY(upload(d, &bn, bnode));
    CUDA_TRY(upload(d, &bv, bcode));
    scatter_u32(bc, bn, bv, (int64_t)bnode.size(), d->stream);
    CUDA_TRY(cudaGetLastError());
  }
  CUDA_TRY(upload(d, &bcv, vals));
  P.bc = bc;
  P.bcval = bcv;
  {
    // FP32 copies for the mixed node update, which would otherwise convert
    // an FP64 value (an FP64-pipe instruction) per constrained component
    std::vector<float> vf(vals.size());
    for (size_t i = 0; i < vals.size(); i++) vf[i] = (float)vals[i];
    float *bcf = nullptr;
    CUDA_TRY(upload(d, &bcf, vf));
    P.bcvalf = bcf;
  }
  // node flags: zero but at the reaction and contact-candidate nodes (and
  // the external surface with a triangle-mesh die), set on the device
  uint8_t *fl = nullptr;
  CUDA_TRY(dalloc(d, &fl, nn));
  for (const auto &lst : {std::make_pair(&d->react_nodes, (uint8_t)NF_REACTION),
                          std::make_pair(&d->cand, (uint8_t)NF_CONTACT)}) {
    std::vector<int32_t> u(*lst.first);
    if (!std::is_sorted(u.begin(), u.end())) std::sort(u.begin(), u.end());
    u.erase(std::unique(u.begin(), u.end()), u.end());
    int32_t *ud = nullptr;
    CUDA_TRY(upload(d, &ud, u));
    or_flags(fl, ud, lst.second, (int64_t)u.size(), d->stream);
    CUDA_TRY(cudaGetLastError());
  }
  P.end_t = d->end_t;
  if (d->tri) {
    std::vector<uint8_t> ext;
    std::vector<double> area, nodlen, nrm, pp;
    if (!ensure_host_lists(d)) return fail(d, WF_ERR_CUDA, "reading back the node lists failed");
    {
      const wf_status hs = host_mesh(d);
      if (hs) return hs;
    }
    part_surface(d, ext, area, nodlen);
    {
      std::vector<int32_t> en;
      for (int64_t n = 0; n < nn; n++)
        if (ext[n]) en.push_back((int32_t)n);
      int32_t *ed = nullptr;
      CUDA_TRY(upload(d, &ed, en));
      or_flags(fl, ed, (uint8_t)NF_CONTACT, (int64_t)en.size(), d->stream);
      CUDA_TRY(cudaGetLastError());
    }
    tri_normals_planes(d->tri_x, d->tri_el, nrm, pp);
    double *tx = nullptr, *tvd = nullptr, *tn = nullptr, *tp = nullptr, *na = nullptr,
           *nl = nullptr;
    int32_t *te = nullptr, *tm = nullptr;
    CUDA_TRY(upload(d, &tx, d->tri_x));
    CUDA_TRY(upload(d, &tvd, d->tri_v));
    CUDA_TRY(upload(d, &tm, d->tri_mid));
    CUDA_TRY(upload(d, &tn, nrm));
    CUDA_TRY(upload(d, &tp, pp));
    CUDA_TRY(upload(d, &te, d->tri_el));
    CUDA_TRY(upload(d, &na, area));
    CUDA_TRY(upload(d, &nl, nodlen));
    P.tri_on = 1;
    P.tri_nn = (int32_t)(d->tri_x.size() / 3);
    P.tri_ne = (int32_t)(d->tri_el.size() / 3);
    P.tri_x = tx;
    P.tri_v = tvd;
    P.tri_nrm = tn;
    P.tri_pp = tp;
    P.tri_el = te;
    P.tri_mid = tm;
    P.node_area = na;
    P.nodlen = nl;
    P.tri_mu_s = d->tri_mu_s;
    P.tri_mu_d = d->tri_mu_d;
    P.tri_pf = d->tri_pf;
    P.tri_E0 = d->mats[0].E;
  }
  P.nflag = fl;
  // materials (Elastic_, Material.cuh:24-27; InitHollomon, :90-104)
  std::vector<MatDev> md(d->mats.size());
  for (size_t i = 0; i < d->mats.size(); i++) {
    const wf_material &m = d->mats[i];
    MatDev &t = md[i];
    t = MatDev{};
    t.E = m.E;
    t.K = m.E / (3.0 * (1.0 - 2.0 * m.nu));
    t.G = m.E / (2.0 * (1.0 + m.nu));
    t.sy0 = m.sy0;
    t.H = m.H;
    t.cs0 = std::sqrt(t.K / m.rho);
    t.model = m.model;
    t.hol_K = m.hol_K;
    t.hol_m = m.hol_m;
    if (m.model == WF_MAT_HOLLOMON) {
      t.eps0 = m.sy0 / m.E;
      t.eps1 = std::pow(m.sy0 / m.hol_K, 1. / m.hol_m);
    }
    if (m.model == WF_MAT_JOHNSON_COOK) {
      const std::array<double, 8> &j = d->jc[i];
      if (!(j[3] > 0)) return fail(d, WF_ERR_STATE, "material %zu: wf_set_johnson_cook not called", i);
      t.jc_B = j[0];
      t.jc_n = j[1];
      t.jc_C = j[2];
      t.jc_eps0 = j[3];
      const double T_h = (j[7] - j[6]) / (j[5] - j[6]);
      t.jc_Th = 1.0 - std::pow(T_h, j[4]);
      t.jc_m = j[4];
      t.jc_Tm = j[5];
      t.jc_Tt = j[6];
    }
    if (m.model == WF_MAT_GMT) {
      // GMT(el, n1, n2, C1, C2, m1, m2, I1, I2, ranges) (Material.cuh:271-290)
      const std::array<double, 15> &g = d->gmt[i];
      if (!(g[8] > 0)) return fail(d, WF_ERR_STATE, "material %zu: wf_set_gmt not called", i);
      t.g_n1 = g[0]; t.g_n2 = g[1]; t.g_C1 = g[2]; t.g_C2 = g[3];
      t.g_m1 = g[4]; t.g_m2 = g[5]; t.g_I1 = g[6]; t.g_I2 = g[7];
      t.g_emin = g[8]; t.g_emax = g[9]; t.g_rmin = g[10]; t.g_rmax = g[11];
      t.g_Tmin = g[12]; t.g_Tmax = g[13]; t.g_T = g[14];
    }
    t.k_T = d->mat_thermal[i][0];
    t.cp_T = d->mat_thermal[i][1];
    t.exp_T = d->mat_thermal[i][2];
  }
  MatDev *mdev = nullptr;
  CUDA_TRY(upload(d, &mdev, md));
  P.mats = mdev;
  for (const MatDev &t : md)
    if (t.model != WF_MAT_BILINEAR) P.mat_general = 1;
  P.k0 = md[0].K;
  if (!d->emat.empty()) {
    int32_t *em = nullptr;
    CUDA_TRY(upload(d, &em, d->emat));
    P.emat = em;
  }
  // batched ensemble tables
  if (d->nspec) {
    const int32_t S_ = d->nspec;
    P.nspec = S_;
    std::vector<uint16_t> es(ne), ns(nn);
    for (int32_t k = 0; k < S_; k++) {
      for (int64_t e = d->spec_eoff[k]; e < d->spec_eoff[k + 1]; e++) es[e] = (uint16_t)k;
      for (int64_t n = d->spec_noff[k]; n < d->spec_noff[k + 1]; n++) ns[n] = (uint16_t)k;
    }
    std::vector<SpecF> sf(S_);
    for (int32_t k = 0; k < S_; k++) {
      const double dt = d->spec_dt[k];
      sf[k] = SpecF{(float)dt, (float)((0.5 - P.beta) * dt), (float)(P.beta * dt * dt),
                    (float)(P.gamma * dt), (float)((1.0 - P.gamma) * dt), 0.f, 0.f, 0.f};
    }
    std::vector<int32_t> rl(d->react_nodes.begin(), d->react_nodes.end());
    std::sort(rl.begin(), rl.end());
    std::vector<int32_t> rloff(S_ + 1, 0);
    for (int32_t n : rl) rloff[ns[n] + 1]++;
    for (int32_t k = 0; k < S_; k++) rloff[k + 1] += rloff[k];
    uint16_t *esd = nullptr, *nsd = nullptr;
    double *sdt = nullptr;
    SpecF *sfd = nullptr;
    int32_t *rld = nullptr, *rlo = nullptr;
    CUDA_TRY(upload(d, &esd, es));
    CUDA_TRY(upload(d, &nsd, ns));
    CUDA_TRY(upload(d, &sdt, d->spec_dt));
    CUDA_TRY(upload(d, &sfd, sf));
    CUDA_TRY(upload(d, &rld, rl));
    CUDA_TRY(upload(d, &rlo, rloff));
    P.espec = esd;
    P.nspec_of = nsd;
    P.spec_dt = sdt;
    P.specf = sfd;
    P.rlist = rld;
    P.rl_off = rlo;
    CUDA_TRY(dalloc(d, &P.rnode, np));
  }
  // reaction history and step state
  d->node_grid = (d->precision == WF_MIXED) ? mix_node_grid(nn) : fp64_node_grid(nn, P.sms);
  CUDA_TRY(dalloc(d, &P.partials, std::max(d->node_grid, 32)));
  d->hist_cap = 1 << 16;
  CUDA_TRY(dalloc(d, &P.hist, d->hist_cap));
  if (d->nspec) CUDA_TRY(dalloc(d, &P.hist_spec, (size_t)d->hist_cap * d->nspec));
  P.hist_cap = d->hist_cap;
  CUDA_TRY(dalloc(d, &P.st, 1));
  CUDA_TRY(cudaMallocHost(&d->st_host, sizeof(StepState)));
  *d->st_host = StepState{};
  d->st_host->first_bad_node = LLONG_MAX;
  CUDA_TRY(cudaMemcpyAsync(&P.st->first_bad_node, &d->st_host->first_bad_node, sizeof(long long),
                           cudaMemcpyHostToDevice, d->stream));
  if (d->energy) {
    P.energy_on = 1;
    CUDA_TRY(dalloc(d, &P.epart, 2 * (size_t)energy_grid(P)));
    CUDA_TRY(dalloc(d, &P.ekin_hist, d->hist_cap));
    CUDA_TRY(dalloc(d, &P.eint_hist, d->hist_cap));
  }

  // FP64 state (also the export target of the mixed state)
  Fp64State &S = d->S;
  CUDA_TRY(dalloc_raw(d, &S.x, 3 * np));
  coords_soa(x_aos, nn, np, S.x, d->stream);
  const bool fp64 = d->precision == WF_FP64;
  CUDA_TRY(dalloc(d, &S.v, 3 * np));
  CUDA_TRY(dalloc(d, &S.pa, 3 * np));
  CUDA_TRY(dalloc(d, &S.u, 3 * np));
  CUDA_TRY(dalloc(d, &S.fi, 3 * np));
  CUDA_TRY(dalloc(d, &S.cf, 3 * np));
  CUDA_TRY(dalloc(d, &S.mass, np));
  CUDA_TRY(dalloc(d, &S.voln, np));
  CUDA_TRY(dalloc(d, &S.vol, ne));
  CUDA_TRY(dalloc(d, &S.vol0, ne));
  CUDA_TRY(dalloc(d, &S.rho, ne));
  CUDA_TRY(dalloc(d, &S.detJ, ne));
  CUDA_TRY(dalloc(d, &S.p, ne));
  CUDA_TRY(dalloc(d, &S.pls, ne));
  CUDA_TRY(dalloc(d, &S.sy, ne));
  CUDA_TRY(dalloc(d, &S.tau, 6 * ne));
  CUDA_TRY(dalloc(d, &S.sig, 6 * ne));
  CUDA_TRY(dalloc(d, &S.eps, 6 * ne));
  CUDA_TRY(dalloc(d, &S.jr, np));
  CUDA_TRY(dalloc(d, &S.s0, np));
  if (d->thermal) {
    // temperature (both precisions: the mixed state exports into S.T)
    CUDA_TRY(upload(d, &S.T, std::vector<double>(np, d->T0)));
    P.thermal = 1;
    P.cp0 = d->mat_thermal[0][1];
    P.tri_hc = d->tri_hc;
    P.tri_Tdie = d->tri_Tdie;
  }
  if (fp64) {
    CUDA_TRY(dalloc(d, &S.vp, 3 * np));
    CUDA_TRY(dalloc(d, &S.ut, 3 * np));
    if (d->thermal) {
      CUDA_TRY(dalloc(d, &S.qc, np));
      CUDA_TRY(dalloc(d, &S.dte, 2 * ne * d->npe));
    }
    CUDA_TRY(dalloc(d, &S.sr, 6 * ne));
    CUDA_TRY(dalloc(d, &S.rr, 6 * ne));
    CUDA_TRY(dalloc(d, &S.fe, (size_t)ne * d->npe * 3));
    if (P.hg_on) CUDA_TRY(dalloc(d, &S.fhg, (size_t)ne * d->npe * 3));
  }
  CUDA_TRY(dalloc_raw(d, &d->rho0_dev, ne));
  fill_values(d->rho0_dev, d->rho_all, ne, d->stream);

  // preamble (Solver_explicit.C:120-268): sigma_y = sy0, eps_p = 0; v = a = u
  // = 0 then ImposeBCV per dimension -- the zeroing sits inside the dimension
  // loop, so only the last dimension's BC values survive into step 1.
  initial_yield(P, S.sy, d->stream);
  initial_velocity(P, S.v, d->stream);
  if (fp64) {
    // initial volumes, densities, nodal volumes and masses (CalcElemInitialVol,
    // calcElemDensity, CalcNodalVol, CalcNodalMassFromVol); the mixed state
    // forms its own in FP32 (mix_init)
    fp64_geometry(P, S, d->stream, true);
    CUDA_TRY(cudaMemcpyAsync(S.vol0, S.vol, sizeof(double) * ne, cudaMemcpyDeviceToDevice,
                             d->stream));
    fp64_density(P, S, d->rho0_dev, d->stream);
    fp64_nodal(P, S, d->stream, 1);
  }
  CUDA_TRY(cudaGetLastError());
  if (!fp64) {
    MixState &M = d->M;
    CUDA_TRY(dalloc(d, &M.xh, 3 * np));
    CUDA_TRY(dalloc(d, &M.x0, 3 * np));
    CUDA_TRY(dalloc(d, &M.v, 3 * np));
    CUDA_TRY(dalloc(d, &M.vp, 3 * np));
    CUDA_TRY(dalloc(d, &M.pa, 3 * np));
    CUDA_TRY(dalloc(d, &M.cf, 3 * np));
    CUDA_TRY(dalloc(d, &M.ut, 3 * np));
    CUDA_TRY(dalloc(d, &M.cfn, d->tri ? np : 1));
    if (d->thermal) {
      // temperature as a compensated pair (T0 split into hi + lo)
      const float hi = (float)d->T0;
      CUDA_TRY(upload(d, &M.T, std::vector<float2>(np, make_float2(hi, (float)(d->T0 - hi)))));
      CUDA_TRY(dalloc(d, &M.qc, np));
      CUDA_TRY(dalloc(d, &M.dte, 2 * ne * d->npe));
      P.f_cp0 = (float)P.cp0;
    }
    if (d->tri) {
      // FP32 die copies relative to the centre of the part's bounding box
      {
        const wf_status hs = host_mesh(d);
        if (hs) return hs;
      }
      double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
      for (int64_t n = 0; n < nn; n++)
        for (int k = 0; k < 3; k++) {
          lo[k] = std::min(lo[k], d->x[3 * n + k]);
          hi[k] = std::max(hi[k], d->x[3 * n + k]);
        }
      for (int k = 0; k < 3; k++) P.tri_ref[k] = 0.5 * (lo[k] + hi[k]);
      std::vector<double> nrm, pp;
      tri_normals_planes(d->tri_x, d->tri_el, nrm, pp);
      const size_t tn = d->tri_x.size() / 3, te = d->tri_el.size() / 3;
      std::vector<float> xf(3 * tn), nf(3 * te), ppf(te);
      for (size_t i = 0; i < 3 * tn; i++) xf[i] = (float)(d->tri_x[i] - P.tri_ref[i % 3]);
      for (size_t e = 0; e < te; e++) {
        const double *p2 = &d->tri_x[3 * d->tri_el[3 * e + 2]];
        double q = 0.0;
        for (int k = 0; k < 3; k++) {
          nf[3 * e + k] = (float)nrm[3 * e + k];
          q += (p2[k] - P.tri_ref[k]) * nrm[3 * e + k];
        }
        ppf[e] = (float)q;
      }
      CUDA_TRY(upload(d, &P.tri_xf, xf));
      CUDA_TRY(upload(d, &P.tri_nf, nf));
      CUDA_TRY(upload(d, &P.tri_ppf, ppf));
    }
    CUDA_TRY(dalloc(d, &M.mass, np));
    CUDA_TRY(dalloc(d, &M.jr, np));
    CUDA_TRY(dalloc(d, &M.nc, np));
    CUDA_TRY(dalloc(d, &M.pls, ne));
    CUDA_TRY(dalloc(d, &M.tau, 6 * ne));
    CUDA_TRY(dalloc(d, &M.fe, (size_t)ne * d->npe * 3));
    if (d->energy) CUDA_TRY(dalloc(d, &M.edot, ne));
    CUDA_TRY(dalloc(d, &d->mvol, ne));
    std::vector<MatF> mf(md.size());
    for (size_t i = 0; i < md.size(); i++) {
      mf[i] = MatF{};
      mf[i].K = (float)md[i].K;
      mf[i].G = (float)md[i].G;
      mf[i].sy0 = (float)md[i].sy0;
      mf[i].H = (float)md[i].H;
      mf[i].cs0 = (float)md[i].cs0;
      mf[i].rho = (float)d->mats[i].rho;
      mf[i].hol_K = (float)md[i].hol_K;
      mf[i].hol_m = (float)md[i].hol_m;
      mf[i].eps0 = (float)md[i].eps0;
      mf[i].eps1 = (float)md[i].eps1;
      mf[i].jc_B = (float)md[i].jc_B;
      mf[i].jc_n = (float)md[i].jc_n;
      mf[i].jc_C = (float)md[i].jc_C;
      mf[i].jc_eps0 = (float)md[i].jc_eps0;
      mf[i].jc_Th = (float)md[i].jc_Th;
      mf[i].E = (float)md[i].E;
      mf[i].jc_m = (float)md[i].jc_m;
      mf[i].jc_Tm = (float)md[i].jc_Tm;
      mf[i].jc_Tt = (float)md[i].jc_Tt;
      mf[i].k_T = (float)md[i].k_T;
      mf[i].cp_T = (float)md[i].cp_T;
      mf[i].exp_T = (float)md[i].exp_T;
      if (md[i].model == WF_MAT_GMT) {
        const MatDev &g = md[i];
        mf[i].jc_Th = (float)g.g_T;
        const double *src[14] = {&g.g_C1, &g.g_C2, &g.g_n1, &g.g_n2, &g.g_m1, &g.g_m2, &g.g_I1,
                                 &g.g_I2, &g.g_emin, &g.g_emax, &g.g_rmin, &g.g_rmax, &g.g_Tmin,
                                 &g.g_Tmax};
        float *dst[14] = {&mf[i].g_C1, &mf[i].g_C2, &mf[i].g_n1, &mf[i].g_n2, &mf[i].g_m1,
                          &mf[i].g_m2, &mf[i].g_I1, &mf[i].g_I2, &mf[i].g_emin, &mf[i].g_emax,
                          &mf[i].g_rmin, &mf[i].g_rmax, &mf[i].g_Tmin, &mf[i].g_Tmax};
        // ranges past the float range (the class defaults are 1e10) stay
        // finite: FLT_MAX keeps their clamps inactive
        for (int q = 0; q < 14; q++) *dst[q] = (float)std::min(*src[q], (double)FLT_MAX);
        const double Tc = std::min(std::max(g.g_T, g.g_Tmin), g.g_Tmax);
        mf[i].g_A = (float)(g.g_C1 * std::exp(g.g_C2 * Tc));
        mf[i].g_n = (float)(g.g_n1 * Tc + g.g_n2);
        mf[i].g_I = (float)(g.g_I1 * Tc + g.g_I2);
        mf[i].g_q = (float)(g.g_m1 * Tc + g.g_m2);
      }
      mf[i].model = md[i].model;
    }
    MatF *mfd = nullptr;
    CUDA_TRY(upload(d, &mfd, mf));
    P.matf = mfd;
    P.f_alpha = (float)P.alpha;
    P.f_fcorr = (float)P.fcorr;
    P.f_hg_coef = (float)P.hg_coef;
    P.f_c_k = (float)P.c_k;
    P.f_c_mu = (float)P.c_mu;
    P.f_av0 = (float)P.av[0];
    P.f_av1 = (float)P.av[1];
    mix_init(P, M, S, d->mvol, d->rho0_dev, d->stream);
    CUDA_TRY(cudaGetLastError());
    d->mix_valid_fp64 = true;
    // element tiles of the tiled step (hexahedra; the kernels leave out
    // specimens, thermal coupling, the energy history and triangle-mesh dies)
    d->tiled = false;
    d->tile_why.clear();
    if (d->npe != 8) d->tile_why = "tetrahedra";
    else if (d->nspec) d->tile_why = "specimens";
    else if (P.thermal) d->tile_why = "thermal coupling";
    else if (P.energy_on) d->tile_why = "energy history";
    else if (P.tri_on) d->tile_why = "triangle-mesh contact";
    else if (d->step_mode != 3) d->tile_why = "step mode 3 not set before wf_init";
    if (d->tile_why.empty()) {
      double bb[6];
      {
        const wf_status hs = host_mesh(d);
        if (hs) return hs;
      }
      host_bbox(d, bb);
      CUDA_TRY(build_tiles(P.elnod, S.x, np, ne, nn, P.off, bb, kSharedThreads, keep_alloc, d,
                           d->stream, d->T, d->tile_why));
      d->tiled = d->tile_why.empty();
    }
    // the column sweep (box meshes of hexahedra; the kernel leaves out
    // specimens, thermal coupling and triangle-mesh dies): the second buffer
    // of each pair it reads for neighbouring columns, and the column partials
    d->sweep = false;
    d->sweep_why.clear();
    d->xh_pair[0] = M.xh;
    d->vp_pair[0] = M.vp;
    d->tau_pair[0] = M.tau;
    d->pls_pair[0] = M.pls;
    d->xh_pair[1] = nullptr;
    d->vp_pair[1] = d->tau_pair[1] = d->pls_pair[1] = nullptr;
    d->parity = 0;
    if (!P.box) d->sweep_why = "not a box mesh of hexahedra";
    else if (d->nspec) d->sweep_why = "specimens";
    else if (P.thermal) d->sweep_why = "thermal coupling";
    else if (P.tri_on) d->sweep_why = "triangle-mesh contact";
    // the dataflow step (same meshes): item table, counters, partials
    d->flow = false;
    d->flow_why = d->sweep_why;
    if (d->flow_why.empty()) {
      d->F = FlowParams{};
      d->F.grid = flow_grid(P);
      if (P.bz + d->flow_lag + 1 > kFlowMaxLayers + 19) {
        d->flow_why = "more element layers than the dataflow step's stage table holds";
      } else if (d->F.grid <= 0) {
        d->flow_why = "the dataflow kernel cannot launch on this device";
      } else {
        std::vector<int> first;
        flow_stages(P, d->flow_tile, d->flow_lag, kFlowSplit, first, d->F);
        int *fs = nullptr;
        CUDA_TRY(upload(d, &fs, first));
        d->F.stage_first = fs;
        for (int k = 0; k < 2; k++) {
          CUDA_TRY(dalloc(d, &d->flow_cnt[k], d->F.ncnt));
          CUDA_TRY(cudaMemsetAsync(d->flow_cnt[k], 0, sizeof(unsigned) * d->F.ncnt, d->stream));
        }
        CUDA_TRY(dalloc(d, &d->F.partials, (size_t)d->F.bz1 * d->F.ntiles[3]));
        d->flow_par = 0;
        d->flow = true;
      }
    }
    if (d->sweep_why.empty()) {
      d->W = SweepParams{};
      d->W.cy = d->sweep_rows;
      const int cols = sweep_columns(P, d->W);
      if (!sweep_fits(P, d->W)) {
        d->sweep_why = "the sweep kernel cannot launch on this device";
      } else {
        CUDA_TRY(dalloc(d, &d->xh_pair[1], 3 * np));
        CUDA_TRY(dalloc(d, &d->vp_pair[1], 3 * np));
        CUDA_TRY(dalloc(d, &d->tau_pair[1], 6 * ne));
        CUDA_TRY(dalloc(d, &d->pls_pair[1], ne));
        CUDA_TRY(dalloc(d, &d->W.partials, cols));
        d->sweep = true;
        set_parity(d, 0);
      }
    }
    if (d->autotune) {
      wf_status ts = autotune_launches(d);
      if (ts) return ts;
    }
    d->cl_blocks = d->cl_bs = 0;
    if (d->ne <= kClusterMaxElems && !d->nspec) {
      // the largest cluster (16 blocks needs the non-portable size) that
      // can be resident, at most one block per 32 elements
      for (int blocks : {16, 8, 4, 2, 1}) {
        if (blocks > 1 && (int64_t)blocks * 32 > d->ne) continue;
        const int64_t per = std::max((d->ne + blocks - 1) / blocks, (d->nn + blocks - 1) / blocks);
        const int bs = per <= 64 ? 64 : (per <= 128 ? 128 : 256);
        if (mix_cluster_fits(P, M, d->mvol, blocks, bs) >= 1) {
          d->cl_blocks = blocks;
          d->cl_bs = bs;
          CUDA_TRY(dalloc(d, &d->cl_part, (size_t)kClusterChunk * blocks));
          break;
        }
      }
    }
  }
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  if (d->init_stage) CUDA_TRY(cudaFreeAsync(d->init_stage, d->stream));
  d->init_stage = nullptr;
  d->initialized = true;
  d->host_step = 0;
  d->host_time = 0.0;
  d->launches = 0;
  d->graph_launches = 0;
  return WF_OK;
}

// ---- run --------------------------------------------------------------------------
namespace {

// One dataflow step: counts in the current counter set, zeroes the other.
void launch_flow(wf_domain *d) {
  if (d->F.split) {
    mix_geometry(d->P, d->M, d->mvol, d->stream, d->cfg[0]);
    mix_nodal(d->P, d->M, d->mvol, d->stream, d->cfg[1]);
  }
  d->F.cnt = d->flow_cnt[d->flow_par];
  d->F.cnt_next = d->flow_cnt[d->flow_par ^ 1];
  mix_flow(d->P, d->M, d->mvol, d->F, d->stream);
  d->flow_par ^= 1;
}

void launch_step(wf_domain *d) {
  const StepParams &P = d->P;
  if (d->precision == WF_FP64) {
    fp64_geometry(P, d->S, d->stream, false);
    fp64_nodal(P, d->S, d->stream, 0);
    fp64_elements(P, d->S, d->stream);
    fp64_nodes(P, d->S, d->stream, d->node_grid);
  } else if (tiled_mode(d)) {
    mix_geometry(P, d->M, d->mvol, d->stream, d->cfg[0]);
    mix_nodal(P, d->M, d->mvol, d->stream, d->cfg[1]);
    mix_tile(P, d->M, d->T, d->stream);
    mix_shared(P, d->M, d->T, d->stream);
  } else if (flow_mode(d)) {
    launch_flow(d);
  } else if (sweep_mode(d)) {
    mix_geometry(P, d->M, d->mvol, d->stream, d->cfg[0]);
    mix_nodal(P, d->M, d->mvol, d->stream, d->cfg[1]);
    mix_sweep(P, d->M, d->W, d->stream);
    set_parity(d, d->parity ^ 1);
  } else {
    mix_geometry(P, d->M, d->mvol, d->stream, d->cfg[0]);
    mix_nodal(P, d->M, d->mvol, d->stream, d->cfg[1]);
    mix_elements(P, d->M, d->mvol, d->stream, d->cfg[2]);
    mix_nodes(P, d->M, d->stream, d->node_grid);
  }
  if (P.nspec) spec_reaction(P, d->stream);
  if (P.energy_on) {
    if (d->precision == WF_FP64)
      energy_fp64(P, d->S, d->stream);
    else
      energy_mixed(P, d->M, d->stream);
  }
}

void launch_step_timed(wf_domain *d, cudaEvent_t *ev) {
  const StepParams &P = d->P;
  cudaEventRecord(ev[0], d->stream);
  if (d->precision == WF_FP64) {
    fp64_geometry(P, d->S, d->stream, false);
    cudaEventRecord(ev[1], d->stream);
    fp64_nodal(P, d->S, d->stream, 0);
    cudaEventRecord(ev[2], d->stream);
    fp64_elements(P, d->S, d->stream);
    cudaEventRecord(ev[3], d->stream);
    fp64_nodes(P, d->S, d->stream, d->node_grid);
  } else if (flow_mode(d)) {
    // the dataflow step is one kernel: timed as the element phase
    cudaEventRecord(ev[1], d->stream);
    cudaEventRecord(ev[2], d->stream);
    launch_flow(d);
    cudaEventRecord(ev[3], d->stream);
  } else {
    // the column sweep is timed as the element phase (the node phase then
    // times nothing but the energy history)
    const bool tl = tiled_mode(d), sw = !tl && sweep_mode(d);
    mix_geometry(P, d->M, d->mvol, d->stream, d->cfg[0]);
    cudaEventRecord(ev[1], d->stream);
    mix_nodal(P, d->M, d->mvol, d->stream, d->cfg[1]);
    cudaEventRecord(ev[2], d->stream);
    if (tl) mix_tile(P, d->M, d->T, d->stream);
    else if (sw) mix_sweep(P, d->M, d->W, d->stream);
    else mix_elements(P, d->M, d->mvol, d->stream, d->cfg[2]);
    cudaEventRecord(ev[3], d->stream);
    if (tl) mix_shared(P, d->M, d->T, d->stream);
    else if (sw) set_parity(d, d->parity ^ 1);
    else mix_nodes(P, d->M, d->stream, d->node_grid);
  }
  if (P.nspec) spec_reaction(P, d->stream);
  if (P.energy_on) {
    if (d->precision == WF_FP64)
      energy_fp64(P, d->S, d->stream);
    else
      energy_mixed(P, d->M, d->stream);
  }
  cudaEventRecord(ev[4], d->stream);
}

// Folds the recorded events into the per-phase sums (waits for them).
wf_status collect_phase_events(wf_domain *d) {
  for (size_t i = 0; i + 5 <= d->ev_used; i += 5) {
    CUDA_TRY(cudaEventSynchronize(d->ev_pool[i + 4]));
    for (int k = 0; k < 4; k++) {
      float ms = 0.f;
      CUDA_TRY(cudaEventElapsedTime(&ms, d->ev_pool[i + k], d->ev_pool[i + k + 1]));
      d->phase_ms[k] += ms;
    }
    d->phase_steps++;
  }
  d->ev_used = 0;
  return WF_OK;
}

// Time-step dependent constants (FP64 and their FP32 roundings).
void set_dt_constants(StepParams &P, double dt) {
  P.dt = dt;
  P.f_dt = (float)dt;
  P.f_cu_pred = (float)((0.5 - P.beta) * dt);
  P.f_cu_corr = (float)(P.beta * dt * dt);
  P.f_cv_corr = (float)(P.gamma * dt);
  P.f_cv_pred = (float)((1.0 - P.gamma) * dt);
}

constexpr int kGraphSteps = 32;

// The graph of `steps` consecutive steps from the current buffer parity
// (captured and instantiated on first use; kept until the launch parameters
// change). Capturing launches nothing: the parity the captured steps advance
// is put back, and launch_graph advances it.
wf_status ensure_graph(wf_domain *d, int64_t steps, cudaGraphExec_t *out) {
  const int64_t key = 4 * steps + 2 * d->flow_par + d->parity;
  auto it = d->graphs.find(key);
  if (it != d->graphs.end()) {
    *out = it->second;
    return WF_OK;
  }
  const int parity = d->parity, flow_par = d->flow_par;
  cudaGraph_t g = nullptr;
  CUDA_TRY(cudaStreamBeginCapture(d->stream, cudaStreamCaptureModeThreadLocal));
  for (int64_t i = 0; i < steps; i++) launch_step(d);
  cudaError_t e = cudaStreamEndCapture(d->stream, &g);
  if (d->sweep) set_parity(d, parity);
  d->flow_par = flow_par;
  if (e != cudaSuccess) return fail(d, WF_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
  cudaGraphExec_t x = nullptr;
  e = cudaGraphInstantiate(&x, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(d, WF_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
  d->graphs[key] = x;
  *out = x;
  return WF_OK;
}

// Replays a graph of `steps` steps captured by ensure_graph at the current
// parity.
wf_status launch_graph(wf_domain *d, cudaGraphExec_t g, int64_t steps) {
  CUDA_TRY(cudaGraphLaunch(g, d->stream));
  if (flow_mode(d) && (steps & 1)) d->flow_par ^= 1;
  else if (sweep_mode(d) && (steps & 1)) set_parity(d, d->parity ^ 1);
  d->graph_launches++;
  return WF_OK;
}

// Grows the device histories (reaction, per-specimen reactions, energies) to
// hold `total` steps, keeping what is recorded so far.
wf_status grow_history(wf_domain *d, int64_t total) {
  if (total > d->hist_cap) {
    // grow the reaction history (device copy of what is recorded so far)
    int64_t cap = d->hist_cap;
    while (cap < total) cap *= 2;
    double *nh = nullptr;
    CUDA_TRY(dalloc(d, &nh, cap));
    CUDA_TRY(cudaMemcpyAsync(nh, d->P.hist, sizeof(double) * d->hist_cap, cudaMemcpyDeviceToDevice,
                             d->stream));
    d->P.hist = nh;
    if (d->nspec) {
      double *ns = nullptr;
      CUDA_TRY(dalloc(d, &ns, (size_t)cap * d->nspec));
      CUDA_TRY(cudaMemcpyAsync(ns, d->P.hist_spec, sizeof(double) * d->hist_cap * d->nspec,
                               cudaMemcpyDeviceToDevice, d->stream));
      d->P.hist_spec = ns;
    }
    if (d->P.energy_on) {
      for (double **h : {&d->P.ekin_hist, &d->P.eint_hist}) {
        double *nh2 = nullptr;
        CUDA_TRY(dalloc(d, &nh2, cap));
        CUDA_TRY(cudaMemcpyAsync(nh2, *h, sizeof(double) * d->hist_cap, cudaMemcpyDeviceToDevice,
                                 d->stream));
        *h = nh2;
      }
    }
    d->P.hist_cap = cap;
    d->hist_cap = cap;
    drop_graphs(d);
  }
  return WF_OK;
}

}  // namespace

WF_API wf_status wf_run(wf_domain *d, int64_t nsteps) {
  if (!d || nsteps < 0) return WF_ERR_ARG;
  if (!d->initialized) return fail(d, WF_ERR_STATE, "wf_init not called");
  if (nsteps == 0) return WF_OK;
  CUDA_TRY(cudaSetDevice(d->device));
  {
    const wf_status gs = grow_history(d, d->host_step + nsteps);
    if (gs) return gs;
  }
  if (!(d->dt > 0.0) && !d->nspec) return fail(d, WF_ERR_STATE, "time step not set (SetDT)");
  set_dt_constants(d->P, d->dt);
  if (d->precision == WF_FP64)
    fp64_predict(d->P, d->S, d->stream);
  else
    mix_predict(d->P, d->M, d->stream);
  CUDA_TRY(cudaGetLastError());
  d->launches += 1;
  int64_t left = nsteps;
  if (d->phase_timing) {
    for (int64_t i = 0; i < nsteps; i++) {
      if (d->ev_used + 5 > d->ev_pool.size()) {
        wf_status cs = collect_phase_events(d);
        if (cs) return cs;
        if (d->ev_pool.size() < 5 * 256) {
          while (d->ev_pool.size() < 5 * 256) {
            cudaEvent_t ev;
            CUDA_TRY(cudaEventCreate(&ev));
            d->ev_pool.push_back(ev);
          }
        }
      }
      launch_step_timed(d, &d->ev_pool[d->ev_used]);
      d->ev_used += 5;
    }
    left = 0;
  }
  if (d->step_mode == 3 && !tiled_mode(d))
    return fail(d, WF_ERR_UNSUPPORTED, "tiled steps need mixed precision and a mesh the tiles "
                                       "cover (%s)", d->tile_why.c_str());
  if (d->step_mode == 5 && !flow_mode(d))
    return fail(d, WF_ERR_UNSUPPORTED, "the dataflow step needs mixed precision and a box mesh "
                                       "of hexahedra (%s)",
                d->precision != WF_MIXED ? "FP64 step" : d->flow_why.c_str());
  if (d->step_mode == 4 && !sweep_mode(d))
    return fail(d, WF_ERR_UNSUPPORTED, "the column sweep needs mixed precision and a box mesh "
                                       "of hexahedra (%s)",
                d->precision != WF_MIXED ? "FP64 step" : d->sweep_why.c_str());
  if (d->step_mode == 2 && !cluster_mode(d))
    return fail(d, WF_ERR_UNSUPPORTED,
                "the cluster run needs mixed precision, a mesh of at most %lld elements, and no "
                "specimens, energy history or phase timing", (long long)kClusterMaxElems);
  if (cluster_mode(d)) {
    // one launch per chunk of steps (kernels stay short)
    while (left > 0) {
      const int64_t chunk = std::min<int64_t>(left, kClusterChunk);
      CUDA_TRY(mix_cluster_run(d->P, d->M, d->mvol, d->cl_part, chunk, d->cl_blocks, d->cl_bs,
                               d->stream));
      d->launches += 1;
      left -= chunk;
    }
  }
  // the split dataflow step launches the geometry and nodal kernels first
  const int per_step = flow_mode(d) ? (d->F.split ? 3 : 1) : (sweep_mode(d) ? 3 : 4);
  d->launches += (per_step + (d->nspec ? 1 : 0) + (d->P.energy_on ? 1 : 0)) * left;
  // graph replays: kGraphSteps at a time, then one graph of the remainder
  if (left >= kGraphSteps) {
    cudaGraphExec_t g = nullptr;
    wf_status s = ensure_graph(d, kGraphSteps, &g);
    if (s) return s;
    while (left >= kGraphSteps) {
      s = launch_graph(d, g, kGraphSteps);
      if (s) return s;
      left -= kGraphSteps;
    }
  }
  if (left > 1) {
    cudaGraphExec_t g = nullptr;
    wf_status s = ensure_graph(d, left, &g);
    if (s) return s;
    s = launch_graph(d, g, left);
    if (s) return s;
    left = 0;
  }
  for (int64_t i = 0; i < left; i++) launch_step(d);
  CUDA_TRY(cudaGetLastError());
  // the step state (its non-finite flag) for the next wf_sync to check
  CUDA_TRY(cudaMemcpyAsync(d->st_host, d->P.st, sizeof(StepState), cudaMemcpyDeviceToHost,
                           d->stream));
  d->st_pending = true;
  for (int64_t i = 0; i < nsteps; i++) d->host_time += d->dt;
  d->host_step += nsteps;
  d->mix_valid_fp64 = false;
  return WF_OK;
}

WF_API wf_status wf_prepare_run(wf_domain *d, int64_t nsteps) {
  if (!d || nsteps < 0) return WF_ERR_ARG;
  if (!d->initialized) return fail(d, WF_ERR_STATE, "wf_init not called");
  if (!(d->dt > 0.0) && !d->nspec) return fail(d, WF_ERR_STATE, "time step not set (SetDT)");
  if (d->phase_timing || cluster_mode(d)) return WF_OK;   // these runs replay no graph
  CUDA_TRY(cudaSetDevice(d->device));
  {
    const wf_status gs = grow_history(d, d->host_step + nsteps);
    if (gs) return gs;
  }
  set_dt_constants(d->P, d->dt);
  cudaGraphExec_t g = nullptr;
  if (nsteps >= kGraphSteps) {
    const wf_status s = ensure_graph(d, kGraphSteps, &g);
    if (s) return s;
  }
  const int64_t rem = nsteps % kGraphSteps;
  if (rem > 1) {
    const wf_status s = ensure_graph(d, rem, &g);
    if (s) return s;
  }
  return WF_OK;
}

// ---- step halves and halo data (slab decomposition) ------------------------------
namespace {
wf_status need_halves(wf_domain *d) {
  if (!d) return WF_ERR_ARG;
  if (!d->initialized) return fail(d, WF_ERR_STATE, "wf_init not called");
  if (d->nspec || d->thermal || d->P.tri_on || d->P.energy_on)
    return fail(d, WF_ERR_UNSUPPORTED, "step halves need a step without specimens, thermal "
                                       "coupling, triangle-mesh contact or energies");
  if (!(d->dt > 0.0)) return fail(d, WF_ERR_STATE, "time step not set (SetDT)");
  return WF_OK;
}
}  // namespace

WF_API wf_status wf_step_begin(wf_domain *d) {
  wf_status s = need_halves(d);
  if (s) return s;
  if (d->half_open) return fail(d, WF_ERR_STATE, "wf_step_end not called after wf_step_begin");
  CUDA_TRY(cudaSetDevice(d->device));
  if ((s = grow_history(d, d->host_step + 1))) return s;
  set_dt_constants(d->P, d->dt);
  const StepParams &P = d->P;
  if (d->precision == WF_FP64) {
    fp64_predict(P, d->S, d->stream);
    fp64_geometry(P, d->S, d->stream, false);
    fp64_nodal(P, d->S, d->stream, 0);
    fp64_elements(P, d->S, d->stream);
  } else {
    // the mixed per-phase kernels, whatever the step mode of wf_run
    mix_predict(P, d->M, d->stream);
    mix_geometry(P, d->M, d->mvol, d->stream, d->cfg[0]);
    mix_nodal(P, d->M, d->mvol, d->stream, d->cfg[1]);
    mix_elements(P, d->M, d->mvol, d->stream, d->cfg[2]);
    d->mix_valid_fp64 = false;
  }
  CUDA_TRY(cudaGetLastError());
  d->launches += 4;
  d->half_open = true;
  return WF_OK;
}

WF_API wf_status wf_step_end(wf_domain *d) {
  wf_status s = need_halves(d);
  if (s) return s;
  if (!d->half_open) return fail(d, WF_ERR_STATE, "wf_step_begin not called");
  CUDA_TRY(cudaSetDevice(d->device));
  if (d->precision == WF_FP64)
    fp64_nodes(d->P, d->S, d->stream, d->node_grid);
  else
    mix_nodes(d->P, d->M, d->stream, d->node_grid);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(d->st_host, d->P.st, sizeof(StepState), cudaMemcpyDeviceToHost,
                           d->stream));
  d->st_pending = true;
  d->launches += 1;
  d->half_open = false;
  d->host_time += d->dt;
  d->host_step += 1;
  return WF_OK;
}

WF_API wf_status wf_get_halo_forces(wf_domain *d, int64_t e0, int64_t e1, double *out) {
  wf_status s = need_halves(d);
  if (s) return s;
  if (!out || e0 < 0 || e1 > d->ne || e0 > e1) return WF_ERR_ARG;
  CUDA_TRY(cudaSetDevice(d->device));
  const size_t k = (size_t)(e1 - e0) * d->npe * 3, at = (size_t)e0 * d->npe * 3;
  if (d->precision == WF_MIXED) {
    // FP32 forces (element force minus hourglass force) [npe * 3][ne]: the
    // element range of every (corner, component) row, widened exactly; the
    // second half (the FP64 step's hourglass forces) is zero
    const size_t m = (size_t)(e1 - e0), rows = (size_t)d->npe * 3;
    std::vector<float> h(rows * m);
    CUDA_TRY(cudaMemcpy2DAsync(h.data(), sizeof(float) * m, d->M.fe + e0,
                               sizeof(float) * d->ne, sizeof(float) * m, rows,
                               cudaMemcpyDeviceToHost, d->stream));
    CUDA_TRY(cudaStreamSynchronize(d->stream));
    for (size_t i = 0; i < rows * m; i++) out[i] = (double)h[i];
    std::fill(out + k, out + 2 * k, 0.0);
    d->d2h_bytes += (int64_t)(sizeof(float) * rows * m);
    return WF_OK;
  }
  CUDA_TRY(cudaMemcpyAsync(out, d->S.fe + at, sizeof(double) * k, cudaMemcpyDeviceToHost,
                           d->stream));
  if (d->S.fhg)
    CUDA_TRY(cudaMemcpyAsync(out + k, d->S.fhg + at, sizeof(double) * k, cudaMemcpyDeviceToHost,
                             d->stream));
  else
    std::fill(out + k, out + 2 * k, 0.0);
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  d->d2h_bytes += (int64_t)(sizeof(double) * 2 * k);
  return WF_OK;
}

WF_API wf_status wf_set_halo_forces(wf_domain *d, int64_t e0, int64_t e1, const double *in) {
  wf_status s = need_halves(d);
  if (s) return s;
  if (!in || e0 < 0 || e1 > d->ne || e0 > e1) return WF_ERR_ARG;
  CUDA_TRY(cudaSetDevice(d->device));
  const size_t k = (size_t)(e1 - e0) * d->npe * 3, at = (size_t)e0 * d->npe * 3;
  if (d->precision == WF_MIXED) {
    const size_t m = (size_t)(e1 - e0), rows = (size_t)d->npe * 3;
    std::vector<float> h(rows * m);
    for (size_t i = 0; i < rows * m; i++) h[i] = (float)in[i];
    CUDA_TRY(cudaMemcpy2DAsync(d->M.fe + e0, sizeof(float) * d->ne, h.data(), sizeof(float) * m,
                               sizeof(float) * m, rows, cudaMemcpyHostToDevice, d->stream));
    CUDA_TRY(cudaStreamSynchronize(d->stream));
    d->h2d_bytes += (int64_t)(sizeof(float) * rows * m);
    return WF_OK;
  }
  CUDA_TRY(cudaMemcpyAsync(d->S.fe + at, in, sizeof(double) * k, cudaMemcpyHostToDevice,
                           d->stream));
  if (d->S.fhg)
    CUDA_TRY(cudaMemcpyAsync(d->S.fhg + at, in + k, sizeof(double) * k, cudaMemcpyHostToDevice,
                             d->stream));
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  d->h2d_bytes += (int64_t)(sizeof(double) * 2 * k);
  return WF_OK;
}

namespace {
// The node state a halo carries between steps: x, v, prev_a, u (SoA fields).
void halo_fields(wf_domain *d, double *f[4]) {
  f[0] = d->S.x;
  f[1] = d->S.v;
  f[2] = d->S.pa;
  f[3] = d->S.u;
}

// The mixed step's node state between steps, 18 values per node as doubles
// (exact): positions hi and lo, velocity, previous acceleration, predicted
// velocity, contact slip; read into out or written from in.
wf_status mixed_halo_nodes(wf_domain *d, int64_t n0, int64_t n1, double *out, const double *in) {
  const size_t m = (size_t)(n1 - n0);
  const int64_t np = d->np;
  std::vector<float2> xh(3 * m);
  std::vector<float> f(12 * m);
  float *rows[4] = {d->M.v, d->M.pa, d->M.vp, d->M.ut};
  if (out) {
    for (int k = 0; k < 3; k++)
      CUDA_TRY(cudaMemcpyAsync(xh.data() + k * m, d->M.xh + k * np + n0, sizeof(float2) * m,
                               cudaMemcpyDeviceToHost, d->stream));
    for (int q = 0; q < 4; q++)
      for (int k = 0; k < 3; k++)
        CUDA_TRY(cudaMemcpyAsync(f.data() + (3 * q + k) * m, rows[q] + k * np + n0,
                                 sizeof(float) * m, cudaMemcpyDeviceToHost, d->stream));
    CUDA_TRY(cudaStreamSynchronize(d->stream));
    for (size_t i = 0; i < 3 * m; i++) {
      out[i] = (double)xh[i].x;
      out[3 * m + i] = (double)xh[i].y;
    }
    for (size_t i = 0; i < 12 * m; i++) out[6 * m + i] = (double)f[i];
    d->d2h_bytes += (int64_t)(sizeof(float) * 18 * m);
    return WF_OK;
  }
  for (size_t i = 0; i < 3 * m; i++) xh[i] = make_float2((float)in[i], (float)in[3 * m + i]);
  for (size_t i = 0; i < 12 * m; i++) f[i] = (float)in[6 * m + i];
  for (int k = 0; k < 3; k++)
    CUDA_TRY(cudaMemcpyAsync(d->M.xh + k * np + n0, xh.data() + k * m, sizeof(float2) * m,
                             cudaMemcpyHostToDevice, d->stream));
  for (int q = 0; q < 4; q++)
    for (int k = 0; k < 3; k++)
      CUDA_TRY(cudaMemcpyAsync(rows[q] + k * np + n0, f.data() + (3 * q + k) * m,
                               sizeof(float) * m, cudaMemcpyHostToDevice, d->stream));
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  d->h2d_bytes += (int64_t)(sizeof(float) * 18 * m);
  d->mix_valid_fp64 = false;
  return WF_OK;
}
}  // namespace

WF_API wf_status wf_get_halo_node_width(const wf_domain *d, int32_t *values_per_node) {
  if (!d || !values_per_node) return WF_ERR_ARG;
  *values_per_node = d->precision == WF_MIXED ? 18 : 12;
  return WF_OK;
}

WF_API wf_status wf_get_halo_nodes(wf_domain *d, int64_t n0, int64_t n1, double *out) {
  wf_status s = need_halves(d);
  if (s) return s;
  if (!out || n0 < 0 || n1 > d->nn || n0 > n1) return WF_ERR_ARG;
  CUDA_TRY(cudaSetDevice(d->device));
  if (d->precision == WF_MIXED) return mixed_halo_nodes(d, n0, n1, out, nullptr);
  double *f[4];
  halo_fields(d, f);
  const size_t m = (size_t)(n1 - n0);
  for (int q = 0; q < 4; q++)
    for (int k = 0; k < 3; k++)
      CUDA_TRY(cudaMemcpyAsync(out + (3 * q + k) * m, f[q] + k * d->np + n0, sizeof(double) * m,
                               cudaMemcpyDeviceToHost, d->stream));
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  d->d2h_bytes += (int64_t)(sizeof(double) * 12 * m);
  return WF_OK;
}

WF_API wf_status wf_set_halo_nodes(wf_domain *d, int64_t n0, int64_t n1, const double *in) {
  wf_status s = need_halves(d);
  if (s) return s;
  if (!in || n0 < 0 || n1 > d->nn || n0 > n1) return WF_ERR_ARG;
  CUDA_TRY(cudaSetDevice(d->device));
  if (d->precision == WF_MIXED) return mixed_halo_nodes(d, n0, n1, nullptr, in);
  double *f[4];
  halo_fields(d, f);
  const size_t m = (size_t)(n1 - n0);
  for (int q = 0; q < 4; q++)
    for (int k = 0; k < 3; k++)
      CUDA_TRY(cudaMemcpyAsync(f[q] + k * d->np + n0, in + (3 * q + k) * m, sizeof(double) * m,
                               cudaMemcpyHostToDevice, d->stream));
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  d->h2d_bytes += (int64_t)(sizeof(double) * 12 * m);
  return WF_OK;
}

WF_API wf_status wf_solve(wf_domain *d, int64_t *nsteps) {
  if (!d) return WF_ERR_ARG;
  if (!d->initialized) return fail(d, WF_ERR_STATE, "wf_init not called");
  if (d->nspec) return fail(d, WF_ERR_UNSUPPORTED, "a batched ensemble runs with wf_run");
  // count the iterations of `while (Time < end_t) { ...; Time += dt; }`
  int64_t n = 0;
  double t = d->host_time;
  while (t < d->end_t) {
    t += d->dt;
    n++;
  }
  wf_status s = wf_run(d, n);
  if (nsteps) *nsteps = n;
  if (s) return s;
  return wf_sync(d);
}

WF_API wf_status wf_sync(wf_domain *d) {
  if (!d) return WF_ERR_ARG;
  CUDA_TRY(cudaSetDevice(d->device));
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  if (d->st_pending && d->st_host) {
    // Solver_explicit.C:777-785 clears a non-finite internal force and
    // prints it; here the node kernels clear it the same way and raise a
    // flag, reported once by this call and then reset on the device
    d->st_pending = false;
    const StepState st = *d->st_host;
    if (st.status & 2u) {
      d->st_host->status &= ~2u;
      CUDA_TRY(cudaMemcpy(&d->P.st->status, &d->st_host->status, sizeof(unsigned),
                          cudaMemcpyHostToDevice));
      return fail(d, WF_ERR_TIMEOUT, "a dependency wait of the dataflow step ran out, in the "
                                     "steps up to step %lld", (long long)st.step);
    }
    if (st.status & 1u) {
      d->st_host->status = 0u;
      d->st_host->first_bad_node = LLONG_MAX;
      CUDA_TRY(cudaMemcpy(&d->P.st->status, &d->st_host->status,
                          offsetof(StepState, first_bad_node) + sizeof(long long) -
                              offsetof(StepState, status),
                          cudaMemcpyHostToDevice));
      return fail(d, WF_ERR_NONFINITE,
                  "non-finite internal force cleared to zero (first at node %lld), in the "
                  "steps up to step %lld",
                  (long long)st.first_bad_node, (long long)st.step);
    }
  }
  return WF_OK;
}

WF_API wf_status wf_get_time(const wf_domain *d, double *t, int64_t *step) {
  if (!d) return WF_ERR_ARG;
  if (t) *t = d->host_time;
  if (step) *step = d->host_step;
  return WF_OK;
}

WF_API wf_status wf_min_edge_length(wf_domain *d, double *hmin) {
  wf_status s = need_mesh(d);
  if (s) return s;
  if (!hmin) return WF_ERR_ARG;
  if (!d->initialized) return fail(d, WF_ERR_STATE, "wf_init not called");
  CUDA_TRY(cudaSetDevice(d->device));
  if (!d->edge_min) CUDA_TRY(dalloc(d, &d->edge_min, 1));
  double *out = d->edge_min;
  if (d->precision == WF_MIXED && !d->mix_valid_fp64) {
    mix_export(d->P, d->M, d->S, d->mvol, d->stream);
    d->mix_valid_fp64 = true;
  }
  if (d->P.box)
    min_edge_length_box(d->S.x, d->np, d->P.bx, d->P.by, d->P.bz, out, d->stream);
  else
    min_edge_length(d->P.elnod, d->S.x, d->np, d->ne, d->npe, out, d->stream);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(hmin, out, sizeof(double), cudaMemcpyDeviceToHost, d->stream));
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  return WF_OK;
}

// ---- readback --------------------------------------------------------------------
namespace {

wf_status ready_for_readback(wf_domain *d) {
  if (!d) return WF_ERR_ARG;
  if (!d->initialized) return fail(d, WF_ERR_STATE, "wf_init not called");
  CUDA_TRY(cudaSetDevice(d->device));
  if (d->precision == WF_MIXED && !d->mix_valid_fp64) {
    mix_export(d->P, d->M, d->S, d->mvol, d->stream);
    CUDA_TRY(cudaGetLastError());
    d->mix_valid_fp64 = true;
  }
  return WF_OK;
}

// SoA [3][np] field -> caller's AoS [nn][3]: transposed on the device into
// a readback buffer kept with the domain, then one copy to the host.
wf_status copy_node3(wf_domain *d, const double *src, double *out) {
  if (!d->readback) CUDA_TRY(dalloc_raw(d, &d->readback, 3 * d->np));
  coords_aos(src, d->nn, d->np, d->readback, d->stream);
  CUDA_TRY(cudaGetLastError());
  const size_t bytes = sizeof(double) * 3 * d->nn;
  d->d2h_bytes += (int64_t)bytes;
  CUDA_TRY(cudaMemcpyAsync(out, d->readback, bytes, cudaMemcpyDeviceToHost, d->stream));
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  return WF_OK;
}

wf_status copy_plain(wf_domain *d, const double *src, double *out, size_t count) {
  d->d2h_bytes += (int64_t)(sizeof(double) * count);
  CUDA_TRY(cudaMemcpyAsync(out, src, sizeof(double) * count, cudaMemcpyDeviceToHost, d->stream));
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  return WF_OK;
}

}  // namespace

WF_API wf_status wf_get_node_field(wf_domain *d, int32_t field, double *out) {
  if (d && out && d->initialized && d->precision == WF_MIXED && !d->mix_valid_fp64 &&
      (field == WF_NODE_U || field == WF_NODE_X)) {
    // positions and displacements straight from the mixed state (no export
    // of the other fields)
    CUDA_TRY(cudaSetDevice(d->device));
    if (!d->readback) CUDA_TRY(dalloc_raw(d, &d->readback, 3 * d->np));
    mix_node_aos(d->P, d->M, field == WF_NODE_U, d->readback, d->stream);
    CUDA_TRY(cudaGetLastError());
    const size_t bytes = sizeof(double) * 3 * d->nn;
    d->d2h_bytes += (int64_t)bytes;
    CUDA_TRY(cudaMemcpyAsync(out, d->readback, bytes, cudaMemcpyDeviceToHost, d->stream));
    CUDA_TRY(cudaStreamSynchronize(d->stream));
    return WF_OK;
  }
  wf_status s = ready_for_readback(d);
  if (s) return s;
  if (!out) return WF_ERR_ARG;
  const Fp64State &S = d->S;
  switch (field) {
    case WF_NODE_X: return copy_node3(d, S.x, out);
    case WF_NODE_V: return copy_node3(d, S.v, out);
    case WF_NODE_A:  // after a step the reference's a equals prev_a
    case WF_NODE_PREV_A: return copy_node3(d, S.pa, out);
    case WF_NODE_U: return copy_node3(d, S.u, out);
    case WF_NODE_FI: return copy_node3(d, S.fi, out);
    case WF_NODE_CONTFORCE: return copy_node3(d, S.cf, out);
  }
  return fail(d, WF_ERR_ARG, "unknown node field %d", field);
}

WF_API wf_status wf_get_node_scalar(wf_domain *d, int32_t field, double *out) {
  wf_status s = ready_for_readback(d);
  if (s) return s;
  if (!out) return WF_ERR_ARG;
  // per-node arrays are padded to np entries: the first nn are the nodes
  if (field == WF_NODE_MASS || field == WF_NODE_VOLN)
    return copy_plain(d, field == WF_NODE_MASS ? d->S.mass : d->S.voln, out, d->nn);
  if (field == WF_NODE_TEMP) {
    if (!d->thermal) return fail(d, WF_ERR_STATE, "thermal coupling is off");
    return copy_plain(d, d->S.T, out, d->nn);
  }
  if (field == WF_NODE_PRESSURE) {
    // calcNodalPressureFromElemental (Mechanical.C:1187-1213), serial order
    s = host_mesh(d);
    if (s) return s;
    std::vector<double> p(d->ne), vol(d->ne);
    s = copy_plain(d, d->S.p, p.data(), d->ne);
    if (s) return s;
    s = copy_plain(d, d->S.vol, vol.data(), d->ne);
    if (s) return s;
    std::vector<double> acc(d->nn, 0.0);
    for (int64_t n = 0; n < d->nn; n++) out[n] = 0.0;
    for (int64_t e = 0; e < d->ne; e++)
      for (int a = 0; a < d->npe; a++) {
        int32_t nid = d->elnod[e * d->npe + a];
        out[nid] += p[e] * vol[e];
        acc[nid] += vol[e];
      }
    for (int64_t n = 0; n < d->nn; n++)
      if (acc[n] > 0.0) out[n] /= acc[n];
    return WF_OK;
  }
  return fail(d, WF_ERR_ARG, "unknown node scalar %d", field);
}

WF_API wf_status wf_get_elem_scalar(wf_domain *d, int32_t field, double *out) {
  wf_status s = ready_for_readback(d);
  if (s) return s;
  if (!out) return WF_ERR_ARG;
  const Fp64State &S = d->S;
  const double *src = nullptr;
  switch (field) {
    case WF_ELEM_VOL: src = S.vol; break;
    case WF_ELEM_VOL0: src = S.vol0; break;
    case WF_ELEM_DETJ: src = S.detJ; break;
    case WF_ELEM_P: src = S.p; break;
    case WF_ELEM_PL_STRAIN: src = S.pls; break;
    case WF_ELEM_SIGMA_Y: src = S.sy; break;
    case WF_ELEM_RHO: src = S.rho; break;
    default: return fail(d, WF_ERR_ARG, "unknown element scalar %d", field);
  }
  if (field == WF_ELEM_DETJ) {
    // refresh detJ for the current coordinates
    fp64_geometry(d->P, d->S, d->stream, true);
    CUDA_TRY(cudaGetLastError());
  }
  return copy_plain(d, src, out, d->ne);
}

WF_API wf_status wf_get_elem_tensor(wf_domain *d, int32_t field, double *out) {
  wf_status s = ready_for_readback(d);
  if (s) return s;
  if (!out) return WF_ERR_ARG;
  const Fp64State &S = d->S;
  const double *src = nullptr;
  switch (field) {
    case WF_ELEM_SIGMA: src = S.sig; break;
    case WF_ELEM_TAU: src = S.tau; break;
    case WF_ELEM_EPS: src = S.eps; break;
    case WF_ELEM_STR_RATE: src = S.sr; break;
    case WF_ELEM_ROT_RATE: src = S.rr; break;
    default: return fail(d, WF_ERR_ARG, "unknown element tensor %d", field);
  }
  if (!src) return fail(d, WF_ERR_UNSUPPORTED, "field not kept in mixed precision");
  std::vector<double> tmp(6 * d->ne);
  s = copy_plain(d, src, tmp.data(), 6 * d->ne);
  if (s) return s;
  for (int64_t e = 0; e < d->ne; e++)
    for (int c = 0; c < 6; c++) out[6 * e + c] = tmp[c * d->ne + e];
  return WF_OK;
}

WF_API wf_status wf_get_disp(wf_domain *d, double *out) { return wf_get_node_field(d, WF_NODE_U, out); }
WF_API wf_status wf_get_vel(wf_domain *d, double *out) { return wf_get_node_field(d, WF_NODE_V, out); }
WF_API wf_status wf_get_pl_strain(wf_domain *d, double *out) {
  return wf_get_elem_scalar(d, WF_ELEM_PL_STRAIN, out);
}

// ---- VTK output: synchronous and from snapshots ---------------------------------
namespace {

// Offsets (in doubles) of the fields in a snapshot slot.
struct SnapLayout {
  size_t x, u, v, a, cf, mass, T, p, pl, vol, vol0, rho, sy, sig, sr, tri, count;
};

SnapLayout snap_layout(const wf_domain *d) {
  const size_t n3 = 3 * (size_t)d->nn, nn = d->nn, ne = d->ne;
  SnapLayout L{};
  size_t o = 0;
  L.x = o; o += n3;
  L.u = o; o += n3;
  L.v = o; o += n3;
  L.a = o; o += n3;
  L.cf = o; o += n3;
  L.mass = o; o += nn;
  L.T = o; o += d->thermal ? nn : 0;
  L.p = o; o += ne;
  L.pl = o; o += ne;
  L.vol = o; o += ne;
  L.vol0 = o; o += ne;
  L.rho = o; o += ne;
  L.sy = o; o += ne;
  L.sig = o; o += 6 * ne;
  L.sr = o; o += d->S.sr ? 6 * ne : 0;
  L.tri = o; o += d->P.tri_on ? 3 * (size_t)d->P.tri_nn : 0;
  L.count = o;
  return L;
}

// The static parts of a VTK view: connectivity, surface, die triangles.
wf_status vtk_static(wf_domain *d, VtkView &v) {
  {
    const wf_status hs = host_mesh(d);
    if (hs) return hs;
  }
  v.nn = d->nn;
  v.ne = d->ne;
  v.npe = d->npe;
  v.elnod = d->elnod.data();
  if (d->P.tri_on) {
    if (d->surf_ext.empty()) {
      std::vector<double> nodlen;
      part_surface(d, d->surf_ext, d->surf_area, nodlen);
    }
    v.ext = d->surf_ext.data();
    v.area = d->surf_area.data();
    v.tri_nn = d->P.tri_nn;
    v.tri_ne = d->P.tri_ne;
    v.tri_el = d->tri_el.data();
    v.T_die = d->tri_Tdie;
  }
  return WF_OK;
}

// The view's field pointers into one buffer of snapshot layout.
void vtk_fields(const wf_domain *d, const SnapLayout &L, const double *b, VtkView &v) {
  v.x = b + L.x;
  v.u = b + L.u;
  v.v = b + L.v;
  v.a = b + L.a;
  v.cf = b + L.cf;
  v.mass = b + L.mass;
  v.T = d->thermal ? b + L.T : nullptr;
  v.p = b + L.p;
  v.pl = b + L.pl;
  v.vol = b + L.vol;
  v.vol0 = b + L.vol0;
  v.rho = b + L.rho;
  v.sy = b + L.sy;
  v.sig = b + L.sig;
  v.sig_soa = true;
  v.sr = d->S.sr ? b + L.sr : nullptr;
  v.sr_soa = true;
  if (d->P.tri_on) v.tri_x = b + L.tri;
}

// Queues on the domain's stream the device copies of the state into dst
// (snapshot layout): node vectors transposed to AoS, the rest as stored.
wf_status queue_state_copy(wf_domain *d, const SnapLayout &L, double *dst) {
  const Fp64State &S = d->S;
  const int64_t nn = d->nn, np = d->np, ne = d->ne;
  const double *node3[5] = {S.x, S.u, S.v, S.pa, S.cf};
  const size_t off3[5] = {L.x, L.u, L.v, L.a, L.cf};
  for (int i = 0; i < 5; i++) coords_aos(node3[i], nn, np, dst + off3[i], d->stream);
  CUDA_TRY(cudaGetLastError());
  auto d2d = [&](size_t off, const double *src, size_t count) {
    return cudaMemcpyAsync(dst + off, src, sizeof(double) * count, cudaMemcpyDeviceToDevice,
                           d->stream);
  };
  CUDA_TRY(d2d(L.mass, S.mass, nn));
  if (d->thermal) CUDA_TRY(d2d(L.T, S.T, nn));
  CUDA_TRY(d2d(L.p, S.p, ne));
  CUDA_TRY(d2d(L.pl, S.pls, ne));
  CUDA_TRY(d2d(L.vol, S.vol, ne));
  CUDA_TRY(d2d(L.vol0, S.vol0, ne));
  CUDA_TRY(d2d(L.rho, S.rho, ne));
  CUDA_TRY(d2d(L.sy, S.sy, ne));
  CUDA_TRY(d2d(L.sig, S.sig, 6 * (size_t)ne));
  if (S.sr) CUDA_TRY(d2d(L.sr, S.sr, 6 * (size_t)ne));
  if (d->P.tri_on) CUDA_TRY(d2d(L.tri, d->P.tri_x, 3 * (size_t)d->P.tri_nn));
  return WF_OK;
}

}  // namespace

WF_API wf_status wf_write_vtk(wf_domain *d, const char *path) {
  if (!path) return WF_ERR_ARG;
  wf_status s = ready_for_readback(d);
  if (s) return s;
  // the same device copies a snapshot takes, read back at once
  const SnapLayout L = snap_layout(d);
  double *dev = nullptr;
  CUDA_TRY(cudaMalloc(&dev, sizeof(double) * std::max<size_t>(L.count, 1)));
  std::vector<double> host(L.count);
  s = queue_state_copy(d, L, dev);
  cudaError_t e = cudaSuccess;
  if (!s) e = cudaMemcpyAsync(host.data(), dev, sizeof(double) * L.count, cudaMemcpyDeviceToHost,
                              d->stream);
  if (!s && e == cudaSuccess) e = cudaStreamSynchronize(d->stream);
  cudaFree(dev);
  if (s) return s;
  if (e != cudaSuccess) return fail(d, WF_ERR_CUDA, "wf_write_vtk: %s", cudaGetErrorString(e));
  d->d2h_bytes += (int64_t)(sizeof(double) * L.count);
  VtkView v;
  s = vtk_static(d, v);
  if (s) return s;
  vtk_fields(d, L, host.data(), v);
  if (!write_vtk_text(path, v)) return fail(d, WF_ERR_ARG, "cannot write %s", path);
  return WF_OK;
}

WF_API wf_status wf_snapshot(wf_domain *d, int32_t *slot) {
  if (!slot) return WF_ERR_ARG;
  wf_status s = ready_for_readback(d);
  if (s) return s;
  int k = d->snap_next;
  if (d->snap[k].state != 0) k = 1 - k;
  if (d->snap[k].state != 0)
    return fail(d, WF_ERR_STATE, "both snapshot slots hold states not yet written");
  wf_domain::Snapshot &sn = d->snap[k];
  const SnapLayout L = snap_layout(d);
  if (!d->out_stream) CUDA_TRY(cudaStreamCreateWithFlags(&d->out_stream, cudaStreamNonBlocking));
  if (sn.count != L.count) {
    if (sn.dev) cudaFree(sn.dev);
    if (sn.host) cudaFreeHost(sn.host);
    sn.dev = nullptr;
    sn.host = nullptr;
    CUDA_TRY(cudaMalloc(&sn.dev, sizeof(double) * std::max<size_t>(L.count, 1)));
    CUDA_TRY(cudaMallocHost(&sn.host, sizeof(double) * std::max<size_t>(L.count, 1)));
    sn.count = L.count;
  }
  if (!sn.ready) CUDA_TRY(cudaEventCreateWithFlags(&sn.ready, cudaEventDisableTiming));
  if (!sn.done) CUDA_TRY(cudaEventCreateWithFlags(&sn.done, cudaEventDisableTiming));
  s = queue_state_copy(d, L, sn.dev);
  if (s) return s;
  CUDA_TRY(cudaEventRecord(sn.ready, d->stream));
  // the host copy runs on the output stream, beside the next steps
  CUDA_TRY(cudaStreamWaitEvent(d->out_stream, sn.ready, 0));
  CUDA_TRY(cudaMemcpyAsync(sn.host, sn.dev, sizeof(double) * L.count, cudaMemcpyDeviceToHost,
                           d->out_stream));
  CUDA_TRY(cudaEventRecord(sn.done, d->out_stream));
  d->d2h_bytes += (int64_t)(sizeof(double) * L.count);
  sn.state = 1;
  d->snap_next = 1 - k;
  *slot = k;
  return WF_OK;
}

WF_API wf_status wf_write_snapshot_vtk(wf_domain *d, int32_t slot, const char *path) {
  if (!d || !path || slot < 0 || slot > 1) return WF_ERR_ARG;
  wf_domain::Snapshot &sn = d->snap[slot];
  if (sn.state != 1) return fail(d, WF_ERR_STATE, "snapshot slot %d holds no state", slot);
  CUDA_TRY(cudaSetDevice(d->device));
  CUDA_TRY(cudaEventSynchronize(sn.done));
  const SnapLayout L = snap_layout(d);
  VtkView v;
  {
    const wf_status vs = vtk_static(d, v);
    if (vs) return vs;
  }
  vtk_fields(d, L, sn.host, v);
  sn.state = 0;
  if (!write_vtk_text(path, v)) return fail(d, WF_ERR_ARG, "cannot write %s", path);
  return WF_OK;
}

WF_API wf_status wf_get_reaction_history(wf_domain *d, double *out, int64_t cap, int64_t *n) {
  if (!d) return WF_ERR_ARG;
  if (!d->initialized) return fail(d, WF_ERR_STATE, "wf_init not called");
  CUDA_TRY(cudaSetDevice(d->device));
  const int64_t have = d->host_step;
  if (n) *n = have;
  const int64_t m = std::min(cap, have);
  if (out && m > 0) {
    d->d2h_bytes += (int64_t)(sizeof(double) * m);
    CUDA_TRY(cudaMemcpyAsync(out, d->P.hist, sizeof(double) * m, cudaMemcpyDeviceToHost, d->stream));
  }
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  return WF_OK;
}

WF_API wf_status wf_get_energy_history(wf_domain *d, double *ekin, double *eint, int64_t cap,
                                       int64_t *n) {
  if (!d || !n) return WF_ERR_ARG;
  if (!d->initialized) return fail(d, WF_ERR_STATE, "wf_init not called");
  if (!d->P.energy_on) return fail(d, WF_ERR_STATE, "energy history not enabled before init");
  CUDA_TRY(cudaSetDevice(d->device));
  *n = d->host_step;
  const int64_t m = std::min(cap, d->host_step);
  if (m > 0) {
    if (ekin) {
      CUDA_TRY(cudaMemcpyAsync(ekin, d->P.ekin_hist, sizeof(double) * m, cudaMemcpyDeviceToHost,
                               d->stream));
    }
    if (eint) {
      CUDA_TRY(cudaMemcpyAsync(eint, d->P.eint_hist, sizeof(double) * m, cudaMemcpyDeviceToHost,
                               d->stream));
    }
    d->d2h_bytes += (int64_t)(sizeof(double) * m * ((ekin ? 1 : 0) + (eint ? 1 : 0)));
  }
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  return WF_OK;
}

WF_API wf_status wf_set_node_state(wf_domain *d, const double *x, const double *v,
                                   const double *prev_a, const double *u) {
  if (!d) return WF_ERR_ARG;
  if (!d->initialized) return fail(d, WF_ERR_STATE, "wf_init not called");
  if (d->precision != WF_FP64)
    return fail(d, WF_ERR_UNSUPPORTED, "node state upload is FP64-only");
  CUDA_TRY(cudaSetDevice(d->device));
  const double *srcs[4] = {x, v, prev_a, u};
  double *dsts[4] = {d->S.x, d->S.v, d->S.pa, d->S.u};
  for (int i = 0; i < 4; i++) {
    if (!srcs[i]) continue;
    std::vector<double> soa(3 * d->np, 0.0);
    for (int64_t n = 0; n < d->nn; n++)
      for (int k = 0; k < 3; k++) soa[k * d->np + n] = srcs[i][3 * n + k];
    CUDA_TRY(cudaMemcpyAsync(dsts[i], soa.data(), sizeof(double) * 3 * d->np,
                             cudaMemcpyHostToDevice, d->stream));
    CUDA_TRY(cudaStreamSynchronize(d->stream));
  }
  return WF_OK;
}



WF_API wf_status wf_set_phase_timing(wf_domain *d, int32_t on) {
  if (!d) return WF_ERR_ARG;
  d->phase_timing = on != 0;
  return WF_OK;
}

WF_API wf_status wf_get_phase_times(wf_domain *d, double ms[4], int64_t *steps, int32_t reset) {
  if (!d || !ms) return WF_ERR_ARG;
  CUDA_TRY(cudaSetDevice(d->device));
  wf_status s = collect_phase_events(d);
  if (s) return s;
  for (int k = 0; k < 4; k++) ms[k] = d->phase_ms[k];
  if (steps) *steps = d->phase_steps;
  if (reset) {
    for (int k = 0; k < 4; k++) d->phase_ms[k] = 0.0;
    d->phase_steps = 0;
  }
  return WF_OK;
}

WF_API wf_status wf_get_launch_count(const wf_domain *d, int64_t *n) {
  if (!d || !n) return WF_ERR_ARG;
  *n = d->launches;
  return WF_OK;
}

WF_API wf_status wf_get_graph_launches(const wf_domain *d, int64_t *n) {
  if (!d || !n) return WF_ERR_ARG;
  *n = d->graph_launches;
  return WF_OK;
}

WF_API wf_status wf_get_stream(const wf_domain *d, void **stream) {
  if (!d || !stream) return WF_ERR_ARG;
  *stream = (void *)d->stream;
  return WF_OK;
}

WF_API wf_status wf_get_transfer_bytes(const wf_domain *d, int64_t *h2d, int64_t *d2h) {
  if (!d) return WF_ERR_ARG;
  if (h2d) *h2d = d->h2d_bytes;
  if (d2h) *d2h = d->d2h_bytes;
  return WF_OK;
}

// ---- adjoint ----------------------------------------------------------------------
namespace {

template <typename T>
cudaError_t adj_alloc(wf_domain *d, T **p, size_t count) {
  void *q = nullptr;
  cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess) return e;
  d->adj_allocs.push_back(q);
  *p = static_cast<T *>(q);
  return cudaMemsetAsync(q, 0, std::max<size_t>(count, 1) * sizeof(T), d->stream);
}

// Checkpoint c holds what the step reads and accumulates: x, v, prev_a, u,
// tau, eps, eps_p and the device step state (step index and Time).
wf_status ck_copy(wf_domain *d, int64_t c, bool save) {
  const size_t nb = sizeof(double) * 3 * d->np, eb = sizeof(double) * d->ne;
  double *node = d->ck_node + (size_t)c * 12 * d->np;
  double *elem = d->ck_elem + (size_t)c * 13 * d->ne;
  Fp64State &S = d->S;
  double *nf[4] = {S.x, S.v, S.pa, S.u};
  const auto kind = cudaMemcpyDeviceToDevice;
  for (int i = 0; i < 4; i++) {
    double *ck = node + (size_t)i * 3 * d->np;
    CUDA_TRY(cudaMemcpyAsync(save ? ck : nf[i], save ? nf[i] : ck, nb, kind, d->stream));
  }
  CUDA_TRY(cudaMemcpyAsync(save ? elem : S.tau, save ? S.tau : elem, 6 * eb, kind, d->stream));
  CUDA_TRY(cudaMemcpyAsync(save ? elem + 6 * d->ne : S.eps, save ? S.eps : elem + 6 * d->ne, 6 * eb,
                           kind, d->stream));
  CUDA_TRY(cudaMemcpyAsync(save ? elem + 12 * d->ne : S.pls, save ? S.pls : elem + 12 * d->ne, eb,
                           kind, d->stream));
  CUDA_TRY(cudaMemcpyAsync(save ? d->ck_st + c : d->P.st, save ? d->P.st : d->ck_st + c,
                           sizeof(StepState), kind, d->stream));
  return WF_OK;
}

wf_status adjoint_buffers(wf_domain *d) {
  if (d->adj_buffers) return WF_OK;
  const size_t np = d->np, ne = d->ne, seg = d->adj_every, npe = d->npe;
  AdjArgs &A = d->A;
  CUDA_TRY(adj_alloc(d, &A.sx, seg * 3 * np));
  CUDA_TRY(adj_alloc(d, &A.sv, seg * 3 * np));
  CUDA_TRY(adj_alloc(d, &A.spa, seg * 3 * np));
  CUDA_TRY(adj_alloc(d, &A.sjr, seg * np));
  CUDA_TRY(adj_alloc(d, &A.smass, seg * np));
  CUDA_TRY(adj_alloc(d, &A.sfi, seg * 3 * np));
  CUDA_TRY(adj_alloc(d, &A.stau, seg * 6 * ne));
  CUDA_TRY(adj_alloc(d, &A.spls, seg * ne));
  CUDA_TRY(adj_alloc(d, &A.X, 3 * np));
  CUDA_TRY(adj_alloc(d, &A.V, 3 * np));
  CUDA_TRY(adj_alloc(d, &A.PA, 3 * np));
  CUDA_TRY(adj_alloc(d, &A.T, 6 * ne));
  CUDA_TRY(adj_alloc(d, &A.EP, ne));
  CUDA_TRY(adj_alloc(d, &A.fib, 3 * np));
  CUDA_TRY(adj_alloc(d, &A.vpb, 3 * np));
  CUDA_TRY(adj_alloc(d, &A.mb, np));
  CUDA_TRY(adj_alloc(d, &A.sb, np));
  CUDA_TRY(adj_alloc(d, &A.cx, npe * 3 * ne));
  CUDA_TRY(adj_alloc(d, &A.cv, npe * 3 * ne));
  CUDA_TRY(adj_alloc(d, &A.cgeo, npe * 3 * ne));
  CUDA_TRY(adj_alloc(d, &A.cj, ne));
  CUDA_TRY(adj_alloc(d, &A.volb, ne));
  CUDA_TRY(adj_alloc(d, &A.gth, 3 * ne));
  CUDA_TRY(adj_alloc(d, &A.inv_s0, np));
  CUDA_TRY(adj_alloc(d, &A.dmds, np));
  CUDA_TRY(adj_alloc(d, &d->adj_seed, d->adj_steps));
  A.seed = d->adj_seed;
  A.s0 = d->S.s0;
  A.rho = d->S.rho;
  adj_node_constants(d->P, A, d->stream);
  CUDA_TRY(cudaGetLastError());
  d->adj_buffers = true;
  return WF_OK;
}

}  // namespace

namespace {

// FP64 steps from the current state with each step's inputs stashed in slots
// first..first+L-1 (the recompute of a segment, or the whole forward run when
// every step is kept).
void run_stashed(wf_domain *d, int64_t first, int64_t L) {
  const StepParams &P = d->P;
  const Fp64State &S = d->S;
  const AdjArgs &A = d->A;
  fp64_predict(P, S, d->stream);
  for (int64_t j = 0; j < L; j++) {
    adj_stash_state(P, S, A, (int)(first + j), d->stream);
    fp64_geometry(P, S, d->stream, false);
    fp64_nodal(P, S, d->stream, 0);
    fp64_elements(P, S, d->stream);
    fp64_nodes(P, S, d->stream, d->node_grid);
    if (P.energy_on) energy_fp64(P, S, d->stream);
    adj_stash_step(P, S, A, (int)(first + j), d->stream);
  }
  d->launches += 1 + (6 + (P.energy_on ? 1 : 0)) * L;
}

}  // namespace

WF_API wf_status wf_adjoint_forward(wf_domain *d, int64_t nsteps, int64_t every) {
  if (!d || nsteps <= 0 || every < -1) return WF_ERR_ARG;
  if (!d->initialized) return fail(d, WF_ERR_STATE, "wf_init not called");
  if (d->precision != WF_FP64)
    return fail(d, WF_ERR_UNSUPPORTED, "the adjoint records the FP64 step");
  if (d->contact || d->nspec || d->thermal || d->press_alg != 0 || d->av[0] != 0.0 ||
      d->av[1] != 0.0)
    return fail(d, WF_ERR_UNSUPPORTED, "the adjoint supports pressure algorithm 0 without contact, "
                                       "thermal coupling, artificial viscosity or specimens");
  const double *sp = &d->stab.alpha_free;
  for (int i = 0; i < 10; i++)
    if (sp[i] != 0.0) return fail(d, WF_ERR_UNSUPPORTED, "the adjoint supports default stabilisation");
  for (const wf_material &m : d->mats)
    if (m.model != WF_MAT_BILINEAR)
      return fail(d, WF_ERR_UNSUPPORTED, "the adjoint supports bilinear (linear hardening) materials");
  if (!(d->dt > 0.0)) return fail(d, WF_ERR_STATE, "time step not set (SetDT)");
  CUDA_TRY(cudaSetDevice(d->device));
  if (every == -1) {
    // keep every step's inputs: no checkpoints, no recompute in the reverse pass
    free_adjoint(d);
    const double need = (double)nsteps * (14.0 * d->np + 7.0 * d->ne) * sizeof(double);
    size_t free_b = 0, total_b = 0;
    CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    if (need > 0.9 * (double)free_b)
      return fail(d, WF_ERR_NOMEM, "keeping %lld steps needs %.1f GB, %.1f GB free: use checkpoints",
                  (long long)nsteps, need / 1e9, free_b / 1e9);
    d->adj_steps = nsteps;
    d->adj_every = nsteps;
    d->adj_nck = 0;
    d->adj_store_all = true;
    d->adj_first = d->host_step;
    wf_status s = adjoint_buffers(d);
    if (s) return s;
    s = grow_history(d, d->host_step + nsteps);
    if (s) return s;
    set_dt_constants(d->P, d->dt);
    run_stashed(d, 0, nsteps);
    CUDA_TRY(cudaGetLastError());
    for (int64_t i = 0; i < nsteps; i++) d->host_time += d->dt;
    d->host_step += nsteps;
    return WF_OK;
  }
  if (every == 0) every = std::max<int64_t>(1, (int64_t)std::llround(std::sqrt((double)nsteps)));
  every = std::min(every, nsteps);
  free_adjoint(d);
  const int64_t nck = (nsteps + every - 1) / every;
  CUDA_TRY(adj_alloc(d, &d->ck_node, (size_t)nck * 12 * d->np));
  CUDA_TRY(adj_alloc(d, &d->ck_elem, (size_t)nck * 13 * d->ne));
  CUDA_TRY(adj_alloc(d, &d->ck_st, nck));
  d->adj_first = d->host_step;
  for (int64_t c = 0; c < nck; c++) {
    wf_status s = ck_copy(d, c, true);
    if (s) return s;
    s = wf_run(d, std::min(every, nsteps - c * every));
    if (s) return s;
  }
  d->adj_steps = nsteps;
  d->adj_every = every;
  d->adj_nck = nck;
  return WF_OK;
}

WF_API wf_status wf_adjoint_backward(wf_domain *d, const double *dL_dR, int32_t reverse_fp32,
                                     double *grad) {
  if (!d || !dL_dR || !grad) return WF_ERR_ARG;
  if (d->adj_steps <= 0) return fail(d, WF_ERR_STATE, "wf_adjoint_forward not called");
  if (d->host_step != d->adj_first + d->adj_steps)
    return fail(d, WF_ERR_STATE, "the domain stepped after wf_adjoint_forward");
  CUDA_TRY(cudaSetDevice(d->device));
  wf_status s = adjoint_buffers(d);
  if (s) return s;
  const int64_t N = d->adj_steps, every = d->adj_every;
  const AdjArgs &A = d->A;
  const size_t np = d->np, ne = d->ne, npe = d->npe;
  CUDA_TRY(cudaMemcpyAsync(d->adj_seed, dL_dR, sizeof(double) * N, cudaMemcpyHostToDevice,
                           d->stream));
  d->h2d_bytes += (int64_t)(sizeof(double) * N);
  for (double *p : {A.X, A.V, A.PA})
    CUDA_TRY(cudaMemsetAsync(p, 0, sizeof(double) * 3 * np, d->stream));
  CUDA_TRY(cudaMemsetAsync(A.T, 0, sizeof(double) * 6 * ne, d->stream));
  CUDA_TRY(cudaMemsetAsync(A.EP, 0, sizeof(double) * ne, d->stream));
  CUDA_TRY(cudaMemsetAsync(A.cgeo, 0, sizeof(double) * npe * 3 * ne, d->stream));
  CUDA_TRY(cudaMemsetAsync(A.gth, 0, sizeof(double) * 3 * ne, d->stream));
  StepParams &P = d->P;
  set_dt_constants(P, d->dt);
  if (d->adj_store_all) {
    // every step's inputs are in the stash: reverse straight away
    for (int64_t j = N - 1; j >= 0; j--)
      adj_reverse_step(P, A, (int)j, j, 1, reverse_fp32 != 0, d->stream);
    CUDA_TRY(cudaGetLastError());
    d->launches += 4 * N;
  }
  for (int64_t c = d->adj_nck - 1; c >= 0; c--) {
    const int64_t c0 = c * every, L = std::min(every, N - c0);
    s = ck_copy(d, c, false);
    if (s) return s;
    // recompute the segment, stashing each step's inputs, then reverse it
    run_stashed(d, 0, L);
    for (int64_t j = L - 1; j >= 0; j--)
      adj_reverse_step(P, A, (int)j, c0 + j, 1, reverse_fp32 != 0, d->stream);
    CUDA_TRY(cudaGetLastError());
    d->launches += 4 * L;
  }
  // back to the state at the end of the forward run
  if (!d->adj_store_all) {
    const int64_t c = d->adj_nck - 1, L = N - c * every;
    s = ck_copy(d, c, false);
    if (s) return s;
    fp64_predict(P, d->S, d->stream);
    for (int64_t j = 0; j < L; j++) launch_step(d);
    CUDA_TRY(cudaGetLastError());
    d->launches += 1 + (4 + (P.energy_on ? 1 : 0)) * L;
  }
  // per-material sums of the element gradients, in element order
  std::vector<double> g(3 * ne);
  CUDA_TRY(cudaMemcpyAsync(g.data(), A.gth, sizeof(double) * 3 * ne, cudaMemcpyDeviceToHost,
                           d->stream));
  d->d2h_bytes += (int64_t)(sizeof(double) * 3 * ne);
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  const size_t nmat = d->mats.size();
  for (size_t i = 0; i < 3 * nmat; i++) grad[i] = 0.0;
  for (size_t e = 0; e < ne; e++) {
    const size_t m = d->emat.empty() ? 0 : (size_t)d->emat[e];
    for (int k = 0; k < 3; k++) grad[3 * m + k] += g[k * ne + e];
  }
  return WF_OK;
}
