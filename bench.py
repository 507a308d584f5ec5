"""Benchmark of the explicit step on the roofline workload (one JSON line).

Workload (default): the rigid-die compression case, 256 x 256 x 128
reduced-integration hexahedra (8,388,608 elements, 8,520,321 nodes, h = 1 mm,
interior nodes perturbed by +-0.1 h), viscous hourglass 0.1, penalty plane
contact with Coulomb friction 0.1, mixed precision (FP32 element arithmetic,
compensated positions, FP64 reaction sums). One "step" is one explicit time
step over the whole mesh. The same steps are run in FP64 for the
mixed/FP64 ratio and the error of the mixed path against FP64.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the CPU implementation of the reference's loop on
the host cores (the C restatement in oracle/, all cores) on a bounded
sample of the same workload and prints the same line with impl=reference.
Under torchrun (N > 1) the workload does not shard: every rank runs an
independent replica on its own GPU and the value is the total over ranks.
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from weldformfem_gb300 import workloads as W  # noqa: E402

METRIC = "element-steps/s"
UNIT = "element-steps/s"

# Algorithmic bytes per launch of each phase, per element (E) and per node (N)
# of the mixed-precision hexahedral kernels: every array touched once.
#   geometry: elnod 32 E + positions 24 N + volume 4 E
#   nodal   : offsets 4 N + slots 32 E + volume 4 E + node constants 8 N + J ratio, mass 8 N
#   elements: elnod 32 E + positions 24 N + predicted velocity 12 N + J ratio 4 N
#             + deviatoric stress RW 48 E + plastic strain RW 8 E + element forces 96 E
#   nodes   : offsets 4 N + slots 32 E + element forces 96 E + BC code, flags, mass 9 N
#             + positions RW 48 N + velocity RW 24 N + accel RW 24 N + predicted velocity 12 N
PHASES = ["geometry", "nodal", "elements", "nodes"]
ALG_BYTES_HEX_MIXED = {"geometry": (36, 24), "nodal": (36, 20), "elements": (184, 40),
                       "nodes": (128, 121)}
# tetrahedra: 4 nodes per element (elnod 16, slots 16, forces 48 B per element)
ALG_BYTES_TET_MIXED = {"geometry": (20, 24), "nodal": (20, 20), "elements": (120, 40),
                       "nodes": (64, 121)}
# box meshes: corners and node lists computed in the kernels (no elnod, slots
# or offsets read)
ALG_BYTES_HEX_MIXED_BOX = {"geometry": (4, 24), "nodal": (4, 16), "elements": (152, 40),
                           "nodes": (96, 117)}
KERNEL_NAMES = {"geometry": "k_mix_geometry", "nodal": "k_mix_nodal",
                "elements": "k_mix_elements", "nodes": "k_mix_nodes",
                "tile": "k_mix_tile", "shared": "k_mix_shared", "sweep": "k_mix_sweep",
                "flow": "k_mix_flow"}
TILED_PHASES = ["geometry", "nodal", "tile", "shared"]
# column sweep (box meshes): element and node phases in one kernel, the
# element forces kept in shared memory
#   sweep: deviatoric stress RW 48 E + plastic strain RW 8 E
#          + staged node inputs 40 N (positions 24, predicted velocity 12, J ratio 4)
#          + node update 93 N (BC code, flags, mass 9; velocity RW 24, accel RW 24;
#            positions 24 and predicted velocity 12 written)
ALG_BYTES_SWEEP = {"sweep": (56, 133)}
SWEEP_PHASES = ["geometry", "nodal", "sweep"]
# dataflow step (box meshes): the four phases in one persistent kernel; every
# array touched once, the intermediates written once (read back from L2)
#   flow: deviatoric stress RW 48 E + plastic strain RW 8 E + volume 4 E
#         + element forces 96 E; positions RW 48 N + predicted velocity RW 24 N
#         + velocity RW 24 N + accel RW 24 N + node constants 8 N + BC code and
#         flags 5 N + J ratio 4 N + mass 4 N
ALG_BYTES_FLOW = {"flow": (156, 141)}


def tiled_alg_bytes(E, N, stats):
    """Algorithmic bytes per launch of the tiled kernels, from the tile counts
    the library reports (tiles, shared nodes, sum of tile nodes, shared-node
    list entries):
      tile  : per tile node 4 (id) + 40 (positions 24, predicted velocity 12,
              volume ratio 4, staged once); per element 4 (id) + 16 (local
              corners) + 48 (deviatoric stress RW) + 8 (plastic strain RW);
              per shared incidence 12 (corner force to HBM); per interior node
              93 (velocity, acceleration, mass, BC code, flags read 33;
              positions, velocity, acceleration, predicted velocity written 60)
      shared: per shared node 4 (id) + 8 (list bounds) + 129 (node update 93,
              positions 24, predicted velocity 12); per list entry 4 + 12
              (slot, corner force)"""
    ntiles, nshared, tile_nodes, shared_slots = stats[:4]
    n_int = N - nshared
    tile = 44 * tile_nodes + 76 * E + 12 * (tile_nodes - n_int) + 93 * n_int
    shared = 141 * nshared + 16 * shared_slots
    return tile, shared


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region.

    nvidia-smi is started before the region (it takes a moment to print its
    first line) and sampled every 50 ms; start() returns once it is live and
    opens the window, stop() closes it and keeps the samples whose timestamps
    fall inside (or the nearest one when the region is shorter than a
    sampling period)."""

    FIELDS = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")
    PERIOD_MS = 50

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", str(self.PERIOD_MS)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        deadline = time.time() + 5.0
        while not self.lines and time.time() < deadline and self.proc.poll() is None:
            time.sleep(0.01)
        self.t0 = datetime.datetime.now()

    def begin(self):
        """Opens the window (when the sampler was started ahead of it)."""
        self.t0 = datetime.datetime.now()

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append((datetime.datetime.now(), ln.strip()))

    def stop(self):
        if not self.proc:
            return None
        self.t1 = datetime.datetime.now()
        time.sleep(self.PERIOD_MS * 1.5e-3)        # the sample that covers the region's end
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for seen, ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f")
            except ValueError:
                ts = seen                           # arrival time of the line instead
            try:
                rows.append((ts, float(parts[1]), float(parts[2]), parts[4:8]))
            except ValueError:
                continue
        if not rows:
            return None
        inside = [r for r in rows if self.t0 <= r[0] <= self.t1]
        if not inside:   # region shorter than a period: the sample nearest to its middle
            mid = self.t0 + (self.t1 - self.t0) / 2
            inside = [min(rows, key=lambda r: abs((r[0] - mid).total_seconds()))]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in inside:
            for nm, val in zip(names, r[3]):
                if val.lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median([r[1] for r in inside])), "sm_max_mhz": inside[-1][2],
                "reasons": sorted(reasons), "samples": len(inside),
                "window_s": round((self.t1 - self.t0).total_seconds(), 3)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def kernel_traffic(phase, workload, elements):
    """DRAM bytes per launch of the full C2 mesh from the committed ncu summary,
    if present; None for other workloads (no capture covers them)."""
    if not (workload.startswith("C2") and elements == 256 * 256 * 128):
        return None
    p = os.path.join(ROOT, "profiles", "kernel_traffic.txt")
    try:
        for ln in open(p):
            parts = ln.split()
            if len(parts) >= 2 and parts[0] == phase:
                return float(parts[1])
    except OSError:
        pass
    return None


def max_over_ranks(values, world, device):
    """Per-rank floats reduced with MAX over the ranks (identity on one rank):
    the slowest rank's times decide the whole-job throughput."""
    if world <= 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def shard(n, rank, world):
    """The contiguous block [lo, hi) of n independent units that rank owns."""
    return n * rank // world, n * (rank + 1) // world


def init_ranks(world, local):
    """One process per GPU: NCCL process group when there is more than one rank."""
    if world <= 1:
        return
    import torch
    import torch.distributed as dist

    torch.cuda.set_device(local)
    dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")


def build_domain(wf, case, prec, x, device):
    d = wf.Domain(prec, device=device)
    W.apply(d, case, x=x)
    d.init()
    d.sync()
    return d


def run_ours(args):
    import torch

    import weldformfem_gb300 as wf

    rank, world, local = dist_env()
    init_ranks(world, local)
    device = local
    torch.cuda.set_device(device)
    case = W.config(args.config, scale=tuple(args.scale) if args.scale else None)
    K, Wm = args.steps, args.warmup
    x = case.coords()
    E = case.n_elem

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    # ---- mixed precision, graph launches: the headline -------------------------
    dm = build_domain(wf, case, wf.WF_MIXED, x, device)
    clocks = ClockSampler(device)
    clocks.start()                   # live before the warm-up
    clocks.begin()                   # window: warm-up, timed steps, phase steps, FP64 steps
    dm.run(Wm)
    dm.sync()
    dm.prepare_run(K)                # the graphs the timed run replays, built untimed
    stream = torch.cuda.ExternalStream(dm.stream_handle(), device=device)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    mode, cl_blocks, cl_bs = dm.step_mode()
    tile_stats = dm.tile_stats()
    barrier()
    torch.cuda.synchronize(device)
    launches0 = dm.launch_count()
    graphs0 = dm.graph_launches()
    ev0.record(stream)
    dm.run(K)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize(device)
    barrier()
    ms_total = ev0.elapsed_time(ev1)
    launches = dm.launch_count() - launches0
    graph_replays = dm.graph_launches() - graphs0
    dm.sync()                        # raises if a non-finite force was cleared
    # per-phase breakdown (direct launches, CUDA events around each kernel)
    dm.set_phase_timing(True)
    kp = max(10, min(K, 100))
    dm.run(kp)
    ms_phase, nph = dm.phase_times()
    dm.set_phase_timing(False)
    ms_phase = ms_phase / max(nph, 1)
    tuned = {p: dict(zip(("block", "items_per_thread"), dm.launch_config(i)[:2]))
             for i, p in enumerate(PHASES[:3])}

    # ---- FP64 plain: same steps from the same initial state ----------------------
    df = build_domain(wf, case, wf.WF_FP64, x, device)
    df.run(Wm)
    df.sync()
    df.prepare_run(K)
    fstream = torch.cuda.ExternalStream(df.stream_handle(), device=device)
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(fstream)
    df.run(K)
    f1.record(fstream)
    f1.synchronize()
    clk = clocks.stop()
    ms_fp64 = f0.elapsed_time(f1)
    df.sync()

    # errors of mixed vs FP64 over the configuration's whole run (outside any
    # timed region): a fresh mixed domain and the FP64 one, same inputs
    nrun = max(Wm + K, case.steps) if not args.short_error else Wm + K
    df.run(nrun - (Wm + K))
    dm2 = build_domain(wf, case, wf.WF_MIXED, x, device)
    dm2.run(nrun)
    dm2.sync()
    df.sync()
    err = mixed_errors(dm2, df, nrun)
    del dm2, df

    # ---- end to end through the C ABI from host buffers ------------------------------
    # the host inputs (coordinates, connectivity, BC lists) are built before
    # the clock starts, the coordinates, connectivity and the displacement
    # output in pinned host memory; every library call that consumes or fills
    # them is timed
    elnod = case.elnod()
    bcs = case.bcs()
    x_pin = torch.empty(x.shape, dtype=torch.float64, pin_memory=True).numpy()
    x_pin[...] = x
    el_pin = torch.empty(elnod.shape, dtype=torch.int32, pin_memory=True).numpy()
    el_pin[...] = elnod
    u_pin = torch.empty(case.n_node * 3, dtype=torch.float64, pin_memory=True).numpy()
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    de = wf.Domain(wf.WF_MIXED, device=device)
    de.set_mesh(x_pin, el_pin)
    t_mesh = time.perf_counter()
    W.apply_options(de, case, x=x_pin, set_dt=False, bcs=bcs)
    t_opts = time.perf_counter()
    de.init()
    t_init = time.perf_counter()
    de.set_dt(W.cfl_dt(case, de.min_edge_length()))   # CFL step from the device reduction
    t_setup = time.perf_counter() - t0
    de.run(K)
    de.sync()
    t_run = time.perf_counter()
    u_host = de.node_vec("u", out=u_pin)
    r_host = de.reaction()
    de.sync()
    t_e2e = time.perf_counter() - t0
    e2e_parts = {"set_mesh": round(t_mesh - t0, 4), "options_bcs": round(t_opts - t_mesh, 4),
                 "init": round(t_init - t_opts, 4), "cfl_dt": round(t0 + t_setup - t_init, 4),
                 "steps": round(t_run - t0 - t_setup, 4),
                 "readback": round(t0 + t_e2e - t_run, 4)}
    h2d, d2h = de.transfer_bytes()
    assert u_host.shape[0] == case.n_node and r_host.shape[0] == K
    del de

    # ---- aggregate over ranks ---------------------------------------------------------------
    ms_total, t_e2e = max_over_ranks([ms_total, t_e2e], world, f"cuda:{device}")
    ms_step = ms_total / K
    value = world * E * K / (ms_total * 1e-3)
    fp64_value = E * K / (ms_fp64 * 1e-3)

    # ---- roofline of the dominant kernel -------------------------------------------------
    peak, peak_kind = measured_peak()
    box = dm.box() != (0, 0, 0)
    alg_table = (ALG_BYTES_TET_MIXED if case.tritetra
                 else ALG_BYTES_HEX_MIXED_BOX if box else ALG_BYTES_HEX_MIXED)
    phase_bytes = {p: alg_table[p][0] * E + alg_table[p][1] * case.n_node for p in PHASES}
    phases = PHASES
    if mode == 3:
        phases = TILED_PHASES
        phase_bytes["tile"], phase_bytes["shared"] = tiled_alg_bytes(E, case.n_node, tile_stats)
    elif mode == 5:
        # the dataflow step is timed as the element phase
        phases = ["flow"]
        ms_phase = ms_phase[2:3]
        phase_bytes["flow"] = ALG_BYTES_FLOW["flow"][0] * E + ALG_BYTES_FLOW["flow"][1] * case.n_node
    elif mode == 4:
        # the sweep is timed as the element phase; the node phase's slot times
        # no kernel of the step
        phases = SWEEP_PHASES
        ms_phase = ms_phase[:3]
        phase_bytes["sweep"] = ALG_BYTES_SWEEP["sweep"][0] * E + \
            ALG_BYTES_SWEEP["sweep"][1] * case.n_node
    dom = int(np.argmax(ms_phase))
    ph = phases[dom]
    alg_bytes = phase_bytes[ph]
    achieved = alg_bytes / (ms_phase[dom] * 1e-3) / 1e9
    roof = {"bound": "hbm", "kernel": KERNEL_NAMES[ph], "box_indexing": box,
            "achieved": round(achieved, 1),
            "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": kernel_traffic(ph + ("_box" if box else ""), case.name, E),
            "alg_bytes_per_launch": int(alg_bytes),
            "ms_per_launch": round(float(ms_phase[dom]), 4),
            "phases_ms": {p: round(float(m), 4) for p, m in zip(phases, ms_phase)},
            "phases_gbs": {p: round(phase_bytes[p] / (float(m) * 1e-3) / 1e9, 1)
                           for p, m in zip(phases, ms_phase)}}
    step_alg = sum(phase_bytes[p] for p in phases)
    roof["step_achieved_gbs"] = round(step_alg / (ms_step * 1e-3) / 1e9, 1)
    # the path's roofline: compulsory bytes of one pass over the state per
    # element-step (mixed: hex 92 + 144 r, tet 76 + 144 r, r = nodes / elements)
    r_ne = case.n_node / E
    b_alg = (76.0 if case.tritetra else 92.0) + 144.0 * r_ne
    path_gbs = b_alg * E / (ms_step * 1e-3) / 1e9
    roof["path"] = {"b_alg_per_element_step": round(b_alg, 1), "achieved": round(path_gbs, 1),
                    "frac": round(path_gbs / peak, 4),
                    "note": "compulsory bytes per element-step x element-steps/s over the "
                            "peak; 'frac' above is the dominant kernel's own bytes"}

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(case, x, args.cpu_steps)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world,
            "steps": K, "warmup": Wm, "ms_per_step": round(ms_step, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (f64-compensated positions, f64 reaction sums)", "data": "synthetic",
            "config": {"workload": case.name, "elements": E, "nodes": case.n_node,
                       "precision": "mixed", "parallelism": "replicas" if world > 1 else "single",
                       "l2": f"~{step_alg / 1e9:.2f} GB touched per step per replica, "
                             f"{'larger' if step_alg > 129e6 else 'smaller'} than the 129 MB L2; "
                             "no flush"},
            "fp64": {"value": round(fp64_value, 1), "ms_per_step": round(ms_fp64 / K, 4),
                     "over_cpu_baseline": (round(fp64_value / cpu["value"], 2) if cpu
                                           else None)},
            "mixed_over_fp64": round(value / world / fp64_value, 3),
            "error_vs_fp64": err,
            "e2e": {"value": round(E * K / t_e2e, 1), "unit": UNIT,
                    "h2d_bytes_per_step": int(h2d / K), "d2h_bytes_per_step": int(d2h / K),
                    "seconds": round(t_e2e, 3), "setup_seconds": round(t_setup, 3),
                    "parts_seconds": e2e_parts,
                    "setup_share": round(t_setup / t_e2e, 3),
                    "includes": "mesh + BC upload from pinned host buffers, init (launch "
                                "shapes from the library's per-process autotune cache: an "
                                "earlier domain of this size was tuned; device memory from the "
                                "library's pool), device CFL dt, K steps (graphs captured in "
                                "the run), displacement readback into a pinned host buffer + "
                                "reaction readback"},
            "gpu_launches": int(launches),
            "step_mode": step_mode_label(mode, cl_blocks, cl_bs, K, graph_replays, launches,
                                         tile_stats),
            "autotuned_launch": tuned,
            "launch_note": "items_per_thread 0 = persistent grid (SMs x resident blocks)",
            "roofline": roof,
            "cpu_baseline": cpu,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def step_mode_label(mode, cl_blocks, cl_bs, K, graph_replays, launches, tile_stats=None):
    """What the timed wf_run(K) launched, as counted by the library."""
    if mode == 2:
        return {"mode": "one cluster launch per run", "cluster_blocks": cl_blocks,
                "block_size": cl_bs, "kernel_launches": int(launches),
                "note": "roofline phases are the per-phase kernels, timed apart"}
    full, rem = divmod(K, 32)
    kernels = ("geometry, nodal, tiled element+assembly, shared-node kernels" if mode == 3
               else "geometry, nodal, column-sweep kernels" if mode == 4
               else "dataflow kernel (one persistent launch per step)" if mode == 5
               else "per-phase kernels")
    extra = {}
    if mode == 3 and tile_stats:
        extra = {"tiles": tile_stats[0], "shared_nodes": tile_stats[1],
                 "threads_per_tile": cl_bs}
    if mode == 4:
        extra = {"columns": cl_blocks, "threads_per_column": cl_bs}
    if mode == 5:
        extra = {"blocks": cl_blocks, "threads_per_block": cl_bs}
    return {**extra, "mode": f"{kernels} replayed from CUDA graphs" if graph_replays
            else f"{kernels}, direct launches",
            "graph_replays": int(graph_replays),
            "graphs": f"{full} x 32 steps" + (f" + 1 x {rem} steps" if rem > 1 else "")
            + (" + 1 direct step" if rem == 1 else ""),
            "graphs_built": "before the timed region (wf_prepare_run)"}


def mixed_errors(dm, df, nrun):
    """Mixed-precision run against the FP64 run of the same inputs: max-norm
    and RMS relative errors of the displacement, the plastic strain and the
    reaction history."""
    rm, rf = dm.reaction()[:nrun], df.reaction()[:nrun]
    um, uf = dm.node_vec("u"), df.node_vec("u")
    plm, plf = dm.elem_scalar("pl_strain"), df.elem_scalar("pl_strain")

    def rel(a, b):
        return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))

    def rms(a, b):
        return float(np.sqrt(np.mean((a - b) ** 2)) / max(np.sqrt(np.mean(b ** 2)), 1e-300))

    has_pl = np.max(np.abs(plf)) > 0
    return {"reaction": rel(rm, rf), "reaction_rms": rms(rm, rf),
            "displacement": rel(um, uf), "displacement_rms": rms(um, uf),
            "pl_strain": rel(plm, plf) if has_pl else 0.0,
            "pl_strain_rms": rms(plm, plf) if has_pl else 0.0,
            "pl_strain_max_fp64": float(np.max(plf)),
            "plastic_elements_fp64": int(np.count_nonzero(plf)),
            "steps": nrun,
            "how": "fresh mixed run vs the FP64 run of the same inputs; max-norm: "
                   "max|a-b|/max|b|, rms: ||a-b||_2/||b||_2"}


def run_ensemble(args):
    """Config 3: 1024 cubes in one batched domain vs one domain per specimen."""
    import torch

    import weldformfem_gb300 as wf

    rank, world, local = dist_env()
    init_ranks(world, local)
    device = local
    torch.cuda.set_device(device)
    full = W.ensemble(n_spec=args.n_spec)
    # specimens are independent: each rank runs its contiguous share, no
    # collective on the data path
    lo, hi = shard(len(full.cases), rank, world)
    batch = W.Batch(full.name, full.cases[lo:hi], full.hg)
    K, Wm = args.steps, args.warmup
    E = batch.n_elem
    d = wf.Domain(wf.WF_MIXED, device=device)
    W.apply_batch(d, batch)
    d.init()
    clocks = ClockSampler(device)
    clocks.start()                   # live before the timed region
    d.run(Wm)
    d.sync()
    stream = torch.cuda.ExternalStream(d.stream_handle(), device=device)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = d.launch_count()
    clocks.begin()
    ev0.record(stream)
    d.run(K)
    ev1.record(stream)
    ev1.synchronize()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    launches = d.launch_count() - launches0
    d.set_phase_timing(True)
    d.run(max(10, min(K, 50)))
    ph, nph = d.phase_times()
    d.set_phase_timing(False)
    tuned = {p: dict(zip(("block", "items_per_thread"), d.launch_config(i)[:2]))
             for i, p in enumerate(PHASES[:3])}
    del d
    # looping the solver: one domain per specimen, same steps, same precision
    loop_ms = 0.0
    kl = 32
    for c in batch.cases:
        one = wf.Domain(wf.WF_MIXED, device=device)
        W.apply(one, c)
        one.init()
        one.run(2)
        one.sync()
        st = torch.cuda.ExternalStream(one.stream_handle(), device=device)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        one.run(kl)
        b.record(st)
        b.synchronize()
        loop_ms += a.elapsed_time(b) / kl
        del one
    ms, loop_ms = max_over_ranks([ms, loop_ms], world, f"cuda:{device}")
    E = full.n_elem
    value = E * K / (ms * 1e-3)
    loop_value = E / (loop_ms * 1e-3)
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world, "steps": K,
        "warmup": Wm, "ms_per_step": round(ms / K, 4), "higher_is_better": True,
        "scaling": "strong" if world > 1 else "weak", "vs_baseline": None,
        "dtype": "f32 (f64-compensated positions, f64 reaction sums)", "data": "synthetic",
        "config": {"workload": full.name, "specimens": len(full.cases), "elements": E,
                   "nodes": full.n_node, "precision": "mixed",
                   "parallelism": f"specimens sharded over {world} ranks" if world > 1
                   else "single"},
        "looped": {"value": round(loop_value, 1), "ms_per_step": round(loop_ms, 4),
                   "how": "one domain per specimen, 32 graph-launched steps each, summed"},
        "batched_over_looped": round(value / loop_value, 2),
        "gpu_launches": int(launches),
        "autotuned_launch": tuned,
        "launch_note": "items_per_thread 0 = persistent grid (SMs x resident blocks)",
        "phases_ms": {p: round(float(m) / max(nph, 1), 4) for p, m in zip(PHASES, ph)},
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def run_adjoint(args):
    """Config 4: material identification on the 32^3 octant cube (24
    parameters), FP64 step with checkpoints every `--every` steps; times the
    plain forward, the checkpointed forward and the reverse pass (FP64 and
    FP32 reverse arithmetic), and checks three gradient components against
    central finite differences of the FP64 forward at full size."""
    import torch

    import weldformfem_gb300 as wf
    from weldformfem_gb300 import adjoint as A

    rank, _, local = dist_env()
    if rank != 0:
        return  # one identification problem: measured on rank 0 only
    device = local
    torch.cuda.set_device(device)
    case = W.config(4, steps=args.adj_steps)
    case.dt = case.time_step()
    N, every = case.steps, args.every
    E = case.n_elem
    th0 = W.material_params(case)
    Rstar, _ = A.solve_with_adjoint(case, th0 * W.target_factors(case), N, every)

    def timed(dom, fn):
        st = torch.cuda.ExternalStream(dom.stream_handle(), device=device)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(device)
        a.record(st)
        out = fn()
        b.record(st)
        b.synchronize()
        return a.elapsed_time(b), out

    def fresh(prec=wf.WF_FP64, theta=th0):
        d = wf.Domain(prec, device=device)
        W.apply(d, W.with_params(case, theta))
        d.init()
        d.sync()
        return d

    # warm-up of every kernel on a short run
    dw = fresh()
    dw.adjoint_forward(2 * every, every)
    dw.adjoint_backward(np.ones(2 * every))
    dw.adjoint_backward(np.ones(2 * every), fp32=True)
    del dw
    clocks = ClockSampler(device)
    clocks.start()
    d = fresh()
    ms_fwd, _ = timed(d, lambda: d.run(N))
    R_plain = d.reaction()
    del d
    d = fresh(wf.WF_MIXED)
    ms_mixed, _ = timed(d, lambda: d.run(N))
    del d
    d = fresh()
    l0 = d.launch_count()
    ms_ck, _ = timed(d, lambda: d.adjoint_forward(N, every))
    R = d.reaction()
    seed = 2.0 * (R - Rstar)
    l1 = d.launch_count()
    ms_b64, g64 = timed(d, lambda: d.adjoint_backward(seed))
    l2 = d.launch_count()
    ms_b32, g32 = timed(d, lambda: d.adjoint_backward(seed, fp32=True))
    del d
    # every step kept in HBM instead of checkpoints: no recompute
    d = fresh()
    ms_ka, _ = timed(d, lambda: d.adjoint_forward(N, -1))
    ms_kb, gk = timed(d, lambda: d.adjoint_backward(seed))
    ms_kb32, _ = timed(d, lambda: d.adjoint_backward(seed, fp32=True))
    assert np.array_equal(gk, g64)
    clk = clocks.stop()
    loss = float(np.sum((R - Rstar) ** 2))
    assert np.array_equal(R, R_plain)

    # three components against central differences of the FP64 forward
    fd = []
    for (i, k) in ((0, 0), (3, 1), (7, 2)):
        h = 1e-6 * th0[i, k]
        Ls = []
        for sgn in (1, -1):
            t = th0.copy()
            t[i, k] += sgn * h
            dd = fresh(theta=t)
            dd.run(N)
            Ls.append(float(np.sum((dd.reaction() - Rstar) ** 2)))
            del dd
        gfd = (Ls[0] - Ls[1]) / (2 * h)
        fd.append({"param": f"{W.PARAM_KEYS[k]}[{i}]", "adjoint": float(g64[i, k]),
                   "fd": gfd, "rel_err": abs(g64[i, k] - gfd) / max(abs(gfd), 1e-300)})
    lg = lambda g: g * th0
    err32 = float(np.abs(lg(g32) - lg(g64)).max() / np.abs(lg(g64)).max())
    line = {
        "metric": "adjoint/forward time", "value": round(ms_b64 / ms_fwd, 3), "unit": "ratio",
        "n_gpus": 1, "steps": N, "warmup": 1, "higher_is_better": False,
        "scaling": "none", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": case.name, "elements": E, "nodes": case.n_node,
                   "parameters": int(th0.size), "checkpoint_every": every,
                   "loss": "sum over steps of (F_top - F_target)^2, target = seeded U[0.8,1.2) "
                           "scaling of the 24 parameters"},
        "ms": {"forward_fp64": round(ms_fwd, 2), "forward_mixed": round(ms_mixed, 2),
               "forward_checkpointed": round(ms_ck, 2), "backward_fp64": round(ms_b64, 2),
               "backward_fp32_reverse": round(ms_b32, 2)},
        "ratios": {"backward_fp64_over_forward": round(ms_b64 / ms_fwd, 3),
                   "backward_fp32_over_forward": round(ms_b32 / ms_fwd, 3),
                   "checkpointed_forward_plus_backward_over_forward":
                       round((ms_ck + ms_b64) / ms_fwd, 3),
                   "all_steps_kept": {
                       "forward_over_forward": round(ms_ka / ms_fwd, 3),
                       "backward_fp64_over_forward": round(ms_kb / ms_fwd, 3),
                       "backward_fp32_over_forward": round(ms_kb32 / ms_fwd, 3),
                       "stash_gb": round(N * (14 * case.n_node + 7 * E) * 8 / 1e9, 2)}},
        "element_steps_per_s_forward_fp64": round(E * N / (ms_fwd * 1e-3), 1),
        "loss": loss,
        "gradient_fd_check": fd,
        "fp32_reverse_rel_err": err32,
        "gpu_launches": {"forward_checkpointed": int(l1 - l0), "backward": int(l2 - l1)},
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def cpu_baseline(case, x, steps):
    """The oracle (C restatement of the reference loop) on all host cores."""
    from oracle import orabind

    threads = os.cpu_count() or 1
    d = orabind.OracleDomain(threads=threads)
    W.apply(d, case, x=x)
    d.init()
    t0 = time.perf_counter()
    d.step(steps)
    t = time.perf_counter() - t0
    return {"value": round(case.n_elem * steps / t, 1), "unit": UNIT, "cores": threads,
            "kind": "port", "sample": f"{case.name}: {steps} steps on the full mesh, setup excluded"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    case = W.config(args.config, scale=tuple(args.scale) if args.scale else None)
    x = case.coords()
    from oracle import orabind

    threads = os.cpu_count() or 1
    d = orabind.OracleDomain(threads=threads)
    W.apply(d, case, x=x)
    d.init()
    # the same warm-up count as the GPU arm, bounded to ~30 s on slow hosts
    t0 = time.perf_counter()
    d.step(1)
    per = time.perf_counter() - t0
    wn = int(max(0, min(args.warmup - 1, 30.0 / max(per, 1e-9))))
    d.step(wn)
    # each step is one full time step of the workload; the count is bounded so
    # that the run ends within a few minutes on the host cores
    n = int(max(1, min(args.steps, 60.0 / max(per, 1e-9))))
    t0 = time.perf_counter()
    d.step(n)
    t = time.perf_counter() - t0
    value = case.n_elem * n / t
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": 0, "steps": n,
        "warmup": args.warmup, "ms_per_step": round(t / n * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference", "warmup_steps_run": 1 + wn,
        "config": {"workload": case.name, "elements": case.n_elem, "nodes": case.n_node,
                   "precision": "fp64"},
        "cpu_baseline": {"value": round(value, 1), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n} time steps of the full workload (bounded to ~60 s)"},
        "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_profile_case(args):
    """A bare run for kernel profiles: one domain of the configuration (FP64 or
    mixed), W + K steps in the library's default step mode, no other work, so
    that the launch sequence under a profiler is init, then the steps. With
    --no-autotune the mixed kernels keep their default launch shapes (no
    tuning launches before the steps)."""
    import torch

    import weldformfem_gb300 as wf

    torch.cuda.set_device(0)
    case = W.config(args.config, scale=tuple(args.scale) if args.scale else None)
    prec = wf.WF_FP64 if args.profile == "fp64" else wf.WF_MIXED
    d = wf.Domain(prec, device=0)
    W.apply(d, case)
    if args.no_autotune:
        d.set_autotune(False)
    if args.step_mode is not None:
        d.set_step_mode(args.step_mode)
    if args.no_box:
        d.set_box_indexing(False)
    if args.sweep_rows:
        d.set_sweep_rows(args.sweep_rows)
    if args.flow_tiles:
        d.set_flow_tiles(*args.flow_tiles)
    d.init()
    d.run(args.warmup)
    d.sync()
    d.prepare_run(args.steps)
    st = torch.cuda.ExternalStream(d.stream_handle(), device=0)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    d.run(args.steps)
    b.record(st)
    b.synchronize()
    d.sync()
    out = {"profile_case": case.name, "precision": args.profile, "elements": case.n_elem,
           "step_mode": d.step_mode()[0], "box": d.box(),
           "ms_per_step": round(a.elapsed_time(b) / args.steps, 4)}
    if args.phase_steps:
        d.set_phase_timing(True)
        d.run(args.phase_steps)
        ms, n = d.phase_times()
        out["phases_ms"] = [round(float(v) / max(n, 1), 4) for v in ms]
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=2)
    ap.add_argument("--scale", type=int, nargs=3, default=None)
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--profile", choices=["mixed", "fp64"], default=None,
                    help="bare run of one domain for kernel profiles (no other measurement)")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--step-mode", type=int, default=None,
                    help="profiling runs: step mode (1 per-phase, 2 cluster, 3 tiled, 4 sweep, "
                         "5 dataflow)")
    ap.add_argument("--sweep-rows", type=int, default=0, choices=[0, 4, 8],
                    help="profiling runs: node rows per column of the column sweep")
    ap.add_argument("--flow-tiles", type=int, nargs=2, default=None,
                    help="profiling runs: dataflow tile size and node-update lag")
    ap.add_argument("--no-box", action="store_true",
                    help="profiling runs: read the connectivity arrays on box meshes too")
    ap.add_argument("--phase-steps", type=int, default=0,
                    help="profiling runs: also time this many steps phase by phase")
    ap.add_argument("--short-error", action="store_true",
                    help="mixed-vs-FP64 errors over W + K steps instead of the whole run")
    ap.add_argument("--n-spec", type=int, default=1024)
    ap.add_argument("--adj-steps", type=int, default=4000)
    ap.add_argument("--every", type=int, default=64)
    args = ap.parse_args()
    if args.profile:
        run_profile_case(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.config == 3:
        run_ensemble(args)
    elif args.config == 4:
        run_adjoint(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
