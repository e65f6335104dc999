"""Benchmark of the coupled cell step: cell-steps/s on the 1M-cell / 161^3-node spheroid.

One step = one ``cell_step`` of the drop-in API: deposit of the cells' O2 uptake (int64 fixed
point) -> red-black SOR to the residual tolerance (warm start, residual checked every
``check_every`` sweeps) -> trilinear sampling -> lifecycle (decide, inclusive scan, one host read,
placement) -> one mechanics substep (hash-grid binning, contact forces + integration).

Workload "spheroid_1M_161" (default): 1,000,000 cells uniform in a 1,200 um ball, radii
N(8, 0.8) clipped to [6, 10] um, 161^3 grid at 15 um (boundary 100 mmHg), D = 2000 um^2/s,
Vmax = 20 amol/s = 5.54e7 mmHg um^3/h, Km = 1 mmHg, SOR omega 1.8 to residual 1e-6, hypoxia
below 5 mmHg, necrosis below 1 mmHg, division ln2/24 per h, k/gamma = 1/h, 20 um hash cells,
dt = 6 min (one mechanics substep). Synthetic seeded inputs (numpy default_rng(0)).

Arms:
  (default)          GB300 kernels through the public API; device-timed K steps (CUDA events,
                     inputs already in HBM), per-stage event timers, an end-to-end pass through
                     host buffers, a CPU baseline sample (the oracle on the host cores) and a
                     full-size bitwise parity check of one step against the oracle.
  --impl reference   the reference's algorithm on the host CPU: WarpBioCell's own Warp CPU path
                     cannot run here (warp-lang is not installed), so this times the C++
                     restatement (oracle/) with every host thread, on the same workload.

Multi-GPU (torchrun, --gpus N): independent replicas, one per GPU (no data-path collective; the
only collectives are the timing barrier and the max/sum reductions of the result); the batched
sweep workload shards its instances over the ranks instead (simulation.sweep.partition_runs).
"""

from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

UNIT = "cell-steps/s"


def metric_for(workload: str) -> str:
    """The metric label of a workload (the cell count and grid it is quoted on)."""
    w = WORKLOADS[workload]
    if w.get("batched"):
        return "cell-steps/s (15-spheroid batched sweep, one launch per stage, graph-captured step)"
    if w.get("adjoint"):
        return "adjoint backward time / forward time (100k cells, 81^3 O2, K=64 contact steps)"
    cells = w["cells"]
    count = f"{cells // 1_000_000}M" if cells % 1_000_000 == 0 else f"{cells // 1000}k"
    n = int(round(w["box_um"] / w["dx_um"])) + 1
    fields = "O2 + glucose + lactate, 106-node networks" if w.get("metabolic") else "O2"
    return f"cell-steps/s @{count} cells+{n}^3 {fields} (coupled cell step)"


def workload_config(workload: str, grid_nodes: int | None = None) -> dict:
    """The `config` object of both arms: the workload's name and defining sizes only."""
    cfg = {"workload": workload, **WORKLOADS[workload]}
    if grid_nodes is not None:
        cfg["grid_nodes"] = grid_nodes
    return cfg

WORKLOADS = {
    "spheroid_1M_161": dict(cells=1_000_000, ball_um=1200.0, box_um=2400.0, dx_um=15.0, boundary=100.0),
    "spheroid_10k_41": dict(cells=10_000, ball_um=250.0, box_um=800.0, dx_um=20.0, boundary=38.0),
    "spheroid_100k_81": dict(cells=100_000, ball_um=600.0, box_um=1600.0, dx_um=20.0, boundary=38.0),
    # oxygen + glucose (uptake 1:6 to O2, 5 mM boundary, 600 um^2/s) + lactate (zero boundary,
    # 800 um^2/s, production 2x the glucose uptake scaled by G/(K_G + G)) on three 81^3 grids, and a
    # 106-node random truth-table network per cell clamped by O2 > 5 mmHg and glucose > 2 mM,
    # updated synchronously once per step; lifecycle in network mode.
    "metabolic_network_100k_81": dict(cells=100_000, ball_um=600.0, box_um=1600.0, dx_um=20.0, boundary=38.0,
                                      metabolic=True, network_nodes=106),
    # 15 spheroids: boundary O2 {10, 20, 38, 60, 100} mmHg x 3 seeds, cell counts log-uniform in
    # [2,000, 200,000] at the 1M-cell workload's density, cubic grids of 41-121 nodes (odd, growing
    # with the count) over a box of 2.5 spheroid radii; advanced as one batch against 15 plain runs.
    # Adjoint calibration: 100,000 cells in a 500 um ball, 81^3 O2 grid at 15 um, K = 64 contact
    # steps, per-cell Vmax log-normal (sigma 0.3), loss = squared L2 error of the steady field +
    # of the cells' distances from their centroid against the model at parameters perturbed by up
    # to +-20% (seeded).
    "adjoint_100k_81": dict(adjoint=True, cells=100_000, ball_um=500.0, nodes=81, dx_um=15.0, steps=64,
                            boundary=38.0, vmax_sigma=0.3),
    "batched_sweep_15": dict(batched=True, boundaries=(10.0, 20.0, 38.0, 60.0, 100.0), seeds=(0, 1, 2),
                             cells_lo=2_000, cells_hi=200_000, nodes_lo=41, nodes_hi=121, box_over_radius=2.5),
}

# ncu figures of one k_sor_resident launch (the initial solve, 780 sweeps) of the 1M-cell / 161^3
# workload, `profiles/k_sor_resident_spheroid_1M_161.md`: DRAM bytes read + written by the launch,
# the sweeps it ran, its warp instructions per node update and its issue-active fraction.
SOR_NCU = {"dram_bytes": 35.4e6, "sweeps": 780, "warp_inst_per_node_update": 10.787e9 / (780 * 4173281.0),
           "issue_active": 0.793, "source": "profiles/k_sor_resident_spheroid_1M_161.md"}

DIFFUSION = 7.2e6  # um^2/h (2000 um^2/s)
VMAX = 20e-18 / 1.3e-21 * 3600.0  # 20 amol/s over O2 solubility 1.3e-21 mol/(um^3 mmHg) -> mmHg um^3/h
KM = 1.0
DT = 0.1  # h (6 min)


def make_params(w: dict):
    from warpbiocell_gb300.cells.lifecycle import LifecycleParams
    from warpbiocell_gb300.cells.mechanics import ContactParams
    from warpbiocell_gb300.fields.diffusion import SolverSettings
    from warpbiocell_gb300.fields.oxygen import OxygenParams
    from warpbiocell_gb300.fields.scalar_field import GridGeometry
    from warpbiocell_gb300.simulation.simulator import TimeStepping

    P = dict(
        geom=GridGeometry.centered_cube(w["box_um"], w["dx_um"]),
        oxygen=OxygenParams(diffusion_coefficient=DIFFUSION, uptake_max=VMAX, michaelis_k=KM,
                            boundary_value=w["boundary"]),
        settings=SolverSettings(omega=1.8, tolerance=1e-6, max_sweeps=2000, check_every=20),
        lifecycle=LifecycleParams(division_rate=math.log(2.0) / 24.0, death_rate=0.0, anoxic_death_rate=0.5,
                                  inhibition_threshold=8, hypoxia_threshold=5.0, death_threshold=1.0),
        contact=ContactParams(stiffness=1.0, damping=1.0, max_radius=10.0, margin=0.0, wall_rate=4.0),
        stepping=TimeStepping(dt_cells=DT, dt_mechanics=DT),
        species=[],
        network=None,
    )
    if w.get("metabolic"):
        from warpbiocell_gb300.fields.species import SpeciesParams, by_state
        from warpbiocell_gb300.network.random_network import random_truth_table_network
        from warpbiocell_gb300.network.runtime import InputClamp, NetworkParams

        glucose_uptake = 20e-18 / 6.0 * 3600.0 / 1e-18  # mol/cell/s -> mM um^3/h (1 mM = 1e-18 mol/um^3)
        P["species"] = [
            SpeciesParams("glucose", "mM", diffusion=600.0 * 3600.0, michaelis_k=0.04, boundary_value=5.0,
                          uptake_max=by_state(glucose_uptake)),
            SpeciesParams("lactate", "mM", diffusion=800.0 * 3600.0, michaelis_k=1.0, boundary_value=0.0,
                          production=by_state(2.0 * glucose_uptake), production_source="glucose"),
        ]
        net = random_truth_table_network(w["network_nodes"], seed=0)
        P["network"] = NetworkParams(net, update="synchronous", updates_per_step=1,
                                     inputs=(InputClamp("Oxygen_supply", "oxygen", 5.0),
                                             InputClamp("Glucose_supply", "glucose", 2.0)))
        P["lifecycle"] = LifecycleParams(division_rate=math.log(2.0) / 24.0, anoxic_death_rate=0.5,
                                         inhibition_threshold=8, hypoxia_threshold=5.0, death_threshold=1.0,
                                         phenotype_model="network", apoptosis_rate=0.02, necrosis_rate=0.1)
    return P


def make_cells(w: dict, seed: int):
    from warpbiocell_gb300.cells.initialization import clipped_normal_radii, uniform_ball

    pos = uniform_ball(w["cells"], w["ball_um"], seed=seed)
    radii = clipped_normal_radii(w["cells"], 8.0, 0.8, 6.0, 10.0, seed=seed + 1)
    return pos, radii


# ---- clocks ------------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu_index = gpu_index
        self.proc = None
        self.path = Path(tempfile.mkstemp(prefix="wbc_clocks_", suffix=".csv")[1])

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu_index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, sm_max, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                sm_max.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        self.path.unlink(missing_ok=True)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(sm_max)), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---- roofline bookkeeping --------------------------------------------------------------------------------
def stage_bytes(stage: str, cells: float, nodes: float, launches: int, daughters: float = 0.0) -> float:
    """Algorithmic (compulsory) bytes a stage moves, summed over its launches."""
    if stage == "sor":  # per colour launch: read the field once, n_eff and write the colour's half
        return launches * 8.0 * nodes
    if stage == "deposit":  # position + state + visiting order per cell, the 32-bit low words cleared
        return 20.0 * cells + 16.0 * nodes
    if stage == "convert":  # read the 4 low-word layers, write n_eff
        return (16.0 + 4.0) * nodes
    if stage == "contact":  # xyzr + id read, position/velocity/count write
        return (16.0 + 4.0 + 12.0 + 12.0 + 4.0) * cells
    if stage == "bin":  # position/radius read, ids + xyzr written
        return (12.0 + 4.0 + 4.0 + 16.0) * cells
    if stage == "sample":
        return (12.0 + 4.0) * cells + 4.0 * nodes
    if stage == "decide":
        return 40.0 * cells
    if stage == "scan":
        return 8.0 * cells
    if stage == "place":
        return 8.0 * cells + 64.0 * daughters
    return 0.0


def load_peaks() -> dict:
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        try:
            return json.loads(path.read_text())
        except ValueError:
            pass
    return {}


# ---- GB300 arm ---------------------------------------------------------------------------------------------
# Stages whose events stay inside the timed steps: the roofline's kernels.
ROOFLINE_STAGES = ("sor", "deposit", "convert")


def run_gpu(args, rank: int, world: int) -> dict | None:
    import torch

    from warpbiocell_gb300 import _lib, profiling
    from warpbiocell_gb300.cells.mechanics import contact_substep, make_neighbor_grid
    from warpbiocell_gb300.cells.state import CellPopulation
    from warpbiocell_gb300.fields.oxygen import OxygenField
    from warpbiocell_gb300.simulation.simulator import cell_step

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if args.sor_tuning:
        from warpbiocell_gb300.fields import diffusion as _diff

        _diff.solver_tuning = tuple(int(v) for v in args.sor_tuning.split(","))
    w = WORKLOADS[args.workload]
    P = make_params(w)
    pos, radii = make_cells(w, seed=args.seed + rank)
    capacity = int(w["cells"] * 1.5)
    pop = CellPopulation.from_numpy(pos, radii, capacity=capacity, device=dev, seed=args.seed + rank)
    network = None
    if P["species"]:
        from warpbiocell_gb300.fields.metabolism import MetabolicFields
        from warpbiocell_gb300.network.runtime import NetworkRuntime

        ox = MetabolicFields(P["geom"], P["oxygen"], P["species"], P["settings"], device=dev)
        if P["network"] is not None:
            network = NetworkRuntime(P["network"], capacity, device=dev, species_names=tuple(ox.names))
            network.initialize(pop)
    else:
        ox = OxygenField(P["geom"], P["oxygen"], P["settings"], device=dev)
    grid = make_neighbor_grid(P["contact"], dev)
    # As the reference's Experiment.run: initial neighbour counts and an initial field solve.
    contact_substep(pop, grid, P["contact"], dt=0.0)
    first = ox.update(pop)

    def step():
        return cell_step(pop, grid, P["lifecycle"], P["contact"], P["stepping"], oxygen=ox, network=network)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    launches0 = _lib.launch_count()
    # Inside the timed steps only the roofline kernels are bracketed by events (they are launched
    # at the step's start, while the device still runs the previous step's contact); the other
    # stages are timed in separate steps below, so that their events do not sit on the host's
    # critical path after the division count.
    profiling.enable(True, only=ROOFLINE_STAGES)
    barrier()
    start_ev = torch.cuda.Event(enable_timing=True)
    end_ev = torch.cuda.Event(enable_timing=True)
    cell_steps = 0
    sweeps = []
    daughters = 0
    start_ev.record()
    torch.cuda.nvtx.range_push("timed_steps")  # the launch lists under profiles/ capture this range
    for _ in range(args.steps):
        cell_steps += pop.count
        rep = step()
        sweeps.append(rep.field_sweeps)
        daughters += rep.daughters
    torch.cuda.nvtx.range_pop()
    end_ev.record()
    barrier()
    elapsed_ms = start_ev.elapsed_time(end_ev)
    stages = profiling.summary()
    launches = _lib.launch_count() - launches0
    clocks = sampler.stop()
    # Every stage, from a few more steps (the breakdown; the roofline stages keep the timed steps')
    profiled_steps = min(args.steps, 5)
    profiling.enable(True)
    for _ in range(profiled_steps):
        step()
    breakdown = profiling.summary()
    profiling.enable(False)
    for k, v in breakdown.items():
        if k not in ROOFLINE_STAGES:
            stages[k] = dict(v, calls=v["calls"] * args.steps / max(1, profiled_steps),
                             ms=v["ms"] * args.steps / max(1, profiled_steps),
                             launches=v["launches"] * args.steps / max(1, profiled_steps))

    # End to end: every step uploads the population from pinned host buffers, runs the step
    # through the public API and reads the updated population back.
    names = ["position", "radius", "cell_state", "cell_type", "age", "oxygen_local", "glucose_local", "rng_state",
             "velocity", "neighbor_count", "fate_flags"]
    host = {k: torch.empty_like(getattr(pop, k), device="cpu").pin_memory() for k in names}
    for k in names:
        host[k].copy_(getattr(pop, k))
    e2e_steps = max(1, args.steps)
    torch.cuda.synchronize()
    h2d = d2h = 0
    e_start = torch.cuda.Event(enable_timing=True)
    e_end = torch.cuda.Event(enable_timing=True)
    e2e_cells = 0
    barrier()
    e_start.record()
    for _ in range(e2e_steps):
        n = pop.count
        for k in names:
            getattr(pop, k)[:n].copy_(host[k][:n], non_blocking=True)
            h2d += host[k][:n].numel() * host[k].element_size()
        e2e_cells += n
        step()
        n = pop.count
        for k in names:
            host[k][:n].copy_(getattr(pop, k)[:n], non_blocking=True)
            d2h += host[k][:n].numel() * host[k].element_size()
    e_end.record()
    barrier()
    e2e_ms = e_start.elapsed_time(e_end)

    from warpbiocell_gb300.fields import diffusion as _diffusion

    result = {
        "sor_path": _diffusion.last_solve.get("path"),
        "sor_tiles": _diffusion.last_solve.get("tiles"),
        "sor_strips": _diffusion.last_solve.get("strips"),
        "sor_autotune": [list(v) for v in _diffusion.autotune_cache.values()],
        "rank": rank,
        "elapsed_ms": elapsed_ms,
        "cell_steps": cell_steps,
        "e2e_ms": e2e_ms,
        "e2e_cell_steps": e2e_cells,
        "h2d": h2d / e2e_steps,
        "d2h": d2h / e2e_steps,
        "launches": launches,
        "stages": stages,
        "sweeps": sweeps,
        "initial_sweeps": first.sweeps,
        "daughters": daughters,
        "clocks": clocks,
        "count": pop.count,
        "nodes": P["geom"].node_count,
    }
    if rank == 0 and not args.skip_cpu:
        result["cpu_baseline"], result["parity_full_size"] = cpu_sample_and_parity(pop, ox, grid, P, step, network)
    if rank == 0 and not P["species"]:
        result["scatter_reference"] = scatter_reference(pop, P["geom"])
    return result


def scatter_reference(pop, geom) -> dict:
    """The deposit's scatter alone, done by a library kernel: torch's index_add_ of the same 8 int64
    fixed-point contributions per cell (corner node indices and weights computed beforehand, not
    timed) into a [4 states x nodes] int64 array, i.e. the same number of 64-bit atomic adds over
    the same footprint. A bound for any atomic-scatter deposit, against which k_deposit (which
    also reads the cells and computes the weights) is compared."""
    import torch

    n = pop.count
    pos = pop.position[:n].double()
    state = pop.cell_state[:n].long()
    nx, ny, nz = geom.shape
    u = (pos - torch.tensor(geom.origin, dtype=torch.float64, device=pos.device)) / geom.dx
    i0 = torch.floor(u).long()
    f = u - i0.double()
    ok = ((i0 >= 0).all(1) & (i0[:, 0] + 1 < nx) & (i0[:, 1] + 1 < ny) & (i0[:, 2] + 1 < nz) & (state >= 0) &
          (state < 4))
    i0, f, state = i0[ok], f[ok], state[ok]
    idx, val = [], []
    nodes = nx * ny * nz
    for di in (0, 1):
        for dj in (0, 1):
            for dk in (0, 1):
                w = ((f[:, 0] if di else 1 - f[:, 0]) * (f[:, 1] if dj else 1 - f[:, 1]) *
                     (f[:, 2] if dk else 1 - f[:, 2]))
                node = ((i0[:, 0] + di) * ny + (i0[:, 1] + dj)) * nz + (i0[:, 2] + dk)
                idx.append(state * nodes + node)
                val.append(torch.floor(w * 16777216.0 + 0.5).long())
    idx = torch.cat(idx)
    val = torch.cat(val)
    acc = torch.zeros(4 * nodes, dtype=torch.int64, device=pos.device)
    times = []
    for rep in range(4):
        acc.zero_()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        acc.index_add_(0, idx, val)
        b.record()
        torch.cuda.synchronize()
        if rep:
            times.append(a.elapsed_time(b))
    ms = float(np.median(times))
    return {"what": "torch index_add_ of the same 8 int64 contributions per cell into [4, nodes] int64 "
                    "(indices precomputed, untimed)", "adds": int(idx.numel()), "us": round(ms * 1e3, 2),
            "adds_per_s": round(idx.numel() / (ms / 1e3), 1)}


def _population_to_oracle(pop):
    from oracle import oracle as orc

    arrays = {k: getattr(pop, k).cpu().numpy().copy() for k in
              ("position", "radius", "cell_state", "cell_type", "age", "oxygen_local", "glucose_local", "velocity",
               "neighbor_count", "divide_flag", "division_offset", "fate_flags")}
    sim = orc.OracleSim(capacity=pop.capacity, count=pop.count, seed=pop.seed,
                        rng_state=pop.rng_state.cpu().numpy().view(np.uint32).copy(), **arrays)
    return sim


def _oracle_species(fields, settings):
    """Oracle mirrors of the GPU fields (one SpeciesField or the species of a MetabolicFields),
    with the GPU's current values; returns (species list, production-source map)."""
    from oracle import oracle as orc

    items = list(fields.species_fields.items()) if hasattr(fields, "species_fields") else [(fields.name, fields)]
    out, src = [], {}
    for name, f in items:
        g = f.geometry
        sp = orc.OracleSpecies(orc.Geometry(g.origin, g.dx, g.shape), tuple(int(b) for b in f.field.boundary_flags),
                               f.field.boundary_value, f.species.diffusion, f.species.uptake_max, f.species.michaelis_k,
                               settings, production=f.species.production, name=name)
        sp.values = f.numpy()
        out.append(sp)
        if f.species.production_source:
            src[name] = f.species.production_source
    return out, src


def _oracle_network(rt, capacity):
    from oracle import oracle as orc

    sources = {"oxygen": 0, "glucose": 1, "constant": 4}
    extra = list(rt.extra_names)
    clamps = tuple((rt.network.index[c.node], sources.get(c.source, 2 + (extra.index(c.source) if c.source in extra else 0)),
                    float(np.float32(c.threshold)), 1 if c.above else 0) for c in rt.params.inputs)
    onet = orc.OracleNetwork({k: v.cpu().numpy() for k, v in rt._arrays.items()}, rt.network.n_nodes, capacity,
                             update=rt.params.update, updates_per_step=rt.params.updates_per_step,
                             time_units_per_h=rt.params.time_units_per_h, max_events=rt.params.max_events_per_step,
                             clamps=clamps, fate_nodes=rt.fate_nodes, extra_names=tuple(extra))
    onet.words[:] = rt.states.cpu().numpy().view(np.uint64)
    return onet


def cpu_sample_and_parity(pop, fields, grid, P, step, network=None):
    """Time one full-size cell step of the oracle on the host cores from the GPU's current state,
    then run the same step on the GPU and compare the two bit for bit."""
    from oracle import oracle as orc

    sim = _population_to_oracle(pop)
    for name, t in pop.extra_local.items():
        sim.extra_local[name] = t.cpu().numpy().copy()
    species, src = _oracle_species(fields, P["settings"])
    onet = _oracle_network(network, pop.capacity) if network is not None else None
    threads = orc.num_threads()
    cells = sim.count
    t0 = time.perf_counter()
    daughters, reports = orc.full_cell_step(sim, P["lifecycle"], P["contact"], P["stepping"].dt_cells,
                                            P["stepping"].dt_mechanics, species, src, network=onet, dim=grid.dim)
    cpu_s = time.perf_counter() - t0
    rep = step()
    n = pop.count
    gpu_fields = [f.numpy() for f in (fields.species_fields.values() if hasattr(fields, "species_fields") else [fields])]
    same = (rep.daughters == daughters and n == sim.count and rep.field_sweeps == sum(r[0] for r in reports)
            and all(np.array_equal(a, s.values) for a, s in zip(gpu_fields, species))
            and np.array_equal(pop.position[:n].cpu().numpy(), sim.position[:n])
            and np.array_equal(pop.cell_state[:n].cpu().numpy(), sim.cell_state[:n])
            and np.array_equal(pop.neighbor_count[:n].cpu().numpy(), sim.neighbor_count[:n])
            and np.array_equal(pop.rng_state[:n].cpu().numpy().view(np.uint32), sim.rng_state[:n])
            and (onet is None or np.array_equal(network.states[:n].cpu().numpy().view(np.uint64), onet.words[:n])))
    sweeps = sum(r[0] for r in reports)
    baseline = {"value": cells / cpu_s, "unit": UNIT, "cores": threads, "kind": "port",
                "sample": f"one full cell step of the same workload ({cells} cells, {sweeps} SOR sweeps) by the "
                          f"C++ restatement with {threads} OpenMP threads, from the GPU run's state; {cpu_s:.2f} s"}
    return baseline, bool(same)


def report_gpu(args, results: list[dict], world: int) -> dict:
    peaks = load_peaks()
    r0 = results[0]
    max_ms = max(r["elapsed_ms"] for r in results)
    total_cells = sum(r["cell_steps"] for r in results)
    value = total_cells / (max_ms / 1e3)
    e2e_ms = max(r["e2e_ms"] for r in results)
    e2e_value = sum(r["e2e_cell_steps"] for r in results) / (e2e_ms / 1e3)
    stages = r0["stages"]
    steps = max(1, args.steps)
    cells_per_step = r0["cell_steps"] / steps
    nodes = r0["nodes"]
    dominant = max(stages, key=lambda k: stages[k]["ms"]) if stages else None
    peak = peaks.get("hbm_gbs", 6800.0)
    peak_source = "measured" if "hbm_gbs" in peaks else "fallback"
    roofline = None
    if dominant == "sor":
        # Unit: one launch of the resident solver = one steady-state solve (all its sweeps and
        # residual checks). Algorithmic bytes: the field read and written once and n_eff read once,
        # 12 B per node (16 with a production term), whatever the sweep count; the solve then runs
        # on chip, so HBM is not its binding roof: the issue rate is, reported beside it.
        s = stages["sor"]
        launch_ms = s["ms"] / max(1, s["calls"])
        sweeps_per_launch = sum(r0["sweeps"]) / max(1, len(r0["sweeps"]))
        nbytes = 12.0 * nodes
        achieved = nbytes / (launch_ms / 1e3) / 1e9
        traffic = None
        if r0.get("sor_path") == 2 and args.workload == "spheroid_1M_161":
            traffic = round(SOR_NCU["dram_bytes"], 0)
        half_us = launch_ms * 1e3 / (2.0 * sweeps_per_launch)
        updates_per_s = nodes * sweeps_per_launch / (launch_ms / 1e3)
        roofline = {"bound": "hbm", "kernel": "k_sor_resident (one launch = one steady-state solve)",
                    "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 6),
                    "traffic": traffic, "peak_source": peak_source, "bytes_per_launch": nbytes,
                    "launch_us": round(launch_ms * 1e3, 2), "sweeps_per_launch": round(sweeps_per_launch, 1),
                    "issue_roof": {
                        "what": "the solve is on chip and bound by instruction issue, not HBM",
                        "node_updates_per_s": round(updates_per_s, 1),
                        "half_sweep_us": round(half_us, 3),
                        "warp_inst_per_node_update_ncu": (round(SOR_NCU["warp_inst_per_node_update"], 3)
                                                          if args.workload == "spheroid_1M_161" else None),
                        "issue_active_ncu": SOR_NCU["issue_active"] if args.workload == "spheroid_1M_161" else None,
                        "source": SOR_NCU["source"] if args.workload == "spheroid_1M_161" else None},
                    "streaming_equivalent_GBps": round(8.0 * nodes / (half_us / 1e6) / 1e9, 1)}
    elif dominant:
        s = stages[dominant]
        unit_ms = s["ms"] / max(1, s["calls"])
        nbytes = stage_bytes(dominant, cells_per_step, nodes, 1)
        achieved = nbytes / (unit_ms / 1e3) / 1e9
        roofline = {"bound": "hbm", "kernel": dominant, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                    "frac": round(achieved / peak, 4), "traffic": None, "peak_source": peak_source,
                    "bytes_per_unit": nbytes, "unit_us": round(unit_ms * 1e3, 3)}
    deposit_roofline = None
    if "deposit" in stages and "convert" in stages:
        # The deposit stage as a whole (atomics + conversion + n_eff), against the compulsory
        # bytes 16 N + 4 M (positions and states in, n_eff out) and the bytes this design moves.
        ms = (stages["deposit"]["ms"] + stages["convert"]["ms"]) / steps
        compulsory = 16.0 * cells_per_step + 4.0 * nodes
        moved = stage_bytes("deposit", cells_per_step, nodes, 1) + stage_bytes("convert", cells_per_step, nodes, 1)
        deposit_roofline = {"bound": "hbm", "achieved": round(compulsory / (ms / 1e3) / 1e9, 1), "peak": peak,
                            "unit": "GB/s", "frac": round(compulsory / (ms / 1e3) / 1e9 / peak, 4),
                            "moved_GBps": round(moved / (ms / 1e3) / 1e9, 1), "us_per_step": round(ms * 1e3, 2),
                            "deposit_us_per_step": round(stages["deposit"]["ms"] / steps * 1e3, 2),
                            "convert_us_per_step": round(stages["convert"]["ms"] / steps * 1e3, 2)}
        if "scatter_reference" in r0:
            ref = dict(r0["scatter_reference"])
            ref["k_deposit_adds_per_s"] = round(8.0 * cells_per_step / (stages["deposit"]["ms"] / steps / 1e3), 1)
            deposit_roofline["scatter_reference"] = ref
    breakdown = {k: {"ms_per_step": round(v["ms"] / steps, 4), "launches_per_step": v["launches"] / steps,
                     "GB/s": round(stage_bytes(k, cells_per_step, nodes, int(v["launches"] / steps)) /
                                   (v["ms"] / steps / 1e3) / 1e9, 1) if v["ms"] > 0 and k != "sor" else None}
                 for k, v in sorted(stages.items(), key=lambda kv: -kv[1]["ms"])}
    out = {
        "metric": metric_for(args.workload),
        "value": round(value, 1),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(max_ms / steps, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32 fields/positions, int64 deposit, uint32 streams",
        "data": "synthetic (seeded uniform ball, clipped-normal radii)",
        "config": workload_config(args.workload, nodes),
        "notes": {"sor": "omega 1.8, tol 1e-6, check every 20, max 2000", "dt_h": DT, "mechanics_substeps": 1,
                  "parallelism": f"replicas x{world}",
                  "l2": "inputs larger than L2: per-step working set (cells ~60 MB + int64 accumulator "
                        f"{4 * 8 * nodes / 1e6:.0f} MB + fields) exceeds the 129 MB L2"},
        "gpu_launches": int(r0["launches"]),
        "e2e": {"value": round(e2e_value, 1), "unit": UNIT, "h2d_bytes_per_step": int(r0["h2d"]),
                "d2h_bytes_per_step": int(r0["d2h"])},
        "roofline": roofline,
        "roofline_deposit": deposit_roofline,
        "stages": breakdown,
        "sor_sweeps_per_step": r0["sweeps"],
        "sor_solver": {"path": "shared-memory resident" if r0.get("sor_path") == 2 else "streaming",
                       "ctas": r0.get("sor_tiles"), "strips": r0.get("sor_strips"),
                       "autotuned": r0.get("sor_autotune")},
        "initial_solve_sweeps": r0["initial_sweeps"],
        "clocks": r0["clocks"],
        "cells_final": r0["count"],
    }
    if "cpu_baseline" in r0:
        out["cpu_baseline"] = r0["cpu_baseline"]
        out["parity_full_size_bitwise"] = r0["parity_full_size"]
    return out


# ---- reference arm (CPU) ---------------------------------------------------------------------------------------
def run_reference(args) -> dict:
    from oracle import oracle as orc

    w = WORKLOADS[args.workload]
    P = make_params(w)
    pos, radii = make_cells(w, seed=args.seed)
    from warpbiocell_gb300.fields.oxygen import species_params

    capacity = int(w["cells"] * 1.5)
    sim = orc.OracleSim.from_numpy(pos, radii, capacity=capacity, seed=args.seed)
    g = P["geom"]
    og = orc.Geometry(g.origin, g.dx, g.shape)
    species = [orc.OracleSpecies(og, (0, 0, 0), s.boundary_value, s.diffusion, s.uptake_max, s.michaelis_k,
                                 P["settings"], production=s.production, name=s.name)
               for s in [species_params(P["oxygen"])] + list(P["species"])]
    src = {s.name: s.production_source for s in P["species"] if s.production_source}
    onet = None
    if P["network"] is not None:
        params = P["network"]
        net = params.network
        sources = {"oxygen": 0, "glucose": 1, "constant": 4}
        clamps = tuple((net.index[c.node], sources[c.source], float(np.float32(c.threshold)), 1 if c.above else 0)
                       for c in params.inputs)
        onet = orc.OracleNetwork(net.programs(), net.n_nodes, capacity, update=params.update,
                                 updates_per_step=params.updates_per_step, clamps=clamps,
                                 fate_nodes=params.fate_node_indices())
        onet.initialize(sim)
    threads = orc.num_threads()
    contact, stepping = P["contact"], P["stepping"]
    sim.contact_substep(contact.query_radius, 128, contact.query_radius, contact.rate, 0.0)
    orc.metabolic_update(sim, species, src)  # initial field solve, as the reference's Experiment.run

    def step(timings=None):
        orc.full_cell_step(sim, P["lifecycle"], contact, stepping.dt_cells, stepping.dt_mechanics, species, src,
                           network=onet, timings=timings)

    for _ in range(args.warmup):
        step()
    cells = 0
    stage_s: dict = {}
    t0 = time.perf_counter()
    done = 0
    budget_s = args.reference_budget_s
    for _ in range(args.steps):
        cells += sim.count
        step(stage_s)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    elapsed = time.perf_counter() - t0
    value = cells / elapsed
    sample = (f"{done} full cell steps of the workload by the C++ restatement of the reference kernels "
              f"(WarpBioCell's Warp CPU path cannot run here: warp-lang is absent) on {threads} OpenMP threads")
    # One more step on one thread: the reference's Warp CPU mode runs its kernels single-threaded.
    orc.set_threads(1)
    try:
        n1 = sim.count
        t1 = time.perf_counter()
        step()
        one_s = time.perf_counter() - t1
    finally:
        orc.set_threads(threads)
    single = {"value": round(n1 / one_s, 1), "unit": UNIT, "cores": 1,
              "sample": f"the next full cell step ({n1} cells) on one thread; {one_s:.2f} s"}
    return {
        "metric": metric_for(args.workload), "value": round(value, 1), "unit": UNIT, "n_gpus": 0, "steps": done,
        "warmup": args.warmup,
        "ms_per_step": round(elapsed * 1e3 / max(1, done), 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 fields/positions, int64 deposit, uint32 streams",
        "data": "synthetic (seeded uniform ball, clipped-normal radii)",
        "config": workload_config(args.workload, g.node_count),
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 1), "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                         "stages_ms_per_step": {k: round(v * 1e3 / max(1, done), 3) for k, v in stage_s.items()},
                         "single_thread": single, "host": host_cpu()},
        "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def host_cpu() -> dict:
    """The host's logical CPU count, architecture and model name (from lscpu where it is present)."""
    import platform

    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"cpu_count": os.cpu_count(), "machine": platform.machine(), "model": model}


def run_reference_batched(args) -> dict:
    """The sweep as the reference runs it: its instances one after another on the host (the
    reference's Sweep runs one Experiment per configuration). A bounded sample: rounds of one step
    of every instance, until the steps are done or the time budget is spent."""
    from oracle import oracle as orc
    from warpbiocell_gb300.cells.initialization import clipped_normal_radii, uniform_ball
    from warpbiocell_gb300.fields.oxygen import OxygenParams, species_params

    w = WORKLOADS[args.workload]
    P = make_params(dict(box_um=800.0, dx_um=20.0, boundary=38.0))
    specs = batch_specs(w, args.seed)
    contact, stepping = P["contact"], P["stepping"]
    runs = []
    for sp in specs:
        pos = uniform_ball(sp["cells"], sp["ball"], seed=sp["seed"])
        radii = clipped_normal_radii(sp["cells"], 8.0, 0.8, 6.0, 10.0, seed=sp["seed"] + 1)
        sim = orc.OracleSim.from_numpy(pos, radii, capacity=3 * sp["cells"], seed=sp["seed"])
        half = 0.5 * (sp["nodes"] - 1) * sp["dx"]
        og = orc.Geometry((-half,) * 3, sp["dx"], (sp["nodes"],) * 3)
        s = species_params(OxygenParams(diffusion_coefficient=DIFFUSION, uptake_max=VMAX, michaelis_k=KM,
                                        boundary_value=sp["boundary"]))
        species = [orc.OracleSpecies(og, (0, 0, 0), s.boundary_value, s.diffusion, s.uptake_max, s.michaelis_k,
                                     P["settings"], production=s.production, name=s.name)]
        sim.contact_substep(contact.query_radius, 128, contact.query_radius, contact.rate, 0.0)
        orc.metabolic_update(sim, species, {})  # initial field solve, as the reference's Experiment.run
        runs.append((sim, species))
    threads = orc.num_threads()

    def step(sim, species):
        orc.full_cell_step(sim, P["lifecycle"], contact, stepping.dt_cells, stepping.dt_mechanics, species, {})

    for _ in range(args.warmup):
        for sim, species in runs:
            step(sim, species)
    cells, done = 0, 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for sim, species in runs:
            cells += sim.count
            step(sim, species)
        done += 1
        if time.perf_counter() - t0 > args.reference_budget_s:
            break
    elapsed = time.perf_counter() - t0
    value = cells / elapsed
    sample = (f"{done} rounds of one full cell step of each of the {len(runs)} instances, one instance after "
              f"another, by the C++ restatement of the reference kernels (WarpBioCell's Warp CPU path cannot "
              f"run here: warp-lang is absent) on {threads} OpenMP threads")
    unit = "cell-steps/s"
    return {
        "metric": metric_for(args.workload),
        "value": round(value, 1), "unit": unit, "n_gpus": 0, "steps": done, "warmup": args.warmup,
        "ms_per_step": round(elapsed * 1e3 / max(1, done), 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 fields/positions, int64 deposit, uint32 streams",
        "data": "synthetic (seeded uniform balls, clipped-normal radii)",
        "config": batch_config(args.workload, specs),
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 1), "unit": unit, "cores": threads, "kind": "port", "sample": sample,
                         "host": host_cpu()},
        "e2e": {"value": round(value, 1), "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def reference_unavailable(args) -> dict | None:
    """The line the reference arm prints for a workload whose metric has no CPU counterpart."""
    if WORKLOADS[args.workload].get("adjoint"):
        return {"impl": "reference",
                "unavailable": "the adjoint workload's metric (backward time over forward time) is timed on the "
                               "reference's Warp tape, which needs warp-lang (absent); the C++ restatement has "
                               "no reverse pass (it re-runs the forward in FP64 for central differences only)"}
    return None


# ---- batched sweep (15 spheroids) ----------------------------------------------------------------------
def batch_specs(w: dict, seed: int) -> list[dict]:
    """The sweep's instances: (cells, ball radius, grid nodes, spacing, boundary, seed) each."""
    rng = np.random.default_rng(2026 + seed)
    density = 1.0e6 / (4.0 / 3.0 * math.pi * 1200.0**3)  # cells per um^3 of the 1M-cell workload
    lo, hi = math.log(w["cells_lo"]), math.log(w["cells_hi"])
    specs = []
    for boundary in w["boundaries"]:
        for s in w["seeds"]:
            u = float(rng.random())
            cells = int(round(math.exp(lo + u * (hi - lo))))
            radius = (3.0 * cells / (4.0 * math.pi * density)) ** (1.0 / 3.0)
            nodes = w["nodes_lo"] + 2 * int(round(u * (w["nodes_hi"] - w["nodes_lo"]) / 2))
            box = w["box_over_radius"] * radius
            specs.append(dict(cells=cells, ball=radius, nodes=nodes, dx=box / (nodes - 1), boundary=boundary,
                              seed=1000 * seed + 17 * len(specs) + s))
    return specs


def batch_config(workload: str, specs: list[dict]) -> dict:
    """The `config` object of both arms of the batched workload."""
    return {"workload": workload, "instances": len(specs), "cells": [sp["cells"] for sp in specs],
            "grid_nodes_per_side": [sp["nodes"] for sp in specs], "boundary_mmHg": [sp["boundary"] for sp in specs]}


def build_member(spec: dict, P: dict, dev):
    import torch  # noqa: F401

    from warpbiocell_gb300.cells.initialization import clipped_normal_radii, uniform_ball
    from warpbiocell_gb300.cells.mechanics import contact_substep, make_neighbor_grid
    from warpbiocell_gb300.cells.state import CellPopulation
    from warpbiocell_gb300.fields.oxygen import OxygenField, OxygenParams
    from warpbiocell_gb300.fields.scalar_field import GridGeometry
    from warpbiocell_gb300.simulation.batch import BatchMember

    pos = uniform_ball(spec["cells"], spec["ball"], seed=spec["seed"])
    radii = clipped_normal_radii(spec["cells"], 8.0, 0.8, 6.0, 10.0, seed=spec["seed"] + 1)
    pop = CellPopulation.from_numpy(pos, radii, capacity=3 * spec["cells"], device=dev, seed=spec["seed"])
    half = 0.5 * (spec["nodes"] - 1) * spec["dx"]
    geom = GridGeometry(origin=(-half, -half, -half), dx=spec["dx"], shape=(spec["nodes"],) * 3)
    oxygen = OxygenField(geom, OxygenParams(diffusion_coefficient=DIFFUSION, uptake_max=VMAX, michaelis_k=KM,
                                            boundary_value=spec["boundary"]), P["settings"], device=dev)
    grid = make_neighbor_grid(P["contact"], dev)
    # As the reference's Experiment.run: initial neighbour counts and an initial field solve.
    contact_substep(pop, grid, P["contact"], dt=0.0)
    oxygen.update(pop)
    return BatchMember(pop, grid, oxygen, P["lifecycle"], P["contact"])


def run_batched(args, rank: int = 0, world: int = 1) -> dict:
    """The batched sweep; with several ranks the instances are sharded (no collective on the data
    path): each rank batches its share, balanced by simulation.sweep.partition_runs."""
    import torch

    from warpbiocell_gb300.simulation.batch import SpheroidBatch
    from warpbiocell_gb300.simulation.simulator import cell_step
    from warpbiocell_gb300.simulation.sweep import partition_runs

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    w = WORKLOADS[args.workload]
    P = make_params(dict(box_um=800.0, dx_um=20.0, boundary=38.0))
    all_specs = batch_specs(w, args.seed)
    if world > len(all_specs):
        raise SystemExit(f"{world} ranks for {len(all_specs)} instances: some ranks would have nothing to run")
    share = partition_runs([float(sp["cells"] + sp["nodes"] ** 3) for sp in all_specs], world)[rank]
    specs = [all_specs[i] for i in share]
    stepping = P["stepping"]

    def timed(fn, name):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.cuda.nvtx.range_push(name)
        out = fn()
        torch.cuda.nvtx.range_pop()
        e1.record()
        torch.cuda.synchronize()
        return out, e0.elapsed_time(e1)

    # 15 plain runs, one after another (warm-up steps, then the timed steps of each run).
    plain = [build_member(sp, P, dev) for sp in specs]

    def run_plain(steps):
        cell_steps = 0
        for m in plain:
            for _ in range(steps):
                cell_steps += m.population.count
                cell_step(m.population, m.grid, m.lifecycle, m.contact, stepping, oxygen=m.oxygen)
        return cell_steps

    run_plain(args.warmup)
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    sampler.start()
    time.sleep(0.3)
    plain_cells, plain_ms = timed(lambda: run_plain(args.steps), "sequential_steps")

    # The same 15 runs as one batch: the first warm-up steps outside the graph, the solve plan
    # re-made from the mean sweep counts of those after the first (which starts from the initial
    # field), then capture.
    members = [build_member(sp, P, dev) for sp in specs]
    batch = SpheroidBatch(members, stepping)
    plan_steps = max(1, min(args.batch_plan_steps, args.warmup))
    history = []
    for k in range(plan_steps):
        batch.step(1)
        if k > 0 or plan_steps == 1:
            history.append([r.sweeps for r in batch.reports()])
    batch.rebalance([sum(col) / len(col) for col in zip(*history)])
    batch.capture()
    if args.warmup > plan_steps:
        batch.step(args.warmup - plan_steps)
    _, batch_ms = timed(lambda: batch.step(args.steps), "timed_steps")
    clocks = sampler.stop()
    counts = batch.sync()
    identical = batch.status_codes() == [0] * len(specs)
    for m, p in zip(members, plain):
        a, b = m.population, p.population
        identical = identical and a.count == b.count
        n = a.count
        for name in ("position", "radius", "cell_state", "age", "oxygen_local", "rng_state", "velocity",
                     "neighbor_count"):
            identical = identical and torch.equal(getattr(a, name)[:n], getattr(b, name)[:n])
        identical = identical and torch.equal(m.oxygen.field.values, p.oxygen.field.values)
    reps = batch.reports()
    if world > 1:
        import torch.distributed as dist

        part = {"plain_cells": plain_cells, "plain_ms": plain_ms, "batch_ms": batch_ms, "identical": bool(identical),
                "counts": counts, "sweeps": [r.sweeps for r in reps], "launches": int(batch.launches_per_step),
                "share": share}
        gathered = [None] * world
        dist.all_gather_object(gathered, part)
        plain_cells = sum(g["plain_cells"] for g in gathered)
        plain_ms = max(g["plain_ms"] for g in gathered)
        batch_ms = max(g["batch_ms"] for g in gathered)
        identical = all(g["identical"] for g in gathered)
        order = [i for g in gathered for i in g["share"]]
        counts = [c for g in gathered for c in g["counts"]]
        counts = [c for _, c in sorted(zip(order, counts))]
        last_sweeps = [s_ for _, s_ in sorted(zip(order, [x for g in gathered for x in g["sweeps"]]))]
        launches = sum(g["launches"] for g in gathered)
        specs = all_specs
    else:
        last_sweeps = [r.sweeps for r in reps]
        launches = int(batch.launches_per_step)
    steps = max(1, args.steps)
    value = plain_cells / (batch_ms / 1e3)
    plain_value = plain_cells / (plain_ms / 1e3)
    nodes = sum(sp["nodes"] ** 3 for sp in specs)
    return {
        "metric": metric_for(args.workload),
        "value": round(value, 1), "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(batch_ms / steps, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 fields/positions, int64 deposit, uint32 streams",
        "data": "synthetic (seeded uniform balls, clipped-normal radii)",
        "config": batch_config(args.workload, specs),
        "notes": {"total_grid_nodes": nodes, "sor": "omega 1.8, tol 1e-6, check every 20, max 2000", "dt_h": DT,
                  "parallelism": "one GPU, instances batched" if world == 1 else
                  f"{world} GPUs, instances sharded by rank and batched on each"},
        "clocks": clocks,
        "sequential": {"value": round(plain_value, 1), "ms_per_step": round(plain_ms / steps, 4),
                       "what": "the same runs through the plain per-run path (cell_step), one after another "
                               "(on each rank, its share)"},
        "speedup_vs_sequential": round(plain_ms / batch_ms, 3),
        "identical_outputs": bool(identical),
        "gpu_launches": int(launches * args.steps),
        "launches_per_step": int(launches),
        "final_counts": counts,
        "last_solve_sweeps": last_sweeps,
        "sor_batch": {"tiles": int(batch.sor.total_tiles), "ctas": int(batch.sor.ctas),
                      "smem_bytes": int(batch.sor.smem_bytes)},
    }


# ---- adjoint (config D) ----------------------------------------------------------------------------------
def run_adjoint(args) -> dict:
    import torch

    from warpbiocell_gb300 import _lib
    from warpbiocell_gb300.cells.initialization import clipped_normal_radii, uniform_ball
    from warpbiocell_gb300.cells.mechanics import ContactParams
    from warpbiocell_gb300.fields.scalar_field import GridGeometry
    from warpbiocell_gb300.simulation.adjoint import AdjointSpheroid, CoupledSteadyState

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    w = WORKLOADS[args.workload]
    rng = np.random.default_rng(args.seed + 11)
    pos = uniform_ball(w["cells"], w["ball_um"], seed=args.seed)
    radii = clipped_normal_radii(w["cells"], 8.0, 0.8, 6.0, 10.0, seed=args.seed + 1)
    half = 0.5 * (w["nodes"] - 1) * w["dx_um"]
    geom = GridGeometry(origin=(-half,) * 3, dx=w["dx_um"], shape=(w["nodes"],) * 3)
    contact = ContactParams(stiffness=1.0, damping=1.0, max_radius=10.0)
    model = AdjointSpheroid(torch.from_numpy(pos), torch.from_numpy(radii), geom, w["steps"], DT, contact=contact,
                            adjoint_tolerance=1e-6, device=dev)
    vmax = (VMAX * np.exp(w["vmax_sigma"] * rng.standard_normal(w["cells"]))).astype(np.float32)
    theta = dict(km=KM, diffusion=DIFFUSION, boundary=w["boundary"], stiffness=1.0)
    pert = {k: v * (1.0 + 0.2 * (2 * rng.random() - 1)) for k, v in theta.items()}
    vmax_t = torch.from_numpy((vmax * (1.0 + 0.2 * (2 * rng.random(vmax.size) - 1))).astype(np.float32)).to(dev)
    with torch.no_grad():
        u_t, x_t = model.forward(vmax_t, pert["km"], pert["diffusion"], pert["boundary"], pert["stiffness"])
    u_t = u_t.double()
    rho_t = (x_t.double() - x_t.double().mean(dim=0)).norm(dim=1)
    v0 = torch.from_numpy(vmax).to(dev)

    def loss_of(u, x):
        xd = x.double()
        return ((u.double() - u_t) ** 2).sum() + (((xd - xd.mean(dim=0)).norm(dim=1) - rho_t) ** 2).sum()

    def timed(fn, name):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.cuda.nvtx.range_push(name)
        out = fn()
        torch.cuda.nvtx.range_pop()
        e1.record()
        torch.cuda.synchronize()
        return out, e0.elapsed_time(e1)

    fwd_ms, bwd_ms = [], []
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    sampler.start()
    time.sleep(0.3)
    launches0 = _lib.launch_count()
    reps = max(1, args.warmup) + max(1, args.steps)
    for rep in range(reps):
        v = v0.clone().requires_grad_(True)
        scal = {k: torch.tensor(val, dtype=torch.float64, requires_grad=True) for k, val in theta.items()}
        (u, x), f_ms = timed(lambda: CoupledSteadyState.apply(v, scal["km"], scal["diffusion"], scal["boundary"],
                                                                scal["stiffness"], model), "adjoint_forward")
        loss = loss_of(u, x)
        _, b_ms = timed(loss.backward, "adjoint_backward")
        if rep >= max(1, args.warmup):
            fwd_ms.append(f_ms)
            bwd_ms.append(b_ms)
    launches = _lib.launch_count() - launches0
    clocks = sampler.stop()
    grads = {k: float(t.grad) for k, t in scal.items()}
    grad_v = v.grad.double().cpu().numpy()
    result = {
        "metric": metric_for(args.workload),
        "value": round(float(np.median(bwd_ms)) / float(np.median(fwd_ms)), 3), "unit": "x forward",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32 forward, fp32 adjoint with fp64 scalar sums",
        "data": "synthetic (seeded uniform ball, clipped-normal radii, log-normal Vmax)",
        "config": workload_config(args.workload),
        "forward_ms": round(float(np.median(fwd_ms)), 3), "backward_ms": round(float(np.median(bwd_ms)), 3),
        "forward_sweeps": model.last_forward_sweeps, "adjoint_sweeps": model.last_adjoint_sweeps,
        "adjoint_converged": model.last_adjoint_converged,
        "gpu_launches": int(launches),
        "launches_per_forward_backward": round(launches / reps, 1),
        "gradients": {**grads, "vmax_norm": float(np.linalg.norm(grad_v))},
        "clocks": clocks,
    }
    if not args.skip_cpu:
        result.update(adjoint_fp64_checks(args, w, pos, radii, geom, vmax, theta, grads, grad_v, u_t, rho_t, rng))
    return result


def adjoint_fp64_checks(args, w, pos, radii, geom, vmax, theta, grads, grad_v, u_t, rho_t, rng) -> dict:
    """The GPU gradients against (a) the oracle's FP64 adjoint of the same model and (b) central
    differences of the oracle's FP64 forward (double contact steps, exact deposit, double SOR to
    1e-13), for all five: Km, D, boundary O2, stiffness and a random per-cell Vmax direction; for
    the stiffness also at smaller steps, each with the count of contact-onset crossings (pairs in
    contact at some step of one of the two trajectories but not the other) the difference spans."""
    sys.path.insert(0, str(ROOT))
    from oracle import oracle as orc

    orc.set_threads(os.cpu_count() or 1)
    t0 = time.perf_counter()
    u64, rho64 = u_t.cpu().numpy(), rho_t.cpu().numpy()
    og = orc.Geometry(geom.origin, geom.dx, geom.shape)
    vm64 = vmax.astype(np.float64)
    qr = 20.0

    def forward64(vm, km, diffusion, boundary, stiffness):
        return orc.adjoint_forward_f64(pos, radii, vm, og, w["steps"], DT, stiffness, qr, qr, 128, diffusion, km,
                                       boundary)[:2]

    def loss64(vm, **th):
        field, p = forward64(vm, **th)
        return float(((field - u64) ** 2).sum() + ((np.linalg.norm(p - p.mean(axis=0), axis=1) - rho64) ** 2).sum())

    def loss_grads(field, p):
        c = p - p.mean(axis=0)
        rho = np.linalg.norm(c, axis=1)
        gx = (2.0 * (rho - rho64))[:, None] * c / rho[:, None]
        return 2.0 * (field - u64), gx - gx.mean(axis=0)

    f64 = orc.adjoint_gradients_f64(pos, radii, vm64, og, w["steps"], DT, theta["stiffness"], 1.0, qr, qr, 128,
                                    theta["diffusion"], theta["km"], theta["boundary"], loss_grads)
    vs_adjoint = {k: abs(grads[k] - f64[k]) / abs(f64[k]) for k in ("km", "diffusion", "boundary", "stiffness")}
    d = np.where(rng.random(vmax.size) < 0.5, -1.0, 1.0)
    gpu_dir = float((grad_v * vm64 * d).sum())
    f64_dir = float((f64["vmax"] * vm64 * d).sum())
    vs_adjoint["vmax_direction"] = abs(gpu_dir - f64_dir) / abs(f64_dir)
    rel = 1e-4
    vs_fd = {}
    fd_values = {}
    for name in ("km", "diffusion", "boundary", "stiffness"):
        h = rel * theta[name]
        hi, lo = dict(theta), dict(theta)
        hi[name] += h
        lo[name] -= h
        fd = (loss64(vm64, **hi) - loss64(vm64, **lo)) / (2 * h)
        fd_values[name] = fd
        vs_fd[name] = abs(grads[name] - fd) / abs(fd)
    fd = (loss64(vm64 * (1 + rel * d), **theta) - loss64(vm64 * (1 - rel * d), **theta)) / (2 * rel)
    vs_fd["vmax_direction"] = abs(gpu_dir - fd) / abs(fd)
    stiffness_steps = {}
    for r in (1e-4, 1e-5, 1e-6):
        hi, lo = dict(theta), dict(theta)
        hi["stiffness"] *= 1 + r
        lo["stiffness"] *= 1 - r
        fd_r = fd_values["stiffness"] if r == rel else \
            (loss64(vm64, **hi) - loss64(vm64, **lo)) / (2 * r * theta["stiffness"])
        crossings = orc.contact_crossings_f64(pos, radii, w["steps"], DT, hi["stiffness"], lo["stiffness"], qr, qr,
                                              128)
        stiffness_steps[f"{r:g}"] = {"gpu_vs_fd": float(f"{abs(grads['stiffness'] - fd_r) / abs(fd_r):.3g}"),
                                     "fp64_adjoint_vs_fd": float(f"{abs(f64['stiffness'] - fd_r) / abs(fd_r):.3g}"),
                                     "contact_crossings": crossings}
    return {"fp64_central_difference_rel_error": {k: float(f"{e:.3g}") for k, e in vs_fd.items()},
            "fp64_adjoint_rel_error": {k: float(f"{e:.3g}") for k, e in vs_adjoint.items()},
            "stiffness_by_step": stiffness_steps,
            "fd_step": rel, "fp64_check_s": round(time.perf_counter() - t0, 1)}


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="spheroid_1M_161")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--skip-cpu", action="store_true", help="skip the CPU baseline sample and parity check")
    ap.add_argument("--reference-budget-s", type=float, default=120.0)
    ap.add_argument("--batch-plan-steps", type=int, default=4,
                    help="batched sweep: warm-up steps before the solve plan is re-made from their mean sweep counts "
                         "(leaving out the first step's; at most --warmup)")
    ap.add_argument("--sor-tuning", default="",
                    help="tiles,strips for the resident solver instead of the autotuner's pick")
    ap.add_argument("--no-extras", action="store_true",
                    help="headline workload only: skip the batched-sweep and adjoint halves of the metric")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        print("note: fewer than 3 warm-up steps", file=sys.stderr)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            out = reference_unavailable(args)
            if out is None:
                out = run_reference_batched(args) if WORKLOADS[args.workload].get("batched") else run_reference(args)
            print(json.dumps(out))
        return
    if WORKLOADS[args.workload].get("batched"):
        if world > 1:
            import torch
            import torch.distributed as dist

            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
            dist.init_process_group("nccl")
        out = run_batched(args, rank, world)
        if rank == 0:
            print(json.dumps(out))
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()
        return
    if WORKLOADS[args.workload].get("adjoint"):
        if rank == 0:
            print(json.dumps(run_adjoint(args)))
        return

    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    result = run_gpu(args, rank, world)
    if world > 1:
        import torch.distributed as dist

        gathered = [None] * world
        dist.all_gather_object(gathered, result)
        results = gathered
    else:
        results = [result]
    if rank == 0:
        line = report_gpu(args, results, world)
        if world == 1 and args.workload == "spheroid_1M_161" and not args.no_extras:
            line.update(metric_extras(args))
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def metric_extras(args) -> dict:
    """The other two parts of the metric, measured on the same GPU after the headline steps: the
    15-spheroid batched sweep against the same runs looped through the plain path, and the
    adjoint's backward time over its forward time with its gradients checked against FP64; then
    the two other single-spheroid configurations (10k cells on 41^3, and the three-species
    100k-cell run with Boolean networks on 81^3), each with its full-size bitwise parity check."""
    import copy

    import torch

    out = {}
    configs = {}
    for workload in ("spheroid_10k_41", "metabolic_network_100k_81"):
        c_args = copy.copy(args)
        c_args.workload = workload
        c_args.steps = min(args.steps, 10)
        c = report_gpu(c_args, [run_gpu(c_args, 0, 1)], 1)
        keep = ("metric", "value", "unit", "ms_per_step", "steps", "warmup", "e2e", "gpu_launches",
                "parity_full_size_bitwise", "cpu_baseline", "clocks", "config")
        configs[workload] = {k: c[k] for k in keep if k in c}
        torch.cuda.empty_cache()
    out["configs"] = configs
    b_args = copy.copy(args)
    b_args.workload = "batched_sweep_15"
    b = run_batched(b_args)
    out["batched"] = {"workload": b_args.workload, "ratio_vs_sequential": b["speedup_vs_sequential"],
                      "identical_outputs": b["identical_outputs"], "batched_ms_per_step": b["ms_per_step"],
                      "sequential_ms_per_step": b["sequential"]["ms_per_step"], "value": b["value"],
                      "unit": b["unit"], "steps": b["steps"], "warmup": b["warmup"],
                      "launches_per_step": b["launches_per_step"], "config": b["config"], "clocks": b["clocks"]}
    torch.cuda.empty_cache()
    a_args = copy.copy(args)
    a_args.workload = "adjoint_100k_81"
    a = run_adjoint(a_args)
    keep = ("value", "unit", "forward_ms", "backward_ms", "forward_sweeps", "adjoint_sweeps", "adjoint_converged",
            "launches_per_forward_backward", "fp64_central_difference_rel_error", "fp64_adjoint_rel_error",
            "stiffness_by_step", "fd_step", "clocks", "config")
    out["adjoint"] = {"workload": a_args.workload, "what": "backward time / forward time", "steps": a["steps"],
                      **{k: a[k] for k in keep if k in a}}
    return out


if __name__ == "__main__":
    main()
