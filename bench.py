#!/usr/bin/env python
"""Throughput benchmark of the force-and-step path on GB300.

Workload: 30,000 flexible three-site waters in a 96.5 A cubic box plus a
solvated 500-bead chain (88,289 atoms after overlap removal), LJ cutoff 12 A
switched from 10 A, Ewald real space (tolerance 1e-5) + PME 96^3 order 4,
bonds/angles/dihedrals, Langevin 300 K, 1 fs, friction 1/ps.  Seeded
synthetic coordinates (no dataset exists for this benchmark).

A "step" is one MD step (one force evaluation + the FP64 update).  Each timed
step is one CUDA-graph replay bracketed by CUDA events on the launching
stream; a 256 MB buffer is rewritten between timed steps to flush the 129 MB
L2 (the working set, ~25 MB, would otherwise stay L2-resident).

Beside the plain form it times the multiple-time-step forms on the same
system: the impulse scheme with PME every k steps (--mts) and the learned
slow force with PME every k steps (--learned; trained first on frame pairs
of a plain Langevin run at 280-320 K).  Each form's NVE drift (100 ps after
20 ps of Langevin) gates it; "chosen" is the fastest form that passes.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

N > 1 runs one independent replica per GPU (torchrun; the path does not
shard): value = all replicas' simulated time / max-over-ranks wall time.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

METRIC = "ns/day & atom-steps/s on 1 GB300 at force err <=1e-4 vs FP64; plain vs chosen"
DT_FS = 1.0
TEMPERATURE = 300.0
FRICTION = 0.001          # 1/ps in 1/fs
CUTOFF, SWITCH, ORDER, EWALD_TOL = 12.0, 10.0, 4, 1e-5
# single-system workloads: waters, box edge (A), chain beads, PME grid
WORKLOADS = {"water90k": (30000, 96.5, 500, 96), "water1m": (333333, 215.0, 0, 224)}
L2_FLUSH_BYTES = 256 << 20
PEAKS = os.path.join(HERE, "MEASURED_PEAKS.json")
PROFILE_INPUTS = os.path.join(HERE, "profiles", "roofline_inputs.json")
FP32_PEAK_TFLOPS_NOMINAL = 152 * 128 * 2 * 2.07e9 / 1e12   # 152 SMs x 128 FP32 lanes x FMA x 2.07 GHz


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3000)
    p.add_argument("--warmup", type=int, default=50)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="water90k", choices=["water90k", "water1m", "batch256"],
                   help="water90k: the 88k-atom water + chain box (default); water1m: 333,333 "
                        "waters (1M atoms) in a 215 A box; batch256: 256 independent water "
                        "boxes of 1.5k-12k atoms in one batch")
    p.add_argument("--boxes", type=int, default=256)
    p.add_argument("--mts", default="2,3,4",
                   help="outer steps (in steps) of the multiple-time-step forms timed beside the "
                        "plain one, comma separated (empty: none)")
    p.add_argument("--learned", default="4",
                   help="outer steps of the learned slow-force forms (trained at the start, "
                        "comma separated; empty: none)")
    p.add_argument("--learned-iters", type=int, default=400,
                   help="training iterations (frame pairs) of each learned form")
    p.add_argument("--learned-threshold", type=float, default=0.05,
                   help="judge threshold of the learned forms (RMS slow-force error over RMS "
                        "total force) above which an interval falls back to the impulse scheme")
    p.add_argument("--profile-learned", type=int, default=0, metavar="K",
                   help="profiling run of the learned form only: the water90k box, feature "
                        "normalisation from one frame pair (no training), 40 plain steps, "
                        "then 40 learned steps with PME every K steps; prints the times")
    p.add_argument("--no-autotune", action="store_true",
                   help="keep the default launch shape instead of timing the alternatives")
    p.add_argument("--waters", type=int, default=None)
    p.add_argument("--box", type=float, default=None)
    p.add_argument("--beads", type=int, default=None)
    p.add_argument("--e2e-steps", type=int, default=100)
    p.add_argument("--kernel-reps", type=int, default=200)
    p.add_argument("--cpu-seconds", type=float, default=20.0)
    p.add_argument("--no-error-check", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--nve-ps", type=float, default=None,
                   help="velocity-Verlet NVE run after the timed region for the energy drift "
                        "(default 100 ps on water90k, 0 elsewhere)")
    a = p.parse_args()
    w, b, beads, grid = WORKLOADS.get(a.workload, WORKLOADS["water90k"])
    a.waters = w if a.waters is None else a.waters
    a.box = b if a.box is None else a.box
    a.beads = beads if a.beads is None else a.beads
    a.grid = grid
    if a.nve_ps is None:
        a.nve_ps = 100.0 if a.workload == "water90k" else 0.0
    if a.workload == "water1m":
        # the FP64 references (all-pairs Coulomb, direct Ewald k-sum) do not
        # finish at 1M atoms; the 88k-atom box carries both numbers
        a.no_error_check = True
        a.no_cpu_baseline = True
    return a


def workload_name(a, n_atoms):
    return ("water%dk_chain%d_%.1fA_%d_atoms_rc%g_sw%g_pme%d_o%d_langevin300K_1fs"
            % (a.waters // 1000, a.beads, a.box, n_atoms, CUTOFF, SWITCH, a.grid, ORDER))


def make_system(a, seed):
    from mdpy_gb300 import systems

    if a.beads == 0:
        return systems.water_box(a.waters, a.box, seed=seed)
    return systems.chain_in_water(n_waters=a.waters, box=a.box, n_beads=a.beads, seed=seed)


def make_ensemble(s, device, grid):
    from mdpy_gb300 import constraint as C
    from mdpy_gb300.ensemble import Ensemble

    ens = Ensemble(s.topology, s.pbc_matrix, device=device)
    nb = C.NonbondedConstraint(s.parameters["nonbonded"], cutoff_radius=CUTOFF,
                               switch_radius=SWITCH, ewald_error=EWALD_TOL)
    pme = C.PMEConstraint(grid_size=grid, order=ORDER, ewald_error=EWALD_TOL,
                          real_space_cutoff=CUTOFF)
    cons = [nb, pme, C.CharmmBondConstraint(s.parameters["bond"]),
            C.CharmmAngleConstraint(s.parameters["angle"])]
    if s.topology.num_dihedrals:
        cons.append(C.CharmmDihedralConstraint(None, float_parameters=s.dihedral_parameters))
    ens.add_constraints(*cons)
    ens.state.set_positions(s.positions)
    ens.state.set_velocities(s.velocities)
    return ens, nb.ewald_beta


BATCH_CUTOFF = 10.0


def make_batch_members(n_boxes, seed):
    """256 water boxes, atom counts log-uniform in [1500, 12000], each with a
    PME grid of ~1 A spacing clipped to 24..48, cutoff 10 A."""
    from mdpy_gb300 import batch, constraint as C, systems

    ws = systems.water_box_batch(n_boxes, 1500, 12000, seed=seed)
    members = []
    for w in ws:
        grid = min(48, max(24, systems.fft_friendly(int(round(w.box[0])))))
        ens = batch.member(w.topology, w.pbc_matrix)
        ens.add_constraints(
            C.NonbondedConstraint(w.parameters["nonbonded"], BATCH_CUTOFF, ewald_error=EWALD_TOL),
            C.PMEConstraint(grid_size=grid, ewald_error=EWALD_TOL, real_space_cutoff=BATCH_CUTOFF),
            C.CharmmBondConstraint(w.parameters["bond"]),
            C.CharmmAngleConstraint(w.parameters["angle"]))
        ens.state.set_positions(w.positions)
        ens.state.set_velocities(w.velocities)
        members.append((w, ens, grid))
    return members


def time_steps(sysm, mask, steps, stream, flush):
    import torch

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for k in range(steps):
        flush.fill_(k & 0xFF)
        starts[k].record(stream)
        sysm.integrate(1, mask, want_energy=False)
        ends[k].record(stream)
    torch.cuda.synchronize()
    return sum(st.elapsed_time(en) for st, en in zip(starts, ends))


def run_batch(a, world, rank, local):
    """Batched form: every box in one device batch (one set of launches per
    step, one CUDA graph per step), against the same boxes run one at a time
    (a sample of every 8th box, scaled by its share of the atoms)."""
    import torch

    from mdpy_gb300 import _lib, batch, unit
    from mdpy_gb300.ensemble import Ensemble
    from mdpy_gb300.integrator import LangevinIntegrator

    torch.cuda.set_device(local)
    members = make_batch_members(a.boxes, seed=rank)
    b = batch.EnsembleBatch([m[1] for m in members], device=local)
    sysm = b.system
    n = sysm.n
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sysm.set_stream(stream.cuda_stream)
    integ = LangevinIntegrator(DT_FS, TEMPERATURE, FRICTION, seed=1000 + rank)
    integ._configure(b)
    mask = b.term_mask
    sysm.set_graph_mode(_lib.GRAPH_STEP)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    shape = sysm.launch_shape if a.no_autotune else sysm.autotune(mask, reps=5)
    sysm.integrate(max(a.warmup, 3), mask, want_energy=False)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier(world)
    torch.cuda.synchronize()
    launches0 = sysm.launch_count
    ms_total = time_steps(sysm, mask, a.steps, stream, flush)
    launches = sysm.launch_count - launches0
    clk = clocks.stop()
    ms_total = reduce_max(ms_total, world, device=torch.device("cuda", local)
                          if world > 1 and os.environ.get("MDG_BENCH_BACKEND", "nccl") == "nccl"
                          else None)
    sysm.check_status()
    ms_step = ms_total / a.steps
    atom_steps = world * n * a.steps / (ms_total / 1000.0)
    # per-box ns/day averaged over boxes = steps/s of the batch
    ns_day_per_box = unit.ns_per_day(a.steps / (ms_total / 1000.0), DT_FS)
    b.update()
    pe = b.potential_energies

    # the same boxes one at a time: every 8th box, each its own system
    sample = members[::8]
    single_ms, single_atoms = 0.0, 0
    for w, _, grid in sample:
        from mdpy_gb300 import constraint as C

        ens = Ensemble(w.topology, w.pbc_matrix, device=local)
        ens.add_constraints(
            C.NonbondedConstraint(w.parameters["nonbonded"], BATCH_CUTOFF, ewald_error=EWALD_TOL),
            C.PMEConstraint(grid_size=grid, ewald_error=EWALD_TOL, real_space_cutoff=BATCH_CUTOFF),
            C.CharmmBondConstraint(w.parameters["bond"]),
            C.CharmmAngleConstraint(w.parameters["angle"]))
        ens.state.set_positions(w.positions)
        ens.state.set_velocities(w.velocities)
        ss = ens.system
        ss.set_stream(stream.cuda_stream)
        integ._configure(ens)
        ss.set_graph_mode(_lib.GRAPH_STEP)
        ss.integrate(5, mask, want_energy=False)
        torch.cuda.synchronize()
        reps = max(10, a.steps // 10)
        single_ms += time_steps(ss, mask, reps, stream, flush) / reps
        single_atoms += w.num_particles
        ss.close()
    one_at_a_time_ms = single_ms * (n / single_atoms)
    if rank == 0:
        sizes = [m[0].num_particles for m in members]
        grids = sorted({m[2] for m in members})
        line = {
            "metric": "atom-steps/s, %d independent water boxes on 1 GB300" % a.boxes,
            "value": atom_steps, "unit": "atom-steps/s", "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "batch%d_water_1.5k-12k_atoms_rc%g_pme%d-%d_o4_langevin300K_1fs"
                                   % (a.boxes, BATCH_CUTOFF, grids[0], grids[-1]),
                       "atoms": n, "boxes": a.boxes, "atoms_min": min(sizes),
                       "atoms_max": max(sizes), "pme_grids": grids,
                       "l2": "flushed between timed steps (256 MB rewrite)", "form": "batched",
                       "launch_shape": shape},
            "ns_per_day_per_box": ns_day_per_box,
            "one_at_a_time": {"ms_per_step_all_boxes": one_at_a_time_ms,
                              "atom_steps_per_s": n / (one_at_a_time_ms / 1000.0),
                              "sample": "every 8th box (%d boxes, %d atoms) timed alone, scaled "
                                        "by atoms" % (len(sample), single_atoms)},
            "speedup_vs_one_at_a_time": one_at_a_time_ms / ms_step,
            "finite_energies": bool(np.all(np.isfinite(pe))),
            "gpu_launches": int(launches), "clocks": clk,
        }
        print(json.dumps(line))
    return 0


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------------
# distributed helpers (replicas; gloo on CPU in the tests)
# --------------------------------------------------------------------------
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if os.environ.get("MDG_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
        if backend == "nccl":
            import torch

            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def reduce_max(value, world, device=None):
    """Max of a float over ranks (the bench's wall-time rule)."""
    if world == 1:
        return float(value)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64,
                     device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def nve_drift(sysm, mask, n_atoms, ps, chunk=500, equilibrate_ps=20.0, seed=0, mts=1,
              learned=None):
    """Total-energy drift of a velocity-Verlet run of ``ps`` picoseconds:
    ``equilibrate_ps`` of Langevin at 300 K first (the lattice start relaxes
    for several ps, which shows as a spurious trend), then the least-squares
    slope of E(t), sampled every ``chunk`` steps, in kT per ns per atom."""
    from mdpy_gb300 import _lib, unit

    sysm.set_mts(1)
    sysm.integrator_config(_lib.INTEGRATOR_LANGEVIN, DT_FS, TEMPERATURE, FRICTION, 77 + seed)
    sysm.integrate(int(equilibrate_ps * 1000.0 / DT_FS), mask, want_energy=False)
    sysm.integrator_config(_lib.INTEGRATOR_VERLET, DT_FS)
    if learned is not None:
        learned.enable(sysm)
        sysm.learned_reset_stats()
    else:
        sysm.set_mts(mts)
    n_chunks = max(2, int(round(ps * 1000.0 / DT_FS / chunk)))
    terms = [t for t in range(_lib.NUM_TERMS) if mask >> t & 1]
    t_fs, e_tot = [], []
    t0 = time.perf_counter()
    for k in range(n_chunks):
        sysm.integrate(chunk, mask, want_energy=True)
        e, ke = sysm.get_energies()
        t_fs.append((k + 1) * chunk * DT_FS)
        e_tot.append(float(sum(e[t] for t in terms) + ke))
    wall = time.perf_counter() - t0
    judge = sysm.learned_stats() if learned is not None else None
    sysm.set_mts(1)
    slope = float(np.polyfit(np.array(t_fs), np.array(e_tot), 1)[0])   # energy unit / fs
    kT = unit.KB * TEMPERATURE
    drift = slope * 1e6 / (n_atoms * kT)
    e0 = e_tot[0]
    half = n_chunks // 2
    halves = [float(np.polyfit(np.array(t_fs[i:j]), np.array(e_tot[i:j]), 1)[0]) * 1e6
              / (n_atoms * kT) for i, j in ((0, half), (half, n_chunks))]
    # standard error of the whole-run slope from the spread of 4 block slopes
    # (a slope's noise grows as T^-1.5 for a window of length T)
    nb = 4
    lb = n_chunks // nb
    blocks = [float(np.polyfit(np.array(t_fs[i * lb:(i + 1) * lb]),
                               np.array(e_tot[i * lb:(i + 1) * lb]), 1)[0]) * 1e6
              / (n_atoms * kT) for i in range(nb)]
    stderr = float(np.std(blocks, ddof=1)) / nb ** 1.5
    return {"kT_per_ns_per_atom": drift, "halves_kT_per_ns_per_atom": halves,
            "block_slopes_kT_per_ns_per_atom": blocks, "stderr_kT_per_ns_per_atom": stderr,
            "ps": n_chunks * chunk * DT_FS / 1000.0,
            "samples": n_chunks, "sample_every_steps": chunk,
            "max_abs_dev_kT_per_atom": float(np.max(np.abs(np.array(e_tot) - e0)) / (n_atoms * kT)),
            "integrator": "velocity Verlet, dt 1 fs%s, after %g ps of Langevin at 300 K"
                          % ((", learned slow force, PME every %d steps" % learned.outer_step)
                             if learned is not None else
                             (", reciprocal force every %d steps (impulse)" % mts) if mts > 1
                             else "", equilibrate_ps),
            "judge": judge, "wall_s": wall}


# --------------------------------------------------------------------------
# CPU arm: the oracle port of the reference path, on the host cores
# --------------------------------------------------------------------------
def cpu_reference_sample(s, seconds):
    """mdpy's CPU step restated by the oracle: LJ (cell list, hard cutoff 12 A)
    + bare Coulomb over all pairs + bonds + angles + dihedrals per force
    evaluation, three evaluations per Langevin step as mdpy's
    LangevinIntegrator runs them (mdpy/integrator/langevin_integrator.py:51-64).
    Times whole force evaluations on the full system until ``seconds`` pass."""
    from oracle import oracle as O

    t = s.topology
    n = s.num_particles
    p = s.parameters["nonbonded"]
    lj = np.array([[p[ty][0], p[ty][1], p[ty][0], p[ty][1]] for ty in t.particle_types])
    q = t.charges.reshape(-1)
    types = t.particle_types
    kb = np.array([s.parameters["bond"]["%s-%s" % (types[i], types[j])] for i, j in t.bonds])
    ka = np.array([s.parameters["angle"]["%s-%s-%s" % (types[i], types[j], types[k])]
                   for i, j, k in t.angles])
    threads = O.num_threads()
    evals, t0 = 0, time.perf_counter()
    while True:
        te = time.perf_counter()
        f1, _ = O.nonbonded(s.positions, s.box, lj, q, t.bonded_particles, t.scaling_particles,
                            CUTOFF, coulomb="none")
        f2, _ = O.nonbonded(s.positions, s.box, np.zeros((n, 4)), q, t.bonded_particles,
                            t.scaling_particles, CUTOFF, lj=False, coulomb="bare")
        O.bonds(s.positions, s.box, t.bonds, kb)
        O.angles(s.positions, s.box, t.angles, ka)
        if t.num_dihedrals:
            O.dihedrals(s.positions, s.box, t.dihedrals, s.dihedral_parameters)
        evals += 1
        if time.perf_counter() - t0 >= seconds or time.perf_counter() - te > seconds / 2:
            break
    per_eval = (time.perf_counter() - t0) / evals
    per_step = 3.0 * per_eval
    sps = 1.0 / per_step
    from mdpy_gb300 import unit

    return {
        "ns_per_day": unit.ns_per_day(sps, DT_FS),
        "atom_steps_per_s": n * sps,
        "cores": threads,
        "host_cores": os.cpu_count(),
        "sample": ("%d full force evaluation(s) of the reference path (LJ cell list rc 12 A + "
                   "bare Coulomb over all %d atom pairs + bonds/angles/dihedrals, FP64 C port, "
                   "%d threads) on the %d-atom system; %.2f s per evaluation, x3 per Langevin "
                   "step as mdpy runs it" % (evals, n, threads, n, per_eval)),
    }


# --------------------------------------------------------------------------
# force error vs the FP64 oracle (a sample of atoms; structure factors use all)
# --------------------------------------------------------------------------
def force_error(s, ens, beta, n_sample=1000, seed=0):
    from oracle import oracle as O

    t = s.topology
    n = s.num_particles
    pos = ens.state.positions
    ens.update()
    f_gpu = ens.forces
    p = s.parameters["nonbonded"]
    lj = np.array([[p[ty][0], p[ty][1], p[ty][0], p[ty][1]] for ty in t.particle_types])
    q = t.charges.reshape(-1)
    rng = np.random.default_rng(seed)
    sub = np.sort(rng.choice(n, size=min(n_sample, n), replace=False))
    f_nb, _ = O.nonbonded(pos, s.box, lj, q, t.bonded_particles, t.scaling_particles, CUTOFF,
                          switch=SWITCH, coulomb="ewald", beta=beta)
    f_rec, _ = O.ewald_recip(pos, s.box, q, beta, O.ewald_kmax(s.box, beta, 1e-9), subset=sub)
    f_ex, _ = O.ewald_exclusions(pos, s.box, q, t.bonded_particles, beta)
    types = t.particle_types
    kb = np.array([s.parameters["bond"]["%s-%s" % (types[i], types[j])] for i, j in t.bonds])
    ka = np.array([s.parameters["angle"]["%s-%s-%s" % (types[i], types[j], types[k])]
                   for i, j, k in t.angles])
    f_b, _ = O.bonds(pos, s.box, t.bonds, kb)
    f_a, _ = O.angles(pos, s.box, t.angles, ka)
    f_d = O.dihedrals(pos, s.box, t.dihedrals, s.dihedral_parameters)[0] \
        if t.num_dihedrals else 0.0
    ref = (f_nb + f_ex + f_b + f_a + f_d)[sub] + f_rec
    err = float(np.sqrt(np.sum((f_gpu[sub] - ref) ** 2) / np.sum(ref ** 2)))
    return err, len(sub)


# --------------------------------------------------------------------------
def run_reference_arm(a, world, rank):
    if rank != 0:
        return 0
    s = make_system(a, seed=0)
    r = cpu_reference_sample(s, a.cpu_seconds)
    line = {
        "metric": METRIC, "value": r["ns_per_day"], "unit": "ns/day", "impl": "reference",
        "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": 1000.0 * s.num_particles / r["atom_steps_per_s"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "atom_steps_per_s": r["atom_steps_per_s"],
        "config": {"workload": workload_name(a, s.num_particles), "atoms": s.num_particles,
                   "l2": "n/a (host)"},
        "cpu_baseline": {"value": r["ns_per_day"], "unit": "ns/day", "cores": r["cores"],
                         "kind": "port", "sample": r["sample"]},
        "e2e": {"value": r["ns_per_day"], "unit": "ns/day", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def profile_learned(a):
    """The short run the learned form's profiles are captured on."""
    import torch

    from mdpy_gb300 import _lib
    from mdpy_gb300.learned import LearnedSlowForce

    s = make_system(a, 0)
    ens, _ = make_ensemble(s, 0, a.grid)
    sysm, mask = ens.system, ens.term_mask
    sysm.set_graph_mode(_lib.GRAPH_STEP)
    lrn = LearnedSlowForce(outer_step=a.profile_learned, threshold=1e9)
    sysm.integrator_config(_lib.INTEGRATOR_LANGEVIN, DT_FS, TEMPERATURE, FRICTION, 5)
    lrn.normalise(sysm, mask)
    out = {}
    for name in ("plain", "learned"):
        if name == "learned":
            lrn.enable(sysm)
        sysm.integrate(12, mask, want_energy=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sysm.integrate(40, mask, want_energy=False)
        torch.cuda.synchronize()
        out[name + "_ms_per_step"] = (time.perf_counter() - t0) / 40 * 1e3
    out["judge"] = sysm.learned_stats()
    print(json.dumps(out))
    return 0


def main():
    a = parse()
    if a.profile_learned:
        return profile_learned(a)
    world, rank, local = dist_setup()
    if a.impl == "reference":
        return run_reference_arm(a, world, rank)
    if a.workload == "batch256":
        return run_batch(a, world, rank, local)

    import torch

    from mdpy_gb300 import _lib, unit
    from mdpy_gb300.integrator import LangevinIntegrator

    torch.cuda.set_device(local)
    s = make_system(a, seed=rank)
    n = s.num_particles
    ens, beta = make_ensemble(s, local, a.grid)
    sysm = ens.system
    # a dedicated stream: the library, the L2 flush and the timing events all
    # go to it (torch's default stream is the legacy stream, handle 0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sysm.set_stream(stream.cuda_stream)
    integ = LangevinIntegrator(DT_FS, TEMPERATURE, FRICTION, seed=1000 + rank)
    integ._configure(ens)
    mask = ens.term_mask
    sysm.set_graph_mode(_lib.GRAPH_STEP)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    shape = sysm.launch_shape if a.no_autotune else sysm.autotune(mask, reps=10)

    # warm-up (graphs captured here)
    sysm.integrate(max(a.warmup, 3), mask, want_energy=False)
    torch.cuda.synchronize()

    # ---- timed region: K single-step graph replays, L2 flushed in between --
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(a.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier(world)
    torch.cuda.synchronize()
    launches0 = sysm.launch_count
    for k in range(a.steps):
        flush.fill_(k & 0xFF)
        starts[k].record(stream)
        sysm.integrate(1, mask, want_energy=False)
        ends[k].record(stream)
    torch.cuda.synchronize()
    barrier(world)
    launches = sysm.launch_count - launches0
    clk = clocks.stop()
    ms_total = sum(st.elapsed_time(en) for st, en in zip(starts, ends))
    ms_total = reduce_max(ms_total, world, device=torch.device("cuda", local)
                          if world > 1 and os.environ.get("MDG_BENCH_BACKEND", "nccl") == "nccl"
                          else None)
    ms_step = ms_total / a.steps
    sps_job = world * a.steps / (ms_total / 1000.0)
    value = unit.ns_per_day(sps_job, DT_FS)
    sysm.check_status()

    # ---- per-stage timing (same flush protocol) ----------------------------
    # single stages accumulate into the force buffer and the update stage
    # moves atoms with it, so the state is saved here and restored after
    x_save, v_save = sysm.get_positions(), sysm.get_velocities()
    ens.update()
    stats = sysm.nonbonded_stats()
    stage_ms = {}
    for name, stage in (("pack", _lib.STAGE_PACK), ("nonbonded", _lib.STAGE_NONBONDED),
                        ("special", _lib.STAGE_SPECIAL), ("pme", _lib.STAGE_PME),
                        ("bonded", _lib.STAGE_BONDED), ("integrate", _lib.STAGE_INTEGRATE),
                        ("reorder", _lib.STAGE_REORDER)):
        reps = a.kernel_reps if name == "nonbonded" else max(20, a.kernel_reps // 4)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(reps)]
        for st, en in ev:
            flush.fill_(1)
            st.record(stream)
            sysm.launch_stage(stage, mask)
            en.record(stream)
        torch.cuda.synchronize()
        stage_ms[name] = float(np.mean([st.elapsed_time(en) for st, en in ev]))
    sysm.set_positions(x_save)
    sysm.set_velocities(v_save)
    ens.update()  # a valid force buffer again

    # pair-kernel roofline: algorithmic bytes = coordinates+charge (16 B) +
    # LJ parameters (8 B) read once and three int64 force words (24 B) written
    # once per atom, plus the cluster box and partner range (40 B per cluster)
    n_pad = 32 * ((n + 31) // 32)
    alg_bytes = 48 * n_pad + 40 * (n_pad // 32)
    t_nb = stage_ms["nonbonded"] * 1e-3
    peaks = {}
    if os.path.exists(PEAKS):
        with open(PEAKS) as fh:
            peaks = json.load(fh)
    hbm_peak = peaks.get("hbm_gbs")
    peak_src = "measured" if hbm_peak else "fallback"
    hbm_peak = hbm_peak or 6800.0
    traffic = None
    issue = None
    pairs_in = stats["pairs_in_cutoff"]
    if os.path.exists(PROFILE_INPUTS):
        with open(PROFILE_INPUTS) as fh:
            prof = json.load(fh)
        # one ncu capture of the 88k box; other sizes scale by the units processed
        traffic = prof["nonbonded_dram_bytes_per_launch"] * alg_bytes / prof["alg_bytes_per_launch"]
        inst = (prof["warp_instructions_per_launch"] * stats["pair_evaluations"]
                / prof["pair_evaluations_per_launch"])
        # the binding limit of this kernel: warp-instruction issue (4 schedulers
        # per SM, one instruction per clock each) at the sampled SM clock
        sm_mhz = None
        try:
            sm_mhz = float(clk.get("sm_mhz")) if clk and clk.get("sm_mhz") else None
        except (TypeError, ValueError):
            sm_mhz = None
        sm_mhz = sm_mhz or 2070.0
        n_sms = torch.cuda.get_device_properties(local).multi_processor_count
        peak_issue = n_sms * 4 * sm_mhz * 1e6
        issue = {"warp_instructions_per_launch": inst, "achieved_per_s": inst / t_nb,
                 "peak_per_s": peak_issue, "frac": inst / t_nb / peak_issue,
                 "source": "instructions per pair evaluation from the ncu capture in "
                           "profiles/roofline_inputs.json x this launch's evaluations; "
                           "peak = SMs x 4 schedulers x sampled SM clock"}
    achieved = alg_bytes / t_nb / 1e9
    flops = 60.0 * pairs_in / t_nb / 1e12
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": traffic, "kernel": "k_nonbonded",
                "peak_source": peak_src, "alg_bytes_per_launch": alg_bytes,
                "launch_ms": stage_ms["nonbonded"],
                "issue": issue,
                "fp32": {"achieved_tflops": flops, "nominal_peak_tflops": FP32_PEAK_TFLOPS_NOMINAL,
                         "frac": flops / FP32_PEAK_TFLOPS_NOMINAL,
                         "flops_per_pair": 60, "pairs_in_cutoff": pairs_in,
                         "pair_evaluations": stats["pair_evaluations"]}}

    # ---- end to end through the public API with pinned host buffers --------
    x_h = torch.empty((n, 3), dtype=torch.float64, pin_memory=True)
    v_h = torch.empty((n, 3), dtype=torch.float64, pin_memory=True)
    sysm.get_positions_ptr(x_h.data_ptr(), _lib.HOST)
    sysm.get_velocities_ptr(v_h.data_ptr(), _lib.HOST)
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    e_terms = np.zeros(_lib.NUM_TERMS)
    for k in range(a.e2e_steps):
        # one C-ABI call: host state in, one step, host state and energies out
        sysm.step_host_ptr(x_h.data_ptr(), v_h.data_ptr(), 1, mask, x_h.data_ptr(),
                           v_h.data_ptr(), e_terms)
    torch.cuda.synchronize()
    e2e_s = reduce_max(time.perf_counter() - t0, world,
                       device=torch.device("cuda", local)
                       if world > 1 and os.environ.get("MDG_BENCH_BACKEND", "nccl") == "nccl"
                       else None)
    e2e_value = unit.ns_per_day(world * a.e2e_steps / e2e_s, DT_FS)
    e2e = {"value": e2e_value, "unit": "ns/day", "h2d_bytes_per_step": 2 * n * 24,
           "d2h_bytes_per_step": 2 * n * 24 + 8 * (_lib.NUM_TERMS + 1) + 4,
           "api": "mdg_step_host: positions + velocities in from pinned host memory (the "
                  "previous call's outputs), one step, wrapped positions + velocities + "
                  "energies out; the incoming positions are compared on the device with the "
                  "state (one 4-byte read and a synchronisation), and equal ones keep their "
                  "forces and cluster order -- other positions trigger a re-sort and a fresh "
                  "force evaluation"}

    # what a multiple-time-step scheme could save at most: the same step
    # with the reciprocal-space term left out (PME runs beside the pair
    # kernel on the side stream, so only its share of the SMs shows)
    from mdpy_gb300 import _lib as L_

    no_pme = mask & ~L_.mask(L_.TERM_COUL_RECIP)
    sysm.integrate(5, no_pme, want_energy=False)
    reps = max(50, a.steps // 4)
    ms_no_pme = time_steps(sysm, no_pme, reps, stream, flush) / reps
    sysm.integrate(5, mask, want_energy=False)
    mts_bound = {"ms_per_step_without_pme": ms_no_pme, "ms_per_step": ms_step,
                 "pme_share_of_step": 1.0 - ms_no_pme / ms_step,
                 "max_saving_pme_every_4_steps": 0.75 * (1.0 - ms_no_pme / ms_step)}

    # the multiple-time-step forms: same shape and protocol, PME every k steps
    forms = []
    for k in [int(t) for t in str(a.mts).split(",") if t.strip() and int(t) > 1]:
        sysm.set_mts(k)
        sysm.integrate(2 * k + 3, mask, want_energy=False)
        reps = max(8 * k, (a.steps // (2 * k)) * k)
        ms_k = time_steps(sysm, mask, reps, stream, flush) / reps
        sysm.set_mts(1)
        sysm.integrate(5, mask, want_energy=False)
        forms.append({"form": "impulse multiple time steps: PME force every %d steps, weight %d"
                              % (k, k), "mts": k,
                      "ms_per_step": ms_k,
                      "ns_per_day": unit.ns_per_day(world * 1000.0 / ms_k, DT_FS),
                      "atom_steps_per_s": n * world * 1000.0 / ms_k, "timed_steps": reps})

    # the learned slow-force forms: trained here on frames of the plain
    # method (Langevin, 280-320 K), then timed with the same protocol; the
    # judge's statistics over the timed steps give the prediction's error
    learned_forms = {}
    for k in [int(t) for t in str(a.learned).split(",") if t.strip() and int(t) > 1]:
        from mdpy_gb300.learned import LearnedSlowForce

        lrn = LearnedSlowForce(outer_step=k, threshold=a.learned_threshold)
        t_tr = time.perf_counter()
        losses = lrn.train(sysm, iterations=a.learned_iters, lr=2e-3, seed=k, mask=mask)
        t_tr = time.perf_counter() - t_tr
        held = float(np.mean(losses[:5])) if losses else None
        sysm.integrator_config(_lib.INTEGRATOR_LANGEVIN, DT_FS, TEMPERATURE, FRICTION, 4242 + k)
        lrn.enable(sysm)
        sysm.integrate(4 * k + 3, mask, want_energy=False)
        sysm.learned_reset_stats()
        reps = max(8 * k, (a.steps // (2 * k)) * k)
        ms_k = time_steps(sysm, mask, reps, stream, flush) / reps
        judge = sysm.learned_stats()
        sysm.set_mts(1)
        sysm.integrate(5, mask, want_energy=False)
        f = {"form": "learned slow force: PME every %d steps, network prediction between, "
                     "impulse fallback above a judged error of %g" % (k, a.learned_threshold),
             "learned": k, "ms_per_step": ms_k,
             "ns_per_day": unit.ns_per_day(world * 1000.0 / ms_k, DT_FS),
             "atom_steps_per_s": n * world * 1000.0 / ms_k, "timed_steps": reps,
             "judge_over_timed_steps": judge,
             "training": {"iterations": a.learned_iters, "seconds": t_tr,
                          "loss_first5": held, "loss_last20": float(np.mean(losses[-20:])),
                          "loss": "sum |G(x1)-G(x0) - dF_slow|^2 / sum |dF_slow|^2 over frame "
                                  "pairs 1..k steps apart (1 = holding the slow force)"}}
        forms.append(f)
        learned_forms[id(f)] = lrn

    # every NVE run starts from the same state, and the state is put back
    # afterwards (a form whose run diverges must not spoil what follows)
    x_keep, v_keep = sysm.get_positions(), sysm.get_velocities()

    def restore():
        sysm.set_mts(1)
        sysm.set_positions(x_keep)
        sysm.set_velocities(v_keep)
        sysm.integrator_config(_lib.INTEGRATOR_LANGEVIN, DT_FS, TEMPERATURE, FRICTION, 4243)

    def drift_of(**kw):
        try:
            return nve_drift(sysm, mask, n, a.nve_ps, **kw)
        except Exception as e:  # noqa: BLE001 -- a diverging form is a result
            return {"diverged": "%s: %s" % (type(e).__name__, e),
                    "kT_per_ns_per_atom": None, "stderr_kT_per_ns_per_atom": None}
        finally:
            restore()

    nve = drift_of() if a.nve_ps > 0 else None
    if a.nve_ps > 0:
        for f in forms:
            f["nve_drift"] = drift_of(mts=f.get("mts", 1), seed=1,
                                      learned=learned_forms.get(id(f)))

    err = None
    cpu = None
    if rank == 0 and world == 1:
        if not a.no_error_check:
            err, nsub = force_error(s, ens, beta)
        if not a.no_cpu_baseline:
            r = cpu_reference_sample(s, a.cpu_seconds)
            cpu = {"value": r["ns_per_day"], "unit": "ns/day", "cores": r["cores"],
                   "kind": "port", "sample": r["sample"],
                   "atom_steps_per_s": r["atom_steps_per_s"]}

    if rank == 0:
        plain = {"form": "plain", "ns_per_day": value, "atom_steps_per_s": n * sps_job,
                 "ms_per_step": ms_step, "nve_drift": nve}
        # the chosen form: the fastest whose NVE drift (when measured) is not
        # shown to exceed 1e-3 kT/ns/atom (|drift| - 2 standard errors)
        def within(f):
            d = f.get("nve_drift")
            if d is None:
                return True
            if d.get("kT_per_ns_per_atom") is None:  # the run diverged
                return False
            return abs(d["kT_per_ns_per_atom"]) - 2 * d["stderr_kT_per_ns_per_atom"] <= 1e-3
        chosen = max([plain] + [f for f in forms if within(f)], key=lambda f: f["ns_per_day"])
        line = {
            "metric": METRIC, "value": value, "unit": "ns/day", "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": workload_name(a, n), "atoms": n, "replicas": world,
                       "l2": "flushed between timed steps (256 MB rewrite)",
                       "precision": "f32 pair/PME arithmetic, int64 fixed-point (2^-32) force "
                                    "accumulation, f64 x/v/energies",
                       "form": "plain", "launch_shape": shape},
            "atom_steps_per_s": n * sps_job,
            "force_rel_rms_err_vs_fp64": err,
            "nve_drift": nve,
            "mts_bound": mts_bound,
            "plain": plain, "chosen": chosen, "forms": forms,
            "roofline": roofline, "stages_ms": stage_ms, "nonbonded_stats": stats,
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
            "clocks": clk,
        }
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
