"""Host-side logic, the C ABI surface, and the oracle boundary (CPU only)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_c_abi_exports_every_declared_symbol(lib):
    """libmdg.so loads and exports every MDG_API function of include/mdg.h."""
    with open(os.path.join(ROOT, "include", "mdg.h")) as fh:
        names = re.findall(r"MDG_API\s+[\w\s\*]+?\b(mdg_\w+)\s*\(", fh.read())
    assert len(names) >= 30
    so = ctypes.CDLL(lib.LIB_PATH)
    for nm in names:
        assert hasattr(so, nm), nm
    lib.load()
    assert set(lib.SIGNATURES) <= set(names) | {"mdg_last_error"}


def test_version_and_error_without_gpu(lib):
    L = lib.load()
    major, minor = ctypes.c_int(), ctypes.c_int()
    assert L.mdg_version(ctypes.byref(major), ctypes.byref(minor)) == 0
    assert major.value >= 1
    # invalid arguments are rejected before any device work
    h = ctypes.c_void_p()
    box = (ctypes.c_double * 3)(10.0, 10.0, 10.0)
    assert L.mdg_system_create(0, -5, box, ctypes.byref(h)) == 1
    assert b"n_atoms" in L.mdg_last_error()
    bad = (ctypes.c_double * 3)(10.0, -1.0, 10.0)
    assert L.mdg_system_create(0, 5, bad, ctypes.byref(h)) == 4


def test_status_codes_map_to_mdpy_exceptions():
    from mdpy_gb300 import error as E

    assert isinstance(E.status_to_exception(4, "x"), E.PBCPoorDefinedError)
    assert isinstance(E.status_to_exception(5, "x"), E.CellListPoorDefinedError)
    assert isinstance(E.status_to_exception(6, "x"), E.ParticleLossError)
    assert isinstance(E.status_to_exception(7, "x"), E.FixedPointOverflowError)
    assert isinstance(E.status_to_exception(9, "x"), E.DeviceTimeoutError)


def test_product_code_never_imports_the_oracle():
    pkg = os.path.join(ROOT, "mdpy_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h")):
                with open(os.path.join(dirpath, f)) as fh:
                    src = fh.read()
                assert "import oracle" not in src and "from oracle" not in src, f
                assert "liborc" not in src, f


def test_unit_constants_match_reference_definitions():
    from mdpy_gb300 import unit

    # values mdpy computes through its float32 Quantity (mdpy/unit/__init__.py:54-58):
    # equal up to float32 rounding (one ulp ~ 1.2e-7 relative)
    assert unit.EPSILON0 == pytest.approx(0.5727653, rel=2.5e-7)
    assert unit.KCAL_PER_MOL == pytest.approx(0.00041840284, rel=2.5e-7)
    assert unit.KB * 300 == pytest.approx(2.4943e-4, rel=1e-3)


def test_topology_particle_api_matches_join():
    from mdpy_gb300 import Particle, Topology
    from mdpy_gb300.error import ModifyJoinedTopologyError, ParticleConflictError

    t = Topology()
    t.add_particles([Particle(particle_id=i, particle_type="C", mass=12, charge=0.1 * i)
                     for i in range(5)])
    t.add_bond([0, 1])
    t.add_bond([1, 2])
    t.add_angle([0, 1, 2])
    t.add_dihedral([0, 1, 2, 3])
    with pytest.raises(ParticleConflictError):
        t.add_bond([0, 0])
    t.join()
    assert t.bonded_particles[0].tolist() == [1, 2]
    assert t.bonded_particles[1].tolist()[:2] == [0, 2]
    assert t.scaling_particles[0, 0] == 3 and t.scaling_particles[3, 0] == 0
    assert t.masses.shape == (5, 1) and t.charges[4, 0] == pytest.approx(0.4)
    with pytest.raises(ModifyJoinedTopologyError):
        t.add_bond([3, 4])
    a = Topology.from_arrays(["C"] * 5, [12] * 5, [0.1 * i for i in range(5)],
                             bonds=[[0, 1], [1, 2]], angles=[[0, 1, 2]], dihedrals=[[0, 1, 2, 3]])
    assert np.array_equal(np.sort(a.bonded_particles, 1), np.sort(t.bonded_particles, 1))
    assert np.array_equal(a.scaling_particles[:, :1], t.scaling_particles[:, :1])


def test_synthetic_workloads():
    from mdpy_gb300 import systems, unit

    w = systems.water_box(900, 30.0, seed=0)
    assert w.num_particles == 2700
    assert np.all(np.abs(w.positions) <= 15.0 + 1e-9)
    o, h1 = w.positions[0], w.positions[1]
    d = h1 - o
    d -= 30.0 * np.round(d / 30.0)
    assert np.linalg.norm(d) == pytest.approx(0.9572, abs=1e-9)
    ke = 0.5 * np.sum(w.topology.masses * w.velocities ** 2)
    assert unit.kinetic_temperature(ke, w.num_particles) == pytest.approx(300, rel=0.05)
    assert abs(np.sum(w.topology.charges)) < 1e-9
    c = systems.chain_in_water(n_waters=460, box=24.0, n_beads=60, seed=5)
    assert c.topology.num_dihedrals == 57 and c.dihedral_parameters.shape == (57, 3)
    assert abs(np.sum(c.topology.charges)) < 1e-9
    batch = systems.water_box_batch(6, seed=1)
    sizes = [b.num_particles for b in batch]
    assert min(sizes) >= 1500 - 3 and max(sizes) <= 12000 + 3
    assert systems.fft_friendly(97) == 100 and systems.fft_friendly(96) == 96


def test_parameter_lookup_like_reference():
    from mdpy_gb300 import Topology, systems
    from mdpy_gb300.constraint import _per_atom_lj, _type_rows
    from mdpy_gb300.error import ParameterPoorDefinedError

    w = systems.water_box(3, 30.0)
    rows = _per_atom_lj(w.parameters["nonbonded"], w.topology)
    assert rows.shape == (9, 4) and rows[0, 0] > 0 and rows[1, 0] == 0
    t = Topology.from_arrays(["XX"], [1.0], [0.0])
    with pytest.raises(ParameterPoorDefinedError):
        _per_atom_lj(w.parameters["nonbonded"], t)
    idx, prm = _type_rows({"A-B-C-D": [[1.0, 2, 0.0], [0.5, 3, 3.14]]},
                          Topology.from_arrays(list("ABCD"), [1] * 4, [0] * 4),
                          [[0, 1, 2, 3]], 3, expand=True)
    assert len(idx) == 2 and prm[1][1] == 3


def test_ewald_beta_rule():
    from mdpy_gb300.constraint import ewald_beta_from_error

    b = ewald_beta_from_error(12.0, 1e-5)
    from math import erfc

    # exp(-(beta rc)^2) = 2 tol, so erfc(beta rc) ~ 2 tol / (beta rc sqrt(pi)) < tol
    assert 1e-6 < erfc(b * 12.0) < 1e-5
    assert b == pytest.approx(0.2744, abs=1e-3)


class _FakeBatchSystem:
    """Records what EnsembleBatch sends to the device batch."""

    def __init__(self, counts, boxes):
        self.n = int(np.sum(counts))
        self.n_systems = len(counts)
        self.counts, self.boxes = np.asarray(counts), np.asarray(boxes)
        self.calls = {}

    def __getattr__(self, name):
        if name.startswith("set_") or name.endswith("_config") or name.endswith("_batch"):
            return lambda *a: self.calls.__setitem__(name, a)
        raise AttributeError(name)


def test_ensemble_batch_concatenates_member_setup(monkeypatch):
    """Host side of a batch: member set-ups recorded, shifted to batch atom
    indices, per-member PME grids, shared settings checked."""
    from mdpy_gb300 import _lib, batch, constraint as C, systems

    monkeypatch.setattr(_lib.System, "batch", classmethod(lambda cls, c, b, d=0: _FakeBatchSystem(c, b)))
    ws = [systems.water_box(n, (3 * n / 0.1) ** (1 / 3), seed=k) for k, n in enumerate((300, 500))]
    members = []
    for w, grid in zip(ws, (24, 28)):
        ens = batch.member(w.topology, w.pbc_matrix)
        ens.add_constraints(C.NonbondedConstraint(w.parameters["nonbonded"], 9.0),
                            C.PMEConstraint(grid_size=grid, real_space_cutoff=9.0),
                            C.CharmmBondConstraint(w.parameters["bond"]))
        ens.state.set_positions(w.positions)
        members.append(ens)
    b = batch.EnsembleBatch(members)
    calls = b.system.calls
    assert b.system.n == 2400 and list(b.system.counts) == [900, 1500]
    idx, prm = calls["set_bonds"]
    assert idx.shape == (600 + 1000, 2) and idx[600:].min() == 900      # second member shifted
    excl = calls["set_exclusions"][0]
    assert excl.shape[0] == 2400 and excl[900:][excl[900:] >= 0].min() >= 900
    assert excl[:900].max() < 900
    grids, order, beta = calls["pme_config_batch"]
    assert grids.tolist() == [[24] * 3, [28] * 3] and order == 4
    assert np.allclose(calls["set_positions"][0][900:], ws[1].positions)
    # shared settings must agree
    other = batch.member(ws[1].topology, ws[1].pbc_matrix)
    other.add_constraints(C.NonbondedConstraint(ws[1].parameters["nonbonded"], 8.0),
                          C.PMEConstraint(grid_size=28, real_space_cutoff=8.0),
                          C.CharmmBondConstraint(ws[1].parameters["bond"]))
    with pytest.raises(ValueError, match="disagree"):
        batch.EnsembleBatch([members[0], other])


def test_pdb_dumper_writes_fixed_column_frames(tmp_path):
    """PDBDumper on a stand-in simulation: CRYST1 once, one MODEL per dump,
    coordinates in columns 31-54 as the PDB format fixes them."""
    from types import SimpleNamespace

    from mdpy_gb300 import systems
    from mdpy_gb300.dumper import PDBDumper
    from mdpy_gb300.error import DumperPoorDefinedError, FileFormatError

    w = systems.water_box(20, 12.0, seed=1)
    frames = [w.positions - 6.0, w.positions - 5.5]
    state = SimpleNamespace(pbc_matrix=np.diag(w.box), positions=None)
    sim = SimpleNamespace(ensemble=SimpleNamespace(topology=w.topology, state=state))
    with pytest.raises(FileFormatError):
        PDBDumper(str(tmp_path / "x.txt"), 1)
    with pytest.raises(DumperPoorDefinedError):
        PDBDumper(str(tmp_path / "x.pdb"), 0)
    d = PDBDumper(str(tmp_path / "t.pdb"), 10)
    for x in frames:
        state.positions = x
        d.dump(sim)
    d.close()
    lines = open(tmp_path / "t.pdb").read().splitlines()
    assert lines[0].startswith("CRYST1") and float(lines[0][6:15]) == pytest.approx(12.0)
    assert sum(ln.startswith("MODEL") for ln in lines) == 2
    atoms = [ln for ln in lines if ln.startswith("ATOM")]
    assert len(atoms) == 2 * 60
    xyz = np.array([[float(ln[30:38]), float(ln[38:46]), float(ln[46:54])] for ln in atoms])
    assert np.allclose(xyz, np.concatenate(frames), atol=5e-4)
    assert atoms[1][12:16].strip() == "HT" and int(atoms[59][6:11]) == 60


def test_charmm_forcefield_emits_device_constraints(monkeypatch):
    """CharmmForcefield.create_ensemble (mdpy/forcefield/charmm_forcefield.py:96-112):
    parameter check, and the constraint set for each long-range solver."""
    from mdpy_gb300 import constraint as C, forcefield, systems
    from mdpy_gb300.error import ParameterPoorDefinedError

    class FakeEnsemble:
        def __init__(self, topology, pbc, device=None):
            self.cons = []

        def add_constraints(self, *cons):
            self.cons.extend(cons)

    monkeypatch.setattr(forcefield, "Ensemble", FakeEnsemble)
    w = systems.water_box(30, 14.0, seed=0)
    ff = forcefield.CharmmForcefield(w.topology, w.pbc_matrix, cutoff_radius=6.0)
    with pytest.raises(ParameterPoorDefinedError):
        ff.check_parameters()
    bad = {k: dict(v) for k, v in w.parameters.items()}
    bad["nonbonded"].pop("HT")
    ff.set_parameters(bad)
    with pytest.raises(ParameterPoorDefinedError, match="HT"):
        ff.check_parameters()
    ff.set_parameters(w.parameters)
    kinds = [type(c) for c in ff.create_ensemble().cons]
    assert kinds == [C.NonbondedConstraint, C.PMEConstraint, C.CharmmBondConstraint,
                     C.CharmmAngleConstraint]
    ff2 = forcefield.CharmmForcefield(w.topology, w.pbc_matrix, cutoff_radius=6.0,
                                      long_range_solver=None)
    ff2.set_parameters(w.parameters)
    kinds = [type(c) for c in ff2.create_ensemble().cons]
    assert kinds[:2] == [C.ElectrostaticConstraint, C.CharmmNonbondedConstraint]
    with pytest.raises(ValueError):
        forcefield.CharmmForcefield(w.topology, w.pbc_matrix, long_range_solver="EWALD")


def test_learned_parameter_layout_matches_library(lib):
    """The Python offsets of the learned network's parameter vector and the
    library's count agree (no GPU needed for the count)."""
    from mdpy_gb300 import learned as Lr

    assert lib.System.learned_num_params() == Lr.N_PARAMS == 27025
    p = Lr.init_params(np.random.default_rng(0), scale=2.0)
    u = Lr.unpack(p)
    assert u["w1"].shape == (64, 128) and u["w3"].shape == (128, 16) and u["scale"] == 2.0
    assert np.all(u["sig"] == 1.0) and np.all(u["mu"] == 0.0)


def test_learned_reference_features_brute_force():
    """The FP64 feature reference (tests/learned_ref.py) against a direct
    double loop on a small periodic system: values, rotation invariance of
    the features and equivariance of the vector basis."""
    from tests import learned_ref as R

    rng = np.random.default_rng(1)
    box = np.array([14.0, 14.0, 14.0])
    pos = rng.uniform(0, 14.0, (60, 3))
    q = rng.uniform(-1, 1, 60)
    rf = 6.0
    feat, vec = R.features(pos, q, box, rf)
    f2 = np.zeros_like(feat)
    v2 = np.zeros_like(vec)
    for i in range(60):
        for j in range(60):
            if i == j:
                continue
            d = pos[i] - pos[j]
            d -= box * np.round(d / box)
            r = np.linalg.norm(d)
            if r >= rf:
                continue
            for b in range(32):
                w = R.bspline3(np.array([r / (rf / 33) - b]))[0]
                f2[i, b] += q[j] * w
                f2[i, 32 + b] += w
            for b in range(16):
                w = R.bspline3(np.array([r / (rf / 17) - b]))[0]
                v2[i, b] += q[i] * q[j] * w * d / rf ** 2
    assert np.allclose(feat, f2, atol=1e-12) and np.allclose(vec, v2, atol=1e-12)
    # basis functions vanish smoothly at rf
    assert R.bspline3(np.array([rf / (rf / 33) - 31]))[0] == 0.0
    # rotation of a cluster far from the box edges: invariant features,
    # rotated vectors
    big = np.array([100.0, 100.0, 100.0])
    c = rng.uniform(-4, 4, (30, 3))
    th = 0.7
    rot = np.array([[np.cos(th), -np.sin(th), 0], [np.sin(th), np.cos(th), 0], [0, 0, 1]])
    fa, va = R.features(c + 50.0, q[:30], big, rf)
    fb, vb = R.features(c @ rot.T + 50.0, q[:30], big, rf)
    assert np.allclose(fa, fb, atol=1e-10)
    assert np.allclose(np.einsum("ab,nkb->nka", rot, va), vb, atol=1e-10)


def test_learned_save_load_round_trip(tmp_path):
    """LearnedSlowForce keeps its parameters and settings through save/load
    (host logic only)."""
    from mdpy_gb300 import learned as Lr

    p = Lr.init_params(np.random.default_rng(3), scale=0.5)
    a = Lr.LearnedSlowForce(outer_step=3, threshold=0.02, rf=5.5, skin=1.2, list_capacity=200,
                            params=p)
    path = str(tmp_path / "slow_force.npz")
    a.save(path)
    b = Lr.LearnedSlowForce.load(path)
    assert np.array_equal(a.params, b.params)
    assert (b.outer_step, b.threshold, b.rf, b.skin, b.list_capacity) == (3, 0.02, 5.5, 1.2, 200)
    with pytest.raises(ValueError):
        Lr.LearnedSlowForce(outer_step=1)


class _FakeLearnedSystem:
    """Records the calls LearnedSlowForce makes (host logic only)."""

    def __init__(self, n=10):
        self.n = n
        self.calls = []
        self.rng = np.random.default_rng(0)
        self.params = None

    def __getattr__(self, name):
        def rec(*args, **kw):
            self.calls.append((name, args))
        return rec

    def learned_set_params(self, p):
        self.calls.append(("learned_set_params", ()))
        self.params = np.array(p, dtype=np.float32)

    def learned_params(self):
        return self.params.copy()

    def learned_frame_data(self, slot):
        n = self.n
        return (self.rng.normal(size=(n, 64)).astype(np.float32),
                self.rng.normal(size=(n, 16, 3)).astype(np.float32),
                self.rng.normal(size=(n, 3)).astype(np.float32),
                np.zeros((n, 3), np.float32))

    def learned_train_step(self, lr, t):
        self.calls.append(("learned_train_step", (lr, t)))
        return 1.0 / t


def test_learned_training_loop_host_logic():
    """LearnedSlowForce.train: frame pairs 1..k steps apart after
    `decorrelate` steps, one Adam step each with a cosine-decayed rate, the
    Langevin temperature redrawn in the given range, the plain form on."""
    from mdpy_gb300 import _lib, learned as Lr

    s = _FakeLearnedSystem()
    lrn = Lr.LearnedSlowForce(outer_step=3)
    losses = lrn.train(s, iterations=7, lr=1e-2, temperatures=(280.0, 320.0), decorrelate=5,
                       redraw_every=3, mask=_lib.MASK_ALL, seed=1)
    assert len(losses) == 7 and lrn.params is not None
    names = [c[0] for c in s.calls]
    assert ("set_mts_learned", (0, 1.0)) in s.calls          # plain method makes the frames
    # normalise: G = 0 parameters, one frame pair k steps apart, a zero-rate step
    steps = [c for c in s.calls if c[0] == "learned_train_step"]
    assert steps[0][1] == (1e-30, 1)
    train = steps[1:]
    assert [t for _, (_, t) in train] == list(range(1, 8))
    rates = [r for _, (r, _) in train]
    assert rates[0] == pytest.approx(1e-2) and all(a > b for a, b in zip(rates, rates[1:]))
    assert rates[-1] > 1e-3
    # per iteration: integrate(decorrelate), frame 0, integrate(gap), frame 1
    ints = [c[1][0] for c in s.calls if c[0] == "integrate"]
    gaps = ints[1:][1::2]     # after normalise's pair: decorrelate, gap, decorrelate, gap ...
    assert ints[0] == 3 and gaps == [1, 2, 3, 1, 2, 3, 1]
    assert all(d == 5 for d in ints[1:][0::2])
    temps = [c[1][2] for c in s.calls if c[0] == "integrator_config" and c[1][0] == _lib.INTEGRATOR_LANGEVIN]
    assert len(temps) >= 1 + 3 and all(280.0 <= t <= 320.0 for t in temps)
    assert names.count("learned_frame") == 2 * 8


def test_reference_binding_imports_the_installed_reference():
    """The reference-side binding's host part: the installed reference
    (baseline/_ref) imports through the stubs, the binding subclasses its
    Constraint, and its Topology of a water box carries the exclusions the
    libmdg constraint hands to the device."""
    from tests import ref_binding as RB

    if not RB.reference_available():
        pytest.skip("the reference is not installed in baseline/_ref")
    from mdpy_gb300 import systems

    w = systems.water_box(10, 10.0, seed=0)
    t = RB.reference_topology(w)
    t.join()   # what the reference's Ensemble does on construction
    assert t.num_particles == 30
    cls = RB.binding_class()
    from mdpy.constraint import Constraint

    assert issubclass(cls, Constraint)
    # 1-2 and 1-3 partners of each atom of a water: the other two atoms
    for i in range(30):
        partners = sorted(int(p) for p in t.bonded_particles[i] if p >= 0)
        m = i // 3
        assert partners == [j for j in range(3 * m, 3 * m + 3) if j != i]


def test_bench_drift_statistics_and_gates():
    """The NVE-drift estimator of bench.py on synthetic energy series: a
    known slope under white noise is recovered within its standard error,
    correlated (random-walk) noise widens the error instead of hiding in it,
    and the gate requires |drift| + 2 sigma below the bar."""
    import bench
    from mdpy_gb300 import unit

    rng = np.random.default_rng(4)
    n_atoms = 1000
    kt = unit.KB * bench.TEMPERATURE
    t = np.arange(1, 5001) * 20.0                  # fs, a sample every 20 steps
    true = 4e-4                                    # kT / ns / atom
    slope = true * n_atoms * kt / 1e6              # energy per fs
    white = slope * t + rng.normal(0.0, 5e-4 * n_atoms * kt, t.size)
    d = bench.drift_statistics(t, white, n_atoms)
    assert abs(d["kT_per_ns_per_atom"] - true) < 4 * d["stderr_kT_per_ns_per_atom"]
    assert 0.5 <= d["autocorrelation_samples"] < 2.0
    walk = slope * t + np.cumsum(rng.normal(0.0, 5e-5 * n_atoms * kt, t.size))
    dw = bench.drift_statistics(t, walk, n_atoms)
    assert dw["autocorrelation_samples"] > 20
    assert dw["stderr_kT_per_ns_per_atom"] > 3 * d["stderr_kT_per_ns_per_atom"]
    assert bench.drift_passes({"kT_per_ns_per_atom": 4e-4, "stderr_kT_per_ns_per_atom": 2e-4})
    assert not bench.drift_passes({"kT_per_ns_per_atom": 4e-4, "stderr_kT_per_ns_per_atom": 4e-4})
    assert not bench.drift_passes({"kT_per_ns_per_atom": -1.2e-3, "stderr_kT_per_ns_per_atom": 0.0})
    assert not bench.drift_passes({"kT_per_ns_per_atom": None, "stderr_kT_per_ns_per_atom": None})
    assert not bench.drift_passes(None)
    assert bench.integrated_autocorrelation_time(np.zeros(10)) == 0.5


def test_bench_reference_arm_runs_the_steps_it_reports():
    """bench.py --impl reference on a small box: exactly --warmup + --steps
    sampled steps, ms_per_step the measured sampled step, the whole-step time
    extrapolated from it and said so."""
    import json
    import subprocess
    import sys

    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, os.path.join(repo, "bench.py"), "--impl", "reference",
                          "--steps", "3", "--warmup", "1", "--waters", "300", "--box", "21",
                          "--beads", "0", "--reference-seconds", "2"],
                         capture_output=True, text=True, timeout=300, cwd=repo)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads([l for l in out.stdout.splitlines() if l.startswith("{")][-1])
    assert line["impl"] == "reference" and line["steps"] == 3 and line["warmup"] == 1
    assert line["ms_per_full_step_extrapolated"] >= line["ms_per_step"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and "extrapolated" in line["cpu_baseline"]["sample"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["value"] > 0


def test_energy_erfc_fit_accuracy():
    """The real-space energy's erfc (erfc_q in the pair kernel header): the
    constants are read from the source, the polynomial is evaluated in
    float32 as the kernel does (t = 1/(1 + p x) rounded to float32), and the
    relative error against scipy's erfc stays below 5e-7 over x in [0, 6]
    (below 1e-7 on average); in float64 the fit itself is within 1e-7."""
    import re

    from scipy.special import erfc

    src = open(os.path.join(ROOT, "mdpy_gb300", "csrc", "mdg_nonbonded_kernel.cuh")).read()
    body = src[src.index("float erfc_q(float t)"):]
    body = body[:body.index("}")]
    tc = float(re.search(r"kEqC = ([-0-9.e]+)f", src).group(1))
    p = float(re.search(r"kAsP = ([-0-9.e]+)f", src).group(1))
    lits = [float(v) for v in re.findall(r"(-?[0-9]+\.[0-9]+(?:e-?[0-9]+)?)f", body)]
    # Horner order in the source: c7, c6 (first fmaf), then c5 .. c0
    coef = [lits[0], lits[1]] + lits[2:]
    assert len(coef) == 8
    x = np.linspace(0.0, 6.0, 200001)
    exact = erfc(x)
    # float64
    t = 1.0 / (1.0 + p * x)
    q = np.full_like(t, coef[0])
    for c in coef[1:]:
        q = q * (t - tc) + c
    assert np.max(np.abs(t * q * np.exp(-x * x) - exact) / exact) < 1e-7
    # float32, as the kernel evaluates it (e^{-x^2} taken exactly here)
    f = np.float32
    x32 = x.astype(f)
    t32 = (f(1) / (f(1) + f(p) * x32)).astype(f)
    u = (t32 - f(tc)).astype(f)
    q32 = np.full_like(u, f(coef[0]))
    for c in coef[1:]:
        q32 = (q32 * u + f(c)).astype(f)
    ex = erfc(x32.astype(np.float64))
    rel = np.abs(t32.astype(np.float64) * q32 * np.exp(-x32.astype(np.float64) ** 2) - ex) / ex
    assert rel.max() < 5e-7 and rel.mean() < 1e-7, (rel.max(), rel.mean())


class _FakeSnapshotSystem:
    """Stands in for _lib.System in the asynchronous dump loop: integrate
    advances a step counter, a snapshot records the energies of that step in
    its slot, and a non-waiting read reports the copy as pending on its first
    poll (as a copy behind queued steps would be)."""

    def __init__(self):
        from mdpy_gb300 import _lib

        self.step = 0
        self.slots = {}
        self.polls = {}
        self.events = []
        self.nterms = _lib.NUM_TERMS

    def integrate(self, n, mask, want_energy=True):
        self.step += int(n)
        self.events.append(("integrate", self.step))

    def energy_snapshot(self, slot):
        assert slot not in self.slots, "slot %d reused before its read" % slot
        self.slots[slot] = self.step
        self.polls[slot] = 0
        self.events.append(("snapshot", slot, self.step))

    def energy_snapshot_read(self, slot, wait=True):
        if not wait and self.polls[slot] == 0:
            self.polls[slot] += 1
            return None
        step = self.slots.pop(slot)
        e = np.zeros(self.nterms)
        e[0] = float(step)            # potential energy = the step number
        self.events.append(("read", slot, step))
        return e, 2.0 * step          # kinetic energy = twice the step


def test_asynchronous_dump_loop_host_logic():
    """Simulation.integrate with asynchronous LogDumpers: one snapshot per
    dump step after that step's integrate, rows in step order with the
    values of their own step, never more snapshots in flight than ring slots
    (a slot is read before it is reused), everything read by the end, and
    the ensemble read back once at the end."""
    from mdpy_gb300 import _lib, unit
    from mdpy_gb300.simulation import LogDumper, Simulation

    class _Ens:
        def __init__(self):
            self.system = _FakeSnapshotSystem()
            self.term_mask = 1
            self.after = 0
            self.topology = type("T", (), {"num_particles": 10})()

        def _after_integrate(self):
            self.after += 1

    class _Integ:
        time_step = 1.0

        def integrate(self, ens, n, read_back=True):
            assert read_back is False
            ens.system.integrate(n, ens.term_mask)

    ens = _Ens()
    sim = Simulation(ens, _Integ())
    logs = [LogDumper(None, dump_frequency=f, asynchronous=True) for f in (2, 5)]
    sim.add_dumpers(*logs)
    n = 3 * _lib.SNAPSHOT_SLOTS * 2 + 7
    sim.integrate(n)
    assert sim.cur_step == n and ens.after == 1 and not ens.system.slots
    for log, f in zip(logs, (2, 5)):
        steps = [int(r[0]) for r in log.rows]
        assert steps == list(range(f, n + 1, f))
        kj = 1.0 / unit.KJ_PER_MOL
        for r in log.rows:
            st = int(r[0])
            assert float(r[1]) == pytest.approx(st * kj, abs=1e-3)
            assert float(r[2]) == pytest.approx(2 * st * kj, abs=1e-3)
    ev = ens.system.events
    in_flight, peak = 0, 0
    for e in ev:
        if e[0] == "snapshot":
            in_flight += 1
            peak = max(peak, in_flight)
        elif e[0] == "read":
            in_flight -= 1
    assert peak <= _lib.SNAPSHOT_SLOTS
    snaps = [e[2] for e in ev if e[0] == "snapshot"]
    assert snaps == sorted(set(range(2, n + 1, 2)) | set(range(5, n + 1, 5)))
