"""The mdpy-facing API on the device: the reference's own unit tests ported
(same set-ups, same known answers), plus ensemble/constraint consistency."""
import numpy as np
import pytest

from tests.helpers import rel_rms

pytestmark = pytest.mark.gpu


def _four(types, masses, charges):
    from mdpy_gb300 import Particle, Topology

    t = Topology()
    t.add_particles([Particle(particle_id=i, particle_type=ty, particle_name=ty, mass=m, charge=c)
                     for i, (ty, m, c) in enumerate(zip(types, masses, charges))])
    return t


def test_charmm_nonbonded_update_known_answer(lib, golden):
    """mdpy/test/test_charmm_nonbonded_constraint.py:93-126."""
    from mdpy_gb300 import constraint as C
    from mdpy_gb300.ensemble import Ensemble
    from mdpy_gb300.error import NonBoundedError

    rows = golden["nb4_params"].astype(np.float64)
    params = {"CA": list(rows[0, :2]), "NY": list(rows[1, :2]), "CPT": list(rows[2, :2])}
    t = _four(["CA", "NY", "CPT", "CA"], [12, 14, 1, 12], [0, 0, 0, 0])
    ens = Ensemble(t, np.eye(3) * 30)
    ens.state.cell_list.set_cutoff_radius(5)
    p = np.array([[0, 0, 0], [0, 10, 0], [0, 21, 0], [0, 11, 0]], dtype=np.float64)
    ens.state.set_positions(p)
    c = C.CharmmNonbondedConstraint(params)
    with pytest.raises(NonBoundedError):
        c._check_bound_state()
    c.set_cutoff_radius(9.1)
    ens.add_constraints(c)
    assert c._parent_ensemble.num_constraints == 1
    c.update()
    forces = c.forces
    assert forces.sum() == pytest.approx(0, abs=1e-8)
    eps = np.sqrt(rows[0, 0] * rows[2, 0])
    sigma = (rows[0, 1] + rows[2, 1]) / 2
    r = 9.0
    sr = sigma / r
    fval = -24 * eps / r * (2 * sr ** 12 - sr ** 6)
    uvec = (p[2] - p[0]) / np.linalg.norm(p[2] - p[0])
    force = fval * -uvec                                      # through the periodic image
    assert forces[0] == pytest.approx(force, abs=1e-8)
    eps = np.sqrt(rows[0, 0] * rows[1, 0])
    sigma = (rows[0, 1] + rows[1, 1]) / 2
    e_ref = 4 * eps * (sigma ** 12 - sigma ** 6)
    assert c.potential_energy == pytest.approx(e_ref, abs=1e-3)


def test_electrostatic_update_known_answer(lib):
    """mdpy/test/test_electrostatic_constraint.py:197-221 (k from mdpy's eps0)."""
    from mdpy_gb300 import constraint as C, unit
    from mdpy_gb300.ensemble import Ensemble

    t = _four(["C", "N", "CA", "C"], [12, 14, 1, 12], [1, 2, 0, 0])
    ens = Ensemble(t, np.eye(3) * 30)
    ens.state.set_positions(np.array([[0, 0, 0], [0, 10, 0], [0, 21, 0], [0, 11, 0]], float))
    c = C.ElectrostaticConstraint()
    ens.state.set_pbc_matrix(np.diag(np.ones(3) * 100))
    ens.add_constraints(c)
    c.update()
    f = c.forces
    assert f[2, 0] == 0 and f[3, 1] == 0
    fval = -unit.COULOMB_K * 1 * 2 / 10 ** 2
    assert f[0] == pytest.approx([0, fval, 0], rel=1e-6, abs=1e-12)
    assert f[1] == pytest.approx([0, -fval, 0], rel=1e-6, abs=1e-12)
    assert c.potential_energy == pytest.approx(unit.COULOMB_K * 2 / 10, rel=1e-6)


def test_ensemble_kinetic_energy_known_answer(lib):
    """mdpy/test/test_ensemble.py:88-101: KE = 13.5 mass*velocity^2 units; PE = 0."""
    t = _four(["C", "N", "H", "C"], [12, 14, 1, 12], [0, 0, 0, 0])
    t.add_bond([0, 1])
    t.add_bond([1, 2])
    t.add_bond([2, 3])
    from mdpy_gb300.ensemble import Ensemble

    ens = Ensemble(t, np.eye(3) * 30)
    ens.state.set_positions(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float))
    ens.state.set_velocities(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float))
    ens.update()
    assert ens.kinetic_energy == pytest.approx(13.5, rel=1e-12)
    assert ens.potential_energy == 0
    assert ens.total_energy == pytest.approx(13.5, rel=1e-12)


def test_ensemble_update_equals_constraint_sum(lib):
    from mdpy_gb300 import constraint as C, systems
    from mdpy_gb300.ensemble import Ensemble
    from mdpy_gb300.error import ConstraintConflictError

    w = systems.water_box(900, 30.0, seed=0)
    ens = Ensemble(w.topology, w.pbc_matrix)
    cons = [C.NonbondedConstraint(w.parameters["nonbonded"], 12.0),
            C.PMEConstraint(grid_size=32), C.CharmmBondConstraint(w.parameters["bond"]),
            C.CharmmAngleConstraint(w.parameters["angle"])]
    ens.add_constraints(*cons)
    with pytest.raises(ConstraintConflictError):
        ens.add_constraints(cons[0])
    ens.state.set_positions(w.positions)
    ens.update()
    total = ens.forces.copy()
    pe = ens.potential_energy
    per = [c.potential_energy for c in cons]
    fsum = sum(c.forces for c in cons)
    assert rel_rms(fsum, total) < 1e-6
    assert sum(per) == pytest.approx(pe, rel=1e-9)
    for c, e in zip(cons, per):
        c.update()
        assert c.potential_energy == pytest.approx(e, rel=1e-9, abs=1e-12)


def test_simulation_with_log_dumper(lib, tmp_path):
    from mdpy_gb300 import constraint as C, systems
    from mdpy_gb300.ensemble import Ensemble
    from mdpy_gb300.error import DumperPoorDefinedError
    from mdpy_gb300.integrator import LangevinIntegrator
    from mdpy_gb300.simulation import LogDumper, Simulation

    w = systems.water_box(500, 25.0, seed=6)
    ens = Ensemble(w.topology, w.pbc_matrix)
    ens.add_constraints(C.NonbondedConstraint(w.parameters["nonbonded"], 10.0),
                        C.PMEConstraint(grid_size=25, real_space_cutoff=10.0),
                        C.CharmmBondConstraint(w.parameters["bond"]),
                        C.CharmmAngleConstraint(w.parameters["angle"]))
    ens.state.set_positions(w.positions)
    ens.state.set_velocities_to_temperature(300, seed=2)
    sim = Simulation(ens, LangevinIntegrator(1.0, 300.0, 0.001, seed=5))
    with pytest.raises(DumperPoorDefinedError):
        sim.integrate(10)
    log = LogDumper(str(tmp_path / "log.txt"), dump_frequency=10)
    sim.add_dumpers(log)
    sim.dump_initial_state()
    sim.integrate(50)
    assert sim.cur_step == 50
    assert len(log.rows) == 6
    temps = [float(r[4]) for r in log.rows]
    # the lattice start relaxes: temperatures move, but stay finite and positive
    assert all(np.isfinite(t) and t > 0 for t in temps)
    assert float(log.rows[-1][5]) > 0   # ns/day column


def test_asynchronous_log_dumper_matches_synchronous(lib):
    """Energy snapshots (mdg_energy_snapshot): an asynchronous LogDumper
    writes the same rows as a synchronous one on the same trajectory (the
    speed column aside), with more dump steps than ring slots in flight, and
    leaves the ensemble's energies as the synchronous path does."""
    from mdpy_gb300 import _lib, constraint as C, systems
    from mdpy_gb300.ensemble import Ensemble
    from mdpy_gb300.integrator import LangevinIntegrator
    from mdpy_gb300.simulation import LogDumper, Simulation

    w = systems.water_box(500, 25.0, seed=6)
    runs = []
    for asynchronous in (False, True):
        ens = Ensemble(w.topology, w.pbc_matrix)
        ens.add_constraints(C.NonbondedConstraint(w.parameters["nonbonded"], 10.0),
                            C.PMEConstraint(grid_size=25, real_space_cutoff=10.0),
                            C.CharmmBondConstraint(w.parameters["bond"]),
                            C.CharmmAngleConstraint(w.parameters["angle"]))
        ens.state.set_positions(w.positions)
        ens.state.set_velocities_to_temperature(300, seed=2)
        sim = Simulation(ens, LangevinIntegrator(1.0, 300.0, 0.001, seed=5))
        logs = [LogDumper(None, dump_frequency=f, asynchronous=asynchronous) for f in (2, 3)]
        sim.add_dumpers(*logs)
        sim.integrate(4 * _lib.SNAPSHOT_SLOTS + 5)
        sim.integrate(7)
        runs.append(([[r[:5] for r in log.rows] for log in logs], ens.potential_energy,
                     ens.kinetic_energy))
    (rows_s, pe_s, ke_s), (rows_a, pe_a, ke_a) = runs
    assert rows_s == rows_a
    assert len(rows_s[0]) == (4 * _lib.SNAPSHOT_SLOTS + 12) // 2
    assert pe_a == pe_s and ke_a == ke_s


def test_energy_snapshot_slots_are_checked(lib):
    from mdpy_gb300 import systems
    from mdpy_gb300.error import NonBoundedError

    w = systems.water_box(50, 12.0, seed=1)
    s = lib.System(w.num_particles, w.box)
    with pytest.raises(ValueError):
        s.energy_snapshot(lib.SNAPSHOT_SLOTS)
    with pytest.raises(NonBoundedError):
        s.energy_snapshot_read(0)   # nothing taken yet


def test_charmm_forcefield_ensemble_runs_on_the_device(lib):
    """An mdpy-style script: CharmmForcefield -> create_ensemble -> update ->
    Simulation.integrate, with PME as the long-range solver; the forces equal
    those of the same constraints added by hand."""
    from mdpy_gb300 import constraint as C, systems
    from mdpy_gb300.ensemble import Ensemble
    from mdpy_gb300.forcefield import CharmmForcefield
    from mdpy_gb300.integrator import LangevinIntegrator
    from mdpy_gb300.simulation import LogDumper, Simulation

    w = systems.water_box(500, 25.0, seed=4)
    ff = CharmmForcefield(w.topology, w.pbc_matrix, cutoff_radius=10.0, long_range_solver="PME",
                          ewald_error=1e-5, pme_grid_spacing=1.0)
    ff.set_parameters(w.parameters)
    ens = ff.create_ensemble()
    ens.state.set_positions(w.positions)
    ens.update()
    ref = Ensemble(w.topology, w.pbc_matrix)
    ref.add_constraints(C.NonbondedConstraint(w.parameters["nonbonded"], 10.0, ewald_error=1e-5),
                        C.PMEConstraint(ewald_error=1e-5, real_space_cutoff=10.0,
                                        grid_spacing=1.0),
                        C.CharmmBondConstraint(w.parameters["bond"]),
                        C.CharmmAngleConstraint(w.parameters["angle"]))
    ref.state.set_positions(w.positions)
    ref.update()
    assert np.array_equal(ens.forces, ref.forces)
    assert ens.potential_energy == ref.potential_energy
    ens.state.set_velocities_to_temperature(300, seed=1)
    sim = Simulation(ens, LangevinIntegrator(1.0, 300.0, 0.001, seed=2))
    sim.add_dumpers(LogDumper(None, dump_frequency=10))
    sim.integrate(20)
    assert np.isfinite(ens.potential_energy) and ens.kinetic_energy > 0
