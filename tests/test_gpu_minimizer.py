"""Energy minimisation on the device: one steepest-descent move equals the
reference's update x + alpha F/|F| (mdpy/minimizer/steepest_descent_minimizer.py:
39-42) applied to the same forces, and minimisation lowers the energy of a
strained water box until the relative change drops below the tolerance."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ensemble(seed=3, jitter=0.6):
    from mdpy_gb300 import constraint as C, systems
    from mdpy_gb300.ensemble import Ensemble

    w = systems.water_box(500, 25.0, seed=seed, jitter=jitter)
    ens = Ensemble(w.topology, w.pbc_matrix)
    ens.add_constraints(C.NonbondedConstraint(w.parameters["nonbonded"], 10.0),
                        C.PMEConstraint(grid_size=25, real_space_cutoff=10.0),
                        C.CharmmBondConstraint(w.parameters["bond"]),
                        C.CharmmAngleConstraint(w.parameters["angle"]))
    ens.state.set_positions(w.positions)
    return ens, w


def test_steepest_descent_move_matches_reference_update(lib):
    ens, w = _ensemble()
    ens.update()
    f = ens.forces.copy()
    x0 = ens.system.get_positions()
    ens.system.minimize_step(0.01)
    x1 = ens.system.get_positions()
    expect = x0 + 0.01 * f / np.linalg.norm(f, axis=1).reshape(-1, 1)
    d = x1 - expect
    d -= w.box * np.round(d / w.box)
    assert np.max(np.abs(d)) < 1e-12
    with pytest.raises(Exception, match="no force evaluation"):
        ens.system.minimize_step(0.01)


def test_steepest_descent_lowers_energy(lib, capsys):
    from mdpy_gb300.minimizer import SteepestDescentMinimizer

    ens, _ = _ensemble(jitter=0.8)
    ens.update()
    e0 = ens.potential_energy
    m = SteepestDescentMinimizer(0.01)
    m.minimize(ens, energy_tolerance=1e-4, max_iterations=300)
    assert ens.potential_energy < e0
    assert m.num_iterations <= 300
    out = capsys.readouterr().out
    assert "Initial potential energy" in out and "kj/mol" in out


def test_simulation_minimize_default(lib):
    from mdpy_gb300.integrator import VerletIntegrator
    from mdpy_gb300.simulation import LogDumper, Simulation

    ens, _ = _ensemble(jitter=0.8)
    sim = Simulation(ens, VerletIntegrator(1.0))
    sim.add_dumpers(LogDumper(None, dump_frequency=1))
    ens.update()
    e0 = ens.potential_energy
    sim.minimize(1e-3, 50)
    assert ens.potential_energy < e0
