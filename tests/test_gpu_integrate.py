"""Integrators: one step against the FP64 textbook oracle, the Philox noise
against the oracle's restatement, the reference's one-step position test,
bit-reproducibility, and energy conservation."""
import numpy as np
import pytest

from tests.helpers import rel_rms

pytestmark = pytest.mark.gpu


def _ensemble(w, rc=12.0, K=32, switch=None, device=0):
    from mdpy_gb300 import constraint as C
    from mdpy_gb300.ensemble import Ensemble

    ens = Ensemble(w.topology, w.pbc_matrix, device=device)
    ens.add_constraints(
        C.NonbondedConstraint(w.parameters["nonbonded"], cutoff_radius=rc, switch_radius=switch),
        C.PMEConstraint(grid_size=K, order=4, real_space_cutoff=rc),
        C.CharmmBondConstraint(w.parameters["bond"]),
        C.CharmmAngleConstraint(w.parameters["angle"]))
    ens.state.set_positions(w.positions)
    ens.state.set_velocities(w.velocities)
    return ens


def test_verlet_one_step_vs_oracle(lib, orc):
    from mdpy_gb300 import systems
    from mdpy_gb300.integrator import VerletIntegrator

    w = systems.water_box(900, 30.0, seed=0)
    ens = _ensemble(w)
    ens.update()
    f0 = ens.forces.copy()
    x0 = w.positions.copy()
    v0 = w.velocities.copy()
    VerletIntegrator(1.0).integrate(ens, 1)
    x1 = ens.state.positions
    v1 = ens.state.velocities
    ens.update()
    f1 = ens.forces
    m = w.topology.masses.reshape(-1, 1)
    x1o = x0 + 1.0 * v0 + 0.5 * f0 / m
    x1o = orc.wrap_positions(x1o, w.box)
    v1o = v0 + 0.5 * (f0 + f1) / m
    d = x1 - x1o
    d -= w.box * np.round(d / w.box)
    assert np.abs(d).max() < 1e-10
    assert np.abs(v1 - v1o).max() < 1e-12 + 1e-9 * np.abs(v1o).max()


def test_langevin_noise_matches_oracle(lib, orc):
    s = lib.System(1000, 30.0)
    s.integrator_config(lib.INTEGRATOR_LANGEVIN, 1.0, 300.0, 0.001, seed=12345)
    for step in (0, 1, 77, 2 ** 33 + 5):
        g = s.langevin_noise(step)
        o = orc.langevin_noise(1000, 12345, step)
        assert np.abs(g - o).max() < 2e-5
    g = s.langevin_noise(3).astype(np.float64).reshape(-1)
    assert abs(g.mean()) < 0.05 and abs(g.std() - 1.0) < 0.05


def test_langevin_one_step_vs_oracle(lib, orc):
    from mdpy_gb300 import systems
    from mdpy_gb300.integrator import LangevinIntegrator

    w = systems.water_box(900, 30.0, seed=0)
    ens = _ensemble(w)
    ens.update()
    f0 = ens.forces.copy()
    integ = LangevinIntegrator(1.0, 300.0, 0.001, seed=99)
    step0 = ens.system.step
    integ.integrate(ens, 1)
    x1 = ens.state.positions
    v1 = ens.state.velocities
    ens.update()
    f1 = ens.forces
    xi = ens.system.langevin_noise(step0).astype(np.float64)
    x1o, v1o, _ = orc.langevin_gjf_step(w.positions, w.velocities, f0, w.topology.masses, 1.0,
                                        300.0, 0.001, xi, lambda x: f1)
    d = x1 - orc.wrap_positions(x1o, w.box)
    d -= w.box * np.round(d / w.box)
    assert np.abs(d).max() < 1e-9
    assert np.abs(v1 - v1o).max() < 1e-9 * max(1.0, np.abs(v1o).max())


def test_reference_one_step_position_bound(lib, golden):
    """mdpy/test/test_verlet_integrator.py:33-47 checks one step moves an atom
    by < 0.01 A from the reference position; the same set-up (27 waters,
    25 A) through the GPU Verlet lands within 0.01 A of the reference's
    one-step positions."""
    from mdpy_gb300 import systems
    from mdpy_gb300 import constraint as C
    from mdpy_gb300.ensemble import Ensemble
    from mdpy_gb300.integrator import VerletIntegrator

    w = systems.water_box(27, 25.0, seed=3)
    ens = Ensemble(w.topology, w.pbc_matrix)
    ens.add_constraints(C.CharmmNonbondedConstraint(w.parameters["nonbonded"], 12),
                        C.ElectrostaticConstraint(), C.CharmmBondConstraint(w.parameters["bond"]),
                        C.CharmmAngleConstraint(w.parameters["angle"]))
    ens.state.set_positions(golden["v81_positions0"].astype(np.float64))
    ens.state.set_velocities(golden["v81_velocities0"].astype(np.float64))
    VerletIntegrator(1).integrate(ens, 1)
    d = ens.state.positions - golden["v81_positions1"].astype(np.float64)
    d -= 25.0 * np.round(d / 25.0)
    assert np.abs(d).max() < 0.01


def test_trajectory_bit_reproducible(lib):
    from mdpy_gb300 import systems
    from mdpy_gb300.integrator import LangevinIntegrator

    w = systems.water_box(900, 30.0, seed=1)
    runs = []
    for _ in range(2):
        ens = _ensemble(w)
        ens.system.set_reorder_interval(10)
        LangevinIntegrator(1.0, 300.0, 0.001, seed=7).integrate(ens, 45)
        runs.append((ens.state.positions, ens.state.velocities, ens.potential_energy))
    assert np.array_equal(runs[0][0], runs[1][0])
    assert np.array_equal(runs[0][1], runs[1][1])
    assert runs[0][2] == runs[1][2]


def test_graph_chunks_equal_eager_steps(lib):
    """The CUDA-graph chunk path and single eager steps give identical states."""
    from mdpy_gb300 import systems
    from mdpy_gb300.integrator import LangevinIntegrator

    w = systems.water_box(600, 27.0, seed=8)
    a = _ensemble(w, rc=11.0, K=28)
    b = _ensemble(w, rc=11.0, K=28)
    a.system.set_reorder_interval(5)
    b.system.set_reorder_interval(5)
    ia, ib = LangevinIntegrator(1.0, 300.0, 0.001, seed=3), LangevinIntegrator(1.0, 300.0, 0.001, seed=3)
    ia.integrate(a, 20)                 # graph chunks
    for _ in range(20):
        ib.integrate(b, 1)              # eager steps
    assert np.array_equal(a.state.positions, b.state.positions)
    assert np.array_equal(a.state.velocities, b.state.velocities)


def test_nve_energy_conservation(lib):
    from mdpy_gb300 import systems
    from mdpy_gb300.integrator import LangevinIntegrator, VerletIntegrator

    w = systems.water_box(900, 30.0, seed=0)
    ens = _ensemble(w, switch=10.0)
    LangevinIntegrator(0.5, 300.0, 0.01, seed=1).integrate(ens, 400)   # relax the lattice
    vv = VerletIntegrator(0.5)
    energies = []
    for _ in range(20):
        vv.integrate(ens, 25)
        energies.append(ens.total_energy)
    e = np.array(energies)
    ke = ens.kinetic_energy
    assert np.all(np.isfinite(e))
    # drift over 250 fs well below the kinetic energy scale
    assert abs(e[-1] - e[0]) < 2e-3 * ke


def test_step_host_equals_separate_calls(lib):
    """mdg_step_host (copies in, n steps, copies out, one synchronisation)
    gives bit for bit what the separate set / integrate / get calls give."""
    from mdpy_gb300 import systems
    from tests.helpers import make_system, water_lj_rows

    w = systems.water_box(600, 26.0, seed=12)
    t = w.topology
    mask = lib.mask(lib.TERM_LJ, lib.TERM_COUL_REAL, lib.TERM_COUL_RECIP)

    def build():
        s = make_system(lib, w.num_particles, w.box, masses=t.masses.reshape(-1),
                        charges=t.charges.reshape(-1), lj=water_lj_rows(w),
                        bonded=t.bonded_particles, cutoff=10.0, coulomb=lib.COUL_EWALD,
                        beta=0.3, positions=w.positions)
        s.pme_config(27, 4, 0.3)
        s.integrator_config(lib.INTEGRATOR_LANGEVIN, 1.0, 300.0, 0.001, 5)
        return s

    a, b = build(), build()
    x = np.ascontiguousarray(w.positions + 0.01)
    v = np.ascontiguousarray(w.velocities)
    a.set_positions(x)
    a.set_velocities(v)
    a.integrate(7, mask, want_energy=True)
    xa, va = a.get_positions(), a.get_velocities()
    ea, kea = a.get_energies()
    xb, vb = np.empty_like(x), np.empty_like(v)
    eb = np.zeros(lib.NUM_TERMS)
    keb = b.step_host_ptr(x.ctypes.data, v.ctypes.data, 7, mask, xb.ctypes.data, vb.ctypes.data,
                          eb)
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)
    assert np.array_equal(ea, eb) and kea == keb
    # outputs only: the state carries on from where it was
    keb2 = b.step_host_ptr(0, 0, 3, mask, xb.ctypes.data, 0, eb)
    a.integrate(3, mask, want_energy=True)
    assert np.array_equal(a.get_positions(), xb) and a.get_energies()[1] == keb2


def test_step_host_continuation_keeps_forces(lib):
    """Feeding mdg_step_host the positions and velocities it returned
    continues the trajectory bit for bit as mdg_integrate does (the forces of
    those positions are kept, no re-sort); changed positions start afresh,
    as mdg_set_positions does."""
    from mdpy_gb300 import systems

    w = systems.water_box(600, 26.0, seed=13)
    ea_, eb_ = _ensemble(w, rc=10.0, K=27), _ensemble(w, rc=10.0, K=27)
    a, b = ea_.system, eb_.system
    mask = ea_.term_mask
    for s in (a, b):
        s.integrator_config(lib.INTEGRATOR_LANGEVIN, 1.0, 300.0, 0.001, 5)
    x = np.ascontiguousarray(w.positions)
    v = np.ascontiguousarray(w.velocities)
    a.set_positions(x)
    a.set_velocities(v)
    xb, vb = x.copy(), v.copy()
    eb = np.zeros(lib.NUM_TERMS)
    for step in range(25):   # crosses the re-sort after 20 steps
        a.integrate(1, mask, want_energy=True)
        keb = b.step_host_ptr(xb.ctypes.data, vb.ctypes.data, 1, mask, xb.ctypes.data,
                              vb.ctypes.data, eb)
        assert np.array_equal(a.get_positions(), xb), step
        assert np.array_equal(a.get_velocities(), vb), step
        ea, kea = a.get_energies()
        assert np.array_equal(ea, eb) and kea == keb, step
    # moved positions: the forces are recomputed, as after mdg_set_positions
    xm = np.ascontiguousarray(xb + 1e-3)
    vm = vb.copy()
    a.set_positions(xm)
    a.set_velocities(vm)
    a.integrate(1, mask, want_energy=True)
    a.check_status()
    b.step_host_ptr(xm.ctypes.data, vm.ctypes.data, 1, mask, xb.ctypes.data, vb.ctypes.data, eb)
    assert np.array_equal(a.get_positions(), xb) and np.array_equal(a.get_velocities(), vb)
    # moved positions without velocities: the speculative step on the old
    # state is undone (velocities and step counter put back) and redone
    xm2 = np.ascontiguousarray(xb - 2e-3)
    a.set_positions(xm2)
    a.integrate(1, mask, want_energy=True)
    keb = b.step_host_ptr(xm2.ctypes.data, 0, 1, mask, xb.ctypes.data, vb.ctypes.data, eb)
    ea, kea = a.get_energies()
    assert np.array_equal(a.get_positions(), xb) and np.array_equal(a.get_velocities(), vb)
    assert np.array_equal(ea, eb) and kea == keb
    assert a.step == b.step
    # and the trajectories carry on together (same Philox step numbers)
    for step in range(3):
        a.integrate(1, mask, want_energy=True)
        b.step_host_ptr(xb.ctypes.data, vb.ctypes.data, 1, mask, xb.ctypes.data,
                        vb.ctypes.data, eb)
        assert np.array_equal(a.get_positions(), xb), step
        assert np.array_equal(a.get_velocities(), vb), step


def test_mts_impulse_equations(lib):
    """Multiple time steps, k = 2: the steps follow the impulse (Verlet-I)
    equations restated in numpy from the library's own term forces -- the
    reciprocal force enters with weight 2 at the end of every second step and
    is absent in between."""
    from mdpy_gb300 import systems

    w = systems.water_box(900, 30.0, seed=0)
    ens = _ensemble(w)
    probe = _ensemble(w)   # term forces at given positions
    s, mask = ens.system, ens.term_mask
    recip = lib.mask(lib.TERM_COUL_RECIP)
    fast = mask & ~recip
    m = w.topology.masses.reshape(-1, 1)

    def forces(x, terms):
        probe.system.set_positions(x)
        probe.system.compute_forces(terms)
        return probe.system.get_forces()

    x, v = w.positions.copy(), w.velocities.copy()
    s.set_positions(x)
    s.set_velocities(v)
    s.integrator_config(lib.INTEGRATOR_VERLET, 1.0)
    s.set_mts(2)
    f = forces(x, fast) + 2.0 * forces(x, recip)      # the outer step starts with the impulse
    for step in range(4):
        s.integrate(1, mask, want_energy=False)
        x = x + v + 0.5 * f / m
        vh = v + 0.5 * f / m
        f = forces(x, fast) + (2.0 * forces(x, recip) if step % 2 == 1 else 0.0)
        v = vh + 0.5 * f / m
        d = s.get_positions() - x
        d -= w.box * np.round(d / w.box)
        # (a wrong weight would be off by ~1e-3 A; float rounding of the
        # probe's forces leaves ~1e-8)
        assert np.abs(d).max() < 1e-7, step
        # (the probe's forces round differently from the running system's:
        # other cluster layouts, FP32 partial sums)
        assert np.abs(s.get_velocities() - v).max() < 2e-6 * np.abs(v).max(), step
    # k = 1 is the ordinary integrator, bit for bit
    a, b = _ensemble(w), _ensemble(w)
    for e in (a, b):
        e.system.integrator_config(lib.INTEGRATOR_VERLET, 1.0)
    a.system.set_mts(1)
    a.system.integrate(10, mask, want_energy=True)
    b.system.integrate(10, mask, want_energy=True)
    assert np.array_equal(a.system.get_positions(), b.system.get_positions())
    assert np.array_equal(a.system.get_energies()[0], b.system.get_energies()[0])


def test_mts_energy_reported_at_inner_steps(lib):
    """Energies of a multiple-time-step run include the reciprocal term on
    every energy step, outer or inner."""
    from mdpy_gb300 import systems

    w = systems.water_box(900, 30.0, seed=1)
    ens = _ensemble(w)
    s, mask = ens.system, ens.term_mask
    s.integrator_config(lib.INTEGRATOR_VERLET, 1.0)
    s.set_mts(4)
    for n in (1, 2, 3, 4):
        s.integrate(1, mask, want_energy=True)
        e, _ = s.get_energies()
        x = s.get_positions()
        probe = _ensemble(w)
        probe.system.set_positions(x)
        probe.system.compute_forces(mask)
        ep, _ = probe.system.get_energies()
        assert abs(e[lib.TERM_COUL_RECIP] - ep[lib.TERM_COUL_RECIP]) < 1e-6 * abs(ep[lib.TERM_COUL_RECIP]) + 1e-6
        probe.system.close()


@pytest.mark.parametrize("bad", ["nan", "far"])
def test_particle_loss_raised_by_the_device(lib, bad):
    """A non-finite position, or one several boxes from the central image
    (mdpy's ParticleLossError rule, mdpy/utils/pbc.py:30-34), set from the
    host through the C ABI: the device re-sort of the next step flags it and
    the status read raises ParticleLossError.  The system stays usable: good
    positions afterwards step normally."""
    from mdpy_gb300 import systems
    from mdpy_gb300.error import ParticleLossError

    w = systems.water_box(300, 21.0, seed=2)
    ens = _ensemble(w, rc=9.0, K=24)
    s = ens.system
    s.integrator_config(lib.INTEGRATOR_LANGEVIN, 1.0, 300.0, 0.001, 3)
    s.integrate(3, ens.term_mask, want_energy=False)
    s.check_status()
    x = s.get_positions()
    v = s.get_velocities()
    x_bad = x.copy()
    if bad == "nan":
        x_bad[17, 1] = np.nan
    else:
        x_bad[17, 0] += 3.0 * w.box[0]
    s.set_positions(x_bad)
    s.integrate(2, ens.term_mask, want_energy=False)
    with pytest.raises(ParticleLossError):
        s.check_status()
    s.set_positions(x)
    s.set_velocities(v)
    s.integrate(2, ens.term_mask, want_energy=True)
    s.check_status()
    e, ke = s.get_energies()
    assert np.all(np.isfinite(e)) and np.isfinite(ke)
