"""Launch shapes of the pair kernel (work items per cluster, grid or
persistent work queue) and of the PME spread/gather blocks: every shape
gives the same pair set and the same forces up to float rounding of partial
sums, each shape is bit-reproducible, and the autotuner keeps one of them."""
import numpy as np
import pytest

from tests.helpers import make_system, pair_keys, rel_rms, water_lj_rows

pytestmark = pytest.mark.gpu


def _system(lib, orc, w):
    t = w.topology
    beta = orc.ewald_beta(10.0, 1e-5)
    s = make_system(lib, w.num_particles, w.box, charges=t.charges.reshape(-1),
                    lj=water_lj_rows(w), bonded=t.bonded_particles, scaling=t.scaling_particles,
                    cutoff=10.0, switch=8.0, coulomb=lib.COUL_EWALD, beta=beta,
                    positions=w.positions)
    s.pme_config(36, 4, beta)
    return s


@pytest.mark.parametrize("edge,n_waters", [(30.0, 900), (53.0, 5000)])  # full scan; columns
def test_every_shape_gives_the_same_forces(lib, orc, edge, n_waters):
    from mdpy_gb300 import systems

    w = systems.water_box(n_waters, edge, seed=8)
    s = _system(lib, orc, w)
    mask = lib.mask(lib.TERM_LJ, lib.TERM_COUL_REAL, lib.TERM_COUL_RECIP)
    ref_pairs = None
    ref_f = None
    for split in (1, 2, 4, 8, 16):
        # persistent 1: few resident warps, so each takes several items per
        # queue atomic (grab > 1)
        for persistent, half in ((0, 0), (20, 0), (1, 0), (0, 1), (20, 1), (0, 2), (12, 2)):
            s.set_launch_shape(split, persistent, (64, 128, 256)[split % 3], split % 2,
                               (split // 2) % 2, split % 4, half)
            pairs = pair_keys(s.pairset())
            s.compute_forces(mask)
            f1 = s.get_forces()
            s.compute_forces(mask)
            f2 = s.get_forces()
            assert np.array_equal(f1, f2), (split, persistent, half)     # reproducible
            if ref_f is None:
                ref_pairs, ref_f = pairs, f1
            else:
                assert np.array_equal(pairs, ref_pairs), (split, persistent, half)
                assert rel_rms(f1, ref_f) < 1e-6, (split, persistent, half)
    with pytest.raises(Exception, match="split"):
        s.set_launch_shape(3, 0, 256)
    with pytest.raises(Exception, match="PME block"):
        s.set_launch_shape(4, 0, 96)
    with pytest.raises(Exception, match="persistent"):
        s.set_launch_shape(4, 25, 256)
    with pytest.raises(Exception, match="pme_tiles"):
        s.set_launch_shape(4, 0, 256, 0, 1, 4)


def test_autotune_keeps_a_valid_shape(lib, orc):
    from mdpy_gb300 import systems

    w = systems.water_box(1400, 35.0, seed=9)
    s = _system(lib, orc, w)
    mask = lib.mask(lib.TERM_LJ, lib.TERM_COUL_REAL, lib.TERM_COUL_RECIP)
    s.compute_forces(mask)
    f0 = s.get_forces()
    r = s.autotune(mask, reps=3)
    assert r["split"] in (2, 4, 8) and r["pme_block"] in (64, 128, 256)
    assert r["persistent"] in (0, 20, 24) and r["side_priority"] in (0, 1)
    assert r["split_rings"] in (0, 1) and r["pme_tiles"] in (0, 1, 2, 3) and r["tuned_ms"] > 0
    assert r["half"] in (0, 1, 2)
    with pytest.raises(Exception, match="no force evaluation"):
        s.get_forces()
    s.compute_forces(mask)
    assert rel_rms(s.get_forces(), f0) < 1e-6


def test_autotune_over_md_steps_restores_the_state(lib, orc):
    """With an integrator configured the autotuner times MD steps; positions,
    velocities and the Langevin noise counter are put back, so the next
    steps are those the system would have taken without tuning."""
    from mdpy_gb300 import constraint as C, systems
    from mdpy_gb300.ensemble import Ensemble

    w = systems.water_box(900, 30.0, seed=10)
    runs = []
    for tune in (False, True):
        ens = Ensemble(w.topology, w.pbc_matrix)
        ens.add_constraints(C.NonbondedConstraint(w.parameters["nonbonded"], 10.0,
                                                  switch_radius=8.0),
                            C.PMEConstraint(grid_size=32, real_space_cutoff=10.0),
                            C.CharmmBondConstraint(w.parameters["bond"]),
                            C.CharmmAngleConstraint(w.parameters["angle"]))
        ens.state.set_positions(w.positions)
        ens.state.set_velocities(w.velocities)
        s, mask = ens.system, ens.term_mask
        s.integrator_config(lib.INTEGRATOR_LANGEVIN, 1.0, 300.0, 0.001, 3)
        s.integrate(5, mask, want_energy=False)
        if tune:
            r = s.autotune(mask, reps=2)
            assert r["tuned_ms"] > 0
            s.set_launch_shape(4, 0, 256, 0, 1, 0, 0)  # compare under one shape
        s.integrate(5, mask, want_energy=True)
        runs.append((s.get_positions(), s.get_velocities()))
    # a re-sort after the restore changes the order of the FP32 partial sums
    # only: after 5 steps the positions differ by ~1e-9 relative (a state that
    # was not restored -- positions, velocities or the noise counter --
    # differs by 1e-4 or more)
    assert rel_rms(runs[1][0], runs[0][0]) < 1e-8
    assert rel_rms(runs[1][1], runs[0][1]) < 1e-6


def test_pme_tiles_are_bit_identical(lib, orc):
    """Spreading and gathering through shared-memory tiles add the same int64
    contributions and read the same potential values as the direct kernels:
    the reciprocal-space forces agree bit for bit (one batch with several
    systems, so blocks that span two systems take the direct path)."""
    from mdpy_gb300 import systems

    ws = [systems.water_box(nw, (3 * nw / 0.1) ** (1 / 3), seed=50 + k)
          for k, nw in enumerate((700, 500, 900))]
    beta = orc.ewald_beta(9.0, 1e-5)
    s = lib.System.batch([w.num_particles for w in ws], [w.box for w in ws])
    s.set_charges(np.concatenate([w.topology.charges.reshape(-1) for w in ws]))
    s.nonbonded_config(9.0, 0.0, False, lib.COUL_EWALD, beta)
    s.pme_config_batch([(27, 27, 27), (25, 25, 25), (30, 30, 30)], 4, beta)
    s.set_positions(np.concatenate([w.positions for w in ws]))
    out = []
    for tiles in range(4):
        for block in (64, 256):
            s.set_launch_shape(4, 0, block, 0, 1, tiles)
            s.compute_forces(lib.mask(lib.TERM_COUL_RECIP))
            out.append((s.get_forces(), s.get_energies_batch()[0]))
    for f, e in out[1:]:
        assert np.array_equal(f, out[0][0]) and np.array_equal(e, out[0][1])
