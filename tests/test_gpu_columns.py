"""Pair search over neighbouring sort columns (large boxes): the pair set is
the all-pairs set of the reference's float32 pair test, bit for bit, at every
reach the search uses (R = 2, R = 3, and the
full-scan fallback when 2R+1 columns no longer fit), also after the atoms
have drifted far from their sort columns without a re-sort; forces match the
FP64 oracle."""
import numpy as np
import pytest

from tests.helpers import (cutoff_band, keys_to_pairs, make_system, pair_keys, ref32_keys,
                           rel_rms, water_lj_rows)


def _same_pairs(orc, gpu, pos, box, rc):
    """The GPU set (pair_keys) equals, bit for bit, the reference's float32
    pair test over all pairs at the positions the system reports."""
    ref = ref32_keys(orc, pos, box, rc)
    assert np.array_equal(gpu, ref), (keys_to_pairs(np.setdiff1d(gpu, ref))[:5].tolist(),
                                      keys_to_pairs(np.setdiff1d(ref, gpu))[:5].tolist())

pytestmark = pytest.mark.gpu


def _box():
    from mdpy_gb300 import systems

    return systems.water_box(5000, 53.0, seed=21)   # 15,000 atoms, 8 x 8 columns


@pytest.mark.parametrize("half", [0, 1, 2])
@pytest.mark.parametrize("rc", [10.0, 14.0, 20.0])
def test_column_pair_set_equals_bruteforce(lib, orc, rc, half):
    w = _box()
    n = w.num_particles
    none = np.full((n, 1), -1)
    s = make_system(lib, n, w.box, lj=water_lj_rows(w), charges=np.zeros(n), bonded=none,
                    cutoff=rc, coulomb=lib.COUL_EWALD, beta=0.3, positions=w.positions)
    s.set_launch_shape(half=half)
    gpu = pair_keys(s.pairset())
    _same_pairs(orc, gpu, s.get_positions(), w.box, rc)
    # with the Ewald term every pair is evaluated (LJ-only runs skip pairs
    # of two atoms without LJ parameters); the force kernel decides r <= rc on
    # its packed float32 coordinates, so its count may differ from the
    # reference-arithmetic set only by pairs within 1e-4 A of the cutoff
    s.compute_forces(lib.mask(lib.TERM_LJ, lib.TERM_COUL_REAL))
    band = cutoff_band(orc, s.get_positions(), w.box, rc)
    assert abs(s.nonbonded_stats()["pairs_in_cutoff"] - len(gpu)) <= len(band)


@pytest.mark.parametrize("half", [0, 1, 2])
@pytest.mark.parametrize("n_waters,edge", [(5000, 53.0), (900, 30.0)])
def test_pair_set_after_drift_without_resort(lib, orc, n_waters, edge, half):
    """400 Langevin steps at 900 K with no re-sort: unbonded H atoms fly
    tens of A, past the periodic box; the pair set still equals the all-pairs
    set (53 A: neighbour-column search; 30 A: full scan with 27 images)."""
    from mdpy_gb300 import systems

    w = systems.water_box(n_waters, edge, seed=21)
    n = w.num_particles
    none = np.full((n, 1), -1)
    s = make_system(lib, n, w.box, masses=w.topology.masses.reshape(-1), lj=water_lj_rows(w),
                    charges=np.zeros(n), bonded=none, cutoff=12.0, positions=w.positions,
                    velocities=systems.maxwell_boltzmann(np.random.default_rng(3),
                                                         w.topology.masses, 900.0))
    s.set_reorder_interval(100000)
    s.set_launch_shape(half=half)
    s.integrator_config(lib.INTEGRATOR_LANGEVIN, 1.0, 900.0, 0.001, 7)
    s.integrate(400, lib.mask(lib.TERM_LJ), want_energy=False)
    x = s.get_positions()
    gpu = pair_keys(s.pairset())
    _same_pairs(orc, gpu, x, w.box, 12.0)


@pytest.mark.parametrize("half", [0, 1, 2])
def test_column_forces_vs_oracle(lib, orc, half):
    w = _box()
    t = w.topology
    n = w.num_particles
    beta = orc.ewald_beta(12.0, 1e-5)
    lj = water_lj_rows(w)
    s = make_system(lib, n, w.box, charges=t.charges.reshape(-1), lj=lj,
                    bonded=t.bonded_particles, scaling=t.scaling_particles, cutoff=12.0,
                    switch=10.0, coulomb=lib.COUL_EWALD, beta=beta, positions=w.positions)
    s.set_launch_shape(half=half)
    s.compute_forces(lib.mask(lib.TERM_LJ, lib.TERM_COUL_REAL))
    f = s.get_forces()
    e, _ = s.get_energies()
    fo, eo = orc.nonbonded(w.positions, w.box, lj, t.charges, t.bonded_particles,
                           t.scaling_particles, 12.0, switch=10.0, coulomb="ewald", beta=beta)
    assert rel_rms(f, fo) <= 1e-5
    assert e[lib.TERM_LJ] == pytest.approx(eo["lj"], rel=1e-5)
    # the real-space Coulomb total of neutral water is a small residual of
    # terms that sum in magnitude to about the self energy: compare on that scale
    scale = abs(orc.ewald_self(t.charges.reshape(-1), beta))
    assert abs(e[lib.TERM_COUL_REAL] - eo["coulomb"]) <= 1e-7 * scale
