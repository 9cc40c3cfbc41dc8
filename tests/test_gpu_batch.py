"""Batches of independent systems: every member's forces, energies and
trajectory equal the ones it has alone.  The pair, special-pair and bonded
sums are int64 fixed point and the batch keeps each member's cluster layout,
so those match bit for bit; the batched FFT may round differently, so PME
terms match to float precision."""
import numpy as np
import pytest

from tests.helpers import rel_rms

pytestmark = pytest.mark.gpu

RC = 9.0
SIZES = (400, 700, 700, 1100)  # waters per member; two share a PME grid


def _boxes():
    from mdpy_gb300 import systems

    out = []
    for k, nw in enumerate(SIZES):
        edge = (3 * nw / 0.1) ** (1.0 / 3.0)
        out.append(systems.water_box(nw, edge, seed=11 + k))
    return out


def _setup(ens, w):
    from mdpy_gb300 import constraint as C, systems

    grid = systems.fft_friendly(int(np.ceil(w.box[0])))
    ens.add_constraints(
        C.NonbondedConstraint(w.parameters["nonbonded"], RC, ewald_error=1e-5),
        C.PMEConstraint(grid_size=grid, ewald_error=1e-5, real_space_cutoff=RC),
        C.CharmmBondConstraint(w.parameters["bond"]),
        C.CharmmAngleConstraint(w.parameters["angle"]))
    ens.state.set_positions(w.positions)
    ens.state.set_velocities(w.velocities)
    return ens


def _singles(ws):
    from mdpy_gb300.ensemble import Ensemble

    return [_setup(Ensemble(w.topology, w.pbc_matrix), w) for w in ws]


def _batch(ws):
    from mdpy_gb300 import batch

    return batch.EnsembleBatch([_setup(batch.member(w.topology, w.pbc_matrix), w) for w in ws])


def test_batch_forces_and_energies_match_singles(lib):
    ws = _boxes()
    singles = _singles(ws)
    b = _batch(ws)
    assert b.system.n_systems == len(SIZES)
    # fixed-point terms: bit for bit
    short = lib.mask(lib.TERM_LJ, lib.TERM_COUL_REAL, lib.TERM_BOND, lib.TERM_ANGLE)
    b.system.compute_forces(short)
    fb = b.system.get_forces()
    eb, _ = b.system.get_energies_batch()
    for q, s in enumerate(singles):
        s.system.compute_forces(short)
        f1 = s.system.get_forces()
        e1, _ = s.system.get_energies()
        assert np.array_equal(fb[b.member_slice(q)], f1), q
        # pair energies are summed per cluster: exact; bonded and kinetic
        # energies are FP64 block sums whose blocks straddle members, so
        # they agree to the fixed-point unit (2^-32) per block
        for t in (lib.TERM_LJ, lib.TERM_COUL_REAL):
            assert eb[q, t] == e1[t], (q, t)
        for t in (lib.TERM_BOND, lib.TERM_ANGLE):
            assert eb[q, t] == pytest.approx(e1[t], abs=1e-7), (q, t)
    # everything, PME included
    b.update()
    for q, s in enumerate(singles):
        s.update()
        assert rel_rms(b.forces(q), s.forces) < 1e-6, q
        e1 = s._energies
        scale = np.abs(e1).sum()
        assert np.all(np.abs(b.energies[q] - e1) <= 1e-7 * scale), (q, b.energies[q], e1)
        assert b.kinetic_energies[q] == pytest.approx(s.kinetic_energy, abs=1e-7)
    # the summed entry point reports the sum over members
    tot, ke = b.system.get_energies()
    assert np.allclose(tot, b.energies.sum(axis=0), rtol=1e-12, atol=1e-9)
    assert ke == pytest.approx(b.kinetic_energies.sum(), rel=1e-12)


def test_batch_pme_grids_of_any_size(lib, orc):
    """Odd grid sizes in several size groups (unaligned grid lengths): each
    member's reciprocal forces match the FP64 PME of its own grid."""
    from mdpy_gb300 import systems

    ws = [systems.water_box(nw, (3 * nw / 0.1) ** (1 / 3), seed=40 + k)
          for k, nw in enumerate((500, 600, 500, 800))]
    grids = [(25, 25, 25), (27, 27, 27), (25, 25, 25), (30, 27, 25)]
    beta = orc.ewald_beta(9.0, 1e-5)
    s = lib.System.batch([w.num_particles for w in ws], [w.box for w in ws])
    s.set_charges(np.concatenate([w.topology.charges.reshape(-1) for w in ws]))
    s.nonbonded_config(9.0, 0.0, False, lib.COUL_EWALD, beta)
    s.pme_config_batch(grids, 4, beta)
    s.set_positions(np.concatenate([w.positions for w in ws]))
    s.compute_forces(lib.mask(lib.TERM_COUL_RECIP))
    f = s.get_forces()
    e, _ = s.get_energies_batch()
    off = 0
    for k, (w, K) in enumerate(zip(ws, grids)):
        q = w.topology.charges.reshape(-1)
        fp, ep = orc.pme(w.positions, w.box, q, beta, K, 4)
        n = w.num_particles
        # no exclusions were set: the slot holds reciprocal + self + net charge
        assert rel_rms(f[off:off + n], fp) <= 2e-5, k
        e_self = orc.ewald_self(q, beta)
        e_ref = ep + e_self + orc.ewald_net_charge(q, w.box, beta)
        assert abs(e[k, lib.TERM_COUL_RECIP] - e_ref) <= 2e-7 * (abs(ep) + abs(e_self)), k
        off += n
    s.close()


def test_batch_trajectory_matches_singles(lib):
    """25 velocity-Verlet steps (one re-sort on the way) without the FFT
    term: positions and velocities equal bit for bit."""
    from mdpy_gb300.integrator import VerletIntegrator

    ws = _boxes()
    singles = _singles(ws)
    b = _batch(ws)
    mask = lib.mask(lib.TERM_LJ, lib.TERM_COUL_REAL, lib.TERM_BOND, lib.TERM_ANGLE)
    b.system.integrator_config(lib.INTEGRATOR_VERLET, 0.5)
    b.system.integrate(25, mask, want_energy=True)
    xb, vb = b.positions(), b.velocities()
    eb, keb = b.system.get_energies_batch()
    for q, s in enumerate(singles):
        s.system.integrator_config(lib.INTEGRATOR_VERLET, 0.5)
        s.system.integrate(25, mask, want_energy=True)
        assert np.array_equal(xb[b.member_slice(q)], s.system.get_positions()), q
        assert np.array_equal(vb[b.member_slice(q)], s.system.get_velocities()), q
        e1, ke1 = s.system.get_energies()
        assert eb[q, lib.TERM_LJ] == e1[lib.TERM_LJ]
        assert keb[q] == pytest.approx(ke1, abs=1e-7)
    # the mdpy-style integrator drives a batch like an ensemble
    VerletIntegrator(0.5).integrate(b, 5)
    assert np.all(np.isfinite(b.potential_energies)) and np.all(b.kinetic_energies > 0)


def test_batch_rejects_terms_across_members(lib):
    s = lib.System.batch([6, 6], [[20.0] * 3, [22.0] * 3])
    with pytest.raises(Exception, match="spans two systems"):
        s.set_bonds(np.array([[0, 7]]), np.array([[1.0, 1.0]]))
    with pytest.raises(Exception, match="partner"):
        b = np.full((12, 1), -1)
        b[2, 0] = 9
        s.set_exclusions(b, np.full((12, 1), -1))
    s.set_bonds(np.array([[0, 1], [6, 7]]), np.array([[1.0, 1.0], [1.0, 1.0]]))
    s.close()
