"""Bonded terms: bond/angle against the reference's own outputs; dihedral and
improper energies against the reference, forces against the exact gradient
(the reference's dihedral force is not -dV/dphi)."""
import numpy as np
import pytest

from tests.helpers import REF_E_TOL, make_system, rel_rms

pytestmark = pytest.mark.gpu


def _bonded_case(lib, golden, key, setter, mask_term):
    pos = golden[key + "_positions"].astype(np.float64)
    s = make_system(lib, 4, 30.0, positions=pos)
    getattr(s, setter)(golden[key + "_idx"], golden[key + "_prm"].astype(np.float64))
    s.compute_forces(lib.mask(mask_term))
    e, _ = s.get_energies()
    return s.get_forces(), e[mask_term], pos


def test_bond_matches_reference(lib, golden):
    f, e, _ = _bonded_case(lib, golden, "bond4", "set_bonds", lib.TERM_BOND)
    ref = golden["bond4_forces"].astype(np.float64)
    assert np.abs(f - ref).max() <= 1e-6 * np.abs(ref).max()
    assert e == pytest.approx(float(golden["bond4_energy"]), rel=1e-6)


def test_angle_matches_reference(lib, golden):
    f, e, _ = _bonded_case(lib, golden, "angle4", "set_angles", lib.TERM_ANGLE)
    ref = golden["angle4_forces"].astype(np.float64)
    assert np.abs(f - ref).max() <= 2e-6 * np.abs(ref).max()
    assert e == pytest.approx(float(golden["angle4_energy"]), rel=1e-6)


@pytest.mark.parametrize("key,setter,term,fn", [
    ("dih4", "set_dihedrals", "TERM_DIHEDRAL", "dihedrals"),
    ("imp4", "set_impropers", "TERM_IMPROPER", "impropers")])
def test_torsions_energy_reference_forces_exact(lib, golden, orc, key, setter, term, fn):
    t = getattr(lib, term)
    f, e, pos = _bonded_case(lib, golden, key, setter, t)
    assert e == pytest.approx(float(golden[key + "_energy"]), rel=1e-5, abs=1e-9)
    fo, eo = getattr(orc, fn)(pos, 30.0, golden[key + "_idx"], golden[key + "_prm"])
    assert eo == pytest.approx(float(golden[key + "_energy"]), rel=1e-5, abs=1e-9)
    assert rel_rms(f, fo) <= 1e-5


def test_water_bonds_angles_match_reference(lib, golden):
    from mdpy_gb300 import systems

    pos = golden["wb900_positions"].astype(np.float64)
    w = systems.water_box(900, 30.0, seed=0)
    t = w.topology
    kb = np.array([w.parameters["bond"]["OT-HT"]] * t.num_bonds)
    ka = np.array([w.parameters["angle"]["HT-OT-HT"]] * t.num_angles)
    s = make_system(lib, pos.shape[0], 30.0, positions=pos)
    s.set_bonds(t.bonds, kb)
    s.set_angles(t.angles, ka)
    for term, key, en in ((lib.TERM_BOND, "wb900_f_bond", "wb900_e_bond"),
                          (lib.TERM_ANGLE, "wb900_f_angle", "wb900_e_angle")):
        s.compute_forces(lib.mask(term))
        e, _ = s.get_energies()
        assert rel_rms(s.get_forces(), golden[key]) <= 1e-5
        assert e[term] == pytest.approx(float(golden[en]), rel=REF_E_TOL)


def test_chain_bonded_vs_oracle(lib, orc):
    from mdpy_gb300 import systems

    c = systems.chain_in_water(n_waters=460, box=24.0, n_beads=80, seed=9)
    t = c.topology
    s = make_system(lib, c.num_particles, c.box, positions=c.positions)
    types = t.particle_types
    kb = np.array([c.parameters["bond"]["%s-%s" % (types[i], types[j])] for i, j in t.bonds])
    ka = np.array([c.parameters["angle"]["%s-%s-%s" % (types[i], types[j], types[k])]
                   for i, j, k in t.angles])
    s.set_bonds(t.bonds, kb)
    s.set_angles(t.angles, ka)
    s.set_dihedrals(t.dihedrals, c.dihedral_parameters)
    imp = t.dihedrals[::7]
    ip = np.stack([np.full(len(imp), 0.01), np.linspace(-2.0, 2.0, len(imp))], 1)
    s.set_impropers(imp, ip)
    s.compute_forces(lib.mask(lib.TERM_BOND, lib.TERM_ANGLE, lib.TERM_DIHEDRAL, lib.TERM_IMPROPER))
    f = s.get_forces()
    e, _ = s.get_energies()
    fb, eb = orc.bonds(c.positions, c.box, t.bonds, kb)
    fa, ea = orc.angles(c.positions, c.box, t.angles, ka)
    fd, ed = orc.dihedrals(c.positions, c.box, t.dihedrals, c.dihedral_parameters)
    fi, ei = orc.impropers(c.positions, c.box, imp, ip)
    assert rel_rms(f, fb + fa + fd + fi) <= 1e-5
    assert e[lib.TERM_BOND] == pytest.approx(eb, rel=1e-5)
    assert e[lib.TERM_ANGLE] == pytest.approx(ea, rel=1e-5)
    assert e[lib.TERM_DIHEDRAL] == pytest.approx(ed, rel=1e-5)
    assert e[lib.TERM_IMPROPER] == pytest.approx(ei, rel=1e-4)
