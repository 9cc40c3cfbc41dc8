"""Pin the oracle against the unmodified reference (golden vectors made by
tests/golden/make_golden.py running mdpy v0.2.1) and against the reference
tests' own known answers.  CPU only."""
import numpy as np
import pytest

from tests.helpers import REF_E_TOL, half_box_tie_atoms, rel_rms_excluding, pairs_to_set, rel_rms


def test_reference_cell_list_restated_exactly(golden, orc):
    """CellList.update/kernel (mdpy/core/cell_list.py:83-116) on 6PO6 coordinates."""
    pos = golden["cl6po6_positions"]
    ncv, idx = orc.ref_cell_index(pos, np.full(3, 30, np.float32), 9.0)
    assert np.array_equal(ncv, golden["cl6po6_num_cell_vec"])
    assert np.array_equal(idx, golden["cl6po6_cell_index"])
    # the padded cell list: ascending atom index per cell, -1 padding
    cl = golden["cl6po6_cell_list"]
    for c in [(0, 0, 0), (1, 2, 0), (2, 2, 2)]:
        members = np.where((idx == np.array(c)).all(1))[0]
        row = cl[c]
        assert np.array_equal(row[:len(members)], members) and np.all(row[len(members):] == -1)


def test_reference_cell_index_water_boxes(golden, orc):
    for key, box in (("w900", 30.0), ("sp50", 50.0)):
        ncv, idx = orc.ref_cell_index(golden[key + "_positions"], np.full(3, box, np.float32), 12.0)
        assert np.array_equal(ncv, golden[key + "_num_cell_vec"])
        assert np.array_equal(idx, golden[key + "_cell_index"])


def test_reference_pair_enumeration_digest(golden, orc):
    pos = golden["w900_positions"]
    ref = orc.ref_pairs(pos, np.full(3, 30.0, np.float32), 12.0, golden["w900_cell_index"],
                        golden["w900_num_cell_vec"], golden["w900_bonded"])
    cnt, deg, dig = orc.pair_set_digest(ref, pos.shape[0])
    assert cnt == int(golden["w900_pairs_count"])
    assert dig == int(golden["w900_pairs_digest"])


def test_reference_float32_pair_test_over_all_pairs(golden, orc):
    """At 3^3 cells the reference's cell walk visits every pair, so its own
    float32 pair test applied to all pairs (the rule the GPU pair dump
    follows) gives exactly the reference's set: same count, degrees and
    digest as the golden vectors of the unmodified reference.  At 4^3 cells
    the all-pairs set contains the reference's set (which drops wrap pairs)."""
    from tests.helpers import ref32_pairs

    pos = golden["w900_positions"]
    n = pos.shape[0]
    allp = orc.pairs_bruteforce_ref32(pos, np.full(3, 30.0, np.float32), 12.0,
                                      golden["w900_bonded"])
    cnt, deg, dig = orc.pair_set_digest(allp, n)
    assert cnt == int(golden["w900_pairs_count"])
    assert dig == int(golden["w900_pairs_digest"])
    assert np.array_equal(deg, golden["w900_pairs_degree"])
    pos50 = golden["sp50_positions"]
    ref = pairs_to_set(orc.ref_pairs(pos50, np.full(3, 50.0, np.float32), 12.0,
                                     golden["sp50_cell_index"], golden["sp50_num_cell_vec"],
                                     np.full((pos50.shape[0], 1), -1)))
    assert ref < ref32_pairs(orc, pos50, 50.0, 12.0)


def test_lj_oracle_matches_reference_on_its_pair_set(golden, orc):
    """The FP64 LJ over the reference's pair set reproduces mdpy's float32
    CharmmNonbondedConstraint forces and energy (900 waters, 3^3 cells, where
    the reference's set is complete)."""
    pos = golden["w900_positions"].astype(np.float64)
    n = pos.shape[0]
    f, e = orc.nonbonded(pos, 30.0, golden["w900_lj_params"], np.zeros(n), golden["w900_bonded"],
                         np.full((n, 1), -1), 12.0, coulomb="none")
    assert rel_rms(f, golden["w900_f_lj"]) <= 1e-5
    # mdpy sums ~2e6 half-pair energies in float32: its own total carries ~1e-4 error
    assert e["lj"] == pytest.approx(float(golden["w900_e_lj"]), rel=REF_E_TOL)


def test_bare_coulomb_oracle_matches_reference(golden, orc):
    """ElectrostaticConstraint: units and constants agree (k = 1/(4 pi eps0))."""
    pos = golden["w900_positions"].astype(np.float64)
    n = pos.shape[0]
    f, e = orc.nonbonded(pos, 30.0, np.zeros((n, 4)), golden["w900_charges"], golden["w900_bonded"],
                         np.full((n, 1), -1), 12.0, lj=False, coulomb="bare")
    # all-pairs minimum image: pairs within float32 resolution of half the
    # box are ties the two codes may break differently (e.g. dy = 15.00000024 A
    # here); the atoms of such pairs are left out, everything else at 1e-5
    ties = half_box_tie_atoms(golden["w900_positions"], 30.0)
    assert len(ties) <= 8
    assert rel_rms_excluding(f, golden["w900_f_coul"], ties) <= 1e-5
    assert e["coulomb"] == pytest.approx(float(golden["w900_e_coul"]), rel=REF_E_TOL)
    pos4 = golden["es4_positions"].astype(np.float64)
    f4, e4 = orc.nonbonded(pos4, 100.0, np.zeros((4, 4)), golden["es4_charges"],
                           np.full((4, 1), -1), np.full((4, 1), -1), 12.0, lj=False, coulomb="bare")
    assert rel_rms(f4, golden["es4_forces"]) < 1e-6
    assert e4["coulomb"] == pytest.approx(float(golden["es4_energy"]), rel=1e-6)


def test_lj_four_atom_known_answer(golden, orc):
    """mdpy/test/test_charmm_nonbonded_constraint.py:93-126 known answers."""
    pos = golden["nb4_positions"].astype(np.float64)
    p = golden["nb4_params"].astype(np.float64)
    f, e = orc.nonbonded(pos, 30.0, p, np.zeros(4), np.full((4, 1), -1), np.full((4, 1), -1),
                         float(golden["nb4_cutoff"]))
    ref = golden["nb4_forces"].astype(np.float64)
    assert np.abs(f[0] - ref[0]).max() < 1e-8          # the reference test's assertion
    assert np.allclose(f, ref, rtol=1e-6, atol=1e-8)   # float32 precision elsewhere
    assert e["lj"] == pytest.approx(float(golden["nb4_energy"]), abs=1e-3)


def test_bond_angle_oracle_match_reference(golden, orc):
    from mdpy_gb300 import systems

    w = systems.water_box(900, 30.0, seed=0)
    pos = golden["wb900_positions"].astype(np.float64)
    t = w.topology
    kb = np.array([w.parameters["bond"]["OT-HT"]] * t.num_bonds)
    ka = np.array([w.parameters["angle"]["HT-OT-HT"]] * t.num_angles)
    fb, eb = orc.bonds(pos, 30.0, t.bonds, kb)
    fa, ea = orc.angles(pos, 30.0, t.angles, ka)
    assert rel_rms(fb, golden["wb900_f_bond"]) <= 1e-5
    assert rel_rms(fa, golden["wb900_f_angle"]) <= 1e-5
    assert eb == pytest.approx(float(golden["wb900_e_bond"]), rel=REF_E_TOL)
    assert ea == pytest.approx(float(golden["wb900_e_angle"]), rel=REF_E_TOL)
    for key, fn in (("bond4", orc.bonds), ("angle4", orc.angles)):
        f, e = fn(golden[key + "_positions"].astype(np.float64), 30.0, golden[key + "_idx"],
                  golden[key + "_prm"])
        assert np.abs(f - golden[key + "_forces"]).max() <= 1e-6 * np.abs(f).max()
        assert e == pytest.approx(float(golden[key + "_energy"]), rel=1e-6)


def test_reference_dihedral_force_is_not_the_gradient(golden, orc):
    """The reference's dihedral energy agrees with the oracle, its force does
    not (mdpy/constraint/charmm_dihedral_constraint.py:81 is not -dV/dphi);
    the oracle's force is the finite-difference gradient."""
    pos = golden["dih4_positions"].astype(np.float64)
    idx, prm = golden["dih4_idx"], golden["dih4_prm"].astype(np.float64)
    f, e = orc.dihedrals(pos, 30.0, idx, prm)
    assert e == pytest.approx(float(golden["dih4_energy"]), rel=1e-5, abs=1e-9)
    h = 1e-6
    g = np.zeros_like(pos)
    for k in range(4):
        for d in range(3):
            xp, xm = pos.copy(), pos.copy()
            xp[k, d] += h
            xm[k, d] -= h
            g[k, d] = -(orc.dihedrals(xp, 30.0, idx, prm)[1] - orc.dihedrals(xm, 30.0, idx, prm)[1]) / (2 * h)
    assert np.abs(f - g).max() < 1e-6 * max(np.abs(g).max(), 1e-12) + 1e-12
    assert np.abs(golden["dih4_forces"] - g).max() > 10 * np.abs(f - g).max()


def test_pbc_wrap_and_unwrap(golden, orc):
    """mdpy/test/test_pbc.py:26-81 inputs/outputs."""
    w = orc.wrap_positions(golden["pbc_wrap_in"].astype(np.float64), 10.0)
    assert np.allclose(w, golden["pbc_wrap_out"])
    d = golden["pbc_unwrap_in"].astype(np.float64)
    assert np.allclose(d - 10.0 * np.round(d / 10.0), golden["pbc_unwrap_out"], atol=1e-6)


def test_four_cell_box_defect_is_visible(golden, orc):
    """At 4^3 reference cells the reference pair set misses wrap pairs that
    brute force finds; the oracle restates both and the reference's LJ forces
    equal the oracle's LJ over the reference set."""
    pos32 = golden["sp50_positions"]
    n = pos32.shape[0]
    excl = np.full((n, 1), -1)
    ref = orc.ref_pairs(pos32, np.full(3, 50.0, np.float32), 12.0, golden["sp50_cell_index"],
                        golden["sp50_num_cell_vec"], excl)
    cnt, _, dig = orc.pair_set_digest(ref, n)
    assert cnt == int(golden["sp50_ref_count"]) and dig == int(golden["sp50_ref_digest"])
    bf = orc.pairs_bruteforce(pos32.astype(np.float64), 50.0, 12.0)
    bcnt, _, bdig = orc.pair_set_digest(bf, n)
    assert bcnt == int(golden["sp50_bf_count"]) and bdig == int(golden["sp50_bf_digest"])
    assert bcnt > cnt
    assert pairs_to_set(ref) <= pairs_to_set(bf)
    # LJ over exactly the reference pair set reproduces the reference forces
    pos = pos32.astype(np.float64)
    p = golden["sp50_lj_params"].astype(np.float64)
    f = np.zeros((n, 3))
    pr = np.asarray(ref, dtype=np.int64)
    d = pos[pr[:, 1]] - pos[pr[:, 0]]
    d -= 50.0 * np.round(d / 50.0)
    r2 = (d ** 2).sum(1)
    eps = np.sqrt(p[pr[:, 0], 0] * p[pr[:, 1], 0])
    sig = 0.5 * (p[pr[:, 0], 1] + p[pr[:, 1], 1])
    s6 = (sig ** 2 / r2) ** 3
    fr = 24 * eps * (2 * s6 * s6 - s6) / r2
    np.add.at(f, pr[:, 1], fr[:, None] * d)
    np.add.at(f, pr[:, 0], -fr[:, None] * d)
    assert rel_rms(f, golden["sp50_forces"]) <= 1e-5


def test_correct_verlet_within_reference_one_step_bound(golden, orc):
    """mdpy/test/test_verlet_integrator.py:33-47 allows 0.01 A after one step;
    the textbook velocity Verlet lands within that of the reference's step
    (whose first step is x + v dt, mdpy/integrator/verlet_integrator.py:26-44)."""
    x0 = golden["v81_positions0"].astype(np.float64)
    v0 = golden["v81_velocities0"].astype(np.float64)
    x1 = golden["v81_positions1"].astype(np.float64)
    d = x0 + v0 - x1
    d -= 25.0 * np.round(d / 25.0)
    assert np.abs(d).max() < 1e-5
