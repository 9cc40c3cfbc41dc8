"""Short-range kernel parity: LJ and bare Coulomb against the reference's own
outputs (golden vectors), Ewald real space and the switch against the FP64
oracle, and the pair set against the reference's cell-list enumeration."""
import numpy as np
import pytest

from tests.helpers import (REF_E_TOL, cutoff_band, half_box_tie_atoms, make_system, pairs_to_set,
                           ref32_pairs, rel_rms, rel_rms_excluding, water_lj_rows)

pytestmark = pytest.mark.gpu


def test_lj_four_atoms_matches_reference(lib, golden):
    """mdpy/test/test_charmm_nonbonded_constraint.py:93-126 set-up."""
    pos = golden["nb4_positions"].astype(np.float64)
    s = make_system(lib, 4, golden["nb4_box"], lj=golden["nb4_params"].astype(np.float64),
                    charges=np.zeros(4), bonded=np.full((4, 1), -1),
                    cutoff=float(golden["nb4_cutoff"]), positions=pos)
    s.compute_forces(lib.mask(lib.TERM_LJ))
    f = s.get_forces()
    e, _ = s.get_energies()
    ref = golden["nb4_forces"].astype(np.float64)
    assert np.abs(f[0] - ref[0]).max() < 1e-8          # the reference test's abs=1e-8
    assert np.allclose(f, ref, rtol=1e-6, atol=1e-8)   # float32 precision elsewhere
    assert abs(f.sum()) < 1e-6
    assert e[lib.TERM_LJ] == pytest.approx(float(golden["nb4_energy"]), abs=1e-3)
    assert e[lib.TERM_LJ] == pytest.approx(float(golden["nb4_energy"]), rel=1e-5)


def test_lj_water_box_matches_reference(lib, golden):
    """900 waters, 30 A, rc 12: forces rel RMS <= 1e-5 vs mdpy's own constraint."""
    pos = golden["w900_positions"].astype(np.float64)
    n = pos.shape[0]
    s = make_system(lib, n, 30.0, lj=golden["w900_lj_params"].astype(np.float64),
                    charges=golden["w900_charges"].reshape(-1), bonded=golden["w900_bonded"],
                    cutoff=12.0, positions=pos)
    s.compute_forces(lib.mask(lib.TERM_LJ))
    f = s.get_forces()
    e, _ = s.get_energies()
    ref = golden["w900_f_lj"].astype(np.float64)
    assert rel_rms(f, ref) <= 1e-5
    # mdpy sums ~2e6 half-pair energies in float32: its own total carries ~1e-4 error
    assert e[lib.TERM_LJ] == pytest.approx(float(golden["w900_e_lj"]), rel=REF_E_TOL)


def test_pair_set_matches_reference_cell_list(lib, golden, orc):
    """3^3 reference cells: the GPU pair set equals, bit for bit, the set the
    reference's kernel visits (mdpy/constraint/charmm_nonbonded_constraint.py:
    75-90).  The dump decides r <= rc with the reference's own float32
    arithmetic, so pairs at the cutoff fall on the reference's side."""
    pos32 = golden["w900_positions"]
    n = pos32.shape[0]
    ref = orc.ref_pairs(pos32, np.full(3, 30.0, np.float32), 12.0, golden["w900_cell_index"],
                        golden["w900_num_cell_vec"], golden["w900_bonded"])
    cnt, deg, dig = orc.pair_set_digest(ref, n)
    assert cnt == int(golden["w900_pairs_count"]) and dig == int(golden["w900_pairs_digest"])
    assert np.array_equal(deg, golden["w900_pairs_degree"])
    s = make_system(lib, n, 30.0, lj=golden["w900_lj_params"].astype(np.float64),
                    charges=np.zeros(n), bonded=golden["w900_bonded"], cutoff=12.0,
                    positions=pos32.astype(np.float64))
    gpu = pairs_to_set(s.pairset())
    refs = pairs_to_set(ref)
    # the pairs within 1e-4 A of the cutoff, where FP32 rounding decides
    band = cutoff_band(orc, pos32, 30.0, 12.0)
    band = {p for p in band if golden["w900_bonded"][p[0]].tolist().count(p[1]) == 0}
    print("cutoff band: %d pairs within 1e-4 A of rc, %d of them in the reference's set"
          % (len(band), len(band & refs)))
    assert gpu == refs, (sorted(gpu - refs)[:5], sorted(refs - gpu)[:5])
    # every form of the pair kernel (i groups of 32, 16 and 8 atoms) finds it
    for half in (1, 2):
        s.set_launch_shape(half=half)
        assert pairs_to_set(s.pairset()) == refs, half


def test_pair_set_4_cells_superset_of_reference(lib, golden, orc):
    """4^3 reference cells: the reference drops pairs across the periodic
    wrap (its cell adjacency misses them).  The GPU set equals, bit for bit,
    the reference's float32 pair test over all pairs; it contains the
    reference's set, and every pair it adds lies in cells the reference's
    walk does not treat as neighbours."""
    pos32 = golden["sp50_positions"]
    n = pos32.shape[0]
    excl = np.full((n, 1), -1)
    ref = pairs_to_set(orc.ref_pairs(pos32, np.full(3, 50.0, np.float32), 12.0,
                                     golden["sp50_cell_index"], golden["sp50_num_cell_vec"], excl))
    assert len(ref) == int(golden["sp50_ref_count"])
    bf = pairs_to_set(orc.pairs_bruteforce(pos32.astype(np.float64), 50.0, 12.0))
    assert len(bf) == int(golden["sp50_bf_count"])
    s = make_system(lib, n, 50.0, lj=golden["sp50_lj_params"].astype(np.float64),
                    charges=np.zeros(n), bonded=excl, cutoff=12.0,
                    positions=pos32.astype(np.float64))
    gpu = pairs_to_set(s.pairset())
    assert gpu == ref32_pairs(orc, pos32, 50.0, 12.0)
    assert ref <= gpu
    # each pair the reference drops sits in cells that are not adjacent mod n,
    # and every GPU pair in adjacent cells is one the reference visits
    ci = golden["sp50_cell_index"]
    ncv = golden["sp50_num_cell_vec"]
    missing_in_ref = gpu - ref
    assert len(missing_in_ref) > 0
    for i, j in gpu:
        d = np.abs(ci[i] - ci[j])
        d = np.minimum(d, ncv - d)
        assert np.any(d > 1) == ((i, j) in missing_in_ref)
    print("4^3 cells: %d pairs, %d dropped by the reference's cell walk"
          % (len(gpu), len(missing_in_ref)))


def test_lj_forces_four_cell_box_match_reference(lib, golden, orc):
    """Where the reference's pair set is incomplete (4^3 cells) its forces
    differ from the GPU's by exactly the contribution of the pairs it drops."""
    pos32 = golden["sp50_positions"]
    pos = pos32.astype(np.float64)
    n = pos.shape[0]
    p = golden["sp50_lj_params"].astype(np.float64)
    s = make_system(lib, n, 50.0, lj=p, charges=np.zeros(n), bonded=np.full((n, 1), -1),
                    cutoff=12.0, positions=pos)
    s.compute_forces(lib.mask(lib.TERM_LJ))
    f = s.get_forces()
    ref = golden["sp50_forces"].astype(np.float64)
    refset = pairs_to_set(orc.ref_pairs(pos32, np.full(3, 50.0, np.float32), 12.0,
                                        golden["sp50_cell_index"], golden["sp50_num_cell_vec"],
                                        np.full((n, 1), -1)))
    dropped = np.array(sorted(pairs_to_set(orc.pairs_bruteforce(pos, 50.0, 12.0)) - refset))
    d = pos[dropped[:, 1]] - pos[dropped[:, 0]]
    d -= 50.0 * np.round(d / 50.0)
    r2 = (d ** 2).sum(1)
    eps = np.sqrt(p[dropped[:, 0], 0] * p[dropped[:, 1], 0])
    sig = 0.5 * (p[dropped[:, 0], 1] + p[dropped[:, 1], 1])
    s6 = (sig ** 2 / r2) ** 3
    fr = 24 * eps * (2 * s6 * s6 - s6) / r2
    f_drop = np.zeros((n, 3))
    np.add.at(f_drop, dropped[:, 1], fr[:, None] * d)
    np.add.at(f_drop, dropped[:, 0], -fr[:, None] * d)
    assert len(dropped) > 0
    assert rel_rms(f, ref + f_drop) <= 1e-5
    # on the atoms of the dropped pairs, the pairs the reference misses account
    # for the GPU-minus-reference difference (elsewhere both agree to float32)
    hit = np.unique(dropped.reshape(-1))
    before = np.sqrt(np.mean((f[hit] - ref[hit]) ** 2))
    after = np.sqrt(np.mean((f[hit] - ref[hit] - f_drop[hit]) ** 2))
    assert after < 0.3 * before


def test_bare_coulomb_four_atoms_matches_reference(lib, golden):
    """mdpy/test/test_electrostatic_constraint.py:197-221 set-up (all pairs)."""
    pos = golden["es4_positions"].astype(np.float64)
    s = make_system(lib, 4, golden["es4_box"], charges=golden["es4_charges"].reshape(-1),
                    lj=np.zeros((4, 4)), bonded=np.full((4, 1), -1), cutoff=12.0, lj_on=False,
                    coulomb=lib.COUL_BARE, positions=pos)
    s.compute_forces(lib.mask(lib.TERM_COUL_REAL))
    f = s.get_forces()
    e, _ = s.get_energies()
    ref = golden["es4_forces"].astype(np.float64)
    assert rel_rms(f, ref) < 1e-6
    assert e[lib.TERM_COUL_REAL] == pytest.approx(float(golden["es4_energy"]), rel=1e-6)


def test_bare_coulomb_water_box_matches_reference(lib, golden):
    pos = golden["w900_positions"].astype(np.float64)
    n = pos.shape[0]
    s = make_system(lib, n, 30.0, charges=golden["w900_charges"].reshape(-1),
                    lj=np.zeros((n, 4)), bonded=golden["w900_bonded"], cutoff=12.0, lj_on=False,
                    coulomb=lib.COUL_BARE, positions=pos)
    s.compute_forces(lib.mask(lib.TERM_COUL_REAL))
    f = s.get_forces()
    e, _ = s.get_energies()
    # all-pairs minimum image: pairs within float32 resolution of half the
    # box are ties the two codes may break differently (e.g. dy = 15.00000024 A
    # here); the atoms of such pairs are left out, everything else at 1e-5
    ties = half_box_tie_atoms(golden["w900_positions"], 30.0)
    assert len(ties) <= 8
    assert rel_rms_excluding(f, golden["w900_f_coul"], ties) <= 1e-5
    assert e[lib.TERM_COUL_REAL] == pytest.approx(float(golden["w900_e_coul"]), rel=REF_E_TOL)


@pytest.mark.parametrize("switch", [None, 10.0])
def test_lj_ewald_real_vs_oracle(lib, orc, switch):
    from mdpy_gb300 import systems

    w = systems.water_box(2000, 27.0, seed=11)
    t = w.topology
    n = w.num_particles
    beta = orc.ewald_beta(12.0, 1e-5)
    lj = water_lj_rows(w)
    s = make_system(lib, n, w.box, charges=t.charges.reshape(-1), lj=lj,
                    bonded=t.bonded_particles, scaling=t.scaling_particles, cutoff=12.0,
                    switch=switch or 0.0, coulomb=lib.COUL_EWALD, beta=beta, positions=w.positions)
    s.compute_forces(lib.mask(lib.TERM_LJ, lib.TERM_COUL_REAL))
    f = s.get_forces()
    e, _ = s.get_energies()
    fo, eo = orc.nonbonded(w.positions, w.box, lj, t.charges, t.bonded_particles,
                           t.scaling_particles, 12.0, switch=switch, coulomb="ewald", beta=beta)
    assert rel_rms(f, fo) <= 1e-5
    assert e[lib.TERM_LJ] == pytest.approx(eo["lj"], rel=1e-5)
    assert e[lib.TERM_COUL_REAL] == pytest.approx(eo["coulomb"], rel=1e-5)


def test_one_four_pairs_and_chain_vs_oracle(lib, orc):
    """A solvated chain: 1-4 pairs take the 1-4 LJ parameters and the normal
    Coulomb term; 1-2/1-3 pairs are excluded."""
    from mdpy_gb300 import systems

    c = systems.chain_in_water(n_waters=460, box=24.0, n_beads=60, seed=5)
    t = c.topology
    n = c.num_particles
    p = c.parameters["nonbonded"]
    lj = np.array([[p[ty][0], p[ty][1], 0.5 * p[ty][0], 0.9 * p[ty][1]] for ty in t.particle_types])
    beta = orc.ewald_beta(11.0, 1e-5)
    s = make_system(lib, n, c.box, charges=t.charges.reshape(-1), lj=lj,
                    bonded=t.bonded_particles, scaling=t.scaling_particles, cutoff=11.0,
                    switch=9.0, coulomb=lib.COUL_EWALD, beta=beta, positions=c.positions)
    s.compute_forces(lib.mask(lib.TERM_LJ, lib.TERM_COUL_REAL))
    f = s.get_forces()
    e, _ = s.get_energies()
    fo, eo = orc.nonbonded(c.positions, c.box, lj, t.charges, t.bonded_particles,
                           t.scaling_particles, 11.0, switch=9.0, coulomb="ewald", beta=beta)
    assert rel_rms(f, fo) <= 1e-5
    assert e[lib.TERM_LJ] == pytest.approx(eo["lj"], rel=1e-5)
    assert e[lib.TERM_COUL_REAL] == pytest.approx(eo["coulomb"], rel=1e-5)


def test_forces_bit_reproducible(lib):
    from mdpy_gb300 import systems

    w = systems.water_box(3000, 31.0, seed=2)
    t = w.topology
    out = []
    for _ in range(2):
        s = make_system(lib, w.num_particles, w.box, charges=t.charges.reshape(-1),
                        lj=water_lj_rows(w), bonded=t.bonded_particles, cutoff=12.0,
                        coulomb=lib.COUL_EWALD, beta=0.27, positions=w.positions)
        s.compute_forces(lib.mask(lib.TERM_LJ, lib.TERM_COUL_REAL))
        out.append(s.get_forces())
        s.compute_forces(lib.mask(lib.TERM_LJ, lib.TERM_COUL_REAL))
        out.append(s.get_forces())
    for o in out[1:]:
        assert np.array_equal(o, out[0])


def test_empty_and_tiny_systems(lib):
    # one atom: no pairs, zero force, energy 0
    s = make_system(lib, 1, 30.0, charges=[0.5], lj=np.array([[1e-4, 3.0, 1e-4, 3.0]]),
                    bonded=np.full((1, 1), -1), cutoff=12.0, coulomb=lib.COUL_EWALD, beta=0.3,
                    positions=np.zeros((1, 3)))
    s.compute_forces(lib.mask(lib.TERM_LJ, lib.TERM_COUL_REAL))
    assert np.all(s.get_forces() == 0)
    assert len(s.pairset()) == 0
    # 33 atoms: one full cluster plus a cluster of one
    rng = np.random.default_rng(0)
    x = rng.uniform(0, 20, size=(33, 3))
    s = make_system(lib, 33, 20.0, charges=np.zeros(33), lj=np.tile([1e-4, 3.0, 1e-4, 3.0], (33, 1)),
                    bonded=np.full((33, 1), -1), cutoff=9.0, positions=x)
    from oracle import oracle as O
    gpu = pairs_to_set(s.pairset())
    assert gpu == ref32_pairs(O, s.get_positions(), 20.0, 9.0)


def test_cutoff_validation(lib):
    from mdpy_gb300.error import CellListPoorDefinedError

    s = lib.System(10, 20.0)
    with pytest.raises(CellListPoorDefinedError):
        s.nonbonded_config(10.5)


def test_overlapping_atoms_raise_fixed_point_overflow(lib):
    """Two LJ atoms 0.2 A apart give forces ~1e13, outside the int64
    fixed-point range (|F| < 2^31 internal units): the kernel's own check
    reports it instead of returning a wrapped sum."""
    from mdpy_gb300.error import FixedPointOverflowError

    x = np.array([[1.0, 1.0, 1.0], [1.2, 1.0, 1.0]])
    s = make_system(lib, 2, 30.0, charges=np.zeros(2),
                    lj=np.tile([6.4e-5, 3.15, 6.4e-5, 3.15], (2, 1)), bonded=np.full((2, 1), -1),
                    cutoff=12.0, positions=x)
    s.compute_forces(lib.mask(lib.TERM_LJ))
    with pytest.raises(FixedPointOverflowError):
        s.get_forces()
    # the status is cleared once reported; a sane configuration works again
    s.set_positions(np.array([[1.0, 1.0, 1.0], [4.5, 1.0, 1.0]]))
    s.compute_forces(lib.mask(lib.TERM_LJ))
    assert np.all(np.isfinite(s.get_forces()))
