"""PME reciprocal space against the FP64 oracle (same grid), and the full
Ewald sum (real + reciprocal + exclusion + self + net charge) against the
FP64 direct Ewald sum.  mdpy has no Ewald/PME: these parities are pinned by
the oracle's mathematics (Madelung constant, convergence), not by the
reference."""
import numpy as np
import pytest

from tests.helpers import make_system, rel_rms, water_lj_rows

pytestmark = pytest.mark.gpu


def _pme_system(lib, w, K, order, beta, rc=None):
    t = w.topology
    n = w.num_particles
    s = make_system(lib, n, w.box, charges=t.charges.reshape(-1), lj=water_lj_rows(w),
                    bonded=t.bonded_particles, scaling=t.scaling_particles,
                    cutoff=rc or 0.45 * float(np.min(w.box)), coulomb=lib.COUL_EWALD, beta=beta,
                    positions=w.positions)
    s.pme_config(K, order, beta)
    return s


@pytest.mark.parametrize("order,K", [(4, 32), (5, 32), (6, (28, 32, 36))])
def test_pme_matches_fp64_pme(lib, orc, order, K):
    from mdpy_gb300 import systems

    w = systems.water_box(900, 30.0, seed=0)
    t = w.topology
    q = t.charges.reshape(-1)
    beta = orc.ewald_beta(12.0, 1e-5)
    s = _pme_system(lib, w, K, order, beta, rc=12.0)
    s.compute_forces(lib.mask(lib.TERM_COUL_RECIP))
    f = s.get_forces()
    e, _ = s.get_energies()
    fp, ep = orc.pme(w.positions, w.box, q, beta, K, order)
    fx, ex = orc.ewald_exclusions(w.positions, w.box, q, t.bonded_particles, beta)
    e_self = orc.ewald_self(q, beta)
    e_ref = ep + ex + e_self + orc.ewald_net_charge(q, w.box, beta)
    assert rel_rms(f, fp + fx) <= 2e-5
    # the slot is a ~1e-3 residual of the self and exclusion terms (~20 units
    # each, opposite signs): compare on the scale of those components
    scale = abs(e_self) + abs(ex) + abs(ep)
    assert abs(e[lib.TERM_COUL_RECIP] - e_ref) <= 2e-7 * scale


def test_pme_non_cubic_box(lib, orc):
    from mdpy_gb300 import systems

    w = systems.water_box(1000, 30.0, seed=4)
    box = np.array([30.0, 33.0, 36.0])
    pos = w.positions * (box / 30.0)
    w.box = box
    w.positions = pos
    beta = 0.3
    K = (30, 32, 36)
    s = _pme_system(lib, w, K, 4, beta, rc=11.0)
    s.compute_forces(lib.mask(lib.TERM_COUL_RECIP))
    f = s.get_forces()
    q = w.topology.charges.reshape(-1)
    fp, _ = orc.pme(pos, box, q, beta, K, 4)
    fx, _ = orc.ewald_exclusions(pos, box, q, w.topology.bonded_particles, beta)
    assert rel_rms(f, fp + fx) <= 2e-5


def test_full_ewald_vs_direct_sum(lib, orc):
    """configs[0] electrostatics: 900 waters, 30 A, rc 12, tolerance 1e-5,
    32^3 grid, order 4 -- total Coulomb force error vs FP64 direct Ewald."""
    from mdpy_gb300 import systems

    w = systems.water_box(900, 30.0, seed=0)
    t = w.topology
    q = t.charges.reshape(-1)
    beta = orc.ewald_beta(12.0, 1e-5)
    s = _pme_system(lib, w, 32, 4, beta, rc=12.0)
    s.compute_forces(lib.mask(lib.TERM_COUL_REAL, lib.TERM_COUL_RECIP))
    f = s.get_forces()
    e, _ = s.get_energies()
    d = orc.ewald_direct(w.positions, w.box, q, t.bonded_particles, beta, 12.0)
    err = rel_rms(f, d["forces"])
    # the same PME in FP64: its error against the direct sum is the grid's
    # discretisation error (2.34e-4 at 32^3 / order 4 in the 30 A box)
    lj0 = np.zeros((w.num_particles, 4))
    f64 = (orc.nonbonded(w.positions, w.box, lj0, q, t.bonded_particles, t.scaling_particles,
                         12.0, lj=False, coulomb="ewald", beta=beta)[0]
           + orc.pme(w.positions, w.box, q, beta, 32, 4)[0]
           + orc.ewald_exclusions(w.positions, w.box, q, t.bonded_particles, beta)[0])
    err64 = rel_rms(f64, d["forces"])
    print("900 waters, 30 A, PME 32^3 o4: Coulomb force rel RMS vs direct Ewald %.3e "
          "(FP64 PME: %.3e)" % (err, err64))
    assert err64 < 2.4e-4
    # FP32 arithmetic adds at most 2e-5 (the GPU-vs-FP64-PME bar above)
    assert err < 2.5e-4
    e_gpu = e[lib.TERM_COUL_REAL] + e[lib.TERM_COUL_RECIP]
    scale = abs(d["e_self"]) + abs(d["e_excl"]) + abs(d["e_real"]) + abs(d["e_recip"])
    # PME discretisation error of the energy at 32^3 / order 4, on the scale of
    # the Ewald components (the total is a small residual of them)
    assert abs(e_gpu - d["energy"]) <= 2e-5 * scale


def test_pme_energy_translation_invariance(lib):
    """Shifting every atom by the same vector leaves the energy unchanged up
    to the grid discretisation (PME is not exactly translation invariant)."""
    from mdpy_gb300 import systems

    w = systems.water_box(900, 30.0, seed=0)
    s = _pme_system(lib, w, 32, 4, 0.27, rc=12.0)
    s.compute_forces(lib.mask(lib.TERM_COUL_REAL, lib.TERM_COUL_RECIP))
    e0, _ = s.get_energies()
    s.set_positions(w.positions + np.array([0.37, -1.21, 2.5]))
    s.compute_forces(lib.mask(lib.TERM_COUL_REAL, lib.TERM_COUL_RECIP))
    e1, _ = s.get_energies()
    tot0 = e0[lib.TERM_COUL_REAL] + e0[lib.TERM_COUL_RECIP]
    tot1 = e1[lib.TERM_COUL_REAL] + e1[lib.TERM_COUL_RECIP]
    # ~20-unit self/exclusion components cancel to ~0.017; the grid breaks
    # translation invariance at the 1e-6 level of the components
    assert abs(tot1 - tot0) <= 2e-6 * 40.0
