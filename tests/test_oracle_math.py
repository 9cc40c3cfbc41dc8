"""Pins of the oracle's own mathematics (CPU).  Ewald, PME, switching and
the exact torsion gradient have no reference implementation in mdpy, so they
are pinned here by known answers and finite differences."""
import math

import numpy as np
import pytest


def _fd(fn, x, k, h=1e-5):
    g = np.zeros(3)
    for d in range(3):
        xp, xm = x.copy(), x.copy()
        xp[k, d] += h
        xm[k, d] -= h
        g[d] = -(fn(xp) - fn(xm)) / (2 * h)
    return g


def test_madelung_constant_rock_salt(orc):
    """Direct Ewald energy of NaCl (unit charges, nearest distance 1): -M per ion pair,
    M = 1.747564594633."""
    n, a = 4, 2.0
    idx = np.stack(np.meshgrid(*[np.arange(2 * n)] * 3, indexing="ij"), -1).reshape(-1, 3)
    pos = idx * (a / 2) + 0.01
    q = np.where(idx.sum(1) % 2 == 0, 1.0, -1.0)
    box = np.full(3, n * a)
    rc = n * a / 2 * 0.999
    r = orc.ewald_direct(pos, box, q, np.full((len(q), 1), -1), 5.5 / rc, rc, eps=1e-16, kcoul=1.0)
    assert -r["energy"] * 2 * (a / 2) / len(q) == pytest.approx(1.747564594633, abs=1e-9)


def test_ewald_two_charges_approach_coulomb(orc):
    """Two opposite charges 3 A apart in boxes of growing size: the Ewald
    energy approaches the bare Coulomb pair energy (the periodic images'
    dipole correction falls off as 1/L^3)."""
    errs = []
    for L in (40.0, 80.0):
        pos = np.array([[0.0, 0.0, 0.0], [3.0, 0.0, 0.0]]) + L / 2
        q = np.array([1.0, -1.0])
        beta = 5.0 / (0.45 * L)
        r = orc.ewald_direct(pos, np.full(3, L), q, np.full((2, 1), -1), beta, 0.45 * L, eps=1e-16,
                             kcoul=1.0)
        errs.append(abs(r["energy"] - (-1.0 / 3.0)))
    assert errs[1] < errs[0] / 6 and errs[1] < 1e-4


def test_pme_converges_to_direct_ewald(orc):
    from mdpy_gb300 import systems

    w = systems.water_box(100, 14.5, seed=1)
    q = w.topology.charges.reshape(-1)
    beta = 0.35
    fr, er = orc.ewald_recip(w.positions, w.box, q, beta, orc.ewald_kmax(w.box, beta, 1e-14))
    prev = None
    for K in (16, 24, 32, 48):
        fp, ep = orc.pme(w.positions, w.box, q, beta, K, 4)
        err = np.sqrt(((fp - fr) ** 2).sum() / (fr ** 2).sum())
        if prev is not None:
            assert err < prev
        prev = err
    assert prev < 1e-4
    assert ep == pytest.approx(er, rel=1e-4)
    f6, e6 = orc.pme(w.positions, w.box, q, beta, 32, 6)
    assert np.sqrt(((f6 - fr) ** 2).sum() / (fr ** 2).sum()) < 5e-5


def test_nonbonded_forces_are_gradients(orc):
    from mdpy_gb300 import systems

    w = systems.water_box(64, 13.0, seed=3)
    t = w.topology
    n = w.num_particles
    p = w.parameters["nonbonded"]
    lj = np.array([[p[ty][0], p[ty][1], 0.7 * p[ty][0], 0.9 * p[ty][1]] for ty in t.particle_types])
    x = w.positions.copy()
    for kw in (dict(coulomb="ewald", beta=0.35, switch=5.0), dict(coulomb="bare")):
        def energy(y):
            _, e = orc.nonbonded(y, w.box, lj, t.charges, t.bonded_particles, t.scaling_particles,
                                 6.4, **kw)
            return e["lj"] + e["coulomb"]
        f, _ = orc.nonbonded(x, w.box, lj, t.charges, t.bonded_particles, t.scaling_particles,
                             6.4, **kw)
        for k in (0, 7, n - 1):
            assert f[k] == pytest.approx(_fd(energy, x, k, 1e-5), rel=2e-4, abs=1e-9)


def test_switch_is_continuous(orc):
    """CHARMM switch: energy and force go to zero continuously at rc."""
    lj = np.array([[1e-4, 3.0, 1e-4, 3.0]] * 2)
    none = np.full((2, 1), -1)
    box = np.full(3, 40.0)
    e = []
    for r in (11.999, 11.9999, 12.0):
        pos = np.array([[0.0, 0, 0], [r, 0, 0]])
        f, en = orc.nonbonded(pos, box, lj, np.zeros(2), none, none, 12.0, switch=10.0)
        e.append((en["lj"], f[1, 0]))
    assert abs(e[0][0]) < 1e-12 and abs(e[1][0]) < 1e-14
    assert abs(e[0][1]) < 1e-8 and abs(e[2][1]) == 0


def test_bonded_forces_are_gradients(orc):
    rng = np.random.default_rng(0)
    x = rng.normal(size=(8, 3)) * 1.2
    cases = [
        (orc.bonds, np.array([[0, 1], [2, 5]]), np.array([[0.2, 1.1], [0.1, 1.4]])),
        (orc.angles, np.array([[0, 1, 2], [3, 4, 5]]), np.array([[0.02, 1.9, 0.01, 2.0], [0.03, 2.1, 0, 0]])),
        (orc.dihedrals, np.array([[0, 1, 2, 3], [4, 5, 6, 7]]), np.array([[0.001, 2, math.pi], [0.002, 3, 0.0]])),
        (orc.impropers, np.array([[0, 1, 2, 3]]), np.array([[0.02, 0.3]])),
    ]
    for fn, idx, prm in cases:
        f, _ = fn(x, 50.0, idx, prm)
        for k in range(8):
            g = _fd(lambda y: fn(y, 50.0, idx, prm)[1], x, k)
            assert f[k] == pytest.approx(g, rel=1e-5, abs=1e-10)


def test_philox_known_answers(orc):
    """Philox4x32-10 known-answer vectors published with Random123
    (Salmon et al., SC'11)."""
    assert orc.philox4x32([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert orc.philox4x32([0xffffffff] * 4, [0xffffffff] * 2) == \
        [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert orc.philox4x32([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                          [0xa4093822, 0x299f31d0]) == [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_langevin_noise_statistics(orc):
    g = orc.langevin_noise(20000, 42, 7).astype(np.float64)
    assert abs(g.mean()) < 0.02
    assert abs(g.std() - 1.0) < 0.02
    assert not np.array_equal(g, orc.langevin_noise(20000, 42, 8))


def test_gjf_reduces_to_velocity_verlet(orc):
    rng = np.random.default_rng(1)
    x, v, f = rng.normal(size=(5, 3)), rng.normal(size=(5, 3)), rng.normal(size=(5, 3))
    m = rng.uniform(1, 16, size=5)
    f1 = rng.normal(size=(5, 3))
    a = orc.langevin_gjf_step(x, v, f, m, 0.5, 300.0, 0.0, np.zeros((5, 3)), lambda y: f1)
    b = orc.verlet_step(x, v, f, m, 0.5, lambda y: f1)
    assert np.allclose(a[0], b[0], rtol=0, atol=1e-15) and np.allclose(a[1], b[1], rtol=0, atol=1e-15)
