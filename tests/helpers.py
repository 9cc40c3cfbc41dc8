"""Shared builders for the tests (no GPU work at import time)."""
import numpy as np


def rel_rms(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.sqrt(np.sum((a - b) ** 2) / max(np.sum(b ** 2), 1e-300)))


def water_lj_rows(sysobj):
    p = sysobj.parameters["nonbonded"]
    return np.array([[p[t][0], p[t][1], p[t][0], p[t][1]] for t in sysobj.topology.particle_types])


def water_bonded(sysobj):
    t = sysobj.topology
    kb = np.array([sysobj.parameters["bond"]["OT-HT"]] * t.num_bonds)
    ka = np.array([sysobj.parameters["angle"]["HT-OT-HT"]] * t.num_angles)
    return kb, ka


def make_system(lib, n, box, masses=None, charges=None, lj=None, bonded=None, scaling=None,
                cutoff=None, switch=0.0, lj_on=True, coulomb=0, beta=0.0, positions=None,
                velocities=None):
    s = lib.System(n, box)
    if masses is not None:
        s.set_masses(masses)
    if charges is not None:
        s.set_charges(charges)
    if lj is not None:
        s.set_lj(lj)
    if bonded is not None or scaling is not None:
        b = np.full((n, 1), -1) if bonded is None else bonded
        c = np.full((n, 1), -1) if scaling is None else scaling
        s.set_exclusions(b, c)
    if cutoff is not None:
        s.nonbonded_config(cutoff, switch, lj_on, coulomb, beta)
    if positions is not None:
        s.set_positions(positions)
    if velocities is not None:
        s.set_velocities(velocities)
    return s


def pairs_to_set(pairs):
    p = np.asarray(pairs, dtype=np.int64)
    lo, hi = np.minimum(p[:, 0], p[:, 1]), np.maximum(p[:, 0], p[:, 1])
    return set(zip(lo.tolist(), hi.tolist()))


def min_image_r(pos, box, pairs):
    pos = np.asarray(pos, dtype=np.float64)
    box = np.broadcast_to(np.asarray(box, float), (3,))
    p = np.asarray(list(pairs), dtype=np.int64).reshape(-1, 2)
    d = pos[p[:, 1]] - pos[p[:, 0]]
    d -= box * np.round(d / box)
    return np.sqrt((d ** 2).sum(1))
