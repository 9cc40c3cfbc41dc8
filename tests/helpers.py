"""Shared builders for the tests (no GPU work at import time)."""
import numpy as np

# Tolerance on totals the reference accumulates in float32 over 10^5-10^6
# terms (its forces are per-atom sums of ~10^3 terms and stay at ~1e-6):
# the reference's own rounding error in such a total reaches ~1e-4.
REF_E_TOL = 2e-4


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


def half_box_tie_atoms(pos, box, tol=2e-6):
    """Atoms of pairs whose separation along some axis lies within ``tol`` of
    half the box: there the minimum image is a tie that float32 and FP64
    (or two rounding rules) may break differently.  All pairs, O(N^2)."""
    pos = np.asarray(pos, dtype=np.float64)
    box = np.broadcast_to(np.asarray(box, float), (3,))
    atoms = set()
    for k in range(3):
        d = np.abs(pos[None, :, k] - pos[:, None, k])
        d = np.abs(d - box[k] * np.round(d / box[k]))
        i, j = np.nonzero(np.abs(d - box[k] / 2) < tol)
        atoms.update(i.tolist())
        atoms.update(j.tolist())
    return np.array(sorted(atoms), dtype=np.int64)


def rel_rms_excluding(a, b, drop):
    keep = np.ones(len(a), dtype=bool)
    keep[np.asarray(drop, dtype=np.int64)] = False
    return rel_rms(np.asarray(a)[keep], np.asarray(b)[keep])


def pair_keys(pairs):
    """Sorted unique int64 keys (lo << 32 | hi) of an (m, 2) pair array: set
    comparisons of millions of pairs without Python tuples."""
    p = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    lo, hi = np.minimum(p[:, 0], p[:, 1]), np.maximum(p[:, 0], p[:, 1])
    return np.unique((lo << 32) | hi)


def keys_to_pairs(keys):
    keys = np.asarray(keys, dtype=np.int64)
    return np.stack([keys >> 32, keys & 0xFFFFFFFF], axis=1)


_REF32_CACHE = {}


def ref32_keys(orc, positions, box, rc, exclusions=None):
    """pair_keys of the pair set the reference's own float32 pair test gives
    over all pairs (oracle ref_within32), from positions as mdg_get_positions
    reports them (wrapped into [-L/2, L/2) as mdpy wraps) rounded to float32.
    Results are kept per input (tests that differ only in launch shape see
    the same positions)."""
    import hashlib

    pos32 = np.ascontiguousarray(np.asarray(positions, dtype=np.float64).astype(np.float32))
    n = pos32.shape[0]
    diag = np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)).astype(np.float32)
    ex = (np.full((n, 1), -1, dtype=np.int32) if exclusions is None
          else np.ascontiguousarray(exclusions, dtype=np.int32))
    h = hashlib.sha1()
    for arr in (pos32, diag, np.float64(rc), ex):
        h.update(np.ascontiguousarray(arr).tobytes())
    key = h.hexdigest()
    if key not in _REF32_CACHE:
        if len(_REF32_CACHE) > 8:
            _REF32_CACHE.clear()
        _REF32_CACHE[key] = pair_keys(orc.pairs_bruteforce_ref32(pos32, diag, float(rc), ex))
    return _REF32_CACHE[key]


def ref32_pairs(orc, positions, box, rc, exclusions=None):
    """The same pair set as ref32_keys, as a set of (i, j) tuples, i < j."""
    k = ref32_keys(orc, positions, box, rc, exclusions)
    return set(zip((k >> 32).tolist(), (k & 0xFFFFFFFF).tolist()))


_BAND_CACHE = {}


def cutoff_band(orc, positions, box, rc, width=1e-4):
    """Pairs whose FP64 minimum-image distance lies within ``width`` A of rc:
    where float32 rounding decides which side a pair falls.  Results are kept
    per input, as for ref32_keys."""
    import hashlib

    pos = np.ascontiguousarray(positions, dtype=np.float64)
    h = hashlib.sha1()
    for arr in (pos, np.asarray(box, dtype=np.float64), np.float64(rc), np.float64(width)):
        h.update(np.ascontiguousarray(arr).tobytes())
    key = h.hexdigest()
    if key not in _BAND_CACHE:
        if len(_BAND_CACHE) > 8:
            _BAND_CACHE.clear()
        outer = np.asarray(orc.pairs_bruteforce(pos, box, rc + width), dtype=np.int64).reshape(-1, 2)
        r = min_image_r(pos, box, outer)
        band = outer[r > rc - width]
        _BAND_CACHE[key] = pairs_to_set(band) if len(band) else set()
    return _BAND_CACHE[key]
