"""Seeded synthetic systems for tests and the benchmark.

No dataset is involved: every workload is generated here from a seed.

* :func:`water_box` -- flexible three-site water (O, H, H) on a jittered cubic
  lattice.  Lattice spacing L / ceil(Nw^(1/3)), O jitter U(+-0.3 A), random
  orientation, r0 = 0.9572 A, theta0 = 104.52 deg, charges O -0.834 /
  H +0.417, LJ on O only (eps 0.1521 kcal/mol, sigma 3.1507 A), bonds
  k = 450 kcal/mol/A^2, angle k = 55 kcal/mol/rad^2, masses 15.9994 / 1.008.
* :func:`chain_in_water` -- the water box plus a 500-bead chain with bonds,
  angles and dihedrals (k U(0.2, 2) kcal/mol, multiplicity 1-3, phase 0 or
  180 deg), bead charges U(+-0.5) e corrected to a net-zero sum; waters
  overlapping the chain are removed.
* :func:`water_box_batch` -- many independent water boxes of uneven size.

Parameters are returned in mdpy's dictionary format (what
``CharmmTopparParser(...).parameters`` yields, in internal units:
mdpy/io/charmm_toppar_parser.py:208-221), so the constraints consume them
exactly as the reference's constraints would.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import unit
from .topology import Topology

WATER_R0 = 0.9572
WATER_THETA0_DEG = 104.52
O_MASS, H_MASS = 15.9994, 1.008
O_CHARGE, H_CHARGE = -0.834, 0.417
O_EPS_KCAL, O_SIGMA = 0.1521, 3.1507
BOND_K_KCAL = 450.0
ANGLE_K_KCAL = 55.0
DENSITY_ATOMS_PER_A3 = 0.1


@dataclass
class SyntheticSystem:
    name: str
    box: np.ndarray                  # (3,) orthorhombic edge lengths, A
    positions: np.ndarray            # (N, 3) float64, A
    velocities: np.ndarray           # (N, 3) float64, A/fs
    topology: Topology
    parameters: dict                 # mdpy-format parameter dictionaries
    dihedral_parameters: np.ndarray = None   # (nd, 3): k, n, delta per dihedral
    settings: dict = field(default_factory=dict)

    @property
    def num_particles(self):
        return self.positions.shape[0]

    @property
    def pbc_matrix(self):
        return np.diag(self.box.astype(np.float64))


def water_parameters():
    kcal = unit.KCAL_PER_MOL
    return {
        "nonbonded": {"OT": [O_EPS_KCAL * kcal, O_SIGMA], "HT": [0.0, 1.0]},
        "bond": {"OT-HT": [BOND_K_KCAL * kcal, WATER_R0], "HT-OT": [BOND_K_KCAL * kcal, WATER_R0]},
        "angle": {"HT-OT-HT": [ANGLE_K_KCAL * kcal, math.radians(WATER_THETA0_DEG), 0.0, 0.0]},
        "dihedral": {},
        "improper": {},
    }


def _random_rotations(rng, n):
    """Uniform random rotation matrices from unit quaternions."""
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
    ], axis=1)


def maxwell_boltzmann(rng, masses, temperature):
    """Velocities (A/fs) drawn from Maxwell-Boltzmann at ``temperature`` K,
    net momentum removed."""
    m = np.asarray(masses, dtype=np.float64).reshape(-1, 1)
    sd = np.sqrt(unit.KB * temperature / m)
    v = rng.normal(size=(m.shape[0], 3)) * sd
    v -= (m * v).sum(0) / m.sum()
    return v


def _water_coordinates(rng, n_waters, box, jitter=0.3):
    box = np.asarray(box, dtype=np.float64)
    per_axis = int(math.ceil(n_waters ** (1.0 / 3.0) - 1e-9))
    spacing = box / per_axis
    grid = np.stack(np.meshgrid(*[np.arange(per_axis)] * 3, indexing="ij"), -1).reshape(-1, 3)
    sites = rng.permutation(grid.shape[0])[:n_waters]
    o = (grid[sites] + 0.5) * spacing + rng.uniform(-jitter, jitter, size=(n_waters, 3))
    half = math.radians(WATER_THETA0_DEG) / 2
    local = np.array([[0.0, 0.0, 0.0],
                      [WATER_R0 * math.sin(half), 0.0, WATER_R0 * math.cos(half)],
                      [-WATER_R0 * math.sin(half), 0.0, WATER_R0 * math.cos(half)]])
    rot = _random_rotations(rng, n_waters)
    xyz = o[:, None, :] + np.einsum("nij,aj->nai", rot, local)
    xyz -= box / 2            # reference convention: wrapped into [-L/2, L/2)
    xyz -= box * np.round(xyz / box)
    return xyz.reshape(-1, 3)


def _water_topology_arrays(n_waters, offset=0):
    base = offset + 3 * np.arange(n_waters)
    bonds = np.stack([np.stack([base, base + 1], 1), np.stack([base, base + 2], 1)], 1).reshape(-1, 2)
    angles = np.stack([base + 1, base, base + 2], 1)
    return bonds, angles


def water_box(n_waters=900, box=30.0, seed=0, temperature=300.0, jitter=0.3):
    """``n_waters`` flexible waters in a cubic box of edge ``box`` A."""
    rng = np.random.default_rng(seed)
    box3 = np.full(3, float(box))
    pos = _water_coordinates(rng, n_waters, box3, jitter)
    types = ["OT", "HT", "HT"] * n_waters
    masses = np.tile([O_MASS, H_MASS, H_MASS], n_waters)
    charges = np.tile([O_CHARGE, H_CHARGE, H_CHARGE], n_waters)
    bonds, angles = _water_topology_arrays(n_waters)
    topo = Topology.from_arrays(types, masses, charges, bonds=bonds, angles=angles)
    vel = maxwell_boltzmann(rng, masses, temperature)
    return SyntheticSystem("water%d" % n_waters, box3, pos, vel, topo, water_parameters(),
                           settings={"temperature": temperature})


def chain_in_water(n_waters=30000, box=96.5, n_beads=500, seed=0, temperature=300.0,
                   clearance=3.0):
    """Water box with a solvated synthetic chain (prepended as atoms 0..n_beads-1)."""
    from scipy.spatial import cKDTree

    rng = np.random.default_rng(seed)
    box3 = np.full(3, float(box))
    wat = _water_coordinates(rng, n_waters, box3).reshape(n_waters, 3, 3)
    # self-avoiding chain: bond 1.53 A, angle 112 deg, random torsion
    bond, ang = 1.53, math.radians(112.0)
    beads = [np.zeros(3), np.array([bond, 0.0, 0.0])]
    d = np.array([math.cos(math.pi - ang), math.sin(math.pi - ang), 0.0])
    beads.append(beads[-1] + bond * d)
    while len(beads) < n_beads:
        b1, b2, b3 = beads[-3], beads[-2], beads[-1]
        for _ in range(200):
            phi = rng.uniform(0, 2 * math.pi)
            bc = (b3 - b2) / np.linalg.norm(b3 - b2)
            nrm = np.cross(b2 - b1, bc)
            nrm /= np.linalg.norm(nrm)
            m = np.cross(nrm, bc)
            dl = np.array([-bond * math.cos(ang), bond * math.sin(ang) * math.cos(phi),
                           bond * math.sin(ang) * math.sin(phi)])
            new = b3 + dl[0] * bc + dl[1] * m + dl[2] * nrm
            prev = np.asarray(beads[:-3])
            if len(prev) == 0:
                break
            dd = new - prev
            dd -= box3 * np.round(dd / box3)
            if np.min(np.einsum("ij,ij->i", dd, dd)) >= 9.0:
                break
        beads.append(new)
    chain = np.asarray(beads)
    chain -= chain.mean(0)
    chain -= box3 * np.round(chain / box3)
    tree = cKDTree(np.mod(chain, box3), boxsize=box3)
    close = tree.query_ball_point(np.mod(wat.reshape(-1, 3), box3), r=clearance)
    hit = np.array([len(c) > 0 for c in close]).reshape(n_waters, 3).any(1)
    wat = wat[~hit]
    nw = wat.shape[0]
    pos = np.concatenate([chain, wat.reshape(-1, 3)], 0)
    q_beads = rng.uniform(-0.5, 0.5, n_beads)
    q_beads -= q_beads.mean()
    types = ["CB"] * n_beads + ["OT", "HT", "HT"] * nw
    masses = np.concatenate([np.full(n_beads, 14.027), np.tile([O_MASS, H_MASS, H_MASS], nw)])
    charges = np.concatenate([q_beads, np.tile([O_CHARGE, H_CHARGE, H_CHARGE], nw)])
    i = np.arange(n_beads)
    cbonds = np.stack([i[:-1], i[1:]], 1)
    cangles = np.stack([i[:-2], i[1:-1], i[2:]], 1)
    cdihed = np.stack([i[:-3], i[1:-2], i[2:-1], i[3:]], 1)
    wbonds, wangles = _water_topology_arrays(nw, offset=n_beads)
    topo = Topology.from_arrays(types, masses, charges,
                                bonds=np.concatenate([cbonds, wbonds]),
                                angles=np.concatenate([cangles, wangles]),
                                dihedrals=cdihed)
    kcal = unit.KCAL_PER_MOL
    params = water_parameters()
    params["nonbonded"]["CB"] = [0.0914 * kcal, 3.6072]
    params["bond"]["CB-CB"] = [300.0 * kcal, 1.53]
    params["angle"]["CB-CB-CB"] = [60.0 * kcal, math.radians(112.0), 0.0, 0.0]
    nd = cdihed.shape[0]
    dih = np.stack([rng.uniform(0.2, 2.0, nd) * kcal,
                    rng.integers(1, 4, nd).astype(np.float64),
                    np.where(rng.random(nd) < 0.5, 0.0, math.pi)], 1)
    vel = maxwell_boltzmann(rng, masses, temperature)
    return SyntheticSystem("chain%d_water%d" % (n_beads, nw), box3, pos, vel, topo, params,
                           dihedral_parameters=dih, settings={"temperature": temperature})


def water_box_batch(n_boxes=256, n_min=1500, n_max=12000, seed=0, temperature=300.0):
    """Independent water boxes, atom counts log-uniform in [n_min, n_max],
    edge L_i = (N_i / rho)^(1/3) with rho = 0.1 atoms/A^3."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(math.log(n_min), math.log(n_max), n_boxes))
    systems = []
    for b, n_atoms in enumerate(sizes):
        nw = max(int(round(n_atoms / 3.0)), 1)
        edge = (3 * nw / DENSITY_ATOMS_PER_A3) ** (1.0 / 3.0)
        systems.append(water_box(nw, edge, seed=seed * 100003 + b + 1, temperature=temperature))
    return systems


def fft_friendly(n, lo=8, hi=512):
    """Smallest 2^a 3^b 5^c >= n within [lo, hi]."""
    best = None
    for a in range(0, 10):
        for b in range(0, 7):
            for c in range(0, 5):
                v = (2 ** a) * (3 ** b) * (5 ** c)
                if v >= max(n, lo) and v <= hi and (best is None or v < best):
                    best = v
    return best
