"""A small topology container with the attribute names of mdpy's
``Topology`` / ``Particle`` (mdpy/core/topology.py, mdpy/core/particle.py).

The GPU constraints and ensemble only read these attributes, so a joined
``mdpy.core.Topology`` works in place of this one.  Two ways to build it:

* particle by particle, exactly like the reference (``add_particles``,
  ``add_bond``, ``add_angle``, ``add_dihedral``, ``join``), used by the
  ported reference tests;
* :meth:`Topology.from_arrays`, which takes dense arrays directly and skips
  the per-particle Python objects -- needed for 10^5-10^6 atom systems.

Exclusion semantics follow ``Topology.join`` (mdpy/core/topology.py:59-80):
``bonded_particles`` holds 1-2 partners (``add_bond``) and 1-3 partners
(``add_angle``), ``scaling_particles`` holds 1-4 partners (``add_dihedral``),
both as dense ``(N, width)`` int arrays padded with -1.  The reference sizes
the 1-4 array with the 1-2/1-3 width (mdpy/core/topology.py:74-76), which
truncates or overflows when the widths differ; here each array gets its own
width.
"""
from __future__ import annotations

import numpy as np

from .error import ModifyJoinedTopologyError, ParticleConflictError, GeomtryDimError


class Particle:
    """Per-particle record with mdpy's ``Particle`` attribute names."""

    def __init__(self, particle_id=0, particle_type="", particle_name="",
                 matrix_id=None, molecule_id=None, molecule_type=None,
                 chain_id=None, mass=None, charge=None):
        self.particle_id = particle_id
        self.particle_type = particle_type
        self.particle_name = particle_name
        self.matrix_id = matrix_id
        self.molecule_id = molecule_id
        self.molecule_type = molecule_type
        self.chain_id = chain_id
        self.mass = 0.0 if mass is None else float(mass)
        self.charge = 0.0 if charge is None else float(charge)
        self.bonded_particles = []
        self.scaling_particles = []

    @property
    def num_bonded_particles(self):
        return len(self.bonded_particles)

    @property
    def num_scaling_particles(self):
        return len(self.scaling_particles)

    def change_matrix_id(self, matrix_id):
        self.matrix_id = matrix_id

    def add_bonded_particle(self, matrix_id):
        if matrix_id == self.matrix_id:
            raise ParticleConflictError("a particle can not be bonded to itself")
        if matrix_id in self.bonded_particles:
            raise ParticleConflictError(
                "particle %d is already bonded to particle %d" % (matrix_id, self.matrix_id))
        self.bonded_particles.append(matrix_id)

    def add_scaling_particle(self, matrix_id, factor=1):
        if matrix_id == self.matrix_id:
            raise ParticleConflictError("a particle can not be its own 1-4 partner")
        if matrix_id not in self.scaling_particles:
            self.scaling_particles.append(matrix_id)


def _dense(lists, n):
    width = max((len(x) for x in lists), default=0)
    out = np.full((n, max(width, 1)), -1, dtype=np.int32)
    for i, row in enumerate(lists):
        if row:
            out[i, :len(row)] = row
    return out


class Topology:
    def __init__(self):
        self._particles = []
        self._bonds, self._angles, self._dihedrals, self._impropers = [], [], [], []
        self._is_joined = False
        self._masses = self._charges = None
        self._bonded_particles = self._scaling_particles = None
        self._particle_types = None
        self._num_particles = 0

    # -- construction, reference style ------------------------------------
    def _check_joined(self):
        if self._is_joined:
            raise ModifyJoinedTopologyError("%s has been joined. No change can be made." % self)

    def add_particles(self, particles):
        self._check_joined()
        for p in particles:
            if not isinstance(p, Particle) and not hasattr(p, "particle_type"):
                raise TypeError("Particle expected, got %s" % type(p))
            p.change_matrix_id(self._num_particles)
            self._particles.append(p)
            self._num_particles += 1

    def _check_ids(self, ids, count, what):
        if len(ids) != count:
            raise GeomtryDimError("%s needs %d particles, got %d" % (what, count, len(ids)))
        for k, i in enumerate(ids):
            if i >= self._num_particles:
                raise ParticleConflictError("matrix id %d is out of range" % i)
            if i in ids[k + 1:]:
                raise ParticleConflictError("particle appears twice in a %s" % what)

    def add_bond(self, bond):
        self._check_joined()
        self._check_ids(bond, 2, "bond")
        p1, p2 = bond
        self._bonds.append(list(bond))
        self._particles[p1].add_bonded_particle(p2)
        self._particles[p2].add_bonded_particle(p1)

    def add_angle(self, angle):
        self._check_joined()
        self._check_ids(angle, 3, "angle")
        p1, _, p3 = angle
        self._angles.append(list(angle))
        self._particles[p1].add_bonded_particle(p3)
        self._particles[p3].add_bonded_particle(p1)

    def add_dihedral(self, dihedral, scaling_factor=1):
        self._check_joined()
        self._check_ids(dihedral, 4, "dihedral")
        p1, _, _, p4 = dihedral
        self._dihedrals.append(list(dihedral))
        self._particles[p1].add_scaling_particle(p4, scaling_factor)
        self._particles[p4].add_scaling_particle(p1, scaling_factor)

    def add_improper(self, improper):
        self._check_joined()
        self._check_ids(improper, 4, "improper")
        self._impropers.append(list(improper))

    def join(self):
        n = self._num_particles
        self._masses = np.array([[p.mass] for p in self._particles], dtype=np.float64).reshape(n, 1)
        self._charges = np.array([[p.charge] for p in self._particles], dtype=np.float64).reshape(n, 1)
        self._bonded_particles = _dense([p.bonded_particles for p in self._particles], n)
        self._scaling_particles = _dense([p.scaling_particles for p in self._particles], n)
        self._particle_types = [p.particle_type for p in self._particles]
        self._is_joined = True

    # -- construction from dense arrays -------------------------------------
    @classmethod
    def from_arrays(cls, particle_types, masses, charges, bonds=(), angles=(),
                    dihedrals=(), impropers=(), bonded_particles=None,
                    scaling_particles=None):
        """Build a joined topology without per-particle objects.

        When ``bonded_particles`` / ``scaling_particles`` are not given they
        are derived as ``join`` would: 1-2 from bonds, 1-3 from angle ends,
        1-4 from dihedral ends, in that insertion order.
        """
        t = cls()
        n = len(masses)
        t._num_particles = n
        t._particle_types = list(particle_types)
        t._masses = np.asarray(masses, dtype=np.float64).reshape(n, 1)
        t._charges = np.asarray(charges, dtype=np.float64).reshape(n, 1)
        t._bonds = np.asarray(bonds, dtype=np.int64).reshape(-1, 2)
        t._angles = np.asarray(angles, dtype=np.int64).reshape(-1, 3)
        t._dihedrals = np.asarray(dihedrals, dtype=np.int64).reshape(-1, 4)
        t._impropers = np.asarray(impropers, dtype=np.int64).reshape(-1, 4)
        if bonded_particles is None:
            bonded_particles = _pairs_to_dense(
                n, [t._bonds[:, [0, 1]], t._angles[:, [0, 2]]])
        if scaling_particles is None:
            scaling_particles = _pairs_to_dense(n, [t._dihedrals[:, [0, 3]]])
        t._bonded_particles = np.asarray(bonded_particles, dtype=np.int32)
        t._scaling_particles = np.asarray(scaling_particles, dtype=np.int32)
        t._is_joined = True
        return t

    # -- attributes read by constraints / ensemble -------------------------
    @property
    def is_joined(self):
        return self._is_joined

    @property
    def particles(self):
        return self._particles

    @property
    def particle_types(self):
        if self._particle_types is None:
            return [p.particle_type for p in self._particles]
        return self._particle_types

    @property
    def num_particles(self):
        return self._num_particles

    @property
    def masses(self):
        return self._masses

    @property
    def charges(self):
        return self._charges

    @property
    def bonded_particles(self):
        return self._bonded_particles

    @property
    def scaling_particles(self):
        return self._scaling_particles

    @property
    def bonds(self):
        return self._bonds

    @property
    def angles(self):
        return self._angles

    @property
    def dihedrals(self):
        return self._dihedrals

    @property
    def impropers(self):
        return self._impropers

    @property
    def num_bonds(self):
        return len(self._bonds)

    @property
    def num_angles(self):
        return len(self._angles)

    @property
    def num_dihedrals(self):
        return len(self._dihedrals)

    @property
    def num_impropers(self):
        return len(self._impropers)

    def __repr__(self):
        return "<mdpy_gb300.Topology: %d particles>" % self._num_particles


def _pairs_to_dense(n, pair_arrays):
    """Symmetric partner lists (insertion order, duplicates dropped) as a
    dense -1 padded array."""
    pairs = [np.asarray(p, dtype=np.int64).reshape(-1, 2) for p in pair_arrays if len(p)]
    if not pairs:
        return np.full((n, 1), -1, dtype=np.int32)
    allp = np.concatenate(pairs, axis=0)
    # directed edges in insertion order: (a->b), (b->a) for each pair
    src = np.stack([allp[:, 0], allp[:, 1]], axis=1).reshape(-1)
    dst = np.stack([allp[:, 1], allp[:, 0]], axis=1).reshape(-1)
    key = src * n + dst
    _, first = np.unique(key, return_index=True)
    first.sort()
    src, dst = src[first], dst[first]
    order = np.argsort(src, kind="stable")
    src, dst = src[order], dst[order]
    counts = np.bincount(src, minlength=n)
    width = max(int(counts.max()), 1)
    out = np.full((n, width), -1, dtype=np.int32)
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    slot = np.arange(len(src)) - starts[src]
    out[src, slot] = dst
    return out
