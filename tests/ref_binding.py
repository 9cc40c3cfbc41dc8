"""The binding a maintainer would add to mdpy to use libmdg from mdpy's own,
unchanged Ensemble: a subclass of the reference's Constraint
(mdpy/constraint/constraint.py:16-73) whose bind_ensemble builds a libmdg
system from the Ensemble's topology and whose update() evaluates LJ, Ewald
real space and PME on the GPU and hands the forces back as the (N, 3) host
array mdpy's Ensemble.update sums (mdpy/ensemble.py:53-61).

The reference is imported from its installed copy (baseline/_ref, made with
pip --target from the reference source tree) with the import stubs of
oracle/refshim for numba, h5py and MDAnalysis, which the reference imports
but this path does not use (numba.njit becomes the identity: the
reference's own NUMBA_DISABLE_JIT test mode).  Test infrastructure only.
"""
import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(REPO, "baseline", "_ref")


def reference_available():
    return os.path.isfile(os.path.join(REF, "mdpy", "__init__.py"))


def import_reference():
    """The unmodified reference package ``mdpy``."""
    for p in (REF, os.path.join(REPO, "oracle", "refshim")):
        if p not in sys.path:
            sys.path.insert(0, p)
    if not hasattr(np, "round_"):  # numpy 2 dropped it; mdpy/utils/pbc.py:42 calls it
        np.round_ = np.round
    import mdpy

    return mdpy


def binding_class():
    """GB300NonbondedConstraint, a subclass of the reference's Constraint."""
    import_reference()
    from mdpy.constraint import Constraint

    from mdpy_gb300 import _lib

    class GB300NonbondedConstraint(Constraint):
        def __init__(self, parameters, cutoff_radius=12, ewald_beta=None, pme_grid=None):
            super().__init__(parameters)
            self._cutoff_radius = cutoff_radius
            self._beta, self._grid = ewald_beta, pme_grid

        def bind_ensemble(self, ensemble):
            self._parent_ensemble = ensemble
            self._force_id = ensemble.constraints.index(self)
            t, box = ensemble.topology, np.diag(ensemble.state.pbc_matrix)
            self._sys = _lib.System(t.num_particles, box)
            self._sys.set_masses(t.masses)
            self._sys.set_charges(t.charges)
            self._sys.set_exclusions(t.bonded_particles, t.scaling_particles)
            rows = [list(self._parameters[p.particle_type]) for p in t.particles]
            self._sys.set_lj(np.array([r * 2 if len(r) == 2 else r for r in rows], float))
            coul = _lib.COUL_EWALD if self._beta else _lib.COUL_NONE
            self._sys.nonbonded_config(self._cutoff_radius, 0.0, True, coul, self._beta or 0.0)
            self._mask = _lib.mask(_lib.TERM_LJ, _lib.TERM_COUL_REAL)
            if self._grid:
                self._sys.pme_config(self._grid, 4, self._beta)
                self._mask |= _lib.mask(_lib.TERM_COUL_RECIP)

        def update(self):
            self._check_bound_state()
            self._sys.set_positions(self._parent_ensemble.state.positions)
            self._sys.compute_forces(self._mask)
            self._forces = self._sys.get_forces()
            e, _ = self._sys.get_energies()
            self._potential_energy = float(e[0] + e[1] + e[2])

    return GB300NonbondedConstraint


def reference_topology(sys_):
    """The reference's Topology (mdpy/core/topology.py) of a system made by
    mdpy_gb300.systems (not yet joined: the reference's Ensemble joins it)."""
    import_reference()
    from mdpy.core import Particle, Topology

    t = Topology()
    tt = sys_.topology
    t.add_particles([Particle(particle_id=i, particle_type=ty, particle_name=ty,
                              molecule_type="W", mass=float(m), charge=float(q))
                     for i, (ty, m, q) in enumerate(zip(tt.particle_types, tt.masses.reshape(-1),
                                                          tt.charges.reshape(-1)))])
    for b in tt.bonds:
        t.add_bond([int(b[0]), int(b[1])])
    for a in tt.angles:
        t.add_angle([int(a[0]), int(a[1]), int(a[2])])
    return t
