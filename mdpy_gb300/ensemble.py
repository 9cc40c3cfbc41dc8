"""Ensemble and State with mdpy's interface, backed by one device system.

mdpy's ``Ensemble`` (mdpy/ensemble.py:15-102) owns a ``State`` with host
positions/velocities and sums every constraint's host force array on each
``update()``.  Here the state lives in HBM (FP64 x and v in libmdg), one
``update()`` is one fused device evaluation of all bound terms, and host
arrays are produced only when a caller reads them.
"""
from __future__ import annotations

import os

import numpy as np

from . import _lib
from . import unit
from .error import (ArrayDimError, CellListPoorDefinedError, ConstraintConflictError,
                    PBCPoorDefinedError)


def _diag_box(pbc_matrix):
    pbc = np.asarray(pbc_matrix, dtype=np.float64)
    if pbc.shape != (3, 3):
        raise ArrayDimError("The pbc matrix should have shape [3, 3], while matrix %s is provided"
                            % (list(pbc.shape),))
    if np.linalg.det(pbc) == 0:
        raise PBCPoorDefinedError("PBC is poor defined. Two or more column vectors are linear "
                                  "corellated")
    if np.any(np.abs(pbc - np.diag(np.diag(pbc))) > 0):
        raise PBCPoorDefinedError("only orthorhombic (diagonal) pbc matrices are supported")
    return np.diag(pbc).copy()


class CellListView:
    """Stand-in for ``state.cell_list`` (mdpy/core/cell_list.py): the device
    code finds neighbours from cluster bounding boxes, so there is no cell
    list to maintain; this keeps the cut-off bookkeeping and the reference's
    validity check (``floor(L / rc) >= 2``, cell_list.py:56-72)."""

    def __init__(self, state, cutoff_radius=12.0):
        self._state = state
        # mdpy's default 12 A, reduced for boxes under 24 A instead of raising
        self._cutoff_radius = float(min(cutoff_radius, np.min(state.box) / 2.0))

    def set_cutoff_radius(self, cutoff_radius):
        rc = float(unit.check_quantity_value(cutoff_radius, "angstrom"))
        if rc == 0:
            raise CellListPoorDefinedError("Cutoff radius is poor defined, current value %.3f" % rc)
        if np.any(np.floor(self._state.box / rc) < 2):
            raise CellListPoorDefinedError("The cutoff_radius is too large to create cell list")
        self._cutoff_radius = rc

    @property
    def cutoff_radius(self):
        return self._cutoff_radius

    def update(self, positions=None):
        """No-op: the device re-sorts its clusters itself."""


class State:
    def __init__(self, ensemble, pbc_matrix):
        self._ensemble = ensemble
        self._num_particles = ensemble.topology.num_particles
        self._matrix_shape = [self._num_particles, 3]
        self.box = _diag_box(pbc_matrix)
        self._cell_list = CellListView(self)

    @property
    def _system(self):
        return self._ensemble.system

    def _check_matrix_shape(self, matrix):
        if not isinstance(matrix, np.ndarray):
            raise TypeError("Matrix should be numpy.ndarray, instead of %s" % type(matrix))
        if matrix.ndim != 2 or list(matrix.shape) != self._matrix_shape:
            raise ArrayDimError("The dimension of array should be %s, while array %s is provided"
                                % (self._matrix_shape, list(matrix.shape)))

    # -- mdpy State API ------------------------------------------------------
    def set_pbc_matrix(self, pbc_matrix):
        self.box = _diag_box(pbc_matrix)
        self._system.set_box(self.box)
        self._ensemble._invalidate()

    def set_positions(self, positions):
        self._check_matrix_shape(positions)
        self._system.set_positions(positions.astype(np.float64))
        self._ensemble._invalidate()

    def set_velocities(self, velocities):
        self._check_matrix_shape(velocities)
        self._system.set_velocities(velocities.astype(np.float64))
        self._ensemble._invalidate_kinetic()

    def set_velocities_to_temperature(self, temperature, seed=None):
        """Maxwell-Boltzmann velocities at ``temperature`` K.  (mdpy draws
        uniform velocities here, mdpy/core/state.py:67-81; a Gaussian is the
        correct distribution.)"""
        from .systems import maxwell_boltzmann

        rng = np.random.default_rng(seed)
        t = float(unit.check_quantity_value(temperature, "kelvin"))
        self.set_velocities(maxwell_boltzmann(rng, self._ensemble.topology.masses, t))

    @property
    def positions(self):
        """(N, 3) FP64 positions wrapped into [-L/2, L/2) (mdpy/utils/pbc.py:28-36)."""
        return self._system.get_positions()

    @property
    def velocities(self):
        return self._system.get_velocities()

    @property
    def matrix_shape(self):
        return self._matrix_shape

    @property
    def pbc_matrix(self):
        return np.diag(self.box)

    @property
    def pbc_inv(self):
        return np.diag(1.0 / self.box)

    @property
    def pbc_info(self):
        return self.pbc_matrix, self.pbc_inv

    @property
    def cell_list(self):
        return self._cell_list


class Ensemble:
    """mdpy.Ensemble on the GPU.  ``device`` selects the CUDA device
    (default: $MDG_DEVICE or 0)."""

    def __init__(self, topology, pbc_matrix, device=None, _system=None):
        if not topology.is_joined:
            topology.join()
        self._topology = topology
        box = _diag_box(pbc_matrix)
        if device is None:
            device = int(os.environ.get("MDG_DEVICE", "0"))
        # _system: a stand-in that records the set-up (batch members)
        self._system = _system if _system is not None else \
            _lib.System(topology.num_particles, box, device)
        self._system.set_masses(np.asarray(topology.masses, dtype=np.float64).reshape(-1))
        self._system.set_charges(np.asarray(topology.charges, dtype=np.float64).reshape(-1))
        self._system.set_exclusions(topology.bonded_particles, topology.scaling_particles)
        self._state = State(self, pbc_matrix)
        self._constraints = []
        self._forces = None
        self._potential_energy = 0.0
        self._kinetic_energy = 0.0
        self._energies = np.zeros(_lib.NUM_TERMS)
        self._fresh = False

    def __repr__(self):
        return "<mdpy_gb300.Ensemble object: %d constraints at %x>" % (len(self._constraints), id(self))

    __str__ = __repr__

    # -- constraints ---------------------------------------------------------
    def add_constraints(self, *constraints):
        for constraint in constraints:
            if constraint in self._constraints:
                raise ConstraintConflictError("%s has added twice to %s" % (constraint, self))
            self._constraints.append(constraint)
            constraint.bind_ensemble(self)
            if constraint.cutoff_radius > self.state.cell_list.cutoff_radius:
                self.state.cell_list.set_cutoff_radius(constraint.cutoff_radius)
        self._configure()

    def _configure(self):
        """Resolve the fused nonbonded kernel's settings from the bound constraints."""
        lj = [c for c in self._constraints if c._term_mask & _lib.mask(_lib.TERM_LJ)]
        coul = [c for c in self._constraints if c._term_mask & _lib.mask(_lib.TERM_COUL_REAL)]
        pme = [c for c in self._constraints if c._term_mask & _lib.mask(_lib.TERM_COUL_RECIP)]
        if len(lj) > 1 or len(coul) > 1 or len(pme) > 1:
            raise ConstraintConflictError("at most one LJ, one short-range Coulomb and one "
                                          "reciprocal-space constraint per ensemble")
        beta = None
        for c in coul + pme:
            b = getattr(c, "ewald_beta", None)
            if b is not None:
                if beta is not None and abs(b - beta) > 1e-12 * max(b, beta):
                    raise ValueError("real- and reciprocal-space constraints use different "
                                     "Ewald beta (%g vs %g)" % (beta, b))
                beta = b
        if lj or coul:
            cut = [c.cutoff_radius for c in lj + coul if getattr(c, "_uses_cutoff", True)]
            if len(set(round(x, 9) for x in cut)) > 1:
                raise ValueError("LJ and real-space Coulomb constraints need the same cutoff")
            # a bare-Coulomb-only ensemble has no cutoff; any valid value will do
            rc = cut[0] if cut else 0.49 * float(np.min(self._state.box))
            mode = coul[0]._coulomb_mode if coul else _lib.COUL_NONE
            sw = lj[0].switch_radius if lj else 0.0
            self._system.nonbonded_config(rc, sw or 0.0, bool(lj), mode, beta or 0.0)
        for c in pme:
            c._configure_system(beta)
        self._invalidate()

    @property
    def term_mask(self):
        m = 0
        for c in self._constraints:
            m |= c._term_mask
        return m

    # -- evaluation ----------------------------------------------------------
    def _invalidate(self):
        self._fresh = False
        self._forces = None
        for c in self._constraints:
            c._stale()

    def _invalidate_kinetic(self):
        self._kinetic_energy = self._system.kinetic_energy()

    def _read_back(self, mask, with_forces=True):
        e, ke = self._system.get_energies()
        self._energies = e
        self._potential_energy = float(sum(e[t] for t in range(_lib.NUM_TERMS) if mask >> t & 1))
        self._kinetic_energy = ke
        self._forces = self._system.get_forces() if with_forces else None
        for c in self._constraints:
            c._from_ensemble(e)
        self._fresh = True

    def update(self):
        """One fused device evaluation of every bound term (mdpy/ensemble.py:53-61)."""
        mask = self.term_mask
        self._system.compute_forces(mask)
        self._read_back(mask)
        self._kinetic_energy = self._system.kinetic_energy()

    def _after_integrate(self):
        self._read_back(self.term_mask, with_forces=False)
        for c in self._constraints:
            c._stale()

    # -- properties ------------------------------------------------------------
    @property
    def system(self):
        return self._system

    @property
    def topology(self):
        return self._topology

    @property
    def state(self):
        return self._state

    @property
    def forces(self):
        if self._forces is None:
            self._forces = self._system.get_forces()
        return self._forces

    @property
    def potential_energy(self):
        return self._potential_energy

    @property
    def kinetic_energy(self):
        return self._kinetic_energy

    @property
    def total_energy(self):
        return self._potential_energy + self._kinetic_energy

    @property
    def energies(self):
        """Per-term energies of the last evaluation, keyed by term name."""
        return dict(zip(_lib.TERM_NAMES, self._energies))

    @property
    def constraints(self):
        return self._constraints

    @property
    def num_constraints(self):
        return len(self._constraints)

    def _update_kinetic_energy(self):
        self._kinetic_energy = self._system.kinetic_energy()
