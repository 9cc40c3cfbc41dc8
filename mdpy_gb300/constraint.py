"""Constraints with mdpy's interface (mdpy/constraint/constraint.py:16-73).

A constraint binds to an ensemble (``bind_ensemble``), and ``update()`` fills
``forces`` ((N, 3) FP64) and ``potential_energy``.  Each class names the
force terms it owns; the ensemble fuses all bound terms into one device
evaluation, and a constraint evaluated alone runs only its own terms.

Reference counterparts:

* ``CharmmNonbondedConstraint`` -- mdpy/constraint/charmm_nonbonded_constraint.py
  (LJ, hard cutoff; optional CHARMM switch)
* ``ElectrostaticConstraint``   -- mdpy/constraint/electrostatic_constraint.py
  (bare Coulomb over all pairs, minimum image)
* ``NonbondedConstraint``       -- LJ + Ewald real-space erfc in one kernel;
  no reference counterpart (mdpy has no Ewald)
* ``PMEConstraint``             -- smooth PME reciprocal space + self, net
  charge and exclusion terms; mdpy names PME (mdpy/constraint/__init__.py:22)
  but has no implementation
* ``CharmmBond/Angle/Dihedral/ImproperConstraint`` -- mdpy/constraint/charmm_*.py
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib
from . import unit
from .error import NonBoundedError, ParameterPoorDefinedError


def ewald_beta_from_error(cutoff, ewald_error):
    """Splitting parameter with erfc(beta rc) ~ ewald_error:
    beta = sqrt(-ln(2 err)) / rc."""
    return math.sqrt(-math.log(2.0 * ewald_error)) / cutoff


class Constraint:
    _term_mask = 0
    _uses_cutoff = True

    def __init__(self, parameters=None, force_id: int = 0, force_group: int = 0):
        self._parameters = parameters
        self._force_id = force_id
        self._force_group = force_group
        self._parent_ensemble = None
        self._forces = None
        self._potential_energy = None
        self._cutoff_radius = 0.0

    def __repr__(self):
        return "<mdpy_gb300.constraint.%s object>" % type(self).__name__

    __str__ = __repr__

    def __eq__(self, o):
        return id(self) == id(o)

    __hash__ = object.__hash__

    def bind_ensemble(self, ensemble):
        self._parent_ensemble = ensemble
        self._force_id = ensemble.constraints.index(self)
        self._bind(ensemble.system, ensemble.topology)

    def _bind(self, system, topology):
        raise NotImplementedError("subclasses bind their parameters to the device system")

    def _check_bound_state(self):
        if self._parent_ensemble is None:
            raise NonBoundedError("%s has not been bounded to any Ensemble instance" % self)

    def update(self):
        """Evaluate this constraint's terms alone."""
        self._check_bound_state()
        system = self._parent_ensemble.system
        system.compute_forces(self._term_mask)
        self._forces = system.get_forces()
        e, _ = system.get_energies()
        self._from_ensemble(e)

    # called by the ensemble after a fused evaluation
    def _from_ensemble(self, energies):
        self._potential_energy = float(sum(energies[t] for t in range(_lib.NUM_TERMS)
                                           if self._term_mask >> t & 1))

    def _stale(self):
        self._forces = None

    @property
    def force_id(self):
        return self._force_id

    @property
    def force_group(self):
        return self._force_group

    @property
    def parent_ensemble(self):
        return self._parent_ensemble

    @property
    def forces(self):
        if self._forces is None and self._parent_ensemble is not None \
                and self._potential_energy is not None:
            self.update()
        return self._forces

    @property
    def potential_energy(self):
        return self._potential_energy

    def set_cutoff_radius(self, val):
        self._cutoff_radius = float(unit.check_quantity_value(val, "angstrom"))

    @property
    def cutoff_radius(self):
        return self._cutoff_radius


def _per_atom_lj(parameters, topology):
    """(N, 4) rows [eps, sigma, eps14, sigma14] as CharmmNonbondedConstraint.bind_ensemble
    builds them (charmm_nonbonded_constraint.py:48-60)."""
    types = np.asarray(topology.particle_types)
    uniq, inv = np.unique(types, return_inverse=True)
    table = np.zeros((len(uniq), 4))
    for k, t in enumerate(uniq):
        if t not in parameters:
            raise ParameterPoorDefinedError("no nonbonded parameter for particle type %s" % t)
        p = parameters[t]
        if len(p) == 2:
            table[k] = [p[0], p[1], p[0], p[1]]
        elif len(p) == 4:
            table[k] = p
        else:
            raise ParameterPoorDefinedError("nonbonded parameter of %s needs 2 or 4 values" % t)
    return table[inv.reshape(-1)]


class CharmmNonbondedConstraint(Constraint):
    """Lennard-Jones 12-6, Lorentz-Berthelot, 1-4 parameters for scaling
    partners, bonded partners excluded, hard cutoff r <= rc -- the reference's
    semantics; ``switch_radius`` adds the CHARMM energy switch on
    [switch_radius, cutoff] (new)."""
    _term_mask = _lib.mask(_lib.TERM_LJ)

    def __init__(self, parameters, cutoff_radius=12, switch_radius=None, force_id: int = 0,
                 force_group: int = 0):
        super().__init__(parameters, force_id=force_id, force_group=force_group)
        self._cutoff_radius = float(unit.check_quantity_value(cutoff_radius, "angstrom"))
        self.switch_radius = None if switch_radius is None else float(switch_radius)
        self._parameters_list = None

    def _bind(self, system, topology):
        self._parameters_list = _per_atom_lj(self._parameters, topology)
        system.set_lj(self._parameters_list)

    def set_cutoff_radius(self, val):
        super().set_cutoff_radius(val)
        if self._parent_ensemble is not None:
            self._parent_ensemble._configure()


class ElectrostaticConstraint(Constraint):
    """Bare Coulomb k q_i q_j / r over all pairs under the minimum image,
    1-2/1-3 pairs excluded (electrostatic_constraint.py:52-79).  O(N^2):
    kept for parity with the reference, not for production."""
    _term_mask = _lib.mask(_lib.TERM_COUL_REAL)
    _coulomb_mode = _lib.COUL_BARE
    _uses_cutoff = False

    def __init__(self, parameters=None, force_id: int = 0, force_group: int = 0):
        super().__init__(parameters, force_id=force_id, force_group=force_group)

    def _bind(self, system, topology):
        pass


class NonbondedConstraint(CharmmNonbondedConstraint):
    """The short-range nonbonded constraint: LJ (+ optional switch) and the
    Ewald real-space term k q_i q_j erfc(beta r)/r for r <= rc, in one pass
    over the pairs.  beta comes from ``ewald_beta`` or from ``ewald_error``
    via erfc(beta rc) = ewald_error."""
    _term_mask = _lib.mask(_lib.TERM_LJ, _lib.TERM_COUL_REAL)
    _coulomb_mode = _lib.COUL_EWALD

    def __init__(self, parameters, cutoff_radius=12, switch_radius=None, ewald_error=1e-5,
                 ewald_beta=None, force_id: int = 0, force_group: int = 0):
        super().__init__(parameters, cutoff_radius, switch_radius, force_id, force_group)
        self.ewald_error = ewald_error
        self._beta = ewald_beta

    @property
    def ewald_beta(self):
        if self._beta is not None:
            return float(self._beta)
        return ewald_beta_from_error(self._cutoff_radius, self.ewald_error)


class PMEConstraint(Constraint):
    """Smooth particle-mesh Ewald reciprocal space (order-p B-splines, cuFFT),
    plus the FP64 self and net-charge terms and the erf correction of the
    excluded pairs, so that NonbondedConstraint + PMEConstraint is the full
    Ewald sum.  ``grid_size`` defaults to the FFT-friendly size at
    ``grid_spacing`` A per point."""
    _term_mask = _lib.mask(_lib.TERM_COUL_RECIP)
    _uses_cutoff = False

    def __init__(self, grid_size=None, order=4, ewald_error=1e-5, ewald_beta=None,
                 real_space_cutoff=12.0, grid_spacing=1.0, force_id: int = 0, force_group: int = 0):
        super().__init__(None, force_id=force_id, force_group=force_group)
        self.grid_size = grid_size
        self.order = int(order)
        self.ewald_error = ewald_error
        self._beta = ewald_beta
        self.real_space_cutoff = float(real_space_cutoff)
        self.grid_spacing = float(grid_spacing)
        self.grid = None

    @property
    def ewald_beta(self):
        if self._beta is not None:
            return float(self._beta)
        return ewald_beta_from_error(self.real_space_cutoff, self.ewald_error)

    def _bind(self, system, topology):
        pass

    def _configure_system(self, beta):
        from .systems import fft_friendly

        box = self._parent_ensemble.state.box
        if self.grid_size is None:
            grid = [fft_friendly(int(math.ceil(L / self.grid_spacing))) for L in box]
        else:
            grid = [int(k) for k in np.broadcast_to(np.asarray(self.grid_size), (3,))]
        self.grid = grid
        self._parent_ensemble.system.pme_config(grid, self.order, beta or self.ewald_beta)


def _type_rows(parameters, topology, index_rows, width_p, sep="-", expand=False):
    types = topology.particle_types
    cache, idx_out, prm_out = {}, [], []
    for row in index_rows:
        key = sep.join(types[int(i)] for i in row)
        if key not in cache:
            if key not in parameters:
                raise ParameterPoorDefinedError("no parameter for %s" % key)
            cache[key] = parameters[key]
        p = cache[key]
        if expand:
            for term in p:
                idx_out.append([int(i) for i in row])
                prm_out.append(list(term)[:width_p])
        else:
            idx_out.append([int(i) for i in row])
            prm_out.append(list(p)[:width_p])
    return idx_out, prm_out


class _Bonded(Constraint):
    _width = 2
    _pwidth = 2
    _expand = False

    def __init__(self, parameters, force_id: int = 0, force_group: int = 0, float_parameters=None):
        super().__init__(parameters, force_id=force_id, force_group=force_group)
        self._explicit = None if float_parameters is None else np.asarray(float_parameters,
                                                                          dtype=np.float64)
        self._int_parameters = None
        self._float_parameters = None

    def _rows(self, topology):
        raise NotImplementedError

    def _bind(self, system, topology):
        rows = np.asarray(self._rows(topology), dtype=np.int64).reshape(-1, self._width)
        if self._explicit is not None:
            idx, prm = rows, self._explicit.reshape(-1, self._pwidth)
        elif len(rows):
            idx, prm = _type_rows(self._parameters, topology, rows, self._pwidth,
                                  expand=self._expand)
        else:
            idx, prm = [], []
        self._int_parameters = np.asarray(idx, dtype=np.int32).reshape(-1, self._width)
        self._float_parameters = np.asarray(prm, dtype=np.float64).reshape(-1, self._pwidth)
        self._set(system, self._int_parameters, self._float_parameters)


class CharmmBondConstraint(_Bonded):
    """V = k (r - r0)^2 (charmm_bond_constraint.py:52-73)."""
    _term_mask = _lib.mask(_lib.TERM_BOND)
    _width, _pwidth = 2, 2

    def _rows(self, topology):
        return topology.bonds

    def _set(self, system, idx, prm):
        system.set_bonds(idx, prm)

    @property
    def num_bonds(self):
        return 0 if self._int_parameters is None else len(self._int_parameters)


class CharmmAngleConstraint(_Bonded):
    """V = k (theta - theta0)^2 + ku (r13 - u0)^2 (charmm_angle_constraint.py:138-179)."""
    _term_mask = _lib.mask(_lib.TERM_ANGLE)
    _width, _pwidth = 3, 4

    def _rows(self, topology):
        return topology.angles

    def _set(self, system, idx, prm):
        system.set_angles(idx, prm)

    @property
    def num_angles(self):
        return 0 if self._int_parameters is None else len(self._int_parameters)


class CharmmDihedralConstraint(_Bonded):
    """V = k (1 + cos(n phi - delta)), one row per Fourier term
    (charmm_dihedral_constraint.py:33-56); forces are -dV/dphi exactly."""
    _term_mask = _lib.mask(_lib.TERM_DIHEDRAL)
    _width, _pwidth = 4, 3
    _expand = True

    def _rows(self, topology):
        return topology.dihedrals

    def _set(self, system, idx, prm):
        system.set_dihedrals(idx, prm)

    @property
    def num_dihedrals(self):
        if self._int_parameters is None:
            return 0
        return len({tuple(r) for r in self._int_parameters.tolist()})


class CharmmImproperConstraint(_Bonded):
    """V = k (psi - psi0)^2 (charmm_improper_constraint.py:56-93)."""
    _term_mask = _lib.mask(_lib.TERM_IMPROPER)
    _width, _pwidth = 4, 2

    def _rows(self, topology):
        return topology.impropers

    def _set(self, system, idx, prm):
        system.set_impropers(idx, prm)

    @property
    def num_impropers(self):
        return 0 if self._int_parameters is None else len(self._int_parameters)
