"""CharmmForcefield with mdpy's interface, emitting the device constraints.

mdpy's ``CharmmForcefield(topology, pbc, cutoff_radius=12,
long_range_solver='PPPM', ewald_error=1e-6)`` stores the long-range solver
and Ewald error but never uses them, and ``create_ensemble`` wires a bare
all-pairs ``ElectrostaticConstraint`` next to the LJ constraint
(mdpy/forcefield/charmm_forcefield.py:20-112).  Here the same call builds a
device ``Ensemble``:

* ``long_range_solver`` 'PME' or 'PPPM' (both mean smooth PME here):
  ``NonbondedConstraint`` (LJ + Ewald real space, beta from ``ewald_error``)
  + ``PMEConstraint`` (grid at ``pme_grid_spacing`` A, order 4);
* ``long_range_solver=None``: the reference's pair of constraints,
  ``CharmmNonbondedConstraint`` + ``ElectrostaticConstraint``;
* bond / angle / dihedral / improper constraints for the terms the topology
  has, as the reference does (:96-112).

Parameter files are parsed by mdpy's own ``CharmmTopparParser`` when mdpy is
importable (``set_param_files``); otherwise pass the parsed dictionaries with
``set_parameters`` (the format of ``CharmmTopparParser(...).parameters``).
"""
from __future__ import annotations

import numpy as np

from . import constraint as C
from .ensemble import Ensemble, _diag_box
from .error import ParameterPoorDefinedError


class CharmmForcefield:
    def __init__(self, topology, pbc_matrix, cutoff_radius=12, long_range_solver="PPPM",
                 ewald_error=1e-6, is_SHAKE=True, switch_radius=None, pme_grid_spacing=1.0,
                 pme_order=4):
        self._topology = topology
        self._pbc_matrix = np.asarray(pbc_matrix, dtype=np.float64)
        _diag_box(self._pbc_matrix)
        self._cutoff_radius = float(cutoff_radius)
        if long_range_solver not in (None, "PME", "PPPM"):
            raise ValueError("long_range_solver must be None, 'PME' or 'PPPM'")
        self._long_range_solver = long_range_solver
        self._ewald_error = float(ewald_error)
        self._is_SHAKE = is_SHAKE     # accepted for API compatibility; no constraint solver
        self._switch_radius = switch_radius
        self._pme_grid_spacing = float(pme_grid_spacing)
        self._pme_order = int(pme_order)
        self._parameters = None

    def set_param_files(self, *file_paths):
        """Parse CHARMM parameter files with mdpy's own parser."""
        try:
            from mdpy.io import CharmmTopparParser
        except ImportError as exc:  # pragma: no cover - depends on mdpy being installed
            raise ImportError("parsing CHARMM files needs mdpy; pass parsed dictionaries with "
                              "set_parameters instead") from exc
        self._parameters = CharmmTopparParser(*file_paths).parameters

    def set_parameters(self, parameters):
        self._parameters = parameters

    @property
    def parameters(self):
        return self._parameters

    def check_parameters(self):
        """Every particle type and bonded term has a parameter
        (mdpy/forcefield/charmm_forcefield.py:38-94)."""
        if self._parameters is None:
            raise ParameterPoorDefinedError("no parameters set")
        t = self._topology
        if not t.is_joined:
            t.join()
        types = t.particle_types
        for ty in set(types):
            if ty not in self._parameters["nonbonded"]:
                raise ParameterPoorDefinedError(
                    "The nonbonded parameter for particle type %s can not be found" % ty)
        for name, width in (("bond", 2), ("angle", 3), ("dihedral", 4), ("improper", 4)):
            rows = np.asarray(getattr(t, name + "s")).reshape(-1, width)
            seen = set()
            for row in rows:
                key = "-".join(types[int(i)] for i in row)
                if key in seen:
                    continue
                seen.add(key)
                if key not in self._parameters[name]:
                    raise ParameterPoorDefinedError(
                        "The parameter for %s %s (%s) can not be found"
                        % (name, "-".join(str(int(i)) for i in row), key))

    def create_ensemble(self, device=None):
        self.check_parameters()
        t = self._topology
        ens = Ensemble(t, self._pbc_matrix, device=device)
        cons = []
        if t.num_particles != 0:
            if self._long_range_solver is None:
                cons.append(C.ElectrostaticConstraint())
                cons.append(C.CharmmNonbondedConstraint(self._parameters["nonbonded"],
                                                        self._cutoff_radius,
                                                        switch_radius=self._switch_radius))
            else:
                cons.append(C.NonbondedConstraint(self._parameters["nonbonded"],
                                                  self._cutoff_radius,
                                                  switch_radius=self._switch_radius,
                                                  ewald_error=self._ewald_error))
                cons.append(C.PMEConstraint(order=self._pme_order, ewald_error=self._ewald_error,
                                            real_space_cutoff=self._cutoff_radius,
                                            grid_spacing=self._pme_grid_spacing))
        if t.num_bonds:
            cons.append(C.CharmmBondConstraint(self._parameters["bond"]))
        if t.num_angles:
            cons.append(C.CharmmAngleConstraint(self._parameters["angle"]))
        if t.num_dihedrals:
            cons.append(C.CharmmDihedralConstraint(self._parameters["dihedral"]))
        if t.num_impropers:
            cons.append(C.CharmmImproperConstraint(self._parameters["improper"]))
        ens.add_constraints(*cons)
        return ens
