"""Batches of independent ensembles evaluated and integrated together.

mdpy drives one ``Ensemble`` per process (mdpy/ensemble.py:15-102).  Many
small systems -- a few thousand atoms each -- leave most of a GB300 idle
when run one at a time, so a batch puts them in one device system
(``mdg_system_create_batch``): every kernel covers every member, each member
keeps its own box, PME grid and energies, and each member's forces and
trajectory are the ones it would have alone (up to float rounding of the
batched FFT).

    members = []
    for w in boxes:
        ens = batch.member(w.topology, w.pbc_matrix)      # records, allocates nothing
        ens.add_constraints(NonbondedConstraint(...), PMEConstraint(...), ...)
        ens.state.set_positions(w.positions)
        members.append(ens)
    b = batch.EnsembleBatch(members)
    LangevinIntegrator(1.0, 300, 0.001, seed=1).integrate(b, 1000)
    b.potential_energies                                   # (n_members,)

Members must agree on everything the batch shares: the cutoff, switch,
Coulomb mode, Ewald beta, PME order and the set of bound terms.
"""
from __future__ import annotations

import os

import numpy as np

from . import _lib
from .ensemble import Ensemble, _diag_box


class _Recorder:
    """Takes the place of a device system while a member ensemble is set up:
    keeps the last value given to each setter."""

    def __init__(self, n_atoms, box):
        self.n = int(n_atoms)
        self.box = np.asarray(box, dtype=np.float64).copy()
        self.calls = {}

    def _keep(name):  # noqa: N805 - decorator factory used in the class body
        def setter(self, *args):
            self.calls[name] = args
        return setter

    set_masses = _keep("set_masses")
    set_charges = _keep("set_charges")
    set_lj = _keep("set_lj")
    set_exclusions = _keep("set_exclusions")
    nonbonded_config = _keep("nonbonded_config")
    pme_config = _keep("pme_config")
    set_bonds = _keep("set_bonds")
    set_angles = _keep("set_angles")
    set_dihedrals = _keep("set_dihedrals")
    set_impropers = _keep("set_impropers")
    set_positions = _keep("set_positions")
    set_velocities = _keep("set_velocities")
    set_reorder_interval = _keep("set_reorder_interval")
    del _keep

    def set_box(self, box):
        self.box = np.asarray(box, dtype=np.float64).copy()

    def kinetic_energy(self):
        return 0.0


def member(topology, pbc_matrix):
    """An ``Ensemble`` whose set-up (constraints, positions, velocities) is
    recorded for an ``EnsembleBatch`` instead of going to a device."""
    return Ensemble(topology, pbc_matrix, _system=_Recorder(topology.num_particles,
                                                             _diag_box(pbc_matrix)))


def _same(values, what):
    first = values[0]
    for v in values[1:]:
        if not (len(v) == len(first) and all(np.array_equal(np.asarray(a), np.asarray(b))
                                             for a, b in zip(v, first))):
            raise ValueError("batch members disagree on %s" % what)
    return first


class EnsembleBatch:
    """The members' systems in one device batch.  Quacks like an ``Ensemble``
    for the integrators (``system``, ``term_mask``), with per-member results."""

    def __init__(self, members, device=None):
        if not members:
            raise ValueError("an empty batch")
        recs = []
        for m in members:
            if not isinstance(m.system, _Recorder):
                raise TypeError("batch members are made with batch.member()")
            recs.append(m.system)
        if device is None:
            device = int(os.environ.get("MDG_DEVICE", "0"))
        masks = {m.term_mask for m in members}
        if len(masks) != 1:
            raise ValueError("batch members bind different sets of terms")
        self._mask = masks.pop()
        self._members = list(members)
        counts = np.array([r.n for r in recs], dtype=np.int64)
        self._offsets = np.concatenate([[0], np.cumsum(counts)])
        boxes = np.stack([r.box for r in recs])
        sysb = _lib.System.batch(counts, boxes, device)
        self._system = sysb
        n = int(counts.sum())

        def cat(name, shape, default=None):
            parts = []
            for r, c in zip(recs, counts):
                if name in r.calls:
                    parts.append(np.asarray(r.calls[name][0], dtype=np.float64).reshape(int(c), *shape))
                elif default is not None:
                    parts.append(np.full((int(c),) + shape, default, dtype=np.float64))
                else:
                    return None
            return np.concatenate(parts)

        sysb.set_masses(cat("set_masses", (), 1.0))
        sysb.set_charges(cat("set_charges", (), 0.0))
        lj = cat("set_lj", (4,))
        if lj is not None:
            sysb.set_lj(lj)
        # exclusion partner lists, shifted to batch atom indices and padded
        # to the widest member
        excl = [r.calls.get("set_exclusions") for r in recs]
        if any(e is not None for e in excl):
            tabs = ([], [])
            for k in range(2):
                width = max(np.asarray(e[k]).reshape(int(c), -1).shape[1] if e is not None else 1
                            for e, c in zip(excl, counts))
                for e, c, off in zip(excl, counts, self._offsets[:-1]):
                    t = np.full((int(c), max(width, 1)), -1, dtype=np.int64)
                    if e is not None:
                        a = np.asarray(e[k], dtype=np.int64).reshape(int(c), -1)
                        t[:, :a.shape[1]] = np.where(a >= 0, a + off, -1)
                    tabs[k].append(t)
            sysb.set_exclusions(np.concatenate(tabs[0]), np.concatenate(tabs[1]))
        nb = [r.calls.get("nonbonded_config") for r in recs]
        if any(c is not None for c in nb):
            if any(c is None for c in nb):
                raise ValueError("batch members disagree on the nonbonded terms")
            sysb.nonbonded_config(*_same(nb, "the nonbonded settings"))
        pme = [r.calls.get("pme_config") for r in recs]
        if any(c is not None for c in pme):
            if any(c is None for c in pme):
                raise ValueError("batch members disagree on PME")
            _same([c[1:] for c in pme], "the PME order and beta")
            grids = np.array([np.broadcast_to(np.asarray(c[0], dtype=np.int64), (3,)) for c in pme])
            sysb.pme_config_batch(grids, pme[0][1], pme[0][2])
        for name in ("set_bonds", "set_angles", "set_dihedrals", "set_impropers"):
            calls = [r.calls.get(name) for r in recs]
            if all(c is None for c in calls):
                continue
            idx, prm = [], []
            for c, off in zip(calls, self._offsets[:-1]):
                if c is None or len(c[0]) == 0:
                    continue
                idx.append(np.asarray(c[0], dtype=np.int64) + off)
                prm.append(np.asarray(c[1], dtype=np.float64))
            if idx:
                getattr(sysb, name)(np.concatenate(idx), np.concatenate(prm))
        ri = [r.calls.get("set_reorder_interval") for r in recs if "set_reorder_interval" in r.calls]
        if ri:
            sysb.set_reorder_interval(*_same(ri, "the re-sort interval"))
        x = cat("set_positions", (3,))
        if x is not None:
            sysb.set_positions(x)
        v = cat("set_velocities", (3,), 0.0)
        sysb.set_velocities(v)
        self._energies = np.zeros((len(recs), _lib.NUM_TERMS))
        self._kinetic = np.zeros(len(recs))
        self._forces = None
        assert n == sysb.n

    # -- what the integrators use ---------------------------------------------
    @property
    def system(self):
        return self._system

    @property
    def term_mask(self):
        return self._mask

    def _after_integrate(self):
        self._energies, self._kinetic = self._system.get_energies_batch()
        self._forces = None

    # -- batch API ------------------------------------------------------------
    @property
    def num_members(self):
        return len(self._members)

    @property
    def members(self):
        return list(self._members)

    def member_slice(self, q):
        return slice(int(self._offsets[q]), int(self._offsets[q + 1]))

    def update(self):
        """One device evaluation of every member's terms."""
        self._system.compute_forces(self._mask)
        self._energies, _ = self._system.get_energies_batch()
        self._kinetic = self._kinetic_now()
        self._forces = self._system.get_forces()

    def _kinetic_now(self):
        self._system.kinetic_energy()   # refreshes every member's kinetic slot
        return self._system.get_energies_batch()[1]

    @property
    def energies(self):
        """(n_members, NUM_TERMS) energies of the last evaluation."""
        return self._energies.copy()

    @property
    def potential_energies(self):
        m = [t for t in range(_lib.NUM_TERMS) if self._mask >> t & 1]
        return self._energies[:, m].sum(axis=1)

    @property
    def kinetic_energies(self):
        return self._kinetic.copy()

    def forces(self, q=None):
        if self._forces is None:
            self._forces = self._system.get_forces()
        return self._forces if q is None else self._forces[self.member_slice(q)]

    def positions(self, q=None):
        x = self._system.get_positions()
        return x if q is None else x[self.member_slice(q)]

    def velocities(self, q=None):
        v = self._system.get_velocities()
        return v if q is None else v[self.member_slice(q)]
