"""Simulation driver and a log dumper with mdpy's interface.

``Simulation.integrate(n)`` runs ``integrator.integrate`` in chunks of the
greatest common divisor of the dumpers' frequencies and dumps after each
chunk, like mdpy/simulation.py:60-70; between dumps the steps stay on the
device as CUDA-graph replays.  ``LogDumper`` writes the columns of
mdpy/dumper/log_dumper.py:105-208 (step, potential / kinetic / total energy
in kJ/mol, temperature, ns/day).
"""
from __future__ import annotations

import math
import time

from . import unit
from .error import DumperPoorDefinedError


class Dumper:
    def __init__(self, dump_frequency: int):
        if int(dump_frequency) <= 0:
            raise DumperPoorDefinedError("dump_frequency must be a positive integer")
        self.dump_frequency = int(dump_frequency)

    def dump(self, simulation):
        raise NotImplementedError


class LogDumper(Dumper):
    """Tab-separated log.  ``file_path=None`` keeps the rows in ``rows``.

    ``asynchronous=True``: when every dumper of a Simulation is asynchronous,
    ``Simulation.integrate`` does not wait for the GPU at a dump step.  It
    enqueues a copy of that step's energies into a pinned ring slot
    (``mdg_energy_snapshot``) and goes on enqueueing steps; rows are written
    as their copies complete (at the latest when the ring is full and at the
    end of ``integrate``).  The rows hold the same values as synchronous
    dumping; the speed column is taken when a row is written."""

    def __init__(self, file_path=None, dump_frequency=1, step=True, potential_energy=True,
                 kinetic_energy=True, total_energy=True, temperature=True, sim_speed=True,
                 seperator="\t", asynchronous=False):
        super().__init__(dump_frequency)
        self.asynchronous = bool(asynchronous)
        self.file_path = file_path
        self.columns = [c for c, on in (("Step", step), ("Potential Energy (kj/mol)", potential_energy),
                                        ("Kinetic Energy (kj/mol)", kinetic_energy),
                                        ("Total Energy (kj/mol)", total_energy),
                                        ("Temperature (K)", temperature),
                                        ("Speed (ns/day)", sim_speed)) if on]
        self.sep = seperator
        self.rows = []
        self._t0 = None
        self._step0 = 0
        if file_path:
            with open(file_path, "w") as fh:
                fh.write(self.sep.join(self.columns) + "\n")

    def dump(self, simulation):
        ens = simulation.ensemble
        self.dump_values(simulation, simulation.cur_step, ens.potential_energy,
                         ens.kinetic_energy)

    def dump_values(self, simulation, step, potential_energy, kinetic_energy):
        """One row from energies read at ``step`` (either path)."""
        now = time.perf_counter()
        if self._t0 is None:
            self._t0, self._step0 = now, step
        kj = 1.0 / unit.KJ_PER_MOL
        vals = {
            "Step": "%d" % step,
            "Potential Energy (kj/mol)": "%.3f" % (potential_energy * kj),
            "Kinetic Energy (kj/mol)": "%.3f" % (kinetic_energy * kj),
            "Total Energy (kj/mol)": "%.3f" % ((potential_energy + kinetic_energy) * kj),
            "Temperature (K)": "%.2f" % unit.kinetic_temperature(
                kinetic_energy, simulation.ensemble.topology.num_particles),
        }
        dt = now - self._t0
        steps = step - self._step0
        vals["Speed (ns/day)"] = ("%.4f" % unit.ns_per_day(steps / dt, simulation.integrator.time_step)
                                  if dt > 0 and steps > 0 else "--")
        row = [vals[c] for c in self.columns]
        self.rows.append(row)
        if self.file_path:
            with open(self.file_path, "a") as fh:
                fh.write(self.sep.join(row) + "\n")


class Simulation:
    def __init__(self, ensemble, integrator, minimizer=None):
        self._ensemble = ensemble
        self._integrator = integrator
        self._minimizer = minimizer
        self._cur_step = 0
        self._dumpers = []
        self._minimum_dump_frequency = 0

    def add_dumpers(self, *dumpers):
        for d in dumpers:
            self._dumpers.append(d)
            self._minimum_dump_frequency = math.gcd(self._minimum_dump_frequency, d.dump_frequency)

    def _dump(self):
        for d in self._dumpers:
            if self._cur_step % d.dump_frequency == 0:
                d.dump(self)

    def dump_initial_state(self):
        self._ensemble.update()
        for d in self._dumpers:
            d.dump(self)

    def reset_simulation_step(self):
        self._cur_step = 0

    def set_minimizer(self, minimizer):
        self._minimizer = minimizer

    def minimize(self, energy_tolerance, max_iterations):
        """mdpy/simulation.py:52-54; the default minimizer is steepest descent
        with alpha 0.01 A (:18)."""
        if self._minimizer is None:
            from .minimizer import SteepestDescentMinimizer

            self._minimizer = SteepestDescentMinimizer(0.01)
        self._minimizer.minimize(self._ensemble, energy_tolerance, max_iterations)
        self._dump()

    def integrate(self, num_steps: int):
        if not self._dumpers or self._minimum_dump_frequency == 0:
            raise DumperPoorDefinedError("No dumper has been added to Simulation yet.")
        if all(getattr(d, "asynchronous", False) for d in self._dumpers):
            return self._integrate_async(int(num_steps))
        target = self._cur_step + int(num_steps)
        while self._cur_step < target:
            chunk = min(self._minimum_dump_frequency, target - self._cur_step)
            self._integrator.integrate(self._ensemble, chunk)
            self._cur_step += chunk
            self._dump()

    def _integrate_async(self, num_steps):
        """The loop of ``integrate`` with energy snapshots instead of reads:
        a dump step enqueues its energies into a ring slot, rows are written
        as the copies complete, and the host waits only when every slot is
        in flight and at the end."""
        from collections import deque

        from . import _lib

        ens = self._ensemble
        sysm = ens.system
        mask = ens.term_mask
        target = self._cur_step + num_steps
        pending = deque()
        slot = 0

        def write(step, slot, wait):
            r = sysm.energy_snapshot_read(slot, wait=wait)
            if r is None:
                return False
            e, ke = r
            pe = float(sum(e[t] for t in range(_lib.NUM_TERMS) if mask >> t & 1))
            for d in self._dumpers:
                if step % d.dump_frequency == 0:
                    d.dump_values(self, step, pe, ke)
            return True

        while self._cur_step < target:
            chunk = min(self._minimum_dump_frequency, target - self._cur_step)
            self._integrator.integrate(ens, chunk, read_back=False)
            self._cur_step += chunk
            if any(self._cur_step % d.dump_frequency == 0 for d in self._dumpers):
                if len(pending) == _lib.SNAPSHOT_SLOTS:
                    write(*pending.popleft(), wait=True)
                sysm.energy_snapshot(slot)
                pending.append((self._cur_step, slot))
                slot = (slot + 1) % _lib.SNAPSHOT_SLOTS
            while pending and write(*pending[0], wait=False):
                pending.popleft()
        while pending:
            write(*pending.popleft(), wait=True)
        ens._after_integrate()

    @property
    def ensemble(self):
        return self._ensemble

    @property
    def integrator(self):
        return self._integrator

    @property
    def dumpers(self):
        return self._dumpers

    @property
    def num_dumpers(self):
        return len(self._dumpers)

    @property
    def cur_step(self):
        return self._cur_step
