"""Integrators with mdpy's interface (mdpy/integrator/integrator.py:14-62).

``integrate(ensemble, num_steps)`` advances the device state; positions and
velocities stay in HBM (FP64) and the steps run as CUDA-graph chunks inside
libmdg.  One force evaluation per step.

* ``VerletIntegrator`` -- velocity Verlet.  mdpy's position-Verlet
  (mdpy/integrator/verlet_integrator.py:20-48) starts with a dt^2 instead of
  dt^2/2 term and reports half the velocity; those are not reproduced.
* ``LangevinIntegrator`` -- Groenbech-Jensen--Farago Langevin, the scheme
  mdpy's LangevinIntegrator writes (mdpy/integrator/langevin_integrator.py:
  18-71), with the force sign of -grad V, one force evaluation per step, and
  seeded counter-based (Philox) noise instead of unseeded numpy randn.
"""
from __future__ import annotations

import os

from . import _lib
from . import unit


class Integrator:
    """``reciprocal_every`` = k > 1: the PME force enters every k-th step with
    weight k (impulse multiple-time-step scheme, outer step k dt).
    ``learned`` = a trained :class:`mdpy_gb300.learned.LearnedSlowForce`:
    full PME every ``learned.outer_step`` steps and the learned prediction of
    the slow force in between (``reciprocal_every`` is then ignored)."""
    _kind = None

    def __init__(self, time_step, reciprocal_every=1, learned=None):
        self._time_step = float(unit.check_quantity_value(time_step, "femtosecond"))
        self.reciprocal_every = int(reciprocal_every)
        self.learned = learned

    def _configure(self, ensemble):
        raise NotImplementedError

    def integrate(self, ensemble, num_steps: int = 1, read_back: bool = True):
        """``read_back=False`` only enqueues the steps (the ensemble's
        energies are read later, e.g. from energy snapshots)."""
        self._configure(ensemble)
        if self.learned is not None:
            self.learned.enable(ensemble.system)
        else:
            ensemble.system.set_mts(self.reciprocal_every)
        ensemble.system.integrate(int(num_steps), ensemble.term_mask, want_energy=True)
        if read_back:
            ensemble._after_integrate()

    def erase_cache(self):
        """mdpy keeps x_{n-1} on the host between calls; the device state
        needs no cache (kept for API compatibility)."""

    @property
    def time_step(self):
        return self._time_step

    @time_step.setter
    def time_step(self, time_step):
        self._time_step = float(unit.check_quantity_value(time_step, "femtosecond"))

    @property
    def is_cached(self):
        return False


class VerletIntegrator(Integrator):
    def __init__(self, time_step, reciprocal_every=1, learned=None):
        super().__init__(time_step, reciprocal_every, learned)

    def _configure(self, ensemble):
        ensemble.system.integrator_config(_lib.INTEGRATOR_VERLET, self._time_step)


class LangevinIntegrator(Integrator):
    """``friction_rate`` is in 1/fs for plain numbers (mdpy's default unit);
    an mdpy Quantity such as ``Quantity(1, 1/picosecond)`` is converted.
    ``seed`` keys the Philox stream; None draws one from the OS."""

    def __init__(self, time_step, temperature, friction_rate, seed=None, reciprocal_every=1,
                 learned=None):
        super().__init__(time_step, reciprocal_every, learned)
        self._temperature = float(unit.check_quantity_value(temperature, "kelvin"))
        if hasattr(friction_rate, "convert_to"):
            import importlib

            u = importlib.import_module("mdpy.unit")
            friction_rate = friction_rate.convert_to(1 / u.femtosecond).value
        self._gamma = float(friction_rate)
        if seed is None:
            seed = int.from_bytes(os.urandom(8), "little")
        self.seed = int(seed) & ((1 << 64) - 1)

    def _configure(self, ensemble):
        ensemble.system.integrator_config(_lib.INTEGRATOR_LANGEVIN, self._time_step,
                                          self._temperature, self._gamma, self.seed)

    @property
    def temperature(self):
        return self._temperature

    @property
    def friction_rate(self):
        return self._gamma
