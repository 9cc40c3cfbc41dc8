"""Energy minimisers with mdpy's interface (mdpy/minimizer/*.py).

``SteepestDescentMinimizer`` runs on the device: each iteration is one
``mdg_minimize_step`` (x_i += alpha F_i/|F_i|, steepest_descent_minimizer.py:
39-42) and one fused force evaluation; only the potential energy comes back
to the host for the convergence test (|dE/E| < energy_tolerance, :44-51).
``ConjugateGradientMinimizer`` follows conjugate_gradient_minimizer.py:33-80
on host copies of the forces, with the force evaluations on the device.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from . import unit


class Minimizer:
    def __init__(self, output_unit=None, output_unit_label="kj/mol", is_verbose=False,
                 log_freq=5):
        # energies are printed in kJ/mol (mdpy's default output_unit)
        self._output_unit = output_unit
        self._output_unit_label = output_unit_label
        self._is_verbose = is_verbose
        self._log_freq = log_freq

    def minimize(self, ensemble, energy_tolerance=0.001, max_iterations: int = 1000):
        raise NotImplementedError(
            "The subclass of mdpy.minimizer.Minimizer class should overload minimize method")

    def _energy2str(self, energy):
        return "%.5f %s" % (float(energy) / unit.KJ_PER_MOL, self._output_unit_label)


def _potential(ensemble, mask):
    e, _ = ensemble.system.get_energies()
    return float(sum(e[t] for t in range(_lib.NUM_TERMS) if mask >> t & 1))


class SteepestDescentMinimizer(Minimizer):
    def __init__(self, alpha=0.01, output_unit=None, output_unit_label="kj/mol",
                 is_verbose=False, log_freq=5):
        super().__init__(output_unit, output_unit_label, is_verbose, log_freq)
        self._alpha = float(unit.check_quantity_value(alpha, "angstrom"))

    def minimize(self, ensemble, energy_tolerance=0.001, max_iterations: int = 1000):
        sysm = ensemble.system
        mask = ensemble.term_mask
        sysm.compute_forces(mask)
        cur = _potential(ensemble, mask)
        pre = cur
        print("Start energy minimization with steepest decent method")
        print("Initial potential energy: %s" % self._energy2str(cur))
        it = 0
        converged = False
        while it < max_iterations:
            sysm.minimize_step(self._alpha)
            sysm.compute_forces(mask)
            cur = _potential(ensemble, mask)
            err = abs((cur - pre) / pre) if pre != 0 else abs(cur - pre)
            it += 1
            if self._is_verbose and it % self._log_freq == 0:
                print("Iteration %d: %s %.4f" % (it + 1, self._energy2str(cur), err))
            if err < energy_tolerance:
                print("Penultimate potential energy %s" % self._energy2str(pre))
                print("Final potential energy %s" % self._energy2str(cur))
                print("Energy error: %e < %e" % (err, energy_tolerance))
                converged = True
                break
            pre = cur
        if not converged:
            print("Final potential energy: %s" % self._energy2str(cur))
        ensemble._read_back(mask)
        self.num_iterations = it
        return None


class ConjugateGradientMinimizer(Minimizer):
    def __init__(self, theta=0.001, force_tol=0.01, max_sub_iterations=10, output_unit=None,
                 output_unit_label="kj/mol", is_verbose=False, log_freq=5):
        super().__init__(output_unit, output_unit_label, is_verbose, log_freq)
        self._theta = float(theta)
        self._force_tol = float(force_tol)
        self._max_sub_iterations = int(max_sub_iterations)

    def minimize(self, ensemble, energy_tolerance=0.001, max_iterations: int = 1000):
        state = ensemble.state
        ensemble.update()
        cur = ensemble.potential_energy
        print("Start energy minimization with steepest decent method")
        print("Initial potential energy: %s" % self._energy2str(cur))
        it = 0
        while it < max_iterations:
            pre = cur
            x0 = state.positions.copy()
            f0 = ensemble.forces.reshape(-1, 1)
            d = np.zeros_like(f0)
            cur_f = f0.copy()
            t = cur_f.copy()
            for _ in range(self._max_sub_iterations):
                state.set_positions(state.positions + self._theta * t.reshape(-1, 3))
                ensemble.update()
                omega = -(ensemble.forces.reshape(-1, 1) - cur_f) / self._theta
                alpha = float(cur_f.T @ cur_f) / float(omega.T @ t)
                d += alpha * t
                cur_f, pre_f = cur_f + alpha * omega, cur_f
                if float((cur_f ** 2).sum()) / float((f0 ** 2).sum()) < self._force_tol:
                    break
                beta = float(cur_f.T @ cur_f) / float(pre_f.T @ pre_f)
                t = cur_f + beta * t
            state.set_positions(x0 + d.reshape(-1, 3))
            ensemble.update()
            cur = ensemble.potential_energy
            err = abs((cur - pre) / pre) if pre != 0 else abs(cur - pre)
            it += 1
            if self._is_verbose and it % self._log_freq == 0:
                print("Iteration %d: %s %.4f" % (it, self._energy2str(cur), err))
            if err < energy_tolerance:
                print("Penultimate potential energy %s" % self._energy2str(pre))
                print("Final potential energy %s" % self._energy2str(cur))
                print("Energy error: %e < %e" % (err, energy_tolerance))
                self.num_iterations = it
                return None
        print("Final potential energy: %s" % self._energy2str(cur))
        self.num_iterations = it
        return None
