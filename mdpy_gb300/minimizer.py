"""Energy minimisers with mdpy's interface (mdpy/minimizer/*.py).

``SteepestDescentMinimizer`` runs on the device: each iteration is one
``mdg_minimize_step`` (x_i += alpha F_i/|F_i|, steepest_descent_minimizer.py:
39-42) and one fused force evaluation; only the potential energy comes back
to the host for the convergence test (|dE/E| < energy_tolerance, :44-51).
mdpy's conjugate-gradient minimiser is not rebuilt (it is not on the
force-and-step path).
"""
from __future__ import annotations

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
