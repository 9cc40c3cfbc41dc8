"""mdpy_gb300 -- GB300-native (sm_103a) force-and-step engine for mdpy.

The package keeps mdpy's constraint / ensemble / integrator / simulation API
and runs the hot path (short-range nonbonded with Ewald real space, PME
reciprocal space, bonded terms, Verlet/Langevin update) in hand-written CUDA
kernels of ``libmdg.so`` through a C ABI (include/mdg.h).  Importing the
high-level classes needs the built library; there is no CPU fallback.
"""
from . import unit, error
from .topology import Particle, Topology

__version__ = "1.0.0"


def __getattr__(name):
    # high-level classes load libmdg lazily so `import mdpy_gb300` works for
    # building and inspection on machines without the library
    if name in ("Ensemble", "State"):
        from . import ensemble
        return getattr(ensemble, name)
    if name == "Simulation":
        from .simulation import Simulation
        return Simulation
    if name == "SteepestDescentMinimizer":
        from . import minimizer
        return getattr(minimizer, name)
    if name == "EnsembleBatch":
        from .batch import EnsembleBatch
        return EnsembleBatch
    if name == "LearnedSlowForce":
        from .learned import LearnedSlowForce
        return LearnedSlowForce
    if name in ("constraint", "integrator", "simulation", "ensemble", "systems", "_lib",
                "minimizer", "batch", "forcefield", "learned"):
        import importlib
        return importlib.import_module("." + name, __name__)
    raise AttributeError(name)


__all__ = ["unit", "error", "Particle", "Topology", "Ensemble", "State", "Simulation",
           "SteepestDescentMinimizer", "EnsembleBatch",
           "LearnedSlowForce", "constraint", "integrator", "simulation", "systems", "minimizer",
           "batch", "forcefield", "learned"]
