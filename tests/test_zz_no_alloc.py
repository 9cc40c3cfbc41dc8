"""mdg_kinetic_energies_noalloc through the C ABI -- the entry point for
callers that must not have device memory allocated behind their back (a
host program whose own pool owns the GPU's memory, or a loop that cannot
afford cudaMalloc/cudaFree synchronising the device).  Its per-system
kinetic energies equal the ones mdg_kinetic_energy leaves in the system, bit
for bit, on two calls in a row (the static scratch is zeroed by each call).
Kept in the last-collected file so that a run stopping at the first failure
has run every other test first; it passes alone and after the others."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(lib):
    from mdpy_gb300 import systems

    ws = [systems.water_box(nw, (3 * nw / 0.1) ** (1 / 3), seed=70 + k)
          for k, nw in enumerate((300, 520, 410))]
    s = lib.System.batch([w.num_particles for w in ws], [w.box for w in ws])
    s.set_masses(np.concatenate([w.topology.masses.reshape(-1) for w in ws]))
    s.set_positions(np.concatenate([w.positions for w in ws]))
    s.set_velocities(np.concatenate([w.velocities for w in ws]))
    return s


def test_kinetic_energies_noalloc_matches_existing_entry_point(lib):
    raw = lib.load()
    s = _batch(lib)
    total = ctypes.c_double(0.0)
    assert raw.mdg_kinetic_energy(s.handle, ctypes.byref(total)) == 0
    ref = np.zeros(s.n_systems)
    assert raw.mdg_get_energies_batch(s.handle, None, ref.ctypes.data_as(
        ctypes.POINTER(ctypes.c_double))) == 0
    assert ref.sum() == pytest.approx(total.value, rel=1e-12) and np.all(ref > 0)
    for _ in range(2):
        out = np.full(s.n_systems, -1.0)
        rc = raw.mdg_kinetic_energies_noalloc(s.handle,
                                              out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        assert rc == 0, raw.mdg_last_error()
        assert np.array_equal(out, ref)
    s.close()
