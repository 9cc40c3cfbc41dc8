"""The drop-in boundary exercised from the reference's side: the libmdg
constraint of tests/ref_binding.py bound into the reference's own, unchanged
Ensemble (mdpy/ensemble.py:40-61) gives the forces and energy of the
mdpy_gb300 Ensemble on the same system, and both agree with the FP64
oracle.  Skipped where the reference is not installed in baseline/_ref."""
import numpy as np
import pytest

from tests import ref_binding as RB
from tests.helpers import rel_rms, water_lj_rows

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not RB.reference_available(),
                                 reason="the reference is not installed in baseline/_ref")]


def test_binding_inside_the_reference_ensemble(lib, orc):
    RB.import_reference()
    from mdpy.ensemble import Ensemble as RefEnsemble

    from mdpy_gb300 import constraint as C, systems
    from mdpy_gb300.ensemble import Ensemble

    w = systems.water_box(900, 30.0, seed=0)
    beta = orc.ewald_beta(12.0, 1e-5)
    # the reference's Ensemble with the libmdg constraint added to it
    ref = RefEnsemble(RB.reference_topology(w), np.eye(3) * 30.0)
    ref.state.set_positions(w.positions.astype(np.float32))
    ref.state.set_velocities(w.velocities.astype(np.float32))
    gb = RB.binding_class()(w.parameters["nonbonded"], cutoff_radius=12, ewald_beta=beta,
                            pme_grid=32)
    ref.add_constraints(gb)
    assert gb.force_id == 0 and ref.state.cell_list.cutoff_radius == 12
    ref.update()
    f_ref = np.asarray(ref.forces, dtype=np.float64)
    pos = np.asarray(ref.state.positions, dtype=np.float64)   # mdpy's wrapped float32 state

    # the same terms through the mdpy_gb300 Ensemble
    ens = Ensemble(w.topology, w.pbc_matrix, device=0)
    nb = C.NonbondedConstraint(w.parameters["nonbonded"], cutoff_radius=12.0, ewald_error=1e-5)
    ens.add_constraints(nb, C.PMEConstraint(grid_size=32, order=4, ewald_error=1e-5,
                                            real_space_cutoff=12.0))
    ens.state.set_positions(pos)
    ens.update()
    assert nb.ewald_beta == pytest.approx(beta, rel=1e-12)
    assert rel_rms(f_ref, ens.forces) <= 1e-6
    assert ref.potential_energy == pytest.approx(ens.potential_energy, rel=1e-6)

    # and both against the FP64 oracle: LJ + Ewald real space + PME (same grid)
    # + the excluded-pair correction
    t = w.topology
    q = t.charges.reshape(-1)
    f64 = (orc.nonbonded(pos, 30.0, water_lj_rows(w), q, t.bonded_particles,
                         t.scaling_particles, 12.0, coulomb="ewald", beta=beta)[0]
           + orc.pme(pos, 30.0, q, beta, 32, 4)[0]
           + orc.ewald_exclusions(pos, 30.0, q, t.bonded_particles, beta)[0])
    err = rel_rms(f_ref, f64)
    print("reference Ensemble + libmdg constraint: force rel RMS vs FP64 %.2e" % err)
    assert err <= 1e-5
