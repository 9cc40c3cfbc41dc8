"""Generate the golden vectors in this directory by running the UNMODIFIED
reference (mdpy v0.2.1) on the CPU.

Run in a container that holds the reference source tree (it is not needed
anywhere else -- the fixtures it writes are committed):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/mdpy-reference

The reference needs numba, h5py and MDAnalysis at import time; none is used
on the paths exercised here, so ``oracle/refshim`` supplies import stubs
(``numba.njit`` becomes the identity, which is the reference's own test mode,
mdpy/test/run_test.py:63).  The reference's kernels therefore run as plain
Python/numpy in float32 (mdpy's default SINGLE precision).

Cases (every array is the reference's own output unless noted):

* ``nb4_*``   -- mdpy/test/test_charmm_nonbonded_constraint.py:93-126 set-up
* ``es4_*``   -- mdpy/test/test_electrostatic_constraint.py:197-221 set-up
* ``bond4_*``, ``angle4_*``, ``dih4_*``, ``imp4_*`` -- the bonded tests' set-ups
* ``pbc_*``   -- mdpy/test/test_pbc.py:26-81 inputs and outputs
* ``cl6po6_*`` -- CellList on the 6PO6 coordinates (mdpy/test/test_cell_list.py:41-59);
  the PDB is read with a fixed-column reader instead of MDAnalysis
* ``w900_*``  -- 900 waters / 30 A (3^3 reference cells): LJ, Coulomb, bond and
  angle forces/energies, the reference cell list and the digest of the pair set
  its nonbonded kernel visits
* ``wb900_*`` -- the same waters displaced by N(0, 0.05 A): bond and angle
  forces/energies away from equilibrium
* ``sp50_*``  -- 1500 random LJ atoms (2.8 A hard core) in a 50 A box (4^3 reference cells): the
  reference LJ forces, its cell list and pair-set digest, and the brute-force
  digest (shows the pairs the reference drops across the periodic wrap)
* ``v81_*``   -- one VerletIntegrator step of 27 waters in a 25 A box
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def main(ref_root):
    sys.path[:0] = [REPO, os.path.join(REPO, "oracle", "refshim"), ref_root]
    if not hasattr(np, "round_"):  # numpy 2 dropped it; mdpy/utils/pbc.py:42 calls it
        np.round_ = np.round
    import mdpy
    from mdpy import env
    from mdpy.core import Particle, Topology, CellList
    from mdpy.ensemble import Ensemble
    from mdpy.constraint import (CharmmNonbondedConstraint, ElectrostaticConstraint,
                                 CharmmBondConstraint, CharmmAngleConstraint,
                                 CharmmDihedralConstraint, CharmmImproperConstraint)
    from mdpy.integrator import VerletIntegrator
    from mdpy.io import CharmmTopparParser
    from mdpy.unit import Quantity, nanometer
    from mdpy.utils import wrap_positions, unwrap_vec
    from oracle import oracle as O
    from mdpy_gb300 import systems

    assert env.precision == "SINGLE" and env.platform == "CPU"
    data = os.path.join(ref_root, "mdpy", "test", "data")
    out = {}
    charmm = CharmmTopparParser(os.path.join(data, "toppar_water_ions_namd.str"),
                                os.path.join(data, "par_all36_prot.prm"),
                                os.path.join(data, "top_all36_na.rtf"))
    params = charmm.parameters

    def four(types, masses, charges):
        t = Topology()
        t.add_particles([Particle(particle_id=i, particle_type=ty, particle_name=ty,
                                  molecule_type="ASN", mass=m, charge=c)
                         for i, (ty, m, c) in enumerate(zip(types, masses, charges))])
        return t

    # -- nonbonded 4-atom (test_charmm_nonbonded_constraint.py:26-66, 93-101)
    t = four(["CA", "NY", "CPT", "CA"], [12, 14, 1, 12], [0, 0, 0, 0])
    p = np.array([[0, 0, 0], [0, 10, 0], [0, 21, 0], [0, 11, 0]], dtype=np.float32)
    ens = Ensemble(t, np.eye(3) * 30)
    ens.state.cell_list.set_cutoff_radius(5)
    ens.state.set_positions(p)
    c = CharmmNonbondedConstraint(params["nonbonded"])
    ens.state.set_pbc_matrix(np.diag(np.ones(3) * 30).astype(np.float32))
    c.set_cutoff_radius(Quantity(0.91, nanometer))
    ens.add_constraints(c)
    ens.state.cell_list.update(ens.state.positions)
    c.update()
    out.update(nb4_positions=ens.state.positions, nb4_params=c._parameters_list,
               nb4_forces=c.forces, nb4_energy=np.float64(c.potential_energy),
               nb4_cutoff=np.float64(c.cutoff_radius), nb4_box=np.float64(30))

    # -- electrostatic 4-atom (test_electrostatic_constraint.py:26-56, 72-94)
    t = four(["C", "N", "CA", "C"], [12, 14, 1, 12], [1, 2, 0, 0])
    ens = Ensemble(t, np.eye(3) * 30)
    ens.state.cell_list.set_cutoff_radius(12)
    ens.state.set_positions(np.array([[0, 0, 0], [0, 10, 0], [0, 21, 0], [0, 11, 0]]))
    c = ElectrostaticConstraint()
    ens.state.set_pbc_matrix(np.diag(np.ones(3) * 100))
    ens.add_constraints(c)
    c.update()
    out.update(es4_positions=ens.state.positions, es4_charges=t.charges,
               es4_forces=c.forces, es4_energy=np.float64(c.potential_energy),
               es4_box=np.float64(100))

    # -- bonded 4-atom cases
    pos4 = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]])

    def bonded_case(types, add, cls, key):
        t = four(types, [12, 14, 1, 12], [0, 0, 0, 0])
        add(t)
        ens = Ensemble(t, np.eye(3) * 30)
        ens.state.cell_list.set_cutoff_radius(12)
        ens.state.set_positions(pos4)
        c = cls(params[key], 0, 0)
        ens.add_constraints(c)
        c.update()
        return ens.state.positions, c._int_parameters, c._float_parameters, c.forces, \
            np.float64(c.potential_energy)

    r = bonded_case(["CA", "N", "HA1", "CA"], lambda t: t.add_bond([0, 3]),
                    CharmmBondConstraint, "bond")
    out.update(zip(["bond4_positions", "bond4_idx", "bond4_prm", "bond4_forces", "bond4_energy"], r))
    r = bonded_case(["CA", "CA", "HA1", "CA"], lambda t: t.add_angle([0, 1, 3]),
                    CharmmAngleConstraint, "angle")
    out.update(zip(["angle4_positions", "angle4_idx", "angle4_prm", "angle4_forces",
                    "angle4_energy"], r))
    r = bonded_case(["CA", "NY", "CPT", "CA"], lambda t: t.add_dihedral([0, 1, 2, 3]),
                    CharmmDihedralConstraint, "dihedral")
    out.update(zip(["dih4_positions", "dih4_idx", "dih4_prm", "dih4_forces", "dih4_energy"], r))
    imp_types = None
    for key in params["improper"]:
        a, b, cc, d = key.split("-")
        if "X" not in (a, b, cc, d):
            imp_types = [a, b, cc, d]
            break
    r = bonded_case(imp_types, lambda t: t.add_improper([0, 1, 2, 3]),
                    CharmmImproperConstraint, "improper")
    out.update(zip(["imp4_positions", "imp4_idx", "imp4_prm", "imp4_forces", "imp4_energy"], r))

    # -- pbc (test_pbc.py)
    pbc = np.diag(np.ones(3) * 10).astype(np.float32)
    pinv = np.linalg.inv(pbc).astype(np.float32)
    wp = np.array([[0, 0, 0], [4, 5, 1], [-4, -1, -5], [6, 8, 9], [8, 0, 1], [-7, -8, 9],
                   [11, 12, 3], [-3, -12., -14]])
    uv = np.array([[0, 9, 0], [0, 1, 0], [9, -1, 0], [0, 1, -8], [0, 6, 1], [-5, -6, 9]],
                  dtype=np.float32)
    out.update(pbc_wrap_in=wp, pbc_wrap_out=wrap_positions(wp, pbc, pinv),
               pbc_unwrap_in=uv, pbc_unwrap_out=unwrap_vec(uv, pbc, pinv))

    # -- cell list on the 6PO6 coordinates (test_cell_list.py:41-59)
    xyz = []
    with open(os.path.join(data, "6PO6.pdb")) as fh:
        for line in fh:
            if line.startswith(("ATOM", "HETATM")):
                xyz.append([float(line[30:38]), float(line[38:46]), float(line[46:54])])
    xyz = np.asarray(xyz, dtype=np.float32)
    cl = CellList(np.diag([30, 30, 30]), 9)
    cl.update(xyz)
    out.update(cl6po6_positions=xyz, cl6po6_cell_index=cl.particle_cell_index,
               cl6po6_cell_list=cl.cell_list, cl6po6_num_cell_vec=cl.num_cell_vec,
               cl6po6_cell_inv=cl.cell_inv)

    # -- 900 waters, 30 A
    def ref_topology(sys_):
        t = Topology()
        tt = sys_.topology
        t.add_particles([Particle(particle_id=i, particle_type=ty, particle_name=ty,
                                  molecule_type="W", mass=float(m), charge=float(q))
                         for i, (ty, m, q) in enumerate(zip(tt.particle_types,
                                                              tt.masses.reshape(-1),
                                                              tt.charges.reshape(-1)))])
        for b in tt.bonds:
            t.add_bond([int(b[0]), int(b[1])])
        for a in tt.angles:
            t.add_angle([int(a[0]), int(a[1]), int(a[2])])
        return t

    w = systems.water_box(900, 30.0, seed=0)
    t = ref_topology(w)
    ens = Ensemble(t, np.eye(3) * 30)
    ens.state.cell_list.set_cutoff_radius(12)
    ens.state.set_positions(w.positions.astype(np.float32))
    cons = {"lj": CharmmNonbondedConstraint(w.parameters["nonbonded"], 12),
            "coul": ElectrostaticConstraint(),
            "bond": CharmmBondConstraint(w.parameters["bond"]),
            "angle": CharmmAngleConstraint(w.parameters["angle"])}
    ens.add_constraints(*cons.values())
    ens.state.cell_list.update(ens.state.positions)
    pos32 = ens.state.positions
    for k, c in cons.items():
        t0 = time.time()
        c.update()
        print("w900 %s: %.1f s" % (k, time.time() - t0), flush=True)
        out["w900_f_" + k] = c.forces
        out["w900_e_" + k] = np.float64(c.potential_energy)
    cl = ens.state.cell_list
    pairs = O.ref_pairs(pos32, np.diag(ens.state.pbc_matrix), 12.0, cl.particle_cell_index,
                        cl.num_cell_vec, t.bonded_particles)
    cnt, deg, dig = O.pair_set_digest(pairs, pos32.shape[0])
    out.update(w900_positions=pos32, w900_cell_index=cl.particle_cell_index,
               w900_num_cell_vec=cl.num_cell_vec, w900_pairs_count=np.int64(cnt),
               w900_pairs_degree=deg, w900_pairs_digest=np.uint64(dig),
               w900_lj_params=cons["lj"]._parameters_list, w900_bonded=t.bonded_particles,
               w900_charges=t.charges, w900_masses=t.masses)

    # -- bonded terms away from equilibrium (the generated waters sit exactly at
    #    r0/theta0, where bond/angle forces are only float32 rounding noise)
    rng = np.random.default_rng(900)
    pert = (pos32 + rng.normal(0.0, 0.05, size=pos32.shape)).astype(np.float32)
    ens.state.set_positions(pert)
    for k in ("bond", "angle"):
        cons[k].update()
        out["wb900_f_" + k] = cons[k].forces
        out["wb900_e_" + k] = np.float64(cons[k].potential_energy)
    out["wb900_positions"] = ens.state.positions

    # -- sparse 50 A box, 4^3 reference cells
    # random sequential addition with a 2.8 A hard core: uniform-random points
    # put pairs far inside the LJ core (forces ~1e11, beyond any physical state)
    rng = np.random.default_rng(50)
    n = 1500
    pts = []
    while len(pts) < n:
        c = rng.uniform(-25, 25, size=3)
        if pts:
            d = np.asarray(pts) - c
            d -= 50.0 * np.round(d / 50.0)
            if np.min(np.einsum("ij,ij->i", d, d)) < 2.8 ** 2:
                continue
        pts.append(c)
    sp = np.asarray(pts).astype(np.float32)
    t = Topology()
    t.add_particles([Particle(particle_id=i, particle_type="OT", particle_name="OT",
                              molecule_type="X", mass=16.0, charge=0.0) for i in range(n)])
    ens = Ensemble(t, np.eye(3) * 50)
    ens.state.cell_list.set_cutoff_radius(12)
    ens.state.set_positions(sp)
    c = CharmmNonbondedConstraint({"OT": [w.parameters["nonbonded"]["OT"][0], 3.1507]}, 12)
    ens.add_constraints(c)
    ens.state.cell_list.update(ens.state.positions)
    t0 = time.time()
    c.update()
    print("sp50 lj: %.1f s" % (time.time() - t0), flush=True)
    cl = ens.state.cell_list
    excl = np.full((n, 1), -1, dtype=np.int32)
    ref_p = O.ref_pairs(ens.state.positions, np.diag(ens.state.pbc_matrix), 12.0,
                        cl.particle_cell_index, cl.num_cell_vec, excl)
    bf_p = O.pairs_bruteforce(ens.state.positions.astype(np.float64), 50.0, 12.0)
    rc_, rdeg, rdig = O.pair_set_digest(ref_p, n)
    bc_, bdeg, bdig = O.pair_set_digest(bf_p, n)
    out.update(sp50_positions=ens.state.positions, sp50_lj_params=c._parameters_list,
               sp50_forces=c.forces, sp50_energy=np.float64(c.potential_energy),
               sp50_cell_index=cl.particle_cell_index, sp50_num_cell_vec=cl.num_cell_vec,
               sp50_ref_count=np.int64(rc_), sp50_ref_digest=np.uint64(rdig),
               sp50_bf_count=np.int64(bc_), sp50_bf_digest=np.uint64(bdig))

    # -- one Verlet step, 27 waters in a 25 A box
    w = systems.water_box(27, 25.0, seed=3)
    t = ref_topology(w)
    ens = Ensemble(t, np.eye(3) * 25)
    ens.state.cell_list.set_cutoff_radius(12)
    ens.state.set_positions(w.positions.astype(np.float32))
    ens.state.set_velocities(w.velocities.astype(np.float32))
    ens.add_constraints(CharmmNonbondedConstraint(w.parameters["nonbonded"], 12),
                        ElectrostaticConstraint(), CharmmBondConstraint(w.parameters["bond"]),
                        CharmmAngleConstraint(w.parameters["angle"]))
    x0 = ens.state.positions.copy()
    v0 = ens.state.velocities.copy()
    VerletIntegrator(1).integrate(ens, 1)
    out.update(v81_positions0=x0, v81_velocities0=v0, v81_positions1=ens.state.positions,
               v81_velocities1=ens.state.velocities)

    out["mdpy_version"] = np.array("0.2.1")
    path = os.path.join(HERE, "reference_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote %s (%d arrays, %.0f KB)" % (path, len(out), os.path.getsize(path) / 1024))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the mdpy v0.2.1 source tree>")
    main(sys.argv[1])
