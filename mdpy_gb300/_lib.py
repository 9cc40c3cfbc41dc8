"""ctypes binding of libmdg (include/mdg.h).

``System`` owns one ``mdg_system``.  Every call checks the returned status
and raises the mdpy-style exception of :mod:`mdpy_gb300.error`.  The shared
library is built in-tree (``python -m mdpy_gb300.build``); if it is missing
the import of this module fails loudly -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .error import status_to_exception

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libmdg.so")

# constants mirrored from include/mdg.h
HOST, DEVICE = 0, 1
TERM_LJ, TERM_COUL_REAL, TERM_COUL_RECIP, TERM_BOND, TERM_ANGLE, TERM_DIHEDRAL, TERM_IMPROPER = range(7)
NUM_TERMS = 7
TERM_NAMES = ("lj", "coulomb_real", "coulomb_recip", "bond", "angle", "dihedral", "improper")
COUL_NONE, COUL_EWALD, COUL_BARE = 0, 1, 2
INTEGRATOR_VERLET, INTEGRATOR_LANGEVIN = 0, 1
MASK_ALL = (1 << NUM_TERMS) - 1
SNAPSHOT_SLOTS = 8


def mask(*terms):
    m = 0
    for t in terms:
        m |= 1 << t
    return m


_c_int_p = ctypes.POINTER(ctypes.c_int)
_c_dbl_p = ctypes.POINTER(ctypes.c_double)
_c_i32_p = ctypes.POINTER(ctypes.c_int32)
_c_i64_p = ctypes.POINTER(ctypes.c_int64)
_c_f32_p = ctypes.POINTER(ctypes.c_float)
_c_u64_p = ctypes.POINTER(ctypes.c_uint64)
_sys_p = ctypes.c_void_p

# name -> argtypes (every function returns int)
SIGNATURES = {
    "mdg_version": [_c_int_p, _c_int_p],
    "mdg_system_create": [ctypes.c_int, ctypes.c_int, _c_dbl_p, ctypes.POINTER(_sys_p)],
    "mdg_system_create_batch": [ctypes.c_int, ctypes.c_int, _c_int_p, _c_dbl_p,
                                ctypes.POINTER(_sys_p)],
    "mdg_num_systems": [_sys_p, _c_int_p],
    "mdg_system_set_boxes": [_sys_p, _c_dbl_p],
    "mdg_pme_config_batch": [_sys_p, _c_int_p, ctypes.c_int, ctypes.c_double],
    "mdg_get_energies_batch": [_sys_p, _c_dbl_p, _c_dbl_p],
    "mdg_system_destroy": [_sys_p],
    "mdg_system_set_stream": [_sys_p, ctypes.c_void_p],
    "mdg_system_set_box": [_sys_p, _c_dbl_p],
    "mdg_set_masses": [_sys_p, _c_dbl_p],
    "mdg_set_charges": [_sys_p, _c_dbl_p],
    "mdg_set_lj": [_sys_p, _c_dbl_p],
    "mdg_set_exclusions": [_sys_p, _c_i32_p, ctypes.c_int, _c_i32_p, ctypes.c_int],
    "mdg_nonbonded_config": [_sys_p, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                             ctypes.c_double],
    "mdg_pme_config": [_sys_p, _c_int_p, ctypes.c_int, ctypes.c_double],
    "mdg_set_reorder_interval": [_sys_p, ctypes.c_int],
    "mdg_set_bonds": [_sys_p, ctypes.c_int, _c_i32_p, _c_dbl_p],
    "mdg_set_angles": [_sys_p, ctypes.c_int, _c_i32_p, _c_dbl_p],
    "mdg_set_dihedrals": [_sys_p, ctypes.c_int, _c_i32_p, _c_dbl_p],
    "mdg_set_impropers": [_sys_p, ctypes.c_int, _c_i32_p, _c_dbl_p],
    "mdg_set_positions": [_sys_p, ctypes.c_void_p, ctypes.c_int],
    "mdg_set_velocities": [_sys_p, ctypes.c_void_p, ctypes.c_int],
    "mdg_get_positions": [_sys_p, ctypes.c_void_p, ctypes.c_int],
    "mdg_get_velocities": [_sys_p, ctypes.c_void_p, ctypes.c_int],
    "mdg_compute_forces": [_sys_p, ctypes.c_uint],
    "mdg_get_forces": [_sys_p, ctypes.c_void_p, ctypes.c_int],
    "mdg_get_energies": [_sys_p, _c_dbl_p, _c_dbl_p],
    "mdg_kinetic_energy": [_sys_p, _c_dbl_p],
    "mdg_energy_snapshot": [_sys_p, ctypes.c_int],
    "mdg_energy_snapshot_read": [_sys_p, ctypes.c_int, ctypes.c_int, _c_dbl_p, _c_dbl_p, _c_int_p],
    "mdg_kinetic_energies_noalloc": [_sys_p, _c_dbl_p],
    "mdg_minimize_step": [_sys_p, ctypes.c_double],
    "mdg_set_mts": [_sys_p, ctypes.c_int],
    "mdg_learned_config": [_sys_p, ctypes.c_double, ctypes.c_double, ctypes.c_int],
    "mdg_learned_num_params": [_c_i32_p],
    "mdg_learned_set_params": [_sys_p, _c_f32_p, ctypes.c_int32],
    "mdg_learned_get_params": [_sys_p, _c_f32_p, ctypes.c_int32],
    "mdg_learned_frame": [_sys_p, ctypes.c_int32],
    "mdg_learned_frame_data": [_sys_p, ctypes.c_int32, _c_f32_p, _c_f32_p, _c_f32_p, _c_f32_p],
    "mdg_learned_train_step": [_sys_p, ctypes.c_float, ctypes.c_int32, _c_dbl_p],
    "mdg_learned_predict": [_sys_p, ctypes.c_int32, _c_f32_p],
    "mdg_set_mts_learned": [_sys_p, ctypes.c_int32, ctypes.c_double],
    "mdg_learned_set_kernel": [_sys_p, ctypes.c_int32],
    "mdg_learned_wait_test": [_sys_p],
    "mdg_learned_set_terms": [_sys_p, ctypes.c_int32, ctypes.c_int32],
    "mdg_learned_stats": [_sys_p, _c_dbl_p],
    "mdg_learned_reset_stats": [_sys_p],
    "mdg_step_host": [_sys_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_uint,
                      ctypes.c_void_p, ctypes.c_void_p, _c_dbl_p, _c_dbl_p],
    "mdg_set_launch_shape": [_sys_p, _c_int_p],
    "mdg_get_launch_shape": [_sys_p, _c_int_p],
    "mdg_autotune": [_sys_p, ctypes.c_uint, ctypes.c_int, _c_dbl_p],
    "mdg_integrator_config": [_sys_p, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                              ctypes.c_double, ctypes.c_uint64],
    "mdg_integrate": [_sys_p, ctypes.c_int, ctypes.c_uint, ctypes.c_int],
    "mdg_get_step": [_sys_p, _c_u64_p],
    "mdg_set_step": [_sys_p, ctypes.c_uint64],
    "mdg_pairset_dump": [_sys_p, _c_i32_p, ctypes.c_int64, _c_i64_p],
    "mdg_langevin_noise": [_sys_p, ctypes.c_uint64, _c_f32_p],
    "mdg_check_status": [_sys_p],
    "mdg_nonbonded_stats": [_sys_p, _c_i64_p],
    "mdg_launch_count": [_sys_p, _c_i64_p],
    "mdg_set_graph_mode": [_sys_p, ctypes.c_int],
    "mdg_launch_stage": [_sys_p, ctypes.c_int, ctypes.c_uint],
}

GRAPH_CHUNK, GRAPH_STEP = 0, 1
STAGE_PACK, STAGE_NONBONDED, STAGE_SPECIAL, STAGE_PME, STAGE_BONDED, STAGE_REORDER, \
    STAGE_INTEGRATE, STAGE_NONBONDED_ENERGY = range(8)

_lib = None


def load():
    """Load libmdg.so; raises ImportError when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libmdg.so not found at %s; build it with `python -m mdpy_gb300.build` "
                          "(this package has no CPU fallback)" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, argtypes in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = ctypes.c_int
    lib.mdg_last_error.argtypes = []
    lib.mdg_last_error.restype = ctypes.c_char_p
    _lib = lib
    return lib


def check(rc):
    if rc != 0:
        msg = load().mdg_last_error().decode("utf-8", "replace")
        raise status_to_exception(rc, msg)


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None and a.shape != tuple(shape):
        a = a.reshape(shape)
    return a


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _dp(a):
    return a.ctypes.data_as(_c_dbl_p)


class System:
    """One device-resident MD system (``mdg_system``).

    ``System.batch(n_atoms_list, boxes)`` makes a batch of independent
    systems that share one set of launches: per-atom arrays are the systems'
    arrays concatenated in order, and ``get_energies_batch`` reports each
    system's energies."""

    def __init__(self, n_atoms, box, device=0, _batch=None):
        self._lib = load()
        self.device = int(device)
        h = _sys_p()
        if _batch is None:
            self.n = int(n_atoms)
            self.n_systems = 1
            self.atoms_per_system = np.array([self.n], dtype=np.int64)
            box = _f64(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
            check(self._lib.mdg_system_create(self.device, self.n, _dp(box), ctypes.byref(h)))
        else:
            counts = np.ascontiguousarray(_batch[0], dtype=np.int32).reshape(-1)
            boxes = _f64(np.broadcast_to(np.asarray(_batch[1], dtype=np.float64),
                                         (counts.size, 3)))
            self.n = int(counts.sum())
            self.n_systems = int(counts.size)
            self.atoms_per_system = counts.astype(np.int64)
            check(self._lib.mdg_system_create_batch(
                self.device, self.n_systems, counts.ctypes.data_as(_c_int_p), _dp(boxes),
                ctypes.byref(h)))
        self._h = h

    @classmethod
    def batch(cls, n_atoms, boxes, device=0):
        return cls(None, None, device=device, _batch=(n_atoms, boxes))

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mdg_system_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    # -- configuration ----------------------------------------------------
    def set_stream(self, stream_ptr):
        check(self._lib.mdg_system_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)))

    def set_box(self, box):
        box = _f64(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
        check(self._lib.mdg_system_set_box(self._h, _dp(box)))

    def set_boxes(self, boxes):
        boxes = _f64(np.broadcast_to(np.asarray(boxes, dtype=np.float64), (self.n_systems, 3)))
        check(self._lib.mdg_system_set_boxes(self._h, _dp(boxes)))

    def set_masses(self, m):
        m = _f64(m).reshape(-1)
        check(self._lib.mdg_set_masses(self._h, _dp(m)))

    def set_charges(self, q):
        q = _f64(q).reshape(-1)
        check(self._lib.mdg_set_charges(self._h, _dp(q)))

    def set_lj(self, params):
        p = _f64(params).reshape(self.n, 4)
        check(self._lib.mdg_set_lj(self._h, _dp(p)))

    def set_exclusions(self, bonded, scaling):
        b = _i32(np.asarray(bonded).reshape(self.n, -1))
        s = _i32(np.asarray(scaling).reshape(self.n, -1))
        check(self._lib.mdg_set_exclusions(self._h, b.ctypes.data_as(_c_i32_p), b.shape[1],
                                           s.ctypes.data_as(_c_i32_p), s.shape[1]))

    def nonbonded_config(self, cutoff, switch_radius=0.0, lj=True, coulomb=COUL_NONE, beta=0.0):
        check(self._lib.mdg_nonbonded_config(self._h, float(cutoff), float(switch_radius or 0.0),
                                             int(bool(lj)), int(coulomb), float(beta)))

    def pme_config(self, grid, order, beta):
        g = (ctypes.c_int * 3)(*[int(k) for k in np.broadcast_to(np.asarray(grid), (3,))])
        check(self._lib.mdg_pme_config(self._h, g, int(order), float(beta)))

    def set_reorder_interval(self, steps):
        check(self._lib.mdg_set_reorder_interval(self._h, int(steps)))

    def _terms(self, fn, idx, prm, wi, wp):
        idx = _i32(np.asarray(idx).reshape(-1, wi))
        prm = _f64(np.asarray(prm, dtype=np.float64).reshape(-1, wp))
        if idx.shape[0] != prm.shape[0]:
            raise ValueError("index and parameter rows differ")
        check(fn(self._h, idx.shape[0], idx.ctypes.data_as(_c_i32_p), _dp(prm)))

    def set_bonds(self, idx, prm):
        self._terms(self._lib.mdg_set_bonds, idx, prm, 2, 2)

    def set_angles(self, idx, prm):
        self._terms(self._lib.mdg_set_angles, idx, prm, 3, 4)

    def set_dihedrals(self, idx, prm):
        self._terms(self._lib.mdg_set_dihedrals, idx, prm, 4, 3)

    def set_impropers(self, idx, prm):
        self._terms(self._lib.mdg_set_impropers, idx, prm, 4, 2)

    def integrator_config(self, kind, dt, temperature=0.0, friction=0.0, seed=0):
        check(self._lib.mdg_integrator_config(self._h, int(kind), float(dt), float(temperature),
                                              float(friction), ctypes.c_uint64(int(seed))))

    # -- state ------------------------------------------------------------
    def set_positions(self, x):
        x = _f64(x).reshape(self.n, 3)
        check(self._lib.mdg_set_positions(self._h, x.ctypes.data, HOST))

    def set_positions_ptr(self, ptr, where=DEVICE):
        check(self._lib.mdg_set_positions(self._h, ctypes.c_void_p(ptr), int(where)))

    def set_velocities(self, v):
        v = _f64(v).reshape(self.n, 3)
        check(self._lib.mdg_set_velocities(self._h, v.ctypes.data, HOST))

    def set_velocities_ptr(self, ptr, where=DEVICE):
        check(self._lib.mdg_set_velocities(self._h, ctypes.c_void_p(ptr), int(where)))

    def get_positions(self, out=None):
        out = np.empty((self.n, 3)) if out is None else out
        check(self._lib.mdg_get_positions(self._h, out.ctypes.data, HOST))
        return out

    def get_positions_ptr(self, ptr, where=DEVICE):
        check(self._lib.mdg_get_positions(self._h, ctypes.c_void_p(ptr), int(where)))

    def get_velocities(self, out=None):
        out = np.empty((self.n, 3)) if out is None else out
        check(self._lib.mdg_get_velocities(self._h, out.ctypes.data, HOST))
        return out

    def get_velocities_ptr(self, ptr, where=DEVICE):
        check(self._lib.mdg_get_velocities(self._h, ctypes.c_void_p(ptr), int(where)))

    # -- forces / energies -------------------------------------------------
    def compute_forces(self, term_mask=MASK_ALL):
        check(self._lib.mdg_compute_forces(self._h, int(term_mask)))

    def get_forces(self, out=None):
        out = np.empty((self.n, 3)) if out is None else out
        check(self._lib.mdg_get_forces(self._h, out.ctypes.data, HOST))
        return out

    def pme_config_batch(self, grids, order, beta):
        g = np.ascontiguousarray(np.broadcast_to(np.asarray(grids, dtype=np.int32),
                                                 (self.n_systems, 3)))
        check(self._lib.mdg_pme_config_batch(self._h, g.ctypes.data_as(_c_int_p), int(order),
                                             float(beta)))

    def get_energies_batch(self):
        """(n_systems, NUM_TERMS) energies and (n_systems,) kinetic energies."""
        e = np.zeros((self.n_systems, NUM_TERMS))
        ke = np.zeros(self.n_systems)
        check(self._lib.mdg_get_energies_batch(self._h, _dp(e), _dp(ke)))
        return e, ke

    def get_energies(self):
        e = np.zeros(NUM_TERMS)
        ke = ctypes.c_double(0.0)
        check(self._lib.mdg_get_energies(self._h, _dp(e), ctypes.byref(ke)))
        return e, ke.value

    def energy_snapshot(self, slot):
        """Enqueue a copy of the current energies into pinned slot ``slot``
        (no synchronisation)."""
        check(self._lib.mdg_energy_snapshot(self._h, int(slot)))

    def energy_snapshot_read(self, slot, wait=True):
        """(energies, kinetic) of snapshot ``slot``; with ``wait=False``
        None if its copy has not completed yet."""
        e = np.zeros(NUM_TERMS)
        ke = ctypes.c_double(0.0)
        ready = ctypes.c_int(0)
        check(self._lib.mdg_energy_snapshot_read(self._h, int(slot), 1 if wait else 0, _dp(e),
                                                 ctypes.byref(ke), ctypes.byref(ready)))
        return (e, ke.value) if ready.value else None

    SHAPE_FIELDS = ("split", "persistent", "pme_block", "side_priority", "split_rings",
                    "pme_tiles", "half")

    def set_launch_shape(self, split=4, persistent=0, pme_block=256, side_priority=0,
                         split_rings=1, pme_tiles=0, half=0):
        """``persistent``: 0 = one CTA per pair work item, n = n resident CTAs
        per SM pulling work items; ``pme_tiles``: bit 0 tiled spreading, bit 1
        tiled gathering; ``half``: 16-atom i groups per half warp."""
        sh = (ctypes.c_int * 7)(int(split), int(persistent), int(pme_block), int(side_priority),
                                int(split_rings), int(pme_tiles), int(half))
        check(self._lib.mdg_set_launch_shape(self._h, sh))

    @property
    def launch_shape(self):
        sh = (ctypes.c_int * 7)()
        check(self._lib.mdg_get_launch_shape(self._h, sh))
        return dict(zip(self.SHAPE_FIELDS, list(sh)))

    def autotune(self, term_mask=MASK_ALL, reps=10):
        """Pick the fastest launch shape (MD steps when an integrator is
        configured, force evaluations otherwise); returns the shape and its
        time (ms per step or evaluation)."""
        best = ctypes.c_double(0.0)
        check(self._lib.mdg_autotune(self._h, int(term_mask), int(reps), ctypes.byref(best)))
        return dict(self.launch_shape, tuned_ms=best.value)

    def step_host_ptr(self, x_in, v_in, n_steps, term_mask, x_out, v_out, energies=None,
                      want_kinetic=True):
        """mdg_step_host with raw host addresses (0 = skip); ``energies``: a
        float64 array of NUM_TERMS or None.  Returns the kinetic energy."""
        ke = ctypes.c_double(0.0)
        check(self._lib.mdg_step_host(
            self._h, ctypes.c_void_p(x_in or None), ctypes.c_void_p(v_in or None), int(n_steps),
            int(term_mask), ctypes.c_void_p(x_out or None), ctypes.c_void_p(v_out or None),
            None if energies is None else _dp(energies),
            ctypes.byref(ke) if want_kinetic else None))
        return ke.value

    def set_mts(self, k):
        """Reciprocal-space force every k-th step, weighted k (impulse MTS)."""
        check(self._lib.mdg_set_mts(self._h, int(k)))

    # ---- learned slow force -------------------------------------------------
    @staticmethod
    def learned_num_params():
        n = ctypes.c_int32(0)
        check(load().mdg_learned_num_params(ctypes.byref(n)))
        return n.value

    def learned_config(self, rf=6.0, skin=1.0, list_capacity=256):
        check(self._lib.mdg_learned_config(self._h, float(rf), float(skin), int(list_capacity)))

    def learned_set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32).ravel()
        check(self._lib.mdg_learned_set_params(self._h, p.ctypes.data_as(_c_f32_p), p.size))

    def learned_params(self):
        p = np.zeros(self.learned_num_params(), dtype=np.float32)
        check(self._lib.mdg_learned_get_params(self._h, p.ctypes.data_as(_c_f32_p), p.size))
        return p

    def learned_frame(self, slot):
        check(self._lib.mdg_learned_frame(self._h, int(slot)))

    def learned_frame_data(self, slot):
        """(features n x 64, vectors n x 16 x 3, slow force n x 3, prediction n x 3)"""
        n = self.n
        feat = np.zeros((n, 64), dtype=np.float32)
        vec = np.zeros((n, 16, 3), dtype=np.float32)
        slow = np.zeros((n, 3), dtype=np.float32)
        pred = np.zeros((n, 3), dtype=np.float32)
        check(self._lib.mdg_learned_frame_data(
            self._h, int(slot), feat.ctypes.data_as(_c_f32_p), vec.ctypes.data_as(_c_f32_p),
            slow.ctypes.data_as(_c_f32_p), pred.ctypes.data_as(_c_f32_p)))
        return feat, vec, slow, pred

    def learned_predict(self, slot=0):
        """G (n x 3) of the inference kernel on the features of a frame"""
        out = np.zeros((self.n, 3), dtype=np.float32)
        check(self._lib.mdg_learned_predict(self._h, int(slot), out.ctypes.data_as(_c_f32_p)))
        return out

    def learned_train_step(self, lr, t):
        loss = ctypes.c_double(0.0)
        check(self._lib.mdg_learned_train_step(self._h, float(lr), int(t), ctypes.byref(loss)))
        return loss.value

    def set_mts_learned(self, k, threshold=1e-3):
        check(self._lib.mdg_set_mts_learned(self._h, int(k), float(threshold)))

    def learned_set_kernel(self, tensor_cores):
        check(self._lib.mdg_learned_set_kernel(self._h, int(bool(tensor_cores))))

    def learned_wait_test(self):
        """Arm the one-shot test of the tcgen05 kernel's bounded waits (its
        next launch gives up on its first wait and reports a timeout)."""
        check(self._lib.mdg_learned_wait_test(self._h))

    def learned_set_terms(self, field_gradient=True, network=True):
        check(self._lib.mdg_learned_set_terms(self._h, int(bool(field_gradient)),
                                              int(bool(network))))

    def learned_stats(self):
        out = np.zeros(8)
        check(self._lib.mdg_learned_stats(self._h, _dp(out)))
        return {"last_err": out[0], "max_err": out[1],
                "mean_err": out[2] / out[3] if out[3] else 0.0, "judged": int(out[3]),
                "fallbacks": int(out[4]), "loss": out[5], "target_norm": out[6],
                "mode": "impulse" if out[7] else "learned"}

    def learned_reset_stats(self):
        check(self._lib.mdg_learned_reset_stats(self._h))

    def minimize_step(self, alpha):
        check(self._lib.mdg_minimize_step(self._h, float(alpha)))

    def kinetic_energy(self):
        ke = ctypes.c_double(0.0)
        check(self._lib.mdg_kinetic_energy(self._h, ctypes.byref(ke)))
        return ke.value

    def integrate(self, n_steps, term_mask=MASK_ALL, want_energy=True):
        check(self._lib.mdg_integrate(self._h, int(n_steps), int(term_mask), int(bool(want_energy))))

    @property
    def step(self):
        v = ctypes.c_uint64(0)
        check(self._lib.mdg_get_step(self._h, ctypes.byref(v)))
        return v.value

    @step.setter
    def step(self, value):
        check(self._lib.mdg_set_step(self._h, ctypes.c_uint64(int(value))))

    # -- diagnostics --------------------------------------------------------
    def pairset(self, capacity=None):
        cap = int(capacity) if capacity is not None else max(1 << 20, self.n * 800)
        while True:
            buf = np.empty((cap, 2), dtype=np.int32)
            cnt = ctypes.c_int64(0)
            rc = self._lib.mdg_pairset_dump(self._h, buf.ctypes.data_as(_c_i32_p), cap,
                                            ctypes.byref(cnt))
            if rc == 10 and cnt.value > cap:   # MDG_ERR_CAPACITY
                cap = int(cnt.value)
                continue
            check(rc)
            return buf[:cnt.value]

    def langevin_noise(self, step):
        out = np.empty((self.n, 3), dtype=np.float32)
        check(self._lib.mdg_langevin_noise(self._h, ctypes.c_uint64(int(step)),
                                           out.ctypes.data_as(_c_f32_p)))
        return out

    def check_status(self):
        check(self._lib.mdg_check_status(self._h))

    def nonbonded_stats(self):
        v = np.zeros(4, dtype=np.int64)
        check(self._lib.mdg_nonbonded_stats(self._h, v.ctypes.data_as(_c_i64_p)))
        return {"pair_evaluations": int(v[0]), "pairs_in_cutoff": int(v[1]),
                "cluster_candidates": int(v[2]), "clusters": int(v[3])}

    def set_graph_mode(self, mode):
        check(self._lib.mdg_set_graph_mode(self._h, int(mode)))

    def launch_stage(self, stage, term_mask=MASK_ALL):
        check(self._lib.mdg_launch_stage(self._h, int(stage), int(term_mask)))

    @property
    def launch_count(self):
        v = ctypes.c_int64(0)
        check(self._lib.mdg_launch_count(self._h, ctypes.byref(v)))
        return v.value
