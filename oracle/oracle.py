"""CPU oracle for the force-and-step path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
and reference arms may import this module, and only as the checker (or as
the timed CPU restatement of the reference).  The shipped package never
imports it and has no CPU fallback.

Layers:

* ``mdg_oracle.c`` (built into ``oracle/_build/liborc.so`` by :func:`build`):
  FP64 pair sums, direct Ewald, PME spread/gather, bonded terms, and the
  reference's own cell-list pair enumeration; see that file's header for
  the reference file:line each function restates.
* numpy here: PME convolution (``numpy.fft``, FP64), the influence function,
  the Ewald parameter choice, and one integrator step in FP64.

Pinning: ``tests/test_oracle_golden.py`` checks these functions against
golden vectors produced by running the unmodified reference (mdpy v0.2.1)
in the development container (``tests/golden/make_golden.py``) and against
the reference tests' own known answers.  Ewald/PME/switching have no
reference implementation; those functions are pinned only by mathematics
(finite differences, the Madelung constant, PME-vs-direct convergence).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "liborc.so")
_lib = None
_lock = threading.Lock()

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)


def build(force=False):
    """Compile mdg_oracle.c with gcc (OpenMP when available)."""
    src = os.path.join(_HERE, "mdg_oracle.c")
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(src)):
        return _LIB_PATH
    os.makedirs(_BUILD, exist_ok=True)
    tmp = _LIB_PATH + ".%d.tmp" % os.getpid()
    # -ffp-contract=off: the float32 restatements round every operation as
    # the reference does, on x86 and on Arm (where gcc would fuse a*b+c)
    base = ["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11", "-o", tmp, src,
            "-lm"]
    try:
        subprocess.run(base[:1] + ["-fopenmp"] + base[1:], check=True, capture_output=True)
    except subprocess.CalledProcessError:
        subprocess.run(base, check=True, capture_output=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            L.orc_pairs_bruteforce_ref32.restype = ctypes.c_long
            L.orc_pairs_bruteforce_ref32.argtypes = [_fp, ctypes.c_int, _fp, ctypes.c_float, _ip,
                                                     ctypes.c_int, _ip, ctypes.c_long]
            L.orc_ref_pairs.restype = ctypes.c_long
            L.orc_ref_pairs.argtypes = [_fp, ctypes.c_int, _fp, ctypes.c_float, _ip, _ip, _ip,
                                        ctypes.c_int, _ip, ctypes.c_long]
            L.orc_pairs_bruteforce.restype = ctypes.c_long
            L.orc_pairs_bruteforce.argtypes = [_dp, ctypes.c_int, _dp, ctypes.c_double, _ip,
                                               ctypes.c_long]
            L.orc_ref_cell_index.argtypes = [_fp, ctypes.c_int, _fp, ctypes.c_float,
                                             ctypes.c_float, _ip, _ip]
            for name in ("orc_ewald_recip", "orc_ewald_exclusions", "orc_bonds", "orc_angles",
                         "orc_dihedrals", "orc_impropers"):
                getattr(L, name).restype = ctypes.c_double
            _lib = L
    return _lib


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_dp)


def _f(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(_fp)


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(_ip)


def num_threads():
    return lib().orc_num_threads()


def set_threads(n):
    lib().orc_set_threads(int(n))


# --------------------------------------------------------------------------
# reference cell list and pair enumeration
# --------------------------------------------------------------------------
def ref_cell_index(positions_f32, pbc_diag, cutoff, skin=2.0):
    """(num_cell_vec, particle_cell_index) as mdpy's CellList computes them
    (mdpy/core/cell_list.py:74-116)."""
    pos, pp = _f(positions_f32)
    diag, dp_ = _f(pbc_diag)
    ncv = np.zeros(3, dtype=np.int32)
    idx = np.zeros((pos.shape[0], 3), dtype=np.int32)
    lib().orc_ref_cell_index(pp, pos.shape[0], dp_, cutoff, skin,
                             ncv.ctypes.data_as(_ip), idx.ctypes.data_as(_ip))
    return ncv, idx


def ref_pairs(positions_f32, pbc_diag, cutoff, cell_index, num_cell_vec, exclusions):
    """Unordered pairs (i<j) the reference's nonbonded kernel visits with
    r <= rc (mdpy/constraint/charmm_nonbonded_constraint.py:75-90)."""
    pos, pp = _f(positions_f32)
    diag, dp_ = _f(pbc_diag)
    ci, cip = _i(cell_index)
    ncv, ncvp = _i(num_cell_vec)
    ex, exp_ = _i(exclusions)
    width = ex.shape[1] if ex.ndim == 2 else 0
    n = pos.shape[0]
    cap = 1 << 16
    while True:
        out = np.zeros((cap, 2), dtype=np.int32)
        got = lib().orc_ref_pairs(pp, n, dp_, cutoff, cip, ncvp, exp_, width,
                                  out.ctypes.data_as(_ip), cap)
        if got <= cap:
            return out[:got]
        cap = int(got)


def pairs_bruteforce_ref32(positions_f32, pbc_diag, cutoff, exclusions):
    """All unordered non-excluded pairs (i<j) that pass the reference's own
    float32 pair test (mdg_oracle.c:ref_within32), over all pairs."""
    pos, pp = _f(positions_f32)
    diag, dp_ = _f(pbc_diag)
    ex, exp_ = _i(exclusions)
    width = ex.shape[1] if ex.ndim == 2 else 0
    cap = 1 << 16
    while True:
        out = np.zeros((cap, 2), dtype=np.int32)
        got = lib().orc_pairs_bruteforce_ref32(pp, pos.shape[0], dp_, cutoff, exp_, width,
                                               out.ctypes.data_as(_ip), cap)
        if got <= cap:
            return out[:got]
        cap = int(got)


def pairs_bruteforce(positions, box, cutoff):
    """All unordered minimum-image pairs with r <= cutoff (FP64)."""
    pos, pp = _d(positions)
    bx, bp = _d(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
    cap = 1 << 16
    while True:
        out = np.zeros((cap, 2), dtype=np.int32)
        got = lib().orc_pairs_bruteforce(pp, pos.shape[0], bp, cutoff,
                                         out.ctypes.data_as(_ip), cap)
        if got <= cap:
            return out[:got]
        cap = int(got)


def pair_keys(pairs, n):
    """Sorted int64 keys i*n+j of unordered pairs (i<j)."""
    p = np.asarray(pairs, dtype=np.int64)
    lo, hi = np.minimum(p[:, 0], p[:, 1]), np.maximum(p[:, 0], p[:, 1])
    return np.sort(lo * n + hi)


def pair_set_digest(pairs, n):
    """Order-independent digest of a pair set: (count, per-atom degree,
    64-bit sum of splitmix64(key))."""
    keys = pair_keys(pairs, n).astype(np.uint64)
    z = keys + np.uint64(0x9E3779B97F4A7C15)
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    z = z ^ (z >> np.uint64(31))
    digest = int(np.sum(z, dtype=np.uint64))
    p = np.asarray(pairs, dtype=np.int64)
    degree = np.bincount(p.reshape(-1), minlength=n).astype(np.int32)
    return len(keys), degree, digest


# --------------------------------------------------------------------------
# nonbonded, Ewald, PME
# --------------------------------------------------------------------------
def nonbonded(positions, box, params, charges, exclusions, scaling, cutoff, *,
              switch=None, lj=True, coulomb="none", beta=0.0, kcoul=None, rows=None):
    """FP64 LJ / Coulomb forces and energies; ``coulomb`` in
    {'none', 'ewald', 'bare'} (see mdg_oracle.c:orc_nonbonded).  With ``rows``
    (atom indices) only those atoms' forces are computed and returned, in
    that order (orc_nonbonded_rows); energies then count only their pairs."""
    from mdpy_gb300 import unit as U

    kc = U.COULOMB_K if kcoul is None else kcoul
    pos, pp = _d(positions)
    n = pos.shape[0]
    bx, bp = _d(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
    prm, prp = _d(np.asarray(params, dtype=np.float64).reshape(n, 4))
    q, qp = _d(np.asarray(charges, dtype=np.float64).reshape(n))
    ex, exp_ = _i(np.asarray(exclusions).reshape(n, -1))
    sc, scp = _i(np.asarray(scaling).reshape(n, -1))
    e = np.zeros(2)
    mode = {"none": 0, "ewald": 1, "bare": 2}[coulomb]
    args = (pp, n, bp, prp, qp, exp_, ex.shape[1], scp, sc.shape[1], ctypes.c_double(cutoff),
            ctypes.c_double(switch or 0.0), int(switch is not None), int(bool(lj)), mode,
            ctypes.c_double(beta), ctypes.c_double(kc))
    if rows is None:
        f = np.zeros((n, 3))
        lib().orc_nonbonded(*args, f.ctypes.data_as(_dp), e.ctypes.data_as(_dp))
    else:
        rw, rwp = _i(np.asarray(rows).reshape(-1))
        if rw.size and (rw.min() < 0 or rw.max() >= n):
            raise IndexError("rows outside 0..%d" % (n - 1))
        f = np.zeros((rw.size, 3))
        lib().orc_nonbonded_rows(*args, rwp, rw.size, f.ctypes.data_as(_dp),
                                 e.ctypes.data_as(_dp))
    return f, {"lj": e[0], "coulomb": e[1]}


def ewald_beta(cutoff, tolerance):
    """beta with erfc(beta rc) ~ tolerance: beta = sqrt(-ln(2 tol)) / rc."""
    return math.sqrt(-math.log(2.0 * tolerance)) / cutoff


def ewald_recip(positions, box, charges, beta, nmax, kcoul=None, subset=None):
    """Direct reciprocal k-sum; with ``subset`` (atom indices) the forces are
    returned only for those atoms (the structure factors still use all)."""
    from mdpy_gb300 import unit as U

    kc = U.COULOMB_K if kcoul is None else kcoul
    pos, pp = _d(positions)
    n = pos.shape[0]
    bx, bp = _d(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
    q, qp = _d(np.asarray(charges).reshape(n))
    nm, nmp = _i(np.broadcast_to(np.asarray(nmax), (3,)))
    if subset is None:
        sub, sp, ns = None, None, 0
        f = np.zeros((n, 3))
    else:
        sub, sp = _i(np.asarray(subset).reshape(-1))
        ns = sub.shape[0]
        f = np.zeros((ns, 3))
    e = lib().orc_ewald_recip(pp, n, bp, qp, ctypes.c_double(beta), nmp, ctypes.c_double(kc),
                              f.ctypes.data_as(_dp), sp, ns)
    return f, e


def ewald_kmax(box, beta, eps=1e-12):
    """Integer cut-off per axis so every dropped term has exp(-pi^2 m^2/beta^2) < eps."""
    mmax = beta * math.sqrt(-math.log(eps)) / math.pi
    return [int(math.ceil(mmax * L)) for L in np.broadcast_to(np.asarray(box, float), (3,))]


def ewald_exclusions(positions, box, charges, exclusions, beta, kcoul=None):
    from mdpy_gb300 import unit as U

    kc = U.COULOMB_K if kcoul is None else kcoul
    pos, pp = _d(positions)
    n = pos.shape[0]
    bx, bp = _d(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
    q, qp = _d(np.asarray(charges).reshape(n))
    ex, exp_ = _i(np.asarray(exclusions).reshape(n, -1))
    f = np.zeros((n, 3))
    e = lib().orc_ewald_exclusions(pp, n, bp, qp, exp_, ex.shape[1], ctypes.c_double(beta),
                                   ctypes.c_double(kc), f.ctypes.data_as(_dp))
    return f, e


def ewald_self(charges, beta, kcoul=None):
    from mdpy_gb300 import unit as U

    kc = U.COULOMB_K if kcoul is None else kcoul
    q = np.asarray(charges, dtype=np.float64).reshape(-1)
    return -kc * beta / math.sqrt(math.pi) * float(np.dot(q, q))


def ewald_net_charge(charges, box, beta, kcoul=None):
    from mdpy_gb300 import unit as U

    kc = U.COULOMB_K if kcoul is None else kcoul
    Q = float(np.sum(np.asarray(charges, dtype=np.float64)))
    V = float(np.prod(np.broadcast_to(np.asarray(box, float), (3,))))
    return -kc * math.pi * Q * Q / (2.0 * beta * beta * V)


def bspline_moduli(K, order):
    out = np.zeros(K)
    lib().orc_bspline_moduli(int(K), int(order), out.ctypes.data_as(_dp))
    return out


def pme_influence(K, box, beta, order):
    """G(m) = exp(-pi^2 m^2/beta^2) / (pi V m^2) / prod_d |sum_k M_p(k+1) e^{2 pi i m_d k/K_d}|^2
    on the numpy rfftn half-spectrum, G(0) = 0."""
    K = list(np.broadcast_to(np.asarray(K), (3,)))
    box = np.broadcast_to(np.asarray(box, float), (3,))
    V = float(np.prod(box))
    mods = [bspline_moduli(k, order) for k in K]
    idx = [np.fft.fftfreq(K[0], 1.0 / K[0]), np.fft.fftfreq(K[1], 1.0 / K[1]),
           np.arange(K[2] // 2 + 1)]
    m0 = idx[0][:, None, None] / box[0]
    m1 = idx[1][None, :, None] / box[1]
    m2 = idx[2][None, None, :] / box[2]
    msq = m0 ** 2 + m1 ** 2 + m2 ** 2
    msq[0, 0, 0] = 1.0
    den = (mods[0][:, None, None] * mods[1][None, :, None]
           * mods[2][None, None, :K[2] // 2 + 1])
    G = np.exp(-math.pi ** 2 * msq / beta ** 2) / (math.pi * V * msq) / den
    G[0, 0, 0] = 0.0
    return G


def pme(positions, box, charges, beta, K, order=4, kcoul=None):
    """FP64 smooth PME reciprocal forces and energy (Essmann et al. 1995)."""
    from mdpy_gb300 import unit as U

    kc = U.COULOMB_K if kcoul is None else kcoul
    K = [int(k) for k in np.broadcast_to(np.asarray(K), (3,))]
    pos, pp = _d(positions)
    n = pos.shape[0]
    bx, bp = _d(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
    q, qp = _d(np.asarray(charges).reshape(n))
    Ka, Kp = _i(np.asarray(K))
    grid = np.zeros(K)
    lib().orc_pme_spread(pp, n, bp, qp, Kp, int(order), grid.ctypes.data_as(_dp))
    F = np.fft.rfftn(grid)
    G = pme_influence(K, bx, beta, order)
    w = np.full(K[2] // 2 + 1, 2.0)
    w[0] = 1.0
    if K[2] % 2 == 0:
        w[-1] = 1.0
    energy = 0.5 * kc * float(np.sum(w[None, None, :] * G * np.abs(F) ** 2))
    phi = np.fft.irfftn(G * F, s=K, axes=(0, 1, 2)) * float(np.prod(K))
    phi = np.ascontiguousarray(phi)
    f = np.zeros((n, 3))
    lib().orc_pme_gather(pp, n, bp, qp, Kp, int(order), phi.ctypes.data_as(_dp),
                         ctypes.c_double(kc), f.ctypes.data_as(_dp))
    return f, energy


def ewald_direct(positions, box, charges, exclusions, beta, cutoff, eps=1e-12, kcoul=None):
    """Complete FP64 Ewald electrostatics with 1-2/1-3 exclusions:
    real space (non-excluded pairs, erfc, r <= cutoff) + reciprocal k-sum +
    exclusion correction + self + net-charge terms."""
    n = np.asarray(positions).shape[0]
    zeros4 = np.zeros((n, 4))
    f_real, e_real = nonbonded(positions, box, zeros4, charges, exclusions,
                               np.full((n, 1), -1), cutoff, lj=False, coulomb="ewald",
                               beta=beta, kcoul=kcoul)
    f_rec, e_rec = ewald_recip(positions, box, charges, beta, ewald_kmax(box, beta, eps), kcoul)
    f_ex, e_ex = ewald_exclusions(positions, box, charges, exclusions, beta, kcoul)
    e_self = ewald_self(charges, beta, kcoul)
    e_net = ewald_net_charge(charges, box, beta, kcoul)
    return {
        "forces": f_real + f_rec + f_ex,
        "f_real": f_real, "f_recip": f_rec, "f_excl": f_ex,
        "e_real": e_real["coulomb"], "e_recip": e_rec, "e_excl": e_ex,
        "e_self": e_self, "e_net": e_net,
        "energy": e_real["coulomb"] + e_rec + e_ex + e_self + e_net,
    }


# --------------------------------------------------------------------------
# bonded terms
# --------------------------------------------------------------------------
def _bonded(fn, positions, box, idx, prm, width_i, width_p):
    pos, pp = _d(positions)
    n = pos.shape[0]
    bx, bp = _d(np.broadcast_to(np.asarray(box, dtype=np.float64), (3,)))
    ii, ip = _i(np.asarray(idx).reshape(-1, width_i))
    pr, prp = _d(np.asarray(prm).reshape(-1, width_p))
    f = np.zeros((n, 3))
    e = fn(pp, bp, ip, prp, ii.shape[0], f.ctypes.data_as(_dp))
    return f, e


def bonds(positions, box, idx, prm):
    return _bonded(lib().orc_bonds, positions, box, idx, prm, 2, 2)


def angles(positions, box, idx, prm):
    return _bonded(lib().orc_angles, positions, box, idx, prm, 3, 4)


def dihedrals(positions, box, idx, prm):
    return _bonded(lib().orc_dihedrals, positions, box, idx, prm, 4, 3)


def impropers(positions, box, idx, prm):
    return _bonded(lib().orc_impropers, positions, box, idx, prm, 4, 2)


# --------------------------------------------------------------------------
# RNG and integrators
# --------------------------------------------------------------------------
def philox4x32(counter, key):
    c = (ctypes.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in counter])
    k = (ctypes.c_uint32 * 2)(*[int(x) & 0xFFFFFFFF for x in key])
    o = (ctypes.c_uint32 * 4)()
    lib().orc_philox4x32(c, k, o)
    return list(o)


def langevin_noise(n, seed, step):
    out = np.zeros((n, 3), dtype=np.float32)
    lib().orc_langevin_noise(int(n), ctypes.c_uint64(int(seed)), ctypes.c_uint64(int(step)),
                             out.ctypes.data_as(_fp))
    return out


def verlet_step(x, v, f, masses, dt, force_fn):
    """Velocity Verlet, FP64: returns (x1, v1, f1)."""
    m = np.asarray(masses, dtype=np.float64).reshape(-1, 1)
    vh = v + 0.5 * dt * f / m
    x1 = x + dt * vh
    f1 = force_fn(x1)
    v1 = vh + 0.5 * dt * f1 / m
    return x1, v1, f1


def langevin_gjf_step(x, v, f, masses, dt, temperature, gamma, xi, force_fn):
    """Groenbech-Jensen--Farago step with supplied N(0,1) noise ``xi`` (N,3):
    x1 = x + b dt v + b dt^2/(2m) f + b dt/(2m) beta,
    v1 = a v + dt/(2m) (a f + f1) + b/m beta,  beta = sqrt(2 m gamma kT dt) xi,
    a = (1 - gamma dt/2)/(1 + gamma dt/2), b = 1/(1 + gamma dt/2).
    mdpy's LangevinIntegrator (mdpy/integrator/langevin_integrator.py:18-71)
    writes this scheme with the force sign flipped; the sign here is -grad V."""
    from mdpy_gb300 import unit as U

    m = np.asarray(masses, dtype=np.float64).reshape(-1, 1)
    kT = U.KB * temperature
    a = (1 - gamma * dt / 2) / (1 + gamma * dt / 2)
    b = 1 / (1 + gamma * dt / 2)
    beta = np.sqrt(2 * m * gamma * kT * dt) * np.asarray(xi, dtype=np.float64)
    x1 = x + b * dt * v + b * dt * dt / (2 * m) * f + b * dt / (2 * m) * beta
    f1 = force_fn(x1)
    v1 = a * v + dt / (2 * m) * (a * f + f1) + b / m * beta
    return x1, v1, f1


def kinetic_energy(v, masses):
    m = np.asarray(masses, dtype=np.float64).reshape(-1, 1)
    return 0.5 * float(np.sum(m * np.asarray(v, dtype=np.float64) ** 2))


def wrap_positions(positions, box):
    """mdpy's wrap_positions (mdpy/utils/pbc.py:28-36): x - L round(x inv),
    with inv the float32 inverse mdpy keeps (State.set_pbc_matrix,
    mdpy/core/state.py:53-54) -- so exact half-box coordinates wrap to the
    side mdpy puts them (+L/2 -> -L/2 when float32(1/L) > 1/L)."""
    b = np.broadcast_to(np.asarray(box, float), (3,))
    inv32 = (1.0 / b).astype(np.float32).astype(np.float64)
    return positions - b * np.round(np.asarray(positions, dtype=np.float64) * inv32)
