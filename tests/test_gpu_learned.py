"""Learned slow force: features and network against FP64 / torch FP32
references, the training gradient, the multiple-time-step equations with
the learned prediction (held slow force when G = 0), the judge and its
impulse fallback, and bit-reproducibility."""
import numpy as np
import pytest

from tests import learned_ref as R

pytestmark = pytest.mark.gpu

RF = 6.0


def _ensemble(w, K=32):
    from tests.test_gpu_integrate import _ensemble as make

    return make(w, K=K)


def _params(seed, scale=1.0, zero_out=False):
    from mdpy_gb300 import learned as Lr

    rng = np.random.default_rng(seed)
    mu = rng.normal(0.0, 0.5, 64).astype(np.float32)
    sig = rng.uniform(0.2, 1.0, 64).astype(np.float32)
    p = Lr.init_params(rng, mu, sig, scale)
    p[Lr.W3:Lr.B3] = rng.normal(0.0, 0.3, 128 * 16)
    p[Lr.B3:Lr.SCALE] = rng.normal(0.0, 0.3, 16)
    if zero_out:
        p[Lr.W3:Lr.SCALE] = 0.0
    return p


def test_features_vs_fp64(lib):
    from mdpy_gb300 import systems, unit

    w = systems.water_box(900, 30.0, seed=3)
    ens = _ensemble(w)
    s = ens.system
    s.learned_config(RF, 1.0, 256)
    s.learned_set_params(_params(0))
    s.learned_frame(0)
    feat, vec, slow, _ = s.learned_frame_data(0)
    q = w.topology.charges * np.sqrt(unit.COULOMB_K)
    rf, rv = R.features(w.positions, q, w.box, RF, molecule=np.arange(len(q)) // 3)
    # FP32 sums of ~90 neighbours: relative error ~1e-6 of the channel scale
    assert np.abs(feat - rf).max() < 1e-4 * np.abs(rf).max()
    assert np.abs(vec - rv).max() < 1e-4 * np.abs(rv).max()
    # the frame's slow force is PME plus the excluded-pair correction
    probe = _ensemble(w)
    probe.system.compute_forces(lib.mask(lib.TERM_COUL_RECIP))
    ref = probe.system.get_forces()
    assert np.abs(slow - ref).max() < 1e-5 * np.abs(ref).max()


def test_forward_vs_torch(lib):
    import torch
    from mdpy_gb300 import systems

    w = systems.water_box(900, 30.0, seed=4)
    ens = _ensemble(w)
    s = ens.system
    s.learned_config(RF, 1.0, 256)
    p = _params(1)
    s.learned_set_params(p)
    s.learned_frame(0)
    feat, vec, _, pred = s.learned_frame_data(0)
    g = R.forward_torch(torch.tensor(p), torch.tensor(feat), torch.tensor(vec)).numpy()
    # FP32 sums in another order can move a BF16 rounding by one step
    assert np.sqrt(np.mean((pred - g) ** 2)) < 2e-3 * np.sqrt(np.mean(g ** 2))
    assert np.mean(np.abs(pred - g) <= 1e-4 * np.abs(g).max()) > 0.95


def test_train_step_loss_and_gradient_sign(lib):
    import torch
    from mdpy_gb300 import systems

    w = systems.water_box(900, 30.0, seed=5)
    ens = _ensemble(w)
    s = ens.system
    s.integrator_config(lib.INTEGRATOR_VERLET, 1.0)
    s.learned_config(RF, 1.0, 256)
    p = _params(2, scale=0.05)
    s.learned_set_params(p)
    s.learned_set_terms(False, True)
    s.learned_frame(0)
    s.integrate(3, ens.term_mask, want_energy=False)
    s.learned_frame(1)
    f0, v0, t0, _ = s.learned_frame_data(0)
    f1, v1, t1, _ = s.learned_frame_data(1)
    lr = 1e-4
    loss = s.learned_train_step(lr, 1)
    q = s.learned_params()
    pt = torch.tensor(p, requires_grad=True)
    g0 = R.forward_torch(pt, torch.tensor(f0), torch.tensor(v0))
    g1 = R.forward_torch(pt, torch.tensor(f1), torch.tensor(v1))
    dT = torch.tensor(t1 - t0, dtype=torch.float64)
    res = (g1 - g0).double() - dT
    L = (res ** 2).sum() / (dT ** 2).sum()
    L.backward()
    assert abs(loss - L.item()) < 1e-3 * L.item()
    grad = pt.grad.numpy()
    from mdpy_gb300 import learned as Lr

    trained = np.arange(Lr.N_PARAMS)
    trained = trained[(trained >= Lr.W1) & (trained != Lr.SCALE)]
    big = trained[np.abs(grad[trained]) > 1e-2 * np.abs(grad[trained]).max()]
    step = q[big] - p[big]
    # the first Adam step moves every parameter by lr against its gradient's sign
    agree = np.mean(np.sign(step) == -np.sign(grad[big]))
    assert agree > 0.99, agree
    assert np.allclose(np.abs(step), lr, rtol=0.05)
    # normalisation and output scale stay fixed
    assert np.array_equal(q[:Lr.W1], p[:Lr.W1]) and q[Lr.SCALE] == p[Lr.SCALE]


def test_learned_held_force_equations(lib):
    """G = 0: inner steps use the slow force of the last full evaluation;
    every k-th step uses the new one (weight 1); the judge reports the
    held force's error."""
    from mdpy_gb300 import systems

    w = systems.water_box(900, 30.0, seed=6)
    ens = _ensemble(w)
    probe = _ensemble(w)
    s, mask = ens.system, ens.term_mask
    recip = lib.mask(lib.TERM_COUL_RECIP)
    fast = mask & ~recip
    m = w.topology.masses.reshape(-1, 1)

    def forces(x, terms):
        probe.system.set_positions(x)
        probe.system.compute_forces(terms)
        return probe.system.get_forces()

    s.learned_config(RF, 1.0, 256)
    s.learned_set_params(_params(3, zero_out=True))
    s.learned_set_terms(False, True)
    s.integrator_config(lib.INTEGRATOR_VERLET, 1.0)
    k = 4
    s.set_mts_learned(k, 1e9)
    x, v = w.positions.copy(), w.velocities.copy()
    held = forces(x, recip)
    f = forces(x, fast) + held
    errs = []
    for step in range(8):
        s.integrate(1, mask, want_energy=False)
        x = x + v + 0.5 * f / m
        vh = v + 0.5 * f / m
        if (step + 1) % k == 0:
            new = forces(x, recip)
            fa = forces(x, fast)
            errs.append(np.sqrt(np.sum((held - new) ** 2) / np.sum((fa + new) ** 2)))
            held = new
            f = fa + new
        else:
            f = forces(x, fast) + held
        v = vh + 0.5 * f / m
        d = s.get_positions() - x
        d -= w.box * np.round(d / w.box)
        # (a wrong force would be off by ~1e-4 A; the probe's FP32 sums
        # round differently from the running system's)
        assert np.abs(d).max() < 5e-7, step
        assert np.abs(s.get_velocities() - v).max() < 5e-6 * np.abs(v).max(), step
    st = s.learned_stats()
    assert st["judged"] == 2 and st["fallbacks"] == 0 and st["mode"] == "learned"
    assert abs(st["last_err"] - errs[-1]) < 1e-3 * errs[-1]


def test_judge_falls_back_to_impulse(lib):
    """Threshold below any error: after the first judgement the intervals
    follow the impulse scheme; the boundary between a learned and an impulse
    interval carries the mean weight (1 + k) / 2."""
    from mdpy_gb300 import systems

    w = systems.water_box(900, 30.0, seed=7)
    ens = _ensemble(w)
    probe = _ensemble(w)
    s, mask = ens.system, ens.term_mask
    recip = lib.mask(lib.TERM_COUL_RECIP)
    fast = mask & ~recip
    m = w.topology.masses.reshape(-1, 1)

    def forces(x, terms):
        probe.system.set_positions(x)
        probe.system.compute_forces(terms)
        return probe.system.get_forces()

    s.learned_config(RF, 1.0, 256)
    s.learned_set_params(_params(4, zero_out=True))
    s.learned_set_terms(False, True)
    s.integrator_config(lib.INTEGRATOR_VERLET, 1.0)
    k = 4
    s.set_mts_learned(k, 1e-12)
    x, v = w.positions.copy(), w.velocities.copy()
    held = forces(x, recip)
    f = forces(x, fast) + held
    mode = "learned"
    for step in range(12):
        s.integrate(1, mask, want_energy=False)
        x = x + v + 0.5 * f / m
        vh = v + 0.5 * f / m
        fa = forces(x, fast)
        if (step + 1) % k == 0:
            new = forces(x, recip)
            w_prev = 1.0 if mode == "learned" else float(k)
            mode = "impulse"
            f = fa + 0.5 * (w_prev + k) * new
            held = new
        else:
            f = fa + (held if mode == "learned" else 0.0)
        v = vh + 0.5 * f / m
        d = s.get_positions() - x
        d -= w.box * np.round(d / w.box)
        assert np.abs(d).max() < 5e-7, step
    st = s.learned_stats()
    assert st["judged"] == 3 and st["fallbacks"] == 3 and st["mode"] == "impulse"


def test_learned_run_bit_reproducible(lib):
    from mdpy_gb300 import systems

    w = systems.water_box(900, 30.0, seed=8)
    out = []
    for _ in range(2):
        ens = _ensemble(w)
        s = ens.system
        s.learned_config(RF, 1.0, 256)
        s.learned_set_params(_params(5, scale=0.02))
        s.integrator_config(lib.INTEGRATOR_LANGEVIN, 1.0, 300.0, 1e-3, 11)
        s.set_mts_learned(4, 1e9)
        s.integrate(21, ens.term_mask, want_energy=True)
        out.append((s.get_positions(), s.get_energies()[0], s.learned_stats()["last_err"]))
        s.close()
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1]) and out[0][2] == out[1][2]


def test_training_runs_and_lowers_loss(lib):
    from mdpy_gb300 import systems
    from mdpy_gb300.learned import LearnedSlowForce

    w = systems.water_box(900, 30.0, seed=9)
    ens = _ensemble(w)
    s = ens.system
    learned = LearnedSlowForce(outer_step=2, rf=RF)
    losses = learned.train(s, iterations=60, lr=3e-3, decorrelate=2, mask=ens.term_mask)
    assert np.all(np.isfinite(losses))
    assert np.mean(losses[-10:]) < np.mean(losses[:10])
    # the trained network drives a learned run
    s.integrator_config(lib.INTEGRATOR_VERLET, 1.0)
    learned.enable(s)
    s.integrate(8, ens.term_mask, want_energy=True)
    st = s.learned_stats()
    assert st["judged"] == 4 and np.isfinite(st["last_err"])


def test_tensor_core_kernel_matches_simt(lib):
    """The tcgen05 inference kernel against the SIMT kernel on the same
    features (FP32 sums in another order: BF16 roundings may differ), and a
    learned run with each."""
    import torch
    from mdpy_gb300 import systems

    w = systems.water_box(900, 30.0, seed=10)
    ens = _ensemble(w)
    s = ens.system
    s.learned_config(RF, 1.0, 256)
    p = _params(6)
    s.learned_set_params(p)
    s.learned_frame(0)
    feat, vec, _, _ = s.learned_frame_data(0)
    s.learned_set_kernel(False)
    g_simt = s.learned_predict(0)
    s.learned_set_kernel(True)
    g_tc = s.learned_predict(0)
    ref = R.forward_torch(torch.tensor(p), torch.tensor(feat), torch.tensor(vec)).numpy()
    scale = np.sqrt(np.mean(ref ** 2))
    for g in (g_simt, g_tc):
        assert np.sqrt(np.mean((g - ref) ** 2)) < 2e-3 * scale
    assert np.sqrt(np.mean((g_tc - g_simt) ** 2)) < 2e-3 * scale
    assert np.mean(np.abs(g_tc - g_simt) <= 1e-4 * np.abs(ref).max()) > 0.95
    # learned runs with either kernel differ far less than either differs
    # from the run with G = 0 (the network's whole effect)
    pos = []
    for tc, scale in ((False, 0.02), (True, 0.02), (False, 0.0)):
        e = _ensemble(w)
        t = e.system
        t.learned_config(RF, 1.0, 256)
        t.learned_set_params(_params(7, scale=scale))
        t.learned_set_kernel(tc)
        t.integrator_config(lib.INTEGRATOR_VERLET, 1.0)
        t.set_mts_learned(4, 1e9)
        t.integrate(8, e.term_mask, want_energy=True)
        pos.append(t.get_positions())
        t.close()

    def dist(a, b):
        d = a - b
        d -= w.box * np.round(d / w.box)
        return np.sqrt(np.mean(d ** 2))

    assert dist(pos[0], pos[1]) < 1e-2 * dist(pos[0], pos[2])


def test_field_gradient_term_vs_finite_differences(lib):
    """With the field-gradient term alone, an inner step's slow force is
    F_slow(x0) + J (x1 - x0) with J_i = d F_slow,i / d x_i: compared with J
    from central differences of the slow force (atom i moved alone)."""
    from mdpy_gb300 import systems

    w = systems.water_box(900, 30.0, seed=11)
    ens = _ensemble(w)
    probe = _ensemble(w)
    s, mask = ens.system, ens.term_mask
    recip = lib.mask(lib.TERM_COUL_RECIP)
    fast = mask & ~recip

    def forces(x, terms):
        probe.system.set_positions(x)
        probe.system.compute_forces(terms)
        return probe.system.get_forces()

    s.learned_config(RF, 1.0, 256)
    s.learned_set_params(_params(8, zero_out=True))
    s.learned_set_terms(True, False)
    s.integrator_config(lib.INTEGRATOR_VERLET, 1.0)
    s.set_mts_learned(4, 1e9)
    x0 = w.positions.copy()
    f_slow0 = forces(x0, recip)
    s.integrate(1, mask, want_energy=False)
    x1 = s.get_positions()
    dx = x1 - x0
    dx -= w.box * np.round(dx / w.box)
    pred = s.get_forces() - forces(x1, fast) - f_slow0     # J (x1 - x0)
    atoms = [3 * m + a for m in (5, 200, 451, 777) for a in range(3)]
    h = 0.01
    err, ref = [], []
    for i in atoms:
        J = np.zeros((3, 3))
        for a in range(3):
            xp, xm = x0.copy(), x0.copy()
            xp[i, a] += h
            xm[i, a] -= h
            J[:, a] = (forces(xp, recip)[i] - forces(xm, recip)[i]) / (2 * h)
        fd = J @ dx[i]
        err.append(pred[i] - fd)
        ref.append(fd)
    err, ref = np.array(err), np.array(ref)
    # (B-spline second derivatives of an order-4 PME grid of ~0.94 A spacing)
    assert np.sqrt(np.mean(err ** 2)) < 0.15 * np.sqrt(np.mean(ref ** 2))


def test_tensor_core_wait_timeout_reports_and_recovers(lib):
    """The tcgen05 kernel's mbarrier waits are bounded by wall time.  The
    one-shot wait test withholds the kernel's first bulk copy, so its first
    wait runs out (10 ms): the call reports DeviceTimeoutError (no MMA or copy
    is in flight, the tensor memory is freed), and the next call works and
    gives the same prediction as before."""
    from mdpy_gb300 import systems
    from mdpy_gb300.error import DeviceTimeoutError

    w = systems.water_box(900, 30.0, seed=10)
    ens = _ensemble(w)
    s = ens.system
    s.learned_config(RF, 1.0, 256)
    s.learned_set_params(_params(6))
    s.learned_frame(0)
    s.learned_set_kernel(True)
    g0 = s.learned_predict(0)
    s.learned_wait_test()
    with pytest.raises(DeviceTimeoutError):
        s.learned_predict(0)
    g1 = s.learned_predict(0)
    assert np.array_equal(g0, g1)
    # and once more, after a second timed-out launch in a row
    s.learned_wait_test()
    with pytest.raises(DeviceTimeoutError):
        s.learned_predict(0)
    assert np.array_equal(s.learned_predict(0), g0)
    s.learned_set_kernel(False)
    with pytest.raises(Exception):
        s.learned_wait_test()   # only the tensor-core kernel has the test
