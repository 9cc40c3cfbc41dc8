"""Learned slow force for the multiple-time-step form (no mdpy counterpart).

Full PME runs every ``outer_step``-th step.  In between, the slow force
(reciprocal space plus the excluded-pair correction) is predicted as
``F_slow(t0) + J (x(t) - x(t0)) + G(x(t)) - G(x(t0))``: J is each atom's
field-gradient matrix from the last PME evaluation (the change of its slow
force as it moves through the field of the others), and G a small
rotation-equivariant network evaluated on the device every step, trained on
what the first term leaves (libmdg: ``mdg_learned_*``; the network is
described in include/mdg.h).  Each full evaluation judges the prediction;
above ``threshold`` (RMS error over RMS total force) the next interval falls
back to the impulse scheme, and the learned form resumes when the judged
error is back under it.

The network is trained on frames the plain method generates: pairs of
configurations ``gap`` steps apart (1 <= gap <= outer_step) from a Langevin
run whose temperature is redrawn in ``temperatures`` every few iterations;
the loss is the squared error of G(x1) - G(x0) against the slow-force change,
relative to that change (1.0 = no better than holding the slow force).
Training and inference kernels are hand-written (BF16 operands, FP32
accumulation); the optimiser is Adam on an FP32 master copy.

    learned = LearnedSlowForce(outer_step=4)
    learned.train(system, iterations=400)
    system.set_mts_learned(4, learned.threshold)   # or Integrator(learned=...)
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib

N_FEAT, N_VEC, N_HIDDEN = 64, 16, 128
# offsets of the parameter vector (include/mdg.h)
MU, SIG = 0, 64
W1 = 128
B1 = W1 + N_FEAT * N_HIDDEN
W2 = B1 + N_HIDDEN
B2 = W2 + N_HIDDEN * N_HIDDEN
W3 = B2 + N_HIDDEN
B3 = W3 + N_HIDDEN * N_VEC
SCALE = B3 + N_VEC
N_PARAMS = SCALE + 1


def unpack(p):
    """Parameter vector -> dict of arrays (weights [in][out])."""
    p = np.asarray(p, dtype=np.float32)
    return {
        "mu": p[MU:SIG], "sig": p[SIG:W1],
        "w1": p[W1:B1].reshape(N_FEAT, N_HIDDEN), "b1": p[B1:W2],
        "w2": p[W2:B2].reshape(N_HIDDEN, N_HIDDEN), "b2": p[B2:W3],
        "w3": p[W3:B3].reshape(N_HIDDEN, N_VEC), "b3": p[B3:SCALE], "scale": p[SCALE],
    }


def init_params(rng, mu=None, sig=None, scale=1.0):
    """He-style initial weights, a small last layer, given normalisation."""
    p = np.zeros(N_PARAMS, dtype=np.float32)
    p[MU:SIG] = 0.0 if mu is None else mu
    p[SIG:W1] = 1.0 if sig is None else sig
    p[W1:B1] = rng.normal(0.0, math.sqrt(2.0 / N_FEAT), N_FEAT * N_HIDDEN)
    p[W2:B2] = rng.normal(0.0, math.sqrt(2.0 / N_HIDDEN), N_HIDDEN * N_HIDDEN)
    p[W3:B3] = rng.normal(0.0, 0.1 / math.sqrt(N_HIDDEN), N_HIDDEN * N_VEC)
    p[SCALE] = scale
    return p


class LearnedSlowForce:
    """Configuration, parameters and training of the learned slow force."""

    def __init__(self, outer_step=4, threshold=2e-3, rf=6.0, skin=1.0, list_capacity=256,
                 params=None, tensor_cores=True, field_gradient=False, network=True):
        if not 2 <= int(outer_step) <= 16:
            raise ValueError("outer_step must be in 2..16")
        self.outer_step = int(outer_step)
        self.threshold = float(threshold)
        self.rf, self.skin, self.list_capacity = float(rf), float(skin), int(list_capacity)
        self.params = None if params is None else np.asarray(params, np.float32).copy()
        self.tensor_cores = bool(tensor_cores)
        self.field_gradient, self.network = bool(field_gradient), bool(network)
        self.history = []
        self._attached = set()

    # ---- device plumbing -----------------------------------------------------
    def attach(self, system):
        """Configure the network's buffers on ``system`` (once) and load the
        parameters, if any."""
        if id(system) not in self._attached:
            system.learned_config(self.rf, self.skin, self.list_capacity)
            self._attached.add(id(system))
        if self.params is not None:
            system.learned_set_params(self.params)
        system.learned_set_kernel(self.tensor_cores)
        system.learned_set_terms(self.field_gradient, self.network)

    def enable(self, system):
        self.attach(system)
        system.set_mts_learned(self.outer_step, self.threshold)

    @staticmethod
    def disable(system):
        system.set_mts_learned(0, 1.0)

    # ---- training ---------------------------------------------------------------
    def _frames(self, system, gap, mask):
        system.learned_frame(0)
        system.integrate(int(gap), mask, want_energy=False)
        system.learned_frame(1)

    def normalise(self, system, mask=_lib.MASK_ALL, seed=0):
        """Feature shift/scale and output scale from one frame pair; fresh
        weights.  Also two diagnostics:

        ``baseline_loss``: the relative loss of G = 0 on the device's target
        (the slow-force change less the field-gradient term when that term is
        on): what the field-gradient term alone leaves of the change.

        ``pair_model_loss``: the slow force is a pair sum of the smooth Ewald
        kernel over all non-excluded pairs, so G with environment-independent
        coefficients C_b reproduces the part of its change that comes from
        pairs within rf; the relative loss of those 16 constants, fitted by
        least squares to the raw change.  Without the field-gradient term
        they become the output biases (the network's starting point)."""
        rng = np.random.default_rng(seed)
        self.attach(system)
        z = init_params(rng)
        z[W3:SCALE] = 0.0  # G = 0
        system.learned_set_params(z)
        self._frames(system, self.outer_step, mask)
        f0, v0, s0, _ = system.learned_frame_data(0)
        _, v1, s1, _ = system.learned_frame_data(1)
        self.baseline_loss = system.learned_train_step(1e-30, 1)
        mu = f0.mean(axis=0)
        sd = f0.std(axis=0)
        sig = np.where(sd > 1e-6, 1.0 / np.maximum(sd, 1e-6), 1.0)
        # outputs of order one: C_b ~ rms |F_slow| / rms |S_b|
        f_rms = float(np.sqrt(np.mean(np.sum(s0.astype(np.float64) ** 2, axis=1))))
        v_rms = float(np.sqrt(np.mean(np.sum(v0.astype(np.float64) ** 2, axis=2))))
        scale = f_rms / v_rms if v_rms > 0 else 1.0
        dv = (v1.astype(np.float64) - v0).transpose(0, 2, 1).reshape(-1, N_VEC)
        dt = (s1.astype(np.float64) - s0).reshape(-1)
        c, *_ = np.linalg.lstsq(dv, dt, rcond=None)
        res = dv @ c - dt
        self.pair_model_loss = float(np.sum(res ** 2) / max(np.sum(dt ** 2), 1e-300))
        self.params = init_params(rng, mu, sig, scale)
        if not self.field_gradient:
            self.params[B3:SCALE] = (c / scale).astype(np.float32)
        system.learned_set_params(self.params)

    def train(self, system, iterations=400, lr=2e-3, temperatures=(280.0, 320.0), dt=1.0,
              friction=1e-3, decorrelate=8, redraw_every=50, mask=_lib.MASK_ALL, seed=0,
              log_every=0):
        """Plain Langevin MD generates frame pairs; one Adam step per pair.
        Leaves the plain integrator configured (learned form off) and the
        parameters in ``self.params``; returns the loss history."""
        rng = np.random.default_rng(seed)
        self.attach(system)
        system.set_mts_learned(0, 1.0)
        system.integrator_config(_lib.INTEGRATOR_LANGEVIN, dt, float(temperatures[0]), friction,
                                 int(rng.integers(1 << 62)))
        if self.params is None:
            self.normalise(system, mask, seed)
        losses = []
        for it in range(int(iterations)):
            if it % int(redraw_every) == 0:
                T = float(rng.uniform(*temperatures))
                system.integrator_config(_lib.INTEGRATOR_LANGEVIN, dt, T, friction,
                                         int(rng.integers(1 << 62)))
            if decorrelate:
                system.integrate(int(decorrelate), mask, want_energy=False)
            gap = 1 + it % self.outer_step
            self._frames(system, gap, mask)
            # cosine decay to a tenth of the initial rate
            rate = lr * (0.1 + 0.9 * 0.5 * (1.0 + math.cos(math.pi * it / max(1, iterations))))
            loss = system.learned_train_step(rate, it + 1)
            losses.append(loss)
            if log_every and (it + 1) % log_every == 0:
                print("learned slow force: iteration %d loss %.4f" % (it + 1, loss), flush=True)
        self.params = system.learned_params()
        self.history.extend(losses)
        return losses

    def evaluate_loss(self, system, pairs=8, mask=_lib.MASK_ALL):
        """Mean relative loss over fresh frame pairs (no update): the
        forward pass of a training step is all that runs."""
        out = []
        for k in range(int(pairs)):
            gap = 1 + k % self.outer_step
            system.integrate(4, mask, want_energy=False)
            self._frames(system, gap, mask)
            _, _, s0, p0 = system.learned_frame_data(0)
            _, _, s1, p1 = system.learned_frame_data(1)
            d = s1 - s0
            r = (p1 - p0) - d
            out.append(float(np.sum(r.astype(np.float64) ** 2) / max(np.sum(d.astype(np.float64) ** 2), 1e-300)))
        return float(np.mean(out))

    # ---- persistence --------------------------------------------------------------
    def save(self, path):
        np.savez(path, params=self.params, outer_step=self.outer_step, threshold=self.threshold,
                 rf=self.rf, skin=self.skin, list_capacity=self.list_capacity)

    @classmethod
    def load(cls, path, **kw):
        z = np.load(path)
        return cls(outer_step=int(z["outer_step"]), threshold=float(z["threshold"]),
                   rf=float(z["rf"]), skin=float(z["skin"]),
                   list_capacity=int(z["list_capacity"]), params=z["params"], **kw)
