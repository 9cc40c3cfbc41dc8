"""NumPy / torch FP32 references of the learned slow-force network (test
infrastructure: the GPU kernels of mdpy_gb300/csrc/mdg_learned*.cu are
checked against these).

Features of atom i (64): for 32 cubic B-spline bins phi_b(r) = B3(r/h1 - b),
h1 = rf/33, over neighbours 0 < r_ij < rf that are not 1-2 / 1-3 partners
of i: sum_j q_j phi_b (first 32) and
sum_j phi_b (next 32).  Vector basis (16 x 3): psi_b(r) = B3(r/h2 - b),
h2 = rf/17, S_ib = q_i sum_j q_j psi_b(r_ij) (x_i - x_j) / rf^2.  Charges are
q sqrt(k_e).  MLP: X = bf16((raw - mu) * sig); H1 = bf16(silu(X W1 + b1));
H2 = bf16(silu(H1 W2 + b2)); C = scale (H2 W3 + b3) (weights bf16, FP32
accumulation); G_i = sum_b C_ib S_ib.
"""
from __future__ import annotations

import numpy as np


def bspline3(t):
    """Centred uniform cubic B-spline (support |t| < 2)."""
    a = np.abs(t)
    out = np.zeros_like(a)
    m1 = a < 1.0
    m2 = (a >= 1.0) & (a < 2.0)
    out[m1] = (4.0 - 6.0 * a[m1] ** 2 + 3.0 * a[m1] ** 3) / 6.0
    out[m2] = (2.0 - a[m2]) ** 3 / 6.0
    return out


def features(pos, q, box, rf=6.0, molecule=None):
    """FP64 features (n, 64) and vector basis (n, 16, 3) of wrapped
    positions ``pos`` (n, 3) with charges ``q`` (q sqrt(k_e)).  Pairs within
    one ``molecule`` (ids per atom; rigid-topology waters: the 1-2 / 1-3
    pairs, which the library leaves out) are skipped."""
    from scipy.spatial import cKDTree

    pos = np.mod(np.asarray(pos, np.float64), box)
    pos = np.where(pos >= box, 0.0, pos)
    q = np.asarray(q, np.float64).ravel()
    n = len(pos)
    tree = cKDTree(pos, boxsize=box)
    pairs = tree.query_pairs(rf, output_type="ndarray")
    i = np.concatenate([pairs[:, 0], pairs[:, 1]])
    j = np.concatenate([pairs[:, 1], pairs[:, 0]])
    d = pos[i] - pos[j]
    d -= box * np.round(d / box)
    r = np.sqrt(np.sum(d * d, axis=1))
    keep = (r < rf) & (r > 0)
    if molecule is not None:
        mol = np.asarray(molecule).ravel()
        keep &= mol[i] != mol[j]
    i, j, d, r = i[keep], j[keep], d[keep], r[keep]
    h1, h2 = rf / 33.0, rf / 17.0
    feat = np.zeros((n, 64))
    vec = np.zeros((n, 16, 3))
    for b in range(32):
        w = bspline3(r / h1 - b)
        np.add.at(feat[:, b], i, q[j] * w)
        np.add.at(feat[:, 32 + b], i, w)
    for b in range(16):
        w = bspline3(r / h2 - b)
        for a in range(3):
            np.add.at(vec[:, b, a], i, q[j] * w * d[:, a])
    vec *= (q / rf ** 2)[:, None, None]
    return feat, vec


def _bf16(t):
    import torch

    return t.to(torch.bfloat16).to(torch.float32)


def forward_torch(params, raw, vec):
    """G (n, 3) of the network in torch FP32 with the kernels' BF16 rounding
    points; differentiable in the parameters (rounding passes gradients)."""
    import torch

    from mdpy_gb300 import learned as Lr

    p = params
    mu, sig = p[Lr.MU:Lr.SIG], p[Lr.SIG:Lr.W1]
    w1 = p[Lr.W1:Lr.B1].reshape(64, 128)
    b1 = p[Lr.B1:Lr.W2]
    w2 = p[Lr.W2:Lr.B2].reshape(128, 128)
    b2 = p[Lr.B2:Lr.W3]
    w3 = p[Lr.W3:Lr.B3].reshape(128, 16)
    b3 = p[Lr.B3:Lr.SCALE]
    scale = p[Lr.SCALE]
    x = _bf16((raw - mu) * sig)
    h1 = _bf16(torch.nn.functional.silu(x @ _bf16(w1) + b1))
    h2 = _bf16(torch.nn.functional.silu(h1 @ _bf16(w2) + b2))
    c = scale * (h2 @ _bf16(w3) + b3)
    return torch.einsum("nb,nba->na", c, vec)
