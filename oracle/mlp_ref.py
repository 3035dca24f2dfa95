"""CPU oracle of the learned warm start (numpy).

TEST INFRASTRUCTURE ONLY: imported by the tests, never by the library.

* ``features`` restates, from the CPU oracle's constraints, operator and rod
  state, the 12 features the GPU computes per collision constraint
  (alens_gb300/csrc/kernels_mlp.cu, ``mlp_features``).
* ``forward`` / ``loss_and_grad`` restate the network (12 -> 64 -> 64 -> 1,
  SiLU) and its backward pass, with the BF16 rounding points of the tensor-core
  kernels when ``rounding`` is on: features, W1, W2, w3, the first hidden
  activation and both pre-activation gradients are rounded to BF16 (round to
  nearest even); everything else is computed here in FP64.  With ``rounding``
  off the functions are the exact network, which the finite-difference test
  pins.

The learned warm start has no counterpart in the reference (aLENS /
SimToolbox start BBPGD from the ConstraintBlock's gamma,
SRC/TubuleSystem.cpp:727-736), so its parity is against this restatement.
"""
from __future__ import annotations

import numpy as np

N_IN = 12
HID = 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + HID * N_IN
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + HID
N_PARAMS = OFF_B3 + 1


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.asarray(x, dtype=np.float64).astype(np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    W1 = p[OFF_W1:OFF_B1].reshape(HID, N_IN)
    b1 = p[OFF_B1:OFF_W2]
    W2 = p[OFF_W2:OFF_B2].reshape(HID, HID)
    b2 = p[OFF_B2:OFF_W3]
    w3 = p[OFF_W3:OFF_B3]
    b3 = p[OFF_B3]
    return W1, b1, W2, b2, w3, b3


def _sig(a):
    return 1.0 / (1.0 + np.exp(-a))


def silu(a):
    return a * _sig(a)


def dsilu(a):
    s = _sig(a)
    return s * (1.0 + a * (1.0 - s))


def forward(p, X, rounding=True):
    """Network output y (n) and the intermediates for the backward pass."""
    r = bf16 if rounding else (lambda v: np.asarray(v, dtype=np.float64))
    W1, b1, W2, b2, w3, b3 = unpack(p)
    X = r(np.asarray(X, dtype=np.float64))
    W1r, W2r, w3r = r(W1), r(W2), r(w3)
    A1 = X @ W1r.T + b1
    H1 = r(silu(A1))
    A2 = H1 @ W2r.T + b2
    H2 = silu(A2)
    y = H2 @ w3r + b3
    return y, dict(X=X, A1=A1, H1=H1, A2=A2, H2=H2, W2r=W2r, w3r=w3r)


def loss_and_grad(p, X, t, rounding=True):
    """Mean squared error (1/n) sum (y - t)^2 and its gradient with respect
    to the parameter vector (same layout as the library's)."""
    r = bf16 if rounding else (lambda v: np.asarray(v, dtype=np.float64))
    y, c = forward(p, X, rounding)
    n = y.shape[0]
    diff = y - np.asarray(t, dtype=np.float64)
    loss = float(np.mean(diff * diff))
    dy = 2.0 * diff / n
    g = np.zeros(N_PARAMS)
    g[OFF_W3:OFF_B3] = c["H2"].T @ dy
    g[OFF_B3] = dy.sum()
    dA2 = r(dy[:, None] * c["w3r"][None, :] * dsilu(c["A2"]))
    g[OFF_W2:OFF_B2] = (dA2.T @ c["H1"]).ravel()
    g[OFF_B2:OFF_W3] = dA2.sum(axis=0)
    dH1 = dA2 @ c["W2r"]
    dA1 = r(dH1 * dsilu(c["A1"]))
    g[OFF_W1:OFF_B1] = (dA1.T @ c["X"]).ravel()
    g[OFF_B1:OFF_W2] = dA1.sum(axis=0)
    return loss, g


def features(con, op, q, rods, cfg, prev=None, dcp=None):
    """Features (n x 12) and scales A_kk/d (n) of the collision constraints.

    con   : oracle constraints (i, j, image, delta0) of the step, before solve
    op    : oracle operator (rowPtr, cols, vals) of the same step
    q     : QP linear term (n)
    rods  : RodState at detect time (positions, quaternions, lengths, radii)
    cfg   : AlensConfig (box, collision ratios)
    prev  : dict {(i, j, image): gamma} of the previous step, or None
    dcp   : function (c1, u1, h1, c2, u2, h2) -> (s, t) closest-point
            parameters (the oracle's segment distance)
    """
    from alens_gb300.workloads import quat_to_axis

    nc = int(con["ncoll"])
    ptr, cols, vals = op["rowPtr"], op["cols"], op["vals"]
    box = np.array([cfg.simBoxHigh[d] - cfg.simBoxLow[d] for d in range(3)])
    ax = quat_to_axis(rods.quat)
    L = rods.length
    rcol = rods.radius * cfg.sylinderDiameterColRatio
    sphere = L < 2.0 * rods.radius
    hcol = np.where(sphere, 0.0, 0.5 * L * cfg.sylinderLengthColRatio)
    counts = np.bincount(np.concatenate([con["i"], con["j"][con["j"] >= 0]]), minlength=rods.n)
    F = np.zeros((nc, N_IN))
    S = np.zeros(nc)
    kinds_unilateral = np.zeros(len(q), bool)
    kinds_unilateral[:nc] = True
    for k in range(nc):
        i, j, img = int(con["i"][k]), int(con["j"][k]), int(con["image"][k])
        d = rcol[i] + rcol[j]
        akk, nb = 0.0, 0.0
        for e in range(ptr[k], ptr[k + 1]):
            l = cols[e]
            if l == k:
                akk = vals[e]
            elif kinds_unilateral[l] and q[l] < 0.0:
                nb += vals[e] * (-q[l])
        if not (akk > 0.0):
            continue
        shift = np.array([img // 9 - 1, (img // 3) % 3 - 1, img % 3 - 1]) * box
        s, t = dcp(rods.pos[i], ax[i], hcol[i], rods.pos[j] + shift, ax[j], hcol[j])
        gp = prev.get((i, j, img), 0.0) if prev else 0.0
        F[k] = [con["delta0"][k] / d, max(0.0, -q[k]) / d, q[k] / d, abs(np.dot(ax[i], ax[j])), L[i], L[j],
                s / hcol[i] if hcol[i] > 0 else 0.0, t / hcol[j] if hcol[j] > 0 else 0.0,
                counts[i] / 8.0, counts[j] / 8.0, gp * akk / d, nb / akk / d]
        S[k] = akk / d
    return F, S
