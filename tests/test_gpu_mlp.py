"""GPU checks of the learned warm start: the tensor-core forward pass, the
gradient of the training kernel and the per-constraint features against the
numpy oracle (oracle/mlp_ref.py), then training and the warm start itself.

Tolerances: the GPU and the oracle round to BF16 at the same points and
accumulate in FP32 (GPU) / FP64 (oracle); an element whose BF16 rounding
falls on the other side of a tie differs by one BF16 step (2^-8 relative),
so outputs are compared within 1e-2 of their scale and gradients within
2e-2 relative L2 per parameter group.
"""
import os
import sys

import numpy as np
import pytest

from alens_gb300 import capi, workloads
from alens_gb300.oracle_api import OracleSystem, dcp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import mlp_ref  # noqa: E402

pytestmark = pytest.mark.gpu

GROUPS = {"W1": (mlp_ref.OFF_W1, mlp_ref.OFF_B1), "b1": (mlp_ref.OFF_B1, mlp_ref.OFF_W2),
          "W2": (mlp_ref.OFF_W2, mlp_ref.OFF_B2), "b2": (mlp_ref.OFF_B2, mlp_ref.OFF_W3),
          "w3": (mlp_ref.OFF_W3, mlp_ref.OFF_B3), "b3": (mlp_ref.OFF_B3, mlp_ref.N_PARAMS)}


def random_batch(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, 12)).astype(np.float32)
    t = rng.standard_normal(n).astype(np.float32)
    return X, t


def test_forward_matches_oracle(gpu_lib):
    m = capi.Mlp(seed=11)
    p = m.params().astype(np.float64)
    for n in (1, 127, 128, 1000, 5000):
        X, _ = random_batch(n, n)
        y = m.predict(X)
        yr, _ = mlp_ref.forward(p, X, rounding=True)
        scale = max(1.0, float(np.max(np.abs(yr))))
        assert np.max(np.abs(y - yr)) <= 1e-2 * scale, n


def test_forward_with_set_params(gpu_lib):
    rng = np.random.default_rng(2)
    p = rng.uniform(-0.6, 0.6, capi.MLP_NUM_PARAMS).astype(np.float32)
    m = capi.Mlp(seed=0)
    m.set_params(p)
    assert np.array_equal(m.params(), p)
    X, _ = random_batch(777, 9)
    y = m.predict(X)
    yr, _ = mlp_ref.forward(p.astype(np.float64), X, rounding=True)
    assert np.max(np.abs(y - yr)) <= 1e-2 * max(1.0, float(np.max(np.abs(yr))))


@pytest.mark.parametrize("n", [100, 1000, 65536 + 300])
def test_gradient_matches_oracle(gpu_lib, n):
    m = capi.Mlp(seed=5)
    p = m.params().astype(np.float64)
    X, t = random_batch(n, 100 + n)
    g, loss = m.gradient(X, t)
    lr_, gr = mlp_ref.loss_and_grad(p, X, t, rounding=True)
    assert abs(loss - lr_) <= 1e-3 * max(1.0, lr_)
    for name, (a, b) in GROUPS.items():
        num = np.linalg.norm(g[a:b] - gr[a:b])
        den = np.linalg.norm(gr[a:b]) + 1e-12
        assert num <= 2e-2 * den, (name, num / den)


def test_training_reduces_loss(gpu_lib):
    """Fit a smooth target of the features with the library's Adam."""
    rng = np.random.default_rng(7)
    X = rng.uniform(-1, 1, (20000, 12)).astype(np.float32)
    t = (np.maximum(0, X[:, 1]) + 0.5 * X[:, 10] * X[:, 3]).astype(np.float32)
    m = capi.Mlp(seed=1, capacity=20000)
    m.add_samples(X, t)
    assert m.dataset_size() == 20000
    loss = m.train(epochs=30, batch=1024, lr=3e-3, seed=4)
    assert np.all(np.isfinite(loss))
    assert loss[-1] < 0.1 * loss[0], loss


def test_features_match_oracle(gpu_lib):
    w = workloads.small_periodic(n=1000, box=5.0, seed=0)
    g = capi.GpuSystem(w.cfg)
    o = OracleSystem(w.cfg)
    g.set_rods(w.rods)
    o.set_rods(w.rods)
    g.set_feature_capture(True)
    # the warm-start modes take the previous multiplier from the constraint
    # build instead of their own search: same features
    gp = capi.GpuSystem(workloads.config_with(w.cfg, warmStart=capi.WARM_PREV))
    gp.set_rods(w.rods)
    gp.set_feature_capture(True)
    prev = None
    for step in range(3):
        pos, quat = o.get_rods()
        rods = capi.RodState(w.rods.gid, pos, quat, w.rods.length, w.rods.radius)
        o.detect()
        con = o.constraints()
        op = o.operator()
        q, _ = o.solver_data()
        Fr, Sr = mlp_ref.features(con, op, q, rods, w.cfg, prev=prev,
                                  dcp=lambda *a: dcp(*a)[:2])
        o.solve()
        con2 = o.constraints()
        prev = {(int(a), int(b), int(c)): float(gm) for a, b, c, gm in
                zip(con2["i"], con2["j"], con2["image"], con2["gamma"])}
        o.advance()
        pg, qg = g.get_rods()
        gp.update_rods(pg, qg)
        g.step()
        F, S = g.features()
        gp.step()
        Fp, Sp = gp.features()
        # same state; the previous multipliers differ only at the solver
        # tolerance (the two systems solved their last step from different
        # starts)
        assert np.array_equal(Sp, S)
        assert np.array_equal(np.delete(Fp, 10, axis=1), np.delete(F, 10, axis=1))
        assert np.max(np.abs(Fp[:, 10] - F[:, 10])) <= 1e-2 * max(1.0, float(np.max(np.abs(F[:, 10]))))
        assert F.shape == Fr.shape
        np.testing.assert_allclose(S, Sr, rtol=1e-5)
        tol = 1e-4 * np.maximum(1.0, np.abs(Fr))
        bad = np.abs(F - Fr) > tol
        # contact parameters of (nearly) parallel pairs are ill-conditioned
        par = Fr[:, 3] > 0.9999
        bad[:, 6:8] &= ~par[:, None]
        assert not bad.any(), (step, np.argwhere(bad)[:5])
        if step > 0:
            assert np.any(F[:, 10] > 0)


def _mean_iterations(w, rods, warm, mlp=None, precision=capi.PREC_FP64, steps=8):
    cfg = workloads.config_with(w.cfg, precision=precision, warmStart=warm)
    g = capi.GpuSystem(cfg)
    g.set_rods(rods)
    if mlp is not None:
        g.attach_mlp(mlp)
    g.step()
    its = []
    for _ in range(steps):
        st = g.step(allow_not_converged=False)
        assert st["converged"] == 1 and st["residual"] <= cfg.conResTol
        its.append(st["iterations"])
    pos, _ = g.get_rods()
    g.close()
    return float(np.mean(its)), pos


def test_learned_warm_start_gain(gpu_lib):
    """Train on FP64 runs of config-1-shaped systems, then compare BBPGD
    iterations per step on held-out systems (other seeds, and the larger
    sparser evaluation shape) against the zero and previous-gamma starts.
    The warm start only seeds the solve: every step still reaches the
    residual tolerance and the trajectory stays within the solver's
    tolerance of the zero-start one."""
    from alens_gb300 import warmstart
    mlp, info = warmstart.build_model(samples=500_000, epochs=15, seed=3, rods=20000)
    assert info["train"]["loss_last"] < 0.2 * info["train"]["loss_first"]
    cases = [warmstart.config1_shaped(20000, 777), workloads.large_eval(60000, 26.0, seed=5)]
    for w in cases:
        g = capi.GpuSystem(w.cfg)
        g.set_rods(w.rods)
        for _ in range(3):
            g.step()
        pos, quat = g.get_rods()
        g.close()
        rods = capi.RodState(w.rods.gid, pos, quat, w.rods.length, w.rods.radius)
        it_zero, p_zero = _mean_iterations(w, rods, capi.WARM_ZERO)
        it_prev, _ = _mean_iterations(w, rods, capi.WARM_PREV)
        it_mlp, p_mlp = _mean_iterations(w, rods, capi.WARM_MLP, mlp)
        it_mlp_mixed, _ = _mean_iterations(w, rods, capi.WARM_MLP, mlp, precision=capi.PREC_MIXED)
        print(f"{w.name}: iterations/step zero {it_zero:.1f} prev {it_prev:.1f} "
              f"mlp {it_mlp:.1f} mlp+mixed {it_mlp_mixed:.1f}")
        assert it_mlp <= 0.92 * min(it_zero, it_prev), (it_zero, it_prev, it_mlp)
        assert it_mlp_mixed <= 0.92 * min(it_zero, it_prev)
        # same physics: trajectories agree to the solver tolerance's scale
        assert np.max(np.abs(p_mlp - p_zero)) < 1e-3
