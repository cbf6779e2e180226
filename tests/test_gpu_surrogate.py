"""The collision-outcome surrogate: BF16 tensor-core MLP kernels checked
against the CPU oracle (oracle/mlp_oracle.py), training, the ensemble's
uncertainty, and a small end-to-end screened sweep that shows what the
network gains over simulating every point."""
import numpy as np
import pytest

from oracle import mlp_oracle
from spacelab_gb300 import batch as B
from spacelab_gb300 import surrogate as S
from spacelab_gb300 import sweep as W

pytestmark = pytest.mark.gpu

ARCH = dict(n_in=8, hidden=256, layers=4, n_out=4)


def _net(seed=1, max_batch=256):
    return S.Mlp(ARCH["n_in"], ARCH["n_out"], ARCH["hidden"], ARCH["layers"], max_batch=max_batch, seed=seed)


def _layer_slices():
    din, dout, offs, _ = mlp_oracle.layout(**ARCH)
    return [(w, w + a * b) for (w, _), a, b in zip(offs, din, dout)] + [(bo, bo + b) for (_, bo), b in zip(offs, dout)]


def test_mlp_forward_matches_cpu_oracle():
    net = _net()
    rng = np.random.default_rng(0)
    x = rng.normal(size=(100, 8)).astype(np.float32)
    y = net.predict(x)
    ref, *_ = mlp_oracle.forward(net.params(), x, **ARCH)
    scale = np.abs(ref).max()
    assert np.abs(y - ref).max() <= 1e-2 * scale


def test_mlp_gradients_match_cpu_oracle():
    net = _net()
    rng = np.random.default_rng(1)
    x = rng.normal(size=(128, 8)).astype(np.float32)
    y = rng.normal(size=(128, 4)).astype(np.float32)
    loss, g = net.gradients(x, y)
    l_ref, g_ref = mlp_oracle.loss_and_grads(net.params(), x, y, **ARCH)
    assert abs(loss - l_ref) <= 1e-3 * l_ref
    for a, b in _layer_slices():
        gr, gg = g_ref[a:b], g[a:b]
        nr = np.linalg.norm(gr)
        if nr == 0:
            assert np.abs(gg).max() == 0
            continue
        assert np.linalg.norm(gg - gr) <= 3e-2 * nr, (a, b)
        assert gg @ gr / (np.linalg.norm(gg) * nr) > 0.999


def test_mlp_learns_a_smooth_map():
    rng = np.random.default_rng(2)
    x = rng.uniform(-1, 1, size=(4096, 8)).astype(np.float32)
    y = np.stack([np.sin(2 * x[:, 0]) + x[:, 1] ** 2, x[:, 2] * x[:, 3], np.cos(x[:, 4] + x[:, 5]),
                  np.abs(x[:, 6]) - x[:, 7]], axis=1).astype(np.float32)
    net = _net(seed=3)
    curve = net.train(x, y, epochs=60, batch=256, lr=2e-3, seed=0)
    assert curve[-1] < curve[0] / 20
    xt = rng.uniform(-1, 1, size=(512, 8)).astype(np.float32)
    yt = np.stack([np.sin(2 * xt[:, 0]) + xt[:, 1] ** 2, xt[:, 2] * xt[:, 3], np.cos(xt[:, 4] + xt[:, 5]),
                   np.abs(xt[:, 6]) - xt[:, 7]], axis=1)
    assert np.mean((net.predict(xt) - yt) ** 2) < 0.05 * yt.var()


def test_ensemble_spread_grows_outside_the_data():
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, size=(2048, 8))
    y = np.stack([x[:, 0] + x[:, 1], x[:, 2] * 2, x[:, 3] ** 2, x[:, 4]], axis=1)
    ens = S.Ensemble(8, 4, members=5, seed=5)
    ens.fit(x, y, epochs=40, batch=256, lr=2e-3)
    _, s_in = ens.predict(rng.uniform(-1, 1, size=(256, 8)))
    _, s_out = ens.predict(rng.uniform(4, 6, size=(256, 8)))
    assert s_out.mean() > 3 * s_in.mean()


def test_screened_sweep_gains_over_simulating_every_point():
    """Small end to end: outcomes of 384 simulated collisions train the
    ensemble; a 3000-point sweep is screened; uncertain points and a 3%
    audit are re-run with the FP64 method.  The network must beat the
    method without it on cost, and on the audit its error must be below
    the outcomes' own spread (it predicts, not just averages)."""
    steps = 600
    train = B.sample_collisions(384, seed=11, nt_range=(16, 40), clearance=W.CLEARANCE, k_speed_div=W.K_SPEED_DIV)
    y, info = W.simulate(train, steps, mode="mixed_df")
    assert info["nonfinite"] == 0
    x = W.features(train)
    ens = S.Ensemble(8, 4, members=5, seed=9)
    ens.fit(x, y, epochs=150, batch=128, lr=1e-3)
    points = W.sample_params(3000, seed=12, nt_range=(16, 40))
    res = W.screen_sweep(ens, points, steps, threshold=1.0, audit=0.03, seed=13, sim_mode="exact")
    assert res["rerun"] < 0.5 * res["points"]
    assert res["cost_ratio"] > 2.0
    mae = np.array(res["audit_mae"])
    spread = np.array(res["outcome_std"])
    informative = spread > 1e-9
    assert np.all(mae[informative] < spread[informative])
