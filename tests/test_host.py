"""Host-side setup: seeded builder, deterministic primitives, spring/dt."""
import math

import numpy as np
import pytest

from spacelab_gb300 import _lib, configs


def test_det_log_exp_accuracy():
    lib = _lib.lib()
    xs = np.concatenate([np.logspace(-300, 300, 301), np.linspace(0.01, 3, 300)])
    for x in xs:
        assert abs(lib.slh_log(x) - math.log(x)) <= 4e-16 * max(1.0, abs(math.log(x)))
    for x in np.linspace(-50, 50, 401):
        assert abs(lib.slh_exp(x) - math.exp(x)) <= 2e-15 * math.exp(x)


def test_cluster_is_seeded_and_non_overlapping():
    a = configs.build_cluster(500, 7, sigma_v=1e-3)
    b = configs.build_cluster(500, 7, sigma_v=1e-3)
    c = configs.build_cluster(500, 8, sigma_v=1e-3)
    assert np.array_equal(a.pos, b.pos) and np.array_equal(a.vel, b.vel)
    assert not np.array_equal(a.pos, c.pos)
    d = np.sqrt(((a.pos[:, None, :] - a.pos[None, :, :]) ** 2).sum(-1))
    s = a.R[:, None] + a.R[None, :]
    np.fill_diagonal(d, np.inf)
    assert (d > s).all()
    com = (a.m[:, None] * a.pos).sum(0) / a.m.sum()
    assert np.abs(com).max() < 1e-18
    assert np.allclose(a.vel.std(), 1e-3, rtol=0.1)
    assert np.array_equal(a.w, np.zeros_like(a.w))
    rc = a.R.max() * (500 / 0.3) ** (1 / 3)
    assert np.linalg.norm(a.pos, axis=1).max() < 1.05 * rc


def test_polydisperse_radii():
    g = configs.build_cluster(2000, 3, sigma_v=1e-2, sigma_ln=0.2)
    med = np.median(g.R)
    assert 0.9e-4 < med < 1.1e-4
    assert g.R.min() >= 0.5e-4 and g.R.max() <= 2e-4
    assert np.allclose(np.log(g.R / 1e-4).std(), 0.2, rtol=0.1)
    np.testing.assert_allclose(g.moi, 0.4 * g.m * g.R ** 2, rtol=1e-15)


def test_collision_layout_and_zero_momentum():
    g = configs.build_collision(400, 100, 100.0, 1.1, 0.3, 1, 2, sigma_v=0.0)
    p = (g.m[:, None] * g.vel).sum(0)
    assert np.abs(p).max() < 1e-12 * (g.m.sum() * 100)
    ct = (g.m[:400, None] * g.pos[:400]).sum(0) / g.m[:400].sum()
    cp = (g.m[400:, None] * g.pos[400:]).sum(0) / g.m[400:].sum()
    Rt = 1e-4 * (400 / 0.3) ** (1 / 3)
    Rp = 1e-4 * (100 / 0.3) ** (1 / 3)
    np.testing.assert_allclose(cp - ct, [1.1 * (Rt + Rp), 0.3 * (Rt + Rp), 0.0], rtol=1e-9, atol=1e-15)
    assert np.all(g.vel[400:, 0] == -100.0)


def test_spring_and_dt_formula():
    kin, kout, dt = configs.spring_and_dt(1e-4, 7.12e-12, 10.0)
    kconsts = 3e3 * (4.0 / 3.0 * math.pi * 1.70) / 0.01
    assert kin == pytest.approx(kconsts * 1e-4 * 100.0, rel=1e-15)
    assert kout == pytest.approx(0.4096 * kin, rel=1e-15)
    assert dt * 50 == pytest.approx(math.pi * math.sqrt(7.12e-12 / (2 * kin)), rel=1e-14)


def test_workloads_shapes():
    w = configs.dust_cluster_1000()
    assert w.n == 1000 and w.steps == 2000 and w.skip == 100
    w1 = configs.aggregate_collision_5000()
    assert w1.n == 5000 and w1.pairs_per_step == 5000 * 4999 // 2
