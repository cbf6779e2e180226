"""Collision outcome metrics (slh_collision_outcome) on hand-built states."""
import numpy as np

from spacelab_gb300 import configs, sweep


def _outcome(pos, R, n_t):
    from spacelab_gb300 import _lib
    import ctypes
    lf, sf, rg = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    nc = ctypes.c_int()
    m = np.ones(len(R))
    assert _lib.lib().slh_collision_outcome(len(R), n_t, _lib.dptr(np.ascontiguousarray(pos.reshape(-1))),
                                            _lib.dptr(R), _lib.dptr(m), 0.1, ctypes.byref(lf), ctypes.byref(sf),
                                            ctypes.byref(rg), ctypes.byref(nc)) == 0
    return lf.value, sf.value, rg.value, nc.value


def test_chain_and_separate_projectile():
    R = np.ones(5)
    # target: three touching spheres on x; projectile: two touching spheres far away
    pos = np.array([[0, 0, 0], [1.95, 0, 0], [3.9, 0, 0], [100, 0, 0], [101.95, 0, 0]], dtype=float)
    lf, sf, rg, nc = _outcome(pos, R, 3)
    assert nc == 2 and abs(lf - 0.6) < 1e-12 and sf == 0.0
    assert abs(rg - np.sqrt(((np.array([0, 1.95, 3.9]) - 1.95) ** 2).mean())) < 1e-12


def test_projectile_stuck_and_gap_threshold():
    R = np.ones(4)
    pos = np.array([[0, 0, 0], [2.05, 0, 0], [4.1, 0, 0], [6.3, 0, 0]], dtype=float)  # gaps 0.05, 0.05, 0.2
    lf, sf, rg, nc = _outcome(pos, R, 3)
    assert nc == 2 and abs(lf - 0.75) < 1e-12 and sf == 0.0
    pos[3, 0] = 6.19  # gap 0.09 < 0.1: the projectile sphere joins
    lf, sf, rg, nc = _outcome(pos, R, 3)
    assert nc == 1 and lf == 1.0 and sf == 1.0


def test_cluster_is_one_remnant_and_measured_rg():
    g = configs.build_cluster(300, 5, sigma_v=0.0)
    # a random packing at phi = 0.3 is not connected by touching: many remnants
    lf, sf, rg, nc = _outcome(g.pos / configs.RADIUS, g.R / configs.RADIUS, 300)
    assert nc > 1
    from spacelab_gb300 import _lib
    import ctypes
    r = ctypes.c_double()
    _lib.lib().slh_radius_of_gyration(300, _lib.dptr(np.ascontiguousarray(g.pos.reshape(-1))), _lib.dptr(g.m),
                                      ctypes.byref(r))
    # a uniform ball of radius a (N / phi)^(1/3) has Rg = sqrt(3/5) of it
    formula = np.sqrt(3.0 / 5.0) * (300 / configs.PHI) ** (1.0 / 3.0)
    assert abs(r.value / configs.RADIUS - formula) < 0.1 * formula
    # the sweep's features build the same cluster from the same seed
    assert sweep.cluster_rg(np.array([300]), np.array([5]))[0] == r.value / configs.RADIUS


def test_sweep_features_are_the_built_clusters_radii_of_gyration():
    from spacelab_gb300 import _lib
    import ctypes
    from spacelab_gb300 import batch as B
    cols = B.sample_collisions(6, seed=77, nt_range=(64, 200))
    x = sweep.features(cols)
    for c, row in zip(cols, x):
        r = ctypes.c_double()
        for lo, hi, col in ((0, c.n_t, 6), (c.n_t, c.n, 7)):
            pos = np.ascontiguousarray(c.group.pos[lo:hi].reshape(-1))
            _lib.lib().slh_radius_of_gyration(hi - lo, _lib.dptr(pos), _lib.dptr(np.ascontiguousarray(c.group.m[lo:hi])),
                                              ctypes.byref(r))
            # the collision shifts the clusters; Rg is about each one's own centre
            assert abs(row[col] - r.value / configs.RADIUS) <= 1e-12 * row[col]
